// eval_device.cuh -- bodies of the elementwise kernels (gather, scatter, fill,
// infix operators, fused chains), shared by the standalone launches (eval.cu)
// and the persistent batched executor (batch.cu).
//
// Memory-level parallelism is the design goal: every thread issues all loads
// of U row chunks (ROW) or of its 16 tile elements (TILE) before it consumes
// any of them, and the element-type switches sit outside the element loops so
// the loads are straight-line code.
#pragma once

#include "plan.h"
#include "program.cuh"

namespace phcu {

constexpr int TILE_THREADS = 256;

// FAST selects how the per-element work runs: the interpreter (FAST_NONE), a
// plain move (FAST_COPY), an in-place binary operator (FAST_BINOP), the
// interpreter reduced to pre-decoded instructions (FAST_FX, program_is_fx) or
// Int32 / Int32 -> Float64 alone (FAST_IDIV, program_is_idiv; 64-bit slots).
enum : int { FAST_NONE = 0, FAST_COPY = 1, FAST_BINOP = 2, FAST_FX = 3, FAST_IDIV = 4 };
constexpr bool interpreted(int fast) { return fast == FAST_NONE || fast == FAST_FX; }

// ----------------------------------------------------------------- ROW
// U chunks of VEC consecutive elements: chunk u is c0 + u * cstep.
template <typename S, int NIN, int VEC, int U, bool STASH, int FAST>
__device__ __forceinline__ void row_group(const EvalPlan& p, const phcu_program_t& prog, uint32_t c0, uint32_t cstep,
                                          uint32_t nchunks, uint32_t& st) {
  constexpr int V = VEC * U;
  const int W = p.sp.rank - 1;
  int64_t off_out[U];
  int64_t off_in[NIN > 0 ? NIN : 1][U];
  bool valid[U];
#pragma unroll
  for (int u = 0; u < U; u++) {
    // a chunk past the end repeats chunk c0 (always valid): its values are
    // computed but not stored, so they raise no spurious status bits
    const uint64_t c64 = (uint64_t)c0 + (uint64_t)u * cstep;
    valid[u] = c64 < nchunks;
    const uint32_t c = valid[u] ? (uint32_t)c64 : c0;
    uint32_t row, col;
    p.lendiv.divmod(c * VEC, row, col);
    off_out[u] = (int64_t)col * p.out.stride[W];
#pragma unroll
    for (int k = 0; k < NIN; k++) off_in[k][u] = (int64_t)col * p.in[k].stride[W];
    for (int a = W - 1; a >= 0; a--) {
      uint32_t q, x;
      p.sp.div[a].divmod(row, q, x);
      row = q;
      off_out[u] += (int64_t)x * p.out.stride[a];
#pragma unroll
      for (int k = 0; k < NIN; k++) off_in[k][u] += (int64_t)x * p.in[k].stride[a];
    }
  }
  S in[NIN > 0 ? NIN : 1][V];
#pragma unroll
  for (int k = 0; k < NIN; k++) {
    if (k >= p.nin) continue;
    const char* base = p.in[k].base;
    const int64_t sw = p.in[k].stride[W];
    const int vm = p.in[k].vmode;
    if constexpr (interpreted(FAST)) {
      if (vm == VM_INDEX) {  // an index operand: Int32 value offset + coordinate . stride
        const int64_t i0 = (int64_t)(uintptr_t)base;
#pragma unroll
        for (int u = 0; u < U; u++)
#pragma unroll
          for (int i = 0; i < VEC; i++) in[k][u * VEC + i] = (S)(uint32_t)(i0 + off_in[k][u] + (int64_t)i * sw);
        continue;
      }
    }
    switch (dtype_size(p.in[k].dtype)) {
      case 4:
#pragma unroll
        for (int u = 0; u < U; u++)
          ld_operand<S, 4, VEC>(base + off_in[k][u] * 4, sw, vm, &in[k][u * VEC]);
        break;
      case 8:
        if constexpr (sizeof(S) == 8) {
#pragma unroll
          for (int u = 0; u < U; u++)
            ld_operand<S, 8, VEC>(base + off_in[k][u] * 8, sw, vm, &in[k][u * VEC]);
        }
        break;
      default:
#pragma unroll
        for (int u = 0; u < U; u++)
          ld_operand<S, 1, VEC>(base + off_in[k][u], sw, vm, &in[k][u * VEC]);
    }
  }
  S acc[V];
  if constexpr (FAST == FAST_COPY) {
#pragma unroll
    for (int v = 0; v < V; v++) acc[v] = in[0][v];
  } else if constexpr (FAST == FAST_BINOP && NIN >= 2) {
    run_binop<S, V>(prog, in[0], in[1], st);
#pragma unroll
    for (int v = 0; v < V; v++) acc[v] = in[0][v];
  } else if constexpr (FAST == FAST_IDIV && NIN >= 2 && sizeof(S) == 8) {
#pragma unroll
    for (int v = 0; v < V; v++) acc[v] = int32_div_f64_bits(si32(in[0][v]), si32(in[1][v]));
  } else if constexpr (FAST == FAST_FX) {
    run_program_fx<S, NIN, V>(prog, in, acc, st);
  } else {
    run_program<S, NIN, V, STASH>(prog, in, acc, st);
  }
  char* obase = (char*)p.out.base;
  const int64_t so = p.out.stride[W];
  const int om = p.out.vmode;
  switch (dtype_size(p.out.dtype)) {
    case 4:
#pragma unroll
      for (int u = 0; u < U; u++)
        if (valid[u]) st_operand<S, 4, VEC>(obase + off_out[u] * 4, so, om, &acc[u * VEC]);
      break;
    case 8:
      if constexpr (sizeof(S) == 8) {
#pragma unroll
        for (int u = 0; u < U; u++)
          if (valid[u]) st_operand<S, 8, VEC>(obase + off_out[u] * 8, so, om, &acc[u * VEC]);
      }
      break;
    default:
#pragma unroll
      for (int u = 0; u < U; u++)
        if (valid[u]) st_operand<S, 1, VEC>(obase + off_out[u], so, om, &acc[u * VEC]);
  }
}

// ----------------------------------------------------------------- TILE
constexpr int TILE_PER_THREAD = TILE * TILE / TILE_THREADS;  // 16

// Loads this thread's 16 elements of a TILE x TILE block of one staged input
// (coalesced along R).  Coordinates past the edge of a partial tile repeat the
// last valid element, so every value the program sees is a real element (no
// spurious status bits).
template <typename S, int ES>
__device__ __forceinline__ void stage_load(const char* base, int64_t sr, int64_t sw, int64_t nr, int64_t nw,
                                           S* v) {
  constexpr int NWARP = TILE_THREADS / 32;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < TILE / NWARP; i++) {
    const int64_t w = min((int64_t)(warp + i * NWARP), nw - 1);
#pragma unroll
    for (int j = 0; j < TILE / 32; j++) {
      const int64_t r = min((int64_t)(lane + 32 * j), nr - 1);
      v[i * (TILE / 32) + j] = ld_elem<S, ES>(base + (r * sr + w * sw) * ES);
    }
  }
}

// Asynchronous global -> shared copies (cp.async, no registers involved): the
// staged tile of an input with 4- or 8-byte elements is copied element by
// element, all copies of all inputs in flight before one wait.
template <int ES>
__device__ __forceinline__ void cp_async_elem(void* smem_dst, const void* gmem_src) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
  if constexpr (ES == 4) asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem_src));
  else asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem_src));
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::);
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

template <typename S, int ES>
__device__ __forceinline__ void stage_async(const char* base, int64_t sr, int64_t sw, int64_t nr, int64_t nw, S* tile) {
  constexpr int LD = TILE + 1;
  constexpr int NWARP = TILE_THREADS / 32;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < TILE / NWARP; i++) {
    const int wt = warp + i * NWARP;
    const int64_t w = min((int64_t)wt, nw - 1);
#pragma unroll
    for (int j = 0; j < TILE / 32; j++) {
      const int rt = lane + 32 * j;
      const int64_t r = min((int64_t)rt, nr - 1);
      cp_async_elem<ES>(&tile[wt * LD + rt], base + (r * sr + w * sw) * ES);
    }
  }
}

template <typename S>
__device__ __forceinline__ void stage_store(const S* v, S* tile) {
  constexpr int LD = TILE + 1;
  constexpr int NWARP = TILE_THREADS / 32;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < TILE / NWARP; i++) {
    const int w = warp + i * NWARP;
#pragma unroll
    for (int j = 0; j < TILE / 32; j++) tile[w * LD + lane + 32 * j] = v[i * (TILE / 32) + j];
  }
}

// Elements handled by one thread in phase 2: rows r = warp + NWARP*i (i < NI),
// columns w = lane + 32*j (j < TILE/32), i.e. NI*2 elements per pass.
template <typename S, int ES, int NI>
__device__ __forceinline__ void tile_direct_load(const char* base, int64_t sr, int64_t sw, int r_first, int64_t nr,
                                                 int64_t nw, S* out) {
  constexpr int NWARP = TILE_THREADS / 32;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NI; i++) {
    const int64_t r = min((int64_t)(r_first + warp + NWARP * i), nr - 1);
#pragma unroll
    for (int j = 0; j < TILE / 32; j++) {
      const int64_t w = min((int64_t)(lane + 32 * j), nw - 1);
      out[i * (TILE / 32) + j] = ld_elem<S, ES>(base + (r * sr + w * sw) * ES);
    }
  }
}

template <typename S, int ES, int NI>
__device__ __forceinline__ void tile_store(char* obase, int64_t so_r, int r_first, int64_t nr, int64_t nw,
                                           const S* acc) {
  constexpr int NWARP = TILE_THREADS / 32;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NI; i++) {
    const int r = r_first + warp + NWARP * i;
#pragma unroll
    for (int j = 0; j < TILE / 32; j++) {
      const int w = lane + 32 * j;
      if (r < nr && w < nw) st_elem<S, ES>(obase + ((int64_t)r * so_r + w) * ES, acc[i * (TILE / 32) + j]);
    }
  }
}

// One TILE x TILE tile t (every thread of the block takes part; contains
// __syncthreads).  smem holds one TILE x (TILE+1) array of S per staged input.
template <typename S, int NIN, bool STASH, int FAST>
__device__ __forceinline__ void tile_body(const EvalPlan& p, const phcu_program_t& prog, uint64_t t, S* smem,
                                          uint32_t& st) {
  const int W = p.sp.rank - 1;
  const int R = p.raxis;
  constexpr int LD = TILE + 1;
  constexpr int NWARP = TILE_THREADS / 32;
  // rows per pass: 8 (16 elements per thread) for copies and in-place binary
  // operators, 4 (8 elements) for interpreted programs; half with 64-bit slots
  constexpr int NI = (!interpreted(FAST) ? 8 : 4) / (sizeof(S) == 4 ? 1 : 2);
  constexpr int V = NI * (TILE / 32);
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  uint32_t rest, tw, tr, b;
  p.tdiv_w.divmod((uint32_t)t, rest, tw);
  p.tdiv_r.divmod(rest, b, tr);
  int64_t off_out = 0;
  int64_t off_in[NIN > 0 ? NIN : 1];
#pragma unroll
  for (int k = 0; k < NIN; k++) off_in[k] = 0;
  uint32_t bb = b;
  for (int a = W - 1; a >= 0; a--) {
    if (a == R) continue;
    uint32_t q, x;
    p.sp.div[a].divmod(bb, q, x);
    bb = q;
    off_out += (int64_t)x * p.out.stride[a];
#pragma unroll
    for (int k = 0; k < NIN; k++) off_in[k] += (int64_t)x * p.in[k].stride[a];
  }
  const int64_t r0 = (int64_t)tr * TILE, w0 = (int64_t)tw * TILE;
  const int64_t nr = min((int64_t)TILE, p.sp.shape[R] - r0);
  const int64_t nw = min((int64_t)TILE, p.sp.shape[W] - w0);

  // phase 1: staged inputs, coalesced along R.  4- and 8-byte elements go
  // straight to shared memory with cp.async (every input's copies in flight
  // at once, no registers); Bool goes through registers.
  {
    int slot = 0;
#pragma unroll
    for (int k = 0; k < NIN; k++) {
      if (k >= p.nin || !(p.staged & (1u << k))) continue;
      S* tile = smem + (size_t)slot * TILE * LD;
      slot++;
      const int64_t sr = p.in[k].stride[R], sw = p.in[k].stride[W];
      if (NIN == 1 && dtype_size(p.in[k].dtype) == 4) {
        // a single input: 16 register loads in flight per thread beat element-wise cp.async
        S v[TILE_PER_THREAD];
        stage_load<S, 4>(p.in[k].base + (off_in[k] + r0 * sr + w0 * sw) * 4, sr, sw, nr, nw, v);
        stage_store<S>(v, tile);
        continue;
      }
      switch (dtype_size(p.in[k].dtype)) {
        case 4: stage_async<S, 4>(p.in[k].base + (off_in[k] + r0 * sr + w0 * sw) * 4, sr, sw, nr, nw, tile); break;
        case 8:
          if constexpr (sizeof(S) == 8)
            stage_async<S, 8>(p.in[k].base + (off_in[k] + r0 * sr + w0 * sw) * 8, sr, sw, nr, nw, tile);
          break;
        default: {
          S v[TILE_PER_THREAD];
          stage_load<S, 1>(p.in[k].base + (off_in[k] + r0 * sr + w0 * sw), sr, sw, nr, nw, v);
          stage_store<S>(v, tile);
        }
      }
    }
    cp_async_wait_all();
  }
  __syncthreads();

  // phase 2: compute and write coalesced along W, V elements per pass
  char* obase = (char*)p.out.base;
  const int64_t so_r = p.out.stride[R];
  const int oes = dtype_size(p.out.dtype);
  obase += (off_out + r0 * so_r + w0) * oes;
#pragma unroll 1
  for (int pass = 0; pass < (TILE / NWARP) / NI; pass++) {
    const int r_first = pass * NI * NWARP;
    S in[NIN > 0 ? NIN : 1][V];
    int s2 = 0;
#pragma unroll
    for (int k = 0; k < NIN; k++) {
      if (k >= p.nin) continue;
      if (p.staged & (1u << k)) {
        const S* tile = smem + (size_t)s2 * TILE * LD;
        s2++;
#pragma unroll
        for (int i = 0; i < NI; i++) {
#pragma unroll
          for (int j = 0; j < TILE / 32; j++)
            in[k][i * (TILE / 32) + j] = tile[(lane + 32 * j) * LD + r_first + warp + NWARP * i];
        }
      } else {
        const int64_t sr = p.in[k].stride[R], sw = p.in[k].stride[W];
        switch (dtype_size(p.in[k].dtype)) {
          case 4:
            tile_direct_load<S, 4, NI>(p.in[k].base + (off_in[k] + r0 * sr + w0 * sw) * 4, sr, sw, r_first, nr, nw,
                                       in[k]);
            break;
          case 8:
            if constexpr (sizeof(S) == 8)
              tile_direct_load<S, 8, NI>(p.in[k].base + (off_in[k] + r0 * sr + w0 * sw) * 8, sr, sw, r_first, nr,
                                         nw, in[k]);
            break;
          default:
            tile_direct_load<S, 1, NI>(p.in[k].base + (off_in[k] + r0 * sr + w0 * sw), sr, sw, r_first, nr, nw,
                                       in[k]);
        }
      }
    }
    S acc[V];
    if constexpr (FAST == FAST_COPY) {
#pragma unroll
      for (int v = 0; v < V; v++) acc[v] = in[0][v];
    } else if constexpr (FAST == FAST_BINOP && NIN >= 2) {
      run_binop<S, V>(prog, in[0], in[1], st);
#pragma unroll
      for (int v = 0; v < V; v++) acc[v] = in[0][v];
    } else if constexpr (FAST == FAST_IDIV && NIN >= 2 && sizeof(S) == 8) {
#pragma unroll
      for (int v = 0; v < V; v++) acc[v] = int32_div_f64_bits(si32(in[0][v]), si32(in[1][v]));
    } else if constexpr (FAST == FAST_FX) {
      run_program_fx<S, NIN, V>(prog, in, acc, st);
    } else {
      run_program<S, NIN, V, STASH>(prog, in, acc, st);
    }
    switch (oes) {
      case 4: tile_store<S, 4, NI>(obase, so_r, r_first, nr, nw, acc); break;
      case 8:
        if constexpr (sizeof(S) == 8) tile_store<S, 8, NI>(obase, so_r, r_first, nr, nw, acc);
        break;
      default: tile_store<S, 1, NI>(obase, so_r, r_first, nr, nw, acc);
    }
  }
  __syncthreads();
}

template <typename S>
inline size_t tile_smem_bytes(uint32_t staged) {
  return (size_t)__builtin_popcount(staged) * TILE * (TILE + 1) * sizeof(S);
}

// ------------------------------------------------------- program traits
// Whether every value the program (and its operands) touches fits 32 bits.
inline bool program_is_32bit(const phcu_program_t& P, const EvalPlan& plan) {
  auto wide = [](int t) { return t == PHCU_I64 || t == PHCU_F64; };
  if (wide(P.out_type) || wide(plan.out.dtype)) return false;
  for (int k = 0; k < plan.nin; k++)
    if (wide(plan.in[k].dtype)) return false;
  for (int i = 0; i < P.n_instr; i++) {
    const phcu_instr_t& I = P.code[i];
    if (wide(I.type) || wide(I.btype)) return false;
    if (I.op == PHCU_I_CVT && wide((int)I.imm.i)) return false;
    if (I.op == PHCU_OP_DIV && is_int_t(I.type)) return false;  // Int / Int -> Float64
  }
  return true;
}

inline bool program_uses_stash(const phcu_program_t& P) {
  for (int i = 0; i < P.n_instr; i++) {
    const phcu_instr_t& I = P.code[i];
    if (I.op == PHCU_I_ST0 || I.op == PHCU_I_ST1 || I.op == PHCU_I_SEL) return true;
  }
  return false;
}

// A plain move: one input, one LD of its own type into an output of that type.
// [ACC = IN0 (its own type); ACC = ACC op IN1 (IN1 already of the compute
// type, or an integer exponent); optional CVT]: runs in place (run_binop).
inline bool plan_has_index(const EvalPlan& plan) {
  for (int k = 0; k < plan.nin; k++)
    if (plan.in[k].vmode == VM_INDEX) return true;
  return false;
}

inline bool program_is_binop(const phcu_program_t& P, const EvalPlan& plan) {
  if (plan.nin != 2 || P.n_instr < 2 || P.n_instr > 3 || plan_has_index(plan)) return false;
  const phcu_instr_t& a = P.code[0];
  const phcu_instr_t& b = P.code[1];
  if (a.op != PHCU_I_LD || a.src != 0 || a.type != a.btype || a.type != plan.in[0].dtype) return false;
  if (b.op >= PHCU_OP_NBINARY || b.src != 1 || (b.flags & 1) || b.type != a.type || b.btype != plan.in[1].dtype)
    return false;
  const bool int_exp = b.op == PHCU_OP_POW && is_float_t(b.type) && is_int_t(b.btype);
  if (!int_exp && b.btype != b.type) return false;
  if (P.n_instr == 3 && P.code[2].op != PHCU_I_CVT) return false;
  return true;
}

// [ACC = IN0 (Int32); ACC = ACC / IN1 (Int32)] into a Float64 output: the
// exact division alone, without the binary operator's run-time dispatch.
inline bool program_is_idiv(const phcu_program_t& P, const EvalPlan& plan) {
  return program_is_binop(P, plan) && P.n_instr == 2 && P.code[1].op == PHCU_OP_DIV && P.code[1].type == PHCU_I32 &&
         plan.in[0].dtype == PHCU_I32 && plan.in[1].dtype == PHCU_I32 && plan.out.dtype == PHCU_F64;
}

inline bool program_is_copy(const phcu_program_t& P, const EvalPlan& plan) {
  return plan.nin == 1 && !plan_has_index(plan) && P.n_instr == 1 && P.code[0].op == PHCU_I_LD && P.code[0].src == 0 &&
         P.code[0].type == P.code[0].btype && P.code[0].type == plan.in[0].dtype && P.out_type == plan.out.dtype &&
         plan.in[0].dtype == plan.out.dtype;
}

}  // namespace phcu
