// eval_device.cuh -- per-chunk and per-tile bodies of the elementwise kernels,
// shared by the standalone launches (eval.cu) and the persistent batched
// executor (batch.cu).
#pragma once

#include "plan.h"
#include "program.cuh"

namespace phcu {

// ROW: VEC consecutive elements (chunk c) of the canonical space.  Inputs k with
// k >= p.nin are skipped, so an NIN=4 instantiation serves any input count.
template <int NIN, int VEC>
__device__ __forceinline__ void row_chunk(const EvalPlan& p, const phcu_program_t& prog, uint32_t c, uint32_t& st) {
  const int W = p.sp.rank - 1;
  const uint32_t e0 = c * VEC;
  uint32_t row, col;
  p.lendiv.divmod(e0, row, col);
  int64_t off_out = (int64_t)col * p.out.stride[W];
  int64_t off_in[NIN > 0 ? NIN : 1];
#pragma unroll
  for (int k = 0; k < NIN; k++) off_in[k] = (int64_t)col * p.in[k].stride[W];
  uint32_t r = row;
  for (int a = W - 1; a >= 0; a--) {
    uint32_t q, x;
    p.sp.div[a].divmod(r, q, x);
    r = q;
    off_out += (int64_t)x * p.out.stride[a];
#pragma unroll
    for (int k = 0; k < NIN; k++) off_in[k] += (int64_t)x * p.in[k].stride[a];
  }
  uint64_t in[NIN > 0 ? NIN : 1][VEC];
#pragma unroll
  for (int k = 0; k < NIN; k++) {
    if (k < p.nin) {
      const int es = dtype_size(p.in[k].dtype);
      load_operand<VEC>(p.in[k].base + off_in[k] * es, p.in[k].stride[W], p.in[k].dtype, p.in[k].vmode, in[k]);
    } else {
#pragma unroll
      for (int v = 0; v < VEC; v++) in[k][v] = 0;
    }
  }
  uint64_t acc[VEC];
  run_program<NIN, VEC>(prog, in, acc, st);
  const int oes = dtype_size(p.out.dtype);
  char* op = (char*)p.out.base + off_out * oes;
  if (p.out.vmode == VM_VEC) store_vec<VEC>(op, p.out.dtype, acc);
  else store_scalar<VEC>(op, p.out.stride[W] * oes, p.out.dtype, acc);
}

constexpr int TILE_THREADS = 256;

// TILE: one TILE x TILE tile t (all threads of the block take part; contains
// __syncthreads).  smem holds one TILE x (TILE+1) slot array per staged input.
template <int NIN>
__device__ __forceinline__ void tile_body(const EvalPlan& p, const phcu_program_t& prog, uint64_t t, uint64_t* smem,
                                          uint32_t& st) {
  const int W = p.sp.rank - 1;
  const int R = p.raxis;
  constexpr int LD = TILE + 1;
  constexpr int NWARP = TILE_THREADS / 32;
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

  // phase 1: staged inputs, coalesced along R
  int slot = 0;
#pragma unroll
  for (int k = 0; k < NIN; k++) {
    if (k >= p.nin || !(p.staged & (1u << k))) continue;
    uint64_t* tile = smem + (size_t)slot * TILE * LD;
    slot++;
    const int es = dtype_size(p.in[k].dtype);
    const int64_t sr = p.in[k].stride[R], sw = p.in[k].stride[W];
    const char* base = p.in[k].base + (off_in[k] + r0 * sr + w0 * sw) * es;
#pragma unroll
    for (int i = 0; i < TILE / NWARP; i++) {
      const int w = warp + i * NWARP;
#pragma unroll
      for (int j = 0; j < TILE / 32; j++) {
        const int r = lane + 32 * j;
        if (w < nw && r < nr) {
          uint64_t v[1];
          load_scalar<1>(base + ((int64_t)r * sr + (int64_t)w * sw) * es, 0, p.in[k].dtype, v);
          tile[w * LD + r] = v[0];
        }
      }
    }
  }
  if (p.staged) __syncthreads();

  // phase 2: compute and write coalesced along W
  const int oes = dtype_size(p.out.dtype);
  char* obase = (char*)p.out.base + (off_out + r0 * p.out.stride[R] + w0) * oes;
#pragma unroll 4
  for (int i = 0; i < TILE / NWARP; i++) {
    const int r = warp + i * NWARP;
#pragma unroll
    for (int j = 0; j < TILE / 32; j++) {
      const int w = lane + 32 * j;
      if (r < nr && w < nw) {
        uint64_t in[NIN > 0 ? NIN : 1][1];
        int s2 = 0;
#pragma unroll
        for (int k = 0; k < NIN; k++) {
          if (k >= p.nin) {
            in[k][0] = 0;
          } else if (p.staged & (1u << k)) {
            in[k][0] = smem[(size_t)s2 * TILE * LD + w * LD + r];
            s2++;
          } else {
            const int es = dtype_size(p.in[k].dtype);
            uint64_t v[1];
            load_scalar<1>(p.in[k].base +
                               (off_in[k] + (r0 + r) * p.in[k].stride[R] + (w0 + w) * p.in[k].stride[W]) * es,
                           0, p.in[k].dtype, v);
            in[k][0] = v[0];
          }
        }
        uint64_t acc[1];
        run_program<NIN, 1>(prog, in, acc, st);
        uint64_t o[1] = {acc[0]};
        store_scalar<1>(obase + ((int64_t)r * p.out.stride[R] + w) * oes, 0, p.out.dtype, o);
      }
    }
  }
  if (p.staged) __syncthreads();
}

inline size_t tile_smem_bytes(uint32_t staged) {
  return (size_t)__builtin_popcount(staged) * TILE * (TILE + 1) * sizeof(uint64_t);
}

}  // namespace phcu
