// tile_tma.cuh -- the TILE launch shape with its staged inputs fetched by the
// Tensor Memory Accelerator.
//
// A staged input (contiguous along the tile's R axis, 4-byte elements) is
// described once per launch by a tensor map over the plan's axes
// [R, W, batch...].  One thread per block issues cp.async.bulk.tensor copies
// of two 32x64 boxes (128-byte rows, 128B swizzle) per input and tile into a
// ring of stages (one to four by kernel kind, tma_stages); an mbarrier per
// stage counts the bytes in.  The other
// threads spend no instructions on staging: each reads 16-byte chunks of four
// consecutive R elements of one W row (the swizzle puts the eight rows of a
// quarter-warp in eight different bank groups, so the transposed reads are
// conflict-free) and writes each of them to its output row, coalesced along W.
// Partial tiles read clamped coordinates (every value the program sees is a
// real element, as in the register-staged path) and guard their stores.
#pragma once

#include <cuda.h>

#include "async_copy.cuh"

namespace phcu {

constexpr uint32_t TMA_BOX_R = 32;                        // 4-byte elements per 128-byte box row
constexpr uint32_t TMA_BOX_BYTES = TILE * 128;            // 64 W rows of 128 bytes
constexpr uint32_t TMA_TILE_BYTES = 2 * TMA_BOX_BYTES;    // one staged input's 64x64 tile

// Tensor maps of the staged inputs, in staging order (bit order of plan.staged).
struct TmaMaps {
  CUtensorMap map[MAXIN];
  int32_t ndim;          // rank of every map: 2 + number of batch axes
  int32_t ext[5];        // extent of each map dimension
  uint32_t flip[MAXIN];  // per map: batch dimensions walked backwards (bit d: coordinate ext[d] - 1 - x)
  int32_t pad[6];
};

struct EvalTmaArgs {  // 64-byte aligned through CUtensorMap
  TmaMaps maps;
  EvalArgs a;
};

// One box of a tensor map into shared memory, completing on bar.
__device__ __forceinline__ void tma_load_box(const CUtensorMap* map, uint32_t dst, uint32_t bar, int ndim,
                                             const int32_t* c) {
  const uint64_t m = reinterpret_cast<uint64_t>(map);
  switch (ndim) {
    case 2:
      asm volatile(
          "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
          "[%4];" ::"r"(dst),
          "l"(m), "r"(c[0]), "r"(c[1]), "r"(bar)
          : "memory");
      break;
    case 3:
      asm volatile(
          "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
          "%4}], [%5];" ::"r"(dst),
          "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(bar)
          : "memory");
      break;
    case 4:
      asm volatile(
          "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
          "%4, %5}], [%6];" ::"r"(dst),
          "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(bar)
          : "memory");
      break;
    default:
      asm volatile(
          "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
          "%4, %5, %6}], [%7];" ::"r"(dst),
          "l"(m), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4]), "r"(bar)
          : "memory");
  }
}

// Tile t's origin, extent and per-operand element offsets; with COORDS, c
// receives the tensor-map coordinates {r0, w0, batch coordinates in axis order}.
template <int NIN, bool COORDS>
__device__ __forceinline__ void tma_tile_geom(const EvalPlan& p, uint64_t t, int64_t& r0, int64_t& w0, int& nr,
                                              int& nw, int64_t& off_out, int64_t* off_in, int32_t* c) {
  const int W = p.sp.rank - 1;
  const int R = p.raxis;
  uint32_t rest, tw, tr, b;
  p.tdiv_w.divmod((uint32_t)t, rest, tw);
  p.tdiv_r.divmod(rest, b, tr);
  off_out = 0;
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
    if constexpr (COORDS) {
      const int ci = 2 + a - (a > R ? 1 : 0);
      if (ci < 5) c[ci] = (int32_t)x;  // plans with more than 3 batch axes never take this path
    }
  }
  r0 = (int64_t)tr * TILE;
  w0 = (int64_t)tw * TILE;
  nr = (int)min((int64_t)TILE, p.sp.shape[R] - r0);
  nw = (int)min((int64_t)TILE, p.sp.shape[W] - w0);
  if constexpr (COORDS) {
    c[0] = (int32_t)r0;
    c[1] = (int32_t)w0;
  }
}

// A tile's origin, extent and per-operand offsets (tma_tile_geom).
template <int NIN>
struct TmaGeom {
  int64_t r0, w0, off_out;
  int64_t off_in[NIN > 0 ? NIN : 1];
  int nr, nw;
};

// Computes and stores one tile whose staged inputs sit in `stage`.
template <typename S, int NIN, bool STASH, int FAST>
__device__ __forceinline__ void tma_tile_body(const EvalPlan& p, const phcu_program_t& prog, const TmaGeom<NIN>& G,
                                              const unsigned char* stage, uint32_t& st) {
  const int64_t r0 = G.r0, w0 = G.w0, off_out = G.off_out;
  const int64_t* off_in = G.off_in;
  const int nr = G.nr, nw = G.nw;
  const int R = p.raxis;
  const int W = p.sp.rank - 1;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wl = lane + 32 * (warp & 1);  // this thread's W row of the tile (output column)
  const int cg = warp >> 1;               // its R range [16 cg, 16 cg + 16)
  const bool full = nr == TILE && nw == TILE;
  const int wc = min(wl, nw - 1);
  // chunks of four R elements per pass: 16 elements per thread in 1, 2 or 4
  // passes (one chunk at a time with 64-bit slots, which need twice the registers)
  constexpr int E = elements_per_thread<S, STASH, FAST>();
  constexpr int QP = sizeof(S) == 8 ? 1 : (E >= 16 ? 4 : (E >= 8 ? 2 : 1));
  constexpr int V = 4 * QP;
  const int64_t so_r = p.out.stride[R];
  const int oes = dtype_size(p.out.dtype);
  char* obase = (char*)p.out.base + (off_out + r0 * so_r + w0) * oes;
#pragma unroll 1
  for (int pass = 0; pass < 4 / QP; pass++) {
    const int rb = 16 * cg + 4 * QP * pass;  // R offset of in[.][0]
    S in[NIN > 0 ? NIN : 1][V];
    int s = 0;
#pragma unroll
    for (int k = 0; k < NIN; k++) {
      if (k >= p.nin) continue;
      if (p.staged & (1u << k)) {
        const unsigned char* tb = stage + (size_t)s * TMA_TILE_BYTES;
        s++;
        if (full) {
          const unsigned char* row = tb + (cg >> 1) * TMA_BOX_BYTES + wl * 128;
#pragma unroll
          for (int qq = 0; qq < QP; qq++) {
            const int cc = (cg & 1) * 4 + QP * pass + qq;
            const uint4 x = *reinterpret_cast<const uint4*>(row + ((cc ^ (wl & 7)) << 4));
            in[k][4 * qq + 0] = (S)x.x;
            in[k][4 * qq + 1] = (S)x.y;
            in[k][4 * qq + 2] = (S)x.z;
            in[k][4 * qq + 3] = (S)x.w;
          }
        } else {
#pragma unroll
          for (int v = 0; v < V; v++) {
            const int rc = min(rb + v, nr - 1);
            const int rr = rc & (int)(TMA_BOX_R - 1);
            in[k][v] = (S) * reinterpret_cast<const uint32_t*>(tb + (rc >> 5) * TMA_BOX_BYTES + wc * 128 +
                                                               (((rr >> 2) ^ (wc & 7)) << 4) + (rr & 3) * 4);
          }
        }
      } else {
        const int64_t sr = p.in[k].stride[R], sw = p.in[k].stride[W];
        const int es = dtype_size(p.in[k].dtype);
        const char* base = p.in[k].base + (off_in[k] + r0 * sr + w0 * sw) * es;
#pragma unroll
        for (int v = 0; v < V; v++) {
          const int64_t rc = full ? rb + v : min(rb + v, nr - 1);
          const int64_t e = rc * sr + (int64_t)wc * sw;
          switch (es) {
            case 4: in[k][v] = ld_elem<S, 4>(base + e * 4); break;
            case 8:
              if constexpr (sizeof(S) == 8) in[k][v] = ld_elem<S, 8>(base + e * 8);
              break;
            default: in[k][v] = ld_elem<S, 1>(base + e);
          }
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
    const bool wok = wl < nw;
    char* o = obase + ((int64_t)rb * so_r + wl) * oes;
    const int64_t ostep = so_r * oes;
    switch (oes) {
      case 4:
#pragma unroll
        for (int v = 0; v < V; v++)
          if (full || (wok && rb + v < nr)) st_elem<S, 4>(o + v * ostep, acc[v]);
        break;
      case 8:
        if constexpr (sizeof(S) == 8) {
#pragma unroll
          for (int v = 0; v < V; v++)
            if (full || (wok && rb + v < nr)) st_elem<S, 8>(o + v * ostep, acc[v]);
        }
        break;
      default:
#pragma unroll
        for (int v = 0; v < V; v++)
          if (full || (wok && rb + v < nr)) st_elem<S, 1>(o + v * ostep, acc[v]);
    }
  }
}

// Issues the copies of tile tt into stage stg (one thread).  Kept out of
// line so its coordinate array does not weigh on the compute loop's registers.
template <int NIN>
static __device__ __noinline__ void tma_issue(const EvalTmaArgs& T, uint64_t tt, int stg, uint32_t sb, uint32_t bar0) {
  const EvalPlan& p = T.a.plan;
  const uint32_t nst = (uint32_t)__popc(p.staged);
  int64_t r0, w0, oo;
  int64_t oi[NIN > 0 ? NIN : 1];
  int32_t c[5] = {0, 0, 0, 0, 0};
  int nr, nw;
  tma_tile_geom<NIN, true>(p, tt, r0, w0, nr, nw, oo, oi, c);
  const bool two = r0 + (int64_t)TMA_BOX_R < p.sp.shape[p.raxis];  // the second box holds R elements
  const uint32_t bar = bar0 + 8u * stg;
  const uint32_t stage_bytes = nst * TMA_TILE_BYTES;
  mbar_expect_tx(bar, nst * (two ? 2u : 1u) * TMA_BOX_BYTES);
  for (uint32_t s = 0; s < nst; s++) {
    const uint32_t dst = sb + stg * stage_bytes + s * TMA_TILE_BYTES;
    int32_t cs[5] = {c[0], c[1], c[2], c[3], c[4]};
    for (int d = 2; d < 5; d++)
      if (T.maps.flip[s] & (1u << d)) cs[d] = T.maps.ext[d] - 1 - c[d];
    tma_load_box(&T.maps.map[s], dst, bar, T.maps.ndim, cs);
    if (two) {
      cs[0] += (int32_t)TMA_BOX_R;
      tma_load_box(&T.maps.map[s], dst + TMA_BOX_BYTES, bar, T.maps.ndim, cs);
    }
  }
}

// Stages of the ring per kernel kind (each stage holds one tile of every
// staged input, 16 KB per input).  Copies keep three tiles in flight per
// block (four stages, 65 KB, three blocks per SM): the permuted gather of
// 512x512x256 Float32 took 86.9 us instead of 94.6 with two stages and
// 95.2 with three.  The Int32 / Int32 -> Float64 division, bound by its
// arithmetic, takes one stage (33 KB) so that four blocks fit instead of
// three: 230.9 us instead of 235.1.  Other kernels with two staged inputs
// keep two stages and three blocks per SM: three stages leave two blocks,
// and the permuted binary then took 143.7 us instead of 127.5 (the
// division 275.9).  At most three stages where four inputs can be staged:
// 3 x 4 x 16 KB + 1 KB stays under the 227 KB a block may use.
template <typename S, int FAST>
constexpr int tma_stages() {
  return FAST == FAST_COPY ? 4 : (FAST == FAST_IDIV ? 1 : 2);
}

// Persistent over tiles t = blockIdx.x + i * gridDim.x with an NST-stage
// ring: the copies of tile i + NST are issued as soon as every thread has
// finished reading tile i.  A copy that has not landed after TMA_WAIT_NS sets
// PHCU_ST_TIMEOUT and ends the block (after the same bounded wait for the
// copies of the other stages still in flight).
template <typename S, int NIN, bool STASH, int FAST>
__global__ void __launch_bounds__(TILE_THREADS, min_blocks<FAST>())
    eval_tma_kernel(const __grid_constant__ EvalTmaArgs T) {
  constexpr int NST = tma_stages<S, FAST>();
  const EvalPlan& p = T.a.plan;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bars[NST];
  const uint32_t raw = (uint32_t)__cvta_generic_to_shared(smem_raw);
  const uint32_t pad = (1024u - (raw & 1023u)) & 1023u;  // 128B swizzle wants 1024-byte aligned boxes
  const uint32_t sb = raw + pad;
  const unsigned char* sg = smem_raw + pad;
  const uint32_t nst = (uint32_t)__popc(p.staged);
  const uint32_t stage_bytes = nst * TMA_TILE_BYTES;
  const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(&bars[0]);
  const uint64_t ntiles = (uint64_t)p.tiles_w * p.tiles_r * p.nbatch;
  const uint64_t g = gridDim.x;

  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NST; j++) mbar_init(bar0 + 8u * j, 1);
    fence_mbar_init();
  }
  __syncthreads();

  uint32_t st = 0;
  uint64_t t = blockIdx.x;
  if (threadIdx.x == 0) {
    for (int j = 0; j < NST; j++)
      if (t + j * g < ntiles) tma_issue<NIN>(T, t + j * g, j, sb, bar0);
  }
  int stg = 0;        // stage of tile i
  uint32_t ph = 0;    // parity of its current use
  for (; t < ntiles; t += g) {
    // The division, bound by its arithmetic, works out the tile's geometry
    // while the copies are in flight (permuted 231.3 -> 225.1 us); the
    // memory-bound kinds lost 1-2% so and do it after the wait.
    TmaGeom<NIN> G;
    if constexpr (FAST == FAST_IDIV) tma_tile_geom<NIN, false>(p, t, G.r0, G.w0, G.nr, G.nw, G.off_out, G.off_in, nullptr);
    const bool ok = mbar_wait_bounded(bar0 + 8u * stg, ph, TMA_WAIT_NS);
    if (!__syncthreads_and(ok)) {
      st |= PHCU_ST_TIMEOUT;
      if (threadIdx.x == 0) {
        for (int j = 1; j < NST; j++) {  // tiles i + 1 .. i + NST - 1 are in flight
          if (t + j * g >= ntiles) break;
          const int s2 = stg + j < NST ? stg + j : stg + j - NST;
          mbar_wait_bounded(bar0 + 8u * s2, stg + j < NST ? ph : ph ^ 1u, TMA_WAIT_NS);
        }
      }
      break;
    }
    if constexpr (FAST != FAST_IDIV) tma_tile_geom<NIN, false>(p, t, G.r0, G.w0, G.nr, G.nw, G.off_out, G.off_in, nullptr);
    tma_tile_body<S, NIN, STASH, FAST>(p, T.a.prog, G, sg + stg * stage_bytes, st);
    __syncthreads();  // every thread is done with this stage
    if (threadIdx.x == 0 && t + NST * g < ntiles) {
      fence_proxy_async();
      tma_issue<NIN>(T, t + NST * g, stg, sb, bar0);
    }
    if (++stg == NST) {
      stg = 0;
      ph ^= 1u;
    }
  }
  if (st) report_status(T.a.status, st);
}

template <typename S, int FAST>
inline size_t tma_smem_bytes(uint32_t staged) {
  return tma_stages<S, FAST>() * (size_t)__builtin_popcount(staged) * TMA_TILE_BYTES + 1024;
}

template <typename S, int NIN, bool STASH, int FAST>
static int32_t launch_tma(const EvalArgs& A) {
  EvalTmaArgs T;
  T.maps = *A.tma;
  T.a = A;
  T.a.tma = nullptr;
  auto kernel = eval_tma_kernel<S, NIN, STASH, FAST>;
  const size_t smem = tma_smem_bytes<S, FAST>(A.plan.staged);
  Context& c = ctx();
  const int per_sm = blocks_per_sm((const void*)kernel, TILE_THREADS, smem);
  const uint64_t ntiles = (uint64_t)A.plan.tiles_w * A.plan.tiles_r * A.plan.nbatch;
  uint64_t grid = (uint64_t)c.sm_count * per_sm;
  if (grid > ntiles) grid = ntiles;
  if (grid < 1) grid = 1;
  kernel<<<(unsigned)grid, TILE_THREADS, smem, c.stream>>>(T);
  count_launch();
  return check_launch("eval_tma_kernel");
}

}  // namespace phcu
