// eval_kernels.cuh -- the standalone ROW and TILE kernels and their launcher,
// instantiated per (slot type, input count) in eval_inst_*.cu so the
// translation units compile in parallel.
#pragma once

#include "eval_device.cuh"

namespace phcu {

struct TmaMaps;

struct EvalArgs {
  EvalPlan plan;
  phcu_program_t prog;
  uint32_t* status;
  const TmaMaps* tma = nullptr;  // host side: tensor maps of the staged inputs, when TMA can fetch them
};

constexpr int ROW_THREADS = 256;

// Copies and the Int32 division get four resident blocks per SM, everything
// else three: the kernels are latency-bound when registers limit residency.
template <int FAST>
constexpr int min_blocks() {
  return (FAST == FAST_COPY || FAST == FAST_IDIV) ? 4 : 3;
}

// ROW kernels of 32-bit in-place binary operators: 8 elements per thread at
// four resident blocks per SM.  Reversed-view binaries on 512x512x256 took
// 123 us per launch so (three blocks: 123, five: 129, six: 138, eight: 158;
// 16 elements at four blocks: 145; 32 at two: 200).  The ROW kernel of a
// pre-decoded 32-bit program fits 64 registers without spills: four resident
// blocks instead of three (fused chain 220 -> 187 us).
// The ROW Int32 / Int32 -> Float64 division over 8-element chunks fits 48
// registers without spills at five blocks per SM: 206 us instead of 221 at
// four on the reversed 512x512x256 views (the TMA division spills at five
// and keeps four; six blocks spill the ROW one too).
template <typename S, int FAST, int VEC>
constexpr int row_min_blocks() {
  return (FAST == FAST_BINOP && sizeof(S) == 4) ? 4
         : (FAST == FAST_FX && sizeof(S) == 4)  ? 4
         : (FAST == FAST_IDIV && VEC == 8)      ? 5
                                                : min_blocks<FAST>();
}

// ROW: each thread handles U grid-strided chunks of VEC elements per iteration.
// Interpreted programs are copied to shared memory first: the interpreter
// reads one instruction per step at a run-time index, which shared memory
// serves with one vector load (kernel-parameter space would serialise it).
template <typename S, int NIN, int VEC, int U, bool STASH, int FAST>
__global__ void __launch_bounds__(ROW_THREADS, row_min_blocks<S, FAST, VEC>())
    eval_row_kernel(const __grid_constant__ EvalArgs A) {
  const uint32_t nchunks = (uint32_t)(A.plan.sp.n / VEC);
  const uint32_t nthreads = gridDim.x * blockDim.x;
  // 64-bit position: the last steps may pass 2^32 when nchunks is close to it
  const uint64_t first = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t step = (uint64_t)nthreads * U;
  uint32_t st = 0;
  if constexpr (interpreted(FAST)) {
    __shared__ __align__(16) phcu_program_t s_prog;
    static_assert(sizeof(phcu_program_t) % 8 == 0, "program copied in 8-byte words");
    constexpr int WORDS = (int)(sizeof(phcu_program_t) / 8);
    for (int i = threadIdx.x; i < WORDS; i += blockDim.x)
      reinterpret_cast<uint2*>(&s_prog)[i] = reinterpret_cast<const uint2*>(&A.prog)[i];
    __syncthreads();
    for (uint64_t c0 = first; c0 < nchunks; c0 += step)
      row_group<S, NIN, VEC, U, STASH, FAST>(A.plan, s_prog, (uint32_t)c0, nthreads, nchunks, st);
  } else {
    for (uint64_t c0 = first; c0 < nchunks; c0 += step)
      row_group<S, NIN, VEC, U, STASH, FAST>(A.plan, A.prog, (uint32_t)c0, nthreads, nchunks, st);
  }
  if (st) report_status(A.status, st);
}

template <typename S, int NIN, bool STASH, int FAST>
__global__ void __launch_bounds__(TILE_THREADS, min_blocks<FAST>()) eval_tile_kernel(const __grid_constant__ EvalArgs A) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  S* smem = reinterpret_cast<S*>(smem_raw);
  uint32_t st = 0;
  const uint64_t ntiles = (uint64_t)A.plan.tiles_w * A.plan.tiles_r * A.plan.nbatch;
  for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) tile_body<S, NIN, STASH, FAST>(A.plan, A.prog, t, smem, st);
  if (st) report_status(A.status, st);
}

template <typename K>
static int32_t launch_grid(K kernel, const EvalArgs& A, uint64_t work_blocks, int threads, size_t smem,
                           const char* what) {
  Context& c = ctx();
  const int per_sm = blocks_per_sm((const void*)kernel, threads, smem);
  uint64_t grid = (uint64_t)c.sm_count * per_sm;
  if (grid > work_blocks) grid = work_blocks;
  if (grid < 1) grid = 1;
  kernel<<<(unsigned)grid, threads, smem, c.stream>>>(A);
  count_launch();
  return check_launch(what);
}

// Elements per thread per iteration: enough independent loads in flight
// without pushing the register count past the residency target (copies carry
// no interpreter state; stash registers cost the most).  32-bit binary
// operators take 8 and more resident blocks instead (row_min_blocks); more
// elements per thread were slower for every kernel measured (16 for
// interpreted programs: 233 -> 338 us on the fused chain).
template <typename S, bool STASH, int FAST>
constexpr int elements_per_thread() {
  return !interpreted(FAST) ? (sizeof(S) == 4 ? (FAST == FAST_BINOP ? 8 : 16) : 8)
                            : STASH ? 4 : (sizeof(S) == 4 ? 8 : 4);
}

template <typename S, int NIN, int VEC, bool STASH, int FAST>
static int32_t launch_row_vec(const EvalArgs& A) {
  constexpr int E = elements_per_thread<S, STASH, FAST>();
  constexpr int U = (VEC == 1) ? (E / 2 > 0 ? E / 2 : 1) : (E / VEC > 0 ? E / VEC : 1);
  const uint64_t n = (uint64_t)A.plan.sp.n;
  const uint64_t wb = (n / VEC + ROW_THREADS * U - 1) / (ROW_THREADS * U);
  return launch_grid(eval_row_kernel<S, NIN, VEC, U, STASH, FAST>, A, wb, ROW_THREADS, 0, "eval_row_kernel");
}

template <typename S, int NIN, bool STASH, int FAST>
static int32_t launch_row(const EvalArgs& A) {
  constexpr int E = elements_per_thread<S, STASH, FAST>();
  switch (A.plan.vec) {
    case 8:  // an 8-aligned plan is also 4-aligned: 4-element chunks when E < 8
      if constexpr (E >= 8) return launch_row_vec<S, NIN, 8, STASH, FAST>(A);
      else return launch_row_vec<S, NIN, 4, STASH, FAST>(A);
    case 4: return launch_row_vec<S, NIN, 4, STASH, FAST>(A);
    case 2: return launch_row_vec<S, NIN, 2, STASH, FAST>(A);
    default: return launch_row_vec<S, NIN, 1, STASH, FAST>(A);
  }
}

template <typename S, int NIN, bool STASH, int FAST>
static int32_t launch_tile(const EvalArgs& A) {
  const size_t smem = tile_smem_bytes<S>(A.plan.staged);
  const uint64_t ntiles = (uint64_t)A.plan.tiles_w * A.plan.tiles_r * A.plan.nbatch;
  return launch_grid(eval_tile_kernel<S, NIN, STASH, FAST>, A, ntiles, TILE_THREADS, smem, "eval_tile_kernel");
}

}  // namespace phcu

#include "tile_tma.cuh"

namespace phcu {

template <typename S, int NIN, bool STASH, int FAST>
static int32_t launch_tile_any(const EvalArgs& A) {
  if constexpr (NIN > 0) {
    if (A.tma) return launch_tma<S, NIN, STASH, FAST>(A);
  }
  return launch_tile<S, NIN, STASH, FAST>(A);
}

template <typename S, int NIN>
int32_t launch_eval_sn(const EvalArgs& A) {
  const bool stash = program_uses_stash(A.prog);
  const bool tile = A.plan.mode == MODE_TILE;
  if constexpr (NIN == 1) {
    if (program_is_copy(A.prog, A.plan))
      return tile ? launch_tile_any<S, NIN, false, FAST_COPY>(A) : launch_row<S, NIN, false, FAST_COPY>(A);
  }
  if constexpr (NIN == 2 && sizeof(S) == 8) {
    if (program_is_idiv(A.prog, A.plan))
      return tile ? launch_tile_any<S, NIN, false, FAST_IDIV>(A) : launch_row<S, NIN, false, FAST_IDIV>(A);
  }
  if constexpr (NIN == 2) {
    if (program_is_binop(A.prog, A.plan))
      return tile ? launch_tile_any<S, NIN, false, FAST_BINOP>(A) : launch_row<S, NIN, false, FAST_BINOP>(A);
  }
  if (!stash && program_is_fx(A.prog))
    return tile ? launch_tile_any<S, NIN, false, FAST_FX>(A) : launch_row<S, NIN, false, FAST_FX>(A);
  if (tile) return stash ? launch_tile_any<S, NIN, true, FAST_NONE>(A) : launch_tile_any<S, NIN, false, FAST_NONE>(A);
  return stash ? launch_row<S, NIN, true, FAST_NONE>(A) : launch_row<S, NIN, false, FAST_NONE>(A);
}

}  // namespace phcu
