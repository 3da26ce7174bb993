// stencil.cu -- explicit 2-D heat step and its CUDA-graph driver.
//
// The Phase program of one step (examples/heat_equation.cr:38-51 generalised to
// 2-D shifted views):
//   c   = u[1..-2, 1..-2]
//   lap = u[0..-3, 1..-2] + u[2.., 1..-2] + u[1..-2, 0..-3] + u[1..-2, 2..] - c * 4
//   u[1..-2, 1..-2] = c + lap * coef
// is fused into one pass: every interior point evaluates the infix chain left to
// right in the element type (no FMA: this file is compiled with -fmad=false),
// the boundary is copied.  Each thread walks a column strip, keeping
// up/centre/down in registers; left/right come from the neighbouring lanes by
// warp shuffle, so each element is read from memory about once per step.
// The Float64 instantiation is the reference run the Float32 error is measured
// against.
#include <map>
#include <tuple>

#include "common.cuh"

namespace phcu {

constexpr int HEAT_COLS = 128;
constexpr int HEAT_ROWS = 16;

template <typename T>
__global__ void __launch_bounds__(HEAT_COLS) heat_step_kernel(const T* __restrict__ u, T* __restrict__ out, int64_t n,
                                                              int64_t m, T coef) {
  const int64_t j = (int64_t)blockIdx.x * HEAT_COLS + threadIdx.x;
  const int64_t i0 = (int64_t)blockIdx.y * HEAT_ROWS;
  const int lane = threadIdx.x & 31;
  const bool jin = j < m;
  const int64_t jc = jin ? j : m - 1;  // lanes past the edge still take part in the shuffles
  // the whole column strip (rows i0-1 .. i0+HEAT_ROWS) is loaded up front, all
  // loads in flight at once; the warp's edge lanes also load their outer
  // neighbour column
  T col[HEAT_ROWS + 2];
#pragma unroll
  for (int r = 0; r < HEAT_ROWS + 2; r++) {
    const int64_t i = i0 - 1 + r;
    col[r] = (i >= 0 && i < n) ? __ldg(u + i * m + jc) : (T)0;
  }
  T side[HEAT_ROWS];
  const bool edge = (lane == 0) || (lane == 31);
  const int64_t js = (lane == 0) ? jc - 1 : jc + 1;
  const bool side_ok = edge && js >= 0 && js < m;
#pragma unroll
  for (int r = 0; r < HEAT_ROWS; r++) {
    const int64_t i = i0 + r;
    side[r] = (side_ok && i < n) ? __ldg(u + i * m + js) : (T)0;
  }
#pragma unroll
  for (int r = 0; r < HEAT_ROWS; r++) {
    const int64_t i = i0 + r;
    if (i >= n) break;  // uniform across the block
    const T up = col[r], c = col[r + 1], down = col[r + 2];
    T left = __shfl_up_sync(0xffffffffu, c, 1);
    T right = __shfl_down_sync(0xffffffffu, c, 1);
    if (lane == 0) left = side[r];
    if (lane == 31) right = side[r];
    if (jin) {
      T res;
      if (i == 0 || i == n - 1 || j == 0 || j == m - 1) {
        res = c;
      } else {
        T lap = up + down;
        lap = lap + left;
        lap = lap + right;
        const T c4 = c * (T)4;
        lap = lap - c4;
        const T d = lap * coef;
        res = c + d;
      }
      out[i * m + j] = res;
    }
  }
}

// Temporal blocking: one launch advances the grid by up to HEAT_K steps.  A
// block loads its output tile (HEAT_TR x HEAT_TC) plus a halo of HEAT_K cells
// into shared memory (HEAT_SR x HEAT_SC = 72 x 128) and applies the step
// HEAT_K times there, ping-ponging between two buffers; after s steps the
// cells at least s from the halo's edge are exact, so after ksteps <= HEAT_K
// steps the centre is, and it is written out.  Every cell evaluates the same
// left-to-right infix chain as the one-step kernel on the same inputs, so the
// result is bit-identical to ksteps single steps; the grid's boundary cells
// copy themselves each step, and cells outside the grid (zero in the halo)
// never reach an exact cell.  Each warp walks its own band of rows; each lane
// takes four consecutive cells of a row with vector accesses (a warp covers
// the whole 128-cell shared row: no bank conflicts).
// Six steps per launch: 1000 steps of 4096^2 take 16.0 ms (four: 17.3 ms,
// eight: 16.0 ms; 104-row tiles: 19-21 ms).
constexpr int HEAT_K = 6;
constexpr int HEAT_SR = 72, HEAT_SC = 128;  // shared tile: rows x columns
constexpr int HEAT_TR = HEAT_SR - 2 * HEAT_K, HEAT_TC = HEAT_SC - 2 * HEAT_K;  // 60 x 116 written
constexpr int HEAT_BLOCK_THREADS = 256;

// four consecutive shared-memory cells (16-byte aligned for Float32, 32 for Float64)
__device__ __forceinline__ void heat_ld4(const float* p, float* v) {
  const float4 x = *reinterpret_cast<const float4*>(p);
  v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
}
__device__ __forceinline__ void heat_ld4(const double* p, double* v) {
  const double2 x = *reinterpret_cast<const double2*>(p);
  const double2 y = *reinterpret_cast<const double2*>(p + 2);
  v[0] = x.x; v[1] = x.y; v[2] = y.x; v[3] = y.y;
}
__device__ __forceinline__ void heat_st4(float* p, const float* v) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void heat_st4(double* p, const double* v) {
  *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
  *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
}

template <typename T>
__global__ void __launch_bounds__(HEAT_BLOCK_THREADS) heat_block_kernel(const T* __restrict__ u, T* __restrict__ out,
                                                                        int64_t n, int64_t m, T coef, int ksteps) {
  extern __shared__ __align__(16) unsigned char heat_smem[];
  T* buf0 = reinterpret_cast<T*>(heat_smem);
  T* buf1 = buf0 + HEAT_SR * HEAT_SC;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t i0 = (int64_t)blockIdx.y * HEAT_TR - HEAT_K;  // global row of local row 0
  const int64_t j0 = (int64_t)blockIdx.x * HEAT_TC - HEAT_K;  // global column of local column 0
  for (int r = warp; r < HEAT_SR; r += HEAT_BLOCK_THREADS / 32) {
    const int64_t i = i0 + r;
    const bool row_in = i >= 0 && i < n;
#pragma unroll
    for (int q = 0; q < HEAT_SC / 32; q++) {
      const int64_t j = j0 + lane + 32 * q;
      buf0[r * HEAT_SC + lane + 32 * q] = (row_in && j >= 0 && j < m) ? __ldg(u + i * m + j) : (T)0;
    }
  }
  // lane l owns local columns 4l .. 4l + 3 (a warp covers a whole shared row);
  // which of them are interior columns of the grid
  bool col_int[4];
#pragma unroll
  for (int e = 0; e < 4; e++) {
    const int64_t j = j0 + 4 * lane + e;
    col_int[e] = j > 0 && j < m - 1;
  }
  __syncthreads();
  T* src = buf0;
  T* dst = buf1;
  // each warp walks a band of consecutive rows, keeping the row above and its
  // current row in registers: one shared-memory row load per row and step
  // instead of three
  constexpr int NWARP = HEAT_BLOCK_THREADS / 32;
  constexpr int BAND = (HEAT_SR - 2 + NWARP - 1) / NWARP;
  const int rb = 1 + warp * BAND;
  const int re = min(rb + BAND, HEAT_SR - 1);
  for (int s = 0; s < ksteps; s++) {
    // rows 1 .. HEAT_SR - 2 (the outer rows have no neighbours); the outer
    // columns are computed from the neighbouring rows' ends and never read back
    // as exact values
    if (rb < re) {
      T up[4], cv[4];
      heat_ld4(src + (rb - 1) * HEAT_SC + 4 * lane, up);
      heat_ld4(src + rb * HEAT_SC + 4 * lane, cv);
      for (int r = rb; r < re; r++) {
        const int64_t i = i0 + r;
        const bool row_int = i > 0 && i < n - 1;
        const int b = r * HEAT_SC + 4 * lane;
        T dn[4], res[4];
        heat_ld4(src + b + HEAT_SC, dn);
        // the neighbouring lanes' end cells; lanes 0 and 31 hold the tile's outer
        // columns, whose results are never exact, so their wrapped values do not matter
        const T lft = __shfl_up_sync(0xffffffffu, cv[3], 1);
        const T rgt = __shfl_down_sync(0xffffffffu, cv[0], 1);
#pragma unroll
        for (int e = 0; e < 4; e++) {
          const T left = e == 0 ? lft : cv[e - 1];
          const T right = e == 3 ? rgt : cv[e + 1];
          res[e] = cv[e];
          if (row_int && col_int[e]) {
            T lap = up[e] + dn[e];
            lap = lap + left;
            lap = lap + right;
            const T c4 = cv[e] * (T)4;
            lap = lap - c4;
            const T d = lap * coef;
            res[e] = cv[e] + d;
          }
        }
        heat_st4(dst + b, res);
#pragma unroll
        for (int e = 0; e < 4; e++) {
          up[e] = cv[e];
          cv[e] = dn[e];
        }
      }
    }
    __syncthreads();
    T* t = src;
    src = dst;
    dst = t;
  }
  for (int r = warp; r < HEAT_TR; r += HEAT_BLOCK_THREADS / 32) {
    const int64_t i = i0 + HEAT_K + r;
    if (i >= n) break;
#pragma unroll
    for (int q = 0; q < HEAT_SC / 32; q++) {
      const int c = lane + 32 * q;
      const int64_t j = j0 + HEAT_K + c;
      if (c < HEAT_TC && j < m) out[i * m + j] = src[(r + HEAT_K) * HEAT_SC + c + HEAT_K];
    }
  }
}

template <typename T>
static void enqueue_heat(const T* u, T* out, int64_t n, int64_t m, T coef, cudaStream_t s) {
  dim3 grid((unsigned)((m + HEAT_COLS - 1) / HEAT_COLS), (unsigned)((n + HEAT_ROWS - 1) / HEAT_ROWS));
  heat_step_kernel<T><<<grid, HEAT_COLS, 0, s>>>(u, out, n, m, coef);
}

template <typename T>
static void enqueue_heat_block(const T* u, T* out, int64_t n, int64_t m, T coef, int ksteps, cudaStream_t s) {
  const size_t smem = 2 * (size_t)HEAT_SR * HEAT_SC * sizeof(T);
  // per launch: the attribute belongs to the current device's context
  cudaFuncSetAttribute(heat_block_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  dim3 grid((unsigned)((m + HEAT_TC - 1) / HEAT_TC), (unsigned)((n + HEAT_TR - 1) / HEAT_TR));
  heat_block_kernel<T><<<grid, HEAT_BLOCK_THREADS, smem, s>>>(u, out, n, m, coef, ksteps);
}

// Enqueues `steps` steps from u: ceil(steps / HEAT_K) blocked launches ping-pong
// between u and tmp; returns whether the result ended in tmp.
template <typename T>
static bool enqueue_heat_steps(T* u, T* tmp, int64_t n, int64_t m, T coef, int32_t steps, cudaStream_t s,
                               int* launches) {
  bool in_tmp = false;
  *launches = 0;
  for (int done = 0; done < steps; done += HEAT_K) {
    const int k = steps - done < HEAT_K ? steps - done : HEAT_K;
    enqueue_heat_block<T>(in_tmp ? tmp : u, in_tmp ? u : tmp, n, m, coef, k, s);
    in_tmp = !in_tmp;
    (*launches)++;
  }
  return in_tmp;
}

// Arguments of a heat call: two distinct, non-overlapping n x m grids of
// `elem`-byte values.
static int32_t check_heat(const void* u, const void* o, int64_t n, int64_t m, size_t elem) {
  if (!u || !o) return fail(PHCU_ERR_INVALID, "heat: null buffer");
  if (n < 1 || m < 1) return fail(PHCU_ERR_SHAPE, "heat: grid %lld x %lld", (long long)n, (long long)m);
  if ((n + HEAT_ROWS - 1) / HEAT_ROWS > 65535) return fail(PHCU_ERR_UNSUPPORTED, "heat: too many rows");
  if (n > (INT64_MAX / (int64_t)elem) / m) return fail(PHCU_ERR_UNSUPPORTED, "heat: grid too large");
  const uintptr_t bytes = (uintptr_t)(n * m) * elem, a = (uintptr_t)u, b = (uintptr_t)o;
  if (a < b + bytes && b < a + bytes) return fail(PHCU_ERR_INVALID, "heat: input and output grids overlap");
  return require_ctx();
}

// instantiated graphs of whole runs, keyed by their parameters
using HeatKey = std::tuple<const void*, const void*, int64_t, int64_t, double, int, cudaStream_t, int>;
static std::map<HeatKey, cudaGraphExec_t> g_heat_graphs;

// Destroys the cached graphs (the context that instantiated them is going away).
void release_heat_graphs() {
  for (auto& kv : g_heat_graphs) cudaGraphExecDestroy(kv.second);
  g_heat_graphs.clear();
}

template <typename T>
static int32_t heat_run(T* u, T* tmp, int64_t n, int64_t m, T coef, int32_t steps, int32_t use_graph) {
  PHCU_TRY(check_heat(u, tmp, n, m, sizeof(T)));
  if (steps < 0) return fail(PHCU_ERR_INVALID, "heat: negative step count");
  if (steps == 0) return PHCU_OK;
  cudaStream_t s = stream();
  const size_t bytes = (size_t)(n * m) * sizeof(T);
  int launches = 0;
  if (!use_graph) {
    const bool in_tmp = enqueue_heat_steps<T>(u, tmp, n, m, coef, steps, s, &launches);
    count_launch((unsigned)launches);
    PHCU_TRY(check_launch("heat_block_kernel"));
    if (in_tmp) PHCU_CUDA(cudaMemcpyAsync(u, tmp, bytes, cudaMemcpyDeviceToDevice, s));
    return PHCU_OK;
  }
  HeatKey key(u, tmp, n, m, (double)coef, steps, s, (int)sizeof(T));
  auto it = g_heat_graphs.find(key);
  cudaGraphExec_t ge;
  launches = (steps + HEAT_K - 1) / HEAT_K;
  if (it == g_heat_graphs.end()) {
    PHCU_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    const bool in_tmp = enqueue_heat_steps<T>(u, tmp, n, m, coef, steps, s, &launches);
    if (in_tmp) cudaMemcpyAsync(u, tmp, bytes, cudaMemcpyDeviceToDevice, s);
    cudaGraph_t g;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture(heat)");
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate(heat)");
    g_heat_graphs[key] = ge;
  } else {
    ge = it->second;
  }
  PHCU_CUDA(cudaGraphLaunch(ge, s));
  count_launch((unsigned)launches);
  return PHCU_OK;
}

}  // namespace phcu

using namespace phcu;

extern "C" {

int32_t phcu_heat_step(const float* u, float* out, int64_t n, int64_t m, float coef) {
  PHCU_TRY(check_heat(u, out, n, m, sizeof(float)));
  enqueue_heat<float>(u, out, n, m, coef, stream());
  count_launch();
  return check_launch("heat_step_kernel");
}

int32_t phcu_heat_run(float* u, float* tmp, int64_t n, int64_t m, float coef, int32_t steps, int32_t use_graph) {
  return heat_run<float>(u, tmp, n, m, coef, steps, use_graph);
}

int32_t phcu_heat_run_f64(double* u, double* tmp, int64_t n, int64_t m, double coef, int32_t steps,
                          int32_t use_graph) {
  return heat_run<double>(u, tmp, n, m, coef, steps, use_graph);
}

}  // extern "C"
