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

template <typename T>
static void enqueue_heat(const T* u, T* out, int64_t n, int64_t m, T coef, cudaStream_t s) {
  dim3 grid((unsigned)((m + HEAT_COLS - 1) / HEAT_COLS), (unsigned)((n + HEAT_ROWS - 1) / HEAT_ROWS));
  heat_step_kernel<T><<<grid, HEAT_COLS, 0, s>>>(u, out, n, m, coef);
}

static int32_t check_heat(const void* u, const void* o, int64_t n, int64_t m) {
  PHCU_TRY(require_ctx());
  if (!u || !o) return fail(PHCU_ERR_INVALID, "heat: null buffer");
  if (u == o) return fail(PHCU_ERR_INVALID, "heat: input and output must differ");
  if (n < 1 || m < 1) return fail(PHCU_ERR_SHAPE, "heat: grid %lld x %lld", (long long)n, (long long)m);
  if ((n + HEAT_ROWS - 1) / HEAT_ROWS > 65535) return fail(PHCU_ERR_UNSUPPORTED, "heat: too many rows");
  return PHCU_OK;
}

// instantiated graphs of whole runs, keyed by their parameters
using HeatKey = std::tuple<const void*, const void*, int64_t, int64_t, double, int, cudaStream_t, int>;
static std::map<HeatKey, cudaGraphExec_t> g_heat_graphs;

template <typename T>
static int32_t heat_run(T* u, T* tmp, int64_t n, int64_t m, T coef, int32_t steps, int32_t use_graph) {
  PHCU_TRY(check_heat(u, tmp, n, m));
  if (steps < 0) return fail(PHCU_ERR_INVALID, "heat: negative step count");
  if (steps == 0) return PHCU_OK;
  cudaStream_t s = stream();
  const size_t bytes = (size_t)(n * m) * sizeof(T);
  if (!use_graph) {
    for (int k = 0; k < steps; k++) {
      enqueue_heat<T>((k & 1) ? tmp : u, (k & 1) ? u : tmp, n, m, coef, s);
      count_launch();
      PHCU_TRY(check_launch("heat_step_kernel"));
    }
    if (steps & 1) PHCU_CUDA(cudaMemcpyAsync(u, tmp, bytes, cudaMemcpyDeviceToDevice, s));
    return PHCU_OK;
  }
  HeatKey key(u, tmp, n, m, (double)coef, steps, s, (int)sizeof(T));
  auto it = g_heat_graphs.find(key);
  cudaGraphExec_t ge;
  if (it == g_heat_graphs.end()) {
    PHCU_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < steps; k++) enqueue_heat<T>((k & 1) ? tmp : u, (k & 1) ? u : tmp, n, m, coef, s);
    if (steps & 1) cudaMemcpyAsync(u, tmp, bytes, cudaMemcpyDeviceToDevice, s);
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
  count_launch((unsigned)steps);
  return PHCU_OK;
}

}  // namespace phcu

using namespace phcu;

extern "C" {

int32_t phcu_heat_step(const float* u, float* out, int64_t n, int64_t m, float coef) {
  PHCU_TRY(check_heat(u, out, n, m));
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
