// stencil.cu -- explicit 2-D heat step and its CUDA-graph driver.
//
// The Phase program of one step (examples/heat_equation.cr:38-51 generalised to
// 2-D shifted views):
//   c   = u[1..-2, 1..-2]
//   lap = u[0..-3, 1..-2] + u[2.., 1..-2] + u[1..-2, 0..-3] + u[1..-2, 2..] - c * 4
//   u[1..-2, 1..-2] = c + lap * coef
// is fused into one pass: every interior point evaluates the infix chain left to
// right in Float32 (no FMA: this file is compiled with -fmad=false), the boundary
// is copied.  Each thread walks a column strip, keeping up/centre/down in
// registers; left/right come from the neighbouring lanes by warp shuffle, so
// each element is read from memory about once per step.
#include <map>
#include <tuple>

#include "common.cuh"

namespace phcu {

constexpr int HEAT_COLS = 128;
constexpr int HEAT_ROWS = 16;

__global__ void __launch_bounds__(HEAT_COLS) heat_step_kernel(const float* __restrict__ u, float* __restrict__ out,
                                                              int64_t n, int64_t m, float coef) {
  const int64_t j = (int64_t)blockIdx.x * HEAT_COLS + threadIdx.x;
  const int64_t i0 = (int64_t)blockIdx.y * HEAT_ROWS;
  const int lane = threadIdx.x & 31;
  const bool jin = j < m;
  const int64_t jc = jin ? j : m - 1;  // lanes past the edge still take part in the shuffles
  float up = (i0 > 0) ? __ldg(u + (i0 - 1) * m + jc) : 0.0f;
  float c = __ldg(u + i0 * m + jc);
#pragma unroll 4
  for (int r = 0; r < HEAT_ROWS; r++) {
    const int64_t i = i0 + r;
    if (i >= n) break;  // uniform across the block
    const float down = (i + 1 < n) ? __ldg(u + (i + 1) * m + jc) : 0.0f;
    float left = __shfl_up_sync(0xffffffffu, c, 1);
    float right = __shfl_down_sync(0xffffffffu, c, 1);
    if (lane == 0) left = (jc > 0) ? __ldg(u + i * m + jc - 1) : 0.0f;
    if (lane == 31) right = (jc + 1 < m) ? __ldg(u + i * m + jc + 1) : 0.0f;
    if (jin) {
      float res;
      if (i == 0 || i == n - 1 || j == 0 || j == m - 1) {
        res = c;
      } else {
        float lap = up + down;
        lap = lap + left;
        lap = lap + right;
        const float c4 = c * 4.0f;
        lap = lap - c4;
        const float d = lap * coef;
        res = c + d;
      }
      out[i * m + j] = res;
    }
    up = c;
    c = down;
  }
}

static int32_t launch_heat(const float* u, float* out, int64_t n, int64_t m, float coef) {
  dim3 grid((unsigned)((m + HEAT_COLS - 1) / HEAT_COLS), (unsigned)((n + HEAT_ROWS - 1) / HEAT_ROWS));
  heat_step_kernel<<<grid, HEAT_COLS, 0, stream()>>>(u, out, n, m, coef);
  count_launch();
  return check_launch("heat_step_kernel");
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
using HeatKey = std::tuple<const void*, const void*, int64_t, int64_t, float, int, cudaStream_t>;
static std::map<HeatKey, cudaGraphExec_t> g_heat_graphs;

}  // namespace phcu

using namespace phcu;

extern "C" {

int32_t phcu_heat_step(const float* u, float* out, int64_t n, int64_t m, float coef) {
  PHCU_TRY(check_heat(u, out, n, m));
  return launch_heat(u, out, n, m, coef);
}

int32_t phcu_heat_run(float* u, float* tmp, int64_t n, int64_t m, float coef, int32_t steps, int32_t use_graph) {
  PHCU_TRY(check_heat(u, tmp, n, m));
  if (steps < 0) return fail(PHCU_ERR_INVALID, "heat: negative step count");
  if (steps == 0) return PHCU_OK;
  cudaStream_t s = stream();
  if (!use_graph) {
    for (int k = 0; k < steps; k++) {
      const float* src = (k & 1) ? tmp : u;
      float* dst = (k & 1) ? u : tmp;
      PHCU_TRY(launch_heat(src, dst, n, m, coef));
    }
    if (steps & 1) PHCU_CUDA(cudaMemcpyAsync(u, tmp, (size_t)(n * m) * sizeof(float), cudaMemcpyDeviceToDevice, s));
    return PHCU_OK;
  }
  HeatKey key(u, tmp, n, m, coef, steps, s);
  auto it = g_heat_graphs.find(key);
  cudaGraphExec_t ge;
  if (it == g_heat_graphs.end()) {
    PHCU_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    int32_t rc = PHCU_OK;
    unsigned long long before = ctx().launches;
    for (int k = 0; k < steps && rc == PHCU_OK; k++) {
      const float* src = (k & 1) ? tmp : u;
      float* dst = (k & 1) ? u : tmp;
      dim3 grid((unsigned)((m + HEAT_COLS - 1) / HEAT_COLS), (unsigned)((n + HEAT_ROWS - 1) / HEAT_ROWS));
      heat_step_kernel<<<grid, HEAT_COLS, 0, s>>>(src, dst, n, m, coef);
    }
    if (steps & 1) cudaMemcpyAsync(u, tmp, (size_t)(n * m) * sizeof(float), cudaMemcpyDeviceToDevice, s);
    cudaGraph_t g;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    ctx().launches = before;
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

}  // extern "C"
