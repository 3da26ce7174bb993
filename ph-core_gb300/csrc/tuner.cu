// tuner.cu -- launch-configuration autotuner and the learned (MLP) tuner.
//
// A configuration of a task is (work-item size, layout): the number of
// elements one block takes from the work queue per item (2^12, 2^13, 2^14 or
// 2^15) and, for elementwise programs, whether the planner's launch shape or
// ROW is used (a reduction keeps the planner's layout under both).
// phcu_tune_measure times a task under every configuration (exhaustive
// autotune) as its share of a batch of copies that fills the GPU; the MLP (24 -> 64 -> 64 -> 1, ReLU, predicts log2 of the time)
// is trained on those timings by the kernels below and then ranks the
// configurations of unseen tasks without timing them.
//
// MLP kernels: one block of 64 threads (one per hidden unit) processes a slice
// of the minibatch with the whole parameter vector in shared memory; forward
// and backward are written out by hand; per-block gradients go to global
// memory with one atomicAdd per parameter per block; Adam runs as a separate
// elementwise kernel.  Explicit fmaf is used for the dot products (this file
// is compiled with -fmad=false, which only stops implicit contraction).
#include <math.h>

#include <algorithm>
#include <vector>

#include "plan.h"

namespace phcu {

constexpr int NCONF = 8;
static const int32_t kChunk[4] = {1 << 12, 1 << 13, 1 << 14, 1 << 15};

static void apply_config(phcu_task_t* t, int c) {
  t->chunk = kChunk[c % 4];
  t->layout = c / 4;
}

// ------------------------------------------------------------ features
static float lg2(double x) { return (float)log2(std::max(1.0, x)); }

static int32_t task_features(const phcu_task_t* t, int config, float* f) {
  for (int i = 0; i < PHCU_TUNE_FEATURES; i++) f[i] = 0.f;
  const phcu_view_t& v = t->in[0];
  const phcu_view_t& src = (t->kind == PHCU_TASK_EVAL && t->n_inputs == 0) ? t->out : v;
  int64_t n = view_size(&src);
  f[0] = (float)src.rank;
  f[1] = lg2((double)n);
  for (int i = 0; i < 4 && i < src.rank; i++) f[2 + i] = lg2((double)src.shape[i] + 1);
  // |stride| of each axis relative to a row-major layout of the view shape
  int64_t rm = 1;
  for (int i = src.rank - 1, j = 0; i >= 0 && j < 4; i--, j++) {
    int64_t s = src.stride[i] < 0 ? -src.stride[i] : src.stride[i];
    f[6 + (src.rank - 1 - i)] = (float)std::min<double>(8.0, rm > 0 ? (double)s / (double)rm : 0.0);
    rm *= std::max<int64_t>(1, src.shape[i]);
  }
  int64_t inner = src.rank ? (src.stride[src.rank - 1] < 0 ? -src.stride[src.rank - 1] : src.stride[src.rank - 1]) : 1;
  f[10] = lg2((double)inner + 1);
  // inversions of the axis order by stride (a permutation measure)
  int inv = 0;
  for (int i = 0; i < src.rank; i++)
    for (int j = i + 1; j < src.rank; j++) {
      int64_t a = src.stride[i] < 0 ? -src.stride[i] : src.stride[i];
      int64_t b = src.stride[j] < 0 ? -src.stride[j] : src.stride[j];
      if (a < b) inv++;
    }
  f[11] = (float)inv;
  f[12] = (src.dtype == PHCU_F32 || src.dtype == PHCU_F64) ? 0.f : 1.f;
  if (t->kind == PHCU_TASK_EVAL) {
    int k = t->n_inputs >= 2 ? (t->prog % 3) : 0;  // +, *, chain by program slot
    f[13 + k] = 1.f;
  } else {
    f[16 + (t->red_op == PHCU_RED_SUM ? 0 : 1)] = 1.f;
  }
  f[18] = lg2((double)view_size(&t->out));
  f[19] = (inner == 1) ? 1.f : 0.f;
  int64_t oin = t->out.rank ? t->out.stride[t->out.rank - 1] : 1;
  f[20] = (oin == 1 || oin == -1) ? 1.f : 0.f;
  f[21] = (float)(config / 4);
  f[22] = lg2((double)kChunk[config % 4]);
  f[23] = lg2((double)n) - lg2((double)kChunk[config % 4]);  // log2 of work items
  return PHCU_OK;
}

// ---------------------------------------------------------------- MLP
constexpr int IN = PHCU_TUNE_FEATURES;
constexpr int H1 = PHCU_MLP_H1;
constexpr int H2 = PHCU_MLP_H2;
constexpr int NP = PHCU_MLP_PARAMS;
constexpr int OFF_W1 = 0, OFF_B1 = H1 * IN, OFF_W2 = OFF_B1 + H1, OFF_B2 = OFF_W2 + H2 * H1, OFF_W3 = OFF_B2 + H2,
              OFF_B3 = OFF_W3 + H2;
static_assert(H1 == 64 && H2 == 64, "one thread per hidden unit");

__device__ __forceinline__ uint32_t hash32(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return (uint32_t)x;
}

// He-uniform weights, zero biases.
__global__ void mlp_init_kernel(float* p, uint64_t seed) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NP; i += gridDim.x * blockDim.x) {
    float u = (hash32(seed * 0x9E3779B97F4A7C15ull + (uint64_t)i) >> 8) * (1.0f / 16777216.0f) * 2.f - 1.f;
    float v = 0.f;
    if (i < OFF_B1) v = u * sqrtf(6.f / IN);
    else if (i >= OFF_W2 && i < OFF_B2) v = u * sqrtf(6.f / H1);
    else if (i >= OFF_W3 && i < OFF_B3) v = u * sqrtf(6.f / H2);
    p[i] = v;
  }
}

constexpr int MLP_SAMPLES_PER_BLOCK = 32;

// Forward (and, with grad != null, backward) of samples [blockIdx*32, +32).
__global__ void __launch_bounds__(64) mlp_fwd_bwd_kernel(const float* __restrict__ params, const float* __restrict__ x,
                                                         const float* __restrict__ y, int batch, float* yhat,
                                                         float* grad, float* loss) {
  __shared__ float P[NP];
  __shared__ float xs[IN];
  __shared__ float a1[H1], a2[H2], d2[H2], red[64];
  const int j = threadIdx.x;
  for (int i = j; i < NP; i += 64) P[i] = params[i];
  // per-thread gradient accumulators for the parameters this thread owns
  float gW1[IN], gb1 = 0.f, gW2[H1], gb2 = 0.f, gW3 = 0.f, gb3 = 0.f, L = 0.f;
#pragma unroll
  for (int k = 0; k < IN; k++) gW1[k] = 0.f;
#pragma unroll
  for (int k = 0; k < H1; k++) gW2[k] = 0.f;
  __syncthreads();
  const int s0 = blockIdx.x * MLP_SAMPLES_PER_BLOCK;
  const int s1 = min(batch, s0 + MLP_SAMPLES_PER_BLOCK);
  for (int s = s0; s < s1; s++) {
    if (j < IN) xs[j] = x[(size_t)s * IN + j];
    __syncthreads();
    float z = P[OFF_B1 + j];
#pragma unroll
    for (int k = 0; k < IN; k++) z = fmaf(P[OFF_W1 + j * IN + k], xs[k], z);
    a1[j] = z > 0.f ? z : 0.f;
    __syncthreads();
    z = P[OFF_B2 + j];
#pragma unroll 16
    for (int k = 0; k < H1; k++) z = fmaf(P[OFF_W2 + j * H1 + k], a1[k], z);
    a2[j] = z > 0.f ? z : 0.f;
    red[j] = P[OFF_W3 + j] * a2[j];
    __syncthreads();
    for (int w = 32; w >= 1; w >>= 1) {
      if (j < w) red[j] += red[j + w];
      __syncthreads();
    }
    const float out = red[0] + P[OFF_B3];
    if (j == 0 && yhat) yhat[s] = out;
    if (grad) {
      const float e = out - y[s];
      const float dy = 2.f * e / (float)batch;
      if (j == 0) {
        L += e * e;
        gb3 += dy;
      }
      gW3 = fmaf(dy, a2[j], gW3);
      d2[j] = a2[j] > 0.f ? dy * P[OFF_W3 + j] : 0.f;
      __syncthreads();
      gb2 += d2[j];
#pragma unroll 16
      for (int k = 0; k < H1; k++) gW2[k] = fmaf(d2[j], a1[k], gW2[k]);
      // d1[j] = sum_i d2[i] * W2[i][j]
      float acc = 0.f;
#pragma unroll 16
      for (int i = 0; i < H2; i++) acc = fmaf(d2[i], P[OFF_W2 + i * H1 + j], acc);
      const float d1 = a1[j] > 0.f ? acc : 0.f;
      gb1 += d1;
#pragma unroll
      for (int k = 0; k < IN; k++) gW1[k] = fmaf(d1, xs[k], gW1[k]);
    }
    __syncthreads();
  }
  if (grad) {
#pragma unroll
    for (int k = 0; k < IN; k++) atomicAdd(&grad[OFF_W1 + j * IN + k], gW1[k]);
    atomicAdd(&grad[OFF_B1 + j], gb1);
#pragma unroll 16
    for (int k = 0; k < H1; k++) atomicAdd(&grad[OFF_W2 + j * H1 + k], gW2[k]);
    atomicAdd(&grad[OFF_B2 + j], gb2);
    atomicAdd(&grad[OFF_W3 + j], gW3);
    if (j == 0) {
      atomicAdd(&grad[OFF_B3], gb3);
      atomicAdd(loss, L);
    }
  }
}

__global__ void adam_kernel(float* p, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NP; i += gridDim.x * blockDim.x) {
    float gi = g[i];
    float mi = b1 * m[i] + (1.f - b1) * gi;
    float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

static int32_t mlp_pass(const float* params, const float* x, const float* y, int batch, float* yhat, float* grad,
                        float* loss_dev) {
  int blocks = (batch + MLP_SAMPLES_PER_BLOCK - 1) / MLP_SAMPLES_PER_BLOCK;
  if (blocks < 1) return PHCU_OK;
  mlp_fwd_bwd_kernel<<<blocks, 64, 0, stream()>>>(params, x, y, batch, yhat, grad, loss_dev);
  count_launch();
  return check_launch("mlp_fwd_bwd_kernel");
}

}  // namespace phcu

using namespace phcu;

extern "C" {

int32_t phcu_tune_n_configs(int32_t* n) {
  *n = NCONF;
  return PHCU_OK;
}

int32_t phcu_tune_features(const phcu_task_t* task, int32_t config, float* features) {
  if (!task || !features || config < 0 || config >= NCONF) return fail(PHCU_ERR_INVALID, "tune_features: bad args");
  return task_features(task, config, features);
}

int32_t phcu_task_run_config(const phcu_task_t* task, const phcu_program_t* programs, int32_t config) {
  PHCU_TRY(require_ctx());
  if (!task || config < 0 || config >= NCONF) return fail(PHCU_ERR_INVALID, "task_run_config: bad args");
  phcu_task_t t = *task;
  apply_config(&t, config);
  int nprog = 0;
  if (t.kind == PHCU_TASK_EVAL) nprog = t.prog + 1;
  return phcu_batch_run(&t, 1, programs, nprog, 0);
}

int32_t phcu_tune_measure(const phcu_task_t* task, const phcu_program_t* programs, int32_t reps, float* ms) {
  PHCU_TRY(require_ctx());
  if (!task || !ms || reps < 1) return fail(PHCU_ERR_INVALID, "tune_measure: bad args");
  const int nprog = task->kind == PHCU_TASK_EVAL ? task->prog + 1 : 0;
  cudaStream_t s = stream();
  cudaEvent_t e0, e1;
  PHCU_CUDA(cudaEventCreate(&e0));
  const cudaError_t ce = cudaEventCreate(&e1);
  if (ce != cudaSuccess) {
    cudaEventDestroy(e0);
    return cuda_fail(ce, "cudaEventCreate(tune_measure)");
  }
  // The task is timed as a batch of R copies that together fill the GPU, and
  // the time is divided by R: a task's cost inside a large batch (its work
  // items interleave with everyone else's) is its share of the throughput,
  // not the latency of a launch that it has to itself.
  // Each copy writes its own contiguous output (scratch of the output's
  // shape), as the tasks of a real batch do: copies sharing one output would
  // turn every store into an L2 hit.
  const phcu_view_t& src = (task->kind == PHCU_TASK_EVAL && task->n_inputs == 0) ? task->out : task->in[0];
  const int64_t n = std::max<int64_t>(1, view_size(&src));
  // 2^25 elements in all: even at the largest work items a batch of big
  // copies has a few items for every block, as the tasks of a real batch do
  const int R = (int)std::min<int64_t>(512, std::max<int64_t>(1, ((int64_t)1 << 25) / n));
  const int64_t out_n = std::max<int64_t>(1, view_size(&task->out));
  const size_t out_bytes = ((size_t)out_n * dtype_size(task->out.dtype) + 255) & ~(size_t)255;
  void* outs = nullptr;
  int32_t rc = scratch_alloc(out_bytes * R, &outs);
  for (int c = 0; c < NCONF && rc == PHCU_OK; c++) {
    phcu_task_t t = *task;
    apply_config(&t, c);
    std::vector<phcu_task_t> copies((size_t)R, t);
    for (int k = 0; k < R; k++) {
      phcu_view_t& o = copies[(size_t)k].out;
      o.base = (char*)outs + (size_t)k * out_bytes;
      o.offset = 0;
      int64_t st = 1;
      for (int i = o.rank - 1; i >= 0; i--) {
        o.stride[i] = st;
        st *= o.shape[i];
      }
    }
    void* b = nullptr;
    rc = phcu_batch_prepare(copies.data(), R, programs, nprog, &b);
    if (rc != PHCU_OK) break;
    rc = phcu_batch_launch(b, 0);  // warm-up
    std::vector<float> v;
    for (int r = 0; r < reps && rc == PHCU_OK; r++) {
      cudaEventRecord(e0, s);
      rc = phcu_batch_launch(b, 0);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float t_ms = 0.f;
      cudaEventElapsedTime(&t_ms, e0, e1);
      v.push_back(t_ms);
    }
    phcu_batch_destroy(b);
    if (rc == PHCU_OK) {
      std::sort(v.begin(), v.end());
      ms[c] = v[v.size() / 2] / (float)R;
    }
  }
  scratch_free(outs);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

int32_t phcu_mlp_init(float* params_dev, uint64_t seed) {
  PHCU_TRY(require_ctx());
  if (!params_dev) return fail(PHCU_ERR_INVALID, "mlp_init: null params");
  mlp_init_kernel<<<(NP + 255) / 256, 256, 0, stream()>>>(params_dev, seed);
  count_launch();
  return check_launch("mlp_init_kernel");
}

int32_t phcu_mlp_forward(const float* params_dev, const float* x_dev, int32_t batch, float* y_dev) {
  PHCU_TRY(require_ctx());
  if (!params_dev || !x_dev || !y_dev || batch < 0) return fail(PHCU_ERR_INVALID, "mlp_forward: bad args");
  return mlp_pass(params_dev, x_dev, nullptr, batch, y_dev, nullptr, nullptr);
}

int32_t phcu_mlp_grad(const float* params_dev, const float* x_dev, const float* y_dev, int32_t batch, float* grad_dev,
                      float* loss) {
  PHCU_TRY(require_ctx());
  if (!params_dev || !x_dev || !y_dev || !grad_dev || batch < 1) return fail(PHCU_ERR_INVALID, "mlp_grad: bad args");
  float* dloss = nullptr;
  PHCU_TRY(scratch_alloc(sizeof(float), (void**)&dloss));
  PHCU_CUDA(cudaMemsetAsync(grad_dev, 0, NP * sizeof(float), stream()));
  PHCU_CUDA(cudaMemsetAsync(dloss, 0, sizeof(float), stream()));
  int32_t rc = mlp_pass(params_dev, x_dev, y_dev, batch, nullptr, grad_dev, dloss);
  float h = 0.f;
  if (rc == PHCU_OK) {
    cudaMemcpyAsync(&h, dloss, sizeof(float), cudaMemcpyDeviceToHost, stream());
    cudaStreamSynchronize(stream());
  }
  scratch_free(dloss);
  if (loss) *loss = h / (float)batch;
  return rc;
}

int32_t phcu_mlp_train(float* params_dev, const float* x_dev, const float* y_dev, int32_t n, int32_t epochs,
                       int32_t batch, float lr, uint64_t seed, float* final_loss) {
  PHCU_TRY(require_ctx());
  if (!params_dev || !x_dev || !y_dev || n < 1 || epochs < 0 || batch < 1)
    return fail(PHCU_ERR_INVALID, "mlp_train: bad args");
  (void)seed;
  cudaStream_t s = stream();
  float *g = nullptr, *m = nullptr, *v = nullptr, *dloss = nullptr;
  PHCU_TRY(scratch_alloc(NP * sizeof(float) * 3 + 16, (void**)&g));
  m = g + NP;
  v = m + NP;
  dloss = v + NP;
  PHCU_CUDA(cudaMemsetAsync(m, 0, 2 * NP * sizeof(float), s));
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  double c1 = 1.0, c2 = 1.0;
  int32_t rc = PHCU_OK;
  // the caller shuffles the samples once; minibatches walk them in order
  for (int ep = 0; ep < epochs && rc == PHCU_OK; ep++) {
    for (int s0 = 0; s0 < n && rc == PHCU_OK; s0 += batch) {
      const int bs = std::min(batch, n - s0);
      cudaMemsetAsync(g, 0, NP * sizeof(float), s);
      rc = mlp_pass(params_dev, x_dev + (size_t)s0 * IN, y_dev + s0, bs, nullptr, g, dloss);
      c1 *= b1;
      c2 *= b2;
      adam_kernel<<<(NP + 255) / 256, 256, 0, s>>>(params_dev, g, m, v, lr, b1, b2, eps, (float)(1.0 - c1),
                                                   (float)(1.0 - c2));
      count_launch();
      if (rc == PHCU_OK) rc = check_launch("adam_kernel");
    }
  }
  if (rc == PHCU_OK && final_loss) {
    // loss over the whole set with the trained parameters
    cudaMemsetAsync(g, 0, NP * sizeof(float), s);
    cudaMemsetAsync(dloss, 0, sizeof(float), s);
    rc = mlp_pass(params_dev, x_dev, y_dev, n, nullptr, g, dloss);
    float h = 0.f;
    cudaMemcpyAsync(&h, dloss, sizeof(float), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    *final_loss = h / (float)n;
  }
  scratch_free(g);
  return rc;
}

}  // extern "C"
