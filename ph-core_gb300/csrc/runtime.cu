// runtime.cu -- context, memory, status word, timers, graphs and errors.
#include <stdarg.h>
#include <stdio.h>

#include "common.cuh"

namespace phcu {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int32_t fail(int32_t code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int32_t cuda_fail(cudaError_t e, const char* what) {
  snprintf(g_err, sizeof(g_err), "CUDA error %d (%s) in %s", (int)e, cudaGetErrorString(e), what);
  if (e == cudaErrorMemoryAllocation) return PHCU_ERR_OOM;
  return PHCU_ERR_CUDA;
}

static Context g_ctx;
Context& ctx() { return g_ctx; }

int32_t require_ctx() {
  if (!g_ctx.ready) return fail(PHCU_ERR_NOT_INIT, "phcu_init has not been called");
  return PHCU_OK;
}

int32_t check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, what);
  return PHCU_OK;
}

int32_t scratch_alloc(size_t bytes, void** p) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMallocAsync(p, bytes, g_ctx.stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync(scratch)");
  return PHCU_OK;
}

void scratch_free(void* p) {
  if (p) cudaFreeAsync(p, g_ctx.stream);
}

struct Timer {
  cudaEvent_t a, b;
};

// Launch-shape cache of blocks_per_sm (one host thread per context).
struct OccEntry {
  const void* fn;
  int threads;
  size_t smem;
  int per_sm;
};
struct SmemLimit {
  const void* fn;
  size_t smem;
};
static OccEntry g_occ[256];
static int g_nocc = 0;
static SmemLimit g_lim[128];
static int g_nlim = 0;

int blocks_per_sm(const void* fn, int threads, size_t smem) {
  if (smem > 48 * 1024) {
    int i = 0;
    while (i < g_nlim && g_lim[i].fn != fn) i++;
    if (i == g_nlim || g_lim[i].smem < smem) {
      cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (i < g_nlim) g_lim[i].smem = smem;
      else if (g_nlim < 128) g_lim[g_nlim++] = {fn, smem};
    }
  }
  for (int i = 0; i < g_nocc; i++)
    if (g_occ[i].fn == fn && g_occ[i].threads == threads && g_occ[i].smem == smem) return g_occ[i].per_sm;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
  if (per_sm < 1) per_sm = 1;
  if (g_nocc < 256) g_occ[g_nocc++] = {fn, threads, smem, per_sm};
  return per_sm;
}

// Frees what a context holds (any subset of it, after a failed init) and
// resets it.
static void release_context(Context& c) {
  if (c.stream && c.stream != c.own_stream) cudaStreamSynchronize(c.stream);  // a caller's stream
  if (c.own_stream) cudaStreamSynchronize(c.own_stream);
  if (c.d2h) cudaStreamSynchronize(c.d2h);
  if (c.h2d) cudaStreamSynchronize(c.h2d);
  for (int i = 0; i < Context::NSIDE; i++)
    if (c.side[i]) cudaStreamSynchronize(c.side[i]);
  release_heat_graphs();
  release_noalloc_scratch();
  if (c.l2_scrub) cudaFree(c.l2_scrub);
  if (c.status) cudaFree(c.status);
  if (c.ev_work) cudaEventDestroy(c.ev_work);
  if (c.ev_h2d) cudaEventDestroy(c.ev_h2d);
  if (c.d2h) cudaStreamDestroy(c.d2h);
  if (c.h2d) cudaStreamDestroy(c.h2d);
  for (int i = 0; i < Context::NSIDE; i++) {
    if (c.ev_join[i]) cudaEventDestroy(c.ev_join[i]);
    if (c.side[i]) cudaStreamDestroy(c.side[i]);
  }
  if (c.ev_fork) cudaEventDestroy(c.ev_fork);
  if (c.own_stream) cudaStreamDestroy(c.own_stream);
  c = Context();
  g_nocc = 0;  // attributes and occupancy belong to this device's context
  g_nlim = 0;
}

static int32_t create_context(Context& c, int32_t device) {
  PHCU_CUDA(cudaSetDevice(device));
  PHCU_CUDA(cudaStreamCreateWithFlags(&c.own_stream, cudaStreamNonBlocking));
  c.stream = c.own_stream;
  PHCU_CUDA(cudaMalloc(&c.status, sizeof(uint32_t)));
  PHCU_CUDA(cudaMemset(c.status, 0, sizeof(uint32_t)));
  cudaDeviceProp prop;
  PHCU_CUDA(cudaGetDeviceProperties(&prop, device));
  c.sm_count = prop.multiProcessorCount;
  c.l2_bytes = prop.l2CacheSize;
  c.smem_optin = (int)prop.sharedMemPerBlockOptin;
  int clk = 0;
  cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, device);
  c.clock_khz = clk;
  // keep freed scratch in the pool instead of returning it to the driver
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  PHCU_CUDA(cudaStreamCreateWithFlags(&c.d2h, cudaStreamNonBlocking));
  PHCU_CUDA(cudaStreamCreateWithFlags(&c.h2d, cudaStreamNonBlocking));
  PHCU_CUDA(cudaEventCreateWithFlags(&c.ev_work, cudaEventDisableTiming));
  PHCU_CUDA(cudaEventCreateWithFlags(&c.ev_h2d, cudaEventDisableTiming));
  PHCU_CUDA(cudaEventCreateWithFlags(&c.ev_fork, cudaEventDisableTiming));
  for (int i = 0; i < Context::NSIDE; i++) {
    PHCU_CUDA(cudaStreamCreateWithFlags(&c.side[i], cudaStreamNonBlocking));
    PHCU_CUDA(cudaEventCreateWithFlags(&c.ev_join[i], cudaEventDisableTiming));
  }
  c.device = device;
  c.launches = 0;
  c.ready = true;
  return PHCU_OK;
}

}  // namespace phcu

using namespace phcu;

extern "C" {

int32_t phcu_init(int32_t device) {
  Context& c = g_ctx;
  if (c.ready && c.device == device) return PHCU_OK;
  if (c.ready) return fail(PHCU_ERR_INVALID, "phcu_init: already initialised on device %d", c.device);
  const int32_t rc = create_context(c, device);
  if (rc != PHCU_OK) {
    char msg[512];
    phcu_last_error(msg, sizeof(msg));
    release_context(c);  // a failed init leaves nothing behind; phcu_init may be called again
    return fail(rc, "%s", msg);
  }
  return PHCU_OK;
}

int32_t phcu_shutdown(void) {
  if (g_ctx.ready) release_context(g_ctx);
  return PHCU_OK;
}

int32_t phcu_set_stream(void* s) {
  PHCU_TRY(require_ctx());
  g_ctx.stream = s ? (cudaStream_t)s : g_ctx.own_stream;
  return PHCU_OK;
}

int32_t phcu_get_stream(void** s) {
  PHCU_TRY(require_ctx());
  if (!s) return fail(PHCU_ERR_INVALID, "phcu_get_stream: null output pointer");
  *s = (void*)g_ctx.stream;
  return PHCU_OK;
}

int32_t phcu_sync(void) {
  PHCU_TRY(require_ctx());
  PHCU_CUDA(cudaStreamSynchronize(g_ctx.stream));
  PHCU_CUDA(cudaStreamSynchronize(g_ctx.d2h));
  PHCU_CUDA(cudaStreamSynchronize(g_ctx.h2d));
  return PHCU_OK;
}

int32_t phcu_last_error(char* buf, size_t len) {
  if (!buf || len == 0) return PHCU_ERR_INVALID;
  snprintf(buf, len, "%s", g_err);
  return PHCU_OK;
}

int32_t phcu_status_word(uint32_t* out, int32_t clear) {
  PHCU_TRY(require_ctx());
  if (!out) return fail(PHCU_ERR_INVALID, "phcu_status_word: null output pointer");
  uint32_t v = 0;
  PHCU_CUDA(cudaMemcpyAsync(&v, g_ctx.status, sizeof(v), cudaMemcpyDeviceToHost, g_ctx.stream));
  PHCU_CUDA(cudaStreamSynchronize(g_ctx.stream));
  if (clear && v) {
    PHCU_CUDA(cudaMemsetAsync(g_ctx.status, 0, sizeof(uint32_t), g_ctx.stream));
    PHCU_CUDA(cudaStreamSynchronize(g_ctx.stream));
  }
  *out = v;
  return PHCU_OK;
}

int32_t phcu_version(int32_t* major, int32_t* minor) {
  if (!major || !minor) return fail(PHCU_ERR_INVALID, "phcu_version: null output pointer");
  *major = PHCU_VERSION_MAJOR;
  *minor = PHCU_VERSION_MINOR;
  return PHCU_OK;
}

int32_t phcu_device_info(int32_t* sm_count, int64_t* l2_bytes, int32_t* smem_per_block,
                         int32_t* clock_khz) {
  PHCU_TRY(require_ctx());
  if (sm_count) *sm_count = g_ctx.sm_count;
  if (l2_bytes) *l2_bytes = g_ctx.l2_bytes;
  if (smem_per_block) *smem_per_block = g_ctx.smem_optin;
  if (clock_khz) *clock_khz = g_ctx.clock_khz;
  return PHCU_OK;
}

int32_t phcu_alloc(size_t bytes, void** dptr) {
  PHCU_TRY(require_ctx());
  if (!dptr) return fail(PHCU_ERR_INVALID, "phcu_alloc: null output pointer");
  if (bytes == 0) bytes = 16;  // keep every array addressable
  cudaError_t e = cudaMallocAsync(dptr, bytes, g_ctx.stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMallocAsync");
  return PHCU_OK;
}

int32_t phcu_free(void* dptr) {
  PHCU_TRY(require_ctx());
  if (!dptr) return PHCU_OK;
  PHCU_CUDA(cudaFreeAsync(dptr, g_ctx.stream));
  return PHCU_OK;
}

int32_t phcu_host_alloc(size_t bytes, void** hptr) {
  PHCU_TRY(require_ctx());
  if (!hptr) return fail(PHCU_ERR_INVALID, "phcu_host_alloc: null output pointer");
  PHCU_CUDA(cudaMallocHost(hptr, bytes ? bytes : 16));
  return PHCU_OK;
}

int32_t phcu_host_free(void* hptr) {
  if (hptr) PHCU_CUDA(cudaFreeHost(hptr));
  return PHCU_OK;
}

int32_t phcu_upload(void* dst, const void* src, size_t bytes) {
  PHCU_TRY(require_ctx());
  if (bytes == 0) return PHCU_OK;
  PHCU_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, g_ctx.stream));
  return PHCU_OK;
}

int32_t phcu_download(void* dst, const void* src, size_t bytes) {
  PHCU_TRY(require_ctx());
  if (bytes == 0) return PHCU_OK;
  PHCU_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, g_ctx.stream));
  PHCU_CUDA(cudaStreamSynchronize(g_ctx.stream));
  return PHCU_OK;
}

// Device -> host behind the library stream: the copy waits for the work
// enqueued so far (an event on the library stream), then runs on the
// device-to-host stream while later kernels proceed.
int32_t phcu_download_async(void* dst, const void* src, size_t bytes) {
  PHCU_TRY(require_ctx());
  if (bytes == 0) return PHCU_OK;
  if (!dst || !src) return fail(PHCU_ERR_INVALID, "phcu_download_async: null pointer");
  PHCU_CUDA(cudaEventRecord(g_ctx.ev_work, g_ctx.stream));
  PHCU_CUDA(cudaStreamWaitEvent(g_ctx.d2h, g_ctx.ev_work, 0));
  PHCU_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, g_ctx.d2h));
  return PHCU_OK;
}

// Host -> device on the host-to-device stream: it waits for the work enqueued
// so far (which may still read dst), and later library work waits for it.
// Outstanding downloads are not waited for, so an upload overlaps them.
int32_t phcu_upload_async(void* dst, const void* src, size_t bytes) {
  PHCU_TRY(require_ctx());
  if (bytes == 0) return PHCU_OK;
  if (!dst || !src) return fail(PHCU_ERR_INVALID, "phcu_upload_async: null pointer");
  PHCU_CUDA(cudaEventRecord(g_ctx.ev_work, g_ctx.stream));
  PHCU_CUDA(cudaStreamWaitEvent(g_ctx.h2d, g_ctx.ev_work, 0));
  PHCU_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, g_ctx.h2d));
  PHCU_CUDA(cudaEventRecord(g_ctx.ev_h2d, g_ctx.h2d));
  PHCU_CUDA(cudaStreamWaitEvent(g_ctx.stream, g_ctx.ev_h2d, 0));
  return PHCU_OK;
}

int32_t phcu_transfer_wait(void) {
  PHCU_TRY(require_ctx());
  PHCU_CUDA(cudaStreamSynchronize(g_ctx.d2h));
  PHCU_CUDA(cudaStreamSynchronize(g_ctx.h2d));
  return PHCU_OK;
}

int32_t phcu_memset(void* dptr, int32_t value, size_t bytes) {
  PHCU_TRY(require_ctx());
  if (bytes == 0) return PHCU_OK;
  PHCU_CUDA(cudaMemsetAsync(dptr, value, bytes, g_ctx.stream));
  return PHCU_OK;
}

int32_t phcu_graph_begin(void) {
  PHCU_TRY(require_ctx());
  if (g_ctx.stream == 0) return fail(PHCU_ERR_INVALID, "cannot capture the legacy default stream");
  PHCU_CUDA(cudaStreamBeginCapture(g_ctx.stream, cudaStreamCaptureModeThreadLocal));
  return PHCU_OK;
}

int32_t phcu_graph_end(void** graph_exec) {
  PHCU_TRY(require_ctx());
  cudaGraph_t g;
  PHCU_CUDA(cudaStreamEndCapture(g_ctx.stream, &g));  // the capture ends whatever follows
  if (!graph_exec) {
    cudaGraphDestroy(g);
    return fail(PHCU_ERR_INVALID, "phcu_graph_end: null output pointer");
  }
  cudaGraphExec_t ge;
  cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
  *graph_exec = (void*)ge;
  return PHCU_OK;
}

int32_t phcu_graph_launch(void* graph_exec) {
  PHCU_TRY(require_ctx());
  PHCU_CUDA(cudaGraphLaunch((cudaGraphExec_t)graph_exec, g_ctx.stream));
  return PHCU_OK;
}

int32_t phcu_graph_destroy(void* graph_exec) {
  if (graph_exec) PHCU_CUDA(cudaGraphExecDestroy((cudaGraphExec_t)graph_exec));
  return PHCU_OK;
}

static void timer_release(Timer* t) {
  if (t->a) cudaEventDestroy(t->a);
  if (t->b) cudaEventDestroy(t->b);
  delete t;
}

int32_t phcu_timer_start(void** timer) {
  PHCU_TRY(require_ctx());
  if (!timer) return fail(PHCU_ERR_INVALID, "phcu_timer_start: null output pointer");
  Timer* t = new Timer{nullptr, nullptr};
  cudaError_t e = cudaEventCreate(&t->a);
  if (e == cudaSuccess) e = cudaEventCreate(&t->b);
  if (e == cudaSuccess) e = cudaEventRecord(t->a, g_ctx.stream);
  if (e != cudaSuccess) {
    timer_release(t);
    return cuda_fail(e, "phcu_timer_start");
  }
  *timer = t;
  return PHCU_OK;
}

// Stops and releases the timer, whether or not the measurement succeeds.
int32_t phcu_timer_stop(void* timer, float* ms) {
  PHCU_TRY(require_ctx());
  if (!timer || !ms) return fail(PHCU_ERR_INVALID, "phcu_timer_stop: null pointer");
  Timer* t = (Timer*)timer;
  cudaError_t e = cudaEventRecord(t->b, g_ctx.stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(t->b);
  if (e == cudaSuccess) e = cudaEventElapsedTime(ms, t->a, t->b);
  timer_release(t);
  if (e != cudaSuccess) return cuda_fail(e, "phcu_timer_stop");
  return PHCU_OK;
}

int32_t phcu_launch_count(uint64_t* n) {
  if (!n) return fail(PHCU_ERR_INVALID, "phcu_launch_count: null output pointer");
  *n = g_ctx.launches;
  return PHCU_OK;
}

int32_t phcu_l2_flush(void) {
  PHCU_TRY(require_ctx());
  Context& c = g_ctx;
  size_t want = (size_t)(c.l2_bytes > 0 ? c.l2_bytes : (128ll << 20)) * 2;
  if (!c.l2_scrub) {
    PHCU_CUDA(cudaMalloc(&c.l2_scrub, want));
    c.l2_scrub_bytes = want;
  }
  PHCU_CUDA(cudaMemsetAsync(c.l2_scrub, c.launches & 0xff, c.l2_scrub_bytes, c.stream));
  return PHCU_OK;
}

}  // extern "C"
