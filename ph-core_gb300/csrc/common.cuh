// common.cuh -- shared internals of libphcuda.so (GB300, sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <string>

#include "phcuda.h"

namespace phcu {

constexpr int MAXR = PHCU_MAX_RANK;
constexpr int MAXIN = PHCU_MAX_INPUTS;

// ------------------------------------------------------------------ errors
void set_error(const char* fmt, ...);
int32_t fail(int32_t code, const char* fmt, ...);
int32_t cuda_fail(cudaError_t e, const char* what);

#define PHCU_CUDA(call)                                   \
  do {                                                    \
    cudaError_t _e = (call);                              \
    if (_e != cudaSuccess) return phcu::cuda_fail(_e, #call); \
  } while (0)

#define PHCU_TRY(call)               \
  do {                               \
    int32_t _rc = (call);            \
    if (_rc != PHCU_OK) return _rc;  \
  } while (0)

// ----------------------------------------------------------------- context
struct Context {
  bool ready = false;
  int device = -1;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  uint32_t* status = nullptr;  // device status word
  int sm_count = 0;
  int64_t l2_bytes = 0;
  int smem_optin = 0;
  int clock_khz = 0;
  void* l2_scrub = nullptr;
  size_t l2_scrub_bytes = 0;
  unsigned long long launches = 0;
  // transfers that run behind the library stream's kernels (one stream per
  // copy direction, so both copy engines and the SMs work at once)
  cudaStream_t d2h = nullptr, h2d = nullptr;
  cudaEvent_t ev_work = nullptr, ev_h2d = nullptr;
  // side streams of a batch launch: its class kernels after the first run
  // beside it, forked from and joined back to the library stream by events
  static constexpr int NSIDE = 4;
  cudaStream_t side[NSIDE] = {};
  cudaEvent_t ev_fork = nullptr;
  cudaEvent_t ev_join[NSIDE] = {};
};
Context& ctx();
int32_t require_ctx();
inline cudaStream_t stream() { return ctx().stream; }
inline void count_launch(unsigned n = 1) { ctx().launches += n; }
int32_t check_launch(const char* what);

// Resident blocks per SM of kernel `fn` at this block size and dynamic
// shared memory, asked of the runtime once per (kernel, threads, smem) and
// remembered: the query costs host time that would otherwise come with every
// launch.  Raises the kernel's dynamic shared-memory limit first when smem
// exceeds the 48 KB default (only ever upwards, once per new maximum).
int blocks_per_sm(const void* fn, int threads, size_t smem);

// Destroys the heat runs' cached CUDA graphs (at shutdown).
void release_heat_graphs();

// Forgets the cached device addresses of the allocation-free reduction's
// static scratch (at shutdown: a later context may load the module anew).
void release_noalloc_scratch();

// stream-ordered scratch
int32_t scratch_alloc(size_t bytes, void** p);
void scratch_free(void* p);

// ------------------------------------------------------------------- dtypes
__host__ __device__ inline int dtype_size(int t) {
  switch (t) {
    case PHCU_BOOL: return 1;
    case PHCU_I32: return 4;
    case PHCU_I64: return 8;
    case PHCU_F32: return 4;
    case PHCU_F64: return 8;
  }
  return 0;
}
inline bool dtype_valid(int t) { return t >= PHCU_BOOL && t <= PHCU_F64; }
__host__ __device__ inline bool is_float_t(int t) { return t == PHCU_F32 || t == PHCU_F64; }
__host__ __device__ inline bool is_int_t(int t) { return t == PHCU_I32 || t == PHCU_I64; }

// ------------------------------------------------------- 32-bit fast divide
// Division of n < 2^32 by an invariant d >= 1 with one high multiply:
// l = ceil(log2 d), m = floor(2^32 (2^l - d) / d) + 1, q = (umulhi(n, m) + n) >> l
// (Granlund & Montgomery, "Division by invariant integers using
// multiplication", 1994, the 33-bit-product variant).
struct FastDiv {
  uint32_t d;
  uint32_t m;
  uint32_t l;
  __host__ __device__ FastDiv() : d(1), m(1), l(0) {}
  __host__ explicit FastDiv(uint32_t div) { init(div); }
  __host__ void init(uint32_t div) {
    d = div ? div : 1;
    l = 0;
    while ((1ull << l) < d) l++;
    uint64_t num = ((1ull << l) - d) << 32;
    m = (uint32_t)(num / d + 1);
  }
  __device__ __forceinline__ uint32_t div(uint32_t n) const {
    uint64_t t = __umulhi(n, m);
    return (uint32_t)((t + n) >> l);
  }
  __host__ uint32_t div_host(uint32_t n) const {
    uint64_t t = ((uint64_t)n * m) >> 32;
    return (uint32_t)((t + n) >> l);
  }
  __device__ __forceinline__ void divmod(uint32_t n, uint32_t& q, uint32_t& r) const {
    q = div(n);
    r = n - q * d;
  }
};

// ------------------------------------------------------------- status word
__device__ __forceinline__ void report_status(uint32_t* st, uint32_t bits) {
  // one atomic per warp that saw a problem
  unsigned mask = __activemask();
  unsigned any = __reduce_or_sync(mask, bits);
  if (any && (threadIdx.x & 31) == (__ffs(mask) - 1)) atomicOr(st, any);
}

// ---------------------------------------------------- canonical operations
// An operand after canonicalisation: byte pointer of element 0 of the
// canonical iteration space plus element strides per canonical axis.
struct Operand {
  const char* base;  // base + offset * es
  int64_t stride[MAXR];
  int32_t dtype;
  int32_t vmode;  // vector mode chosen by the planner (see plan.cpp)
};

// Canonical iteration space shared by the output and all inputs.
struct Space {
  int32_t rank;
  int32_t pad;
  int64_t n;              // number of elements
  int64_t shape[MAXR];
  FastDiv div[MAXR];
};

enum VMode : int32_t {
  VM_SCALAR = 0,   // scalar loads/stores with the canonical inner stride
  VM_VEC = 1,      // inner stride +1 and aligned: vector access
  VM_VEC_REV = 2,  // inner stride -1 and aligned at the low end: reversed vector access
  VM_INDEX = 3,    // an index operand (PHCU_INDEX): the value is computed, base holds its offset
};

}  // namespace phcu
