// common.cuh -- shared device helpers and the per-call context of the GB300
// partitioning library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <utility>
#include <vector>

#include "../../include/parrsb.h"

namespace prsb {

typedef long long ll;

// --------------------------------------------------------------------------
// Error handling: every CUDA call is checked; failures unwind to the C-ABI,
// which returns PARRSB_ERR_CUDA.  The library never exits the process.
// --------------------------------------------------------------------------
struct CudaError {
  cudaError_t err;
  const char *file;
  int line;
};

#define CK(call)                                                              \
  do {                                                                        \
    cudaError_t e_ = (call);                                                  \
    if (e_ != cudaSuccess) throw ::prsb::CudaError{e_, __FILE__, __LINE__};   \
  } while (0)

#define CK_LAUNCH()                                                           \
  do {                                                                        \
    ::prsb::ctx().kernel_launches++;                                          \
    cudaError_t e_ = cudaGetLastError();                                      \
    if (e_ != cudaSuccess) throw ::prsb::CudaError{e_, __FILE__, __LINE__};   \
  } while (0)

struct ArgError {
  int code;
  const char *msg;
};

// --------------------------------------------------------------------------
// Device buffer (RAII) and a per-thread context that owns the stream, event
// pool and statistics of the current call.
// --------------------------------------------------------------------------
// Stream-ordered device allocation on the library stream (memory is kept in
// the device's default pool between calls; see Ctx::init).
void *dev_alloc(size_t bytes);
void dev_free(void *p);

template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  DBuf() {}
  explicit DBuf(size_t count) { alloc(count); }
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr, o.n = 0; }
  DBuf &operator=(DBuf &&o) noexcept {
    release();
    p = o.p, n = o.n;
    o.p = nullptr, o.n = 0;
    return *this;
  }
  void alloc(size_t count) {
    release();
    if (count == 0) count = 1;
    p = (T *)dev_alloc(count * sizeof(T));
    n = count;
  }
  void ensure(size_t count) {
    if (count > n || p == nullptr) alloc(count);
  }
  void release() {
    if (p) dev_free(p);
    p = nullptr, n = 0;
  }
  ~DBuf() { release(); }
  T *get() const { return p; }
};

// Device buffer that lives across calls (the cached upload / download
// buffers of the host entry points): plain cudaMalloc / cudaFree instead of
// the stream-ordered pool, so that the pool's growth and reuse by the
// temporaries of a call never touch the pages the host copies land in.
template <typename T>
struct PBuf {
  T *p = nullptr;
  size_t n = 0;
  PBuf() {}
  PBuf(const PBuf &) = delete;
  PBuf &operator=(const PBuf &) = delete;
  void ensure(size_t count) {
    if (count == 0) count = 1;
    if (p && count <= n) return;
    release();
    CK(cudaMalloc(reinterpret_cast<void **>(&p), count * sizeof(T)));
    n = count;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr, n = 0;
  }
  ~PBuf() { release(); }
};

// One per host thread.  Every call runs on the device that is current when
// it starts: init() selects that device's stream (created on first use) and
// workspace, so a thread may switch devices between calls.
constexpr int MAX_DEVICES = 64;
struct Ctx {
  cudaStream_t stream = nullptr;  // the current device's library stream
  int device = 0;
  cudaStream_t streams[MAX_DEVICES] = {};
  parrsb_stats stats;
  long long kernel_launches = 0;
  bool timing = false;  // time SpMV launches with events
  void init();
};

Ctx &ctx();

// Programmatic dependent launch.  A kernel launched through launch_pdl may be
// scheduled while its predecessor on the stream drains; its first statement,
// pdl_entry(), waits (griddepcontrol.wait) until the predecessor grid has
// completed and its writes are visible, so nothing is read early, and then
// lets the next such kernel be scheduled.  For a kernel launched without the
// attribute the wait returns at once.  PARRSB_GPU_PDL=0 launches without it.
__device__ __forceinline__ void pdl_entry() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
bool pdl_enabled();
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kern)(KArgs...), unsigned grid, unsigned block, size_t smem,
                       cudaStream_t st, Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr;
  attr.id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr.val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  ctx().kernel_launches++;
  CK(cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...));
}

// Stage timer using CUDA events on the context stream.
struct StageTimer {
  cudaEvent_t a = nullptr, b = nullptr;
  int stage;
  explicit StageTimer(int s) : stage(s) {
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, ctx().stream));
  }
  ~StageTimer() {
    if (cudaEventRecord(b, ctx().stream) == cudaSuccess &&
        cudaEventSynchronize(b) == cudaSuccess) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, a, b) == cudaSuccess)
        ctx().stats.stage_ms[stage] += ms;
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

template <typename T>
inline void h2d(T *d, const T *h, size_t n) {
  if (n) CK(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx().stream));
}
template <typename T>
inline void d2h(T *h, const T *d, size_t n) {
  if (n) CK(cudaMemcpyAsync(h, d, n * sizeof(T), cudaMemcpyDeviceToHost, ctx().stream));
}
inline void sync() { CK(cudaStreamSynchronize(ctx().stream)); }

// cudaFuncSetAttribute acts on the current device only.  Raise `func`'s
// dynamic shared-memory limit to at least `bytes` on the current device,
// once per (kernel, device); thread-safe.
cudaError_t smem_limit_on_device(const void *func, int bytes);
template <typename K>
inline void ensure_smem_limit(K *func, int bytes) {
  CK(smem_limit_on_device(reinterpret_cast<const void *>(func), bytes));
}

inline unsigned grid_for(ll n, int threads) {
  ll g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  return (unsigned)g;
}

// --------------------------------------------------------------------------
// Device helpers
// --------------------------------------------------------------------------
// Order-preserving map of an IEEE double to uint64 (numeric order; -0.0 and
// +0.0 map to the same key, matching a '<' comparison sort).
__device__ __forceinline__ unsigned long long ordered_key(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  if (x == 0.0) b = 0ull;  // -0.0 -> +0.0
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Shuffle-down tree over the 32 lanes (offsets 16, 8, 4, 2, 1); lane 0 holds
// the canonical tile sum.  Additions use __dadd_rn so that no FMA forms.
__device__ __forceinline__ double warp_tree_sum(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1)
    v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, off));
  return v;
}

__device__ __forceinline__ double warp_min(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, off));
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, off));
  return v;
}

// Number of elements held by the first ceil(p/2) of p virtual ranks after a
// balanced sort of n elements (the first p - n%p ranks get n/p, the rest one
// more), mirroring the reference's element distribution.
__host__ __device__ inline ll lower_count(ll n, int p) {
  ll h = (p + 1) / 2;
  ll nelt = n / p, nrem = n - (ll)p * nelt;
  if (nrem == 0) return h * nelt;
  ll s = p - nrem;
  return h * nelt + (h > s ? h - s : 0);
}

}  // namespace prsb
