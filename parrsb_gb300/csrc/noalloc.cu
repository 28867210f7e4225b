// noalloc.cu -- RCB partition of a small mesh without any allocation.
//
// For callers that cannot allocate device memory at the time of the call: a
// caller whose device memory all comes from its own pool or arena, a
// long-running service or solver loop that must not grow or fragment the
// device heap between steps, or code that runs where the runtime may not
// allocate.  Inputs and outputs are the caller's device buffers; every
// intermediate lives in one file-scope __device__ array of fixed size, and
// the kernels run on the caller's stream.
//
// Same result as parrsb_part_mesh with partitioner = 1 (RCB, src/rcb.c:7-137)
// for meshes of at most NA_MAX elements: the same centroids (sequential
// corner sums, then a division by nv; src/parrsb.c:103-166), order-preserving
// coordinate ranks, and the same CTA-per-segment recursion kernel.
#include <mutex>

#include "../../include/parrsb.h"
#include "bisect.cuh"

namespace prsb {
namespace {

constexpr int NA_MAX = 8192;  // elements (the CTA-resident recursion limit)
constexpr int NA_MAXDEV = 64;

constexpr size_t na_round(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t NA_CENT = 0;                                           // double [3][NA_MAX]
constexpr size_t NA_UNIQ = NA_CENT + na_round(3 * NA_MAX * sizeof(double));  // double [3][NA_MAX]
constexpr size_t NA_RANK = NA_UNIQ + na_round(3 * NA_MAX * sizeof(double));  // u32 [3][NA_MAX]
constexpr size_t NA_PERM = NA_RANK + na_round(3 * NA_MAX * sizeof(u32));     // int [NA_MAX]
constexpr size_t NA_SEG = NA_PERM + na_round(NA_MAX * sizeof(int));          // 2 ll + 2 int
constexpr size_t NA_BYTES = NA_SEG + 256;                                    // 524,544 bytes

// Nothing in it needs to start at zero: every word a kernel reads is written
// earlier in the same call (ranks index only written `uniq` slots).
static __device__ __align__(256) unsigned char na_scratch[NA_BYTES];

struct NaDev {
  unsigned char *ptr = nullptr;
  bool ready = false;
};
NaDev na_dev[NA_MAXDEV];
std::mutex na_mu;

__global__ void k_na_ranks(const double *__restrict__ cent, int n, u32 *__restrict__ rank,
                           double *__restrict__ uniq);

// Once per device, with that device current: the scratch address and the
// shared-memory limits of the rank and recursion kernels.
cudaError_t na_setup(int dev, unsigned char **out) {
  std::lock_guard<std::mutex> lk(na_mu);
  if (!na_dev[dev].ready) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, na_scratch);
    if (e != cudaSuccess) return e;
    e = rcb_small_prepare();
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(k_na_ranks, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             NA_MAX * (int)sizeof(unsigned long long));
    if (e != cudaSuccess) return e;
    na_dev[dev].ptr = static_cast<unsigned char *>(p);
    na_dev[dev].ready = true;
  }
  *out = na_dev[dev].ptr;
  return cudaSuccess;
}

// centroids with the arithmetic of the allocating path, identity order and
// the single segment [0, n) of nparts ranks
__global__ void k_na_init(const double *__restrict__ xyz, int n, int nv, int ndim, int nparts,
                          double *__restrict__ cent, int *__restrict__ perm,
                          ll *__restrict__ seg_ll, int *__restrict__ seg_int) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e == 0) seg_ll[0] = 0, seg_ll[1] = n, seg_int[0] = nparts, seg_int[1] = 0;
  if (e >= n) return;
  double c[3] = {0.0, 0.0, 0.0};
  const double *x = xyz + (ll)e * nv * ndim;
  for (int v = 0; v < nv; v++)
    for (int d = 0; d < ndim; d++) c[d] = __dadd_rn(c[d], x[v * ndim + d]);
  for (int d = 0; d < ndim; d++) c[d] = __ddiv_rn(c[d], (double)nv);
  for (int d = 0; d < 3; d++) cent[(ll)d * n + e] = c[d];
  perm[e] = e;
}

// rank = number of centroids strictly below on the axis (ties share a rank,
// the order is that of the values); uniq[rank] = the value.  Block (x, a)
// ranks 256 elements of axis a against all n keys held in shared memory.
__global__ void __launch_bounds__(256)
k_na_ranks(const double *__restrict__ cent, int n, u32 *__restrict__ rank,
           double *__restrict__ uniq) {
  extern __shared__ unsigned long long na_keys[];
  const int a = blockIdx.y;
  const double *c = cent + (ll)a * n;
  for (int j = threadIdx.x; j < n; j += blockDim.x) na_keys[j] = ordered_key(c[j]);
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long k = na_keys[i];
  u32 r = 0;
  for (int j = 0; j < n; j++) r += na_keys[j] < k;
  rank[(ll)a * n + i] = r;
  const double v = c[i];
  uniq[(ll)a * n + r] = v == 0.0 ? 0.0 : v;  // -0 and +0 share a rank
}

}  // namespace
}  // namespace prsb

using namespace prsb;

extern "C" PARRSB_API int parrsb_part_mesh_rcb_noalloc(int *d_part, const double *d_xyz,
                                                       int nel, int nv, int nparts,
                                                       void *stream) {
  if (nel < 0 || (nel > 0 && (!d_part || !d_xyz)) || (nv != 4 && nv != 8) || nparts < 1)
    return PARRSB_ERR_ARGS;
  if (nel > NA_MAX) return PARRSB_ERR_UNSUPPORTED;  // more than 8192 elements
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAXDEV) return PARRSB_ERR_CUDA;
  unsigned char *base = nullptr;
  if (na_setup(dev, &base) != cudaSuccess) return PARRSB_ERR_CUDA;
  if (nel == 0) return PARRSB_OK;  // setup only
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int ndim = nv == 8 ? 3 : 2;
  const int P = nparts > nel ? nel : nparts;
  double *cent = reinterpret_cast<double *>(base + NA_CENT);
  double *uniq = reinterpret_cast<double *>(base + NA_UNIQ);
  u32 *rank = reinterpret_cast<u32 *>(base + NA_RANK);
  int *perm = reinterpret_cast<int *>(base + NA_PERM);
  ll *seg_ll = reinterpret_cast<ll *>(base + NA_SEG);
  int *seg_int = reinterpret_cast<int *>(base + NA_SEG + 2 * sizeof(ll));
  k_na_init<<<(nel + 255) / 256, 256, 0, st>>>(d_xyz, nel, nv, ndim, P, cent, perm, seg_ll,
                                               seg_int);
  if (cudaGetLastError() != cudaSuccess) return PARRSB_ERR_CUDA;
  if (P == 1) {
    if (cudaMemsetAsync(d_part, 0, (size_t)nel * sizeof(int), st) != cudaSuccess)
      return PARRSB_ERR_CUDA;
    return PARRSB_OK;
  }
  dim3 grid((nel + 255) / 256, ndim);
  k_na_ranks<<<grid, 256, (size_t)nel * sizeof(unsigned long long), st>>>(cent, nel, rank, uniq);
  if (cudaGetLastError() != cudaSuccess) return PARRSB_ERR_CUDA;
  if (rcb_small_launch(perm, rank, uniq, nel, ndim, seg_ll, seg_ll + 1, seg_int, seg_int + 1, 1,
                       false, d_part, st) != cudaSuccess)
    return PARRSB_ERR_CUDA;
  return PARRSB_OK;
}
