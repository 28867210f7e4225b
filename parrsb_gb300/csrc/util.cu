// util.cu -- three-phase exclusive scan and segment-table helpers.
#include <map>
#include <mutex>
#include <utility>

#include "util.cuh"

namespace prsb {

namespace {

constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <typename T>
__device__ ll load_as_ll(const T *in, ll i, ll n) {
  return i < n ? (ll)in[i] : 0ll;
}

__device__ ll block_excl_scan(ll v, ll *total) {
  __shared__ ll ws[32];
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  ll x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    ll y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int nw = blockDim.x >> 5;
    ll s = lane < nw ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      ll y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < nw) ws[lane] = s;
  }
  __syncthreads();
  ll excl = (warp ? ws[warp - 1] : 0) + x - v;
  *total = ws[(blockDim.x >> 5) - 1];
  __syncthreads();
  return excl;
}

template <typename T>
__global__ void k_block_sums(const T *in, ll n, ll *bsum) {
  ll base = (ll)blockIdx.x * SCAN_TILE + (ll)threadIdx.x * SCAN_ITEMS;
  ll s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) s += load_as_ll(in, base + k, n);
  ll total;
  block_excl_scan(s, &total);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

template <typename T>
__global__ void k_block_scan(const T *in, ll *out, ll n, const ll *boff) {
  ll base = (ll)blockIdx.x * SCAN_TILE + (ll)threadIdx.x * SCAN_ITEMS;
  ll v[SCAN_ITEMS];
  ll s = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) v[k] = load_as_ll(in, base + k, n), s += v[k];
  ll total;
  ll excl = block_excl_scan(s, &total) + boff[blockIdx.x];
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    if (base + k < n) out[base + k] = excl;
    excl += v[k];
  }
}

// want_total = false: the total is not returned (-1) and the host never waits
template <typename T>
ll scan_impl(const T *in, ll *out, ll n, bool want_total = true) {
  cudaStream_t st = ctx().stream;
  if (n <= 0) return 0;
  ll nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  DBuf<ll> bsum((size_t)nb + 1);
  ll total = -1;
  if (nb == 1 && !want_total) {
    CK(cudaMemsetAsync(bsum.p, 0, sizeof(ll), st));  // offset of the only block
    k_block_scan<T><<<1, SCAN_THREADS, 0, st>>>(in, out, n, bsum.p);
    CK_LAUNCH();
    return total;
  }
  k_block_sums<T><<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, n, bsum.p);
  CK_LAUNCH();
  if (nb == 1) {
    CK(cudaMemsetAsync(bsum.p + 1, 0, sizeof(ll), st));
    // offset of block 0 is 0; total is bsum[0]
    ll t0;
    d2h(&t0, bsum.p, 1);
    sync();
    total = t0;
    CK(cudaMemsetAsync(bsum.p, 0, sizeof(ll), st));
  } else {
    total = scan_impl<ll>(bsum.p, bsum.p, nb, want_total);
  }
  k_block_scan<T><<<(unsigned)nb, SCAN_THREADS, 0, st>>>(in, out, n, bsum.p);
  CK_LAUNCH();
  return total;
}

__global__ void k_fill_seg_of_pos(const ll *start, ll nseg, int *seg_of_pos,
                                  ll N) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  ll lo = 0, hi = nseg - 1;
  while (lo < hi) {  // last segment with start <= i
    ll mid = (lo + hi + 1) >> 1;
    if (start[mid] <= i)
      lo = mid;
    else
      hi = mid - 1;
  }
  seg_of_pos[i] = (int)lo;
}

}  // namespace

ll exclusive_scan_ll(const ll *in, ll *out, ll n) { return scan_impl<ll>(in, out, n); }
ll exclusive_scan_int_to_ll(const int *in, ll *out, ll n) {
  return scan_impl<int>(in, out, n);
}
void exclusive_scan_int_to_ll_async(const int *in, ll *out, ll n) {
  scan_impl<int>(in, out, n, false);
}

void fill_seg_of_pos(const SegTable &t, int *seg_of_pos, ll N) {
  if (N <= 0) return;
  k_fill_seg_of_pos<<<grid_for(N, 256), 256, 0, ctx().stream>>>(t.start.p, t.count,
                                                                 seg_of_pos, N);
  CK_LAUNCH();
}

cudaError_t smem_limit_on_device(const void *func, int bytes) {
  static std::mutex mu;
  static std::map<std::pair<const void *, int>, int> done;  // (kernel, device) -> bytes set
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(mu);
  auto key = std::make_pair(func, dev);
  auto it = done.find(key);
  if (it != done.end() && it->second >= bytes) return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess) done[key] = bytes;
  return e;
}

}  // namespace prsb
