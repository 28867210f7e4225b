// sort.cu -- segmented stable LSD radix sort for sm_103a.
//
// Replaces the reference's distributed stable sorts (parallel_sort_,
// src/sort.c:182-213, bin sort src/sort-bin.c:36-50, local gslib sorts
// src/sort.c:72-104).  A segmented sort by (segment, key) is an LSD sort on
// the key bytes followed by the segment-id bytes; every pass is stable, so
// ties keep their current order (the canonical tie-break).
//
// Per pass: a tile histogram kernel (4096 items per 512-thread CTA), a
// per-digit exclusive scan over tiles, and a scatter kernel that loads its
// 8 items per thread up front, ranks them stably inside the CTA with
// __match_any_sync (warp w owns items [w*256, w*256+256) of the tile,
// processed 32 at a time in order), stages the tile in shared memory in
// digit order and writes each digit's run with consecutive addresses.  One
// up-front kernel builds the global digit histograms of every pass; passes
// whose digit is constant over all items are skipped.
#include "sort.cuh"

namespace prsb {

namespace {

constexpr int SORT_THREADS = 512;
constexpr int ITEMS_PER_THREAD = 8;
constexpr int NWARP = SORT_THREADS / 32;
constexpr int TILE = SORT_THREADS * ITEMS_PER_THREAD;  // 4096
constexpr int MAX_PASSES = 12;                           // 8 key + 4 seg bytes
constexpr size_t SCATTER_SMEM = (size_t)TILE * (8 + 4 + 1);  // staged keys, values, digits

struct PassDesc {
  int is_seg;
  int shift;
};

__device__ __forceinline__ u32 digit_of(u64 key, int val, const int *seg_of_val,
                                         int is_seg, int shift) {
  if (is_seg) return ((u32)seg_of_val[val] >> shift) & 255u;
  return (u32)(key >> shift) & 255u;
}

__global__ void k_hist_all(const u64 *__restrict__ keys, const int *__restrict__ vals,
                           ll n, const int *__restrict__ seg_of_val, int nkey,
                           int nseg_pass, u32 *__restrict__ hist_all) {
  __shared__ u32 h[MAX_PASSES][256];
  int np = nkey + nseg_pass;
  for (int i = threadIdx.x; i < np * 256; i += blockDim.x) (&h[0][0])[i] = 0;
  __syncthreads();
  ll stride = (ll)gridDim.x * blockDim.x;
  for (ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    u64 k = keys[i];
    for (int b = 0; b < nkey; b++) atomicAdd(&h[b][(u32)(k >> (8 * b)) & 255u], 1u);
    if (nseg_pass) {
      u32 s = (u32)seg_of_val[vals[i]];
      for (int b = 0; b < nseg_pass; b++)
        atomicAdd(&h[nkey + b][(s >> (8 * b)) & 255u], 1u);
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < np * 256; i += blockDim.x) {
    u32 c = (&h[0][0])[i];
    if (c) atomicAdd(&hist_all[i], c);
  }
}

__global__ void __launch_bounds__(SORT_THREADS)
k_tile_hist(const u64 *__restrict__ keys, const int *__restrict__ vals, ll n,
            const int *__restrict__ seg_of_val, int is_seg, int shift,
            u32 *__restrict__ counts, int ntiles) {
  __shared__ u32 h[NWARP][256];
  int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < NWARP * 256; i += blockDim.x) (&h[0][0])[i] = 0;
  __syncthreads();
  ll base = (ll)blockIdx.x * TILE + warp * (32 * ITEMS_PER_THREAD);
  u32 d[ITEMS_PER_THREAD];
#pragma unroll
  for (int r = 0; r < ITEMS_PER_THREAD; r++) {
    ll i = base + r * 32 + lane;
    d[r] = i < n ? digit_of(keys[i], is_seg ? vals[i] : 0, seg_of_val, is_seg, shift) : 256u;
  }
#pragma unroll
  for (int r = 0; r < ITEMS_PER_THREAD; r++)
    if (d[r] < 256) atomicAdd(&h[warp][d[r]], 1u);
  __syncthreads();
  for (int dd = threadIdx.x; dd < 256; dd += blockDim.x) {
    u32 s = 0;
#pragma unroll
    for (int w = 0; w < NWARP; w++) s += h[w][dd];
    counts[(ll)dd * ntiles + blockIdx.x] = s;
  }
}

// One CTA per digit: exclusive prefix of counts[d][0..ntiles) in place.
__global__ void k_tile_scan(u32 *__restrict__ counts, int ntiles,
                            u32 *__restrict__ totals) {
  __shared__ u32 wsum[32];
  __shared__ u32 carry_s;
  u32 *row = counts + (ll)blockIdx.x * ntiles;
  if (threadIdx.x == 0) carry_s = 0;
  __syncthreads();
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int nw = blockDim.x >> 5;
  for (int base = 0; base < ntiles; base += blockDim.x) {
    int i = base + threadIdx.x;
    u32 v = i < ntiles ? row[i] : 0u;
    u32 x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      u32 y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
      u32 s = lane < nw ? wsum[lane] : 0u;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        u32 y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      if (lane < nw) wsum[lane] = s;
    }
    __syncthreads();
    u32 carry = carry_s;
    u32 excl = carry + (warp ? wsum[warp - 1] : 0u) + x - v;
    if (i < ntiles) row[i] = excl;
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry_s = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) totals[blockIdx.x] = carry_s;
}

__global__ void __launch_bounds__(SORT_THREADS)
k_scatter(const u64 *__restrict__ kin, const int *__restrict__ vin,
          u64 *__restrict__ kout, int *__restrict__ vout, ll n,
          const int *__restrict__ seg_of_val, int is_seg, int shift,
          const u32 *__restrict__ counts, const u32 *__restrict__ totals,
          int ntiles) {
  __shared__ u32 wcnt[NWARP][256];
  __shared__ u32 dbase[256];
  __shared__ u32 tl[256];  // tile-local start of each digit
  __shared__ u32 ws[8], ws2[8];
  extern __shared__ __align__(16) unsigned char sc_smem[];
  u64 *skey = reinterpret_cast<u64 *>(sc_smem);             // TILE
  int *sval = reinterpret_cast<int *>(skey + TILE);          // TILE
  unsigned char *sdig = reinterpret_cast<unsigned char *>(sval + TILE);  // TILE
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int i = threadIdx.x; i < NWARP * 256; i += blockDim.x) (&wcnt[0][0])[i] = 0;
  // global start of every digit in this tile: exclusive scan of the 256
  // digit totals (threads 0..255, one digit each) plus the tile's offset
  {
    const u32 v = threadIdx.x < 256 ? totals[threadIdx.x] : 0u;
    u32 x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      u32 y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (threadIdx.x < 256 && lane == 31) ws[warp] = x;
    __syncthreads();
    if (threadIdx.x < 256) {
      u32 off = 0;
      for (int w = 0; w < warp; w++) off += ws[w];
      dbase[threadIdx.x] = off + x - v + counts[(ll)threadIdx.x * ntiles + blockIdx.x];
    }
  }
  // every load of the tile is issued before the ranking loop
  u64 key[ITEMS_PER_THREAD];
  int val[ITEMS_PER_THREAD];
  u32 rank[ITEMS_PER_THREAD];
  u32 dig[ITEMS_PER_THREAD];
  const unsigned lt_mask = (1u << lane) - 1u;
  const ll base = (ll)blockIdx.x * TILE + warp * (32 * ITEMS_PER_THREAD);
#pragma unroll
  for (int r = 0; r < ITEMS_PER_THREAD; r++) {
    const ll i = base + r * 32 + lane;
    if (i < n) {
      key[r] = kin[i];
      val[r] = vin[i];
    }
  }
#pragma unroll
  for (int r = 0; r < ITEMS_PER_THREAD; r++) {
    const ll i = base + r * 32 + lane;
    dig[r] = i < n ? digit_of(key[r], val[r], seg_of_val, is_seg, shift) : 256u;
  }
  // stable rank within the warp's items (32 at a time, in order)
#pragma unroll
  for (int r = 0; r < ITEMS_PER_THREAD; r++) {
    const u32 d = dig[r];
    const bool valid = d < 256;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    u32 before = 0;
    if (valid) before = wcnt[warp][d];
    __syncwarp();
    if (valid) {
      rank[r] = before + __popc(peers & lt_mask);
      if (lane == __ffs(peers) - 1) wcnt[warp][d] = before + __popc(peers);
    }
    __syncwarp();
  }
  __syncthreads();
  // exclusive scan over warps per digit, then over the digits of the tile
  {
    u32 run = 0;
    if (threadIdx.x < 256) {
      const int d = threadIdx.x;
#pragma unroll
      for (int w = 0; w < NWARP; w++) {
        u32 t = wcnt[w][d];
        wcnt[w][d] = run;
        run += t;
      }
    }
    u32 x = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      u32 y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (threadIdx.x < 256 && lane == 31) ws2[warp] = x;
    __syncthreads();
    if (threadIdx.x < 256) {
      u32 off = 0;
      for (int w = 0; w < warp; w++) off += ws2[w];
      tl[threadIdx.x] = off + x - run;
    }
  }
  __syncthreads();
  // stage the tile in digit order, then write every digit run with
  // consecutive addresses (coalesced stores instead of 256 scattered streams)
#pragma unroll
  for (int r = 0; r < ITEMS_PER_THREAD; r++) {
    if (dig[r] < 256) {
      const u32 lp = tl[dig[r]] + wcnt[warp][dig[r]] + rank[r];
      skey[lp] = key[r];
      sval[lp] = val[r];
      sdig[lp] = (unsigned char)dig[r];
    }
  }
  __syncthreads();
  const ll t0 = (ll)blockIdx.x * TILE;
  const int tn = (int)(n - t0 < TILE ? n - t0 : TILE);
  for (int t = threadIdx.x; t < tn; t += blockDim.x) {
    const u32 d = sdig[t];
    const u32 pos = dbase[d] + ((u32)t - tl[d]);
    kout[pos] = skey[t];
    vout[pos] = sval[t];
  }
}

int bits_for(ll nseg) {
  int b = 0;
  while (nseg > 1 && ((ll)1 << b) < nseg) b++;
  return b;
}

}  // namespace

void seg_sort_pairs(DBuf<u64> &keys, DBuf<int> &vals, ll n,
                    const int *seg_of_val, ll nseg, SortWs &ws) {
  if (n <= 1) return;
  cudaStream_t st = ctx().stream;
  int seg_bits = seg_of_val ? bits_for(nseg) : 0;
  int nseg_pass = (seg_bits + 7) / 8;
  int nkey = 8;
  int np = nkey + nseg_pass;
  int ntiles = (int)((n + TILE - 1) / TILE);
  ws.ktmp.ensure((size_t)n);
  ws.vtmp.ensure((size_t)n);
  ws.counts.ensure((size_t)256 * ntiles);
  ws.totals.ensure(256);
  ws.hist_all.ensure((size_t)MAX_PASSES * 256);
  CK(cudaMemsetAsync(ws.hist_all.p, 0, (size_t)np * 256 * sizeof(u32), st));
  int gblocks = (int)((n + 255) / 256);
  if (gblocks > 152 * 8) gblocks = 152 * 8;
  k_hist_all<<<gblocks, 256, 0, st>>>(keys.p, vals.p, n, seg_of_val, nkey,
                                       nseg_pass, ws.hist_all.p);
  CK_LAUNCH();
  std::vector<u32> h((size_t)np * 256);
  d2h(h.data(), ws.hist_all.p, h.size());
  sync();
  PassDesc passes[MAX_PASSES];
  int npasses = 0;
  for (int b = 0; b < np; b++) {
    bool trivial = false;
    for (int d = 0; d < 256; d++)
      if (h[(size_t)b * 256 + d] == (u32)n) trivial = true;
    if (trivial) continue;
    passes[npasses].is_seg = b >= nkey;
    passes[npasses].shift = b >= nkey ? 8 * (b - nkey) : 8 * b;
    npasses++;
  }
  ensure_smem_limit(k_scatter, (int)SCATTER_SMEM);  // staging exceeds the 48 KB default
  for (int q = 0; q < npasses; q++) {
    const PassDesc &pd = passes[q];
    k_tile_hist<<<ntiles, SORT_THREADS, 0, st>>>(keys.p, vals.p, n, seg_of_val,
                                                 pd.is_seg, pd.shift,
                                                 ws.counts.p, ntiles);
    CK_LAUNCH();
    k_tile_scan<<<256, 1024, 0, st>>>(ws.counts.p, ntiles, ws.totals.p);
    CK_LAUNCH();
    k_scatter<<<ntiles, SORT_THREADS, SCATTER_SMEM, st>>>(keys.p, vals.p, ws.ktmp.p,
                                               ws.vtmp.p, n, seg_of_val,
                                               pd.is_seg, pd.shift, ws.counts.p,
                                               ws.totals.p, ntiles);
    CK_LAUNCH();
    std::swap(keys.p, ws.ktmp.p);
    std::swap(keys.n, ws.ktmp.n);
    std::swap(vals.p, ws.vtmp.p);
    std::swap(vals.n, ws.vtmp.n);
  }
}

}  // namespace prsb
