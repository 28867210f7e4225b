// bisect.cu -- element centroids and the segmented RCB / RIB engine.
//
// Restates, for all groups of a recursion level at once:
//   rcb / rcb_level / rcb_local / get_axis_len   src/rcb.c:7-137
//   rib / rib_level / rib_local / get_rib_axis   src/rib.c:6-111
//   power_serial                                  src/fiedler.c:38-73
//   load_balance centroids                        src/parrsb.c:139-145
// A group of p virtual ranks is a segment [start, start+n) of the element
// order; each recursion step sorts every active segment stably along its
// axis (one segmented radix sort for the whole level) and splits it at the
// element count of its lower ceil(p/2) ranks.  Arithmetic that decides the
// order (centroid sums, RIB means, inertia sums, power iteration, projection
// keys) uses round-to-nearest intrinsics with no FMA, so keys are bit-equal
// to the CPU restatement's.  Group sums use the canonical 32-wide tile tree.
#include <float.h>

#include "bisect.cuh"

#include <type_traits>

namespace prsb {

namespace {

__global__ void k_centroids(const double *__restrict__ xyz, int nel, int nv,
                            int ndim, double *__restrict__ cent) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  double c[3] = {0.0, 0.0, 0.0};
  if (xyz) {
    const double *x = xyz + (ll)e * nv * ndim;
    for (int v = 0; v < nv; v++)
      for (int d = 0; d < ndim; d++) c[d] = __dadd_rn(c[d], x[v * ndim + d]);
    for (int d = 0; d < ndim; d++) c[d] = __ddiv_rn(c[d], (double)nv);
  }
  cent[e] = c[0];
  cent[(ll)nel + e] = c[1];
  cent[2 * (ll)nel + e] = c[2];
}

enum Gen { GEN_MEAN = 1, GEN_INERTIA = 2, GEN_ARRAY = 3 };

// Segment "active" rule shared by all kernels.
__device__ __forceinline__ bool seg_active(int p, ll n, int do_local) {
  return p > 1 || (do_local && p == 1 && n >= 2);
}

__device__ __forceinline__ ll find_seg(const ll *off, ll nseg, ll w) {
  ll lo = 0, hi = nseg - 1;  // last s with off[s] <= w
  while (lo < hi) {
    ll mid = (lo + hi + 1) >> 1;
    if (off[mid] <= w)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// One warp per 32-item tile of a segment.  Level 0 generates values from
// elements; later levels reduce the previous level's tile values.
// Values are sums (canonical shuffle tree).
template <int V, int GEN>
__global__ void k_seg_tree(const int *__restrict__ perm,
                           const double *__restrict__ cent, ll N,
                           const ll *__restrict__ seg_start,
                           const ll *__restrict__ seg_cnt,  // items per segment
                           ll nseg, const ll *__restrict__ tile_off,
                           ll ntiles, const double *__restrict__ in,
                           const ll *__restrict__ in_off,
                           const double *__restrict__ avg,
                           double *__restrict__ out) {
  ll w = ((ll)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (w >= ntiles) return;
  ll s = find_seg(tile_off, nseg, w);
  ll t = w - tile_off[s];
  ll m = seg_cnt[s];
  ll i = t * 32 + lane;
  bool valid = i < m;
  double v[V];
#pragma unroll
  for (int q = 0; q < V; q++) v[q] = 0.0;
  if (valid) {
    if (GEN == GEN_ARRAY) {
      ll src = (in_off[s] + i) * V;
#pragma unroll
      for (int q = 0; q < V; q++) v[q] = in[src + q];
    } else {
      int e = perm[seg_start[s] + i];
      double c0 = cent[e], c1 = cent[N + e], c2 = cent[2 * N + e];
      if (GEN == GEN_MEAN) {
        v[0] = c0, v[1] = c1;
        if (V > 2) v[V - 1] = c2;
      } else {  // inertia products (00, 01, 02, 11, 12, 22)
        const double *a = avg + 3 * s;
        double x = __dsub_rn(c0, a[0]), y = __dsub_rn(c1, a[1]),
               z = __dsub_rn(c2, a[2]);
        v[0] = __dmul_rn(x, x);
        v[1] = __dmul_rn(x, y);
        if (V > 2) {
          v[2] = __dmul_rn(x, z);
          v[3] = __dmul_rn(y, y);
          v[4] = __dmul_rn(y, z);
          v[5] = __dmul_rn(z, z);
        }
      }
    }
  }
  // A segment whose previous level already produced a single value is
  // copied, not reduced again (the canonical tree stops at one value).
  bool copy_only = (GEN == GEN_ARRAY) && m == 1;
#pragma unroll
  for (int q = 0; q < V; q++) {
    double r;
    if (copy_only)
      r = v[q];
    else
      r = warp_tree_sum(v[q]);
    if (lane == 0) out[w * V + q] = r;
  }
}

__global__ void k_tile_counts(const ll *__restrict__ cnt, ll nseg,
                              ll *__restrict__ tiles) {
  ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nseg) tiles[s] = (cnt[s] + 31) / 32;
}

// RCB boxes on the dense coordinate ranks: per segment and axis the minimum
// rank (slots 0..2) and the minimum complemented rank (slots 3..5, i.e. the
// maximum).  Integer atomics are order-independent, so the box does not
// depend on the grid; uniq[rank] turns a rank back into the exact coordinate.
// A thread reduces RBOX_ITEMS consecutive positions, a warp and then the
// block combine when they cover one segment (the common case), and only the
// threads that straddle a segment boundary issue their own atomics.
constexpr int RBOX_THREADS = 256, RBOX_ITEMS = 16;

__device__ __forceinline__ void rbox_flush(u32 *rbox, int s, int ndim, const u32 *v) {
  for (int a = 0; a < ndim; a++) {
    atomicMin(&rbox[6 * (ll)s + a], v[a]);
    atomicMin(&rbox[6 * (ll)s + 3 + a], v[3 + a]);
  }
}

__global__ void __launch_bounds__(RBOX_THREADS)
k_rank_box(const int *__restrict__ perm, const u32 *__restrict__ rank, ll N, int ndim,
           const int *__restrict__ seg_of_pos, u32 *__restrict__ rbox) {
  constexpr int NWB = RBOX_THREADS / 32;
  __shared__ int wseg[NWB];
  __shared__ u32 wval[NWB][6];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const ll i0 = ((ll)blockIdx.x * RBOX_THREADS + threadIdx.x) * RBOX_ITEMS;
  int sg[RBOX_ITEMS], el[RBOX_ITEMS];
#pragma unroll
  for (int r = 0; r < RBOX_ITEMS; r++) {
    const bool ok = i0 + r < N;
    sg[r] = ok ? seg_of_pos[i0 + r] : -1;
    el[r] = ok ? perm[i0 + r] : 0;
  }
  u32 rk[3][RBOX_ITEMS];
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int r = 0; r < RBOX_ITEMS; r++)
      rk[a][r] = (a < ndim && sg[r] >= 0) ? rank[(ll)a * N + el[r]] : 0u;
  int s = -1;
  u32 v[6];
#pragma unroll
  for (int q = 0; q < 6; q++) v[q] = ~0u;
#pragma unroll
  for (int r = 0; r < RBOX_ITEMS; r++) {
    if (sg[r] < 0) continue;
    if (sg[r] != s) {  // a segment boundary inside this thread's run
      if (s >= 0) rbox_flush(rbox, s, ndim, v);
#pragma unroll
      for (int q = 0; q < 6; q++) v[q] = ~0u;
      s = sg[r];
    }
#pragma unroll
    for (int a = 0; a < 3; a++) {
      v[a] = min(v[a], rk[a][r]);
      v[3 + a] = min(v[3 + a], ~rk[a][r]);
    }
  }
  // warp: one segment among the lanes that hold one -> shuffle-free reduce
  const int smin = (int)__reduce_min_sync(0xffffffffu, (unsigned)(s >= 0 ? s : 0x7fffffff));
  const int smax = (int)__reduce_max_sync(0xffffffffu, (unsigned)(s + 1)) - 1;
  if (smax >= 0 && smin == smax) {
#pragma unroll
    for (int q = 0; q < 6; q++) v[q] = __reduce_min_sync(0xffffffffu, v[q]);
    if (lane == 0) {
      wseg[warp] = smax;
#pragma unroll
      for (int q = 0; q < 6; q++) wval[warp][q] = v[q];
    }
  } else {
    if (s >= 0) rbox_flush(rbox, s, ndim, v);
    if (lane == 0) wseg[warp] = -1;
  }
  __syncthreads();
  if (warp == 0) {
    const int ws = lane < NWB ? wseg[lane] : -1;
    const int bmin = (int)__reduce_min_sync(0xffffffffu, (unsigned)(ws >= 0 ? ws : 0x7fffffff));
    const int bmax = (int)__reduce_max_sync(0xffffffffu, (unsigned)(ws + 1)) - 1;
    u32 bv[6];
#pragma unroll
    for (int q = 0; q < 6; q++) bv[q] = ws >= 0 ? wval[lane < NWB ? lane : 0][q] : ~0u;
    if (bmax >= 0 && bmin == bmax) {
#pragma unroll
      for (int q = 0; q < 6; q++) bv[q] = __reduce_min_sync(0xffffffffu, bv[q]);
      if (lane == 0) rbox_flush(rbox, bmax, ndim, bv);
    } else if (ws >= 0) {
      rbox_flush(rbox, ws, ndim, bv);
    }
  }
}

// Longest box edge per segment from the rank boxes (strictly longer wins, so
// ties keep the lower axis, as with coordinate boxes).
__global__ void k_rcb_axis_rank(const u32 *__restrict__ rbox, const double *__restrict__ uniq,
                                ll N, const int *__restrict__ p, const ll *__restrict__ n,
                                ll nseg, int ndim, int do_local, int *__restrict__ axis) {
  ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  double len[3] = {0.0, 0.0, 0.0};
  if (n[s] > 0)
    for (int d = 0; d < ndim; d++) {
      const u32 lo = rbox[6 * s + d], hi = ~rbox[6 * s + 3 + d];
      len[d] = __dsub_rn(uniq[(ll)d * N + hi], uniq[(ll)d * N + lo]);
    }
  int ax = 0;
  for (int d = 1; d < ndim; d++)
    if (len[d] > len[ax]) ax = d;
  axis[s] = seg_active(p[s], n[s], do_local) ? ax : -1;
}

// Power iteration (fixed start vector (31, 17, 43)/50) on the first N*N
// entries of the row-major 3x3 tensor, as power_serial reads it.
__device__ void power_serial_dev(double *y, int N, const double *A) {
  const double start[3] = {31.0 / 50.0, 17.0 / 50.0, 43.0 / 50.0};
  double norm = 0.0;
  for (int i = 0; i < N; i++) {
    y[i] = start[i];
    norm = __dadd_rn(norm, __dmul_rn(y[i], y[i]));
  }
  double normi = __ddiv_rn(1.0, __dsqrt_rn(norm));
  for (int i = 0; i < N; i++) y[i] = __dmul_rn(y[i], normi);
  double Ay[3];
  double err = 1.0, lambda = 0.0;
  for (int i = 0; i < 100; i++) {
    norm = 0.0;
    for (int j = 0; j < N; j++) {
      Ay[j] = 0.0;
      for (int k = 0; k < N; k++) Ay[j] = __dadd_rn(Ay[j], __dmul_rn(A[j * N + k], y[k]));
      norm = __dadd_rn(norm, __dmul_rn(Ay[j], Ay[j]));
    }
    double sn = __dsqrt_rn(norm);
    if (i > 0) err = __ddiv_rn(__dsub_rn(sn, lambda), lambda);
    lambda = sn;
    normi = __ddiv_rn(1.0, sn);
    for (int j = 0; j < N; j++) y[j] = __dmul_rn(Ay[j], normi);
    if (fabs(err) < 1e-12) break;
  }
}

// RIB axis per segment.  Group segments (p > 1) use the tree sums in
// sums/isums; rank-local segments (p == 1) sum sequentially over their
// elements in order, as get_rib_axis does with c == NULL.
__global__ void k_rib_mean_local(const int *__restrict__ perm,
                                 const double *__restrict__ cent, ll N,
                                 const ll *__restrict__ seg_start,
                                 const ll *__restrict__ seg_n,
                                 const int *__restrict__ p, ll nseg,
                                 int do_local, double *__restrict__ avg) {
  ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  if (!(do_local && p[s] == 1 && seg_n[s] >= 2)) return;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  ll st = seg_start[s], n = seg_n[s];
  for (ll i = 0; i < n; i++) {
    int e = perm[st + i];
    a0 = __dadd_rn(a0, cent[e]);
    a1 = __dadd_rn(a1, cent[N + e]);
    a2 = __dadd_rn(a2, cent[2 * N + e]);
  }
  double dn = (double)n;
  avg[3 * s + 0] = __ddiv_rn(a0, dn);
  avg[3 * s + 1] = __ddiv_rn(a1, dn);
  avg[3 * s + 2] = __ddiv_rn(a2, dn);
}

__global__ void k_rib_mean_group(const double *__restrict__ sums,
                                 const ll *__restrict__ seg_n,
                                 const int *__restrict__ p, ll nseg,
                                 double *__restrict__ avg) {
  ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg || p[s] <= 1) return;
  double dn = (double)seg_n[s];
  for (int d = 0; d < 3; d++) avg[3 * s + d] = __ddiv_rn(sums[3 * s + d], dn);
}

__global__ void k_rib_axis(const int *__restrict__ perm,
                           const double *__restrict__ cent, ll N,
                           const ll *__restrict__ seg_start,
                           const ll *__restrict__ seg_n,
                           const int *__restrict__ p, ll nseg, int ndim,
                           int do_local, const double *__restrict__ avg,
                           const double *__restrict__ isums,
                           double *__restrict__ ev, int *__restrict__ act) {
  ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  int active = seg_active(p[s], seg_n[s], do_local);
  act[s] = active;
  if (!active) return;
  double I6[6];
  if (p[s] > 1) {
    for (int q = 0; q < 6; q++) I6[q] = isums[6 * s + q];
  } else {
    for (int q = 0; q < 6; q++) I6[q] = 0.0;
    const double *a = avg + 3 * s;
    ll st = seg_start[s], n = seg_n[s];
    for (ll i = 0; i < n; i++) {
      int e = perm[st + i];
      double x = __dsub_rn(cent[e], a[0]), y = __dsub_rn(cent[N + e], a[1]),
             z = __dsub_rn(cent[2 * N + e], a[2]);
      I6[0] = __dadd_rn(I6[0], __dmul_rn(x, x));
      I6[1] = __dadd_rn(I6[1], __dmul_rn(x, y));
      I6[2] = __dadd_rn(I6[2], __dmul_rn(x, z));
      I6[3] = __dadd_rn(I6[3], __dmul_rn(y, y));
      I6[4] = __dadd_rn(I6[4], __dmul_rn(y, z));
      I6[5] = __dadd_rn(I6[5], __dmul_rn(z, z));
    }
  }
  double I[9] = {I6[0], I6[1], I6[2], I6[1], I6[3], I6[4], I6[2], I6[4], I6[5]};
  double y[3] = {0.0, 0.0, 0.0};
  power_serial_dev(y, ndim, I);
  ev[3 * s + 0] = y[0];
  ev[3 * s + 1] = y[1];
  ev[3 * s + 2] = ndim == 3 ? y[2] : 0.0;
}

template <int KIND>
__global__ void k_keys(const int *__restrict__ perm, const double *__restrict__ cent,
                       const u32 *__restrict__ rank, ll N, const int *__restrict__ seg_of_pos,
                       const int *__restrict__ axis_or_act,
                       const double *__restrict__ avg,
                       const double *__restrict__ ev, u64 *__restrict__ keys,
                       int *__restrict__ vals, int *__restrict__ seg_of_elem) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int s = seg_of_pos[i];
  int e = perm[i];
  u64 k = 0;
  if (KIND == BISECT_RCB) {  // segment id above the dense rank of the coordinate
    int ax = axis_or_act[s];
    k = (u64)(unsigned)s << 32;
    if (ax >= 0) k |= rank[(ll)ax * N + e];
  } else {
    if (axis_or_act[s]) {
      const double *a = avg + 3 * s, *v = ev + 3 * s;
      double x = __dsub_rn(cent[e], a[0]), y = __dsub_rn(cent[N + e], a[1]),
             z = __dsub_rn(cent[2 * N + e], a[2]);
      double key = __dadd_rn(__dadd_rn(__dmul_rn(x, v[0]), __dmul_rn(y, v[1])),
                             __dmul_rn(z, v[2]));
      k = ordered_key(key);
    }
  }
  keys[i] = k;
  vals[i] = e;
  if (KIND != BISECT_RCB) seg_of_elem[e] = s;
}

__global__ void k_child_counts(const int *__restrict__ p, const ll *__restrict__ n,
                               ll nseg, int do_local, int *__restrict__ cnt,
                               int *__restrict__ nactive) {
  ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  int a = seg_active(p[s], n[s], do_local);
  cnt[s] = a ? 2 : 1;
  if (a) atomicAdd(nactive, 1);
}

__global__ void k_children(const ll *__restrict__ st, const ll *__restrict__ n,
                           const int *__restrict__ p, const int *__restrict__ r0,
                           ll nseg, int do_local, const ll *__restrict__ off,
                           ll *__restrict__ st2, ll *__restrict__ n2,
                           int *__restrict__ p2, int *__restrict__ r02) {
  ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  ll o = off[s];
  if (!seg_active(p[s], n[s], do_local)) {
    st2[o] = st[s], n2[o] = n[s], p2[o] = p[s], r02[o] = r0[s];
    return;
  }
  ll L;
  int h, pl, pr;
  if (p[s] > 1) {
    L = lower_count(n[s], p[s]);
    h = (p[s] + 1) / 2;
    pl = h, pr = p[s] - h;
  } else {
    L = n[s] / 2;
    h = 0;
    pl = 1, pr = 1;
  }
  st2[o] = st[s], n2[o] = L, p2[o] = pl, r02[o] = r0[s];
  st2[o + 1] = st[s] + L, n2[o + 1] = n[s] - L, p2[o + 1] = pr, r02[o + 1] = r0[s] + h;
}

__global__ void k_part_from_segs(const int *__restrict__ perm,
                                 const int *__restrict__ seg_of_pos,
                                 const int *__restrict__ r0, ll N,
                                 int *__restrict__ part) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) part[perm[i]] = r0[seg_of_pos[i]];
}

// ---------------------------------------------------------------------------
// Dense coordinate ranks.  RCB only ever compares centroid coordinates along
// one axis and takes min / max for the bounding boxes, so every coordinate
// can be replaced by its dense rank among all centroids on that axis (equal
// values -> equal rank): stable sorts by rank give the same order as stable
// sorts by value, and a box edge is uniq[max rank] - uniq[min rank], the same
// difference of the same two doubles.  Ranks are 32-bit keys (fewer radix
// passes than 64-bit ordered doubles) and are computed once per call.
// ---------------------------------------------------------------------------
__global__ void k_axis_keys(const double *__restrict__ cent, ll N, int a,
                            u64 *__restrict__ keys, int *__restrict__ vals) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  keys[i] = ordered_key(cent[(ll)a * N + i]);
  vals[i] = (int)i;
}

__global__ void k_rank_flags(const u64 *__restrict__ keys, ll N, int *__restrict__ flag) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) flag[i] = (i > 0 && keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void k_rank_write(const u64 *__restrict__ keys, const int *__restrict__ vals,
                             const int *__restrict__ flag, const ll *__restrict__ excl, ll N,
                             u32 *__restrict__ rank, double *__restrict__ uniq) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  ll r = excl[i] + flag[i];
  rank[vals[i]] = (u32)r;
  if (i == 0 || flag[i]) {
    u64 k = keys[i];
    u64 bits = (k >> 63) ? (k ^ 0x8000000000000000ull) : ~k;
    uniq[r] = __longlong_as_double((long long)bits);
  }
}

// ---------------------------------------------------------------------------
// Whole-recursion RCB of one small segment per CTA (n <= SMALL_MAX).
// Every recursion level of the segment runs inside the CTA: the sub-range of
// position x at depth d follows from (n, p) alone (rank split at
// lower_count(len, p) while p > 1, then, with LOCAL, halving at len / 2 as
// rcb_local does, src/rcb.c:39-72).  The dense ranks of the segment's
// elements sit in shared memory for the whole recursion; a thread keeps the
// sub-range of each of its positions in registers and advances it by one
// split per level.  Per level:
//   boxes   - a warp-segmented min / max over every round of 32 positions;
//             a sub-range inside one round takes its axis at once, a long one
//             (more than SMALL_SHORT) goes through shared-memory atomics
//             (table slot start / SMALL_SHORT: long sub-ranges are disjoint
//             and longer than SMALL_SHORT, so their slots differ), and a
//             short one crossing a round boundary is reduced sequentially;
//   axis    - longest edge, uniq[max] - uniq[min] per axis;
//   order   - stable sort of each sub-range by its axis rank.  When no
//             sub-range exceeds SMALL_CMP elements, an element's new place
//             is the number of elements of its sub-range before it in
//             (rank, position) order; otherwise an LSD radix in shared memory
//             over the varying bytes of the rank, then of the sub-range start
//             (warp w ranks positions [SMALL_SPAN w, SMALL_SPAN (w + 1)) in order with
//             __match_any_sync).
// Gives exactly the order of the level-by-level global path.
// ---------------------------------------------------------------------------
constexpr int SMALL_MAX = 8192;
constexpr int SMALL_THREADS = 1024;
constexpr int SMALL_WARPS = SMALL_THREADS / 32;
constexpr int SMALL_ITEMS = SMALL_MAX / SMALL_THREADS;  // positions per thread
constexpr int SMALL_SPAN = 32 * SMALL_ITEMS;            // positions per warp
constexpr int SMALL_CMP = 64;     // comparison ranking up to this sub-range length
constexpr int SMALL_SHORT = 32;   // sequential boxes up to this sub-range length
constexpr int SMALL_NLONG = SMALL_MAX / SMALL_SHORT;  // box table slots

struct SubR {
  int st, len, p, rank;
};

template <bool LOCAL>
__device__ __forceinline__ SubR descend(int x, int n, int p0, int d) {
  SubR r{0, n, p0, 0};
  for (int k = 0; k < d; k++) {
    int L, h;
    if (r.p > 1) {
      L = (int)lower_count(r.len, r.p);
      h = (r.p + 1) / 2;
    } else if (LOCAL && r.len >= 2) {
      L = r.len / 2;
      h = 0;
    } else {
      continue;  // finished sub-range keeps its place
    }
    if (x < r.st + L) {
      r.len = L;
      r.p = r.p > 1 ? h : r.p;
    } else {
      r.st += L;
      r.len -= L;
      r.rank += h;
      r.p = r.p > 1 ? r.p - h : r.p;
    }
  }
  return r;
}

template <bool LOCAL>
__device__ __forceinline__ bool sub_active(const SubR &r) {
  return r.p > 1 || (LOCAL && r.len >= 2);
}

// lower_count for the small segments (n <= SMALL_MAX): 32-bit arithmetic
__device__ __forceinline__ int lower_count_small(int n, int p) {
  const int h = (p + 1) / 2;
  const int nelt = n / p, nrem = n - p * nelt;
  if (nrem == 0) return h * nelt;
  const int s = p - nrem;
  return h * nelt + (h > s ? h - s : 0);
}

// Longest box edge from rank boxes: uniq[max] - uniq[min] per axis, the
// first strictly longest wins.
__device__ __forceinline__ unsigned char small_axis(const double *__restrict__ uniq, ll N,
                                                    int ndim, const u32 *mn, const u32 *mx) {
  double l[3];
#pragma unroll
  for (int q = 0; q < 3; q++)
    l[q] = q < ndim ? __dsub_rn(uniq[(ll)q * N + mx[q]], uniq[(ll)q * N + mn[q]]) : 0.0;
  int ax = 0;
#pragma unroll
  for (int q = 1; q < 3; q++)
    if (q < ndim && l[q] > l[ax]) ax = q;
  return (unsigned char)ax;
}

// Items of k_rcb_small: local id in bits 0-15, sub-range start in bits
// 16-30, bit 31 set while the sub-range is active.
constexpr u32 ITEM_ACTIVE = 0x80000000u;
__device__ __forceinline__ u32 item_st(u32 it) { return (it >> 16) & 0x7FFFu; }
// axis rank of an item; 0 for inactive sub-ranges (their axis slot is unset)
__device__ __forceinline__ u32 kx_key(const u32 *rk, const unsigned char *sax, u32 it) {
  return (it & ITEM_ACTIVE) ? rk[sax[item_st(it)] * SMALL_MAX + (it & 0xFFFFu)] : 0u;
}

// shared memory of k_rcb_small
constexpr size_t small_smem_bytes() {
  return (size_t)SMALL_MAX * (3 * 4 /*rk*/ + 4 + 4 /*item, item2*/ + 4 /*kx*/ + 1 /*sax*/) +
         (size_t)SMALL_WARPS * 256 * 2 /*wcnt*/ + (size_t)SMALL_NLONG * 6 * 4 /*box*/;
}

template <bool LOCAL>
__global__ void __launch_bounds__(SMALL_THREADS)
k_rcb_small(int *__restrict__ perm, const u32 *__restrict__ rank,
            const double *__restrict__ uniq, ll N, int ndim,
            const ll *__restrict__ seg_start, const ll *__restrict__ seg_n,
            const int *__restrict__ seg_p, const int *__restrict__ seg_r0,
            int *__restrict__ part) {
  extern __shared__ u32 smem_u32[];
  u32 *rk = smem_u32;                  // [3][SMALL_MAX] dense ranks by local id
  u32 *item = rk + 3 * SMALL_MAX;      // (sub-range start << 16) | local id
  u32 *item2 = item + SMALL_MAX;
  u32 *kx = item2 + SMALL_MAX;         // axis rank per position
  u32 *box = kx + SMALL_MAX;           // [SMALL_NLONG][6] min0..2, max0..2
  unsigned short *wcnt = (unsigned short *)(box + SMALL_NLONG * 6);  // [SMALL_WARPS][256]
  unsigned char *sax = (unsigned char *)(wcnt + SMALL_WARPS * 256);  // axis by sub-range start
  __shared__ unsigned dbase[256];
  __shared__ u32 s_and, s_or, s_stand, s_stor;
  __shared__ int s_maxlen;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const ll sg = blockIdx.x;
  const ll start = seg_start[sg];
  const int n = (int)seg_n[sg], p0 = seg_p[sg], r0 = seg_r0[sg];
  bool seg_act = p0 > 1 || (LOCAL && p0 == 1 && n >= 2);
  if (n <= 0 || p0 <= 0) return;
  if (!seg_act || n > SMALL_MAX) {
    if (part && n <= SMALL_MAX && p0 == 1)
      for (int x = threadIdx.x; x < n; x += blockDim.x) part[perm[start + x]] = r0;
    return;
  }
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    const int e = perm[start + x];
    for (int q = 0; q < ndim; q++) rk[q * SMALL_MAX + x] = rank[(ll)q * N + e];
    item[x] = (u32)x;
  }
  // The level loop, instantiated for segments with one virtual rank (only
  // the local halving, no per-position rank counts) and for the general case.
  auto levels = [&](auto pone) {
    constexpr bool PONE = decltype(pone)::value;
    const unsigned lt_mask = (1u << lane) - 1u;
    // Sub-range of each own position at the current depth, advanced by one
    // split per level: start | length << 16, and its virtual-rank count.
    u32 sl_r[SMALL_ITEMS];
    int p_r[PONE ? 1 : SMALL_ITEMS];  // with one virtual rank (PONE) p stays 1
  #pragma unroll
    for (int r = 0; r < SMALL_ITEMS; r++) {
      sl_r[r] = (u32)n << 16;
      if (!PONE) p_r[r] = p0;
    }
    for (int d = 0; d < 64; d++) {
      if (d > 0) {
  #pragma unroll
        for (int r = 0; r < SMALL_ITEMS; r++) {
          const int x = warp * SMALL_SPAN + r * 32 + lane;
          int st = (int)(sl_r[r] & 0xFFFFu), ln = (int)(sl_r[r] >> 16), p = PONE ? 1 : p_r[r];
          int L, h;
          if (p > 1) {
            L = lower_count_small(ln, p);
            h = (p + 1) / 2;
          } else if (LOCAL && ln >= 2) {
            L = ln / 2;
            h = 0;
          } else {
            continue;  // finished sub-range keeps its place
          }
          if (x < st + L) {
            ln = L;
            p = p > 1 ? h : p;
          } else {
            st += L;
            ln -= L;
            p = p > 1 ? p - h : p;
          }
          sl_r[r] = (u32)st | ((u32)ln << 16);
          if (!PONE) p_r[r] = p;
        }
      }
      if (threadIdx.x == 0) s_maxlen = 0;
      for (int t = threadIdx.x; t < SMALL_NLONG * 6; t += blockDim.x)
        box[t] = (t % 6) < 3 ? 0xFFFFFFFFu : 0u;
      __syncthreads();
      u32 act_mask = 0;  // bit r: position r lies in an active sub-range
      int mylen = 0;
  #pragma unroll
      for (int r = 0; r < SMALL_ITEMS; r++) {
        const int x = warp * SMALL_SPAN + r * 32 + lane;
        const int ln = (int)(sl_r[r] >> 16);
        if (x < n && ((!PONE && p_r[r] > 1) || (LOCAL && ln >= 2)))
          act_mask |= 1u << r, mylen = max(mylen, ln);
      }
      if (mylen) atomicMax(&s_maxlen, mylen);
      if (!__syncthreads_or(act_mask != 0)) break;
      const int maxlen = s_maxlen;
      // ---- bounding boxes on dense ranks, axis of each sub-range.  A warp
      // whose 256 positions all lie in one active sub-range folds them per
      // lane and reduces once; other warps reduce each round of 32 positions
      // with a segmented shuffle tree.
      const int st0 = (int)(sl_r[0] & 0xFFFFu);
      bool one = act_mask == (1u << SMALL_ITEMS) - 1u;
#pragma unroll
      for (int r = 1; r < SMALL_ITEMS; r++) one = one && (int)(sl_r[r] & 0xFFFFu) == st0;
      const int st0_lane0 = __shfl_sync(0xffffffffu, st0, 0);  // every lane takes part
      const bool warp_one = __all_sync(0xffffffffu, one && st0 == st0_lane0);
      if (warp_one) {
        u32 mn[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, mx[3] = {0u, 0u, 0u};
#pragma unroll
        for (int r = 0; r < SMALL_ITEMS; r++) {
          const u32 id = item[warp * SMALL_SPAN + r * 32 + lane] & 0xFFFFu;
#pragma unroll
          for (int q = 0; q < 3; q++)
            if (q < ndim) {
              const u32 k = rk[q * SMALL_MAX + id];
              mn[q] = min(mn[q], k);
              mx[q] = max(mx[q], k);
            }
        }
#pragma unroll
        for (int q = 0; q < 3; q++) {
          mn[q] = __reduce_min_sync(0xffffffffu, mn[q]);
          mx[q] = __reduce_max_sync(0xffffffffu, mx[q]);
        }
        const int ln0 = (int)(sl_r[0] >> 16);
        if (lane == 0) {
          if (st0 == warp * SMALL_SPAN && ln0 == SMALL_SPAN) {
            sax[st0] = small_axis(uniq, N, ndim, mn, mx);  // the whole sub-range
          } else {  // longer than SMALL_SHORT: box table slot
            const int o = st0 / SMALL_SHORT;
#pragma unroll
            for (int q = 0; q < 3; q++)
              if (q < ndim) {
                atomicMin(&box[6 * o + q], mn[q]);
                atomicMax(&box[6 * o + 3 + q], mx[q]);
              }
          }
        }
      }
#pragma unroll
      for (int r = 0; r < SMALL_ITEMS; r++) {
        const bool act = (act_mask >> r) & 1u;
        if (warp_one || !__any_sync(0xffffffffu, act)) continue;  // warp-uniform
        const int x = warp * SMALL_SPAN + r * 32 + lane;
        const int st = (int)(sl_r[r] & 0xFFFFu), ln = (int)(sl_r[r] >> 16);
        const int segkey = act ? st : -1 - lane;
        u32 mn[3], mx[3];
        const u32 id = act ? (item[x] & 0xFFFFu) : 0u;
  #pragma unroll
        for (int q = 0; q < 3; q++) {
          const u32 k = (act && q < ndim) ? rk[q * SMALL_MAX + id] : 0u;
          mn[q] = act ? k : 0xFFFFFFFFu;
          mx[q] = k;
        }
  #pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
          const int ok = __shfl_down_sync(0xffffffffu, segkey, off);
          const bool same = (lane + off < 32) && ok == segkey;
  #pragma unroll
          for (int q = 0; q < 3; q++) {
            const u32 a2 = __shfl_down_sync(0xffffffffu, mn[q], off);
            const u32 b2 = __shfl_down_sync(0xffffffffu, mx[q], off);
            if (same) mn[q] = min(mn[q], a2), mx[q] = max(mx[q], b2);
          }
        }
        const int prevkey = __shfl_up_sync(0xffffffffu, segkey, 1);
        if (act && (lane == 0 || prevkey != segkey)) {  // first position of a run
          const int rend = warp * SMALL_SPAN + r * 32 + 32;
          if (x == st && st + ln <= rend) {
            sax[st] = small_axis(uniq, N, ndim, mn, mx);  // whole sub-range in this round
          } else if (ln > SMALL_SHORT) {
            const int o = st / SMALL_SHORT;
  #pragma unroll
            for (int q = 0; q < 3; q++)
              if (q < ndim) {
                atomicMin(&box[6 * o + q], mn[q]);
                atomicMax(&box[6 * o + 3 + q], mx[q]);
              }
          }
        }
      }
      __syncthreads();
      // sub-ranges spanning more than one round: long ones from the box table,
      // short ones (crossing a round boundary) by a sequential loop
  #pragma unroll
      for (int r = 0; r < SMALL_ITEMS; r++) {
        const int x = warp * SMALL_SPAN + r * 32 + lane;
        const int st = (int)(sl_r[r] & 0xFFFFu), ln = (int)(sl_r[r] >> 16);
        const int rend = warp * SMALL_SPAN + r * 32 + 32;
        const bool whole_warp = st == warp * SMALL_SPAN && ln == SMALL_SPAN;
        if (((act_mask >> r) & 1u) && x == st && st + ln > rend && !(warp_one && whole_warp)) {
          u32 mn[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu}, mx[3] = {0u, 0u, 0u};
          if (ln > SMALL_SHORT) {
            const int o = st / SMALL_SHORT;
  #pragma unroll
            for (int q = 0; q < 3; q++) mn[q] = box[6 * o + q], mx[q] = box[6 * o + 3 + q];
          } else {
            for (int y = st; y < st + ln; y++) {
              const u32 id = item[y] & 0xFFFFu;
  #pragma unroll
              for (int q = 0; q < 3; q++)
                if (q < ndim) {
                  const u32 k = rk[q * SMALL_MAX + id];
                  mn[q] = min(mn[q], k);
                  mx[q] = max(mx[q], k);
                }
            }
          }
          sax[st] = small_axis(uniq, N, ndim, mn, mx);
        }
      }
      __syncthreads();
      // ---- keys: rank along the sub-range's axis
      u32 kand = 0xFFFFFFFFu, kor = 0u, stand = 0xFFFFFFFFu, stor = 0u;
  #pragma unroll
      for (int r = 0; r < SMALL_ITEMS; r++) {
        const int x = warp * SMALL_SPAN + r * 32 + lane;
        if (x >= n) continue;
        const u32 st = sl_r[r] & 0xFFFFu;
        const bool act = (act_mask >> r) & 1u;
        const u32 id = item[x] & 0xFFFFu;
        const u32 k = act ? rk[sax[st] * SMALL_MAX + id] : 0u;
        kx[x] = k;
        item[x] = (st << 16) | id | (act ? ITEM_ACTIVE : 0u);
        kand &= k, kor |= k, stand &= st, stor |= st;
      }
      __syncthreads();
      if (maxlen <= SMALL_CMP) {
        // ---- comparison ranking inside each sub-range
  #pragma unroll
        for (int r = 0; r < SMALL_ITEMS; r++) {
          const int x = warp * SMALL_SPAN + r * 32 + lane;
          if (x >= n) continue;
          const int len = ((act_mask >> r) & 1u) ? (int)(sl_r[r] >> 16) : 0;
          const int st = (int)(sl_r[r] & 0xFFFFu);
          if (!len) {
            item2[x] = item[x];
            continue;
          }
          const u32 k = kx[x];
          int c = 0;
          for (int y = st; y < st + len; y++) {
            const u32 k2 = kx[y];
            c += (k2 < k) || (k2 == k && y < x);
          }
          item2[st + c] = item[x];
        }
        __syncthreads();
        u32 *t = item;
        item = item2;
        item2 = t;
      } else {
        // ---- stable LSD passes over the varying bytes: rank, then start
        if (threadIdx.x == 0) s_and = 0xFFFFFFFFu, s_or = 0u, s_stand = 0xFFFFFFFFu, s_stor = 0u;
        __syncthreads();
        atomicAnd(&s_and, kand);
        atomicOr(&s_or, kor);
        atomicAnd(&s_stand, stand);
        atomicOr(&s_stor, stor);
        __syncthreads();
        const u32 kdiff = s_and ^ s_or, sdiff = s_stand ^ s_stor;
        for (int b = 0; b < 6; b++) {
          const bool is_st = b >= 4;
          const int shift = is_st ? 8 * (b - 4) : 8 * b;
          if ((((is_st ? sdiff : kdiff) >> shift) & 255u) == 0) continue;
          for (int i = threadIdx.x; i < SMALL_WARPS * 256; i += blockDim.x) wcnt[i] = 0;
          __syncthreads();
          unsigned rd[SMALL_ITEMS];  // digit << 16 | rank among the warp's equal digits
          u32 itv[SMALL_ITEMS];
  #pragma unroll
          for (int r = 0; r < SMALL_ITEMS; r++) {
            const int x = warp * SMALL_SPAN + r * 32 + lane;
            unsigned dgt = 256;
            itv[r] = 0;
            if (x < n) {
              const u32 it = item[x];
              itv[r] = it;
              // inactive positions carry key 0 (their sub-range keeps its order)
              const u32 k = is_st ? item_st(it) : kx_key(rk, sax, it);
              dgt = (k >> shift) & 255u;
            }
            unsigned peers = __match_any_sync(0xffffffffu, dgt);
            unsigned before = 0;
            if (dgt < 256) before = wcnt[warp * 256 + dgt];
            __syncwarp();
            if (dgt < 256) {
              rd[r] = (dgt << 16) | (before + __popc(peers & lt_mask));
              if (lane == __ffs(peers) - 1)
                wcnt[warp * 256 + dgt] = (unsigned short)(before + __popc(peers));
            }
            if (dgt >= 256) rd[r] = 256u << 16;
            __syncwarp();
          }
          __syncthreads();
          if (threadIdx.x < 256) {
            unsigned run = 0;
            for (int w = 0; w < SMALL_WARPS; w++) {
              unsigned t = wcnt[w * 256 + threadIdx.x];
              wcnt[w * 256 + threadIdx.x] = (unsigned short)run;
              run += t;
            }
            dbase[threadIdx.x] = run;
          }
          __syncthreads();
          if (threadIdx.x < 32) {  // exclusive scan of the 256 digit totals
            unsigned v[8], s2 = 0;
            for (int j = 0; j < 8; j++) v[j] = dbase[threadIdx.x * 8 + j], s2 += v[j];
            unsigned incl = s2;
            for (int o = 1; o < 32; o <<= 1) {
              unsigned y = __shfl_up_sync(0xffffffffu, incl, o);
              if (threadIdx.x >= o) incl += y;
            }
            unsigned run = incl - s2;
            for (int j = 0; j < 8; j++) dbase[threadIdx.x * 8 + j] = run, run += v[j];
          }
          __syncthreads();
  #pragma unroll
          for (int r = 0; r < SMALL_ITEMS; r++) {
            const unsigned dgr = rd[r] >> 16;
            if (dgr < 256) item2[dbase[dgr] + wcnt[warp * 256 + dgr] + (rd[r] & 0xFFFFu)] = itv[r];
          }
          __syncthreads();
          u32 *t = item;
          item = item2;
          item2 = t;
        }
      }
    }
    // ---- write the order (and ranks) back: read every old entry, then write
    int ev[SMALL_ITEMS];
  #pragma unroll
    for (int r = 0; r < SMALL_ITEMS; r++) {
      const int x = warp * SMALL_SPAN + r * 32 + lane;
      ev[r] = x < n ? perm[start + (item[x] & 0xFFFFu)] : 0;
    }
    __syncthreads();
  #pragma unroll
    for (int r = 0; r < SMALL_ITEMS; r++) {
      const int x = warp * SMALL_SPAN + r * 32 + lane;
      if (x < n) {
        perm[start + x] = ev[r];
        if (part) part[ev[r]] = r0 + descend<LOCAL>(x, n, p0, 64).rank;
      }
    }
  };
  if (p0 == 1)
    levels(std::true_type{});
  else
    levels(std::false_type{});
}

__global__ void k_max_active_n(const int *__restrict__ p, const ll *__restrict__ n, ll nseg,
                               int do_local, unsigned long long *__restrict__ mx) {
  ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s < nseg && seg_active(p[s], n[s], do_local)) atomicMax(mx, (unsigned long long)n[s]);
}

// Run the tile tree over every segment of `t` until one value per segment
// is left; result in out_final (nseg * V values).
template <int V, int GEN0>
void seg_tree_reduce(const int *perm, const double *cent, ll N, SegTable &t,
                     const double *avg, BisectWs &ws, double *out_final) {
  cudaStream_t st = ctx().stream;
  ll nseg = t.count;
  DBuf<ll> cnt((size_t)nseg), off((size_t)nseg + 1), in_off((size_t)nseg + 1);
  CK(cudaMemcpyAsync(cnt.p, t.n.p, nseg * sizeof(ll), cudaMemcpyDeviceToDevice, st));
  const double *in = nullptr;
  bool first = true;
  DBuf<double> *bufs[2] = {&ws.red_a, &ws.red_b};
  int cur = 0;
  for (int level = 0; level < 16; level++) {
    DBuf<ll> tiles((size_t)nseg);
    k_tile_counts<<<grid_for(nseg, 256), 256, 0, st>>>(cnt.p, nseg, tiles.p);
    CK_LAUNCH();
    ll ntiles = exclusive_scan_ll(tiles.p, off.p, nseg);
    DBuf<double> &ob = *bufs[cur];
    ob.ensure((size_t)ntiles * V);
    unsigned blocks = grid_for(ntiles * 32, 256);
    if (first)
      k_seg_tree<V, GEN0><<<blocks, 256, 0, st>>>(perm, cent, N, t.start.p,
                                                        cnt.p, nseg, off.p, ntiles,
                                                        nullptr, nullptr, avg, ob.p);
    else
      k_seg_tree<V, GEN_ARRAY><<<blocks, 256, 0, st>>>(
          perm, cent, N, t.start.p, cnt.p, nseg, off.p, ntiles, in, in_off.p, avg,
          ob.p);
    CK_LAUNCH();
    if (ntiles == nseg) {  // every segment has a single value
      CK(cudaMemcpyAsync(out_final, ob.p, (size_t)nseg * V * sizeof(double),
                         cudaMemcpyDeviceToDevice, st));
      return;
    }
    in = ob.p;
    CK(cudaMemcpyAsync(in_off.p, off.p, nseg * sizeof(ll), cudaMemcpyDeviceToDevice, st));
    CK(cudaMemcpyAsync(cnt.p, tiles.p, nseg * sizeof(ll), cudaMemcpyDeviceToDevice, st));
    first = false;
    cur ^= 1;
  }
  throw ArgError{PARRSB_ERR_CHECK, "tree reduction did not converge"};
}

}  // namespace

int rcb_small_max() { return SMALL_MAX; }

cudaError_t rcb_small_prepare() {
  cudaError_t e = cudaFuncSetAttribute(k_rcb_small<false>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)small_smem_bytes());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_rcb_small<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)small_smem_bytes());
}

cudaError_t rcb_small_launch(int *perm, const u32 *rank, const double *uniq, ll N, int ndim,
                             const ll *seg_start, const ll *seg_n, const int *seg_p,
                             const int *seg_r0, ll nseg, bool local, int *part,
                             cudaStream_t stream) {
  if (local)
    k_rcb_small<true><<<(unsigned)nseg, SMALL_THREADS, small_smem_bytes(), stream>>>(
        perm, rank, uniq, N, ndim, seg_start, seg_n, seg_p, seg_r0, part);
  else
    k_rcb_small<false><<<(unsigned)nseg, SMALL_THREADS, small_smem_bytes(), stream>>>(
        perm, rank, uniq, N, ndim, seg_start, seg_n, seg_p, seg_r0, part);
  return cudaGetLastError();
}

void compute_centroids(const double *xyz, int nel, int nv, double *cent) {
  int ndim = (nv == 8) ? 3 : 2;
  k_centroids<<<grid_for(nel, 256), 256, 0, ctx().stream>>>(xyz, nel, nv, ndim, cent);
  CK_LAUNCH();
}

// ---------------------------------------------------------------------------
// RCB on presorted coordinate lists, used when every axis rank is unique (no
// two centroids share a coordinate on any axis).  Then a stable sort of a
// segment by its axis rank does not depend on the segment's current order,
// so each level needs no sort: every segment keeps, per axis a, the list of
// its elements in increasing rank a (lists[a], in the segment's positions).
// Its box is the ranks of the first and last entry of each list; its cut
// sends the first `split` entries of the cut axis' list to the lower child;
// the other lists are partitioned stably by that side (a segmented prefix
// count, no comparison).  The tree, the cuts and the final order are those
// of the sort-per-level path (the order of a segment that is not cut again
// is its list along the axis of the cut that made it).  A level moves about
// 130 B per element instead of four or five radix passes.
// ---------------------------------------------------------------------------
constexpr int PS_THREADS = 1024, PS_ITEMS = 4, PS_TILE = PS_THREADS * PS_ITEMS;

// per segment: cut axis (-1: not cut at this level) and the lower child's size
__global__ void k_ps_axis(const int *__restrict__ lists, const u32 *__restrict__ rank,
                          const double *__restrict__ uniq, ll N, int ndim,
                          const ll *__restrict__ st, const ll *__restrict__ n,
                          const int *__restrict__ p, ll nseg, int do_local,
                          int *__restrict__ axis, ll *__restrict__ split) {
  const ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  if (!seg_active(p[s], n[s], do_local)) {
    axis[s] = -1;
    split[s] = n[s];
    return;
  }
  double len[3] = {0.0, 0.0, 0.0};
  if (n[s] > 0)
    for (int d = 0; d < ndim; d++) {
      const u32 lo = rank[(ll)d * N + lists[(ll)d * N + st[s]]];
      const u32 hi = rank[(ll)d * N + lists[(ll)d * N + st[s] + n[s] - 1]];
      len[d] = __dsub_rn(uniq[(ll)d * N + hi], uniq[(ll)d * N + lo]);
    }
  int ax = 0;
  for (int d = 1; d < ndim; d++)
    if (len[d] > len[ax]) ax = d;  // strictly longer wins: ties keep the lower axis
  axis[s] = ax;
  split[s] = p[s] > 1 ? lower_count(n[s], p[s]) : n[s] / 2;
}

// side of every element of a cut segment: 1 for the upper child
__global__ void k_ps_side(const int *__restrict__ lists, ll N, const int *__restrict__ seg_of_pos,
                          const ll *__restrict__ st, const int *__restrict__ axis,
                          const ll *__restrict__ split, unsigned char *__restrict__ side) {
  const ll j = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const int s = seg_of_pos[j];
  const int a = axis[s];
  if (a < 0) return;
  side[lists[(ll)a * N + j]] = (j - st[s]) >= split[s] ? 1 : 0;
}

__device__ __forceinline__ int ps_block_excl(int v, int *total) {
  __shared__ int ws[PS_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int t = lane < PS_THREADS / 32 ? ws[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < PS_THREADS / 32) ws[lane] = t;
  }
  __syncthreads();
  const int excl = (warp ? ws[warp - 1] : 0) + x - v;
  *total = ws[PS_THREADS / 32 - 1];
  __syncthreads();
  return excl;
}

// per tile of PS_TILE positions (PS_TILE / 32 words): the lower-child flags
// of every list as one bit per position (warp ballots; a position of a
// segment that is not cut gets 0), each word's count of lower flags before
// it inside the tile, and the tile's count
constexpr int PS_WORDS = PS_TILE / 32;
__global__ void __launch_bounds__(PS_THREADS)
k_ps_flags(const int *__restrict__ lists, ll N, int ndim, const int *__restrict__ seg_of_pos,
           const int *__restrict__ axis, const unsigned char *__restrict__ side,
           u32 *__restrict__ bits, int *__restrict__ wpre, int *__restrict__ bsum, int nblk) {
  __shared__ int wtot[3][PS_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const ll nw = (N + 31) >> 5;
  const ll w0 = (ll)blockIdx.x * PS_WORDS + (ll)warp * PS_ITEMS;  // this warp's first word
  bool cut[PS_ITEMS];
#pragma unroll
  for (int r = 0; r < PS_ITEMS; r++) {
    const ll j = (w0 + r) * 32 + lane;
    cut[r] = j < N && axis[seg_of_pos[j]] >= 0;
  }
  int pre[3][PS_ITEMS];
#pragma unroll
  for (int b = 0; b < 3; b++) {
    if (b >= ndim) break;
    int c = 0;
#pragma unroll
    for (int r = 0; r < PS_ITEMS; r++) {
      const ll j = (w0 + r) * 32 + lane;
      const bool f = cut[r] && side[lists[(ll)b * N + j]] == 0;
      const u32 bal = __ballot_sync(0xffffffffu, f);
      if (lane == 0 && w0 + r < nw) bits[(ll)b * nw + w0 + r] = bal;
      pre[b][r] = c;
      c += __popc(bal);
    }
    if (lane == 0) wtot[b][warp] = c;
  }
  __syncthreads();
#pragma unroll
  for (int b = 0; b < 3; b++) {
    if (b >= ndim) break;
    const int v = wtot[b][lane];  // PS_THREADS / 32 == 32
    int inc = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    const int base = __shfl_sync(0xffffffffu, inc - v, warp);
    if (lane < PS_ITEMS && w0 + lane < nw) {
      int pv = pre[b][0];
#pragma unroll
      for (int r = 1; r < PS_ITEMS; r++)
        if (lane == r) pv = pre[b][r];
      wpre[(ll)b * nw + w0 + lane] = base + pv;
    }
    const int total = __shfl_sync(0xffffffffu, inc, 31);
    if (threadIdx.x == 0) bsum[(ll)b * nblk + blockIdx.x] = total;
  }
}

// per list (blockIdx.x): exclusive scan of its tiles' counts, in place
__global__ void __launch_bounds__(PS_THREADS) k_ps_bscan(int *__restrict__ bsum, int nblk) {
  int *v = bsum + (ll)blockIdx.x * nblk;
  const int per = (nblk + PS_THREADS - 1) / PS_THREADS;
  const int i0 = threadIdx.x * per;
  int c = 0;
  for (int k = 0; k < per; k++)
    if (i0 + k < nblk) c += v[i0 + k];
  int total;
  int run = ps_block_excl(c, &total);
  for (int k = 0; k < per; k++)
    if (i0 + k < nblk) {
      const int x = v[i0 + k];
      v[i0 + k] = run;
      run += x;
    }
}

// lower flags of list b before position x: the tiles before it, the words
// before it in its tile, the bits below it in its word
__device__ __forceinline__ ll ps_before(const u32 *__restrict__ bits,
                                        const int *__restrict__ wpre,
                                        const int *__restrict__ bsum, ll x) {
  const ll w = x >> 5;
  return (ll)bsum[w / PS_WORDS] + wpre[w] + __popc(bits[w] & ((1u << (x & 31)) - 1u));
}

// stable partition of every cut segment of each list by side, and the
// segment of every position in the children's table (child_off: the first
// child of each segment, the lower one of a cut)
__global__ void k_ps_scatter(const int *__restrict__ lists, ll N, int ndim,
                             const int *__restrict__ seg_of_pos, const ll *__restrict__ st,
                             const int *__restrict__ axis, const ll *__restrict__ split,
                             const u32 *__restrict__ bits, const int *__restrict__ wpre,
                             const int *__restrict__ bsum, int nblk,
                             const ll *__restrict__ child_off, int *__restrict__ lists2,
                             int *__restrict__ seg_of_pos2) {
  const ll j = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const int s = seg_of_pos[j];
  const ll s0 = st[s];
  const bool cut = axis[s] >= 0;
  seg_of_pos2[j] = (int)(child_off[s] + ((cut && j - s0 >= split[s]) ? 1 : 0));
  const ll nw = (N + 31) >> 5;
  for (int b = 0; b < ndim; b++) {
    const int e = lists[(ll)b * N + j];
    ll dest = j;
    if (cut) {
      const u32 *bb = bits + (ll)b * nw;
      const int *wp = wpre + (ll)b * nw, *bs = bsum + (ll)b * nblk;
      const ll c = ps_before(bb, wp, bs, j) - ps_before(bb, wp, bs, s0);  // lower entries before j
      dest = ((bb[j >> 5] >> (j & 31)) & 1u) ? s0 + c : s0 + split[s] + (j - s0 - c);
    }
    lists2[(ll)b * N + dest] = e;
  }
}

// the axis whose list orders each child: the cut's axis, or the parent's
__global__ void k_ps_oaxis(const int *__restrict__ axis, const int *__restrict__ oax, ll nseg,
                           const ll *__restrict__ off, int *__restrict__ oax2) {
  const ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const ll o = off[s];
  if (axis[s] >= 0)
    oax2[o] = oax2[o + 1] = axis[s];
  else
    oax2[o] = oax[s];
}

__global__ void k_ps_seg_keys(const int *__restrict__ sorted, const int *__restrict__ seg_of_elem,
                              ll N, u64 *__restrict__ keys, int *__restrict__ vals) {
  const ll r = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= N) return;
  const int e = sorted[r];
  keys[r] = (u64)(unsigned)seg_of_elem[e];
  vals[r] = e;
}

__global__ void k_ps_seg_of_elem(const int *__restrict__ perm, const int *__restrict__ seg_of_pos,
                                 ll N, int *__restrict__ seg_of_elem) {
  const ll j = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < N) seg_of_elem[perm[j]] = seg_of_pos[j];
}

// The groups of RSB's next level are the halves of this level's (each old
// group becomes one or two consecutive new segments over its own positions),
// so the next call's lists are this call's group lists partitioned stably by
// half.  Per old group: its first child in the new table, whether it has two
// (axis 0, else -1) and the first child's size; `bad` is set when the new
// table does not refine the old one that way.
__global__ void k_inherit_tab(const ll *__restrict__ ost, const ll *__restrict__ on, ll ocount,
                              const ll *__restrict__ nst, const ll *__restrict__ nn,
                              const int *__restrict__ nseg_of_pos, int *__restrict__ axis,
                              ll *__restrict__ split, ll *__restrict__ child_off,
                              int *__restrict__ bad) {
  const ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= ocount) return;
  const ll s0 = ost[s], n = on[s];
  axis[s] = -1, split[s] = n, child_off[s] = 0;
  if (n <= 0) return;
  const int c0 = nseg_of_pos[s0], c1 = nseg_of_pos[s0 + n - 1];
  bool ok = nst[c0] == s0 && (c1 == c0 || c1 == c0 + 1) && nst[c1] + nn[c1] == s0 + n;
  if (c1 == c0 + 1) ok = ok && nst[c1] == s0 + nn[c0];
  if (!ok) atomicOr(bad, 1);
  axis[s] = c1 == c0 + 1 ? 0 : -1;
  split[s] = nn[c0];
  child_off[s] = c0;
}

// side of every element in its old group: 1 for the second child
__global__ void k_inherit_side(const int *__restrict__ perm, ll N,
                               const int *__restrict__ oseg_of_pos,
                               const int *__restrict__ nseg_of_pos,
                               const ll *__restrict__ child_off, unsigned char *__restrict__ side) {
  const ll j = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  side[perm[j]] = nseg_of_pos[j] != (int)child_off[oseg_of_pos[j]] ? 1 : 0;
}

__global__ void k_ps_final(const int *__restrict__ lists, ll N, const int *__restrict__ seg_of_pos,
                           const int *__restrict__ oax, int *__restrict__ perm) {
  const ll j = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const int a = oax[seg_of_pos[j]];
  if (a >= 0) perm[j] = lists[(ll)a * N + j];
}

// The remaining levels of every segment of at most SMALL_MAX elements in
// one CTA each, on presorted lists (every rank unique).  An element's local
// id is its place in the segment's axis-0 list at launch; the CTA holds the
// segment's three lists of local ids in shared memory and, per level, for
// every active sub-range (tracked per position in registers as k_rcb_small
// does): its cut axis from the first and last entry of each list, the side
// of each element from the cut axis' list, and a stable partition of every
// list by side.  The partition counts lower flags with one warp ballot per
// 32 positions: the count before a position is the totals of the warps
// before its warp (a shuffle scan), the totals of the rounds before its
// round inside its warp, and the ballot's bits below its lane.  All three
// lists move to three spare buffers in the same pass, so a level takes four
// CTA barriers.  Same tree, same order as the sort-per-level kernels;
// without LOCAL a sub-range that is no longer cut keeps the list of the axis
// that cut it last.
constexpr int SMALL_ROUNDS = SMALL_MAX / 32;  // ballots per list
constexpr size_t pss_smem_bytes() {
  // local id -> element (int); six list buffers and the lower child's size
  // by sub-range start (u16); side and cut axis (u8); per list the ballots
  // (u32) and the in-warp prefix of each round (u16)
  return (size_t)SMALL_MAX * (sizeof(int) + 7 * sizeof(unsigned short) + 2) +
         (size_t)3 * SMALL_ROUNDS * (sizeof(u32) + sizeof(unsigned short));
}

struct PssSmem {
  int *gl;               // local id -> element
  u32 *bal;              // [3][SMALL_ROUNDS] lower flags, one word per 32 positions
  unsigned short *buf;   // [6][SMALL_MAX]: three lists and three spares
  unsigned short *spl;   // lower child's size by sub-range start
  unsigned short *wpre;  // [3][SMALL_ROUNDS] lower flags before the round in its warp
  unsigned char *side;   // side by local id
  unsigned char *sax;    // cut axis by sub-range start
};

__device__ __forceinline__ PssSmem pss_carve(unsigned char *s) {
  PssSmem m;
  m.gl = reinterpret_cast<int *>(s);
  m.bal = reinterpret_cast<u32 *>(m.gl + SMALL_MAX);
  m.buf = reinterpret_cast<unsigned short *>(m.bal + 3 * SMALL_ROUNDS);
  m.spl = m.buf + 6 * SMALL_MAX;
  m.wpre = m.spl + SMALL_MAX;
  m.side = reinterpret_cast<unsigned char *>(m.wpre + 3 * SMALL_ROUNDS);
  m.sax = m.side + SMALL_MAX;
  return m;
}

// The level loop of k_rcb_small_ps; PONE: the segment has one virtual rank
// (only the local halving: no rank counts to track, every part is r0).
template <bool LOCAL, bool PONE>
__device__ __forceinline__ void pss_levels(int *__restrict__ perm, const double *__restrict__ cent,
                                           ll N, int ndim, ll start, int n, int p0, int r0,
                                           int *__restrict__ part, const PssSmem &m,
                                           int (*wsum)[SMALL_WARPS]) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const u32 lt = (1u << lane) - 1u;
  // sub-range of each own position (start | length << 16), its virtual
  // ranks, and the axis that cut it last
  u32 sl_r[SMALL_ITEMS];
  int p_r[PONE ? 1 : SMALL_ITEMS], rk_r[PONE ? 1 : SMALL_ITEMS];  // virtual ranks, first rank
  signed char oax_r[SMALL_ITEMS];
#pragma unroll
  for (int r = 0; r < SMALL_ITEMS; r++) {
    sl_r[r] = (u32)n << 16, oax_r[r] = -1;
    if (!PONE) p_r[r] = p0, rk_r[r] = 0;
  }
  int cur = 0;  // the lists are in buffers 3 cur .. 3 cur + 2, the spares in the others
  for (int d = 0; d < 64; d++) {
    if (d > 0) {  // advance every position's sub-range by the previous cut
#pragma unroll
      for (int r = 0; r < SMALL_ITEMS; r++) {
        const int x = warp * SMALL_SPAN + r * 32 + lane;
        int st = (int)(sl_r[r] & 0xFFFFu), ln = (int)(sl_r[r] >> 16), p = PONE ? 1 : p_r[r];
        if (!(p > 1 || (LOCAL && ln >= 2))) continue;  // no longer cut
        const int L = m.spl[st], h = p > 1 ? (p + 1) / 2 : 0;
        oax_r[r] = (signed char)m.sax[st];
        if (x < st + L) {
          ln = L;
          p = p > 1 ? h : p;
        } else {
          st += L;
          ln -= L;
          p = p > 1 ? p - h : p;
          if (!PONE) rk_r[r] += h;
        }
        sl_r[r] = (u32)st | ((u32)ln << 16);
        if (!PONE) p_r[r] = p;
      }
    }
    u32 act = 0;
#pragma unroll
    for (int r = 0; r < SMALL_ITEMS; r++) {
      const int x = warp * SMALL_SPAN + r * 32 + lane;
      const int ln = (int)(sl_r[r] >> 16);
      if (x < n && ((!PONE && p_r[r] > 1) || (LOCAL && ln >= 2))) act |= 1u << r;
    }
    // barrier: the reads of sax and spl above and the previous level's
    // partition are done before the cut axes are written and the lists read
    if (!__syncthreads_or(act != 0)) break;
    const unsigned short *Lc = m.buf + 3 * cur * SMALL_MAX;   // current lists
    unsigned short *Ls = m.buf + 3 * (cur ^ 1) * SMALL_MAX;  // spares
    // cut axis of each active sub-range: the coordinates of the first and
    // last entry of each list
#pragma unroll
    for (int r = 0; r < SMALL_ITEMS; r++) {
      const int x = warp * SMALL_SPAN + r * 32 + lane;
      const int st = (int)(sl_r[r] & 0xFFFFu), ln = (int)(sl_r[r] >> 16);
      if (!((act >> r) & 1u) || x != st) continue;
      double len[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int q = 0; q < 3; q++) {
        if (q >= ndim) break;
        const unsigned short *Lq = Lc + q * SMALL_MAX;
        const int lo = m.gl[Lq[st]], hi = m.gl[Lq[st + ln - 1]];
        len[q] = __dsub_rn(cent[(ll)q * N + hi], cent[(ll)q * N + lo]);
      }
      int ax = 0;
      for (int q = 1; q < ndim; q++)
        if (len[q] > len[ax]) ax = q;
      m.sax[st] = (unsigned char)ax;
      const int p = PONE ? 1 : p_r[r];
      m.spl[st] = (unsigned short)(p > 1 ? lower_count_small(ln, p) : ln / 2);
    }
    __syncthreads();
    // side of every element of a cut sub-range, from the cut axis' list
#pragma unroll
    for (int r = 0; r < SMALL_ITEMS; r++) {
      if (!((act >> r) & 1u)) continue;
      const int x = warp * SMALL_SPAN + r * 32 + lane;
      const int st = (int)(sl_r[r] & 0xFFFFu);
      m.side[Lc[m.sax[st] * SMALL_MAX + x]] = (x - st) >= (int)m.spl[st] ? 1 : 0;
    }
    __syncthreads();
    // lower flags of every list: one ballot per round of 32 positions, the
    // in-warp prefix of each round and each warp's total
    for (int q = 0; q < ndim; q++) {
      const unsigned short *Lq = Lc + q * SMALL_MAX;
      int cnt = 0;
#pragma unroll
      for (int r = 0; r < SMALL_ITEMS; r++) {
        const int x = warp * SMALL_SPAN + r * 32 + lane;
        const bool f = ((act >> r) & 1u) && m.side[Lq[x]] == 0;  // act implies x < n
        const u32 b = __ballot_sync(0xffffffffu, f);
        if (lane == 0) {
          m.bal[q * SMALL_ROUNDS + warp * SMALL_ITEMS + r] = b;
          m.wpre[q * SMALL_ROUNDS + warp * SMALL_ITEMS + r] = (unsigned short)cnt;
        }
        cnt += __popc(b);
      }
      if (lane == 0) wsum[q][warp] = cnt;
    }
    __syncthreads();
    // stable partition of each list by side into its spare buffer; a
    // position outside a cut sub-range keeps its place
    for (int q = 0; q < ndim; q++) {
      const int wv = wsum[q][lane];  // SMALL_WARPS == 32
      int inc = wv;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
      }
      const int exc = inc - wv;  // lane w: lower flags of the warps before w
      const int base_x = __shfl_sync(0xffffffffu, exc, warp);
      const unsigned short *Lq = Lc + q * SMALL_MAX;
      unsigned short *Tq = Ls + q * SMALL_MAX;
      const u32 *bq = m.bal + q * SMALL_ROUNDS;
      const unsigned short *wq = m.wpre + q * SMALL_ROUNDS;
#pragma unroll
      for (int r = 0; r < SMALL_ITEMS; r++) {
        const int x = warp * SMALL_SPAN + r * 32 + lane;
        const bool a = (act >> r) & 1u;
        const int st = a ? (int)(sl_r[r] & 0xFFFFu) : x;
        const int base_st = __shfl_sync(0xffffffffu, exc, st / SMALL_SPAN);
        if (x >= n) continue;
        const unsigned short id = Lq[x];
        int dest = x;
        if (a) {
          const int k = warp * SMALL_ITEMS + r, ks = st >> 5;
          const u32 bx = bq[k];
          const int before = (base_x + (int)wq[k] + __popc(bx & lt)) -
                             (base_st + (int)wq[ks] + __popc(bq[ks] & ((1u << (st & 31)) - 1u)));
          dest = ((bx >> lane) & 1u) ? st + before : st + (int)m.spl[st] + (x - st - before);
        }
        Tq[dest] = id;
      }
    }
    cur ^= 1;
  }
  // order: a LOCAL recursion ends in single elements (every list agrees);
  // otherwise each position takes the list of the axis that cut it last
  const unsigned short *Lc = m.buf + 3 * cur * SMALL_MAX;
#pragma unroll
  for (int r = 0; r < SMALL_ITEMS; r++) {
    const int x = warp * SMALL_SPAN + r * 32 + lane;
    if (x < n) {
      const int a = oax_r[r] < 0 ? 0 : oax_r[r];
      const int e = m.gl[Lc[a * SMALL_MAX + x]];
      perm[start + x] = e;
      if (part) part[e] = r0 + (PONE ? 0 : rk_r[r]);
    }
  }
}

template <bool LOCAL>
__global__ void __launch_bounds__(SMALL_THREADS)
k_rcb_small_ps(int *__restrict__ perm, const int *__restrict__ lists, int *__restrict__ loc,
               const double *__restrict__ cent, ll N, int ndim,
               const ll *__restrict__ seg_start, const ll *__restrict__ seg_n,
               const int *__restrict__ seg_p, const int *__restrict__ seg_r0,
               int *__restrict__ part) {
  extern __shared__ __align__(16) unsigned char pss_smem[];
  const PssSmem m = pss_carve(pss_smem);
  __shared__ int wsum[3][SMALL_WARPS];
  const ll sg = blockIdx.x;
  const ll start = seg_start[sg];
  const int n = (int)seg_n[sg], p0 = seg_p[sg], r0 = seg_r0[sg];
  if (n <= 0 || p0 <= 0) return;
  const bool seg_act = p0 > 1 || (LOCAL && p0 == 1 && n >= 2);
  if (!seg_act || n > SMALL_MAX) {
    if (part && n <= SMALL_MAX && p0 == 1)
      for (int x = threadIdx.x; x < n; x += blockDim.x) part[perm[start + x]] = r0;
    return;
  }
  const int *gl0 = lists + start;  // local id k -> element gl0[k]
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    const int e = gl0[x];
    loc[e] = x;
    m.gl[x] = e;
  }
  __syncthreads();
  for (int x = threadIdx.x; x < n; x += blockDim.x) {
    m.buf[x] = (unsigned short)x;
    for (int d = 1; d < ndim; d++)
      m.buf[d * SMALL_MAX + x] = (unsigned short)loc[lists[(ll)d * N + start + x]];
  }
  __syncthreads();
  if (p0 == 1)
    pss_levels<LOCAL, true>(perm, cent, N, ndim, start, n, p0, r0, part, m, wsum);
  else
    pss_levels<LOCAL, false>(perm, cent, N, ndim, start, n, p0, r0, part, m, wsum);
}

static void rcb_presorted(DBuf<int> &perm, SegTable &t, const double *cent, ll N, int ndim,
                          bool do_local, int *part_of_elem, BisectWs &ws) {
  cudaStream_t st = ctx().stream;
  const ll n3 = (ll)ndim * N;
  ws.lists.ensure((size_t)n3);
  ws.lists2.ensure((size_t)n3);
  ws.side.ensure((size_t)N);
  const int nblk = (int)((N + PS_TILE - 1) / PS_TILE);
  ws.bsum.ensure((size_t)ndim * nblk);
  ws.seg_of_pos2.ensure((size_t)N);
  ws.pbits.ensure((size_t)ndim * ((N + 31) >> 5));
  ws.pwpre.ensure((size_t)ndim * ((N + 31) >> 5));
  // lists of the initial segments: the global rank order of each axis,
  // grouped stably by segment; when the segments are the halves of the
  // previous call's (RSB's next level), that call's lists partitioned by half
  fill_seg_of_pos(t, ws.seg_of_pos.p, N);
  bool built = false;
  if (t.count == 1) {
    CK(cudaMemcpyAsync(ws.lists.p, ws.sorted.p, (size_t)n3 * sizeof(int),
                       cudaMemcpyDeviceToDevice, st));
    built = true;
  } else if (ws.g_ok && ws.g_N == N && ws.g_ndim == ndim && ws.gt.count > 0 &&
             t.count <= 2 * ws.gt.count) {
    const ll oc = ws.gt.count;
    ws.oseg.ensure((size_t)N);
    fill_seg_of_pos(ws.gt, ws.oseg.p, N);
    ws.axis.ensure((size_t)oc);
    ws.split.ensure((size_t)oc);
    ws.child_off.ensure((size_t)oc + 1);
    DBuf<int> bad(1);
    CK(cudaMemsetAsync(bad.p, 0, sizeof(int), st));
    k_inherit_tab<<<grid_for(oc, 256), 256, 0, st>>>(ws.gt.start.p, ws.gt.n.p, oc, t.start.p,
                                                     t.n.p, ws.seg_of_pos.p, ws.axis.p,
                                                     ws.split.p, ws.child_off.p, bad.p);
    CK_LAUNCH();
    int h_bad = 1;
    d2h(&h_bad, bad.p, 1);
    sync();
    if (!h_bad) {
      k_inherit_side<<<grid_for(N, 256), 256, 0, st>>>(perm.p, N, ws.oseg.p, ws.seg_of_pos.p,
                                                       ws.child_off.p, ws.side.p);
      CK_LAUNCH();
      k_ps_flags<<<(unsigned)nblk, PS_THREADS, 0, st>>>(ws.glists.p, N, ndim, ws.oseg.p,
                                                        ws.axis.p, ws.side.p, ws.pbits.p,
                                                        ws.pwpre.p, ws.bsum.p, nblk);
      CK_LAUNCH();
      k_ps_bscan<<<(unsigned)ndim, PS_THREADS, 0, st>>>(ws.bsum.p, nblk);
      CK_LAUNCH();
      k_ps_scatter<<<grid_for(N, 256), 256, 0, st>>>(
          ws.glists.p, N, ndim, ws.oseg.p, ws.gt.start.p, ws.axis.p, ws.split.p, ws.pbits.p,
          ws.pwpre.p, ws.bsum.p, nblk, ws.child_off.p, ws.lists.p, ws.seg_of_pos2.p);
      CK_LAUNCH();
      built = true;
    }
  }
  if (!built) {
    k_ps_seg_of_elem<<<grid_for(N, 256), 256, 0, st>>>(perm.p, ws.seg_of_pos.p, N,
                                                        ws.seg_of_elem.p);
    CK_LAUNCH();
    for (int a = 0; a < ndim; a++) {
      k_ps_seg_keys<<<grid_for(N, 256), 256, 0, st>>>(ws.sorted.p + (ll)a * N, ws.seg_of_elem.p,
                                                      N, ws.keys.p, ws.vals.p);
      CK_LAUNCH();
      seg_sort_pairs(ws.keys, ws.vals, N, nullptr, 1, ws.sort);
      CK(cudaMemcpyAsync(ws.lists.p + (ll)a * N, ws.vals.p, (size_t)N * sizeof(int),
                         cudaMemcpyDeviceToDevice, st));
    }
  }
  // this call's group lists and table, for the next call's lists
  ws.glists.ensure((size_t)n3);
  CK(cudaMemcpyAsync(ws.glists.p, ws.lists.p, (size_t)n3 * sizeof(int),
                     cudaMemcpyDeviceToDevice, st));
  ws.gt.reserve(t.count);
  CK(cudaMemcpyAsync(ws.gt.start.p, t.start.p, (size_t)t.count * sizeof(ll),
                     cudaMemcpyDeviceToDevice, st));
  CK(cudaMemcpyAsync(ws.gt.n.p, t.n.p, (size_t)t.count * sizeof(ll), cudaMemcpyDeviceToDevice,
                     st));
  ws.gt.count = t.count;
  ws.g_ok = true, ws.g_N = N, ws.g_ndim = ndim;
  ws.oax.ensure((size_t)t.count);
  CK(cudaMemsetAsync(ws.oax.p, 0xFF, (size_t)t.count * sizeof(int), st));  // -1: input order
  DBuf<int> nact_d(1);
  DBuf<unsigned long long> maxn_d(1);
  for (int level = 0; level < 200; level++) {
    const ll nseg = t.count;
    ws.child_cnt.ensure((size_t)nseg);
    CK(cudaMemsetAsync(nact_d.p, 0, sizeof(int), st));
    CK(cudaMemsetAsync(maxn_d.p, 0, sizeof(unsigned long long), st));
    k_child_counts<<<grid_for(nseg, 256), 256, 0, st>>>(t.p.p, t.n.p, nseg, do_local,
                                                        ws.child_cnt.p, nact_d.p);
    CK_LAUNCH();
    k_max_active_n<<<grid_for(nseg, 256), 256, 0, st>>>(t.p.p, t.n.p, nseg, do_local, maxn_d.p);
    CK_LAUNCH();
    int nact = 0;
    unsigned long long maxn = 0;
    d2h(&nact, nact_d.p, 1);
    d2h(&maxn, maxn_d.p, 1);
    sync();
    // (seg_of_pos follows the table: filled before the loop, then written
    // for the children by k_ps_scatter)
    if (nact == 0) break;
    if (maxn <= (unsigned long long)SMALL_MAX) {
      // every remaining level in one CTA per segment, on the segment's lists
      // (k_rcb_small_ps); a segment that is no longer cut takes its list here
      k_ps_final<<<grid_for(N, 256), 256, 0, st>>>(ws.lists.p, N, ws.seg_of_pos.p, ws.oax.p,
                                                    perm.p);
      CK_LAUNCH();
      ws.loc.ensure((size_t)N);
      const size_t smem = pss_smem_bytes();
      if (do_local) {
        ensure_smem_limit(k_rcb_small_ps<true>, (int)smem);
        k_rcb_small_ps<true><<<(unsigned)nseg, SMALL_THREADS, smem, st>>>(
            perm.p, ws.lists.p, ws.loc.p, cent, N, ndim, t.start.p, t.n.p, t.p.p, t.r0.p,
            part_of_elem);
      } else {
        ensure_smem_limit(k_rcb_small_ps<false>, (int)smem);
        k_rcb_small_ps<false><<<(unsigned)nseg, SMALL_THREADS, smem, st>>>(
            perm.p, ws.lists.p, ws.loc.p, cent, N, ndim, t.start.p, t.n.p, t.p.p, t.r0.p,
            part_of_elem);
      }
      CK_LAUNCH();
      return;
    }
    ws.axis.ensure((size_t)nseg);
    ws.split.ensure((size_t)nseg);
    k_ps_axis<<<grid_for(nseg, 256), 256, 0, st>>>(ws.lists.p, ws.rank.p, ws.uniq.p, N, ndim,
                                                   t.start.p, t.n.p, t.p.p, nseg, do_local,
                                                   ws.axis.p, ws.split.p);
    CK_LAUNCH();
    k_ps_side<<<grid_for(N, 256), 256, 0, st>>>(ws.lists.p, N, ws.seg_of_pos.p, t.start.p,
                                                ws.axis.p, ws.split.p, ws.side.p);
    CK_LAUNCH();
    k_ps_flags<<<(unsigned)nblk, PS_THREADS, 0, st>>>(ws.lists.p, N, ndim, ws.seg_of_pos.p,
                                                      ws.axis.p, ws.side.p, ws.pbits.p,
                                                      ws.pwpre.p, ws.bsum.p, nblk);
    CK_LAUNCH();
    k_ps_bscan<<<(unsigned)ndim, PS_THREADS, 0, st>>>(ws.bsum.p, nblk);
    CK_LAUNCH();
    // children (a cut segment has two, the others one)
    ws.child_off.ensure((size_t)nseg + 1);
    exclusive_scan_int_to_ll_async(ws.child_cnt.p, ws.child_off.p, nseg);
    const ll nchild = nseg + nact;
    k_ps_scatter<<<grid_for(N, 256), 256, 0, st>>>(
        ws.lists.p, N, ndim, ws.seg_of_pos.p, t.start.p, ws.axis.p, ws.split.p, ws.pbits.p,
        ws.pwpre.p, ws.bsum.p, nblk, ws.child_off.p, ws.lists2.p, ws.seg_of_pos2.p);
    CK_LAUNCH();
    std::swap(ws.lists.p, ws.lists2.p);
    std::swap(ws.lists.n, ws.lists2.n);
    std::swap(ws.seg_of_pos.p, ws.seg_of_pos2.p);
    std::swap(ws.seg_of_pos.n, ws.seg_of_pos2.n);
    // the children's table, and the list that orders each of them
    ws.t2.reserve(nchild);
    k_children<<<grid_for(nseg, 256), 256, 0, st>>>(
        t.start.p, t.n.p, t.p.p, t.r0.p, nseg, do_local, ws.child_off.p, ws.t2.start.p,
        ws.t2.n.p, ws.t2.p.p, ws.t2.r0.p);
    CK_LAUNCH();
    ws.oax2.ensure((size_t)nchild);
    k_ps_oaxis<<<grid_for(nseg, 256), 256, 0, st>>>(ws.axis.p, ws.oax.p, nseg, ws.child_off.p,
                                                    ws.oax2.p);
    CK_LAUNCH();
    std::swap(ws.oax.p, ws.oax2.p);
    std::swap(ws.oax.n, ws.oax2.n);
    ws.t2.count = nchild;
    std::swap(t.start, ws.t2.start);
    std::swap(t.n, ws.t2.n);
    std::swap(t.p, ws.t2.p);
    std::swap(t.r0, ws.t2.r0);
    std::swap(t.count, ws.t2.count);
  }
  k_ps_final<<<grid_for(N, 256), 256, 0, st>>>(ws.lists.p, N, ws.seg_of_pos.p, ws.oax.p, perm.p);
  CK_LAUNCH();
  if (part_of_elem) {
    k_part_from_segs<<<grid_for(N, 256), 256, 0, st>>>(perm.p, ws.seg_of_pos.p, t.r0.p, N,
                                                        part_of_elem);
    CK_LAUNCH();
  }
}

void bisect_segments(BisectKind kind, DBuf<int> &perm, SegTable &t,
                     const double *cent, ll N, int ndim, bool do_local,
                     int *part_of_elem, BisectWs &ws) {
  cudaStream_t st = ctx().stream;
  if (N <= 0) return;
  ws.seg_of_pos.ensure((size_t)N);
  ws.seg_of_elem.ensure((size_t)N);
  ws.keys.ensure((size_t)N);
  ws.vals.ensure((size_t)N);
  DBuf<int> nact_d(1);
  DBuf<unsigned long long> maxn_d(1);
  const size_t small_smem = small_smem_bytes();
  // PARRSB_GPU_LEVEL_LOG=1: per-level times on stderr (synchronises)
  const bool level_log = getenv("PARRSB_GPU_LEVEL_LOG") != nullptr;
  cudaEvent_t lg_e0 = nullptr, lg_e1 = nullptr, lg_part[4] = {};
  float lg_sum[4] = {};  // box + axis, keys, sort, children: summed over levels
  if (level_log) {
    CK(cudaEventCreate(&lg_e0));
    CK(cudaEventCreate(&lg_e1));
    for (auto &e : lg_part) CK(cudaEventCreate(&e));
    CK(cudaEventRecord(lg_e0, st));
  }
  auto lg_mark = [&](int i) {
    if (level_log && kind == BISECT_RCB) CK(cudaEventRecord(lg_part[i], st));
  };
  if (kind == BISECT_RCB && ws.rank_of != cent) {
    // dense ranks of the centroid coordinates, once per set of centroids
    ws.rank.ensure((size_t)3 * N);
    ws.uniq.ensure((size_t)3 * N);
    ws.sorted.ensure((size_t)ndim * N);
    DBuf<int> flag((size_t)N);
    DBuf<ll> excl((size_t)N);
    ws.unique = true;
    for (int a = 0; a < ndim; a++) {
      k_axis_keys<<<grid_for(N, 256), 256, 0, st>>>(cent, N, a, ws.keys.p, ws.vals.p);
      CK_LAUNCH();
      seg_sort_pairs(ws.keys, ws.vals, N, nullptr, 1, ws.sort);
      k_rank_flags<<<grid_for(N, 256), 256, 0, st>>>(ws.keys.p, N, flag.p);
      CK_LAUNCH();
      const ll changes = exclusive_scan_int_to_ll(flag.p, excl.p, N);
      if (changes != N - 1) ws.unique = false;  // two centroids share a coordinate
      k_rank_write<<<grid_for(N, 256), 256, 0, st>>>(ws.keys.p, ws.vals.p, flag.p, excl.p, N,
                                                      ws.rank.p + (ll)a * N,
                                                      ws.uniq.p + (ll)a * N);
      CK_LAUNCH();
      CK(cudaMemcpyAsync(ws.sorted.p + (ll)a * N, ws.vals.p, (size_t)N * sizeof(int),
                         cudaMemcpyDeviceToDevice, st));
    }
    ws.rank_of = cent;
    ws.g_ok = false;  // lists of other centroids
  }
  // PARRSB_GPU_RCB_PRESORT=0: the sort-per-level path even for unique ranks
  if (kind == BISECT_RCB && ws.unique) {
    const char *e = getenv("PARRSB_GPU_RCB_PRESORT");
    if (!(e && atoi(e) == 0)) {
      rcb_presorted(perm, t, cent, N, ndim, do_local, part_of_elem, ws);
      return;
    }
  }
  ws.g_ok = false;  // the next presorted call builds its lists afresh
  for (int level = 0; level < 200; level++) {
    ll nseg = t.count;
    // active segments, their largest size, and children counts
    ws.child_cnt.ensure((size_t)nseg);
    CK(cudaMemsetAsync(nact_d.p, 0, sizeof(int), st));
    CK(cudaMemsetAsync(maxn_d.p, 0, sizeof(unsigned long long), st));
    k_child_counts<<<grid_for(nseg, 256), 256, 0, st>>>(t.p.p, t.n.p, nseg, do_local,
                                                        ws.child_cnt.p, nact_d.p);
    CK_LAUNCH();
    k_max_active_n<<<grid_for(nseg, 256), 256, 0, st>>>(t.p.p, t.n.p, nseg, do_local, maxn_d.p);
    CK_LAUNCH();
    int nact = 0;
    unsigned long long maxn = 0;
    d2h(&nact, nact_d.p, 1);
    d2h(&maxn, maxn_d.p, 1);
    sync();
    if (level_log && kind == BISECT_RCB) {  // time of the global levels so far
      CK(cudaEventRecord(lg_e1, st));
      CK(cudaEventSynchronize(lg_e1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, lg_e0, lg_e1));
      if (level > 0) {
        float d[4];
        CK(cudaEventElapsedTime(&d[0], lg_e0, lg_part[0]));
        for (int i = 1; i < 4; i++) CK(cudaEventElapsedTime(&d[i], lg_part[i - 1], lg_part[i]));
        for (int i = 0; i < 4; i++) lg_sum[i] += d[i];
      }
      fprintf(stderr, "parrsb_gb300: rcb level %d segments=%lld active=%d max_n=%llu: %.3f ms"
              " (sums box %.2f keys %.2f sort %.2f children %.2f)\n",
              level, (long long)nseg, nact, maxn, ms, lg_sum[0], lg_sum[1], lg_sum[2], lg_sum[3]);
      CK(cudaEventRecord(lg_e0, st));
    }
    if (kind == BISECT_RCB && nact > 0 && maxn <= (unsigned long long)SMALL_MAX) {
      // every remaining level of every segment in one launch
      if (do_local) {
        CK(cudaFuncSetAttribute(k_rcb_small<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)small_smem));
        k_rcb_small<true><<<(unsigned)nseg, SMALL_THREADS, small_smem, st>>>(
            perm.p, ws.rank.p, ws.uniq.p, N, ndim, t.start.p, t.n.p, t.p.p, t.r0.p,
            part_of_elem);
      } else {
        CK(cudaFuncSetAttribute(k_rcb_small<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)small_smem));
        k_rcb_small<false><<<(unsigned)nseg, SMALL_THREADS, small_smem, st>>>(
            perm.p, ws.rank.p, ws.uniq.p, N, ndim, t.start.p, t.n.p, t.p.p, t.r0.p,
            part_of_elem);
      }
      CK_LAUNCH();
      if (level_log) {
        CK(cudaEventRecord(lg_e1, st));
        CK(cudaEventSynchronize(lg_e1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, lg_e0, lg_e1));
        fprintf(stderr, "parrsb_gb300: rcb small-segment kernel segments=%lld: %.3f ms\n",
                (long long)nseg, ms);
        cudaEventDestroy(lg_e0);
        cudaEventDestroy(lg_e1);
        for (auto &e : lg_part) cudaEventDestroy(e);
      }
      return;
    }
    if (level_log && kind == BISECT_RCB) CK(cudaEventRecord(lg_e0, st));
    fill_seg_of_pos(t, ws.seg_of_pos.p, N);
    if (nact == 0) break;
    ws.axis.ensure((size_t)nseg);
    if (kind == BISECT_RCB) {
      ws.rbox.ensure((size_t)nseg * 6);
      CK(cudaMemsetAsync(ws.rbox.p, 0xFF, (size_t)nseg * 6 * sizeof(u32), st));
      k_rank_box<<<grid_for(N, RBOX_THREADS * RBOX_ITEMS), RBOX_THREADS, 0, st>>>(
          perm.p, ws.rank.p, N, ndim, ws.seg_of_pos.p, ws.rbox.p);
      CK_LAUNCH();
      k_rcb_axis_rank<<<grid_for(nseg, 256), 256, 0, st>>>(ws.rbox.p, ws.uniq.p, N, t.p.p,
                                                           t.n.p, nseg, ndim, do_local,
                                                           ws.axis.p);
      CK_LAUNCH();
      lg_mark(0);
      k_keys<BISECT_RCB><<<grid_for(N, 256), 256, 0, st>>>(
          perm.p, cent, ws.rank.p, N, ws.seg_of_pos.p, ws.axis.p, nullptr, nullptr, ws.keys.p,
          ws.vals.p, ws.seg_of_elem.p);
      CK_LAUNCH();
      lg_mark(1);
    } else {
      DBuf<double> sums((size_t)nseg * 3), avg((size_t)nseg * 3),
          isums((size_t)nseg * 6);
      ws.ev.ensure((size_t)nseg * 3);
      seg_tree_reduce<3, GEN_MEAN>(perm.p, cent, N, t, nullptr, ws, sums.p);
      k_rib_mean_group<<<grid_for(nseg, 256), 256, 0, st>>>(sums.p, t.n.p, t.p.p, nseg,
                                                            avg.p);
      CK_LAUNCH();
      if (do_local) {
        k_rib_mean_local<<<grid_for(nseg, 128), 128, 0, st>>>(
            perm.p, cent, N, t.start.p, t.n.p, t.p.p, nseg, 1, avg.p);
        CK_LAUNCH();
      }
      seg_tree_reduce<6, GEN_INERTIA>(perm.p, cent, N, t, avg.p, ws, isums.p);
      k_rib_axis<<<grid_for(nseg, 128), 128, 0, st>>>(
          perm.p, cent, N, t.start.p, t.n.p, t.p.p, nseg, ndim, do_local ? 1 : 0,
          avg.p, isums.p, ws.ev.p, ws.axis.p);
      CK_LAUNCH();
      k_keys<BISECT_RIB><<<grid_for(N, 256), 256, 0, st>>>(
          perm.p, cent, nullptr, N, ws.seg_of_pos.p, ws.axis.p, avg.p, ws.ev.p, ws.keys.p,
          ws.vals.p, ws.seg_of_elem.p);
      CK_LAUNCH();
    }
    // RCB keys carry the segment id above the rank; RIB keys are full doubles
    if (kind == BISECT_RCB)
      seg_sort_pairs(ws.keys, ws.vals, N, nullptr, 1, ws.sort);
    else
      seg_sort_pairs(ws.keys, ws.vals, N, ws.seg_of_elem.p, nseg, ws.sort);
    lg_mark(2);
    std::swap(perm.p, ws.vals.p);
    std::swap(perm.n, ws.vals.n);
    // children
    ws.child_off.ensure((size_t)nseg + 1);
    ll nchild = exclusive_scan_int_to_ll(ws.child_cnt.p, ws.child_off.p, nseg);
    ws.t2.reserve(nchild);
    k_children<<<grid_for(nseg, 256), 256, 0, st>>>(
        t.start.p, t.n.p, t.p.p, t.r0.p, nseg, do_local, ws.child_off.p, ws.t2.start.p,
        ws.t2.n.p, ws.t2.p.p, ws.t2.r0.p);
    CK_LAUNCH();
    lg_mark(3);
    ws.t2.count = nchild;
    std::swap(t.start, ws.t2.start);
    std::swap(t.n, ws.t2.n);
    std::swap(t.p, ws.t2.p);
    std::swap(t.r0, ws.t2.r0);
    std::swap(t.count, ws.t2.count);
  }
  if (part_of_elem) {
    k_part_from_segs<<<grid_for(N, 256), 256, 0, st>>>(perm.p, ws.seg_of_pos.p, t.r0.p,
                                                        N, part_of_elem);
    CK_LAUNCH();
  }
}

}  // namespace prsb
