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

enum Gen { GEN_BBOX = 0, GEN_MEAN = 1, GEN_INERTIA = 2, GEN_ARRAY = 3 };

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
// For GEN_BBOX values 0..2 are minima, 3..5 maxima; otherwise sums.
template <int V, int GEN, bool BBOX>
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
  for (int q = 0; q < V; q++) {
    if (BBOX)
      v[q] = q < 3 ? DBL_MAX : -DBL_MAX;
    else
      v[q] = 0.0;
  }
  if (valid) {
    if (GEN == GEN_ARRAY) {
      ll src = (in_off[s] + i) * V;
#pragma unroll
      for (int q = 0; q < V; q++) v[q] = in[src + q];
    } else {
      int e = perm[seg_start[s] + i];
      double c0 = cent[e], c1 = cent[N + e], c2 = cent[2 * N + e];
      if (GEN == GEN_BBOX) {
        v[0] = c0, v[1] = c1, v[2] = c2;
        v[3] = c0, v[4] = c1, v[5] = c2;
      } else if (GEN == GEN_MEAN) {
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
    else if (BBOX)
      r = q < 3 ? warp_min(v[q]) : warp_max(v[q]);
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

__global__ void k_rcb_axis(const double *__restrict__ bbox, const int *__restrict__ p,
                           const ll *__restrict__ n, ll nseg, int ndim,
                           int do_local, int *__restrict__ axis) {
  ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const double *b = bbox + 6 * s;
  double len[3];
  for (int d = 0; d < ndim; d++) len[d] = __dsub_rn(b[3 + d], b[d]);
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
                       ll N, const int *__restrict__ seg_of_pos,
                       const int *__restrict__ axis_or_act,
                       const double *__restrict__ avg,
                       const double *__restrict__ ev, u64 *__restrict__ keys,
                       int *__restrict__ vals, int *__restrict__ seg_of_elem) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int s = seg_of_pos[i];
  int e = perm[i];
  u64 k = 0;
  if (KIND == BISECT_RCB) {
    int ax = axis_or_act[s];
    if (ax >= 0) k = ordered_key(cent[(ll)ax * N + e]);
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
  seg_of_elem[e] = s;
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

// Run the tile tree over every segment of `t` until one value per segment
// is left; result in out_final (nseg * V values).
template <int V, int GEN0, bool BBOX>
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
      k_seg_tree<V, GEN0, BBOX><<<blocks, 256, 0, st>>>(perm, cent, N, t.start.p,
                                                        cnt.p, nseg, off.p, ntiles,
                                                        nullptr, nullptr, avg, ob.p);
    else
      k_seg_tree<V, GEN_ARRAY, BBOX><<<blocks, 256, 0, st>>>(
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

void compute_centroids(const double *xyz, int nel, int nv, double *cent) {
  int ndim = (nv == 8) ? 3 : 2;
  k_centroids<<<grid_for(nel, 256), 256, 0, ctx().stream>>>(xyz, nel, nv, ndim, cent);
  CK_LAUNCH();
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
  for (int level = 0; level < 200; level++) {
    ll nseg = t.count;
    // active segments and children counts
    ws.child_cnt.ensure((size_t)nseg);
    CK(cudaMemsetAsync(nact_d.p, 0, sizeof(int), st));
    k_child_counts<<<grid_for(nseg, 256), 256, 0, st>>>(t.p.p, t.n.p, nseg, do_local,
                                                        ws.child_cnt.p, nact_d.p);
    CK_LAUNCH();
    int nact = 0;
    d2h(&nact, nact_d.p, 1);
    sync();
    fill_seg_of_pos(t, ws.seg_of_pos.p, N);
    if (nact == 0) break;
    ws.axis.ensure((size_t)nseg);
    if (kind == BISECT_RCB) {
      DBuf<double> bbox((size_t)nseg * 6);
      seg_tree_reduce<6, GEN_BBOX, true>(perm.p, cent, N, t, nullptr, ws, bbox.p);
      k_rcb_axis<<<grid_for(nseg, 256), 256, 0, st>>>(bbox.p, t.p.p, t.n.p, nseg, ndim,
                                                      do_local, ws.axis.p);
      CK_LAUNCH();
      k_keys<BISECT_RCB><<<grid_for(N, 256), 256, 0, st>>>(
          perm.p, cent, N, ws.seg_of_pos.p, ws.axis.p, nullptr, nullptr, ws.keys.p,
          ws.vals.p, ws.seg_of_elem.p);
      CK_LAUNCH();
    } else {
      DBuf<double> sums((size_t)nseg * 3), avg((size_t)nseg * 3),
          isums((size_t)nseg * 6);
      ws.ev.ensure((size_t)nseg * 3);
      seg_tree_reduce<3, GEN_MEAN, false>(perm.p, cent, N, t, nullptr, ws, sums.p);
      k_rib_mean_group<<<grid_for(nseg, 256), 256, 0, st>>>(sums.p, t.n.p, t.p.p, nseg,
                                                            avg.p);
      CK_LAUNCH();
      if (do_local) {
        k_rib_mean_local<<<grid_for(nseg, 128), 128, 0, st>>>(
            perm.p, cent, N, t.start.p, t.n.p, t.p.p, nseg, 1, avg.p);
        CK_LAUNCH();
      }
      seg_tree_reduce<6, GEN_INERTIA, false>(perm.p, cent, N, t, avg.p, ws, isums.p);
      k_rib_axis<<<grid_for(nseg, 128), 128, 0, st>>>(
          perm.p, cent, N, t.start.p, t.n.p, t.p.p, nseg, ndim, do_local ? 1 : 0,
          avg.p, isums.p, ws.ev.p, ws.axis.p);
      CK_LAUNCH();
      k_keys<BISECT_RIB><<<grid_for(N, 256), 256, 0, st>>>(
          perm.p, cent, N, ws.seg_of_pos.p, ws.axis.p, avg.p, ws.ev.p, ws.keys.p,
          ws.vals.p, ws.seg_of_elem.p);
      CK_LAUNCH();
    }
    seg_sort_pairs(ws.keys, ws.vals, N, ws.seg_of_elem.p, nseg, ws.sort);
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
