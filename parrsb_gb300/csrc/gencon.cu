// gencon.cu -- tolerance-based unique-vertex numbering on the GPU.
//
// Restates parrsb_conn_mesh for one rank (src/con.c:189-295):
//   mesh_init (symmetric corner order, src/con.c:14-50)
//   find_min_neighbor_distance (src/con.c:68-103)
//   find_unique_vertices (src/con-unique-vertices.c:445-505): ndim*ndim
//     passes; each sorts every current segment of points by one coordinate
//     and starts a new segment where (dx_j)^2 > min(dx2_j, dx2_{j-1}) tol^2
//   set_global_id / send_back (src/con.c:108-148)
//   element_check / face_check (src/con-check.c:197-288)
//   compressPeriodicVertices (identity without periodic faces)
// Every segmented sort is stable (the reference's per-segment heapsort,
// src/con-unique-vertices.c:6-58, is replaced by the canonical stable order;
// both give the same ids unless a split decision sits on an exact tie).
#include "gencon.cuh"

namespace prsb {

namespace {

__constant__ int c_pre_to_sym[8] = {0, 1, 3, 2, 4, 5, 7, 6};
__constant__ int c_nbr[8][3] = {{1, 2, 4}, {0, 3, 5}, {0, 3, 6}, {1, 2, 7},
                                {0, 5, 6}, {1, 4, 7}, {2, 4, 7}, {3, 5, 6}};
// faces in symmetric corner order (0-based), src/con-periodic.c:8-10
__constant__ int c_face_mask3[6] = {
    (1 << 0) | (1 << 4) | (1 << 6) | (1 << 2), (1 << 1) | (1 << 3) | (1 << 7) | (1 << 5),
    (1 << 0) | (1 << 1) | (1 << 5) | (1 << 4), (1 << 2) | (1 << 6) | (1 << 7) | (1 << 3),
    (1 << 0) | (1 << 2) | (1 << 3) | (1 << 1), (1 << 4) | (1 << 5) | (1 << 7) | (1 << 6)};

__device__ __forceinline__ double dsq(double a, double b) {
  double t = __dsub_rn(a, b);
  return __dmul_rn(t, t);
}

// Points in symmetric order and their min squared neighbour distance.
__global__ void k_points(const double *__restrict__ coord, ll nel, int ndim,
                         double *__restrict__ x0, double *__restrict__ x1,
                         double *__restrict__ x2, double *__restrict__ dx) {
  ll e = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  int nv = ndim == 2 ? 4 : 8;
  double px[8][3];
  const double *c = coord + e * nv * ndim;
  for (int k = 0; k < nv; k++) {
    int j = c_pre_to_sym[k];
    px[k][0] = c[j * ndim + 0];
    px[k][1] = c[j * ndim + 1];
    px[k][2] = ndim == 3 ? c[j * ndim + 2] : 0.0;
  }
  for (int k = 0; k < nv; k++) {
    ll p = e * nv + k;
    x0[p] = px[k][0];
    x1[p] = px[k][1];
    x2[p] = px[k][2];
    double m = 1.7976931348623157e308;
    for (int q = 0; q < ndim; q++) {
      int nb = c_nbr[k][q];
      double d = __dadd_rn(dsq(px[k][0], px[nb][0]), dsq(px[k][1], px[nb][1]));
      if (ndim == 3) d = __dadd_rn(d, dsq(px[k][2], px[nb][2]));
      m = (m < d) ? m : d;
    }
    dx[p] = m;
  }
}

__global__ void k_gc_keys(const int *__restrict__ ord, const double *__restrict__ x,
                          const ll *__restrict__ segid, ll np,
                          u64 *__restrict__ keys, int *__restrict__ vals,
                          int *__restrict__ seg_of_pt) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  int p = ord[i];
  keys[i] = ordered_key(x[p]);
  vals[i] = p;
  if (seg_of_pt) seg_of_pt[p] = (int)segid[i];
}

__global__ void k_iota(int *__restrict__ a, ll n) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = (int)i;
}

// flag[j] |= gap between sorted neighbours j-1, j along coordinate x.
__global__ void k_gaps(const int *__restrict__ ord, const double *__restrict__ x,
                       const double *__restrict__ dx, ll np, double tol2,
                       int first_pass, int *__restrict__ flag) {
  ll j = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= np) return;
  if (j == 0) {
    flag[0] = 1;
    return;
  }
  int pj = ord[j], pk = ord[j - 1];
  double d = dsq(x[pj], x[pk]);
  double m = __dmul_rn(dx[pj] < dx[pk] ? dx[pj] : dx[pk], tol2);
  int f = d > m ? 1 : 0;
  if (first_pass)
    flag[j] = f;
  else if (f)
    flag[j] = 1;
}

// segid = inclusive prefix of flags minus one, from the exclusive scan.
__global__ void k_segid(const int *__restrict__ flag, ll *__restrict__ scan, ll np) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < np) scan[i] = scan[i] + flag[i] - 1;
}

__global__ void k_ids(const int *__restrict__ ord, const ll *__restrict__ segid,
                      ll np, ll *__restrict__ ids) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < np) ids[ord[i]] = segid[i];
}

__global__ void k_seg_starts(const int *__restrict__ flag, const ll *__restrict__ segid,
                             ll np, ll nseg, ll *__restrict__ seg_start) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < np && flag[i]) seg_start[segid[i]] = i;
  if (i == np - 1) seg_start[nseg] = np;
}

__global__ void k_element_check(const ll *__restrict__ ids, ll nel, int nv,
                                int *__restrict__ err) {
  ll e = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  ll g[8];
  for (int k = 0; k < nv; k++) g[k] = ids[e * nv + k];
  for (int a = 0; a < nv; a++)
    for (int b = a + 1; b < nv; b++)
      if (g[a] == g[b]) {
        atomicOr(err, 1);
        return;
      }
}

// face_check: an element e that contains exactly 3 of the 4 corners of a
// face of element i is an error.  Candidates e are the elements sharing a
// vertex with i (the points of i's vertex segments); e is examined once, at
// the lowest corner of i that it contains.
__global__ void k_face_check(const ll *__restrict__ ids, const int *__restrict__ ord,
                             const ll *__restrict__ seg_start, ll nseg, ll nel,
                             int *__restrict__ err) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nel) return;
  const int nv = 8;
  ll gi[8];
  for (int k = 0; k < nv; k++) gi[k] = ids[i * nv + k];
  for (int k = 0; k < nv; k++) {
    ll s = gi[k];
    ll b = seg_start[s], e = seg_start[s + 1];
    for (ll q = b; q < e; q++) {
      ll el = ord[q] / nv;
      unsigned mask = 0;
      for (int a = 0; a < nv; a++) {
        ll ga = ids[el * nv + a];
        for (int c = 0; c < nv; c++)
          if (ga == gi[c]) mask |= 1u << c;
      }
      if ((__ffs(mask) - 1) != k) continue;  // seen at a lower corner
      for (int f = 0; f < 6; f++)
        if (__popc(mask & c_face_mask3[f]) == 3) {
          atomicOr(err, 1);
          return;
        }
    }
  }
}

__global__ void k_plus_one(const ll *__restrict__ ids, ll n, long long *__restrict__ out) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = ids[i] + 1;
}

}  // namespace

int gencon_device(long long *d_vtx, const double *d_coord, ll nel, int ndim,
                  double tol, GenconWs &ws, ll *nseg_out, ll *d_ids_out) {
  cudaStream_t st = ctx().stream;
  int nv = ndim == 2 ? 4 : 8;
  ll np = nel * nv;
  if (np == 0) {
    if (nseg_out) *nseg_out = 0;
    return PARRSB_OK;
  }
  for (int d = 0; d < 3; d++) ws.x[d].ensure((size_t)np);
  ws.dx.ensure((size_t)np);
  ws.keys.ensure((size_t)np);
  ws.ord.ensure((size_t)np);
  ws.flag.ensure((size_t)np);
  ws.segid.ensure((size_t)np + 1);
  ws.seg_of_pt.ensure((size_t)np);
  ws.ids.ensure((size_t)np);
  ws.vals.ensure((size_t)np);
  k_points<<<grid_for(nel, 128), 128, 0, st>>>(d_coord, nel, ndim, ws.x[0].p, ws.x[1].p,
                                               ws.x[2].p, ws.dx.p);
  CK_LAUNCH();
  k_iota<<<grid_for(np, 256), 256, 0, st>>>(ws.ord.p, np);
  CK_LAUNCH();
  double tol2 = tol * tol;
  ll nseg = 1;
  for (int t = 0; t < ndim; t++) {
    for (int d = 0; d < ndim; d++) {
      bool first = (t == 0 && d == 0);
      k_gc_keys<<<grid_for(np, 256), 256, 0, st>>>(ws.ord.p, ws.x[d].p, ws.segid.p, np,
                                                   ws.keys.p, ws.vals.p,
                                                   first ? nullptr : ws.seg_of_pt.p);
      CK_LAUNCH();
      seg_sort_pairs(ws.keys, ws.vals, np, first ? nullptr : ws.seg_of_pt.p, nseg,
                     ws.sort);
      std::swap(ws.ord.p, ws.vals.p);
      std::swap(ws.ord.n, ws.vals.n);
      k_gaps<<<grid_for(np, 256), 256, 0, st>>>(ws.ord.p, ws.x[d].p, ws.dx.p, np, tol2,
                                                first ? 1 : 0, ws.flag.p);
      CK_LAUNCH();
      ll total = exclusive_scan_int_to_ll(ws.flag.p, ws.segid.p, np);
      k_segid<<<grid_for(np, 256), 256, 0, st>>>(ws.flag.p, ws.segid.p, np);
      CK_LAUNCH();
      nseg = total;
    }
  }
  if (nseg_out) *nseg_out = nseg;
  k_ids<<<grid_for(np, 256), 256, 0, st>>>(ws.ord.p, ws.segid.p, np, ws.ids.p);
  CK_LAUNCH();
  if (d_ids_out)
    CK(cudaMemcpyAsync(d_ids_out, ws.ids.p, np * sizeof(ll), cudaMemcpyDeviceToDevice, st));
  DBuf<int> err(1);
  CK(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  {
    StageTimer tm(PARRSB_STAGE_CHECK);
    k_element_check<<<grid_for(nel, 256), 256, 0, st>>>(ws.ids.p, nel, nv, err.p);
    CK_LAUNCH();
    int h_err = 0;
    d2h(&h_err, err.p, 1);
    sync();
    if (h_err) return 1;
    if (ndim == 3) {  // in 2D an edge has two corners: a count of 3 is impossible
      DBuf<ll> seg_start((size_t)nseg + 1);
      k_seg_starts<<<grid_for(np, 256), 256, 0, st>>>(ws.flag.p, ws.segid.p, np, nseg,
                                                      seg_start.p);
      CK_LAUNCH();
      k_face_check<<<grid_for(nel, 128), 128, 0, st>>>(ws.ids.p, ws.ord.p, seg_start.p,
                                                       nseg, nel, err.p);
      CK_LAUNCH();
      d2h(&h_err, err.p, 1);
      sync();
      if (h_err) return 1;
    }
  }
  if (d_vtx) {
    k_plus_one<<<grid_for(np, 256), 256, 0, st>>>(ws.ids.p, np, d_vtx);
    CK_LAUNCH();
  }
  return PARRSB_OK;
}

}  // namespace prsb
