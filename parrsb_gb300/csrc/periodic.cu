// periodic.cu -- periodic-face matching after gencon (match_periodic_faces,
// src/con-periodic.c:245-288).
//
// Input: the 0-based ids of every corner point (sequence order, symmetric
// corner numbering) and the points' coordinates, as gencon leaves them, and
// the caller's periodic face records (element, face, partner element,
// partner face; 1-based, faces in preprocessor numbering, src/con.c:38-46).
// Steps, all on the device:
//   1. decode the records and order them stably by element (the boundary
//      array is sorted by elementId before matching, :193-230);
//   2. a face j is paired with every face i before it whose (element, face)
//      equals j's partner (findConnectedPeriodicFaces, :157-170): a sorted
//      key table and a binary search replace the quadratic loop;
//   3. one thread per pair centres both faces, picks the cyclic shift of the
//      reversed corner order with the least squared distance, rejects the
//      pair when that distance exceeds 1e-3 of the largest coordinate
//      magnitude, and emits (min id, max id) per corner
//      (findConnectedPeriodicPairs, :104-155);
//   4. every id takes the smallest id of its class under those pairs
//      (renumberPeriodicVertices, :64-102): min-label hooking plus pointer
//      jumping, repeated until no label changes;
//   5. the surviving ids are renumbered consecutively in increasing order
//      (compressPeriodicVertices, :24-55).
// The reference exits the process on a face mismatch; here the call
// returns PARRSB_ERR_CHECK.
#include "../../include/parrsb.h"
#include "periodic.cuh"

namespace prsb {
namespace {

__constant__ int c_pre_to_sym_face[6] = {2, 1, 3, 0, 4, 5};
__constant__ int c_faces3d[6][4] = {{1, 5, 7, 3}, {2, 4, 8, 6}, {1, 2, 6, 5},
                                    {3, 7, 8, 4}, {1, 3, 4, 2}, {5, 6, 8, 7}};
__constant__ int c_faces2d[4][2] = {{3, 1}, {2, 4}, {1, 2}, {4, 3}};

// record -> (element, symmetric face) keys; bad records set *bad
__global__ void k_pf_decode(const long long *__restrict__ pinfo, int npf, ll nel, int nfaces,
                            u64 *__restrict__ ekey, int *__restrict__ eidx,
                            u64 *__restrict__ fkey, int *__restrict__ fidx,
                            ll *__restrict__ self, ll *__restrict__ partner,
                            int *__restrict__ bad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npf) return;
  const long long e = pinfo[4 * i] - 1, f = pinfo[4 * i + 1] - 1;
  const long long be = pinfo[4 * i + 2] - 1, bf = pinfo[4 * i + 3] - 1;
  if (e < 0 || e >= nel || f < 0 || f >= nfaces || be < 0 || be >= nel || bf < 0 ||
      bf >= nfaces) {
    atomicOr(bad, 1);
    self[i] = partner[i] = -1;
    ekey[i] = fkey[i] = 0;
  } else {
    self[i] = e * 8 + c_pre_to_sym_face[f];
    partner[i] = be * 8 + c_pre_to_sym_face[bf];
    ekey[i] = (u64)e;
    fkey[i] = (u64)self[i];
  }
  eidx[i] = i;
  fidx[i] = i;
}

__global__ void k_pf_rank(const int *__restrict__ ord, int npf, int *__restrict__ pos) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < npf) pos[ord[q]] = q;
}

// face j: every earlier face i (in element order) whose key is j's partner
__global__ void k_pf_pairs(const u64 *__restrict__ skey, const int *__restrict__ sface, int npf,
                           const ll *__restrict__ partner, const int *__restrict__ pos,
                           int *__restrict__ npairs, int2 *__restrict__ pairs, int cap) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= npf || partner[j] < 0) return;
  const u64 want = (u64)partner[j];
  int lo = 0, hi = npf;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (skey[mid] < want)
      lo = mid + 1;
    else
      hi = mid;
  }
  for (int q = lo; q < npf && skey[q] == want; q++) {
    const int i = sface[q];
    if (pos[i] < pos[j]) {
      int o = atomicAdd(npairs, 1);
      if (o < cap) pairs[o] = make_int2(i, j);
    }
  }
}

__device__ __forceinline__ double dsq(double a, double b) {
  double d = __dsub_rn(a, b);
  return __dmul_rn(d, d);
}

// one thread per matched face pair: corner correspondence, (min, max) ids
__global__ void k_pf_match(const int2 *__restrict__ pairs, int n, const ll *__restrict__ self,
                           const ll *__restrict__ ids, const double *__restrict__ x0,
                           const double *__restrict__ x1, const double *__restrict__ x2,
                           int ndim, ll *__restrict__ pmin, ll *__restrict__ pmax,
                           int *__restrict__ mismatch) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int nv = ndim == 3 ? 8 : 4, nvf = nv / 2;
  const double *xs[3] = {x0, x1, x2};
  double fx[4][3], gx[4][3];
  ll fid[4], gid[4];
  const ll sf = self[pairs[t].x], sg = self[pairs[t].y];
  for (int j = 0; j < nvf; j++) {
    const int cf = (ndim == 3 ? c_faces3d[sf & 7][j] : c_faces2d[sf & 7][j]) - 1;
    const int cg = (ndim == 3 ? c_faces3d[sg & 7][j] : c_faces2d[sg & 7][j]) - 1;
    const ll pf = (sf >> 3) * nv + cf, pg = (sg >> 3) * nv + cg;
    fid[j] = ids[pf];
    gid[j] = ids[pg];
    for (int d = 0; d < ndim; d++) fx[j][d] = xs[d][pf], gx[j][d] = xs[d][pg];
  }
  double fmax = 0.0, gmax = 0.0;
  for (int d = 0; d < ndim; d++) {
    double mf = 0.0, mg = 0.0;
    for (int j = 0; j < nvf; j++) {
      fmax = fmax > fabs(fx[j][d]) ? fmax : fabs(fx[j][d]);
      gmax = gmax > fabs(gx[j][d]) ? gmax : fabs(gx[j][d]);
      mf = __dadd_rn(mf, fx[j][d]);
      mg = __dadd_rn(mg, gx[j][d]);
    }
    const double cf = __ddiv_rn(mf, (double)nvf), cg = __ddiv_rn(mg, (double)nvf);
    for (int j = 0; j < nvf; j++) {
      fx[j][d] = __dsub_rn(fx[j][d], cf);
      gx[j][d] = __dsub_rn(gx[j][d], cg);
    }
  }
  int shift = 0;
  double d2min = 1.e20;
  for (int s = 0; s < nvf; s++) {
    double d2 = 0.0;
    for (int j = 0; j < nvf; j++) {
      const int k = nvf - 1 - (j + s) % nvf;
      double dd = __dadd_rn(dsq(fx[j][0], gx[k][0]), dsq(fx[j][1], gx[k][1]));
      if (ndim == 3) dd = __dadd_rn(dd, dsq(fx[j][2], gx[k][2]));
      d2 = __dadd_rn(d2, dd);
    }
    if (d2 < d2min) d2min = d2, shift = s;
  }
  const double fg = fmax > gmax ? fmax : gmax;
  if (__dsqrt_rn(d2min) > __dmul_rn(1e-3, fg)) atomicOr(mismatch, 1);
  for (int j = 0; j < nvf; j++) {
    const int k = nvf - 1 - (j + shift) % nvf;
    pmin[t * nvf + j] = fid[j] < gid[k] ? fid[j] : gid[k];
    pmax[t * nvf + j] = fid[j] < gid[k] ? gid[k] : fid[j];
  }
}

__global__ void k_pf_iota(ll *__restrict__ lab, ll n) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) lab[i] = i;
}

// hook: both ends of a pair, and their current labels, take the smaller
// label.  lab is read and written by other threads: no __restrict__, so no
// read-only loads.
__global__ void k_pf_hook(const ll *__restrict__ pmin, const ll *__restrict__ pmax, ll n,
                          unsigned long long *lab, int *changed) {
  ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const ll a = pmin[t], b = pmax[t];
  const unsigned long long la = lab[a], lb = lab[b];
  if (la == lb) return;
  const unsigned long long m = la < lb ? la : lb;
  atomicMin(&lab[a], m);
  atomicMin(&lab[b], m);
  atomicMin(&lab[la], m);
  atomicMin(&lab[lb], m);
  *changed = 1;
}

// pointer jumping: a label never points above itself
__global__ void k_pf_jump(unsigned long long *lab, ll n, int *changed) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long l = lab[i];
  for (int it = 0; it < 64; it++) {
    const unsigned long long l2 = lab[l];
    if (l2 >= l) break;
    l = l2;
  }
  if (l != lab[i]) {
    lab[i] = l;
    *changed = 1;
  }
}

__global__ void k_pf_roots(const ll *__restrict__ lab, ll n, int *__restrict__ root) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) root[i] = lab[i] == i;
}

__global__ void k_pf_apply(ll *__restrict__ ids, ll np, const ll *__restrict__ lab,
                           const ll *__restrict__ rank) {
  ll p = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < np) ids[p] = rank[lab[ids[p]]];
}

__global__ void k_pf_plus_one(const ll *__restrict__ ids, ll n, long long *__restrict__ out) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = ids[i] + 1;
}

}  // namespace

void plus_one(const ll *d_ids, ll n, long long *d_out) {
  if (n <= 0) return;
  k_pf_plus_one<<<grid_for(n, 256), 256, 0, ctx().stream>>>(d_ids, n, d_out);
  CK_LAUNCH();
}

int periodic_device(ll *d_ids, const double *d_x0, const double *d_x1, const double *d_x2,
                    ll nel, int ndim, ll nseg, const long long *pinfo, int npf, SortWs &sws,
                    ll *nseg_out) {
  cudaStream_t st = ctx().stream;
  const int nv = ndim == 3 ? 8 : 4, nvf = nv / 2, nfaces = ndim == 3 ? 6 : 4;
  const ll np = nel * nv;
  if (nseg_out) *nseg_out = nseg;
  if (np == 0) return PARRSB_OK;
  DBuf<int> flags(4);  // 0 bad record, 1 pair count, 2 mismatch, 3 changed
  CK(cudaMemsetAsync(flags.p, 0, 4 * sizeof(int), st));
  ll npairs = 0;
  DBuf<ll> pmin, pmax;
  if (npf > 0) {
    DBuf<long long> d_pinfo((size_t)npf * 4);
    h2d(d_pinfo.p, pinfo, (size_t)npf * 4);
    DBuf<u64> ekey((size_t)npf), fkey((size_t)npf);
    DBuf<int> eidx((size_t)npf), fidx((size_t)npf), pos((size_t)npf);
    DBuf<ll> self((size_t)npf), partner((size_t)npf);
    k_pf_decode<<<grid_for(npf, 256), 256, 0, st>>>(d_pinfo.p, npf, nel, nfaces, ekey.p, eidx.p,
                                                     fkey.p, fidx.p, self.p, partner.p,
                                                     flags.p);
    CK_LAUNCH();
    int bad = 0;
    d2h(&bad, flags.p, 1);
    sync();
    if (bad) return PARRSB_ERR_ARGS;
    seg_sort_pairs(ekey, eidx, npf, nullptr, 1, sws);  // boundary order: by element
    k_pf_rank<<<grid_for(npf, 256), 256, 0, st>>>(eidx.p, npf, pos.p);
    CK_LAUNCH();
    seg_sort_pairs(fkey, fidx, npf, nullptr, 1, sws);  // lookup table by (element, face)
    // a face pairs with every earlier face holding its partner's key; the
    // count is read back and the buffer grown when repeated records exceed npf
    int cap = npf;
    DBuf<int2> pairs;
    for (int attempt = 0; attempt < 2; attempt++) {
      pairs.ensure((size_t)cap);
      CK(cudaMemsetAsync(flags.p + 1, 0, sizeof(int), st));
      k_pf_pairs<<<grid_for(npf, 256), 256, 0, st>>>(fkey.p, fidx.p, npf, partner.p, pos.p,
                                                     flags.p + 1, pairs.p, cap);
      CK_LAUNCH();
      int hn = 0;
      d2h(&hn, flags.p + 1, 1);
      sync();
      npairs = hn;
      if (hn <= cap) break;
      cap = hn;
    }
    if (npairs > 0) {
      pmin.ensure((size_t)npairs * nvf);
      pmax.ensure((size_t)npairs * nvf);
      k_pf_match<<<grid_for(npairs, 128), 128, 0, st>>>(pairs.p, (int)npairs, self.p, d_ids,
                                                        d_x0, d_x1, d_x2, ndim, pmin.p,
                                                        pmax.p, flags.p + 2);
      CK_LAUNCH();
      int mism = 0;
      d2h(&mism, flags.p + 2, 1);
      sync();
      if (mism) return PARRSB_ERR_CHECK;
    }
  }
  // class minimum of every id under the matched pairs
  DBuf<ll> lab((size_t)nseg);
  k_pf_iota<<<grid_for(nseg, 256), 256, 0, st>>>(lab.p, nseg);
  CK_LAUNCH();
  const ll ne = npairs * nvf;
  if (ne > 0) {
    unsigned long long *ul = reinterpret_cast<unsigned long long *>(lab.p);
    int it = 0;
    for (; it < 100000; it++) {
      CK(cudaMemsetAsync(flags.p + 3, 0, sizeof(int), st));
      k_pf_hook<<<grid_for(ne, 256), 256, 0, st>>>(pmin.p, pmax.p, ne, ul, flags.p + 3);
      CK_LAUNCH();
      k_pf_jump<<<grid_for(nseg, 256), 256, 0, st>>>(ul, nseg, flags.p + 3);
      CK_LAUNCH();
      int ch = 0;
      d2h(&ch, flags.p + 3, 1);
      sync();
      if (!ch) break;
    }
    if (it == 100000) throw ArgError{PARRSB_ERR_CHECK, "periodic renumbering did not settle"};
  }
  // consecutive renumbering of the class minima
  DBuf<int> root((size_t)nseg);
  DBuf<ll> rank((size_t)nseg);
  k_pf_roots<<<grid_for(nseg, 256), 256, 0, st>>>(lab.p, nseg, root.p);
  CK_LAUNCH();
  ll nroot = exclusive_scan_int_to_ll(root.p, rank.p, nseg);
  k_pf_apply<<<grid_for(np, 256), 256, 0, st>>>(d_ids, np, lab.p, rank.p);
  CK_LAUNCH();
  if (nseg_out) *nseg_out = nroot;
  return PARRSB_OK;
}

}  // namespace prsb
