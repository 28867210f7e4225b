// quality.cu -- partition quality on the element dual graph.
//
// Edge cut (weighted, pairs, face pairs), part sizes and imbalance, and the
// shared-vertex communication volume that parrsb_get_part_stat reports as
// `nss` (src/helpers.c:132-224): sum over vertices of m (m - 1), where m is
// the number of distinct parts touching the vertex.
#include <algorithm>

#include "rsb.cuh"

namespace prsb {

namespace {

__global__ void k_cut(const ll *__restrict__ rowptr, const int *__restrict__ col,
                      const unsigned char *__restrict__ w, const int *__restrict__ part,
                      ll N, int face_w, unsigned long long *__restrict__ acc,
                      int *__restrict__ cnt_part) {
  ll a = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  int pa = part[a];
  atomicAdd(&cnt_part[pa], 1);
  unsigned long long cw = 0, ce = 0, cf = 0;
  for (ll q = rowptr[a]; q < rowptr[a + 1]; q++) {
    int b = col[q];
    if (b > a && part[b] != pa) {
      cw += w[q];
      ce += 1;
      cf += (w[q] >= face_w);
    }
  }
  if (ce) {
    atomicAdd(&acc[0], cw);
    atomicAdd(&acc[1], ce);
    atomicAdd(&acc[2], cf);
  }
}

// one thread per vertex run: distinct parts m, volume m (m - 1)
__global__ void k_vertex_parts(const int *__restrict__ sorted_slot,
                               const ll *__restrict__ run_start, ll nruns, int nv,
                               const int *__restrict__ part,
                               unsigned long long *__restrict__ vol) {
  ll r = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nruns) return;
  ll b = run_start[r], e = run_start[r + 1];
  unsigned long long m = 0;
  for (ll q = b; q < e; q++) {
    int pq = part[sorted_slot[q] / nv];
    bool seen = false;
    for (ll t = b; t < q && !seen; t++) seen = part[sorted_slot[t] / nv] == pq;
    if (!seen) m++;
  }
  if (m > 1) atomicAdd(vol, m * (m - 1));
}

__global__ void k_cut_pairs(const ll *__restrict__ rowptr, const int *__restrict__ col,
                            const int *__restrict__ part, ll N, int nparts,
                            unsigned long long *__restrict__ npair,
                            u64 *__restrict__ pairs, ll cap) {
  ll a = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= N) return;
  int pa = part[a];
  for (ll q = rowptr[a]; q < rowptr[a + 1]; q++) {
    int pb = part[col[q]];
    if (pb != pa) {
      unsigned long long o = atomicAdd(npair, 1ull);
      if ((ll)o < cap) pairs[o] = (u64)pa * (u64)nparts + (u64)pb;
    }
  }
}

__global__ void k_vid_keys_q(const long long *__restrict__ vtx, ll ns, u64 *__restrict__ keys,
                             int *__restrict__ vals) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns) return;
  keys[i] = (u64)vtx[i] ^ 0x8000000000000000ull;
  vals[i] = (int)i;
}

__global__ void k_runs(const u64 *__restrict__ keys, ll ns, int *__restrict__ flag) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ns) flag[i] = (i == 0 || keys[i] != keys[i - 1]);
}

__global__ void k_run_start(const int *__restrict__ flag, const ll *__restrict__ excl, ll ns,
                            ll nruns, ll *__restrict__ run_start) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns) return;
  if (flag[i]) run_start[excl[i]] = i;
  if (i == ns - 1) run_start[nruns] = ns;
}

}  // namespace

void part_quality_device(const long long *d_vtx, const int *d_part, ll N, int nv, int nparts,
                         double *q) {
  cudaStream_t st = ctx().stream;
  for (int i = 0; i < 8; i++) q[i] = 0.0;
  if (N == 0) return;
  SortWs sws;
  Graph G;
  build_dual_graph(d_vtx, N, nv, G, sws);
  DBuf<unsigned long long> acc(4);
  DBuf<int> cnt((size_t)nparts);
  CK(cudaMemsetAsync(acc.p, 0, 4 * sizeof(unsigned long long), st));
  CK(cudaMemsetAsync(cnt.p, 0, (size_t)nparts * sizeof(int), st));
  k_cut<<<grid_for(N, 256), 256, 0, st>>>(G.rowptr.p, G.col.p, G.w.p, d_part, N,
                                          nv == 8 ? 4 : 2, acc.p, cnt.p);
  CK_LAUNCH();
  // vertex runs
  ll ns = N * nv;
  DBuf<u64> keys((size_t)ns);
  DBuf<int> vals((size_t)ns), flag((size_t)ns);
  DBuf<ll> excl((size_t)ns);
  k_vid_keys_q<<<grid_for(ns, 256), 256, 0, st>>>(d_vtx, ns, keys.p, vals.p);
  CK_LAUNCH();
  seg_sort_pairs(keys, vals, ns, nullptr, 1, sws);
  k_runs<<<grid_for(ns, 256), 256, 0, st>>>(keys.p, ns, flag.p);
  CK_LAUNCH();
  ll nruns = exclusive_scan_int_to_ll(flag.p, excl.p, ns);
  DBuf<ll> run_start((size_t)nruns + 1);
  k_run_start<<<grid_for(ns, 256), 256, 0, st>>>(flag.p, excl.p, ns, nruns, run_start.p);
  CK_LAUNCH();
  k_vertex_parts<<<grid_for(nruns, 256), 256, 0, st>>>(vals.p, run_start.p, nruns, nv, d_part,
                                                        acc.p + 3);
  CK_LAUNCH();
  unsigned long long h[4];
  d2h(h, acc.p, 4);
  std::vector<int> hc(nparts);
  d2h(hc.data(), cnt.p, nparts);
  sync();
  q[0] = (double)h[0], q[1] = (double)h[1], q[2] = (double)h[2], q[6] = (double)h[3];
  int mx = 0, mn = (int)N;
  for (int p = 0; p < nparts; p++) mx = std::max(mx, hc[p]), mn = std::min(mn, hc[p]);
  q[3] = mx, q[4] = mn, q[5] = (double)mx * nparts / (double)N;
  // neighbour parts per part: unique (pa, pb) pairs of cut dual edges
  ll cap = 2 * (ll)h[1] + 16;
  DBuf<u64> pk((size_t)cap);
  DBuf<int> pv((size_t)cap);
  DBuf<unsigned long long> np(1);
  CK(cudaMemsetAsync(np.p, 0, sizeof(unsigned long long), st));
  k_cut_pairs<<<grid_for(N, 256), 256, 0, st>>>(G.rowptr.p, G.col.p, d_part, N, nparts, np.p,
                                                pk.p, cap);
  CK_LAUNCH();
  unsigned long long hn = 0;
  d2h(&hn, np.p, 1);
  sync();
  ll n2 = std::min<ll>((ll)hn, cap);
  if (n2 > 0) {
    std::vector<u64> hp(n2);
    d2h(hp.data(), pk.p, n2);
    sync();
    std::sort(hp.begin(), hp.end());
    std::vector<int> nb(nparts, 0);
    for (ll i = 0; i < n2; i++)
      if (i == 0 || hp[i] != hp[i - 1]) nb[hp[i] / nparts]++;
    int m = 0;
    for (int v : nb) m = std::max(m, v);
    q[7] = m;
  }
}

}  // namespace prsb
