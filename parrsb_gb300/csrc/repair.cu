// repair.cu -- repair of disconnected parts (parrsb_options.repair = 1).
//
// The reference parses the `repair` option and never uses it
// (src/parrsb.c:65); it only counts the components of each bisection's
// halves (src/components.c:160-328).  This library gives the option a
// meaning, applied after the partition is complete:
//   every part keeps its largest vertex-connected component (ties: the one
//   holding the part's first element); every other component of the part
//   moves, whole, to the neighbouring part it shares the largest dual-graph
//   weight with (shared-vertex count; ties: the smallest part number); a
//   component with no neighbour in another part stays.
// One pass: the moved components join their targets as they are.  Part
// sizes change by the moved elements (repair trades exact balance for
// connected parts).  With repair = 0 (the default) nothing runs.
#include "rsb.cuh"

namespace prsb {
namespace {

typedef unsigned long long u64;

// component sizes, indexed by root position
__global__ void k_rp_sizes(const int *__restrict__ lab, ll N, int *__restrict__ size) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) atomicAdd(&size[lab[i]], 1);
}

// per part: the largest component, packed (size << 32) | ~root so that the
// maximum is the largest and, among equal sizes, the smallest root
__global__ void k_rp_largest(const int *__restrict__ lab, const int *__restrict__ grp,
                             const int *__restrict__ size, ll N, u64 *__restrict__ best) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || lab[i] != i || grp[i] < 0) return;
  const u64 key = ((u64)(unsigned)size[i] << 32) | (u64)(0xFFFFFFFFu - (unsigned)i);
  atomicMax(&best[grp[i]], key);
}

__device__ __forceinline__ bool rp_small(int i, const int *lab, const int *grp, const u64 *best) {
  const int g = grp[i];
  if (g < 0) return false;
  const unsigned keep = 0xFFFFFFFFu - (unsigned)(best[g] & 0xFFFFFFFFull);
  return (unsigned)lab[i] != keep;
}

// entries of the cross-part edges of elements outside their part's largest
// component: pass 1 counts per position, pass 2 writes (root << 32 | other
// part, weight) at the scanned offsets
template <bool FILL>
__global__ void k_rp_edges(const int *__restrict__ perm, const int *__restrict__ lab,
                           const int *__restrict__ grp, const u64 *__restrict__ best,
                           const int *__restrict__ part, const ll *__restrict__ rowptr,
                           const int *__restrict__ col, const unsigned char *__restrict__ w,
                           ll N, int *__restrict__ cnt, const ll *__restrict__ off,
                           u64 *__restrict__ keys, int *__restrict__ vals) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int c = 0;
  if (rp_small((int)i, lab, grp, best)) {
    const int e = perm[i];
    const int pe = part[e];
    ll o = FILL ? off[i] : 0;
    for (ll q = rowptr[e]; q < rowptr[e + 1]; q++) {
      const int pf = part[col[q]];
      if (pf == pe) continue;
      if (FILL) {
        keys[o] = ((u64)(unsigned)lab[i] << 32) | (u64)(unsigned)pf;
        vals[o] = (int)w[q];
        o++;
      }
      c++;
    }
  }
  if (!FILL) cnt[i] = c;
}

// sorted entries: sum the weights of equal keys (run heads accumulate with
// integer atomics: exact), then per root keep the best (weight, smallest
// part) by a packed maximum
__global__ void k_rp_runs(const u64 *__restrict__ keys, const int *__restrict__ vals, ll n,
                          int *__restrict__ head_of, int *__restrict__ sum) {
  const ll q = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  ll h = q;
  while (h > 0 && keys[h - 1] == keys[q]) h--;  // runs are short (one root, one part)
  head_of[q] = (int)h;
  atomicAdd(&sum[h], vals[q]);
}

__global__ void k_rp_pick(const u64 *__restrict__ keys, const int *__restrict__ head_of,
                          const int *__restrict__ sum, ll n, u64 *__restrict__ target) {
  const ll q = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n || head_of[q] != q) return;
  const unsigned root = (unsigned)(keys[q] >> 32), pf = (unsigned)(keys[q] & 0xFFFFFFFFull);
  atomicMax(&target[root], ((u64)(unsigned)sum[q] << 32) | (u64)(0xFFFFFFFFu - pf));
}

__global__ void k_rp_apply(const int *__restrict__ perm, const int *__restrict__ lab,
                           const int *__restrict__ grp, const u64 *__restrict__ best,
                           const u64 *__restrict__ target, ll N, int *__restrict__ part,
                           unsigned long long *__restrict__ moved) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || !rp_small((int)i, lab, grp, best)) return;
  const u64 t = target[lab[i]];
  if (t == 0) return;  // no neighbour in another part: stays
  part[perm[i]] = (int)(0xFFFFFFFFu - (unsigned)(t & 0xFFFFFFFFull));
  atomicAdd(&moved[0], 1ull);
  if (lab[i] == i) atomicAdd(&moved[1], 1ull);
}

}  // namespace

void repair_parts_device(const long long *d_vtx, ll N, int nv, int nparts, int *d_part,
                         long long *moved_components, long long *moved_elements) {
  cudaStream_t st = ctx().stream;
  *moved_components = 0, *moved_elements = 0;
  if (N < 2 || nparts < 2) return;
  GroupLevel gl;
  DBuf<int> lab;
  part_component_labels(d_vtx, N, nv, d_part, nparts, gl, lab);
  DBuf<int> size((size_t)N);
  DBuf<u64> best((size_t)nparts);
  CK(cudaMemsetAsync(size.p, 0, (size_t)N * sizeof(int), st));
  CK(cudaMemsetAsync(best.p, 0, (size_t)nparts * sizeof(u64), st));
  k_rp_sizes<<<grid_for(N, 256), 256, 0, st>>>(lab.p, N, size.p);
  CK_LAUNCH();
  k_rp_largest<<<grid_for(N, 256), 256, 0, st>>>(lab.p, gl.grp.p, size.p, N, best.p);
  CK_LAUNCH();
  SortWs sws;
  Graph G;
  build_dual_graph(d_vtx, N, nv, G, sws);
  DBuf<int> cnt((size_t)N);
  DBuf<ll> off((size_t)N + 1);
  k_rp_edges<false><<<grid_for(N, 256), 256, 0, st>>>(
      gl.perm.p, lab.p, gl.grp.p, best.p, d_part, G.rowptr.p, G.col.p, G.w.p, N, cnt.p, nullptr,
      nullptr, nullptr);
  CK_LAUNCH();
  const ll ne = exclusive_scan_int_to_ll(cnt.p, off.p, N);
  if (ne == 0) return;
  DBuf<u64> keys((size_t)ne);
  DBuf<int> vals((size_t)ne), head((size_t)ne), sum((size_t)ne);
  k_rp_edges<true><<<grid_for(N, 256), 256, 0, st>>>(gl.perm.p, lab.p, gl.grp.p, best.p, d_part,
                                                     G.rowptr.p, G.col.p, G.w.p, N, nullptr,
                                                     off.p, keys.p, vals.p);
  CK_LAUNCH();
  seg_sort_pairs(keys, vals, ne, nullptr, 1, sws);
  CK(cudaMemsetAsync(sum.p, 0, (size_t)ne * sizeof(int), st));
  k_rp_runs<<<grid_for(ne, 256), 256, 0, st>>>(keys.p, vals.p, ne, head.p, sum.p);
  CK_LAUNCH();
  DBuf<u64> target((size_t)N);
  CK(cudaMemsetAsync(target.p, 0, (size_t)N * sizeof(u64), st));
  k_rp_pick<<<grid_for(ne, 256), 256, 0, st>>>(keys.p, head.p, sum.p, ne, target.p);
  CK_LAUNCH();
  DBuf<unsigned long long> moved(2);
  CK(cudaMemsetAsync(moved.p, 0, 2 * sizeof(unsigned long long), st));
  k_rp_apply<<<grid_for(N, 256), 256, 0, st>>>(gl.perm.p, lab.p, gl.grp.p, best.p, target.p, N,
                                               d_part, moved.p);
  CK_LAUNCH();
  unsigned long long h[2] = {0, 0};
  d2h(h, moved.p, 2);
  sync();
  *moved_elements = (long long)h[0];
  *moved_components = (long long)h[1];
}

}  // namespace prsb
