// bisect.cuh -- centroids and the segmented coordinate / inertial bisection
// engine (RCB, RIB and their rank-local recursions).
#pragma once
#include "sort.cuh"
#include "util.cuh"

namespace prsb {

// cent[d*N + e] = centroid coordinate d of element e (d < 3; 0 for 2D z):
// sequential sum over the nv corners, then a division by nv.
void compute_centroids(const double *xyz, int nel, int nv, double *cent);

enum BisectKind { BISECT_RCB = 0, BISECT_RIB = 1 };

// The CTA-per-segment RCB recursion on its own, for callers that manage
// every buffer themselves (no allocation, no library stream).  rank / uniq:
// ndim x N order-preserving coordinate ranks (equal values -> equal rank)
// and the coordinate value of each rank; segments of at most rcb_small_max()
// elements.  rcb_small_prepare() sets the kernels' shared-memory limit on the
// current device (once per device, before the first launch).
int rcb_small_max();
cudaError_t rcb_small_prepare();
cudaError_t rcb_small_launch(int *perm, const u32 *rank, const double *uniq, ll N, int ndim,
                             const ll *seg_start, const ll *seg_n, const int *seg_p,
                             const int *seg_r0, ll nseg, bool local, int *part,
                             cudaStream_t stream);

struct BisectWs {
  SortWs sort;
  DBuf<u64> keys;
  DBuf<int> vals;
  DBuf<int> seg_of_pos, seg_of_elem, axis;
  DBuf<double> red_a, red_b, ev;   // reduction partials, eigenvectors
  DBuf<ll> tile_off, child_off;
  DBuf<int> child_cnt;
  SegTable t2;
  // RCB: dense rank of every centroid coordinate per axis (3 x N) and the
  // distinct values by rank (3 x N), built once for the centroids `rank_of`
  DBuf<u32> rank;
  DBuf<double> uniq;
  DBuf<u32> rbox;  // per segment: min rank (3), min complemented rank (3)
  const double *rank_of = nullptr;
  // presorted-list RCB (every axis rank unique): the elements in rank order
  // per axis (3 x N, with the ranks), the per-segment lists and their
  // partition scratch
  DBuf<int> sorted;
  bool unique = false;
  DBuf<int> lists, lists2, oax, oax2, bsum, loc;
  DBuf<u32> pbits;  // lower-child flags, one bit per list position
  DBuf<int> seg_of_pos2;  // the children's segment of every position
  // the group lists and table of the last presorted call (the next call's
  // lists when its segments are their halves), and its segment of every position
  DBuf<int> glists, oseg;
  SegTable gt;
  bool g_ok = false;
  ll g_N = 0;
  int g_ndim = 0;
  DBuf<int> pwpre;  // per flag word: lower flags before it in its tile
  DBuf<unsigned char> side;
  DBuf<ll> split;
};

// Recursive bisection of every segment of `t` (segments tile [0, N) of the
// order `perm`).  A segment with p > 1 virtual ranks is split at
// lower_count(n, p) after a stable sort along its axis (RCB: longest
// bounding-box edge; RIB: dominant inertia eigenvector).  With do_local, a
// segment with p == 1 is then recursively halved at n/2 the same way
// (rcb_local / rib_local), which only reorders it.  On return `perm` holds
// the final order and, if part_of_elem is not null, part_of_elem[e] is the
// rank (r0 of the final segment) of element e.
void bisect_segments(BisectKind kind, DBuf<int> &perm, SegTable &t,
                     const double *cent, ll N, int ndim, bool do_local,
                     int *part_of_elem, BisectWs &ws);

}  // namespace prsb
