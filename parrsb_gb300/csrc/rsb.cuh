// rsb.cuh -- recursive spectral bisection on one GPU.
#pragma once
#include <vector>
#include "bisect.cuh"

namespace prsb {

// Element dual graph in original element order (CSR).  Weight of (a, b) =
// number of (corner of a, corner of b) pairs with the same vertex id.
struct Graph {
  DBuf<ll> rowptr;
  DBuf<int> col;
  DBuf<unsigned char> w;
  ll n = 0, nnz = 0;
  int max_row = 0, max_w = 0;
};

void build_dual_graph(const long long *d_vtx, ll nel, int nv, Graph &g,
                      SortWs &sws);

struct RsbOpts {
  int pre = 1;          // 0 none, 1 RCB, 2 RIB
  int miter = 50;
  int mpass = 50;
  double tol = 1e-5;
  int find_comps = 1;
  int fp32 = 0;         // FP32 Lanczos vectors (FP64 dots / T / eigensolve)
  int check_resid = 1;  // FP64 eigen-residual of every Fiedler vector
  int profile = 0;
  int use_graphs = 1;   // capture each Lanczos pass in a CUDA graph
  int batched = 1;      // all groups of a level per launch (0: one group at a time)
};

// Starting point of a recursion other than one group of all elements:
// tagged partitioning (src/parrsb.c:379-561) starts from one group per tag.
// perm[i] is the element at position i; group g covers positions
// [start[g], start[g] + n[g]) and is split among p[g] ranks numbered from
// r0[g].
struct StartGroups {
  std::vector<int> perm;
  std::vector<ll> start, n;
  std::vector<int> p, r0;
};

// Partition N elements (vertex ids d_vtx, centroids cent) into P parts, or,
// with sg, each start group into its own ranks.
void rsb_device(const long long *d_vtx, const double *cent, ll N, int nv,
                int P, const RsbOpts &o, int *d_part, int *d_seq = nullptr,
                const StartGroups *sg = nullptr);

// Fiedler vectors of independent element groups: group g is the elements
// e with group_of[e] == g, taken in element order (that order defines the
// start vector, as the current order does inside RSB).  f receives the
// normalised Fiedler vector per element (0 for groups of one element);
// iters / resid (host, ngroups) the Lanczos steps and FP64 eigen-residual.
void fiedler_groups_device(const long long *d_vtx, ll N, int nv,
                           const int *d_group_of, int ngroups,
                           const RsbOpts &o, double *d_f, long long *iters,
                           double *resid);

// Vertex-connected components of each group (group_of[e] < 0: no group);
// counts (host, ngroups) receives the number per group.
void components_device(const long long *d_vtx, ll N, int nv, const int *d_group_of,
                       int ngroups, int *counts);

// The element dual graph as built for RSB (rows in element order, each row's
// columns in first-occurrence order), copied to the host.
void dual_graph_device(const long long *d_vtx, ll N, int nv, std::vector<ll> &rowptr,
                       std::vector<int> &col, std::vector<unsigned char> &w);

// d[i] = i for i < N on the library stream.
void iota_device(int *d, ll N);

// Quality of a partition (see parrsb_part_quality).
void part_quality_device(const long long *d_vtx, const int *d_part, ll N,
                         int nv, int nparts, double *q);

}  // namespace prsb
