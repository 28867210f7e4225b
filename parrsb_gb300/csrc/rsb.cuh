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

// A level's graph: the dual graph restricted to the current groups and
// re-indexed into the current element order, as sliced ELL (slices of 32
// consecutive rows, column-major inside a slice, one packed uint32 per
// entry: column in bits 0-27, weight in bits 28-31; padding entries have
// weight 0).
struct Level {
  DBuf<unsigned> ell;
  DBuf<ll> slice_off;
  DBuf<int> slice_w;
  ll nnz = 0;    // restricted nonzeros of the active rows
  ll rows = 0;   // active rows
  int max_w = 0; // widest slice
};

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
  // Start vector of every Lanczos run: 0 the reference's step vector
  // (src/fiedler.c:574-578), 1 a seeded random vector.  With warm != 0 the
  // learned warm start is judged against it per group (lower FP64
  // eigen-residual wins) for groups of at least warm_min elements.
  int start = 0;
  int warm = 0;
  ll warm_min = 0;
  // Stopping rule: 0 the reference's (a restart ends when the CG residual
  // falls below tol times its start, src/fiedler.c:448,500, or after miter
  // steps; Lanczos ends after a restart that needed fewer than miter steps);
  // 1 also restart until the Ritz vector's FP64 eigen-residual
  // ||L f - rho f|| / ||f|| is at most tol (or mpass restarts).
  int resid_stop = 0;
  // reorthogonalise every new Lanczos residual against the earlier ones
  // (classical Gram-Schmidt, FP64 coefficients)
  int reorth = 0;
  // with resid_stop: a restart's own CG exit at tol * cg_factor (a tighter
  // exit makes every restart count: at the same tol restarts end after a
  // step or two once the vector is close, without improving it)
  double cg_factor = 0.1;
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

// Elements of groups given per element (group_of[e] in [0, ngroups), or < 0
// for none), ordered by group (stable: element order inside a group), with
// the level graph of the groups: perm[i] = element at position i, grp[i] =
// its group (-1 after the grouped elements), group g at positions
// [gstart[g], gstart[g] + gn[g]).
struct GroupLevel {
  DBuf<int> perm, grp;
  std::vector<ll> gstart, gn;
  Level lv;
  ll N = 0;
};
void build_group_level(const long long *d_vtx, ll N, int nv, const int *d_group_of,
                       int ngroups, GroupLevel &out);

// Components of every part (part[e] in [0, nparts)): the part-ordered
// level graph in gl and, per position of gl.perm, the label of its
// component (the smallest position of the component).
void part_component_labels(const long long *d_vtx, ll N, int nv, const int *d_part, int nparts,
                           GroupLevel &gl, DBuf<int> &labels);

// options.repair = 1: every part keeps its largest component; each other
// component moves to the neighbouring part it shares the most dual-graph
// weight with (ties: smallest part); isolated components stay.  d_part is
// updated in place.
void repair_parts_device(const long long *d_vtx, ll N, int nv, int nparts, int *d_part,
                         long long *moved_components, long long *moved_elements);

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
