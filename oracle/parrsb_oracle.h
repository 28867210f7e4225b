/*
 * parrsb_oracle.h -- CPU restatement of parRSB's partitioning and gencon
 * paths, used ONLY as the parity checker by the tests, by the smoke check and
 * by the CPU baseline leg of the benchmark.  It is test infrastructure: the
 * product library never links, loads or calls it.
 *
 * MPI ranks of the reference become "virtual ranks": a group of p ranks is a
 * contiguous segment of the element order, and every collective becomes a
 * loop over that segment.  Where the reference's result depends on MPI
 * arrival order or on rank count (ties in sorts, FP64 reduction order), a
 * canonical rule is fixed here and shared with the GPU implementation:
 *   - every sort is stable in the current element order;
 *   - RIB's means and inertia sums use tree_sum (32-wide tiles, shuffle-down
 *     tree, repeated until one value);
 *   - RIB's power iteration starts from (31, 17, 43)/50 instead of rand();
 *   - a Fiedler vector is oriented so that sum_i f_i s_i >= 0, s_i = +1 on
 *     the first half of the group's order and -1 on the second (the
 *     reference's sign is whatever tqli's rotations give).
 * Parity against the real reference is UNPINNED: the reference needs MPI and
 * gslib (neither exists here) and ships no golden outputs for this path.
 */
#ifndef PARRSB_ORACLE_H
#define PARRSB_ORACLE_H

#include "../include/parrsb.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  long long total_iters;   /* Lanczos steps summed over bisections */
  int nbisect;             /* bisections that ran Lanczos */
  int unconverged;         /* bisections that used every restart */
  int max_components;      /* max component count over halves */
  double max_resid;        /* max FP64 ||Lf - rho f||/||f|| over bisections */
  int levels;              /* cuts performed */
  long long row_iters;     /* Lanczos steps x group rows, summed */
} oracle_rsb_info;

/* parrsb_part_mesh with nparts virtual ranks.  order (optional, nel) gets
 * the final element order (concatenation of the parts in rank order). */
int oracle_part_mesh(int *part, int *order, const long long *vtx,
                     const double *xyz, int nel, int nv,
                     parrsb_options *options, int nparts,
                     oracle_rsb_info *info);

/* One RSB level (one cut of every segment; the loop body of rsb,
 * src/rsb.c:276-343) on the element order a[nel].  seg_in: nseg records
 * (start, n, p, r0) as long long; seg_out (room for 2 * nseg records)
 * receives the next level's segments; returns their number.  cent: 3 per
 * element (oracle_centroids).  info (optional) accumulates. */
int oracle_rsb_level(int *a, const long long *seg_in, int nseg, long long *seg_out,
                     const long long *vtx, const double *cent, int nel, int nv,
                     const parrsb_options *o, oracle_rsb_info *info);

/* Host threads used by the oracle (OpenMP builds; 1 otherwise).  n > 0 sets
 * the count; returns the count in effect.  Results do not depend on it. */
int oracle_threads(int n);

/* parrsb_conn_mesh on one rank.  heapsort_mode = 1 restates the reference's
 * per-segment heapsort (src/con-unique-vertices.c:6-58); 0 uses stable sorts
 * (the canonical rule the GPU follows).  ids (optional, nel*nv) receives the
 * 0-based segment ids in sequence order even when a check fails.
 * nseg (optional) receives the number of distinct ids. */
int oracle_conn_mesh(long long *vtx, const double *coord, unsigned int nel,
                     unsigned ndim, double tol, int heapsort_mode,
                     long long *ids, long long *nseg);
/* The same with periodic face records (element, face, partner element,
 * partner face; 1-based, preprocessor face numbering), matched as
 * match_periodic_faces does (src/con-periodic.c:245-288). */
int oracle_conn_mesh_periodic(long long *vtx, const double *coord, unsigned int nel,
                              unsigned ndim, double tol, int heapsort_mode,
                              const long long *pinfo, int npinfo, long long *ids,
                              long long *nseg);

/* Pieces exposed for unit tests. */
void oracle_centroids(double *cent, const double *xyz, int nel, int nv);
double oracle_tree_sum(const double *x, long long n);
int oracle_power_serial(double *y, int N, const double *A);
int oracle_tqli(double *evec, double *eval, int n, const double *diag,
                const double *upper);
/* y = L x on the dual graph of all nel elements (weights = shared slots). */
void oracle_laplacian(double *y, const double *x, const long long *vtx,
                      int nel, int nv);
/* Dual graph CSR: rowptr (nel+1), col/w (nnz) in original element order,
 * columns ascending.  Returns nnz, or -1 if cap is too small. */
long long oracle_dual_graph(long long *rowptr, int *col, int *w,
                            long long cap, const long long *vtx, int nel,
                            int nv);
/* Number of vertex-connected components among elements with mask[e] != 0. */
int oracle_components(const long long *vtx, const int *mask, int nel, int nv);
/* Quality figures, same layout as parrsb_part_quality. */
void oracle_part_quality(double *q, const int *part, const long long *vtx,
                         int nel, int nv, int nparts);
/* Fiedler vector of one connected set of elements by the reference's
 * Lanczos (initv from the given order).  Returns Lanczos steps. */
int oracle_fiedler(double *f, const long long *vtx, int nel, int nv,
                   int miter, int mpass, double tol);

#ifdef __cplusplus
}
#endif

#endif
