/*
 * parrsb.h -- drop-in C ABI of the GB300 partitioning library.
 *
 * The two entry points keep the names, argument order, argument meaning,
 * ownership rules and return codes of parRSB's public header
 * (src/parRSB.h:21-48 and src/parRSB.h:62-70).  The one change is the
 * communicator: an MPI_Comm argument becomes an explicit part count
 * (`nparts`), because the whole mesh lives on one GPU and the reference's
 * "one MPI rank per part" becomes "one virtual rank per part".
 *
 * All pointers are caller-owned HOST memory unless an entry point's name
 * ends in `_device`, in which case they are device pointers on the current
 * CUDA device.  Outputs are written only on success (return value 0).
 * Every call runs on the CUDA device that is current when it is made; the
 * library keeps one stream and one cached workspace per host thread and
 * device, so a thread may change device between calls.
 *
 * Return codes (the reference returns 0 / 1 / the gencon check error and
 * otherwise aborts the process; this library never exits):
 *   PARRSB_OK            0  success
 *   PARRSB_ERR_ARGS      1  bad arguments (also: tagged == 1 with tag NULL,
 *                           as in src/parrsb.c:873-877; tagged with nparts
 *                           not a multiple of the number of tags, where the
 *                           reference exits; gencon: element or face check
 *                           failed, as in src/con.c:238-257; a periodic face
 *                           record out of range)
 *   PARRSB_ERR_CUDA      2  a CUDA call failed (message on stderr)
 *   PARRSB_ERR_CHECK     3  an internal consistency check failed (also:
 *                           paired periodic faces that do not coincide,
 *                           where the reference exits)
 *   PARRSB_ERR_UNSUPPORTED 4 option outside the GPU path (rsb_algo = 1
 *                           multigrid; tagged with a partitioner other than
 *                           0, 1, 2)
 */
#ifndef PARRSB_GB300_H
#define PARRSB_GB300_H

#if defined(__GNUC__)
#define PARRSB_API __attribute__((visibility("default")))
#else
#define PARRSB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define PARRSB_OK 0
#define PARRSB_ERR_ARGS 1
#define PARRSB_ERR_CUDA 2
#define PARRSB_ERR_CHECK 3
#define PARRSB_ERR_UNSUPPORTED 4

/* Byte-identical to parrsb_options in src/parRSB.h:21-41 (14 ints and one
 * double, same field order).  Environment variables PARRSB_<FIELD> override
 * the caller's values and are written back into the struct, as in
 * update_options (src/parrsb.c:48-77). */
typedef struct {
  int partitioner;             /* 0 RSB, 1 RCB, 2 RIB (default 0) */
  int tagged;                  /* tagged partitioning: tag[e] groups elements */
  int levels;                  /* 1 or 2; clamped to <= 2 (default 2) */
  int find_disconnected_comps; /* count components per bisection (1) */
  int repair;                  /* 1: repair disconnected parts after the
                                  partition (no counterpart in the reference,
                                  which parses it and does nothing; 0) */
  int verbose_level;           /* 0 quiet, >=1 prints options and time (1) */
  int profile_level;           /* >=1 prints per-level stage times (0) */
  int rsb_algo;                /* 0 Lanczos (1 = multigrid: unsupported) */
  int rsb_pre;                 /* 0 none, 1 RCB, 2 RIB pre-partition (1) */
  int rsb_max_iter;            /* Lanczos steps per restart (50) */
  int rsb_max_passes;          /* Lanczos restarts (50) */
  double rsb_tol;              /* Lanczos tolerance (1e-5) */
  int rsb_dump_stats;          /* accepted, no effect (as in the reference) */
  int rsb_mg_grammian;         /* multigrid only: accepted, no effect */
  int rsb_mg_factor;           /* multigrid only: accepted, no effect */
} parrsb_options;

/* Defaults of src/parrsb.c:26-44. */
extern PARRSB_API parrsb_options parrsb_default_options;

/* Partition `nel` elements of `nv` vertices (nv == 8: hex, 3D; otherwise
 * quad, 2D) into `nparts` parts; part[e] receives the part of element e.
 * Replaces parrsb_part_mesh (src/parRSB.h:45-48, src/parrsb.c:853-906);
 * `comm` becomes `nparts`.  vtx: nel*nv global vertex ids (may be NULL for
 * RCB/RIB); xyz: nel*nv*ndim corner coordinates (may be NULL: rsb_pre is then
 * set to 0, as src/parrsb.c:250 does).  With options->tagged == 1 and a
 * tag array (parrsb_part_mesh_v1, src/parrsb.c:379-561): nparts must be a
 * multiple of the number of distinct tags; the elements of the t-th
 * smallest tag, in input order, are partitioned among nparts / ntags parts
 * numbered from t * nparts / ntags, independently of the other tags (all
 * tags run in the same GPU launches). */
PARRSB_API int parrsb_part_mesh(int *part, const long long *vtx, const double *xyz,
                     const int *tag, int nel, int nv, parrsb_options *options,
                     int nparts);

/* Tolerance-based vertex numbering ("gencon").  Replaces parrsb_conn_mesh
 * (src/parRSB.h:62-64, src/con.c:189-295) without the communicator.
 * coord: nel * nv * nDim doubles, corners in Nek preprocessor order;
 * vtx: nel * nv output ids in symmetric corner order (1-based, dense).
 * periodicInfo: nPeriodicFaces records (element, face, partner element,
 * partner face), 1-based, faces in preprocessor numbering; paired faces'
 * corners are merged (match_periodic_faces, src/con-periodic.c:245-288).
 * Returns 1 when the element or face check fails or a record is out of
 * range, 3 when paired faces do not coincide (vtx is then untouched). */
PARRSB_API int parrsb_conn_mesh(long long *vtx, double *coord, unsigned int nel,
                     unsigned nDim, long long *periodicInfo,
                     int nPeriodicFaces, double tol);

/* Fortran binding of parrsb_conn_mesh (src/parRSB.h:66-70, src/con.c:300-306)
 * with the communicator argument removed; *err receives the return code. */
PARRSB_API void fparrsb_conn_mesh(long long *vtx, double *coord, int *nel, int *nDim,
                       long long *periodicInfo, int *nPeriodicFaces,
                       double *tol, int *err);

/* Mesh files (src/parRSB.h:75-83, src/io.c), read and written by one host
 * process instead of MPI-IO.  parrsb_read_mesh reads <name>.re2 (read & 1:
 * corner coordinates in preprocessor order, periodic faces as (eid, fid, e1,
 * e2)) and/or <name>.co2 (read & 2: vertex ids); outputs are malloc'ed and
 * owned by the caller.  parrsb_dump_con writes <name>.co2.  parrsb_dump_map
 * writes <name>.ma2; it takes the part array explicitly because there is no
 * per-rank element distribution to take it from. */
PARRSB_API int parrsb_read_mesh(unsigned *nel, unsigned *nv, long long **vl, double **coord,
                                unsigned *nbcs, long long **bcs, char *name, int read);
PARRSB_API int parrsb_dump_con(char *name, unsigned nelt, unsigned nv, long long *vl);
PARRSB_API int parrsb_dump_map(char *name, unsigned nelt, unsigned nv, long long *vtx,
                               const int *part);

/* ------------------------------------------------------------------------
 * Extensions (no counterpart in the reference).
 * ---------------------------------------------------------------------- */

/* parrsb_part_mesh that also returns seq[e], the position of element e
 * inside part[e] in the final element order (the `seq` output documented in
 * the reference's README.md:46-66).  For RCB / RIB this order is the one
 * rcb_local / rib_local leave (src/rcb.c:39-72, src/rib.c:58-74); for RSB it
 * is the order after the last bisection. */
PARRSB_API int parrsb_part_mesh_seq(int *part, int *seq, const long long *vtx,
                                    const double *xyz, const int *tag, int nel, int nv,
                                    parrsb_options *options, int nparts);

/* Same as parrsb_part_mesh / parrsb_conn_mesh with every array a DEVICE
 * pointer on the current device (inputs already resident in HBM). */
PARRSB_API int parrsb_part_mesh_device(int *d_part, const long long *d_vtx,
                            const double *d_xyz, int nel, int nv,
                            parrsb_options *options, int nparts);
PARRSB_API int parrsb_conn_mesh_device(long long *d_vtx, const double *d_coord,
                            unsigned int nel, unsigned nDim, double tol);

/* Statistics of the last parrsb_part_mesh / parrsb_conn_mesh call on this
 * thread.  Stage times come from CUDA events; counts from device state. */
typedef struct {
  double total_ms;        /* whole call, host-measured */
  double stage_ms[12];    /* see PARRSB_STAGE_* */
  long long lanczos_iters;    /* sum over all bisections of Lanczos steps */
  long long lanczos_row_iters;/* sum over bisections of steps * rows */
  long long spmv_launches;    /* SpMV kernel launches */
  double spmv_ms;             /* summed CUDA-event time of SpMV launches */
  long long spmv_bytes;       /* algorithmic bytes moved by those launches */
  long long kernel_launches;  /* all kernels launched by the call */
  int levels;                 /* bisection levels run */
  int max_components;         /* max component count over all halves */
  double max_fiedler_resid;   /* max FP64 ||Lf - rho f|| / ||f|| (if checked) */
  int unconverged;            /* bisections that used all restarts */
  long long nnz;              /* off-diagonal nonzeros of the dual graph */
  long long gencon_segments;  /* gencon: number of distinct ids */
  double lanczos_ms[6];       /* timing mode: p update, r update, eigensolve,
                                 Ritz vector, pass set-up, host per pass */
  long long lanczos_passes;   /* graph launches (Lanczos restarts of a level) */
  long long warm_tried;       /* groups whose learned warm start was judged */
  long long warm_used;        /* of those, groups that started from it */
  double warm_ms;             /* warm-start network inference (all levels) */
  double start_resid_fallback;/* geometric mean of the judged groups' start */
  double start_resid_warm;    /*   residuals: fallback and learned starts */
  long long level_steps[16];  /* Lanczos steps per bisection level (last: 15+) */
  long long repair_components;/* repair = 1: components moved to another part */
  long long repair_elements;  /*   and their elements */
  double lanczos_host_ms[4];  /* host clock: start vectors (prediction +
                                 judge), pass graph capture + instantiation,
                                 the restart loop, the FP64 residual check +
                                 download of each level */
} parrsb_stats;

enum {
  PARRSB_STAGE_UPLOAD = 0,
  PARRSB_STAGE_SETUP = 1,     /* centroids, dual graph */
  PARRSB_STAGE_PRE = 2,       /* RCB / RIB pre-partition */
  PARRSB_STAGE_LANCZOS = 3,
  PARRSB_STAGE_TQLI = 4,      /* tridiagonal solves + Ritz vectors */
  PARRSB_STAGE_SORT = 5,      /* Fiedler sort + split */
  PARRSB_STAGE_COMPONENTS = 6,
  PARRSB_STAGE_BALANCE = 7,
  PARRSB_STAGE_RESTRICT = 8,  /* per-level graph restriction */
  PARRSB_STAGE_DOWNLOAD = 9,
  PARRSB_STAGE_GENCON = 10,
  PARRSB_STAGE_CHECK = 11
};

PARRSB_API int parrsb_get_stats(parrsb_stats *out);

/* Batched level solve: the Fiedler vector of every group of elements
 * (group[e] in [0, ngroups); a group's elements in element order define its
 * start vector, as the current order does inside RSB).  All groups run in
 * the same kernel launches when batched != 0, one group at a time
 * otherwise.  fiedler[e]: normalised Fiedler value of element e (0 for
 * groups of one element); iters[g] / resid[g]: Lanczos steps and FP64
 * eigen-residual ||L f - rho f|| / ||f|| of group g (may be NULL).  Uses
 * rsb_max_iter, rsb_max_passes and rsb_tol of *options (environment
 * overrides applied).  Host arrays. */
PARRSB_API int parrsb_fiedler_groups(double *fiedler, long long *iters, double *resid,
                                     const long long *vtx, const int *group, int nel,
                                     int nv, int ngroups, parrsb_options *options,
                                     int batched);

/* Partition quality on the element dual graph (weight = shared vertices):
 * q[0] weighted edge cut, q[1] cut dual edges, q[2] cut face-sharing pairs,
 * q[3] max part size, q[4] min part size, q[5] imbalance max*nparts/nel,
 * q[6] shared-vertex communication volume summed over parts (the `nss`
 * figure of src/helpers.c:132-224), q[7] max neighbour parts of a part.
 * Host arrays; computed on the GPU. */
PARRSB_API int parrsb_part_quality(double *q, const int *part, const long long *vtx,
                        int nel, int nv, int nparts);

/* The element dual graph that RSB's Laplacian is built on (two elements are
 * adjacent when they share a vertex id; the weight is the number of
 * (corner, corner) pairs with equal ids), built on the GPU: the matrix of
 * gs_weighted_init / gs_weighted (src/laplacian.c:159-205) and of the CSR
 * Laplacian (src/mat.c:17-61), without the diagonal.  rowptr[nel + 1] is
 * always written and *nnz receives the number of entries; col / weight
 * (0-based element index, weight) are written, row by row with each row in
 * the order of its first shared vertex, when neither is NULL and
 * cap >= *nnz.  Host arrays. */
PARRSB_API int parrsb_dual_graph(long long *rowptr, int *col, unsigned char *weight,
                                 long long *nnz, long long cap, const long long *vtx, int nel,
                                 int nv);

/* Number of vertex-connected components of each group of elements
 * (get_components_v2, src/components.c:160-328, count only): group[e] in
 * [0, ngroups), or negative to leave element e out; ncomp[g] receives the
 * count of group g (0 for an empty group).  The same GPU kernels as the
 * component check of each bisection.  Host arrays. */
PARRSB_API int parrsb_components(int *ncomp, const long long *vtx, const int *group, int nel,
                                 int nv, int ngroups);

/* ------------------------------------------------------------------------
 * Learned warm start (no counterpart in the reference, which starts every
 * Lanczos run from a step vector in the current element order,
 * src/fiedler.c:574-578).  A three-layer message-passing network (width 64,
 * BF16 weights and activations, FP32 accumulation on the tensor cores)
 * predicts each group's Fiedler vector from its elements' centroids (in the
 * group's principal frame) and weighted degrees, over the graph Lanczos
 * itself multiplies by.  With PARRSB_GPU_WARM=1, RSB judges the prediction
 * of every group of at least PARRSB_GPU_WARM_MIN elements against the
 * fallback start (PARRSB_GPU_START: 0 the reference's step vector, 1 a
 * seeded random vector) by their FP64 eigen-residuals ||L f - rho f|| /
 * ||f|| and starts Lanczos from the better one; Lanczos then iterates to
 * rsb_tol as usual.  The network is installed per device with
 * parrsb_warm_install, or read from the raw FP32 file named by
 * PARRSB_GPU_WARM_WEIGHTS.  The batch entry points train it on the GPU with
 * the same kernels (device pointers on the current device).
 * ---------------------------------------------------------------------- */
#define PARRSB_WARM_NPARAM 17665

/* Install the network's parameters (host FP32, PARRSB_WARM_NPARAM values:
 * W1[16][64], b1[64], W2[128][64], b2[64], W3[128][64], b3[64], wo[64], bo)
 * for the current device. */
PARRSB_API int parrsb_warm_install(const float *params);

typedef struct parrsb_warm_batch parrsb_warm_batch;

/* A training batch: the elements of each group (d_group[e] in [0, ngroups))
 * form one mesh; its graph and input features are built once.  d_vtx:
 * nel * nv vertex ids, d_xyz: nel * nv * ndim corner coordinates. */
PARRSB_API int parrsb_warm_batch_create(parrsb_warm_batch **batch, const long long *d_vtx,
                                        const double *d_xyz, const int *d_group, int nel,
                                        int nv, int ngroups);
PARRSB_API int parrsb_warm_batch_destroy(parrsb_warm_batch *batch);

/* The batch's input features, nel x 8 FP32 in element order. */
PARRSB_API int parrsb_warm_batch_features(parrsb_warm_batch *batch, float *d_feat);

/* Forward pass with parameters d_params (device FP32); d_pred (optional):
 * the prediction per element.  With d_label (per element, FP64): the mean
 * over groups of the sign-invariant loss 1 - cos^2(prediction, label) (both
 * centred) in *loss and, if d_grad is not NULL, its gradient with respect to
 * every parameter (device FP32, PARRSB_WARM_NPARAM values). */
PARRSB_API int parrsb_warm_batch_step(parrsb_warm_batch *batch, const float *d_params,
                                      const double *d_label, float *d_grad, float *d_pred,
                                      double *loss);

/* One Adam step (beta1 0.9, beta2 0.999, eps 1e-8; step >= 1) on n device
 * parameters with moment buffers d_m, d_v. */
PARRSB_API int parrsb_warm_adam(float *d_params, float *d_m, float *d_v, const float *d_grad,
                                int n, int step, float lr);

/* Release the device workspace cached by earlier calls on this thread. */
PARRSB_API void parrsb_gpu_finalize(void);

/* RCB partition (same result as parrsb_part_mesh with partitioner = 1) of a
 * mesh of at most 8192 elements that allocates nothing: no cudaMalloc /
 * cudaFree and no allocating library call.  No counterpart in the
 * reference.  For callers that cannot allocate device memory during the
 * call: their device memory comes from their own pool or arena, or a
 * long-running loop must not grow or fragment the device heap.  Every
 * intermediate lives in one fixed file-scope device array (about 512 KB per
 * device).
 *   d_part  device int[nel], written;  d_xyz device double[nel][nv][ndim]
 *   stream  cudaStream_t to run on (NULL: the legacy default stream); the
 *           result is ready when the stream reaches it (no synchronisation).
 * Returns PARRSB_ERR_UNSUPPORTED for nel > 8192 (nothing is launched),
 * PARRSB_ERR_ARGS for bad arguments, PARRSB_ERR_CUDA for a launch error.
 * The first call on a device (nel = 0 does only this) resolves the scratch
 * address and sets a kernel attribute; make it before any stream capture.
 * The scratch is shared by every call on a device: calls that overlap in
 * time (other streams, other threads) race on it and must be serialised by
 * the caller.  The call returns before its kernels finish, so two calls made
 * one after the other on the host but on different streams also overlap on
 * the device: order them (cudaEventRecord on the first stream, then
 * cudaStreamWaitEvent on the second) or use one stream. */
PARRSB_API int parrsb_part_mesh_rcb_noalloc(int *d_part, const double *d_xyz, int nel, int nv,
                                            int nparts, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* PARRSB_GB300_H */
