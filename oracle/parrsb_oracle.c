/*
 * parrsb_oracle.c -- CPU restatement of parRSB's partitioning (RSB, RCB, RIB)
 * and connectivity (gencon) paths.  TEST INFRASTRUCTURE ONLY: the tests, the
 * smoke check and the benchmark's CPU-baseline leg use it as the parity
 * checker; the product library never links or calls it.
 *
 * Each function names the reference lines (paths inside the parRSB project)
 * whose behaviour it restates.  MPI ranks become virtual ranks: a group of p
 * ranks is a contiguous range [s, s+n) of the current element order, and the
 * element distribution inside a group follows set_proc_from_idx
 * (src/sort.c:48-70).  Canonical rules where the reference is not
 * deterministic or not reproducible without MPI/gslib are listed in
 * parrsb_oracle.h.  Compile with -ffp-contract=off: the reference is ISO C99
 * (Makefile:2), where GCC does not contract a*b+c into an FMA.
 */
#include "parrsb_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef long long ll;

#define SCALAR_TOL 1e-12 /* src/parrsb-impl.h:20 */

/* ------------------------------------------------------------------------ */
/* Host threads (OpenMP when the oracle is built with it).  The reference    */
/* runs one MPI rank per part; here the threads split the work of the       */
/* independent groups of a level, or of one large group's vectors, and     */
/* every result is independent of the thread count:                        */
/*   - element-wise loops write disjoint entries;                          */
/*   - sums over more than RBLK values add fixed blocks of RBLK in order    */
/*     and then the block sums in order (a single block: the plain         */
/*     sequential sum);                                                     */
/*   - recursive bisections run their two halves as tasks on disjoint      */
/*     index ranges with disjoint scratch.                                  */
/* ------------------------------------------------------------------------ */
#define RBLK 65536
#define TASK_MIN 32768

int oracle_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

static int in_parallel(void) {
#ifdef _OPENMP
  return omp_in_parallel();
#else
  return 0;
#endif
}

/* sum_{i<n} f(i) in fixed blocks of RBLK (see above) */
#define BLOCKED_SUM(OUT, N, EXPR)                                               \
  do {                                                                          \
    ll n_ = (N), nb_ = (n_ + RBLK - 1) / RBLK;                                  \
    if (nb_ <= 1) {                                                             \
      double s_ = 0.0;                                                          \
      for (ll i = 0; i < n_; i++) s_ += (EXPR);                                 \
      OUT = s_;                                                                 \
    } else {                                                                    \
      double *pb_ = (double *)malloc((size_t)nb_ * sizeof(double));             \
      _Pragma("omp parallel for schedule(static) if(!in_parallel())")           \
      for (ll b_ = 0; b_ < nb_; b_++) {                                         \
        ll e_ = (b_ + 1) * RBLK < n_ ? (b_ + 1) * RBLK : n_;                    \
        double s_ = 0.0;                                                        \
        for (ll i = b_ * RBLK; i < e_; i++) s_ += (EXPR);                       \
        pb_[b_] = s_;                                                           \
      }                                                                         \
      double t_ = 0.0;                                                          \
      for (ll b_ = 0; b_ < nb_; b_++) t_ += pb_[b_];                            \
      free(pb_);                                                                \
      OUT = t_;                                                                 \
    }                                                                           \
  } while (0)

/* ------------------------------------------------------------------------ */
/* Options: defaults src/parrsb.c:26-44, env overrides src/parrsb.c:48-77.   */
/* ------------------------------------------------------------------------ */
static void oracle_update_options(parrsb_options *o) {
#define UPD(F, S, INT)                                                         \
  do {                                                                         \
    const char *v = getenv(S);                                                 \
    if (v) {                                                                   \
      if (INT)                                                                 \
        o->F = atoi(v);                                                        \
      else                                                                     \
        o->F = atof(v);                                                        \
    }                                                                          \
  } while (0)
  UPD(partitioner, "PARRSB_PARTITIONER", 1);
  UPD(tagged, "PARRSB_TAGGED", 1);
  UPD(levels, "PARRSB_LEVELS", 1);
  UPD(find_disconnected_comps, "PARRSB_FIND_DISCONNECTED_COMPONENTS", 1);
  UPD(repair, "PARRSB_REPAIR", 1);
  UPD(verbose_level, "PARRSB_VERBOSE_LEVEL", 1);
  UPD(profile_level, "PARRSB_PROFILE_LEVEL", 1);
  UPD(rsb_algo, "PARRSB_RSB_ALGO", 1);
  UPD(rsb_pre, "PARRSB_RSB_PRE", 1);
  UPD(rsb_max_iter, "PARRSB_RSB_MAX_ITER", 1);
  UPD(rsb_max_passes, "PARRSB_RSB_MAX_PASSES", 1);
  UPD(rsb_tol, "PARRSB_RSB_TOL", 0);
  UPD(rsb_mg_grammian, "PARRSB_RSB_MG_GRAMMIAN", 1);
  UPD(rsb_mg_factor, "PARRSB_RSB_MG_FACTOR", 1);
#undef UPD
}

/* ------------------------------------------------------------------------ */
/* Stable merge sort of an index range by double keys (numeric order, so    */
/* -0.0 == +0.0).  Stands in for gslib's stable sorts (src/sort.c:72-104).  */
/* ------------------------------------------------------------------------ */
static void msort(int *a, int *tmp, ll n, const double *key) {
  if (n < 2) return;
  for (ll width = 1; width < n; width *= 2) {
    for (ll lo = 0; lo < n; lo += 2 * width) {
      ll mid = lo + width < n ? lo + width : n;
      ll hi = lo + 2 * width < n ? lo + 2 * width : n;
      ll i = lo, j = mid, k = lo;
      while (i < mid && j < hi) {
        if (key[a[j]] < key[a[i]])
          tmp[k++] = a[j++];
        else
          tmp[k++] = a[i++];
      }
      while (i < mid) tmp[k++] = a[i++];
      while (j < hi) tmp[k++] = a[j++];
    }
    memcpy(a, tmp, (size_t)n * sizeof(int));
  }
}

/* Stable sort by an integer key (used for the sort by globalId). */
static void msort_int(int *a, int *tmp, ll n) {
  if (n < 2) return;
  for (ll width = 1; width < n; width *= 2) {
    for (ll lo = 0; lo < n; lo += 2 * width) {
      ll mid = lo + width < n ? lo + width : n;
      ll hi = lo + 2 * width < n ? lo + 2 * width : n;
      ll i = lo, j = mid, k = lo;
      while (i < mid && j < hi) {
        if (a[j] < a[i])
          tmp[k++] = a[j++];
        else
          tmp[k++] = a[i++];
      }
      while (i < mid) tmp[k++] = a[i++];
      while (j < hi) tmp[k++] = a[j++];
    }
    memcpy(a, tmp, (size_t)n * sizeof(int));
  }
}

/* ------------------------------------------------------------------------ */
/* Element centroids: load_balance, src/parrsb.c:139-145 (sequential sum over */
/* the corners, then a division by nv).                                      */
/* ------------------------------------------------------------------------ */
void oracle_centroids(double *cent, const double *xyz, int nel, int nv) {
  int ndim = (nv == 8) ? 3 : 2;
  for (ll e = 0; e < nel; e++) {
    double c[3] = {0.0, 0.0, 0.0};
    if (xyz) {
      for (int v = 0; v < nv; v++)
        for (int n = 0; n < ndim; n++) c[n] += xyz[e * ndim * nv + v * ndim + n];
      for (int n = 0; n < ndim; n++) c[n] /= nv;
    }
    cent[3 * e + 0] = c[0], cent[3 * e + 1] = c[1], cent[3 * e + 2] = c[2];
  }
}

/* Number of elements held by the first h = ceil(p/2) of p ranks after a
 * balanced parallel sort of n elements: set_proc_from_idx, src/sort.c:48-70
 * (the first p - nrem ranks get n/p elements, the rest one more). */
static ll lower_count(ll n, int p) {
  ll h = (p + 1) / 2;
  ll nelt = n / p, nrem = n - (ll)p * nelt;
  if (nrem == 0) return h * nelt;
  ll s = p - nrem;
  return h * nelt + (h > s ? h - s : 0);
}

/* Canonical tree sum shared with the GPU: tiles of 32 consecutive values
 * (padded with +0.0) reduced by the shuffle-down tree (offsets 16..1), the
 * tile sums reduced the same way until one value is left. */
double oracle_tree_sum(const double *x, ll n) {
  if (n <= 0) return 0.0;
  double *buf = (double *)malloc((size_t)n * sizeof(double));
  memcpy(buf, x, (size_t)n * sizeof(double));
  do {
    ll m = (n + 31) / 32;
    for (ll t = 0; t < m; t++) {
      double v[32];
      for (int i = 0; i < 32; i++) v[i] = (t * 32 + i < n) ? buf[t * 32 + i] : 0.0;
      for (int off = 16; off > 0; off >>= 1)
        for (int i = 0; i < off; i++) v[i] = v[i] + v[i + off];
      buf[t] = v[0];
    }
    n = m;
  } while (n > 1);
  double r = buf[0];
  free(buf);
  return r;
}

/* Power iteration of src/fiedler.c:38-73 with a fixed start vector
 * (31, 17, 43)/50 in place of rand() % 50 / 50 seeded by time(). */
int oracle_power_serial(double *y, int N, const double *A) {
  static const double start[3] = {31.0 / 50.0, 17.0 / 50.0, 43.0 / 50.0};
  double norm = 0.0;
  for (int i = 0; i < N; i++) {
    y[i] = start[i];
    norm += y[i] * y[i];
  }
  double normi = 1.0 / sqrt(norm);
  for (int i = 0; i < N; i++) y[i] *= normi;

  double Ay[3];
  double err = 1.0, lambda = 0.0;
  int i;
  for (i = 0; i < 100; i++) {
    norm = 0.0;
    for (int j = 0; j < N; j++) {
      Ay[j] = 0.0;
      for (int k = 0; k < N; k++) Ay[j] += A[j * N + k] * y[k];
      norm += Ay[j] * Ay[j];
    }
    if (i > 0) err = (sqrt(norm) - lambda) / lambda;
    lambda = sqrt(norm);
    normi = 1.0 / sqrt(norm);
    for (int j = 0; j < N; j++) y[j] = Ay[j] * normi;
    if (fabs(err) < 1e-12) break;
  }
  return i;
}

/* ------------------------------------------------------------------------ */
/* RCB: src/rcb.c.  get_axis_len :7-37, rcb_local :39-72, rcb_level :74-114, */
/* rcb :116-137.                                                             */
/* ------------------------------------------------------------------------ */
static int bbox_axis(const int *a, ll n, const double *cent, int ndim) {
  double mn[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, mx[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
  for (ll i = 0; i < n; i++) {
    const double *c = &cent[3 * (ll)a[i]];
    for (int d = 0; d < ndim; d++) {
      if (c[d] < mn[d]) mn[d] = c[d];
      if (c[d] > mx[d]) mx[d] = c[d];
    }
  }
  double len[3];
  for (int d = 0; d < ndim; d++) len[d] = mx[d] - mn[d];
  int axis = 0;
  for (int d = 1; d < ndim; d++)
    if (len[d] > len[axis]) axis = d;
  return axis;
}

typedef struct {
  const double *cent; /* 3 per element */
  double *key;        /* scratch key per element */
  int *tmp;           /* scratch aligned with the order array a_base */
  const int *a_base;
  int ndim;
} geo_ctx;

/* scratch for the index range starting at a: disjoint ranges get disjoint
 * scratch, so the two halves of a bisection can run at the same time */
#define TMP(g, a) ((g)->tmp + ((a) - (g)->a_base))

static void sort_by_coord(int *a, ll n, geo_ctx *g, int axis) {
  for (ll i = 0; i < n; i++) g->key[a[i]] = g->cent[3 * (ll)a[i] + axis];
  msort(a, TMP(g, a), n, g->key);
}

/* rcb_local (src/rcb.c:39-72): start/end are indices local to the rank. */
static void rcb_local(int *a, ll start, ll end, geo_ctx *g) {
  ll size = end - start;
  if (size <= 1) return;
  int axis = bbox_axis(a + start, size, g->cent, g->ndim);
  sort_by_coord(a + start, size, g, axis);
  ll mid = (start + end) / 2;
#pragma omp task if(size >= TASK_MIN)
  rcb_local(a, start, mid, g);
  rcb_local(a, mid, end, g);
#pragma omp taskwait
}

/* Recursive RCB over virtual ranks; leaves get rcb_local and their rank. */
static void rcb_rec(int *a, ll n, int p, int r0, geo_ctx *g, int *rank_of,
                    int do_local) {
  if (n == 0) return;
  if (p <= 1) {
    if (do_local) rcb_local(a, 0, n, g);
    if (rank_of)
      for (ll i = 0; i < n; i++) rank_of[a[i]] = r0;
    return;
  }
  int axis = bbox_axis(a, n, g->cent, g->ndim);
  sort_by_coord(a, n, g, axis);
  ll L = lower_count(n, p);
  int h = (p + 1) / 2;
#pragma omp task if(n >= TASK_MIN)
  rcb_rec(a, L, h, r0, g, rank_of, do_local);
  rcb_rec(a + L, n - L, p - h, r0 + h, g, rank_of, do_local);
#pragma omp taskwait
}

/* ------------------------------------------------------------------------ */
/* RIB: src/rib.c.  get_rib_axis :6-56 (group sums use tree_sum), rib_local  */
/* :58-74 (sequential sums, as with c == NULL), rib :90-111.                 */
/* ------------------------------------------------------------------------ */
static void rib_keys(int *a, ll n, geo_ctx *g, int tree) {
  double avg[3], I[9];
  double *buf = NULL;
  if (tree) buf = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
  for (int d = 0; d < 3; d++) {
    if (tree) {
      for (ll i = 0; i < n; i++) buf[i] = g->cent[3 * (ll)a[i] + d];
      avg[d] = oracle_tree_sum(buf, n);
    } else {
      avg[d] = 0.0;
      for (ll i = 0; i < n; i++) avg[d] += g->cent[3 * (ll)a[i] + d];
    }
  }
  for (int d = 0; d < 3; d++) avg[d] /= (double)n;
  /* I[j][k] = sum (c_j - avg_j)(c_k - avg_k); I[k][j] is the same value. */
  for (int j = 0; j < 3; j++) {
    for (int k = j; k < 3; k++) {
      double s = 0.0;
      if (tree) {
        for (ll i = 0; i < n; i++) {
          const double *c = &g->cent[3 * (ll)a[i]];
          buf[i] = (c[j] - avg[j]) * (c[k] - avg[k]);
        }
        s = oracle_tree_sum(buf, n);
      } else {
        for (ll i = 0; i < n; i++) {
          const double *c = &g->cent[3 * (ll)a[i]];
          s += (c[j] - avg[j]) * (c[k] - avg[k]);
        }
      }
      I[3 * j + k] = s, I[3 * k + j] = s;
    }
  }
  if (buf) free(buf);
  /* power_serial(ev, ndim, I): for ndim == 2 it reads the first four entries
   * of the row-major 3x3 tensor as a 2x2 matrix (src/rib.c:30-47); ev[2] is
   * defined as 0 here. */
  double ev[3] = {0.0, 0.0, 0.0};
  oracle_power_serial(ev, g->ndim, I);
  for (ll i = 0; i < n; i++) {
    const double *c = &g->cent[3 * (ll)a[i]];
    double x = c[0] - avg[0], y = c[1] - avg[1], z = c[2] - avg[2];
    g->key[a[i]] = x * ev[0] + y * ev[1] + z * ev[2];
  }
}

static void rib_local(int *a, ll start, ll end, geo_ctx *g) {
  ll size = end - start;
  if (size <= 1) return;
  rib_keys(a + start, size, g, 0);
  msort(a + start, TMP(g, a + start), size, g->key);
  ll mid = (start + end) / 2;
#pragma omp task if(size >= TASK_MIN)
  rib_local(a, start, mid, g);
  rib_local(a, mid, end, g);
#pragma omp taskwait
}

static void rib_rec(int *a, ll n, int p, int r0, geo_ctx *g, int *rank_of,
                    int do_local) {
  if (n == 0) return;
  if (p <= 1) {
    if (do_local) rib_local(a, 0, n, g);
    if (rank_of)
      for (ll i = 0; i < n; i++) rank_of[a[i]] = r0;
    return;
  }
  rib_keys(a, n, g, 1);
  msort(a, TMP(g, a), n, g->key);
  ll L = lower_count(n, p);
  int h = (p + 1) / 2;
#pragma omp task if(n >= TASK_MIN)
  rib_rec(a, L, h, r0, g, rank_of, do_local);
  rib_rec(a + L, n - L, p - h, r0 + h, g, rank_of, do_local);
#pragma omp taskwait
}

/* Run a recursive bisection on the calling thread's team: inside a parallel
 * region the tasks join it; outside, a region is opened for them. */
static void rcb_run(int *a, ll n, int p, int r0, geo_ctx *g, int *rank_of, int do_local) {
  if (in_parallel()) {
    rcb_rec(a, n, p, r0, g, rank_of, do_local);
    return;
  }
#pragma omp parallel
#pragma omp single
  rcb_rec(a, n, p, r0, g, rank_of, do_local);
}
static void rib_run(int *a, ll n, int p, int r0, geo_ctx *g, int *rank_of, int do_local) {
  if (in_parallel()) {
    rib_rec(a, n, p, r0, g, rank_of, do_local);
    return;
  }
#pragma omp parallel
#pragma omp single
  rib_rec(a, n, p, r0, g, rank_of, do_local);
}

/* ------------------------------------------------------------------------ */
/* Element dual graph.  The gather-scatter Laplacian of src/laplacian.c:     */
/* 159-205 equals L = D - A with A[a][b] = number of (slot of a, slot of b)  */
/* pairs carrying the same vertex id (b != a) and D = row sums of A; this is */
/* also the matrix of find_nbrs/compress_nbrs (src/mat.c:17-61,203-249).     */
/* ------------------------------------------------------------------------ */
typedef struct {
  ll vid;
  int slot;
} slot_t;

static int cmp_slot(const void *x, const void *y) {
  const slot_t *a = (const slot_t *)x, *b = (const slot_t *)y;
  if (a->vid != b->vid) return a->vid < b->vid ? -1 : 1;
  return a->slot < b->slot ? -1 : (a->slot > b->slot);
}

typedef struct {
  ll n;
  ll *rowptr;
  int *col;
  int *w;
} csr_t;

static void csr_free(csr_t *m) {
  free(m->rowptr), free(m->col), free(m->w);
  m->rowptr = NULL, m->col = NULL, m->w = NULL;
}

/* Stable LSD radix sort of slots by vertex id (16-bit digits; a digit that
 * is the same for every slot is skipped).  Equals qsort by (vid, slot) when
 * the input is in slot order. */
static void radix_slots(slot_t *s, ll n) {
  if (n < 2) return;
  slot_t *t = (slot_t *)malloc((size_t)n * sizeof(slot_t));
  ll *cnt = (ll *)malloc((size_t)65536 * sizeof(ll));
  slot_t *src = s, *dst = t;
  for (int shift = 0; shift < 64; shift += 16) {
    memset(cnt, 0, (size_t)65536 * sizeof(ll));
    for (ll i = 0; i < n; i++)
      cnt[(((unsigned long long)src[i].vid ^ 0x8000000000000000ull) >> shift) & 0xFFFF]++;
    int trivial = 0;
    for (int d = 0; d < 65536; d++)
      if (cnt[d] == n) trivial = 1;
    if (trivial) continue;
    ll acc = 0;
    for (int d = 0; d < 65536; d++) {
      ll c = cnt[d];
      cnt[d] = acc;
      acc += c;
    }
    for (ll i = 0; i < n; i++) {
      unsigned d = (unsigned)((((unsigned long long)src[i].vid ^ 0x8000000000000000ull) >> shift) &
                              0xFFFF);
      dst[cnt[d]++] = src[i];
    }
    slot_t *x = src;
    src = dst, dst = x;
  }
  if (src != s) memcpy(s, src, (size_t)n * sizeof(slot_t));
  free(t), free(cnt);
}

/* Graph of the elements elems[0..n) (local index = position); vertex ids
 * of element e are vtx[e*nv .. e*nv+nv).  Row a lists every b != a sharing
 * a vertex with a, columns ascending, weight = number of (slot of a, slot
 * of b) pairs with equal ids.  Rows are independent: counted, then filled,
 * in parallel. */
static ll graph_row(ll a, int nv, const slot_t *s, const ll *gs, const ll *ge, const ll *inv,
                    int **bufp, ll *bcapp, int *col, int *w) {
  ll nb = 0;
  int *buf = *bufp;
  for (int k = 0; k < nv; k++) {
    ll pos = inv[a * nv + k];
    ll len = ge[pos] - gs[pos];
    if (nb + len > *bcapp) {
      *bcapp = 2 * (nb + len) + 64;
      buf = (int *)realloc(buf, (size_t)*bcapp * sizeof(int));
      *bufp = buf;
    }
    for (ll q = gs[pos]; q < ge[pos]; q++) {
      int b = s[q].slot / nv;
      if (b != a) buf[nb++] = b;
    }
  }
  /* insertion sort, then run-length = weight */
  for (ll i = 1; i < nb; i++) {
    int v = buf[i];
    ll j = i - 1;
    while (j >= 0 && buf[j] > v) buf[j + 1] = buf[j], j--;
    buf[j + 1] = v;
  }
  ll nnz = 0;
  for (ll i = 0; i < nb;) {
    ll j = i + 1;
    while (j < nb && buf[j] == buf[i]) j++;
    if (col) col[nnz] = buf[i], w[nnz] = (int)(j - i);
    nnz++;
    i = j;
  }
  return nnz;
}

static void build_graph(csr_t *m, const int *elems, ll n, const long long *vtx,
                        int nv) {
  ll ns = n * nv;
  slot_t *s = (slot_t *)malloc((size_t)(ns > 0 ? ns : 1) * sizeof(slot_t));
#pragma omp parallel for schedule(static) if(!in_parallel() && n >= TASK_MIN)
  for (ll i = 0; i < n; i++)
    for (int k = 0; k < nv; k++) {
      s[i * nv + k].vid = vtx[(ll)elems[i] * nv + k];
      s[i * nv + k].slot = (int)(i * nv + k);
    }
  radix_slots(s, ns);
  ll *gs = (ll *)malloc((size_t)(ns > 0 ? ns : 1) * sizeof(ll));
  ll *ge = (ll *)malloc((size_t)(ns > 0 ? ns : 1) * sizeof(ll));
  ll *inv = (ll *)malloc((size_t)(ns > 0 ? ns : 1) * sizeof(ll));
  for (ll i = 0; i < ns;) {
    ll j = i + 1;
    while (j < ns && s[j].vid == s[i].vid) j++;
    for (ll k = i; k < j; k++) gs[k] = i, ge[k] = j, inv[s[k].slot] = k;
    i = j;
  }
  m->n = n;
  m->rowptr = (ll *)malloc((size_t)(n + 1) * sizeof(ll));
  m->rowptr[0] = 0;
#pragma omp parallel if(!in_parallel() && n >= TASK_MIN)
  {
    int *buf = NULL;
    ll bcap = 0;
#pragma omp for schedule(static)
    for (ll a = 0; a < n; a++)
      m->rowptr[a + 1] = graph_row(a, nv, s, gs, ge, inv, &buf, &bcap, NULL, NULL);
    free(buf);
  }
  for (ll a = 0; a < n; a++) m->rowptr[a + 1] += m->rowptr[a];
  ll nnz = m->rowptr[n];
  m->col = (int *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int));
  m->w = (int *)malloc((size_t)(nnz > 0 ? nnz : 1) * sizeof(int));
#pragma omp parallel if(!in_parallel() && n >= TASK_MIN)
  {
    int *buf = NULL;
    ll bcap = 0;
#pragma omp for schedule(static)
    for (ll a = 0; a < n; a++)
      graph_row(a, nv, s, gs, ge, inv, &buf, &bcap, m->col + m->rowptr[a], m->w + m->rowptr[a]);
    free(buf);
  }
  free(s), free(gs), free(ge), free(inv);
}

/* y = L x in the difference form y_a = sum_b w_ab (x_a - x_b). */
static void lap_apply(double *y, const double *x, const csr_t *m) {
#pragma omp parallel for schedule(static) if(!in_parallel() && m->n >= TASK_MIN)
  for (ll a = 0; a < m->n; a++) {
    double acc = 0.0;
    for (ll q = m->rowptr[a]; q < m->rowptr[a + 1]; q++)
      acc += m->w[q] * (x[a] - x[m->col[q]]);
    y[a] = acc;
  }
}

void oracle_laplacian(double *y, const double *x, const long long *vtx,
                      int nel, int nv) {
  int *el = (int *)malloc((size_t)(nel > 0 ? nel : 1) * sizeof(int));
  for (int i = 0; i < nel; i++) el[i] = i;
  csr_t m;
  build_graph(&m, el, nel, vtx, nv);
  lap_apply(y, x, &m);
  csr_free(&m);
  free(el);
}

long long oracle_dual_graph(long long *rowptr, int *col, int *w, long long cap,
                            const long long *vtx, int nel, int nv) {
  int *el = (int *)malloc((size_t)(nel > 0 ? nel : 1) * sizeof(int));
  for (int i = 0; i < nel; i++) el[i] = i;
  csr_t m;
  build_graph(&m, el, nel, vtx, nv);
  ll nnz = m.rowptr[nel];
  if (nnz <= cap) {
    memcpy(rowptr, m.rowptr, (size_t)(nel + 1) * sizeof(ll));
    memcpy(col, m.col, (size_t)nnz * sizeof(int));
    memcpy(w, m.w, (size_t)nnz * sizeof(int));
  } else {
    nnz = -1;
  }
  csr_free(&m);
  free(el);
  return nnz;
}

/* ------------------------------------------------------------------------ */
/* Fiedler vector: src/fiedler.c.  dot :13-18, ortho :20-30, tqli :328-432,  */
/* lanczos_aux :434-511, lanczos :513-561, fiedler :563-621.                 */
/* ------------------------------------------------------------------------ */
static double dot(const double *y, const double *x, ll n) {
  double r;
  BLOCKED_SUM(r, n, x[i] * y[i]);
  return r;
}

#define PAR_FOR _Pragma("omp parallel for schedule(static) if(!in_parallel() && n >= TASK_MIN)")

static void ortho(double *q, ll n) {
  double sum;
  BLOCKED_SUM(sum, n, q[i]);
  sum /= (double)n;
  PAR_FOR
  for (ll i = 0; i < n; i++) q[i] -= sum;
}

static double sign_of(double a, double b) {
  double m = b >= 0.0 ? 1.0 : -1.0;
  return fabs(a) * m;
}

int oracle_tqli(double *eVectors, double *eValues, int n, const double *diagonal,
                const double *upper) {
  if (n == 0) return 0;
  double *d = (double *)calloc((size_t)(2 * n), sizeof(double)), *e = d + n;
  int i, j, k, l, iter, m;
  for (i = 0; i < n; i++) d[i] = diagonal[i];
  for (i = 0; i < n - 1; i++) e[i] = upper[i];
  e[n - 1] = 0.0;
  for (i = 0; i < n; i++) {
    for (j = 0; j < n; j++) eVectors[i * n + j] = 0;
    eVectors[i * n + i] = 1;
  }
  for (l = 0; l < n; l++) {
    iter = 0;
    do {
      for (m = l; m < n - 1; m++) {
        double dd = fabs(d[m]) + fabs(d[m + 1]);
        if (fabs(e[m]) / dd < SCALAR_TOL) break;
      }
      if (m != l) {
        if (iter++ == 30) {
          for (i = 0; i < n; i++) eValues[i] = d[i];
          free(d);
          return 1;
        }
        double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
        double r = sqrt(g * g + 1.0);
        g = d[m] - d[l] + e[l] / (g + sign_of(r, g));
        double s = 1.0, c = 1.0, p = 0.0;
        for (i = m - 1; i >= l; i--) {
          double f = s * e[i];
          double b = c * e[i];
          if (fabs(f) >= fabs(g)) {
            c = g / f;
            r = sqrt(c * c + 1.0);
            e[i + 1] = f * r;
            s = 1.0 / r;
            c = c * s;
          } else {
            s = f / g;
            r = sqrt(s * s + 1.0);
            e[i + 1] = g * r;
            c = 1.0 / r;
            s = s * c;
          }
          g = d[i + 1] - p;
          r = (d[i] - g) * s + 2.0 * c * b;
          p = s * r;
          d[i + 1] = g + p;
          g = c * r - b;
          for (k = 0; k < n; k++) {
            f = eVectors[k * n + i + 1];
            eVectors[k * n + i + 1] = s * eVectors[k * n + i] + c * f;
            eVectors[k * n + i] = c * eVectors[k * n + i] - s * f;
          }
        }
        if (r < SCALAR_TOL && i >= l) continue;
        d[l] -= p;
        e[l] = g;
        e[m] = 0.0;
      }
    } while (m != l);
  }
  for (i = 0; i < n; i++)
    for (j = 0; j < i; j++) {
      double t = eVectors[i * n + j];
      eVectors[i * n + j] = eVectors[j * n + i];
      eVectors[j * n + i] = t;
    }
  for (k = 0; k < n; k++) {
    e[k] = 0;
    for (i = 0; i < n; i++) e[k] += eVectors[k * n + i] * eVectors[k * n + i];
    if (e[k] > 0.0) e[k] = sqrt(fabs(e[k]));
    double scale = 1.0 / e[k];
    for (i = 0; i < n; i++) eVectors[k * n + i] *= scale;
  }
  for (i = 0; i < n; i++) eValues[i] = d[i];
  free(d);
  return 0;
}

static int lanczos_aux(double *diag, double *upper, double *rr, ll n,
                       int niter, double tol, const double *f,
                       const csr_t *L) {
  double *r = (double *)calloc((size_t)(3 * n), sizeof(double));
  double *p = r + n, *w = p + n;
  PAR_FOR
  for (ll i = 0; i < n; i++) r[i] = f[i];
  ortho(r, n);
  double rtz1 = 1, pap = 0, alpha, beta, rtz2, pap_old;
  double rtr = dot(r, r, n);
  double rnorm = sqrt(rtr), rtol = rnorm * tol;
  double rni = 1.0 / rnorm;
  PAR_FOR
  for (ll i = 0; i < n; i++) rr[i] = r[i] * rni;
  int iter;
  for (iter = 0; iter < niter; iter++) {
    rtz2 = rtz1, rtz1 = rtr;
    beta = rtz1 / rtz2;
    if (iter == 0) beta = 0.0;
    PAR_FOR
    for (ll i = 0; i < n; i++) p[i] = beta * p[i] + r[i];
    ortho(p, n);
    lap_apply(w, p, L);
    pap_old = pap, pap = dot(w, p, n);
    alpha = rtz1 / pap;
    PAR_FOR
    for (ll i = 0; i < n; i++) r[i] = r[i] - alpha * w[i];
    rtr = dot(r, r, n);
    rnorm = sqrt(rtr), rni = 1.0 / rnorm;
    PAR_FOR
    for (ll i = 0; i < n; i++) rr[(iter + 1) * n + i] = r[i] * rni;
    if (iter == 0) {
      diag[iter] = pap / rtz1;
    } else {
      diag[iter] = (beta * beta * pap_old + pap) / rtz1;
      upper[iter - 1] = -beta * pap_old / sqrt(rtz2 * rtz1);
    }
    if (rnorm < rtol) {
      iter++;
      break;
    }
  }
  free(r);
  return iter;
}

/* Returns the number of Lanczos steps, *(ipass_out) the passes used. */
static int lanczos(double *fiedler, ll n, double *initv, const csr_t *L,
                   int miter, int mpass, double tol, int *passes_out) {
  if (n < miter) miter = (int)n;
  double *alpha = (double *)calloc((size_t)(2 * miter), sizeof(double));
  double *beta = alpha + miter;
  double *rr = (double *)calloc((size_t)(miter + 1) * (size_t)n, sizeof(double));
  double *eVectors = (double *)calloc((size_t)miter * miter, sizeof(double));
  double *eValues = (double *)calloc((size_t)miter, sizeof(double));
  int iter = miter, ipass;
  for (ipass = 0; iter == miter && ipass < mpass; ipass++) {
    iter = lanczos_aux(alpha, beta, rr, n, miter, tol, initv, L);
    oracle_tqli(eVectors, eValues, iter, alpha, beta);
    double eValMin = fabs(eValues[0]);
    int eValMinI = 0;
    for (int i = 1; i < iter; i++)
      if (fabs(eValues[i]) < eValMin) eValMin = fabs(eValues[i]), eValMinI = i;
    PAR_FOR
    for (ll i = 0; i < n; i++) {
      fiedler[i] = 0.0;
      for (int j = 0; j < iter; j++)
        fiedler[i] += rr[(ll)j * n + i] * eVectors[eValMinI * iter + j];
    }
    ortho(fiedler, n);
    PAR_FOR
    for (ll i = 0; i < n; i++) initv[i] = fiedler[i];
  }
  free(alpha), free(rr), free(eVectors), free(eValues);
  if (passes_out) *passes_out = ipass;
  return (ipass - 1) * miter + iter;
}

/* fiedler (src/fiedler.c:563-621) for a group given as a local graph. */
static int fiedler_group(double *f, const csr_t *L, int miter, int mpass,
                         double tol, int *passes_out) {
  ll n = L->n;
  double *initv = (double *)calloc((size_t)n, sizeof(double));
  PAR_FOR
  for (ll i = 0; i < n; i++) {
    initv[i] = i + 1.0;
    if (i < n / 2) initv[i] += 1000 * n;
  }
  ortho(initv, n);
  double rtr = dot(initv, initv, n);
  double rni = 1.0 / sqrt(rtr);
  PAR_FOR
  for (ll i = 0; i < n; i++) initv[i] *= rni;
  int iter = lanczos(f, n, initv, L, miter, mpass, tol, passes_out);
  double norm;
  BLOCKED_SUM(norm, n, f[i] * f[i]);
  double normi = 1.0 / sqrt(norm);
  PAR_FOR
  for (ll i = 0; i < n; i++) f[i] *= normi;
  /* Canonical orientation (shared with the GPU): the reference's sign comes
   * from tqli's accumulated rotations; here f is oriented like the step of
   * the start vector, sum_i f_i s_i >= 0 with s_i = +1 for i < n/2 and -1
   * otherwise.  A flip swaps the two halves of the bisection. */
  double orient;
  BLOCKED_SUM(orient, n, (i < n / 2) ? f[i] : -f[i]);
  if (orient < 0.0) {
    PAR_FOR
    for (ll i = 0; i < n; i++) f[i] = -f[i];
  }
  free(initv);
  return iter;
}

/* FP64 eigen-residual ||L f - rho f|| / ||f||, rho = f'Lf / f'f. */
static double fiedler_resid(const double *f, const csr_t *L) {
  ll n = L->n;
  double *y = (double *)malloc((size_t)(n > 0 ? n : 1) * sizeof(double));
  lap_apply(y, f, L);
  double ff = dot(f, f, n), fLf = dot(f, y, n);
  double rho = fLf / ff, s;
  BLOCKED_SUM(s, n, (y[i] - rho * f[i]) * (y[i] - rho * f[i]));
  free(y);
  return sqrt(s) / sqrt(ff);
}

int oracle_fiedler(double *f, const long long *vtx, int nel, int nv, int miter,
                   int mpass, double tol) {
  int *el = (int *)malloc((size_t)(nel > 0 ? nel : 1) * sizeof(int));
  for (int i = 0; i < nel; i++) el[i] = i;
  csr_t m;
  build_graph(&m, el, nel, vtx, nv);
  int it = fiedler_group(f, &m, miter, mpass, tol, NULL);
  csr_free(&m);
  free(el);
  return it;
}

/* ------------------------------------------------------------------------ */
/* Connected components (count only): get_components_v2,                    */
/* src/components.c:160-328, counts vertex-connected components of a group. */
/* ------------------------------------------------------------------------ */
static int uf_find(int *par, int x) {
  while (par[x] != x) par[x] = par[par[x]], x = par[x];
  return x;
}

static int count_components(const int *elems, ll n, const long long *vtx,
                            int nv) {
  if (n == 0) return 0;
  ll ns = n * nv;
  slot_t *s = (slot_t *)malloc((size_t)ns * sizeof(slot_t));
  for (ll i = 0; i < n; i++)
    for (int k = 0; k < nv; k++) {
      s[i * nv + k].vid = vtx[(ll)elems[i] * nv + k];
      s[i * nv + k].slot = (int)(i * nv + k);
    }
  radix_slots(s, ns);
  int *par = (int *)malloc((size_t)n * sizeof(int));
  for (ll i = 0; i < n; i++) par[i] = (int)i;
  for (ll i = 0; i < ns;) {
    ll j = i + 1;
    int a = uf_find(par, s[i].slot / nv);
    while (j < ns && s[j].vid == s[i].vid) {
      int b = uf_find(par, s[j].slot / nv);
      if (a != b) par[b] = a;
      j++;
    }
    i = j;
  }
  int nc = 0;
  for (ll i = 0; i < n; i++)
    if (uf_find(par, (int)i) == i) nc++;
  free(par), free(s);
  return nc;
}

int oracle_components(const long long *vtx, const int *mask, int nel, int nv) {
  int *el = (int *)malloc((size_t)(nel > 0 ? nel : 1) * sizeof(int));
  ll n = 0;
  for (int i = 0; i < nel; i++)
    if (!mask || mask[i]) el[n++] = i;
  int nc = count_components(el, n, vtx, nv);
  free(el);
  return nc;
}

/* ------------------------------------------------------------------------ */
/* balance_partitions (src/rsb.c:118-229) on one bisected group.            */
/* a[0..n) is sorted by Fiedler value; a[0..*L) is the lower half (h ranks). */
/* ------------------------------------------------------------------------ */
static int cmp_ll(const void *x, const void *y) {
  ll a = *(const ll *)x, b = *(const ll *)y;
  return a < b ? -1 : (a > b);
}

static int in_sorted(const ll *v, ll n, ll key) {
  ll lo = 0, hi = n;
  while (lo < hi) {
    ll mid = (lo + hi) / 2;
    if (v[mid] < key)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo < n && v[lo] == key;
}

static void balance(int *a, ll n, int p, ll *L, const double *fiedler,
                    const long long *vtx, int nv, int *tmp, double *key,
                    char *moved) {
  if (p <= 1) return;
  int h = (p + 1) / 2;
  ll ne_ = n / p, nrem = n - ne_ * p;
  ll expA = ne_ * h + nrem / 2 + (nrem % 2);
  ll expB = ne_ * (p - h) + nrem / 2;
  ll sendA = *L - expA > 0 ? *L - expA : 0;
  ll sendB = (n - *L) - expB > 0 ? (n - *L) - expB : 0;
  if (sendA == 0 && sendB == 0) return;
  int senderA = sendA > 0;
  ll send = senderA ? sendA : sendB;
  ll s0 = senderA ? 0 : *L, sn = senderA ? *L : n - *L; /* sender range */
  ll r0 = senderA ? *L : 0, rn = senderA ? n - *L : *L; /* receiver range */
  double mul = senderA ? -1.0 : 1.0; /* sid == 0 <=> receiver is lower half */
  /* vertex ids of the receiver */
  ll *rv = (ll *)malloc((size_t)(rn * nv + 1) * sizeof(ll));
  for (ll i = 0; i < rn; i++)
    for (int k = 0; k < nv; k++) rv[i * nv + k] = vtx[(ll)a[r0 + i] * nv + k];
  qsort(rv, (size_t)(rn * nv), sizeof(ll), cmp_ll);
  /* boundary elements of the sender, in current order */
  int *bd = (int *)malloc((size_t)(sn + 1) * sizeof(int));
  ll nb = 0;
  for (ll i = 0; i < sn; i++) {
    int e = a[s0 + i];
    for (int k = 0; k < nv; k++)
      if (in_sorted(rv, rn * nv, vtx[(ll)e * nv + k])) {
        bd[nb++] = e;
        break;
      }
  }
  free(rv);
  if (nb < send) { /* not enough boundary elements: no change */
    free(bd);
    return;
  }
  for (ll i = 0; i < nb; i++) key[bd[i]] = mul * fiedler[bd[i]];
  msort(bd, tmp, nb, key);
  /* moved elements: bd[0..send); moved[] is indexed by element id */
  for (ll q = 0; q < send; q++) moved[bd[q]] = 1;
  int *newa = (int *)malloc((size_t)n * sizeof(int));
  ll k = 0;
  if (senderA) {
    /* new A = A minus moved; new B = stable sort by Fiedler value of the
     * moved elements (in their current order) followed by B */
    for (ll i = 0; i < *L; i++)
      if (!moved[a[i]]) newa[k++] = a[i];
    ll nbeg = k;
    for (ll i = 0; i < *L; i++)
      if (moved[a[i]]) newa[k++] = a[i];
    for (ll i = *L; i < n; i++) newa[k++] = a[i];
    for (ll i = nbeg; i < n; i++) key[newa[i]] = fiedler[newa[i]];
    msort(newa + nbeg, tmp, n - nbeg, key);
    *L = nbeg;
  } else {
    /* new A = stable sort by Fiedler value of A followed by the moved
     * elements (in their current order); new B = B minus moved */
    for (ll i = 0; i < *L; i++) newa[k++] = a[i];
    for (ll i = *L; i < n; i++)
      if (moved[a[i]]) newa[k++] = a[i];
    ll nA = k;
    for (ll i = 0; i < nA; i++) key[newa[i]] = fiedler[newa[i]];
    msort(newa, tmp, nA, key);
    for (ll i = *L; i < n; i++)
      if (!moved[a[i]]) newa[k++] = a[i];
    *L = nA;
  }
  memcpy(a, newa, (size_t)n * sizeof(int));
  for (ll q = 0; q < send; q++) moved[bd[q]] = 0;
  free(newa), free(bd);
}

/* ------------------------------------------------------------------------ */
/* parrsb_part_mesh: src/parrsb.c:853-906 -> parrsb_part_mesh_v0 :236-290,  */
/* rsb src/rsb.c:262-350 (one node: level 0 has no cuts, the last level     */
/* makes ceil(log2 P) cuts, get_level_cuts :244-260, get_bin :231-242).     */
/* ------------------------------------------------------------------------ */
typedef struct {
  ll s, n;
  int p, r0;
} seg_t;

/* Result of one group's bisection (merged into the info in group order). */
typedef struct {
  ll iters, L;
  int unconverged, comps;
  double resid;
} bis_t;

/* One group's cut (the body of rsb's loop, src/rsb.c:276-343): pre-partition,
 * Fiedler vector, sort, component count, balance.  a: the group's order,
 * tmp: scratch aligned with a; key / fied / moved are indexed by element
 * id (disjoint between groups). */
static void rsb_group(int *a, int *tmp, ll n, int p, const long long *vtx, int nv,
                      const double *cent, int ndim, const parrsb_options *o, double *key,
                      double *fied, char *moved, int want_info, bis_t *out) {
  geo_ctx g = {cent, key, tmp, a, ndim};
  /* pre-partition (src/rsb.c:282-292) */
  if (o->rsb_pre == 0)
    msort_int(a, tmp, n);
  else if (o->rsb_pre == 1)
    rcb_run(a, n, p, 0, &g, NULL, 1);
  else if (o->rsb_pre == 2)
    rib_run(a, n, p, 0, &g, NULL, 1);
  /* Fiedler vector (src/rsb.c:300-302) */
  csr_t Lg;
  build_graph(&Lg, a, n, vtx, nv);
  double *f = (double *)calloc((size_t)n, sizeof(double));
  int passes = 0;
  int miter = o->rsb_max_iter, mpass = o->rsb_max_passes;
  int it = fiedler_group(f, &Lg, miter, mpass, o->rsb_tol, &passes);
  memset(out, 0, sizeof(*out));
  out->iters = it;
  if (want_info) {
    int mi = (int)(n < miter ? n : miter);
    out->unconverged = (it == mi * mpass);
    out->resid = fiedler_resid(f, &Lg);
  }
  csr_free(&Lg);
  for (ll i = 0; i < n; i++) fied[a[i]] = f[i];
  free(f);
  /* sort by Fiedler value (src/rsb.c:307-309) */
  msort(a, tmp, n, fied);
  ll L = lower_count(n, p);
  /* components of each half (src/rsb.c:319-327), count only */
  if (o->find_disconnected_comps && want_info) {
    int c0 = count_components(a, L, vtx, nv);
    int c1 = count_components(a + L, n - L, vtx, nv);
    out->comps = c0 > c1 ? c0 : c1;
  }
  /* balance (src/rsb.c:333-335) */
  balance(a, n, p, &L, fied, vtx, nv, tmp, key, moved);
  out->L = L;
}

/* One level of RSB over all its segments.  seg_in[k] = (start, n, p, r0) of
 * segment k in the order a; seg_out receives the next level's segments (two
 * per segment with p > 1 and n > 0, the segment itself otherwise); returns
 * their number.  Groups run in parallel when there are at least as many as
 * threads, otherwise one after the other with their vectors split among the
 * threads; the result is the same either way. */
int oracle_rsb_level(int *a, const long long *seg_in, int nseg, long long *seg_out,
                     const long long *vtx, const double *cent, int nel, int nv,
                     const parrsb_options *o, oracle_rsb_info *info) {
  int ndim = (nv == 8) ? 3 : 2;
  int *tmp = (int *)malloc((size_t)(nel > 0 ? nel : 1) * sizeof(int));
  double *key = (double *)malloc((size_t)(nel > 0 ? nel : 1) * sizeof(double));
  double *fied = (double *)calloc((size_t)(nel > 0 ? nel : 1), sizeof(double));
  char *moved = (char *)calloc((size_t)(nel > 0 ? nel : 1), 1);
  int *act = (int *)malloc((size_t)(nseg > 0 ? nseg : 1) * sizeof(int));
  bis_t *res = (bis_t *)calloc((size_t)(nseg > 0 ? nseg : 1), sizeof(bis_t));
  int na = 0;
  for (int k = 0; k < nseg; k++)
    if (seg_in[4 * k + 2] > 1 && seg_in[4 * k + 1] > 0) act[na++] = k;
  int nthr = oracle_threads(0);
  int want = info != NULL;
  if (na >= nthr) {
#pragma omp parallel for schedule(dynamic, 1)
    for (int q = 0; q < na; q++) {
      const long long *sg = seg_in + 4 * act[q];
      rsb_group(a + sg[0], tmp + sg[0], sg[1], (int)sg[2], vtx, nv, cent, ndim, o, key, fied,
                moved, want, &res[act[q]]);
    }
  } else {
    for (int q = 0; q < na; q++) {
      const long long *sg = seg_in + 4 * act[q];
      rsb_group(a + sg[0], tmp + sg[0], sg[1], (int)sg[2], vtx, nv, cent, ndim, o, key, fied,
                moved, want, &res[act[q]]);
    }
  }
  int nn = 0;
  for (int k = 0; k < nseg; k++) {
    const long long *sg = seg_in + 4 * k;
    long long *d = seg_out + 4 * nn;
    if (!(sg[2] > 1 && sg[1] > 0)) {
      d[0] = sg[0], d[1] = sg[1], d[2] = sg[2], d[3] = sg[3];
      nn++;
      continue;
    }
    const bis_t *r = &res[k];
    if (info) {
      info->total_iters += r->iters;
      info->row_iters += r->iters * sg[1];
      info->nbisect++;
      info->unconverged += r->unconverged;
      if (r->resid > info->max_resid) info->max_resid = r->resid;
      if (r->comps > info->max_components) info->max_components = r->comps;
    }
    int h = (int)((sg[2] + 1) / 2);
    d[0] = sg[0], d[1] = r->L, d[2] = h, d[3] = sg[3];
    d[4] = sg[0] + r->L, d[5] = sg[1] - r->L, d[6] = sg[2] - h, d[7] = sg[3] + h;
    nn += 2;
  }
  if (info && na > 0) info->levels++;
  free(tmp), free(key), free(fied), free(moved), free(act), free(res);
  return nn;
}

/* ------------------------------------------------------------------------ */
/* parrsb_part_mesh: src/parrsb.c:853-906 -> parrsb_part_mesh_v0 :236-290,  */
/* rsb src/rsb.c:262-350 (one node: level 0 has no cuts, the last level     */
/* makes ceil(log2 P) cuts, get_level_cuts :244-260, get_bin :231-242).     */
/* ------------------------------------------------------------------------ */
int oracle_part_mesh(int *part, int *order, const long long *vtx,
                     const double *xyz, int nel, int nv,
                     parrsb_options *options, int nparts,
                     oracle_rsb_info *info) {
  if (info) memset(info, 0, sizeof(*info));
  if (!options || !part || nel < 0 || nparts < 1) return PARRSB_ERR_ARGS;
  oracle_update_options(options);
  if (options->tagged == 1) return PARRSB_ERR_UNSUPPORTED;
  if (vtx == NULL && xyz == NULL) return PARRSB_ERR_ARGS;
  if (xyz == NULL) options->rsb_pre = 0;
  if (options->levels > 2) options->levels = 2;
  if (options->partitioner == 0 && vtx == NULL) return PARRSB_ERR_ARGS;
  if (options->partitioner == 0 && options->rsb_algo != 0)
    return PARRSB_ERR_UNSUPPORTED;
  if (nel == 0) return PARRSB_OK;

  int ndim = (nv == 8) ? 3 : 2;
  int P = nparts < nel ? nparts : nel; /* ranks without elements drop out */
  double *cent = (double *)malloc((size_t)nel * 3 * sizeof(double));
  oracle_centroids(cent, xyz, nel, nv);
  int *a = (int *)malloc((size_t)nel * sizeof(int));
  int *tmp = (int *)malloc((size_t)nel * sizeof(int));
  double *key = (double *)malloc((size_t)nel * sizeof(double));
  for (int i = 0; i < nel; i++) a[i] = i;
  geo_ctx g = {cent, key, tmp, a, ndim};

  int rc = PARRSB_OK;
  if (options->partitioner == 1) {
    rcb_run(a, nel, P, 0, &g, part, 1);
  } else if (options->partitioner == 2) {
    rib_run(a, nel, P, 0, &g, part, 1);
  } else if (options->partitioner == 0) {
    int ncuts = 0;
    for (int pw = 1; pw < P; pw <<= 1) ncuts++;
    long long *segs = (long long *)malloc((size_t)8 * P * sizeof(long long));
    long long *nsegs = (long long *)malloc((size_t)8 * P * sizeof(long long));
    int nseg = 1;
    segs[0] = 0, segs[1] = nel, segs[2] = P, segs[3] = 0;
    for (int cut = 0; cut < ncuts; cut++) {
      nseg = oracle_rsb_level(a, segs, nseg, nsegs, vtx, cent, nel, nv, options, info);
      long long *t = segs;
      segs = nsegs, nsegs = t;
    }
    for (int si = 0; si < nseg; si++)
      for (ll i = 0; i < segs[4 * si + 1]; i++)
        part[a[segs[4 * si] + i]] = (int)segs[4 * si + 3];
    free(segs), free(nsegs);
  } else {
    /* unknown partitioner: elements stay on their load_balance rank
     * (src/parrsb.c:112-137: the first nrem ranks get nstar + 1). */
    ll nstar = nel / nparts, nrem = nel - nstar * nparts;
    ll lower = (nstar + 1) * nrem;
    for (ll e = 0; e < nel; e++) {
      ll eg = e + 1;
      if (nstar == 0)
        part[e] = (int)(eg - 1);
      else if (eg <= lower)
        part[e] = (int)((eg - 1) / (nstar + 1));
      else
        part[e] = (int)((eg - 1 - lower) / nstar + nrem);
    }
  }
  if (order) memcpy(order, a, (size_t)nel * sizeof(int));
  free(cent), free(a), free(tmp), free(key);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* gencon: src/con.c (mesh_init :14-50, find_min_neighbor_distance :68-103,  */
/* set_global_id :108-136, send_back :138-148), src/con-unique-vertices.c   */
/* (find_unique_vertices :445-505 and helpers), src/con-check.c             */
/* (element_check :265-288, face_check :197-263), compressPeriodicVertices  */
/* src/con-periodic.c:24-55 (identity without periodic faces).              */
/* ------------------------------------------------------------------------ */
static const int PRE_TO_SYM_VERTEX[8] = {0, 1, 3, 2, 4, 5, 7, 6};
static const int NEIGHBOR_MAP[8][3] = {{1, 2, 4}, {0, 3, 5}, {0, 3, 6},
                                       {1, 2, 7}, {0, 5, 6}, {1, 4, 7},
                                       {2, 4, 7}, {3, 5, 6}};
static const int FACES3D[6][4] = {{1, 5, 7, 3}, {2, 4, 8, 6}, {1, 2, 6, 5},
                                  {3, 7, 8, 4}, {1, 3, 4, 2}, {5, 6, 8, 7}};
static const int FACES2D[4][2] = {{3, 1}, {2, 4}, {1, 2}, {4, 3}};

static double diff_sqr(double x, double y) { return (x - y) * (x - y); }

/* Heapsort of tuple_sort_ (src/con-unique-vertices.c:6-58): the classic
 * in-place heapsort over 1-based positions, keys compared with '<'. */
static void heap_sort(int *ra, ll n, const double *key) {
  if (n < 2) return;
#define A(i) ra[(i)-1]
#define K(v) key[v]
  ll l = n / 2 + 1, ir = n, i, j;
  int rra;
  for (;;) {
    if (l > 1) {
      rra = A(--l);
    } else {
      rra = A(ir);
      A(ir) = A(1);
      if (--ir == 1) {
        A(1) = rra;
        break;
      }
    }
    i = l;
    j = l + l;
    while (j <= ir) {
      if (j < ir && K(A(j)) < K(A(j + 1))) j++;
      if (K(rra) < K(A(j))) {
        A(i) = A(j);
        i = j;
        j = 2 * j;
      } else
        break;
    }
    A(i) = rra;
  }
#undef A
#undef K
}

typedef struct {
  ll vid, elem;
} ve_t;

static int cmp_ve(const void *x, const void *y) {
  const ve_t *a = (const ve_t *)x, *b = (const ve_t *)y;
  if (a->vid != b->vid) return a->vid < b->vid ? -1 : 1;
  return a->elem < b->elem ? -1 : (a->elem > b->elem);
}

static int element_check(const ll *ids, ll nel, int nv) {
  for (ll i = 0; i < nel; i++) {
    ll g[8];
    for (int j = 0; j < nv; j++) g[j] = ids[i * nv + j];
    qsort(g, (size_t)nv, sizeof(ll), cmp_ll);
    for (int j = 0; j < nv - 1; j++)
      if (g[j] == g[j + 1]) return 1;
  }
  return 0;
}

static int face_check(const ll *ids, ll nel, int ndim) {
  int nv = (ndim == 3) ? 8 : 4, nf = (ndim == 3) ? 6 : 4, nfv = (ndim == 3) ? 4 : 2;
  ll np = nel * nv;
  ve_t *ve = (ve_t *)malloc((size_t)(np + 1) * sizeof(ve_t));
  for (ll p = 0; p < np; p++) ve[p].vid = ids[p], ve[p].elem = p / nv;
  qsort(ve, (size_t)np, sizeof(ve_t), cmp_ve);
  /* unique (vid, elem) pairs; CSR by vid */
  ll nu = 0;
  for (ll p = 0; p < np; p++)
    if (nu == 0 || ve[p].vid != ve[nu - 1].vid || ve[p].elem != ve[nu - 1].elem)
      ve[nu++] = ve[p];
  int err = 0;
  ll *sh = (ll *)malloc((size_t)(4 * 64 + 16) * sizeof(ll));
  ll shcap = 4 * 64 + 16;
  for (ll i = 0; i < nel && !err; i++) {
    for (int j = 0; j < nf && !err; j++) {
      ll ns = 0;
      for (int k = 0; k < nfv; k++) {
        int lv = (ndim == 3 ? FACES3D[j][k] : FACES2D[j][k]) - 1;
        ll vid = ids[i * nv + lv];
        /* binary search the first pair with this vid */
        ll lo = 0, hi = nu;
        while (lo < hi) {
          ll mid = (lo + hi) / 2;
          if (ve[mid].vid < vid)
            lo = mid + 1;
          else
            hi = mid;
        }
        for (ll q = lo; q < nu && ve[q].vid == vid; q++) {
          if (ns >= shcap) {
            shcap *= 2;
            sh = (ll *)realloc(sh, (size_t)shcap * sizeof(ll));
          }
          sh[ns++] = ve[q].elem;
        }
      }
      qsort(sh, (size_t)ns, sizeof(ll), cmp_ll);
      for (ll q = 0; q < ns;) {
        ll r = q + 1;
        while (r < ns && sh[r] == sh[q]) r++;
        if (r - q == 3) {
          err = 1;
          break;
        }
        q = r;
      }
    }
  }
  free(sh), free(ve);
  return err;
}

/* match_periodic_faces (src/con-periodic.c:245-288) on one rank.
 * pinfo: npinfo records (element, face, partner element, partner face),
 * 1-based, preprocessor face numbering (src/con.c:38-46).  ids: 0-based ids
 * of the points in sequence order, renumbered in place.  Returns 0,
 * PARRSB_ERR_ARGS for a record out of range, PARRSB_ERR_CHECK when paired
 * faces do not coincide (the reference exits the process there). */
static const int PRE_TO_SYM_FACE[6] = {2, 1, 3, 0, 4, 5};

typedef struct {
  ll elem, face, bc0, bc1, idx;
} bface_t;

static int cmp_bface_elem(const void *a, const void *b) {
  const bface_t *x = (const bface_t *)a, *y = (const bface_t *)b;
  if (x->elem != y->elem) return x->elem < y->elem ? -1 : 1;
  return x->idx < y->idx ? -1 : (x->idx > y->idx); /* stable */
}

static int match_periodic(ll *ids, double *const x[3], ll nelt, int ndim, ll nids,
                          const long long *pinfo, int npinfo, ll *nseg_out) {
  int nv = ndim == 3 ? 8 : 4, nvf = nv / 2, nfaces = ndim == 3 ? 6 : 4;
  ll np = nelt * nv;
  bface_t *b = (bface_t *)malloc((size_t)(npinfo + 1) * sizeof(bface_t));
  for (int i = 0; i < npinfo; i++) {
    ll e = pinfo[4 * i] - 1, f = pinfo[4 * i + 1] - 1;
    ll be = pinfo[4 * i + 2] - 1, bf = pinfo[4 * i + 3] - 1;
    if (e < 0 || e >= nelt || f < 0 || f >= nfaces || be < 0 || be >= nelt || bf < 0 ||
        bf >= nfaces) {
      free(b);
      return PARRSB_ERR_ARGS;
    }
    b[i].elem = e, b[i].face = PRE_TO_SYM_FACE[f];
    b[i].bc0 = be, b[i].bc1 = PRE_TO_SYM_FACE[bf], b[i].idx = i;
  }
  /* setPeriodicFaceCoordinates sorts the boundary array by elementId */
  qsort(b, (size_t)npinfo, sizeof(bface_t), cmp_bface_elem);
  /* findConnectedPeriodicFaces / findConnectedPeriodicPairs (:104-170) */
  ll cap = 16, nm = 0;
  ll *mmin = (ll *)malloc((size_t)cap * sizeof(ll)), *mmax = (ll *)malloc((size_t)cap * sizeof(ll));
  int err = 0;
  for (int i = 0; i < npinfo - 1 && !err; i++)
    for (int j = i + 1; j < npinfo && !err; j++) {
      if (b[j].bc0 != b[i].elem || b[j].bc1 != b[i].face) continue;
      double fx[4][3], gx[4][3];
      ll fid[4], gid[4];
      for (int q = 0; q < nvf; q++) {
        int cf = (ndim == 3 ? FACES3D[b[i].face][q] : FACES2D[b[i].face][q]) - 1;
        int cg = (ndim == 3 ? FACES3D[b[j].face][q] : FACES2D[b[j].face][q]) - 1;
        ll pf = b[i].elem * nv + cf, pg = b[j].elem * nv + cg;
        fid[q] = ids[pf], gid[q] = ids[pg];
        for (int d = 0; d < ndim; d++) fx[q][d] = x[d][pf], gx[q][d] = x[d][pg];
      }
      double fMax = 0.0, gMax = 0.0;
      for (int d = 0; d < ndim; d++) {
        double meanF = 0.0, meanG = 0.0;
        for (int q = 0; q < nvf; q++) {
          fMax = fMax > fabs(fx[q][d]) ? fMax : fabs(fx[q][d]);
          gMax = gMax > fabs(gx[q][d]) ? gMax : fabs(gx[q][d]);
          meanF += fx[q][d];
          meanG += gx[q][d];
        }
        for (int q = 0; q < nvf; q++) {
          fx[q][d] -= meanF / nvf;
          gx[q][d] -= meanG / nvf;
        }
      }
      int shift = 0;
      double d2Min = 1.e20;
      for (int s = 0; s < nvf; s++) {
        double d2 = 0.0;
        for (int q = 0; q < nvf; q++) {
          int k = nvf - 1 - (q + s) % nvf;
          double dd = diff_sqr(fx[q][0], gx[k][0]) + diff_sqr(fx[q][1], gx[k][1]);
          if (ndim == 3) dd = dd + diff_sqr(fx[q][2], gx[k][2]);
          d2 += dd;
        }
        if (d2 < d2Min) d2Min = d2, shift = s;
      }
      double fg = fMax > gMax ? fMax : gMax;
      if (sqrt(d2Min) > 1e-3 * fg) {
        err = PARRSB_ERR_CHECK;
        break;
      }
      for (int q = 0; q < nvf; q++) {
        int k = nvf - 1 - (q + shift) % nvf;
        if (nm == cap) {
          cap *= 2;
          mmin = (ll *)realloc(mmin, (size_t)cap * sizeof(ll));
          mmax = (ll *)realloc(mmax, (size_t)cap * sizeof(ll));
        }
        mmin[nm] = fid[q] < gid[k] ? fid[q] : gid[k];
        mmax[nm] = fid[q] < gid[k] ? gid[k] : fid[q];
        nm++;
      }
    }
  if (!err) {
    /* renumberPeriodicVertices (:64-102): repeat min over the pairs until
     * nothing changes; every id ends at the smallest id of its class */
    ll *lab = (ll *)malloc((size_t)(nids + 1) * sizeof(ll));
    for (ll v = 0; v < nids; v++) lab[v] = v;
    int changed = 1;
    while (changed) {
      changed = 0;
      for (ll t = 0; t < nm; t++) {
        ll a = lab[mmin[t]], c = lab[mmax[t]];
        ll m = a < c ? a : c;
        if (lab[mmin[t]] != m) lab[mmin[t]] = m, changed = 1;
        if (lab[mmax[t]] != m) lab[mmax[t]] = m, changed = 1;
      }
    }
    /* compressPeriodicVertices (:24-55): consecutive in increasing order */
    ll *rank = (ll *)malloc((size_t)(nids + 1) * sizeof(ll));
    ll nroot = 0;
    for (ll v = 0; v < nids; v++) rank[v] = (lab[v] == v) ? nroot++ : -1;
    for (ll p = 0; p < np; p++) ids[p] = rank[lab[ids[p]]];
    if (nseg_out) *nseg_out = nroot;
    free(lab), free(rank);
  }
  free(b), free(mmin), free(mmax);
  return err;
}

int oracle_conn_mesh_periodic(long long *vtx, const double *coord, unsigned int nelt,
                              unsigned ndim, double tol, int heapsort_mode,
                              const long long *pinfo, int npinfo, long long *ids_out,
                              long long *nseg_out) {
  if (ndim < 2 || ndim > 3) return PARRSB_ERR_ARGS;
  if (npinfo < 0 || (npinfo > 0 && !pinfo)) return PARRSB_ERR_ARGS;
  int nv = (ndim == 2) ? 4 : 8;
  ll np = (ll)nelt * nv;
  if (np == 0) {
    if (nseg_out) *nseg_out = 0;
    return PARRSB_OK;
  }
  double *x[3];
  for (int d = 0; d < 3; d++) x[d] = (double *)calloc((size_t)np, sizeof(double));
  double *dx = (double *)malloc((size_t)np * sizeof(double));
  for (ll i = 0; i < nelt; i++)
    for (int k = 0; k < nv; k++) {
      int j = PRE_TO_SYM_VERTEX[k];
      for (unsigned l = 0; l < ndim; l++)
        x[l][i * nv + k] = coord[i * nv * ndim + j * ndim + l];
    }
  for (ll i = 0; i < nelt; i++)
    for (int j = 0; j < nv; j++) {
      ll p = i * nv + j;
      double m = DBL_MAX;
      for (unsigned k = 0; k < ndim; k++) {
        ll q = i * nv + NEIGHBOR_MAP[j][k];
        double d = diff_sqr(x[0][p], x[0][q]) + diff_sqr(x[1][p], x[1][q]);
        if (ndim == 3) d = d + diff_sqr(x[2][p], x[2][q]);
        m = (m < d) ? m : d;
      }
      dx[p] = m;
    }
  int *ord = (int *)malloc((size_t)np * sizeof(int));
  int *tmp = (int *)malloc((size_t)np * sizeof(int));
  char *flag = (char *)calloc((size_t)np, 1);
  for (ll p = 0; p < np; p++) ord[p] = (int)p;
  double tol2 = tol * tol;
  for (unsigned t = 0; t < ndim; t++) {
    for (unsigned d = 0; d < ndim; d++) {
      if (t == 0 && d == 0) {
        /* all points form one shared segment: stable parallel sort */
        msort(ord, tmp, np, x[0]);
        memset(flag, 0, (size_t)np);
        flag[0] = 1;
      } else {
        /* sort_segments_local (src/con-unique-vertices.c:63-89) */
        ll s = 0;
        while (s < np) {
          ll e = s + 1;
          while (e < np && flag[e] == 0) e++;
          if (s < np - 1 && e - s > 1) {
            if (heapsort_mode)
              heap_sort(ord + s, e - s, x[d]);
            else
              msort(ord + s, tmp, e - s, x[d]);
          }
          s = e;
        }
      }
      /* find_segments (src/con-unique-vertices.c:303-320) */
      for (ll j = 1; j < np; j++) {
        int pj = ord[j], pk = ord[j - 1];
        double dd = diff_sqr(x[d][pj], x[d][pk]);
        double m = (dx[pj] < dx[pk] ? dx[pj] : dx[pk]) * tol2;
        if (dd > m) flag[j] = 1;
      }
    }
  }
  ll *ids = (ll *)malloc((size_t)np * sizeof(ll));
  ll cnt = -1;
  for (ll p = 0; p < np; p++) {
    if (flag[p]) cnt++;
    ids[ord[p]] = cnt;
  }
  if (nseg_out) *nseg_out = cnt + 1;
  if (ids_out) memcpy(ids_out, ids, (size_t)np * sizeof(ll));
  int err = element_check(ids, nelt, nv);
  if (!err) err = face_check(ids, nelt, ndim);
  if (!err) {
    ll nseg2 = cnt + 1;
    err = match_periodic(ids, x, nelt, (int)ndim, cnt + 1, pinfo, npinfo, &nseg2);
    if (!err && nseg_out) *nseg_out = nseg2;
  }
  if (!err && vtx)
    for (ll p = 0; p < np; p++) vtx[p] = ids[p] + 1;
  for (int d = 0; d < 3; d++) free(x[d]);
  free(dx), free(ord), free(tmp), free(flag), free(ids);
  return err;
}

int oracle_conn_mesh(long long *vtx, const double *coord, unsigned int nelt,
                     unsigned ndim, double tol, int heapsort_mode,
                     long long *ids_out, long long *nseg_out) {
  return oracle_conn_mesh_periodic(vtx, coord, nelt, ndim, tol, heapsort_mode, NULL, 0,
                                   ids_out, nseg_out);
}

/* ------------------------------------------------------------------------ */
/* Partition quality (new; comm volume as parrsb_get_part_stat's nss,       */
/* src/helpers.c:132-224).                                                  */
/* ------------------------------------------------------------------------ */
void oracle_part_quality(double *q, const int *part, const long long *vtx,
                         int nel, int nv, int nparts) {
  for (int i = 0; i < 8; i++) q[i] = 0.0;
  int *el = (int *)malloc((size_t)(nel > 0 ? nel : 1) * sizeof(int));
  for (int i = 0; i < nel; i++) el[i] = i;
  csr_t m;
  build_graph(&m, el, nel, vtx, nv);
  int fw = (nv == 8) ? 4 : 2;
  for (ll a = 0; a < nel; a++)
    for (ll k = m.rowptr[a]; k < m.rowptr[a + 1]; k++) {
      int b = m.col[k];
      if (b > a && part[a] != part[b]) {
        q[0] += m.w[k];
        q[1] += 1;
        if (m.w[k] >= fw) q[2] += 1;
      }
    }
  csr_free(&m);
  ll *cnt = (ll *)calloc((size_t)nparts, sizeof(ll));
  for (int e = 0; e < nel; e++) cnt[part[e]]++;
  ll mx = 0, mn = nel;
  for (int p = 0; p < nparts; p++) {
    if (cnt[p] > mx) mx = cnt[p];
    if (cnt[p] < mn) mn = cnt[p];
  }
  q[3] = (double)mx, q[4] = (double)mn;
  q[5] = nel > 0 ? (double)mx * nparts / nel : 0.0;
  /* vertex -> distinct parts */
  ll np = (ll)nel * nv;
  ve_t *ve = (ve_t *)malloc((size_t)(np + 1) * sizeof(ve_t));
  for (ll p = 0; p < np; p++) ve[p].vid = vtx[p], ve[p].elem = part[p / nv];
  qsort(ve, (size_t)np, sizeof(ve_t), cmp_ve);
  /* neighbour sets per part: collect (p, q) pairs */
  ll pcap = 1024, npairs = 0;
  ll *pairs = (ll *)malloc((size_t)pcap * sizeof(ll));
  double vol = 0.0;
  for (ll i = 0; i < np;) {
    ll j = i + 1;
    while (j < np && ve[j].vid == ve[i].vid) j++;
    /* distinct parts in ve[i..j) (sorted by part within the vid) */
    ll dstart = i;
    ll md = 0;
    ll dl[64];
    for (ll k = dstart; k < j; k++)
      if (k == dstart || ve[k].elem != ve[k - 1].elem) {
        if (md < 64) dl[md] = ve[k].elem;
        md++;
      }
    vol += (double)md * (double)(md - 1);
    for (ll u = 0; u < md && u < 64; u++)
      for (ll v = 0; v < md && v < 64; v++)
        if (u != v) {
          if (npairs >= pcap) {
            pcap *= 2;
            pairs = (ll *)realloc(pairs, (size_t)pcap * sizeof(ll));
          }
          pairs[npairs++] = dl[u] * (ll)nparts + dl[v];
        }
    i = j;
  }
  q[6] = vol;
  qsort(pairs, (size_t)npairs, sizeof(ll), cmp_ll);
  ll *nb = (ll *)calloc((size_t)nparts, sizeof(ll));
  for (ll i = 0; i < npairs; i++)
    if (i == 0 || pairs[i] != pairs[i - 1]) nb[pairs[i] / nparts]++;
  ll mnb = 0;
  for (int p = 0; p < nparts; p++)
    if (nb[p] > mnb) mnb = nb[p];
  q[7] = (double)mnb;
  free(nb), free(pairs), free(ve), free(cnt), free(el);
}
