// capi.cu -- the drop-in C ABI (include/parrsb.h).
//
// parrsb_part_mesh restates parrsb_part_mesh / parrsb_part_mesh_v0
// (src/parrsb.c:236-290, 853-906) with `nparts` virtual ranks instead of an
// MPI communicator; parrsb_conn_mesh restates src/con.c:189-295 on one rank.
// Option handling (defaults, PARRSB_* environment overrides written back into
// the caller's struct, levels clamped to 2, rsb_pre = 0 without coordinates)
// follows src/parrsb.c:26-77, 229, 250.  Errors are returned, never exit().
#include <stdarg.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <stdexcept>

#include "bisect.cuh"
#include "gencon.cuh"
#include "periodic.cuh"
#include "rsb.cuh"
#include "warm.cuh"

extern "C" {
parrsb_options parrsb_default_options = {
    /*partitioner*/ 0, /*tagged*/ 0, /*levels*/ 2, /*find_disconnected_comps*/ 1,
    /*repair*/ 0, /*verbose_level*/ 1, /*profile_level*/ 0, /*rsb_algo*/ 0,
    /*rsb_pre*/ 1, /*rsb_max_iter*/ 50, /*rsb_max_passes*/ 50, /*rsb_tol*/ 1e-5,
    /*rsb_dump_stats*/ 0, /*rsb_mg_grammian*/ 0, /*rsb_mg_factor*/ 2};
}

namespace prsb {

static thread_local Ctx g_ctx;
Ctx &ctx() { return g_ctx; }

void *dev_alloc(size_t bytes) {
  void *p = nullptr;
  CK(cudaMallocAsync(&p, bytes, ctx().stream));
  return p;
}

void dev_free(void *p) { cudaFreeAsync(p, ctx().stream); }

bool pdl_enabled() {
  static const bool on = [] {
    const char *e = getenv("PARRSB_GPU_PDL");
    return !(e && atoi(e) == 0);
  }();
  return on;
}

void Ctx::init() {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) throw ArgError{PARRSB_ERR_UNSUPPORTED, "device index >= 64"};
  if (!streams[dev]) {
    CK(cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking));
    cudaMemPool_t pool;
    CK(cudaDeviceGetDefaultMemPool(&pool, dev));
    unsigned long long keep = ~0ull;  // keep freed blocks for reuse
    CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  }
  device = dev;
  stream = streams[dev];
  memset(&stats, 0, sizeof(stats));
  kernel_launches = 0;
  const char *t = getenv("PARRSB_GPU_TIMING");
  timing = t && atoi(t) != 0;
}

namespace {

struct Workspace {
  GenconWs gc;
  PBuf<long long> vtx;  // host inputs land here (cudaMalloc, kept across calls)
  PBuf<double> xyz;
  DBuf<double> cent;
  PBuf<int> part;
  DBuf<long long> ids;
};
// per thread and device: buffers cached by earlier calls on the device that
// is current now (Ctx::init has selected it)
thread_local Workspace *g_ws[MAX_DEVICES] = {};
Workspace &ws() {
  Workspace *&w = g_ws[ctx().device];
  if (!w) w = new Workspace();
  return *w;
}

void print_if(int verbose, const char *fmt, ...) {
  if (verbose <= 0) return;
  va_list ap;
  va_start(ap, fmt);
  vprintf(fmt, ap);
  va_end(ap);
  printf("\n");
  fflush(stdout);
}

void update_options(parrsb_options *o) {
#define UPD(F, S, INT)                     \
  do {                                     \
    const char *v = getenv(S);             \
    if (v) {                               \
      if (INT)                             \
        o->F = atoi(v);                    \
      else                                 \
        o->F = atof(v);                    \
    }                                      \
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

void print_options(const parrsb_options *o) {
  int v = o->verbose_level;
  print_if(v, "PARRSB_PARTITIONER = %d", o->partitioner);
  print_if(v, "PARRSB_TAGGED = %d", o->tagged);
  print_if(v, "PARRSB_LEVELS = %d", o->levels);
  print_if(v, "PARRSB_FIND_DISCONNECTED_COMPONENTS = %d", o->find_disconnected_comps);
  print_if(v, "PARRSB_REPAIR = %d", o->repair);
  print_if(v, "PARRSB_VERBOSE_LEVEL = %d", o->verbose_level);
  print_if(v, "PARRSB_PROFILE_LEVEL = %d", o->profile_level);
  print_if(v, "PARRSB_RSB_ALGO = %d", o->rsb_algo);
  print_if(v, "PARRSB_RSB_PRE = %d", o->rsb_pre);
  print_if(v, "PARRSB_RSB_MAX_ITER = %d", o->rsb_max_iter);
  print_if(v, "PARRSB_RSB_MAX_PASSES = %d", o->rsb_max_passes);
  print_if(v, "PARRSB_RSB_TOL = %lf", o->rsb_tol);
  print_if(v, "PARRSB_RSB_MG_GRAMMIAN = %d", o->rsb_mg_grammian);
  print_if(v, "PARRSB_RSB_MG_FACTOR = %d", o->rsb_mg_factor);
}

double env_double(const char *name, double def) {
  const char *v = getenv(name);
  return v ? atof(v) : def;
}

int env_int(const char *name, int def) {
  const char *v = getenv(name);
  return v ? atoi(v) : def;
}

// Validates and normalises options (shared by the host and device entries).
int prepare_options(const long long *vtx, const double *xyz, int nel, int nv,
                    parrsb_options *o, int nparts, const int *tag, bool print) {
  if (!o) return PARRSB_ERR_ARGS;
  update_options(o);
  if (print) {
    print_if(o->verbose_level, "Running parRSB ..., nv = %d, nelg = %lld", nv, (long long)nel);
    print_options(o);
  }
  if (o->tagged == 1 && !tag) {
    print_if(o->verbose_level, "Tagged partitioning requested but tag array is NULL..");
    return PARRSB_ERR_ARGS;
  }
  if (nel < 0 || nparts < 1 || nv < 1 || nv > 8) return PARRSB_ERR_ARGS;
  if (vtx == nullptr && xyz == nullptr) {
    print_if(o->verbose_level,
             "parrsb_part_mesh_v0: Both vertices and coordinates can't be NULL");
    return PARRSB_ERR_ARGS;
  }
  if (xyz == nullptr) o->rsb_pre = 0;
  if (o->levels > 2) o->levels = 2;
  if (o->partitioner == 0) {
    if (o->rsb_algo != 0) return PARRSB_ERR_UNSUPPORTED;
    if (vtx == nullptr) return PARRSB_ERR_ARGS;
  }
  return PARRSB_OK;
}

// Host inputs into device buffers.  When the host buffer is page-locked and
// mapped into the device's address space (cudaHostAlloc / cudaHostRegister
// memory under unified addressing), the GPU's SMs read it directly over the
// host link with 16-byte loads; otherwise a cudaMemcpyAsync stages it.
// (Measured on a GB300 with 2.15 GB of pinned inputs: SM reads 10.2 ms on
// every call, the link's 211 GB/s; copy-engine transfers of the same
// buffers 10-21 ms, slower after RSB calls, and 25-90 ms in some
// processes.)  PARRSB_GPU_UPLOAD=copy forces the copy engine.
__global__ void k_pull_host(const uint4 *__restrict__ src, uint4 *__restrict__ dst, ll n16) {
  for (ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x; i < n16;
       i += (ll)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

__global__ void k_pull_host_tail(const unsigned char *__restrict__ src,
                                 unsigned char *__restrict__ dst, ll n) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i];
}

template <typename T>
void upload(T *d, const T *h, size_t n) {
  if (!n) return;
  static const bool force_copy = [] {
    const char *e = getenv("PARRSB_GPU_UPLOAD");
    return e && strcmp(e, "copy") == 0;
  }();
  cudaPointerAttributes a;
  const size_t bytes = n * sizeof(T);
  if (!force_copy && cudaPointerGetAttributes(&a, h) == cudaSuccess &&
      a.type == cudaMemoryTypeHost && a.devicePointer != nullptr &&
      reinterpret_cast<uintptr_t>(a.devicePointer) % 16 == 0 &&
      reinterpret_cast<uintptr_t>(d) % 16 == 0) {
    const ll n16 = (ll)(bytes / 16);
    const unsigned grid = (unsigned)std::min<ll>(std::max<ll>(1, (n16 + 255) / 256), 152 * 16);
    if (n16 > 0) {
      k_pull_host<<<grid, 256, 0, ctx().stream>>>(static_cast<const uint4 *>(a.devicePointer),
                                                  reinterpret_cast<uint4 *>(d), n16);
      CK_LAUNCH();
    }
    const ll tail = (ll)(bytes - (size_t)n16 * 16);
    if (tail > 0) {
      k_pull_host_tail<<<1, 256, 0, ctx().stream>>>(
          static_cast<const unsigned char *>(a.devicePointer) + n16 * 16,
          reinterpret_cast<unsigned char *>(d) + n16 * 16, tail);
      CK_LAUNCH();
    }
    return;
  }
  cudaGetLastError();  // a pageable pointer is not an error
  h2d(d, h, n);
}

// PARRSB_GPU_WARM_WEIGHTS=<file>: the warm-start network's parameters as
// raw little-endian FP32 (MP_NPARAM values), installed on the current device
// the first time a call asks for the warm start there.
void load_warm_weights_from_env() {
  if (warm_net_ready()) return;
  const char *path = getenv("PARRSB_GPU_WARM_WEIGHTS");
  if (!path) throw ArgError{PARRSB_ERR_ARGS, "PARRSB_GPU_WARM=1 without an installed network "
                                             "(parrsb_warm_install or PARRSB_GPU_WARM_WEIGHTS)"};
  FILE *fp = fopen(path, "rb");
  if (!fp) throw ArgError{PARRSB_ERR_ARGS, "cannot open PARRSB_GPU_WARM_WEIGHTS"};
  std::vector<float> w(MP_NPARAM);
  const size_t got = fread(w.data(), sizeof(float), MP_NPARAM, fp);
  fclose(fp);
  if (got != (size_t)MP_NPARAM) throw ArgError{PARRSB_ERR_ARGS, "PARRSB_GPU_WARM_WEIGHTS too short"};
  warm_net_install(w.data());
}

__global__ void k_block_part(int *part, ll nel, int nparts) {
  ll e = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  ll nstar = nel / nparts, nrem = nel - nstar * nparts, lower = (nstar + 1) * nrem;
  ll eg = e + 1;
  int p;
  if (nstar == 0)
    p = (int)(eg - 1);
  else if (eg <= lower)
    p = (int)((eg - 1) / (nstar + 1));
  else
    p = (int)((eg - 1 - lower) / nstar + nrem);
  part[e] = p;
}

// Device-resident partitioning: inputs and output already in HBM.
__global__ void k_seq_from_order(const int *__restrict__ perm, const int *__restrict__ part,
                                 ll N, int *__restrict__ first, int *__restrict__ seq) {
  // parts are contiguous and in rank order in the final element order
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int e = perm[i];
  int r = part[e];
  if (i == 0 || part[perm[i - 1]] != r) first[r] = (int)i;
}

__global__ void k_seq_write(const int *__restrict__ perm, const int *__restrict__ part, ll N,
                            const int *__restrict__ first, int *__restrict__ seq) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int e = perm[i];
  seq[e] = (int)(i - first[part[e]]);
}

void part_mesh_dev_impl(int *d_part, const long long *d_vtx, const double *d_xyz, int nel,
                        int nv, const parrsb_options *o, int nparts, int *d_seq,
                        const StartGroups *sg);

// The partition, then (options->repair == 1, with vertex ids) the repair of
// disconnected parts (repair.cu); the within-part order seq, if asked for,
// is the order before the repair.
void part_mesh_dev(int *d_part, const long long *d_vtx, const double *d_xyz, int nel, int nv,
                   const parrsb_options *o, int nparts, int *d_seq = nullptr,
                   const StartGroups *sg = nullptr) {
  part_mesh_dev_impl(d_part, d_vtx, d_xyz, nel, nv, o, nparts, d_seq, sg);
  if (o->repair == 1 && d_vtx && nel > 0) {
    long long mc = 0, me = 0;
    repair_parts_device(d_vtx, nel, nv, nparts, d_part, &mc, &me);
    ctx().stats.repair_components = mc;
    ctx().stats.repair_elements = me;
  }
}

void part_mesh_dev_impl(int *d_part, const long long *d_vtx, const double *d_xyz, int nel,
                        int nv, const parrsb_options *o, int nparts, int *d_seq,
                        const StartGroups *sg) {
  cudaStream_t st = ctx().stream;
  if (nel == 0) return;
  int ndim = (nv == 8) ? 3 : 2;
  ll N = nel;
  int P = nparts < nel ? nparts : nel;
  Workspace &W = ws();
  W.cent.ensure((size_t)3 * N);
  {
    StageTimer tm(PARRSB_STAGE_SETUP);
    compute_centroids(d_xyz, nel, nv, W.cent.p);
  }
  if (o->partitioner == 1 || o->partitioner == 2) {
    StageTimer tm(PARRSB_STAGE_PRE);
    BisectWs bws;
    DBuf<int> perm((size_t)N);
    SegTable t;
    if (sg) {  // tagged: one segment per tag
      const ll ng = (ll)sg->start.size();
      h2d(perm.p, sg->perm.data(), N);
      t.reserve(ng);
      h2d(t.start.p, sg->start.data(), ng);
      h2d(t.n.p, sg->n.data(), ng);
      h2d(t.p.p, sg->p.data(), ng);
      h2d(t.r0.p, sg->r0.data(), ng);
      t.count = ng;
    } else {
      iota_device(perm.p, N);
      t.reserve(1);
      ll s0 = 0, n0 = N;
      int p0 = P, r00 = 0;
      h2d(t.start.p, &s0, 1);
      h2d(t.n.p, &n0, 1);
      h2d(t.p.p, &p0, 1);
      h2d(t.r0.p, &r00, 1);
      t.count = 1;
    }
    bisect_segments(o->partitioner == 1 ? BISECT_RCB : BISECT_RIB, perm, t, W.cent.p, N, ndim,
                    d_seq != nullptr, d_part, bws);
    if (d_seq) {
      DBuf<int> first((size_t)nparts);
      k_seq_from_order<<<grid_for(N, 256), 256, 0, st>>>(perm.p, d_part, N, first.p, d_seq);
      CK_LAUNCH();
      k_seq_write<<<grid_for(N, 256), 256, 0, st>>>(perm.p, d_part, N, first.p, d_seq);
      CK_LAUNCH();
    }
    sync();
  } else if (o->partitioner == 0) {
    RsbOpts ro;
    ro.pre = o->rsb_pre;
    ro.miter = o->rsb_max_iter;
    ro.mpass = o->rsb_max_passes;
    ro.tol = o->rsb_tol;
    ro.find_comps = o->find_disconnected_comps;
    ro.profile = o->profile_level;
    ro.fp32 = env_int("PARRSB_GPU_FP32", 0);
    ro.check_resid = env_int("PARRSB_GPU_CHECK_RESID", 1);
    ro.use_graphs = env_int("PARRSB_GPU_GRAPHS", 1);
    ro.batched = env_int("PARRSB_GPU_BATCHED", 1);
    ro.start = env_int("PARRSB_GPU_START", 0);
    ro.warm = env_int("PARRSB_GPU_WARM", 0);
    ro.warm_min = env_int("PARRSB_GPU_WARM_MIN", 0);
    ro.resid_stop = env_int("PARRSB_GPU_RESID_STOP", 0);
    ro.cg_factor = env_double("PARRSB_GPU_RESID_CG_FACTOR", 0.1);
    ro.reorth = env_int("PARRSB_GPU_REORTH", 0);
    if (ro.warm) load_warm_weights_from_env();
    rsb_device(d_vtx, W.cent.p, N, nv, P, ro, d_part, d_seq, sg);
    sync();
  } else {
    k_block_part<<<grid_for(N, 256), 256, 0, st>>>(d_part, N, nparts);
    CK_LAUNCH();
    if (d_seq) {  // elements stay in input order inside their block
      DBuf<int> perm((size_t)N), first((size_t)nparts);
      iota_device(perm.p, N);
      k_seq_from_order<<<grid_for(N, 256), 256, 0, st>>>(perm.p, d_part, N, first.p, d_seq);
      CK_LAUNCH();
      k_seq_write<<<grid_for(N, 256), 256, 0, st>>>(perm.p, d_part, N, first.p, d_seq);
      CK_LAUNCH();
    }
    sync();
  }
}

const char *stage_names[12] = {"upload", "setup", "pre-partition", "lanczos",
                               "tqli+ritz", "sort", "components", "balance",
                               "restrict", "download", "gencon", "check"};

void print_profile(const parrsb_options *o) {
  if (o->profile_level <= 0) return;
  const parrsb_stats &S = ctx().stats;
  for (int i = 0; i < 12; i++)
    if (S.stage_ms[i] > 0) printf("  %-14s %10.3f ms\n", stage_names[i], S.stage_ms[i]);
  printf("  lanczos steps %lld, levels %d, max components %d, max residual %.3e\n",
         S.lanczos_iters, S.levels, S.max_components, S.max_fiedler_resid);
  fflush(stdout);
}

template <typename F>
int guarded(F &&fn) {
  try {
    return fn();
  } catch (const CudaError &e) {
    fprintf(stderr, "parrsb_gb300: CUDA error %s at %s:%d\n", cudaGetErrorString(e.err), e.file,
            e.line);
    cudaGetLastError();
    return PARRSB_ERR_CUDA;
  } catch (const ArgError &e) {
    fprintf(stderr, "parrsb_gb300: %s\n", e.msg);
    return e.code;
  } catch (const std::bad_alloc &) {
    fprintf(stderr, "parrsb_gb300: host allocation failed\n");
    return PARRSB_ERR_CUDA;
  }
}

// Host-side fault injection for tests: PARRSB_FAULT=<stage> makes that stage
// fail with PARRSB_ERR_CHECK after everything before it ran.
void maybe_fault(const char *stage) {
  const char *f = getenv("PARRSB_FAULT");
  if (f && strcmp(f, stage) == 0) throw ArgError{PARRSB_ERR_CHECK, "injected fault"};
}

}  // namespace
}  // namespace prsb

using namespace prsb;

static int part_mesh_host(int *part, int *seq, const long long *vtx, const double *xyz,
                          const int *tag, int nel, int nv, parrsb_options *options,
                          int nparts);

extern "C" int parrsb_part_mesh(int *part, const long long *vtx, const double *xyz,
                                const int *tag, int nel, int nv, parrsb_options *options,
                                int nparts) {
  return part_mesh_host(part, nullptr, vtx, xyz, tag, nel, nv, options, nparts);
}

extern "C" int parrsb_part_mesh_seq(int *part, int *seq, const long long *vtx,
                                    const double *xyz, const int *tag, int nel, int nv,
                                    parrsb_options *options, int nparts) {
  if (nel > 0 && !seq) return PARRSB_ERR_ARGS;
  return part_mesh_host(part, seq, vtx, xyz, tag, nel, nv, options, nparts);
}

// Tagged partitioning (parrsb_part_mesh_v1, src/parrsb.c:379-561): tags are
// numbered in increasing order; nparts must be a multiple of their number;
// the elements of tag number t, in input order, are partitioned among the
// nparts / ntags ranks starting at t * nparts / ntags, independently of the
// other tags.  Here all tags run in the same launches: the recursion starts
// from one group per tag.
static int tagged_groups(const int *tag, int nel, int nparts, int verbose, StartGroups &sg) {
  std::vector<int> u(tag, tag + nel);
  std::sort(u.begin(), u.end());
  u.erase(std::unique(u.begin(), u.end()), u.end());
  const int ntags = (int)u.size();
  print_if(verbose, "Num tags: %d", ntags);
  if (ntags == 0) return PARRSB_OK;
  if (nparts % ntags != 0) {
    print_if(1, "Number of processes must be a multiple of number of tags: "
                "processes = %d, tags = %d.", nparts, ntags);
    return PARRSB_ERR_ARGS;
  }
  const int chunk = nparts / ntags;
  std::vector<ll> cnt(ntags + 1, 0);
  std::vector<int> tn(nel);
  for (int e = 0; e < nel; e++) {
    tn[e] = (int)(std::lower_bound(u.begin(), u.end(), tag[e]) - u.begin());
    cnt[tn[e] + 1]++;
  }
  for (int t = 0; t < ntags; t++) cnt[t + 1] += cnt[t];
  sg.perm.assign(nel, 0);
  std::vector<ll> fill(cnt.begin(), cnt.end() - 1);
  for (int e = 0; e < nel; e++) sg.perm[fill[tn[e]]++] = e;  // stable: input order
  for (int t = 0; t < ntags; t++) {
    const ll n = cnt[t + 1] - cnt[t];
    sg.start.push_back(cnt[t]);
    sg.n.push_back(n);
    sg.p.push_back((int)std::min<ll>(chunk, n));  // fewer elements than ranks
    sg.r0.push_back(t * chunk);
  }
  return PARRSB_OK;
}

static int part_mesh_host(int *part, int *seq, const long long *vtx, const double *xyz,
                          const int *tag, int nel, int nv, parrsb_options *options,
                          int nparts) {
  auto t0 = std::chrono::steady_clock::now();
  int rc = prepare_options(vtx, xyz, nel, nv, options, nparts, tag, true);
  if (rc != PARRSB_OK) return rc;
  if (nel > 0 && !part) return PARRSB_ERR_ARGS;
  StartGroups sg;
  const bool tagged = options->tagged == 1 && nel > 0;
  if (tagged) {
    if (options->partitioner < 0 || options->partitioner > 2) return PARRSB_ERR_UNSUPPORTED;
    rc = tagged_groups(tag, nel, nparts, options->verbose_level, sg);
    if (rc != PARRSB_OK) return rc;
  }
  rc = guarded([&]() -> int {
    ctx().init();
    Workspace &W = ws();
    ll N = nel;
    if (N == 0) return PARRSB_OK;
    int ndim = (nv == 8) ? 3 : 2;
    {
      StageTimer tm(PARRSB_STAGE_UPLOAD);
      if (vtx) {
        W.vtx.ensure((size_t)N * nv);
        upload(W.vtx.p, vtx, (size_t)N * nv);
      }
      if (xyz) {
        W.xyz.ensure((size_t)N * nv * ndim);
        upload(W.xyz.p, xyz, (size_t)N * nv * ndim);
      }
      W.part.ensure((size_t)N);
    }
    maybe_fault("upload");
    DBuf<int> dseq;
    if (seq) dseq.alloc((size_t)N);
    part_mesh_dev(W.part.p, vtx ? W.vtx.p : nullptr, xyz ? W.xyz.p : nullptr, nel, nv, options,
                  nparts, seq ? dseq.p : nullptr, tagged ? &sg : nullptr);
    maybe_fault("partition");
    {
      StageTimer tm(PARRSB_STAGE_DOWNLOAD);
      d2h(part, W.part.p, (size_t)N);
      if (seq) d2h(seq, dseq.p, (size_t)N);
    }
    sync();
    return PARRSB_OK;
  });
  double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  ctx().stats.total_ms = sec * 1e3;
  ctx().stats.kernel_launches = ctx().kernel_launches;
  static const char *ALGO[3] = {"RSB", "RCB", "RIB"};
  if (rc == PARRSB_OK) {
    int pa = options->partitioner;
    print_if(options->verbose_level, "par%s finished in %g seconds.",
             (pa >= 0 && pa < 3) ? ALGO[pa] : "RSB", sec);
    print_profile(options);
  }
  return rc;
}

extern "C" int parrsb_part_mesh_device(int *d_part, const long long *d_vtx, const double *d_xyz,
                                       int nel, int nv, parrsb_options *options, int nparts) {
  auto t0 = std::chrono::steady_clock::now();
  int rc = prepare_options(d_vtx, d_xyz, nel, nv, options, nparts, nullptr, false);
  if (rc != PARRSB_OK) return rc;
  rc = guarded([&]() -> int {
    ctx().init();
    part_mesh_dev(d_part, d_vtx, d_xyz, nel, nv, options, nparts);
    return PARRSB_OK;
  });
  ctx().stats.total_ms =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() * 1e3;
  ctx().stats.kernel_launches = ctx().kernel_launches;
  return rc;
}

extern "C" int parrsb_conn_mesh(long long *vtx, double *coord, unsigned int nel, unsigned nDim,
                                long long *periodicInfo, int nPeriodicFaces, double tol) {
  int verbose = 1;
  if (const char *v = getenv("PARRSB_VERBOSE_LEVEL")) verbose = atoi(v);
  if (nDim < 2 || nDim > 3) return PARRSB_ERR_ARGS;
  if (nPeriodicFaces < 0 || (nPeriodicFaces > 0 && !periodicInfo)) return PARRSB_ERR_ARGS;
  if (nel > 0 && (!vtx || !coord)) return PARRSB_ERR_ARGS;
  auto t0 = std::chrono::steady_clock::now();
  print_if(verbose, "Running parCon ...");
  int rc = guarded([&]() -> int {
    ctx().init();
    Workspace &W = ws();
    int nv = nDim == 2 ? 4 : 8;
    ll np = (ll)nel * nv;
    if (np == 0) return PARRSB_OK;
    {
      StageTimer tm(PARRSB_STAGE_UPLOAD);
      W.xyz.ensure((size_t)np * nDim);
      upload(W.xyz.p, coord, (size_t)np * nDim);
      W.ids.ensure((size_t)np);
    }
    ll nseg = 0;
    int r;
    {
      StageTimer tm(PARRSB_STAGE_GENCON);
      r = gencon_device(nullptr, W.xyz.p, nel, (int)nDim, tol, W.gc, &nseg, nullptr);
    }
    ctx().stats.gencon_segments = nseg;
    if (r != PARRSB_OK) {
      print_if(1, "\t%s:%d element_check / face_check failed.", __FILE__, __LINE__);
      return r;
    }
    {
      // periodic faces (src/con.c:261-264); without any, the consecutive
      // renumbering leaves the ids as they are
      StageTimer tm(PARRSB_STAGE_GENCON);
      r = periodic_device(W.gc.ids.p, W.gc.x[0].p, W.gc.x[1].p, W.gc.x[2].p, nel, (int)nDim,
                          nseg, periodicInfo, nPeriodicFaces, W.gc.sort, &nseg);
      ctx().stats.gencon_segments = nseg;
      if (r != PARRSB_OK) {
        print_if(1, "\t%s:%d periodic faces did not match.", __FILE__, __LINE__);
        return r;
      }
      plus_one(W.gc.ids.p, np, W.ids.p);
    }
    {
      StageTimer tm(PARRSB_STAGE_DOWNLOAD);
      d2h(vtx, W.ids.p, (size_t)np);
      sync();
    }
    return PARRSB_OK;
  });
  double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  ctx().stats.total_ms = sec * 1e3;
  ctx().stats.kernel_launches = ctx().kernel_launches;
  if (rc == PARRSB_OK) print_if(verbose, "parCon (tol = %e) finished in %g s", tol, sec);
  return rc;
}

extern "C" int parrsb_conn_mesh_device(long long *d_vtx, const double *d_coord, unsigned int nel,
                                       unsigned nDim, double tol) {
  if (nDim < 2 || nDim > 3) return PARRSB_ERR_ARGS;
  auto t0 = std::chrono::steady_clock::now();
  int rc = guarded([&]() -> int {
    ctx().init();
    ll nseg = 0;
    int r = gencon_device(d_vtx, d_coord, nel, (int)nDim, tol, ws().gc, &nseg, nullptr);
    ctx().stats.gencon_segments = nseg;
    sync();
    return r;
  });
  ctx().stats.total_ms =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() * 1e3;
  ctx().stats.kernel_launches = ctx().kernel_launches;
  return rc;
}

extern "C" void fparrsb_conn_mesh(long long *vtx, double *coord, int *nel, int *nDim,
                                  long long *periodicInfo, int *nPeriodicFaces, double *tol,
                                  int *err) {
  *err = 1;
  *err = parrsb_conn_mesh(vtx, coord, (unsigned)*nel, (unsigned)*nDim, periodicInfo,
                          *nPeriodicFaces, *tol);
}

extern "C" int parrsb_get_stats(parrsb_stats *out) {
  if (!out) return PARRSB_ERR_ARGS;
  *out = ctx().stats;
  return PARRSB_OK;
}

extern "C" int parrsb_fiedler_groups(double *fiedler, long long *iters, double *resid,
                                     const long long *vtx, const int *group, int nel, int nv,
                                     int ngroups, parrsb_options *options, int batched) {
  if (!options || nel < 0 || nv < 1 || nv > 8 || ngroups < 1) return PARRSB_ERR_ARGS;
  if (nel > 0 && (!fiedler || !vtx || !group)) return PARRSB_ERR_ARGS;
  update_options(options);
  for (int e = 0; e < nel; e++)
    if (group[e] < 0 || group[e] >= ngroups) return PARRSB_ERR_ARGS;
  return guarded([&]() -> int {
    ctx().init();
    ll N = nel;
    std::vector<long long> it(ngroups, 0);
    std::vector<double> rs(ngroups, 0.0);
    if (N > 0) {
      DBuf<long long> dv((size_t)N * nv);
      DBuf<int> dg((size_t)N);
      DBuf<double> df((size_t)N);
      h2d(dv.p, vtx, (size_t)N * nv);
      h2d(dg.p, group, (size_t)N);
      RsbOpts ro;
      ro.miter = options->rsb_max_iter;
      ro.mpass = options->rsb_max_passes;
      ro.tol = options->rsb_tol;
      ro.fp32 = env_int("PARRSB_GPU_FP32", 0);
      ro.use_graphs = env_int("PARRSB_GPU_GRAPHS", 1);
      ro.batched = batched ? 1 : 0;
      ro.start = env_int("PARRSB_GPU_START", 0);
      ro.resid_stop = env_int("PARRSB_GPU_RESID_STOP", 0);
      ro.cg_factor = env_double("PARRSB_GPU_RESID_CG_FACTOR", 0.1);
      ro.reorth = env_int("PARRSB_GPU_REORTH", 0);
      fiedler_groups_device(dv.p, N, nv, dg.p, ngroups, ro, df.p, it.data(), rs.data());
      d2h(fiedler, df.p, (size_t)N);
      sync();
    }
    if (iters)
      for (int g = 0; g < ngroups; g++) iters[g] = it[g];
    if (resid)
      for (int g = 0; g < ngroups; g++) resid[g] = rs[g];
    ctx().stats.kernel_launches = ctx().kernel_launches;
    return PARRSB_OK;
  });
}

extern "C" int parrsb_part_quality(double *q, const int *part, const long long *vtx, int nel,
                                   int nv, int nparts) {
  if (!q || nel < 0 || nparts < 1 || nv < 1 || nv > 8) return PARRSB_ERR_ARGS;
  if (nel > 0 && (!part || !vtx)) return PARRSB_ERR_ARGS;
  for (int i = 0; i < nel; i++)
    if (part[i] < 0 || part[i] >= nparts) return PARRSB_ERR_ARGS;
  return guarded([&]() -> int {
    ctx().init();
    ll N = nel;
    if (N == 0) {
      for (int i = 0; i < 8; i++) q[i] = 0.0;
      return PARRSB_OK;
    }
    DBuf<long long> dv((size_t)N * nv);
    DBuf<int> dp((size_t)N);
    h2d(dv.p, vtx, (size_t)N * nv);
    h2d(dp.p, part, (size_t)N);
    part_quality_device(dv.p, dp.p, N, nv, nparts, q);
    return PARRSB_OK;
  });
}

extern "C" int parrsb_dual_graph(long long *rowptr, int *col, unsigned char *weight,
                                 long long *nnz, long long cap, const long long *vtx, int nel,
                                 int nv) {
  if (!nnz || nel < 0 || nv < 1 || nv > 8 || cap < 0) return PARRSB_ERR_ARGS;
  if (nel > 0 && (!vtx || !rowptr)) return PARRSB_ERR_ARGS;
  return guarded([&]() -> int {
    ctx().init();
    ll N = nel;
    *nnz = 0;
    if (N == 0) {
      if (rowptr) rowptr[0] = 0;
      return PARRSB_OK;
    }
    DBuf<long long> dv((size_t)N * nv);
    h2d(dv.p, vtx, (size_t)N * nv);
    std::vector<ll> rp;
    std::vector<int> c;
    std::vector<unsigned char> w;
    dual_graph_device(dv.p, N, nv, rp, c, w);
    *nnz = (long long)c.size();
    memcpy(rowptr, rp.data(), (size_t)(N + 1) * sizeof(long long));
    if (col && weight && (ll)c.size() <= cap) {
      memcpy(col, c.data(), c.size() * sizeof(int));
      memcpy(weight, w.data(), w.size());
    }
    ctx().stats.kernel_launches = ctx().kernel_launches;
    return PARRSB_OK;
  });
}

extern "C" int parrsb_components(int *ncomp, const long long *vtx, const int *group, int nel,
                                 int nv, int ngroups) {
  if (!ncomp || nel < 0 || nv < 1 || nv > 8 || ngroups < 1) return PARRSB_ERR_ARGS;
  if (nel > 0 && (!vtx || !group)) return PARRSB_ERR_ARGS;
  for (int e = 0; e < nel; e++)
    if (group[e] >= ngroups) return PARRSB_ERR_ARGS;
  return guarded([&]() -> int {
    ctx().init();
    ll N = nel;
    std::vector<int> c(ngroups, 0);
    if (N > 0) {
      DBuf<long long> dv((size_t)N * nv);
      DBuf<int> dg((size_t)N);
      h2d(dv.p, vtx, (size_t)N * nv);
      h2d(dg.p, group, (size_t)N);
      components_device(dv.p, N, nv, dg.p, ngroups, c.data());
    }
    for (int g = 0; g < ngroups; g++) ncomp[g] = c[g];
    ctx().stats.kernel_launches = ctx().kernel_launches;
    return PARRSB_OK;
  });
}

extern "C" void parrsb_gpu_finalize(void) {
  // every device this thread used: free its workspace on its own stream,
  // trim its pool and destroy the stream, with that device current
  int cur = 0;
  if (cudaGetDevice(&cur) != cudaSuccess) return;
  for (int dev = 0; dev < MAX_DEVICES; dev++) {
    if (!g_ws[dev] && !g_ctx.streams[dev]) continue;
    if (cudaSetDevice(dev) != cudaSuccess) continue;
    g_ctx.device = dev;
    g_ctx.stream = g_ctx.streams[dev];
    if (g_ws[dev]) {
      delete g_ws[dev];
      g_ws[dev] = nullptr;
    }
    if (g_ctx.stream) {
      cudaStreamSynchronize(g_ctx.stream);
      cudaMemPool_t pool;
      if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
      cudaStreamDestroy(g_ctx.stream);
      g_ctx.streams[dev] = nullptr;
    }
  }
  g_ctx.stream = nullptr;
  cudaSetDevice(cur);
}
