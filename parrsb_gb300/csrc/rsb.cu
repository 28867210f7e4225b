// rsb.cu -- recursive spectral bisection on one GB300.
//
// Restates, for every group of a recursion level at once (one segment of the
// element order per group of virtual ranks):
//   rsb                          src/rsb.c:262-350 (one node: ceil(log2 P)
//                                cuts, get_level_cuts :244-260, get_bin :231)
//   balance_partitions           src/rsb.c:118-229
//   fiedler / lanczos /
//   lanczos_aux / tqli           src/fiedler.c:13-30, 328-621
//   gs_weighted (Laplacian)      src/laplacian.c:159-205
//   get_components_v2 (count)    src/components.c:160-328
//
// Data layout in HBM: the dual graph is built once in original element
// order (CSR, int32 columns, uint8 weights).  Each level restricts it to the
// current groups and re-indexes it into the current element order as a
// sliced ELL matrix: slices of 32 consecutive rows, column-major inside a
// slice, one packed uint32 per entry (column in bits 0-27, weight in bits
// 28-31).  The Laplacian is applied in difference form y_i = sum_j w_ij
// (x_i - x_j) (exact integer weights).  Lanczos vectors are FP64 or FP32;
// every dot product, the tridiagonal matrix and the eigensolve are FP64.
// Dot products reduce per tile (512 to 8192 rows by the group's size; fixed
// trees) and then per group over its tiles (fixed order), so results are
// bitwise repeatable.  With FP32 vectors the residual check forms L f
// exactly in 64-bit fixed point.
#include <math.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>

#include "rsb.cuh"
#include "warm.cuh"

namespace prsb {

namespace {

constexpr int LZ_THREADS = 256;
constexpr ll LZ_TILE = 8192;  // largest tile (rows)

// Rows per tile of a group of n rows: big groups keep few partials per
// reduction, smaller ones get enough blocks to fill the GPU.
inline ll tile_rows(ll n) {
  return n >= (1ll << 22) ? LZ_TILE : n >= (1ll << 16) ? 2048 : 512;
}
constexpr int MAX_MITER = 120;

// ----------------------------------------------------------------------------
// Dual graph build
// ----------------------------------------------------------------------------
__global__ void k_vid_keys(const long long *__restrict__ vtx, ll ns,
                           u64 *__restrict__ keys, int *__restrict__ vals) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns) return;
  keys[i] = (u64)vtx[i] ^ 0x8000000000000000ull;
  vals[i] = (int)i;
}

__global__ void k_run_flags(const u64 *__restrict__ keys, ll ns, int *__restrict__ flag) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ns) flag[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void k_run_bounds(const int *__restrict__ flag, const ll *__restrict__ excl,
                             ll ns, ll nruns, int *__restrict__ runid,
                             ll *__restrict__ run_start) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns) return;
  ll r = excl[i] + flag[i] - 1;
  runid[i] = (int)r;
  if (flag[i]) run_start[r] = i;
  if (i == ns - 1) run_start[nruns] = ns;
}

__global__ void k_scatter_inv(const int *__restrict__ vals, ll n, int *__restrict__ inv) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) inv[vals[i]] = (int)i;
}

// Dual-graph rows, one warp per element a (src/con.c's element graph: two
// elements are adjacent when they share a vertex, weighted by the number of
// shared vertex pairs).  The candidates of a are the elements of the runs of
// its vertices, vertex by vertex, each run in slot order; an element b != a
// occurs once per (vertex of a, equal vertex of b) pair, so its weight is its
// number of occurrences, and the row lists every b at its first occurrence.
// Up to GR_CAP candidates sit in shared memory, where a per-warp open-
// addressing table (GR_HASH slots: element, count, first index) counts each
// element's occurrences and keeps its first one in O(C) instead of
// comparing every pair; a longer list is read from the runs again and
// compared pairwise.  FILL = false: row lengths and the largest weight;
// FILL = true: columns and weights at rowptr[a].
constexpr int GR_WARPS = 4;
constexpr int GR_CAP = 256;
constexpr int GR_HASH = 256;  // power of two >= GR_CAP: more slots than distinct keys

__device__ __forceinline__ int gr_slot0(int b) {
  return (int)(((unsigned)b * 2654435761u) >> 24);  // Fibonacci hashing to 8 bits
}

template <bool FILL>
__global__ void __launch_bounds__(GR_WARPS * 32)
k_graph_rows(int nv, ll N, const int *__restrict__ sorted_slot, const int *__restrict__ inv,
             const int *__restrict__ runid, const ll *__restrict__ run_start,
             const ll *__restrict__ rowptr, int *__restrict__ col,
             unsigned char *__restrict__ wout, ll *__restrict__ rowlen, int *__restrict__ maxw) {
  __shared__ __align__(16) int cand[GR_WARPS][GR_CAP + 4];
  __shared__ int hkey[GR_WARPS][GR_HASH], hcnt[GR_WARPS][GR_HASH], hfirst[GR_WARPS][GR_HASH];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int h = lane; h < GR_HASH; h += 32)  // empty: key -1, count 0, first INT_MAX
    hkey[wid][h] = -1, hcnt[wid][h] = 0, hfirst[wid][h] = 0x7fffffff;
  __syncwarp();
  const unsigned lt = (1u << lane) - 1u;
  const ll a = (ll)blockIdx.x * GR_WARPS + wid;
  int wmax = 0;
  if (a < N) {  // warp-uniform
    // run of each vertex of a (lane k < nv), then every lane holds all of them
    // (slot positions and candidate counts fit 32 bits: N < 2^28, nv <= 8)
    int rs = 0, rl = 0;
    if (lane < nv) {
      const int r = runid[inv[a * nv + lane]];
      rs = (int)run_start[r];
      rl = (int)(run_start[r + 1] - run_start[r]);
    }
    int RS[8], EX[8];
    int C = 0;
#pragma unroll
    for (int k = 0; k < 8; k++) {
      RS[k] = __shfl_sync(0xffffffffu, rs, k);
      EX[k] = C;
      C += __shfl_sync(0xffffffffu, rl, k);  // lanes >= nv hold 0
    }
    auto cand_at = [&](int t) -> int {  // element of candidate t
      int base = RS[0] - EX[0];
#pragma unroll
      for (int k = 1; k < 8; k++)
        if (k < nv && t >= EX[k]) base = RS[k] - EX[k];
      return sorted_slot[base + t] / nv;
    };
    const bool staged = C <= GR_CAP;
    if (staged) {
      for (int t = lane; t < C; t += 32) {
        const int b = cand_at(t);
        cand[wid][t] = b;
        if (b == (int)a) continue;
        int h = gr_slot0(b);
        for (;;) {  // fewer distinct keys than slots (a != b): a free or equal slot exists
          const int prev = atomicCAS(&hkey[wid][h], -1, b);
          if (prev == -1 || prev == b) break;
          h = (h + 1) & (GR_HASH - 1);
        }
        atomicAdd(&hcnt[wid][h], 1);
        atomicMin(&hfirst[wid][h], (int)t);
      }
      __syncwarp();
    }
    ll out = 0;
    for (int t0 = 0; t0 < C; t0 += 32) {
      const int t = t0 + lane;
      bool first = false;
      int b = -1, cnt = 0;
      if (t < C) {
        b = staged ? cand[wid][t] : cand_at(t);
        if (b != (int)a) {
          if (staged) {
            int h = gr_slot0(b);
            while (hkey[wid][h] != b) h = (h + 1) & (GR_HASH - 1);  // b was inserted
            cnt = hcnt[wid][h];
            first = hfirst[wid][h] == (int)t;
          } else {
            int before = 0;  // occurrences of b ahead of t
            for (int j = 0; j < C; j++) {
              const int m = cand_at(j) == b;
              cnt += m;
              before += m & (j < t);
            }
            first = before == 0;
          }
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, first);
      if (first) {
        if (FILL) {
          const ll pos = rowptr[a] + out + __popc(m & lt);
          col[pos] = b;
          wout[pos] = (unsigned char)(cnt > 255 ? 255 : cnt);
        }
        wmax = max(wmax, cnt);
      }
      out += __popc(m);
    }
    if (!FILL && lane == 0) rowlen[a] = out;
    if (staged) {  // empty the table again: find every used slot, then clear
      __syncwarp();
      int hs[GR_CAP / 32];
#pragma unroll
      for (int k = 0; k < GR_CAP / 32; k++) {
        const int t = lane + 32 * k;
        hs[k] = -1;
        if (t < C) {
          const int b = cand[wid][t];
          if (b != (int)a) {
            int h = gr_slot0(b);
            while (hkey[wid][h] != b) h = (h + 1) & (GR_HASH - 1);
            hs[k] = h;
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int k = 0; k < GR_CAP / 32; k++)
        if (hs[k] >= 0) hkey[wid][hs[k]] = -1, hcnt[wid][hs[k]] = 0, hfirst[wid][hs[k]] = 0x7fffffff;
      __syncwarp();
    }
  }
  if (!FILL) {  // one atomic per warp; every lane reaches the shuffles
    for (int off = 16; off > 0; off >>= 1)
      wmax = max(wmax, __shfl_xor_sync(0xffffffffu, wmax, off));
    if (lane == 0 && wmax) atomicMax(maxw, wmax);
  }
}

__global__ void k_max_ll(const ll *__restrict__ v, ll n, unsigned long long *__restrict__ m) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long x = i < n ? (unsigned long long)v[i] : 0ull;
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long y = __shfl_xor_sync(0xffffffffu, x, off);
    x = y > x ? y : x;
  }
  if ((threadIdx.x & 31) == 0 && x) atomicMax(m, x);  // one atomic per warp
}

// ----------------------------------------------------------------------------
// Level restriction to sliced ELL (current order, same-group entries only)
// ----------------------------------------------------------------------------
__global__ void k_inv_perm(const int *__restrict__ perm, ll N, int *__restrict__ inv) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) inv[perm[i]] = (int)i;
}

// The level-matrix kernels walk a dual-graph row per thread through two
// dependent gathers per entry (position inv[col], its group); eight entries
// at a time keep eight of each in flight instead of one.
__global__ void k_ell_count(const int *__restrict__ perm, const int *__restrict__ inv,
                            const int *__restrict__ grp, const ll *__restrict__ rowptr,
                            const int *__restrict__ col, ll N, int *__restrict__ rowlen) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int g = grp[i];
  int cnt = 0;
  if (g >= 0) {
    int a = perm[i];
    const ll q0 = rowptr[a], q1 = rowptr[a + 1];
    ll q = q0;
    for (; q + 8 <= q1; q += 8) {
      int j[8];
#pragma unroll
      for (int u = 0; u < 8; u++) j[u] = inv[col[q + u]];
#pragma unroll
      for (int u = 0; u < 8; u++) cnt += grp[j[u]] == g;
    }
    for (; q < q1; q++) cnt += grp[inv[col[q]]] == g;
  }
  rowlen[i] = cnt;
}

__global__ void k_max_int(const int *__restrict__ a, ll n, int *__restrict__ mx) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  int v = i < n ? a[i] : 0;
  for (int off = 16; off > 0; off >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, off));
  if ((threadIdx.x & 31) == 0 && v > 0) atomicMax(mx, v);
}

__global__ void k_slice_w(const int *__restrict__ rowlen, ll N, ll nslice,
                          ll *__restrict__ slots, int *__restrict__ width) {
  ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslice) return;
  int m = 0;
  for (int l = 0; l < 32; l++) {
    ll i = s * 32 + l;
    if (i < N && rowlen[i] > m) m = rowlen[i];
  }
  width[s] = m;
  slots[s] = (ll)m * 32;
}

__global__ void k_ell_fill(const int *__restrict__ perm, const int *__restrict__ inv,
                           const int *__restrict__ grp, const ll *__restrict__ rowptr,
                           const int *__restrict__ col, const unsigned char *__restrict__ w,
                           ll N, const ll *__restrict__ slice_off,
                           const int *__restrict__ width, unsigned *__restrict__ ell) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  ll s = i >> 5;
  unsigned *out = ell + slice_off[s] + (i & 31);
  int wd = width[s];
  int k = 0;
  int g = grp[i];
  if (g >= 0) {
    int a = perm[i];
    const ll q0 = rowptr[a], q1 = rowptr[a + 1];
    ll q = q0;
    for (; q + 8 <= q1; q += 8) {  // same entries in the same order, eight gathers in flight
      int j[8], gj[8];
#pragma unroll
      for (int u = 0; u < 8; u++) j[u] = inv[col[q + u]];
#pragma unroll
      for (int u = 0; u < 8; u++) gj[u] = grp[j[u]];
#pragma unroll
      for (int u = 0; u < 8; u++)
        if (gj[u] == g) {
          out[(ll)k * 32] = (unsigned)j[u] | ((unsigned)w[q + u] << 28);
          k++;
        }
    }
    for (; q < q1; q++) {
      int j = inv[col[q]];
      if (grp[j] == g) {
        out[(ll)k * 32] = (unsigned)j | ((unsigned)w[q] << 28);
        k++;
      }
    }
  }
  for (; k < wd; k++) out[(ll)k * 32] = (unsigned)i;  // weight 0 padding
}

// ----------------------------------------------------------------------------
// Segmented Lanczos
// ----------------------------------------------------------------------------
struct GState {
  double rtz1, rtz2, beta, pap, alpha, c, rtol, rnorm;
  double resid, ff;
  ll start, n;
  ll total_iters;
  int tile0, ntiles, miter, run, iters, done, active, npass;
  int warm;  // start from the learned prediction (else the fallback start)
  int stall;          // residual-stop mode: restarts in a row without progress
  double prev_resid;  //   and the residual of the restart before
  int stopreq;        // a Ritz residual check asks to end the pass (k_ritz_bound)
  int rb_it;          //   the step of the group's last computed check in this pass,
  double rb_theta;    //   its smallest Ritz value and its bound
  double rb_bound;
};

__device__ __forceinline__ double block_sum(double v, double *sh) {
  v = warp_tree_sum(v);
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0) {
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s = __dadd_rn(s, sh[w]);
  }
  return s;
}

enum Gate { GATE_ALL = 0, GATE_ACTIVE = 1, GATE_RUN = 2 };

__device__ __forceinline__ bool gate_ok(const GState &s, int gate) {
  if (gate == GATE_RUN) return s.run != 0;
  if (gate == GATE_ACTIVE) return s.active != 0;
  return true;
}

// initial vector of the first pass: initv[i] = i + 1 (+ 1000 n if i < n/2)
// in the group's current order (src/fiedler.c:574-578).
__device__ __forceinline__ double initv_formula(ll li, ll n) {
  double v = (double)li + 1.0;
  if (li < n / 2) v = v + (double)(1000 * n);
  return v;
}


enum FinOp {
  FIN_IV_MEAN = 0,
  FIN_IV_NORM,
  FIN_INIT_MEAN,
  FIN_INIT_RTR,
  FIN_PMEAN,
  FIN_PAP,
  FIN_RTR,
  FIN_RITZ_MEAN,
  FIN_PASS_END,
  FIN_NORM,
  FIN_RESID1,
  FIN_RESID2,
  FIN_ORIENT,
  FIN_PASS_END_R,  // pass end when the eigen-residual decides the restarts
  FIN_RESID_GATE   // residual of the Ritz vector; restart while above tol
};

// The scalar update OP of group g from its reduced tile partials tot, by
// one thread.  owner = false leaves the per-group arrays (diagT, upperT,
// vnorm) untouched: the persistent step kernel applies the step updates in
// every block that holds a tile of the group (same inputs, same result) and
// lets one block write them.
template <int OP>
__device__ __forceinline__ void fin_apply(GState &s, int g, double tot0, double tot1, int it,
                                          int MI, double tol, int mpass,
                                          double *__restrict__ diagT,
                                          double *__restrict__ upperT,
                                          double *__restrict__ vnorm,
                                          int *__restrict__ any_active, bool owner);

// One block per group: reduce the group's tile partials in a fixed order
// (thread-strided sequential sums, then the block tree of LZ_THREADS
// threads) and apply the scalar update OP.  Run by a whole block: either the
// dedicated k_fin launch or, fused, the last tile block of the group to
// finish.
template <int OP, bool WIDE = false>
__device__ void fin_body(GState &s, int g, const double *__restrict__ part, int it, int MI,
                         double tol, int mpass, double *__restrict__ diagT,
                         double *__restrict__ upperT, double *__restrict__ vnorm,
                         int *__restrict__ any_active, double *sh) {
  const int nv = (OP == FIN_RESID1) ? 2 : 1;
  double tot[2] = {0.0, 0.0};
  if (OP != FIN_PASS_END) {
    for (int v = 0; v < nv; v++) {
      double acc = 0.0;
      const int bd = blockDim.x;
      if (WIDE) {  // up to eight loads in flight per thread, then the adds in order
        for (int q = threadIdx.x; q < s.ntiles; q += 8 * bd) {
          double x[8];
#pragma unroll
          for (int u = 0; u < 8; u++)
            x[u] = q + u * bd < s.ntiles ? __ldcg(&part[(ll)nv * (s.tile0 + q + u * bd) + v])
                                         : 0.0;
#pragma unroll
          for (int u = 0; u < 8; u++)
            if (q + u * bd < s.ntiles) acc = __dadd_rn(acc, x[u]);
        }
      } else {  // the same adds with fewer registers (inlined into the tile kernels)
        int q = threadIdx.x;
        for (; q + 7 * bd < s.ntiles; q += 8 * bd) {
          double x[8];
#pragma unroll
          for (int u = 0; u < 8; u++) x[u] = __ldcg(&part[(ll)nv * (s.tile0 + q + u * bd) + v]);
#pragma unroll
          for (int u = 0; u < 8; u++) acc = __dadd_rn(acc, x[u]);
        }
        for (; q < s.ntiles; q += bd)
          acc = __dadd_rn(acc, __ldcg(&part[(ll)nv * (s.tile0 + q) + v]));
      }
      tot[v] = block_sum(acc, sh);
      __syncthreads();
    }
  }
  if (threadIdx.x != 0) return;
  fin_apply<OP>(s, g, tot[0], tot[1], it, MI, tol, mpass, diagT, upperT, vnorm, any_active,
                true);
}

template <int OP>
__device__ __forceinline__ void fin_apply(GState &s, int g, double tot0, double tot1, int it,
                                          int MI, double tol, int mpass,
                                          double *__restrict__ diagT,
                                          double *__restrict__ upperT,
                                          double *__restrict__ vnorm,
                                          int *__restrict__ any_active, bool owner) {
  const double tot[2] = {tot0, tot1};
  double dn = (double)s.n;
  if (OP == FIN_IV_MEAN || OP == FIN_INIT_MEAN || OP == FIN_PMEAN || OP == FIN_RITZ_MEAN) {
    s.c = __ddiv_rn(tot[0], dn);
  } else if (OP == FIN_IV_NORM) {
    s.alpha = __ddiv_rn(1.0, __dsqrt_rn(tot[0]));
  } else if (OP == FIN_INIT_RTR) {
    double rtr = tot[0];
    double rnorm = __dsqrt_rn(rtr);
    s.rnorm = rnorm;
    s.rtol = __dmul_rn(rnorm, tol);
    if (owner) vnorm[(ll)g * (MI + 1)] = rnorm;
    s.rtz2 = 1.0;
    s.rtz1 = rtr;
    s.beta = 0.0;
    s.pap = 0.0;
    s.run = 1;
    s.iters = 0;
    s.done = 0;
    s.stopreq = 0;
    s.rb_it = -1;
    s.rb_theta = 0.0;
    s.rb_bound = 1e300;
  } else if (OP == FIN_PAP) {
    double pap = tot[0], pap_old = s.pap;
    s.pap = pap;
    s.alpha = __ddiv_rn(s.rtz1, pap);
    if (!owner) {
    } else if (it == 0) {
      diagT[(ll)g * MI] = __ddiv_rn(pap, s.rtz1);
    } else {
      double bb = __dmul_rn(s.beta, s.beta);
      diagT[(ll)g * MI + it] = __ddiv_rn(__dadd_rn(__dmul_rn(bb, pap_old), pap), s.rtz1);
      upperT[(ll)g * MI + it - 1] =
          __ddiv_rn(__dmul_rn(-s.beta, pap_old), __dsqrt_rn(__dmul_rn(s.rtz2, s.rtz1)));
    }
  } else if (OP == FIN_RTR) {
    double rtr = tot[0];
    double rnorm = __dsqrt_rn(rtr);
    if (owner) vnorm[(ll)g * (MI + 1) + it + 1] = rnorm;
    s.rnorm = rnorm;
    s.iters = it + 1;
    if (rnorm < s.rtol) {
      s.done = 1;
      s.run = 0;
    } else if (it + 1 >= s.miter) {
      s.run = 0;
    }
    s.rtz2 = s.rtz1;
    s.rtz1 = rtr;
    s.beta = __ddiv_rn(s.rtz1, s.rtz2);
    // the off-diagonal that the next step's FIN_PAP enters (the same
    // expression on the same values), known now for the Ritz residual bound
    if (owner && it + 1 < MI)
      upperT[(ll)g * MI + it] =
          __ddiv_rn(__dmul_rn(-s.beta, s.pap), __dsqrt_rn(__dmul_rn(s.rtz2, s.rtz1)));
  } else if (OP == FIN_PASS_END) {
    s.total_iters += s.iters;
    s.npass += 1;
    s.active = (s.iters == s.miter && s.npass < mpass) ? 1 : 0;
    if (s.active) atomicOr(any_active, 1);
    atomicMax(any_active + 1, s.iters);
  } else if (OP == FIN_PASS_END_R) {
    s.total_iters += s.iters;
    s.npass += 1;
    atomicMax(any_active + 1, s.iters);  // active stays set until FIN_RESID_GATE
  } else if (OP == FIN_RESID_GATE) {
    // restart while the residual is above tol, at most mpass restarts, and
    // stop after three restarts in a row within 2 tol that did not lower it
    // by 10% (the vector has reached what the working precision allows;
    // farther from tol a slow group keeps restarting)
    s.resid = __ddiv_rn(__dsqrt_rn(tot[0]), __dsqrt_rn(s.ff));
    if (s.resid < 2.0 * tol && s.resid > 0.9 * s.prev_resid) s.stall += 1; else s.stall = 0;
    s.prev_resid = s.resid;
    s.active = (!(s.resid <= tol) && s.npass < mpass && s.stall < 3) ? 1 : 0;
    if (s.active) atomicOr(any_active, 1);
  } else if (OP == FIN_NORM) {
    s.c = __ddiv_rn(1.0, __dsqrt_rn(tot[0]));
  } else if (OP == FIN_RESID1) {
    s.ff = tot[1];
    s.c = __ddiv_rn(tot[0], tot[1]);  // Rayleigh quotient
  } else if (OP == FIN_RESID2) {
    s.resid = __ddiv_rn(__dsqrt_rn(tot[0]), __dsqrt_rn(s.ff));
  } else if (OP == FIN_ORIENT) {
    if (tot[0] < 0.0) s.c = -s.c;  // canonical sign: sum_i s_i f_i >= 0
  }
}

template <int OP, int GATE>
__global__ void k_fin(GState *__restrict__ gs, int ngroups, const double *__restrict__ part,
                      int it, int MI, double tol, int mpass,
                      double *__restrict__ diagT, double *__restrict__ upperT,
                      double *__restrict__ vnorm, int *__restrict__ any_active) {
  pdl_entry();
  __shared__ double sh[32];
  int g = blockIdx.x;
  if (g >= ngroups) return;
  GState &s = gs[g];
  if (!gate_ok(s, GATE)) return;
  fin_body<OP, true>(s, g, part, it, MI, tol, mpass, diagT, upperT, vnorm, any_active, sh);
}

// Fused finalisation: after a tile block has written its partial, the last
// block of the group (per-group arrival counter) runs fin_body.
struct FinArgs {
  int *cnt;  // per-group arrival counters (zero between uses)
  int it, MI, mpass;
  double tol;
  double *diagT, *upperT, *vnorm;
  int *any;
};

template <int OP>
__device__ __forceinline__ void fused_fin(GState *gs, int g, const double *part,
                                          const FinArgs &fa, double *sh) {
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    int prev = atomicAdd(&fa.cnt[g], 1);
    s_last = (prev == gs[g].ntiles - 1);
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  fin_body<OP>(gs[g], g, part, fa.it, fa.MI, fa.tol, fa.mpass, fa.diagT, fa.upperT, fa.vnorm,
               fa.any, sh);
  if (threadIdx.x == 0) fa.cnt[g] = 0;
}

// Small non-negative integer (< 2^23) to float without a conversion
// instruction: 2^23 + w has w in the low mantissa bits.
__device__ __forceinline__ float small_u2f(unsigned w) {
  return __int_as_float(0x4B000000 | w) - 8388608.0f;
}

// Generic per-tile pass.  MODE selects the element-wise work.
enum TileMode {
  TM_IV_SUM = 0,     // sum of initv formula
  TM_IV_SQ = 1,      // sum of (initv - c)^2
  TM_IV_WRITE = 2,   // f = (initv - c) * scale   (scale in alpha)
  TM_SUM_F = 3,      // sum f
  TM_INIT_R = 4,     // r = f - c, V0 = r, sum r^2
  TM_P = 5,          // k_pr: p = beta (p - c) + r, sum p      (r = V[it])
  TM_R = 6,          // k_pr: V[it+1] = V[it] - alpha w, sum V[it+1]^2
  TM_SUB_C = 7,      // f -= c
  TM_SQ_F = 8,       // sum f^2
  TM_SCALE_F = 9,    // f *= c
  TM_RESID1 = 10,    // y = L f in FP64 -> y64; sums f.y, f.f
  TM_RESID2 = 11,    // sum (y - rho f)^2
  TM_SUM_F_WARM = 12, // same as TM_SUM_F but for a warm start vector
  TM_ORIENT = 13,     // sum s_i f_i, s = +1 on the first half of the group, -1 after
  TM_LOAD_Y = 14,     // f = y (FP64 per position, passed as y64)
  TM_RANDOM = 15,     // f = seeded uniform values in [-1, 1)
  TM_SELECT = 16      // groups without the warm flag: f = V (the saved fallback)
};

// SplitMix64 (Steele, Lea and Flood, 2014): the seeded random start vector
// of position li of a group, uniform in [-1, 1).
__device__ __forceinline__ double random_start(ll li) {
  unsigned long long z = (unsigned long long)li * 0x9E3779B97F4A7C15ull + 0x2545F4914F6CDD1Dull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (double)(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
}

// Canonical per-tile reductions.  A tile's rows are cut into 32-row chunks
// aligned to the ELL slices; a warp owns whole chunks (lane = row % 32), a
// chunk is reduced by a fixed shuffle tree and the tile partial is the sum of
// its chunk values in chunk order.  The result therefore does not depend on
// the CTA size, which the autotuner is free to choose.
//   FP32 terms: compensated (TwoSum / TwoProduct) pairs through the tree;
//   FP64 terms: plain FP64 tree.
__device__ __forceinline__ void two_sum_pair(float &s, float &c, float s2, float c2) {
  float t = s + s2;
  float bp = t - s;
  float e = (s - (t - bp)) + (s2 - bp);
  s = t;
  c = c + c2 + e;
}

__device__ __forceinline__ double chunk_sum_pair(float s, float c) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    float s2 = __shfl_down_sync(0xffffffffu, s, off);
    float c2 = __shfl_down_sync(0xffffffffu, c, off);
    two_sum_pair(s, c, s2, c2);
  }
  return (double)s + (double)c;
}

template <typename VT>
struct Term {  // one row's contribution to a dot product
  VT s = (VT)0, c = (VT)0;
  __device__ __forceinline__ void set(VT x) { s = x, c = (VT)0; }
  __device__ __forceinline__ void set_prod(VT a, VT b) {
    s = a * b;
    c = (VT)fma(a, b, -s);
  }
  __device__ __forceinline__ double chunk() const;
};
template <>
__device__ __forceinline__ double Term<float>::chunk() const { return chunk_sum_pair(s, c); }
template <>
__device__ __forceinline__ double Term<double>::chunk() const { return warp_tree_sum(s + c); }

// Tile partial from its chunk values cs[0..nc), run by warp 0: lane l sums
// cs[l], cs[l + 32], ... in order, then the fixed shuffle tree; the result
// (lane 0) depends only on the chunk values, never on the CTA size.
__device__ __forceinline__ double tile_total(const double *cs, int nc) {
  double t = 0.0;
  for (int q = threadIdx.x & 31; q < nc; q += 32) t = __dadd_rn(t, cs[q]);
  return warp_tree_sum(t);
}

// FP32 kernels keep the compensated pair through the chunk and the tile:
// the chunk value is the pair left by the fixed shuffle tree, and the tile
// partial sums the chunk pairs (lane l: chunks l, l + 32, ... in order, then
// the fixed tree) before one conversion to FP64.  GB300's FP64 pipe issues a
// warp instruction about every 16 cycles per SM, so a per-chunk conversion
// and FP64 add would cost more than the memory traffic of the chunk.
__device__ __forceinline__ float2 chunk_pair(float s, float c) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    float s2 = __shfl_down_sync(0xffffffffu, s, off);
    float c2 = __shfl_down_sync(0xffffffffu, c, off);
    two_sum_pair(s, c, s2, c2);
  }
  return make_float2(s, c);
}
__device__ __forceinline__ double tile_total_pair(const float2 *cs, int nc) {
  float s = 0.f, c = 0.f;
  for (int q = threadIdx.x & 31; q < nc; q += 32) two_sum_pair(s, c, cs[q].x, cs[q].y);
  const float2 t = chunk_pair(s, c);
  return (double)t.x + (double)t.y;
}

template <typename VT, int MODE, int GATE, int FUSE>
__global__ void __launch_bounds__(512)
k_tile(const ll *__restrict__ tbeg, const ll *__restrict__ tend,
       const int *__restrict__ tgrp, GState *__restrict__ gs, VT *__restrict__ f,
       VT *__restrict__ V, ll N, int it, double *__restrict__ part,
       const unsigned *__restrict__ ell, const ll *__restrict__ slice_off,
       const int *__restrict__ slice_w, double *__restrict__ y64, FinArgs fa) {
  pdl_entry();
  __shared__ double sh[32];
  __shared__ double cs[2][LZ_TILE / 32 + 1];
  int t = blockIdx.x;
  int g = tgrp[t];
  const GState &s = gs[g];
  if (!gate_ok(s, GATE)) return;
  const VT c = (VT)s.c;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const ll b = tbeg[t], e = tend[t];
  const ll c0 = b >> 5;
  const int nc = (int)(((e - 1) >> 5) - c0 + 1);
  constexpr bool has_sum = !(MODE == TM_IV_WRITE || MODE == TM_SUB_C || MODE == TM_SCALE_F ||
                             MODE == TM_LOAD_Y || MODE == TM_RANDOM || MODE == TM_SELECT);
  constexpr bool fp64_term = (MODE == TM_IV_SUM || MODE == TM_IV_SQ || MODE == TM_RESID1 ||
                              MODE == TM_RESID2);
  for (int q = warp; q < nc; q += nw) {
    ll i = (c0 + q) * 32 + lane;
    bool valid = i >= b && i < e;
    Term<VT> tv;
    double d1 = 0.0, d2 = 0.0;  // FP64 terms of the setup / check passes
    if (valid) {
      if (MODE == TM_IV_SUM) {
        d1 = initv_formula(i - s.start, s.n);
      } else if (MODE == TM_IV_SQ) {
        double v = __dsub_rn(initv_formula(i - s.start, s.n), s.c);
        d1 = __dmul_rn(v, v);
      } else if (MODE == TM_IV_WRITE) {
        double v = __dsub_rn(initv_formula(i - s.start, s.n), s.c);
        f[i] = (VT)__dmul_rn(v, s.alpha);
      } else if (MODE == TM_SUM_F || MODE == TM_SUM_F_WARM) {
        tv.set(f[i]);
      } else if (MODE == TM_INIT_R) {
        VT qv = f[i] - c;
        V[i] = qv;  // r_0 is row 0 of the Krylov basis
        tv.set_prod(qv, qv);
      } else if (MODE == TM_SUB_C) {
        f[i] = f[i] - c;
      } else if (MODE == TM_SQ_F) {
        tv.set_prod(f[i], f[i]);
      } else if (MODE == TM_ORIENT) {
        tv.set((i - s.start) < s.n / 2 ? f[i] : -f[i]);
      } else if (MODE == TM_SCALE_F) {
        f[i] = (VT)((double)f[i] * s.c);
      } else if (MODE == TM_LOAD_Y) {
        f[i] = (VT)y64[i];
      } else if (MODE == TM_RANDOM) {
        f[i] = (VT)random_start(i - s.start);
      } else if (MODE == TM_SELECT) {
        if (!s.warm) f[i] = V[i];
      } else if (MODE == TM_RESID1) {
        double fi = (double)f[i];
        ll sl = i >> 5;
        const unsigned *ep = ell + slice_off[sl] + (i & 31);
        int wd = slice_w[sl];
        double yv = 0.0;
        for (int k = 0; k < wd; k++) {
          unsigned x = ep[(ll)k * 32];
          yv = __dadd_rn(yv, __dmul_rn((double)(x >> 28),
                                       __dsub_rn(fi, (double)f[x & 0x0FFFFFFFu])));
        }
        y64[i] = yv;
        d1 = __dmul_rn(fi, yv);
        d2 = __dmul_rn(fi, fi);
      } else if (MODE == TM_RESID2) {
        double v = __dsub_rn(y64[i], __dmul_rn(s.c, (double)f[i]));
        d1 = __dmul_rn(v, v);
      }
    }
    if (has_sum) {
      double v1 = fp64_term ? warp_tree_sum(d1) : tv.chunk();
      if (MODE == TM_RESID1) {
        double v2 = warp_tree_sum(d2);
        if (lane == 0) cs[1][q] = v2;
      }
      if (lane == 0) cs[0][q] = v1;
    }
  }
  if (has_sum) {
    __syncthreads();
    if (threadIdx.x < 32) {
      if (MODE == TM_RESID1) {
        double v0 = tile_total(cs[0], nc), v1 = tile_total(cs[1], nc);
        if (threadIdx.x == 0) part[2 * t] = v0, part[2 * t + 1] = v1;
      } else {
        double v0 = tile_total(cs[0], nc);
        if (threadIdx.x == 0) part[t] = v0;
      }
    }
    if (FUSE >= 0) fused_fin<FUSE>(gs, g, part, fa, sh);
  }
}

// ---------------------------------------------------------------------------
// y = L f of the residual check for FP32 vectors, exact in 64-bit fixed
// point on the integer pipe instead of one FP64 subtract, multiply and add
// (plus two conversions) per nonzero on the FP64 pipe, which runs at 1/64 of
// the FP32 rate.  Each group's f is scaled by 2^S_g so that its largest
// |f| lies in [2^46, 2^47) and truncated to integers Fq (entries at least
// 2^-22 of the group's largest are exact; smaller ones lose at most
// 2^-47 of it).  Then y_i = d_i Fq_i - sum_j w_ij Fq_j is exact in int64
// for rows of fewer than 2048 stored entries (|terms| < 2^51 each) and is
// rounded once to FP64.  The sums f.y, f.f and (y - rho f)^2 stay FP64 but
// each lane first accumulates its own rows (one FMA per row and sum) before
// one warp tree per warp: a tree per 32-row chunk, as k_tile's FP64 form
// does, costs five more FP64 adds per row, and the FP64 pipe, not the
// gathers, bounded that form.
// ---------------------------------------------------------------------------
constexpr int RQ_MAX_WIDTH = 2048;  // widest ELL slice the integer form accepts
constexpr int RQ_THREADS = 256;     // the tile sums' order depends on it

// per tile: the largest |f| of the tile's rows (IEEE bits, which order like
// the magnitudes)
template <int GATE>
__global__ void __launch_bounds__(512)
k_rq_max(const ll *__restrict__ tbeg, const ll *__restrict__ tend, const int *__restrict__ tgrp,
         const GState *__restrict__ gs, const float *__restrict__ f, unsigned *__restrict__ tmax) {
  pdl_entry();
  __shared__ unsigned wm[16];
  const int t = blockIdx.x, g = tgrp[t];
  if (!gate_ok(gs[g], GATE)) return;
  unsigned m = 0;
  for (ll i = tbeg[t] + threadIdx.x; i < tend[t]; i += blockDim.x)
    m = max(m, __float_as_uint(f[i]) & 0x7FFFFFFFu);
  for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x >> 5); k++) m = max(m, wm[k]);
    tmax[t] = m;
  }
}

// the group's largest |f| from its tiles' maxima (every block of the group
// computes it; the block of the group's first tile also stores it)
__device__ __forceinline__ unsigned rq_group_max(const GState &s, int t,
                                                 const unsigned *__restrict__ tmax,
                                                 unsigned *__restrict__ gmax, int g) {
  __shared__ unsigned wm[16];
  unsigned m = 0;
  for (int q = threadIdx.x; q < s.ntiles; q += blockDim.x) m = max(m, tmax[s.tile0 + q]);
  for (int off = 16; off > 0; off >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
  __syncthreads();
  m = wm[0];
  for (int k = 1; k < (int)(blockDim.x >> 5); k++) m = max(m, wm[k]);
  if (threadIdx.x == 0 && t == s.tile0) gmax[g] = m;
  return m;
}

// S_g - 150 + 23 folded: an entry of biased exponent E is shifted by
// E - Emax + 23 (Emax: biased exponent of the group's largest |f|)
__device__ __forceinline__ ll rq_quantize(float x, unsigned gm) {
  const unsigned u = __float_as_uint(x);
  const int E = (int)((u >> 23) & 0xFF);
  if (E == 0) return 0;  // zero and subnormals (below 2^-126)
  const ll m = (ll)((u & 0x7FFFFFu) | 0x800000u);
  const int sh = E - (int)(gm >> 23) + 23;
  const ll v = sh >= 0 ? (m << sh) : (sh > -24 ? (m >> -sh) : 0);
  return (u >> 31) ? -v : v;
}

template <int GATE>
__global__ void __launch_bounds__(512)
k_rq_quant(const ll *__restrict__ tbeg, const ll *__restrict__ tend, const int *__restrict__ tgrp,
           const GState *__restrict__ gs, const float *__restrict__ f,
           const unsigned *__restrict__ tmax, unsigned *__restrict__ gmax,
           ll *__restrict__ fq) {
  pdl_entry();
  const int t = blockIdx.x, g = tgrp[t];
  if (!gate_ok(gs[g], GATE)) return;
  const unsigned gm = rq_group_max(gs[g], t, tmax, gmax, g);
  for (ll i = tbeg[t] + threadIdx.x; i < tend[t]; i += blockDim.x) fq[i] = rq_quantize(f[i], gm);
}

template <int GATE>
__global__ void __launch_bounds__(RQ_THREADS)
k_rq_resid1(const ll *__restrict__ tbeg, const ll *__restrict__ tend,
            const int *__restrict__ tgrp, const GState *__restrict__ gs,
            const float *__restrict__ f, const ll *__restrict__ fq,
            const unsigned *__restrict__ gmax, const unsigned *__restrict__ ell,
            const ll *__restrict__ slice_off, const int *__restrict__ slice_w,
            double *__restrict__ y64, double *__restrict__ part) {
  pdl_entry();
  __shared__ double cs[2][RQ_THREADS / 32];
  const int t = blockIdx.x, g = tgrp[t];
  if (!gate_ok(gs[g], GATE)) return;
  const unsigned gm = gmax[g];
  // 2^-S_g with S_g = 46 - (Emax - 127); a group whose largest |f| is not
  // finite gets NaN (its residual then never wins and never passes)
  const bool finite = gm < 0x7F800000u;
  const double unscale =
      __longlong_as_double((ll)(1023 - 46 + ((int)(gm >> 23) - 127)) << 52);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const ll b = tbeg[t], e = tend[t];
  const ll c0 = b >> 5;
  const int nc = (int)(((e - 1) >> 5) - c0 + 1);
  double a1 = 0.0, a2 = 0.0;  // this lane's f.y and f.f over its rows, in slice order
  for (int q = warp; q < nc; q += RQ_THREADS / 32) {
    const ll i = (c0 + q) * 32 + lane;
    if (i < b || i >= e) continue;
    const ll sl = i >> 5;
    const unsigned *ep = ell + slice_off[sl] + (i & 31);
    const int wd = slice_w[sl];
    ll acc = 0;
    int dsum = 0;
    int k = 0;
#pragma unroll 1
    for (; k + 8 <= wd; k += 8) {
      unsigned x[8];
#pragma unroll
      for (int u = 0; u < 8; u++) x[u] = __ldcs(ep + (ll)(k + u) * 32);
      ll fj[8];
#pragma unroll
      for (int u = 0; u < 8; u++) fj[u] = fq[x[u] & 0x0FFFFFFFu];
#pragma unroll
      for (int u = 0; u < 8; u++) {
        acc += (ll)(x[u] >> 28) * fj[u];
        dsum += (int)(x[u] >> 28);
      }
    }
    for (; k < wd; k++) {
      const unsigned x = __ldcs(ep + (ll)k * 32);
      acc += (ll)(x >> 28) * fq[x & 0x0FFFFFFFu];
      dsum += (int)(x >> 28);
    }
    const ll yq = (ll)dsum * fq[i] - acc;
    const double yv = finite ? __dmul_rn(__ll2double_rn(yq), unscale)
                             : __longlong_as_double(0x7FF8000000000000ll);
    y64[i] = yv;
    const double fi = (double)f[i];
    a1 = __fma_rn(fi, yv, a1);
    a2 = __fma_rn(fi, fi, a2);  // fi * fi is exact
  }
  const double v1 = warp_tree_sum(a1), v2 = warp_tree_sum(a2);
  if (lane == 0) cs[0][warp] = v1, cs[1][warp] = v2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s1 = 0.0, s2 = 0.0;
    for (int w = 0; w < RQ_THREADS / 32; w++) s1 = __dadd_rn(s1, cs[0][w]), s2 = __dadd_rn(s2, cs[1][w]);
    part[2 * t] = s1, part[2 * t + 1] = s2;
  }
}

// sum (y - rho f)^2 per tile for the FP32 residual check (rho in the group
// state's c): a thread's rows in order, warp trees, the warps in order
template <int GATE>
__global__ void __launch_bounds__(RQ_THREADS)
k_rq_resid2(const ll *__restrict__ tbeg, const ll *__restrict__ tend,
            const int *__restrict__ tgrp, const GState *__restrict__ gs,
            const float *__restrict__ f, const double *__restrict__ y64,
            double *__restrict__ part) {
  pdl_entry();
  __shared__ double cs[RQ_THREADS / 32];
  const int t = blockIdx.x, g = tgrp[t];
  const GState &s = gs[g];
  if (!gate_ok(s, GATE)) return;
  const double rho = s.c;
  double a = 0.0;
  for (ll i = tbeg[t] + threadIdx.x; i < tend[t]; i += RQ_THREADS) {
    const double v = __fma_rn(-rho, (double)f[i], y64[i]);
    a = __fma_rn(v, v, a);
  }
  const double w = warp_tree_sum(a);
  if ((threadIdx.x & 31) == 0) cs[threadIdx.x >> 5] = w;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s1 = 0.0;
    for (int k = 0; k < RQ_THREADS / 32; k++) s1 = __dadd_rn(s1, cs[k]);
    part[t] = s1;
  }
}

// Rows per lane of the vectorised tile kernels: one 16-byte load per array.
template <typename VT>
struct VecOf;
template <>
struct VecOf<float> {
  using T = float4;
  static constexpr int R = 4;
  __device__ static __forceinline__ void get(const T &v, float *x) {
    x[0] = v.x, x[1] = v.y, x[2] = v.z, x[3] = v.w;
  }
  __device__ static __forceinline__ T make(const float *x) {
    return make_float4(x[0], x[1], x[2], x[3]);
  }
};
template <>
struct VecOf<double> {
  using T = double2;
  static constexpr int R = 2;
  __device__ static __forceinline__ void get(const T &v, double *x) { x[0] = v.x, x[1] = v.y; }
  __device__ static __forceinline__ T make(const double *x) { return make_double2(x[0], x[1]); }
};

// rows [i0, i0 + R) of a, restricted to the tile [b, e) (others read as 0)
template <typename VT>
__device__ __forceinline__ void load_rows(const VT *__restrict__ a, ll i0, ll b, ll e,
                                          VT *x) {
  using V = VecOf<VT>;
  if (i0 >= b && i0 + V::R <= e) {
    V::get(*reinterpret_cast<const typename V::T *>(a + i0), x);
  } else {
#pragma unroll
    for (int k = 0; k < V::R; k++) x[k] = (i0 + k >= b && i0 + k < e) ? a[i0 + k] : (VT)0;
  }
}
template <typename VT>
__device__ __forceinline__ void store_rows(VT *__restrict__ a, ll i0, ll b, ll e,
                                           const VT *x) {
  using V = VecOf<VT>;
  if (i0 >= b && i0 + V::R <= e) {
    *reinterpret_cast<typename V::T *>(a + i0) = V::make(x);
  } else {
#pragma unroll
    for (int k = 0; k < V::R; k++)
      if (i0 + k >= b && i0 + k < e) a[i0 + k] = x[k];
  }
}

// A lane's running sum of its rows' terms: compensated pair in FP32, plain
// FP64 otherwise; chunk() reduces the warp's pairs with the fixed tree.
template <typename VT>
struct LaneSum {
  VT s = (VT)0, c = (VT)0;
  __device__ __forceinline__ void add(const Term<VT> &t);
  __device__ __forceinline__ double chunk() const;
  __device__ __forceinline__ float2 pair() const { return chunk_pair((float)s, (float)c); }
};
template <>
__device__ __forceinline__ void LaneSum<float>::add(const Term<float> &t) {
  two_sum_pair(s, c, t.s, t.c);
}
template <>
__device__ __forceinline__ void LaneSum<double>::add(const Term<double> &t) {
  s = s + (t.s + t.c);
}
template <>
__device__ __forceinline__ double LaneSum<float>::chunk() const { return chunk_sum_pair(s, c); }
template <>
__device__ __forceinline__ double LaneSum<double>::chunk() const { return warp_tree_sum(s); }

// The two vector updates of a Lanczos step (src/fiedler.c:233-262, CG form),
// R consecutive rows per lane and PR_U chunks of 32 R rows per warp in flight
// (16-byte loads).  r is row `it` of the Krylov basis V.
//   TM_P: p = r (it 0) or beta (p - c) + r; tile partial of sum p
//   TM_R: V[it+1] = V[it] - alpha w; tile partial of sum V[it+1]^2
// The chunk decomposition (32 R rows, aligned to multiples of 32 R) does not
// depend on the CTA size.  The last tile block of a group finalises it.
// k_pr: PR_U chunks per warp in flight on big levels (at least PR_BIG rows),
// one chunk per warp on smaller ones so that enough warps fill the GPU
constexpr ll PR_BIG = 1ll << 22;

// One tile [b, e) of a vector update: the rows, then (thread 0) the tile
// partial into *out.  Called by every thread of the block.
template <typename VT, int MODE, int PR_U>
__device__ __forceinline__ void pr_tile(ll b, ll e, VT c, VT beta, VT alpha, int it,
                                        VT *__restrict__ p, const VT *__restrict__ w,
                                        VT *__restrict__ V, ll N, double *cs, float2 *cs2,
                                        double *__restrict__ part, int t) {
  using Vec = VecOf<VT>;
  constexpr int R = Vec::R, CH = 32 * R;
  const VT *__restrict__ rv = V + (ll)it * N;
  VT *__restrict__ rn = V + (ll)(it + 1) * N;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const ll c0 = b / CH;
  const int nc = (int)((e - 1) / CH - c0 + 1);
  for (int q0 = PR_U * warp; q0 < nc; q0 += PR_U * nw) {
    ll i0[PR_U];
    VT x[PR_U][R], y[PR_U][R];
#pragma unroll
    for (int u = 0; u < PR_U; u++) {
      i0[u] = (c0 + q0 + u) * CH + (ll)lane * R;
      if (q0 + u < nc) {  // warp-uniform
        load_rows(rv, i0[u], b, e, x[u]);
        if (MODE == TM_R || it > 0) load_rows(MODE == TM_P ? (const VT *)p : w, i0[u], b, e, y[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < PR_U; u++) {
      if (q0 + u >= nc) break;
      LaneSum<VT> acc;
      VT o[R];
#pragma unroll
      for (int k = 0; k < R; k++) {
        Term<VT> tv;
        if (MODE == TM_P) {
          o[k] = it == 0 ? x[u][k] : (VT)fma(beta, y[u][k] - c, x[u][k]);
          tv.set(o[k]);
        } else {
          o[k] = (VT)fma(-alpha, y[u][k], x[u][k]);
          tv.set_prod(o[k], o[k]);
        }
        if (i0[u] + k >= b && i0[u] + k < e) acc.add(tv);
      }
      store_rows(MODE == TM_P ? p : rn, i0[u], b, e, o);
      if constexpr (sizeof(VT) == 4) {
        const float2 v = acc.pair();
        if (lane == 0) cs2[q0 + u] = v;
      } else {
        const double v = acc.chunk();
        if (lane == 0) cs[q0 + u] = v;
      }
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const double v0 = sizeof(VT) == 4 ? tile_total_pair(cs2, nc) : tile_total(cs, nc);
    if (threadIdx.x == 0) part[t] = v0;
  }
}

template <typename VT, int MODE, int PR_U, bool FUSE = true>
__global__ void __launch_bounds__(512)
k_pr(const ll *__restrict__ tbeg, const ll *__restrict__ tend, const int *__restrict__ tgrp,
     GState *__restrict__ gs, VT *__restrict__ p, const VT *__restrict__ w,
     VT *__restrict__ V, ll N, double *__restrict__ part, FinArgs fa) {
  pdl_entry();
  constexpr int CH = 32 * VecOf<VT>::R;
  constexpr int OP = MODE == TM_P ? FIN_PMEAN : FIN_RTR;
  __shared__ double sh[32];
  __shared__ double cs[LZ_TILE / CH + 2];
  __shared__ float2 cs2[LZ_TILE / CH + 2];  // chunk pairs (FP32)
  const int t = blockIdx.x;
  const int g = tgrp[t];
  const GState &s = gs[g];
  if (!s.run) return;
  pr_tile<VT, MODE, PR_U>(tbeg[t], tend[t], (VT)s.c, (VT)s.beta, (VT)s.alpha, fa.it, p, w, V, N,
                          cs, cs2, part, t);
  if (FUSE) fused_fin<OP>(gs, g, part, fa, sh);
}

// threads per block of k_pr / k_ritz for tiles of at most `rows` rows
template <typename VT>
inline int vec_threads(ll rows, int chunks_per_warp) {
  const ll ch = 32 * VecOf<VT>::R;
  ll warps = (rows / ch + chunks_per_warp - 1) / chunks_per_warp;
  if (warps < 1) warps = 1;
  if (warps > 16) warps = 16;
  return (int)warps * 32;
}

// w = L p and sum w_i (p_i - c) per tile.  FP32: difference form
// w_i = sum_j w_ij (p_i - p_j) with FFMA.  FP64: w_i = d_i p_i - sum_j w_ij p_j
// (the gather-scatter form of the reference, src/laplacian.c:188-205) with
// one DFMA per nonzero and the weights taken from a shared-memory table.
// A warp processes one 32-row ELL slice at a time (fully coalesced index
// loads, uniform width).  The index stream is read with the evict-first
// policy so that the vectors (p, w, the Krylov rows) stay in L2 between the
// launches of a step.
// One tile [b, e) of the SpMV: w = L p on the tile's rows, then (thread 0)
// the tile partial of sum w (p - c) into *out.  Called by every thread of
// the block; wlut holds the weights 0..15 as doubles (FP64 form).
template <typename VT>
__device__ __forceinline__ void spmv_tile(ll b, ll e, VT c, const unsigned *__restrict__ ell,
                                          const ll *__restrict__ slice_off,
                                          const int *__restrict__ slice_w,
                                          const VT *__restrict__ p, VT *__restrict__ w,
                                          const double *wlut, double *cs, float2 *cs2,
                                          double *__restrict__ part, int t) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const ll c0 = b >> 5;
  const int nc = (int)(((e - 1) >> 5) - c0 + 1);
  for (int q = warp; q < nc; q += nw) {
    const ll sl = c0 + q;
    const ll i = sl * 32 + lane;
    const bool valid = i >= b && i < e;
    const unsigned *ep = ell + slice_off[sl] + lane;
    // lanes outside the tile skip the row (slots of rows >= N are never written)
    const int wd = valid ? slice_w[sl] : 0;
    const VT pi = valid ? p[i] : (VT)0;
    VT y;
    if (sizeof(VT) == 4) {
      float sum = 0.f;
      int k = 0;
#pragma unroll 1
      for (; k + 8 <= wd; k += 8) {
        unsigned x[8];
#pragma unroll
        for (int u = 0; u < 8; u++) x[u] = __ldcs(ep + (ll)(k + u) * 32);
        float pj[8];
#pragma unroll
        for (int u = 0; u < 8; u++) pj[u] = (float)p[x[u] & 0x0FFFFFFFu];
#pragma unroll
        for (int u = 0; u < 8; u++) sum = fmaf(small_u2f(x[u] >> 28), (float)pi - pj[u], sum);
      }
      for (; k < wd; k++) {
        unsigned x = __ldcs(ep + (ll)k * 32);
        sum = fmaf(small_u2f(x >> 28), (float)pi - (float)p[x & 0x0FFFFFFFu], sum);
      }
      y = (VT)sum;
    } else {
      double sum = 0.0;
      unsigned dsum = 0;
      int k = 0;
#pragma unroll 1
      for (; k + 8 <= wd; k += 8) {
        unsigned x[8];
#pragma unroll
        for (int u = 0; u < 8; u++) x[u] = __ldcs(ep + (ll)(k + u) * 32);
        double pj[8];
#pragma unroll
        for (int u = 0; u < 8; u++) pj[u] = (double)p[x[u] & 0x0FFFFFFFu];
#pragma unroll
        for (int u = 0; u < 8; u++) {
          sum = fma(wlut[x[u] >> 28], pj[u], sum);
          dsum += x[u] >> 28;
        }
      }
      for (; k < wd; k++) {
        unsigned x = __ldcs(ep + (ll)k * 32);
        sum = fma(wlut[x >> 28], (double)p[x & 0x0FFFFFFFu], sum);
        dsum += x >> 28;
      }
      y = (VT)fma((double)dsum, (double)pi, -sum);
    }
    Term<VT> tv;
    if (valid) {
      w[i] = y;
      tv.set_prod(y, pi - c);
    }
    if constexpr (sizeof(VT) == 4) {
      const float2 v = chunk_pair(tv.s, tv.c);
      if (lane == 0) cs2[q] = v;
    } else {
      const double v = tv.chunk();
      if (lane == 0) cs[q] = v;
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const double v0 = sizeof(VT) == 4 ? tile_total_pair(cs2, nc) : tile_total(cs, nc);
    if (threadIdx.x == 0) part[t] = v0;
  }
}

template <typename VT>
__global__ void __launch_bounds__(512)
k_spmv(const ll *__restrict__ tbeg, const ll *__restrict__ tend,
       const int *__restrict__ tgrp, GState *__restrict__ gs,
       const unsigned *__restrict__ ell, const ll *__restrict__ slice_off,
       const int *__restrict__ slice_w, const VT *__restrict__ p, VT *__restrict__ w,
       double *__restrict__ part, FinArgs fa, int fuse, int force) {
  pdl_entry();
  __shared__ double sh[32];
  __shared__ double cs[LZ_TILE / 32 + 1];
  __shared__ float2 cs2[LZ_TILE / 32 + 1];  // chunk pairs (FP32)
  __shared__ double wlut[16];
  if (threadIdx.x < 16) wlut[threadIdx.x] = (double)threadIdx.x;
  __syncthreads();
  int t = blockIdx.x;
  int g = tgrp[t];
  if (!gs[g].run && !force) return;
  spmv_tile<VT>(tbeg[t], tend[t], (VT)gs[g].c, ell, slice_off, slice_w, p, w, wlut, cs, cs2,
                part, t);
  if (fuse) fused_fin<FIN_PAP>(gs, g, part, fa, sh);
}

// ---------------------------------------------------------------------------
// SpMV with the index stream staged by the Tensor Memory Accelerator.
// Same arithmetic and reduction order as k_spmv (bitwise the same w and tile
// partials), but the ELL words of SP_SS consecutive slices are copied into
// shared memory by one cp.async.bulk per stage (SP_NST stages in flight,
// completion counted on an mbarrier), so the warps only wait on the gathers
// of p, never on the DRAM latency of the index stream.  Warp w handles slice
// w of every stage.  A wait gives up after about two seconds of clock and
// sets err[0]; every thread still meets every __syncthreads.
// ---------------------------------------------------------------------------
constexpr int SP_NST = 3;  // stages in flight per block

__device__ __forceinline__ u32 smem_u32addr(const void *p) {
  return (u32)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(u32 bar, u32 count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(u32 bar, u32 bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(u32 bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_test(u32 bar, u32 parity) {
  u32 ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// bounded wait: false after ~2 s of SM clock
__device__ __forceinline__ bool mbar_wait(u32 bar, u32 parity) {
  if (mbar_test(bar, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_test(bar, parity)) {
    if (clock64() - t0 > 4000000000ll) return false;
    __nanosleep(20);
  }
  return true;
}
__device__ __forceinline__ void bulk_g2s(u32 dst, const void *src, u32 bytes, u32 bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(dst),
      "l"(src), "r"(bytes), "r"(bar)
      : "memory");
}

__global__ void __launch_bounds__(512)
k_spmv_tma(const ll *__restrict__ tbeg, const ll *__restrict__ tend,
           const int *__restrict__ tgrp, GState *__restrict__ gs,
           const unsigned *__restrict__ ell, const ll *__restrict__ slice_off,
           const int *__restrict__ slice_w, const float *__restrict__ p, float *__restrict__ w,
           double *__restrict__ part, FinArgs fa, int fuse, int force, int stage_bytes,
           int *__restrict__ err) {
  pdl_entry();
  extern __shared__ __align__(128) unsigned char sp_smem[];
  __shared__ double sh[32];
  __shared__ float2 cs[LZ_TILE / 32 + 1];  // chunk pairs
  __shared__ ll soff[LZ_TILE / 32 + 2];
  __shared__ __align__(8) unsigned long long bars[SP_NST];
  const int t = blockIdx.x;
  const int g = tgrp[t];
  if (!gs[g].run && !force) return;
  const float c = (float)gs[g].c;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const ll b = tbeg[t], e = tend[t];
  const ll c0 = b >> 5;
  const int nc = (int)(((e - 1) >> 5) - c0 + 1);
  const int nst = (nc + nw - 1) / nw;  // stages of nw slices
  for (int q = threadIdx.x; q <= nc; q += blockDim.x) soff[q] = slice_off[c0 + q];
  if (threadIdx.x == 0) {
    for (int k = 0; k < SP_NST; k++) mbar_init(smem_u32addr(&bars[k]), 1);
    mbar_fence_init();
  }
  __syncthreads();
  // Thread 0 issues the copies; a stage larger than its buffer is never
  // copied (issue_bad).  `bad` is block-uniform (barrier-reduced): once a
  // wait gives up or a stage is oversized, no further copy is issued, the
  // block stops computing, drains the copies still in flight (bounded
  // waits) and reports through err.
  bool issue_bad = false;
  int issued = 0;  // stages issued so far (thread 0)
  auto issue = [&](int j) {  // thread 0: stage j into buffer j % SP_NST
    const int q0 = j * nw, q1 = min(q0 + nw, nc);
    const u32 bytes = (u32)((soff[q1] - soff[q0]) * 4);
    const u32 bar = smem_u32addr(&bars[j % SP_NST]);
    issued = j + 1;
    if (bytes > (u32)stage_bytes) {  // never copy past the stage buffer
      issue_bad = true;
      mbar_arrive(bar);
    } else if (bytes == 0) {
      mbar_arrive(bar);
    } else {
      mbar_expect_tx(bar, bytes);
      bulk_g2s(smem_u32addr(sp_smem + (size_t)(j % SP_NST) * stage_bytes), ell + soff[q0],
               bytes, bar);
    }
  };
  if (threadIdx.x == 0)
    for (int j = 0; j < SP_NST && j < nst; j++) issue(j);
  bool bad = false;
  int j = 0;
  for (; j < nst; j++) {
    const int buf = j % SP_NST;
    const bool ok = mbar_wait(smem_u32addr(&bars[buf]), (u32)((j / SP_NST) & 1));
    bad = __syncthreads_or(!ok || issue_bad) != 0;
    if (bad) break;
    const int q = j * nw + warp;
    if (q < nc) {
      const ll sl = c0 + q;
      const ll i = sl * 32 + lane;
      const bool valid = i >= b && i < e;
      const int wd = valid ? slice_w[sl] : 0;
      const float pi = valid ? p[i] : 0.f;
      const unsigned *ep = reinterpret_cast<const unsigned *>(
                               sp_smem + (size_t)buf * stage_bytes) +
                           (soff[q] - soff[j * nw]) + lane;
      float sum = 0.f;
      int k = 0;
#pragma unroll 1
      for (; k + 8 <= wd; k += 8) {
        unsigned x[8];
#pragma unroll
        for (int u = 0; u < 8; u++) x[u] = ep[(k + u) * 32];
        float pj[8];
#pragma unroll
        for (int u = 0; u < 8; u++) pj[u] = p[x[u] & 0x0FFFFFFFu];
#pragma unroll
        for (int u = 0; u < 8; u++) sum = fmaf(small_u2f(x[u] >> 28), pi - pj[u], sum);
      }
      for (; k < wd; k++) {
        unsigned x = ep[k * 32];
        sum = fmaf(small_u2f(x >> 28), pi - p[x & 0x0FFFFFFFu], sum);
      }
      Term<float> tv;
      if (valid) {
        w[i] = sum;
        tv.set_prod(sum, pi - c);
      }
      const float2 v = chunk_pair(tv.s, tv.c);
      if (lane == 0) cs[q] = v;
    } else if (q < nc && lane == 0) {
      cs[q] = make_float2(0.f, 0.f);
    }
    __syncthreads();  // buffer j % SP_NST is free again
    if (threadIdx.x == 0 && j + SP_NST < nst) issue(j + SP_NST);
  }
  if (bad) {
    // stages j .. issued - 1 may still be in flight (stage j's wait gave up
    // or it was oversized): wait for each once more, bounded, so that no
    // copy is left writing into this block's shared memory if it can end
    if (threadIdx.x == 0)
      for (int k = j; k < issued; k++) mbar_wait(smem_u32addr(&bars[k % SP_NST]), (u32)((k / SP_NST) & 1));
    __syncthreads();
  }
  if (threadIdx.x < 32) {
    const double v0 = bad ? 0.0 : tile_total_pair(cs, nc);
    if (threadIdx.x == 0) {
      if (bad) atomicExch(err, 1);
      part[t] = v0;
    }
  }
  if (fuse) fused_fin<FIN_PAP>(gs, g, part, fa, sh);
}

// ---------------------------------------------------------------------------
// Persistent segmented step kernel: every Lanczos step of a pass
// (src/fiedler.c:458-504) for all groups of the level in one cooperative
// launch, in place of the six launches per step (P update, its
// finalisation, SpMV, finalisation, R update, finalisation).  Block b owns
// tiles b, b + G, b + 2G, ... (G blocks, all resident: a cooperative launch
// refuses a grid that does not fit).  A step is three phases separated by
// grid barriers; each phase runs the same tile body as the stand-alone
// kernel (pr_tile, spmv_tile) and writes the same tile partials, into a
// partial array of its own.  After a barrier every block reduces, for each
// of its tiles whose group runs, the group's partials in the order of k_fin
// (256 virtual threads: strided sequential sums, warp trees, the warps in
// order) and applies the scalar update to its own copy of the group state
// in shared memory; the block holding the group's first tile writes the
// per-group arrays and, at the end, the state.  Results are bitwise those of
// the launch-per-kernel pass.  Each barrier wait gives up after about one
// second (globaltimer), sets err and returns; a block that sees err set
// returns at its next barrier, so the kernel always ends.
// ---------------------------------------------------------------------------
constexpr int PS_THREADS = LZ_THREADS;  // the finalisation order is k_fin's
constexpr int PS_SLOTS = 32;            // tiles per block at most

struct StepArgs {
  const ll *tbeg, *tend;
  const int *tgrp;
  GState *gs;
  void *p, *w, *V;
  ll VS;
  const unsigned *ell;
  const ll *slice_off;
  const int *slice_w;
  double *part;  // 3 T: the P, SpMV and R tile partials
  double *diagT, *upperT, *vnorm;
  unsigned *bar;  // barrier arrivals (zero at launch)
  int *run_cnt;   // per step: groups still running after it (zero at launch)
  int *err;       // 2: a barrier wait gave up
  int T, MI;
  double tol;
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__global__ void k_ps_reset(unsigned *__restrict__ bar, int *__restrict__ run_cnt, int MI) {
  pdl_entry();
  if (threadIdx.x == 0) bar[0] = 0u;
  for (int i = threadIdx.x; i < MI; i += blockDim.x) run_cnt[i] = 0;
}

// Grid barrier number k (targets k G arrivals).  False when it gave up or
// another block did.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned target, int *err) {
  __shared__ int ok_s;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(bar, 1u);
    int ok = 1;
    const unsigned long long t0 = global_ns();
    for (unsigned n = 0;; n++) {
      if (ld_acquire_u32(bar) >= target) break;
      if (*(volatile int *)err) {
        ok = 0;
        break;
      }
      if ((n & 63) == 63 && (global_ns() - t0 > 1000000000ull || n > (1u << 26))) {
        atomicExch(err, 2);  // about one second, or 2^26 polls of at least 64 ns
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    __threadfence();
    ok_s = ok;
  }
  __syncthreads();
  __threadfence();  // every thread: later loads see the other blocks' writes
  return ok_s != 0;
}

// The step finalisation OP for every slot of the block whose group runs, in
// k_fin's reduction order (256 threads: strided sequential sums, warp trees,
// the warps in order).  A group of more than 256 tiles is reduced by the
// whole block with k_fin's own code (eight loads in flight per thread); a
// smaller one by one warp that stands in for the 256 threads (each holds at
// most one partial), all of its loads issued before the trees.
template <int OP>
__device__ __forceinline__ void step_fin(GState *st, const int *sg, int nslot,
                                         const double *__restrict__ part, const StepArgs &a,
                                         int it, double *sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < nslot; k++) {  // big groups: the whole block
    GState &s = st[k];
    if (!s.run || s.ntiles <= PS_THREADS) continue;  // block-uniform
    double acc = 0.0;
    for (int q = threadIdx.x; q < s.ntiles; q += 8 * PS_THREADS) {  // as fin_body
      double x[8];
#pragma unroll
      for (int u = 0; u < 8; u++)
        x[u] = q + u * PS_THREADS < s.ntiles ? __ldcg(&part[s.tile0 + q + u * PS_THREADS]) : 0.0;
#pragma unroll
      for (int u = 0; u < 8; u++)
        if (q + u * PS_THREADS < s.ntiles) acc = __dadd_rn(acc, x[u]);
    }
    const double tot = block_sum(acc, sh);
    if (threadIdx.x == 0) {
      const int t = blockIdx.x + k * gridDim.x;
      fin_apply<OP>(s, sg[k], tot, 0.0, it, a.MI, a.tol, 0, a.diagT, a.upperT, a.vnorm, nullptr,
                    t == s.tile0);
    }
    __syncthreads();
  }
  for (int k = warp; k < nslot; k += PS_THREADS / 32) {  // small groups: a warp each
    GState &s = st[k];
    if (!s.run || s.ntiles > PS_THREADS) continue;  // warp-uniform
    double x[PS_THREADS / 32];
#pragma unroll
    for (int u = 0; u < PS_THREADS / 32; u++) {
      const int q = lane + 32 * u;
      x[u] = q < s.ntiles ? __dadd_rn(0.0, __ldcg(&part[s.tile0 + q])) : 0.0;
    }
    double tot = 0.0;
#pragma unroll
    for (int u = 0; u < PS_THREADS / 32; u++) {
      const double ws = warp_tree_sum(x[u]);
      if (lane == 0) tot = __dadd_rn(tot, ws);
    }
    if (lane == 0) {
      const int t = blockIdx.x + k * gridDim.x;
      fin_apply<OP>(s, sg[k], tot, 0.0, it, a.MI, a.tol, 0, a.diagT, a.upperT, a.vnorm, nullptr,
                    t == s.tile0);
    }
  }
}

template <typename VT>
__global__ void __launch_bounds__(PS_THREADS, 8) k_steps(StepArgs a) {
  __shared__ GState st[PS_SLOTS];
  __shared__ int sg[PS_SLOTS];
  __shared__ double cs[LZ_TILE / 32 + 2];
  __shared__ float2 cs2[LZ_TILE / 32 + 2];
  __shared__ double wlut[16];
  __shared__ double sh[32];
  const int G = gridDim.x;
  const int nslot = (a.T - (int)blockIdx.x + G - 1) / G;  // tiles blockIdx.x + k G < T
  VT *p = static_cast<VT *>(a.p), *w = static_cast<VT *>(a.w), *V = static_cast<VT *>(a.V);
  double *partP = a.part, *partS = a.part + a.T, *partR = a.part + 2 * (ll)a.T;
  for (int k = threadIdx.x; k < nslot; k += PS_THREADS) {
    sg[k] = a.tgrp[blockIdx.x + k * G];
    st[k] = a.gs[sg[k]];
  }
  if (threadIdx.x < 16) wlut[threadIdx.x] = (double)threadIdx.x;
  __syncthreads();
  unsigned nbar = 0;
  for (int it = 0; it < a.MI; it++) {
    // p = r (step 0) or beta (p - c) + r; partials of sum p
    for (int k = 0; k < nslot; k++) {
      if (!st[k].run) continue;  // block-uniform
      const int t = blockIdx.x + k * G;
      pr_tile<VT, TM_P, 1>(a.tbeg[t], a.tend[t], (VT)st[k].c, (VT)st[k].beta, (VT)st[k].alpha,
                           it, p, w, V, a.VS, cs, cs2, partP, t);
      __syncthreads();
    }
    if (!grid_barrier(a.bar, ++nbar * (unsigned)G, a.err)) return;
    if (it > 0 && ld_acquire_u32(reinterpret_cast<const unsigned *>(a.run_cnt) + it - 1) == 0)
      break;  // no group of the level runs (the same value in every block)
    step_fin<FIN_PMEAN>(st, sg, nslot, partP, a, it, sh);
    __syncthreads();
    // w = L p; partials of sum w (p - c)
    for (int k = 0; k < nslot; k++) {
      if (!st[k].run) continue;
      const int t = blockIdx.x + k * G;
      spmv_tile<VT>(a.tbeg[t], a.tend[t], (VT)st[k].c, a.ell, a.slice_off, a.slice_w, p, w, wlut,
                    cs, cs2, partS, t);
      __syncthreads();
    }
    if (!grid_barrier(a.bar, ++nbar * (unsigned)G, a.err)) return;
    step_fin<FIN_PAP>(st, sg, nslot, partS, a, it, sh);
    __syncthreads();
    // V[it+1] = V[it] - alpha w; partials of sum V[it+1]^2
    for (int k = 0; k < nslot; k++) {
      if (!st[k].run) continue;
      const int t = blockIdx.x + k * G;
      pr_tile<VT, TM_R, 1>(a.tbeg[t], a.tend[t], (VT)st[k].c, (VT)st[k].beta, (VT)st[k].alpha,
                           it, p, w, V, a.VS, cs, cs2, partR, t);
      __syncthreads();
    }
    if (!grid_barrier(a.bar, ++nbar * (unsigned)G, a.err)) return;
    step_fin<FIN_RTR>(st, sg, nslot, partR, a, it, sh);
    __syncthreads();
    if (threadIdx.x == 0) {
      int running = 0;
      for (int k = 0; k < nslot; k++)
        if (blockIdx.x + k * G == st[k].tile0 && st[k].run) running++;
      if (running) atomicAdd(&a.run_cnt[it], running);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nslot; k += PS_THREADS)
    if ((int)blockIdx.x + k * G == st[k].tile0) a.gs[sg[k]] = st[k];
}

// Ritz vector f_i = sum_j coef_j V_j[i] (j < iters, src/fiedler.c:520-535)
// and the tile partial of sum f, R rows per lane (16-byte loads of each
// basis row).  FP32: compensated dot (Ogita, Rump and Oishi's Dot2) with each
// coefficient split into two floats, so the sum keeps about twice single
// precision before its one rounding to float.  FP64: DFMA chain.
template <typename VT>
__global__ void __launch_bounds__(512)
k_ritz(const ll *__restrict__ tbeg, const ll *__restrict__ tend,
       const int *__restrict__ tgrp, const GState *__restrict__ gs,
       const VT *__restrict__ V, ll N, const double *__restrict__ coef, int MI,
       VT *__restrict__ f, double *__restrict__ part) {
  pdl_entry();
  using Vec = VecOf<VT>;
  constexpr int R = Vec::R, CH = 32 * R;
  __shared__ double cf[MAX_MITER];
  __shared__ float ch[MAX_MITER], cl[MAX_MITER];
  __shared__ double cs[LZ_TILE / CH + 2];
  const int t = blockIdx.x;
  const int g = tgrp[t];
  const GState &s = gs[g];
  if (!s.active) return;
  const int n = s.iters;
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    double v = coef[(ll)g * MI + j];
    float hi = __double2float_rn(v);
    cf[j] = v;
    ch[j] = hi;
    cl[j] = __double2float_rn(__dsub_rn(v, (double)hi));
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const ll b = tbeg[t], e = tend[t];
  const ll c0 = b / CH;
  const int nc = (int)((e - 1) / CH - c0 + 1);
  for (int q = warp; q < nc; q += nw) {
    const ll i0 = (c0 + q) * CH + (ll)lane * R;
    LaneSum<VT> acc;
    VT o[R];
    if (i0 >= b && i0 + R <= e) {
      // whole vector inside the tile: the j loop over 16-byte loads
      if (sizeof(VT) == 4) {
        float sh_[R], sc_[R];
#pragma unroll
        for (int k = 0; k < R; k++) sh_[k] = 0.f, sc_[k] = 0.f;
#pragma unroll 4
        for (int j = 0; j < n; j++) {
          VT x[R];
          Vec::get(*reinterpret_cast<const typename Vec::T *>(V + (ll)j * N + i0), x);
          const float hj = ch[j], lj = cl[j];
#pragma unroll
          for (int k = 0; k < R; k++) {
            float xv = (float)x[k];
            float pr = xv * hj;
            float pe = fmaf(xv, hj, -pr);
            pe = fmaf(xv, lj, pe);
            float t1 = sh_[k] + pr;
            float bp = t1 - sh_[k];
            float er = (sh_[k] - (t1 - bp)) + (pr - bp);
            sh_[k] = t1;
            sc_[k] = sc_[k] + (er + pe);
          }
        }
#pragma unroll
        for (int k = 0; k < R; k++) o[k] = (VT)((double)sh_[k] + (double)sc_[k]);
      } else {
        double a_[R];
#pragma unroll
        for (int k = 0; k < R; k++) a_[k] = 0.0;
#pragma unroll 4
        for (int j = 0; j < n; j++) {
          VT x[R];
          Vec::get(*reinterpret_cast<const typename Vec::T *>(V + (ll)j * N + i0), x);
#pragma unroll
          for (int k = 0; k < R; k++) a_[k] = fma((double)x[k], cf[j], a_[k]);
        }
#pragma unroll
        for (int k = 0; k < R; k++) o[k] = (VT)a_[k];
      }
    } else {
#pragma unroll
      for (int k = 0; k < R; k++) {
        const ll i = i0 + k;
        o[k] = (VT)0;
        if (i < b || i >= e) continue;
        if (sizeof(VT) == 4) {
          float sh1 = 0.f, sc1 = 0.f;
          for (int j = 0; j < n; j++) {
            float xv = (float)V[(ll)j * N + i];
            float pr = xv * ch[j];
            float pe = fmaf(xv, ch[j], -pr);
            pe = fmaf(xv, cl[j], pe);
            float t1 = sh1 + pr;
            float bp = t1 - sh1;
            float er = (sh1 - (t1 - bp)) + (pr - bp);
            sh1 = t1;
            sc1 = sc1 + (er + pe);
          }
          o[k] = (VT)((double)sh1 + (double)sc1);
        } else {
          double a1 = 0.0;
          for (int j = 0; j < n; j++) a1 = fma((double)V[(ll)j * N + i], cf[j], a1);
          o[k] = (VT)a1;
        }
      }
    }
#pragma unroll
    for (int k = 0; k < R; k++) {
      Term<VT> tv;
      tv.set(o[k]);
      if (i0 + k >= b && i0 + k < e) acc.add(tv);
    }
    store_rows(f, i0, b, e, o);
    double v = acc.chunk();
    if (lane == 0) cs[q] = v;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    double v0 = tile_total(cs, nc);
    if (threadIdx.x == 0) part[t] = v0;
  }
}

// ---------------------------------------------------------------------------
// Reorthogonalisation (opt-in, PARRSB_GPU_REORTH=1).  The reference keeps
// the Krylov basis orthogonal only to the constant vector (ortho,
// src/fiedler.c:20-30, 470); in finite precision the residuals r_0 .. r_k
// (rows of V) lose their mutual orthogonality as Ritz values converge.
// Here every new residual is orthogonalised against all earlier ones by
// classical Gram-Schmidt with FP64 coefficients:
//   r_{k+1} <- r_{k+1} - sum_j (r_j . r_{k+1} / |r_j|^2) r_j,
// before its norm enters the recurrence (beta, the stopping test, T).
// k_rdot: tile partials of d_j = r_j . r_{k+1}; each thread keeps its rows
// of r_{k+1} in registers (at most 32: tiles of at most 8192 rows and 256
// threads), sums its products in the vector type and the block adds the
// threads' sums in a fixed order (FP64).
// ---------------------------------------------------------------------------
constexpr int RO_THREADS = 256;
constexpr int RO_ROWS = LZ_TILE / RO_THREADS;  // 32

template <typename VT>
__global__ void __launch_bounds__(RO_THREADS)
k_rdot(const ll *__restrict__ tbeg, const ll *__restrict__ tend, const int *__restrict__ tgrp,
       const GState *__restrict__ gs, const VT *__restrict__ V, ll VS, int it, int MI,
       double *__restrict__ part2) {
  pdl_entry();
  const int t = blockIdx.x;
  const int g = tgrp[t];
  if (!gs[g].run) return;
  const ll b = tbeg[t], e = tend[t];
  const VT *__restrict__ rn = V + (ll)(it + 1) * VS;
  VT x[RO_ROWS];
#pragma unroll
  for (int q = 0; q < RO_ROWS; q++) {
    const ll i = b + threadIdx.x + (ll)q * RO_THREADS;
    x[q] = i < e ? rn[i] : (VT)0;
  }
  __shared__ double sh[RO_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int j = 0; j <= it; j++) {
    const VT *__restrict__ rj = V + (ll)j * VS;
    VT acc = (VT)0;
#pragma unroll
    for (int q = 0; q < RO_ROWS; q++) {
      const ll i = b + threadIdx.x + (ll)q * RO_THREADS;
      if (i < e) acc = acc + x[q] * rj[i];
    }
    double v = warp_tree_sum((double)acc);
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int w = 0; w < RO_THREADS / 32; w++) s = __dadd_rn(s, sh[w]);
      part2[(ll)t * (MI + 1) + j] = s;
    }
    __syncthreads();
  }
}

// One block per group: h_j = (sum over the group's tiles, in order, of d_j)
// / |r_j|^2 (vnorm holds |r_j|).
__global__ void k_rdot_fin(const GState *__restrict__ gs, int ngroups,
                           const double *__restrict__ part2, const double *__restrict__ vnorm,
                           int it, int MI, double *__restrict__ h) {
  pdl_entry();
  const int g = blockIdx.x;
  if (g >= ngroups) return;
  const GState &s = gs[g];
  if (!s.run) return;
  for (int j = threadIdx.x; j <= it; j += blockDim.x) {
    double d = 0.0;
    for (int q = 0; q < s.ntiles; q++) d = __dadd_rn(d, part2[(ll)(s.tile0 + q) * (MI + 1) + j]);
    const double nj = vnorm[(ll)g * (MI + 1) + j];
    h[(ll)g * (MI + 1) + j] = nj > 0.0 ? __ddiv_rn(d, __dmul_rn(nj, nj)) : 0.0;
  }
}

// r_{k+1} -= sum_j h_j r_j, and the tile partial of |r_{k+1}|^2 (for the
// recurrence's finalisation, in place of the plain update's).
template <typename VT>
__global__ void __launch_bounds__(RO_THREADS)
k_rupd(const ll *__restrict__ tbeg, const ll *__restrict__ tend, const int *__restrict__ tgrp,
       const GState *__restrict__ gs, VT *__restrict__ V, ll VS, int it, int MI,
       const double *__restrict__ h, double *__restrict__ part) {
  pdl_entry();
  const int t = blockIdx.x;
  const int g = tgrp[t];
  if (!gs[g].run) return;
  __shared__ VT hs[MAX_MITER + 1];
  for (int j = threadIdx.x; j <= it; j += blockDim.x) hs[j] = (VT)h[(ll)g * (MI + 1) + j];
  __syncthreads();
  const ll b = tbeg[t], e = tend[t];
  VT *__restrict__ rn = V + (ll)(it + 1) * VS;
  double acc = 0.0;
  for (ll i = b + threadIdx.x; i < e; i += RO_THREADS) {
    VT v = rn[i];
    for (int j = 0; j <= it; j++) v = v - hs[j] * V[(ll)j * VS + i];
    rn[i] = v;
    acc += (double)(v * v);
  }
  __shared__ double sh[RO_THREADS / 32];
  const double w = warp_tree_sum(acc);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = w;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int q = 0; q < RO_THREADS / 32; q++) s = __dadd_rn(s, sh[q]);
    part[t] = s;
  }
}

// Tridiagonal eigensolve for the Ritz vector, one warp per group.
// GB300 runs long dependent FP64 chains slowly, so instead of the implicit
// QL sweep of the reference (tqli, src/fiedler.c:328-432, about 2000
// dependent rotations with divisions and square roots for n = 50):
//   1. the eigenvalue of least modulus (the one lanczos picks,
//      src/fiedler.c:538-545) by warp multisection: 32 lanes evaluate a
//      division-free Sturm count at 32 shifts per round, the bracket
//      shrinks 33x per round;
//   2. its eigenvector by inverse iteration on T (LU with partial
//      pivoting, two solves, Newton reciprocals), normalised.
// The vector's sign is fixed later, on the final Fiedler vector (canonical
// orientation).  Writes coef[j] = y_j / |r_j|.

// number of eigenvalues of T below x (Sturm sequence of the leading
// principal minors).  Only the two multiplies and the subtraction of each
// step use the FP64 pipe (GB300 runs FP64 at 1/64 of the FP32 rate): signs,
// zero tests and the range check read the bit pattern with integer
// instructions, and the rescaling multiplies by exact powers of two.
__device__ __forceinline__ int sturm_count(const double *d, const double *e2, int n, double x) {
  const double TINY = 1e-300;
  double pm = 1.0, p = __dsub_rn(d[0], x);
  long long pb = __double_as_longlong(p);
  if ((pb << 1) == 0) p = -TINY, pb = __double_as_longlong(p);
  int cnt = pb < 0;
  for (int i = 1; i < n; i++) {
    double pn = fma(__dsub_rn(d[i], x), p, -__dmul_rn(e2[i - 1], pm));
    long long nb = __double_as_longlong(pn);
    if ((nb << 1) == 0) {  // exact zero: sign opposite to p
      pn = pb < 0 ? TINY : -TINY;
      nb = __double_as_longlong(pn);
    }
    cnt += (nb ^ pb) < 0;
    pm = p;
    p = pn;
    pb = nb;
    const int ex = (int)((nb >> 52) & 0x7FF);
    if (ex > 1023 + 600) {
      p = __dmul_rn(p, 0x1p-600), pm = __dmul_rn(pm, 0x1p-600);
      pb = __double_as_longlong(p);
    } else if (ex < 1023 - 600) {
      p = __dmul_rn(p, 0x1p600), pm = __dmul_rn(pm, 0x1p600);
      pb = __double_as_longlong(p);
    }
  }
  return cnt;
}

// y / x with a single-precision reciprocal refined by two Newton steps
__device__ __forceinline__ double fast_div(double y, double x) {
  double ax = fabs(x);
  double r;
  if (ax > 1e-30 && ax < 1e30) {
    r = (double)__frcp_rn((float)x);
    r = fma(r, fma(-x, r, 1.0), r);
    r = fma(r, fma(-x, r, 1.0), r);
  } else {
    r = __ddiv_rn(1.0, x);
  }
  double q = __dmul_rn(y, r);
  return fma(r, fma(-x, q, y), q);  // one correction of the quotient
}

__device__ void tri_solve_pivot(int n, const double *a0, const double *e, double lam,
                                double *x, double *a, double *b, double *c, double *c2,
                                int *piv, double tiny) {
  // factor (T - lam I) = P L U with U having two super-diagonals (dgttrf)
  for (int i = 0; i < n; i++) a[i] = __dsub_rn(a0[i], lam);
  for (int i = 0; i < n - 1; i++) b[i] = e[i], c[i] = e[i], c2[i] = 0.0;
  for (int i = 0; i < n - 1; i++) {
    if (fabs(a[i]) >= fabs(b[i])) {
      piv[i] = 0;
      if (a[i] == 0.0) a[i] = tiny;
      double fact = fast_div(b[i], a[i]);
      b[i] = fact;
      a[i + 1] = fma(-fact, c[i], a[i + 1]);
      c2[i] = 0.0;
    } else {
      piv[i] = 1;
      double fact = fast_div(a[i], b[i]);
      a[i] = b[i];
      b[i] = fact;
      double t = c[i];
      c[i] = a[i + 1];
      a[i + 1] = fma(-fact, a[i + 1], t);
      if (i < n - 2) {
        c2[i] = c[i + 1];
        c[i + 1] = __dmul_rn(-fact, c[i + 1]);
      } else {
        c2[i] = 0.0;
      }
    }
  }
  if (n > 0 && a[n - 1] == 0.0) a[n - 1] = tiny;
  for (int i = 0; i < n - 1; i++) {  // L with row interchanges
    if (piv[i]) {
      double t = x[i];
      x[i] = x[i + 1];
      x[i + 1] = fma(-b[i], x[i], t);
    } else {
      x[i + 1] = fma(-b[i], x[i], x[i + 1]);
    }
  }
  for (int i = n - 1; i >= 0; i--) {  // U
    double v = x[i];
    if (i + 1 < n) v = fma(-c[i], x[i + 1], v);
    if (i + 2 < n) v = fma(-c2[i], x[i + 2], v);
    x[i] = fast_div(v, a[i]);
  }
}

__device__ __forceinline__ double warp_min_d(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}
__device__ __forceinline__ double warp_max_d(double v) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
  return v;
}

// k-th smallest eigenvalue (0-based) by multisection inside [lo, hi], to a
// bracket of relative width rel
__device__ double eig_index(const double *d, const double *e2, int n, int k, double lo,
                            double hi, double rel = 2.2e-16) {
  const int lane = threadIdx.x;
  double a = lo, b = hi;
  for (int round = 0; round < 24; round++) {
    double w = __dsub_rn(b, a);
    if (!(w > rel * fmax(fabs(a), fabs(b)) + 1e-300)) break;
    double x = fma(w, (double)(lane + 1) / 33.0, a);
    int cnt = sturm_count(d, e2, n, x);
    unsigned ball = __ballot_sync(0xffffffffu, cnt > k);
    int first = ball ? __ffs(ball) - 1 : 32;
    double xl = __shfl_sync(0xffffffffu, x, first > 0 ? first - 1 : 0);
    double xr = __shfl_sync(0xffffffffu, x, first < 32 ? first : 31);
    double na = first > 0 ? xl : a;
    double nb = first < 32 ? xr : b;
    if (!(nb < b || na > a)) break;  // no progress at this precision
    a = na, b = nb;
  }
  return 0.5 * (a + b);
}

__global__ void k_tri_eig(GState *__restrict__ gs, int ngroups,
                          const double *__restrict__ diagT, const double *__restrict__ upperT,
                          const double *__restrict__ vnorm, int MI, double *__restrict__ coef) {
  pdl_entry();
  extern __shared__ double eig_sm[];
  const int g = blockIdx.x, lane = threadIdx.x;
  if (g >= ngroups) return;
  GState &st = gs[g];
  if (!st.active) return;
  const int n = st.iters;
  double *D0 = eig_sm, *E0 = D0 + MI, *e2 = E0 + MI;
  double *a = e2 + MI, *b = a + MI, *c = b + MI, *c2 = c + MI, *x = c2 + MI;
  int *piv = (int *)(x + MI);
  for (int i = lane; i < n; i += 32) {
    D0[i] = diagT[(ll)g * MI + i];
    if (i < n - 1) {
      double ev = upperT[(ll)g * MI + i];
      E0[i] = ev;
      e2[i] = __dmul_rn(ev, ev);
    }
  }
  __syncwarp();
  // Gershgorin interval
  double glo = 1e300, ghi = -1e300;
  for (int i = lane; i < n; i += 32) {
    double r = (i > 0 ? fabs(E0[i - 1]) : 0.0) + (i < n - 1 ? fabs(E0[i]) : 0.0);
    glo = fmin(glo, __dsub_rn(D0[i], r));
    ghi = fmax(ghi, __dadd_rn(D0[i], r));
  }
  glo = warp_min_d(glo);
  ghi = warp_max_d(ghi);
  double pad = fmax(1e-300, 2.2e-16 * fmax(fabs(glo), fabs(ghi))) * 4.0;
  glo -= pad, ghi += pad;
  // eigenvalue of least modulus: the negative one closest to 0 or the
  // smallest non-negative one
  int c0 = sturm_count(D0, e2, n, 0.0);  // eigenvalues below 0 (all lanes agree)
  double lam;
  if (c0 == 0) {
    lam = eig_index(D0, e2, n, 0, glo, ghi);
  } else if (c0 >= n) {
    lam = eig_index(D0, e2, n, n - 1, glo, ghi);
  } else {
    double ln = eig_index(D0, e2, n, c0 - 1, glo, ghi);
    double lp = eig_index(D0, e2, n, c0, glo, ghi);
    lam = fabs(lp) < fabs(ln) ? lp : ln;
  }
  if (lane == 0) {
    double tnorm = fmax(fabs(glo), fabs(ghi));
    double tiny = fmax(tnorm, 1e-300) * 1e-16;
    for (int i = 0; i < n; i++) x[i] = 1.0;
    for (int sweep = 0; sweep < 2; sweep++) {
      tri_solve_pivot(n, D0, E0, lam, x, a, b, c, c2, piv, tiny);
      double nrm = 0.0;
      for (int i = 0; i < n; i++) nrm = fma(x[i], x[i], nrm);
      double inv = nrm > 0.0 ? fast_div(1.0, __dsqrt_rn(nrm)) : 0.0;
      for (int i = 0; i < n; i++) x[i] = __dmul_rn(x[i], inv);
    }
  }
  __syncwarp();
  for (int j = lane; j < n; j += 32)
    coef[(ll)g * MI + j] = fast_div(x[j], vnorm[(ll)g * (MI + 1) + j]);
}

// Residual of the current Ritz pair of a running group after step it: with
// T_k (k = it + 1) the tridiagonal matrix of the pass so far, theta its
// smallest eigenvalue and y the normalised eigenvector, the Lanczos relation
// L V_k = V_k T_k + b_k v_(k+1) e_k^T gives |L V_k y - theta V_k y| = |b_k y_k|
// for an orthonormal basis, b_k = upperT[it] being the off-diagonal that
// step it + 1 enters (FIN_RTR of step it writes it).  theta by multisection
// to a relative 1e-10; y_k from the bottom twist of T_k - theta I: the
// pivots d_i of its LDL^T factorisation (positive below the last for the
// smallest eigenvalue) and z_(k-1) = 1, z_i = -e_i z_(i+1) / d_i,
// y_k = 1 / |z|.  Writes the bound to bound_out[g MI + it] (when given) and,
// when it is below stop_below, asks to end the group's pass (stopreq).
// It runs on a second stream beside the next steps: it reads only entries
// of T that step it completed (each written with the same value wherever it
// is written), whether the group ran step it, and its own fields of the
// group state, so its answer does not depend on how far the other stream
// has got; k_apply_stop turns the request into run = 0 at a fixed step after
// joining the streams.  To spend little of the FP64 pipe, a group whose
// last bound was above 30 stop_below is computed again only `span` steps
// after it, and the multisection starts from [0.99 theta', theta'], theta'
// the last check's Ritz value (the smallest Ritz value never grows with the
// steps of a pass; both ends are checked by Sturm counts, else Gershgorin's
// interval).  One warp per group; a group whose T_k has an eigenvalue below
// 0 is left alone.
__global__ void k_ritz_bound(GState *__restrict__ gs, int ngroups,
                             const double *__restrict__ diagT, const double *__restrict__ upperT,
                             int MI, int it, double stop_below, int span,
                             double *__restrict__ bound_out) {
  pdl_entry();
  extern __shared__ double rb_sm[];
  const int g = blockIdx.x, lane = threadIdx.x;
  if (g >= ngroups) return;
  GState &st = gs[g];
  if (!st.active || *(volatile const int *)&st.iters < it + 1) return;  // step it not run
  if (!bound_out && st.rb_it >= 0 && st.rb_bound > 30.0 * stop_below && it - st.rb_it < span)
    return;  // far from stopping: not yet
  const int n = it + 1;
  double *D0 = rb_sm, *E0 = D0 + MI, *e2 = E0 + MI;
  for (int i = lane; i < n; i += 32) {
    D0[i] = diagT[(ll)g * MI + i];
    if (i < n - 1) {
      const double ev = upperT[(ll)g * MI + i];
      E0[i] = ev;
      e2[i] = __dmul_rn(ev, ev);
    }
  }
  __syncwarp();
  double glo = 1e300, ghi = -1e300;
  for (int i = lane; i < n; i += 32) {
    const double r = (i > 0 ? fabs(E0[i - 1]) : 0.0) + (i < n - 1 ? fabs(E0[i]) : 0.0);
    glo = fmin(glo, __dsub_rn(D0[i], r));
    ghi = fmax(ghi, __dadd_rn(D0[i], r));
  }
  glo = warp_min_d(glo);
  ghi = warp_max_d(ghi);
  const double pad = fmax(1e-300, 2.2e-16 * fmax(fabs(glo), fabs(ghi))) * 4.0;
  glo -= pad, ghi += pad;
  // lane 0: eigenvalues below 0; lanes 1, 2: the warm bracket's ends
  const double th0 = st.rb_theta;
  const double xq = lane == 1 ? 0.99 * th0 : th0;
  const int cq = (lane == 0 || (th0 > 0.0 && lane < 3)) ? sturm_count(D0, e2, n, lane ? xq : 0.0)
                                                          : 0;
  const int c0 = __shfl_sync(0xffffffffu, cq, 0), clo = __shfl_sync(0xffffffffu, cq, 1),
            chi = __shfl_sync(0xffffffffu, cq, 2);
  const bool pd = c0 == 0;
  const bool warm = th0 > 0.0 && clo == 0 && chi >= 1;
  const double theta =
      pd ? (warm ? eig_index(D0, e2, n, 0, 0.99 * th0, th0, 1e-10)
                 : eig_index(D0, e2, n, 0, glo, ghi, 1e-10))
         : 0.0;
  if (lane != 0) return;
  double bound = 1e300;
  if (pd) {
    // pivots of T_k - theta I, then z from the bottom (scaled to stay finite)
    double *dv = e2 + MI;
    double d = __dsub_rn(D0[0], theta);
    dv[0] = d;
    for (int i = 1; i < n; i++) {
      d = __dsub_rn(__dsub_rn(D0[i], theta), fast_div(e2[i - 1], d));
      dv[i] = d;
    }
    double z = 1.0, zl = 1.0, ss = 1.0;  // current z_i, z_(k-1), sum of squares
    for (int i = n - 2; i >= 0; i--) {
      z = fast_div(__dmul_rn(-E0[i], z), dv[i]);
      if (!(fabs(z) < 1e150)) {
        if (!isfinite(z)) {  // a zero pivot: the pair is exact to working precision
          zl = 0.0;
          ss = 1.0;
          break;
        }
        z = __dmul_rn(z, 1e-150), zl = __dmul_rn(zl, 1e-150), ss = __dmul_rn(ss, 1e-300);
      }
      ss = fma(z, z, ss);
    }
    const double yk = fast_div(fabs(zl), __dsqrt_rn(ss));
    bound = __dmul_rn(fabs(upperT[(ll)g * MI + it]), yk);
  }
  if (bound_out) bound_out[(ll)g * MI + it] = bound;
  st.rb_it = it;
  st.rb_theta = pd ? theta : 0.0;
  st.rb_bound = bound;
  if (bound < stop_below) st.stopreq = 1;
}

// the stop requests of the last Ritz residual check take effect
__global__ void k_apply_stop(GState *__restrict__ gs, int ngroups) {
  pdl_entry();
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngroups) return;
  GState &st = gs[g];
  if (st.stopreq) {
    st.run = 0;
    st.stopreq = 0;
  }
}

__global__ void k_set_active(GState *__restrict__ gs, int ngroups) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < ngroups) {
    gs[g].active = 1;
    gs[g].npass = 0;
    gs[g].total_iters = 0;
    gs[g].run = 0;
    gs[g].stall = 0;
    gs[g].prev_resid = 1e300;
  }
}

__global__ void k_set_warm(GState *__restrict__ gs, int ngroups, const int *__restrict__ use) {
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g < ngroups) gs[g].warm = use[g];
}

// Restarts driven on the device (a conditional while node of the pass
// graph): the body zeroes the pass flags, runs one restart of every active
// group and then k_loop_next folds the pass into the counters and sets the
// condition: another restart only while a group is still active and fewer
// than mpass restarts have run (so the loop always ends).
__global__ void k_loop_zero(int *__restrict__ any) {
  any[0] = 0;
  any[1] = 0;
}

__global__ void k_loop_next(cudaGraphConditionalHandle h, const int *__restrict__ any,
                            long long *__restrict__ ctr, int mpass) {
  const long long np = ctr[0] + 1;
  ctr[0] = np;
  ctr[1] += any[1];  // steps of the longest group this restart
  cudaGraphSetConditional(h, (any[0] != 0 && np < mpass) ? 1u : 0u);
}

// ----------------------------------------------------------------------------
// Host-side segmented Lanczos engine
// ----------------------------------------------------------------------------
template <typename VT>
struct Lanczos {
  int A = 0;      // groups
  int T = 0;      // tiles
  int MI = 0;
  ll N = 0;
  DBuf<GState> gs;
  DBuf<ll> tbeg, tend;
  DBuf<int> tgrp;
  DBuf<VT> f, p, w, V;  // Fiedler iterate, CG direction, L p, Krylov basis
  DBuf<double> part, diagT, upperT, vnorm, coef, y64;
  DBuf<int> any;  // [0] any group active for another pass, [1] max steps
  DBuf<int> cnt;  // per-group arrival counters of the fused finalisation
  std::vector<GState> hgs;
  std::vector<cudaEvent_t> ev;  // SpMV start/stop events (timing mode)
  std::vector<cudaEvent_t> evk; // p / r per step, then init, eig, ritz (timing mode)
  int bd = 256;                  // threads per tile block (autotuned per level)
  int sp_kind = 0;               // SpMV variant (autotuned): 0 k_spmv, 1 k_spmv_tma
  DBuf<int> err;                 // [0]: a staged-SpMV wait gave up
  int pr_bd = 256;               // threads per block of k_pr
  int pr_u = 4;                  // chunks per warp in flight in k_pr
  // The vector updates write tile partials and a separate one-block-per-group
  // launch finalises (measured faster than finalising in the last tile block
  // of each group, which every block pays for with a fence, an atomic and
  // barriers); PARRSB_GPU_PR_FUSED=1 selects the fused form (same bits).
  bool pr_fused = false;
  // the same choice for the SpMV (PARRSB_GPU_SPMV_FUSED=1: fused)
  bool sp_fused = false;
  int ritz_bd = 256;             // threads per block of k_ritz
  DBuf<long long> loop_ctr;      // device restart loop: passes, SpMV steps
  bool reorth = false;           // reorthogonalise every residual (opt-in)
  DBuf<double> part2, hro;       //   its tile partials and coefficients
  // persistent step kernel (k_steps): with PARRSB_GPU_PERSIST=1, unless per-
  // kernel timing, reorthogonalisation or a fused finalisation is asked for,
  // and when the level's tiles fit its resident grid
  bool persist = false;
  int ps_grid = 0;               //   its blocks
  DBuf<unsigned> ps_bar;         //   barrier arrivals
  DBuf<int> ps_run;              //   groups still running after each step
  DBuf<ll> fq;                   // fixed-point f of the residual check (FP32)
  DBuf<unsigned> gmax, tmax;     //   each group's and tile's largest |f| (IEEE bits)
  bool resid_stop = false;       // restarts decided by the FP64 eigen-residual
  // early pass exit (residual-stop mode): after step it with it + 1 =
  // early_min + j early_stride, a group whose Ritz residual bound is below
  // early * rsb_tol ends its pass before step it + early_delay
  // (k_ritz_bound, k_apply_stop; 1 <= early_delay <= early_stride); 0: off
  double early = 0.0;
  int early_min = 3, early_stride = 3, early_delay = 3;
  bool bound_log = false;        // PARRSB_GPU_PASS_LOG=2: the bound after every step
  DBuf<double> bnd;              //   [A][MI]
  cudaStream_t side = nullptr;   // the bound checks' stream, forked from and joined to
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;  //   the pass's stream
  int side_prio = 0;             //   its priority (the device's highest)

  Lanczos() = default;
  Lanczos(const Lanczos &) = delete;
  Lanczos &operator=(const Lanczos &) = delete;
  ~Lanczos() {
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_join) cudaEventDestroy(ev_join);
    if (side) cudaStreamDestroy(side);
  }
  double resid_tol = 0.0;        // its bound (rsb_tol); passes then use
  double cg_factor = 1.0;        //   tol * cg_factor for their own CG exit
  ll VS = 0;                     // row stride of V (N rounded up to 64: 16-byte rows)

  void setup(const std::vector<ll> &gstart, const std::vector<ll> &gn, ll N_, int miter) {
    N = N_;
    A = (int)gstart.size();
    MI = miter;
    std::vector<ll> hb, he;
    std::vector<int> hg;
    hgs.assign(A, GState());
    for (int g = 0; g < A; g++) {
      GState &s = hgs[g];
      memset(&s, 0, sizeof(s));
      s.start = gstart[g];
      s.n = gn[g];
      s.miter = (int)std::min<ll>(miter, gn[g]);
      s.tile0 = (int)hb.size();
      // tile rows depend only on the group's size (never on the other groups
      // of the level), so batched and one-group-at-a-time runs agree bitwise
      const ll tr = tile_rows(gn[g]);
      for (ll b = gstart[g]; b < gstart[g] + gn[g]; b += tr) {
        hb.push_back(b);
        he.push_back(std::min(b + tr, gstart[g] + gn[g]));
        hg.push_back(g);
      }
      s.ntiles = (int)hb.size() - s.tile0;
    }
    T = (int)hb.size();
    ll max_tile = 0;
    for (int g = 0; g < A; g++) max_tile = std::max(max_tile, std::min(tile_rows(gn[g]), gn[g]));
    pr_u = N >= PR_BIG ? 4 : 1;
    {
      const char *v = getenv("PARRSB_GPU_PR_FUSED");
      pr_fused = v && atoi(v) != 0;
      const char *v2 = getenv("PARRSB_GPU_SPMV_FUSED");
      sp_fused = v2 && atoi(v2) != 0;
    }
    // FP32: four warps per block (fewer tiles per SM wait on one block's
    // reduction tail; measured fastest on 8M-row levels); the chunk order of
    // the reduction does not depend on the block size
    pr_bd = sizeof(VT) == 4 ? std::min(vec_threads<VT>(max_tile, pr_u), 128)
                            : vec_threads<VT>(max_tile, pr_u);
    if (const char *v = getenv("PARRSB_GPU_PR_THREADS"))  // 32..512, a multiple of 32
      pr_bd = std::max(32, std::min(512, atoi(v) / 32 * 32));
    ritz_bd = vec_threads<VT>(max_tile, 1);
    VS = (N + 63) & ~(ll)63;
    gs.ensure(A);
    tbeg.ensure(T), tend.ensure(T), tgrp.ensure(T);
    h2d(gs.p, hgs.data(), A);
    h2d(tbeg.p, hb.data(), T);
    h2d(tend.p, he.data(), T);
    h2d(tgrp.p, hg.data(), T);
    f.ensure(N), p.ensure(N), w.ensure(N);
    V.ensure((size_t)(MI + 1) * VS);
    part.ensure((size_t)3 * T + 2);
    diagT.ensure((size_t)A * MI), upperT.ensure((size_t)A * MI);
    vnorm.ensure((size_t)A * (MI + 1)), coef.ensure((size_t)A * MI);
    any.ensure(2);
    err.ensure(1);
    CK(cudaMemsetAsync(err.p, 0, sizeof(int), ctx().stream));
    cnt.ensure(A);
    CK(cudaMemsetAsync(cnt.p, 0, (size_t)A * sizeof(int), ctx().stream));

  }

  // a Ritz residual bound after step it (k_ritz_bound); with early exit its
  // stop requests apply before step it + early_delay (k_apply_stop)
  bool bound_at(int it) const {
    if (bound_log) return true;
    return early > 0.0 && it + 1 >= early_min && (it + 1 - early_min) % early_stride == 0 &&
           it + early_delay < MI;
  }
  int bound_launches() const {
    int c = 0;
    for (int it = 0; it < MI; it++) c += bound_at(it) ? 1 : 0;
    return c * (early > 0.0 ? 2 : 1);
  }

  // shared memory of k_tri_eig: 8 arrays of MI doubles and MI ints
  size_t eig_smem() const {
    return (size_t)8 * MI * sizeof(double) + (size_t)(MI + 2) * sizeof(int) + 16;
  }

  FinArgs fargs(int it, double tol, int mpass) {
    FinArgs fa;
    fa.cnt = cnt.p;
    fa.it = it;
    fa.MI = MI;
    fa.mpass = mpass;
    fa.tol = tol;
    fa.diagT = diagT.p;
    fa.upperT = upperT.p;
    fa.vnorm = vnorm.p;
    fa.any = any.p;
    return fa;
  }

  // y_in / v_in replace the y64 and V arguments (TM_LOAD_Y, TM_SELECT)
  template <int MODE, int GATE, int FUSE = -1>
  void tile(int it = 0, const Level *lv = nullptr, double tol = 0.0, int mpass = 0,
            const double *y_in = nullptr, VT *v_in = nullptr) {
    launch_pdl(k_tile<VT, MODE, GATE, FUSE>, T, bd, 0, ctx().stream, tbeg.p, tend.p, tgrp.p,
               gs.p, f.p, v_in ? v_in : V.p, N, it, part.p, lv ? lv->ell.p : nullptr,
               lv ? lv->slice_off.p : nullptr, lv ? lv->slice_w.p : nullptr,
               y_in ? const_cast<double *>(y_in) : y64.p, fargs(it, tol, mpass));
  }
  template <int OP, int GATE>
  void fin(int it = 0, double tol = 0.0, int mpass = 0) {
    launch_pdl(k_fin<OP, GATE>, A, LZ_THREADS, 0, ctx().stream, gs.p, A, part.p, it, MI, tol,
               mpass, diagT.p, upperT.p, vnorm.p, any.p);
  }

  void initial_vector() {
    tile<TM_IV_SUM, GATE_ALL>();
    fin<FIN_IV_MEAN, GATE_ALL>();
    tile<TM_IV_SQ, GATE_ALL>();
    fin<FIN_IV_NORM, GATE_ALL>();
    tile<TM_IV_WRITE, GATE_ALL>();
  }

  // Seeded random start (uniform in [-1, 1) per position of a group); the
  // first pass removes its mean and normalises it.
  void random_vector() { tile<TM_RANDOM, GATE_ALL>(); }

  // Start vectors with a predicted candidate y (FP64 per position): every
  // group starts from y or from the fallback start (start_kind 1: random,
  // otherwise the reference's step vector), whichever has the lower FP64
  // eigen-residual ||L f - rho f|| / ||f|| (the judge).  Leaves the start
  // in f.
  void choose_start(const Level &lv, const double *y, int start_kind) {
    cudaStream_t st = ctx().stream;
    k_set_active<<<grid_for(A, 128), 128, 0, st>>>(gs.p, A);
    CK_LAUNCH();
    if (start_kind == 1) random_vector(); else initial_vector();
    residual(lv);
    download(hgs);
    std::vector<double> r_fb(A);
    for (int g = 0; g < A; g++) r_fb[g] = hgs[g].resid;
    CK(cudaMemcpyAsync(p.p, f.p, (size_t)N * sizeof(VT), cudaMemcpyDeviceToDevice, st));
    tile<TM_LOAD_Y, GATE_ALL>(0, nullptr, 0.0, 0, y);
    tile<TM_SUM_F, GATE_ALL>();
    fin<FIN_RITZ_MEAN, GATE_ALL>();
    tile<TM_SUB_C, GATE_ALL>();
    residual(lv);
    download(hgs);
    parrsb_stats &S = ctx().stats;
    double lf = 0.0, lw = 0.0;
    long long tried = 0;
    std::vector<int> use(A, 0);
    for (int g = 0; g < A; g++) {
      const double rw = hgs[g].resid;
      tried++;
      lf += log10(std::max(r_fb[g], 1e-300));
      lw += log10(std::max(rw, 1e-300));
      // (a group with two axes of nearly the same length has its guess
      // along RCB's cut axis, the axis of the fallback's step)
      use[g] = rw < r_fb[g] ? 1 : 0;  // NaN never wins
      S.warm_used += use[g];
    }
    // running geometric means over every judged group of the call
    const long long t0 = S.warm_tried;
    if (tried > 0) {
      const double pf = t0 ? log10(S.start_resid_fallback) * t0 : 0.0;
      const double pw = t0 ? log10(S.start_resid_warm) * t0 : 0.0;
      S.start_resid_fallback = pow(10.0, (pf + lf) / (double)(t0 + tried));
      S.start_resid_warm = pow(10.0, (pw + lw) / (double)(t0 + tried));
      S.warm_tried = t0 + tried;
    }
    DBuf<int> du(A);
    h2d(du.p, use.data(), A);
    k_set_warm<<<grid_for(A, 128), 128, 0, st>>>(gs.p, A, du.p);
    CK_LAUNCH();
    tile<TM_SELECT, GATE_ALL>(0, nullptr, 0.0, 0, nullptr, p.p);
    sync();
  }

  // One Lanczos pass (restart) for the active groups: the body that the
  // CUDA graph captures.
  // event record inside a pass: an external event node while the pass is
  // captured, a plain record when it runs without a graph
  void record(cudaEvent_t e) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CK(cudaStreamIsCapturing(ctx().stream, &cs));
    CK(cudaEventRecordWithFlags(
        e, ctx().stream,
        cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault));
  }
  void mark(int k) {
    if (!evk.empty()) record(evk[k]);
  }
  // evk layout: [4 it .. 4 it + 3] p start/stop, r start/stop of step it;
  // then 4 MI + 0..5: init start/stop, eig start/stop, ritz start/stop
  void pass_body(const Level &lv, double tol, int mpass, long long *spmv_launches) {
    cudaStream_t st = ctx().stream;
    bool forked = false;  // bound checks on the side stream (joined at the end)
    mark(4 * MI + 0);
    tile<TM_SUM_F, GATE_ACTIVE>();
    fin<FIN_INIT_MEAN, GATE_ACTIVE>();
    tile<TM_INIT_R, GATE_ACTIVE>();
    fin<FIN_INIT_RTR, GATE_ACTIVE>(0, tol);
    mark(4 * MI + 1);
    if (persist) {
      steps_persistent(lv, tol);
      *spmv_launches += MI;
    }
    int pending = -1;  // step of the bound check whose stop requests are due
    for (int it = 0; it < (persist ? 0 : MI); it++) {
      if (pending >= 0 && it == pending + early_delay) {  // join, then apply the requests
        CK(cudaEventRecord(ev_join, side));
        CK(cudaStreamWaitEvent(st, ev_join, 0));
        k_apply_stop<<<grid_for(A, 128), 128, 0, st>>>(gs.p, A);
        CK_LAUNCH();
        ctx().kernel_launches++;
        pending = -1;
      }
      // three launches per step: each finalises its group scalars in the
      // last tile block of the group
      mark(4 * it + 0);
      if (pr_fused) {
        launch_pdl(pr_u == 4 ? k_pr<VT, TM_P, 4> : k_pr<VT, TM_P, 1>, T, pr_bd, 0, st, tbeg.p,
                   tend.p, tgrp.p, gs.p, p.p, w.p, V.p, VS, part.p, fargs(it, tol, mpass));
      } else {  // tile partials, then one block per group
        launch_pdl(pr_u == 4 ? k_pr<VT, TM_P, 4, false> : k_pr<VT, TM_P, 1, false>, T, pr_bd, 0,
                   st, tbeg.p, tend.p, tgrp.p, gs.p, p.p, w.p, V.p, VS, part.p,
                   fargs(it, tol, mpass));
        fin<FIN_PMEAN, GATE_RUN>(it, tol, mpass);
      }
      mark(4 * it + 1);
      if (!ev.empty()) record(ev[2 * it]);
      spmv(lv, sp_kind, bd, fargs(it, tol, mpass), sp_fused ? 1 : 0, 0);
      if (!sp_fused) fin<FIN_PAP, GATE_RUN>(it, tol, mpass);
      if (!ev.empty()) record(ev[2 * it + 1]);
      (*spmv_launches)++;
      mark(4 * it + 2);
      if (pr_fused && !reorth) {
        launch_pdl(pr_u == 4 ? k_pr<VT, TM_R, 4> : k_pr<VT, TM_R, 1>, T, pr_bd, 0, st, tbeg.p,
                   tend.p, tgrp.p, gs.p, p.p, w.p, V.p, VS, part.p, fargs(it, tol, mpass));
      } else {
        launch_pdl(pr_u == 4 ? k_pr<VT, TM_R, 4, false> : k_pr<VT, TM_R, 1, false>, T, pr_bd, 0,
                   st, tbeg.p, tend.p, tgrp.p, gs.p, p.p, w.p, V.p, VS, part.p,
                   fargs(it, tol, mpass));
        if (reorth) {  // against r_0 .. r_it; rewrites the partials of |r_{it+1}|^2
          launch_pdl(k_rdot<VT>, T, RO_THREADS, 0, st, tbeg.p, tend.p, tgrp.p, gs.p, V.p, VS, it,
                     MI, part2.p);
          launch_pdl(k_rdot_fin, A, 64, 0, st, gs.p, A, part2.p, vnorm.p, it, MI, hro.p);
          launch_pdl(k_rupd<VT>, T, RO_THREADS, 0, st, tbeg.p, tend.p, tgrp.p, gs.p, V.p, VS, it,
                     MI, hro.p, part.p);
        }
        fin<FIN_RTR, GATE_RUN>(it, tol, mpass);
      }
      if (bound_at(it)) {  // on the side stream, beside the next steps
        CK(cudaEventRecord(ev_fork, st));
        CK(cudaStreamWaitEvent(side, ev_fork, 0));
        // (at the highest priority: its blocks take the first free slots
        // while the step kernels fill the GPU)
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)A);
        cfg.blockDim = dim3(32);
        cfg.dynamicSmemBytes = (size_t)4 * MI * sizeof(double);
        cfg.stream = side;
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributePriority;
        attr.val.priority = side_prio;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        CK(cudaLaunchKernelEx(&cfg, k_ritz_bound, gs.p, A, (const double *)diagT.p,
                              (const double *)upperT.p, MI, it, early * resid_tol,
                              3 * early_stride, bound_log ? bnd.p : nullptr));
        ctx().kernel_launches++;
        forked = true;
        if (early > 0.0) pending = it;
      }
      mark(4 * it + 3);
    }
    mark(4 * MI + 2);
    launch_pdl(k_tri_eig, A, 32, eig_smem(), st, gs.p, A, diagT.p, upperT.p, vnorm.p, MI, coef.p);
    mark(4 * MI + 3);
    mark(4 * MI + 4);
    launch_pdl(k_ritz<VT>, T, ritz_bd, 0, st, tbeg.p, tend.p, tgrp.p, gs.p, V.p, VS, coef.p, MI,
               f.p, part.p);
    mark(4 * MI + 5);
    fin<FIN_RITZ_MEAN, GATE_ACTIVE>();
    tile<TM_SUB_C, GATE_ACTIVE>();
    if (!resid_stop) {
      fin<FIN_PASS_END, GATE_ACTIVE>(0, tol, mpass);
    } else {
      // restart until the Ritz vector's FP64 eigen-residual is at most tol
      fin<FIN_PASS_END_R, GATE_ACTIVE>(0, tol, mpass);
      resid1<GATE_ACTIVE>(lv);
      fin<FIN_RESID1, GATE_ACTIVE>();
      resid2<GATE_ACTIVE>(lv);
      fin<FIN_RESID_GATE, GATE_ACTIVE>(0, resid_tol, mpass);
    }
    if (forked) {  // every bound check ends before the pass does
      CK(cudaEventRecord(ev_join, side));
      CK(cudaStreamWaitEvent(st, ev_join, 0));
    }
  }

  // kernels of the steps of one pass
  long long step_kernels() const {
    if (persist) return 2;
    return (long long)MI * ((pr_fused && !reorth) ? 3 : 5) + (sp_fused ? 0 : MI) +
           (reorth ? 3ll * MI : 0) + bound_launches();
  }

  // all steps of the pass in one cooperative launch (k_steps)
  void steps_persistent(const Level &lv, double tol) {
    cudaStream_t st = ctx().stream;
    // (a kernel, not memset nodes, in front of the cooperative launch)
    k_ps_reset<<<1, 128, 0, st>>>(ps_bar.p, ps_run.p, MI);
    CK_LAUNCH();
    StepArgs sa;
    sa.tbeg = tbeg.p, sa.tend = tend.p, sa.tgrp = tgrp.p, sa.gs = gs.p;
    sa.p = p.p, sa.w = w.p, sa.V = V.p, sa.VS = VS;
    sa.ell = lv.ell.p, sa.slice_off = lv.slice_off.p, sa.slice_w = lv.slice_w.p;
    sa.part = part.p;
    sa.diagT = diagT.p, sa.upperT = upperT.p, sa.vnorm = vnorm.p;
    sa.bar = ps_bar.p, sa.run_cnt = ps_run.p, sa.err = err.p;
    sa.T = T, sa.MI = MI, sa.tol = tol;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)ps_grid);
    cfg.blockDim = dim3(PS_THREADS);
    cfg.stream = st;
    cudaLaunchAttribute attr;
    attr.id = cudaLaunchAttributeCooperative;
    attr.val.cooperative = 1;
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    ctx().kernel_launches++;
    CK(cudaLaunchKernelEx(&cfg, k_steps<VT>, sa));
  }

  // whether this level runs its steps in k_steps, and with how many blocks
  bool want_persist() {
    const char *e = getenv("PARRSB_GPU_PERSIST");
    if (!e || atoi(e) == 0) return false;  // opt-in
    if (reorth || pr_fused || sp_fused || !ev.empty() || T <= 0) return false;
    int dev = 0, sms = 0, per_sm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_steps<VT>, PS_THREADS, 0));
    const ll cap = (ll)sms * per_sm;
    if (cap <= 0) return false;
    ps_grid = (int)std::min<ll>(T, cap);
    if ((T + ps_grid - 1) / ps_grid > PS_SLOTS) return false;
    ps_bar.ensure(1);
    ps_run.ensure((size_t)MI);
    return true;
  }

  // shared memory of one k_spmv_tma stage (nw slices of the widest width)
  static size_t sp_stage_bytes(const Level &lv, int threads) {
    return (size_t)(threads / 32) * (size_t)std::max(lv.max_w, 1) * 128;
  }
  bool sp_tma_ok(const Level &lv, int threads) const {
    return sizeof(VT) == 4 && SP_NST * sp_stage_bytes(lv, threads) <= 200 * 1024;
  }
  void spmv(const Level &lv, int kind, int threads, const FinArgs &fa, int fuse, int force) {
    cudaStream_t st = ctx().stream;
    if (kind == 1 && sizeof(VT) == 4) {
      const size_t sb = sp_stage_bytes(lv, threads);
      launch_pdl(k_spmv_tma, T, threads, SP_NST * sb, st, tbeg.p, tend.p, tgrp.p, gs.p,
                 lv.ell.p, lv.slice_off.p, lv.slice_w.p, reinterpret_cast<const float *>(p.p),
                 reinterpret_cast<float *>(w.p), part.p, fa, fuse, force, (int)sb, err.p);
    } else {
      launch_pdl(k_spmv<VT>, T, threads, 0, st, tbeg.p, tend.p, tgrp.p, gs.p, lv.ell.p,
                 lv.slice_off.p, lv.slice_w.p, p.p, w.p, part.p, fa, fuse, force);
    }
  }

  // Autotuner: threads per tile block for this level.  Candidates are timed
  // on the level's own matrix (three forced SpMV launches each, CUDA
  // events); the tile reductions are canonical, so the choice never changes
  // a result.  Decisions are cached per (tiles, groups, rows) for the thread.
  void autotune(const Level &lv) {
    // PARRSB_GPU_SPMV: 0 = k_spmv only, 1 = k_spmv_tma only, unset = time both
    // per device (a later call may run on another device), before the cached
    // decision is used
    ensure_smem_limit(k_spmv_tma, 200 * 1024);
    const char *force_env = getenv("PARRSB_GPU_SPMV");
    const int force_kind = force_env ? atoi(force_env) : -1;
    static thread_local std::vector<std::pair<std::array<ll, 5>, int>> cache;
    // PARRSB_GPU_SPMV_THREADS: only this block size (128, 256 or 512)
    const char *th_env = getenv("PARRSB_GPU_SPMV_THREADS");
    const int force_th = th_env ? atoi(th_env) : 0;
    std::array<ll, 5> key = {(ll)T, (ll)A, N, (ll)lv.max_w, (ll)force_kind * 1024 + force_th};
    for (auto &kv : cache)
      if (kv.first == key) {
        sp_kind = kv.second >> 16;
        bd = kv.second & 0xFFFF;
        return;
      }
    cudaStream_t st = ctx().stream;
    std::vector<std::pair<int, int>> cand;
    for (int th : {128, 256, 512}) {
      if (force_th && th != force_th) continue;
      if (force_kind < 0 || force_kind == 0) cand.push_back({0, th});
      if ((force_kind < 0 || force_kind == 1) && sp_tma_ok(lv, th)) cand.push_back({1, th});
    }
    if (cand.empty()) cand.push_back({0, 256});
    float best = 1e30f;
    std::pair<int, int> pick = cand[0];
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    for (auto &c : cand) {
      spmv(lv, c.first, c.second, fargs(0, 0.0, 0), 0, 1);
      CK(cudaEventRecord(e0, st));
      for (int rep = 0; rep < 3; rep++) spmv(lv, c.first, c.second, fargs(0, 0.0, 0), 0, 1);
      CK(cudaEventRecord(e1, st));
      CK(cudaEventSynchronize(e1));
      float ms = 0.f;
      CK(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best * 0.97f) best = ms, pick = c;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    sp_kind = pick.first;
    bd = pick.second;
    cache.push_back({key, (pick.first << 16) | pick.second});
    if (getenv("PARRSB_GPU_AUTOTUNE_LOG"))
      fprintf(stderr, "parrsb_gb300: SpMV autotune tiles=%d groups=%d rows=%lld -> %s x %d\n", T,
              A, (long long)N, pick.first ? "k_spmv_tma" : "k_spmv", pick.second);
  }

  // Runs all passes; f holds the normalised Fiedler vectors afterwards.
  // warm: f already holds the start vectors; otherwise start_kind selects
  // the reference's step vector (0) or a random one (1).
  void run(const Level &lv, double tol, int mpass, bool use_graph, bool warm,
           int start_kind = 0) {
    cudaStream_t st = ctx().stream;
    if (resid_stop) {
      resid_bufs();
      resid_tol = tol;
      tol = tol * cg_factor;  // a pass's own CG exit
    }
    // PARRSB_GPU_PASS_LOG=1 (host restart loop): each pass's residuals of the
    // first groups on stderr; =2 also the Ritz residual bound after every step
    const int pass_log = [] {
      const char *v = getenv("PARRSB_GPU_PASS_LOG");
      return v ? atoi(v) : 0;
    }();
    // early pass exit (residual-stop mode only; the persistent step kernel
    // takes no checks): after steps 3, 6, 9, ... a group whose Ritz residual
    // bound is below 0.7 rsb_tol ends its pass three steps later (the check
    // runs beside the next two); the FP64 residual of its Ritz vector still
    // decides whether it restarts.
    // PARRSB_GPU_EARLY=<factor> (0: off), _MIN, _STRIDE (at least 2)
    early = 0.0;
    if (resid_stop) {
      early = 0.7, early_min = 3, early_stride = 3;
      if (const char *v = getenv("PARRSB_GPU_EARLY")) early = std::max(0.0, atof(v));
      if (const char *v = getenv("PARRSB_GPU_EARLY_MIN")) early_min = std::max(1, atoi(v));
      if (const char *v = getenv("PARRSB_GPU_EARLY_STRIDE")) early_stride = std::max(1, atoi(v));
      // (a request applies at the latest before the step of the next check)
      early_delay = early_stride;
      if (const char *v = getenv("PARRSB_GPU_EARLY_DELAY")) early_delay = atoi(v);
      early_delay = std::max(1, std::min(early_delay, early_stride));
    }
    // (a fused finalisation counts arrivals per group: its tile blocks must
    // agree on the gate, so no checks run beside it)
    if (pr_fused || sp_fused) early = 0.0;
    bound_log = resid_stop && pass_log >= 2 && !pr_fused && !sp_fused;
    if (bound_log) early = 0.0;  // (the log checks every step and stops nothing)
    if (bound_log) bnd.ensure((size_t)A * MI);
    if ((early > 0.0 || bound_log) && !side) {
      int least = 0;
      CK(cudaDeviceGetStreamPriorityRange(&least, &side_prio));
      CK(cudaStreamCreateWithPriority(&side, cudaStreamNonBlocking, side_prio));
      CK(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
      CK(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming));
    }
    // the vectors are scratch until the first pass initialises them
    CK(cudaMemsetAsync(p.p, 0, (size_t)N * sizeof(VT), st));
    if (eig_smem() > 48 * 1024)
      CK(cudaFuncSetAttribute(k_tri_eig, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)eig_smem()));
    autotune(lv);
    k_set_active<<<grid_for(A, 128), 128, 0, st>>>(gs.p, A);
    CK_LAUNCH();
    if (!warm) {
      if (start_kind == 1)
        random_vector();
      else
        initial_vector();
    }
    long long launches = 0;
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph = nullptr;
    if (ctx().timing) {
      ev.assign(2 * MI, nullptr);
      for (auto &e : ev) CK(cudaEventCreate(&e));
      evk.assign(4 * MI + 6, nullptr);
      for (auto &e : evk) CK(cudaEventCreate(&e));
    }
    // the whole restart loop as one graph launch (no host round trip per
    // restart), unless per-launch timing is on (no event nodes in a
    // conditional body) or PARRSB_GPU_DEVICE_LOOP=0
    const bool device_loop_env = [] {
      const char *e = getenv("PARRSB_GPU_DEVICE_LOOP");
      return !(e && atoi(e) == 0);
    }();
    // sticky fallbacks after a graph could not be built (any thread, any device)
    static std::atomic<bool> device_loop_broken{false};
    static std::atomic<bool> persist_broken{false};  // a graph with k_steps failed once
    persist = !persist_broken && want_persist();
    for (int attempt = 0;
         attempt < 2 && !exec && use_graph && ev.empty() && device_loop_env && !device_loop_broken;
         attempt++) try {
      const auto h0 = std::chrono::steady_clock::now();
      CK(cudaGraphCreate(&graph, 0));
      cudaGraphConditionalHandle hnd;
      CK(cudaGraphConditionalHandleCreate(&hnd, graph, 1, cudaGraphCondAssignDefault));
      cudaGraphNodeParams cp = {};
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = hnd;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      cudaGraphNode_t node;
      CK(cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &cp));
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      loop_ctr.ensure(2);
      CK(cudaMemsetAsync(loop_ctr.p, 0, 2 * sizeof(long long), st));
      CK(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0,
                                       cudaStreamCaptureModeThreadLocal));
      long long kl = ctx().kernel_launches;
      k_loop_zero<<<1, 1, 0, st>>>(any.p);
      pass_body(lv, tol, mpass, &launches);
      k_loop_next<<<1, 1, 0, st>>>(hnd, any.p, loop_ctr.p, mpass);
      ctx().kernel_launches = kl;
      CK(cudaStreamEndCapture(st, &body));
      CK(cudaGraphInstantiate(&exec, graph, 0));
      ctx().stats.lanczos_host_ms[1] +=
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - h0)
              .count();
    } catch (const CudaError &e) {
      // the graph could not be built or instantiated here: end any capture,
      // report once, and run the restarts from the host from now on
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
        cudaGraph_t g2 = nullptr;
        cudaStreamEndCapture(st, &g2);
        if (g2) cudaGraphDestroy(g2);
      }
      cudaGetLastError();
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
      exec = nullptr, graph = nullptr;
      if (persist) {  // try again with the launch-per-kernel steps
        persist_broken = true;
        persist = false;
        fprintf(stderr, "parrsb_gb300: persistent step kernel unavailable in graphs (%s)\n",
                cudaGetErrorString(e.err));
        continue;
      }
      device_loop_broken = true;
      fprintf(stderr, "parrsb_gb300: device restart loop unavailable (%s); host loop used\n",
              cudaGetErrorString(e.err));
    }
    if (exec) {  // the device loop was built
      const auto h1 = std::chrono::steady_clock::now();
      CK(cudaGraphLaunch(exec, st));
      long long hc[2] = {0, 0};
      d2h(hc, loop_ctr.p, 2);
      sync();
      const long long per_pass_kernels =
          6 + step_kernels() + 5 + (resid_stop ? 3 + resid1_launches(lv) : 0);
      ctx().kernel_launches += per_pass_kernels * hc[0];
      ctx().stats.lanczos_passes += hc[0];
      ctx().stats.spmv_launches += hc[1];
      ctx().stats.lanczos_host_ms[2] +=
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - h1)
              .count();
      cudaGraphExecDestroy(exec);
      cudaGraphDestroy(graph);
      exec = nullptr, graph = nullptr;
      finish_run();
      return;
    }
    for (int attempt = 0; attempt < 2 && use_graph && !exec; attempt++) try {
      const auto h0 = std::chrono::steady_clock::now();
      CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      long long kl = ctx().kernel_launches;
      pass_body(lv, tol, mpass, &launches);
      ctx().kernel_launches = kl;
      CK(cudaStreamEndCapture(st, &graph));
      CK(cudaGraphInstantiate(&exec, graph, 0));
      ctx().stats.lanczos_host_ms[1] +=
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - h0).count();
    } catch (const CudaError &e) {
      if (!persist) throw;
      cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
      if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
        cudaGraph_t g2 = nullptr;
        cudaStreamEndCapture(st, &g2);
        if (g2) cudaGraphDestroy(g2);
      }
      cudaGetLastError();
      if (exec) cudaGraphExecDestroy(exec);
      if (graph) cudaGraphDestroy(graph);
      exec = nullptr, graph = nullptr;
      persist_broken = true;
      persist = false;
      fprintf(stderr, "parrsb_gb300: persistent step kernel unavailable in graphs (%s)\n",
              cudaGetErrorString(e.err));
    }
    const long long per_pass_kernels =
        4 + step_kernels() + 5 + (resid_stop ? 3 + resid1_launches(lv) : 0);
    launches = 0;
    // PARRSB_GPU_LEVEL_LOG=1 (timing mode): one line per level on stderr
    const bool level_log = !ev.empty() && getenv("PARRSB_GPU_LEVEL_LOG");
    const double spmv0 = ctx().stats.spmv_ms, pass0 = ctx().stats.lanczos_ms[5];
    int npass = 0;
    const auto hp0 = std::chrono::steady_clock::now();
    for (int pass = 0; pass < mpass; pass++) {
      CK(cudaMemsetAsync(any.p, 0, 2 * sizeof(int), st));
      if (bound_log)  // 0x7F bytes: a large positive double where no step ran
        CK(cudaMemsetAsync(bnd.p, 0x7F, (size_t)A * MI * sizeof(double), st));
      if (use_graph) {
        CK(cudaGraphLaunch(exec, st));
        ctx().kernel_launches += per_pass_kernels;
      } else {
        long long dummy = 0;
        pass_body(lv, tol, mpass, &dummy);
      }
      int h_any[2] = {0, 0};
      d2h(h_any, any.p, 2);
      sync();
      launches += h_any[1];  // SpMV launches that did work this pass
      ctx().stats.lanczos_passes++;
      npass++;
      if (pass_log) log_pass(pass);
      if (!ev.empty()) {
        auto el = [&](cudaEvent_t a, cudaEvent_t b) {
          float ms = 0.f;
          CK(cudaEventElapsedTime(&ms, a, b));
          return (double)ms;
        };
        double *lm = ctx().stats.lanczos_ms;
        for (int it = 0; it < MI; it++) {
          if (it < h_any[1]) ctx().stats.spmv_ms += el(ev[2 * it], ev[2 * it + 1]);
          lm[0] += el(evk[4 * it + 0], evk[4 * it + 1]);
          lm[1] += el(evk[4 * it + 2], evk[4 * it + 3]);
        }
        lm[4] += el(evk[4 * MI + 0], evk[4 * MI + 1]);
        lm[2] += el(evk[4 * MI + 2], evk[4 * MI + 3]);
        lm[3] += el(evk[4 * MI + 4], evk[4 * MI + 5]);
        // wall time of the whole pass on the device minus its parts
        lm[5] += el(evk[4 * MI + 0], evk[4 * MI + 5]);
      }
      if (!h_any[0]) break;
    }
    ctx().stats.lanczos_host_ms[2] +=
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - hp0).count();
    if (level_log)
      fprintf(stderr,
              "parrsb_gb300: level rows=%lld groups=%d tiles=%d passes=%d steps=%lld "
              "spmv_ms=%.2f (%.4f per step) pass_ms=%.2f\n",
              (long long)N, A, T, npass, launches, ctx().stats.spmv_ms - spmv0,
              launches ? (ctx().stats.spmv_ms - spmv0) / launches : 0.0,
              ctx().stats.lanczos_ms[5] - pass0);
    for (auto &e : ev) cudaEventDestroy(e);
    ev.clear();
    for (auto &e : evk) cudaEventDestroy(e);
    evk.clear();
    ctx().stats.spmv_launches += launches;
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    finish_run();
  }

  // one stderr line per group (the first four) after a pass of the host loop
  void log_pass(int pass) {
    const int ng = std::min(A, 4);
    std::vector<GState> h(ng);
    d2h(h.data(), gs.p, ng);
    std::vector<double> hb;
    if (bound_log) {
      hb.resize((size_t)ng * MI);
      d2h(hb.data(), bnd.p, hb.size());
    }
    sync();
    const double th[5] = {1e-4, 3e-5, 1e-5, 5e-6, 2e-6};
    for (int g = 0; g < ng; g++) {
      fprintf(stderr, "parrsb_gb300: pass %d group %d n=%lld iters=%d resid=%.3e active=%d", pass,
              g, (long long)h[g].n, h[g].iters, h[g].resid, h[g].active);
      if (bound_log) {
        fprintf(stderr, " bound<=[1e-4,3e-5,1e-5,5e-6,2e-6] at");
        for (double t : th) {
          int at = -1;
          for (int it = 0; it < h[g].iters && at < 0; it++)
            if (hb[(size_t)g * MI + it] <= t) at = it + 1;
          fprintf(stderr, " %d", at);
        }
        if (h[g].iters > 0) fprintf(stderr, " last=%.3e", hb[(size_t)g * MI + h[g].iters - 1]);
      }
      fprintf(stderr, "\n");
    }
  }

  // after the restarts: the staged SpMV's error flag, then normalise
  // (src/fiedler.c:606-613) and fix the sign canonically: sum_i s_i f_i >= 0
  // with s = +1 on the first half of the group's order
  void finish_run() {
    {
      int h_err = 0;
      d2h(&h_err, err.p, 1);
      sync();
      if (h_err) throw CudaError{cudaErrorLaunchTimeout, __FILE__, __LINE__};  // a stage wait gave up
    }
    tile<TM_SQ_F, GATE_ALL>();
    fin<FIN_NORM, GATE_ALL>();
    tile<TM_ORIENT, GATE_ALL>();
    fin<FIN_ORIENT, GATE_ALL>();
    tile<TM_SCALE_F, GATE_ALL>();
  }

  // y64 = L f and the tile partials of f.y and f.f, for FIN_RESID1: the
  // exact fixed-point form for FP32 vectors (k_rq_*), else FP64 (k_tile)
  bool resid_int(const Level &lv) const { return sizeof(VT) == 4 && lv.max_w <= RQ_MAX_WIDTH; }
  // Buffers of the residual check.  Every buffer a pass graph uses must
  // exist before its capture starts: an allocation from the stream-ordered
  // pool on a capturing stream becomes a node of the graph (memory the graph
  // owns, not allowed in a conditional body at all).
  void resid_bufs() {
    y64.ensure((size_t)N);
    if (sizeof(VT) == 4) {
      fq.ensure((size_t)N);
      gmax.ensure((size_t)A);
      tmax.ensure((size_t)T);
    }
  }
  int resid1_launches(const Level &lv) const { return resid_int(lv) ? 3 : 1; }
  template <int GATE>
  void resid1(const Level &lv) {
    if constexpr (sizeof(VT) == 4) {
      if (resid_int(lv)) {
        cudaStream_t st = ctx().stream;
        resid_bufs();  // (allocated before any capture: a no-op here then)
        launch_pdl(k_rq_max<GATE>, T, 256, 0, st, tbeg.p, tend.p, tgrp.p, gs.p, f.p, tmax.p);
        launch_pdl(k_rq_quant<GATE>, T, 256, 0, st, tbeg.p, tend.p, tgrp.p, gs.p, f.p, tmax.p,
                   gmax.p, fq.p);
        launch_pdl(k_rq_resid1<GATE>, T, RQ_THREADS, 0, st, tbeg.p, tend.p, tgrp.p, gs.p, f.p,
                   fq.p, gmax.p, lv.ell.p, lv.slice_off.p, lv.slice_w.p, y64.p, part.p);
        return;
      }
    }
    tile<TM_RESID1, GATE>(0, &lv);
  }
  // the tile partials of sum (y - rho f)^2, for FIN_RESID2 / FIN_RESID_GATE
  template <int GATE>
  void resid2(const Level &lv) {
    if constexpr (sizeof(VT) == 4) {
      if (resid_int(lv)) {
        launch_pdl(k_rq_resid2<GATE>, T, RQ_THREADS, 0, ctx().stream, tbeg.p, tend.p, tgrp.p,
                   gs.p, f.p, y64.p, part.p);
        return;
      }
    }
    tile<TM_RESID2, GATE>(0, &lv);
  }

  void residual(const Level &lv) {
    resid_bufs();
    resid1<GATE_ALL>(lv);
    fin<FIN_RESID1, GATE_ALL>();
    resid2<GATE_ALL>(lv);
    fin<FIN_RESID2, GATE_ALL>();
  }

  void download(std::vector<GState> &out) {
    out.resize(A);
    d2h(out.data(), gs.p, A);
    sync();
  }
};

// ----------------------------------------------------------------------------
// RSB level helpers
// ----------------------------------------------------------------------------
inline bool env_flag(const char *name) {
  const char *v = getenv(name);
  return v && atoi(v) != 0;
}

struct HGroup {
  ll start, n;
  int p, r0;
};

__global__ void k_fied_keys(const double *__restrict__ f_pos, const int *__restrict__ grp,
                            ll N, u64 *__restrict__ keys, int *__restrict__ vals) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  keys[i] = grp[i] >= 0 ? ordered_key(f_pos[i]) : 0ull;
  vals[i] = (int)i;
}

template <typename VT>
__global__ void k_to_double(const VT *__restrict__ in, ll N, double *__restrict__ out) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) out[i] = (double)in[i];
}

__global__ void k_gather_perm(const int *__restrict__ idx, const int *__restrict__ perm_in,
                              const double *__restrict__ f_in, ll N,
                              int *__restrict__ perm_out, double *__restrict__ f_out) {
  ll j = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  int i = idx[j];
  perm_out[j] = perm_in[i];
  f_out[j] = f_in[i];
}

__global__ void k_keys_elem_id(const int *__restrict__ perm, const int *__restrict__ grp,
                               ll N, u64 *__restrict__ keys, int *__restrict__ vals) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  keys[i] = grp[i] >= 0 ? (u64)perm[i] : 0ull;
  vals[i] = (int)i;
}

__global__ void k_gather_int(const int *__restrict__ idx, const int *__restrict__ in, ll N,
                             int *__restrict__ out) {
  ll j = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (j < N) out[j] = in[idx[j]];
}

// Component count by min-label hooking + pointer jumping on the level graph
// restricted to each half.
__global__ void k_cc_init(int *__restrict__ lab, ll N) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) lab[i] = (int)i;
}

__global__ void k_cc_hook(const unsigned *__restrict__ ell, const ll *__restrict__ slice_off,
                          const int *__restrict__ slice_w, const int *__restrict__ half,
                          ll N, int *__restrict__ lab, int *__restrict__ changed) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int h = half[i];
  if (h < 0) return;
  ll sl = i >> 5;
  const unsigned *ep = ell + slice_off[sl] + (i & 31);
  int wd = slice_w[sl];
  for (int k = 0; k < wd; k++) {
    unsigned x = ep[(ll)k * 32];
    if ((x >> 28) == 0) continue;
    int j = x & 0x0FFFFFFF;
    if (half[j] != h) continue;
    int a = lab[i], b = lab[j];
    if (a == b) continue;
    int hi = a > b ? a : b, lo = a > b ? b : a;
    atomicMin(&lab[hi], lo);
    *changed = 1;
  }
}

// Afforest-style start: hook every row to its r-th neighbour in its half
// (one edge per row), so most of a half joins one tree before full rounds.
__global__ void k_cc_sample(const unsigned *__restrict__ ell, const ll *__restrict__ slice_off,
                            const int *__restrict__ slice_w, const int *__restrict__ half, ll N,
                            int r, int *__restrict__ lab) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int h = half[i];
  if (h < 0) return;
  ll sl = i >> 5;
  const unsigned *ep = ell + slice_off[sl] + (i & 31);
  int wd = slice_w[sl], seen = 0;
  for (int k = 0; k < wd; k++) {
    unsigned x = ep[(ll)k * 32];
    if ((x >> 28) == 0) continue;
    int j = x & 0x0FFFFFFF;
    if (half[j] != h) continue;
    if (seen++ < r) continue;
    int a = lab[i], b = lab[j];
    if (a != b) atomicMin(&lab[a > b ? a : b], a > b ? b : a);
    return;
  }
}

// the root of a half's first row: presumed root of the half's largest part
__global__ void k_cc_giant(const ll *__restrict__ hstart, int nh, const int *__restrict__ lab,
                           int *__restrict__ giant) {
  int h = blockIdx.x * blockDim.x + threadIdx.x;
  if (h < nh) giant[h] = lab[hstart[h]];
}

// full round for the rows outside their half's presumed giant tree: an edge
// between a skipped row and another row is seen from the other row (the
// graph is symmetric), and an edge between two skipped rows joins nothing
// new, so skipping never loses a hook
__global__ void k_cc_hook_rest(const unsigned *__restrict__ ell, const ll *__restrict__ slice_off,
                               const int *__restrict__ slice_w, const int *__restrict__ half,
                               const int *__restrict__ giant, ll N, int *__restrict__ lab,
                               int *__restrict__ changed) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int h = half[i];
  if (h < 0 || lab[i] == giant[h]) return;
  ll sl = i >> 5;
  const unsigned *ep = ell + slice_off[sl] + (i & 31);
  int wd = slice_w[sl];
  for (int k = 0; k < wd; k++) {
    unsigned x = ep[(ll)k * 32];
    if ((x >> 28) == 0) continue;
    int j = x & 0x0FFFFFFF;
    if (half[j] != h) continue;
    int a = lab[i], b = lab[j];
    if (a == b) continue;
    int hi = a > b ? a : b, lo = a > b ? b : a;
    atomicMin(&lab[hi], lo);
    *changed = 1;
  }
}

__global__ void k_cc_compress(int *__restrict__ lab, ll N) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int l = lab[i];
  while (lab[l] != l) l = lab[l];
  lab[i] = l;
}

__global__ void k_cc_count(const int *__restrict__ lab, const int *__restrict__ half, ll N,
                           int *__restrict__ cnt) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N && half[i] >= 0 && lab[i] == i) atomicAdd(&cnt[half[i]], 1);
}

// Balance: mark sender rows with a neighbour in the receiver half.
__global__ void k_bd_flag(const unsigned *__restrict__ ell, const ll *__restrict__ slice_off,
                          const int *__restrict__ slice_w, const int *__restrict__ half,
                          const int *__restrict__ send_half,  // per half id: receiver id or -1
                          ll N, int *__restrict__ flag, int *__restrict__ cnt) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int h = half[i];
  int f = 0;
  if (h >= 0 && send_half[h] >= 0) {
    int recv = send_half[h];
    ll sl = i >> 5;
    const unsigned *ep = ell + slice_off[sl] + (i & 31);
    int wd = slice_w[sl];
    for (int k = 0; k < wd && !f; k++) {
      unsigned x = ep[(ll)k * 32];
      if ((x >> 28) && half[x & 0x0FFFFFFF] == recv) f = 1;
    }
    if (f) atomicAdd(&cnt[h], 1);
  }
  flag[i] = f;
}

__global__ void k_bd_keys(const int *__restrict__ flag, const ll *__restrict__ excl,
                          const double *__restrict__ f_pos, const int *__restrict__ half,
                          const double *__restrict__ mul_of_half, ll N,
                          u64 *__restrict__ keys, int *__restrict__ vals,
                          int *__restrict__ seg_of_val) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || !flag[i]) return;
  ll o = excl[i];
  keys[o] = ordered_key(__dmul_rn(mul_of_half[half[i]], f_pos[i]));
  vals[o] = (int)i;
  seg_of_val[i] = half[i];
}

__global__ void k_bd_moved(const int *__restrict__ vals, ll nb, const ll *__restrict__ off,
                           const ll *__restrict__ sendc, const int *__restrict__ half,
                           int *__restrict__ moved) {
  ll q = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nb) return;
  int i = vals[q];
  int h = half[i];
  if (q - off[h] < sendc[h]) moved[i] = 1;
}

// New arrangement of balanced groups.  Each position gets a segment id that
// increases with position (active group a owns ids base[a] and base[a] + 1;
// frozen groups keep the id in segpos) and a key: the Fiedler value where a
// half must be re-sorted, 0 to keep the current order.
__global__ void k_rebal_keys(const int *__restrict__ half, const int *__restrict__ moved,
                             const int *__restrict__ mode_of_group,  // 0 none, 1 A sends, 2 B sends
                             const int *__restrict__ base, const int *__restrict__ segpos,
                             const double *__restrict__ f_pos, ll N,
                             u64 *__restrict__ keys, int *__restrict__ vals,
                             int *__restrict__ seg_of_val) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  int h = half[i];
  u64 k = 0;
  if (h >= 0) {
    int g = h >> 1, isB = h & 1;
    int mode = mode_of_group[g];
    int sub = isB;
    if (mode == 1) {  // A sends to B: moved A elements join B; B re-sorted
      if (!isB && moved[i]) sub = 1;
      if (sub == 1) k = ordered_key(f_pos[i]);
    } else if (mode == 2) {  // B sends to A: moved B elements join A; A re-sorted
      if (isB && moved[i]) sub = 0;
      if (sub == 0) k = ordered_key(f_pos[i]);
    }
    seg_of_val[i] = base[g] + sub;
  } else {
    seg_of_val[i] = segpos[i];
  }
  keys[i] = k;
  vals[i] = (int)i;
}

__global__ void k_part_scatter(const int *__restrict__ perm, const int *__restrict__ grp, ll N,
                               int *__restrict__ part) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) part[perm[i]] = grp[i];
}

__global__ void k_seq_rel(const int *__restrict__ perm, const int *__restrict__ gstart, ll N,
                          int *__restrict__ seq) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) seq[perm[i]] = (int)(i - gstart[i]);
}

__global__ void k_fill_grp(const ll *__restrict__ gstart, const ll *__restrict__ gn,
                           const int *__restrict__ gid, int ng, int *__restrict__ grp) {
  // one block per group, loop over its range
  int g = blockIdx.x;
  if (g >= ng) return;
  for (ll i = gstart[g] + threadIdx.x; i < gstart[g] + gn[g]; i += blockDim.x) grp[i] = gid[g];
}

// Fill pos -> id for host-described contiguous groups.
void fill_groups(const std::vector<ll> &st, const std::vector<ll> &n, const std::vector<int> &id,
                 int *d_out, ll N) {
  int ng = (int)st.size();
  if (ng == 0) return;
  DBuf<ll> a(ng), b(ng);
  DBuf<int> c(ng);
  h2d(a.p, st.data(), ng);
  h2d(b.p, n.data(), ng);
  h2d(c.p, id.data(), ng);
  k_fill_grp<<<ng, 256, 0, ctx().stream>>>(a.p, b.p, c.p, ng, d_out);
  CK_LAUNCH();
  sync();
}

void build_level(const Graph &g, const int *perm, const int *inv, const int *grp, ll N,
                 Level &lv) {
  cudaStream_t st = ctx().stream;
  DBuf<int> rowlen((size_t)N);
  k_ell_count<<<grid_for(N, 256), 256, 0, st>>>(perm, inv, grp, g.rowptr.p, g.col.p, N,
                                                rowlen.p);
  CK_LAUNCH();
  ll nslice = (N + 31) / 32;
  DBuf<ll> slots((size_t)nslice + 1);
  lv.slice_w.ensure((size_t)nslice);
  lv.slice_off.ensure((size_t)nslice + 1);
  k_slice_w<<<grid_for(nslice, 256), 256, 0, st>>>(rowlen.p, N, nslice, slots.p, lv.slice_w.p);
  CK_LAUNCH();
  ll total = exclusive_scan_ll(slots.p, lv.slice_off.p, nslice);
  h2d(lv.slice_off.p + nslice, &total, 1);  // end of the last slice
  lv.ell.ensure((size_t)total + 32);
  k_ell_fill<<<grid_for(N, 256), 256, 0, st>>>(perm, inv, grp, g.rowptr.p, g.col.p, g.w.p, N,
                                               lv.slice_off.p, lv.slice_w.p, lv.ell.p);
  CK_LAUNCH();
  // restricted nnz of active rows (for the algorithmic byte count)
  DBuf<ll> rl64((size_t)N);
  ll nnz = exclusive_scan_int_to_ll(rowlen.p, rl64.p, N);
  lv.nnz = nnz;
  DBuf<int> mw(1);
  CK(cudaMemsetAsync(mw.p, 0, sizeof(int), st));
  k_max_int<<<grid_for(nslice, 256), 256, 0, st>>>(lv.slice_w.p, nslice, mw.p);
  CK_LAUNCH();
  d2h(&lv.max_w, mw.p, 1);
  sync();
}

// Number of vertex-connected components of every half (get_components_v2,
// src/components.c:160-328, count only): min-label hooking plus pointer
// jumping on the level graph restricted to each half.  half[i] is the half
// id of position i (-1: none); hstart[h] is a position inside half h (its
// first one).  Two one-edge hooking rounds join most of a half into one
// tree; full rounds then visit only the rows outside the tree of hstart[h]
// (PARRSB_GPU_CC_FULL=1: every row every round).  Returns the counts by id.
std::vector<int> count_components_level(const Level &lv, const int *half, ll N,
                                        const std::vector<ll> &hstart,
                                        DBuf<int> *labels_out = nullptr) {
  cudaStream_t st = ctx().stream;
  const int nh = (int)hstart.size();
  std::vector<int> hc(nh, 0);
  if (nh == 0 || N == 0) return hc;
  DBuf<int> lab((size_t)N), changed(1), cnt((size_t)nh);
  k_cc_init<<<grid_for(N, 256), 256, 0, st>>>(lab.p, N);
  CK_LAUNCH();
  const bool full = env_flag("PARRSB_GPU_CC_FULL");
  DBuf<int> giant((size_t)nh);
  if (!full) {
    for (int r = 0; r < 2; r++) {
      k_cc_sample<<<grid_for(N, 256), 256, 0, st>>>(lv.ell.p, lv.slice_off.p, lv.slice_w.p, half,
                                                    N, r, lab.p);
      CK_LAUNCH();
      k_cc_compress<<<grid_for(N, 256), 256, 0, st>>>(lab.p, N);
      CK_LAUNCH();
    }
    DBuf<ll> hs((size_t)nh);
    h2d(hs.p, hstart.data(), nh);
    k_cc_giant<<<grid_for(nh, 256), 256, 0, st>>>(hs.p, nh, lab.p, giant.p);
    CK_LAUNCH();
  }
  for (int round = 0; round < 100000; round++) {
    CK(cudaMemsetAsync(changed.p, 0, sizeof(int), st));
    if (full)
      k_cc_hook<<<grid_for(N, 256), 256, 0, st>>>(lv.ell.p, lv.slice_off.p, lv.slice_w.p, half, N,
                                                  lab.p, changed.p);
    else
      k_cc_hook_rest<<<grid_for(N, 256), 256, 0, st>>>(lv.ell.p, lv.slice_off.p, lv.slice_w.p,
                                                       half, giant.p, N, lab.p, changed.p);
    CK_LAUNCH();
    k_cc_compress<<<grid_for(N, 256), 256, 0, st>>>(lab.p, N);
    CK_LAUNCH();
    int h = 0;
    d2h(&h, changed.p, 1);
    sync();
    if (!h) break;
  }
  CK(cudaMemsetAsync(cnt.p, 0, (size_t)nh * sizeof(int), st));
  k_cc_count<<<grid_for(N, 256), 256, 0, st>>>(lab.p, half, N, cnt.p);
  CK_LAUNCH();
  d2h(hc.data(), cnt.p, nh);
  sync();
  if (labels_out) *labels_out = std::move(lab);  // label = root position of the component
  return hc;
}

// y_warm (optional): learned start candidates per position (FP64), judged
// per group against the fallback start before Lanczos runs.
template <typename VT>
void run_fiedler_level(Lanczos<VT> &lz, const Level &lv, const RsbOpts &o,
                       const std::vector<ll> &gstart, const std::vector<ll> &gn, ll N,
                       double *f_pos, std::vector<GState> &res,
                       const double *y_warm = nullptr) {
  lz.setup(gstart, gn, N, o.miter);
  lz.reorth = o.reorth != 0;
  if (lz.reorth) {
    lz.part2.ensure((size_t)lz.T * (o.miter + 1) + 1);
    lz.hro.ensure((size_t)lz.A * (o.miter + 1) + 1);
  }
  lz.resid_stop = o.resid_stop != 0;
  lz.cg_factor = o.cg_factor;
  {
    StageTimer tm(PARRSB_STAGE_LANCZOS);
    const auto h0 = std::chrono::steady_clock::now();
    if (y_warm) lz.choose_start(lv, y_warm, o.start);
    ctx().stats.lanczos_host_ms[0] +=
        std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - h0).count();
    lz.run(lv, o.tol, o.mpass, o.use_graphs != 0, y_warm != nullptr, o.start);
  }
  const auto h1 = std::chrono::steady_clock::now();
  // the residual-stop rule has already computed every group's FP64
  // eigen-residual at its last restart (normalising and orienting the
  // vector afterwards does not change it)
  if (o.check_resid && !o.resid_stop) lz.residual(lv);
  k_to_double<VT><<<grid_for(N, 256), 256, 0, ctx().stream>>>(lz.f.p, N, f_pos);
  CK_LAUNCH();
  lz.download(res);
  ctx().stats.lanczos_host_ms[3] +=
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - h1).count();
}

// ----------------------------------------------------------------------------
// Coarse-graph start (PARRSB_GPU_COARSE=1): for the groups of a level with at
// least PARRSB_GPU_COARSE_MIN elements, aggregates of elements whose
// centroids fall in the same cell of two element spacings per axis (on a
// mesh of near-uniform hexes: blocks of 2x2x2 elements) form a coarse graph
// with the Laplacian P^T L P (P the aggregation: a coarse row sums its fine
// rows, entries inside an aggregate cancel in the difference form, an
// entry's weight is the sum of the fine weights between the two
// aggregates, split into 4-bit pieces so the coarse matrix is an ordinary
// level matrix).  One Lanczos pass on it from the geometric start,
// prolonged to the fine positions, becomes the group's warm start candidate
// (judged as any other).  A group's spacing per axis is its centroid extent
// over its number of element layers, round(extent / h) + 1, with h the mean
// |d| of face neighbours whose displacement lies mostly along that axis.
// ----------------------------------------------------------------------------
constexpr int CR_CAP = 512;  // fine entries of one coarse row
constexpr int CS_BITS = 14;  // cell index bits per axis in the sort key

// per coarse-eligible group (sel[a] >= 0): ordered-key min / max of the
// centroid per axis, and per axis the sum and count of |d| over face
// neighbours (weight wface) displaced mostly along it
__global__ void k_cs_stats(const unsigned *__restrict__ ell, const ll *__restrict__ slice_off,
                           const int *__restrict__ slice_w, const int *__restrict__ perm,
                           const int *__restrict__ grp, const int *__restrict__ sel,
                           const double *__restrict__ cent, ll nel, ll N, unsigned wface,
                           unsigned long long *__restrict__ mn, unsigned long long *__restrict__ mx,
                           double *__restrict__ hsum, unsigned long long *__restrict__ hcnt) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int g = -1;
  double c[3] = {0.0, 0.0, 0.0}, s[3] = {0.0, 0.0, 0.0};
  unsigned n[3] = {0u, 0u, 0u};
  if (i < N) {
    const int a = grp[i];
    g = a >= 0 ? sel[a] : -1;
  }
  if (g >= 0) {
    const int e = perm[i];
    for (int d = 0; d < 3; d++) c[d] = cent[(ll)d * nel + e];
    const unsigned *ep = ell + slice_off[i >> 5] + (i & 31);
    const int wd = slice_w[i >> 5];
    for (int k = 0; k < wd; k++) {
      const unsigned x = ep[(ll)k * 32];
      if ((x >> 28) != wface) continue;
      const int ej = perm[x & 0x0FFFFFFFu];
      double dd[3], best = -1.0;
      int ax = 0;
      for (int d = 0; d < 3; d++) {
        dd[d] = fabs(cent[(ll)d * nel + ej] - c[d]);
        if (dd[d] > best) best = dd[d], ax = d;
      }
      s[ax] += dd[ax];
      n[ax] += 1u;
    }
  }
  // one atomic per warp and quantity when the warp lies in one group
  const int g0 = __shfl_sync(0xffffffffu, g, 0);
  const bool same = __all_sync(0xffffffffu, g == g0);
  if (same) {
    if (g0 < 0) return;
    for (int d = 0; d < 3; d++) {
      double v = s[d];
      unsigned cn = n[d];
      double lo = c[d], hi = c[d];
      for (int o = 16; o > 0; o >>= 1) {
        v += __shfl_xor_sync(0xffffffffu, v, o);
        cn += __shfl_xor_sync(0xffffffffu, cn, o);
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
      }
      if (lane == 0) {
        atomicAdd(&hsum[3 * g0 + d], v);
        atomicAdd(&hcnt[3 * g0 + d], (unsigned long long)cn);
        atomicMin(&mn[3 * g0 + d], ordered_key(lo));
        atomicMax(&mx[3 * g0 + d], ordered_key(hi));
      }
    }
  } else if (g >= 0) {
    for (int d = 0; d < 3; d++) {
      atomicAdd(&hsum[3 * g + d], s[d]);
      atomicAdd(&hcnt[3 * g + d], (unsigned long long)n[d]);
      atomicMin(&mn[3 * g + d], ordered_key(c[d]));
      atomicMax(&mx[3 * g + d], ordered_key(c[d]));
    }
  }
}

// sort key of every position: (coarse group, cell z, y, x); ~0 outside
__global__ void k_cs_keys(const int *__restrict__ perm, const int *__restrict__ grp,
                          const int *__restrict__ sel, const double *__restrict__ cent, ll nel,
                          ll N, const double *__restrict__ cmin, const double *__restrict__ ch,
                          const int *__restrict__ nlay, u64 *__restrict__ keys,
                          int *__restrict__ vals) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int a = grp[i];
  const int g = a >= 0 ? sel[a] : -1;
  u64 key = ~0ull;
  if (g >= 0) {
    const int e = perm[i];
    key = (u64)g << (3 * CS_BITS);
    for (int d = 0; d < 3; d++) {
      int idx = (int)floor((cent[(ll)d * nel + e] - cmin[3 * g + d]) / ch[3 * g + d] + 0.5);
      idx = idx < 0 ? 0 : (idx >= nlay[3 * g + d] ? nlay[3 * g + d] - 1 : idx);
      key |= (u64)(idx >> 1) << (CS_BITS * d);
    }
  }
  keys[i] = key;
  vals[i] = (int)i;
}

// runs of equal keys after the sort: flag[s] = 1 at a run's first entry
__global__ void k_cs_flags(const u64 *__restrict__ keys, ll N, int *__restrict__ flag) {
  const ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= N) return;
  flag[s] = (keys[s] != ~0ull && (s == 0 || keys[s] != keys[s - 1])) ? 1 : 0;
}

// aggregate of every position (cmap), each aggregate's first sorted entry
// (agg_off) and each coarse group's first aggregate (cst_dev)
__global__ void k_cs_aggs(const u64 *__restrict__ keys, const int *__restrict__ vals,
                          const int *__restrict__ flag, const ll *__restrict__ excl, ll N,
                          int *__restrict__ cmap, ll *__restrict__ agg_off,
                          ll *__restrict__ cst_dev) {
  const ll s = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= N || keys[s] == ~0ull) return;
  const ll agg = excl[s] + flag[s] - 1;
  cmap[vals[s]] = (int)agg;
  if (flag[s]) {
    agg_off[agg] = s;
    const u64 g = keys[s] >> (3 * CS_BITS);
    if (s == 0 || (keys[s - 1] >> (3 * CS_BITS)) != g) cst_dev[g] = agg;
  }
}

// One warp per coarse row: its fine rows' entries (coarse column, weight) in
// row and slot order, a bitonic sort by (column, weight), the weights summed
// per column, emitted in column order as pieces of at most 15.  Count mode
// writes the row's entry count; fill mode writes the entries and the
// weight-0 padding of its slice.  err: a coarse row had more than CR_CAP
// fine entries (the caller then keeps the geometric start).
template <bool FILL>
__global__ void __launch_bounds__(256)
k_coarse_rows(const unsigned *__restrict__ ell, const ll *__restrict__ slice_off,
              const int *__restrict__ slice_w, const int *__restrict__ cmap,
              const ll *__restrict__ agg_off, const int *__restrict__ agg_pos, ll Nc,
              int *__restrict__ rowlen, const ll *__restrict__ cslice_off,
              const int *__restrict__ cslice_w, unsigned *__restrict__ cell,
              int *__restrict__ err) {
  __shared__ unsigned long long sbuf[8][CR_CAP];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const ll I = (ll)blockIdx.x * 8 + wib;
  if (I >= Nc) return;  // the whole warp
  unsigned long long *buf = sbuf[wib];
  int m = 0;
  for (ll t = agg_off[I]; t < agg_off[I + 1]; t++) {
    const ll i = agg_pos[t];
    const unsigned *ep = ell + slice_off[i >> 5] + (i & 31);
    const int wd = slice_w[i >> 5];
    for (int k0 = 0; k0 < wd; k0 += 32) {
      const int k = k0 + lane;
      bool ok = false;
      unsigned long long key = 0;
      if (k < wd) {
        const unsigned x = ep[(ll)k * 32];
        const unsigned w = x >> 28;
        if (w) {
          const int J = cmap[x & 0x0FFFFFFFu];
          if (J >= 0 && (ll)J != I) {
            ok = true;
            key = ((unsigned long long)(unsigned)J << 8) | w;
          }
        }
      }
      const unsigned b = __ballot_sync(0xffffffffu, ok);
      const int pos = m + __popc(b & ((1u << lane) - 1u));
      if (ok && pos < CR_CAP) buf[pos] = key;
      m += __popc(b);
    }
  }
  if (m > CR_CAP) {
    if (lane == 0) atomicOr(err, 1);
    m = CR_CAP;
  }
  int p2 = 1;
  while (p2 < m) p2 <<= 1;
  for (int q = m + lane; q < p2; q += 32) buf[q] = ~0ull;
  __syncwarp();
  for (int kk = 2; kk <= p2; kk <<= 1)
    for (int jj = kk >> 1; jj > 0; jj >>= 1) {
      for (int q = lane; q < p2; q += 32) {
        const int r = q ^ jj;
        if (r > q) {
          const unsigned long long a = buf[q], c = buf[r];
          if ((q & kk) == 0 ? a > c : a < c) buf[q] = c, buf[r] = a;
        }
      }
      __syncwarp();
    }
  if (lane != 0) return;
  const ll sl = I >> 5;
  unsigned *out = FILL ? cell + cslice_off[sl] + (I & 31) : nullptr;
  const int cwd = FILL ? cslice_w[sl] : 0;
  int e = 0, q = 0;
  while (q < m) {
    const unsigned J = (unsigned)(buf[q] >> 8);
    unsigned W = 0;
    while (q < m && (unsigned)(buf[q] >> 8) == J) W += (unsigned)(buf[q] & 0xFFu), q++;
    while (W > 0) {
      const unsigned c = W > 15u ? 15u : W;
      if (FILL && e < cwd) out[(ll)e * 32] = J | (c << 28);
      e++;
      W -= c;
    }
  }
  if (FILL) {
    for (; e < cwd; e++) out[(ll)e * 32] = (unsigned)I;  // weight-0 padding
  } else {
    rowlen[I] = e;
  }
}

// coarse centroids (the mean of the aggregate's) and element spacings (the
// sums of the aggregate's; only their ratios between axes matter)
__global__ void k_coarse_cent(const int *__restrict__ perm, const double *__restrict__ cent,
                              ll nel, const float4 *__restrict__ esp,
                              const ll *__restrict__ agg_off, const int *__restrict__ agg_pos,
                              ll Nc, double *__restrict__ cent_c, float4 *__restrict__ esp_c) {
  const ll I = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= Nc) return;
  double sx = 0.0, sy = 0.0, sz = 0.0;
  float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
  const ll t0 = agg_off[I], t1 = agg_off[I + 1];
  for (ll t = t0; t < t1; t++) {
    const int el = perm[agg_pos[t]];
    sx += cent[el], sy += cent[nel + el], sz += cent[2 * nel + el];
    if (esp) {
      const float4 v = esp[el];
      q.x += v.x, q.y += v.y, q.z += v.z, q.w += v.w;
    }
  }
  const double inv = 1.0 / (double)(t1 - t0);
  cent_c[I] = sx * inv, cent_c[Nc + I] = sy * inv, cent_c[2 * Nc + I] = sz * inv;
  if (esp) esp_c[I] = q;
}

__global__ void k_coarse_prolong(const int *__restrict__ cmap, const double *__restrict__ fc,
                                 ll N, double *__restrict__ y) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int c = cmap[i];
  if (c >= 0) y[i] = fc[c];
}

__global__ void k_iota_int(int *__restrict__ a, ll n) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = (int)i;
}

__host__ __device__ inline double key_to_double(unsigned long long k) {
  const unsigned long long bits = (k >> 63) ? (k ^ 0x8000000000000000ull) : ~k;
  double d;
  memcpy(&d, &bits, sizeof d);
  return d;
}

// The coarse start of the level's 3D groups of at least cmin elements
// (active group a: positions [ast[a], ast[a] + an[a]), grp: active group of
// every position): y (the geometric start of every group) takes the
// prolonged coarse Fiedler vector on those groups.  Returns false (y
// untouched) when no group qualifies or a coarse row overflowed.
template <typename VT>
bool coarse_predict_level(const Level &lv, const int *perm, const int *grp, const double *cent,
                          const float4 *esp, ll N, int ndim, const std::vector<ll> &ast,
                          const std::vector<ll> &an, const RsbOpts &o, ll cmin, double *y,
                          SortWs &sws) {
  cudaStream_t st = ctx().stream;
  if (ndim != 3) return false;
  const int na = (int)ast.size();
  std::vector<int> sel(na, -1), gof;  // coarse group of each active group, and back
  for (int a = 0; a < na; a++)
    if (an[a] >= cmin && an[a] >= 64) sel[a] = (int)gof.size(), gof.push_back(a);
  if (gof.empty()) return false;
  const int ncg = (int)gof.size();
  // spacings and extents per group and axis
  DBuf<int> d_sel((size_t)na);
  h2d(d_sel.p, sel.data(), (size_t)na);
  DBuf<unsigned long long> mn((size_t)3 * ncg), mx((size_t)3 * ncg), hcnt((size_t)3 * ncg);
  DBuf<double> hsum((size_t)3 * ncg);
  CK(cudaMemsetAsync(mn.p, 0xFF, (size_t)3 * ncg * sizeof(unsigned long long), st));
  CK(cudaMemsetAsync(mx.p, 0, (size_t)3 * ncg * sizeof(unsigned long long), st));
  CK(cudaMemsetAsync(hcnt.p, 0, (size_t)3 * ncg * sizeof(unsigned long long), st));
  CK(cudaMemsetAsync(hsum.p, 0, (size_t)3 * ncg * sizeof(double), st));
  k_cs_stats<<<grid_for(N, 256), 256, 0, st>>>(lv.ell.p, lv.slice_off.p, lv.slice_w.p, perm, grp,
                                               d_sel.p, cent, N, N, 4u, mn.p, mx.p, hsum.p,
                                               hcnt.p);
  CK_LAUNCH();
  std::vector<unsigned long long> hmn(3 * ncg), hmx(3 * ncg), hc(3 * ncg);
  std::vector<double> hs(3 * ncg);
  d2h(hmn.data(), mn.p, hmn.size());
  d2h(hmx.data(), mx.p, hmx.size());
  d2h(hc.data(), hcnt.p, hc.size());
  d2h(hs.data(), hsum.p, hs.size());
  sync();
  std::vector<double> cmin_h(3 * ncg), ch_h(3 * ncg);
  std::vector<int> nlay(3 * ncg);
  for (int g = 0; g < ncg; g++)
    for (int d = 0; d < 3; d++) {
      const int q = 3 * g + d;
      const double lo = key_to_double(hmn[q]), hi = key_to_double(hmx[q]);
      const double ext = hi - lo;
      const double h = hc[q] ? hs[q] / (double)hc[q] : 0.0;
      int nl = (h > 0.0 && ext > 0.0) ? (int)std::llround(ext / h) + 1 : 1;
      if (nl < 1 || nl >= (2 << CS_BITS)) return false;  // too many layers for the key
      cmin_h[q] = lo;
      ch_h[q] = nl > 1 ? ext / (double)(nl - 1) : 1.0;
      nlay[q] = nl;
    }
  DBuf<double> d_cmin((size_t)3 * ncg), d_ch((size_t)3 * ncg);
  DBuf<int> d_nlay((size_t)3 * ncg);
  h2d(d_cmin.p, cmin_h.data(), cmin_h.size());
  h2d(d_ch.p, ch_h.data(), ch_h.size());
  h2d(d_nlay.p, nlay.data(), nlay.size());
  // aggregates: runs of a sort by (coarse group, cell)
  DBuf<u64> keys((size_t)N);
  DBuf<int> vals((size_t)N), flag((size_t)N), cmap((size_t)N), err(1);
  DBuf<ll> excl((size_t)N), cst_dev((size_t)ncg);
  k_cs_keys<<<grid_for(N, 256), 256, 0, st>>>(perm, grp, d_sel.p, cent, N, N, d_cmin.p, d_ch.p,
                                              d_nlay.p, keys.p, vals.p);
  CK_LAUNCH();
  seg_sort_pairs(keys, vals, N, nullptr, 1, sws);
  k_cs_flags<<<grid_for(N, 256), 256, 0, st>>>(keys.p, N, flag.p);
  CK_LAUNCH();
  const ll Nc = exclusive_scan_int_to_ll(flag.p, excl.p, N);
  if (Nc <= 0) return false;
  DBuf<ll> agg_off((size_t)Nc + 1);
  CK(cudaMemsetAsync(cmap.p, 0xFF, (size_t)N * sizeof(int), st));
  k_cs_aggs<<<grid_for(N, 256), 256, 0, st>>>(keys.p, vals.p, flag.p, excl.p, N, cmap.p,
                                              agg_off.p, cst_dev.p);
  CK_LAUNCH();
  ll M = 0;  // eligible positions: the end of the last aggregate
  for (int g = 0; g < ncg; g++) M += an[gof[g]];
  h2d(agg_off.p + Nc, &M, 1);
  std::vector<ll> cst(ncg), cn(ncg);
  d2h(cst.data(), cst_dev.p, (size_t)ncg);
  sync();
  for (int g = 0; g < ncg; g++) cn[g] = (g + 1 < ncg ? cst[g + 1] : Nc) - cst[g];
  std::vector<int> cid(ncg);
  for (int g = 0; g < ncg; g++) cid[g] = g;
  DBuf<int> cgrp((size_t)Nc), rowlen((size_t)Nc);
  fill_groups(cst, cn, cid, cgrp.p, Nc);
  // coarse level matrix
  CK(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  const unsigned cb = (unsigned)((Nc + 7) / 8);
  k_coarse_rows<false><<<cb, 256, 0, st>>>(lv.ell.p, lv.slice_off.p, lv.slice_w.p, cmap.p,
                                           agg_off.p, vals.p, Nc, rowlen.p, nullptr, nullptr,
                                           nullptr, err.p);
  CK_LAUNCH();
  Level lvc;
  const ll nslice = (Nc + 31) / 32;
  DBuf<ll> slots((size_t)nslice + 1);
  lvc.slice_w.ensure((size_t)nslice);
  lvc.slice_off.ensure((size_t)nslice + 1);
  k_slice_w<<<grid_for(nslice, 256), 256, 0, st>>>(rowlen.p, Nc, nslice, slots.p, lvc.slice_w.p);
  CK_LAUNCH();
  const ll total = exclusive_scan_ll(slots.p, lvc.slice_off.p, nslice);
  h2d(lvc.slice_off.p + nslice, &total, 1);
  lvc.ell.ensure((size_t)total + 32);
  k_coarse_rows<true><<<cb, 256, 0, st>>>(lv.ell.p, lv.slice_off.p, lv.slice_w.p, cmap.p,
                                          agg_off.p, vals.p, Nc, rowlen.p, lvc.slice_off.p,
                                          lvc.slice_w.p, lvc.ell.p, err.p);
  CK_LAUNCH();
  {
    DBuf<ll> rl64((size_t)Nc);
    lvc.nnz = exclusive_scan_int_to_ll(rowlen.p, rl64.p, Nc);
    DBuf<int> mw(1);
    CK(cudaMemsetAsync(mw.p, 0, sizeof(int), st));
    k_max_int<<<grid_for(nslice, 256), 256, 0, st>>>(lvc.slice_w.p, nslice, mw.p);
    CK_LAUNCH();
    int h_err = 0;
    d2h(&lvc.max_w, mw.p, 1);
    d2h(&h_err, err.p, 1);
    sync();
    if (h_err) return false;
  }
  // coarse centroids, spacings and the geometric start on the coarse graph
  DBuf<double> cent_c((size_t)3 * Nc), yc((size_t)Nc), fc((size_t)Nc);
  DBuf<float4> esp_c(esp ? (size_t)Nc : 1);
  DBuf<int> ident((size_t)Nc);
  k_iota_int<<<grid_for(Nc, 256), 256, 0, st>>>(ident.p, Nc);
  CK_LAUNCH();
  k_coarse_cent<<<grid_for(Nc, 256), 256, 0, st>>>(perm, cent, N, esp, agg_off.p, vals.p, Nc,
                                                   cent_c.p, esp ? esp_c.p : nullptr);
  CK_LAUNCH();
  geometric_predict_level(lvc, ident.p, cgrp.p, cent_c.p, Nc, ndim, cst, cn, Nc, yc.p, nullptr,
                          esp ? esp_c.p : nullptr);
  // one Lanczos pass on the coarse graph
  RsbOpts oc = o;
  oc.mpass = 1;
  Lanczos<VT> lzc;
  std::vector<GState> resc;
  run_fiedler_level<VT>(lzc, lvc, oc, cst, cn, Nc, fc.p, resc, yc.p);
  k_coarse_prolong<<<grid_for(N, 256), 256, 0, st>>>(cmap.p, fc.p, N, y);
  CK_LAUNCH();
  return true;
}

}  // namespace

// ----------------------------------------------------------------------------
// Public (library-internal) entry points
// ----------------------------------------------------------------------------
void build_dual_graph(const long long *d_vtx, ll nel, int nv, Graph &g, SortWs &sws) {
  cudaStream_t st = ctx().stream;
  ll ns = nel * nv;
  g.n = nel;
  g.rowptr.ensure((size_t)nel + 1);
  if (nel == 0) {
    CK(cudaMemsetAsync(g.rowptr.p, 0, sizeof(ll), st));
    g.nnz = 0;
    return;
  }
  DBuf<u64> keys((size_t)ns);
  DBuf<int> vals((size_t)ns);
  k_vid_keys<<<grid_for(ns, 256), 256, 0, st>>>(d_vtx, ns, keys.p, vals.p);
  CK_LAUNCH();
  seg_sort_pairs(keys, vals, ns, nullptr, 1, sws);
  DBuf<int> flag((size_t)ns), runid((size_t)ns), inv((size_t)ns);
  DBuf<ll> excl((size_t)ns);
  k_run_flags<<<grid_for(ns, 256), 256, 0, st>>>(keys.p, ns, flag.p);
  CK_LAUNCH();
  ll nruns = exclusive_scan_int_to_ll(flag.p, excl.p, ns);
  DBuf<ll> run_start((size_t)nruns + 1);
  k_run_bounds<<<grid_for(ns, 256), 256, 0, st>>>(flag.p, excl.p, ns, nruns, runid.p,
                                                  run_start.p);
  CK_LAUNCH();
  k_scatter_inv<<<grid_for(ns, 256), 256, 0, st>>>(vals.p, ns, inv.p);
  CK_LAUNCH();
  keys.release();
  excl.release();
  flag.release();
  DBuf<ll> rowlen((size_t)nel + 1);
  DBuf<int> maxw(1);
  CK(cudaMemsetAsync(maxw.p, 0, sizeof(int), st));
  CK(cudaMemsetAsync(rowlen.p + nel, 0, sizeof(ll), st));
  const unsigned gr_blocks = grid_for(nel, GR_WARPS);
  k_graph_rows<false><<<gr_blocks, GR_WARPS * 32, 0, st>>>(
      nv, nel, vals.p, inv.p, runid.p, run_start.p, nullptr, nullptr, nullptr, rowlen.p, maxw.p);
  CK_LAUNCH();
  g.nnz = exclusive_scan_ll(rowlen.p, g.rowptr.p, nel + 1);
  DBuf<unsigned long long> mrow(1);
  CK(cudaMemsetAsync(mrow.p, 0, sizeof(unsigned long long), st));
  k_max_ll<<<grid_for(nel, 256), 256, 0, st>>>(rowlen.p, nel, mrow.p);
  CK_LAUNCH();
  unsigned long long hm = 0;
  int hw = 0;
  d2h(&hm, mrow.p, 1);
  d2h(&hw, maxw.p, 1);
  sync();
  g.max_row = (int)hm;
  g.max_w = hw;
  g.col.ensure((size_t)g.nnz + 1);
  g.w.ensure((size_t)g.nnz + 1);
  k_graph_rows<true><<<gr_blocks, GR_WARPS * 32, 0, st>>>(
      nv, nel, vals.p, inv.p, runid.p, run_start.p, g.rowptr.p, g.col.p, g.w.p, nullptr,
      nullptr);
  CK_LAUNCH();
}

template <typename VT>
static void rsb_impl(const long long *d_vtx, const double *cent, ll N, int nv, int P,
                     const RsbOpts &o, int *d_part, int *d_seq, const StartGroups *sg) {
  cudaStream_t st = ctx().stream;
  int ndim = (nv == 8) ? 3 : 2;
  parrsb_stats &S = ctx().stats;
  Graph G;
  SortWs sws;
  {
    StageTimer tm(PARRSB_STAGE_SETUP);
    build_dual_graph(d_vtx, N, nv, G, sws);
  }
  S.nnz = G.nnz;
  if (G.max_w >= 16 || N >= (1ll << 28))
    throw ArgError{PARRSB_ERR_UNSUPPORTED,
                   "dual-graph weight >= 16 or more than 2^28 elements"};
  DBuf<int> perm((size_t)N), inv((size_t)N), grp((size_t)N), half((size_t)N),
      segpos((size_t)N), idx((size_t)N), moved((size_t)N), flag((size_t)N);
  DBuf<double> f_pos((size_t)N), f_tmp((size_t)N), y_pred;
  DBuf<float4> esp;  // element spacings (warm starts only)
  DBuf<u64> keys((size_t)N);
  DBuf<int> vals((size_t)N), perm2((size_t)N);
  std::vector<HGroup> groups;
  if (sg) {
    h2d(perm.p, sg->perm.data(), N);
    for (size_t g = 0; g < sg->start.size(); g++)
      groups.push_back({sg->start[g], sg->n[g], sg->p[g], sg->r0[g]});
  } else {
    iota_device(perm.p, N);
    groups.push_back({0, N, P, 0});
  }
  int ncuts = 0;
  for (ll pw = 1; pw < P; pw <<= 1) ncuts++;
  BisectWs bws;
  Lanczos<VT> lz;
  Level lv;
  // coarse-graph start (geometric start mode): groups of at least this many
  // elements; 0: off
  const ll coarse_min = [] {
    const char *e = getenv("PARRSB_GPU_COARSE");
    if (!(e && atoi(e) != 0)) return (ll)0;
    const char *m = getenv("PARRSB_GPU_COARSE_MIN");
    return m ? std::max<ll>(16, atoll(m)) : (ll)1 << 20;
  }();
  for (int cut = 0; cut < ncuts; cut++) {
    // active groups
    std::vector<ll> ast, an;
    std::vector<int> aid;
    std::vector<ll> all_st, all_n;
    std::vector<int> all_id, all_active_id;
    int na = 0;
    for (size_t gi = 0; gi < groups.size(); gi++) {
      const HGroup &g = groups[gi];
      all_st.push_back(g.start), all_n.push_back(g.n), all_id.push_back((int)gi);
      if (g.p > 1 && g.n > 0) {
        ast.push_back(g.start), an.push_back(g.n), aid.push_back(na);
        all_active_id.push_back(na);
        na++;
      } else {
        all_active_id.push_back(-1);
      }
    }
    if (na == 0) break;
    S.levels++;
    // ---- pre-partition (src/rsb.c:282-292)
    {
      StageTimer tm(PARRSB_STAGE_PRE);
      if (o.pre == 1 || o.pre == 2) {
        SegTable t;
        t.reserve((ll)groups.size());
        std::vector<int> hp, hr;
        for (auto &g : groups) hp.push_back(g.p > 1 ? g.p : 0), hr.push_back(g.r0);
        t.count = (ll)groups.size();
        h2d(t.start.p, all_st.data(), groups.size());
        h2d(t.n.p, all_n.data(), groups.size());
        h2d(t.p.p, hp.data(), groups.size());
        h2d(t.r0.p, hr.data(), groups.size());
        bisect_segments(o.pre == 1 ? BISECT_RCB : BISECT_RIB, perm, t, cent, N, ndim, true,
                        nullptr, bws);
      } else {
        fill_groups(all_st, all_n, all_active_id, grp.p, N);
        fill_groups(all_st, all_n, all_id, segpos.p, N);
        k_keys_elem_id<<<grid_for(N, 256), 256, 0, st>>>(perm.p, grp.p, N, keys.p, vals.p);
        CK_LAUNCH();
        seg_sort_pairs(keys, vals, N, segpos.p, (ll)groups.size(), sws);
        k_gather_int<<<grid_for(N, 256), 256, 0, st>>>(vals.p, perm.p, N, perm2.p);
        CK_LAUNCH();
        std::swap(perm, perm2);
      }
    }
    // ---- level graph
    {
      StageTimer tm(PARRSB_STAGE_RESTRICT);
      fill_groups(all_st, all_n, all_active_id, grp.p, N);
      fill_groups(all_st, all_n, all_id, segpos.p, N);
      k_inv_perm<<<grid_for(N, 256), 256, 0, st>>>(perm.p, N, inv.p);
      CK_LAUNCH();
      build_level(G, perm.p, inv.p, grp.p, N, lv);
    }
    // ---- learned warm start: predictions for the groups of this level
    // that are large enough (the judge in Lanczos::choose_start decides)
    // (the network where groups have at least warm_min elements; with
    // start 2 the geometric guess elsewhere)
    const double *y_warm = nullptr;
    if ((o.warm || o.start == 2) && nv == 8) {
      ll biggest = 0;
      for (int g = 0; g < na; g++) biggest = std::max(biggest, an[g]);
      const bool use_net = o.warm && biggest >= std::max<ll>(o.warm_min, 2);
      if (use_net || o.start == 2) {
        if (use_net && !warm_net_ready())
          throw ArgError{PARRSB_ERR_ARGS, "warm start requested but no network installed"};
        cudaEvent_t w0, w1;
        CK(cudaEventCreate(&w0));
        CK(cudaEventCreate(&w1));
        CK(cudaEventRecord(w0, st));
        y_pred.ensure((size_t)N);
        if (!esp.p) {  // once per call: element spacings from the dual graph
          esp.ensure((size_t)N);
          element_spacings(G, cent, N, ndim, esp.p);
        }
        if (use_net)
          warm_predict_level(lv, perm.p, grp.p, cent, N, ndim, ast, an, N, y_pred.p, nullptr,
                             esp.p);
        else  // start 2: the geometric guess
          geometric_predict_level(lv, perm.p, grp.p, cent, N, ndim, ast, an, N, y_pred.p,
                                  nullptr, esp.p);
        // PARRSB_GPU_COARSE=1: groups of at least PARRSB_GPU_COARSE_MIN
        // elements (default 2^20) start from their coarse graph's vector
        if (!use_net && coarse_min > 0)
          coarse_predict_level<VT>(lv, perm.p, grp.p, cent, esp.p, N, ndim, ast, an, o,
                                   coarse_min, y_pred.p, sws);
        CK(cudaEventRecord(w1, st));
        CK(cudaEventSynchronize(w1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, w0, w1));
        S.warm_ms += ms;
        cudaEventDestroy(w0);
        cudaEventDestroy(w1);
        y_warm = y_pred.p;
      }
    }
    // ---- Fiedler vectors (src/rsb.c:300-302)
    std::vector<GState> res;
    if (o.batched) {
      run_fiedler_level<VT>(lz, lv, o, ast, an, N, f_pos.p, res, y_warm);
    } else {
      // plain path: every group of the level solved by its own launches
      RsbOpts o1 = o;
      o1.use_graphs = 0;
      for (int g = 0; g < na; g++) {
        std::vector<GState> r1;
        std::vector<ll> s1 = {ast[g]}, n1 = {an[g]};
        run_fiedler_level<VT>(lz, lv, o1, s1, n1, N, f_tmp.p, r1, y_warm);
        CK(cudaMemcpyAsync(f_pos.p + ast[g], f_tmp.p + ast[g], an[g] * sizeof(double),
                           cudaMemcpyDeviceToDevice, st));
        res.push_back(r1[0]);
      }
    }
    ll rows = 0;
    for (int g = 0; g < na; g++) {
      S.level_steps[std::min(cut, 15)] += res[g].total_iters;
      S.lanczos_iters += res[g].total_iters;
      S.lanczos_row_iters += res[g].total_iters * res[g].n;
      rows += res[g].n;
      if (res[g].total_iters == (ll)res[g].miter * o.mpass) S.unconverged++;
      if (res[g].resid > S.max_fiedler_resid) S.max_fiedler_resid = res[g].resid;
    }
    // algorithmic bytes of the SpMV launches of this level: per row and
    // step 4 B per stored nonzero plus the row's own p read and w write
    {
      long long row_iters = 0;
      for (int g = 0; g < na; g++) row_iters += res[g].total_iters * res[g].n;
      double per_row = rows > 0 ? 4.0 * (double)lv.nnz / (double)rows + 2.0 * sizeof(VT) : 0.0;
      S.spmv_bytes += (long long)(per_row * (double)row_iters);
    }
    // ---- sort by Fiedler value (src/rsb.c:307-309)
    {
      StageTimer tm(PARRSB_STAGE_SORT);
      k_fied_keys<<<grid_for(N, 256), 256, 0, st>>>(f_pos.p, grp.p, N, keys.p, vals.p);
      CK_LAUNCH();
      seg_sort_pairs(keys, vals, N, segpos.p, (ll)groups.size(), sws);
      k_gather_perm<<<grid_for(N, 256), 256, 0, st>>>(vals.p, perm.p, f_pos.p, N, perm2.p,
                                                      f_tmp.p);
      CK_LAUNCH();
      std::swap(perm, perm2);
      std::swap(f_pos, f_tmp);
    }
    // ---- split into halves (bin = rank >= ceil(p/2))
    std::vector<ll> Ls(groups.size(), 0);
    std::vector<ll> hst, hn;
    std::vector<int> hid;
    for (size_t gi = 0; gi < groups.size(); gi++) {
      const HGroup &g = groups[gi];
      if (all_active_id[gi] < 0) continue;
      Ls[gi] = lower_count(g.n, g.p);
      int a = all_active_id[gi];
      hst.push_back(g.start), hn.push_back(Ls[gi]), hid.push_back(2 * a);
      hst.push_back(g.start + Ls[gi]), hn.push_back(g.n - Ls[gi]), hid.push_back(2 * a + 1);
    }
    CK(cudaMemsetAsync(half.p, 0xff, (size_t)N * sizeof(int), st));
    fill_groups(hst, hn, hid, half.p, N);
    // ---- connected components of each half (src/rsb.c:319-327)
    if (o.find_comps) {
      StageTimer tm(PARRSB_STAGE_COMPONENTS);
      std::vector<ll> hs_by_id(2 * na, 0);
      for (size_t q = 0; q < hid.size(); q++) hs_by_id[hid[q]] = hst[q];
      std::vector<int> hc = count_components_level(lv, half.p, N, hs_by_id);
      for (int v : hc) S.max_components = std::max(S.max_components, v);
    }
    // ---- balance (src/rsb.c:118-229)
    {
      StageTimer tm(PARRSB_STAGE_BALANCE);
      std::vector<int> mode(na, 0), send_half(2 * na, -1);
      std::vector<ll> sendc(2 * na, 0);
      std::vector<double> mul(2 * na, 0.0);
      bool any = false;
      for (size_t gi = 0; gi < groups.size(); gi++) {
        int a = all_active_id[gi];
        if (a < 0) continue;
        const HGroup &g = groups[gi];
        int h = (g.p + 1) / 2;
        ll ne_ = g.n / g.p, nrem = g.n - ne_ * g.p;
        ll expA = ne_ * h + nrem / 2 + (nrem % 2);
        ll expB = ne_ * (g.p - h) + nrem / 2;
        ll L = Ls[gi];
        ll sA = std::max<ll>(0, L - expA), sB = std::max<ll>(0, (g.n - L) - expB);
        if (sA > 0) {
          mode[a] = 1, send_half[2 * a] = 2 * a + 1, sendc[2 * a] = sA, mul[2 * a] = -1.0;
          any = true;
        } else if (sB > 0) {
          mode[a] = 2, send_half[2 * a + 1] = 2 * a, sendc[2 * a + 1] = sB, mul[2 * a + 1] = 1.0;
          any = true;
        }
      }
      if (any) {
        DBuf<int> d_send_half((size_t)2 * na), cnt((size_t)2 * na);
        h2d(d_send_half.p, send_half.data(), 2 * na);
        CK(cudaMemsetAsync(cnt.p, 0, (size_t)2 * na * sizeof(int), st));
        k_bd_flag<<<grid_for(N, 256), 256, 0, st>>>(lv.ell.p, lv.slice_off.p, lv.slice_w.p,
                                                    half.p, d_send_half.p, N, flag.p, cnt.p);
        CK_LAUNCH();
        std::vector<int> hc(2 * na);
        d2h(hc.data(), cnt.p, 2 * na);
        sync();
        // groups without enough boundary elements keep their split
        for (int a = 0; a < na; a++) {
          int sh = mode[a] == 1 ? 2 * a : (mode[a] == 2 ? 2 * a + 1 : -1);
          if (sh >= 0 && hc[sh] < sendc[sh]) mode[a] = 0, sendc[sh] = 0;
        }
        bool still = false;
        for (int a = 0; a < na; a++) still = still || mode[a] != 0;
        if (still) {
          // compact flagged rows (only halves that still send)
          for (int a = 0; a < na; a++)
            if (mode[a] == 0) send_half[2 * a] = send_half[2 * a + 1] = -1;
          h2d(d_send_half.p, send_half.data(), 2 * na);
          CK(cudaMemsetAsync(cnt.p, 0, (size_t)2 * na * sizeof(int), st));
          k_bd_flag<<<grid_for(N, 256), 256, 0, st>>>(lv.ell.p, lv.slice_off.p,
                                                      lv.slice_w.p, half.p, d_send_half.p, N,
                                                      flag.p, cnt.p);
          CK_LAUNCH();
          d2h(hc.data(), cnt.p, 2 * na);
          DBuf<ll> excl((size_t)N + 1);
          ll nb = exclusive_scan_int_to_ll(flag.p, excl.p, N);
          DBuf<u64> bk((size_t)nb + 1);
          DBuf<int> bv((size_t)nb + 1), bseg((size_t)N);
          DBuf<double> dmul((size_t)2 * na);
          h2d(dmul.p, mul.data(), 2 * na);
          k_bd_keys<<<grid_for(N, 256), 256, 0, st>>>(flag.p, excl.p, f_pos.p, half.p, dmul.p,
                                                      N, bk.p, bv.p, bseg.p);
          CK_LAUNCH();
          seg_sort_pairs(bk, bv, nb, bseg.p, 2 * na, sws);
          std::vector<ll> off(2 * na, 0);
          ll acc = 0;
          for (int h = 0; h < 2 * na; h++) off[h] = acc, acc += hc[h];
          DBuf<ll> doff((size_t)2 * na), dsend((size_t)2 * na);
          h2d(doff.p, off.data(), 2 * na);
          h2d(dsend.p, sendc.data(), 2 * na);
          CK(cudaMemsetAsync(moved.p, 0, (size_t)N * sizeof(int), st));
          k_bd_moved<<<grid_for(nb, 256), 256, 0, st>>>(bv.p, nb, doff.p, dsend.p, half.p,
                                                        moved.p);
          CK_LAUNCH();
          // segment ids in position order: an active group takes two ids
          // (kept / re-sorted part), a frozen group one
          std::vector<int> base_active(na, 0), fz_id;
          std::vector<ll> fz_st, fz_n;
          int nid = 0;
          for (size_t gi = 0; gi < groups.size(); gi++) {
            int a = all_active_id[gi];
            fz_st.push_back(groups[gi].start), fz_n.push_back(groups[gi].n);
            fz_id.push_back(nid);
            if (a >= 0) {
              base_active[a] = nid;
              nid += 2;
            } else {
              nid += 1;
            }
          }
          fill_groups(fz_st, fz_n, fz_id, segpos.p, N);
          DBuf<int> dmode(na), dbase(na), seg_of_val((size_t)N);
          h2d(dmode.p, mode.data(), na);
          h2d(dbase.p, base_active.data(), na);
          k_rebal_keys<<<grid_for(N, 256), 256, 0, st>>>(half.p, moved.p, dmode.p, dbase.p,
                                                         segpos.p, f_pos.p, N, keys.p, vals.p,
                                                         seg_of_val.p);
          CK_LAUNCH();
          seg_sort_pairs(keys, vals, N, seg_of_val.p, nid, sws);
          k_gather_perm<<<grid_for(N, 256), 256, 0, st>>>(vals.p, perm.p, f_pos.p, N, perm2.p,
                                                          f_tmp.p);
          CK_LAUNCH();
          std::swap(perm, perm2);
          std::swap(f_pos, f_tmp);
          for (size_t gi = 0; gi < groups.size(); gi++) {
            int a = all_active_id[gi];
            if (a < 0) continue;
            if (mode[a] == 1) Ls[gi] -= sendc[2 * a];
            if (mode[a] == 2) Ls[gi] += sendc[2 * a + 1];
          }
          sync();
        }
      }
    }
    // ---- next level groups
    std::vector<HGroup> next;
    for (size_t gi = 0; gi < groups.size(); gi++) {
      const HGroup &g = groups[gi];
      if (all_active_id[gi] < 0) {
        next.push_back(g);
        continue;
      }
      int h = (g.p + 1) / 2;
      ll L = Ls[gi];
      next.push_back({g.start, L, h, g.r0});
      next.push_back({g.start + L, g.n - L, g.p - h, g.r0 + h});
    }
    groups.swap(next);
  }
  // part[perm[i]] = r0 of the group holding position i
  std::vector<ll> st_, n_;
  std::vector<int> r_;
  for (auto &g : groups) st_.push_back(g.start), n_.push_back(g.n), r_.push_back(g.r0);
  fill_groups(st_, n_, r_, grp.p, N);
  k_part_scatter<<<grid_for(N, 256), 256, 0, st>>>(perm.p, grp.p, N, d_part);
  CK_LAUNCH();
  if (d_seq) {
    std::vector<int> pos_;
    for (auto &g : groups) pos_.push_back((int)g.start);
    fill_groups(st_, n_, pos_, segpos.p, N);
    k_seq_rel<<<grid_for(N, 256), 256, 0, st>>>(perm.p, segpos.p, N, d_seq);
    CK_LAUNCH();
  }
}

__global__ void k_group_keys(const int *__restrict__ group_of, ll N, u64 *__restrict__ keys,
                             int *__restrict__ vals, int *__restrict__ cnt) {
  ll e = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= N) return;
  int g = group_of[e];
  keys[e] = (u64)(unsigned)g;
  vals[e] = (int)e;
  atomicAdd(&cnt[g], 1);
}

__global__ void k_scatter_f(const int *__restrict__ perm, const double *__restrict__ f_pos,
                            ll N, double *__restrict__ f) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) f[perm[i]] = f_pos[i];
}

template <typename VT>
static void fiedler_groups_impl(const long long *d_vtx, ll N, int nv, const int *d_group_of,
                                int ngroups, const RsbOpts &o, double *d_f, long long *iters,
                                double *resid) {
  cudaStream_t st = ctx().stream;
  SortWs sws;
  Graph G;
  {
    StageTimer tm(PARRSB_STAGE_SETUP);
    build_dual_graph(d_vtx, N, nv, G, sws);
  }
  if (G.max_w >= 16 || N >= (1ll << 28))
    throw ArgError{PARRSB_ERR_UNSUPPORTED, "dual-graph weight >= 16 or more than 2^28 elements"};
  // order elements by group (stable: element order inside a group)
  DBuf<u64> keys((size_t)N);
  DBuf<int> perm((size_t)N), cnt((size_t)ngroups), inv((size_t)N), grp((size_t)N);
  CK(cudaMemsetAsync(cnt.p, 0, (size_t)ngroups * sizeof(int), st));
  k_group_keys<<<grid_for(N, 256), 256, 0, st>>>(d_group_of, N, keys.p, perm.p, cnt.p);
  CK_LAUNCH();
  seg_sort_pairs(keys, perm, N, nullptr, 1, sws);
  std::vector<int> hc(ngroups);
  d2h(hc.data(), cnt.p, ngroups);
  sync();
  std::vector<ll> ast, an, all_st, all_n;
  std::vector<int> act_id, gidx;
  ll pos = 0;
  for (int g = 0; g < ngroups; g++) {
    all_st.push_back(pos), all_n.push_back(hc[g]);
    if (hc[g] >= 2) {
      act_id.push_back((int)ast.size());
      gidx.push_back(g);
      ast.push_back(pos), an.push_back(hc[g]);
    } else {
      act_id.push_back(-1);
    }
    pos += hc[g];
  }
  fill_groups(all_st, all_n, act_id, grp.p, N);
  k_inv_perm<<<grid_for(N, 256), 256, 0, st>>>(perm.p, N, inv.p);
  CK_LAUNCH();
  Level lv;
  {
    StageTimer tm(PARRSB_STAGE_RESTRICT);
    build_level(G, perm.p, inv.p, grp.p, N, lv);
  }
  DBuf<double> f_pos((size_t)N);
  CK(cudaMemsetAsync(f_pos.p, 0, (size_t)N * sizeof(double), st));
  for (int g = 0; g < ngroups; g++) iters[g] = 0, resid[g] = 0.0;
  Lanczos<VT> lz;
  auto collect = [&](const std::vector<GState> &res, const std::vector<int> &which) {
    for (size_t q = 0; q < res.size(); q++) {
      int g = gidx[which[q]];
      iters[g] = res[q].total_iters;
      resid[g] = res[q].resid;
      ctx().stats.lanczos_iters += res[q].total_iters;
      ctx().stats.lanczos_row_iters += res[q].total_iters * res[q].n;
      if (res[q].resid > ctx().stats.max_fiedler_resid)
        ctx().stats.max_fiedler_resid = res[q].resid;
    }
  };
  if (ast.empty()) {
  } else if (o.batched) {
    std::vector<GState> res;
    run_fiedler_level<VT>(lz, lv, o, ast, an, N, f_pos.p, res);
    std::vector<int> which(ast.size());
    for (size_t q = 0; q < which.size(); q++) which[q] = (int)q;
    collect(res, which);
  } else {
    // one group at a time: every kernel launch covers one subgraph
    RsbOpts o1 = o;
    o1.use_graphs = 0;
    DBuf<double> f_one((size_t)N);
    for (size_t q = 0; q < ast.size(); q++) {
      std::vector<GState> res;
      std::vector<ll> s1 = {ast[q]}, n1 = {an[q]};
      run_fiedler_level<VT>(lz, lv, o1, s1, n1, N, f_one.p, res);
      CK(cudaMemcpyAsync(f_pos.p + ast[q], f_one.p + ast[q], an[q] * sizeof(double),
                         cudaMemcpyDeviceToDevice, st));
      collect(res, std::vector<int>{(int)q});
    }
  }
  k_scatter_f<<<grid_for(N, 256), 256, 0, st>>>(perm.p, f_pos.p, N, d_f);
  CK_LAUNCH();
  sync();
}

void fiedler_groups_device(const long long *d_vtx, ll N, int nv, const int *d_group_of,
                           int ngroups, const RsbOpts &o, double *d_f, long long *iters,
                           double *resid) {
  if (o.miter > MAX_MITER || o.miter < 1)
    throw ArgError{PARRSB_ERR_UNSUPPORTED, "rsb_max_iter outside [1, 120]"};
  if (o.fp32)
    fiedler_groups_impl<float>(d_vtx, N, nv, d_group_of, ngroups, o, d_f, iters, resid);
  else
    fiedler_groups_impl<double>(d_vtx, N, nv, d_group_of, ngroups, o, d_f, iters, resid);
}

// keys for ordering elements by group; elements without a group (< 0) go last
__global__ void k_group_keys_opt(const int *__restrict__ group_of, ll N, int ngroups,
                                 u64 *__restrict__ keys, int *__restrict__ vals,
                                 int *__restrict__ cnt) {
  ll e = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= N) return;
  int g = group_of[e];
  keys[e] = g >= 0 ? (u64)(unsigned)g : (u64)(unsigned)ngroups;
  vals[e] = (int)e;
  if (g >= 0) atomicAdd(&cnt[g], 1);
}

__global__ void k_iota(int *__restrict__ a, ll N) {
  ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) a[i] = (int)i;
}

void iota_device(int *d, ll N) {
  if (N <= 0) return;
  k_iota<<<grid_for(N, 256), 256, 0, ctx().stream>>>(d, N);
  CK_LAUNCH();
}

void build_group_level(const long long *d_vtx, ll N, int nv, const int *d_group_of,
                       int ngroups, GroupLevel &out) {
  cudaStream_t st = ctx().stream;
  out.N = N;
  out.gstart.assign(ngroups, 0);
  out.gn.assign(ngroups, 0);
  if (N == 0) return;
  SortWs sws;
  Graph G;
  build_dual_graph(d_vtx, N, nv, G, sws);
  if (G.max_w >= 16 || N >= (1ll << 28))
    throw ArgError{PARRSB_ERR_UNSUPPORTED, "dual-graph weight >= 16 or more than 2^28 elements"};
  DBuf<u64> keys((size_t)N);
  DBuf<int> cnt((size_t)ngroups), inv((size_t)N);
  out.perm.ensure((size_t)N), out.grp.ensure((size_t)N);
  CK(cudaMemsetAsync(cnt.p, 0, (size_t)ngroups * sizeof(int), st));
  k_group_keys_opt<<<grid_for(N, 256), 256, 0, st>>>(d_group_of, N, ngroups, keys.p, out.perm.p,
                                                     cnt.p);
  CK_LAUNCH();
  seg_sort_pairs(keys, out.perm, N, nullptr, 1, sws);
  std::vector<int> hc(ngroups);
  d2h(hc.data(), cnt.p, ngroups);
  sync();
  std::vector<ll> st_, n_;
  std::vector<int> id_;
  ll pos = 0;
  for (int g = 0; g < ngroups; g++) {
    out.gstart[g] = pos, out.gn[g] = hc[g];
    st_.push_back(pos), n_.push_back(hc[g]), id_.push_back(g);
    pos += hc[g];
  }
  CK(cudaMemsetAsync(out.grp.p, 0xff, (size_t)N * sizeof(int), st));  // no group: -1
  fill_groups(st_, n_, id_, out.grp.p, N);
  k_inv_perm<<<grid_for(N, 256), 256, 0, st>>>(out.perm.p, N, inv.p);
  CK_LAUNCH();
  build_level(G, out.perm.p, inv.p, out.grp.p, N, out.lv);
}

void components_device(const long long *d_vtx, ll N, int nv, const int *d_group_of, int ngroups,
                       int *counts) {
  for (int g = 0; g < ngroups; g++) counts[g] = 0;
  if (N == 0) return;
  GroupLevel gl;
  build_group_level(d_vtx, N, nv, d_group_of, ngroups, gl);
  std::vector<ll> hstart(ngroups, 0);
  for (int g = 0; g < ngroups; g++) hstart[g] = gl.gn[g] ? gl.gstart[g] : 0;  // any valid row
  std::vector<int> c = count_components_level(gl.lv, gl.grp.p, N, hstart);
  for (int g = 0; g < ngroups; g++) counts[g] = gl.gn[g] ? c[g] : 0;
}

void part_component_labels(const long long *d_vtx, ll N, int nv, const int *d_part, int nparts,
                           GroupLevel &gl, DBuf<int> &labels) {
  build_group_level(d_vtx, N, nv, d_part, nparts, gl);
  std::vector<ll> hstart(nparts, 0);
  for (int g = 0; g < nparts; g++) hstart[g] = gl.gn[g] ? gl.gstart[g] : 0;
  count_components_level(gl.lv, gl.grp.p, N, hstart, &labels);
}

void dual_graph_device(const long long *d_vtx, ll N, int nv, std::vector<ll> &rowptr,
                       std::vector<int> &col, std::vector<unsigned char> &w) {
  SortWs sws;
  Graph G;
  build_dual_graph(d_vtx, N, nv, G, sws);
  rowptr.assign((size_t)N + 1, 0);
  col.assign((size_t)G.nnz, 0);
  w.assign((size_t)G.nnz, 0);
  d2h(rowptr.data(), G.rowptr.p, (size_t)N + 1);
  d2h(col.data(), G.col.p, (size_t)G.nnz);
  d2h(w.data(), G.w.p, (size_t)G.nnz);
  sync();
}

void rsb_device(const long long *d_vtx, const double *cent, ll N, int nv, int P,
                const RsbOpts &o, int *d_part, int *d_seq, const StartGroups *sg) {
  if (o.miter > MAX_MITER || o.miter < 1)
    throw ArgError{PARRSB_ERR_UNSUPPORTED, "rsb_max_iter outside [1, 120]"};
  if (o.fp32)
    rsb_impl<float>(d_vtx, cent, N, nv, P, o, d_part, d_seq, sg);
  else
    rsb_impl<double>(d_vtx, cent, N, nv, P, o, d_part, d_seq, sg);
}

}  // namespace prsb
