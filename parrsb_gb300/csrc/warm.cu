// warm.cu -- learned warm start for the Fiedler vectors of an RSB level.
//
// The reference starts every Lanczos run from a step vector in the current
// element order (src/fiedler.c:574-578: initv[i] = i + 1, plus 1000 n on the
// first half).  This file predicts a start vector instead: a three-layer
// message-passing network over the level's own sliced-ELL graph (the
// restricted dual graph Lanczos multiplies by), with inputs per element
//   x~  = R^T (c - mu) / s   the centroid in the group's principal frame
//                            (R: eigenvectors of the group's centroid
//                            scatter matrix, largest first; s = sqrt(3
//                            lambda_1 / n), so the longest axis spans about
//                            [-1, 1])
//   deg = sum_j w_ij / 56    the element's weighted degree in the group
// and per layer
//   h_l = relu([h_{l-1} | a_l] W_l + b_l),  a_l,i = sum_j w_ij h_{l-1},j /
//                                                    sum_j w_ij
// (BF16 activations and weights, FP32 accumulation on the tensor cores with
// mma.sync m16n8k16), then y = g + h_3 . wo + bo: the head corrects the
// geometric guess g = -sin(pi x~_1 / 2), which is also an input.  The
// training step (forward,
// sign-invariant cosine loss against the Fiedler vectors of the plain
// method, backward, Adam) runs on the same kernels; its C entry points are
// at the end of this file.
#include <cuda_bf16.h>

#include <mutex>

#include "warm.cuh"

namespace prsb {

typedef __nv_bfloat16 bf16;

namespace {

constexpr int MP_ROWS = 64;        // rows per tile of the layer kernels (4 warps x 16)
constexpr int MP_THREADS = 128;
constexpr int MP_FTILE = 16384;    // rows per tile of the group-frame reductions
constexpr int MP_FRAME = 16;       // doubles per group frame
constexpr double MP_DEG_SCALE = 1.0 / 56.0;  // hex: 6 x 4 + 12 x 2 + 8 x 1

// Block-wide sum in a fixed order (shuffle tree per warp, then the warps in
// order); the result is valid in thread 0.
__device__ __forceinline__ double mp_block_sum(double v, double *sh) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += sh[w];
  return s;  // valid in thread 0
}

// ---------------------------------------------------------------------------
// Parameters on the device
// ---------------------------------------------------------------------------
// Wf[l]: [64][K_l] (k contiguous, the B operand of the forward MMA);
// Wb[l]: [K_l][64] (n contiguous, the B operand of dA = dZ W^T); p: the
// FP32 flat vector (biases, head).
struct NetDev {
  bf16 *Wf[3] = {nullptr, nullptr, nullptr};
  bf16 *Wb[3] = {nullptr, nullptr, nullptr};
  float *p = nullptr;
};

__host__ __device__ constexpr int layer_k(int l) { return l == 0 ? MP_K1 : MP_K2; }
__host__ __device__ constexpr int layer_w_off(int l) {
  return l == 0 ? MP_OFF_W1 : (l == 1 ? MP_OFF_W2 : MP_OFF_W3);
}
__host__ __device__ constexpr int layer_b_off(int l) {
  return l == 0 ? MP_OFF_B1 : (l == 1 ? MP_OFF_B2 : MP_OFF_B3);
}

__global__ void k_mp_pack(const float *__restrict__ p, bf16 *__restrict__ wf0,
                          bf16 *__restrict__ wf1, bf16 *__restrict__ wf2,
                          bf16 *__restrict__ wb0, bf16 *__restrict__ wb1,
                          bf16 *__restrict__ wb2) {
  const int l = blockIdx.y;
  const int K = layer_k(l);
  bf16 *wf = l == 0 ? wf0 : (l == 1 ? wf1 : wf2);
  bf16 *wb = l == 0 ? wb0 : (l == 1 ? wb1 : wb2);
  const float *W = p + layer_w_off(l);
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < K * MP_HID;
       q += gridDim.x * blockDim.x) {
    const int k = q / MP_HID, n = q % MP_HID;
    const bf16 v = __float2bfloat16_rn(W[q]);
    wf[n * K + k] = v;
    wb[k * MP_HID + n] = v;
  }
}

// Packed copy of the parameters for a flat FP32 vector already on the device
// (training: repacked after every optimiser step).
struct PackedNet {
  DBuf<bf16> wf[3], wb[3];
  NetDev dev(float *p) {
    NetDev d;
    for (int l = 0; l < 3; l++) d.Wf[l] = wf[l].p, d.Wb[l] = wb[l].p;
    d.p = p;
    return d;
  }
  void pack(float *d_params) {
    for (int l = 0; l < 3; l++) {
      wf[l].ensure((size_t)layer_k(l) * MP_HID);
      wb[l].ensure((size_t)layer_k(l) * MP_HID);
    }
    k_mp_pack<<<dim3(8, 3), 256, 0, ctx().stream>>>(d_params, wf[0].p, wf[1].p, wf[2].p,
                                                    wb[0].p, wb[1].p, wb[2].p);
    CK_LAUNCH();
  }
};

// Installed network, one per device.  Its buffers come from cudaMalloc (not
// the stream-ordered pool) because they outlive every call.
struct InstalledNet {
  bool ready = false;
  float *p = nullptr;
  bf16 *wf[3] = {nullptr, nullptr, nullptr}, *wb[3] = {nullptr, nullptr, nullptr};
};
InstalledNet g_net[MAX_DEVICES];
std::mutex g_net_mu;

// ---------------------------------------------------------------------------
// Group frames: centroid mean, principal axes and scale per group
// ---------------------------------------------------------------------------
struct FTile {
  ll b, e;
  int g;
};

// Element spacing per axis.  The graph Laplacian sees element counts, not
// lengths: a box of 256 x 256 x 128 elements on the unit cube has its
// Fiedler vector along x or y although z is as long.  So centroids are
// measured in element spacings: per group and axis a, h_a^2 = mean over the
// face neighbour pairs (weight wface) of (c_i,a - c_j,a)^2, and the frame
// is built from c_a / h_a.  Per tile: the three sums and the pair count.
__global__ void __launch_bounds__(256)
k_mp_spacing(const FTile *__restrict__ tiles, const int *__restrict__ perm,
             const double *__restrict__ cent, ll nel, const unsigned *__restrict__ ell,
             const ll *__restrict__ slice_off, const int *__restrict__ slice_w, unsigned wface,
             double *__restrict__ part) {
  const FTile t = tiles[blockIdx.x];
  double s[4] = {0, 0, 0, 0};
  for (ll i = t.b + threadIdx.x; i < t.e; i += blockDim.x) {
    const int e = perm[i];
    const ll sl = i >> 5;
    const unsigned *ep = ell + slice_off[sl] + (i & 31);
    const int wd = slice_w[sl];
    for (int k = 0; k < wd; k++) {
      const unsigned x = ep[(ll)k * 32];
      if ((x >> 28) != wface) continue;
      const int f = perm[x & 0x0FFFFFFFu];
      for (int a = 0; a < 3; a++) {
        const double d = cent[(ll)a * nel + e] - cent[(ll)a * nel + f];
        s[a] += d * d;
      }
      s[3] += 1.0;
    }
  }
  __shared__ double sh[32];
  for (int q = 0; q < 4; q++) {
    const double v = mp_block_sum(s[q], sh);
    if (threadIdx.x == 0) part[(ll)blockIdx.x * 4 + q] = v;
    __syncthreads();
  }
}

// The same sums from per-element values (esp[e] = the element's own sums
// over all its face neighbours, computed once per call from the dual graph):
// a coalesced pass per level instead of the neighbour gathers.
__global__ void __launch_bounds__(256)
k_mp_spacing_elem(const FTile *__restrict__ tiles, const int *__restrict__ perm,
                  const float4 *__restrict__ esp, double *__restrict__ part) {
  const FTile t = tiles[blockIdx.x];
  double s[4] = {0, 0, 0, 0};
  for (ll i = t.b + threadIdx.x; i < t.e; i += blockDim.x) {
    const float4 v = esp[perm[i]];
    s[0] += v.x, s[1] += v.y, s[2] += v.z, s[3] += v.w;
  }
  __shared__ double sh[32];
  for (int q = 0; q < 4; q++) {
    const double v = mp_block_sum(s[q], sh);
    if (threadIdx.x == 0) part[(ll)blockIdx.x * 4 + q] = v;
    __syncthreads();
  }
}

__global__ void k_elem_spacing(const ll *__restrict__ rowptr, const int *__restrict__ col,
                               const unsigned char *__restrict__ w, const double *__restrict__ cent,
                               ll nel, unsigned wface, float4 *__restrict__ esp) {
  const ll e = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nel) return;
  double s[4] = {0, 0, 0, 0};
  for (ll q = rowptr[e]; q < rowptr[e + 1]; q++) {
    if (w[q] != wface) continue;
    const int f = col[q];
    for (int a = 0; a < 3; a++) {
      const double d = cent[(ll)a * nel + e] - cent[(ll)a * nel + f];
      s[a] += d * d;
    }
    s[3] += 1.0;
  }
  esp[e] = make_float4((float)s[0], (float)s[1], (float)s[2], (float)s[3]);
}

// sa[g][a] = 1 / h_a (1 where an axis has no spacing: 2D z, no pairs)
__global__ void k_mp_scales(const double *__restrict__ part, const int *__restrict__ tile0,
                            const int *__restrict__ ntile, int ngroups,
                            double *__restrict__ sa) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngroups) return;
  double s[4] = {0, 0, 0, 0};
  for (int t = tile0[g]; t < tile0[g] + ntile[g]; t++)
    for (int q = 0; q < 4; q++) s[q] += part[(ll)t * 4 + q];
  for (int a = 0; a < 3; a++) {
    const double h2 = s[3] > 0.0 ? s[a] / s[3] : 0.0;
    sa[(ll)g * 3 + a] = h2 > 0.0 ? 1.0 / sqrt(h2) : 1.0;
  }
}

// per tile: sum of (c - o), sum of (c - o)(c - o)^T (6) about the group's
// origin o = centroid of its first position (numerically safe raw moments),
// coordinates in element spacings; and the tile's bounding box of the raw
// centroids (min x y z, max x y z), from which RCB picks its cut axis.
// Each thread accumulates its elements' terms in FP32 (c - o in FP64 first,
// so any coordinate range is safe; 64 elements per thread), the block sums
// its threads in FP64: FP64 arithmetic per element, at 1/64 of the FP32
// rate, bounded this kernel.  The box is kept on order-preserving integer
// keys of the doubles (the integer pipe).
__device__ __forceinline__ unsigned long long mp_okey(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double mp_okey_inv(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}

__global__ void __launch_bounds__(256)
k_mp_moments(const FTile *__restrict__ tiles, const ll *__restrict__ gstart,
             const int *__restrict__ perm, const double *__restrict__ cent, ll nel,
             const double *__restrict__ sa, double *__restrict__ part,
             double *__restrict__ box) {
  const FTile t = tiles[blockIdx.x];
  const int e0 = perm[gstart[t.g]];
  const double o[3] = {cent[e0], cent[nel + e0], cent[2 * nel + e0]};
  const double *k = sa + (ll)t.g * 3;
  const float kf[3] = {(float)k[0], (float)k[1], (float)k[2]};
  float s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  unsigned long long lo[3], hi[3];
  for (int a = 0; a < 3; a++) lo[a] = hi[a] = mp_okey(o[a]);
  for (ll i = t.b + threadIdx.x; i < t.e; i += blockDim.x) {
    const int e = perm[i];
    const double c[3] = {cent[e], cent[nel + e], cent[2 * nel + e]};
    const float x = (float)(c[0] - o[0]) * kf[0], y = (float)(c[1] - o[1]) * kf[1],
                z = (float)(c[2] - o[2]) * kf[2];
    s[0] += x, s[1] += y, s[2] += z;
    s[3] = fmaf(x, x, s[3]), s[4] = fmaf(y, y, s[4]), s[5] = fmaf(z, z, s[5]);
    s[6] = fmaf(x, y, s[6]), s[7] = fmaf(x, z, s[7]), s[8] = fmaf(y, z, s[8]);
    for (int a = 0; a < 3; a++) {
      const unsigned long long q = mp_okey(c[a]);
      lo[a] = min(lo[a], q), hi[a] = max(hi[a], q);
    }
  }
  __shared__ double sh[32];
  for (int q = 0; q < 9; q++) {
    const double v = mp_block_sum((double)s[q], sh);
    if (threadIdx.x == 0) part[(ll)blockIdx.x * 9 + q] = v;
    __syncthreads();
  }
  // the box: o lies in the group, so starting from it leaves min / max exact
  __shared__ unsigned long long bx[6][8];
  for (int a = 0; a < 3; a++) {
    for (int off = 16; off > 0; off >>= 1) {
      lo[a] = min(lo[a], __shfl_down_sync(0xffffffffu, lo[a], off));
      hi[a] = max(hi[a], __shfl_down_sync(0xffffffffu, hi[a], off));
    }
  }
  if ((threadIdx.x & 31) == 0)
    for (int a = 0; a < 3; a++) bx[a][threadIdx.x >> 5] = lo[a], bx[3 + a][threadIdx.x >> 5] = hi[a];
  __syncthreads();
  if (threadIdx.x < 6) {
    unsigned long long v = bx[threadIdx.x][0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++)
      v = threadIdx.x < 3 ? min(v, bx[threadIdx.x][w]) : max(v, bx[threadIdx.x][w]);
    box[(ll)blockIdx.x * 6 + threadIdx.x] = mp_okey_inv(v);
  }
}

// Eigen-decomposition of a symmetric 3x3 matrix by the cyclic Jacobi method
// (Golub and Van Loan, Matrix Computations, section 8.5): rotations that
// zero the off-diagonal entries in turn until they are negligible.  On
// return d holds the eigenvalues and the columns of V the eigenvectors.
__device__ void jacobi3(double A[3][3], double d[3], double V[3][3]) {
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) V[i][j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 32; sweep++) {
    const double off = fabs(A[0][1]) + fabs(A[0][2]) + fabs(A[1][2]);
    const double dia = fabs(A[0][0]) + fabs(A[1][1]) + fabs(A[2][2]);
    if (off <= 1e-15 * dia || off == 0.0) break;
    for (int p = 0; p < 2; p++)
      for (int q = p + 1; q < 3; q++) {
        if (A[p][q] == 0.0) continue;
        const double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), sn = t * c;
        for (int k = 0; k < 3; k++) {  // A <- A J
          const double akp = A[k][p], akq = A[k][q];
          A[k][p] = c * akp - sn * akq;
          A[k][q] = sn * akp + c * akq;
        }
        for (int k = 0; k < 3; k++) {  // A <- J^T A
          const double apk = A[p][k], aqk = A[q][k];
          A[p][k] = c * apk - sn * aqk;
          A[q][k] = sn * apk + c * aqk;
        }
        for (int k = 0; k < 3; k++) {  // V <- V J
          const double vkp = V[k][p], vkq = V[k][q];
          V[k][p] = c * vkp - sn * vkq;
          V[k][q] = sn * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < 3; i++) d[i] = A[i][i];
}

// One thread per group: mean, scatter matrix, principal axes (largest
// variance first; each axis signed so that its largest component is
// positive), scale.  When the two largest variances are within 5% the
// frame is the coordinate axes with RCB's cut axis first (the longest edge
// of the raw centroids' bounding box, ties to the lower axis) and the scale
// of the variance along it: the reference's step start separates the two
// halves of exactly that axis, and a guess along the same coordinate axis
// excites the same modes of a nearly degenerate pair (any other direction
// in their plane would excite both).  degen[g] = 1 for such a group.
// frame[g] = {mu[3], R[3][3] (rows = axes), 1/s, sa[3]}: mu in element
// spacings, x~ = R (c * sa - mu) / s.
__global__ void k_mp_frames(const FTile *__restrict__ tiles, const double *__restrict__ part,
                            const int *__restrict__ tile0, const int *__restrict__ ntile,
                            const ll *__restrict__ gstart, const ll *__restrict__ gn,
                            const int *__restrict__ perm, const double *__restrict__ cent, ll nel,
                            int ngroups, int ndim, const double *__restrict__ sa,
                            const double *__restrict__ box, double *__restrict__ frame,
                            int *__restrict__ degen) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngroups) return;
  double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int t = tile0[g]; t < tile0[g] + ntile[g]; t++)
    for (int q = 0; q < 9; q++) s[q] += part[(ll)t * 9 + q];
  const double n = (double)gn[g];
  const int e0 = perm[gstart[g]];
  const double *k = sa + (ll)g * 3;
  const double o[3] = {cent[e0] * k[0], cent[nel + e0] * k[1], cent[2 * nel + e0] * k[2]};
  double m[3] = {s[0] / n, s[1] / n, s[2] / n};
  double A[3][3];
  A[0][0] = s[3] - n * m[0] * m[0];
  A[1][1] = s[4] - n * m[1] * m[1];
  A[2][2] = s[5] - n * m[2] * m[2];
  A[0][1] = A[1][0] = s[6] - n * m[0] * m[1];
  A[0][2] = A[2][0] = s[7] - n * m[0] * m[2];
  A[1][2] = A[2][1] = s[8] - n * m[1] * m[2];
  if (ndim == 2) A[0][2] = A[2][0] = A[1][2] = A[2][1] = A[2][2] = 0.0;
  double Ac[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) Ac[i][j] = A[i][j];
  double d[3], V[3][3];
  jacobi3(Ac, d, V);
  int ord[3] = {0, 1, 2};  // eigenvalues descending
  for (int i = 0; i < 3; i++)
    for (int j = i + 1; j < 3; j++)
      if (d[ord[j]] > d[ord[i]]) {
        const int x = ord[i];
        ord[i] = ord[j], ord[j] = x;
      }
  double R[3][3];
  for (int a = 0; a < 3; a++)
    for (int k = 0; k < 3; k++) R[a][k] = V[k][ord[a]];
  double l1 = d[ord[0]];
  const double l2 = d[ord[1]];
  const bool dg = l1 > 0.0 && (l1 - l2) <= 0.05 * l1;
  degen[g] = dg ? 1 : 0;
  if (dg) {
    double lo[3], hi[3];
    for (int a = 0; a < 3; a++) lo[a] = box[(ll)tile0[g] * 6 + a], hi[a] = box[(ll)tile0[g] * 6 + 3 + a];
    for (int t = tile0[g] + 1; t < tile0[g] + ntile[g]; t++)
      for (int a = 0; a < 3; a++)
        lo[a] = fmin(lo[a], box[(ll)t * 6 + a]), hi[a] = fmax(hi[a], box[(ll)t * 6 + 3 + a]);
    int ax = 0;  // RCB's rule: strictly longer wins
    for (int a = 1; a < ndim; a++)
      if (hi[a] - lo[a] > hi[ax] - lo[ax]) ax = a;
    for (int a = 0, r = 1; a < 3; a++) {
      for (int q = 0; q < 3; q++) R[a == ax ? 0 : r][q] = a == q ? 1.0 : 0.0;
      if (a != ax) r++;
    }
    l1 = A[ax][ax];
  }
  for (int a = 0; a < 3; a++) {
    int big = 0;
    for (int k = 1; k < 3; k++)
      if (fabs(R[a][k]) > fabs(R[a][big])) big = k;
    if (R[a][big] < 0.0)
      for (int k = 0; k < 3; k++) R[a][k] = -R[a][k];
  }
  const double var = l1 > 0.0 ? l1 / n : 0.0;
  const double inv_s = var > 0.0 ? 1.0 / sqrt(3.0 * var) : 0.0;
  double *f = frame + (ll)g * MP_FRAME;
  for (int q = 0; q < 3; q++) f[q] = o[q] + m[q];
  for (int a = 0; a < 3; a++)
    for (int q = 0; q < 3; q++) f[3 + 3 * a + q] = R[a][q];
  f[12] = inv_s;
  for (int q = 0; q < 3; q++) f[13 + q] = k[q];
}

// x~ of element e in frame f (3 values)
__device__ __forceinline__ void frame_coords(const double *f, const double *cent, ll nel, int e,
                                             double out[3]) {
  const double x = cent[e] * f[13] - f[0], y = cent[nel + e] * f[14] - f[1],
               z = cent[2 * nel + e] * f[15] - f[2];
  for (int a = 0; a < 3; a++) out[a] = (f[3 + 3 * a] * x + f[4 + 3 * a] * y + f[5 + 3 * a] * z) * f[12];
}

// Input features of every position: X[i] = (x~ (3), deg / 56, g, 0, 0, 0)
// with g = -sin(pi x~_1 / 2), in FP32 (the first layer multiplies them as a pair of BF16 values, high
// and low part, so positions keep about 16 significant bits: a group may
// be thousands of elements long); rows outside the groups (grp < 0) and
// padding rows are zero.
// wsum[i] = sum_j w_ij in the level graph (FP32, reused by the backward).
__global__ void k_mp_features(const int *__restrict__ perm, const int *__restrict__ grp,
                              const double *__restrict__ cent, ll nel,
                              const double *__restrict__ frame, const unsigned *__restrict__ ell,
                              const ll *__restrict__ slice_off, const int *__restrict__ slice_w,
                              ll N, ll Npad, float *__restrict__ X, float *__restrict__ wsum) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Npad) return;
  float v[MP_FIN] = {0, 0, 0, 0, 0, 0, 0, 0};
  float ws = 0.f;
  const int g = i < N ? grp[i] : -1;
  if (g >= 0) {
    const int e = perm[i];
    const double *f = frame + (ll)g * MP_FRAME;
    double xt[3];
    frame_coords(f, cent, nel, e, xt);
    for (int a = 0; a < 3; a++) v[a] = (float)xt[a];
    const ll sl = i >> 5;
    const unsigned *ep = ell + slice_off[sl] + (i & 31);
    const int wd = slice_w[sl];
    unsigned acc = 0;
    for (int k = 0; k < wd; k++) acc += ep[(ll)k * 32] >> 28;
    ws = (float)acc;
    v[3] = (float)((double)acc * MP_DEG_SCALE);
    // the geometric guess -sin(pi x~_1 / 2) (the Fiedler vector of a uniform
    // bar along the first axis): an input, and the start the head corrects
    v[4] = (float)(-sin(1.5707963267948966 * xt[0]));
  }
  float4 *o = reinterpret_cast<float4 *>(X + i * MP_FIN);
  o[0] = make_float4(v[0], v[1], v[2], v[3]);
  o[1] = make_float4(v[4], v[5], v[6], v[7]);
  if (wsum) wsum[i] = ws;
}

// ---------------------------------------------------------------------------
// Layer kernels
// ---------------------------------------------------------------------------
// D += A B for one m16n8k16 BF16 tile (FP32 accumulators; fragment layouts
// of the PTX ISA's mma.m16n8k16 with .row.col operands).
__device__ __forceinline__ void mma_bf16(float *c, unsigned a0, unsigned a1, unsigned a2,
                                         unsigned a3, unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, {%0, %1, %2, %3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ unsigned pack_bf16(bf16 lo, bf16 hi) {
  return (unsigned)__bfloat16_as_ushort(lo) | ((unsigned)__bfloat16_as_ushort(hi) << 16);
}

// Weighted neighbour mean of DIN features: 8 features (one 16-byte load per
// neighbour) of row i starting at column c8 * 8.
template <int DIN>
__device__ __forceinline__ void gather_mean(const bf16 *__restrict__ H, const unsigned *ep,
                                            int wd, int c8, float inv, float acc[8]) {
#pragma unroll
  for (int q = 0; q < 8; q++) acc[q] = 0.f;
  for (int k = 0; k < wd; k++) {
    const unsigned x = ep[(ll)k * 32];
    const unsigned w = x >> 28;
    if (!w) continue;
    const ll j = x & 0x0FFFFFFFu;
    const uint4 hv = *reinterpret_cast<const uint4 *>(H + j * DIN + c8 * 8);
    const bf16 *hb = reinterpret_cast<const bf16 *>(&hv);
    const float fw = (float)w;
#pragma unroll
    for (int q = 0; q < 8; q++) acc[q] = fmaf(fw, __bfloat162float(hb[q]), acc[q]);
  }
#pragma unroll
  for (int q = 0; q < 8; q++) acc[q] *= inv;
}

// One layer, tiles of 64 rows (grid-stride):
//   A = [h_prev | weighted neighbour mean of h_prev]   (64 x 2 DIN, BF16, smem)
//   Z = A W + b (tensor cores, FP32), h = relu(Z) -> Hout (BF16)
// AG (optional): the neighbour means, kept for the backward pass.
// HEAD: also y = h . wo + bo (FP32) per row.
// F32IN (first layer): inputs and neighbour means in FP32, split into a
// high and a low BF16 part; Z = A_hi W + A_lo W (two MMAs), AG in FP32.
template <int DIN, bool HEAD, bool F32IN = false>
__global__ void __launch_bounds__(MP_THREADS)
k_mp_fwd(const void *__restrict__ Hin_, const unsigned *__restrict__ ell,
         const ll *__restrict__ slice_off, const int *__restrict__ slice_w,
         const float *__restrict__ wsum, ll N, ll Npad, const bf16 *__restrict__ Wf,
         const float *__restrict__ bias, bf16 *__restrict__ Hout, void *__restrict__ AG_,
         const float *__restrict__ wo, const float *__restrict__ bo, float *__restrict__ y,
         const float *__restrict__ Xg) {
  constexpr int K = 2 * DIN, KP = K + 8;
  const bf16 *__restrict__ Hin = static_cast<const bf16 *>(Hin_);
  bf16 *__restrict__ AG = static_cast<bf16 *>(AG_);
  __shared__ __align__(16) bf16 sA[MP_ROWS * KP];
  __shared__ __align__(16) bf16 sAlo[F32IN ? MP_ROWS * KP : 8];
  __shared__ __align__(16) bf16 sW[MP_HID * KP];
  for (int q = threadIdx.x; q < MP_HID * (K / 8); q += blockDim.x) {
    const int n = q / (K / 8), k8 = q % (K / 8);
    *reinterpret_cast<uint4 *>(sW + n * KP + k8 * 8) =
        *reinterpret_cast<const uint4 *>(Wf + n * K + k8 * 8);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, tig = lane & 3;
  constexpr int LPR = DIN / 8;           // lanes per row in the gather
  constexpr int RPP = MP_THREADS / LPR;  // rows per pass of the block
  const ll ntiles = Npad / MP_ROWS;
  for (ll tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const ll base = tile * MP_ROWS;
    __syncthreads();  // sA is free again (and sW is loaded)
    if (F32IN) {  // one thread per row, 8 FP32 features
      const float *Hf = static_cast<const float *>(Hin_);
      float *AGf = static_cast<float *>(AG_);
      for (int r = threadIdx.x; r < MP_ROWS; r += MP_THREADS) {
        const ll i = base + r;
        float sv[8] = {0, 0, 0, 0, 0, 0, 0, 0}, acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        if (i < N) {
          const float4 a = reinterpret_cast<const float4 *>(Hf + i * 8)[0];
          const float4 b = reinterpret_cast<const float4 *>(Hf + i * 8)[1];
          sv[0] = a.x, sv[1] = a.y, sv[2] = a.z, sv[3] = a.w;
          sv[4] = b.x, sv[5] = b.y, sv[6] = b.z, sv[7] = b.w;
          const ll sl = i >> 5;
          const unsigned *ep = ell + slice_off[sl] + (i & 31);
          const int wd = slice_w[sl];
          for (int k = 0; k < wd; k++) {
            const unsigned x = ep[(ll)k * 32];
            const unsigned w = x >> 28;
            if (!w) continue;
            const ll j = x & 0x0FFFFFFFu;
            const float4 c = reinterpret_cast<const float4 *>(Hf + j * 8)[0];
            const float4 d = reinterpret_cast<const float4 *>(Hf + j * 8)[1];
            const float fw = (float)w;
            acc[0] = fmaf(fw, c.x, acc[0]), acc[1] = fmaf(fw, c.y, acc[1]);
            acc[2] = fmaf(fw, c.z, acc[2]), acc[3] = fmaf(fw, c.w, acc[3]);
            acc[4] = fmaf(fw, d.x, acc[4]), acc[5] = fmaf(fw, d.y, acc[5]);
            acc[6] = fmaf(fw, d.z, acc[6]), acc[7] = fmaf(fw, d.w, acc[7]);
          }
          const float ws = wsum[i];
          const float inv = ws > 0.f ? 1.f / ws : 0.f;
#pragma unroll
          for (int q = 0; q < 8; q++) acc[q] *= inv;
        }
#pragma unroll
        for (int q = 0; q < 8; q++) {
          const bf16 h0 = __float2bfloat16_rn(sv[q]), h1 = __float2bfloat16_rn(acc[q]);
          sA[r * KP + q] = h0;
          sAlo[r * KP + q] = __float2bfloat16_rn(sv[q] - __bfloat162float(h0));
          sA[r * KP + DIN + q] = h1;
          sAlo[r * KP + DIN + q] = __float2bfloat16_rn(acc[q] - __bfloat162float(h1));
        }
        if (AGf && i < Npad) {
          reinterpret_cast<float4 *>(AGf + i * 8)[0] = make_float4(acc[0], acc[1], acc[2], acc[3]);
          reinterpret_cast<float4 *>(AGf + i * 8)[1] = make_float4(acc[4], acc[5], acc[6], acc[7]);
        }
      }
    } else
    for (int r = threadIdx.x / LPR; r < MP_ROWS; r += RPP) {
      const int c8 = threadIdx.x % LPR;
      const ll i = base + r;
      float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      uint4 self = make_uint4(0u, 0u, 0u, 0u);
      if (i < N) {
        self = *reinterpret_cast<const uint4 *>(Hin + i * DIN + c8 * 8);
        const ll sl = i >> 5;
        const float ws = wsum[i];
        gather_mean<DIN>(Hin, ell + slice_off[sl] + (i & 31), slice_w[sl], c8,
                         ws > 0.f ? 1.f / ws : 0.f, acc);
      }
      __align__(16) bf16 ag[8];
#pragma unroll
      for (int q = 0; q < 8; q++) ag[q] = __float2bfloat16_rn(acc[q]);
      *reinterpret_cast<uint4 *>(sA + r * KP + c8 * 8) = self;
      *reinterpret_cast<uint4 *>(sA + r * KP + DIN + c8 * 8) = *reinterpret_cast<uint4 *>(ag);
      if (AG) *reinterpret_cast<uint4 *>(AG + i * DIN + c8 * 8) = *reinterpret_cast<uint4 *>(ag);
    }
    __syncthreads();
    float c[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; nt++) c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.f;
    const bf16 *ar0 = sA + (warp * 16 + g) * KP, *ar1 = ar0 + 8 * KP;
#pragma unroll
    for (int ks = 0; ks < K / 16; ks++) {
      const int k0 = ks * 16 + 2 * tig;
      const unsigned a0 = *reinterpret_cast<const unsigned *>(ar0 + k0);
      const unsigned a1 = *reinterpret_cast<const unsigned *>(ar1 + k0);
      const unsigned a2 = *reinterpret_cast<const unsigned *>(ar0 + k0 + 8);
      const unsigned a3 = *reinterpret_cast<const unsigned *>(ar1 + k0 + 8);
#pragma unroll
      for (int nt = 0; nt < 8; nt++) {
        const bf16 *bp = sW + (nt * 8 + g) * KP + k0;
        mma_bf16(c[nt], a0, a1, a2, a3, *reinterpret_cast<const unsigned *>(bp),
                 *reinterpret_cast<const unsigned *>(bp + 8));
      }
      if (F32IN) {  // the low parts of the inputs, same weights
        const bf16 *lr0 = sAlo + (warp * 16 + g) * KP, *lr1 = lr0 + 8 * KP;
        const unsigned l0 = *reinterpret_cast<const unsigned *>(lr0 + k0);
        const unsigned l1 = *reinterpret_cast<const unsigned *>(lr1 + k0);
        const unsigned l2 = *reinterpret_cast<const unsigned *>(lr0 + k0 + 8);
        const unsigned l3 = *reinterpret_cast<const unsigned *>(lr1 + k0 + 8);
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
          const bf16 *bp = sW + (nt * 8 + g) * KP + k0;
          mma_bf16(c[nt], l0, l1, l2, l3, *reinterpret_cast<const unsigned *>(bp),
                   *reinterpret_cast<const unsigned *>(bp + 8));
        }
      }
    }
    const ll r0 = base + warp * 16 + g, r1 = r0 + 8;
    float y0 = 0.f, y1 = 0.f;
#pragma unroll
    for (int nt = 0; nt < 8; nt++) {
      const int n = nt * 8 + 2 * tig;
      const float h00 = fmaxf(c[nt][0] + bias[n], 0.f), h01 = fmaxf(c[nt][1] + bias[n + 1], 0.f);
      const float h10 = fmaxf(c[nt][2] + bias[n], 0.f), h11 = fmaxf(c[nt][3] + bias[n + 1], 0.f);
      if (Hout) {
        *reinterpret_cast<unsigned *>(Hout + r0 * MP_HID + n) =
            pack_bf16(__float2bfloat16_rn(h00), __float2bfloat16_rn(h01));
        *reinterpret_cast<unsigned *>(Hout + r1 * MP_HID + n) =
            pack_bf16(__float2bfloat16_rn(h10), __float2bfloat16_rn(h11));
      }
      if (HEAD) {
        // the head reads the BF16-rounded activations, as the backward does
        y0 = fmaf(__bfloat162float(__float2bfloat16_rn(h00)), wo[n], y0);
        y0 = fmaf(__bfloat162float(__float2bfloat16_rn(h01)), wo[n + 1], y0);
        y1 = fmaf(__bfloat162float(__float2bfloat16_rn(h10)), wo[n], y1);
        y1 = fmaf(__bfloat162float(__float2bfloat16_rn(h11)), wo[n + 1], y1);
      }
    }
    if (HEAD) {
      y0 += __shfl_xor_sync(0xffffffffu, y0, 1);
      y0 += __shfl_xor_sync(0xffffffffu, y0, 2);
      y1 += __shfl_xor_sync(0xffffffffu, y1, 1);
      y1 += __shfl_xor_sync(0xffffffffu, y1, 2);
      if (tig == 0) {  // the head corrects the geometric guess (feature 4)
        y[r0] = y0 + bo[0] + Xg[r0 * MP_FIN + 4];
        y[r1] = y1 + bo[0] + Xg[r1 * MP_FIN + 4];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Loss and backward kernels (training)
// ---------------------------------------------------------------------------
// One block per group: sign-invariant cosine loss between the centred
// prediction yc = y - mean(y) and the centred label fc:
//   loss_g = 1 - (yc . fc)^2 / (|yc|^2 |fc|^2)
// and dloss_g / dy_i = (-2 c / (s ff) fc_i + 2 c^2 / (s^2 ff) yc_i) / G with
// c = yc . fc, s = |yc|^2, ff = |fc|^2 (the centring adds nothing: both
// vectors sum to zero).  G = number of groups (the loss is their mean).
__global__ void __launch_bounds__(256)
k_mp_loss(const float *__restrict__ y, const double *__restrict__ lab,
          const ll *__restrict__ gstart, const ll *__restrict__ gn, int G,
          float *__restrict__ dy, double *__restrict__ loss) {
  const int g = blockIdx.x;
  const ll b = gstart[g], n = gn[g];
  __shared__ double sh[32];
  __shared__ double bc[5];
  double sy = 0.0, sl = 0.0;
  for (ll i = b + threadIdx.x; i < b + n; i += blockDim.x) sy += y[i], sl += lab[i];
  sy = mp_block_sum(sy, sh);
  sl = mp_block_sum(sl, sh);
  if (threadIdx.x == 0) bc[0] = sy / (double)n, bc[1] = sl / (double)n;
  __syncthreads();
  const double my = bc[0], ml = bc[1];
  double c = 0.0, s = 0.0, ff = 0.0;
  for (ll i = b + threadIdx.x; i < b + n; i += blockDim.x) {
    const double yc = (double)y[i] - my, fc = lab[i] - ml;
    c += yc * fc, s += yc * yc, ff += fc * fc;
  }
  c = mp_block_sum(c, sh);
  s = mp_block_sum(s, sh);
  ff = mp_block_sum(ff, sh);
  if (threadIdx.x == 0) {
    const bool ok = s > 1e-30 && ff > 1e-30;
    bc[2] = ok ? -2.0 * c / (s * ff) / (double)G : 0.0;
    bc[3] = ok ? 2.0 * c * c / (s * s * ff) / (double)G : 0.0;
    loss[g] = ok ? 1.0 - c * c / (s * ff) : 1.0;
  }
  __syncthreads();
  const double ka = bc[2], kb = bc[3];
  for (ll i = b + threadIdx.x; i < b + n; i += blockDim.x)
    dy[i] = (float)(ka * (lab[i] - ml) + kb * ((double)y[i] - my));
}

constexpr int MP_GB = 304;  // blocks of the backward kernels (fixed: partial sums in order)

// Head and last ReLU: dZ3 = (dy wo) * [h3 > 0] (BF16); per block partial
// sums of dwo = sum_i dy_i h3_i and dbo = sum_i dy_i -> part[block][65].
__global__ void __launch_bounds__(MP_THREADS)
k_mp_head_bwd(const float *__restrict__ dy, const bf16 *__restrict__ H3, ll Npad,
              const float *__restrict__ wo, bf16 *__restrict__ dZ, float *__restrict__ part) {
  const int c8 = threadIdx.x & 7;
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0}, accb = 0.f;
  for (ll i = (ll)blockIdx.x * (MP_THREADS / 8) + (threadIdx.x >> 3); i < Npad;
       i += (ll)gridDim.x * (MP_THREADS / 8)) {
    const float d = dy[i];
    const uint4 hv = *reinterpret_cast<const uint4 *>(H3 + i * MP_HID + c8 * 8);
    const bf16 *hb = reinterpret_cast<const bf16 *>(&hv);
    __align__(16) bf16 o[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const float h = __bfloat162float(hb[q]);
      acc[q] = fmaf(d, h, acc[q]);
      o[q] = __float2bfloat16_rn(h > 0.f ? d * wo[c8 * 8 + q] : 0.f);
    }
    if (c8 == 0) accb += d;
    *reinterpret_cast<uint4 *>(dZ + i * MP_HID + c8 * 8) = *reinterpret_cast<const uint4 *>(o);
  }
  __shared__ float sh[MP_THREADS][9];
#pragma unroll
  for (int q = 0; q < 8; q++) sh[threadIdx.x][q] = acc[q];
  sh[threadIdx.x][8] = accb;
  __syncthreads();
  if (threadIdx.x < MP_HID + 1) {
    float s = 0.f;
    if (threadIdx.x < MP_HID) {
      const int n = threadIdx.x;
      for (int t = n / 8; t < MP_THREADS; t += 8) s += sh[t][n % 8];
    } else {
      for (int t = 0; t < MP_THREADS; t += 8) s += sh[t][8];
    }
    part[(ll)blockIdx.x * (MP_HID + 1) + threadIdx.x] = s;
  }
}

// Backward of one layer, tiles of 64 rows, MP_GB blocks (grid-stride):
//   dA = dZ W^T (tensor cores): the first DIN columns are dL/dh_prev through
//   the self term -> dH (FP32); the last DIN are dL/da, divided by the
//   row's weight sum -> U (BF16), scattered to the neighbours by
//   k_mp_gather_bwd (the graph is symmetric, so the scatter is a gather);
//   dW += A^T dZ, db += sum of dZ rows (per block, FP32) -> partials.
// INPUT_GRAD = false for the first layer (its inputs are the features).
// F32IN (first layer): Hprev (the features) and AG in FP32, split into high
// and low BF16 parts for dW += A_hi^T dZ + A_lo^T dZ.
template <int DIN, bool INPUT_GRAD, bool F32IN = false>
__global__ void __launch_bounds__(MP_THREADS)
k_mp_bwd(const bf16 *__restrict__ dZ, const void *__restrict__ Hprev_,
         const void *__restrict__ AG_, const float *__restrict__ wsum, ll Npad,
         const bf16 *__restrict__ Wb, float *__restrict__ dH, bf16 *__restrict__ U,
         float *__restrict__ part_w, float *__restrict__ part_b) {
  constexpr int K = 2 * DIN, KP = K + 8, ZP = MP_HID + 8;
  constexpr int NPAIR = (K / 16) * 8;              // (m-tile, n-tile) pairs of dW
  constexpr int PPW = NPAIR / (MP_THREADS / 32);  // per warp
  const bf16 *__restrict__ Hprev = static_cast<const bf16 *>(Hprev_);
  const bf16 *__restrict__ AG = static_cast<const bf16 *>(AG_);
  __shared__ __align__(16) bf16 sZ[MP_ROWS * ZP];
  __shared__ __align__(16) bf16 sA[MP_ROWS * KP];
  __shared__ __align__(16) bf16 sAlo[F32IN ? MP_ROWS * KP : 8];
  __shared__ __align__(16) bf16 sW[INPUT_GRAD ? K * ZP : 8];
  if (INPUT_GRAD)
    for (int q = threadIdx.x; q < K * (MP_HID / 8); q += blockDim.x) {
      const int k = q / (MP_HID / 8), h8 = q % (MP_HID / 8);
      *reinterpret_cast<uint4 *>(sW + k * ZP + h8 * 8) =
          *reinterpret_cast<const uint4 *>(Wb + k * MP_HID + h8 * 8);
    }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int g = lane >> 2, tig = lane & 3;
  float cw[PPW][4];
#pragma unroll
  for (int j = 0; j < PPW; j++) cw[j][0] = cw[j][1] = cw[j][2] = cw[j][3] = 0.f;
  float cb = 0.f;  // thread t: column t % 64, rows of half t / 64
  const ll ntiles = Npad / MP_ROWS;
  for (ll tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const ll base = tile * MP_ROWS;
    __syncthreads();
    for (int q = threadIdx.x; q < MP_ROWS * (MP_HID / 8); q += blockDim.x) {
      const int r = q / (MP_HID / 8), h8 = q % (MP_HID / 8);
      *reinterpret_cast<uint4 *>(sZ + r * ZP + h8 * 8) =
          *reinterpret_cast<const uint4 *>(dZ + (base + r) * MP_HID + h8 * 8);
    }
    if (F32IN) {
      const float *Hf = static_cast<const float *>(Hprev_), *Af = static_cast<const float *>(AG_);
      for (int q = threadIdx.x; q < MP_ROWS * K; q += blockDim.x) {
        const int r = q / K, k = q % K;
        const float v = k < DIN ? Hf[(base + r) * DIN + k] : Af[(base + r) * DIN + k - DIN];
        const bf16 h = __float2bfloat16_rn(v);
        sA[r * KP + k] = h;
        sAlo[r * KP + k] = __float2bfloat16_rn(v - __bfloat162float(h));
      }
    } else {
      for (int q = threadIdx.x; q < MP_ROWS * (K / 8); q += blockDim.x) {
        const int r = q / (K / 8), k8 = q % (K / 8);
        const bf16 *src = k8 < DIN / 8 ? Hprev + (base + r) * DIN + k8 * 8
                                       : AG + (base + r) * DIN + (k8 - DIN / 8) * 8;
        *reinterpret_cast<uint4 *>(sA + r * KP + k8 * 8) = *reinterpret_cast<const uint4 *>(src);
      }
    }
    __syncthreads();
    if (INPUT_GRAD) {
      constexpr int NT = K / 8;
      float c[NT][4];
#pragma unroll
      for (int nt = 0; nt < NT; nt++) c[nt][0] = c[nt][1] = c[nt][2] = c[nt][3] = 0.f;
      const bf16 *ar0 = sZ + (warp * 16 + g) * ZP, *ar1 = ar0 + 8 * ZP;
#pragma unroll
      for (int ks = 0; ks < MP_HID / 16; ks++) {
        const int k0 = ks * 16 + 2 * tig;
        const unsigned a0 = *reinterpret_cast<const unsigned *>(ar0 + k0);
        const unsigned a1 = *reinterpret_cast<const unsigned *>(ar1 + k0);
        const unsigned a2 = *reinterpret_cast<const unsigned *>(ar0 + k0 + 8);
        const unsigned a3 = *reinterpret_cast<const unsigned *>(ar1 + k0 + 8);
#pragma unroll
        for (int nt = 0; nt < NT; nt++) {
          const bf16 *bp = sW + (nt * 8 + g) * ZP + k0;
          mma_bf16(c[nt], a0, a1, a2, a3, *reinterpret_cast<const unsigned *>(bp),
                   *reinterpret_cast<const unsigned *>(bp + 8));
        }
      }
      const ll r0 = base + warp * 16 + g, r1 = r0 + 8;
      const float w0 = wsum[r0], w1 = wsum[r1];
      const float i0 = w0 > 0.f ? 1.f / w0 : 0.f, i1 = w1 > 0.f ? 1.f / w1 : 0.f;
#pragma unroll
      for (int nt = 0; nt < NT; nt++) {
        const int n = nt * 8 + 2 * tig;
        if (n < DIN) {
          *reinterpret_cast<float2 *>(dH + r0 * DIN + n) = make_float2(c[nt][0], c[nt][1]);
          *reinterpret_cast<float2 *>(dH + r1 * DIN + n) = make_float2(c[nt][2], c[nt][3]);
        } else {
          *reinterpret_cast<unsigned *>(U + r0 * DIN + (n - DIN)) = pack_bf16(
              __float2bfloat16_rn(c[nt][0] * i0), __float2bfloat16_rn(c[nt][1] * i0));
          *reinterpret_cast<unsigned *>(U + r1 * DIN + (n - DIN)) = pack_bf16(
              __float2bfloat16_rn(c[nt][2] * i1), __float2bfloat16_rn(c[nt][3] * i1));
        }
      }
    }
    // dW += A^T dZ over this tile's 64 rows (k dimension of the MMA)
#pragma unroll
    for (int j = 0; j < PPW; j++) {
      const int pr = warp + j * (MP_THREADS / 32);
      const int mt = pr / 8, nt = pr % 8;
#pragma unroll
      for (int ks = 0; ks < MP_ROWS / 16; ks++) {
        const int rk = ks * 16 + 2 * tig;
        const bf16 *x0 = sA + rk * KP + mt * 16 + g;
        const unsigned a0 = pack_bf16(x0[0], x0[KP]);
        const unsigned a1 = pack_bf16(x0[8], x0[KP + 8]);
        const unsigned a2 = pack_bf16(x0[8 * KP], x0[9 * KP]);
        const unsigned a3 = pack_bf16(x0[8 * KP + 8], x0[9 * KP + 8]);
        const bf16 *z0 = sZ + rk * ZP + nt * 8 + g;
        const unsigned b0 = pack_bf16(z0[0], z0[ZP]);
        const unsigned b1 = pack_bf16(z0[8 * ZP], z0[9 * ZP]);
        mma_bf16(cw[j], a0, a1, a2, a3, b0, b1);
        if (F32IN) {
          const bf16 *y0 = sAlo + rk * KP + mt * 16 + g;
          mma_bf16(cw[j], pack_bf16(y0[0], y0[KP]), pack_bf16(y0[8], y0[KP + 8]),
                   pack_bf16(y0[8 * KP], y0[9 * KP]), pack_bf16(y0[8 * KP + 8], y0[9 * KP + 8]),
                   b0, b1);
        }
      }
    }
    {
      const int n = threadIdx.x % MP_HID, half = threadIdx.x / MP_HID;
      for (int r = half * 32; r < half * 32 + 32; r++) cb += __bfloat162float(sZ[r * ZP + n]);
    }
  }
  // partials of this block
  float *pw = part_w + (ll)blockIdx.x * K * MP_HID;
#pragma unroll
  for (int j = 0; j < PPW; j++) {
    const int pr = warp + j * (MP_THREADS / 32);
    const int mt = pr / 8, nt = pr % 8;
    const int m0 = mt * 16 + g, n0 = nt * 8 + 2 * tig;
    pw[m0 * MP_HID + n0] = cw[j][0];
    pw[m0 * MP_HID + n0 + 1] = cw[j][1];
    pw[(m0 + 8) * MP_HID + n0] = cw[j][2];
    pw[(m0 + 8) * MP_HID + n0 + 1] = cw[j][3];
  }
  __shared__ float sb[MP_THREADS];
  sb[threadIdx.x] = cb;
  __syncthreads();
  if (threadIdx.x < MP_HID)
    part_b[(ll)blockIdx.x * MP_HID + threadIdx.x] = sb[threadIdx.x] + sb[threadIdx.x + MP_HID];
}

// dL/dh_prev = dH (self term) + sum_j w_ij U_j (neighbour terms), then the
// previous layer's ReLU: dZ_prev = dL/dh_prev * [h_prev > 0] (BF16).
__global__ void __launch_bounds__(MP_THREADS)
k_mp_gather_bwd(const float *__restrict__ dH, const bf16 *__restrict__ U,
                const bf16 *__restrict__ Hprev, const unsigned *__restrict__ ell,
                const ll *__restrict__ slice_off, const int *__restrict__ slice_w, ll N,
                ll Npad, bf16 *__restrict__ dZ) {
  const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  const ll i = t >> 3;
  const int c8 = (int)(t & 7);
  if (i >= Npad) return;
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (i < N) {
    const ll sl = i >> 5;
    gather_mean<MP_HID>(U, ell + slice_off[sl] + (i & 31), slice_w[sl], c8, 1.f, acc);
  }
  const uint4 hv = *reinterpret_cast<const uint4 *>(Hprev + i * MP_HID + c8 * 8);
  const bf16 *hb = reinterpret_cast<const bf16 *>(&hv);
  __align__(16) bf16 o[8];
#pragma unroll
  for (int q = 0; q < 8; q++) {
    const float d = dH[i * MP_HID + c8 * 8 + q] + acc[q];
    o[q] = __float2bfloat16_rn(__bfloat162float(hb[q]) > 0.f ? d : 0.f);
  }
  *reinterpret_cast<uint4 *>(dZ + i * MP_HID + c8 * 8) = *reinterpret_cast<const uint4 *>(o);
}

// Flat gradient from the per-block partials, summed in block order.
__global__ void k_mp_grad_reduce(const float *__restrict__ pw0, const float *__restrict__ pb0,
                                 const float *__restrict__ pw1, const float *__restrict__ pb1,
                                 const float *__restrict__ pw2, const float *__restrict__ pb2,
                                 const float *__restrict__ ph, int nblk, float *__restrict__ grad) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= MP_NPARAM) return;
  const float *src;
  ll stride;
  int off;
  if (q < MP_OFF_B1) src = pw0, stride = MP_K1 * MP_HID, off = q - MP_OFF_W1;
  else if (q < MP_OFF_W2) src = pb0, stride = MP_HID, off = q - MP_OFF_B1;
  else if (q < MP_OFF_B2) src = pw1, stride = MP_K2 * MP_HID, off = q - MP_OFF_W2;
  else if (q < MP_OFF_W3) src = pb1, stride = MP_HID, off = q - MP_OFF_B2;
  else if (q < MP_OFF_B3) src = pw2, stride = MP_K2 * MP_HID, off = q - MP_OFF_W3;
  else if (q < MP_OFF_WO) src = pb2, stride = MP_HID, off = q - MP_OFF_B3;
  else src = ph, stride = MP_HID + 1, off = q - MP_OFF_WO;
  float s = 0.f;
  for (int b = 0; b < nblk; b++) s += src[(ll)b * stride + off];
  grad[q] = s;
}

// Adam (Kingma and Ba, 2015): m = b1 m + (1 - b1) g, v = b2 v + (1 - b2) g^2,
// p -= lr (m / c1) / (sqrt(v / c2) + eps) with c1 = 1 - b1^t, c2 = 1 - b2^t.
__global__ void k_mp_adam(float *__restrict__ p, float *__restrict__ m, float *__restrict__ v,
                          const float *__restrict__ g, int n, float lr, float b1, float b2,
                          float eps, float c1, float c2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const float gq = g[q];
  const float mq = b1 * m[q] + (1.f - b1) * gq;
  const float vq = b2 * v[q] + (1.f - b2) * gq * gq;
  m[q] = mq, v[q] = vq;
  p[q] -= lr * (mq / c1) / (sqrtf(vq / c2) + eps);
}

__global__ void k_mp_to_pos(const int *__restrict__ perm, const double *__restrict__ lab_elem,
                            ll N, double *__restrict__ lab_pos) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) lab_pos[i] = lab_elem[perm[i]];
}

__global__ void k_mp_pred_to_elem(const int *__restrict__ perm, const float *__restrict__ y,
                                  ll N, float *__restrict__ out) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) out[perm[i]] = y[i];
}

__global__ void k_mp_feat_to_elem(const int *__restrict__ perm, const float *__restrict__ X, ll N,
                                  float *__restrict__ out) {
  const ll t = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= N * MP_FIN) return;
  const ll i = t / MP_FIN;
  const int k = (int)(t % MP_FIN);
  out[(ll)perm[i] * MP_FIN + k] = X[t];
}

// Geometric start: y = -sin(pi x~_1 / 2) along the group's principal axis,
// the Fiedler vector of a uniform bar (a cosine over its length).  x~_1 in
// FP64 (its axis only), the sine in FP32 (sinpif): a start vector needs no
// more, and FP64 transcendentals at 1/64 of the FP32 rate bounded this pass.
__global__ void k_mp_geometric(const int *__restrict__ perm, const int *__restrict__ grp,
                               const double *__restrict__ cent, ll nel,
                               const double *__restrict__ frame, ll N, double *__restrict__ y) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int g = grp[i];
  double v = 0.0;
  if (g >= 0) {
    const int e = perm[i];
    const double *f = frame + (ll)g * MP_FRAME;
    const double x = fma(cent[e], f[13], -f[0]), yy = fma(cent[nel + e], f[14], -f[1]),
                 z = fma(cent[2 * nel + e], f[15], -f[2]);
    const double x1 = fma(f[3], x, fma(f[4], yy, f[5] * z)) * f[12];
    v = -(double)sinpif(0.5f * (float)x1);
  }
  y[i] = v;
}

__global__ void k_mp_y_to_double(const float *__restrict__ y, const int *__restrict__ grp, ll N,
                                 double *__restrict__ out) {
  const ll i = (ll)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < N) out[i] = grp[i] >= 0 ? (double)y[i] : 0.0;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
// The rows the network runs on: a level graph in position order, the
// element at each position, the group of each position (-1: none) and the
// groups as contiguous position ranges.
struct MpView {
  const Level *lv = nullptr;
  const int *perm = nullptr;
  const int *grp = nullptr;
  ll N = 0, Npad = 0;
  std::vector<ll> gstart, gn;
};

struct MpBuffers {
  DBuf<float> X, AG0;  // first layer: FP32 features and neighbour means
  DBuf<bf16> H[3], AG[3];
  DBuf<float> wsum, y;
  DBuf<float> dy, dH, part_w[3], part_b[3], part_head, grad;
  DBuf<bf16> dZa, dZb, U;
  DBuf<double> loss, lab_pos;
  DBuf<ll> d_gstart, d_gn;
};

inline unsigned mp_grid(ll Npad) {
  const ll tiles = Npad / MP_ROWS;
  return (unsigned)std::max<ll>(1, std::min<ll>(tiles, 152 * 8));
}

void mp_frames(const MpView &v, const double *cent, ll nel, int ndim, DBuf<double> &frame,
               std::vector<int> *degen = nullptr, const float4 *esp = nullptr);

void mp_features(const MpView &v, const double *cent, ll nel, int ndim, MpBuffers &B,
                 std::vector<int> *degen = nullptr, const float4 *esp = nullptr) {
  cudaStream_t st = ctx().stream;
  B.X.ensure((size_t)v.Npad * MP_FIN);
  B.wsum.ensure((size_t)v.Npad);
  DBuf<double> frame;
  mp_frames(v, cent, nel, ndim, frame, degen, esp);
  k_mp_features<<<grid_for(v.Npad, 256), 256, 0, st>>>(
      v.perm, v.grp, cent, nel, frame.p, v.lv->ell.p, v.lv->slice_off.p, v.lv->slice_w.p, v.N,
      v.Npad, B.X.p, B.wsum.p);
  CK_LAUNCH();
}

// Per group: {mu[3], R[3][3], 1/s} (k_mp_frames); degen (optional): per
// group, 1 when its two largest centroid variances are within 5% (its frame
// is then RCB's cut axis first).
void mp_frames(const MpView &v, const double *cent, ll nel, int ndim, DBuf<double> &frame,
               std::vector<int> *degen, const float4 *esp) {
  cudaStream_t st = ctx().stream;
  const int G = (int)v.gstart.size();
  std::vector<FTile> tiles;
  std::vector<int> t0(G), nt(G);
  for (int g = 0; g < G; g++) {
    t0[g] = (int)tiles.size();
    for (ll b = v.gstart[g]; b < v.gstart[g] + v.gn[g]; b += MP_FTILE)
      tiles.push_back({b, std::min(b + MP_FTILE, v.gstart[g] + v.gn[g]), g});
    nt[g] = (int)tiles.size() - t0[g];
  }
  frame.ensure((size_t)std::max(G, 1) * MP_FRAME);
  DBuf<int> dg((size_t)std::max(G, 1));
  DBuf<double> sa((size_t)std::max(G, 1) * 3);
  if (G > 0 && !tiles.empty()) {
    DBuf<FTile> dt(tiles.size());
    DBuf<int> d0(G), dn(G);
    DBuf<ll> gs(G), gn(G);
    h2d(dt.p, tiles.data(), tiles.size());
    h2d(d0.p, t0.data(), G);
    h2d(dn.p, nt.data(), G);
    h2d(gs.p, v.gstart.data(), G);
    h2d(gn.p, v.gn.data(), G);
    DBuf<double> part(tiles.size() * 9), box(tiles.size() * 6);
    const unsigned wface = ndim == 3 ? 4u : 2u;  // face (3D) or edge (2D) neighbours
    if (esp)
      k_mp_spacing_elem<<<(unsigned)tiles.size(), 256, 0, st>>>(dt.p, v.perm, esp, part.p);
    else
      k_mp_spacing<<<(unsigned)tiles.size(), 256, 0, st>>>(dt.p, v.perm, cent, nel,
                                                          v.lv->ell.p, v.lv->slice_off.p,
                                                          v.lv->slice_w.p, wface, part.p);
    CK_LAUNCH();
    k_mp_scales<<<grid_for(G, 128), 128, 0, st>>>(part.p, d0.p, dn.p, G, sa.p);
    CK_LAUNCH();
    k_mp_moments<<<(unsigned)tiles.size(), 256, 0, st>>>(dt.p, gs.p, v.perm, cent, nel, sa.p,
                                                        part.p, box.p);
    CK_LAUNCH();
    k_mp_frames<<<grid_for(G, 128), 128, 0, st>>>(dt.p, part.p, d0.p, dn.p, gs.p, gn.p, v.perm,
                                                  cent, nel, G, ndim, sa.p, box.p, frame.p,
                                                  dg.p);
    CK_LAUNCH();
  }
  if (degen) {
    degen->assign(G, 0);
    d2h(degen->data(), dg.p, (size_t)G);
    sync();
  }
}

// keep: store every layer's activations and neighbour means for backward.
void mp_forward(const MpView &v, const NetDev &net, MpBuffers &B, bool keep) {
  cudaStream_t st = ctx().stream;
  const size_t nh = (size_t)v.Npad * MP_HID;
  B.H[0].ensure(nh), B.H[1].ensure(nh), B.y.ensure((size_t)v.Npad);
  if (keep) {
    B.H[2].ensure(nh);
    B.AG0.ensure((size_t)v.Npad * MP_FIN), B.AG[1].ensure(nh), B.AG[2].ensure(nh);
  }
  const Level &lv = *v.lv;
  const unsigned grid = mp_grid(v.Npad);
  const float *p = net.p;
  k_mp_fwd<MP_FIN, false, true><<<grid, MP_THREADS, 0, st>>>(
      B.X.p, lv.ell.p, lv.slice_off.p, lv.slice_w.p, B.wsum.p, v.N, v.Npad, net.Wf[0],
      p + MP_OFF_B1, B.H[0].p, keep ? B.AG0.p : nullptr, nullptr, nullptr, nullptr, nullptr);
  CK_LAUNCH();
  k_mp_fwd<MP_HID, false><<<grid, MP_THREADS, 0, st>>>(
      B.H[0].p, lv.ell.p, lv.slice_off.p, lv.slice_w.p, B.wsum.p, v.N, v.Npad, net.Wf[1],
      p + MP_OFF_B2, B.H[1].p, keep ? B.AG[1].p : nullptr, nullptr, nullptr, nullptr, nullptr);
  CK_LAUNCH();
  k_mp_fwd<MP_HID, true><<<grid, MP_THREADS, 0, st>>>(
      B.H[1].p, lv.ell.p, lv.slice_off.p, lv.slice_w.p, B.wsum.p, v.N, v.Npad, net.Wf[2],
      p + MP_OFF_B3, keep ? B.H[2].p : nullptr, keep ? B.AG[2].p : nullptr, p + MP_OFF_WO,
      p + MP_OFF_BO, B.y.p, B.X.p);
  CK_LAUNCH();
}

// Loss against lab_pos (per position), gradient into B.grad; returns the
// mean loss over the groups.
double mp_backward(const MpView &v, const NetDev &net, MpBuffers &B) {
  cudaStream_t st = ctx().stream;
  const int G = (int)v.gstart.size();
  const size_t nh = (size_t)v.Npad * MP_HID;
  B.dy.ensure((size_t)v.Npad), B.loss.ensure((size_t)std::max(G, 1));
  B.dZa.ensure(nh), B.dZb.ensure(nh), B.U.ensure(nh), B.dH.ensure(nh);
  for (int l = 0; l < 3; l++) {
    B.part_w[l].ensure((size_t)MP_GB * layer_k(l) * MP_HID);
    B.part_b[l].ensure((size_t)MP_GB * MP_HID);
  }
  B.part_head.ensure((size_t)MP_GB * (MP_HID + 1));
  B.grad.ensure(MP_NPARAM);
  B.d_gstart.ensure((size_t)std::max(G, 1)), B.d_gn.ensure((size_t)std::max(G, 1));
  h2d(B.d_gstart.p, v.gstart.data(), G);
  h2d(B.d_gn.p, v.gn.data(), G);
  CK(cudaMemsetAsync(B.dy.p, 0, (size_t)v.Npad * sizeof(float), st));
  if (G > 0) {
    k_mp_loss<<<G, 256, 0, st>>>(B.y.p, B.lab_pos.p, B.d_gstart.p, B.d_gn.p, G, B.dy.p, B.loss.p);
    CK_LAUNCH();
  }
  const Level &lv = *v.lv;
  const float *p = net.p;
  k_mp_head_bwd<<<MP_GB, MP_THREADS, 0, st>>>(B.dy.p, B.H[2].p, v.Npad, p + MP_OFF_WO, B.dZa.p,
                                              B.part_head.p);
  CK_LAUNCH();
  const unsigned gg = grid_for(v.Npad * 8, MP_THREADS);
  k_mp_bwd<MP_HID, true><<<MP_GB, MP_THREADS, 0, st>>>(B.dZa.p, B.H[1].p, B.AG[2].p, B.wsum.p,
                                                       v.Npad, net.Wb[2], B.dH.p, B.U.p,
                                                       B.part_w[2].p, B.part_b[2].p);
  CK_LAUNCH();
  k_mp_gather_bwd<<<gg, MP_THREADS, 0, st>>>(B.dH.p, B.U.p, B.H[1].p, lv.ell.p, lv.slice_off.p,
                                             lv.slice_w.p, v.N, v.Npad, B.dZb.p);
  CK_LAUNCH();
  k_mp_bwd<MP_HID, true><<<MP_GB, MP_THREADS, 0, st>>>(B.dZb.p, B.H[0].p, B.AG[1].p, B.wsum.p,
                                                       v.Npad, net.Wb[1], B.dH.p, B.U.p,
                                                       B.part_w[1].p, B.part_b[1].p);
  CK_LAUNCH();
  k_mp_gather_bwd<<<gg, MP_THREADS, 0, st>>>(B.dH.p, B.U.p, B.H[0].p, lv.ell.p, lv.slice_off.p,
                                             lv.slice_w.p, v.N, v.Npad, B.dZa.p);
  CK_LAUNCH();
  k_mp_bwd<MP_FIN, false, true><<<MP_GB, MP_THREADS, 0, st>>>(
      B.dZa.p, B.X.p, B.AG0.p, B.wsum.p, v.Npad, nullptr, nullptr, nullptr, B.part_w[0].p,
      B.part_b[0].p);
  CK_LAUNCH();
  k_mp_grad_reduce<<<grid_for(MP_NPARAM, 256), 256, 0, st>>>(
      B.part_w[0].p, B.part_b[0].p, B.part_w[1].p, B.part_b[1].p, B.part_w[2].p, B.part_b[2].p,
      B.part_head.p, MP_GB, B.grad.p);
  CK_LAUNCH();
  std::vector<double> hl(std::max(G, 1), 0.0);
  d2h(hl.data(), B.loss.p, (size_t)G);
  sync();
  double s = 0.0;
  for (int g = 0; g < G; g++) s += hl[g];
  return G ? s / G : 0.0;
}

}  // namespace

// ---------------------------------------------------------------------------
// Library-internal interface (warm.cuh)
// ---------------------------------------------------------------------------
void warm_net_install(const float *host_params) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) throw ArgError{PARRSB_ERR_UNSUPPORTED, "device index >= 64"};
  std::lock_guard<std::mutex> lk(g_net_mu);
  InstalledNet &n = g_net[dev];
  if (!n.p) {
    CK(cudaMalloc(&n.p, MP_NPARAM * sizeof(float)));
    for (int l = 0; l < 3; l++) {
      CK(cudaMalloc(&n.wf[l], (size_t)layer_k(l) * MP_HID * sizeof(bf16)));
      CK(cudaMalloc(&n.wb[l], (size_t)layer_k(l) * MP_HID * sizeof(bf16)));
    }
  }
  CK(cudaMemcpy(n.p, host_params, MP_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
  k_mp_pack<<<dim3(8, 3), 256>>>(n.p, n.wf[0], n.wf[1], n.wf[2], n.wb[0], n.wb[1], n.wb[2]);
  CK(cudaGetLastError());
  CK(cudaDeviceSynchronize());
  n.ready = true;
}

bool warm_net_ready() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return false;
  std::lock_guard<std::mutex> lk(g_net_mu);
  return g_net[dev].ready;
}

void element_spacings(const Graph &g, const double *cent, ll nel, int ndim, float4 *esp) {
  if (nel <= 0) return;
  k_elem_spacing<<<grid_for(nel, 256), 256, 0, ctx().stream>>>(
      g.rowptr.p, g.col.p, g.w.p, cent, nel, ndim == 3 ? 4u : 2u, esp);
  CK_LAUNCH();
}

void geometric_predict_level(const Level &lv, const int *perm, const int *grp,
                             const double *cent, ll nel, int ndim, const std::vector<ll> &gstart,
                             const std::vector<ll> &gn, ll N, double *y,
                             std::vector<int> *degen, const float4 *esp) {
  MpView v;
  v.lv = &lv, v.perm = perm, v.grp = grp, v.N = N, v.Npad = (N + MP_ROWS - 1) / MP_ROWS * MP_ROWS;
  v.gstart = gstart, v.gn = gn;
  DBuf<double> frame;
  mp_frames(v, cent, nel, ndim, frame, degen, esp);
  k_mp_geometric<<<grid_for(N, 256), 256, 0, ctx().stream>>>(perm, grp, cent, nel, frame.p, N, y);
  CK_LAUNCH();
}

void warm_predict_level(const Level &lv, const int *perm, const int *grp, const double *cent,
                        ll nel, int ndim, const std::vector<ll> &gstart,
                        const std::vector<ll> &gn, ll N, double *y, std::vector<int> *degen,
                        const float4 *esp) {
  int dev = 0;
  CK(cudaGetDevice(&dev));
  NetDev net;
  {
    std::lock_guard<std::mutex> lk(g_net_mu);
    const InstalledNet &n = g_net[dev];
    if (!n.ready) throw ArgError{PARRSB_ERR_ARGS, "no warm-start network installed"};
    for (int l = 0; l < 3; l++) net.Wf[l] = n.wf[l], net.Wb[l] = n.wb[l];
    net.p = n.p;
  }
  MpView v;
  v.lv = &lv, v.perm = perm, v.grp = grp, v.N = N, v.Npad = (N + MP_ROWS - 1) / MP_ROWS * MP_ROWS;
  v.gstart = gstart, v.gn = gn;
  MpBuffers B;
  mp_features(v, cent, nel, ndim, B, degen, esp);
  mp_forward(v, net, B, false);
  k_mp_y_to_double<<<grid_for(N, 256), 256, 0, ctx().stream>>>(B.y.p, grp, N, y);
  CK_LAUNCH();
}

}  // namespace prsb

// ---------------------------------------------------------------------------
// C ABI of the warm start (include/parrsb.h)
// ---------------------------------------------------------------------------
using namespace prsb;

struct parrsb_warm_batch {
  GroupLevel gl;
  DBuf<double> cent;
  int ndim = 3;
  ll nel = 0;
  MpView view;
  MpBuffers B;
  PackedNet pk;
  int device = 0;
};

namespace {
template <typename F>
int warm_guarded(F &&fn) {
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
}  // namespace

extern "C" PARRSB_API int parrsb_warm_install(const float *params) {
  if (!params) return PARRSB_ERR_ARGS;
  return warm_guarded([&]() -> int {
    warm_net_install(params);
    return PARRSB_OK;
  });
}

extern "C" PARRSB_API int parrsb_warm_batch_create(parrsb_warm_batch **batch,
                                                   const long long *d_vtx, const double *d_xyz,
                                                   const int *d_group, int nel, int nv,
                                                   int ngroups) {
  if (!batch || nel < 1 || !d_vtx || !d_xyz || !d_group || (nv != 8 && nv != 4) || ngroups < 1)
    return PARRSB_ERR_ARGS;
  *batch = nullptr;
  return warm_guarded([&]() -> int {
    ctx().init();
    parrsb_warm_batch *b = new parrsb_warm_batch();
    b->device = ctx().device;
    try {
      b->nel = nel;
      b->ndim = nv == 8 ? 3 : 2;
      build_group_level(d_vtx, nel, nv, d_group, ngroups, b->gl);
      b->cent.ensure((size_t)3 * nel);
      compute_centroids(d_xyz, nel, nv, b->cent.p);
      MpView &v = b->view;
      v.lv = &b->gl.lv, v.perm = b->gl.perm.p, v.grp = b->gl.grp.p, v.N = nel;
      v.Npad = ((ll)nel + MP_ROWS - 1) / MP_ROWS * MP_ROWS;
      for (int g = 0; g < ngroups; g++)  // groups with at least two elements
        if (b->gl.gn[g] >= 2) v.gstart.push_back(b->gl.gstart[g]), v.gn.push_back(b->gl.gn[g]);
      mp_features(v, b->cent.p, nel, b->ndim, b->B);
      sync();
    } catch (...) {
      delete b;
      throw;
    }
    *batch = b;
    return PARRSB_OK;
  });
}

extern "C" PARRSB_API int parrsb_warm_batch_destroy(parrsb_warm_batch *batch) {
  if (!batch) return PARRSB_OK;
  return warm_guarded([&]() -> int {
    int cur = 0;
    CK(cudaGetDevice(&cur));
    CK(cudaSetDevice(batch->device));
    ctx().init();
    delete batch;
    sync();
    CK(cudaSetDevice(cur));
    return PARRSB_OK;
  });
}

extern "C" PARRSB_API int parrsb_warm_batch_features(parrsb_warm_batch *batch, float *d_feat) {
  if (!batch || !d_feat) return PARRSB_ERR_ARGS;
  return warm_guarded([&]() -> int {
    ctx().init();
    const ll N = batch->nel;
    k_mp_feat_to_elem<<<grid_for(N * MP_FIN, 256), 256, 0, ctx().stream>>>(
        batch->gl.perm.p, batch->B.X.p, N, d_feat);
    CK_LAUNCH();
    sync();
    return PARRSB_OK;
  });
}

extern "C" PARRSB_API int parrsb_warm_batch_step(parrsb_warm_batch *batch, const float *d_params,
                                                 const double *d_label, float *d_grad,
                                                 float *d_pred, double *loss) {
  if (!batch || !d_params || (d_grad && !d_label)) return PARRSB_ERR_ARGS;
  return warm_guarded([&]() -> int {
    ctx().init();
    cudaStream_t st = ctx().stream;
    const MpView &v = batch->view;
    MpBuffers &B = batch->B;
    batch->pk.pack(const_cast<float *>(d_params));
    NetDev net = batch->pk.dev(const_cast<float *>(d_params));
    const bool train = d_label != nullptr;
    mp_forward(v, net, B, train);
    if (d_pred) {
      k_mp_pred_to_elem<<<grid_for(v.N, 256), 256, 0, st>>>(v.perm, B.y.p, v.N, d_pred);
      CK_LAUNCH();
    }
    if (train) {
      B.lab_pos.ensure((size_t)v.Npad);
      k_mp_to_pos<<<grid_for(v.N, 256), 256, 0, st>>>(v.perm, d_label, v.N, B.lab_pos.p);
      CK_LAUNCH();
      const double l = mp_backward(v, net, B);
      if (loss) *loss = l;
      if (d_grad)
        CK(cudaMemcpyAsync(d_grad, B.grad.p, MP_NPARAM * sizeof(float), cudaMemcpyDeviceToDevice,
                           st));
    }
    sync();
    return PARRSB_OK;
  });
}

extern "C" PARRSB_API int parrsb_warm_adam(float *d_params, float *d_m, float *d_v,
                                           const float *d_grad, int n, int step, float lr) {
  if (!d_params || !d_m || !d_v || !d_grad || n < 1 || step < 1) return PARRSB_ERR_ARGS;
  return warm_guarded([&]() -> int {
    ctx().init();
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = (float)(1.0 - pow(0.9, step)), c2 = (float)(1.0 - pow(0.999, step));
    k_mp_adam<<<grid_for(n, 256), 256, 0, ctx().stream>>>(d_params, d_m, d_v, d_grad, n, lr, b1,
                                                         b2, 1e-8f, c1, c2);
    CK_LAUNCH();
    sync();
    return PARRSB_OK;
  });
}
