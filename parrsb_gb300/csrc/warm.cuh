// warm.cuh -- learned warm start for the Fiedler vectors of an RSB level: a
// three-layer message-passing network on the level's graph, with
// hand-written BF16 forward and backward kernels (tensor-core MMA, FP32
// accumulation) and its own training step.
#pragma once
#include <vector>

#include "rsb.cuh"

namespace prsb {

// Network shape.  Per element: 8 input features (the element centroid in
// its group's principal frame, scaled so the longest axis spans about
// [-1, 1]; the element's weighted degree / 56; the geometric guess
// g = -sin(pi x~_1 / 2); three zeros), three layers
//   h_l = relu([h_{l-1} | mean_w(h_{l-1} over the graph neighbours)] W_l + b_l)
// of width 64, and a head that corrects the guess: y = g + h_3 . wo + bo.
constexpr int MP_HID = 64;
constexpr int MP_FIN = 8;
constexpr int MP_K1 = 2 * MP_FIN;   // 16
constexpr int MP_K2 = 2 * MP_HID;   // 128
// Offsets in the flat FP32 parameter vector (W_l row-major [k][n]).
constexpr int MP_OFF_W1 = 0;
constexpr int MP_OFF_B1 = MP_OFF_W1 + MP_K1 * MP_HID;
constexpr int MP_OFF_W2 = MP_OFF_B1 + MP_HID;
constexpr int MP_OFF_B2 = MP_OFF_W2 + MP_K2 * MP_HID;
constexpr int MP_OFF_W3 = MP_OFF_B2 + MP_HID;
constexpr int MP_OFF_B3 = MP_OFF_W3 + MP_K2 * MP_HID;
constexpr int MP_OFF_WO = MP_OFF_B3 + MP_HID;
constexpr int MP_OFF_BO = MP_OFF_WO + MP_HID;
constexpr int MP_NPARAM = MP_OFF_BO + 1;  // 17,665

// Installs network parameters (host FP32, MP_NPARAM values) for the current
// device; warm_net_ready() tells whether the current device has some.
void warm_net_install(const float *host_params);
bool warm_net_ready();

// Predicted Fiedler vectors of the groups [gstart[g], gstart[g] + gn[g]) of
// a level (perm: element at each position; grp: group of each position, -1
// for none; cent: centroids [3][nel] in element order): y[i] for every
// position i (0 outside the groups), FP64, on the library stream.  degen
// (optional, host): per group, 1 when the two largest variances of its
// centroids are within 5% (two axes of nearly the same length: the leading
// eigenvalues of the group's Laplacian are nearly equal, and no prediction
// can say which combination Lanczos will settle on; the reference's step
// start keeps the split of the pre-partition).
void warm_predict_level(const Level &lv, const int *perm, const int *grp, const double *cent,
                        ll nel, int ndim, const std::vector<ll> &gstart,
                        const std::vector<ll> &gn, ll N, double *y,
                        std::vector<int> *degen = nullptr, const float4 *esp = nullptr);

// The geometric start of the same groups: -sin(pi x~_1 / 2) along each
// group's principal axis (x~_1 as in the network's first input feature).
void geometric_predict_level(const Level &lv, const int *perm, const int *grp,
                             const double *cent, ll nel, int ndim, const std::vector<ll> &gstart,
                             const std::vector<ll> &gn, ll N, double *y,
                             std::vector<int> *degen = nullptr, const float4 *esp = nullptr);

// Per element, over its face neighbours in the dual graph g (weight 4 in 3D,
// 2 in 2D): the sums of the squared centroid differences per axis and the
// neighbour count (the element-spacing input of the frames; esp may then be
// passed to the predictions above instead of their per-level pass).
void element_spacings(const Graph &g, const double *cent, ll nel, int ndim, float4 *esp);

}  // namespace prsb
