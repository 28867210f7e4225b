// util.cuh -- device scans and small helpers shared by the kernels.
#pragma once
#include "common.cuh"

namespace prsb {

// out[i] = sum_{j<i} in[j] (exclusive); returns the total (synchronises).
// `in` and `out` may alias.
ll exclusive_scan_ll(const ll *in, ll *out, ll n);
// Same for int inputs; output int64.
ll exclusive_scan_int_to_ll(const int *in, ll *out, ll n);
// the same without returning the total: nothing waits on the device
void exclusive_scan_int_to_ll_async(const int *in, ll *out, ll n);

// Segment table kept on the device (structure of arrays).
struct SegTable {
  DBuf<ll> start, n;
  DBuf<int> p, r0;
  ll count = 0;
  void reserve(ll c) {
    start.ensure((size_t)c);
    n.ensure((size_t)c);
    p.ensure((size_t)c);
    r0.ensure((size_t)c);
  }
};

// seg_of_pos[i] = index of the segment containing position i, for segments
// that tile [0, N) contiguously in order.
void fill_seg_of_pos(const SegTable &t, int *seg_of_pos, ll N);

}  // namespace prsb
