// periodic.cuh -- periodic-face matching after gencon.
#pragma once
#include "sort.cuh"
#include "util.cuh"

namespace prsb {

// d_ids: np = nel * nv 0-based gencon ids (sequence order, symmetric corner
// numbering), renumbered in place; d_x0..2: the points' coordinates in the
// same order; pinfo: npf host records (element, face, partner element,
// partner face), 1-based, preprocessor face numbering.  Returns 0,
// PARRSB_ERR_ARGS for a record out of range, PARRSB_ERR_CHECK when matched
// faces do not coincide after centring.  *nseg_out: distinct ids after.
int periodic_device(ll *d_ids, const double *d_x0, const double *d_x1, const double *d_x2,
                    ll nel, int ndim, ll nseg, const long long *pinfo, int npf, SortWs &sws,
                    ll *nseg_out);

// d_out[i] = d_ids[i] + 1 (the 1-based ids of the C ABI)
void plus_one(const ll *d_ids, ll n, long long *d_out);

}  // namespace prsb
