// gencon.cuh -- tolerance-based vertex numbering (parrsb_conn_mesh).
#pragma once
#include "sort.cuh"
#include "util.cuh"

namespace prsb {

struct GenconWs {
  SortWs sort;
  DBuf<double> x[3], dx;
  DBuf<u64> keys;
  DBuf<int> ord, vals, flag, seg_of_pt;
  DBuf<ll> segid, ids;
};

// Device-resident gencon.  d_coord: nel*nv*ndim corner coordinates in
// preprocessor order; d_vtx (may be null): nel*nv ids (1-based) written only
// on success.  Returns 0, or 1 when the element / face check fails.
// d_ids_out (optional): 0-based segment ids in sequence order, written even
// when a check fails.
int gencon_device(long long *d_vtx, const double *d_coord, ll nel, int ndim,
                  double tol, GenconWs &ws, ll *nseg_out, ll *d_ids_out);

}  // namespace prsb
