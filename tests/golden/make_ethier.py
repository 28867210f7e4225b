"""Writes tests/golden/ethier.npz from the reference's example mesh
examples/ethier.re2 (32 hex elements, the mesh the reference's CI runs
through gencon and genmap): its corner coordinates as read by the library's
.re2 reader, the oracle's gencon ids at tol 0.2, and the oracle's RCB and RSB
partitions of the numbered mesh into 4 parts.

Run in a checkout that has the reference tree:
    python tests/golden/make_ethier.py <reference>/examples/ethier
The GPU machine has no reference tree; the tests read the .npz.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def main(stem):
    import parrsb_gb300 as P
    from oracle import oracle as O
    m = P.read_mesh(stem, read=1)
    coord = np.ascontiguousarray(m["coord"], np.float64)
    rc, vtx, _, nseg = O.conn_mesh(coord, 3, 0.2)
    assert rc == 0
    rc1, rcb, _, _, _ = O.part_mesh(vtx, coord, 4, partitioner=1)
    rc0, rsb, _, info, _ = O.part_mesh(vtx, coord, 4, partitioner=0)
    assert rc1 == 0 and rc0 == 0
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ethier.npz")
    np.savez_compressed(out, coord=coord, periodic=np.asarray(m["periodic"], np.int64),
                        vtx=vtx, nseg=np.int64(nseg), rcb4=rcb, rsb4=rsb,
                        rsb4_iters=np.int64(info.total_iters))
    print(out, coord.shape, "distinct ids", nseg)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else
         os.environ.get("PARRSB_ETHIER", "examples/ethier"))
