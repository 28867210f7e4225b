"""Repair of disconnected parts (parrsb_options.repair = 1), a meaning this
library gives to an option the reference parses and ignores
(src/parrsb.c:65): every part keeps its largest component, every other
component joins the neighbouring part it shares the most dual-graph weight
with.  Checked bit-exact against the restatement in oracle/oracle.py, on
meshes whose parts fall apart (sub-boxes with deleted elements, as in the
batched level-solve workload), and the default (repair = 0) changes
nothing."""
import numpy as np
import pytest

import parrsb_gb300 as P
from parrsb_gb300 import meshgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _gpu(lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    yield
    P.finalize()


@pytest.mark.parametrize("partitioner,seed", [(0, 4), (0, 5), (1, 6), (2, 7)])
def test_repair_matches_restatement(oracle, partitioner, seed):
    vtx, xyz, _ = meshgen.subboxes(10, smin=60, smax=700, delete=0.1, seed=seed)
    nparts = 24
    base = P.part_mesh(vtx, xyz, nparts, partitioner=partitioner)
    assert P.last_stats().repair_components == 0
    fixed = P.part_mesh(vtx, xyz, nparts, partitioner=partitioner, repair=1)
    st = P.last_stats()
    want, mc, me = oracle.repair_parts(base, vtx, nparts)
    np.testing.assert_array_equal(fixed, want)
    assert st.repair_components == mc and st.repair_elements == me
    assert mc > 0  # these meshes do fall apart
    # after the repair no part has more components than before
    before = P.components(vtx, base, nparts)
    after = P.components(vtx, fixed, nparts)
    assert after.sum() <= before.sum() - mc // 2


def test_repair_leaves_connected_parts_alone(oracle):
    vtx, xyz = meshgen.box_hex(20, 16, 12, jitter=0.1, seed=3)
    a = P.part_mesh(vtx, xyz, 16, partitioner=1)
    b = P.part_mesh(vtx, xyz, 16, partitioner=1, repair=1)
    want, mc, _ = oracle.repair_parts(a, vtx, 16)
    np.testing.assert_array_equal(b, want)
    if mc == 0:
        np.testing.assert_array_equal(a, b)
