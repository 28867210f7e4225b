"""Failure handling on the GPU path without faulting the GPU: a host-side
injected failure (PARRSB_FAULT) makes a stage return an error code; the
library unwinds cleanly and the next call succeeds with the same result."""
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
    yield


@pytest.mark.parametrize("stage", ["upload", "partition"])
def test_injected_fault_unwinds(monkeypatch, stage):
    vtx, xyz = meshgen.box_hex(8, 8, 4, jitter=0.1, seed=1)
    good = P.part_mesh(vtx, xyz, 4, partitioner=0)
    monkeypatch.setenv("PARRSB_FAULT", stage)
    with pytest.raises(P.ParrsbError) as ei:
        P.part_mesh(vtx, xyz, 4, partitioner=0)
    assert ei.value.code == P.ERR_CHECK
    monkeypatch.delenv("PARRSB_FAULT")
    again = P.part_mesh(vtx, xyz, 4, partitioner=0)
    np.testing.assert_array_equal(good, again)


def test_unsupported_options_do_not_touch_gpu_state():
    vtx, xyz = meshgen.box_hex(4, 4, 4, jitter=0.1, seed=2)
    with pytest.raises(P.ParrsbError) as ei:
        P.part_mesh(vtx, xyz, 4, partitioner=0, rsb_max_iter=500)
    assert ei.value.code == P.ERR_UNSUPPORTED
    part = P.part_mesh(vtx, xyz, 4, partitioner=1)
    assert np.bincount(part).tolist() == [16] * 4
