"""Batched level solve (config 4 shape, reduced): Fiedler vectors of many
independent subgraphs in one segmented launch sequence.  Checked against
the oracle's Lanczos per subgraph and against one-subgraph-at-a-time
launches, which must give bitwise the same vectors (per-group reductions
have a fixed order regardless of the other groups)."""
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


@pytest.fixture(scope="module")
def mesh():
    return meshgen.subboxes(24, smin=60, smax=2000, delete=0.05, seed=4)


def test_batched_equals_per_group(mesh):
    vtx, xyz, seg = mesh
    ng = int(seg.max()) + 1
    fb, ib, rb = P.fiedler_groups(vtx, seg, ng, batched=True)
    fs, is_, rs = P.fiedler_groups(vtx, seg, ng, batched=False)
    np.testing.assert_array_equal(fb, fs)
    np.testing.assert_array_equal(ib, is_)


def test_batched_matches_oracle(oracle, mesh):
    vtx, xyz, seg = mesh
    ng = int(seg.max()) + 1
    f, it, rs = P.fiedler_groups(vtx, seg, ng, batched=True)
    for g in range(ng):
        m = seg == g
        fo, ito = oracle.fiedler(vtx[m], 50, 50, 1e-5)
        fg = f[m]
        assert abs(np.linalg.norm(fg) - 1.0) < 1e-9
        ncomp = oracle.components(vtx[m])
        if ncomp == 1:
            # same eigenvector up to sign, same step count within one restart,
            # and the same FP64 eigen-residual as the oracle's vector.  (The
            # reference stops on the CG residual |r_k| < tol |r_0|, which on
            # these small subgraphs leaves eigen-residuals far above tol; the
            # GPU reproduces that, it does not hide it.)
            assert abs(abs(fg @ fo) - 1.0) < 1e-4, (g, fg @ fo)
            assert abs(int(it[g]) - ito) <= 50
            yo = oracle.laplacian(fo, vtx[m])
            ro = np.linalg.norm(yo - (fo @ yo) * fo)
            assert abs(rs[g] - ro) <= 1e-3 * ro + 1e-6, (g, rs[g], ro)
        else:
            # disconnected subgraph (deleted elements): lambda_2 = 0 and the
            # vector lies in a degenerate null space; only its norm is defined
            assert np.isfinite(rs[g])


def test_batched_fp32(monkeypatch, mesh):
    vtx, xyz, seg = mesh
    ng = int(seg.max()) + 1
    f64, _, _ = P.fiedler_groups(vtx, seg, ng)
    monkeypatch.setenv("PARRSB_GPU_FP32", "1")
    f32, _, rs = P.fiedler_groups(vtx, seg, ng)
    for g in range(ng):
        m = seg == g
        if m.sum() > 100:
            assert abs(abs(f32[m] @ f64[m]) - 1.0) < 1e-3


def test_fp32_residual_check_matches_fp64(oracle, monkeypatch, mesh):
    """With FP32 vectors the residual check computes L f exactly in 64-bit
    fixed point: the reported ||L f - rho f|| / ||f|| of every returned
    vector equals the FP64 value computed from that vector to 1e-8."""
    vtx, xyz, seg = mesh
    ng = int(seg.max()) + 1
    monkeypatch.setenv("PARRSB_GPU_FP32", "1")
    f, _, rs = P.fiedler_groups(vtx, seg, ng)
    for g in range(ng):
        m = seg == g
        fg = f[m]
        y = oracle.laplacian(fg, vtx[m])
        rho = (fg @ y) / (fg @ fg)
        ro = np.linalg.norm(y - rho * fg) / np.linalg.norm(fg)
        assert abs(rs[g] - ro) <= 1e-8 * ro + 1e-13, (g, rs[g], ro)
