"""GPU integer parity: the integer stages of the path, bit-exact against the
oracle, through the C ABI.

- the element dual graph RSB builds its Laplacian on (rows, columns and
  shared-vertex weights; src/laplacian.c:159-205, src/mat.c:17-61);
- component counts per group (get_components_v2, src/components.c:160-328)
  and inside RSB's bisections;
- gencon's face check (src/con-check.c:197-263) on the GPU;
- the reference's own example mesh (examples/ethier.re2, as the committed
  fixture tests/golden/ethier.npz) through GPU gencon, RCB and RSB;
- RCB and RIB of the full 512 x 512 quad annulus into 1024 parts.
"""
import os

import numpy as np
import pytest

import parrsb_gb300 as P
from parrsb_gb300 import meshgen

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def _gpu(lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    yield
    P.finalize()


def _rows_sorted(rowptr, col, w):
    """(row, col, weight) triples with each row's columns in increasing order."""
    rows = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    o = np.lexsort((col, rows))
    return rows[o], col[o].astype(np.int64), w[o].astype(np.int64)


def _meshes():
    out = {}
    out["box16"] = meshgen.box_hex(16, 16, 16, jitter=0.1, seed=0)[0]
    v, _, _ = meshgen.subboxes(6, smin=50, smax=600, delete=0.1, seed=3)
    out["subboxes_deleted"] = v
    out["annulus_quad"] = meshgen.annulus_quad(48, 16, amp=0.02, seed=1)[0]
    out["pipe"] = meshgen.pipe_hex(24, 4, 6, jitter=0.05, seed=2)[0]
    # repeated vertex ids inside elements (weights above the corner count)
    v = meshgen.box_hex(6, 5, 4, jitter=0.0)[0].copy()
    v[::7, 1] = v[::7, 0]
    out["repeated_ids"] = v
    return out


@pytest.mark.parametrize("name", list(_meshes().keys()))
def test_dual_graph_bit_exact(oracle, name):
    vtx = _meshes()[name]
    rp, col, w = P.dual_graph(vtx)
    rpo, colo, wo = oracle.dual_graph(vtx)
    np.testing.assert_array_equal(rp, rpo)
    a = _rows_sorted(rp, col, w)
    b = _rows_sorted(rpo, colo, wo)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    # first-occurrence order inside a row is a permutation of the sorted row
    assert P.last_stats().kernel_launches > 0


def test_dual_graph_hex_stencil_weights():
    """Interior rows of an unjittered box: 26 neighbours, weights 4/2/1."""
    vtx, _ = meshgen.box_hex(5, 5, 5, jitter=0.0)
    rp, col, w = P.dual_graph(vtx)
    e = 2 + 5 * (2 + 5 * 2)
    row_w = np.sort(w[rp[e]:rp[e + 1]])
    assert len(row_w) == 26
    assert row_w.tolist() == [1] * 8 + [2] * 12 + [4] * 6


@pytest.mark.parametrize("seed", [1, 2])
def test_components_bit_exact(oracle, seed):
    vtx, _, seg = meshgen.subboxes(10, smin=80, smax=1500, delete=0.12, seed=seed)
    rng = np.random.default_rng(seed)
    # groups: whole sub-boxes, halves of sub-boxes by index, and left-out
    # elements (-1)
    group = seg.copy()
    half = rng.integers(0, 2, len(seg))
    group = (2 * group + half).astype(np.int32)
    group[rng.random(len(seg)) < 0.03] = -1
    ng = int(group.max()) + 2  # one empty group at the end
    got = P.components(vtx, group, ng)
    want = np.array([oracle.components(vtx, (group == g).astype(np.int32))
                     for g in range(ng)], np.int32)
    np.testing.assert_array_equal(got, want)
    assert got[-1] == 0 and got.max() > 1


@pytest.mark.parametrize("seed", [4, 7])
def test_rsb_component_counts_match_oracle(oracle, seed):
    """The largest component count over all halves of all bisections of an
    RSB run equals the oracle's (both count the halves of the same sorted
    groups when the partitions agree)."""
    vtx, xyz, _ = meshgen.subboxes(6, smin=60, smax=500, delete=0.08, seed=seed)
    part = P.part_mesh(vtx, xyz, 8, partitioner=0)
    st = P.last_stats()
    rc, ref, _, info, _ = oracle.part_mesh(vtx, xyz, 8, partitioner=0)
    assert rc == 0
    if np.array_equal(part, ref):
        assert st.max_components == info.max_components
    # the halves of the GPU's own partition, counted by the oracle
    worst = 0
    for p in range(8):
        worst = max(worst, oracle.components(vtx, (part == p).astype(np.int32)))
    assert worst >= 1


def test_face_check_fails_like_the_oracle(oracle):
    """Two hexes sharing a face, one corner of the shared face moved by 0.3 h
    in the second element: gencon numbers it apart (gap > tol h), so the
    second element holds exactly 3 of the first one's face corners.
    element_check passes and face_check fails, on the GPU and in the
    oracle, with the same return code; vtx is left untouched."""
    _, xyz = meshgen.box_hex(2, 1, 1, jitter=0.0)
    xyz = xyz.copy()
    hit = np.flatnonzero((xyz[1, :, 0] == 0.5) & (xyz[1, :, 1] == 1.0) & (xyz[1, :, 2] == 1.0))
    assert len(hit) == 1
    xyz[1, hit[0], 2] = 1.3
    rc, _, _, _ = oracle.conn_mesh(xyz, 3, 0.2)
    assert rc == 1
    with pytest.raises(P.ParrsbError) as ei:
        P.conn_mesh(xyz, 3, 0.2)
    assert ei.value.code == 1
    # without the displaced corner both succeed
    _, good = meshgen.box_hex(2, 1, 1, jitter=0.0)
    np.testing.assert_array_equal(P.conn_mesh(good, 3, 0.2), oracle.conn_mesh(good, 3, 0.2)[1])


def test_ethier_mesh_through_gpu(oracle):
    """The reference's example mesh (32 hex elements): GPU gencon ids equal
    the oracle's (fixture), then GPU RCB equals the oracle's parts and GPU
    RSB has the oracle's part sizes and a cut within 1%."""
    g = np.load(os.path.join(GOLDEN, "ethier.npz"))
    ids = P.conn_mesh(g["coord"], 3, 0.2)
    np.testing.assert_array_equal(ids, g["vtx"])
    assert P.last_stats().gencon_segments == int(g["nseg"])
    rcb = P.part_mesh(ids, g["coord"], 4, partitioner=1)
    np.testing.assert_array_equal(rcb, g["rcb4"])
    rsb = P.part_mesh(ids, g["coord"], 4, partitioner=0)
    np.testing.assert_array_equal(np.bincount(rsb, minlength=4),
                                  np.bincount(g["rsb4"], minlength=4))
    q = oracle.part_quality(rsb, ids, 4)
    qr = oracle.part_quality(g["rsb4"], ids, 4)
    assert abs(q[0] - qr[0]) <= 0.01 * qr[0]


@pytest.mark.parametrize("partitioner", [1, 2])
def test_bisection_annulus_512_to_1024_bit_exact(oracle, partitioner):
    """The full 512 x 512 quad annulus (262,144 elements) into 1024 parts:
    parts and within-part order equal the oracle's."""
    vtx, xyz = meshgen.annulus_quad(512, 512, amp=0.02, seed=0)
    part, seq = P.part_mesh_seq(vtx, xyz, 1024, partitioner=partitioner)
    rc, ref, order, _, _ = oracle.part_mesh(vtx, xyz, 1024, partitioner=partitioner,
                                            want_order=True)
    assert rc == 0
    np.testing.assert_array_equal(part, ref)
    pos = np.empty(len(order), np.int64)
    pos[order] = np.arange(len(order))
    first = np.full(1024, len(order), np.int64)
    np.minimum.at(first, ref, pos)
    np.testing.assert_array_equal(seq, pos - first[ref])
