"""The FP64 restatement of the warm-start network (oracle/warm_oracle.py),
checked on the CPU: its gradient against central finite differences, its
features against first principles (an axis-aligned box), and the BF16
rounding against exhaustive known values."""
import numpy as np

from oracle import warm_oracle as W
from parrsb_gb300 import meshgen


def _graph(vtx, group):
    from oracle import oracle as O
    rp, col, w = O.dual_graph(vtx)
    return W.restrict(rp, col, w, group)


def _params(seed, scale=0.3):
    rng = np.random.default_rng(seed)
    p = rng.normal(0.0, scale, W.NPARAM)
    return p


def test_bf16_rounding_known_values():
    x = np.array([1.0, 1.00390625, 1.005859375, 3.14159265, -2.5e-3, 0.0], np.float32)
    r = W.bf16_round(x)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: even mantissa -> 1
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert r[3] == 3.140625 and r[5] == 0.0
    assert abs(r[4] - (-2.5e-3)) < 2.5e-3 * 2 ** -8


def test_features_axis_aligned_box():
    """A 12 x 6 x 3 unjittered box: the first axis is x and spans about
    [-1, 1] (uniform distribution: sqrt(3) sigma), interior degree 56."""
    vtx, xyz = meshgen.box_hex(12, 6, 3, jitter=0.0)
    from oracle import oracle as O
    cent = O.centroids(xyz, 8)
    group = np.zeros(len(vtx), np.int64)
    rows, col, w = _graph(vtx, group)
    X = W.features(cent, group, rows, col, w)
    assert np.allclose(np.abs(X[:, 0]).max(), 11 / 12 * np.sqrt(12 ** 2 / (12 ** 2 - 1)), rtol=1e-9)
    assert np.all(np.diff(X[:12, 0]) > 0)  # x increases along the first row
    assert np.isclose(X[:, 3].max(), 1.0)
    np.testing.assert_allclose(X[:, 4], -np.sin(np.pi * X[:, 0] / 2))
    assert np.all(X[:, 5:] == 0)


def test_gradient_matches_finite_differences():
    vtx, xyz, seg = meshgen.subboxes(3, smin=30, smax=80, delete=0.1, seed=5)
    from oracle import oracle as O
    cent = O.centroids(xyz, 8)
    group = seg.astype(np.int64)
    rows, col, w = _graph(vtx, group)
    X = W.features(cent, group, rows, col, w)
    rng = np.random.default_rng(1)
    label = rng.normal(size=len(vtx))
    p = _params(2)
    L, g = W.gradient(X, rows, col, w, p, label, group, round_weights=False)
    idx = rng.choice(W.NPARAM, 60, replace=False)
    idx = np.concatenate([idx, [W.OFF["bo"][0], W.OFF["wo"][0], W.OFF["b1"][0]]])
    eps = 1e-6
    for q in idx:
        pp, pm = p.copy(), p.copy()
        pp[q] += eps
        pm[q] -= eps
        fp = W.loss_and_dy(W.forward(X, rows, col, w, pp, False)[0], label, group)[0]
        fm = W.loss_and_dy(W.forward(X, rows, col, w, pm, False)[0], label, group)[0]
        fd = (fp - fm) / (2 * eps)
        assert abs(fd - g[q]) <= 1e-5 * max(1.0, abs(fd)) + 1e-7, (q, fd, g[q])
    # the loss of the label itself is zero, and it is sign invariant
    assert abs(W.loss_and_dy(label, label, group)[0]) < 1e-12
    assert abs(W.loss_and_dy(-3 * label + 2, label, group)[0]) < 1e-12
