"""FP64 restatement of the warm-start network (parrsb_gb300/csrc/warm.cu):
group frames and input features, forward pass, the sign-invariant cosine
loss and its gradient with respect to every parameter.

Test infrastructure only: the tests use it to check the GPU's features,
forward pass and gradients; the product never imports it.  It has no
counterpart in the reference (parRSB starts Lanczos from a step vector,
src/fiedler.c:574-578); the network it restates is this project's own.

Parameters are the flat FP32 vector of the library (W_l row-major [k][n]):
    W1 [16][64], b1 [64], W2 [128][64], b2, W3 [128][64], b3, wo [64], bo
The graph is the dual graph restricted to each group (CSR with integer
weights), rows in the same element order as the features.
"""
import numpy as np

HID, FIN = 64, 8
K1, K2 = 2 * FIN, 2 * HID
OFF = {}
_o = 0
for _name, _size in (("W1", K1 * HID), ("b1", HID), ("W2", K2 * HID), ("b2", HID),
                     ("W3", K2 * HID), ("b3", HID), ("wo", HID), ("bo", 1)):
    OFF[_name] = (_o, _o + _size)
    _o += _size
NPARAM = _o
DEG_SCALE = 1.0 / 56.0


def unpack(p):
    p = np.asarray(p, np.float64)
    get = lambda k: p[OFF[k][0]:OFF[k][1]]
    return {"W1": get("W1").reshape(K1, HID), "b1": get("b1"),
            "W2": get("W2").reshape(K2, HID), "b2": get("b2"),
            "W3": get("W3").reshape(K2, HID), "b3": get("b3"),
            "wo": get("wo"), "bo": get("bo")[0]}


def pack(d):
    out = np.zeros(NPARAM, np.float64)
    for k, (a, b) in OFF.items():
        out[a:b] = np.ravel(d[k]) if k != "bo" else [d[k]]
    return out


def bf16_round(x):
    """Round FP32 values to the nearest BF16 (ties to even), as float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def restrict(rowptr, col, w, group):
    """The dual graph keeping only edges inside a group (group >= 0)."""
    rows = np.repeat(np.arange(len(rowptr) - 1), np.diff(rowptr))
    keep = (group[rows] >= 0) & (group[rows] == group[col])
    return rows[keep], np.asarray(col)[keep], np.asarray(w, np.float64)[keep]


def spacings(cent, group, rows, cols, w, wface=4):
    """Per group and axis: 1 / h_a with h_a^2 the mean of (c_i,a - c_j,a)^2
    over the face neighbour pairs (weight wface) inside the group."""
    out = {}
    face = w == wface
    for g in np.unique(group[group >= 0]):
        sel = face & (group[rows] == g)
        d = cent[rows[sel]] - cent[cols[sel]]
        cnt = sel.sum()
        h2 = (d * d).sum(axis=0) / cnt if cnt else np.zeros(3)
        out[int(g)] = np.where(h2 > 0, 1.0 / np.sqrt(np.where(h2 > 0, h2, 1.0)), 1.0)
    return out


def frames(cent, group, rows, cols, w):
    """Per group: mean, principal axes (rows, largest variance first, largest
    component positive) and 1 / sqrt(3 l1 / n), all of the centroids
    measured in element spacings (spacings()).  When the two largest
    variances are within 5% the axes are the coordinate axes with RCB's cut
    axis first (longest edge of the raw centroids' bounding box, ties to the
    lower axis) and l1 is the scatter along it."""
    out = {}
    sp = spacings(cent, group, rows, cols, w)
    for g in np.unique(group[group >= 0]):
        c = cent[group == g] * sp[int(g)]
        n = len(c)
        mu = c.mean(axis=0)
        d = c - mu
        A = d.T @ d
        lam, V = np.linalg.eigh(A)
        o = np.argsort(-lam, kind="stable")
        lam, R = lam[o], V[:, o].T.copy()
        if lam[0] > 0 and lam[0] - lam[1] <= 0.05 * lam[0]:
            raw = cent[group == g]
            ext = raw.max(axis=0) - raw.min(axis=0)
            ax = 0  # (a 2D mesh has ext[2] = 0, which is never strictly longer)
            for a in range(1, 3):
                if ext[a] > ext[ax]:
                    ax = a
            R = np.eye(3)[[ax] + [a for a in range(3) if a != ax]]
            lam = lam.copy()
            lam[0] = A[ax, ax]
        for a in range(3):
            if R[a, np.argmax(np.abs(R[a]))] < 0:
                R[a] = -R[a]
        inv_s = 1.0 / np.sqrt(3.0 * lam[0] / n) if lam[0] > 0 else 0.0
        out[int(g)] = (mu, R, inv_s, sp[int(g)])
    return out


def features(cent, group, rows, cols, w):
    """Input features per element: x~ (3), weighted degree / 56, the
    geometric guess -sin(pi x~_1 / 2), zeros."""
    X = np.zeros((len(cent), FIN))
    for g, (mu, R, inv_s, k) in frames(cent, group, rows, cols, w).items():
        sel = group == g
        X[sel, :3] = ((cent[sel] * k - mu) @ R.T) * inv_s
        X[sel, 4] = -np.sin(np.pi * X[sel, 0] / 2)
    deg = np.bincount(rows, weights=w, minlength=len(cent))
    X[:, 3] = np.where(group >= 0, deg * DEG_SCALE, 0.0)
    return X


def _mean_agg(H, rows, col, w, wsum):
    agg = np.zeros_like(H)
    np.add.at(agg, rows, w[:, None] * H[col])
    inv = np.where(wsum > 0, 1.0 / np.where(wsum > 0, wsum, 1.0), 0.0)
    return agg * inv[:, None]


def forward(X, rows, col, w, params, round_weights=True):
    P = unpack(params)
    rw = bf16_round if round_weights else (lambda a: a)
    wsum = np.bincount(rows, weights=w, minlength=len(X))
    cache = {"wsum": wsum, "H": [X]}
    H = X
    for l, (Wk, bk) in enumerate((("W1", "b1"), ("W2", "b2"), ("W3", "b3"))):
        A = np.concatenate([H, _mean_agg(H, rows, col, w, wsum)], axis=1)
        Z = A @ rw(P[Wk]) + P[bk]
        H = np.maximum(Z, 0.0)
        cache.setdefault("A", []).append(A)
        cache.setdefault("Z", []).append(Z)
        cache["H"].append(H)
    y = H @ P["wo"] + P["bo"] + X[:, 4]  # the head corrects the geometric guess
    return y, cache


def loss_and_dy(y, label, group):
    """Mean over groups of 1 - cos^2(y - mean y, f - mean f), and dL/dy."""
    gs = np.unique(group[group >= 0])
    G = len(gs)
    dy = np.zeros_like(y)
    tot = 0.0
    for g in gs:
        sel = group == g
        yc = y[sel] - y[sel].mean()
        fc = label[sel] - label[sel].mean()
        c, s, ff = yc @ fc, yc @ yc, fc @ fc
        tot += 1.0 - c * c / (s * ff)
        dy[sel] = (-2 * c / (s * ff) * fc + 2 * c * c / (s * s * ff) * yc) / G
    return tot / G, dy


def gradient(X, rows, col, w, params, label, group, round_weights=True):
    """(loss, flat gradient) in FP64, with the BF16-rounded weights the GPU
    multiplies by (round_weights=False: the exact weights, for finite
    differences)."""
    P = unpack(params)
    rw = bf16_round if round_weights else (lambda a: a)
    y, C = forward(X, rows, col, w, params, round_weights)
    L, dy = loss_and_dy(y, label, group)
    grad = {}
    H3 = C["H"][3]
    grad["wo"] = H3.T @ dy
    grad["bo"] = dy.sum()
    dH = np.outer(dy, P["wo"])
    wsum = C["wsum"]
    for l in (2, 1, 0):
        Wk, bk = ("W1", "b1") if l == 0 else (("W2", "b2") if l == 1 else ("W3", "b3"))
        dZ = dH * (C["Z"][l] > 0)
        grad[Wk] = C["A"][l].T @ dZ
        grad[bk] = dZ.sum(axis=0)
        if l == 0:
            break
        dA = dZ @ rw(P[Wk]).T
        din = dA.shape[1] // 2
        dself, dagg = dA[:, :din], dA[:, din:]
        u = dagg * np.where(wsum > 0, 1.0 / np.where(wsum > 0, wsum, 1.0), 0.0)[:, None]
        back = np.zeros_like(dself)
        np.add.at(back, col, w[:, None] * u[rows])
        dH = dself + back
    return L, pack(grad)
