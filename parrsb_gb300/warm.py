"""Learned warm start for RSB's Lanczos runs: data, training and weights.

The network and its forward / backward kernels live in the CUDA library
(csrc/warm.cu, declared in include/parrsb.h under "Learned warm start");
this module drives them through the C ABI:

* ``training_meshes(count, seed)`` -- the seeded training set: jittered hex
  sub-boxes (distinct side lengths, so every box has a well separated
  Fiedler vector) and annular hex cylinders with more elements along the
  axis than around it, 1k-64k elements each, log-uniform;
* ``label(vtx, group, ngroups)`` -- their Fiedler vectors by the plain
  method (parrsb_fiedler_groups: batched Lanczos, FP64 vectors);
* ``train(...)`` -- Adam on the sign-invariant cosine loss, every step a
  forward and backward pass of the library's kernels on the GPU;
* ``save`` / ``load`` / ``install`` -- the raw FP32 parameter file that
  ``PARRSB_GPU_WARM_WEIGHTS`` names (``WEIGHTS``: the trained network that
  ships with the package).

PyTorch only provides device buffers here; every computation is a library
kernel.
"""
import ctypes
import os
import time

import numpy as np

from . import library, fiedler_groups, ParrsbError, OK
from . import meshgen

NPARAM = 17665
HID, FIN, K1, K2 = 64, 8, 16, 128
WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "warm_weights.f32")


def init_params(seed=0):
    """He-style initialisation of the flat parameter vector (FP32)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    parts = []
    for k in (K1, K2, K2):
        parts.append(rng.normal(0.0, np.sqrt(2.0 / k), k * HID))
        parts.append(np.zeros(HID))
    # small head: the network starts at the geometric guess it corrects
    parts.append(rng.normal(0.0, 1e-3, HID))
    parts.append(np.zeros(1))
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == NPARAM
    return p


def save(path, params):
    np.asarray(params, np.float32).tofile(path)


def load(path=WEIGHTS):
    p = np.fromfile(path, dtype=np.float32)
    if p.size != NPARAM:
        raise ValueError(f"{path}: {p.size} values, expected {NPARAM}")
    return p


def install(params=None):
    """Install parameters (default: the shipped weights) on the current
    device for PARRSB_GPU_WARM=1."""
    p = np.ascontiguousarray(load() if params is None else params, np.float32)
    rc = library().parrsb_warm_install(p.ctypes.data_as(ctypes.c_void_p))
    if rc != OK:
        raise ParrsbError(rc, "parrsb_warm_install")


def _box_dims(rng, target):
    """Side lengths with target elements, longest / second >= 1.2."""
    while True:
        a = np.exp(rng.uniform(0.0, np.log(4.0), 3))
        a = np.sort(a)[::-1]
        if a[0] >= 1.2 * a[1]:
            break
    s = (target / np.prod(a)) ** (1.0 / 3.0)
    d = np.maximum(2, np.round(a * s)).astype(int)
    return int(d[0]), int(d[1]), int(d[2])


def training_meshes(count=2000, seed=0, smin=1000, smax=64000):
    """`count` seeded meshes with disjoint vertex ids: (vtx, xyz, group)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    vts, xys, grs = [], [], []
    off = 0
    for m in range(count):
        target = float(np.exp(rng.uniform(np.log(smin), np.log(smax))))
        if rng.uniform() < 0.7:
            nx, ny, nz = _box_dims(rng, target)
            perm = rng.permutation(3)  # the long side along any axis
            dims = np.array([nx, ny, nz])[perm]
            h = np.ones(3)
            hi = dims * h / dims.max()
            v, x = meshgen.box_hex(int(dims[0]), int(dims[1]), int(dims[2]), jitter=0.1,
                                   seed=seed * 7919 + m, hi=tuple(hi), id_offset=off)
            off += int(np.prod(dims + 1))
        else:
            # annular cylinder, r in [1, 2], near-cubic elements, more
            # elements along the axis than around it (the graph Laplacian
            # sees element counts, not lengths: its Fiedler vector then runs
            # along the axis, like the centroids' principal axis)
            nr = max(2, min(8, int((target / 75.0) ** (1.0 / 3.0))))
            nt = max(8, int(round(2 * np.pi * 1.5 * nr)))
            nz = max(int(np.ceil(0.8 * nt)), int(round(target / (nt * nr))))
            v, x = meshgen.pipe_hex(nt, nr, nz, jitter=0.05, seed=seed * 7919 + m,
                                    length=nz / nr)
            v = v + off
            off += nt * (nr + 1) * (nz + 1)
        vts.append(v)
        xys.append(x)
        grs.append(np.full(len(v), m, np.int32))
    return (np.ascontiguousarray(np.concatenate(vts)), np.ascontiguousarray(np.concatenate(xys)),
            np.concatenate(grs))


def label(vtx, group, ngroups, **kw):
    """Fiedler vectors of every group by the plain method (FP64 vectors,
    batched Lanczos from the reference's start), restarted until each
    vector's eigen-residual is at most rsb_tol (default 1e-6)."""
    kw.setdefault("rsb_tol", 1e-6)
    kw.setdefault("rsb_max_passes", 400)
    old = {k: os.environ.get(k) for k in ("PARRSB_GPU_RESID_STOP", "PARRSB_GPU_FP32")}
    os.environ["PARRSB_GPU_RESID_STOP"] = "1"
    os.environ["PARRSB_GPU_FP32"] = "0"
    try:
        f, it, rs = fiedler_groups(vtx, group, ngroups, batched=True, **kw)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    return f, it, rs


class Batch:
    """A training batch on the current device (parrsb_warm_batch_*)."""

    def __init__(self, vtx, xyz, group, ngroups):
        import torch
        self.torch = torch
        self.nel, self.nv = vtx.shape
        self.ngroups = ngroups
        self.d_vtx = torch.from_numpy(np.ascontiguousarray(vtx, np.int64)).cuda()
        self.d_xyz = torch.from_numpy(np.ascontiguousarray(xyz, np.float64).ravel()).cuda()
        self.d_grp = torch.from_numpy(np.ascontiguousarray(group, np.int32)).cuda()
        h = ctypes.c_void_p()
        rc = library().parrsb_warm_batch_create(ctypes.byref(h), self._p(self.d_vtx),
                                                self._p(self.d_xyz), self._p(self.d_grp),
                                                self.nel, self.nv, ngroups)
        if rc != OK:
            raise ParrsbError(rc, "parrsb_warm_batch_create")
        self.h = h

    @staticmethod
    def _p(t):
        return None if t is None else ctypes.c_void_p(t.data_ptr())

    def features(self):
        out = self.torch.zeros((self.nel, FIN), dtype=self.torch.float32, device="cuda")
        rc = library().parrsb_warm_batch_features(self.h, self._p(out))
        if rc != OK:
            raise ParrsbError(rc, "parrsb_warm_batch_features")
        return out

    def step(self, d_params, d_label=None, d_grad=None, want_pred=False):
        pred = (self.torch.zeros(self.nel, dtype=self.torch.float32, device="cuda")
                if want_pred else None)
        loss = ctypes.c_double(0.0)
        rc = library().parrsb_warm_batch_step(self.h, self._p(d_params), self._p(d_label),
                                              self._p(d_grad), self._p(pred),
                                              ctypes.byref(loss))
        if rc != OK:
            raise ParrsbError(rc, "parrsb_warm_batch_step")
        return loss.value, pred

    def close(self):
        if self.h:
            library().parrsb_warm_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def adam(d_params, d_m, d_v, d_grad, step, lr):
    rc = library().parrsb_warm_adam(ctypes.c_void_p(d_params.data_ptr()),
                                    ctypes.c_void_p(d_m.data_ptr()),
                                    ctypes.c_void_p(d_v.data_ptr()),
                                    ctypes.c_void_p(d_grad.data_ptr()), NPARAM, step, lr)
    if rc != OK:
        raise ParrsbError(rc, "parrsb_warm_adam")


def train(count=2000, seed=0, epochs=200, nbatch=8, lr=3e-3, params=None, log=None):
    """Train on `count` seeded meshes split into `nbatch` batches; returns
    (params, history).  history: per epoch mean training loss, and the
    loss of the held-out last batch."""
    import torch
    vtx, xyz, group = training_meshes(count, seed)
    t0 = time.time()
    f, it, rs = label(vtx, group, count)
    t_label = time.time() - t0
    order = np.arange(count)
    cut = np.array_split(order, nbatch)
    batches = []
    for ids in cut:
        sel = np.isin(group, ids)
        remap = np.full(count, -1, np.int32)
        remap[ids] = np.arange(len(ids), dtype=np.int32)
        b = Batch(vtx[sel], xyz[sel], remap[group[sel]], len(ids))
        lab = torch.from_numpy(np.ascontiguousarray(f[sel])).cuda()
        batches.append((b, lab))
    train_b, held = batches[:-1], batches[-1]
    p = torch.from_numpy(init_params(seed) if params is None else
                         np.asarray(params, np.float32)).cuda()
    m = torch.zeros_like(p)
    v = torch.zeros_like(p)
    g = torch.zeros_like(p)
    hist = []
    step = 0
    t1 = time.time()
    for ep in range(epochs):
        tot = 0.0
        for b, lab in train_b:
            loss, _ = b.step(p, lab, g)
            step += 1
            # cosine decay of the learning rate over the run
            lr_t = lr * 0.5 * (1.0 + np.cos(np.pi * step / (epochs * len(train_b))))
            adam(p, m, v, g, step, float(max(lr_t, lr * 0.02)))
            tot += loss
        hl, _ = held[0].step(p, held[1])
        hist.append({"epoch": ep, "train_loss": tot / len(train_b), "heldout_loss": hl})
        if log:
            log(hist[-1])
    info = {"label_s": t_label, "train_s": time.time() - t1, "elements": int(len(vtx)),
            "label_steps_mean": float(np.mean(it)), "label_resid_max": float(np.max(rs)),
            "label_resid_p90": float(np.percentile(rs, 90)),
            "history": hist}
    for b, _ in batches:
        b.close()
    return p.cpu().numpy(), info


if __name__ == "__main__":
    import argparse
    import json
    import torch
    ap = argparse.ArgumentParser(description="train the warm-start network on the GPU")
    ap.add_argument("--count", type=int, default=2000)
    ap.add_argument("--epochs", type=int, default=200)
    ap.add_argument("--lr", type=float, default=3e-3)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--out", default=WEIGHTS)
    ap.add_argument("--log", default=None)
    a = ap.parse_args()
    torch.cuda.set_device(0)
    p, info = train(a.count, a.seed, a.epochs, lr=a.lr, log=lambda h: print(json.dumps(h),
                                                                            flush=True))
    save(a.out, p)
    info["weights"] = a.out
    if a.log:
        with open(a.log, "w") as fh:
            json.dump(info, fh, indent=1)
    print(json.dumps({k: v for k, v in info.items() if k != "history"}))
