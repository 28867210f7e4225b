"""ctypes wrapper of the C oracle (parrsb_oracle.c).

Test infrastructure only: used by tests/, by ``__graft_entry__.smoke()`` and
by the CPU-baseline leg of ``bench.py``.  The product library never imports
this module.  ``build()`` compiles the C restatement with gcc into
``oracle/_build/`` (no FMA contraction, like the reference's ISO C99 build).
"""
import ctypes
import os
import subprocess

import numpy as np

from parrsb_gb300.options import ParrsbOptions

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "parrsb_oracle.c")
HDR = os.path.join(HERE, "parrsb_oracle.h")
LIB = os.path.join(HERE, "_build", "libparrsb_oracle.so")

_lib = None


def build(force=False):
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    newest = max(os.path.getmtime(SRC), os.path.getmtime(HDR))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    base = ["gcc", "-O2", "-std=gnu99", "-ffp-contract=off", "-fPIC", "-shared",
            "-o", LIB + ".tmp", SRC, "-lm"]
    # OpenMP when the compiler has it (host threads for large meshes; the
    # results do not depend on the thread count), plain otherwise
    if subprocess.run(base + ["-fopenmp"], capture_output=True).returncode != 0:
        subprocess.run(base, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class RsbInfo(ctypes.Structure):
    _fields_ = [("total_iters", ctypes.c_longlong), ("nbisect", ctypes.c_int),
                ("unconverged", ctypes.c_int), ("max_components", ctypes.c_int),
                ("max_resid", ctypes.c_double), ("levels", ctypes.c_int),
                ("row_iters", ctypes.c_longlong)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        L.oracle_part_mesh.argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(ParrsbOptions),
                                       ctypes.c_int, ctypes.POINTER(RsbInfo)]
        L.oracle_conn_mesh.argtypes = [P, P, ctypes.c_uint, ctypes.c_uint,
                                       ctypes.c_double, ctypes.c_int, P, P]
        L.oracle_conn_mesh_periodic.argtypes = [P, P, ctypes.c_uint, ctypes.c_uint,
                                                ctypes.c_double, ctypes.c_int, P,
                                                ctypes.c_int, P, P]
        L.oracle_centroids.argtypes = [P, P, ctypes.c_int, ctypes.c_int]
        L.oracle_tree_sum.argtypes = [P, ctypes.c_longlong]
        L.oracle_tree_sum.restype = ctypes.c_double
        L.oracle_power_serial.argtypes = [P, ctypes.c_int, P]
        L.oracle_tqli.argtypes = [P, P, ctypes.c_int, P, P]
        L.oracle_laplacian.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int]
        L.oracle_dual_graph.argtypes = [P, P, P, ctypes.c_longlong, P,
                                        ctypes.c_int, ctypes.c_int]
        L.oracle_dual_graph.restype = ctypes.c_longlong
        L.oracle_components.argtypes = [P, P, ctypes.c_int, ctypes.c_int]
        L.oracle_part_quality.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int]
        L.oracle_fiedler.argtypes = [P, P, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_double]
        L.oracle_rsb_level.argtypes = [P, P, ctypes.c_int, P, P, P, ctypes.c_int,
                                       ctypes.c_int, ctypes.POINTER(ParrsbOptions),
                                       ctypes.POINTER(RsbInfo)]
        L.oracle_rsb_level.restype = ctypes.c_int
        L.oracle_threads.argtypes = [ctypes.c_int]
        L.oracle_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def part_mesh(vtx, xyz, nparts, want_order=False, **opts):
    """Oracle parrsb_part_mesh.  Returns (rc, part, order, info, options)."""
    nel = len(vtx) if vtx is not None else len(xyz)
    nv = (vtx.shape[1] if vtx is not None else xyz.shape[1])
    vtx = None if vtx is None else np.ascontiguousarray(vtx, np.int64)
    xyz = None if xyz is None else np.ascontiguousarray(xyz, np.float64)
    opts.setdefault("verbose_level", 0)
    o = ParrsbOptions.make(**opts)
    part = np.full(nel, -1, np.int32)
    order = np.full(nel, -1, np.int32) if want_order else None
    info = RsbInfo()
    rc = lib().oracle_part_mesh(_p(part), _p(order), _p(vtx), _p(xyz), nel, nv,
                                ctypes.byref(o), nparts, ctypes.byref(info))
    return rc, part, order, info, o


def threads(n=0):
    """Host threads of the oracle (n > 0 sets them); returns the count."""
    return lib().oracle_threads(int(n))


class RsbLevels:
    """RSB of the oracle one level at a time (oracle_rsb_level), for timing
    the levels of a large run separately.  state() / restore() copy the
    element order and segment table at a level boundary."""

    def __init__(self, vtx, xyz, nparts, **opts):
        self.vtx = np.ascontiguousarray(vtx, np.int64)
        self.nel, self.nv = self.vtx.shape
        opts.setdefault("verbose_level", 0)
        self.opts = ParrsbOptions.make(partitioner=0, **opts)
        self.cent = centroids(xyz, self.nv)
        self.P = min(nparts, self.nel)
        self.a = np.arange(self.nel, dtype=np.int32)
        self.segs = np.array([[0, self.nel, self.P, 0]], np.int64)
        self.info = RsbInfo()
        self.ncuts = 0
        while (1 << self.ncuts) < self.P:
            self.ncuts += 1

    def state(self):
        return self.a.copy(), self.segs.copy()

    def restore(self, st):
        self.a, self.segs = st[0].copy(), st[1].copy()

    def level(self):
        out = np.zeros((2 * len(self.segs), 4), np.int64)
        n = lib().oracle_rsb_level(_p(self.a), _p(self.segs), len(self.segs), _p(out),
                                   _p(self.vtx), _p(self.cent), self.nel, self.nv,
                                   ctypes.byref(self.opts), ctypes.byref(self.info))
        self.segs = out[:n].copy()

    def part(self):
        part = np.full(self.nel, -1, np.int32)
        for s0, n, p, r0 in self.segs:
            part[self.a[s0:s0 + n]] = r0
        return part


def conn_mesh(coord, ndim, tol=0.2, heapsort=False, periodic=None):
    """Oracle parrsb_conn_mesh.  periodic: optional (n, 4) face records.
    Returns (rc, vtx, ids, nseg); ids are the ids before periodic matching,
    nseg the number of distinct ids after it."""
    coord = np.ascontiguousarray(coord, np.float64)
    nv = 4 if ndim == 2 else 8
    nel = coord.size // (nv * ndim)
    vtx = np.zeros(nel * nv, np.int64)
    ids = np.zeros(nel * nv, np.int64)
    nseg = ctypes.c_longlong(0)
    pinfo = None if periodic is None else np.ascontiguousarray(periodic, np.int64)
    npf = 0 if pinfo is None else len(pinfo)
    rc = lib().oracle_conn_mesh_periodic(_p(vtx), _p(coord), nel, ndim, tol,
                                         1 if heapsort else 0, _p(pinfo), npf, _p(ids),
                                         ctypes.byref(nseg))
    return rc, vtx.reshape(nel, nv), ids.reshape(nel, nv), nseg.value


def part_mesh_tagged(vtx, xyz, tag, nparts, **opts):
    """Oracle of tagged partitioning (parrsb_part_mesh_v1,
    src/parrsb.c:379-561): tags numbered in increasing order, nparts a
    multiple of their number; the elements of tag number t, in input order,
    are partitioned by parrsb_part_mesh_v0 among nparts / ntags ranks, whose
    part numbers start at t * nparts / ntags.  Returns (rc, part)."""
    tag = np.asarray(tag)
    u = np.unique(tag)
    if nparts % len(u):
        return 1, None
    chunk = nparts // len(u)
    part = np.full(len(tag), -1, np.int32)
    for t, val in enumerate(u):
        sel = np.flatnonzero(tag == val)
        rc, p, _, _, _ = part_mesh(None if vtx is None else vtx[sel],
                                   None if xyz is None else xyz[sel], chunk, **opts)
        if rc:
            return rc, None
        part[sel] = p + t * chunk
    return 0, part


def centroids(xyz, nv):
    xyz = np.ascontiguousarray(xyz, np.float64)
    nel = xyz.shape[0]
    out = np.zeros((nel, 3), np.float64)
    lib().oracle_centroids(_p(out), _p(xyz), nel, nv)
    return out


def tree_sum(x):
    x = np.ascontiguousarray(x, np.float64)
    return lib().oracle_tree_sum(_p(x), len(x))


def power_serial(A, N):
    A = np.ascontiguousarray(A, np.float64).ravel()
    y = np.zeros(3, np.float64)
    it = lib().oracle_power_serial(_p(y), N, _p(A))
    return y[:N], it


def tqli(diag, upper):
    n = len(diag)
    diag = np.ascontiguousarray(diag, np.float64)
    upper = np.ascontiguousarray(np.concatenate([upper, [0.0]])[:max(n, 1)],
                                 np.float64)
    ev = np.zeros((n, n), np.float64)
    ew = np.zeros(n, np.float64)
    rc = lib().oracle_tqli(_p(ev), _p(ew), n, _p(diag), _p(upper))
    return rc, ew, ev


def laplacian(x, vtx):
    vtx = np.ascontiguousarray(vtx, np.int64)
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros_like(x)
    lib().oracle_laplacian(_p(y), _p(x), _p(vtx), len(vtx), vtx.shape[1])
    return y


def dual_graph(vtx):
    vtx = np.ascontiguousarray(vtx, np.int64)
    nel, nv = vtx.shape
    cap = nel * 64 + 16
    rowptr = np.zeros(nel + 1, np.int64)
    col = np.zeros(cap, np.int32)
    w = np.zeros(cap, np.int32)
    nnz = lib().oracle_dual_graph(_p(rowptr), _p(col), _p(w), cap, _p(vtx),
                                  nel, nv)
    assert nnz >= 0
    return rowptr, col[:nnz].copy(), w[:nnz].copy()


def components(vtx, mask=None):
    vtx = np.ascontiguousarray(vtx, np.int64)
    m = None if mask is None else np.ascontiguousarray(mask, np.int32)
    return lib().oracle_components(_p(vtx), _p(m), len(vtx), vtx.shape[1])


def part_quality(part, vtx, nparts):
    vtx = np.ascontiguousarray(vtx, np.int64)
    part = np.ascontiguousarray(part, np.int32)
    q = np.zeros(8, np.float64)
    lib().oracle_part_quality(_p(q), _p(part), _p(vtx), len(vtx),
                              vtx.shape[1], nparts)
    return q


def fiedler(vtx, miter=50, mpass=50, tol=1e-5):
    vtx = np.ascontiguousarray(vtx, np.int64)
    f = np.zeros(len(vtx), np.float64)
    it = lib().oracle_fiedler(_p(f), _p(vtx), len(vtx), vtx.shape[1], miter,
                              mpass, tol)
    return f, it


def repair_parts(part, vtx, nparts):
    """Restatement of the library's repair of disconnected parts
    (parrsb_options.repair = 1; the reference parses the option and does
    nothing with it, src/parrsb.c:65): every part keeps its largest
    vertex-connected component (ties: the one holding the part's smallest
    element index); every other component moves, whole, to the part it
    shares the largest dual-graph weight with (ties: smallest part number);
    a component without a neighbour in another part stays.
    Returns (new part, moved components, moved elements)."""
    from scipy.sparse import coo_matrix
    from scipy.sparse.csgraph import connected_components
    part = np.asarray(part, np.int64)
    n = len(part)
    rowptr, col, w = dual_graph(vtx)
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    same = part[rows] == part[col]
    A = coo_matrix((np.ones(int(same.sum())), (rows[same], col[same])), shape=(n, n))
    ncomp, comp = connected_components(A, directed=False)
    size = np.bincount(comp, minlength=ncomp)
    first = np.full(ncomp, n, np.int64)
    np.minimum.at(first, comp, np.arange(n))
    cpart = part[first]
    keep = {}
    for c in np.lexsort((first, -size)):  # largest first, then smallest first element
        keep.setdefault(int(cpart[c]), int(c))
    out = part.copy()
    moved_c = moved_e = 0
    cross = ~same
    for c in range(ncomp):
        if keep[int(cpart[c])] == c:
            continue
        sel = cross & (comp[rows] == c)
        if not sel.any():
            continue
        wsum = np.bincount(part[col[sel]], weights=w[sel], minlength=nparts)
        tgt = int(np.argmax(wsum))  # first maximum: the smallest part
        out[comp == c] = tgt
        moved_c += 1
        moved_e += int(size[c])
    return out.astype(np.int32), moved_c, moved_e
