"""parrsb_gb300 -- GB300 (sm_103a) implementation of parRSB's partitioning
(RSB / RCB / RIB) and connectivity (gencon) path behind a drop-in C ABI.

The compute path is the in-tree CUDA library ``libparrsb_gb300.so`` (built by
``parrsb_gb300.build``).  This module binds its C ABI with ctypes and mirrors
the reference entry points:

* ``part_mesh(vtx, xyz, nparts, **options)`` -- parrsb_part_mesh
  (src/parRSB.h:45-48) with an explicit part count instead of MPI_Comm.
* ``conn_mesh(coord, ndim, tol)`` -- parrsb_conn_mesh (src/parRSB.h:62-64).

There is no CPU fallback: importing works without a GPU (so option handling
and argument checks can be tested), but any call that reaches the GPU raises
``ParrsbError`` when the library or the device is missing.
"""
import ctypes
import os

import numpy as np

from .options import (ERR_ARGS, ERR_CHECK, ERR_CUDA, ERR_UNSUPPORTED, OK,
                      ParrsbOptions, DEFAULTS)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libparrsb_gb300.so")

# Exported symbols declared in include/parrsb.h
EXPORTS = ["parrsb_default_options", "parrsb_part_mesh", "parrsb_conn_mesh",
           "fparrsb_conn_mesh", "parrsb_part_mesh_device",
           "parrsb_conn_mesh_device", "parrsb_get_stats", "parrsb_part_quality",
           "parrsb_gpu_finalize", "parrsb_fiedler_groups", "parrsb_part_mesh_seq",
           "parrsb_read_mesh", "parrsb_dump_con", "parrsb_dump_map",
           "parrsb_part_mesh_rcb_noalloc", "parrsb_dual_graph", "parrsb_components",
           "parrsb_warm_install", "parrsb_warm_batch_create", "parrsb_warm_batch_destroy",
           "parrsb_warm_batch_features", "parrsb_warm_batch_step", "parrsb_warm_adam"]


class ParrsbError(RuntimeError):
    def __init__(self, code, what):
        super().__init__(f"{what} failed with code {code}")
        self.code = code


class Stats(ctypes.Structure):
    _fields_ = [("total_ms", ctypes.c_double),
                ("stage_ms", ctypes.c_double * 12),
                ("lanczos_iters", ctypes.c_longlong),
                ("lanczos_row_iters", ctypes.c_longlong),
                ("spmv_launches", ctypes.c_longlong),
                ("spmv_ms", ctypes.c_double),
                ("spmv_bytes", ctypes.c_longlong),
                ("kernel_launches", ctypes.c_longlong),
                ("levels", ctypes.c_int),
                ("max_components", ctypes.c_int),
                ("max_fiedler_resid", ctypes.c_double),
                ("unconverged", ctypes.c_int),
                ("nnz", ctypes.c_longlong),
                ("gencon_segments", ctypes.c_longlong),
                ("lanczos_ms", ctypes.c_double * 6),
                ("lanczos_passes", ctypes.c_longlong),
                ("warm_tried", ctypes.c_longlong),
                ("warm_used", ctypes.c_longlong),
                ("warm_ms", ctypes.c_double),
                ("start_resid_fallback", ctypes.c_double),
                ("start_resid_warm", ctypes.c_double),
                ("level_steps", ctypes.c_longlong * 16),
                ("repair_components", ctypes.c_longlong),
                ("repair_elements", ctypes.c_longlong),
                ("lanczos_host_ms", ctypes.c_double * 4)]

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if name in ("stage_ms", "lanczos_ms", "level_steps", "lanczos_host_ms") else v
        return d


STAGES = ["upload", "setup", "pre", "lanczos", "tqli", "sort", "components",
          "balance", "restrict", "download", "gencon", "check"]

_lib = None


def library(build_if_missing=False):
    """Load the CUDA library (raises if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if build_if_missing:
            from .build import build
            build()
        else:
            raise ParrsbError(ERR_CUDA, f"CUDA library not built ({LIB_PATH})")
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.c_void_p
    L.parrsb_part_mesh.argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_int,
                                   ctypes.POINTER(ParrsbOptions), ctypes.c_int]
    L.parrsb_part_mesh.restype = ctypes.c_int
    L.parrsb_part_mesh_seq.argtypes = [P, P, P, P, P, ctypes.c_int, ctypes.c_int,
                                       ctypes.POINTER(ParrsbOptions), ctypes.c_int]
    L.parrsb_part_mesh_seq.restype = ctypes.c_int
    L.parrsb_part_mesh_device.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ParrsbOptions),
                                          ctypes.c_int]
    L.parrsb_conn_mesh.argtypes = [P, P, ctypes.c_uint, ctypes.c_uint, P,
                                   ctypes.c_int, ctypes.c_double]
    L.parrsb_conn_mesh.restype = ctypes.c_int
    L.parrsb_conn_mesh_device.argtypes = [P, P, ctypes.c_uint, ctypes.c_uint,
                                          ctypes.c_double]
    L.fparrsb_conn_mesh.argtypes = [P, P, P, P, P, P, P, P]
    L.fparrsb_conn_mesh.restype = None
    L.parrsb_get_stats.argtypes = [ctypes.POINTER(Stats)]
    L.parrsb_part_quality.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int]
    L.parrsb_fiedler_groups.argtypes = [P, P, P, P, P, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.POINTER(ParrsbOptions),
                                        ctypes.c_int]
    L.parrsb_read_mesh.argtypes = [P, P, P, P, P, P, ctypes.c_char_p, ctypes.c_int]
    L.parrsb_dump_con.argtypes = [ctypes.c_char_p, ctypes.c_uint, ctypes.c_uint, P]
    L.parrsb_dump_map.argtypes = [ctypes.c_char_p, ctypes.c_uint, ctypes.c_uint, P, P]
    L.parrsb_gpu_finalize.argtypes = []
    L.parrsb_gpu_finalize.restype = None
    L.parrsb_part_mesh_rcb_noalloc.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
    L.parrsb_part_mesh_rcb_noalloc.restype = ctypes.c_int
    L.parrsb_dual_graph.argtypes = [P, P, P, P, ctypes.c_longlong, P, ctypes.c_int,
                                    ctypes.c_int]
    L.parrsb_dual_graph.restype = ctypes.c_int
    L.parrsb_components.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.parrsb_components.restype = ctypes.c_int
    L.parrsb_warm_install.argtypes = [P]
    L.parrsb_warm_batch_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), P, P, P,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.parrsb_warm_batch_destroy.argtypes = [P]
    L.parrsb_warm_batch_features.argtypes = [P, P]
    L.parrsb_warm_batch_step.argtypes = [P, P, P, P, P, ctypes.POINTER(ctypes.c_double)]
    L.parrsb_warm_adam.argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_float]
    _lib = L
    return L


def default_options():
    """Copy of the library's exported parrsb_default_options."""
    o = ParrsbOptions.in_dll(library(), "parrsb_default_options")
    return ParrsbOptions(**o.as_dict())


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def part_mesh(vtx, xyz, nparts, options=None, tag=None, **kw):
    """Partition elements into `nparts` parts (parrsb_part_mesh).

    vtx: (nel, nv) int64 vertex ids or None; xyz: (nel, nv, ndim) float64
    corner coordinates or None.  Options may be a ParrsbOptions (mutated in
    place with environment overrides, as the reference does) or keywords.
    Returns part (nel,) int32.  Raises ParrsbError on a nonzero return."""
    if options is None:
        kw.setdefault("verbose_level", 0)
        options = ParrsbOptions.make(**kw)
    nel = len(vtx) if vtx is not None else len(xyz)
    nv = vtx.shape[1] if vtx is not None else xyz.shape[1]
    vtx = None if vtx is None else np.ascontiguousarray(vtx, np.int64)
    xyz = None if xyz is None else np.ascontiguousarray(xyz, np.float64)
    tag = None if tag is None else np.ascontiguousarray(tag, np.int32)
    part = np.full(nel, -1, np.int32)
    rc = library().parrsb_part_mesh(_ptr(part), _ptr(vtx), _ptr(xyz), _ptr(tag),
                                    nel, nv, ctypes.byref(options), nparts)
    if rc != OK:
        raise ParrsbError(rc, "parrsb_part_mesh")
    return part


def part_mesh_seq(vtx, xyz, nparts, **kw):
    """parrsb_part_mesh_seq: (part, seq) where seq[e] is the position of
    element e inside its part in the final order."""
    kw.setdefault("verbose_level", 0)
    options = ParrsbOptions.make(**kw)
    nel = len(vtx) if vtx is not None else len(xyz)
    nv = vtx.shape[1] if vtx is not None else xyz.shape[1]
    vtx = None if vtx is None else np.ascontiguousarray(vtx, np.int64)
    xyz = None if xyz is None else np.ascontiguousarray(xyz, np.float64)
    part = np.full(nel, -1, np.int32)
    seq = np.full(nel, -1, np.int32)
    rc = library().parrsb_part_mesh_seq(_ptr(part), _ptr(seq), _ptr(vtx), _ptr(xyz), None,
                                        nel, nv, ctypes.byref(options), nparts)
    if rc != OK:
        raise ParrsbError(rc, "parrsb_part_mesh_seq")
    return part, seq


def conn_mesh(coord, ndim, tol=0.2, periodic=None):
    """Vertex ids from corner coordinates (parrsb_conn_mesh).  coord:
    (nel, nv, ndim) in Nek preprocessor corner order.  Returns (nel, nv)
    int64 ids in symmetric corner order.  Raises ParrsbError (code 1 when
    the element or face check fails)."""
    coord = np.ascontiguousarray(coord, np.float64)
    nv = 4 if ndim == 2 else 8
    nel = coord.size // (nv * ndim)
    vtx = np.zeros(nel * nv, np.int64)
    npf = 0 if periodic is None else len(periodic)
    pinfo = None if periodic is None else np.ascontiguousarray(periodic, np.int64)
    rc = library().parrsb_conn_mesh(_ptr(vtx), _ptr(coord), nel, ndim,
                                    _ptr(pinfo), npf, tol)
    if rc != OK:
        raise ParrsbError(rc, "parrsb_conn_mesh")
    return vtx.reshape(nel, nv)


def part_quality(part, vtx, nparts):
    """Quality figures of a partition, computed on the GPU (see
    include/parrsb.h parrsb_part_quality)."""
    vtx = np.ascontiguousarray(vtx, np.int64)
    part = np.ascontiguousarray(part, np.int32)
    q = np.zeros(8, np.float64)
    rc = library().parrsb_part_quality(_ptr(q), _ptr(part), _ptr(vtx), len(vtx),
                                       vtx.shape[1], nparts)
    if rc != OK:
        raise ParrsbError(rc, "parrsb_part_quality")
    return q


def fiedler_groups(vtx, group, ngroups, batched=True, **kw):
    """Batched level solve (parrsb_fiedler_groups): the Fiedler vector of
    every group of elements.  Returns (fiedler[nel], iters[ngroups],
    resid[ngroups])."""
    kw.setdefault("verbose_level", 0)
    options = ParrsbOptions.make(**kw)
    vtx = np.ascontiguousarray(vtx, np.int64)
    group = np.ascontiguousarray(group, np.int32)
    nel, nv = vtx.shape
    f = np.zeros(nel, np.float64)
    it = np.zeros(ngroups, np.int64)
    rs = np.zeros(ngroups, np.float64)
    rc = library().parrsb_fiedler_groups(_ptr(f), _ptr(it), _ptr(rs), _ptr(vtx),
                                         _ptr(group), nel, nv, ngroups,
                                         ctypes.byref(options), 1 if batched else 0)
    if rc != OK:
        raise ParrsbError(rc, "parrsb_fiedler_groups")
    return f, it, rs


def dual_graph(vtx):
    """The element dual graph built on the GPU (parrsb_dual_graph): (rowptr,
    col, weight), each row's columns in first-occurrence order."""
    vtx = np.ascontiguousarray(vtx, np.int64)
    nel, nv = vtx.shape
    rowptr = np.zeros(nel + 1, np.int64)
    nnz = ctypes.c_longlong(0)
    rc = library().parrsb_dual_graph(_ptr(rowptr), None, None, ctypes.byref(nnz), 0, _ptr(vtx),
                                     nel, nv)
    if rc != OK:
        raise ParrsbError(rc, "parrsb_dual_graph")
    col = np.zeros(max(nnz.value, 1), np.int32)
    w = np.zeros(max(nnz.value, 1), np.uint8)
    rc = library().parrsb_dual_graph(_ptr(rowptr), _ptr(col), _ptr(w), ctypes.byref(nnz),
                                     len(col), _ptr(vtx), nel, nv)
    if rc != OK:
        raise ParrsbError(rc, "parrsb_dual_graph")
    return rowptr, col[:nnz.value], w[:nnz.value]


def components(vtx, group, ngroups):
    """Vertex-connected components per group, on the GPU (parrsb_components);
    group[e] < 0 leaves element e out."""
    vtx = np.ascontiguousarray(vtx, np.int64)
    group = np.ascontiguousarray(group, np.int32)
    out = np.zeros(ngroups, np.int32)
    rc = library().parrsb_components(_ptr(out), _ptr(vtx), _ptr(group), len(vtx), vtx.shape[1],
                                     ngroups)
    if rc != OK:
        raise ParrsbError(rc, "parrsb_components")
    return out


_libc = None


def _free(ptr):
    global _libc
    if _libc is None:
        _libc = ctypes.CDLL(None)
        _libc.free.argtypes = [ctypes.c_void_p]
    _libc.free(ptr)


def read_mesh(name, read=1):
    """parrsb_read_mesh: returns dict with 'coord' (nel, nv, ndim) and
    'periodic' (nbcs, 4) for read & 1, 'vtx' (nel, nv) for read & 2."""
    nel, nv, nb = ctypes.c_uint(0), ctypes.c_uint(0), ctypes.c_uint(0)
    vl, co, bc = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    rc = library().parrsb_read_mesh(ctypes.byref(nel), ctypes.byref(nv), ctypes.byref(vl),
                                    ctypes.byref(co), ctypes.byref(nb), ctypes.byref(bc),
                                    name.encode(), read)
    if rc != OK:
        raise ParrsbError(rc, "parrsb_read_mesh")
    out = {}
    n, v = nel.value, nv.value
    nd = 3 if v == 8 else 2
    if read & 1:
        a = np.ctypeslib.as_array(ctypes.cast(co, ctypes.POINTER(ctypes.c_double)),
                                  shape=(max(n * v * nd, 1),))
        out["coord"] = a[:n * v * nd].reshape(n, v, nd).copy()
        b = np.ctypeslib.as_array(ctypes.cast(bc, ctypes.POINTER(ctypes.c_longlong)),
                                  shape=(max(4 * nb.value, 1),))
        out["periodic"] = b[:4 * nb.value].reshape(nb.value, 4).copy()
        _free(co)
        _free(bc)
    if read & 2:
        a = np.ctypeslib.as_array(ctypes.cast(vl, ctypes.POINTER(ctypes.c_longlong)),
                                  shape=(max(n * v, 1),))
        out["vtx"] = a[:n * v].reshape(n, v).copy()
        _free(vl)
    return out


def dump_con(name, vtx):
    vtx = np.ascontiguousarray(vtx, np.int64)
    rc = library().parrsb_dump_con(name.encode(), len(vtx), vtx.shape[1], _ptr(vtx))
    if rc != OK:
        raise ParrsbError(rc, "parrsb_dump_con")


def dump_map(name, vtx, part):
    vtx = np.ascontiguousarray(vtx, np.int64)
    part = np.ascontiguousarray(part, np.int32)
    rc = library().parrsb_dump_map(name.encode(), len(vtx), vtx.shape[1], _ptr(vtx), _ptr(part))
    if rc != OK:
        raise ParrsbError(rc, "parrsb_dump_map")


def write_re2(name, coord, periodic=()):
    """Write a Nek5000 .re2 file (the layout parrsb_read_mesh reads) from
    corner coordinates (nel, nv, ndim) in preprocessor order."""
    coord = np.asarray(coord, np.float64)
    nel, nv, nd = coord.shape
    with open(name + ".re2", "wb") as f:
        hdr = f"#v003 {nel:10d} {nd:2d} {nel:10d} synthetic".ljust(80)
        f.write(hdr.encode()[:80])
        f.write(np.float32(6.54321).tobytes())
        rec = np.zeros((nel, 1 + nv * nd))
        rec[:, 1:] = coord.transpose(0, 2, 1).reshape(nel, nv * nd)
        f.write(rec.tobytes())
        f.write(np.float64(0.0).tobytes())  # no curves
        f.write(np.float64(len(periodic)).tobytes())
        for eid, fid, e1, e2 in periodic:
            f.write(np.array([eid, fid, e1, e2, 0, 0, 0], np.float64).tobytes())
            f.write(b"P       ")


def last_stats():
    s = Stats()
    library().parrsb_get_stats(ctypes.byref(s))
    return s


def finalize():
    if _lib is not None:
        _lib.parrsb_gpu_finalize()


__all__ = ["part_mesh", "part_mesh_seq", "conn_mesh", "read_mesh", "dump_con",
           "dump_map", "write_re2", "part_quality", "last_stats", "fiedler_groups",
           "dual_graph", "components",
           "default_options", "ParrsbOptions", "ParrsbError", "DEFAULTS",
           "library", "finalize", "OK", "ERR_ARGS", "ERR_CUDA", "ERR_CHECK",
           "ERR_UNSUPPORTED"]
