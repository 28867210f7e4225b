"""CPU tests of the C ABI: the library loads and exports every symbol that
include/parrsb.h declares, the option/stat structs have the C layout, and
the argument checks and option handling that run before any GPU work behave
like the reference (src/parrsb.c:48-77, 244-250, 873-877; src/con.c)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import parrsb_gb300 as P
from parrsb_gb300 import meshgen
from parrsb_gb300.options import ParrsbOptions

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "parrsb.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    funcs = re.findall(r"PARRSB_API\s+(?:int|void)\s+(\w+)\s*\(", text)
    data = re.findall(r"extern\s+PARRSB_API\s+\w+\s+(\w+)\s*;", text)
    return funcs + data


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert "parrsb_part_mesh" in syms and "parrsb_conn_mesh" in syms
    assert "parrsb_default_options" in syms
    for s in syms:
        getattr(lib, s)  # raises AttributeError if not exported
    assert sorted(syms) == sorted(P.EXPORTS)


def _c_layout(tmp_path):
    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "parrsb.h"\n'
        "#define O(P, T, f) printf(P #f \" %zu\\n\", offsetof(T, f))\n"
        "int main(void) {\n"
        '  printf("sizeof_options %zu\\n", sizeof(parrsb_options));\n'
        '  printf("sizeof_stats %zu\\n", sizeof(parrsb_stats));\n'
        + "".join(f'  O("opt_", parrsb_options, {f});\n' for f, _ in ParrsbOptions._fields_)
        + "".join(f'  O("st_", parrsb_stats, {f});\n' for f, _ in P.Stats._fields_)
        + "  return 0;\n}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout
    return dict((k, int(v)) for k, v in (l.split() for l in out.splitlines()))


def test_struct_layouts_match_c(tmp_path):
    c = _c_layout(tmp_path)
    assert c["sizeof_options"] == ctypes.sizeof(ParrsbOptions)
    assert c["sizeof_stats"] == ctypes.sizeof(P.Stats)
    for f, _ in ParrsbOptions._fields_:
        assert c["opt_" + f] == getattr(ParrsbOptions, f).offset, f
    for f, _ in P.Stats._fields_:
        assert c["st_" + f] == getattr(P.Stats, f).offset, f


def test_default_options_match_reference(lib):
    # src/parrsb.c:26-44
    d = P.default_options().as_dict()
    assert d == dict(partitioner=0, tagged=0, levels=2, find_disconnected_comps=1,
                     repair=0, verbose_level=1, profile_level=0, rsb_algo=0, rsb_pre=1,
                     rsb_max_iter=50, rsb_max_passes=50, rsb_tol=1e-5, rsb_dump_stats=0,
                     rsb_mg_grammian=0, rsb_mg_factor=2)


def _call(lib, vtx, xyz, nparts, opts, tag=None, nel=None, nv=None):
    part = np.zeros(0 if vtx is None and xyz is None else max(1, len(vtx if vtx is not None else xyz)), np.int32)
    P_ = lambda a: None if a is None else a.ctypes.data_as(ctypes.c_void_p)
    if nel is None:
        nel = 0 if (vtx is None and xyz is None) else len(vtx if vtx is not None else xyz)
    if nv is None:
        nv = 8
    return lib.parrsb_part_mesh(P_(part), P_(vtx), P_(xyz), P_(tag), nel, nv,
                                ctypes.byref(opts), nparts)


def test_tagged_without_tag_returns_1(lib):
    vtx, xyz = meshgen.box_hex(2, 2, 2)
    o = ParrsbOptions.make(tagged=1, verbose_level=0)
    assert _call(lib, vtx, xyz, 2, o) == 1  # src/parrsb.c:873-877


def test_tagged_parts_must_be_a_multiple_of_tags(lib):
    # the reference exits (src/parrsb.c:431-439); here: code 1, before any GPU work
    vtx, xyz = meshgen.box_hex(2, 2, 2)
    o = ParrsbOptions.make(tagged=1, verbose_level=0)
    tag = np.array([0, 0, 1, 1, 2, 2, 3, 3], np.int32)
    assert _call(lib, vtx, xyz, 6, o, tag=tag) == 1


def test_oracle_tagged_composition(oracle):
    """Tags are numbered in increasing order and partition independently:
    tag number t owns parts [t * chunk, (t + 1) * chunk)."""
    vtx, xyz = meshgen.box_hex(6, 5, 4, jitter=0.1, seed=1)
    tag = np.repeat(np.array([7, 3, 9, 3]), 30).astype(np.int32)  # z layers
    rc, part = oracle.part_mesh_tagged(vtx, xyz, tag, 9, partitioner=1)
    assert rc == 0
    for t, val in enumerate([3, 7, 9]):
        got = np.unique(part[tag == val])
        np.testing.assert_array_equal(got, np.arange(3 * t, 3 * t + 3))
    rc, _ = oracle.part_mesh_tagged(vtx, xyz, tag, 8, partitioner=1)
    assert rc == 1  # 8 parts over 3 tags


def test_both_inputs_null_is_an_error(lib):
    # the reference calls MPI_Abort (src/parrsb.c:244-249); here: code 1
    o = ParrsbOptions.make(verbose_level=0)
    assert _call(lib, None, None, 2, o, nel=4, nv=8) == 1


def test_bad_arguments(lib):
    vtx, xyz = meshgen.box_hex(2, 2, 2)
    o = ParrsbOptions.make(verbose_level=0)
    assert _call(lib, vtx, xyz, 0, o) == 1          # nparts < 1
    assert _call(lib, vtx, xyz, 2, o, nel=-1) == 1  # nel < 0
    assert _call(lib, vtx, xyz, 2, o, nv=9) == 1    # nv > 8
    o = ParrsbOptions.make(verbose_level=0, rsb_algo=1)
    assert _call(lib, vtx, xyz, 2, o) == P.ERR_UNSUPPORTED  # multigrid RSB
    o = ParrsbOptions.make(verbose_level=0, partitioner=0)
    assert _call(lib, None, xyz, 2, o) == 1          # RSB needs vertices


def test_env_overrides_written_back(lib, monkeypatch):
    """update_options (src/parrsb.c:48-77): PARRSB_* variables override the
    caller's struct and stay in it after the call; levels is clamped."""
    monkeypatch.setenv("PARRSB_RSB_MAX_ITER", "33")
    monkeypatch.setenv("PARRSB_RSB_TOL", "1e-7")
    monkeypatch.setenv("PARRSB_LEVELS", "5")
    monkeypatch.setenv("PARRSB_TAGGED", "1")  # makes the call stop before GPU work
    vtx, xyz = meshgen.box_hex(2, 2, 2)
    o = ParrsbOptions.make(verbose_level=0)
    assert _call(lib, vtx, xyz, 2, o) == 1
    assert o.rsb_max_iter == 33 and o.rsb_tol == 1e-7 and o.tagged == 1
    assert o.levels == 5  # returned before clamping, like the reference


def test_conn_mesh_argument_checks(lib):
    P_ = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    coord = np.zeros(8 * 3, np.float64)
    vtx = np.zeros(8, np.int64)
    assert lib.parrsb_conn_mesh(P_(vtx), P_(coord), 1, 4, None, 0, 0.2) == 1
    # periodic records: a negative count, or a count without records
    pinfo = np.ones(4, np.int64)
    assert lib.parrsb_conn_mesh(P_(vtx), P_(coord), 1, 3, P_(pinfo), -1, 0.2) == 1
    assert lib.parrsb_conn_mesh(P_(vtx), P_(coord), 1, 3, None, 1, 0.2) == 1
    err = ctypes.c_int(0)
    nel, nd, npf, tol = ctypes.c_int(1), ctypes.c_int(3), ctypes.c_int(1), ctypes.c_double(0.2)
    lib.fparrsb_conn_mesh(P_(vtx), P_(coord), ctypes.byref(nel), ctypes.byref(nd),
                          None, ctypes.byref(npf), ctypes.byref(tol), ctypes.byref(err))
    assert err.value == 1


def test_quality_rejects_out_of_range_parts(lib):
    vtx, _ = meshgen.box_hex(2, 1, 1)
    part = np.array([0, 5], np.int32)
    q = np.zeros(8)
    P_ = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    assert lib.parrsb_part_quality(P_(q), P_(part), P_(vtx), 2, 8, 2) == 1


def test_product_does_not_import_oracle():
    """The shipped package never imports or loads the oracle."""
    pkg = os.path.join(ROOT, "parrsb_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                text = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in text.lower().replace("the oracle", ""), f
