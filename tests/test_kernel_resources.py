"""CPU checks of the compiled kernels' resources (nvcc -Xptxas -v, no GPU).

The SpMV of the Lanczos steps is bound by the latency of its gathers, and
its speed depends on its register allocation: an 8-byte spill in
k_spmv<float> (caused by edits to the inlined finalisation code) took it from
0.176 to 0.237 ms per launch on the 8M-element benchmark.  These tests pin the
allocations that the measured kernels rely on."""
import os
import re
import shutil
import subprocess

import pytest

from parrsb_gb300 import build as B

pytestmark = pytest.mark.skipif(shutil.which(B.NVCC) is None, reason="nvcc not found")


def _ptxas_report(src):
    out = os.path.join(B.BUILD, "resources_" + src[:-3] + ".o")
    os.makedirs(B.BUILD, exist_ok=True)
    cmd = [B.NVCC] + B.ARCH + B.FLAGS + ["-Xptxas", "-v", "-c", os.path.join(B.CSRC, src),
                                         "-o", out]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr[-2000:]
    return p.stderr


def _entries(report):
    """{mangled entry name: (registers, spill store bytes, spill load bytes)}"""
    res, name, spill = {}, None, (0, 0)
    for line in report.splitlines():
        m = re.search(r"Compiling entry function '(\S+)'", line)
        if m:
            name = m.group(1)
            continue
        m = re.search(r"(\d+) bytes spill stores, (\d+) bytes spill loads", line)
        if m and name:
            spill = (int(m.group(1)), int(m.group(2)))
            continue
        m = re.search(r"Used (\d+) registers", line)
        if m and name:
            res[name] = (int(m.group(1)),) + spill
            name, spill = None, (0, 0)
    return res


@pytest.fixture(scope="module")
def rsb_entries():
    return _entries(_ptxas_report("rsb.cu"))


def test_spmv_float_does_not_spill(rsb_entries):
    spmv = {k: v for k, v in rsb_entries.items() if "k_spmvIf" in k}
    assert spmv, "k_spmv<float> not found in the ptxas report"
    for name, (regs, st, ld) in spmv.items():
        assert st == 0 and ld == 0, (name, regs, st, ld)
        assert regs <= 32, (name, regs)  # 64 resident warps per SM


def test_vector_updates_do_not_spill(rsb_entries):
    pr = {k: v for k, v in rsb_entries.items() if "k_prIf" in k}
    assert pr
    for name, (regs, st, ld) in pr.items():
        assert st == 0 and ld == 0, (name, regs, st, ld)


def test_sort_scatter_does_not_spill():
    ent = _entries(_ptxas_report("sort.cu"))
    sc = {k: v for k, v in ent.items() if "k_scatter" in k}
    assert sc
    for name, (regs, st, ld) in sc.items():
        assert st == 0 and ld == 0, (name, regs, st, ld)
