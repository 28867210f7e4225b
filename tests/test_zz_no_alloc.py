"""parrsb_part_mesh_rcb_noalloc: the allocation-free RCB entry point, called
through the C ABI on caller-owned device buffers, against the allocating
parrsb_part_mesh (partitioner = 1) and against the oracle's RCB.  RCB parts
are integers: the bar is equality.  Collected last so that it runs alone and
after every other test."""
import ctypes

import numpy as np
import pytest

import parrsb_gb300 as P
from oracle import oracle as O
from parrsb_gb300 import meshgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    return torch


def _noalloc(torch, xyz, nel, nv, nparts):
    d_xyz = torch.from_numpy(np.ascontiguousarray(xyz, dtype=np.float64).ravel()).cuda()
    d_part = torch.full((nel,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = P.library().parrsb_part_mesh_rcb_noalloc(
        ctypes.c_void_p(d_part.data_ptr()), ctypes.c_void_p(d_xyz.data_ptr()), nel, nv, nparts,
        ctypes.c_void_p(stream))
    torch.cuda.synchronize()
    return rc, d_part.cpu().numpy()


@pytest.mark.parametrize("mesh,nparts", [("box", 8), ("box", 13), ("box", 1),
                                         ("annulus", 100), ("ties", 7), ("full", 1024)])
def test_noalloc_rcb_matches_part_mesh(cuda, mesh, nparts):
    if mesh == "box":
        vtx, xyz = meshgen.box_hex(20, 16, 12, jitter=0.1, seed=3)
    elif mesh == "annulus":
        vtx, xyz = meshgen.annulus_quad(64, 32, amp=0.02, seed=5)
    elif mesh == "ties":
        vtx, xyz = meshgen.box_hex(16, 12, 9, jitter=0.0)
    else:
        vtx, xyz = meshgen.box_hex(32, 16, 16, jitter=0.1, seed=6)  # 8192 elements
    nel, nv = vtx.shape
    ref = P.part_mesh(vtx, xyz, nparts, partitioner=1)
    rc_o, ref_o, _, _, _ = O.part_mesh(vtx, xyz, nparts, partitioner=1)
    assert rc_o == 0
    np.testing.assert_array_equal(ref, ref_o)
    for call in range(2):  # two calls in a row reuse the same scratch
        rc, part = _noalloc(cuda, xyz, nel, nv, nparts)
        assert rc == 0
        np.testing.assert_array_equal(part, ref)
        np.testing.assert_array_equal(part, ref_o)


def test_noalloc_leaves_free_device_memory_unchanged(cuda):
    """The call's promise: no device allocation.  After one call has loaded
    the kernels, two more calls leave cudaMemGetInfo's free bytes as they
    were (the buffers are the caller's, allocated before)."""
    torch = cuda
    vtx, xyz = meshgen.box_hex(24, 16, 12, jitter=0.1, seed=9)
    nel, nv = vtx.shape
    d_xyz = torch.from_numpy(np.ascontiguousarray(xyz, dtype=np.float64).ravel()).cuda()
    d_part = torch.full((nel,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    lib = P.library()

    def call():
        return lib.parrsb_part_mesh_rcb_noalloc(
            ctypes.c_void_p(d_part.data_ptr()), ctypes.c_void_p(d_xyz.data_ptr()), nel, nv, 16,
            ctypes.c_void_p(stream))

    assert call() == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert call() == 0
    assert call() == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    rc_o, ref_o, _, _, _ = O.part_mesh(vtx, xyz, 16, partitioner=1)
    np.testing.assert_array_equal(d_part.cpu().numpy(), ref_o)


def test_noalloc_rejects_large_meshes(cuda):
    vtx, xyz = meshgen.box_hex(32, 16, 17, jitter=0.1, seed=1)  # 8704 > 8192
    nel, nv = vtx.shape
    rc, part = _noalloc(cuda, xyz, nel, nv, 8)
    assert rc == 4  # PARRSB_ERR_UNSUPPORTED, nothing launched
    assert (part == -1).all()
