"""Mesh file I/O (src/io.c formats) on the host: .re2 read, .co2 write/read
round trip, .ma2 layout, and the reference's own example mesh when the
reference tree is available (it is not on the GPU machine)."""
import os

import numpy as np
import pytest

import parrsb_gb300 as P
from parrsb_gb300 import meshgen

# stem of the reference's examples/ethier mesh (only where a reference tree
# is available; the committed fixture stands in for it elsewhere)
ETHIER = os.environ.get("PARRSB_ETHIER", "")
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ethier.npz")


def test_re2_roundtrip(tmp_path, lib):
    _, xyz = meshgen.box_hex(5, 4, 3, jitter=0.1, seed=1)
    name = str(tmp_path / "box")
    P.write_re2(name, xyz, periodic=[(1, 2, 7, 4)])
    m = P.read_mesh(name, read=1)
    np.testing.assert_array_equal(m["coord"], xyz)
    assert m["periodic"].tolist() == [[1, 2, 7, 4]]


def test_re2_roundtrip_2d(tmp_path, lib):
    _, xyz = meshgen.annulus_quad(16, 8, seed=2)
    name = str(tmp_path / "ann")
    P.write_re2(name, xyz)
    m = P.read_mesh(name, read=1)
    np.testing.assert_array_equal(m["coord"], xyz)
    assert m["periodic"].shape == (0, 4)


def test_co2_roundtrip(tmp_path, lib):
    vtx, xyz = meshgen.box_hex(3, 3, 2, jitter=0.0)
    name = str(tmp_path / "c")
    P.write_re2(name, xyz)
    P.dump_con(name, vtx)
    m = P.read_mesh(name, read=3)
    np.testing.assert_array_equal(m["vtx"], vtx)
    raw = open(name + ".co2", "rb").read()
    assert raw[:5] == b"#v001" and len(raw) == 132 + 4 + len(vtx) * 9 * 4
    ints = np.frombuffer(raw[136:], np.int32).reshape(len(vtx), 9)
    assert ints[:, 0].tolist() == list(range(1, len(vtx) + 1))


def test_ma2_layout(tmp_path, lib):
    vtx, _ = meshgen.box_hex(4, 2, 2, jitter=0.0)
    part = (np.arange(len(vtx)) % 3).astype(np.int32)
    name = str(tmp_path / "m")
    P.dump_map(name, vtx, part)
    raw = open(name + ".ma2", "rb").read()
    hdr = raw[:132].decode().split()
    assert hdr[0] == "#v001" and int(hdr[1]) == 16 and int(hdr[3]) == 4 and int(hdr[4]) == 16
    ints = np.frombuffer(raw[136:], np.int32).reshape(16, 9)
    np.testing.assert_array_equal(ints[:, 0], part)
    np.testing.assert_array_equal(ints[:, 1:], vtx)


def test_missing_file_is_an_error(tmp_path, lib):
    with pytest.raises(P.ParrsbError):
        P.read_mesh(str(tmp_path / "nope"), read=1)


@pytest.mark.skipif(not os.path.exists(ETHIER + ".re2"),
                    reason="set PARRSB_ETHIER to the stem of the reference's examples/ethier")
def test_ethier_mesh_through_gencon_oracle(oracle, lib):
    """examples/ethier.re2 (32 hex elements, used by the reference's CI):
    read, number with the oracle's gencon, check the connectivity, and
    check that the committed fixture was made from this file."""
    m = P.read_mesh(ETHIER, read=1)
    coord = m["coord"]
    assert coord.shape == (32, 8, 3)
    rc, ids, _, nseg = oracle.conn_mesh(coord, 3, 0.2)
    assert rc == 0
    assert ids.min() == 1 and ids.max() == nseg
    rch, idsh, _, _ = oracle.conn_mesh(coord, 3, 0.2, heapsort=True)
    assert rch == 0
    np.testing.assert_array_equal(ids, idsh)
    g = np.load(GOLDEN)
    np.testing.assert_array_equal(g["coord"], coord)


def test_ethier_fixture_pins_the_oracle(oracle):
    """The committed ethier fixture (tests/golden/make_ethier.py): the
    oracle's gencon ids, heapsort mode included, and its RCB / RSB parts."""
    g = np.load(GOLDEN)
    rc, ids, _, nseg = oracle.conn_mesh(g["coord"], 3, 0.2)
    assert rc == 0 and nseg == int(g["nseg"])
    np.testing.assert_array_equal(ids, g["vtx"])
    rch, idsh, _, _ = oracle.conn_mesh(g["coord"], 3, 0.2, heapsort=True)
    assert rch == 0
    np.testing.assert_array_equal(idsh, g["vtx"])
    rc1, rcb, _, _, _ = oracle.part_mesh(g["vtx"], g["coord"], 4, partitioner=1)
    np.testing.assert_array_equal(rcb, g["rcb4"])
    rc0, rsb, _, _, _ = oracle.part_mesh(g["vtx"], g["coord"], 4, partitioner=0)
    np.testing.assert_array_equal(rsb, g["rsb4"])
