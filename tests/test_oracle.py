"""CPU tests pinning the oracle with known answers derived from first
principles (the reference ships no golden vectors and cannot be built here:
it needs MPI and gslib).  Each test names the reference behaviour it pins.
"""
import math

import numpy as np
import pytest

from parrsb_gb300 import meshgen

SYM = [0, 1, 3, 2, 4, 5, 7, 6]  # preprocessor -> symmetric corner order


def py_tree_sum(x):
    """Independent restatement of the canonical 32-wide tile tree."""
    buf = list(map(float, x))
    if not buf:
        return 0.0
    while True:
        out = []
        for t in range(0, len(buf), 32):
            v = buf[t:t + 32] + [0.0] * (32 - len(buf[t:t + 32]))
            off = 16
            while off:
                for i in range(off):
                    v[i] = v[i] + v[i + off]
                off //= 2
            out.append(v[0])
        buf = out
        if len(buf) == 1:
            return buf[0]


@pytest.mark.parametrize("n", [0, 1, 2, 31, 32, 33, 1000, 40000])
def test_tree_sum_matches_restatement(oracle, n):
    x = np.random.default_rng(n).standard_normal(n)
    assert oracle.tree_sum(x) == py_tree_sum(x)
    if n:
        assert math.isclose(oracle.tree_sum(x), math.fsum(x), rel_tol=1e-12, abs_tol=1e-12)


def test_power_serial_dominant_eigenvector(oracle):
    """power_serial (src/fiedler.c:38-73) converges to the dominant
    eigenvector of a symmetric 3x3 tensor."""
    A = np.array([[4.0, 1.0, 0.5], [1.0, 3.0, 0.2], [0.5, 0.2, 1.0]])
    y, it = oracle.power_serial(A, 3)
    w, V = np.linalg.eigh(A)
    assert abs(abs(y @ V[:, -1]) - 1.0) < 1e-6
    assert it < 100


def test_power_serial_2d_reads_first_four_entries(oracle):
    """In 2D, get_rib_axis passes the 3x3 tensor with N = 2, so the matrix
    seen is [[I00, I01], [I02, I10]] (src/rib.c:30-47)."""
    I = np.array([[5.0, 0.3, 0.0], [0.3, 2.0, 0.0], [0.0, 0.0, 0.0]])
    y, _ = oracle.power_serial(I.ravel(), 2)
    A2 = I.ravel()[:4].reshape(2, 2)  # [[5, .3], [0, .3]]
    w, V = np.linalg.eig(A2)
    v = V[:, np.argmax(abs(w))].real
    assert abs(abs(y @ v) / np.linalg.norm(v) - 1.0) < 1e-6


def test_tqli_eigenpairs(oracle):
    """tqli (src/fiedler.c:328-432) returns the eigenvalues of the symmetric
    tridiagonal matrix and normalised eigenvectors (rows)."""
    rng = np.random.default_rng(1)
    n = 40
    d = rng.uniform(1, 3, n)
    e = rng.uniform(-1, 1, n - 1)
    rc, ew, ev = oracle.tqli(d, e)
    assert rc == 0
    T = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    np.testing.assert_allclose(np.sort(ew), np.linalg.eigvalsh(T), rtol=1e-10, atol=1e-10)
    for k in range(n):
        np.testing.assert_allclose(T @ ev[k], ew[k] * ev[k], atol=1e-9)
        assert abs(np.linalg.norm(ev[k]) - 1.0) < 1e-12


def test_dual_graph_box_stencil(oracle):
    """The gather-scatter Laplacian (src/laplacian.c:159-205) of a hex box is
    the 27-point stencil with weights 4 (face), 2 (edge), 1 (corner)."""
    n = 4
    vtx, _ = meshgen.box_hex(n, n, n, jitter=0.0)
    rowptr, col, w = oracle.dual_graph(vtx)
    idx = lambda i, j, k: i + n * (j + n * k)
    for (i, j, k) in [(1, 1, 1), (0, 0, 0), (3, 1, 2)]:
        a = idx(i, j, k)
        got = dict(zip(col[rowptr[a]:rowptr[a + 1]].tolist(), w[rowptr[a]:rowptr[a + 1]].tolist()))
        want = {}
        for di in (-1, 0, 1):
            for dj in (-1, 0, 1):
                for dk in (-1, 0, 1):
                    if (di, dj, dk) == (0, 0, 0):
                        continue
                    ii, jj, kk = i + di, j + dj, k + dk
                    if 0 <= ii < n and 0 <= jj < n and 0 <= kk < n:
                        want[idx(ii, jj, kk)] = 4 >> (abs(di) + abs(dj) + abs(dk) - 1)
        assert got == want
    # interior row: 26 neighbours, diagonal 6*4 + 12*2 + 8*1 = 56
    a = idx(1, 1, 1)
    assert rowptr[a + 1] - rowptr[a] == 26 and w[rowptr[a]:rowptr[a + 1]].sum() == 56


def test_laplacian_apply_matches_csr(oracle):
    vtx, _ = meshgen.box_hex(5, 4, 3, jitter=0.0)
    x = np.random.default_rng(0).standard_normal(len(vtx))
    y = oracle.laplacian(x, vtx)
    rowptr, col, w = oracle.dual_graph(vtx)
    ref = np.array([sum(w[q] * (x[a] - x[col[q]]) for q in range(rowptr[a], rowptr[a + 1]))
                    for a in range(len(vtx))])
    np.testing.assert_allclose(y, ref, rtol=1e-13, atol=1e-12)
    assert abs(y.sum()) < 1e-9  # L 1 = 0


def test_fiedler_of_chain_is_cosine(oracle):
    """A 1D chain of hexes is a path graph (weight 4): its Fiedler vector is
    cos(pi (i + 1/2) / n) up to sign."""
    n = 48
    vtx, _ = meshgen.box_hex(n, 1, 1, jitter=0.0)
    f, it = oracle.fiedler(vtx, 50, 50, 1e-8)
    ref = np.cos(np.pi * (np.arange(n) + 0.5) / n)
    ref /= np.linalg.norm(ref)
    assert abs(abs(f @ ref) - 1.0) < 1e-6


def test_rcb_cube_octants(oracle):
    """RCB of an unjittered 8^3 cube into 8 parts: first cut on x (ties in
    the bounding box pick the first axis), then y, then z
    (src/rcb.c:74-137)."""
    n = 8
    vtx, xyz = meshgen.box_hex(n, n, n, jitter=0.0)
    rc, part, order, _, _ = oracle.part_mesh(vtx, xyz, 8, partitioner=1, want_order=True)
    assert rc == 0
    e = np.arange(n ** 3)
    i, j, k = e % n, (e // n) % n, e // (n * n)
    np.testing.assert_array_equal(part, 4 * (i >= 4) + 2 * (j >= 4) + (k >= 4))
    assert sorted(order.tolist()) == list(range(n ** 3))


def test_rcb_slabs_and_counts(oracle):
    """A 64x1x1 chain into 5 parts: set_proc_from_idx gives the first
    p - n%p ranks n/p elements and the others one more (src/sort.c:48-70);
    bisection splits ceil(p/2) / floor(p/2) ranks (src/rcb.c:126)."""
    vtx, xyz = meshgen.box_hex(64, 1, 1, jitter=0.0)
    rc, part, _, _, _ = oracle.part_mesh(vtx, xyz, 5, partitioner=1)
    sizes = np.bincount(part)
    assert sizes.sum() == 64 and sizes.max() - sizes.min() <= 1
    assert np.all(np.diff(part) >= 0)  # slabs in x order


def test_gencon_box_recovers_lattice(oracle):
    """gencon on a jittered box with duplicated corners numbers the (n+1)^3
    lattice vertices; the ids are a bijection of the lattice ids (the test of
    examples/gencon.c:6-68 checks exactly this equivalence)."""
    for shape in [(6, 5, 4), (16, 16, 16)]:
        vtx, xyz = meshgen.box_hex(*shape, jitter=0.1, seed=2)
        rc, ids, _, nseg = oracle.conn_mesh(xyz, 3, 0.2)
        assert rc == 0
        nx, ny, nz = shape
        assert nseg == (nx + 1) * (ny + 1) * (nz + 1)
        pairs = set(zip(vtx[:, SYM].ravel().tolist(), ids.ravel().tolist()))
        assert len(pairs) == nseg
        assert ids.min() == 1 and ids.max() == nseg


def test_gencon_heapsort_and_stable_agree(oracle):
    """The reference's per-segment heapsort and the stable order give the
    same ids on these meshes (no split decision sits on an exact tie)."""
    for (vtx, xyz), nd in [(meshgen.box_hex(7, 6, 5, jitter=0.1, seed=3), 3),
                           (meshgen.annulus_quad(64, 32, seed=1), 2)]:
        a = oracle.conn_mesh(xyz, nd, 0.2, heapsort=False)
        b = oracle.conn_mesh(xyz, nd, 0.2, heapsort=True)
        assert a[0] == b[0] == 0
        np.testing.assert_array_equal(a[1], b[1])


def test_gencon_dense_annulus_fails(oracle):
    """Documented behaviour of the reference algorithm: on the 512x512
    annulus at tol 0.2 the one-coordinate gaps cannot separate vertices, so
    element_check fails and parrsb_conn_mesh returns 1."""
    _, xyz = meshgen.annulus_quad(512, 512, amp=0.02, seed=0)
    rc, _, ids, nseg = oracle.conn_mesh(xyz, 2, 0.2)
    assert rc == 1 and nseg < 512 * 513


def test_gencon_face_check_detects_hanging_corner(oracle):
    """face_check (src/con-check.c:197-263): an element sharing exactly 3
    corners of another element's face is an error."""
    _, xyz = meshgen.box_hex(2, 1, 1, jitter=0.0)
    xyz = xyz.copy()
    # move one corner of the shared face of element 1 away (non-conforming)
    xyz[1, 3] = xyz[1, 3] + np.array([0.0, 0.0, 0.3])
    rc, _, _, _ = oracle.conn_mesh(xyz, 3, 0.05)
    assert rc == 1


def test_components_two_boxes(oracle):
    v1, _ = meshgen.box_hex(3, 3, 3, jitter=0.0)
    v2, _ = meshgen.box_hex(2, 2, 2, jitter=0.0, id_offset=1000)
    vtx = np.concatenate([v1, v2])
    assert oracle.components(vtx) == 2
    mask = np.zeros(len(vtx), np.int32)
    mask[:27] = 1
    assert oracle.components(vtx, mask) == 1


def test_rsb_cube_is_balanced_and_converges(oracle):
    vtx, xyz = meshgen.box_hex(16, 16, 16, jitter=0.1, seed=0)
    rc, part, _, info, _ = oracle.part_mesh(vtx, xyz, 8, partitioner=0)
    assert rc == 0
    assert np.bincount(part).tolist() == [512] * 8
    assert info.levels == 3 and info.nbisect == 7 and info.unconverged == 0
    assert info.max_components == 1
    assert info.max_resid < 1e-4


def test_rsb_uneven_sizes(oracle):
    """With n % p != 0 the halves follow balance_partitions' expected counts
    (src/rsb.c:138-140); final part sizes differ by at most one."""
    vtx, xyz = meshgen.box_hex(10, 9, 7, jitter=0.1, seed=3)
    for p in (3, 5, 7):
        rc, part, _, info, _ = oracle.part_mesh(vtx, xyz, p, partitioner=0)
        s = np.bincount(part, minlength=p)
        assert s.sum() == 630 and s.max() - s.min() <= 1, s


def test_part_quality_counts(oracle):
    n = 4
    vtx, _ = meshgen.box_hex(n, n, n, jitter=0.0)
    e = np.arange(n ** 3)
    part = (e % n >= 2).astype(np.int32)  # cut the box in x
    q = oracle.part_quality(part, vtx, 2)
    assert q[2] == n * n                          # face pairs across the plane
    assert q[1] == n * n + 2 * 2 * n * (n - 1) + 4 * (n - 1) ** 2  # +edge +corner pairs
    assert q[3] == q[4] == 32 and q[5] == 1.0
    assert q[6] == 2 * (n + 1) ** 2               # shared plane vertices, counted twice
    assert q[7] == 1


def test_unknown_partitioner_block_distribution(oracle):
    vtx, xyz = meshgen.box_hex(5, 2, 1, jitter=0.0)
    rc, part, _, _, _ = oracle.part_mesh(vtx, xyz, 3, partitioner=7)
    # first nel % p ranks get one more element (src/parrsb.c:112-137)
    assert np.bincount(part).tolist() == [4, 3, 3]


# ------------------------------------------------------------- periodic gencon
def test_oracle_periodic_one_sided_records_pair_nothing(oracle):
    """A face pairs only with a face that is itself listed
    (src/con-periodic.c:157-170): records from one side alone merge nothing."""
    nx, ny, nz = 5, 4, 3
    _, xyz = meshgen.box_hex(nx, ny, nz, jitter=0.1, seed=2)
    rc, _, _, nseg = oracle.conn_mesh(xyz, 3, 0.2,
                                      periodic=meshgen.periodic_x_faces(nx, ny, nz, False))
    assert rc == 0 and nseg == (nx + 1) * (ny + 1) * (nz + 1)


def test_oracle_periodic_box_wraps_x(oracle):
    """Periodic x faces of a jittered hex box: the x = 0 and x = 1 vertices
    merge, giving nx (ny + 1)(nz + 1) ids, and every id equals the lattice
    id with i taken modulo nx."""
    nx, ny, nz = 5, 4, 3
    vtx, xyz = meshgen.box_hex(nx, ny, nz, jitter=0.1, seed=2)
    rc, ids, _, nseg = oracle.conn_mesh(xyz, 3, 0.2,
                                        periodic=meshgen.periodic_x_faces(nx, ny, nz))
    assert rc == 0
    assert nseg == nx * (ny + 1) * (nz + 1)
    # lattice (i, j, k) of each corner in symmetric order, i wrapped
    lat = vtx - 1
    i, rest = lat % (nx + 1), lat // (nx + 1)
    wrapped = (i % nx) + nx * rest
    sym = [0, 1, 3, 2, 4, 5, 7, 6]
    w = wrapped[:, sym]
    # equal lattice points <-> equal ids
    pairs = {}
    for a, b in zip(w.ravel(), ids.ravel()):
        assert pairs.setdefault(a, b) == b
    assert len(set(ids.ravel())) == nseg


def test_oracle_periodic_quad_and_errors(oracle):
    nx, ny = 6, 4
    _, xyz = meshgen.box_quad(nx, ny, jitter=0.1, seed=3)
    rc, _, _, nseg = oracle.conn_mesh(xyz, 2, 0.2, periodic=meshgen.periodic_x_faces(nx, ny))
    assert rc == 0 and nseg == nx * (ny + 1)
    rc, _, _, _ = oracle.conn_mesh(xyz, 2, 0.2, periodic=[(1, 4, 99, 2)])
    assert rc == 1  # record out of range
    # an x-low face paired with the x-high face of a jittered interior element
    _, xyz3 = meshgen.box_hex(5, 4, 3, jitter=0.1, seed=2)
    rc, _, _, _ = oracle.conn_mesh(xyz3, 3, 0.2, periodic=[(1, 4, 27, 2), (27, 2, 1, 4)])
    assert rc == 3  # faces do not coincide


def _rows_by_occurrence(vtx):
    """The GPU dual-graph rows' enumeration, restated in numpy: slots sorted
    stably by vertex id; the candidates of element a are the runs of its
    vertices, vertex by vertex; b's weight is its number of occurrences and
    it is listed at its first occurrence."""
    nel, nv = vtx.shape
    flat = vtx.reshape(-1)
    order = np.argsort(flat, kind="stable")  # sorted slots
    sorted_ids = flat[order]
    starts = np.flatnonzero(np.r_[True, sorted_ids[1:] != sorted_ids[:-1]])
    ends = np.r_[starts[1:], len(flat)]
    run_of_pos = np.repeat(np.arange(len(starts)), ends - starts)
    pos_of_slot = np.empty_like(order)
    pos_of_slot[order] = np.arange(len(order))
    rows = []
    for a in range(nel):
        cand = []
        for k in range(nv):
            r = run_of_pos[pos_of_slot[a * nv + k]]
            cand.extend((order[starts[r]:ends[r]] // nv).tolist())
        seen, row = {}, []
        for b in cand:
            if b == a:
                continue
            if b not in seen:
                seen[b] = 0
                row.append(b)
            seen[b] += 1
        rows.append([(b, seen[b]) for b in row])
    return rows


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_dual_graph_weights_are_run_occurrences(oracle, seed):
    """Counting an element's occurrences in the vertex runs of another gives
    the number of equal (corner, corner) pairs, repeated vertex ids inside
    an element included: the rows equal the oracle's dual graph."""
    rng = np.random.default_rng(seed)
    nel, nv = 60, 8
    vtx = rng.integers(1, 90, size=(nel, nv)).astype(np.int64)  # repeats within elements
    rowptr, col, w = oracle.dual_graph(vtx)
    rows = _rows_by_occurrence(vtx)
    for a in range(nel):
        want = dict(zip(col[rowptr[a]:rowptr[a + 1]].tolist(),
                        w[rowptr[a]:rowptr[a + 1]].tolist()))
        got = dict(rows[a])
        assert got == want, a
        assert len(rows[a]) == len(got)  # each neighbour listed once


def test_oracle_threads_do_not_change_results(oracle):
    """The oracle splits sums into fixed blocks of 65,536 values and runs
    the halves of a bisection on disjoint scratch: 1 or 4 host threads give
    bitwise the same partition, Lanczos steps and residual."""
    from parrsb_gb300 import meshgen
    vtx, xyz = meshgen.box_hex(48, 40, 40, jitter=0.1, seed=3)  # 76,800 > one block
    res = []
    for t in (1, 4):
        oracle.threads(t)
        rc, part, _, info, _ = oracle.part_mesh(vtx, xyz, 16, partitioner=0)
        assert rc == 0
        res.append((part, info.total_iters, info.max_resid))
    oracle.threads(0)
    np.testing.assert_array_equal(res[0][0], res[1][0])
    assert res[0][1] == res[1][1] and res[0][2] == res[1][2]
