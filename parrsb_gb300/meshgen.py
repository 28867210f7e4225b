"""Seeded synthetic meshes for tests and benchmarks.

Every generator returns corner coordinates in Nek5000 *preprocessor* corner
order (the order ``parrsb_conn_mesh`` expects, src/con-impl.h:8-16): for a
quad (i,j),(i+1,j),(i+1,j+1),(i,j+1); for a hex the same four at the lower
``k`` followed by the four at ``k+1``.  Vertex ids are 1-based lattice ids.

Random jitter uses PCG64 integers scaled by 2**-53 and separate numpy ufuncs
(no fused multiply-add), so a given seed gives the same bits on x86 and Arm.
Generators that use sin/cos (annulus, pipe) can differ in the last bit
between platforms; parity tests generate once and feed the same arrays to
the GPU path and to the oracle.
"""
import numpy as np

# preprocessor-order corner offsets
QUAD_CORNERS = np.array([[0, 0], [1, 0], [1, 1], [0, 1]], dtype=np.int64)
HEX_CORNERS = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                        [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]],
                       dtype=np.int64)


def _uniform_pm1(rng, shape):
    """Uniform values in [-1, 1) built from 53-bit integers (exact)."""
    u = rng.integers(0, 2 ** 53, size=shape, dtype=np.int64).astype(np.float64)
    u = u * (2.0 ** -53)
    return u * 2.0 - 1.0


def _hex_elements(nx, ny, nz):
    """Element lattice corners (nel, 8, 3) as integer (i, j, k)."""
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx),
                          indexing="ij")
    base = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1)  # x fastest
    return base[:, None, :] + HEX_CORNERS[None, :, :]


def box_hex(nx, ny, nz, jitter=0.1, seed=0, lo=(0.0, 0.0, 0.0),
            hi=(1.0, 1.0, 1.0), id_offset=0):
    """Structured hex box on [lo, hi] with uniform jitter of +-jitter*h on
    interior lattice vertices.  Returns (vtx[nel,8] int64, xyz[nel,8,3])."""
    rng = np.random.Generator(np.random.PCG64(seed))
    lo = np.asarray(lo, np.float64)
    hi = np.asarray(hi, np.float64)
    n = np.array([nx, ny, nz])
    h = (hi - lo) / n
    axes = [lo[d] + np.arange(n[d] + 1, dtype=np.float64) * h[d]
            for d in range(3)]
    X = np.empty((nz + 1, ny + 1, nx + 1, 3), np.float64)
    X[..., 0] = axes[0][None, None, :]
    X[..., 1] = axes[1][None, :, None]
    X[..., 2] = axes[2][:, None, None]
    if jitter:
        J = _uniform_pm1(rng, (nz - 1, ny - 1, nx - 1, 3))
        amp = np.asarray(jitter * h, np.float64)
        X[1:nz, 1:ny, 1:nx, :] = X[1:nz, 1:ny, 1:nx, :] + J * amp
    c = _hex_elements(nx, ny, nz)  # (nel, 8, 3) ints
    vid = c[..., 0] + (nx + 1) * (c[..., 1] + (ny + 1) * c[..., 2])
    xyz = X[c[..., 2], c[..., 1], c[..., 0]]
    vtx = (vid + 1 + id_offset).astype(np.int64)
    return np.ascontiguousarray(vtx), np.ascontiguousarray(xyz)


def box_quad(nx, ny, jitter=0.1, seed=0):
    """2D quad box on [0, 1]^2 with uniform jitter of +-jitter*h on interior
    lattice vertices.  Returns (vtx[nel,4] int64, xyz[nel,4,2]); elements
    are x-fastest."""
    rng = np.random.Generator(np.random.PCG64(seed))
    h = np.array([1.0 / nx, 1.0 / ny])
    X = np.empty((ny + 1, nx + 1, 2), np.float64)
    X[..., 0] = (np.arange(nx + 1, dtype=np.float64) * h[0])[None, :]
    X[..., 1] = (np.arange(ny + 1, dtype=np.float64) * h[1])[:, None]
    if jitter:
        J = _uniform_pm1(rng, (ny - 1, nx - 1, 2))
        X[1:ny, 1:nx, :] = X[1:ny, 1:nx, :] + J * np.asarray(jitter * h, np.float64)
    j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    base = np.stack([i.ravel(), j.ravel()], axis=1)
    c = base[:, None, :] + QUAD_CORNERS[None, :, :]
    xyz = X[c[..., 1], c[..., 0]]
    vid = c[..., 0] + (nx + 1) * c[..., 1]
    return np.ascontiguousarray((vid + 1).astype(np.int64)), np.ascontiguousarray(xyz)


def periodic_x_faces(nx, ny, nz=None, both=True):
    """Periodic face records (element, face, partner element, partner face;
    1-based, preprocessor face numbers 4 = x-low, 2 = x-high) joining the
    x = 0 and x = 1 sides of box_hex(nx, ny, nz) or, with nz None, of
    box_quad(nx, ny).  both: list every pair from both sides, as Nek's .re2
    boundary section does."""
    layers = 1 if nz is None else nz
    out = []
    for k in range(layers):
        for j in range(ny):
            lo = 1 + nx * (j + ny * k)
            hi = lo + nx - 1
            out.append((lo, 4, hi, 2))
            if both:
                out.append((hi, 2, lo, 4))
    return np.array(out, dtype=np.int64).reshape(-1, 4)


def annulus_quad(nt, nr, amp=0.02, seed=0):
    """2D quad annulus r in [1, 2]: nt elements around, nr across.  The
    radius carries a seeded sinusoidal perturbation of amplitude `amp`
    (mode 3..8, random phase) that vanishes on both circles.  Returns
    (vtx[nel,4] int64, xyz[nel,4,2]); every element holds its own copy of
    its corner coordinates."""
    rng = np.random.Generator(np.random.PCG64(seed))
    mode = int(rng.integers(3, 9))
    phase = float(rng.integers(0, 2 ** 53)) * (2.0 ** -53) * 2.0 * np.pi
    i = np.arange(nt + 1, dtype=np.float64)
    j = np.arange(nr + 1, dtype=np.float64)
    th = i * (2.0 * np.pi / nt)
    r = 1.0 + j / nr
    R = r[None, :] + amp * np.sin(mode * th + phase)[:, None] * \
        np.sin(np.pi * j / nr)[None, :]
    X = R * np.cos(th)[:, None]
    Y = R * np.sin(th)[:, None]
    X[nt, :] = X[0, :]
    Y[nt, :] = Y[0, :]
    jj, ii = np.meshgrid(np.arange(nr), np.arange(nt), indexing="ij")
    base = np.stack([ii.ravel(), jj.ravel()], axis=1)  # tangential fastest
    c = base[:, None, :] + QUAD_CORNERS[None, :, :]
    xyz = np.stack([X[c[..., 0], c[..., 1]], Y[c[..., 0], c[..., 1]]], -1)
    vid = (c[..., 0] % nt) + nt * c[..., 1]
    return (np.ascontiguousarray((vid + 1).astype(np.int64)),
            np.ascontiguousarray(xyz))


def pipe_hex(nt, nr, nz, jitter=0.05, seed=0, length=4.0):
    """Hex annular cylinder r in [1, 2], z in [0, length]: nt elements
    around, nr across, nz along.  Interior lattice vertices are jittered by
    +-jitter*h (h per lattice direction).  Returns (vtx, xyz[nel,8,3])."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ti = np.arange(nt, dtype=np.float64)  # periodic: index nt wraps to 0
    rj = np.arange(nr + 1, dtype=np.float64)
    zk = np.arange(nz + 1, dtype=np.float64)
    T, Rr, Z = np.meshgrid(ti, rj, zk, indexing="ij")  # (nt, nr+1, nz+1)
    if jitter:
        J = _uniform_pm1(rng, (nt, nr - 1, nz - 1, 3)) * jitter
        T[:, 1:nr, 1:nz] = T[:, 1:nr, 1:nz] + J[..., 0]
        Rr[:, 1:nr, 1:nz] = Rr[:, 1:nr, 1:nz] + J[..., 1]
        Z[:, 1:nr, 1:nz] = Z[:, 1:nr, 1:nz] + J[..., 2]
    th = T * (2.0 * np.pi / nt)
    r = 1.0 + Rr / nr
    X = r * np.cos(th)
    Y = r * np.sin(th)
    Zc = Z * (length / nz)
    kk, jj, ii = np.meshgrid(np.arange(nz), np.arange(nr), np.arange(nt),
                             indexing="ij")
    base = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1)
    c = base[:, None, :] + HEX_CORNERS[None, :, :]
    a, b, d = c[..., 0] % nt, c[..., 1], c[..., 2]
    xyz = np.stack([X[a, b, d], Y[a, b, d], Zc[a, b, d]], -1)
    vid = a + nt * (b + (nr + 1) * d)
    return (np.ascontiguousarray((vid + 1).astype(np.int64)),
            np.ascontiguousarray(xyz))


def subboxes(count, smin=200, smax=20000, delete=0.05, seed=0, jitter=0.1):
    """`count` disjoint jittered hex sub-boxes with log-uniform element counts
    in [smin, smax] and a fraction `delete` of elements removed at random.
    Returns (vtx, xyz, seg) where seg[e] is the sub-box of element e (the
    boxes are concatenated in order and never share vertex ids)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    vts, xys, segs = [], [], []
    off = 0
    for b in range(count):
        u = float(rng.integers(0, 2 ** 53)) * (2.0 ** -53)
        target = float(np.exp(np.log(smin) + u * (np.log(smax) - np.log(smin))))
        # box shape: nx >= ny >= nz roughly cubic
        side = max(2, int(round(target ** (1.0 / 3.0))))
        nz = max(1, side - int(rng.integers(0, 2)))
        ny = side
        nx = max(2, int(round(target / (ny * nz))))
        v, x = box_hex(nx, ny, nz, jitter=jitter, seed=seed * 100003 + b + 1,
                       lo=(3.0 * b, 0.0, 0.0), hi=(3.0 * b + 1.0, 1.0, 1.0),
                       id_offset=off)
        off += (nx + 1) * (ny + 1) * (nz + 1)
        keep = rng.integers(0, 2 ** 53, size=len(v)) * (2.0 ** -53) >= delete
        if keep.sum() < 2:
            keep[:2] = True
        vts.append(v[keep])
        xys.append(x[keep])
        segs.append(np.full(int(keep.sum()), b, np.int32))
    return (np.ascontiguousarray(np.concatenate(vts)),
            np.ascontiguousarray(np.concatenate(xys)),
            np.concatenate(segs))


def duplicate_corner_coords(xyz):
    """Coordinates for gencon: already one copy per element corner."""
    return np.ascontiguousarray(xyz.reshape(len(xyz), -1))


def lattice_ids_hex(nx, ny, nz):
    """Expected gencon ids for an unjittered or mildly jittered box are an
    equivalence of the lattice ids; returned for equivalence checks."""
    c = _hex_elements(nx, ny, nz)
    return c[..., 0] + (nx + 1) * (c[..., 1] + (ny + 1) * c[..., 2])
