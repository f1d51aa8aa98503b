"""Seeded synthetic node coordinates, cell lists and initial states of the
benchmark workloads, in plain numpy.

This module imports nothing from the package, so code that must not load the
native library (the CPU oracle's side of the benchmark) can load it by path.
:mod:`solvcon_gb300.meshgen` re-exports it and adds the mesh builds.

* :func:`tri_square` -- unit square, n x n quads each cut on the same
  diagonal into 2 triangles, interior nodes jittered by U(-j h, j h).
* :func:`tet_cube` -- unit cube, n^3 hexes each cut into the 6 Kuhn
  tetrahedra around the v0-v6 diagonal, interior nodes jittered likewise.
* :func:`quad_square`, :func:`hex_cube`, :func:`prism_slab` -- the other
  cell types on the same grids.
* :func:`quadrant_state` -- four-quadrant Riemann state drawn from a seed.
* :func:`blast_state` -- spherical blast, (rho, p) = (1, 1) inside r < 0.2.
* :func:`sod_tube_state` -- a Sod-type 1D tube with random states.
"""

import numpy as np

# Cell type ids (the reference's StaticMesh constants).
QUADRILATERAL, TRIANGLE, HEXAHEDRON, TETRAHEDRON, PRISM = 3, 4, 5, 6, 7


def _jitter(coord, nside, ndim, frac, seed):
    rng = np.random.Generator(np.random.PCG64(seed))
    h = 1.0 / nside
    idx = np.indices((nside + 1,) * ndim).reshape(ndim, -1)[::-1].T
    interior = np.all((idx > 0) & (idx < nside), axis=1)
    noise = rng.uniform(-frac * h, frac * h, size=coord.shape)
    coord[interior] += noise[interior]
    return coord


def tri_square(nside, jitter=0.2, seed=0):
    """Jittered triangulated unit square: (ndcrd, cltpn, clnds)."""
    n = int(nside)
    xs = np.linspace(0.0, 1.0, n + 1)
    gx, gy = np.meshgrid(xs, xs, indexing="xy")
    ndcrd = np.stack([gx.ravel(), gy.ravel()], axis=1)
    if jitter:
        ndcrd = _jitter(ndcrd, n, 2, jitter, seed)
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a = (j * (n + 1) + i).ravel()
    b = a + 1
    c = a + n + 2
    d = a + n + 1
    t1 = np.stack([a, b, c], axis=1)
    t2 = np.stack([a, c, d], axis=1)
    tri = np.empty((2 * n * n, 3), dtype="int32")
    tri[0::2] = t1
    tri[1::2] = t2
    clnds = np.full((tri.shape[0], 9), -1, dtype="int32")
    clnds[:, 0] = 3
    clnds[:, 1:4] = tri
    cltpn = np.full(tri.shape[0], TRIANGLE, dtype="int32")
    return ndcrd, cltpn, clnds


def quad_square(nside, jitter=0.0, seed=0):
    """(Jittered) quadrilateral unit square: (ndcrd, cltpn, clnds)."""
    n = int(nside)
    xs = np.linspace(0.0, 1.0, n + 1)
    gx, gy = np.meshgrid(xs, xs, indexing="xy")
    ndcrd = np.stack([gx.ravel(), gy.ravel()], axis=1)
    if jitter:
        ndcrd = _jitter(ndcrd, n, 2, jitter, seed)
    j, i = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    a = (j * (n + 1) + i).ravel()
    clnds = np.full((n * n, 9), -1, dtype="int32")
    clnds[:, 0] = 4
    clnds[:, 1:5] = np.stack([a, a + 1, a + n + 2, a + n + 1], axis=1)
    cltpn = np.full(n * n, QUADRILATERAL, dtype="int32")
    return ndcrd, cltpn, clnds


# The 6 Kuhn tetrahedra of a hex around its v0-v6 diagonal, as local vertex
# ids with v0=(0,0,0) v1=(1,0,0) v2=(1,1,0) v3=(0,1,0) v4=(0,0,1) v5=(1,0,1)
# v6=(1,1,1) v7=(0,1,1).
_KUHN = np.array([[0, 1, 2, 6], [0, 1, 5, 6], [0, 3, 2, 6],
                  [0, 3, 7, 6], [0, 4, 5, 6], [0, 4, 7, 6]], dtype="int64")


def tet_cube(nside, jitter=0.15, seed=0):
    """Jittered Kuhn-tetrahedralised unit cube: (ndcrd, cltpn, clnds)."""
    n = int(nside)
    xs = np.linspace(0.0, 1.0, n + 1)
    gz, gy, gx = np.meshgrid(xs, xs, xs, indexing="ij")
    ndcrd = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1)
    if jitter:
        ndcrd = _jitter(ndcrd, n, 3, jitter, seed)
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n),
                          indexing="ij")
    s = n + 1
    base = (k * s * s + j * s + i).ravel()
    off = np.array([0, 1, 1 + s, s, s * s, 1 + s * s, 1 + s + s * s,
                    s + s * s], dtype="int64")
    verts = base[:, None] + off[None, :]             # [nhex, 8]
    tets = verts[:, _KUHN].reshape(-1, 4)           # [6 nhex, 4]
    # Orient every tetrahedron positively.
    p = ndcrd[tets]
    det = np.einsum("ij,ij->i", p[:, 1] - p[:, 0],
                    np.cross(p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]))
    neg = det < 0
    tets[neg, 1], tets[neg, 2] = tets[neg, 2].copy(), tets[neg, 1].copy()
    clnds = np.full((tets.shape[0], 9), -1, dtype="int32")
    clnds[:, 0] = 4
    clnds[:, 1:5] = tets
    cltpn = np.full(tets.shape[0], TETRAHEDRON, dtype="int32")
    return ndcrd, cltpn, clnds


def hex_cube(nside, jitter=0.0, seed=0):
    """(Jittered) hexahedral unit cube: (ndcrd, cltpn, clnds)."""
    n = int(nside)
    xs = np.linspace(0.0, 1.0, n + 1)
    gz, gy, gx = np.meshgrid(xs, xs, xs, indexing="ij")
    ndcrd = np.stack([gx.ravel(), gy.ravel(), gz.ravel()], axis=1)
    if jitter:
        ndcrd = _jitter(ndcrd, n, 3, jitter, seed)
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n),
                          indexing="ij")
    s = n + 1
    base = (k * s * s + j * s + i).ravel()
    off = np.array([0, 1, 1 + s, s, s * s, 1 + s * s, 1 + s + s * s,
                    s + s * s], dtype="int64")
    clnds = np.full((base.size, 9), -1, dtype="int32")
    clnds[:, 0] = 8
    clnds[:, 1:9] = base[:, None] + off[None, :]
    cltpn = np.full(base.size, HEXAHEDRON, dtype="int32")
    return ndcrd, cltpn, clnds


def prism_slab(nside, nz, jitter=0.0, seed=0):
    """Triangulated unit square (:func:`tri_square`) extruded into nz layers
    of prisms over z in [0, 1]: (ndcrd, cltpn, clnds)."""
    x2, _, c2 = tri_square(nside, jitter, seed)
    nn = x2.shape[0]
    zs = np.linspace(0.0, 1.0, nz + 1)
    ndcrd = np.concatenate([np.column_stack([x2, np.full(nn, z)])
                            for z in zs])
    tri = c2[:, 1:4].astype("int64")
    cells = []
    for layer in range(nz):
        lo = tri + layer * nn
        cells.append(np.concatenate([lo, lo + nn], axis=1))
    pr = np.concatenate(cells)
    clnds = np.full((pr.shape[0], 9), -1, dtype="int32")
    clnds[:, 0] = 6
    clnds[:, 1:7] = pr
    cltpn = np.full(pr.shape[0], PRISM, dtype="int32")
    return ndcrd, cltpn, clnds


def conserved(rho, vel, p, gamma):
    """Conserved rows [rho, rho v, p/(gamma-1) + rho |v|^2 / 2]."""
    rho = np.asarray(rho, dtype="float64")
    vel = np.asarray(vel, dtype="float64")
    gamma = np.broadcast_to(np.asarray(gamma, dtype="float64"), rho.shape)
    out = np.empty(rho.shape + (vel.shape[-1] + 2,), dtype="float64")
    out[..., 0] = rho
    out[..., 1:-1] = rho[..., None] * vel
    out[..., -1] = p / (gamma - 1.0) + 0.5 * rho * np.sum(vel * vel, axis=-1)
    return out


def quadrant_state(clcnd, seed=0, gamma=1.4):
    """Four-quadrant Riemann state split at x = y = 0.5, drawn from a seed:
    (rho, p) ~ U[0.1, 1.5], u, v ~ U[-0.8, 0.8] per quadrant."""
    rng = np.random.Generator(np.random.PCG64(seed + 7919))
    rho_q = rng.uniform(0.1, 1.5, 4)
    p_q = rng.uniform(0.1, 1.5, 4)
    v_q = rng.uniform(-0.8, 0.8, (4, 2))
    q = (clcnd[:, 0] >= 0.5).astype(int) + 2 * (clcnd[:, 1] >= 0.5)
    return conserved(rho_q[q], v_q[q], p_q[q], gamma)


def blast_state(clcnd, gamma=1.4, center=(0.5, 0.5, 0.5), radius=0.2):
    """Spherical blast: (rho, p) = (1, 1) inside r < radius, (0.125, 0.1)
    outside, at rest."""
    r = np.linalg.norm(clcnd - np.asarray(center)[None, :], axis=1)
    inside = r < radius
    rho = np.where(inside, 1.0, 0.125)
    p = np.where(inside, 1.0, 0.1)
    return conserved(rho, np.zeros_like(clcnd), p, gamma)


def sod_tube_state(ncoord, seed):
    """A Sod-type tube on [-1, 1]: random left/right (rho, p), at rest;
    returns (coordinates, so0 [ncoord, 3], dt)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    rl, rr = rng.uniform(0.5, 1.5), rng.uniform(0.1, 0.5)
    pl, pr = rng.uniform(0.5, 1.5), rng.uniform(0.05, 0.3)
    x = np.linspace(-1.0, 1.0, ncoord)
    so0 = np.zeros((ncoord, 3))
    left = x < 0.0
    so0[:, 0] = np.where(left, rl, rr)
    so0[:, 2] = np.where(left, pl, pr) / 0.4
    return x, so0, tube_dt(ncoord)


def tube_dt(ncoord):
    """dt of a tube: CFL 0.8 for the largest wave speed the random states
    can produce (acoustic speed <= 2.05, post-shock |u| + c below 4.5), so
    it depends on the size only and a tube slot serves every request of its
    size."""
    return 0.8 * (2.0 / (ncoord - 1)) / 4.5


# Padding elements on each side of a spacetime grid (core.hpp:105).
ST_BOUND_COUNT = 2


def grid_xloc(xmin, xmax, ncelm):
    """CE boundaries of ``Grid(xmin, xmax, ncelm)`` (spacetime/core.cpp
    :14-45): xmin, then repeated additions of the spacing, then xmax."""
    space = (xmax - xmin) / ncelm
    steps = np.full(ncelm, space)
    steps[0] = xmin
    xloc = np.empty(ncelm + 1)
    xloc[:ncelm] = np.cumsum(steps)  # sequential, as the reference's loop
    xloc[ncelm] = xmax
    return xloc


def grid_xcoord(xloc):
    """All coordinates of a spacetime grid from its CE boundaries
    (Grid::init_from_array, spacetime/core.cpp:47-96): boundaries at the even
    places, CE centres between them, ST_BOUND_COUNT mirrored points on each
    side."""
    b = ST_BOUND_COUNT
    ncelm = xloc.size - 1
    nx = ncelm * 2 + 1 + b * 2
    x = np.zeros(nx)
    x[b:b + 2 * xloc.size - 1:2] = xloc
    ref = np.arange(ncelm) * 2 + b + 1
    x[ref] = (x[ref - 1] + x[ref + 1]) / 2
    for it in range(1, b + 1):
        x[b - it] = x[b] + x[b] - x[b + it]
        r = nx - b - 1
        x[r + it] = x[r] + x[r] - x[r - it]
    return x
