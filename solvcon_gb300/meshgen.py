"""Seeded synthetic meshes and initial states of the benchmark workloads.

The reference ships no mesh generator at these scales, so these vectorised
builders produce the node coordinates and cell lists, and
:func:`build_mesh` runs them through :class:`~solvcon_gb300.mesh.StaticMesh`
(interior, boundary, ghost) exactly as a reference user would.

* :func:`tri_square` -- unit square, n x n quads each cut on the same
  diagonal into 2 triangles, interior nodes jittered by U(-j h, j h).
* :func:`tet_cube` -- unit cube, n^3 hexes each cut into the 6 Kuhn
  tetrahedra around the v0-v6 diagonal, interior nodes jittered likewise.
* :func:`quadrant_state` -- four-quadrant Riemann state drawn from a seed.
* :func:`blast_state` -- spherical blast, (rho, p) = (1, 1) inside r < 0.2.
"""

import numpy as np

from .mesh import StaticMesh

__all__ = ["tri_square", "tet_cube", "quad_square", "hex_cube", "prism_slab", "build_mesh",
           "quadrant_state", "blast_state", "conserved", "set_state"]


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
    cltpn = np.full(tri.shape[0], StaticMesh.TRIANGLE, dtype="int32")
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
    cltpn = np.full(n * n, StaticMesh.QUADRILATERAL, dtype="int32")
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
    cltpn = np.full(tets.shape[0], StaticMesh.TETRAHEDRON, dtype="int32")
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
    cltpn = np.full(base.size, StaticMesh.HEXAHEDRON, dtype="int32")
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
    cltpn = np.full(pr.shape[0], StaticMesh.PRISM, dtype="int32")
    return ndcrd, cltpn, clnds


# Gmsh element type of each solvcon cell type, and the Gmsh corner order:
# Gmsh corner k is solvcon node GMSH_ORDER[type][k] (the prism's Gmsh
# corners run the other way round each triangle).
GMSH_TYPE = {2: 1, 3: 3, 4: 2, 5: 5, 6: 4, 7: 6, 8: 7}
GMSH_ORDER = {7: (0, 2, 1, 3, 5, 4)}


def to_gmsh(ndim, ndcrd, cltpn, clnds, lower=(), names=(), second_order=()):
    """A Gmsh MSH 2.2 ASCII file (str) of a mesh given as node coordinates
    ``ndcrd`` [nnode, ndim], cell types ``cltpn`` and solvcon cell node lists
    ``clnds`` (first column the node count).

    :param lower: lower-dimension elements to write before the cells, as
        (gmsh type, physical tag, node ids) tuples (boundary lines, points).
    :param names: (dim, tag, name) physical names.
    :param second_order: indices of triangle cells to write as 6-node
        triangles (Gmsh type 9); their mid-edge nodes are appended to the node
        list, unused by any cell.
    """
    x = np.asarray(ndcrd, dtype="float64")
    nnode = x.shape[0]
    extra = []
    elems = []
    for gtype, tag, nds in lower:
        elems.append((int(gtype), int(tag), [int(v) for v in nds]))
    so = set(int(i) for i in second_order)
    for icl, (tp, row) in enumerate(zip(cltpn, clnds)):
        tp = int(tp)
        n = int(row[0])
        nds = [int(v) for v in row[1:n + 1]]
        order = GMSH_ORDER.get(tp, tuple(range(n)))
        g = [nds[order[k]] for k in range(n)]
        gtype = GMSH_TYPE[tp]
        if icl in so and tp == 4:
            for a, b in ((0, 1), (1, 2), (2, 0)):
                extra.append((x[g[a]] + x[g[b]]) / 2)
                g.append(nnode + len(extra) - 1)
            gtype = 9
        elems.append((gtype, 1, g))
    allx = np.vstack([x] + [np.asarray(extra)]) if extra else x
    out = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat"]
    if names:
        out += ["$PhysicalNames", str(len(names))]
        out += ['%d %d "%s"' % (d, t, nm) for d, t, nm in names]
        out += ["$EndPhysicalNames"]
    out += ["$Nodes", str(allx.shape[0])]
    for i, p in enumerate(allx):
        xyz = list(p) + [0.0] * (3 - len(p))
        out.append("%d %s" % (i + 1, " ".join(repr(float(v)) for v in xyz)))
    out += ["$EndNodes", "$Elements", str(len(elems))]
    for k, (gtype, tag, nds) in enumerate(elems):
        out.append("%d %d 2 %d %d %s" % (k + 1, gtype, tag, tag,
                                         " ".join(str(v + 1) for v in nds)))
    out += ["$EndElements"]
    return "\n".join(out) + "\n"


def to_plot3d(blocks):
    """A Plot3D multi-block ASCII grid file (str) of structured blocks, each
    an array of node coordinates [nk, nj, ni, 3] (grid index i fastest in
    the file)."""
    out = [str(len(blocks))]
    for b in blocks:
        nk, nj, ni = b.shape[:3]
        out.append("%d %d %d" % (ni, nj, nk))
    for b in blocks:
        flat = np.asarray(b, dtype="float64").reshape(-1, 3)
        for d in range(3):
            vals = [repr(float(v)) for v in flat[:, d]]
            for k in range(0, len(vals), 6):
                out.append(" ".join(vals[k:k + 6]))
    return "\n".join(out) + "\n"


def build_mesh(ndim, ndcrd, cltpn, clnds, bcs=()):
    """A :class:`StaticMesh` with interior, boundary and ghost layer built."""
    m = StaticMesh(ndim=ndim, nnode=len(ndcrd), nface=0, ncell=len(cltpn))
    m.ndcrd.ndarray[...] = ndcrd
    m.cltpn.ndarray[...] = cltpn
    cl = np.asarray(clnds)
    m.clnds.ndarray[:, :cl.shape[1]] = cl
    m.build_interior(do_metric=True, build_edge=False)
    for name, faces in bcs:
        m.add_bc(name, faces)
    m.build_boundary()
    m.build_ghost()
    return m


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


def set_state(core, mesh, state, gamma):
    """Initialise a core: gamma everywhere, so0n body rows = state, ghosts
    primed with bc_soln/bc_dsoln (the reference drivers' start-up,
    pilot/apps/obsrefl/_driver.py:505-508)."""
    core.init_solution(gamma=gamma, rho=1.0, v=[0.0] * mesh.ndim, p=1.0)
    so0n = core.so0n
    so0n.ndarray[core.ngstcell:] = state
    core.bc_soln()
    core.bc_dsoln()
