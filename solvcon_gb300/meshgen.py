"""Seeded synthetic meshes and initial states of the benchmark workloads.

The reference ships no mesh generator at these scales, so vectorised
builders (:mod:`solvcon_gb300.synth`, re-exported here) produce the node
coordinates and cell lists, and :func:`build_mesh` runs them through
:class:`~solvcon_gb300.mesh.StaticMesh` (interior, boundary, ghost) exactly
as a reference user would.

* :func:`tri_square` -- unit square, n x n quads each cut on the same
  diagonal into 2 triangles, interior nodes jittered by U(-j h, j h).
* :func:`tet_cube` -- unit cube, n^3 hexes each cut into the 6 Kuhn
  tetrahedra around the v0-v6 diagonal, interior nodes jittered likewise.
* :func:`quadrant_state` -- four-quadrant Riemann state drawn from a seed.
* :func:`blast_state` -- spherical blast, (rho, p) = (1, 1) inside r < 0.2.
"""

import numpy as np

from .mesh import StaticMesh
from .synth import (_jitter, blast_state, conserved, hex_cube,  # noqa: F401
                    prism_slab, quad_square, quadrant_state, tet_cube,
                    tri_square)

__all__ = ["tri_square", "tet_cube", "quad_square", "hex_cube", "prism_slab", "build_mesh",
           "quadrant_state", "blast_state", "conserved", "set_state"]


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


def set_state(core, mesh, state, gamma):
    """Initialise a core: gamma everywhere, so0n body rows = state, ghosts
    primed with bc_soln/bc_dsoln (the reference drivers' start-up,
    pilot/apps/obsrefl/_driver.py:505-508)."""
    core.init_solution(gamma=gamma, rho=1.0, v=[0.0] * mesh.ndim, p=1.0)
    so0n = core.so0n
    so0n.ndarray[core.ngstcell:] = state
    core.bc_soln()
    core.bc_dsoln()
