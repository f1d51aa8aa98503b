"""Generate the golden fixtures of tests/golden/ from the reference itself.

Runs the reference solvcon implementation (oracle/_ref/libsolvcon_ref.so,
built from the reference's own sources by ``make -C oracle ref``) on small
seeded cases and stores its outputs as .npz files:

* mesh_<case>.npz -- every StaticMesh table after build_interior,
  build_boundary and build_ghost (the mesh builder's golden vectors);
* march_<case>.npz -- initial state, boundary setup and the EulerCore arrays
  after a number of march steps (the march's golden vectors);
* e1d_sod.npz -- the Euler1DCore Sod tube after march_alpha2;
* gmsh_<case>.npz -- a Gmsh MSH 2.2 file written by meshgen.to_gmsh (its text
  in "msh") and every StaticMesh table the reference's Gmsh reader builds
  from it;
* plot3d_<case>.npz -- the same for Plot3D grid files (text in "p3d");
* st_<solver>_a<alpha>.npz -- a spacetime LinearScalarSolver /
  InviscidBurgersSolver on a non-uniform grid: its CE boundaries, dt, the
  initial so0/so1 and the so0/so1/cfl tables after march_alpha<alpha>.

Usage: python tests/golden/make_golden.py [gmsh|plot3d|spacetime]   (needs
oracle/_ref built; a mode argument writes only those fixtures)
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import refbind as rb  # noqa: E402
from solvcon_gb300 import meshgen  # noqa: E402

MESH_ARRAYS = ("ndcrd", "fccnd", "fcnml", "fcara", "clcnd", "clvol", "fctpn",
               "cltpn", "fcnds", "fccls", "clnds", "clfcs", "ednds", "bndfcs")


def fixture_cases():
    """Hand-built fixture meshes of the reference tests
    (tests/test_multidim.py:152-281, 810-827) plus seeded jittered meshes."""
    cases = {
        "tri3": (2, [(0, 0), (-1, -1), (1, -1), (0, 1)], [4, 4, 4],
                 [(3, 0, 1, 2), (3, 0, 2, 3), (3, 0, 3, 1)]),
        "quad1": (2, [(0, 0), (1, 0), (1, 1), (0, 1)], [3],
                  [(4, 0, 1, 2, 3)]),
        "mixed": (2, [(0, 0), (1, 0), (2, 0), (0, 1), (1, 1), (2, 1)],
                  [3, 4, 4], [(4, 0, 1, 4, 3), (3, 1, 2, 4, 0),
                              (3, 2, 5, 4, 0)]),
        "tet1": (3, [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)], [6],
                 [(4, 0, 1, 2, 3)]),
        "hex1": (3, [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1),
                     (1, 0, 1), (1, 1, 1), (0, 1, 1)], [5],
                 [(8, 0, 1, 2, 3, 4, 5, 6, 7)]),
        "prism1": (3, [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1),
                       (1, 0, 1), (0, 1, 1)], [7], [(6, 0, 1, 2, 3, 4, 5)]),
        "pyr1": (3, [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0),
                     (0.5, 0.5, 1)], [8], [(5, 0, 1, 2, 3, 4)]),
    }
    x, t, c = meshgen.tri_square(12, 0.2, seed=11)
    cases["tri12"] = (2, x, t, c[:, :4])
    x, t, c = meshgen.quad_square(8, 0.15, seed=12)
    cases["quad8"] = (2, x, t, c[:, :5])
    x, t, c = meshgen.tet_cube(3, 0.15, seed=13)
    cases["tet3"] = (3, x, t, c[:, :5])
    return cases


def mesh_golden(name, nd, x, t, c):
    r = rb.RefMesh(nd, x, t, c)
    out = {"ndim": nd, "ndcrd_in": np.asarray(x, dtype="float64"),
           "cltpn_in": np.asarray(t, dtype="int32"),
           "clnds_in": np.asarray(c, dtype="int32")}
    sizes = r.sizes()
    out["sizes"] = np.array([sizes[k] for k in
                             ("ndim", "nnode", "nface", "ncell", "nbound",
                              "ngstnode", "ngstface", "ngstcell", "nedge",
                              "nbcs")], dtype="int64")
    for a in MESH_ARRAYS:
        out[a] = r.array(a)
    np.savez_compressed(os.path.join(HERE, "mesh_%s.npz" % name), **out)
    return r


def march_golden(name, mesh, nd, state, bc_kind, dt, steps):
    e = rb.RefEuler(mesh, dt)
    e.init_solution(1.4, 1.0, [0.0] * nd, 1.0)
    ng = mesh.sizes()["ngstcell"]
    so = e.get("so0n")
    so[ng:] = state
    e.set("so0n", so)
    faces = mesh.array("bndfcs").reshape(-1, 3)[:, 0]
    e.add_bc(bc_kind, faces)
    e.call("bc_soln")
    e.call("bc_dsoln")
    out = {"dt": dt, "steps": steps, "bc_kind": bc_kind,
           "state0": np.asarray(state), "faces": faces}
    e.march(steps)
    for a in ("cevol", "cecnd", "so0c", "so0n", "so0t", "so1c", "so1n",
              "cflo", "cflc"):
        out[a] = e.get(a)
    np.savez_compressed(os.path.join(HERE, "march_%s.npz" % name), **out)


def e1d_golden():
    # Sod tube of the 1D configuration: 201 points on [-1, 1],
    # dt = 2 * 0.8 * dx / 2.19 (post-shock max |u| + c), 28 steps.
    n = 201
    dx = 2.0 / (n - 1)
    dt = 2 * 0.8 * dx / 2.19
    c = rb.RefEuler1D(n, dt)
    x = np.linspace(-1, 1, n)
    c.set("coord", x)
    g = 1.4
    so0 = np.zeros((n, 3))
    left = x < 0.0
    so0[:, 0] = np.where(left, 1.0, 0.125)
    so0[:, 2] = np.where(left, 1.0 / (g - 1), 0.1 / (g - 1))
    c.set("so0", so0)
    c.set("so1", np.zeros((n, 3)))
    c.set("gamma", np.full(n, g))
    c.set("cfl", np.zeros(n))
    c.setup_march()
    out = {"dt": dt, "steps": 28, "coord": x, "so0_in": so0}
    c.march_alpha(2, 28)
    for a in ("so0", "so1", "cfl"):
        out[a] = c.get(a)
    np.savez_compressed(os.path.join(HERE, "e1d_sod.npz"), **out)


def spacetime_cases():
    """Spacetime solver cases on non-uniform grids (CE boundaries jittered
    by up to 30% of the mean spacing, seeded): the linear scalar advecting
    sin(x) (so1 = cos(x)), and inviscid Burgers from u = 0.5 + sin(x), which
    steepens into a shock at t = 1 and is marched to t ~ 2.  dt gives a CFL
    number of 0.9 on the smallest half spacing at the largest speed.  Returns
    {name: (kind, alpha, xloc, dt, steps, so0 at CE boundaries / centres,
    so1)} with so0/so1 given as functions of the grid's coordinates."""
    out = {}
    for name, kind, ncelm, umax, steps in (("linear", 0, 80, 1.0, 60),
                                           ("burgers", 1, 200, 1.5, 240)):
        rng = np.random.Generator(np.random.PCG64(4242 + kind))
        h = 2 * np.pi / ncelm
        xloc = np.arange(ncelm + 1) * h
        xloc[1:-1] += rng.uniform(-0.3, 0.3, ncelm - 1) * h
        hmin = np.diff(xloc).min() / 2
        dt = 0.9 * 2 * hmin / umax
        for alpha in (1, 2):
            out["%s_a%d" % (name, alpha)] = (kind, alpha, xloc, dt, steps)
    return out


def spacetime_golden(name, kind, alpha, xloc, dt, steps):
    s = rb.RefSpacetime(kind, xloc, dt)
    x = s.get("xcoord")
    so0 = np.sin(x) + (0.5 if kind == 1 else 0.0)
    so1 = np.cos(x)
    s.set("so0", so0)
    s.set("so1", so1)
    # The two outermost entries of cfl are never written by the solver
    # (core.hpp:954-962 covers selms -1 .. nselm-1 only); start from zeros so
    # the fixture holds no uninitialised memory.
    s.set("cfl", np.zeros_like(x))
    s.setup_march()
    out = {"kind": kind, "alpha": alpha, "xloc": xloc, "dt": dt,
           "steps": steps, "xcoord": x, "so0_in": so0, "so1_in": so1}
    s.march_alpha(alpha, steps)
    for a in ("so0", "so1", "cfl"):
        out[a] = s.get(a)
    np.savez_compressed(os.path.join(HERE, "st_%s.npz" % name), **out)


def gmsh_cases():
    """Gmsh files of the reader's fixtures: (text, ndim, ndcrd, cltpn, clnds)
    where the last three are the mesh the file describes (None when the file
    carries nodes no cell uses)."""
    out = {}
    # The reference test's triangle fan (tests/test_gmsh.py:19-40), with a
    # boundary line, a point and a physical name besides the cells.
    x = [(0.0, 0.0), (-1.0, -1.0), (1.0, -1.0), (0.0, 1.0)]
    t = [4, 4, 4]
    c = [(3, 0, 1, 2), (3, 0, 2, 3), (3, 0, 3, 1)]
    txt = meshgen.to_gmsh(2, x, t, c, lower=[(15, 7, [1]), (1, 5, [1, 2])],
                          names=[(1, 5, "wall"), (2, 1, "fluid")])
    out["tri3"] = (txt, 2, x, t, c)
    # Quads with every third one split into two triangles, boundary lines.
    xq, tq, cq = meshgen.quad_square(6, 0.15, seed=21)
    cells, types = [], []
    for k, row in enumerate(cq):
        a, b, cc, d = (int(v) for v in row[1:5])
        if k % 3 == 0:
            cells += [(3, a, b, cc), (3, a, cc, d)]
            types += [4, 4]
        else:
            cells.append((4, a, b, cc, d))
            types.append(3)
    clnds = np.full((len(cells), 5), -1, dtype="int32")
    for k, row in enumerate(cells):
        clnds[k, :len(row)] = row
    lines = [(1, 3, [i, i + 1]) for i in range(6)]
    txt = meshgen.to_gmsh(2, xq, types, clnds, lower=lines,
                          names=[(1, 3, "bottom")])
    out["mixed2d"] = (txt, 2, xq, types, clnds)
    # The same with some triangles written as 6-node triangles: their
    # mid-edge nodes are in $Nodes but in no cell.
    tri = [k for k, tp in enumerate(types) if tp == 4][::2]
    txt = meshgen.to_gmsh(2, xq, types, clnds, second_order=tri)
    out["order2"] = (txt, 2, None, None, None)
    # 3D: a hexahedral block, a prism slab beside it, a pyramid and a
    # tetrahedron (four components, every 3D type and the prism's Gmsh
    # corner order).
    xh, th, ch = meshgen.hex_cube(2, 0.1, seed=22)
    xp, tp, cp = meshgen.prism_slab(2, 1, 0.1, seed=23)
    xp = xp + np.array([1.5, 0.0, 0.0])
    xy = np.array([(3.0, 0, 0), (4, 0, 0), (4, 1, 0), (3, 1, 0),
                   (3.5, 0.5, 1), (5, 0, 0), (6, 0, 0), (5, 1, 0),
                   (5, 0, 1)], dtype="float64")
    nh, npr = len(xh), len(xp)
    x3 = np.vstack([xh, xp, xy])
    t3 = list(th) + list(tp) + [8, 6]
    c3 = np.full((len(t3), 9), -1, dtype="int32")
    c3[:len(th), :9] = ch[:, :9]
    c3[len(th):len(th) + len(tp), :7] = cp[:, :7] + np.array([0] + [nh] * 6)
    base = nh + npr
    c3[-2, :6] = [5] + [base + i for i in range(5)]
    c3[-1, :5] = [4] + [base + 5 + i for i in range(4)]
    txt = meshgen.to_gmsh(3, x3, t3, c3)
    out["mixed3d"] = (txt, 3, x3, t3, c3)
    return out


def plot3d_cases():
    """Plot3D files of the reader's fixtures: a jittered single block, and
    three blocks of different shapes side by side."""
    rng = np.random.Generator(np.random.PCG64(31))

    def block(ni, nj, nk, x0, jitter):
        g = np.stack(np.meshgrid(np.arange(nk), np.arange(nj), np.arange(ni),
                                 indexing="ij"), axis=-1)[..., ::-1]
        g = g.astype("float64") + rng.uniform(-jitter, jitter, g.shape)
        g[..., 0] += x0
        return g
    return {"cube": meshgen.to_plot3d([block(4, 3, 3, 0.0, 0.2)]),
            "blocks": meshgen.to_plot3d([block(3, 2, 2, 0.0, 0.1),
                                         block(2, 3, 2, 5.0, 0.1),
                                         block(2, 2, 4, 10.0, 0.0)])}


def mesh_golden_from(name, r, extra):
    out = dict(extra)
    sizes = r.sizes()
    out["sizes"] = np.array([sizes[k] for k in
                             ("ndim", "nnode", "nface", "ncell", "nbound",
                              "ngstnode", "ngstface", "ngstcell", "nedge",
                              "nbcs")], dtype="int64")
    for a in MESH_ARRAYS:
        out[a] = r.array(a)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


def gmsh_golden(name, text):
    r = rb.RefMesh.from_gmsh(text.encode())
    out = {"msh": np.array(text)}
    sizes = r.sizes()
    out["sizes"] = np.array([sizes[k] for k in
                             ("ndim", "nnode", "nface", "ncell", "nbound",
                              "ngstnode", "ngstface", "ngstcell", "nedge",
                              "nbcs")], dtype="int64")
    for a in MESH_ARRAYS:
        out[a] = r.array(a)
    np.savez_compressed(os.path.join(HERE, "gmsh_%s.npz" % name), **out)


def main():
    if sys.argv[1:] == ["gmsh"]:
        for name, case in gmsh_cases().items():
            gmsh_golden(name, case[0])
        print("gmsh fixtures written to", HERE)
        return
    if sys.argv[1:] == ["spacetime"]:
        for name, case in spacetime_cases().items():
            spacetime_golden(name, *case)
        print("spacetime fixtures written to", HERE)
        return
    if sys.argv[1:] == ["plot3d"]:
        for name, text in plot3d_cases().items():
            mesh_golden_from("plot3d_" + name,
                             rb.RefMesh.from_plot3d(text.encode()),
                             {"p3d": np.array(text)})
        print("plot3d fixtures written to", HERE)
        return
    cases = fixture_cases()
    meshes = {k: mesh_golden(k, *v) for k, v in cases.items()}
    for name, kind in (("tri12", 1), ("quad8", 0), ("tet3", 1)):
        mesh = meshes[name]
        nd = cases[name][0]
        clcnd = mesh.array("clcnd").reshape(-1, nd)[mesh.sizes()["ngstcell"]:]
        state = meshgen.quadrant_state(clcnd[:, :2], seed=5) if nd == 2 \
            else meshgen.blast_state(clcnd, center=(0.5, 0.5, 0.5),
                                     radius=0.35)
        march_golden(name, mesh, nd, state, kind, 2e-3, 6)
    e1d_golden()
    for name, case in spacetime_cases().items():
        spacetime_golden(name, *case)
    for name, case in gmsh_cases().items():
        gmsh_golden(name, case[0])
    for name, text in plot3d_cases().items():
        mesh_golden_from("plot3d_" + name,
                         rb.RefMesh.from_plot3d(text.encode()),
                         {"p3d": np.array(text)})
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
