"""Pin the CPU oracle before trusting it.

The oracle (oracle/cese_oracle.c) restates the reference march; here it is
checked against the golden vectors produced by the reference itself
(tests/golden/, made by tests/golden/make_golden.py), against the reference
library directly where it is built on this host (oracle/_ref), and against
the known-answer properties the reference's own tests assert.
"""

import numpy as np
import pytest

from _util import golden
from test_mesh import _build


def _oracle_from_golden(case):
    from oracle import oracle as ora
    gm = golden("mesh_" + case)
    g = golden("march_" + case)
    mesh = _build(gm)
    o = ora.OracleEuler(mesh, float(g["dt"]))
    o.init_solution(1.4, 1.0, [0.0] * mesh.ndim, 1.0)
    o.so0n[o.ngstcell:] = g["state0"]
    o.add_bc(int(g["bc_kind"]), g["faces"])
    o.call("bc_soln")
    o.call("bc_dsoln")
    return mesh, o, g


@pytest.mark.parametrize("case", ["tri12", "quad8", "tet3"])
def test_oracle_reproduces_reference_march(case):
    mesh, o, g = _oracle_from_golden(case)
    for a in ("cevol", "cecnd"):
        np.testing.assert_array_equal(getattr(o, a), g[a])
    o.march(int(g["steps"]))
    for a in ("so0c", "so0n", "so0t", "so1c", "so1n", "cflo", "cflc"):
        np.testing.assert_allclose(getattr(o, a), g[a], rtol=0, atol=1e-13,
                                   err_msg=a)


def test_oracle_reproduces_reference_sod():
    from oracle import oracle as ora
    g = golden("e1d_sod")
    n = g["coord"].size
    o = ora.OracleEuler1D(n, float(g["dt"]))
    o.coord[:] = g["coord"]
    o.so0[:] = g["so0_in"]
    o.gamma[:] = 1.4
    o.setup_march()
    o.march_alpha(2, int(g["steps"]))
    for a in ("so0", "so1", "cfl"):
        np.testing.assert_allclose(getattr(o, a), g[a], rtol=0, atol=1e-14)


def test_oracle_spacetime_known_answers():
    """The reference's spacetime known answers
    (tests/test_spacetime_linear_scalar.py:106-113,
    test_spacetime_inviscid_burgers.py:47-52) hold for the oracle."""
    from oracle import oracle as ora
    from solvcon_gb300.spacetime import Grid
    res = 8
    xcrd = np.arange(res + 1) / res * 2 * np.pi
    grid = Grid(xcrd)
    nstep = int(np.ceil(2 * np.pi / ((grid.xmax - grid.xmin) / grid.ncelm)))
    dt = 2 * np.pi / nstep
    o = ora.OracleSpacetime(0, grid.xcoord, dt)
    o.so0[2:2 + 2 * res + 1:2] = np.sin(xcrd)
    o.so1[2:2 + 2 * res + 1:2] = np.cos(xcrd)
    o.setup_march()
    o.march_alpha(2, nstep * 10)
    np.testing.assert_allclose(o.so0[2:2 + 2 * res + 1:2], np.sin(xcrd),
                               rtol=0, atol=1e-14)
    np.testing.assert_allclose(o.cfl[2:2 + 2 * res + 1:2], 1.0, rtol=0,
                               atol=1e-14)
    b = ora.OracleSpacetime(1, grid.xcoord, dt)
    b.so0[2:2 + 2 * res + 1:2] = np.sin(xcrd)
    b.so1[2:2 + 2 * res + 1:2] = np.cos(xcrd)
    b.setup_march()
    for _ in range(nstep * 2):
        b.march_alpha(2, 1)
        ev = b.so0[2:2 + 2 * res + 1:2]
        assert ev.max() <= 1 and ev.min() >= -1


def test_oracle_free_stream_and_linear_field():
    """Known answers of the reference tests (tests/test_multidim.py:657-708):
    a uniform state is preserved exactly; a linear field's gradient is
    recovered exactly."""
    from oracle import oracle as ora
    from solvcon_gb300 import meshgen
    x, t, c = meshgen.tri_square(6, 0.2, 2)
    mesh = meshgen.build_mesh(2, x, t, c)
    o = ora.OracleEuler(mesh, 0.01)
    row = np.array([1.2, 0.36, -0.18, 0.9 / 0.4 + 0.5 * 1.2 * 0.1125])
    o.gamma[:] = 1.4
    o.so0c[:] = row
    o.so1c[:] = 0.0
    o.call("calc_solt")
    o.call("calc_soln")
    np.testing.assert_allclose(o.so0n[o.ngstcell:], np.broadcast_to(
        row, (o.ncell, 4)), rtol=1e-12)
    g = np.array([[0.1 * (i + 1) + 0.01 * (d + 1) for d in range(2)]
                  for i in range(4)])
    ng = o.ngstcell
    pts = np.array(o.cecnd[:, :2])
    pts[:ng] = np.array(mesh.clcnd.ndarray)[:ng]
    vals = 0.5 + pts @ g.T
    o.so0c[:] = vals
    o.so0n[:] = vals
    o.so0t[:] = 0.0
    o.so1c[:] = g[None]
    o.cflc[:] = 0.5
    o.call("calc_dsoln")
    np.testing.assert_allclose(o.so1n[ng:], np.broadcast_to(g, (o.ncell, 4, 2)),
                               rtol=1e-9)


def test_oracle_against_reference_library():
    from oracle import oracle as ora
    from oracle import refbind as rb
    if not rb.available():
        pytest.skip("reference library not built on this host")
    from solvcon_gb300 import meshgen
    for nd, (x, t, c) in ((2, meshgen.quad_square(7, 0.2, 3)),
                          (3, meshgen.hex_cube(2, 0.1, 3)),
                          (3, meshgen.prism_slab(3, 2, 0.1, 3))):
        mesh = meshgen.build_mesh(nd, x, t, c)
        r = rb.RefMesh(nd, x, t, c)
        ref = rb.RefEuler(r, 3e-3)
        o = ora.OracleEuler(mesh, 3e-3)
        ng = o.ngstcell
        clcnd = np.array(mesh.clcnd.ndarray)[ng:]
        st = meshgen.quadrant_state(clcnd[:, :2], 4) if nd == 2 else \
            meshgen.blast_state(clcnd, radius=0.4)
        st = st if nd == 2 else st
        for core in (o, ref):
            core.init_solution(1.4, 1.0, [0.0] * nd, 1.0)
        so = ref.get("so0n")
        so[ng:] = st
        ref.set("so0n", so)
        o.so0n[ng:] = st
        faces = np.array(mesh.bndfcs.ndarray[:, 0])
        ref.add_bc(0, faces[::2])
        o.add_bc(0, faces[::2])
        ref.add_bc(1, faces[1::2])
        o.add_bc(1, faces[1::2])
        ref.call("bc_soln")
        ref.call("bc_dsoln")
        o.call("bc_soln")
        o.call("bc_dsoln")
        ref.march(3)
        o.march(3)
        for a in ("so0n", "so1n", "so0t", "cflc"):
            np.testing.assert_array_equal(getattr(o, a), ref.get(a), a)


ST_CASES = ["linear_a1", "linear_a2", "burgers_a1", "burgers_a2"]


@pytest.mark.parametrize("case", ST_CASES)
def test_oracle_reproduces_reference_spacetime(case):
    """The spacetime oracle against the reference's own solvers
    (spacetime/core.hpp:946-1036, kernel/linear_scalar.hpp,
    kernel/inviscid_burgers.hpp) on non-uniform grids: a linear-scalar wave
    and a Burgers state that steepens into a shock, alpha 1 and 2
    (fixtures generated from the reference)."""
    from oracle import oracle as ora
    g = golden("st_" + case)
    o = ora.OracleSpacetime(int(g["kind"]), g["xcoord"], float(g["dt"]))
    o.so0[:] = g["so0_in"]
    o.so1[:] = g["so1_in"]
    o.setup_march()
    o.march_alpha(int(g["alpha"]), int(g["steps"]))
    for a in ("so0", "so1", "cfl"):
        np.testing.assert_array_equal(getattr(o, a), g[a], a)


def test_oracle_spacetime_against_reference_library():
    """The same comparison against the reference library live, on other
    grids and states, marched half a step at a time and in one call."""
    from oracle import oracle as ora
    from oracle import refbind as rb
    if not rb.available():
        pytest.skip("reference library not built on this host")
    rng = np.random.default_rng(99)
    for kind, ncelm in ((0, 57), (1, 131)):
        h = 3.0 / ncelm
        xloc = -1.0 + np.arange(ncelm + 1) * h
        xloc[1:-1] += rng.uniform(-0.35, 0.35, ncelm - 1) * h
        dt = 0.8 * np.diff(xloc).min() / 1.6
        for alpha in (1, 2):
            ref = rb.RefSpacetime(kind, xloc, dt)
            x = ref.get("xcoord")
            so0 = np.where(x < 0.2, 1.2, -0.3) + 0.1 * np.sin(7 * x)
            so1 = np.zeros_like(x)
            ref.set("so0", so0)
            ref.set("so1", so1)
            ref.set("cfl", np.zeros_like(x))
            o = ora.OracleSpacetime(kind, x, dt)
            o.so0[:] = so0
            o.so1[:] = so1
            ref.setup_march()
            o.setup_march()
            for k in (1, 1, 5, 40):
                ref.march_alpha(alpha, k)
                o.march_alpha(alpha, k)
                for a in ("so0", "so1", "cfl"):
                    np.testing.assert_array_equal(getattr(o, a), ref.get(a),
                                                  "%d %d %s" % (kind, alpha,
                                                                a))


MESH_CASES = ("tri3", "quad1", "mixed", "tet1", "hex1", "prism1", "pyr1",
              "tri12", "quad8", "tet3")
MESH_TABLES = ("fctpn", "cltpn", "fcnds", "fccls", "clfcs", "bndfcs",
               "ndcrd", "fccnd", "fcnml", "fcara", "clcnd", "clvol")


def _oracle_mesh_equals(m, tables, sizes, clnds_full=None):
    got = [m.ndim, m.nnode, m.nface, m.ncell, m.nbound, m.ngstnode,
           m.ngstface, m.ngstcell]
    assert got == [int(x) for x in sizes[:8]]
    for name in MESH_TABLES:
        np.testing.assert_array_equal(np.asarray(getattr(m, name)).ravel(),
                                      np.asarray(tables[name]).ravel(), name)
    want = np.asarray(tables["clnds"]).reshape(m.clnds.shape)
    for row in range(want.shape[0]):
        n = want[row, 0]
        assert np.array_equal(m.clnds[row, :n + 1], want[row, :n + 1]), row


@pytest.mark.parametrize("case", MESH_CASES)
def test_oracle_mesh_matches_reference_golden(case):
    """The oracle's own StaticMesh build (oracle/mesh_oracle.c) gives the
    reference's tables entry for entry: interior, boundary and ghost."""
    from oracle import oracle as ora
    g = golden("mesh_" + case)
    m = ora.OracleMesh(int(g["ndim"]), g["ndcrd_in"], g["cltpn_in"],
                       g["clnds_in"])
    _oracle_mesh_equals(m, g, g["sizes"])


def test_oracle_mesh_against_reference_library():
    from oracle import oracle as ora
    from oracle import refbind as rb
    if not rb.available():
        pytest.skip("reference library not built on this host")
    from solvcon_gb300 import synth
    for nd, (x, t, c) in ((2, synth.tri_square(30, 0.2, 8)),
                          (2, synth.quad_square(11, 0.15, 8)),
                          (3, synth.tet_cube(5, 0.15, 8)),
                          (3, synth.hex_cube(4, 0.1, 8)),
                          (3, synth.prism_slab(5, 3, 0.1, 8))):
        r = rb.RefMesh(nd, x, t, c)
        s = r.sizes()
        m = ora.OracleMesh(nd, x, t, c)
        _oracle_mesh_equals(m, {k: r.array(k) for k in MESH_TABLES +
                                ("clnds",)},
                            [s[k] for k in ("ndim", "nnode", "nface", "ncell",
                                            "nbound", "ngstnode", "ngstface",
                                            "ngstcell")])


def test_oracle_mesh_equals_the_library_mesh_builder():
    """The two restatements of the mesh build -- the oracle's in C and the
    library's host builder -- agree table for table on the workloads'
    generators, so a march on either mesh is the same march."""
    from oracle import oracle as ora
    from solvcon_gb300 import meshgen
    for nd, (x, t, c) in ((2, meshgen.tri_square(40, 0.2, 3)),
                          (3, meshgen.tet_cube(5, 0.15, 3))):
        m = ora.OracleMesh(nd, x, t, c)
        lib_mesh = meshgen.build_mesh(nd, x, t, c)
        tables = {k: np.asarray(getattr(lib_mesh, k).ndarray)
                  for k in MESH_TABLES + ("clnds",)}
        _oracle_mesh_equals(m, tables, [getattr(lib_mesh, k) for k in (
            "ndim", "nnode", "nface", "ncell", "nbound", "ngstnode",
            "ngstface", "ngstcell")])
