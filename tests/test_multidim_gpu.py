"""GPU EulerCore: behaviour of the reference's EulerCore tests and parity
with the oracle, per operation and over multi-step marches.

Modelled on the reference's tests/test_multidim.py (solution storage, CFL,
flux homogeneity, free stream, linear-field gradient recovery, boundary
conditions, bounded channel march), compared with the CPU oracle (a bit-exact
restatement of the reference, pinned in test_oracle.py).

Tolerances (FP64): one operation on the same inputs agrees with the oracle to
1e-12 relative to the largest magnitude of the compared array (the GPU
evaluates the same mathematics in a different operation order); marches of a
few steps agree to 1e-10.
"""

import numpy as np
import pytest

from _util import FIXTURES, assert_rel, fixture_mesh, quad_channel

pytestmark = pytest.mark.gpu

GAMMA, RHO, PRES = 1.4, 1.2, 0.9
VEL = (0.3, -0.15, 0.05)


def _core(mesh, dt=0.01, precision="fp64"):
    import solvcon_gb300 as sg
    return sg.EulerCore(mesh=mesh, time_increment=dt, precision=precision)


def _uniform_row(nd):
    v = VEL[:nd]
    e = PRES / (GAMMA - 1.0) + 0.5 * RHO * sum(c * c for c in v)
    return [RHO] + [RHO * c for c in v] + [e]


def _flux(u, gamma):
    nd = u.size - 2
    rho, mom, en = u[0], u[1:1 + nd], u[nd + 1]
    vel = mom / rho
    p = (gamma - 1.0) * (en - 0.5 * rho * vel @ vel)
    f = np.zeros((u.size, nd))
    for d in range(nd):
        f[0, d] = mom[d]
        for k in range(nd):
            f[1 + k, d] = mom[k] * vel[d] + (p if k == d else 0.0)
        f[nd + 1, d] = (en + p) * vel[d]
    return f


# -- solution storage and initialisation (test_multidim.py:450-599) ---------

@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_storage_and_init(name):
    mesh = fixture_mesh(name)
    ec = _core(mesh)
    nd, neq = mesh.ndim, mesh.ndim + 2
    tot = ec.ngstcell + ec.ncell
    assert ec.neq == neq
    for a in ("so0c", "so0n", "so0t", "stm"):
        assert getattr(ec, a).shape == (tot, neq)
    for a in ("so1c", "so1n"):
        assert getattr(ec, a).shape == (tot, neq, nd)
    for a in ("cflo", "cflc", "gamma"):
        assert getattr(ec, a).shape == (tot,)
    ec.init_solution(gamma=GAMMA, rho=RHO, v=list(VEL[:nd]), p=PRES)
    row = _uniform_row(nd)
    for icl in range(ec.ncell):
        np.testing.assert_allclose([ec.so0n[icl, k] for k in range(neq)], row)
    for icl in range(-ec.ngstcell, 0):
        assert all(ec.so0n[icl, k] == 0.0 for k in range(neq))
    np.testing.assert_allclose(ec.gamma.ndarray, GAMMA)
    for bad in (dict(v=[0.1] * (nd - 1)), dict(gamma=1.0), dict(rho=0.0),
                dict(p=-1.0)):
        args = dict(gamma=GAMMA, rho=RHO, v=list(VEL[:nd]), p=PRES)
        args.update(bad)
        with pytest.raises(ValueError):
            ec.init_solution(**args)
    assert ec.sigma0 == 3.0 and ec.taumin == 0.0 and ec.tauscale == 1.0
    ec.sigma0, ec.taumin, ec.tauscale = 2.5, 0.1, 0.7
    assert (ec.sigma0, ec.taumin, ec.tauscale) == (2.5, 0.1, 0.7)


@pytest.mark.parametrize("name", ["tri3", "mixed", "tet1", "hex1"])
def test_calc_cfl_uniform_and_negative_pressure(name):
    mesh = fixture_mesh(name)
    ec = _core(mesh)
    nd = mesh.ndim
    v = VEL[:nd]
    ec.init_solution(gamma=GAMMA, rho=RHO, v=list(v), p=PRES)
    ec.calc_cfl()
    hdt = ec.time_increment / 2.0
    wspd = np.sqrt(GAMMA * PRES / RHO) + np.sqrt(sum(c * c for c in v))
    cecnd = ec.cecnd
    for icl in range(ec.ncell):
        nfc = mesh.clfcs[icl, 0]
        dist = min(np.sqrt(sum((cecnd[icl, f * nd + d] - cecnd[icl, d]) ** 2
                               for d in range(nd))) for f in range(1, nfc + 1))
        np.testing.assert_allclose(ec.cflo[icl], hdt * wspd / dist, rtol=1e-13)
        np.testing.assert_allclose(ec.cflc[icl], ec.cflo[icl], rtol=1e-13)
    for icl in range(ec.ncell):
        ec.so0n[icl, nd + 1] = 0.0
    ec.calc_cfl()
    ke = sum((RHO * c) ** 2 for c in v) / (2.0 * RHO)
    for icl in range(ec.ncell):
        np.testing.assert_allclose(ec.cflc[icl], 1.0, rtol=1e-14)
        np.testing.assert_allclose(ec.so0n[icl, nd + 1], ke, rtol=1e-13)


def test_update_swaps_buffers():
    ec = _core(fixture_mesh("mixed"))
    ec.init_solution(gamma=GAMMA, rho=RHO, v=[0.3, -0.15], p=PRES)
    view = ec.so1n.ndarray
    view[...] = np.arange(view.size, dtype="float64").reshape(view.shape)
    before = {a: np.array(getattr(ec, a).ndarray)
              for a in ("so0c", "so0n", "so1c", "so1n")}
    ec.update()
    np.testing.assert_array_equal(ec.so0c.ndarray, before["so0n"])
    np.testing.assert_array_equal(ec.so0n.ndarray, before["so0c"])
    np.testing.assert_array_equal(ec.so1c.ndarray, before["so1n"])
    np.testing.assert_array_equal(ec.so1n.ndarray, before["so1c"])
    # The view taken before update() still aliases the same table.
    np.testing.assert_array_equal(view, ec.so1c.ndarray)


# -- marching primitives (test_multidim.py:600-789) -------------------------

@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_calc_solt_is_minus_flux_combination(name):
    mesh = fixture_mesh(name)
    ec = _core(mesh)
    nd, neq = mesh.ndim, mesh.ndim + 2
    row = np.array(_uniform_row(nd))
    coef = np.array([0.7, -1.3, 0.4][:nd])
    so0c, so1c, gamma = (np.array(ec.so0c.ndarray), np.array(ec.so1c.ndarray),
                         np.array(ec.gamma.ndarray))
    ng = ec.ngstcell
    gamma[ng:] = GAMMA
    so0c[ng:] = row
    so1c[ng:] = row[None, :, None] * coef[None, None, :]
    ec.gamma.ndarray[...] = gamma
    ec.so0c.ndarray[...] = so0c
    ec.so1c.ndarray[...] = so1c
    ec.calc_solt()
    expect = -(_flux(row, GAMMA) * coef[None, :]).sum(axis=1)
    got = np.array(ec.so0t.ndarray)[ng:]
    np.testing.assert_allclose(got, np.broadcast_to(expect, got.shape),
                               rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_calc_soln_preserves_free_stream(name):
    mesh = fixture_mesh(name)
    ec = _core(mesh)
    row = _uniform_row(mesh.ndim)
    ec.gamma.ndarray[...] = GAMMA
    ec.so0c.ndarray[...] = row
    ec.so0t.ndarray[...] = 0.0
    ec.so1c.ndarray[...] = 0.0
    ec.calc_solt()
    ec.calc_soln()
    got = np.array(ec.so0n.ndarray)[ec.ngstcell:]
    np.testing.assert_allclose(got, np.broadcast_to(row, got.shape),
                               rtol=1e-12)


@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_calc_dsoln_recovers_linear_field(name):
    mesh = fixture_mesh(name)
    ec = _core(mesh)
    nd, neq = mesh.ndim, mesh.ndim + 2
    g = np.array([[0.1 * (i + 1) + 0.01 * (d + 1) for d in range(nd)]
                  for i in range(neq)])
    c = np.array([0.5 + 0.3 * i for i in range(neq)])
    cecnd = np.array(ec.cecnd.ndarray)
    clcnd = np.array(mesh.clcnd.ndarray)
    ng = ec.ngstcell
    pts = np.where(np.arange(-ng, ec.ncell)[:, None] >= 0, cecnd[:, :nd],
                   clcnd)
    vals = c[None, :] + pts @ g.T
    ec.so0c.ndarray[...] = vals
    ec.so0n.ndarray[...] = vals
    ec.so0t.ndarray[...] = 0.0
    ec.so1c.ndarray[...] = g[None]
    ec.cflc.ndarray[...] = 0.5
    ec.calc_dsoln()
    got = np.array(ec.so1n.ndarray)[ng:]
    np.testing.assert_allclose(got, np.broadcast_to(g, got.shape), rtol=1e-9,
                               atol=1e-10)


# -- boundary conditions (test_multidim.py:810-1084) ------------------------

def _bnd(mesh):
    faces = [int(f) for f in mesh.bndfcs.ndarray[:, 0]]
    return faces, [(f, mesh.fccls[f, 0], mesh.fccls[f, 1]) for f in faces]


@pytest.mark.parametrize("name", ["tri3", "quad1", "mixed", "tet1", "hex1",
                                  "prism1", "pyr1"])
def test_boundary_conditions(name):
    mesh = fixture_mesh(name)
    nd, neq = mesh.ndim, mesh.ndim + 2
    faces, bnd = _bnd(mesh)
    eye = np.eye(nd)
    # normal matrix: orthonormal, first row the outward normal.
    ec = _core(mesh)
    for f in faces:
        mat = np.array(ec.get_normal_matrix(f))
        np.testing.assert_allclose(mat @ mat.T, eye, atol=1e-12)
        np.testing.assert_allclose(mat[0], [mesh.fcnml[f, d]
                                            for d in range(nd)], atol=1e-12)
        np.testing.assert_allclose(np.linalg.det(mat), 1.0, atol=1e-12)
    with pytest.raises(IndexError):
        ec.get_normal_matrix(10 ** 7)
    # non-reflective
    ec = _core(mesh)
    body = np.array(ec.so0n.ndarray)
    for icl in range(ec.ncell):
        body[icl + ec.ngstcell] = [1.0 + 0.1 * icl + 0.37 * k
                                   for k in range(neq)]
    ec.so0n.ndarray[...] = body
    g1 = np.array(ec.so1c.ndarray)
    for icl in range(ec.ncell):
        for k in range(neq):
            for d in range(nd):
                g1[icl + ec.ngstcell, k, d] = 0.2 + 0.1 * k - 0.05 * d + \
                    0.03 * icl
    ec.so1c.ndarray[...] = g1
    ec.add_nonrefl(faces)
    ec.bc_soln()
    ec.bc_dsoln()
    for f, icl, jcl in bnd:
        n = np.array([mesh.fcnml[f, d] for d in range(nd)])
        np.testing.assert_allclose(ec.so0n[jcl], ec.so0n[icl], rtol=1e-15)
        gi, gg = ec.so1c[icl], ec.so1n[jcl]
        np.testing.assert_allclose(gg, gi - np.outer(gi @ n, n), atol=1e-12)
    # slip wall
    ec.clear_bc()
    ec.add_slipwall(faces)
    ec.bc_soln()
    ec.bc_dsoln()
    for f, icl, jcl in bnd:
        n = np.array([mesh.fcnml[f, d] for d in range(nd)])
        refl = eye - 2.0 * np.outer(n, n)
        mi, mg = ec.so0n[icl][1:1 + nd], ec.so0n[jcl][1:1 + nd]
        np.testing.assert_allclose(mg, refl @ mi, atol=1e-12)
        assert ec.so0n[jcl, 0] == ec.so0n[icl, 0]
        assert ec.so0n[jcl, neq - 1] == ec.so0n[icl, neq - 1]
        for k in (0, neq - 1):
            np.testing.assert_allclose(ec.so1n[jcl][k], refl @ ec.so1c[icl][k],
                                       atol=1e-12)
        gmi = ec.so1c[icl][1:1 + nd]
        np.testing.assert_allclose(ec.so1n[jcl][1:1 + nd], refl @ gmi @ refl,
                                   atol=1e-12)
    # inlet
    ec.clear_bc()
    val = [1.3] + [2.0, 0.3, -0.1][:nd] + [0.8, GAMMA]
    ec.add_inlet(faces, value=val)
    ec.bc_soln()
    ec.bc_dsoln()
    en = 0.8 / (GAMMA - 1.0) + 0.5 * 1.3 * sum(c * c for c in val[1:1 + nd])
    for f, icl, jcl in bnd:
        np.testing.assert_allclose(
            ec.so0n[jcl], [1.3] + [1.3 * c for c in val[1:1 + nd]] + [en])
        assert not np.any(ec.so1n[jcl])
    # validation
    with pytest.raises(ValueError):
        ec.add_inlet(faces, value=[1.0] * (nd + 2))
    for bad in ([0.0] + [0.0] * nd + [1.0, 1.4],
                [1.0] + [0.0] * nd + [-1.0, 1.4],
                [1.0] + [0.0] * nd + [1.0, 1.0]):
        with pytest.raises(ValueError):
            ec.add_inlet(faces, value=bad)
    with pytest.raises(ValueError):
        ec.add_nonrefl([10 ** 7])


def test_channel_march_bounded():
    lx, ly = 4.0, 2.0
    mesh = quad_channel(4, 2, lx, ly)
    left, right, walls = [], [], []
    for f in mesh.bndfcs.ndarray[:, 0]:
        f = int(f)
        cx = mesh.fccnd[f, 0]
        (left if abs(cx) < 1e-9 else right if abs(cx - lx) < 1e-9
         else walls).append(f)
    ec = _core(mesh, dt=0.04)
    ec.init_solution(gamma=1.4, rho=1.0, v=[2.0, 0.0], p=1.0)
    ec.add_inlet(left, value=[1.0, 2.0, 0.0, 1.0, 1.4])
    ec.add_nonrefl(right)
    ec.add_slipwall(walls)
    ec.bc_soln()
    ec.bc_dsoln()
    ec.march(steps=5)
    so0n = np.array(ec.so0n.ndarray)
    assert np.all(np.isfinite(so0n))
    np.testing.assert_allclose(so0n[ec.ngstcell:, 0], 1.0, atol=1e-6)
    for f in left:
        np.testing.assert_allclose(ec.so0n[mesh.fccls[f, 1], 0], 1.0)


# -- parity with the oracle ---------------------------------------------------

def _meshes():
    from solvcon_gb300 import meshgen
    out = {}
    for name, (nd, gen, args) in {
            "tri": (2, meshgen.tri_square, (7, 0.2, 4)),
            "quad": (2, meshgen.quad_square, (6, 0.15, 5)),
            "tet": (3, meshgen.tet_cube, (2, 0.15, 6)),
            "hex": (3, meshgen.hex_cube, (3, 0.1, 7)),
            "prism": (3, meshgen.prism_slab, (3, 2, 0.1, 8))}.items():
        x, t, c = gen(*args)
        out[name] = meshgen.build_mesh(nd, x, t, c)
    for name in ("mixed", "pyr1", "prism1"):
        out[name] = fixture_mesh(name)
    return out


_MESHES = None


def meshes():
    global _MESHES
    if _MESHES is None:
        _MESHES = _meshes()
    return _MESHES


MESH_NAMES = ["tri", "quad", "tet", "hex", "prism", "mixed", "pyr1", "prism1"]


def _random_state(ec, seed):
    rng = np.random.default_rng(seed)
    nd, neq = ec.ndim, ec.neq
    tot = ec.ncell + ec.ngstcell
    rho = rng.uniform(0.5, 1.5, tot)
    v = rng.uniform(-0.5, 0.5, (tot, nd))
    p = rng.uniform(0.5, 1.5, tot)
    from solvcon_gb300 import meshgen
    so0 = meshgen.conserved(rho, v, p, GAMMA)
    so1 = rng.uniform(-0.3, 0.3, (tot, neq, nd))
    so0t = rng.uniform(-0.3, 0.3, (tot, neq))
    return so0, so1, so0t


def _pair(name, dt=0.01, precision="fp64"):
    from oracle import oracle as ora
    mesh = meshes()[name]
    return mesh, _core(mesh, dt, precision), ora.OracleEuler(mesh, dt)


def _load(ec, ref, **arrays):
    for k, v in arrays.items():
        getattr(ec, k).ndarray[...] = v
        getattr(ref, k)[...] = v


@pytest.mark.parametrize("name", MESH_NAMES)
def test_prepare_ce_matches_oracle(name):
    mesh, ec, ref = _pair(name)
    for a in ("cevol", "cecnd", "sfcnd", "sfnml"):
        assert_rel(ec.__getattribute__(a).ndarray, getattr(ref, a), 1e-14, a)


@pytest.mark.parametrize("name", MESH_NAMES)
def test_each_operation_matches_oracle(name):
    mesh, ec, ref = _pair(name)
    so0, so1, so0t = _random_state(ec, 11)
    gamma = np.full(ec.ncell + ec.ngstcell, GAMMA)
    _load(ec, ref, so0c=so0, so1c=so1, so0t=so0t, gamma=gamma)
    ec.calc_solt()
    ref.call("calc_solt")
    assert_rel(ec.so0t.ndarray, ref.so0t, 1e-12, "calc_solt")
    _load(ec, ref, so0t=so0t)
    ec.calc_soln()
    ref.call("calc_soln")
    ng = ec.ngstcell
    assert_rel(np.array(ec.so0n.ndarray)[ng:], ref.so0n[ng:], 1e-12,
               "calc_soln")
    _load(ec, ref, so0n=np.array(ref.so0n))
    ec.calc_cfl()
    ref.call("calc_cfl")
    assert_rel(ec.cflo.ndarray, ref.cflo, 1e-13, "cflo")
    assert_rel(ec.cflc.ndarray, ref.cflc, 1e-13, "cflc")
    assert_rel(ec.so0n.ndarray, ref.so0n, 1e-13, "cfl energy")
    _load(ec, ref, so0n=np.array(ref.so0n), cflc=np.array(ref.cflc))
    ec.calc_dsoln()
    ref.call("calc_dsoln")
    assert_rel(np.array(ec.so1n.ndarray)[ng:], ref.so1n[ng:], 1e-11,
               "calc_dsoln")
    mask = ec.limiter_mask()
    assert np.array_equal(mask, ref.limiter[:ec.ncell])
    faces = [int(f) for f in mesh.bndfcs.ndarray[:, 0]]
    for kind in (0, 1, 2):
        _load(ec, ref, so1c=so1)
        ec.clear_bc()
        ref._bcs = []
        val = [1.3] + [0.4, -0.2, 0.1][:ec.ndim] + [0.8, GAMMA]
        half = faces[: max(1, len(faces) // 2)]
        ec._add_bc(kind, half, val if kind == 2 else ())
        ref.add_bc(kind, half, val if kind == 2 else ())
        ec.bc_soln()
        ec.bc_dsoln()
        ref.call("bc_soln")
        ref.call("bc_dsoln")
        assert_rel(ec.so0n.ndarray, ref.so0n, 1e-14, "bc_soln %d" % kind)
        assert_rel(ec.so1n.ndarray, ref.so1n, 1e-14, "bc_dsoln %d" % kind)


@pytest.mark.parametrize("name", MESH_NAMES)
def test_march_matches_oracle(name):
    from solvcon_gb300 import meshgen
    mesh, ec, ref = _pair(name, dt=2e-3)
    ng = ec.ngstcell
    clcnd = np.array(mesh.clcnd.ndarray)[ng:]
    if mesh.ndim == 2:
        state = meshgen.quadrant_state(clcnd[:, :2], seed=9)
    else:
        state = meshgen.blast_state(clcnd, radius=0.4)
    faces = [int(f) for f in mesh.bndfcs.ndarray[:, 0]]
    for core in (ec, ref):
        core.init_solution(GAMMA, 1.0, [0.0] * mesh.ndim, 1.0)
        core.add_slipwall(faces)
    ec.so0n.ndarray[ng:] = state
    ref.so0n[ng:] = state
    ec.bc_soln()
    ec.bc_dsoln()
    ref.call("bc_soln")
    ref.call("bc_dsoln")
    ec.march(4)
    ref.march(4)
    for a in ("so0c", "so0n", "so0t", "so1c", "so1n", "cflo", "cflc"):
        assert_rel(getattr(ec, a).ndarray, getattr(ref, a), 1e-10, a)
    ec.march_substep()
    ref.call("march_substep")
    for a in ("so0n", "so1n", "so0t"):
        assert_rel(getattr(ec, a).ndarray, getattr(ref, a), 1e-10, a)
    tot = ec.totals()
    vol = np.array(mesh.clvol.ndarray)[ng:]
    q = np.array(ref.so0n)[ng:] * vol[:, None]
    want = q.sum(axis=0)
    # Totals that cancel (a momentum component at rest) are compared against
    # the sum of magnitudes they cancel from.
    np.testing.assert_allclose(tot, want, rtol=1e-12,
                               atol=1e-13 * np.abs(q).sum())
    lo, hi = ec.cfl_range()
    np.testing.assert_allclose([lo, hi], [ref.cflo[ng:].min(),
                                          ref.cflo[ng:].max()], rtol=1e-12)


def test_march_matches_reference_golden():
    """The march of the golden fixtures generated from the reference."""
    from _util import golden
    from test_mesh import _build
    for case in ("tri12", "quad8", "tet3"):
        gm = golden("mesh_" + case)
        g = golden("march_" + case)
        mesh = _build(gm)
        ec = _core(mesh, dt=float(g["dt"]))
        ec.init_solution(1.4, 1.0, [0.0] * mesh.ndim, 1.0)
        ec.so0n.ndarray[ec.ngstcell:] = g["state0"]
        ec._add_bc(int(g["bc_kind"]), g["faces"])
        ec.bc_soln()
        ec.bc_dsoln()
        ec.march(int(g["steps"]))
        for a in ("so0c", "so0n", "so0t", "so1c", "so1n", "cflo", "cflc"):
            assert_rel(getattr(ec, a).ndarray, g[a], 1e-10, case + " " + a)


# -- FP32-state variants: error against the FP64 oracle -----------------------

@pytest.mark.parametrize("kind", ["tri", "tet", "quad", "hex", "prism"])
def test_fp32_state_error_against_oracle(kind):
    """FP32 forms of the march -- ``fp32`` (FP32 state and flux arithmetic
    with compensated face sums, FP64 geometry tables) and ``fp32-geom32``
    (the geometry stored FP32 too) -- against the FP64 oracle at the
    workloads' CFL: the 3D spherical blast (CFL 0.7) and a 2D four-quadrant
    state (CFL 0.8), 60 steps, relative L1 <= 1e-5 per conserved variable
    (measured on GB300: 2D triangles 1.5e-6 with FP64 geometry, 3.9e-6 with
    FP32 geometry; 3D 3.4e-7).  Totals: FP64 totals of the FP32 march within
    1e-6 relative of the oracle's for mass and energy.  Triangles and
    tetrahedra run the kernels compiled for one simplex type (neighbour
    terms carried); quadrilaterals, hexahedra and prisms the kernels that
    dispatch on the cell type (neighbour records gathered twice)."""
    import bench
    from oracle import oracle as ora
    from solvcon_gb300 import meshgen
    ndim = 2 if kind in ("tri", "quad") else 3
    if kind == "tri":
        x, t, c = meshgen.tri_square(48, 0.2, seed=31)
    elif kind == "quad":
        x, t, c = meshgen.quad_square(48, 0.15, seed=31)
    elif kind == "tet":
        x, t, c = meshgen.tet_cube(8, 0.15, seed=31)
    elif kind == "hex":
        x, t, c = meshgen.hex_cube(12, 0.1, seed=31)
    else:
        x, t, c = meshgen.prism_slab(12, 6, 0.1, seed=31)
    mesh = meshgen.build_mesh(ndim, x, t, c)
    ng = mesh.ngstcell
    clcnd = np.array(mesh.clcnd.ndarray)[ng:]
    state = meshgen.quadrant_state(clcnd[:, :2], seed=31) if ndim == 2 \
        else meshgen.blast_state(clcnd)
    faces = np.array(mesh.bndfcs.ndarray[:, 0])
    dt = bench.dt_for_cfl(mesh, state, faces, 0.8 if ndim == 2 else 0.7)
    steps = 60
    ref = ora.OracleEuler(mesh, dt)
    ref.init_solution(GAMMA, 1.0, [0.0] * ndim, 1.0)
    ref.so0n[ng:] = state
    ref.add_slipwall(faces)
    ref.call("bc_soln")
    ref.call("bc_dsoln")
    ref.march(steps)
    want = np.array(ref.so0n)[ng:]
    vol = np.array(mesh.clvol.ndarray)[ng:]
    twant = (want * vol[:, None]).sum(axis=0)
    per_var = 1e-5
    for prec in ("fp32", "fp32-geom32"):
        ec = bench.setup_core(mesh, state, faces, dt, prec)
        ec.march(steps)
        got = np.array(ec.so0n[...])[ng:]
        d = np.abs(got - want)
        for k in range(ndim + 2):
            l1 = d[:, k].sum() / np.abs(want[:, k]).sum()
            assert l1 < per_var, (prec, k, l1)
        assert d.sum() / np.abs(want).sum() < 1e-5
        tgot = ec.totals()
        for k in (0, ndim + 1):
            assert abs(tgot[k] - twant[k]) <= 1e-6 * abs(twant[k]), (prec, k)


# -- connectivity written by a caller is checked before any kernel uses it ---

@pytest.mark.parametrize("what", ["face", "face_cell", "node", "count"])
def test_core_rejects_inconsistent_connectivity(what):
    import solvcon_gb300 as sg
    mesh = fixture_mesh("mixed")
    ng, ngf = int(mesh.ngstcell), int(mesh.ngstface)
    clfcs = mesh.clfcs.ndarray
    fccls = mesh.fccls.ndarray
    fcnds = mesh.fcnds.ndarray
    ifc = int(clfcs[ng + 1, 1])
    if what == "face":
        clfcs[ng + 1, 1] = mesh.nface + 7
    elif what == "face_cell":
        # The face no longer lists cell 1 among its two cells.
        fccls[ngf + ifc, 0] = 0 if fccls[ngf + ifc, 0] != 0 else 2
        fccls[ngf + ifc, 1] = 0 if fccls[ngf + ifc, 1] != 0 else 2
    elif what == "node":
        fcnds[ngf + ifc, 1] = mesh.nnode + 3
    else:
        clfcs[ng + 1, 0] = 9
    with pytest.raises(ValueError, match="connectivity of cell"):
        sg.EulerCore(mesh=mesh, time_increment=0.01)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_reset_state_gives_a_fresh_core(precision):
    """reset_state (not in the reference) puts a used core back to a new
    core's state: the same march from the same start gives the same bits."""
    from solvcon_gb300 import meshgen
    x, t, c = meshgen.tri_square(12, 0.2, seed=9)
    mesh = meshgen.build_mesh(2, x, t, c)
    clcnd = np.array(mesh.clcnd.ndarray)[mesh.ngstcell:]
    state = meshgen.quadrant_state(clcnd, seed=9)
    faces = [int(f) for f in mesh.bndfcs.ndarray[:, 0]]

    def start(core):
        core.init_solution(GAMMA, 1.0, [0.0, 0.0], 1.0)
        core.so0n[0:] = state
        core.bc_soln()
        core.bc_dsoln()

    used = _core(mesh, 2e-3, precision)
    used.add_slipwall(faces)
    start(used)
    used.march(3)
    used.update()  # leave the buffer bookkeeping off its initial state
    used.reset_state()
    for name in ("so0c", "so0n", "so1n", "cflo", "gamma"):
        assert not np.array(getattr(used, name)[...]).any(), name
    start(used)
    used.march(2)
    fresh = _core(mesh, 2e-3, precision)
    fresh.add_slipwall(faces)
    start(fresh)
    fresh.march(2)
    for name in ("so0c", "so0n", "so0t", "so1c", "so1n", "cflo", "cflc"):
        np.testing.assert_array_equal(getattr(used, name).ndarray,
                                      getattr(fresh, name).ndarray, name)


def test_core_on_a_reference_built_mesh():
    """EulerCore on a mesh built by reference code (the reference's golden
    tables behind its StaticMesh surface, taken over verbatim) marches as
    the reference did."""
    from _util import golden
    from test_mesh import _foreign_from_golden
    for case in ("tri12", "tet3"):
        g = golden("march_" + case)
        foreign = _foreign_from_golden(golden("mesh_" + case))
        ec = _core(foreign, dt=float(g["dt"]))
        ec.init_solution(1.4, 1.0, [0.0] * foreign.ndim, 1.0)
        ec.so0n.ndarray[ec.ngstcell:] = g["state0"]
        ec._add_bc(int(g["bc_kind"]), g["faces"])
        ec.bc_soln()
        ec.bc_dsoln()
        ec.march(int(g["steps"]))
        for a in ("so0n", "so1n", "cflo"):
            assert_rel(getattr(ec, a).ndarray, g[a], 1e-10, case + " " + a)


def test_geometry_rounding_is_round_to_nearest_even():
    """The FP32 march rounds its FP64 geometry tables to FP32 with integer
    instructions; on the device that rounding equals IEEE
    round-to-nearest-even (numpy's float64 -> float32) bit for bit over the
    FP32 normal range: random values, exact ties, near-ties, mantissa
    carries into the exponent (up to infinity from the top binade).  Values
    below the normal range become a signed zero.  Larger ones are not taken:
    a core of the FP32 form refuses a mesh whose geometry holds them (tested
    below)."""
    from solvcon_gb300._lib import check, lib, ptr
    rng = np.random.default_rng(5)
    n = 1 << 20
    bits = rng.integers(0, 2 ** 63, n, dtype=np.uint64)
    bits |= rng.integers(0, 2, n, dtype=np.uint64) << np.uint64(63)
    exp = rng.integers(880, 1170, n, dtype=np.uint64)
    bits = (bits & ~np.uint64(0x7FF << 52)) | (exp << np.uint64(52))
    low = np.uint64(0x1FFFFFFF)
    for k, pat in enumerate((0x10000000, 0x0FFFFFFF, 0x10000001)):
        sl = slice(k * 50000, (k + 1) * 50000)
        bits[sl] = (bits[sl] & ~low) | np.uint64(pat)
    bits[200000:250000] |= np.uint64((1 << 52) - 1)
    x = bits.view(np.float64).copy()
    x[:10] = [0.0, -0.0, 1e-40, -3e-39, 1e39, np.inf, -np.inf, np.nan,
              5e-324, -1e-310]
    got = np.empty(n, dtype=np.float32)
    check(lib.scg_geometry_round(ptr(x), ptr(got), n))
    with np.errstate(over="ignore"):
        want = x.astype(np.float32)
    e = (x.view(np.uint64) >> np.uint64(52)) & np.uint64(0x7FF)
    normal = (e >= 897) & (e <= 1150)
    g, w = got.view(np.uint32), want.view(np.uint32)
    same = g[normal] == w[normal]
    assert same.all(), x[normal][~same][:5]
    tiny = e < 897
    assert tiny.sum() >= 6
    assert (got[tiny] == 0).all()
    assert (np.signbit(got[tiny]) == np.signbit(x[tiny])).all()



def test_fp32_form_refuses_geometry_outside_fp32_range():
    """The FP32 form keeps FP64 geometry and rounds it where it is used,
    without an overflow check; a mesh whose geometry goes beyond FP32's
    range (a unit square scaled by 1e25: areas of 1e50) is refused when the
    core is built, and marches in FP64 as before."""
    import solvcon_gb300 as sg
    from solvcon_gb300 import meshgen
    x, t, c = meshgen.tri_square(6, 0.2, seed=1)
    mesh = meshgen.build_mesh(2, x * 1e25, t, c)
    with pytest.raises(ValueError, match="beyond FP32's range"):
        sg.EulerCore(mesh, 1e20, precision="fp32")
    ec = sg.EulerCore(mesh, 1e20, precision="fp64")
    assert ec.ncell == mesh.ncell

@pytest.mark.parametrize("precision", ["fp32", "fp32-geom32"])
def test_fp32_state_keeps_its_rounding_residual(precision):
    """An FP32 core's state is its FP32 so0 plus the rounding residual it
    carries: an FP64 so0n written through the API reads back to ~1e-14
    (not to FP32's 6e-8), and its totals are the FP64 totals of what was
    written."""
    from solvcon_gb300 import meshgen
    x, t, c = meshgen.tri_square(20, 0.2, seed=5)
    mesh = meshgen.build_mesh(2, x, t, c)
    ec = _core(mesh, 1e-3, precision)
    ec.init_solution(GAMMA, 1.0, [0.0, 0.0], 1.0)
    rng = np.random.default_rng(3)
    ng = ec.ngstcell
    so0 = np.array(ec.so0n.ndarray)
    so0[ng:] = rng.uniform(0.5, 1.5, so0[ng:].shape)
    ec.so0n.ndarray[...] = so0
    ec.release_views()
    got = np.array(ec.so0n.ndarray)
    assert np.abs(got[ng:] - so0[ng:]).max() < 1e-14
    vol = np.array(mesh.clvol.ndarray)[ng:]
    want = (so0[ng:] * vol[:, None]).sum(0)
    np.testing.assert_allclose(ec.totals(), want, rtol=1e-14)


@pytest.mark.parametrize("precision", ["fp32", "fp32-geom32"])
def test_fp32_totals_track_fp64(precision):
    """The FP32 march feeds each cell's rounding residual back into the
    cell's next value, so the roundings of the state cancel in the totals
    instead of accumulating: the FP32 totals stay within 3e-9 of the FP64
    march's on the 3D blast (200 steps, 20^3 x 6 tetrahedra; measured on
    GB300 7.3e-10 with FP64 geometry, 1.3e-9 with FP32 geometry), where
    rounding alone drifts them ~1e-8 and growing."""
    import bench
    w, mesh, state, faces = bench.make_workload("tet3d", nside=20)
    dt = bench.dt_for_cfl(mesh, state, faces, 0.7)
    ref = bench.setup_core(mesh, state, faces, dt, "fp64")
    ec = bench.setup_core(mesh, state, faces, dt, precision)
    worst = 0.0
    for _ in range(10):
        ref.march(20)
        ec.march(20)
        a, b = np.array(ec.totals()), np.array(ref.totals())
        worst = max(worst, float(np.max(np.abs(a - b)[[0, 4]] /
                                        np.abs(b)[[0, 4]])))
    print("%s: FP32 mass/energy totals within %.2e of FP64" % (precision,
                                                              worst))
    assert worst < 3e-9
