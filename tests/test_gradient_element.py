"""GradientElement, the per-cell gradient geometry of the CESE dual mesh.

Structural and geometric checks follow the reference's own GradientElement
tests (tests/test_multidim.py:284-421): accessor bounds, the sub-element
table, displacement-matrix rank, the idis/jdis identity, the tau = 0 shift,
per-sub-element non-singularity and exact recovery of a linear field.  The CE
geometry (``cecnd``) comes from the oracle on the CPU and from the device
EulerCore on the GPU.

calc_dsoln is then checked against an independent weighting written on top
of ``GradientElement.solve_gradient`` (the reference does the same in
tests/test_multidim.py:97-149 and :740-768): a non-linear field makes the
sub-element gradients differ, so the W-1/2 weights and the W-3/4 limiter are
live, not the trivial linear-field case.  On the CPU that pins the oracle's
calc_dsoln; on the GPU (``-m gpu``) the device kernel, to 1e-10 absolute
(FP64; the sums run in another order).
"""

import types

import numpy as np
import pytest

from _util import FIXTURES, fixture_mesh

# Sub-elements per cell type (GradientElement.cpp:16-79): quadrilateral 4,
# triangle 3, hexahedron 8, tetrahedron 4, prism 6, pyramid 6.
NFGE = {3: 4, 4: 3, 5: 8, 6: 4, 7: 6, 8: 6}

GENERATED = {
    "tri_square3": ("tri_square", (3, 0.2, 1)),
    "quad_square3": ("quad_square", (3, 0.15, 2)),
    "tet_cube2": ("tet_cube", (2, 0.15, 3)),
    "hex_cube2": ("hex_cube", (2, 0.1, 4)),
    "prism_slab2": ("prism_slab", (2, 2, 0.1, 5)),
}
MESHES = sorted(FIXTURES) + sorted(GENERATED)


def _mesh(name):
    if name in FIXTURES:
        return fixture_mesh(name)
    from solvcon_gb300 import meshgen
    fn, args = GENERATED[name]
    x, t, c = getattr(meshgen, fn)(*args)
    return meshgen.build_mesh(x.shape[1], x, t, c)


def _oracle_ce(mesh, dt=0.01):
    """The oracle core of ``mesh`` and its CE centroids as a ghost-indexed
    SimpleArray, the argument GradientElement takes."""
    from oracle import oracle as ora
    from solvcon_gb300.buffer import SimpleArray
    o = ora.OracleEuler(mesh, dt)
    return o, SimpleArray(lambda: o.cecnd, nghost=o.ngstcell)


def _ge(mesh, cecnd, icl, tau=1.0):
    from solvcon_gb300 import GradientElement
    return GradientElement(mesh=mesh, cecnd=cecnd, icl=icl, tau=tau)


def _points(mesh, cecnd):
    """Solution points of every row, ghosts first: the CE centroid of an
    interior cell, the cell centroid of a ghost."""
    nd, ng = mesh.ndim, int(mesh.ngstcell)
    pts = np.array(np.asarray(cecnd)[:, :nd])
    pts[:ng] = np.asarray(mesh.clcnd.ndarray)[:ng]
    return pts


# -- structure (tests/test_multidim.py:284-351) ------------------------------

@pytest.mark.parametrize("name", MESHES)
def test_basic_properties(name):
    mesh = _mesh(name)
    _, cecnd = _oracle_ce(mesh)
    for icl in range(mesh.ncell):
        ge = _ge(mesh, cecnd, icl)
        assert ge.icl == icl
        assert ge.ndim == mesh.ndim
        assert ge.clnfc == mesh.clfcs[icl, 0]
        assert ge.nfge == NFGE[int(mesh.cltpn[icl])]
        assert ge.nfge_inverse == 1.0 / ge.nfge
        for ifl in range(ge.clnfc):
            ifc = mesh.clfcs[icl, ifl + 1]
            pair = {int(mesh.fccls[ifc, 0]), int(mesh.fccls[ifc, 1])}
            assert pair == {icl, ge.rcl(ifl)}


@pytest.mark.parametrize("name", ["tri3", "quad1", "hex1", "pyr1"])
def test_accessor_index_bounds(name):
    mesh = _mesh(name)
    _, cecnd = _oracle_ce(mesh)
    ge = _ge(mesh, cecnd, 0)
    nfc, nd = ge.clnfc, ge.ndim
    for ifl in range(nfc):
        ge.rcl(ifl)
        for d in range(nd):
            ge.idis(ifl, d)
            ge.jdis(ifl, d)
    for ifl in (-1, nfc):
        for call in (lambda: ge.rcl(ifl), lambda: ge.idis(ifl, 0),
                     lambda: ge.jdis(ifl, 0)):
            with pytest.raises(IndexError):
                call()
    for d in (-1, nd):
        with pytest.raises(IndexError):
            ge.idis(0, d)
        with pytest.raises(IndexError):
            ge.jdis(0, d)


@pytest.mark.parametrize("name", sorted(FIXTURES))
def test_fge_table(name):
    mesh = _mesh(name)
    _, cecnd = _oracle_ce(mesh)
    ge = _ge(mesh, cecnd, 0)
    used = set()
    for ifge in range(ge.nfge):
        faces = ge.faces(ifge)
        assert len(faces) == mesh.ndim
        assert len(set(faces)) == mesh.ndim
        assert all(1 <= f <= ge.clnfc for f in faces)
        used.update(faces)
    # Every face of the cell takes part in some sub-element.
    assert used == set(range(1, ge.clnfc + 1))


@pytest.mark.parametrize("name", ["tri3", "tet1", "prism1"])
def test_ifge_and_udf_checks(name):
    mesh = _mesh(name)
    _, cecnd = _oracle_ce(mesh)
    ge = _ge(mesh, cecnd, 0)
    nd = mesh.ndim
    for ifge in (-1, ge.nfge):
        with pytest.raises(IndexError):
            ge.faces(ifge)
        with pytest.raises(IndexError):
            ge.displacement_matrix(ifge)
        with pytest.raises(IndexError):
            ge.solve_gradient(ifge, [0.0] * nd)
    for n in (nd - 1, nd + 1):
        with pytest.raises(ValueError):
            ge.solve_gradient(0, [0.0] * n)


def test_ndim_must_be_2_or_3():
    from solvcon_gb300 import GradientElement
    with pytest.raises(ValueError):
        GradientElement(types.SimpleNamespace(ndim=1), None, 0, 1.0)


# -- geometry (tests/test_multidim.py:354-421) -------------------------------

@pytest.mark.parametrize("name", MESHES)
def test_displacements_span_space(name):
    mesh = _mesh(name)
    _, cecnd = _oracle_ce(mesh)
    nd = mesh.ndim
    for icl in range(mesh.ncell):
        ge = _ge(mesh, cecnd, icl)
        mat = np.array([[ge.idis(ifl, d) for d in range(nd)]
                        for ifl in range(ge.clnfc)])
        assert np.linalg.matrix_rank(mat) == nd, icl
        for ifge in range(ge.nfge):
            sub = np.array(ge.displacement_matrix(ifge))
            assert sub.shape == (nd, nd)
            assert abs(np.linalg.det(sub)) > 1e-10, (icl, ifge)
            rows = np.array([mat[f - 1] for f in ge.faces(ifge)])
            np.testing.assert_array_equal(sub, rows)


@pytest.mark.parametrize("name", MESHES)
def test_idis_jdis_meet_at_one_point(name):
    """idis from the cell's solution point and jdis from the neighbour's
    reach the same gradient evaluation point."""
    mesh = _mesh(name)
    _, cecnd = _oracle_ce(mesh)
    nd, ng = mesh.ndim, int(mesh.ngstcell)
    pts = _points(mesh, cecnd)
    for icl in range(mesh.ncell):
        ge = _ge(mesh, cecnd, icl, tau=0.37)
        for ifl in range(ge.clnfc):
            jcl = ge.rcl(ifl)
            for d in range(nd):
                a = ge.idis(ifl, d) + pts[ng + icl, d]
                b = ge.jdis(ifl, d) + pts[ng + jcl, d]
                assert abs(a - b) <= 1e-12 * max(1.0, abs(a))


@pytest.mark.parametrize("name", MESHES)
def test_tau_zero_puts_points_on_face_centroids(name):
    """At tau = 0 the evaluation points are the CE's face centroids, moved
    all by one common shift."""
    mesh = _mesh(name)
    _, cecnd = _oracle_ce(mesh)
    nd = mesh.ndim
    ce = np.asarray(cecnd)[int(mesh.ngstcell):]
    for icl in range(mesh.ncell):
        ge = _ge(mesh, cecnd, icl, tau=0.0)
        pos = np.array([[ge.idis(ifl, d) + ce[icl, d] for d in range(nd)]
                        for ifl in range(ge.clnfc)])
        bce = ce[icl, nd:(ge.clnfc + 1) * nd].reshape(ge.clnfc, nd)
        shift = pos - bce
        np.testing.assert_allclose(shift, np.broadcast_to(shift[0],
                                                          shift.shape),
                                   rtol=0, atol=1e-12)


@pytest.mark.parametrize("name", MESHES)
def test_solve_gradient_recovers_linear_field(name):
    mesh = _mesh(name)
    _, cecnd = _oracle_ce(mesh)
    nd = mesh.ndim
    grad = np.array([1.5, -2.7, 0.9][:nd])
    rng = np.random.default_rng(7)
    for icl in range(mesh.ncell):
        ge = _ge(mesh, cecnd, icl)
        for ifge in range(ge.nfge):
            dst = np.array(ge.displacement_matrix(ifge))
            got = np.array(ge.solve_gradient(ifge, (dst @ grad).tolist()))
            np.testing.assert_allclose(got, grad, rtol=1e-9, atol=1e-9)
            # Any right-hand side: the cofactor solve agrees with LAPACK.
            udf = rng.standard_normal(nd)
            np.testing.assert_allclose(ge.solve_gradient(ifge, udf.tolist()),
                                       np.linalg.solve(dst, udf),
                                       rtol=1e-10, atol=1e-12)


# -- calc_dsoln against the GradientElement weighting ------------------------

def _field(pts, neq):
    """A smooth non-linear state and an unrelated non-uniform so1c."""
    x = pts[:, 0]
    y = pts[:, 1]
    z = pts[:, -1]
    so0 = np.stack([1.0 + 0.1 * k + 0.6 * x + 0.5 * x * x - 0.3 * x * y
                    + 0.25 * z for k in range(neq)], axis=1)
    nd = pts.shape[1]
    so1 = np.stack([np.stack([0.1 * (k + 1) + 0.05 * (d + 1) * x
                              for d in range(nd)], axis=1)
                    for k in range(neq)], axis=1)
    return so0, so1


def dsoln_by_gradient_elements(mesh, cecnd, so0c, so0t, so0n, so1c, cflc,
                               dt, sigma0, taumin, tauscale):
    """so1n of every interior cell from per-sub-element gradients solved by
    GradientElement, weighted by inverse gradient magnitude and limited so
    no weight leaves [0, 1] and no deviation exceeds sigma0/|cfl|
    (the order-1 weighting of EulerCore::calc_dsoln,
    cpp/solvcon/multidim/euler_gradient.cpp:23-134).  Arrays are whole buffers,
    ghost rows first.  Returns (so1n, whether any weight deviates from the
    uniform one)."""
    nd, ng, ncell = mesh.ndim, int(mesh.ngstcell), int(mesh.ncell)
    neq = nd + 2
    hdt, tiny = 0.5 * dt, 1e-200
    out = np.zeros((ncell, neq, nd))
    live = False
    for icl in range(ncell):
        cfl = abs(cflc[ng + icl])
        ge = _ge(mesh, cecnd, icl, tau=taumin + cfl * tauscale)
        # Solution change from the cell's point to every evaluation point,
        # each extrapolated from the neighbour across that face.
        du = np.empty((ge.clnfc, neq))
        for ifl in range(ge.clnfc):
            j = ng + ge.rcl(ifl)
            jd = np.array([ge.jdis(ifl, d) for d in range(nd)])
            du[ifl] = so0c[j] + hdt * so0t[j] + so1c[j] @ jd - so0n[ng + icl]
        grads = np.array([[ge.solve_gradient(k, du[[f - 1 for f in
                                                    ge.faces(k)], e].tolist())
                           for e in range(neq)] for k in range(ge.nfge)])
        w = 1.0 / np.sqrt((grads * grads).sum(axis=2) + tiny)
        ofg = ge.nfge_inverse
        dev = w / w.sum(axis=0) - ofg
        hi = np.maximum(dev.max(axis=0), 0.0)
        lo = np.minimum(dev.min(axis=0), 0.0)
        sig = np.minimum(np.minimum((1.0 - ofg) / (hi + tiny),
                                    -ofg / (lo - tiny)), sigma0 / cfl)
        live = live or bool(np.abs(dev).max() > 1e-9)
        out[icl] = ((ofg + sig * dev)[:, :, None] * grads).sum(axis=0)
    return out, live


@pytest.mark.parametrize("name", MESHES)
def test_oracle_calc_dsoln_matches_gradient_elements(name):
    mesh = _mesh(name)
    o, cecnd = _oracle_ce(mesh)
    neq, ng = mesh.ndim + 2, o.ngstcell
    so0, so1 = _field(_points(mesh, cecnd), neq)
    o.so0c[:] = so0
    o.so0n[:] = so0
    o.so0t[:] = 0.02 * so0
    o.so1c[:] = so1
    o.cflc[:] = 0.45
    o.call("calc_dsoln")
    ref, live = dsoln_by_gradient_elements(
        mesh, cecnd, o.so0c, o.so0t, o.so0n, o.so1c, o.cflc,
        o.time_increment, o.sigma0, o.taumin, o.tauscale)
    assert live, "every sub-element gradient equal; the limiter is idle"
    np.testing.assert_allclose(o.so1n[ng:], ref, rtol=0,
                               atol=1e-12 * max(1.0, np.abs(ref).max()))


@pytest.mark.gpu
@pytest.mark.parametrize("name", MESHES)
def test_calc_dsoln_matches_gradient_elements(name):
    import solvcon_gb300 as sg
    mesh = _mesh(name)
    ec = sg.EulerCore(mesh=mesh, time_increment=0.01, precision="fp64")
    neq, ng = mesh.ndim + 2, ec.ngstcell
    so0, so1 = _field(_points(mesh, ec.cecnd), neq)
    ec.so0c.ndarray[...] = so0
    ec.so0n.ndarray[...] = so0
    ec.so0t.ndarray[...] = 0.02 * so0
    ec.so1c.ndarray[...] = so1
    ec.cflc.ndarray[...] = 0.45
    ec.calc_dsoln()
    ref, live = dsoln_by_gradient_elements(
        mesh, ec.cecnd, np.array(ec.so0c.ndarray), np.array(ec.so0t.ndarray),
        np.array(ec.so0n.ndarray), np.array(ec.so1c.ndarray),
        np.array(ec.cflc.ndarray), ec.time_increment, ec.sigma0, ec.taumin,
        ec.tauscale)
    assert live, "every sub-element gradient equal; the limiter is idle"
    got = np.array(ec.so1n.ndarray)[ng:]
    np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-10)
