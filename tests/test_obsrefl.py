"""Oblique-shock reflection: relations, channel meshes and the GPU driver.

The relations are checked against the oblique-shock tables (M1 = 3,
theta = 10 deg: beta = 27.38 deg, p2/p1 = 2.054, rho2/rho1 = 1.655,
M2 = 2.505; NACA Report 1135) and their own inversions; the meshes against
the properties the reference mesher promises (counter-clockwise cells, at
most one boundary face per cell, one boundary group per edge); the driver's
GPU march against the CPU oracle on the same mesh, and its steady state
against the analytic zone states.
"""

import math

import numpy as np
import pytest


def _rel():
    from solvcon_gb300.obsrefl import ObliqueShockRelation
    return ObliqueShockRelation(gamma=1.4)


def test_relation_table_values():
    r = _rel()
    theta = math.radians(10.0)
    beta = r.calc_shock_angle(3.0, theta)
    assert abs(math.degrees(beta) - 27.38) < 0.01
    assert abs(r.calc_pressure_ratio(3.0, beta) - 2.054) < 2e-3
    assert abs(r.calc_density_ratio(3.0, beta) - 1.655) < 2e-3
    assert abs(r.calc_dmach(3.0, theta=theta) - 2.505) < 2e-3
    assert abs(r.calc_temperature_ratio(3.0, beta) -
               r.calc_pressure_ratio(3.0, beta) /
               r.calc_density_ratio(3.0, beta)) < 1e-15
    # A normal shock at M = 2: M2 = 0.5774.
    assert abs(r.calc_normal_dmach(2.0) - 0.57735) < 1e-4


def test_relation_inversions_and_errors():
    r = _rel()
    for mach in (1.8, 3.0, 6.0):
        for deg in (2.0, 8.0, 15.0):
            theta = math.radians(deg)
            weak = r.calc_shock_angle(mach, theta, delta=1)
            strong = r.calc_shock_angle(mach, theta, delta=0)
            assert strong > weak
            for beta in (weak, strong):
                assert abs(r.calc_flow_angle(mach, beta) - theta) < 1e-10
            assert abs(r.calc_dmach(mach, beta=weak) -
                       r.calc_dmach(mach, theta=theta)) < 1e-10
    with pytest.raises(ValueError):
        r.calc_shock_angle(1.5, math.radians(20.0))
    with pytest.raises(ValueError):
        r.calc_dmach(3.0)
    with pytest.raises(ValueError):
        r.calc_dmach(3.0, beta=0.5, theta=0.1)


@pytest.mark.parametrize("flavor", ["quad", "triangle", "unstructured"])
def test_meshes(flavor):
    from solvcon_gb300.obsrefl import ObliqueShockMesher
    ms = ObliqueShockMesher(nx=16, ny=6)
    mh = ms.make_mesh(cell_type=flavor)
    ng = mh.ngstcell
    vol = np.asarray(mh.clvol.ndarray)[ng:]
    assert (vol > 0).all()
    assert abs(vol.sum() - 4.0) < 1e-12
    if flavor == "quad":
        assert mh.ncell == 16 * 6
    elif flavor == "triangle":
        assert mh.ncell == 2 * 16 * 6
    # At most one boundary face per cell for the triangle flavors.
    fccls = np.asarray(mh.fccls.ndarray)[mh.ngstface:]
    clfcs = np.asarray(mh.clfcs.ndarray)[ng:]
    if flavor != "quad":
        for icl in range(mh.ncell):
            faces = clfcs[icl, 1:clfcs[icl, 0] + 1]
            assert (fccls[faces, 1] < 0).sum() <= 1
    counts = {b.name: b.nbound for b in mh.bcs}
    assert counts == {"left": 6, "top": 16, "bottom": 16, "right": 6}
    assert mh.nbound == 44
    # Deterministic.
    again = ms.make_mesh(cell_type=flavor)
    assert np.array_equal(np.asarray(again.clnds.ndarray),
                          np.asarray(mh.clnds.ndarray))


def test_driver_constants_and_path():
    from solvcon_gb300.obsrefl import ObliqueShock
    d = ObliqueShock()
    with pytest.raises(ValueError):
        d.build_numerical()
    d.build_constant(mach=3.0, angle=10.0)
    z1, z2, z3 = d.zone_states()
    assert z1 == (1.0, d.velocity, 0.0, 1.0)
    assert abs(z2[0] - 1.655) < 2e-3 and abs(z2[3] - 2.054) < 2e-3
    assert z3[3] > z2[3] > z1[3] and z3[2] == 0.0
    assert abs(math.atan2(-z2[2], z2[1]) - math.radians(10.0)) < 1e-12
    with pytest.raises(ValueError):
        d.shock_path()


def _oracle_like(d, steps):
    from oracle import oracle as ora
    mesh = d.mesh
    o = ora.OracleEuler(mesh, d.svr.time_increment)
    o.init_solution(d.gamma, d.density, [d.velocity, 0.0], d.pressure)
    left, top, bottom, right = (mesh.bc(n).facn.ndarray[:, 0]
                                for n in d.mesher.BOUNDARY_NAMES)
    o.add_inlet(left, [d.density, d.velocity, 0.0, d.pressure, d.gamma])
    o.add_inlet(top, [d.density2, d.velocity2[0], d.velocity2[1],
                      d.pressure2, d.gamma])
    o.add_slipwall(bottom)
    o.add_nonrefl(right)
    o.call("bc_soln")
    o.call("bc_dsoln")
    o.march(steps)
    return o


@pytest.mark.gpu
def test_driver_march_matches_oracle():
    from _util import assert_rel
    from solvcon_gb300.obsrefl import ObliqueShock
    d = ObliqueShock()
    d.build_constant(mach=3.0, angle=10.0)
    d.build_numerical(cell_type="unstructured", time_increment=2e-3,
                      nx=32, ny=8)
    d.march(20)
    o = _oracle_like(d, 20)
    # The gradients at the Mach-3 shock pass through the limiter's
    # non-smooth weights, which amplify last-bit differences (FMA
    # contraction on the GPU) far more than in the values: 1e-8 relative for
    # so1n, 1e-10 for the rest.
    for a, tol in (("so0n", 1e-10), ("so1n", 1e-8), ("cflo", 1e-10)):
        assert_rel(getattr(d.svr, a).ndarray, getattr(o, a), tol, a)


@pytest.mark.gpu
def test_driver_reaches_the_analytic_zones():
    """After the flow has crossed the channel several times the computed
    state matches the analytic one inside each zone: zone 1 near the inlet,
    zone 2 under the top boundary behind the incident shock, zone 3 behind
    the reflected shock near the outflow."""
    from solvcon_gb300 import EulerField
    from solvcon_gb300.obsrefl import ObliqueShock
    d = ObliqueShock()
    d.build_constant(mach=3.0, angle=10.0)
    d.build_numerical(cell_type="unstructured", time_increment=2e-3,
                      nx=64, ny=16)
    d.march(3000)
    fld = EulerField(d.svr, d.mesh)
    rho, p = fld.density, fld.pressure
    assert np.isfinite(rho).all()
    xy = fld.centroid
    zones = d.zone_states()
    for (x, y), z, tol in (((0.3, 0.3), zones[0], 0.01),
                           ((2.6, 0.85), zones[1], 0.03),
                           ((3.6, 0.12), zones[2], 0.05)):
        near = np.hypot(xy[:, 0] - x, xy[:, 1] - y) < 0.1
        assert near.sum() >= 3
        assert abs(rho[near].mean() / z[0] - 1) < tol, (x, y)
        assert abs(p[near].mean() / z[3] - 1) < tol, (x, y)


@pytest.mark.parametrize("nx,ny", [(64, 16), (24, 6)])
def test_unstructured_mesh_is_the_references(nx, ny):
    """The unstructured flavor triangulates exactly the reference mesher's
    points into exactly its triangles (fixtures made by running the
    reference's ObliqueShockMesher, _driver.py:127-260): the same scattered
    points bit for bit, the same corner-ear Steiner points, the same
    triangle set.  Only the numbering differs where the reference's follows
    its Bowyer-Watson insertion order: the Steiner points are appended, and
    the cells listed, in another order."""
    from _util import golden
    from solvcon_gb300.obsrefl import ObliqueShockMesher
    g = golden("obsrefl_%dx%d" % (nx, ny))
    m = ObliqueShockMesher(nx=nx, ny=ny)
    pts, tris = m._triangulate(m._scattered_nodes())
    ours = np.asarray(pts, dtype="float64")
    ref = g["points"]
    assert ours.shape == ref.shape
    index = {tuple(p): k for k, p in enumerate(ref.tolist())}
    to_ref = np.array([index[tuple(p)] for p in ours.tolist()])
    assert sorted(to_ref.tolist()) == list(range(len(ref)))

    def canon(t):
        t = list(t)
        k = t.index(min(t))
        return tuple(t[k:] + t[:k])
    mapped = {canon(to_ref[list(t)]) for t in tris}
    assert mapped == {canon(t) for t in g["triangles"].tolist()}
    assert len(tris) == len(g["triangles"])
