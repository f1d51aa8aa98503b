"""Spacetime scalar solvers (linear scalar, inviscid Burgers) on the GPU.

Known answers of the reference's tests/test_spacetime_linear_scalar.py and
test_spacetime_inviscid_burgers.py: sin(x) advected ten periods at CFL 1
returns to 1e-14 with CFL identically 1, the fine-grained and one-call
marches agree bit for bit, Burgers stays within [-1, 1]; plus parity with the
oracle on a long grid (which exercises the CUDA-graph replay).
"""

import numpy as np
import pytest

from _util import assert_rel


def test_grid_layout():
    from solvcon_gb300.spacetime import Grid
    g = Grid(0.0, 1.0, 4)
    assert (g.ncelm, g.nselm, g.xsize) == (4, 5, 13)
    np.testing.assert_allclose(g.xcoord[2:11:2], [0, 0.25, 0.5, 0.75, 1.0])
    np.testing.assert_allclose(g.xcoord[3:10:2], [0.125, 0.375, 0.625, 0.875])
    np.testing.assert_allclose(g.xcoord[:2], [-0.25, -0.125])
    with pytest.raises(ValueError):
        Grid(1.0, 0.0, 4)
    with pytest.raises(ValueError):
        Grid(0.0, 1.0, 0)
    with pytest.raises(ValueError):
        Grid(np.array([0.0, 0.5, 0.2]))


def _build(cls, resolution):
    from solvcon_gb300 import spacetime as st
    xcrd = np.arange(resolution + 1) / resolution * 2 * np.pi
    grid = st.Grid(xcrd)
    dx = (grid.xmax - grid.xmin) / grid.ncelm
    nstep = int(np.ceil(2 * np.pi / dx))
    dt = 2 * np.pi / nstep
    svr = getattr(st, cls)(grid=grid, time_increment=dt)
    svr.set_so0(0, np.sin(xcrd))
    svr.set_so1(0, np.cos(xcrd))
    svr.setup_march()
    return nstep, xcrd, svr


@pytest.mark.gpu
def test_linear_scalar_returns_after_ten_periods():
    nstep, xcrd, svr = _build("LinearScalarSolver", 8)
    assert svr.nvar == 1
    assert svr.xctr().tolist() == xcrd.tolist()
    assert len(svr.xctr(odd_plane=True)) == svr.grid.ncelm
    assert svr.get_so0(0).ndarray.tolist() == np.sin(xcrd).tolist()
    with pytest.raises(IndexError, match="out of nvar range"):
        svr.get_so0(1)
    svr.march_alpha2(nstep * 10)
    np.testing.assert_allclose(svr.get_so0(0), np.sin(xcrd), rtol=0,
                               atol=1e-14)
    np.testing.assert_allclose(svr.get_cfl(), np.ones(svr.grid.nselm),
                               rtol=0, atol=1e-14)
    v1 = [e.get_so0(0) for e in svr.selms(odd_plane=True)]
    assert v1 == svr.get_so0(0, odd_plane=True).ndarray.tolist()


@pytest.mark.gpu
def test_fine_interface_equals_march_alpha2():
    nstep, xcrd, a = _build("LinearScalarSolver", 8)
    _, _, b = _build("LinearScalarSolver", 8)
    for _ in range(nstep * 3):
        a.march_half_so0(odd_plane=False)
        a.treat_boundary_so0()
        a.update_cfl(odd_plane=True)
        a.march_half_so1_alpha2(odd_plane=False)
        a.treat_boundary_so1()
        a.march_half_so0(odd_plane=True)
        a.update_cfl(odd_plane=False)
        a.march_half_so1_alpha2(odd_plane=True)
        b.march_alpha2(steps=1)
        assert a.get_so0(0).ndarray.tolist() == b.get_so0(0).ndarray.tolist()


@pytest.mark.gpu
def test_burgers_bounded():
    nstep, xcrd, svr = _build("InviscidBurgersSolver", 8)
    for _ in range(nstep * 2):
        res = svr.get_so0(0).ndarray
        assert res.max() <= 1 and res.min() >= -1
        svr.march_alpha2(1)


@pytest.mark.gpu
@pytest.mark.parametrize("cls,kind", [("LinearScalarSolver", 0),
                                      ("InviscidBurgersSolver", 1)])
@pytest.mark.parametrize("alpha", [1, 2])
def test_matches_oracle(cls, kind, alpha):
    from oracle import oracle as ora
    nstep, xcrd, svr = _build(cls, 4000)
    ref = ora.OracleSpacetime(kind, svr.grid.xcoord, svr.time_increment)
    ref.so0[:] = svr.so0.ndarray[:, 0]
    ref.so1[:] = svr.so1.ndarray[:, 0]
    ref.setup_march()
    svr.march_alpha1(70) if alpha == 1 else svr.march_alpha2(70)
    ref.march_alpha(alpha, 70)
    assert_rel(svr.so0.ndarray[:, 0], ref.so0, 1e-12, "so0")
    assert_rel(svr.so1.ndarray[:, 0], ref.so1, 1e-10, "so1")
    assert_rel(svr.cfl.ndarray, ref.cfl, 1e-12, "cfl")


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["linear_a1", "linear_a2", "burgers_a1",
                                  "burgers_a2"])
def test_matches_reference_golden(case):
    """The GPU solvers against the reference's own output on a non-uniform
    grid (fixtures made by running the reference): a linear-scalar wave, and
    a Burgers state that has steepened into a shock."""
    from _util import golden
    from solvcon_gb300 import spacetime as st
    g = golden("st_" + case)
    grid = st.Grid(g["xloc"])
    np.testing.assert_array_equal(grid.xcoord, g["xcoord"])
    cls = (st.LinearScalarSolver, st.InviscidBurgersSolver)[int(g["kind"])]
    svr = cls(grid=grid, time_increment=float(g["dt"]))
    svr.so0.ndarray[:, 0] = g["so0_in"]
    svr.so1.ndarray[:, 0] = g["so1_in"]
    svr.setup_march()
    if int(g["alpha"]) == 1:
        svr.march_alpha1(int(g["steps"]))
    else:
        svr.march_alpha2(int(g["steps"]))
    assert_rel(svr.so0.ndarray[:, 0], g["so0"], 1e-12, "so0")
    assert_rel(svr.so1.ndarray[:, 0], g["so1"], 1e-10, "so1")
    assert_rel(svr.cfl.ndarray, g["cfl"], 1e-12, "cfl")


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["linear_a1", "linear_a2", "burgers_a1",
                                  "burgers_a2"])
def test_reference_golden_bit_for_bit(case):
    """Compiled without contraction, the GPU half steps (their grid
    quotients formed from tabulated reciprocals) reproduce the reference's
    marches bit for bit."""
    from _util import golden
    from solvcon_gb300 import spacetime as st
    g = golden("st_" + case)
    grid = st.Grid(g["xloc"])
    cls = (st.LinearScalarSolver, st.InviscidBurgersSolver)[int(g["kind"])]
    svr = cls(grid=grid, time_increment=float(g["dt"]))
    svr.so0.ndarray[:, 0] = g["so0_in"]
    svr.so1.ndarray[:, 0] = g["so1_in"]
    svr.setup_march()
    if int(g["alpha"]) == 1:
        svr.march_alpha1(int(g["steps"]))
    else:
        svr.march_alpha2(int(g["steps"]))
    for name, got in (("so0", svr.so0.ndarray[:, 0]),
                      ("so1", svr.so1.ndarray[:, 0]), ("cfl", svr.cfl.ndarray)):
        want = np.asarray(g[name]).reshape(np.shape(got))
        assert (np.asarray(got).view(np.uint64) ==
                want.view(np.uint64)).all(), name
