"""1D Euler: the exact shock-tube solution (CPU) and the GPU Euler1DCore.

Known answers are those of the reference's tests/test_onedim_euler.py
(shock strength, zone states, wave locations); the GPU core is compared with
the oracle and with the reference's own Sod output (tests/golden/e1d_sod.npz),
and its fine-grained and one-call marches must agree bit for bit, as the
reference's test_march_fine_interface requires.
"""

import numpy as np
import pytest

from _util import assert_rel, golden


def _tube():
    from solvcon_gb300.onedim import ShockTube
    st = ShockTube()
    st.build_constant(gamma=1.4, pressure1=1.0, density1=1.0, pressure5=0.1,
                      density5=0.125)
    return st


def test_shock_tube_constants():
    st = _tube()
    np.testing.assert_allclose(st.calc_pressure45(), 3.0313017805064697,
                               rtol=1e-7)
    np.testing.assert_allclose(
        [st.density1, st.density3, st.density4, st.density5],
        [1.0, 0.42631942817849494, 0.2655737117053072, 0.125], rtol=1e-7)
    assert st.pressure3 == st.pressure4
    np.testing.assert_allclose(
        [st.pressure1, st.pressure3, st.pressure4, st.pressure5],
        [1.0, 0.303130178050647, 0.303130178050647, 0.1], rtol=1e-7)
    np.testing.assert_allclose(
        [st.velocity1, st.velocity3, st.velocity4, st.velocity5],
        [0.0, 0.9274526200489503, 0.9274526200489503, 0.0], rtol=1e-7)
    np.testing.assert_allclose(
        st.calc_locations(t=0.1),
        [-0.11832159566199232, -0.007027281256118345, 0.09274526200489504,
         0.17521557320301784], rtol=1e-7)
    assert st.speedofsound1 == np.sqrt(st.gamma)


def test_shock_tube_field_at_t0():
    st = _tube()
    st.build_field(t=0.0, coord=np.linspace(-1, 1, num=11))
    assert st.svr is None and len(st.coord_field) == 11
    np.testing.assert_equal(0, st.velocity_field)
    left = st.coord_field < 0
    np.testing.assert_equal(st.pressure1, st.pressure_field[left])
    np.testing.assert_equal(st.pressure5, st.pressure_field[~left])
    np.testing.assert_equal(st.density1, st.density_field[left])
    np.testing.assert_equal(st.density5, st.density_field[~left])


@pytest.mark.gpu
def test_core_arrays_and_errors():
    from solvcon_gb300.onedim import Euler1DCore, Euler1DSolver
    svr = Euler1DSolver(xmin=0.0, xmax=2 * np.pi, ncoord=9,
                        time_increment=0.1)
    assert svr.nvar == 3 and svr.ncoord == 9
    assert svr.coord.shape == (9,) and svr.so0.shape == (9, 3)
    np.testing.assert_allclose(svr.coord.ndarray, np.linspace(0, 2 * np.pi, 9))
    with pytest.raises(ValueError):
        Euler1DCore(ncoord=10, time_increment=0.1)
    c = svr.clone()
    np.testing.assert_array_equal(c.coord.ndarray, svr.coord.ndarray)


@pytest.mark.gpu
def test_fine_interface_equals_march_alpha2():
    from solvcon_gb300.onedim import ShockTube
    a, b = _tube(), _tube()
    a.build_numerical(-1, 1, 41, time_increment=0.01)
    b.build_numerical(-1, 1, 41, time_increment=0.01)
    s = a.svr
    for _ in range(15):
        s.march_half_so0(odd_plane=False)
        s.treat_boundary_so0()
        s.update_cfl(odd_plane=True)
        s.march_half_so1_alpha2(odd_plane=False)
        s.treat_boundary_so1()
        s.march_half_so0(odd_plane=True)
        s.update_cfl(odd_plane=False)
        s.march_half_so1_alpha2(odd_plane=True)
        b.svr.march_alpha2(steps=1)
        assert s.so0.tolist() == b.svr.so0.tolist()
    del ShockTube


def _gpu_sod(n, steps, alpha=2, precision="fp64", stretched=False):
    from solvcon_gb300.onedim import Euler1DCore
    g = golden("e1d_sod") if n == 201 and not stretched else None
    x = np.linspace(-1, 1, n)
    if stretched:  # finest at the diaphragm, 4x coarser at the ends
        x = np.sinh(2.0947 * x) / np.sinh(2.0947)
    dt = float(g["dt"]) if g is not None else \
        2 * 0.8 * float(np.diff(x).min()) / 2.19
    c = Euler1DCore(n, dt, precision=precision)
    so0 = np.zeros((n, 3))
    left = x < 0.0
    so0[:, 0] = np.where(left, 1.0, 0.125)
    so0[:, 2] = np.where(left, 1.0 / 0.4, 0.1 / 0.4)
    c.coord[...] = x
    c.so0[...] = so0
    c.so1.fill(0)
    c.gamma.fill(1.4)
    c.cfl.fill(0)
    c.setup_march()
    getattr(c, "march_alpha%d" % alpha)(steps)
    return c, x, so0, dt


@pytest.mark.gpu
def test_sod_matches_reference_golden_and_oracle():
    from oracle import oracle as ora
    g = golden("e1d_sod")
    c, x, so0, dt = _gpu_sod(201, int(g["steps"]))
    for a in ("so0", "so1", "cfl"):
        assert_rel(getattr(c, a).ndarray, g[a], 1e-12, a)
    for alpha in (1, 2):
        c, x, so0, dt = _gpu_sod(1001, 70, alpha)
        o = ora.OracleEuler1D(1001, dt)
        o.coord[:] = x
        o.so0[:] = so0
        o.setup_march()
        o.march_alpha(alpha, 70)
        for a in ("so0", "so1", "cfl"):
            assert_rel(getattr(c, a).ndarray, getattr(o, a), 1e-11,
                       "alpha%d %s" % (alpha, a))


@pytest.mark.gpu
def test_sod_accuracy_against_exact_solution():
    """Sod tube at t = 0.2 on 201 points, CFL 0.8 (the 1D configuration):
    the density's mean absolute error against the exact solution."""
    g = golden("e1d_sod")
    c, x, so0, dt = _gpu_sod(201, int(g["steps"]))
    st = _tube()
    t = dt * int(g["steps"])
    st.build_field(t=t, coord=x[2:-2:2])
    rho = np.array(c.so0.ndarray)[2:-2:2, 0]
    l1 = np.abs(rho - st.density_field).mean()
    assert l1 < 8e-3, l1


@pytest.mark.gpu
def test_long_tube_graph_path_matches_oracle():
    """100,001 points, 70 steps: the march replays captured CUDA graphs."""
    from oracle import oracle as ora
    c, x, so0, dt = _gpu_sod(100001, 70)
    o = ora.OracleEuler1D(100001, dt)
    o.coord[:] = x
    o.so0[:] = so0
    o.setup_march()
    o.march_alpha(2, 70)
    assert_rel(c.so0.ndarray, o.so0, 1e-11, "so0")
    assert_rel(c.so1.ndarray, o.so1, 1e-10, "so1")


@pytest.mark.gpu
@pytest.mark.parametrize("n,steps", [(201, None), (10001, 700)])
def test_fp32_tube_against_fp64(n, steps):
    """FP32 state (not in the reference) against the FP64 march on the same
    Sod tube: relative L1 per variable <= 1e-5 (201 points to t = 0.2, and
    10,001 points for 700 steps through the graph path); the FP32 core
    reports its precision, keeps it through clone() and rounds a host write
    to FP32."""
    g = golden("e1d_sod")
    steps = int(g["steps"]) if steps is None else steps
    c32, x, so0, dt = _gpu_sod(n, steps, precision="fp32")
    c64, _, _, _ = _gpu_sod(n, steps)
    assert c32.precision == "fp32" and c64.precision == "fp64"
    a = np.array(c32.so0.ndarray)
    b = np.array(c64.so0.ndarray)
    for k in range(3):
        l1 = np.abs(a[:, k] - b[:, k]).sum() / np.abs(b[:, k]).sum()
        assert l1 < 1e-5, (k, l1)
    twin = c32.clone()
    assert twin.precision == "fp32"
    np.testing.assert_array_equal(twin.so0.ndarray, c32.so0.ndarray)
    twin.so0[...] = so0 * (1 + 1e-12)
    twin.update_cfl(odd_plane=False)  # pushes so0, reads it, keeps it
    np.testing.assert_array_equal(np.array(twin.so0[...]),
                                  (so0 * (1 + 1e-12)).astype("float32"))


@pytest.mark.gpu
def test_fp32_tube_stretched_grid_and_clone():
    """FP32 state on a non-uniform grid (the spacing tables are formed from
    the coordinates written after construction) against FP64: relative L1
    per variable <= 1e-5; a clone carries the spacing and marches on to the
    same bits as the original."""
    c32, x, so0, dt = _gpu_sod(2001, 300, precision="fp32", stretched=True)
    c64, _, _, _ = _gpu_sod(2001, 300, stretched=True)
    a = np.array(c32.so0.ndarray)
    b = np.array(c64.so0.ndarray)
    for k in range(3):
        l1 = np.abs(a[:, k] - b[:, k]).sum() / np.abs(b[:, k]).sum()
        assert l1 < 1e-5, (k, l1)
    twin = c32.clone()
    c32.march_alpha2(20)
    twin.march_alpha2(20)
    for name in ("so0", "so1", "cfl"):
        np.testing.assert_array_equal(np.array(getattr(twin, name).ndarray),
                                      np.array(getattr(c32, name).ndarray),
                                      err_msg=name)
    # A coordinate write rebuilds the spacing: a uniform grid written into
    # the stretched core marches as a core built uniform from the start.
    u32, xu, so0u, dtu = _gpu_sod(2001, 0, precision="fp32")
    re = c32.clone()
    re.coord[...] = xu
    re.so0[...] = so0u
    re.so1.fill(0)
    re.cfl.fill(0)
    re.setup_march()
    from solvcon_gb300.onedim import Euler1DCore
    fresh = Euler1DCore(2001, c32.time_increment, precision="fp32")
    fresh.coord[...] = xu
    fresh.so0[...] = so0u
    fresh.so1.fill(0)
    fresh.gamma.fill(1.4)
    fresh.cfl.fill(0)
    fresh.setup_march()
    re.march_alpha2(50)
    fresh.march_alpha2(50)
    np.testing.assert_array_equal(np.array(re.so0.ndarray),
                                  np.array(fresh.so0.ndarray))


def test_tube_precision_must_be_known():
    from solvcon_gb300.onedim import Euler1DCore
    with pytest.raises(ValueError):
        Euler1DCore(11, 0.1, precision="fp16")
