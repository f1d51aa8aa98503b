"""EulerField: body-cell fields derived on the device.

Each field must equal the reference EulerField's numpy formula
(solvcon/multidim/euler/_field.py:80-148) applied to the host copy of the
same state, to FP64 round-off; the overall mass and CFL range come from
device reductions and must match the numpy sums.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(ndim, precision):
    import solvcon_gb300 as sg
    from solvcon_gb300 import meshgen
    if ndim == 2:
        x, t, c = meshgen.tri_square(20, 0.2, 5)
    else:
        x, t, c = meshgen.tet_cube(5, 0.1, 5)
    mesh = meshgen.build_mesh(ndim, x, t, c)
    clcnd = np.array(mesh.clcnd.ndarray)[mesh.ngstcell:]
    state = meshgen.quadrant_state(clcnd[:, :2], 5, 1.3) if ndim == 2 \
        else meshgen.blast_state(clcnd, 1.3)
    core = sg.EulerCore(mesh, 2e-4, precision=precision)
    core.init_solution(1.3, 1.0, [0.0] * ndim, 1.0)
    core.so0n[0:] = state
    core.add_slipwall(np.array(mesh.bndfcs.ndarray[:, 0]))
    core.bc_soln()
    core.bc_dsoln()
    core.march(4)
    return mesh, core


def _reference_fields(cons, gamma, cflo, ndim):
    # The reference EulerField's formulas, in numpy.
    rho = cons[:, 0]
    vel = cons[:, 1:1 + ndim] / rho[:, None]
    speed = np.sqrt((vel ** 2).sum(axis=1))
    energy = cons[:, 1 + ndim]
    pressure = (gamma - 1.0) * (energy - 0.5 * rho * speed ** 2)
    out = {"density": rho, "velx": vel[:, 0], "vely": vel[:, 1],
           "speed": speed, "pressure": pressure,
           "mach": speed / np.sqrt(gamma * pressure / rho),
           "total_energy": energy, "cfl": cflo}
    if ndim == 3:
        out["velz"] = vel[:, 2]
    return out


@pytest.mark.parametrize("ndim,precision", [(2, "fp64"), (3, "fp64"),
                                            (2, "fp32")])
def test_fields_match_reference_formulas(ndim, precision):
    from solvcon_gb300 import EulerField
    mesh, core = _run(ndim, precision)
    ng = core.ngstcell
    cons = np.array(core.so0n[...], dtype="float64")[ng:]
    gamma = np.array(core.gamma[...], dtype="float64")[ng:]
    cflo = np.array(core.cflo[...], dtype="float64")[ng:]
    want = _reference_fields(cons, gamma, cflo, ndim)
    fld = EulerField(core, mesh)
    for name in EulerField.FIELDS:
        got = fld.field(name)
        assert got.shape == (mesh.ncell,)
        np.testing.assert_allclose(got, want[name], rtol=1e-13, atol=1e-15,
                                   err_msg=name)
    vel = fld.vel
    assert vel.shape == (mesh.ncell, ndim)
    if ndim == 3:
        np.testing.assert_allclose(vel[:, 2], want["velz"], rtol=1e-13,
                                   atol=1e-15)
    vol = np.array(mesh.clvol.ndarray)[mesh.ngstcell:]
    mass = float(np.sum(cons[:, 0] * vol))
    assert abs(fld.calc_overall_mass() - mass) <= 1e-13 * abs(mass)
    lo, hi = fld.calc_cfl_range()
    assert lo == cflo.min() and hi == cflo.max()
    assert fld.conserveds[0] == "density" and len(fld.conserveds) == ndim + 2
    np.testing.assert_array_equal(fld.conserved, cons if precision == "fp64"
                                  else fld.conserved)


def test_field_errors():
    from solvcon_gb300 import EulerField
    mesh, core = _run(2, "fp64")
    fld = EulerField(core, mesh)
    with pytest.raises(ValueError):
        fld.field("vorticity")
    with pytest.raises(ValueError):
        core.device_field("velz")
