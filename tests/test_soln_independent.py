"""calc_soln against an independent restatement of the CESE flux integral.

The reference's tests pin calc_soln with a NumPy re-implementation that takes
the Euler flux Jacobian by finite differences (tests/test_multidim.py:52-94,
:710-738).  Here the integral is restated once more with the Jacobian taken
by the complex-step derivative, J[:, j] = Im f(u + i h e_j) / h, which is
exact to round-off (no truncation error, no cancellation), so the comparison
holds to 1e-12 relative.  The state is non-uniform, with non-zero so0t and
so1c and ghost rows that differ from their interior cells, so the spatial
Taylor terms, the temporal flux and the Jacobian products all contribute.
On the CPU it checks the oracle's calc_soln; on the GPU (``-m gpu``) the
device kernel's, each with its own CE tables.
"""

import numpy as np
import pytest

from _util import FIXTURES, fixture_mesh

GAMMA = 1.4


def euler_flux(u, gamma):
    """f[i, d] of one conserved row (real or complex)."""
    nd = u.size - 2
    rho, mom, en = u[0], u[1:1 + nd], u[nd + 1]
    vel = mom / rho
    ke = sum(mom[k] * vel[k] for k in range(nd)) * 0.5
    p = (gamma - 1.0) * (en - ke)
    f = np.zeros((u.size, nd), dtype=np.result_type(u, 1.0))
    for d in range(nd):
        f[0, d] = mom[d]
        for k in range(nd):
            f[1 + k, d] = mom[k] * vel[d] + (p if k == d else 0.0)
        f[nd + 1, d] = (en + p) * vel[d]
    return f


def jacobian_cs(u, gamma, h=1e-30):
    """J[i, j, d] = d f[i, d] / d u[j] by the complex-step derivative."""
    neq = u.size
    jac = np.zeros((neq, neq, neq - 2))
    for j in range(neq):
        z = u.astype(complex)
        z[j] += 1j * h
        jac[:, j, :] = euler_flux(z, gamma).imag / h
    return jac


def soln_reference(mesh, tab, dt):
    """so0n of every interior cell.  ``tab`` holds whole buffers, ghost rows
    first: cevol, cecnd, sfcnd, sfnml (interior rows only), so0c, so0t,
    so1c."""
    nd, ng, ncell = mesh.ndim, int(mesh.ngstcell), int(mesh.ncell)
    neq = nd + 2
    qdt, hdt = 0.25 * dt, 0.5 * dt
    clfcs = np.asarray(mesh.clfcs.ndarray)
    fccls = np.asarray(mesh.fccls.ndarray)
    fcnds = np.asarray(mesh.fcnds.ndarray)
    clcnd = np.asarray(mesh.clcnd.ndarray)
    ngf = int(mesh.ngstface)
    nsub = tab["sfcnd"].shape[1] // (clfcs.shape[1] - 1)
    out = np.zeros((ncell, neq))
    for icl in range(ncell):
        r = ng + icl
        acc = np.zeros(neq)
        for ifl in range(1, clfcs[r, 0] + 1):
            ifc = clfcs[r, ifl]
            jcl = fccls[ngf + ifc, 0] + fccls[ngf + ifc, 1] - icl
            jr = ng + jcl
            jce = tab["cecnd"][jr, :nd] if jcl >= 0 else clcnd[jr, :nd]
            bce = tab["cecnd"][r, ifl * nd:(ifl + 1) * nd]
            u, ut, g = tab["so0c"][jr], tab["so0t"][jr], tab["so1c"][jr]
            acc += (u + g @ (bce - jce)) * tab["cevol"][r, ifl]
            f = euler_flux(u, GAMMA)
            jac = jacobian_cs(u, GAMMA)
            for inf in range(fcnds[ngf + ifc, 0]):
                k = (ifl - 1) * nsub + inf
                sc, sn = tab["sfcnd"][icl, k], tab["sfnml"][icl, k]
                us = qdt * ut + g @ (sc - jce)
                acc -= hdt * ((f + np.einsum("ijd,j->id", jac, us)) @ sn)
        out[icl] = acc / tab["cevol"][r, 0]
    return out


def _state(mesh, cecnd):
    """A smooth non-uniform state, so0t and so1c on every row; ghost rows get
    values of their own (not copies of the interior)."""
    nd, ng = mesh.ndim, int(mesh.ngstcell)
    neq = nd + 2
    pts = np.array(np.asarray(cecnd)[:, :nd])
    pts[:ng] = np.asarray(mesh.clcnd.ndarray)[:ng, :nd]
    x = pts[:, 0]
    y = pts[:, 1]
    rho = 1.1 + 0.2 * x - 0.1 * y
    vel = np.stack([0.3 + 0.1 * y, -0.2 + 0.15 * x, 0.05 + 0.0 * x][:nd],
                   axis=1)
    p = 0.9 + 0.3 * x * y
    so0 = np.empty((len(x), neq))
    so0[:, 0] = rho
    so0[:, 1:1 + nd] = rho[:, None] * vel
    so0[:, -1] = p / (GAMMA - 1.0) + 0.5 * rho * (vel * vel).sum(axis=1)
    so0[:ng] *= 1.03  # ghosts differ from what the interior would give
    so0t = np.stack([0.3 * (k + 1) * (1 + x) for k in range(neq)], axis=1)
    so1 = np.stack([np.stack([0.02 * (k + 1) * (d + 1) + 0.01 * y
                              for d in range(nd)], axis=1)
                    for k in range(neq)], axis=1)
    return so0, so0t, so1


MESHES = sorted(FIXTURES)


@pytest.mark.parametrize("name", MESHES)
def test_oracle_calc_soln_matches_complex_step_restatement(name):
    from oracle import oracle as ora
    mesh = fixture_mesh(name)
    dt = 0.05
    o = ora.OracleEuler(mesh, dt)
    so0, so0t, so1 = _state(mesh, o.cecnd)
    o.gamma[:] = GAMMA
    o.so0c[:] = so0
    o.so0t[:] = so0t
    o.so1c[:] = so1
    o.call("calc_soln")
    tab = {k: np.array(getattr(o, k)) for k in
           ("cevol", "cecnd", "sfcnd", "sfnml", "so0c", "so0t", "so1c")}
    want = soln_reference(mesh, tab, dt)
    got = np.array(o.so0n)[o.ngstcell:]
    np.testing.assert_allclose(got, want, rtol=0,
                               atol=1e-12 * np.abs(want).max())


@pytest.mark.gpu
@pytest.mark.parametrize("name", MESHES)
def test_calc_soln_matches_complex_step_restatement(name):
    import solvcon_gb300 as sg
    mesh = fixture_mesh(name)
    dt = 0.05
    ec = sg.EulerCore(mesh=mesh, time_increment=dt, precision="fp64")
    so0, so0t, so1 = _state(mesh, ec.cecnd)
    ec.gamma.ndarray[...] = GAMMA
    ec.so0c.ndarray[...] = so0
    ec.so0t.ndarray[...] = so0t
    ec.so1c.ndarray[...] = so1
    ec.calc_soln()
    tab = {k: np.array(getattr(ec, k).ndarray) for k in
           ("cevol", "cecnd", "sfcnd", "sfnml", "so0c", "so0t", "so1c")}
    want = soln_reference(mesh, tab, dt)
    got = np.array(ec.so0n.ndarray)[ec.ngstcell:]
    np.testing.assert_allclose(got, want, rtol=0,
                               atol=1e-12 * np.abs(want).max())
