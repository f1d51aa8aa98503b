"""FP64 GPU march against the oracle on meshes that span many thread blocks.

The per-operation parity tests use meshes of a few dozen cells; these cases
run the workloads' own generators at sizes where every kernel launch covers
hundreds of blocks and every neighbour gather crosses block boundaries:

* 2D: the unit square, 100 x 100 quads x 2 triangles (20,000 cells), nodes
  jittered by U(-0.2h, 0.2h), a seeded four-quadrant Riemann state, slip
  walls, dt for CFL 0.8 (the plain FP64 workload at 1/100 of its cells);
* 3D: the unit cube, 12^3 hexahedra x 6 tetrahedra (10,368 cells), nodes
  jittered by U(-0.15h, 0.15h), the spherical blast, slip walls, dt for
  CFL 0.7.

Checked, against the oracle (a restatement of the reference march that equals
the compiled reference bit for bit):

1. all 13 arrays of the EulerCore surface after each of the first two
   substeps (euler_march.cpp:339-359), to 1e-12 relative to each array's
   largest magnitude;
2. after 50 full steps: relative L1 (volume weighted) and Linf per conserved
   variable, the mass / momentum / energy totals sum(so0n * clvol) to 1e-12
   relative (a momentum total that cancels is compared against the sum of
   the magnitudes it cancels from), and the W-3/4 limiter firing pattern of
   the last calc_dsoln (fired <=> sigma_max < sigma0/|cflc|,
   euler_gradient.cpp:102-108) as a Hamming fraction over cells x equations.

The FP32 form (FP32 state and flux, FP64 geometry) marches the same two
cases against the same FP64 oracle: relative L1 per conserved variable within
1e-5 after 50 steps (the precision contract's bound), the totals against the
oracle's within 5e-8 (the reference march is not conservative, so FP32
rounding moves its totals; measured 2.3e-9 to 1.8e-8 on the four-quadrant
triangles, 3.5e-10 to 4.9e-9 on the blast), and the firing pattern on
resolved pairs within 5% (an FP32 gradient near the W-3/4 threshold may
decide the other way; measured 3.1% and 0).

The firing bit of an equation in a cell whose state is still uniform is
decided by round-off: the per-element gradients there are noise of order
1e-16, their inverse-magnitude weights scatter by O(1), and the cap binds or
not at random.  The reference itself flips up to 45% of all bits on these cases
when its input is perturbed by 1e-15 relative, and none on (cell, equation)
pairs whose gradient is resolved (|so1n| above 1e-10 of the equation's
largest).  The firing pattern is therefore required to match exactly on the
resolved pairs; the fraction over all pairs is reported.
"""

import numpy as np
import pytest

from _util import assert_rel

pytestmark = pytest.mark.gpu

ARRAYS = ("cevol", "cecnd", "sfcnd", "sfnml", "so0c", "so0n", "so0t", "stm",
          "so1c", "so1n", "cflo", "cflc", "gamma")

CASES = {
    # kind: (ndim, generator args, cfl)
    "tri20k": (2, (100, 0.2, 2026), 0.8),
    "tet10k": (3, (12, 0.15, 2026), 0.7),
}

STEPS = 50
# Gradient magnitude, relative to the equation's largest, above which a
# (cell, equation) pair's limiter decision is not round-off.
RESOLVED = 1e-10


def _setup(kind, precision="fp64"):
    import bench
    from oracle import oracle as ora
    from solvcon_gb300 import meshgen
    nd, args, cfl = CASES[kind]
    gen = meshgen.tri_square if nd == 2 else meshgen.tet_cube
    mesh = meshgen.build_mesh(nd, *gen(*args))
    ng = mesh.ngstcell
    clcnd = np.array(mesh.clcnd.ndarray)[ng:]
    state = meshgen.quadrant_state(clcnd, seed=args[2]) if nd == 2 \
        else meshgen.blast_state(clcnd)
    faces = np.array(mesh.bndfcs.ndarray[:, 0])
    dt = bench.dt_for_cfl(mesh, state, faces, cfl)
    gpu = bench.setup_core(mesh, state, faces, dt, precision)
    ref = ora.OracleEuler(mesh, dt)
    ref.init_solution(1.4, 1.0, [0.0] * nd, 1.0)
    ref.so0n[ng:] = state
    ref.add_slipwall(faces)
    ref.call("bc_soln")
    ref.call("bc_dsoln")
    return mesh, gpu, ref


def march_comparison(gpu, ref, mesh):
    """Relative L1/Linf per variable, totals and limiter Hamming fraction of
    the GPU core's newest state against the oracle's."""
    ng, nd = mesh.ngstcell, mesh.ndim
    neq = nd + 2
    vol = np.array(mesh.clvol.ndarray)[ng:]
    got = np.array(gpu.so0n.ndarray)[ng:]
    want = np.array(ref.so0n)[ng:]
    d = np.abs(got - want)
    l1 = (d * vol[:, None]).sum(0) / (np.abs(want) * vol[:, None]).sum(0)
    linf = d.max(0) / np.abs(want).max(0)
    q = want * vol[:, None]
    tref = q.sum(0)
    scale = np.maximum(np.abs(tref), np.abs(q).sum(0))
    tgot = gpu.totals()
    tot_rel = np.abs(tgot - tref) / scale
    mg = gpu.limiter_mask().astype(np.uint8)
    mo = ref.limiter[:mesh.ncell].astype(np.uint8)
    diff = np.unpackbits((mg ^ mo)[:, None], axis=1,
                         bitorder="little")[:, :neq].astype(bool)
    fired = np.unpackbits(mo[:, None], axis=1, bitorder="little")[:, :neq]
    grad = np.linalg.norm(np.array(ref.so1n)[ng:], axis=2)
    resolved = grad > RESOLVED * grad.max(axis=0)[None, :]
    return {"rel_l1": l1, "rel_linf": linf, "totals_rel": tot_rel,
            "hamming": float(diff.mean()),
            "hamming_resolved": float(diff[resolved].mean())
            if resolved.any() else 0.0,
            "resolved_fraction": float(resolved.mean()),
            "fired_fraction": float(fired.mean())}


@pytest.mark.parametrize("kind", sorted(CASES))
def test_substeps_match_oracle_every_array(kind):
    mesh, gpu, ref = _setup(kind)
    assert mesh.ncell >= 10000
    for sub in range(2):
        gpu.march_substep()
        ref.call("march_substep")
        for a in ARRAYS:
            assert_rel(getattr(gpu, a).ndarray, getattr(ref, a), 1e-12,
                       "%s substep %d %s" % (kind, sub + 1, a))


@pytest.mark.parametrize("kind", sorted(CASES))
def test_march_matches_oracle_at_scale(kind):
    mesh, gpu, ref = _setup(kind)
    gpu.march(STEPS)
    ref.march(STEPS)
    r = march_comparison(gpu, ref, mesh)
    print("%s %d cells, %d steps: rel L1 %s, rel Linf %s, totals %s, "
          "limiter Hamming %.3e on resolved pairs (%.3f of all), %.3e on "
          "all (oracle fired %.3f)" % (
              kind, mesh.ncell, STEPS, r["rel_l1"], r["rel_linf"],
              r["totals_rel"], r["hamming_resolved"], r["resolved_fraction"],
              r["hamming"], r["fired_fraction"]))
    # Measured on GB300: tri 6.4e-13 / 5.9e-10, tet 4.8e-15 / 9.6e-15.
    assert np.all(r["rel_l1"] < 1e-11), r["rel_l1"]
    assert np.all(r["rel_linf"] < 1e-8), r["rel_linf"]
    assert np.all(r["totals_rel"] <= 1e-12), r["totals_rel"]
    # The limiter must actually fire on resolved pairs for the pattern to
    # mean anything.
    assert r["fired_fraction"] > 1e-2 and r["resolved_fraction"] > 0.5
    assert r["hamming_resolved"] == 0.0, r["hamming_resolved"]


@pytest.mark.parametrize("kind", sorted(CASES))
def test_fp32_form_march_against_the_oracle_at_scale(kind):
    mesh, gpu, ref = _setup(kind, "fp32")
    gpu.march(STEPS)
    ref.march(STEPS)
    r = march_comparison(gpu, ref, mesh)
    print("FP32 form, %s %d cells, %d steps: rel L1 %s, rel Linf %s, totals "
          "%s, limiter Hamming %.3e on resolved pairs (%.3f of all), %.3e on "
          "all" % (kind, mesh.ncell, STEPS, r["rel_l1"], r["rel_linf"],
                   r["totals_rel"], r["hamming_resolved"],
                   r["resolved_fraction"], r["hamming"]))
    assert np.all(r["rel_l1"] < 1e-5), r["rel_l1"]
    assert np.all(r["rel_linf"] < 1e-3), r["rel_linf"]
    assert np.all(r["totals_rel"] < 5e-8), r["totals_rel"]
    assert r["hamming_resolved"] < 0.05, r["hamming_resolved"]
