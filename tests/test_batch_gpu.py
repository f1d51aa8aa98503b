"""Batched march: many independent cores in one launch per substep.

Each core's result must be bit-identical to marching it alone (the batch runs
the same per-thread substep with the same arguments), for cores of different
sizes, time steps and gas constants, in FP64 and FP32, in 2D and 3D, with
every block size and grid policy of the autotuner.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cores(ndim, precision, seeds, dt_scale=1.0, mixed=False):
    import solvcon_gb300 as sg
    from solvcon_gb300 import meshgen
    out = []
    for k, seed in enumerate(seeds):
        rng = np.random.default_rng(seed)
        if ndim == 2:
            n = int(rng.integers(4, 24))
            gen = meshgen.quad_square if mixed and k % 2 else \
                meshgen.tri_square
            x, t, c = gen(n, 0.2, seed)
        else:
            n = int(rng.integers(2, 5))
            gen = meshgen.tet_cube if k % 2 == 0 else meshgen.hex_cube
            x, t, c = gen(n, 0.1, seed)
        mesh = meshgen.build_mesh(ndim, x, t, c)
        gamma = float(rng.uniform(1.1, 1.67))
        dt = dt_scale * float(rng.uniform(5e-4, 2e-3))
        core = sg.EulerCore(mesh, dt, precision=precision)
        clcnd = np.array(mesh.clcnd.ndarray)[mesh.ngstcell:]
        state = meshgen.quadrant_state(clcnd[:, :2], seed, gamma) \
            if ndim == 2 else meshgen.blast_state(clcnd, gamma, radius=0.4)
        core.init_solution(gamma, 1.0, [0.0] * ndim, 1.0)
        core.so0n[0:] = state
        faces = [int(f) for f in mesh.bndfcs.ndarray[:, 0]]
        core.add_slipwall(faces[0::2])
        core.add_nonrefl(faces[1::2])
        core.bc_soln()
        core.bc_dsoln()
        out.append((mesh, core))
    return out


@pytest.mark.parametrize("ndim,precision", [(2, "fp64"), (2, "fp32"),
                                            (2, "fp32-geom32"), (3, "fp64"),
                                            (3, "fp32"), (3, "fp32-geom32")])
def test_batch_equals_individual_marches(ndim, precision):
    from solvcon_gb300.batch import EulerBatch
    seeds = [3, 11, 17, 29, 41]
    alone = _cores(ndim, precision, seeds)
    together = _cores(ndim, precision, seeds)
    for _, core in alone:
        core.march(3)
    b = EulerBatch([c for _, c in together], block=128, persistent=True)
    assert b.ncore == len(seeds)
    assert b.ncell == sum(c.ncell for _, c in together)
    b.march(2)
    b.march(1)
    for (_, a), (_, t) in zip(alone, together):
        for name in ("so0c", "so0n", "so0t", "so1c", "so1n", "cflo", "cflc"):
            np.testing.assert_array_equal(getattr(t, name).ndarray,
                                          getattr(a, name).ndarray, name)
    # The cores keep working on their own after a batched march.
    for (_, a), (_, t) in zip(alone, together):
        a.march(1)
        t.march(1)
        np.testing.assert_array_equal(t.so0n.ndarray, a.so0n.ndarray)


@pytest.mark.parametrize("precision", ["fp64", "fp32", "fp32-geom32"])
def test_mixed_2d_batch_equals_individual_marches(precision):
    """Triangle and quadrilateral meshes in one batch: the batch compiles
    the cell code of both types into one kernel, each core alone a
    single-type kernel, and the two still round alike."""
    from solvcon_gb300.batch import EulerBatch
    seeds = [3, 11, 17, 29]
    alone = _cores(2, precision, seeds, mixed=True)
    together = _cores(2, precision, seeds, mixed=True)
    for _, core in alone:
        core.march(3)
    EulerBatch([c for _, c in together], block=128).march(3)
    for (_, a), (_, t) in zip(alone, together):
        for name in ("so0n", "so0t", "so1n", "cflo", "cflc"):
            np.testing.assert_array_equal(getattr(t, name).ndarray,
                                          getattr(a, name).ndarray, name)


def test_autotune_candidates_agree():
    from solvcon_gb300.batch import EulerBatch, autotune
    seeds = [5, 7, 9]
    ref = _cores(2, "fp32", seeds)
    for _, c in ref:
        c.march(3)
    for block in (64, 256):
        for pers in (True, False):
            cores = _cores(2, "fp32", seeds)
            EulerBatch([c for _, c in cores], block=block,
                       persistent=pers).march(3)
            for (_, a), (_, t) in zip(ref, cores):
                np.testing.assert_array_equal(t.so0n.ndarray, a.so0n.ndarray)
    cores = _cores(2, "fp32", seeds)
    best, table = autotune([c for _, c in cores], steps=1, repeat=1)
    assert len(table) == 6 and best["ms_per_step"] > 0
    assert best["ordering"] == "native"
    other = _cores(2, "fp32", seeds)
    best, table = autotune([c for _, c in cores], steps=1, repeat=1,
                           blocks=(64,), persistents=(True,),
                           orderings={"again": [c for _, c in other]})
    assert [r["ordering"] for r in table] == ["native", "again"]
    assert best["ordering"] in ("native", "again")


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_cell_renumbering_leaves_the_march_unchanged(precision):
    """The same mesh with its cells in Morton order marches to the same
    state, cell for cell, to round-off: each cell sums over its faces in its
    own node order, but a shared face belongs to (and its geometry is
    computed from) the lower-numbered of its two cells, so the geometry's
    rounding follows the numbering (measured: 1.4e-14 absolute in FP64
    after 5 steps)."""
    import sys
    import os
    sys.path.insert(0, os.path.dirname(os.path.dirname(
        os.path.abspath(__file__))))
    import bench
    from solvcon_gb300.batch import EulerBatch
    got = {}
    for order in ("native", "morton"):
        m, s, f, g = bench.batch_mesh(5, 3000, 1.4, 2026, order)
        dt = bench.dt_for_cfl_g(m, s, 0.8, g)
        c = bench.setup_core_g(m, s, f, dt, precision, g)
        EulerBatch([c], block=64).march(5)
        cl = np.array(m.clnds.ndarray)[m.ngstcell:, :4]
        got[order] = (cl, np.array(c.so0n.ndarray)[c.ngstcell:],
                      np.array(c.so1n.ndarray)[c.ngstcell:])
    key = {tuple(r): i for i, r in enumerate(got["native"][0].tolist())}
    perm = np.array([key[tuple(r)] for r in got["morton"][0].tolist()])
    tol = 1e-12 if precision == "fp64" else 2e-5
    for k in (1, 2):
        want = got["native"][k][perm]
        np.testing.assert_allclose(got["morton"][k], want, rtol=0,
                                   atol=tol * np.abs(want).max())


def test_batch_rejects_mixed_cores():
    from solvcon_gb300.batch import EulerBatch
    a = _cores(2, "fp64", [1])
    b = _cores(2, "fp32", [2])
    with pytest.raises(ValueError):
        EulerBatch([a[0][1], b[0][1]])
    with pytest.raises(ValueError):
        EulerBatch([a[0][1]], block=100)


def test_retarget_keeps_results_exact():
    """A batch pointed at another set of cores marches them exactly as
    marching each alone; a set that needs another kernel is refused."""
    from solvcon_gb300.batch import EulerBatch
    seeds = [3, 11, 17, 29]
    alone = _cores(2, "fp32", seeds)
    together = _cores(2, "fp32", seeds)
    for _, c in alone[:3]:
        c.march(2)
    for _, c in alone[1:]:
        c.march(3)
    b = EulerBatch([c for _, c in together[:3]], block=64)
    b.march(2)
    assert b.retarget([c for _, c in together[1:]])
    assert b.ncore == 3
    assert b.ncell == sum(c.ncell for _, c in together[1:])
    b.march(3)
    for (_, a), (_, t) in zip(alone, together):
        np.testing.assert_array_equal(t.so0n.ndarray, a.so0n.ndarray)
        np.testing.assert_array_equal(t.so1n.ndarray, a.so1n.ndarray)
    other = _cores(2, "fp64", [5])
    assert not b.retarget([other[0][1]])
    assert b.ncore == 3


def test_retarget_through_growing_and_shrinking_sets():
    """Member sets that grow past the work list's capacity (its device table
    is reallocated and the step graph captured again) and shrink back (the
    graph's nodes updated in place), each marched right after the retarget:
    every core still equals its march alone."""
    from solvcon_gb300.batch import EulerBatch
    seeds = [3, 11, 17, 29, 31, 37]
    alone = _cores(2, "fp32", seeds)
    together = _cores(2, "fp32", seeds)
    plan = [([0], 2), ([0, 1, 2], 3), ([1, 2, 3, 4, 5], 2), ([2], 4),
            ([0, 1, 2, 3, 4, 5], 1), ([3, 4], 3), ([5, 0, 1, 2, 3, 4], 2)]
    b = None
    for members, steps in plan:
        for k in members:
            alone[k][1].march(steps)
        cores = [together[k][1] for k in members]
        if b is None:
            b = EulerBatch(cores, block=64)
        else:
            assert b.retarget(cores)
        assert b.ncore == len(members)
        b.march(steps)
    for (_, a), (_, t) in zip(alone, together):
        np.testing.assert_array_equal(t.so0n.ndarray, a.so0n.ndarray)
        np.testing.assert_array_equal(t.so1n.ndarray, a.so1n.ndarray)
