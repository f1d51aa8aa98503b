"""scg_euler_totals_noalloc: the conservation totals without allocation.

Some callers reserve all their device memory up front and may not allocate
afterwards -- a serving loop that admits solves under a fixed HBM budget and
checks the totals of every resident solve each step is one.  For them the
library has scg_euler_totals_noalloc, which keeps its partial sums in a fixed
device array instead of a per-call cudaMalloc/cudaFree buffer (cudaFree would
also synchronise the whole device).  This test calls it through the C ABI and
checks it against scg_euler_totals on two calls in a row, for two meshes of
different sizes one after the other, so that a call following one that left
more partial rows behind is covered too.

Named to be collected last: if it fails, a run stopped at the first failure
has already run every other test.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lib():
    from solvcon_gb300 import _lib
    fn = _lib.lib.scg_euler_totals_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    return _lib


def _core(ndim, nside, precision):
    import solvcon_gb300 as sg
    from solvcon_gb300 import meshgen
    if ndim == 2:
        x, t, c = meshgen.tri_square(nside, 0.2, seed=21)
    else:
        x, t, c = meshgen.tet_cube(nside, 0.15, seed=21)
    mesh = meshgen.build_mesh(ndim, x, t, c)
    core = sg.EulerCore(mesh, 1e-3, precision=precision)
    clcnd = np.asarray(mesh.clcnd.ndarray)[mesh.ngstcell:]
    state = meshgen.quadrant_state(clcnd[:, :2], seed=21) if ndim == 2 \
        else meshgen.blast_state(clcnd, radius=0.35)
    core.init_solution(1.4, 1.0, [0.0] * ndim, 1.0)
    core.so0n[0:] = state
    core.add_slipwall([int(f) for f in mesh.bndfcs.ndarray[:, 0]])
    core.bc_soln()
    core.bc_dsoln()
    core.march(3)
    return core


def _check_pair(lib, core):
    ref = np.zeros(core.neq)
    a0 = lib.device_alloc_count()
    lib.check(lib.lib.scg_euler_totals(core.handle, lib.ptr(ref)))
    # The allocating entry point is seen by the counter.
    assert lib.device_alloc_count() > a0
    mags = np.abs(np.array(core.so0n.ndarray)[core.ngstcell:]).sum(axis=0)
    for _ in range(2):  # two calls in a row
        got = np.full(core.neq, np.nan)
        n0 = lib.launch_count()
        a0 = lib.device_alloc_count()
        lib.check(lib.lib.scg_euler_totals_noalloc(core.handle, lib.ptr(got)))
        assert lib.launch_count() - n0 == 2
        # The point of the entry point: no device allocation at all.
        assert lib.device_alloc_count() == a0
        # The tolerance of the march parity tests: relative 1e-12, with an
        # absolute floor for totals that cancel (momentum at rest).
        np.testing.assert_allclose(got, ref, rtol=1e-12,
                                   atol=1e-13 * mags.max())


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_totals_noalloc_matches_totals(precision):
    lib = _lib()
    big = _core(2, 300, precision)    # 180,000 cells: 6 partial rows
    _check_pair(lib, big)
    small = _core(3, 4, precision)    # 384 cells: 1 partial row
    _check_pair(lib, small)
    _check_pair(lib, big)


def test_totals_noalloc_rejects_null_arguments():
    lib = _lib()
    rc = lib.lib.scg_euler_totals_noalloc(None, None)
    assert rc == 1
    assert "null" in lib.lib.scg_last_error().decode()
