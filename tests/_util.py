"""Helpers shared by the tests: fixture meshes, golden files, comparisons."""

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as f:
        return {k: f[k] for k in f.files}


# Hand-built fixture meshes in the style of the reference's tests
# (tests/test_multidim.py:152-281): name -> (ndim, nodes, types, cell lists).
FIXTURES = {
    "tri3": (2, [(0, 0), (-1, -1), (1, -1), (0, 1)], [4, 4, 4],
             [(3, 0, 1, 2), (3, 0, 2, 3), (3, 0, 3, 1)]),
    "quad1": (2, [(0, 0), (1, 0), (1, 1), (0, 1)], [3], [(4, 0, 1, 2, 3)]),
    "mixed": (2, [(0, 0), (1, 0), (2, 0), (0, 1), (1, 1), (2, 1)], [3, 4, 4],
              [(4, 0, 1, 4, 3), (3, 1, 2, 4, 0), (3, 2, 5, 4, 0)]),
    "tet1": (3, [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)], [6],
             [(4, 0, 1, 2, 3)]),
    "hex1": (3, [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1),
                 (1, 0, 1), (1, 1, 1), (0, 1, 1)], [5],
             [(8, 0, 1, 2, 3, 4, 5, 6, 7)]),
    "prism1": (3, [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1),
                   (0, 1, 1)], [7], [(6, 0, 1, 2, 3, 4, 5)]),
    "pyr1": (3, [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0.5, 0.5, 1)],
             [8], [(5, 0, 1, 2, 3, 4)]),
}


def fixture_mesh(name):
    from solvcon_gb300 import meshgen
    nd, x, t, c = FIXTURES[name]
    return meshgen.build_mesh(nd, np.asarray(x, dtype="float64"), t,
                              np.asarray(c))


def quad_channel(nx, ny, lx, ly):
    """Structured nx x ny quadrilateral channel over [0, lx] x [0, ly]."""
    from solvcon_gb300 import meshgen
    xs = np.linspace(0.0, lx, nx + 1)
    ys = np.linspace(0.0, ly, ny + 1)
    gx, gy = np.meshgrid(xs, ys, indexing="xy")
    nd = np.stack([gx.ravel(), gy.ravel()], axis=1)
    cl = []
    for j in range(ny):
        for i in range(nx):
            a = j * (nx + 1) + i
            cl.append((4, a, a + 1, a + nx + 2, a + nx + 1))
    return meshgen.build_mesh(2, nd, [3] * len(cl), np.asarray(cl))


def relerr(a, b):
    a = np.asarray(a, dtype="float64")
    b = np.asarray(b, dtype="float64")
    scale = max(float(np.abs(b).max()) if b.size else 0.0, 1e-300)
    return float(np.abs(a - b).max()) / scale if b.size else 0.0


def assert_rel(a, b, tol, what="", atol=1e-13):
    """max|a - b| <= tol * max|b| + atol.  The absolute floor matters only
    for arrays that are round-off noise in the reference (e.g. the temporal
    derivative of an exactly uniform state)."""
    a = np.asarray(a, dtype="float64")
    b = np.asarray(b, dtype="float64")
    if b.size == 0:
        return
    diff = float(np.abs(a - b).max())
    bound = tol * float(np.abs(b).max()) + atol
    assert np.isfinite(diff) and diff <= bound, \
        "%s: max abs diff %.3e > %.3e (rel %.3e)" % (
            what, diff, bound, relerr(a, b))
