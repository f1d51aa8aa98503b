"""build_interior on the GPU: every table equal to the host builder's.

The device builder (mesh_device.cu) extracts, de-duplicates and numbers the
faces with sorts and prefix sums and evaluates the metrics per face and per
cell; the host builder restates the reference's sequential passes.  They must
agree entry for entry (integers exactly, reals bit for bit: both evaluate the
same expressions in the same order without FMA contraction) on every cell
type, on mixed meshes, and against the reference's golden tables.
"""

import numpy as np
import pytest

from _util import golden
from test_mesh import CASES, INT_ARRAYS, REAL_ARRAYS, SIZES

pytestmark = pytest.mark.gpu

ALL = INT_ARRAYS + REAL_ARRAYS + ("clnds",)


def _mesh(nd, x, t, c, device, ghost=True):
    from solvcon_gb300 import StaticMesh
    c = np.asarray(c)
    m = StaticMesh(ndim=nd, nnode=len(x), nface=0, ncell=len(t))
    m.ndcrd[:, :] = np.asarray(x)
    m.cltpn[:] = np.asarray(t)
    m.clnds[:, :c.shape[1]] = c
    m.build_interior(do_metric=True, build_edge=True, device=device)
    if ghost:
        m.build_boundary()
        m.build_ghost()
    return m


def _same(a, b, what):
    for k in SIZES:
        assert getattr(a, k) == getattr(b, k), (what, k)
    for arr in ALL:
        x = np.asarray(getattr(a, arr).ndarray)
        y = np.asarray(getattr(b, arr).ndarray)
        assert x.shape == y.shape and np.array_equal(x, y), (what, arr)


def _meshes():
    import os
    import sys
    from solvcon_gb300 import meshgen
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_golden
    out = {}
    out["tri"] = (2,) + meshgen.tri_square(40, 0.2, 3)
    out["quad"] = (2,) + meshgen.quad_square(30, 0.15, 4)
    out["tet"] = (3,) + meshgen.tet_cube(8, 0.15, 5)
    out["hex"] = (3,) + meshgen.hex_cube(7, 0.1, 6)
    out["prism"] = (3,) + meshgen.prism_slab(9, 3, 0.1, 7)
    for name in ("mixed2d", "mixed3d"):
        _, nd, x, t, c = make_golden.gmsh_cases()[name]
        out[name] = (nd, x, t, c)
    return out


@pytest.mark.parametrize("ghost", [False, True])
def test_device_build_equals_host_build(ghost):
    for name, (nd, x, t, c) in _meshes().items():
        _same(_mesh(nd, x, t, c, True, ghost), _mesh(nd, x, t, c, False, ghost),
              name)


@pytest.mark.parametrize("case", CASES)
def test_device_build_matches_reference_golden(case):
    from test_mesh import _same_as_golden
    g = golden("mesh_" + case)
    m = _mesh(int(g["ndim"]), g["ndcrd_in"], g["cltpn_in"], g["clnds_in"],
              True)
    _same_as_golden(m, g)


def test_device_build_default_and_errors():
    from solvcon_gb300 import StaticMesh, meshgen
    # Large meshes take the device path by default; same tables.
    x, t, c = meshgen.tri_square(200, 0.2, 9)
    assert len(t) >= StaticMesh.DEVICE_BUILD_CELLS
    a = _mesh(2, x, t, c, None)
    b = _mesh(2, x, t, c, False)
    _same(a, b, "auto")
    # A cell of another dimension is refused by the device builder.
    m = StaticMesh(ndim=3, nnode=4, nface=0, ncell=1)
    m.ndcrd[:, :] = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1)]
    m.cltpn[:] = [StaticMesh.TRIANGLE]
    m.clnds[:, :4] = [(3, 0, 1, 2)]
    with pytest.raises(ValueError):
        m.build_interior(device=True)
