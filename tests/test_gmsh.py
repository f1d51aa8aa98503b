"""Gmsh MSH 2.2 reader: the mesh read equals the reference reader's.

Fixtures (tests/golden/gmsh_*.npz, written by tests/golden/make_golden.py)
hold Gmsh files written by meshgen.to_gmsh and every StaticMesh table the
reference's own reader (cpp/solvcon/inout/gmsh.cpp) builds from them: a
triangle fan with boundary lines, points and physical names (the reference
test's case), a tri/quad mix, the same with 6-node triangles, and a 3D file
with every cell type.  The reader must give the same tables entry for entry,
the same tables as building the described mesh directly, and the reference's
errors for malformed files.
"""

import numpy as np
import pytest

from _util import golden
from test_mesh import INT_ARRAYS, REAL_ARRAYS, SIZES

CASES = ("tri3", "mixed2d", "order2", "mixed3d")


def _read(text):
    from solvcon_gb300 import Gmsh
    return Gmsh(text).to_block()


def _same_tables(m, g):
    assert [getattr(m, k) for k in SIZES] == list(g["sizes"])
    for name in INT_ARRAYS:
        got = np.asarray(getattr(m, name).ndarray).ravel()
        assert np.array_equal(got, g[name]), name
    got = np.asarray(m.clnds.ndarray)
    want = np.asarray(g["clnds"]).reshape(got.shape)
    for row in range(got.shape[0]):
        n = want[row, 0]
        assert np.array_equal(got[row, :n + 1], want[row, :n + 1])
    for name in REAL_ARRAYS:
        got = np.asarray(getattr(m, name).ndarray).ravel()
        np.testing.assert_allclose(got, g[name], rtol=1e-14, atol=1e-15,
                                   err_msg=name)


@pytest.mark.parametrize("case", CASES)
def test_reader_matches_reference_golden(case):
    g = golden("gmsh_" + case)
    _same_tables(_read(str(g["msh"])), g)


def test_reference_test_known_answers():
    # tests/test_gmsh.py:19-40 of the reference: node and cell tables.
    m = _read(str(golden("gmsh_tri3")["msh"]))
    assert (m.nnode, m.ngstnode, m.ncell) == (4, 3, 3)
    np.testing.assert_almost_equal(
        [[m.ndcrd[i, d] for d in range(m.ndim)] for i in range(m.nnode)],
        [[0.0, 0.0], [-1.0, -1.0], [1.0, -1.0], [0.0, 1.0]])
    assert list(m.cltpn[0:3]) == [4, 4, 4]
    assert [[m.clnds[i, j] for j in range(4)] for i in range(m.ncell)] == \
        [[3, 0, 1, 2], [3, 0, 2, 3], [3, 0, 3, 1]]


def test_reader_matches_direct_build():
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_golden
    from solvcon_gb300 import meshgen
    for name, (text, nd, x, t, c) in make_golden.gmsh_cases().items():
        if x is None:
            continue
        a = _read(text)
        b = meshgen.build_mesh(nd, np.asarray(x), np.asarray(t),
                               np.asarray(c))
        b.build_edge()  # build_mesh leaves the edge table out
        for k in SIZES:
            assert getattr(a, k) == getattr(b, k), (name, k)
        for arr in INT_ARRAYS + REAL_ARRAYS + ("clnds",):
            assert np.array_equal(np.asarray(getattr(a, arr).ndarray),
                                  np.asarray(getattr(b, arr).ndarray)), \
                (name, arr)


def test_reader_matches_reference_library_on_more_files():
    from oracle import refbind as rb
    if not rb.available():
        pytest.skip("reference library not built here")
    from solvcon_gb300 import meshgen
    for seed in (3, 4):
        x, t, c = meshgen.tet_cube(2, 0.15, seed)
        text = meshgen.to_gmsh(3, x, t, c)
        r = rb.RefMesh.from_gmsh(text.encode())
        g = {"sizes": [r.sizes()[k] for k in SIZES]}
        for a in INT_ARRAYS + REAL_ARRAYS + ("clnds",):
            g[a] = r.array(a)
        _same_tables(_read(text), g)


def _file(version="2.2", nodes=True, elements=True, order=None):
    parts = {
        "fmt": ["$MeshFormat", "%s 0 8" % version, "$EndMeshFormat"],
        "nodes": ["$Nodes", "3", "1 0 0 0", "2 1 0 0", "3 0 1 0",
                  "$EndNodes"],
        "elems": ["$Elements", "1", "1 2 2 1 1 1 2 3", "$EndElements"],
    }
    seq = order or ["fmt"] + (["nodes"] if nodes else []) + \
        (["elems"] if elements else [])
    return "\n".join(sum((parts[k] for k in seq), [])) + "\n"


def test_malformed_files():
    from solvcon_gb300 import Gmsh
    assert Gmsh(_file()).to_block().ncell == 1
    with pytest.raises(ValueError, match="does not support msh file ver"):
        Gmsh(_file(version="4.1"))
    with pytest.raises(ValueError, match="Incorrect msh file format"):
        Gmsh(_file(elements=False))
    with pytest.raises(ValueError, match="Incorrect msh file format"):
        Gmsh(_file(order=["nodes", "fmt", "elems"]))
    with pytest.raises(IndexError):
        Gmsh(_file().replace("1 2 2 1 1 1 2 3", "1 2 2 1 1 1 2 9"))


@pytest.mark.gpu
def test_march_on_a_gmsh_mesh():
    """The GPU march on a mesh read from a file equals the march on the same
    mesh built from its arrays, bit for bit."""
    import solvcon_gb300 as sg
    from solvcon_gb300 import meshgen
    g = golden("gmsh_mixed2d")
    a = _read(str(g["msh"]))
    x = np.asarray(a.ndcrd.ndarray)[a.ngstnode:]
    t = np.asarray(a.cltpn.ndarray)[a.ngstcell:]
    c = np.asarray(a.clnds.ndarray)[a.ngstcell:]
    b = meshgen.build_mesh(2, x, t, c)
    out = []
    for mesh in (a, b):
        core = sg.EulerCore(mesh, 2e-3)
        clcnd = np.asarray(mesh.clcnd.ndarray)[mesh.ngstcell:]
        core.init_solution(1.4, 1.0, [0.0, 0.0], 1.0)
        core.so0n[0:] = meshgen.quadrant_state(clcnd, 3)
        core.add_slipwall(np.asarray(mesh.bndfcs.ndarray[:, 0]))
        core.bc_soln()
        core.bc_dsoln()
        core.march(5)
        out.append(np.array(core.so0n.ndarray))
    np.testing.assert_array_equal(out[0], out[1])
