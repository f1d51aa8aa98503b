"""Host mesh builder parity: the StaticMesh tables equal the reference's.

Golden vectors come from the reference itself (tests/golden/make_golden.py);
where the reference library is built here (oracle/_ref) the same checks run
against it directly on extra seeded meshes.
"""

import numpy as np
import pytest

from _util import golden

CASES = ("tri3", "quad1", "mixed", "tet1", "hex1", "prism1", "pyr1", "tri12",
         "quad8", "tet3")
INT_ARRAYS = ("fctpn", "cltpn", "fcnds", "fccls", "clfcs", "ednds", "bndfcs")
REAL_ARRAYS = ("ndcrd", "fccnd", "fcnml", "fcara", "clcnd", "clvol")
SIZES = ("ndim", "nnode", "nface", "ncell", "nbound", "ngstnode", "ngstface",
         "ngstcell", "nedge", "nbcs")


def _build(g):
    from solvcon_gb300 import StaticMesh
    nd = int(g["ndim"])
    x, t, c = g["ndcrd_in"], g["cltpn_in"], g["clnds_in"]
    m = StaticMesh(ndim=nd, nnode=len(x), nface=0, ncell=len(t))
    m.ndcrd[:, :] = x
    m.cltpn[:] = t
    m.clnds[:, :c.shape[1]] = c
    m.build_interior(do_metric=True, build_edge=True)
    m.build_boundary()
    m.build_ghost()
    return m


@pytest.mark.parametrize("case", CASES)
def test_mesh_matches_reference_golden(case):
    g = golden("mesh_" + case)
    _same_as_golden(_build(g), g)


def _same_as_golden(m, g):
    assert [getattr(m, k) for k in SIZES] == list(g["sizes"])
    for name in INT_ARRAYS:
        got = np.asarray(getattr(m, name).ndarray).ravel()
        assert np.array_equal(got, g[name]), name
    # clnds: the reference leaves unused columns uninitialised; compare the
    # node counts and node lists only.
    got = np.asarray(m.clnds.ndarray)
    want = g["clnds"].reshape(got.shape)
    for row in range(got.shape[0]):
        n = want[row, 0]
        assert np.array_equal(got[row, :n + 1], want[row, :n + 1])
    for name in REAL_ARRAYS:
        got = np.asarray(getattr(m, name).ndarray).ravel()
        np.testing.assert_allclose(got, g[name], rtol=1e-14, atol=1e-15,
                                   err_msg=name)


def test_ghost_indexing_and_views():
    from _util import fixture_mesh
    m = fixture_mesh("tri3")
    assert m.ngstcell == 3 and m.clcnd.nghost == 3
    full = np.asarray(m.clcnd.ndarray)
    assert m.clcnd[-1, 0] == full[2, 0]
    assert m.clcnd[0, 1] == full[3, 1]
    with pytest.raises(IndexError):
        m.clcnd[-4, 0]
    with pytest.raises(IndexError):
        m.clcnd[3, 0]
    # A view taken before a rebuild keeps its old buffer alive.
    assert m.fccls[0, 0] >= 0


def test_add_bc_validation():
    from solvcon_gb300 import StaticMesh
    m = StaticMesh(ndim=2, nnode=4, nface=0, ncell=1)
    m.ndcrd[:, :] = [(0, 0), (1, 0), (1, 1), (0, 1)]
    m.cltpn[:] = [StaticMesh.QUADRILATERAL]
    m.clnds[:, :5] = [(4, 0, 1, 2, 3)]
    m.build_interior()
    with pytest.raises(ValueError):
        m.add_bc("", [0])
    with pytest.raises(ValueError):
        m.add_bc("x", [99])
    b = m.add_bc("left", [3])
    assert b.name == "left"
    with pytest.raises(ValueError):
        m.add_bc("left", [2])
    with pytest.raises(ValueError):
        m.add_bc("again", [3])
    m.build_boundary()
    assert m.nbound == 4 and m.nbcs == 2
    assert m.bc("left").facn[0, 0] == 3
    assert [b.name for b in m.bcs] == ["left", "<NONAME>"]
    with pytest.raises(RuntimeError):
        m.build_boundary()


def test_bad_inputs_raise():
    from solvcon_gb300 import StaticMesh
    with pytest.raises(ValueError):
        StaticMesh(ndim=4, nnode=1, nface=0, ncell=1)
    m = StaticMesh(ndim=2, nnode=3, nface=0, ncell=1)
    m.cltpn[:] = [StaticMesh.TRIANGLE]
    m.clnds[:, :4] = [(3, 0, 1, 7)]
    with pytest.raises(IndexError):
        m.build_interior()


def _ref():
    from oracle import refbind
    if not refbind.available():
        pytest.skip("reference library not built on this host")
    return refbind


@pytest.mark.parametrize("seed", [1, 2])
def test_mesh_matches_reference_library(seed):
    rb = _ref()
    from solvcon_gb300 import meshgen
    for nd, (x, t, c) in ((2, meshgen.tri_square(9, 0.2, seed)),
                          (3, meshgen.tet_cube(3, 0.15, seed))):
        m = meshgen.build_mesh(nd, x, t, c)
        r = rb.RefMesh(nd, x, t, c[:, :5])
        m.build_edge()
        for name in INT_ARRAYS + REAL_ARRAYS:
            got = np.asarray(getattr(m, name).ndarray).ravel()
            assert np.array_equal(got, r.array(name)), name


class _ForeignMesh:
    """A mesh built by other code, with the reference StaticMesh surface:
    size properties and whole-buffer tables (ghost rows first) whose
    ``.ndarray`` is a numpy array, as the reference's pybind11 wrapper
    exposes them (wrap_StaticMesh.cpp:61-181)."""

    class _Arr:
        def __init__(self, a):
            self.ndarray = a

    class _Bc:
        def __init__(self, name, facn):
            self.name = name
            self.facn = _ForeignMesh._Arr(facn)

    def __init__(self, sizes, tables, bcs=()):
        for k, v in zip(SIZES, sizes):
            setattr(self, k, int(v))
        for k, v in tables.items():
            setattr(self, k, self._Arr(v))
        self.bcs = [self._Bc(n, f) for n, f in bcs]


def _foreign_from_golden(g):
    s = [int(x) for x in g["sizes"]]
    tables = {k: g[k] for k in INT_ARRAYS + REAL_ARRAYS + ("clnds",)}
    # The fixtures carry no clgrp; the reference fills it with -1 (no group).
    tables["clgrp"] = np.full(s[7] + s[3], -1, dtype="int32")
    return _ForeignMesh(s, tables, [("walls", np.arange(s[4] * 3,
                                                        dtype="int32"))])


@pytest.mark.parametrize("case", CASES)
def test_from_mesh_takes_reference_tables_verbatim(case):
    """StaticMesh.from_mesh on a mesh the reference built (its golden
    tables behind the reference's surface): every table and size comes over
    unchanged, boundary groups included."""
    from solvcon_gb300 import StaticMesh
    g = golden("mesh_" + case)
    foreign = _foreign_from_golden(g)
    m = StaticMesh.from_mesh(foreign)
    _same_as_golden(m, g)
    np.testing.assert_array_equal(np.asarray(m.clnds.ndarray).ravel(),
                                  g["clnds"])
    assert [b.name for b in m.bcs] == ["walls"]
    np.testing.assert_array_equal(m.bcs[0].facn.ndarray.ravel(),
                                  np.arange(int(g["sizes"][4]) * 3))


def test_from_mesh_rejects_short_tables():
    from solvcon_gb300 import StaticMesh
    g = golden("mesh_tri12")
    foreign = _foreign_from_golden(g)
    foreign.fccls = _ForeignMesh._Arr(g["fccls"][:-4])
    with pytest.raises(ValueError, match="fccls"):
        StaticMesh.from_mesh(foreign)


def test_from_mesh_of_the_live_reference_library():
    """A mesh built by the reference library itself (where it is built
    here) taken over by StaticMesh.from_mesh equals the host builder's."""
    from oracle import refbind as rb
    if not rb.available():
        pytest.skip("reference library not built on this host")
    from solvcon_gb300 import StaticMesh, meshgen
    x, t, c = meshgen.tet_cube(3, 0.15, seed=17)
    r = rb.RefMesh(3, x, t, c)
    s = r.sizes()
    foreign = _ForeignMesh([s[k] for k in SIZES],
                           {k: r.array(k) for k in INT_ARRAYS + REAL_ARRAYS +
                            ("clnds", "clgrp")})
    m = StaticMesh.from_mesh(foreign)
    assert m.nedge == s["nedge"] > 0
    np.testing.assert_array_equal(np.asarray(m.ednds.ndarray).ravel(),
                                  r.array("ednds"))
    # build_mesh builds no edges; every other table is compared.
    ours = meshgen.build_mesh(3, x, t, c)
    for k in set(INT_ARRAYS + REAL_ARRAYS) - {"ednds"}:
        np.testing.assert_array_equal(np.asarray(getattr(m, k).ndarray),
                                      np.asarray(getattr(ours, k).ndarray), k)
