"""Plot3D reader: the mesh read equals the reference reader's.

Fixtures (tests/golden/plot3d_*.npz, written by tests/golden/make_golden.py)
hold Plot3D files written by meshgen.to_plot3d (a jittered block; three
blocks of different shapes side by side) and every StaticMesh table the
reference's own reader (cpp/solvcon/inout/plot3d.cpp) builds from them.
"""

import numpy as np
import pytest

from _util import golden
from test_gmsh import _same_tables


def _read(text):
    from solvcon_gb300 import Plot3d
    return Plot3d(text).to_block()


@pytest.mark.parametrize("case", ("cube", "blocks"))
def test_reader_matches_reference_golden(case):
    g = golden("plot3d_" + case)
    _same_tables(_read(str(g["p3d"])), g)


def test_reference_test_known_answers():
    # tests/test_plot3d.py:13-41 of the reference: one 2x2x2 block.
    data = ("1\n2 2 2\n0 0 0 0 1 1 1 1\n0 0 1 1 0 0 1 1\n"
            "0 1 0 1 0 1 0 1\n")
    m = _read(data)
    assert (m.nnode, m.ncell) == (8, 1)
    np.testing.assert_almost_equal(
        np.asarray(m.ndcrd.ndarray)[24:].tolist(),
        [[0, 0, 0], [0, 0, 1], [0, 1, 0], [0, 1, 1], [1, 0, 0], [1, 0, 1],
         [1, 1, 0], [1, 1, 1]])
    assert np.asarray(m.cltpn.ndarray)[6:].tolist() == [5]
    assert np.asarray(m.clnds.ndarray)[6:].tolist() == \
        [[8, 0, 2, 6, 4, 1, 3, 7, 5]]


def test_blocks_keep_their_own_nodes():
    g = golden("plot3d_blocks")
    m = _read(str(g["p3d"]))
    # 3*2*2 + 2*3*2 + 2*2*4 nodes; 2 + 2 + 3 cells, none across blocks.
    assert (m.nnode, m.ncell) == (40, 7)
    c = np.asarray(m.clnds.ndarray)[m.ngstcell:, 1:9]
    assert c[:2].max() < 12 and 12 <= c[2:4].min() and c[2:4].max() < 24
    assert c[4:].min() >= 24


def test_malformed_files():
    from solvcon_gb300 import Plot3d
    with pytest.raises(ValueError):
        Plot3d("1\n2 2 2\n0 0 0 0 1 1 1 1\n")
    with pytest.raises(ValueError):
        Plot3d("2\n2 2 2\n")
