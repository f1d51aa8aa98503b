"""Conservation-element geometry: the reference's known answers
(tests/test_euler_multidim.py:62-120) on the oracle (CPU) and on the device
core (``-m gpu``).

* every cell's BCE volumes sum to its CCE volume (the FP32 march's delta form
  relies on this identity: sum_f bvol_f u0 / cevol = u0);
* hand-computed volumes: cell 0 of the three-triangle fan has BCEs 1/2, 2/3,
  1/2; the unit square quad has four BCEs of 1/2 and a CCE of 2;
* prepare_ce run again gives the same tables.
"""

import numpy as np
import pytest

from _util import FIXTURES, fixture_mesh

GENERATED = {"tri": ("tri_square", (6, 0.2, 1)),
             "quad": ("quad_square", (5, 0.15, 2)),
             "tet": ("tet_cube", (3, 0.15, 3)),
             "hex": ("hex_cube", (3, 0.1, 4)),
             "prism": ("prism_slab", (3, 2, 0.1, 5))}
MESHES = sorted(FIXTURES) + sorted(GENERATED)


def _mesh(name):
    if name in FIXTURES:
        return fixture_mesh(name)
    from solvcon_gb300 import meshgen
    fn, args = GENERATED[name]
    x, t, c = getattr(meshgen, fn)(*args)
    return meshgen.build_mesh(x.shape[1], x, t, c)


def _check_bce_sums(mesh, cevol):
    ng = int(mesh.ngstcell)
    clfcs = np.asarray(mesh.clfcs.ndarray)[ng:]
    body = np.asarray(cevol)[ng:]
    for icl in range(int(mesh.ncell)):
        nfc = clfcs[icl, 0]
        total = body[icl, 1:nfc + 1].sum()
        assert abs(total - body[icl, 0]) <= 1e-12 * abs(body[icl, 0]), icl
        assert body[icl, 0] > 0.0


def _check_known(name, cevol, ng):
    row = np.asarray(cevol)[ng]
    if name == "tri3":
        np.testing.assert_allclose(row[1:4], [0.5, 2.0 / 3.0, 0.5],
                                   rtol=0, atol=1e-12)
        np.testing.assert_allclose(row[0], 0.5 + 2.0 / 3.0 + 0.5, atol=1e-12)
    elif name == "quad1":
        np.testing.assert_allclose(row[1:5], [0.5] * 4, rtol=0, atol=1e-12)
        np.testing.assert_allclose(row[0], 2.0, atol=1e-12)


@pytest.mark.parametrize("name", MESHES)
def test_oracle_ce_known_answers(name):
    from oracle import oracle as ora
    mesh = _mesh(name)
    o = ora.OracleEuler(mesh, 0.01)
    _check_bce_sums(mesh, o.cevol)
    _check_known(name, o.cevol, o.ngstcell)


@pytest.mark.gpu
@pytest.mark.parametrize("name", MESHES)
def test_device_ce_known_answers(name):
    import solvcon_gb300 as sg
    mesh = _mesh(name)
    ec = sg.EulerCore(mesh=mesh, time_increment=0.01)
    cevol = np.array(ec.cevol.ndarray)
    _check_bce_sums(mesh, cevol)
    _check_known(name, cevol, ec.ngstcell)
    before = {k: np.array(getattr(ec, k).ndarray)
              for k in ("cevol", "cecnd", "sfcnd", "sfnml")}
    ec.prepare_ce()
    for k, v in before.items():
        np.testing.assert_array_equal(np.array(getattr(ec, k).ndarray), v,
                                      err_msg=k)
