"""Generate tests/golden/obsrefl_<nx>x<ny>.npz from the reference's own
oblique-shock mesher.

Runs ``ObliqueShockMesher._jitter_points`` and ``_split_double_boundary``
(solvcon/pilot/apps/obsrefl/_driver.py:127-260: the scattered points, the
Bowyer-Watson triangulation and the corner-ear refinement) of the reference
tree named by SOLVCON_REF_TREE, loaded unmodified.  The module's only
dependency on the compiled library is the PointPad point container, which a
plain-Python stand-in with the same four calls provides here.  Stores the
final points (Steiner points appended) and the triangles in the reference's
order.

Usage: SOLVCON_REF_TREE=<reference tree> python tests/golden/make_obsrefl_golden.py
"""

import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class PointPad:
    """The four PointPadFp64 calls the mesher makes: append, len, x_at,
    y_at."""

    def __init__(self, ndim=2):
        self.ndim = ndim
        self.xy = []

    def append(self, x, y):
        self.xy.append((float(x), float(y)))

    def __len__(self):
        return len(self.xy)

    def x_at(self, i):
        return self.xy[i][0]

    def y_at(self, i):
        return self.xy[i][1]


def load_driver(tree):
    core = types.SimpleNamespace(PointPadFp64=PointPad)
    for name in ("solvcon", "solvcon.pilot", "solvcon.pilot.apps",
                 "solvcon.pilot.apps.obsrefl"):
        mod = types.ModuleType(name)
        mod.__path__ = []
        sys.modules[name] = mod
    sys.modules["solvcon"].core = core
    path = os.path.join(tree, "solvcon", "pilot", "apps", "obsrefl",
                        "_driver.py")
    spec = importlib.util.spec_from_file_location(
        "solvcon.pilot.apps.obsrefl._driver", path)
    drv = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(drv)
    return drv


def main():
    tree = os.environ.get("SOLVCON_REF_TREE") or "/root/reference"
    drv = load_driver(tree)
    for nx, ny in ((64, 16), (24, 6)):
        mesher = drv.ObliqueShockMesher(nx=nx, ny=ny)
        pad = mesher._jitter_points()
        tris = mesher._split_double_boundary(pad)
        np.savez_compressed(
            os.path.join(HERE, "obsrefl_%dx%d.npz" % (nx, ny)),
            nx=nx, ny=ny, points=np.array(pad.xy, dtype="float64"),
            triangles=np.array(tris, dtype="int32"))
        print("obsrefl %dx%d: %d points, %d triangles" %
              (nx, ny, len(pad), len(tris)))


if __name__ == "__main__":
    main()
