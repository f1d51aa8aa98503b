"""Batched march of many independent Euler cores, and its autotuner.

:class:`EulerBatch` marches a list of :class:`~solvcon_gb300.EulerCore`
objects together: one kernel launch per substep over a work list of
(core, row tile) pairs, the two launches of a step captured once in a CUDA
graph and replayed.  Each core keeps its own buffers, so cores of different
sizes, time steps and gas constants batch together, and every core's result is
bit-identical to marching it alone.

:func:`autotune` picks the tile (block) size, the grid policy (persistent
blocks striding over the work list, or one block per tile) and, when given
the same meshes in other cell orders (e.g. :func:`morton_order` of
:func:`node_average`), the cell ordering, by timing a few steps of each
candidate.
"""

import ctypes
import time

import numpy as np

from . import _lib
from ._lib import check, ptr

__all__ = ["EulerBatch", "autotune", "morton_order", "node_average"]

_vp = ctypes.c_void_p
lib = _lib.bind_more({
    "scg_batch_create": ([_vp, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                          _vp], ctypes.c_int),
    "scg_batch_destroy": ([_vp], ctypes.c_int),
    "scg_batch_retarget": ([_vp, _vp, ctypes.c_int64, _vp], ctypes.c_int),
    "scg_batch_info": ([_vp, _vp], ctypes.c_int),
    "scg_batch_march": ([_vp, ctypes.c_int64], ctypes.c_int),
    "scg_batch_last_ms": ([_vp, _vp], ctypes.c_int),
    "scg_batch_stream": ([_vp, _vp], ctypes.c_int),
})


class EulerBatch:
    """March many cores in one launch per substep.

    :param cores: EulerCore objects of one ndim and precision.
    :param block: threads per tile (64, 128 or 256).
    :param persistent: size the grid to the GPU's resident capacity and let
        blocks stride over the work list; otherwise one block per tile.
    """

    def __init__(self, cores, block=128, persistent=True):
        self.cores = list(cores)
        arr = (ctypes.c_void_p * len(self.cores))(
            *[c.handle.value for c in self.cores])
        h = ctypes.c_void_p()
        check(lib.scg_batch_create(arr, len(self.cores), int(block),
                                   int(bool(persistent)), ctypes.byref(h)))
        self._h = h
        info = np.zeros(5, dtype="int64")
        check(lib.scg_batch_info(h, ptr(info)))
        self.ncore, self.ncell, self.ntiles, self.grid, self.block = \
            (int(x) for x in info)
        self.persistent = bool(persistent)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.scg_batch_destroy(h)
            self._h = None

    def retarget(self, cores):
        """March another set of cores with this batch (its stream, device
        tables and occupancy kept; the step graph is captured again).
        Returns False, changing nothing, when the set needs another kernel
        (other ndim or precision, or another cell-type specialisation)."""
        cores = list(cores)
        arr = (ctypes.c_void_p * len(cores))(*[c.handle.value for c in cores])
        done = ctypes.c_int()
        check(lib.scg_batch_retarget(self._h, arr, len(cores),
                                     ctypes.byref(done)))
        if not done.value:
            return False
        self.cores = cores
        info = np.zeros(5, dtype="int64")
        check(lib.scg_batch_info(self._h, ptr(info)))
        self.ncore, self.ncell, self.ntiles, self.grid, self.block = \
            (int(x) for x in info)
        return True

    def march(self, steps):
        """Advance every core ``steps`` full steps (synchronous)."""
        for c in self.cores:
            c._flush()
        check(lib.scg_batch_march(self._h, int(steps)))
        for c in self.cores:
            c._after(0)

    @property
    def last_ms(self):
        """Device time (CUDA events) of the last march's kernels, in ms."""
        ms = ctypes.c_double()
        check(lib.scg_batch_last_ms(self._h, ctypes.byref(ms)))
        return ms.value


def morton_order(points):
    """Permutation that sorts 2D/3D points along a Morton (Z-order) curve."""
    pts = np.asarray(points, dtype="float64")
    lo = pts.min(axis=0)
    span = np.maximum(pts.max(axis=0) - lo, 1e-300)
    nd = pts.shape[1]
    bits = 21 if nd == 3 else 31
    q = ((pts - lo) / span * ((1 << bits) - 1)).astype("uint64")
    code = np.zeros(len(pts), dtype="uint64")
    for b in range(bits):
        for d in range(nd):
            code |= ((q[:, d] >> np.uint64(b)) & np.uint64(1)) << \
                np.uint64(b * nd + d)
    return np.argsort(code, kind="stable")


def node_average(ndcrd, clnds):
    """Node average of every cell (clnds rows: count, then node ids), the
    point a cell ordering sorts by."""
    x = np.asarray(ndcrd, dtype="float64")
    c = np.asarray(clnds)
    n = c[:, 0].astype("int64")
    out = np.zeros((len(c), x.shape[1]))
    for k in range(1, c.shape[1]):
        has = n >= k
        out[has] += x[c[has, k]]
    return out / n[:, None]


def autotune(cores, steps=2, blocks=(64, 128, 256),
             persistents=(True, False), repeat=2, orderings=None):
    """Time each (block, persistent) candidate on ``cores``; return the
    fastest configuration and the table of timings (ms per step).

    ``orderings`` optionally maps a name to the same meshes with their cells
    in another order (``cores`` are "native"); every (ordering, block,
    persistent) candidate is timed and the fastest one's ordering is
    returned with it.  The cores are marched ``(1 + repeat) * steps`` steps
    per candidate, so pass scratch copies when their state matters."""
    sets = {"native": cores}
    sets.update(orderings or {})
    table = []
    for name, cs in sets.items():
        for block in blocks:
            for pers in persistents:
                b = EulerBatch(cs, block=block, persistent=pers)
                b.march(steps)  # warm-up (graph capture)
                best = float("inf")
                for _ in range(repeat):
                    b.march(steps)
                    best = min(best, b.last_ms / steps)
                table.append({"ordering": name, "block": block,
                              "persistent": pers, "ms_per_step": best,
                              "grid": b.grid})
                del b
    fastest = min(table, key=lambda r: r["ms_per_step"])
    return fastest, table


def time_sequential(cores, steps):
    """Wall time of marching the cores one after the other (each its own
    launches), for comparison with a batch."""
    for c in cores:
        c.sync()
    t0 = time.perf_counter()
    for c in cores:
        c.march(steps)
    return (time.perf_counter() - t0) * 1e3
