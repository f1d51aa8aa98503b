"""GPU spacetime scalar CESE solvers with solvcon's spacetime surface.

Mirrors ``solvcon.spacetime`` (cpp/solvcon/spacetime/pymod/wrap_spacetime.*):
:class:`Grid` (CE boundaries plus centres and two mirrored ghost points on
each side, core.cpp:14-99), and :class:`LinearScalarSolver` /
:class:`InviscidBurgersSolver` with ``get_so0/set_so0/get_so1/set_so1/
get_cfl/get_so0p``, ``x``/``xctr``, ``selm``/``selms``/``celm``/``celms``,
the fine-grained half steps and ``march_alpha1``/``march_alpha2``.  The march
runs on the GPU; the generic ``Solver`` whose kernel is a set of Python
callbacks has no GPU counterpart.
"""

import ctypes

import numpy as np

from . import _lib
from ._lib import check, ptr
from .buffer import SimpleArray
from .synth import ST_BOUND_COUNT as BOUND_COUNT, grid_xcoord, grid_xloc

__all__ = ["Grid", "LinearScalarSolver", "InviscidBurgersSolver"]

_vp = ctypes.c_void_p
lib = _lib.bind_more({
    "scg_st_create": ([ctypes.c_int, _vp, ctypes.c_int64, ctypes.c_double,
                       _vp], ctypes.c_int),
    "scg_st_destroy": ([_vp], ctypes.c_int),
    "scg_st_set_time_increment": ([_vp, ctypes.c_double], ctypes.c_int),
    "scg_st_get": ([_vp, ctypes.c_int, _vp, ctypes.c_int64], ctypes.c_int),
    "scg_st_set": ([_vp, ctypes.c_int, _vp, ctypes.c_int64], ctypes.c_int),
    "scg_st_op": ([_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int],
                  ctypes.c_int),
    "scg_st_march": ([_vp, ctypes.c_int, ctypes.c_int64], ctypes.c_int),
    "scg_st_sync": ([_vp], ctypes.c_int),
    "scg_st_stream": ([_vp, _vp], ctypes.c_int),
})



class Grid:
    """1D space-time grid (core.hpp:96-214).  ``Grid(xmin, xmax, ncelm)``
    or ``Grid(xloc)`` with the CE boundaries."""

    def __init__(self, *args):
        if len(args) == 3:
            xmin, xmax, ncelm = float(args[0]), float(args[1]), int(args[2])
            if ncelm < 1:
                raise ValueError("Grid::Grid(xmin=%g, xmax=%g, ncelm=%d) "
                                 "invalid argument: ncelm smaller than 1"
                                 % (xmin, xmax, ncelm))
            if xmin >= xmax:
                raise ValueError("Grid::Grid(xmin=%g, xmax=%g, ncelm=%d) "
                                 "invalid arguments: xmin >= xmax"
                                 % (xmin, xmax, ncelm))
            xloc = grid_xloc(xmin, xmax, ncelm)
        elif len(args) == 1:
            xloc = np.asarray(args[0], dtype="float64")
        else:
            raise TypeError("Grid(xmin, xmax, ncelm) or Grid(xloc)")
        self._init_from_array(xloc)

    def _init_from_array(self, xloc):
        if xloc.size < 2:
            raise ValueError("Grid::init_from_array(xloc) invalid arguments: "
                             "xloc.size()=%d smaller than 2" % xloc.size)
        if np.any(xloc[:-1] >= xloc[1:]):
            raise ValueError("Grid::init_from_array(xloc) invalid arguments: "
                             "coordinates not ascending")
        self.ncelm = xloc.size - 1
        self.xmin = float(xloc[0])
        self.xmax = float(xloc[-1])
        self.xcoord = grid_xcoord(xloc)

    @property
    def nselm(self):
        return self.ncelm + 1

    @property
    def xsize(self):
        return self.xcoord.size

    def __str__(self):
        return "Grid(xmin=%g, xmax=%g, ncelm=%d)" % (self.xmin, self.xmax,
                                                      self.ncelm)


class _Selm:
    """Host view of one solution element (core.hpp:460-560)."""

    def __init__(self, svr, index, odd_plane):
        self._svr = svr
        self.index = int(index)
        self.on_odd_plane = bool(odd_plane)
        self.on_even_plane = not self.on_odd_plane
        self.xindex = BOUND_COUNT + 2 * self.index + int(self.on_odd_plane)

    def _x(self, off):
        return float(self._svr._host("x")[self.xindex + off])

    x = property(lambda self: self._x(0))
    xneg = property(lambda self: self._x(-1))
    xpos = property(lambda self: self._x(1))
    xctr = property(lambda self: (self.xneg + self.xpos) / 2)
    dx = property(lambda self: self.xpos - self.xneg)
    dxneg = property(lambda self: self.x - self.xneg)
    dxpos = property(lambda self: self.xpos - self.x)

    def get_so0(self, iv):
        return float(self._svr._host("so0")[self.xindex])

    def get_so1(self, iv):
        return float(self._svr._host("so1")[self.xindex])

    def get_cfl(self):
        return float(self._svr._host("cfl")[self.xindex])

    def so0p(self, iv):
        hdt = self._svr.time_increment / 2
        return self.get_so0(iv) + (self.x - self.xctr) * self.get_so1(iv) \
            - hdt * self.get_so1(iv)


class _Celm:
    """Host view of one conservation element (core.hpp:574-690)."""

    def __init__(self, svr, index, odd_plane):
        self._svr = svr
        self.index = int(index)
        self.on_odd_plane = bool(odd_plane)
        self.on_even_plane = not self.on_odd_plane
        self.xindex = 1 + BOUND_COUNT + 2 * self.index + int(odd_plane)

    x = property(lambda self: float(self._svr._host("x")[self.xindex]))
    xctr = property(lambda self: self.x)

    def selm_xn(self):
        return _Selm(self._svr, self.index, self.on_odd_plane)

    def selm_xp(self):
        return _Selm(self._svr, self.index + 1, self.on_odd_plane)

    def selm_tp(self):
        return _Selm(self._svr, self.index + int(self.on_odd_plane),
                     not self.on_odd_plane)

    selm_tn = selm_tp


class _ScalarSolver:
    KIND = None
    nvar = 1

    def __init__(self, grid, time_increment):
        self.grid = grid
        self._dt = float(time_increment)
        h = ctypes.c_void_p()
        xc = np.ascontiguousarray(grid.xcoord)
        check(lib.scg_st_create(self.KIND, ptr(xc), grid.ncelm, self._dt,
                                ctypes.byref(h)))
        self._h = h
        self._cache = {}
        self._valid = set()
        self._dirty = set()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.scg_st_destroy(h)
            self._h = None

    _IDS = {"x": 0, "so0": 1, "so1": 2, "cfl": 3}

    def _host(self, name):
        if name not in self._valid:
            buf = self._cache.get(name)
            if buf is None:
                buf = np.empty(self.grid.xsize)
                self._cache[name] = buf
            check(lib.scg_st_get(self._h, self._IDS[name], ptr(buf),
                                 buf.size))
            self._valid.add(name)
        return self._cache[name]

    def _flush(self):
        for name in sorted(self._dirty):
            buf = self._cache[name]
            check(lib.scg_st_set(self._h, self._IDS[name], ptr(buf),
                                 buf.size))
        self._dirty.clear()

    def _op(self, op, odd=False, alpha=2):
        self._flush()
        check(lib.scg_st_op(self._h, op, int(bool(odd)), alpha))
        self._valid.clear()

    # -- properties ---------------------------------------------------------

    @property
    def time_increment(self):
        return self._dt

    def set_time_increment(self, dt):
        self._dt = float(dt)
        check(lib.scg_st_set_time_increment(self._h, self._dt))

    dt = property(lambda self: self._dt)
    hdt = property(lambda self: self._dt / 2)
    qdt = property(lambda self: self._dt / 4)

    def _whole(self, name):
        return SimpleArray(lambda: self._host(name).reshape(-1, 1)
                           if name in ("so0", "so1") else self._host(name),
                           on_write=lambda: self._dirty.add(name))

    so0 = property(lambda self: self._whole("so0"))
    so1 = property(lambda self: self._whole("so1"))
    cfl = property(lambda self: self._whole("cfl"))

    def _plane(self, odd_plane):
        n = self.grid.nselm - int(bool(odd_plane))
        start = BOUND_COUNT + int(bool(odd_plane))
        return slice(start, start + 2 * n - 1, 2), n

    def _check_iv(self, iv, what):
        if iv < 0 or iv >= self.nvar:
            raise IndexError("%s(): out of nvar range" % what)

    def x(self, odd_plane=False):
        sl, _ = self._plane(odd_plane)
        return self._host("x")[sl].copy()

    def xctr(self, odd_plane=False):
        sl, n = self._plane(odd_plane)
        x = self._host("x")
        idx = np.arange(sl.start, sl.stop, 2)
        return (x[idx - 1] + x[idx + 1]) / 2

    def _get(self, name, iv, odd_plane):
        if iv is not None:
            self._check_iv(iv, "get_" + name)
        sl, _ = self._plane(odd_plane)
        arr = self._host(name)[sl].copy()
        return SimpleArray(lambda: arr)

    def _set(self, name, iv, arr, odd_plane):
        if iv is not None:
            self._check_iv(iv, "set_" + name)
        sl, n = self._plane(odd_plane)
        arr = np.asarray(arr, dtype="float64")
        if arr.ndim != 1:
            raise IndexError("set_%s(): input not 1D" % name)
        if arr.size != n:
            raise IndexError("set_%s(): arr size %d != nselm %d" % (
                name, arr.size, n))
        self._host(name)[sl] = arr
        self._dirty.add(name)

    def get_so0(self, iv, odd_plane=False):
        return self._get("so0", iv, odd_plane)

    def get_so1(self, iv, odd_plane=False):
        return self._get("so1", iv, odd_plane)

    def get_cfl(self, odd_plane=False):
        return self._get("cfl", None, odd_plane)

    def set_so0(self, iv, arr, odd_plane=False):
        self._set("so0", iv, arr, odd_plane)

    def set_so1(self, iv, arr, odd_plane=False):
        self._set("so1", iv, arr, odd_plane)

    def set_cfl(self, arr, odd_plane=False):
        self._set("cfl", None, arr, odd_plane)

    def get_so0p(self, iv, odd_plane=False):
        self._check_iv(iv, "get_so0p")
        return np.array([e.so0p(iv) for e in self.selms(odd_plane)])

    def selm(self, ielm, odd_plane=False):
        return _Selm(self, ielm, odd_plane)

    def celm(self, ielm, odd_plane=False):
        return _Celm(self, ielm, odd_plane)

    def selms(self, odd_plane=False):
        n = self.grid.nselm - int(bool(odd_plane))
        return [_Selm(self, i, odd_plane) for i in range(n)]

    def celms(self, odd_plane=False):
        n = self.grid.ncelm - int(bool(odd_plane))
        return [_Celm(self, i, odd_plane) for i in range(n)]

    # -- marching -----------------------------------------------------------

    def update_cfl(self, odd_plane):
        self._op(0, odd_plane)

    def march_half_so0(self, odd_plane):
        self._op(1, odd_plane)

    def march_half_so1_alpha1(self, odd_plane):
        self._op(2, odd_plane, 1)

    def march_half_so1_alpha2(self, odd_plane):
        self._op(2, odd_plane, 2)

    def treat_boundary_so0(self):
        self._op(3)

    def treat_boundary_so1(self):
        self._op(4)

    def setup_march(self):
        self._op(5)

    def march_half1_alpha1(self):
        self._op(6, False, 1)

    def march_half1_alpha2(self):
        self._op(6, False, 2)

    def march_half2_alpha1(self):
        self._op(7, True, 1)

    def march_half2_alpha2(self):
        self._op(7, True, 2)

    def _march(self, alpha, steps):
        self._flush()
        check(lib.scg_st_march(self._h, alpha, int(steps)))
        check(lib.scg_st_sync(self._h))
        self._valid.clear()

    def march_alpha1(self, steps):
        self._march(1, steps)

    def march_alpha2(self, steps):
        self._march(2, steps)


class LinearScalarSolver(_ScalarSolver):
    """u_t + u_x = 0 (kernel/linear_scalar.hpp)."""
    KIND = 0


class InviscidBurgersSolver(_ScalarSolver):
    """u_t + (u^2/2)_x = 0 (kernel/inviscid_burgers.hpp)."""
    KIND = 1
