"""ctypes binding of oracle/_ref/libsolvcon_ref.so (test infrastructure only).

The library is the reference solvcon implementation itself (its own mesh,
multidim and onedim sources, built by ``make -C oracle ref``) behind the thin C
driver in oracle/ref_driver.cpp.  It is only present where the reference source
tree was available at build time; :func:`available` says whether it is.  Only
tests and the golden-vector generator use it, to pin the oracle and the
fixtures to the reference's own results.
"""

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "_ref", "libsolvcon_ref.so")

_lib = None

MESH_INT_ARRAYS = ("fctpn", "cltpn", "clgrp", "fcnds", "fccls", "clnds",
                   "clfcs", "ednds", "bndfcs")
MESH_REAL_ARRAYS = ("ndcrd", "fccnd", "fcnml", "fcara", "clcnd", "clvol")
EULER_ARRAYS = ("cevol", "cecnd", "sfcnd", "sfnml", "so0c", "so0n", "so0t",
                "so1c", "so1n", "stm", "cflo", "cflc", "gamma")
OPS = {"update": 0, "calc_solt": 1, "calc_soln": 2, "bc_soln": 3,
       "calc_cfl": 4, "calc_dsoln": 5, "bc_dsoln": 6, "march_substep": 7}


def available():
    return os.path.exists(LIBPATH)


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(LIBPATH)
        _lib.ref_last_error.restype = ctypes.c_char_p
    return _lib


def _check(rc):
    if rc != 0:
        raise ValueError(lib().ref_last_error().decode())


def _dp(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class RefMesh:
    """The reference StaticMesh, built from node coordinates and cell lists."""

    def __init__(self, ndim, ndcrd, cltpn, clnds, bcs=(), ghost=True):
        ndcrd = np.ascontiguousarray(ndcrd, dtype="float64")
        cltpn = np.ascontiguousarray(cltpn, dtype="int32")
        full = np.full((len(cltpn), 9), -1, dtype="int32")
        clnds = np.asarray(clnds, dtype="int32")
        full[:, :clnds.shape[1]] = clnds
        h = ctypes.c_void_p()
        _check(lib().ref_mesh_create(ndim, ndcrd.shape[0], len(cltpn),
                                     _dp(ndcrd), _dp(cltpn), _dp(full),
                                     ctypes.byref(h)))
        self.h = h
        _check(lib().ref_mesh_build(h, 0))
        for name, faces in bcs:
            f = np.ascontiguousarray(faces, dtype="int32")
            _check(lib().ref_mesh_add_bc(h, name.encode(), _dp(f), len(f)))
        if ghost:
            _check(lib().ref_mesh_build(h, 1))
            _check(lib().ref_mesh_build(h, 2))

    @classmethod
    def from_gmsh(cls, data):
        """The reference's Gmsh reader on a MSH file's contents."""
        self = cls.__new__(cls)
        h = ctypes.c_void_p()
        lib().ref_gmsh_load.argtypes = [ctypes.c_char_p, ctypes.c_longlong,
                                        ctypes.c_void_p]
        _check(lib().ref_gmsh_load(bytes(data), len(data), ctypes.byref(h)))
        self.h = h
        return self

    @classmethod
    def from_plot3d(cls, data):
        """The reference's Plot3D reader on a file's contents."""
        self = cls.__new__(cls)
        h = ctypes.c_void_p()
        lib().ref_plot3d_load.argtypes = [ctypes.c_char_p,
                                          ctypes.c_longlong, ctypes.c_void_p]
        _check(lib().ref_plot3d_load(bytes(data), len(data),
                                     ctypes.byref(h)))
        self.h = h
        return self

    def sizes(self):
        out = (ctypes.c_longlong * 10)()
        _check(lib().ref_mesh_sizes(self.h, out))
        keys = ("ndim", "nnode", "nface", "ncell", "nbound", "ngstnode",
                "ngstface", "ngstcell", "nedge", "nbcs")
        return dict(zip(keys, list(out)))

    def array(self, name):
        cnt = ctypes.c_longlong()
        _check(lib().ref_mesh_array(self.h, name.encode(), None,
                                    ctypes.byref(cnt)))
        dt = "int32" if name in MESH_INT_ARRAYS else "float64"
        out = np.empty(cnt.value, dtype=dt)
        _check(lib().ref_mesh_array(self.h, name.encode(), _dp(out),
                                    ctypes.byref(cnt)))
        return out

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.ref_mesh_destroy(self.h)
            self.h = None


class RefEuler:
    """The reference EulerCore on a :class:`RefMesh`."""

    def __init__(self, mesh, time_increment):
        h = ctypes.c_void_p()
        lib().ref_euler_create.argtypes = [ctypes.c_void_p, ctypes.c_double,
                                           ctypes.c_void_p]
        _check(lib().ref_euler_create(mesh.h, time_increment,
                                      ctypes.byref(h)))
        self.h = h
        self.mesh = mesh
        s = mesh.sizes()
        self.ndim, self.ncell, self.ngstcell = s["ndim"], s["ncell"], \
            s["ngstcell"]
        self.neq = self.ndim + 2

    def shape(self, name):
        nd, neq, tot = self.ndim, self.neq, self.ncell + self.ngstcell
        return {"cevol": (tot, 7), "cecnd": (tot, 7 * nd),
                "sfcnd": (self.ncell, 24, nd), "sfnml": (self.ncell, 24, nd),
                "so1c": (tot, neq, nd), "so1n": (tot, neq, nd),
                "cflo": (tot,), "cflc": (tot,), "gamma": (tot,)}.get(
                    name, (tot, neq))

    def get(self, name):
        cnt = ctypes.c_longlong()
        _check(lib().ref_euler_array(self.h, name.encode(), None,
                                     ctypes.byref(cnt)))
        out = np.empty(cnt.value, dtype="float64")
        _check(lib().ref_euler_array(self.h, name.encode(), _dp(out),
                                     ctypes.byref(cnt)))
        return out.reshape(self.shape(name))

    def set(self, name, value):
        arr = np.ascontiguousarray(value, dtype="float64").reshape(
            self.shape(name))
        _check(lib().ref_euler_set_array(self.h, name.encode(), _dp(arr)))

    def init_solution(self, gamma, rho, v, p):
        vv = np.zeros(3, dtype="float64")
        vv[:len(v)] = v
        lib().ref_euler_init.argtypes = [ctypes.c_void_p, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_void_p,
                                         ctypes.c_double]
        _check(lib().ref_euler_init(self.h, gamma, rho, _dp(vv), p))

    def set_params(self, sigma0=3.0, taumin=0.0, tauscale=1.0):
        lib().ref_euler_params.argtypes = [ctypes.c_void_p] + \
            [ctypes.c_double] * 3
        _check(lib().ref_euler_params(self.h, sigma0, taumin, tauscale))

    def add_bc(self, kind, faces, value=()):
        f = np.ascontiguousarray(faces, dtype="int32")
        v = np.ascontiguousarray(value, dtype="float64")
        if v.size == 0:
            v = np.zeros(1, dtype="float64")
            nv = 0
        else:
            nv = v.size
        _check(lib().ref_euler_add_bc(self.h, kind, _dp(f), len(f), _dp(v),
                                      nv))

    def call(self, op):
        _check(lib().ref_euler_call(self.h, OPS[op]))

    def march(self, steps):
        _check(lib().ref_euler_march(self.h, steps))

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.ref_euler_destroy(self.h)
            self.h = None


class RefEuler1D:
    """The reference onedim Euler1DCore."""

    NAMES = {"coord": 0, "cfl": 1, "so0": 2, "so1": 3, "gamma": 4}

    def __init__(self, ncoord, time_increment):
        h = ctypes.c_void_p()
        lib().ref_e1d_create.argtypes = [ctypes.c_int, ctypes.c_double,
                                         ctypes.c_void_p]
        _check(lib().ref_e1d_create(ncoord, time_increment, ctypes.byref(h)))
        self.h = h
        self.ncoord = ncoord

    def _shape(self, name):
        return (self.ncoord, 3) if name in ("so0", "so1") else (self.ncoord,)

    def get(self, name):
        out = np.empty(self._shape(name), dtype="float64")
        _check(lib().ref_e1d_array(self.h, self.NAMES[name], _dp(out), None))
        return out

    def set(self, name, value):
        arr = np.ascontiguousarray(value, dtype="float64").reshape(
            self._shape(name))
        _check(lib().ref_e1d_array(self.h, self.NAMES[name], None, _dp(arr)))

    def setup_march(self):
        _check(lib().ref_e1d_march(self.h, 0, 0))

    def march_alpha(self, alpha, steps):
        _check(lib().ref_e1d_march(self.h, alpha, steps))

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.ref_e1d_destroy(self.h)
            self.h = None


class RefSpacetime:
    """The reference spacetime LinearScalarSolver (kind 0) or
    InviscidBurgersSolver (kind 1) on a Grid built from the CE boundaries
    ``xloc``; tables are whole [2 ncelm + 5] arrays (nvar = 1)."""

    NAMES = {"xcoord": 0, "so0": 1, "so1": 2, "cfl": 3}

    def __init__(self, kind, xloc, time_increment):
        xloc = np.ascontiguousarray(xloc, dtype="float64")
        h = ctypes.c_void_p()
        lib().ref_st_create.argtypes = [ctypes.c_int, ctypes.c_void_p,
                                        ctypes.c_longlong, ctypes.c_double,
                                        ctypes.c_void_p]
        lib().ref_st_array.argtypes = [ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p]
        lib().ref_st_march.argtypes = [ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_longlong]
        _check(lib().ref_st_create(kind, _dp(xloc), xloc.size,
                                   time_increment, ctypes.byref(h)))
        self.h = h
        cnt = ctypes.c_longlong()
        _check(lib().ref_st_array(h, 0, None, None, ctypes.byref(cnt)))
        self.xsize = cnt.value

    def get(self, name):
        out = np.empty(self.xsize, dtype="float64")
        cnt = ctypes.c_longlong()
        _check(lib().ref_st_array(self.h, self.NAMES[name], _dp(out), None,
                                  ctypes.byref(cnt)))
        return out

    def set(self, name, value):
        arr = np.ascontiguousarray(value, dtype="float64").reshape(
            self.xsize)
        cnt = ctypes.c_longlong()
        _check(lib().ref_st_array(self.h, self.NAMES[name], None, _dp(arr),
                                  ctypes.byref(cnt)))

    def setup_march(self):
        _check(lib().ref_st_march(self.h, 0, 0))

    def march_alpha(self, alpha, steps):
        _check(lib().ref_st_march(self.h, alpha, steps))

    def __del__(self):
        if getattr(self, "h", None) is not None and _lib is not None:
            _lib.ref_st_destroy(self.h)
            self.h = None
