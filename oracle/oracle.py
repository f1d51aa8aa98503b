"""Python front of the C oracle (oracle/cese_oracle.c) -- TEST INFRASTRUCTURE.

The oracle restates the reference CESE march on the CPU; tests,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline and reference
arm use it, to check results against and to time.  The product never imports
this module.
"""

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(_HERE, "_build", "libcese_oracle.so")

_lib = None

MESH_NAMES = ("ndcrd", "fccnd", "fcnml", "clcnd", "fcnds", "fccls", "clfcs",
              "cltpn")


def build():
    """Compile the oracle (``make -C oracle port``)."""
    subprocess.run(["make", "-s", "-C", _HERE, "port"], check=True)
    return LIBPATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            build()
        _lib = ctypes.CDLL(LIBPATH)
        for name in ("ora_prepare_ce", "ora_calc_solt", "ora_calc_soln",
                     "ora_bc_soln", "ora_calc_cfl", "ora_calc_dsoln",
                     "ora_bc_dsoln", "ora_update", "ora_march_substep"):
            getattr(_lib, name).argtypes = [ctypes.c_void_p]
            getattr(_lib, name).restype = None
        _lib.ora_march.argtypes = [ctypes.c_void_p, ctypes.c_int64]
        _lib.ora_march.restype = None
        _lib.ora_set_threads.argtypes = [ctypes.c_int]
        _lib.ora_set_threads.restype = None
        _lib.ora_e1d_march.argtypes = [ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_int64]
        _lib.ora_e1d_update_cfl.argtypes = [ctypes.c_void_p, ctypes.c_int]
        _lib.ora_e1d_march_half_so0.argtypes = [ctypes.c_void_p,
                                                ctypes.c_int]
        _lib.ora_e1d_march_half_so1.argtypes = [ctypes.c_void_p,
                                                ctypes.c_int, ctypes.c_int]
        _lib.ora_e1d_treat_boundary_so0.argtypes = [ctypes.c_void_p]
        _lib.ora_e1d_treat_boundary_so1.argtypes = [ctypes.c_void_p]
    return _lib


def set_threads(n):
    """Threads for the per-cell loops of the multidim march (1 by default,
    the reference's serial order per cell; the results are bit-identical for
    any count)."""
    lib().ora_set_threads(int(n))


_P = ctypes.c_void_p


class _OraMesh(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int32), ("nnode", ctypes.c_int64),
                ("nface", ctypes.c_int64), ("ncell", ctypes.c_int64),
                ("ngstnode", ctypes.c_int64), ("ngstface", ctypes.c_int64),
                ("ngstcell", ctypes.c_int64)] + \
        [(n, _P) for n in MESH_NAMES]


_EULER_ARRAYS = ("cevol", "cecnd", "sfcnd", "sfnml", "so0c", "so0n", "so0t",
                 "stm", "so1c", "so1n", "cflo", "cflc", "gamma")


class _OraEuler(ctypes.Structure):
    _fields_ = [("m", _OraMesh), ("dt", ctypes.c_double),
                ("sigma0", ctypes.c_double), ("taumin", ctypes.c_double),
                ("tauscale", ctypes.c_double)] + \
        [(n, _P) for n in _EULER_ARRAYS] + \
        [("limiter", _P), ("nbnd", ctypes.c_int32), ("bkind", _P),
         ("boff", _P), ("bfaces", _P), ("bval", _P)]


def mesh_tables(mesh):
    """Whole-buffer copies of the tables the march reads, plus sizes, from
    any object with the StaticMesh surface."""
    t = {n: np.ascontiguousarray(np.array(getattr(getattr(mesh, n), "ndarray",
                                                  getattr(mesh, n))))
         for n in MESH_NAMES}
    sizes = {k: int(getattr(mesh, k)) for k in
             ("ndim", "nnode", "nface", "ncell", "ngstnode", "ngstface",
              "ngstcell")}
    return t, sizes


class _OraBuilt(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int32)] + \
        [(k, ctypes.c_int64) for k in ("nnode", "nface", "ncell", "nbound",
                                       "ngstnode", "ngstface", "ngstcell")] + \
        [(k, _P) for k in ("ndcrd", "fccnd", "fcnml", "fcara", "clcnd",
                           "clvol", "fctpn", "cltpn", "clgrp", "fcnds",
                           "fccls", "clnds", "clfcs", "bndfcs")]


class OracleMesh:
    """A mesh built by the oracle's own restatement of the reference's
    StaticMesh build (oracle/mesh_oracle.c): build_interior with metrics,
    build_boundary with every boundary face in one group, build_ghost.

    ``OracleMesh(ndim, ndcrd, cltpn, clnds)`` (clnds as [ncell, 1 + nodes]
    rows, count first).  The sizes are attributes and every table is a whole
    numpy array with its ghost rows first, in the reference's shapes, so
    :class:`OracleEuler` runs on it directly.  The GPU library is not used.
    """

    WIDTHS = {"fcara": 0, "clvol": 0, "fctpn": 0, "cltpn": 0, "clgrp": 0,
              "fcnds": 5, "fccls": 4, "clnds": 9, "clfcs": 7, "bndfcs": 3}

    def __init__(self, ndim, ndcrd, cltpn, clnds):
        ndcrd = np.ascontiguousarray(ndcrd, dtype="float64")
        cltpn = np.ascontiguousarray(cltpn, dtype="int32")
        full = np.full((len(cltpn), 9), -1, dtype="int32")
        c = np.asarray(clnds, dtype="int32")
        full[:, :c.shape[1]] = c
        out = _OraBuilt()
        L = lib()
        L.ora_mesh_build.argtypes = [ctypes.c_int, ctypes.c_int64,
                                     ctypes.c_int64, _P, _P, _P, _P]
        L.ora_mesh_free.argtypes = [_P]
        rc = L.ora_mesh_build(int(ndim), ndcrd.shape[0], cltpn.size,
                              ndcrd.ctypes.data, cltpn.ctypes.data,
                              full.ctypes.data, ctypes.byref(out))
        if rc != 0:
            raise ValueError("ora_mesh_build failed")
        try:
            self.ndim = int(out.ndim)
            for k in ("nnode", "nface", "ncell", "nbound", "ngstnode",
                      "ngstface", "ngstcell"):
                setattr(self, k, int(getattr(out, k)))
            rows = {"node": self.ngstnode + self.nnode,
                    "face": self.ngstface + self.nface,
                    "cell": self.ngstcell + self.ncell}
            kind = {"ndcrd": "node", "fccnd": "face", "fcnml": "face",
                    "fcara": "face", "clcnd": "cell", "clvol": "cell",
                    "fctpn": "face", "cltpn": "cell", "clgrp": "cell",
                    "fcnds": "face", "fccls": "face", "clnds": "cell",
                    "clfcs": "cell"}
            for name, _ in _OraBuilt._fields_[8:]:
                n = self.nbound if name == "bndfcs" else rows[kind[name]]
                w = self.WIDTHS.get(name, self.ndim)
                real = name in ("ndcrd", "fccnd", "fcnml", "fcara", "clcnd",
                                "clvol")
                ctype = ctypes.c_double if real else ctypes.c_int32
                size = n * max(w, 1)
                buf = np.ctypeslib.as_array(
                    (ctype * max(size, 1)).from_address(getattr(out, name)))
                arr = np.array(buf[:size])
                setattr(self, name, arr.reshape((n, w)) if w else arr)
        finally:
            L.ora_mesh_free(ctypes.byref(out))

    @property
    def boundary_faces(self):
        return self.bndfcs[:, 0].copy()


class OracleEuler:
    """The reference EulerCore restated on the CPU.

    Arrays are numpy buffers in the reference layout (ghost rows first),
    accessible as attributes (``so0n``, ``so1n``, ...).
    """

    def __init__(self, mesh, time_increment, tables=None):
        t, s = tables if tables is not None else mesh_tables(mesh)
        self._t = t
        self.ndim = nd = s["ndim"]
        self.ncell = s["ncell"]
        self.ngstcell = s["ngstcell"]
        self.neq = neq = nd + 2
        tot = self.ncell + self.ngstcell
        self.time_increment = float(time_increment)
        shapes = {"cevol": (tot, 7), "cecnd": (tot, 7 * nd),
                  "sfcnd": (self.ncell, 24, nd), "sfnml": (self.ncell, 24, nd),
                  "so1c": (tot, neq, nd), "so1n": (tot, neq, nd),
                  "cflo": (tot,), "cflc": (tot,), "gamma": (tot,)}
        self._a = {n: np.zeros(shapes.get(n, (tot, neq)), dtype="float64")
                   for n in _EULER_ARRAYS}
        self.limiter = np.zeros(max(self.ncell, 1), dtype="uint8")
        self._s = _OraEuler()
        m = self._s.m
        for k in ("ndim", "nnode", "nface", "ncell", "ngstnode", "ngstface",
                  "ngstcell"):
            setattr(m, k, s[k])
        for n in MESH_NAMES:
            setattr(m, n, t[n].ctypes.data)
        self._s.dt = self.time_increment
        self.sigma0, self.taumin, self.tauscale = 3.0, 0.0, 1.0
        self._bcs = []
        self._sync_ptrs()
        self._set_bc_struct()
        lib().ora_prepare_ce(ctypes.byref(self._s))

    def __getattr__(self, name):
        a = self.__dict__.get("_a")
        if a is not None and name in a:
            return a[name]
        raise AttributeError(name)

    def _sync_ptrs(self):
        for n in _EULER_ARRAYS:
            setattr(self._s, n, self._a[n].ctypes.data)
        self._s.limiter = self.limiter.ctypes.data
        self._s.sigma0 = self.sigma0
        self._s.taumin = self.taumin
        self._s.tauscale = self.tauscale

    def _readback(self):
        # The C march swaps so0c/so0n and so1c/so1n by pointer; map back.
        byaddr = {self._a[n].ctypes.data: self._a[n] for n in
                  ("so0c", "so0n", "so1c", "so1n")}
        for n in ("so0c", "so0n", "so1c", "so1n"):
            self._a[n] = byaddr[getattr(self._s, n)]

    def _set_bc_struct(self):
        nd = self.ndim
        kinds = np.array([b[0] for b in self._bcs] or [0], dtype="int32")
        off = np.zeros(len(self._bcs) + 1, dtype="int64")
        faces = []
        vals = np.zeros((max(len(self._bcs), 1), nd + 3), dtype="float64")
        for i, (k, f, v) in enumerate(self._bcs):
            faces.extend(f)
            off[i + 1] = len(faces)
            if len(v):
                vals[i] = v
        self._bc_arrays = (kinds, off, np.array(faces or [0], dtype="int32"),
                           vals)
        self._s.nbnd = len(self._bcs)
        self._s.bkind = kinds.ctypes.data
        self._s.boff = off.ctypes.data
        self._s.bfaces = self._bc_arrays[2].ctypes.data
        self._s.bval = vals.ctypes.data

    def add_bc(self, kind, faces, value=()):
        self._bcs.append((int(kind), [int(x) for x in faces],
                          [float(x) for x in value]))
        self._set_bc_struct()

    def add_nonrefl(self, faces):
        self.add_bc(0, faces)

    def add_slipwall(self, faces):
        self.add_bc(1, faces)

    def add_inlet(self, faces, value):
        self.add_bc(2, faces, value)

    def init_solution(self, gamma, rho, v, p):
        nd = self.ndim
        vsq = sum(float(x) * float(x) for x in v[:nd])
        energy = p / (gamma - 1.0) + 0.5 * rho * vsq
        self._a["gamma"][:] = gamma
        body = self._a["so0n"][self.ngstcell:]
        body[:, 0] = rho
        for d in range(nd):
            body[:, 1 + d] = rho * v[d]
        body[:, nd + 1] = energy

    def call(self, op):
        self._sync_ptrs()
        getattr(lib(), "ora_" + op)(ctypes.byref(self._s))
        self._readback()

    def march(self, steps):
        self._sync_ptrs()
        lib().ora_march(ctypes.byref(self._s), int(steps))
        self._readback()


class _OraE1D(ctypes.Structure):
    _fields_ = [("ncoord", ctypes.c_int64), ("dt", ctypes.c_double),
                ("coord", _P), ("cfl", _P), ("so0", _P), ("so1", _P),
                ("gamma", _P)]


class OracleEuler1D:
    """The reference onedim Euler1DCore restated on the CPU."""

    def __init__(self, ncoord, time_increment):
        if ncoord % 2 == 0:
            raise ValueError("ncoord cannot be even")
        self.ncoord = ncoord
        self.coord = np.zeros(ncoord)
        self.cfl = np.zeros(ncoord)
        self.so0 = np.zeros((ncoord, 3))
        self.so1 = np.zeros((ncoord, 3))
        self.gamma = np.full(ncoord, 1.4)
        self._s = _OraE1D(ncoord, float(time_increment), self.coord.ctypes.data,
                          self.cfl.ctypes.data, self.so0.ctypes.data,
                          self.so1.ctypes.data, self.gamma.ctypes.data)

    def setup_march(self):
        lib().ora_e1d_update_cfl(ctypes.byref(self._s), 0)

    def march_alpha(self, alpha, steps):
        lib().ora_e1d_march(ctypes.byref(self._s), int(alpha), int(steps))


class _OraST(ctypes.Structure):
    _fields_ = [("ncelm", ctypes.c_int64), ("kind", ctypes.c_int32),
                ("dt", ctypes.c_double), ("xcoord", _P), ("so0", _P),
                ("so1", _P), ("cfl", _P)]


class OracleSpacetime:
    """The reference spacetime LinearScalar (kind 0) / InviscidBurgers
    (kind 1) solver restated on the CPU; arrays are whole [2 ncelm + 5]
    tables."""

    def __init__(self, kind, xcoord, time_increment):
        self.xcoord = np.ascontiguousarray(xcoord, dtype="float64").copy()
        n = self.xcoord.size
        self.ncelm = (n - 5) // 2
        self.so0 = np.zeros(n)
        self.so1 = np.zeros(n)
        self.cfl = np.zeros(n)
        self._s = _OraST(self.ncelm, int(kind), float(time_increment),
                         self.xcoord.ctypes.data, self.so0.ctypes.data,
                         self.so1.ctypes.data, self.cfl.ctypes.data)
        lib().ora_st_setup.argtypes = [ctypes.c_void_p]
        lib().ora_st_march.argtypes = [ctypes.c_void_p, ctypes.c_int,
                                       ctypes.c_int64]

    def setup_march(self):
        lib().ora_st_setup(ctypes.byref(self._s))

    def march_alpha(self, alpha, steps):
        lib().ora_st_march(ctypes.byref(self._s), int(alpha), int(steps))
