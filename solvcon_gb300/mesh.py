"""Unstructured mixed-element mesh with a mirrored ghost layer.

Mirrors solvcon's ``StaticMesh`` Python surface
(cpp/solvcon/mesh/pymod/wrap_StaticMesh.cpp:61-181): the constructor
``StaticMesh(ndim, nnode, nface=0, ncell=0)``, the cell-type constants, the
size properties, ``build_interior``/``build_boundary``/``build_ghost``/
``build_edge``, ``add_bc``/``bc``/``bcs`` and the fifteen table properties as
ghost-aware :class:`~solvcon_gb300.buffer.SimpleArray` views.  The tables live
in the native library (host memory) and the views alias them.
"""

import ctypes

import numpy as np

from ._lib import check, lib, ptr
from .buffer import SimpleArray

__all__ = ["StaticMesh", "StaticMeshBc", "Gmsh", "Plot3d"]

_ARRAYS = ("ndcrd", "fccnd", "fcnml", "fcara", "clcnd", "clvol", "fctpn",
           "cltpn", "clgrp", "fcnds", "fccls", "clnds", "clfcs", "ednds",
           "bndfcs")


_GPUS = None


def _gpu_count():
    global _GPUS
    if _GPUS is None:
        n = ctypes.c_int()
        check(lib.scg_device_count(ctypes.byref(n)))
        _GPUS = n.value
    return _GPUS


class StaticMeshBc:
    """A boundary group of a :class:`StaticMesh` (StaticMesh.hpp:159-251)."""

    def __init__(self, name, facn):
        self.name = name
        # [nbound, 3] face table as a SimpleArray (facn.ndarray is the
        # numpy array, as in the reference's BC object).
        self.facn = SimpleArray(lambda: facn)

    @property
    def nbound(self):
        return self.facn.shape[0]


class StaticMesh:
    """Mixed-element unstructured mesh (StaticMesh.hpp:264-456)."""

    NONCELLTYPE = 0
    POINT = 1
    LINE = 2
    QUADRILATERAL = 3
    TRIANGLE = 4
    HEXAHEDRON = 5
    TETRAHEDRON = 6
    PRISM = 7
    PYRAMID = 8

    FCMND = 4
    CLMND = 8
    CLMFC = 6
    FCREL = 4
    BFREL = 3

    def __init__(self, ndim, nnode, nface=0, ncell=0):
        h = ctypes.c_void_p()
        check(lib.scg_mesh_create(int(ndim), int(nnode), int(nface),
                                  int(ncell), ctypes.byref(h)))
        self._h = h

    _SIZES = ("ndim", "nnode", "nface", "ncell", "nbound", "ngstnode",
              "ngstface", "ngstcell", "nedge")

    @classmethod
    def from_mesh(cls, other):
        """Not in the reference: take over a mesh built by other code -- the
        reference's own ``solvcon.StaticMesh`` (from its Gmsh reader, a pilot
        driver, or ``build_interior``/``build_boundary``/``build_ghost``) or
        any object with the same surface -- with every table copied
        verbatim and nothing rebuilt, so that its cells, faces and ghost
        layer march on the GPU exactly as numbered there.

        ``other`` needs the size properties (``ndim`` ... ``nedge``), the
        fifteen table properties whose ``.ndarray`` is the whole buffer with
        the ghost rows first (wrap_StaticMesh.cpp:61-181), and optionally
        ``bcs`` (objects with ``name`` and ``facn``)."""
        sizes = np.array([int(getattr(other, k)) for k in cls._SIZES],
                         dtype="int64")
        nd, nnode, nface, ncell, nbound, gnode, gface, gcell, nedge = \
            (int(x) for x in sizes)
        rows = {"node": gnode + nnode, "face": gface + nface,
                "cell": gcell + ncell}
        shape = {"ndcrd": ("node", nd), "fccnd": ("face", nd),
                 "fcnml": ("face", nd), "fcara": ("face", 1),
                 "clcnd": ("cell", nd), "clvol": ("cell", 1),
                 "fctpn": ("face", 1), "cltpn": ("cell", 1),
                 "clgrp": ("cell", 1), "fcnds": ("face", cls.FCMND + 1),
                 "fccls": ("face", cls.FCREL),
                 "clnds": ("cell", cls.CLMND + 1),
                 "clfcs": ("cell", cls.CLMFC + 1)}
        keep = []
        ptrs = (ctypes.c_void_p * len(_ARRAYS))()
        for i, name in enumerate(_ARRAYS):
            dtype = "int32" if i >= _ARRAYS.index("fctpn") else "float64"
            arr = getattr(other, name)
            arr = getattr(arr, "ndarray", arr)
            buf = np.ascontiguousarray(arr, dtype=dtype)
            if name == "ednds":
                want = nedge * 2
            elif name == "bndfcs":
                want = nbound * cls.BFREL
            else:
                kind, width = shape[name]
                want = rows[kind] * width
            if buf.size != want:
                raise ValueError("StaticMesh.from_mesh: %s holds %d values, "
                                 "the sizes need %d" % (name, buf.size, want))
            keep.append(buf)
            ptrs[i] = buf.ctypes.data if buf.size else None
        h = ctypes.c_void_p()
        check(lib.scg_mesh_from_tables(ptr(sizes), ptrs, ctypes.byref(h)))
        self = cls._adopt(h)
        for bc in getattr(other, "bcs", ()) or ():
            facn = getattr(bc.facn, "ndarray", bc.facn)
            facn = np.ascontiguousarray(facn, dtype="int32").reshape(-1, 3)
            check(lib.scg_mesh_adopt_bc(h, str(bc.name).encode(), ptr(facn),
                                        facn.shape[0]))
        return self

    @classmethod
    def _adopt(cls, handle):
        """Wrap a native scg_mesh handle (the wrapper destroys it)."""
        self = cls.__new__(cls)
        self._h = handle
        return self

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.scg_mesh_destroy(h)
            self._h = None

    @property
    def handle(self):
        """The native scg_mesh handle (for the C ABI)."""
        return self._h

    # -- sizes --------------------------------------------------------------

    def _sizes(self):
        out = np.zeros(10, dtype="int64")
        check(lib.scg_mesh_sizes(self._h, ptr(out)))
        return out

    ndim = property(lambda self: int(self._sizes()[0]))
    nnode = property(lambda self: int(self._sizes()[1]))
    nface = property(lambda self: int(self._sizes()[2]))
    ncell = property(lambda self: int(self._sizes()[3]))
    nbound = property(lambda self: int(self._sizes()[4]))
    ngstnode = property(lambda self: int(self._sizes()[5]))
    ngstface = property(lambda self: int(self._sizes()[6]))
    ngstcell = property(lambda self: int(self._sizes()[7]))
    nedge = property(lambda self: int(self._sizes()[8]))
    nbcs = property(lambda self: int(self._sizes()[9]))

    # -- builds -------------------------------------------------------------

    #: Meshes at least this large build their interior on the GPU when one
    #: is present (``build_interior(device=None)``).
    DEVICE_BUILD_CELLS = 65536

    def build_interior(self, do_metric=True, build_edge=True, device=None):
        """Faces, face-cell relations and (with ``do_metric``) the metrics
        (StaticMesh::build_interior).  ``device=True`` builds them on the GPU,
        ``False`` on the host; ``None`` picks the GPU for meshes of at least
        :attr:`DEVICE_BUILD_CELLS` cells when one is present.  Both give the
        same tables entry for entry."""
        if device is None:
            device = self.ncell >= self.DEVICE_BUILD_CELLS and _gpu_count() > 0
        fn = lib.scg_mesh_build_interior_device if device else \
            lib.scg_mesh_build_interior
        check(fn(self._h, int(bool(do_metric)), int(bool(build_edge))))

    def build_edge(self):
        check(lib.scg_mesh_build_edge(self._h))

    def build_boundary(self):
        check(lib.scg_mesh_build_boundary(self._h))

    def build_ghost(self):
        check(lib.scg_mesh_build_ghost(self._h))

    def add_bc(self, name, faces):
        f = np.ascontiguousarray(faces, dtype="int32")
        check(lib.scg_mesh_add_bc(self._h, name.encode(), ptr(f), f.size))
        return self.bc(self.nbcs - 1)

    def bc(self, key):
        if isinstance(key, str):
            for b in self.bcs:
                if b.name == key:
                    return b
            raise KeyError(key)
        buf = ctypes.create_string_buffer(256)
        nb = ctypes.c_int64()
        check(lib.scg_mesh_bc(self._h, int(key), buf, 256, None,
                              ctypes.byref(nb)))
        facn = np.zeros((nb.value, 3), dtype="int32")
        check(lib.scg_mesh_bc(self._h, int(key), buf, 256, ptr(facn),
                              ctypes.byref(nb)))
        return StaticMeshBc(buf.value.decode(), facn)

    @property
    def bcs(self):
        return [self.bc(i) for i in range(self.nbcs)]

    # -- tables -------------------------------------------------------------

    def _table(self, which):
        data = ctypes.c_void_p()
        shape = np.zeros(3, dtype="int64")
        nd = ctypes.c_int()
        ngh = ctypes.c_int64()
        dt = ctypes.c_int()
        check(lib.scg_mesh_array(self._h, which, ctypes.byref(data),
                                 ptr(shape), ctypes.byref(nd),
                                 ctypes.byref(ngh), ctypes.byref(dt)))
        ctype = ctypes.c_double if dt.value == 0 else ctypes.c_int32
        dtype = "float64" if dt.value == 0 else "int32"
        n = int(shape[0] * shape[1])
        shp = (int(shape[0]), int(shape[1])) if nd.value == 2 else \
            (int(shape[0]),)
        if n == 0 or not data.value:
            return np.zeros(shp, dtype=dtype), int(ngh.value)
        raw = (ctype * n).from_address(data.value)
        raw._owner = self  # keep the mesh (and its buffers) alive
        return np.frombuffer(raw, dtype=dtype).reshape(shp), int(ngh.value)

    def _view(self, which):
        return SimpleArray(lambda: self._table(which)[0],
                           nghost=self._table(which)[1])


def _make_prop(i):
    return property(lambda self: self._view(i))


for _i, _name in enumerate(_ARRAYS):
    setattr(StaticMesh, _name, _make_prop(_i))
del _i, _name, _make_prop


class Gmsh:
    """Gmsh MSH 2.2 (ASCII) reader (cpp/solvcon/inout/gmsh.hpp:70-285,
    wrapped as ``solvcon.Gmsh``): ``Gmsh(data).to_block()`` gives the
    :class:`StaticMesh` of the file's highest-dimension elements, with the
    interior, boundary and ghost tables built.  ``data`` is the file's
    contents (bytes or str); the parsing is native."""

    def __init__(self, data):
        if isinstance(data, str):
            data = data.encode()
        self._data = bytes(data)
        # Parse now, as the reference's constructor does, so a malformed
        # file raises here.
        self._mesh = self._read()

    def _read(self):
        h = ctypes.c_void_p()
        check(lib.scg_mesh_from_gmsh(self._data, len(self._data),
                                     ctypes.byref(h)))
        return StaticMesh._adopt(h)

    def to_block(self):
        """The mesh (a new StaticMesh on each call)."""
        mesh, self._mesh = self._mesh, None
        return mesh if mesh is not None else self._read()


class Plot3d:
    """Plot3D multi-block ASCII grid reader (cpp/solvcon/inout/plot3d.hpp:
    22-80, wrapped as ``solvcon.core.Plot3d``): ``Plot3d(data).to_block()``
    gives the :class:`StaticMesh` of one hexahedron per grid cell, with the
    interior, boundary and ghost tables built.  The parsing is native."""

    def __init__(self, data):
        if isinstance(data, str):
            data = data.encode()
        self._data = bytes(data)
        self._mesh = self._read()

    def _read(self):
        h = ctypes.c_void_p()
        check(lib.scg_mesh_from_plot3d(self._data, len(self._data),
                                       ctypes.byref(h)))
        return StaticMesh._adopt(h)

    def to_block(self):
        """The mesh (a new StaticMesh on each call)."""
        mesh, self._mesh = self._mesh, None
        return mesh if mesh is not None else self._read()

