"""GPU multi-dimensional Euler CESE core with solvcon's EulerCore surface.

``EulerCore(mesh, time_increment)`` mirrors the reference class bound in
cpp/solvcon/multidim/pymod/wrap_multidim.cpp:184-414 (methods, properties,
argument names, exception types).  The solution lives on the GPU; every array
property returns a ghost-aware :class:`~solvcon_gb300.buffer.SimpleArray`
backed by a host mirror that this class keeps coherent:

* a read fetches the table from the device once and serves it from the mirror
  until the next device operation;
* a write (``arr[i, j] = v``, ``arr.fill``, or writes through ``arr.ndarray``)
  is pushed back to the device before the next device operation;
* ``update()`` swaps the so0c/so0n and so1c/so1n mirrors as the reference swaps
  its buffers (euler.hpp:123-127), so a view taken before keeps aliasing the
  same physical table.

``march`` runs entirely on the device; nothing is copied unless an array is
read.
"""

import ctypes

import numpy as np

from ._lib import check, lib, ptr
from .buffer import SimpleArray

__all__ = ["EulerCore", "GradientElement", "PRECISIONS"]

ARRAYS = ("cevol", "cecnd", "sfcnd", "sfnml", "so0c", "so0n", "so0t", "so1c",
          "so1n", "stm", "cflo", "cflc", "gamma")
_ID = {n: i for i, n in enumerate(ARRAYS)}
_OPS = {"prepare_ce": 0, "update": 1, "calc_solt": 2, "calc_soln": 3,
        "bc_soln": 4, "calc_cfl": 5, "calc_dsoln": 6, "bc_dsoln": 7,
        "march_substep": 8, "reset_state": 9}
# "fp32" is the FP32 form (FP32 state and flux, FP64 geometry tables);
# "fp32-geom64" names the same; "fp32-geom32" also stores the geometry FP32.
PRECISIONS = {"fp64": 0, "fp32": 1, "fp32-geom64": 1, "fp32-geom32": 2}
_SWAP = (("so0c", "so0n"), ("so1c", "so1n"))


class EulerCore:
    """Solve the Euler equations with the CESE method on the GPU.

    :param mesh: a :class:`~solvcon_gb300.mesh.StaticMesh` with its ghost
        layer built, or a mesh built by other code with the reference
        StaticMesh surface (the reference's own ``solvcon.StaticMesh``),
        whose tables are then taken over verbatim
        (:meth:`StaticMesh.from_mesh`).
    :param time_increment: the fixed time step.
    :param precision: ``"fp64"`` (the reference's arithmetic), ``"fp32"``
        (not in the reference: FP32 state and flux arithmetic with
        compensated face sums, the mesh geometry in FP64 tables, totals and
        the CFL reduction in FP64; ``"fp32-geom64"`` is the same) or
        ``"fp32-geom32"`` (the same march with the geometry, computed in FP64,
        stored in FP32: less traffic, slightly larger error).
    """

    SUBSTEP_RUN = 2

    def __init__(self, mesh, time_increment, precision="fp64"):
        if precision not in PRECISIONS:
            raise ValueError("EulerCore: precision must be one of %s" %
                             sorted(PRECISIONS))
        if not hasattr(mesh, "handle"):
            from .mesh import StaticMesh
            mesh = StaticMesh.from_mesh(mesh)
        h = ctypes.c_void_p()
        check(lib.scg_euler_create(mesh.handle, float(time_increment),
                                   PRECISIONS[precision], ctypes.byref(h)))
        self._h = h
        self._mesh = mesh
        self._precision = precision
        info = np.zeros(5, dtype="int64")
        check(lib.scg_euler_info(h, ptr(info)))
        self._ndim, self._ncell, self._ngstcell, self._neq = \
            (int(x) for x in info[:4])
        self._cache = {}
        self._valid = set()
        self._dirty = set()
        self._exposed = set()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.scg_euler_destroy(h)
            self._h = None

    # -- plain properties ---------------------------------------------------

    handle = property(lambda self: self._h)
    mesh = property(lambda self: self._mesh)
    ndim = property(lambda self: self._ndim)
    ncell = property(lambda self: self._ncell)
    ngstcell = property(lambda self: self._ngstcell)
    neq = property(lambda self: self._neq)
    precision = property(lambda self: self._precision)

    def _param(self, which):
        v = ctypes.c_double()
        check(lib.scg_euler_get_param(self._h, which, ctypes.byref(v)))
        return v.value

    def _set_param(self, which, value):
        check(lib.scg_euler_set_param(self._h, which, float(value)))

    time_increment = property(lambda self: self._param(3))
    sigma0 = property(lambda self: self._param(0),
                      lambda self, v: self._set_param(0, v))
    taumin = property(lambda self: self._param(1),
                      lambda self, v: self._set_param(1, v))
    tauscale = property(lambda self: self._param(2),
                        lambda self, v: self._set_param(2, v))

    @property
    def device_bytes(self):
        out = ctypes.c_int64()
        check(lib.scg_euler_device_bytes(self._h, ctypes.byref(out)))
        return out.value

    # -- host mirror --------------------------------------------------------

    def _shape(self, i):
        shape = np.zeros(3, dtype="int64")
        nd = ctypes.c_int()
        ngh = ctypes.c_int64()
        check(lib.scg_euler_array_shape(self._h, i, ptr(shape),
                                        ctypes.byref(nd), ctypes.byref(ngh)))
        return tuple(int(s) for s in shape[:nd.value]), int(ngh.value)

    def _host(self, name):
        if name not in self._valid:
            i = _ID[name]
            shape, _ = self._shape(i)
            buf = self._cache.get(name)
            if buf is None or buf.shape != shape:
                buf = np.empty(shape, dtype="float64")
                self._cache[name] = buf
            check(lib.scg_euler_get(self._h, i, ptr(buf), buf.size))
            self._valid.add(name)
        return self._cache[name]

    def _written(self, name):
        self._dirty.add(name)

    def _exposed_view(self, name):
        # A caller holding the raw buffer may write through it at any time:
        # push it before, and refresh it after, every device operation.
        self._dirty.add(name)
        self._exposed.add(name)

    def _flush(self):
        for name in sorted(self._dirty | self._exposed):
            if name in self._valid:
                buf = self._cache[name]
                check(lib.scg_euler_set(self._h, _ID[name], ptr(buf),
                                        buf.size))
        self._dirty.clear()

    def _after(self, nswap=0):
        self._valid.clear()
        if nswap % 2:
            for a, b in _SWAP:
                ca, cb = self._cache.get(a), self._cache.get(b)
                self._cache[a], self._cache[b] = cb, ca
                for s in (self._exposed,):
                    ina, inb = a in s, b in s
                    s.discard(a)
                    s.discard(b)
                    if ina:
                        s.add(b)
                    if inb:
                        s.add(a)
                for k in (a, b):
                    if self._cache.get(k) is None:
                        self._cache.pop(k, None)
        for name in list(self._exposed):
            self._host(name)

    def _array(self, name):
        _, ngh = self._shape(_ID[name])
        return SimpleArray(lambda: self._host(name), nghost=ngh,
                           on_write=lambda: self._written(name),
                           on_expose=lambda: self._exposed_view(name))

    def release_views(self):
        """Stop mirroring the raw buffers handed out by ``arr.ndarray``
        (writes through them are no longer pushed to the device)."""
        self._flush()
        self._exposed.clear()

    # -- operations ---------------------------------------------------------

    def _op(self, name, nswap=0):
        self._flush()
        check(lib.scg_euler_op(self._h, _OPS[name]))
        self._after(nswap)

    def prepare_ce(self):
        self._op("prepare_ce")

    def init_solution(self, gamma, rho, v, p):
        v = [float(x) for x in v]
        if len(v) != self._ndim:
            raise ValueError("EulerCore::init_solution: velocity size %d "
                             "must equal ndim %d" % (len(v), self._ndim))
        self._flush()
        vv = np.asarray(v + [0.0] * (3 - len(v)), dtype="float64")
        check(lib.scg_euler_init_solution(self._h, float(gamma), float(rho),
                                          ptr(vv), len(v), float(p)))
        self._after()

    def update(self):
        self._op("update", nswap=1)

    def reset_state(self):
        """Not in the reference: put the solution state back to that of a
        new core (all solution arrays, CFL numbers and gamma zero), keeping
        the mesh, the CE geometry and the boundary conditions, so a core can
        be reused for another solve on the same mesh."""
        self._op("reset_state")

    def calc_solt(self):
        self._op("calc_solt")

    def calc_soln(self):
        self._op("calc_soln")

    def calc_cfl(self):
        self._op("calc_cfl")

    def calc_dsoln(self):
        self._op("calc_dsoln")

    def bc_soln(self):
        self._op("bc_soln")

    def bc_dsoln(self):
        self._op("bc_dsoln")

    def march_substep(self):
        self._op("march_substep", nswap=1)

    def march(self, steps):
        """Advance ``steps`` full steps (SUBSTEP_RUN substeps each) and wait
        for the device."""
        self.march_async(steps)
        self.sync()

    def march_async(self, steps):
        """Enqueue ``steps`` full steps on the core's stream and return."""
        self._flush()
        check(lib.scg_euler_march(self._h, int(steps)))
        self._valid.clear()
        if self._exposed:
            self.sync()
            self._after(0)

    def sync(self):
        check(lib.scg_euler_sync(self._h))

    # -- host tables exchanged every step (not in the reference) -------------

    def host_table(self, name):
        """A :class:`~solvcon_gb300.host.HostTable` shaped for array ``name``
        (``"so0n"``, ``"so1n"``, ...), ghost rows first."""
        from .host import HostTable
        shape, _ = self._shape(_ID[name])
        return HostTable(shape)

    def deliver(self, so0n=None, so1n=None):
        """Have every later march leave its new so0n / so1n in these
        :class:`~solvcon_gb300.host.HostTable` objects (None: stop), as it
        computes them (FP64) or right after (FP32); scg_euler_deliver."""
        for name, t in (("so0n", so0n), ("so1n", so1n)):
            if t is None:
                check(lib.scg_euler_deliver(self._h, _ID[name], None, 0))
            else:
                check(lib.scg_euler_deliver(self._h, _ID[name],
                                            ctypes.c_void_p(t.address), t.size))

    def march_from_host(self, so0n, so1n, steps):
        """Set so0n and so1n from host tables and advance ``steps`` full
        steps, waiting for the device; with :class:`HostTable` tables the
        upload runs while the first substep already marches the cells whose
        rows are up (scg_euler_march_from_host).  Same state as setting the
        two arrays and calling :meth:`march`, bit for bit."""
        tabs = []
        for name, t in (("so0n", so0n), ("so1n", so1n)):
            shape, _ = self._shape(_ID[name])
            if hasattr(t, "address"):
                if tuple(t.shape) != tuple(shape):
                    raise ValueError("EulerCore.march_from_host: %s has shape "
                                     "%s, not %s" % (name, t.shape, shape))
                tabs.append((ctypes.c_void_p(t.address), t.size))
            else:
                arr = np.ascontiguousarray(t, dtype="float64")
                if arr.shape != tuple(shape):
                    raise ValueError("EulerCore.march_from_host: %s has shape "
                                     "%s, not %s" % (name, arr.shape, shape))
                tabs.append((ptr(arr), arr.size, arr))
        self._flush()
        check(lib.scg_euler_march_from_host(self._h, tabs[0][0], tabs[0][1],
                                            tabs[1][0], tabs[1][1], int(steps)))
        self._valid.clear()
        self.sync()
        if self._exposed:
            self._after(0)

    def set_stream(self, cuda_stream):
        """Run on a caller-owned cudaStream_t (an int address or None)."""
        check(lib.scg_euler_set_stream(self._h, ctypes.c_void_p(
            int(cuda_stream) if cuda_stream else None)))

    # -- boundary conditions ------------------------------------------------

    def _add_bc(self, kind, faces, value=()):
        f = np.ascontiguousarray([int(x) for x in faces], dtype="int32")
        v = np.ascontiguousarray([float(x) for x in value], dtype="float64")
        check(lib.scg_euler_add_bc(self._h, kind, ptr(f), f.size,
                                   ptr(v) if v.size else None, v.size))

    def add_nonrefl(self, faces):
        self._add_bc(0, faces)

    def add_slipwall(self, faces):
        self._add_bc(1, faces)

    def add_inlet(self, faces, value):
        self._add_bc(2, faces, value)

    def clear_bc(self):
        check(lib.scg_euler_clear_bc(self._h))

    def get_normal_matrix(self, ifc):
        out = np.zeros(self._ndim * self._ndim, dtype="float64")
        check(lib.scg_euler_normal_matrix(self._h, int(ifc), ptr(out)))
        return out.reshape(self._ndim, self._ndim).tolist()

    # -- diagnostics beyond the reference surface ---------------------------

    def limiter_mask(self):
        """W-3/4 firing bits of the last calc_dsoln, one uint8 per body cell
        (bit i: equation i had sigma_max capped below sigma0/|cfl|)."""
        out = np.zeros(max(self._ncell, 1), dtype="uint8")
        check(lib.scg_euler_limiter_mask(self._h, ptr(out)))
        return out[:self._ncell]

    def totals(self):
        """FP64 totals of so0n * clvol over the body cells, per equation."""
        self._flush()
        out = np.zeros(self._neq, dtype="float64")
        check(lib.scg_euler_totals(self._h, ptr(out)))
        return out

    def cfl_range(self):
        """(min, max) of cflo over the body cells."""
        self._flush()
        out = np.zeros(2, dtype="float64")
        check(lib.scg_euler_cfl_range(self._h, ptr(out)))
        return float(out[0]), float(out[1])

    #: Scalar fields :meth:`device_field` derives on the device, by id.
    DEVICE_FIELDS = {"density": 0, "velx": 1, "vely": 2, "velz": 3,
                     "speed": 4, "pressure": 5, "mach": 6,
                     "total_energy": 7, "cfl": 8}

    def device_field(self, name):
        """One scalar field of the newest solution over the body cells
        (one of :attr:`DEVICE_FIELDS`), derived on the device in FP64; only
        ``ncell`` doubles cross to the host."""
        if name not in self.DEVICE_FIELDS:
            raise ValueError("unknown field '%s'" % name)
        self._flush()
        out = np.zeros(max(self._ncell, 1), dtype="float64")
        check(lib.scg_euler_field(self._h, self.DEVICE_FIELDS[name], ptr(out)))
        return out[:self._ncell]


def _make_prop(name):
    return property(lambda self: self._array(name))


for _n in ARRAYS:
    setattr(EulerCore, _n, _make_prop(_n))
del _n


class GradientElement:
    """Per-cell gradient element geometry: solvcon's GradientElement
    (cpp/solvcon/multidim/GradientElement.cpp:137-290, the sub-element table
    at :16-79) with the bounds-checked accessors of its Python wrapper
    (cpp/solvcon/multidim/pymod/wrap_multidim.cpp:42-204).

    Host-side helper with the reference's accessors (``rcl``, ``idis``,
    ``jdis``, ``faces``, ``displacement_matrix``, ``solve_gradient``); the
    march itself evaluates the same geometry inside its kernels.  Face and
    dimension indices out of range raise ``IndexError``; a ``udf`` whose
    length is not ``ndim`` raises ``ValueError``.
    """

    _FGE = {
        3: [(1, 2), (2, 3), (3, 4), (4, 1)],
        4: [(1, 2), (2, 3), (3, 1)],
        5: [(2, 3, 5), (6, 3, 2), (4, 3, 6), (5, 3, 4),
            (5, 1, 2), (2, 1, 6), (6, 1, 4), (4, 1, 5)],
        6: [(3, 1, 2), (2, 1, 4), (4, 1, 3), (2, 4, 3)],
        7: [(5, 2, 4), (3, 2, 5), (4, 2, 3), (4, 1, 5), (5, 1, 3),
            (3, 1, 4)],
        8: [(1, 5, 2), (2, 5, 3), (3, 5, 4), (4, 5, 1), (1, 3, 4),
            (3, 1, 2)],
    }

    def __init__(self, mesh, cecnd, icl, tau):
        nd = mesh.ndim
        if nd not in (2, 3):
            raise ValueError("GradientElement: ndim must be 2 or 3")
        self.icl = int(icl)
        self.ndim = nd
        self.clnfc = int(mesh.clfcs[icl, 0])
        self._fge = self._FGE[int(mesh.cltpn[icl])]
        self.nfge = len(self._fge)
        self.nfge_inverse = 1.0 / self.nfge
        ice = np.array([cecnd[icl, d] for d in range(nd)])
        gp = np.zeros((self.clnfc, nd))
        jd = np.zeros((self.clnfc, nd))
        self._rcl = []
        for ifl in range(self.clnfc):
            ifc = mesh.clfcs[icl, ifl + 1]
            jcl = mesh.fccls[ifc, 0] + mesh.fccls[ifc, 1] - icl
            self._rcl.append(int(jcl))
            mid = np.array([cecnd[icl, (ifl + 1) * nd + d]
                            for d in range(nd)])
            jce = np.array([cecnd[jcl, d] if jcl >= 0 else mesh.clcnd[jcl, d]
                            for d in range(nd)])
            gp[ifl] = mid + tau * (jce - mid)
            jd[ifl] = gp[ifl] - jce
        avg = gp.mean(axis=0)
        cnd = np.zeros(nd)
        voc = 0.0
        for fl in self._fge:
            idx = [f - 1 for f in fl]
            sub = (avg + gp[idx].sum(axis=0)) / (nd + 1)
            vob = np.linalg.det(gp[idx] - avg)
            voc += vob
            cnd += sub * vob
        cnd /= voc
        self._idis = gp - cnd
        self._jdis = jd + ice - cnd

    def _chk_ifl(self, ifl):
        if ifl < 0 or ifl >= self.clnfc:
            raise IndexError("GradientElement: ifl %d out of range [0, %d)" %
                             (ifl, self.clnfc))

    def _chk_d(self, d):
        if d < 0 or d >= self.ndim:
            raise IndexError("GradientElement: d %d out of range [0, %d)" %
                             (d, self.ndim))

    def _chk_ifge(self, ifge):
        if ifge < 0 or ifge >= self.nfge:
            raise IndexError("GradientElement: ifge %d out of range [0, %d)"
                             % (ifge, self.nfge))

    def rcl(self, ifl):
        self._chk_ifl(ifl)
        return self._rcl[ifl]

    def idis(self, ifl, d):
        self._chk_ifl(ifl)
        self._chk_d(d)
        return float(self._idis[ifl, d])

    def jdis(self, ifl, d):
        self._chk_ifl(ifl)
        self._chk_d(d)
        return float(self._jdis[ifl, d])

    def faces(self, ifge):
        self._chk_ifge(ifge)
        return list(self._fge[ifge])

    def displacement_matrix(self, ifge):
        self._chk_ifge(ifge)
        return self._idis[[f - 1 for f in self._fge[ifge]]].tolist()

    def solve_gradient(self, ifge, udf):
        self._chk_ifge(ifge)
        if len(udf) != self.ndim:
            raise ValueError("GradientElement: udf size %d must equal ndim %d"
                             % (len(udf), self.ndim))
        # Cramer's rule with the inverse's columns written as cross products
        # of the rows (3D) or the rotated rows (2D): grad = adj(dst) udf /
        # det(dst), as the reference computes it, so a degenerate element
        # gives inf/nan rather than an exception.
        r = np.array(self.displacement_matrix(ifge), dtype="float64")
        u = np.asarray(udf, dtype="float64")
        if self.ndim == 2:
            c = np.array([[r[1, 1], -r[0, 1]], [-r[1, 0], r[0, 0]]])
            det = r[0, 0] * r[1, 1] - r[0, 1] * r[1, 0]
        else:
            c = np.stack([np.cross(r[1], r[2]), np.cross(r[2], r[0]),
                          np.cross(r[0], r[1])], axis=1)
            det = float(r[0] @ c[:, 0])
        with np.errstate(divide="ignore", invalid="ignore"):
            return (c @ u / np.float64(det)).tolist()
