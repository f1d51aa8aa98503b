"""GPU 1D Euler CESE solver with solvcon's onedim surface.

* :class:`Euler1DCore` mirrors ``solvcon.onedim`` ``Euler1DCore``
  (cpp/solvcon/onedim/pymod/wrap_onedim.cpp:18-162): arrays ``coord``, ``cfl``,
  ``so0``, ``so1``, ``gamma``; derived ``density``, ``velocity``,
  ``pressure``, ``temperature``, ``internal_energy``, ``entropy``; the
  fine-grained half-step methods and ``march_alpha1``/``march_alpha2``.
* :class:`Euler1DSolver` and :class:`ShockTube` mirror
  solvcon/onedim/euler1d.py:21-393 (grid set-up and the exact Riemann solution
  of the shock tube).
"""

import ctypes

import numpy as np

from . import _lib
from ._lib import check, ptr
from .buffer import SimpleArray

__all__ = ["Euler1DCore", "Euler1DSolver", "ShockTube"]

_vp = ctypes.c_void_p
lib = _lib.bind_more({
    "scg_e1d_create": ([ctypes.c_int64, ctypes.c_double, _vp], ctypes.c_int),
    "scg_e1d_create_precision": ([ctypes.c_int64, ctypes.c_double,
                                  ctypes.c_int, _vp], ctypes.c_int),
    "scg_e1d_precision": ([_vp, _vp], ctypes.c_int),
    "scg_e1d_destroy": ([_vp], ctypes.c_int),
    "scg_e1d_clone": ([_vp, _vp], ctypes.c_int),
    "scg_e1d_info": ([_vp, _vp, _vp], ctypes.c_int),
    "scg_e1d_get": ([_vp, ctypes.c_int, _vp, ctypes.c_int64], ctypes.c_int),
    "scg_e1d_set": ([_vp, ctypes.c_int, _vp, ctypes.c_int64], ctypes.c_int),
    "scg_e1d_op": ([_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int],
                   ctypes.c_int),
    "scg_e1d_march": ([_vp, ctypes.c_int, ctypes.c_int64], ctypes.c_int),
    "scg_e1d_sync": ([_vp], ctypes.c_int),
    "scg_e1d_stream": ([_vp, _vp], ctypes.c_int),
})

_IDS = {"coord": 0, "cfl": 1, "so0": 2, "so1": 3, "gamma": 4}
R_GAS = 8.31446261815324  # Euler1DCore::R (Euler1DCore.hpp:48)
TINY = 1.e-100            # Euler1DCore::TINY (Euler1DCore.hpp:47)


_E1D_PRECISIONS = {"fp64": 0, "fp32": 2}


class Euler1DCore:
    """1D Euler CESE core on the GPU (Euler1DCore.hpp:39-142).

    :param precision: ``"fp64"`` (the reference's arithmetic) or ``"fp32"``
        (FP32 state, CFL and gamma, marched in delta form; coordinates
        kept FP64 and the spacing between them rounded once to FP32; not
        in the reference).
    """

    nvar = 3

    def __init__(self, ncoord, time_increment, precision="fp64",
                 _handle=None):
        h = ctypes.c_void_p()
        if _handle is None:
            if precision not in _E1D_PRECISIONS:
                raise ValueError("Euler1DCore: precision must be one of %s"
                                 % sorted(_E1D_PRECISIONS))
            check(lib.scg_e1d_create_precision(
                int(ncoord), float(time_increment),
                _E1D_PRECISIONS[precision], ctypes.byref(h)))
        else:
            h = _handle
        self._h = h
        n = ctypes.c_int64()
        dt = ctypes.c_double()
        check(lib.scg_e1d_info(h, ctypes.byref(n), ctypes.byref(dt)))
        self._n, self._dt = n.value, dt.value
        code = ctypes.c_int()
        check(lib.scg_e1d_precision(h, ctypes.byref(code)))
        self._precision = {v: k for k, v in _E1D_PRECISIONS.items()}[
            code.value]
        self._cache = {}
        self._valid = set()
        self._dirty = set()
        self._exposed = set()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib.scg_e1d_destroy(h)
            self._h = None

    def __str__(self):
        return "Euler1DCore(ncoord=%d, time_increment=%g)" % (self._n,
                                                              self._dt)

    def clone(self):
        self._flush()
        h = ctypes.c_void_p()
        check(lib.scg_e1d_clone(self._h, ctypes.byref(h)))
        return Euler1DCore(0, 0.0, _handle=h)

    ncoord = property(lambda self: self._n)
    time_increment = property(lambda self: self._dt)
    precision = property(lambda self: self._precision)

    # -- host mirror (same coherence rules as multidim.EulerCore) -----------

    def _host(self, name):
        if name not in self._valid:
            shape = (self._n, 3) if name in ("so0", "so1") else (self._n,)
            buf = self._cache.get(name)
            if buf is None:
                buf = np.empty(shape, dtype="float64")
                self._cache[name] = buf
            check(lib.scg_e1d_get(self._h, _IDS[name], ptr(buf), buf.size))
            self._valid.add(name)
        return self._cache[name]

    def _flush(self):
        for name in sorted(self._dirty | self._exposed):
            if name in self._valid:
                buf = self._cache[name]
                check(lib.scg_e1d_set(self._h, _IDS[name], ptr(buf),
                                      buf.size))
        self._dirty.clear()

    def _after(self):
        self._valid.clear()
        for name in list(self._exposed):
            self._host(name)

    def _array(self, name):
        def expose():
            self._dirty.add(name)
            self._exposed.add(name)
        return SimpleArray(lambda: self._host(name), nghost=0,
                           on_write=lambda: self._dirty.add(name),
                           on_expose=expose)

    def release_views(self):
        self._flush()
        self._exposed.clear()

    coord = property(lambda self: self._array("coord"))
    cfl = property(lambda self: self._array("cfl"))
    so0 = property(lambda self: self._array("so0"))
    so1 = property(lambda self: self._array("so1"))
    gamma = property(lambda self: self._array("gamma"))

    # -- derived quantities (Euler1DCore.hpp:106-168) ----------------------

    @property
    def density(self):
        return self._host("so0")[:, 0].copy()

    @property
    def velocity(self):
        s = self._host("so0")
        return s[:, 1] / (s[:, 0] + TINY)

    @property
    def pressure(self):
        s = self._host("so0")
        g = self._host("gamma")
        ret = s[:, 1] * s[:, 1]
        ret /= 2.0 * s[:, 0] + TINY
        ret = s[:, 2] - ret
        ret *= g - 1.0
        return ret

    @property
    def temperature(self):
        s = self._host("so0")
        g = self._host("gamma")
        return (g - 1.0) / R_GAS * (s[:, 2] / s[:, 0] - 0.5 * s[:, 1] ** 2 /
                                    s[:, 0] ** 2)

    @property
    def internal_energy(self):
        s = self._host("so0")
        return s[:, 2] / s[:, 0] - 0.5 * (s[:, 1] ** 2 / s[:, 0] ** 2)

    @property
    def entropy(self):
        s = self._host("so0")
        return self.pressure / s[:, 0] ** self._host("gamma")

    # -- marching -----------------------------------------------------------

    def _op(self, op, odd=False, alpha=2):
        self._flush()
        check(lib.scg_e1d_op(self._h, op, int(bool(odd)), alpha))
        self._after()

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
        check(lib.scg_e1d_march(self._h, alpha, int(steps)))
        check(lib.scg_e1d_sync(self._h))
        self._after()

    def march_alpha1(self, steps):
        self._march(1, steps)

    def march_alpha2(self, steps):
        self._march(2, steps)

    @property
    def handle(self):
        return self._h


class Euler1DSolver:
    """Grid and field set-up over :class:`Euler1DCore`
    (solvcon/onedim/euler1d.py:21-62)."""

    def __init__(self, xmin, xmax, ncoord, time_increment=0.05,
                 keep_edge=False):
        self._core = self.init_solver(xmin, xmax, ncoord, time_increment,
                                      gamma=1.4)
        last = self.ncoord - 1
        start = 0 if keep_edge else 2
        stop = last if keep_edge else last - 2
        num = (stop - start) // 2 + 1
        self.xindices = np.linspace(start, stop, num, dtype="int32")

    def __getattr__(self, name):
        return getattr(self._core, name)

    @staticmethod
    def init_solver(xmin, xmax, ncoord, time_increment, gamma):
        svr = Euler1DCore(ncoord=ncoord, time_increment=time_increment)
        svr.coord[...] = np.linspace(xmin, xmax, num=ncoord)
        svr.cfl.fill(0)
        svr.gamma.fill(gamma)
        svr.so0[...] = 0.0
        svr.so1[...] = 0.0
        return svr

    @staticmethod
    def calc_u2(gamma, density, velocity, pressure):
        ie = 1.0 / (gamma - 1) * pressure / density
        ke = velocity * velocity / 2
        return density * (ie + ke)


class ShockTube:
    """Exact solution of the shock tube (zones 1 | 2 expansion | 3 | 4 |
    shock | 5) and the numerical solver set-up
    (solvcon/onedim/euler1d.py:64-393)."""

    R = R_GAS

    def __init__(self):
        self.gamma = None
        for zone in "12345":
            for q in ("velocity", "pressure", "density", "temperature",
                      "internal_energy", "entropy", "speedofsound"):
                setattr(self, q + zone, None)
        self.velocity_shock = None
        self.velocity_con = None
        self.coord_field = None
        self.density_field = None
        self.velocity_field = None
        self.pressure_field = None
        self.temperature_field = None
        self.internal_energy_field = None
        self.entropy_field = None
        self.svr = None

    def build_numerical(self, xmin, xmax, ncoord, time_increment=0.05,
                        xdiaphragm=0.0, keep_edge=False):
        if self.gamma is None:
            raise ValueError("constants are not set; call build_constant()")
        self.svr = Euler1DSolver(xmin, xmax, ncoord,
                                 time_increment=time_increment,
                                 keep_edge=keep_edge)
        self.svr.gamma.fill(self.gamma)
        coord = np.array(self.svr.coord.ndarray)
        left = coord < xdiaphragm
        so0 = np.zeros((ncoord, 3))
        so0[:, 0] = np.where(left, self.density1, self.density5)
        so0[:, 2] = np.where(
            left,
            Euler1DSolver.calc_u2(self.gamma, self.density1, 0.0,
                                  self.pressure1),
            Euler1DSolver.calc_u2(self.gamma, self.density5, 0.0,
                                  self.pressure5))
        self.svr.so0[...] = so0
        self.svr.so1.fill(0)
        self.svr.setup_march()

    def build_constant(self, gamma, pressure1, density1, pressure5,
                       density5):
        self.gamma = gamma
        for z, p, rho in (("1", pressure1, density1),
                          ("5", pressure5, density5)):
            setattr(self, "velocity" + z, 0.0)
            setattr(self, "pressure" + z, p)
            setattr(self, "density" + z, rho)
            setattr(self, "temperature" + z, p / (rho * self.R))
            setattr(self, "speedofsound" + z,
                    self.calc_speedofsound(pressure=p, density=rho))
            setattr(self, "internal_energy" + z,
                    self.calc_internal_energy(p, rho))
            setattr(self, "entropy" + z, self.calc_entropy(p, rho))
        p45 = self.calc_pressure45()
        self.velocity4 = self.calc_velocity4(pressure45=p45)
        self.pressure4 = p45 * self.pressure5
        self.density4 = self.calc_density45(pressure45=p45) * self.density5
        self.temperature4 = self.calc_temperature45(p45) * self.temperature5
        self.speedofsound4 = self.calc_speedofsound(pressure=self.pressure4,
                                                    density=self.density4)
        self.internal_energy4 = self.calc_internal_energy(self.pressure4,
                                                          self.density4)
        self.entropy4 = self.calc_entropy(self.pressure4, self.density4)
        self.velocity_shock = self.speedofsound5 * np.sqrt(
            (gamma + 1) / (2 * gamma) * (p45 - 1) + 1)
        self.velocity_con = self.velocity4
        self.velocity3 = self.velocity4
        self.pressure3 = self.pressure4
        self.density3 = self.calc_density2(x=0, t=0,
                                           velocity2=self.velocity3)
        self.temperature3 = self.calc_temperature2(x=0, t=0,
                                                   velocity2=self.velocity3)
        self.internal_energy3 = self.calc_internal_energy(self.pressure3,
                                                          self.density3)
        self.entropy3 = self.calc_entropy(self.pressure3, self.density3)
        self.speedofsound3 = self.calc_speedofsound(pressure=self.pressure3,
                                                    density=self.density3)

    def calc_pressure45(self, tolerance=1.e-10, maxiter=50):
        """Shock strength p4/p5 from the shock-tube equation, by secant
        iteration."""
        g = self.gamma
        p15 = self.pressure1 / self.pressure5
        a51 = self.speedofsound5 / self.speedofsound1

        def residual(p45):
            v = p45 - 1
            frac = (g - 1) * a51 * v / np.sqrt(2 * g * (2 * g + (g + 1) * v))
            return p15 - p45 * (1 - frac) ** (-2 * g / (g - 1))

        x0, x1 = p15, p15 / 2
        f0, f1 = residual(x0), residual(x1)
        for _ in range(maxiter):
            if abs(f1) <= tolerance:
                break
            x0, x1 = x1, x1 - f1 * (x1 - x0) / (f1 - f0)
            f0, f1 = f1, residual(x1)
        return x1

    def calc_density45(self, pressure45):
        gpn1 = (self.gamma + 1) / (self.gamma - 1)
        return (1 + gpn1 * pressure45) / (gpn1 + pressure45)

    def calc_temperature45(self, pressure45):
        gpn1 = (self.gamma + 1) / (self.gamma - 1)
        return pressure45 * ((gpn1 + pressure45) / (1 + gpn1 * pressure45))

    def calc_velocity4(self, pressure45):
        g = self.gamma
        return (self.speedofsound5 / g * (pressure45 - 1) *
                np.sqrt(2 * g / (g + 1) / (pressure45 + (g - 1) / (g + 1))))

    def calc_velocity2(self, x, t):
        return 2 / (self.gamma + 1) * (self.speedofsound1 + x / t)

    def calc_speedofsound2_ratio(self, x, t, velocity2=None):
        if velocity2 is None:
            velocity2 = self.calc_velocity2(x, t)
        return 1 - (self.gamma - 1) / 2 * velocity2 / self.speedofsound1

    def calc_pressure2(self, x, t):
        return self.pressure1 * self.calc_speedofsound2_ratio(x, t) ** (
            2 * self.gamma / (self.gamma - 1))

    def calc_density2(self, x, t, velocity2=None):
        return self.density1 * self.calc_speedofsound2_ratio(
            x, t, velocity2=velocity2) ** (2 / (self.gamma - 1))

    def calc_temperature2(self, x, t, velocity2=None):
        return self.temperature1 * self.calc_speedofsound2_ratio(
            x, t, velocity2=velocity2) ** 2

    def calc_speedofsound(self, pressure, density):
        return np.sqrt(self.gamma * pressure / density)

    def calc_internal_energy(self, pressure, density):
        return pressure / (density * (self.gamma - 1))

    def calc_entropy(self, pressure, density):
        return pressure / (density ** self.gamma)

    def calc_locations(self, t):
        """[x_12, x_23, x_34, x_45]: head of the expansion, its tail, the
        contact surface and the shock at time t."""
        return np.array([-self.speedofsound1 * t,
                         (self.velocity3 - self.speedofsound3) * t,
                         self.velocity3 * t,
                         self.velocity_shock * t], dtype="float64")

    def build_field(self, t, coord=None):
        if coord is None:
            coord = np.array(self.svr.coord.ndarray)[self.svr.xindices]
        self.coord_field = np.array(coord, dtype="float64", copy=True)
        x = self.coord_field
        l12, l23, l34, l45 = self.calc_locations(t=t)
        zones = [(x < l12, "1"), ((x >= l23) & (x < l34), "3"),
                 ((x >= l34) & (x < l45), "4"), (x >= l45, "5")]
        names = ("density", "velocity", "pressure", "temperature",
                 "internal_energy", "entropy")
        fields = {n: np.zeros_like(x) for n in names}
        for sel, z in zones:
            for n in names:
                fields[n][sel] = getattr(self, n + z)
        fan = (x >= l12) & (x < l23)
        for i in np.nonzero(fan)[0]:
            xi = x[i]
            rho = self.calc_density2(xi, t)
            vel = self.calc_velocity2(xi, t)
            p = self.calc_pressure2(xi, t)
            fields["density"][i] = rho
            fields["velocity"][i] = vel
            fields["pressure"][i] = p
            fields["temperature"][i] = self.calc_temperature2(xi, t, vel)
            fields["internal_energy"][i] = self.calc_internal_energy(p, rho)
            fields["entropy"][i] = self.calc_entropy(p, rho)
        for n in names:
            setattr(self, n + "_field", fields[n])
