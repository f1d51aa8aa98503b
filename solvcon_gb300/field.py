"""Body-cell fields of one Euler run, derived on the device.

:class:`EulerField` keeps the interface of the reference's ``EulerField``
(solvcon/multidim/euler/_field.py:16-148): the same constructor, ``FIELDS``,
``MOMENTA``, properties and methods.  The derived scalars (density, velocity
components, speed, pressure, Mach number, total energy, CFL) are computed by a
kernel from the device-resident solution and only the ``[ncell]`` result is
copied to the host; the overall mass and the CFL range are device reductions
(FP64, compensated), so no call copies the whole state.  ``conserved`` is the
body-row view of the solver's ``so0n`` mirror, so writing into it seeds the
field as in the reference.
"""

import numpy as np

__all__ = ["EulerField"]


class EulerField:
    """Read the body-cell fields of one Euler run.

    :ivar svr: the :class:`~solvcon_gb300.EulerCore` holding the solution.
    :ivar mesh: the :class:`~solvcon_gb300.StaticMesh` it runs on.
    """

    FIELDS = ("density", "velx", "vely", "speed", "pressure", "mach",
              "total_energy", "cfl")

    #: Momentum components in axis order; the solution carries the first
    #: ``ndim`` of them.
    MOMENTA = ("momx", "momy", "momz")

    def __init__(self, svr, mesh):
        self.svr = svr
        self.mesh = mesh

    @property
    def conserveds(self):
        """The conserved variables in the order :attr:`conserved` holds
        them."""
        return (("density",) + self.MOMENTA[:self.svr.ndim] +
                ("total_energy",))

    @property
    def conserved(self):
        """The newest order-0 solution, ``[ncell, neq]`` (a view of the
        solver's ``so0n`` body rows)."""
        arr = self.svr.so0n
        return arr.ndarray[arr.nghost:]

    @property
    def density(self):
        """The newest density over the body cells, ``[ncell]``."""
        return self.svr.device_field("density")

    @property
    def gamma(self):
        """The per-cell ratio of specific heats, ``[ncell]``."""
        arr = self.svr.gamma
        return arr.ndarray[arr.nghost:]

    @property
    def centroid(self):
        """The body-cell centroid, ``[ncell, ndim]``."""
        arr = self.mesh.clcnd
        return arr.ndarray[arr.nghost:]

    @property
    def volume(self):
        """The body-cell volume, ``[ncell]``."""
        arr = self.mesh.clvol
        return arr.ndarray[arr.nghost:]

    @property
    def vel(self):
        """The body-cell velocity, ``[ncell, ndim]``."""
        names = ("velx", "vely", "velz")[:self.svr.ndim]
        return np.stack([self.svr.device_field(n) for n in names], axis=1)

    @property
    def velx(self):
        """The x component of velocity, ``[ncell]``."""
        return self.svr.device_field("velx")

    @property
    def vely(self):
        """The y component of velocity, ``[ncell]``."""
        return self.svr.device_field("vely")

    @property
    def speed(self):
        """The velocity magnitude, ``[ncell]``."""
        return self.svr.device_field("speed")

    @property
    def total_energy(self):
        """The total energy per unit volume, ``[ncell]``."""
        return self.svr.device_field("total_energy")

    @property
    def pressure(self):
        """The pressure of the ideal gas, ``[ncell]``."""
        return self.svr.device_field("pressure")

    @property
    def mach(self):
        """The Mach number against the local speed of sound, ``[ncell]``."""
        return self.svr.device_field("mach")

    @property
    def cfl(self):
        """The CFL number the last step ran at (the unclamped ``cflo``),
        ``[ncell]``."""
        return self.svr.device_field("cfl")

    def field(self, name):
        """Return the scalar field named by one of :attr:`FIELDS`."""
        if name not in self.FIELDS:
            raise ValueError("unknown field '%s'" % name)
        return getattr(self, name)

    def calc_overall_mass(self):
        """Return the density integrated over the whole domain (an FP64
        device reduction of so0n[:, 0] * clvol)."""
        return float(self.svr.totals()[0])

    def calc_cfl_range(self):
        """Return the smallest and the largest CFL number in the domain."""
        return self.svr.cfl_range()
