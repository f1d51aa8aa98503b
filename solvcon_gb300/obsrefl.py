"""Oblique-shock reflection driven on the GPU Euler core.

The numerical side of the reference's oblique-shock reflection application
(solvcon/pilot/apps/obsrefl/_driver.py:21-553) without its GUI:

* :class:`ObliqueShockMesher` meshes the rectangular channel in one of three
  flavors (structured quadrilaterals, structured triangles, or a Delaunay
  triangulation of deterministically jittered points) with one named boundary
  group per domain edge;
* :class:`ObliqueShockRelation` gives the jumps across an oblique shock (the
  relations of Anderson, *Modern Compressible Flow*, 3rd ed., chapter 4, and
  the closed-form inversion of the theta-beta-Mach relation);
* :class:`ObliqueShock` fixes the free stream and the post-shock states and
  builds an :class:`~solvcon_gb300.EulerCore` with the free stream imposed on
  the left, the post-shock state on the top (anchoring the incident shock at
  the upper-left corner), a slip wall at the bottom and a non-reflective
  outflow on the right; its march runs on the GPU.
"""

import math

import numpy as np

from .mesh import StaticMesh
from .multidim import EulerCore

__all__ = ["ObliqueShockMesher", "ObliqueShockRelation", "ObliqueShock"]


class ObliqueShockMesher:
    """Mesh of the rectangle from ``ll`` to ``ur`` on an ``nx`` by ``ny``
    grid of boxes (_driver.py:21-296)."""

    #: Boundary group name per domain edge, in the order
    #: :meth:`classify_boundary` returns the edges.
    BOUNDARY_NAMES = ("left", "top", "bottom", "right")

    def __init__(self, nx=64, ny=16, ll=(0.0, 0.0), ur=(4.0, 1.0)):
        self.nx = nx
        self.ny = ny
        (self.x0, self.y0), (self.x1, self.y1) = ll, ur

    @property
    def cell_extent(self):
        """The (width, height) of one grid box: the resolution of the mesh
        whatever the flavor."""
        return ((self.x1 - self.x0) / self.nx, (self.y1 - self.y0) / self.ny)

    def _xy(self, it, jt):
        # The reference's expression (_driver.py:45-47), so that the points,
        # and the triangulation built on them, are the same to the last bit.
        return (self.x0 + it * (self.x1 - self.x0) / self.nx,
                self.y0 + jt * (self.y1 - self.y0) / self.ny)

    def _grid_nodes(self):
        return [self._xy(it, jt) for jt in range(self.ny + 1)
                for it in range(self.nx + 1)]

    def _nid(self, it, jt):
        return jt * (self.nx + 1) + it

    def _scattered_nodes(self):
        """The unstructured flavor's points: the grid's boundary nodes in a
        counter-clockwise walk from the lower-left corner, then each interior
        grid node displaced in grid units by a fixed phase (up to 0.3 box per
        axis, irregular but free of random numbers)."""
        nx, ny = self.nx, self.ny
        walk = [(it, 0) for it in range(nx + 1)]
        walk += [(nx, jt) for jt in range(1, ny + 1)]
        walk += [(it, ny) for it in range(nx - 1, -1, -1)]
        walk += [(0, jt) for jt in range(ny - 1, 0, -1)]
        pts = [self._xy(it, jt) for it, jt in walk]
        for jt in range(1, ny):
            for it in range(1, nx):
                pts.append(self._xy(
                    it + 0.3 * math.sin(12.9898 * it + 78.233 * jt),
                    jt + 0.3 * math.cos(26.651 * it + 41.347 * jt)))
        return pts

    @staticmethod
    def _delaunay(pts):
        """Counter-clockwise Delaunay triangles of the points."""
        from scipy.spatial import Delaunay
        xy = np.asarray(pts, dtype="float64")
        tri = Delaunay(xy).simplices.astype("int64")
        a, b, c = xy[tri[:, 0]], xy[tri[:, 1]], xy[tri[:, 2]]
        cw = ((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) -
              (c[:, 0] - a[:, 0]) * (b[:, 1] - a[:, 1])) < 0.0
        tri[cw] = tri[cw][:, [0, 2, 1]]
        return [tuple(int(v) for v in t) for t in tri]

    @classmethod
    def _triangulate(cls, pts):
        """Triangulate, then add a point at the centroid of every triangle
        with two boundary edges (a corner ear with one interior neighbour,
        which the CESE scheme handles badly) and triangulate again, until no
        triangle has two boundary edges.  The boundary points never move."""
        pts = list(pts)
        for _ in range(16):
            tris = cls._delaunay(pts)
            count = {}
            for t in tris:
                for k in range(3):
                    e = frozenset((t[k], t[(k + 1) % 3]))
                    count[e] = count.get(e, 0) + 1
            ears = [t for t in tris if sum(
                count[frozenset((t[k], t[(k + 1) % 3]))] == 1
                for k in range(3)) >= 2]
            if not ears:
                return pts, tris
            for t in ears:
                pts.append((sum(pts[v][0] for v in t) / 3.0,
                            sum(pts[v][1] for v in t) / 3.0))
        raise RuntimeError("boundary-cell refinement did not converge")

    def make_mesh(self, cell_type="unstructured"):
        """The mesh of the flavor ``cell_type``: ``'quad'`` (one
        quadrilateral per box), ``'triangle'`` (each box cut along its
        lower-left to upper-right diagonal, the other diagonal in the
        upper-left and lower-right corner boxes so that no triangle has two
        boundary faces) or ``'unstructured'`` (the Delaunay triangulation of
        the scattered points, refined until no triangle has two boundary
        faces).  Cells are counter-clockwise; the mesh carries one boundary
        group per domain edge (:attr:`BOUNDARY_NAMES`) and has its interior,
        boundary and ghost tables built."""
        nx, ny = self.nx, self.ny
        if cell_type == "quad":
            pts = self._grid_nodes()
            cells = [(self._nid(i, j), self._nid(i + 1, j),
                      self._nid(i + 1, j + 1), self._nid(i, j + 1))
                     for j in range(ny) for i in range(nx)]
            tpn = StaticMesh.QUADRILATERAL
        elif cell_type == "triangle":
            pts = self._grid_nodes()
            cells = []
            for j in range(ny):
                for i in range(nx):
                    ll, lr = self._nid(i, j), self._nid(i + 1, j)
                    ur, ul = self._nid(i + 1, j + 1), self._nid(i, j + 1)
                    if (i, j) in ((0, ny - 1), (nx - 1, 0)):
                        cells += [(ll, lr, ul), (lr, ur, ul)]
                    else:
                        cells += [(ll, lr, ur), (ll, ur, ul)]
            tpn = StaticMesh.TRIANGLE
        elif cell_type == "unstructured":
            pts, cells = self._triangulate(self._scattered_nodes())
            tpn = StaticMesh.TRIANGLE
        else:
            raise ValueError("unknown cell_type '%s'" % cell_type)
        nn = len(cells[0])
        mh = StaticMesh(ndim=2, nnode=len(pts), nface=0, ncell=len(cells))
        mh.ndcrd[:, :] = np.asarray(pts, dtype="float64")
        mh.cltpn.fill(tpn)
        mh.clnds[:, :nn + 1] = np.column_stack(
            [np.full(len(cells), nn), np.asarray(cells)])
        mh.build_interior(do_metric=True)
        for name, faces in zip(self.BOUNDARY_NAMES,
                               self.classify_boundary(mh)):
            mh.add_bc(name, faces)
        mh.build_boundary()
        mh.build_ghost()
        return mh

    @staticmethod
    def classify_boundary(mh, tol=1e-9):
        """The boundary faces of ``mh`` (faces without a second cell) per
        domain edge, as sorted face lists ``(left, top, bottom, right)``:
        by face centre on the extreme x (or y) of the boundary face centres
        and by outward normal direction; the rest is the bottom."""
        fccls = np.asarray(mh.fccls.ndarray)[mh.ngstface:]
        fccnd = np.asarray(mh.fccnd.ndarray)[mh.ngstface:]
        fcnml = np.asarray(mh.fcnml.ndarray)[mh.ngstface:]
        bf = np.nonzero(fccls[:mh.nface, 1] < 0)[0]
        xc, yc = fccnd[bf, 0], fccnd[bf, 1]
        nxs, nys = fcnml[bf, 0], fcnml[bf, 1]
        xmin, xmax, ymax = xc.min(), xc.max(), yc.max()
        left = (np.abs(xc - xmin) <= tol) & (nxs < 0.0)
        right = ~left & (np.abs(xc - xmax) <= tol) & (nxs > 0.0)
        top = ~left & ~right & (np.abs(yc - ymax) <= tol) & (nys > 0.0)
        bottom = ~left & ~right & ~top
        return tuple(sorted(int(f) for f in bf[m])
                     for m in (left, top, bottom, right))


class ObliqueShockRelation:
    """Jumps across an oblique shock (_driver.py:298-405).  ``beta`` is the
    shock angle and ``theta`` the flow deflection, in radians from the
    upstream flow direction; ``delta`` picks the weak (1) or strong (0)
    branch."""

    def __init__(self, gamma):
        self.gamma = gamma

    def _mn1sq(self, mach1, beta):
        return (mach1 * math.sin(beta)) ** 2

    def calc_density_ratio(self, mach1, beta):
        """rho2 / rho1 = (g + 1) Mn1^2 / ((g - 1) Mn1^2 + 2)."""
        g, m = self.gamma, self._mn1sq(mach1, beta)
        return (g + 1) * m / ((g - 1) * m + 2)

    def calc_pressure_ratio(self, mach1, beta):
        """p2 / p1 = 1 + 2 g / (g + 1) (Mn1^2 - 1)."""
        g, m = self.gamma, self._mn1sq(mach1, beta)
        return 1 + 2 * g / (g + 1) * (m - 1)

    def calc_temperature_ratio(self, mach1, beta):
        """T2 / T1 = (p2 / p1) / (rho2 / rho1)."""
        return (self.calc_pressure_ratio(mach1, beta) /
                self.calc_density_ratio(mach1, beta))

    def calc_normal_dmach(self, mach_n1):
        """Downstream normal Mach number of a normal shock at ``mach_n1``:
        Mn2^2 = ((g - 1) Mn1^2 + 2) / (2 g Mn1^2 - (g - 1))."""
        g, m = self.gamma, mach_n1 * mach_n1
        return math.sqrt(((g - 1) * m + 2) / (2 * g * m - (g - 1)))

    def calc_dmach(self, mach1, beta=None, theta=None, delta=1):
        """Downstream Mach number M2 = Mn2 / sin(beta - theta), from either
        the shock angle or the deflection."""
        if (beta is None) == (theta is None):
            raise ValueError("got (beta=%s, theta=%s), but I need to take "
                             "either beta or theta" % (beta, theta))
        if beta is None:
            beta = self.calc_shock_angle(mach1, theta, delta=delta)
        else:
            theta = self.calc_flow_angle(mach1, beta)
        return (self.calc_normal_dmach(mach1 * math.sin(beta)) /
                math.sin(beta - theta))

    def calc_flow_angle(self, mach1, beta):
        """The deflection theta of a shock of angle beta."""
        return math.atan(self.calc_flow_tangent(mach1, beta))

    def calc_flow_tangent(self, mach1, beta):
        """tan(theta) = 2 cot(beta) (M1^2 sin^2 beta - 1) /
        (M1^2 (g + cos 2 beta) + 2): the theta-beta-M relation."""
        g, m = self.gamma, mach1 * mach1
        return (2.0 / math.tan(beta) * (m * math.sin(beta) ** 2 - 1) /
                (m * (g + math.cos(2 * beta)) + 2))

    def calc_shock_angle(self, mach1, theta, delta=1):
        """The shock angle beta for a deflection theta."""
        return math.atan(self.calc_shock_tangent(mach1, theta, delta))

    def calc_shock_tangent(self, mach1, theta, delta):
        """tan(beta) from the closed-form inversion of the theta-beta-M
        relation: (M1^2 - 1 + 2 lambda cos((4 pi delta + acos chi) / 3)) /
        (3 (1 + (g - 1) / 2 M1^2) tan theta)."""
        g, m = self.gamma, mach1 * mach1
        lmbd, chi = self.calc_shock_tangent_aux(mach1, theta)
        num = m - 1 + 2 * lmbd * math.cos(
            (4 * math.pi * delta + math.acos(chi)) / 3)
        return num / (3 * (1 + (g - 1) / 2 * m) * math.tan(theta))

    def calc_shock_tangent_aux(self, mach1, theta):
        """(lambda, chi) of the inversion:
        lambda^2 = (M1^2 - 1)^2 - 3 (1 + (g - 1)/2 M1^2)(1 + (g + 1)/2 M1^2)
        tan^2 theta, chi = ((M1^2 - 1)^3 - 9 (1 + (g - 1)/2 M1^2)
        (1 + (g - 1)/2 M1^2 + (g + 1)/4 M1^4) tan^2 theta) / lambda^3.
        No attached shock exists when lambda^2 <= 0 (ValueError)."""
        g, m = self.gamma, mach1 * mach1
        t2 = math.tan(theta) ** 2
        a = 1 + (g - 1) / 2 * m
        lsq = (m - 1) ** 2 - 3 * a * (1 + (g + 1) / 2 * m) * t2
        if lsq <= 0.0:
            raise ValueError("no attached shock for mach1=%g and theta=%g "
                             "deg" % (mach1, math.degrees(theta)))
        lmbd = math.sqrt(lsq)
        chi = ((m - 1) ** 3 - 9 * a * (a + (g + 1) / 4 * m * m) * t2) / \
            lmbd ** 3
        return lmbd, chi


class ObliqueShock:
    """Drive the Euler core over the oblique-shock reflection
    (_driver.py:408-553)."""

    def __init__(self):
        for name in ("gamma", "density", "pressure", "mach",
                     "speedofsound", "velocity", "relation", "theta",
                     "shock_angle", "density2", "pressure2", "mach2",
                     "velocity2", "shock_angle2", "density3", "pressure3",
                     "mach3", "velocity3", "mesher", "mesh", "svr"):
            setattr(self, name, None)

    def build_constant(self, gamma=1.4, density=1.0, pressure=1.0, mach=3.0,
                       angle=10.0):
        """The free stream (zone 1, horizontal at Mach ``mach``), the state
        behind the incident shock that turns it ``angle`` degrees down
        (zone 2, imposed on the top boundary) and the state behind the
        reflected shock that turns it back to horizontal (zone 3, for
        validation)."""
        self.gamma = gamma
        self.density = density
        self.pressure = pressure
        self.mach = mach
        self.speedofsound = math.sqrt(gamma * pressure / density)
        self.velocity = mach * self.speedofsound
        rel = self.relation = ObliqueShockRelation(gamma=gamma)
        self.theta = theta = math.radians(angle)
        self.shock_angle = beta = rel.calc_shock_angle(mach, theta)
        self.density2 = density * rel.calc_density_ratio(mach, beta)
        self.pressure2 = pressure * rel.calc_pressure_ratio(mach, beta)
        self.mach2 = rel.calc_dmach(mach, beta=beta)
        speed2 = self.mach2 * math.sqrt(gamma * self.pressure2 /
                                        self.density2)
        self.velocity2 = (speed2 * math.cos(theta), -speed2 * math.sin(theta))
        self.shock_angle2 = beta2 = rel.calc_shock_angle(self.mach2, theta)
        self.density3 = self.density2 * rel.calc_density_ratio(self.mach2,
                                                                beta2)
        self.pressure3 = self.pressure2 * rel.calc_pressure_ratio(self.mach2,
                                                                  beta2)
        self.mach3 = rel.calc_dmach(self.mach2, beta=beta2)
        speed3 = self.mach3 * math.sqrt(gamma * self.pressure3 /
                                        self.density3)
        self.velocity3 = (speed3, 0.0)

    def build_numerical(self, cell_type="unstructured", time_increment=2.e-3,
                        sigma0=3.0, taumin=0.0, tauscale=1.0,
                        precision="fp64", **mesher_kw):
        """Mesh the channel and build the GPU core :attr:`svr` with the free
        stream as its initial state and the boundary conditions above.
        ``precision`` selects the core's arithmetic (``fp64`` is the
        reference's)."""
        if self.gamma is None:
            raise ValueError("constants are not set; call build_constant()")
        self.mesher = ObliqueShockMesher(**mesher_kw)
        self.mesh = self.mesher.make_mesh(cell_type=cell_type)
        svr = EulerCore(mesh=self.mesh, time_increment=time_increment,
                        precision=precision)
        svr.sigma0 = sigma0
        svr.taumin = taumin
        svr.tauscale = tauscale
        svr.init_solution(gamma=self.gamma, rho=self.density,
                          v=[self.velocity, 0.0], p=self.pressure)
        left, top, bottom, right = (
            self.mesh.bc(name).facn.ndarray[:, 0].tolist()
            for name in self.mesher.BOUNDARY_NAMES)
        svr.add_inlet(left, value=[self.density, self.velocity, 0.0,
                                   self.pressure, self.gamma])
        svr.add_inlet(top, value=[self.density2, self.velocity2[0],
                                  self.velocity2[1], self.pressure2,
                                  self.gamma])
        svr.add_slipwall(bottom)
        svr.add_nonrefl(right)
        svr.bc_soln()
        svr.bc_dsoln()
        self.svr = svr

    def march(self, steps):
        """March the core ``steps`` full CESE steps on the GPU."""
        self.svr.march(steps=steps)

    def zone_states(self):
        """The analytic (rho, vx, vy, p) of zones 1, 2 and 3."""
        return [(self.density, self.velocity, 0.0, self.pressure),
                (self.density2, self.velocity2[0], self.velocity2[1],
                 self.pressure2),
                (self.density3, self.velocity3[0], self.velocity3[1],
                 self.pressure3)]

    def shock_path(self):
        """The analytic shock polyline over the mesh: the upper-left corner,
        the reflection point on the bottom wall and where the reflected
        shock leaves the domain (two points if the incident shock leaves
        through the outflow first)."""
        if self.mesher is None:
            raise ValueError("mesh is not built; call build_numerical()")
        m = self.mesher
        xhit = m.x0 + (m.y1 - m.y0) / math.tan(self.shock_angle)
        if xhit >= m.x1:
            return [(m.x0, m.y1),
                    (m.x1, m.y1 - (m.x1 - m.x0) * math.tan(self.shock_angle))]
        slope = math.tan(self.shock_angle2 - self.theta)
        xend = min(m.x1, xhit + (m.y1 - m.y0) / slope)
        return [(m.x0, m.y1), (xhit, m.y0),
                (xend, m.y0 + (xend - xhit) * slope)]
