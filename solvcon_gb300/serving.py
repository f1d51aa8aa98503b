"""A request loop that serves CESE solves with continuous batching.

Requests are 2D Euler meshes (marched in FP32 by one batched launch per
substep, :mod:`solvcon_gb300.batch`) or 1D Euler tubes (FP64, each on its own
stream), each asking for a number of march steps.  The loop

* admits arrived requests while their device memory fits the HBM budget: a
  request takes a *slot*, a resident solver of its mesh (or tube size) that
  is created on first use of the shape and reused by later requests of the
  same shape, so device memory is allocated only when a new shape arrives;
* keeps every admitted request's state on the device between ticks;
* each tick advances all resident requests together -- the 2D ones in one
  batched march, the 1D ones on their own streams at the same time -- by the
  largest step count that finishes no request early;
* reads back and releases finished requests, which frees their slots and
  budget for the next arrivals; requests that arrive while others run join
  at the next tick.

Latency is measured from a request's arrival to the moment its result is on
the host.  A request's result is bit-identical to marching it alone with the
same precision (batched marches are per-core exact).
"""

import collections
import time

import numpy as np

from .batch import EulerBatch
from .multidim import EulerCore
from .onedim import Euler1DCore, lib as lib1d
from ._lib import check
from .synth import sod_tube_state, tube_dt

__all__ = ["Request", "Server", "poisson_arrivals", "sod_tube_state"]


class Request:
    """One solve.  ``kind`` is "2d" (``mesh_key`` selects a prepared mesh)
    or "1d" (``ncoord`` points); ``steps`` full march steps."""

    def __init__(self, rid, kind, steps, arrival, mesh_key=None, ncoord=None,
                 seed=0):
        self.rid = rid
        self.kind = kind
        self.steps = int(steps)
        self.arrival = float(arrival)
        self.mesh_key = mesh_key
        self.ncoord = ncoord
        self.seed = seed
        self.done = 0
        self.t_admit = None
        self.t_done = None
        self.result = None
        self.cells = None

    @property
    def latency(self):
        return None if self.t_done is None else self.t_done - self.arrival


def poisson_arrivals(rate, n, seed=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.cumsum(rng.exponential(1.0 / rate, n))


# Tube sizes served: 16 log-spaced odd sizes over [1k, 100k] points.
TUBE_SIZES = tuple(int(v) | 1 for v in np.geomspace(1000, 100000, 16))


class _MeshSpec:
    """A prepared 2D mesh: state, boundary faces, gamma and dt."""

    def __init__(self, mesh, state, faces, gamma, dt):
        self.mesh = mesh
        self.state = state
        self.faces = faces
        self.gamma = gamma
        self.dt = dt


class _Slot:
    def __init__(self, key, solver, nbytes):
        self.key = key
        self.solver = solver
        self.nbytes = nbytes
        self.busy = False


class Server:
    """Continuous-batching server of 2D and 1D CESE solves.

    :param meshes: dict mesh_key -> _MeshSpec (see :meth:`add_mesh`).
    :param hbm_budget: device bytes the resident solvers may hold.
    :param max_chunk: most steps one tick advances (measured on the mixed
        workload of 1D tubes and 2D meshes: 32 gave 3.68 G cell-steps/s
        aggregate, 16 gave 3.28, 64 3.46, 128 3.30, 256 3.12).
    :param precision: precision of the 2D solves; the 1D tubes run in FP32
        state for either FP32 form and in FP64 otherwise.
    """

    def __init__(self, hbm_budget=120 * 2 ** 30, max_chunk=32,
                 precision="fp32", block=64, persistent=True):
        self.meshes = {}
        self.hbm_budget = int(hbm_budget)
        self.max_chunk = int(max_chunk)
        self.precision = precision
        self.block = block
        self.persistent = persistent
        self.slots = collections.defaultdict(list)
        self.held = 0
        self.ticks = 0
        # Where a run's wall time went: building batches (a resident set
        # that changed), marching them, and waiting for the 1D tubes.
        self.rebuilds = 0
        self.t_rebuild = 0.0
        self.t_batch = 0.0
        self.t_tubes = 0.0
        self.t_load = 0.0
        self.t_result = 0.0
        self.peak_resident = 0
        self.peak_held = 0
        self.rejected = []

    # -- preparation ------------------------------------------------------

    def add_mesh(self, key, mesh, state, faces, gamma, dt):
        self.meshes[key] = _MeshSpec(mesh, state, faces, gamma, dt)

    @staticmethod
    def tube_bytes(ncoord):
        return 11 * 8 * int(ncoord)

    def _evict_idle(self, need):
        """Free idle slots (least recently created first) until ``need``
        more bytes fit the budget; returns whether they fit."""
        for key in list(self.slots):
            if self.held + need <= self.hbm_budget:
                break
            keep = []
            for s in self.slots[key]:
                if not s.busy and self.held + need > self.hbm_budget:
                    self.held -= s.nbytes
                    s.solver = None
                else:
                    keep.append(s)
            self.slots[key] = keep
        return self.held + need <= self.hbm_budget

    def _slot_for(self, req):
        key = (req.kind, req.mesh_key if req.kind == "2d" else req.ncoord)
        for s in self.slots[key]:
            if not s.busy:
                return s
        if req.kind == "2d":
            spec = self.meshes[req.mesh_key]
            est = int(spec.mesh.ncell * 1200)
            if not self._evict_idle(est):
                return None
            core = EulerCore(spec.mesh, spec.dt, precision=self.precision)
            core.add_slipwall(spec.faces)
            slot = _Slot(key, core, core.device_bytes)
        else:
            est = self.tube_bytes(req.ncoord)
            if not self._evict_idle(est):
                return None
            slot = _Slot(key, Euler1DCore(req.ncoord, tube_dt(req.ncoord),
                                          precision=_tube_precision(
                                              self.precision)),
                         est)
        self.held += slot.nbytes
        self.slots[key].append(slot)
        return slot

    def _load(self, slot, req):
        if req.kind == "2d":
            spec = self.meshes[req.mesh_key]
            core = slot.solver
            # A reused slot starts from the same all-zero tables as a new
            # solver, so the result does not depend on the slot's history.
            core.reset_state()
            core.init_solution(spec.gamma, 1.0, [0.0] * spec.mesh.ndim, 1.0)
            core.so0n[0:] = spec.state
            core.bc_soln()
            core.bc_dsoln()
            core.release_views()
            req.cells = core.ncell
        else:
            x, so0, dt = sod_tube_state(req.ncoord, req.seed)
            tube = slot.solver
            tube.coord[...] = x
            tube.so0[...] = so0
            tube.so1.fill(0.0)
            tube.gamma.fill(1.4)
            tube.cfl.fill(0.0)
            tube.setup_march()
            req.cells = req.ncoord

    def _result(self, slot, req):
        if req.kind == "2d":
            core = slot.solver
            return np.array(core.so0n[...])[core.ngstcell:]
        return np.array(slot.solver.so0[...])

    # -- the loop -----------------------------------------------------------

    def run(self, requests, clock=time.perf_counter):
        """Serve ``requests`` (arrival times in seconds from the start);
        returns the list of finished requests."""
        pending = sorted(requests, key=lambda r: r.arrival)
        self.ticks = self.rebuilds = 0
        self.t_rebuild = self.t_batch = self.t_tubes = 0.0
        self.t_load = self.t_result = 0.0
        queue = collections.deque()
        active = {}
        finished = []
        batch = None
        batch_members = ()
        t0 = clock()
        i = 0
        while i < len(pending) or queue or active:
            now = clock() - t0
            while i < len(pending) and pending[i].arrival <= now:
                queue.append(pending[i])
                i += 1
            # Admission in arrival order while budget and slots allow.
            while queue:
                req = queue[0]
                slot = self._slot_for(req)
                if slot is None and not active:
                    # Too large for the whole budget: reject it rather than
                    # wait for memory that will never be freed.
                    queue.popleft()
                    self.rejected.append(req)
                    continue
                if slot is None:
                    break
                queue.popleft()
                slot.busy = True
                tl = clock()
                self._load(slot, req)
                self.t_load += clock() - tl
                req.t_admit = clock() - t0
                active[req.rid] = (req, slot)
            if not active:
                if i < len(pending):
                    wait = pending[i].arrival - (clock() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.002))
                continue
            self.peak_resident = max(self.peak_resident, len(active))
            self.peak_held = max(self.peak_held, self.held)
            chunk = min(self.max_chunk,
                        min(r.steps - r.done for r, _ in active.values()))
            tubes = [(r, s) for r, s in active.values() if r.kind == "1d"]
            meshes = [(r, s) for r, s in active.values() if r.kind == "2d"]
            # 1D tubes first, asynchronously on their own streams, so they
            # overlap with the 2D batch on the device.
            for r, s in tubes:
                s.solver._flush()
                check(lib1d.scg_e1d_march(s.solver.handle, 2, chunk))
            if meshes:
                members = tuple(sorted(r.rid for r, _ in meshes))
                if batch is None or members != batch_members:
                    tb = clock()
                    solvers = [s.solver for _, s in meshes]
                    if batch is None or not batch.retarget(solvers):
                        batch = EulerBatch(solvers, block=self.block,
                                           persistent=self.persistent)
                    batch_members = members
                    self.rebuilds += 1
                    self.t_rebuild += clock() - tb
                tb = clock()
                batch.march(chunk)
                self.t_batch += clock() - tb
            tb = clock()
            for r, s in tubes:
                check(lib1d.scg_e1d_sync(s.solver.handle))
                s.solver._after()
            self.t_tubes += clock() - tb
            self.ticks += 1
            for rid in list(active):
                r, s = active[rid]
                r.done += chunk
                if r.done >= r.steps:
                    tl = clock()
                    r.result = self._result(s, r)
                    self.t_result += clock() - tl
                    r.t_done = clock() - t0
                    s.busy = False
                    del active[rid]
                    finished.append(r)
        self.makespan = clock() - t0
        return finished


def stats(finished, makespan):
    lat = np.array([r.latency for r in finished])
    work = sum(r.cells * r.steps for r in finished)
    return {"requests": len(finished),
            "p50_latency_s": float(np.percentile(lat, 50)),
            "p99_latency_s": float(np.percentile(lat, 99)),
            "mean_latency_s": float(lat.mean()),
            "makespan_s": makespan,
            "cell_steps": int(work),
            "cell_steps_per_s": work / makespan}


def _tube_precision(precision):
    """The 1D cores' precision for a server of the given 2D precision: FP32
    state for either FP32 form, else the reference's FP64."""
    return "fp64" if precision == "fp64" else "fp32"


def alone(server, req, precision):
    """March one request alone (its own solver, its own launches) and return
    (result, seconds)."""
    if req.kind == "2d":
        spec = server.meshes[req.mesh_key]
        core = EulerCore(spec.mesh, spec.dt, precision=precision)
        core.add_slipwall(spec.faces)
        core.init_solution(spec.gamma, 1.0, [0.0] * spec.mesh.ndim, 1.0)
        core.so0n[0:] = spec.state
        core.bc_soln()
        core.bc_dsoln()
        core.release_views()
        core.sync()
        t0 = time.perf_counter()
        core.march(req.steps)
        secs = time.perf_counter() - t0
        return np.array(core.so0n[...])[core.ngstcell:], secs
    x, so0, dt = sod_tube_state(req.ncoord, req.seed)
    tube = Euler1DCore(req.ncoord, dt, precision=_tube_precision(precision))
    tube.coord[...] = x
    tube.so0[...] = so0
    tube.so1.fill(0.0)
    tube.gamma.fill(1.4)
    tube.cfl.fill(0.0)
    tube.setup_march()
    t0 = time.perf_counter()
    tube.march_alpha2(req.steps)
    secs = time.perf_counter() - t0
    return np.array(tube.so0[...]), secs


def make_requests(n, rate, mesh_keys, seed=0, frac_1d=0.3, steps=(200, 2000)):
    """n requests with Poisson arrivals at ``rate``/s: a fraction frac_1d of
    1D tubes (sizes from TUBE_SIZES, 1k-100k points), the rest 2D meshes
    drawn from ``mesh_keys``; steps uniform in ``steps``."""
    rng = np.random.Generator(np.random.PCG64(seed + 17))
    arr = poisson_arrivals(rate, n, seed)
    out = []
    for k in range(n):
        nsteps = int(rng.integers(steps[0], steps[1] + 1))
        if rng.uniform() < frac_1d:
            npts = TUBE_SIZES[int(rng.integers(0, len(TUBE_SIZES)))]
            out.append(Request(k, "1d", nsteps, arr[k], ncoord=npts,
                               seed=seed * 100000 + k))
        else:
            key = mesh_keys[int(rng.integers(0, len(mesh_keys)))]
            out.append(Request(k, "2d", nsteps, arr[k], mesh_key=key))
    return out

