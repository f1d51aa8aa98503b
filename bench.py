#!/usr/bin/env python
"""Benchmark of the GPU CESE march: cell-steps/s on the 2D plain-FP64 workload.

Workload (default, ``--workload tri2d``): the unit square cut into
1000 x 1000 quads, each split on the same diagonal into 2 triangles
(2,000,000 cells), interior nodes jittered by U(-0.2h, 0.2h) from a seed;
four-quadrant Riemann state (rho, p in [0.1, 1.5], |u|, |v| <= 0.8) from a
seed; gamma 1.4; slip walls on every boundary face; dt set for CFL 0.8 from a
probe calc_cfl; plain FP64.  One bench "step" is one full march step (two
CESE substeps) of the whole mesh.  The state (about 1.3 GB with geometry) is
far larger than the 129 MB L2, so no flush is needed between steps.

Printed (one JSON line on rank 0): ``value`` = cell-steps/s with the state
resident in HBM; ``e2e`` = the same metric through the C ABI with the state in
pinned host memory copied in and out every step; ``roofline`` of the fused
substep kernel (HBM bytes are the algorithmic bytes of one cell-substep); the
FP64-pipe roofline beside it; ``cpu_baseline`` = the CPU oracle on a bounded
sample; clocks sampled during the timed region.

``--impl reference`` times the reference algorithm on the host CPU instead,
one process per host core (the C oracle, a restatement of the reference
march that equals the compiled reference bit for bit: the reference library
is built from the reference's sources, which a machine without them cannot
do).  The line then carries that rate in ``value``, ``cpu_baseline`` and
``e2e``.
With ``--gpus N`` (N > 1) every rank marches its own mesh on its own GPU
(replicas: a single mesh is not decomposed), times are maxed over ranks and
the value is the sum.  Launched without a launcher, the command starts its N
ranks itself under ``torch.distributed.run`` (rendezvous on 127.0.0.1).
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic HBM bytes of one cell-substep of the fused march: compulsory
# reads of the neighbour-summed state, the cell's geometry and ids, and writes
# of so0n, so1n, cflo, cflc.  2D triangles: FP64 520 B, FP32 state with FP64
# geometry (the FP32 form, "fp32") 412 B, FP32 geometry too ("fp32-geom32")
# 268 B; 3D tetrahedra: 1,100 / 928 / 560 B.
ALG_BYTES = {("tri2d", "fp64"): 520, ("tri2d", "fp32"): 412,
             ("tri2d", "fp32-geom32"): 268, ("tet3d", "fp64"): 1100,
             ("tet3d", "fp32"): 928, ("tet3d", "fp32-geom32"): 560}
ALG_BYTES.update({(w, "fp32-geom64"): ALG_BYTES[(w, "fp32")]
                  for w in ("tri2d", "tet3d")})

# DRAM bytes (read + write) and FP64 flops (DFMA counted as 2) of the fused
# substep kernel per cell-substep, each from one ncu capture of the kernel on
# a smaller mesh of the same workload, larger than L2 (tri2d: 500^2 x 2 cells
# FP64, 700^2 x 2 FP32; tet3d: 40^3 x 6 FP64, 60^3 x 6 FP32), divided by its
# cells; absent until captured.  The FP64 records carry a primitive cache
# (192 B instead of 128 B), which trades DRAM bytes, idle in the FP64-bound
# march, for FP64 operations.
NCU_TRAFFIC_PER_CELL = {("tri2d", "fp64"): 769.5,
                        ("tri2d", "fp32"): 546.6,
                        ("tri2d", "fp32-geom32"): 270.2,
                        ("tet3d", "fp64"): 1337.3,
                        ("tet3d", "fp32"): 1199.1,
                        ("tet3d", "fp32-geom32"): 627.1}
NCU_DP_FLOPS_PER_CELL = {("tri2d", "fp64"): 1159.6, ("tet3d", "fp64"): 2717.4}

WORKLOADS = {
    "tri2d": dict(ndim=2, nside=1000, jitter=0.2, cfl=0.8, seed=2026),
    "tet3d": dict(ndim=3, nside=160, jitter=0.15, cfl=0.7, seed=2026),
}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock and throttle-reason samples during a region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,"
             "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" +
                 self.QUERY, "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        return False

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap")
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(name, nside=None, seed_offset=0):
    from solvcon_gb300 import meshgen
    w = dict(WORKLOADS[name])
    if nside:
        w["nside"] = nside
    if w["ndim"] == 2:
        x, t, c = meshgen.tri_square(w["nside"], w["jitter"],
                                     w["seed"] + seed_offset)
    else:
        x, t, c = meshgen.tet_cube(w["nside"], w["jitter"],
                                   w["seed"] + seed_offset)
    mesh = meshgen.build_mesh(w["ndim"], x, t, c)
    clcnd = np.asarray(mesh.clcnd.ndarray)[mesh.ngstcell:]
    if w["ndim"] == 2:
        state = meshgen.quadrant_state(clcnd, seed=w["seed"] + seed_offset)
    else:
        state = meshgen.blast_state(clcnd)
    faces = np.asarray(mesh.bndfcs.ndarray[:, 0]).copy()
    return w, mesh, state, faces


def dt_for_cfl(mesh, state, faces, cfl, precision="fp64"):
    """dt giving max(cflo) = cfl for the initial state (cflo is linear in
    dt): a probe core with dt = 1 runs calc_cfl."""
    import solvcon_gb300 as sg
    probe = sg.EulerCore(mesh, 1.0, precision=precision)
    probe.init_solution(1.4, 1.0, [0.0] * mesh.ndim, 1.0)
    probe.so0n.ndarray[probe.ngstcell:] = state
    probe.calc_cfl()
    cmax = probe.cfl_range()[1]
    del probe
    return cfl / cmax


def setup_core(mesh, state, faces, dt, precision):
    import solvcon_gb300 as sg
    core = sg.EulerCore(mesh, dt, precision=precision)
    core.init_solution(1.4, 1.0, [0.0] * mesh.ndim, 1.0)
    core.add_slipwall(faces)
    core.so0n[0:] = state
    core.bc_soln()
    core.bc_dsoln()
    core.release_views()
    core.sync()
    return core


def time_resident(core, steps):
    """K march steps on the core's stream, CUDA events on that stream."""
    from solvcon_gb300._lib import check, launch_count, lib
    stream = ctypes.c_void_p()
    check(lib.scg_euler_stream(core.handle, ctypes.byref(stream)))
    e0, e1 = ctypes.c_void_p(), ctypes.c_void_p()
    check(lib.scg_event_create(ctypes.byref(e0)))
    check(lib.scg_event_create(ctypes.byref(e1)))
    check(lib.scg_euler_profile(core.handle, 1))
    core.sync()
    n0 = launch_count()
    check(lib.scg_event_record(e0, stream))
    core.march_async(steps)
    check(lib.scg_event_record(e1, stream))
    ms = ctypes.c_double()
    check(lib.scg_event_elapsed(e0, e1, ctypes.byref(ms)))
    launches = launch_count() - n0
    kms = ctypes.c_double()
    kn = ctypes.c_int64()
    check(lib.scg_euler_profile_stats(core.handle, ctypes.byref(kms),
                                      ctypes.byref(kn)))
    check(lib.scg_euler_profile(core.handle, 0))
    check(lib.scg_event_destroy(e0))
    check(lib.scg_event_destroy(e1))
    return ms.value, launches, kms.value, kn.value


def time_e2e(core, steps):
    """K steps through the C ABI with host state: per step the state (so0n,
    so1n) is copied from pinned host memory, one march step runs, and the new
    state comes back into the same pinned buffers.  scg_euler_march_from_host
    takes the state from the buffers while the step's first substep marches
    the cells whose rows are already up; the buffers are registered once with
    scg_euler_deliver: an FP64 march's last substep writes the new state over
    the host link as it computes it, an FP32 march queues a coalesced gather
    into them after it; the step ends when scg_euler_sync returns with the
    state in host memory.  Wall time around the whole loop."""
    from solvcon_gb300._lib import check, lib
    ids = {"so0n": 5, "so1n": 8}
    bufs = {}
    for name in ("so0n", "so1n"):
        arr = np.array(getattr(core, name)[...])
        p = ctypes.c_void_p()
        check(lib.scg_host_alloc(arr.nbytes, ctypes.byref(p)))
        view = np.ctypeslib.as_array((ctypes.c_double * arr.size)
                                     .from_address(p.value)).reshape(arr.shape)
        view[...] = arr
        bufs[name] = (p, view)
    h2d = bufs["so0n"][1].nbytes + bufs["so1n"][1].nbytes
    d2h = h2d
    h = core.handle
    for name in ("so0n", "so1n"):
        p, view = bufs[name]
        check(lib.scg_euler_deliver(h, ids[name], p, view.size))
    core.sync()
    (p0, v0), (p1, v1) = bufs["so0n"], bufs["so1n"]
    t0 = time.perf_counter()
    for _ in range(steps):
        check(lib.scg_euler_march_from_host(h, p0, v0.size, p1, v1.size, 1))
        check(lib.scg_euler_sync(h))
    t1 = time.perf_counter()
    for name in ("so0n", "so1n"):
        check(lib.scg_euler_deliver(h, ids[name], None, 0))
    for p, _ in bufs.values():
        check(lib.scg_host_free(p))
    return (t1 - t0) * 1e3, h2d, d2h


_SYNTH = None


def synth():
    """The workload generators (solvcon_gb300/synth.py, plain numpy), loaded
    by path: the CPU arms build their samples without importing the package
    and its native library."""
    global _SYNTH
    if _SYNTH is None:
        import importlib.util
        path = os.path.join(ROOT, "solvcon_gb300", "synth.py")
        spec = importlib.util.spec_from_file_location("_scg_synth", path)
        _SYNTH = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(_SYNTH)
    return _SYNTH


def tube_state(ncoord, seed):
    """The 1D workload: a Sod-type tube on [-1, 1] (random left/right
    density and pressure, at rest), its dt for CFL 0.8."""
    return synth().sod_tube_state(ncoord, seed)


def scalar_state(ncelm):
    """The spacetime workload: sin(x) / cos(x) on [0, 2 pi] with ncelm
    conservation elements, dt for CFL 0.8 at unit wave speed; returns the
    grid, so0, so1 (whole tables) and dt."""
    from solvcon_gb300.spacetime import Grid
    grid = Grid(0.0, 2.0 * np.pi, int(ncelm))
    x = np.asarray(grid.xcoord)
    dt = 0.8 * (2.0 * np.pi / ncelm)
    return grid, np.sin(x), np.cos(x), dt


def _oracle_setup(workload, size, seed_offset):
    """One seeded sample of a workload on the CPU oracle: returns (units per
    step, march(steps)).  The sample (grid, mesh and state) is built with
    the plain-numpy generators and the oracle's own mesh build, so nothing
    of the GPU library is loaded."""
    from oracle import oracle as ora
    sy = synth()
    if workload == "tube1d":
        x, so0, dt = tube_state(size, 2026 + seed_offset)
        o = ora.OracleEuler1D(size, dt)
        o.coord[:] = x
        o.so0[:] = so0
        o.setup_march()
        return size, lambda k: o.march_alpha(2, k)
    if workload == "spacetime":
        x = sy.grid_xcoord(sy.grid_xloc(0.0, 2.0 * np.pi, int(size)))
        o = ora.OracleSpacetime(0, x, 0.8 * (2.0 * np.pi / size))
        o.so0[:] = np.sin(x)
        o.so1[:] = np.cos(x)
        o.setup_march()
        return x.size - 4, lambda k: o.march_alpha(2, k)
    w = dict(WORKLOADS[workload])
    seed = w["seed"] + seed_offset
    gen = sy.tri_square if w["ndim"] == 2 else sy.tet_cube
    mesh = ora.OracleMesh(w["ndim"], *gen(size, w["jitter"], seed))
    clcnd = mesh.clcnd[mesh.ngstcell:]
    state = sy.quadrant_state(clcnd, seed=seed) if w["ndim"] == 2 else \
        sy.blast_state(clcnd)
    faces = mesh.bndfcs[:, 0]
    o = ora.OracleEuler(mesh, 1e-4)
    o.init_solution(1.4, 1.0, [0.0] * mesh.ndim, 1.0)
    o.so0n[o.ngstcell:] = state
    o.add_slipwall(faces)
    o.call("bc_soln")
    o.call("bc_dsoln")
    return mesh.ncell, o.march


def _oracle_worker(workload, size, seed_offset, warmup, steps, barrier, out):
    """One CPU process of the oracle throughput run: build its own sample,
    warm up, wait for the others, march, report (units, seconds)."""
    units, march = _oracle_setup(workload, size, seed_offset)
    march(warmup)
    barrier.wait()
    t0 = time.perf_counter()
    march(steps)
    out.put((units, time.perf_counter() - t0))


def oracle_throughput(workload, size, steps, warmup=1, nproc=None):
    """The CPU oracle (restatement of the reference march, which is serial)
    on every host core at once: one process per core, each marching its own
    seeded sample of the workload.  Returns (aggregate unit-steps/s over the
    wall time of the concurrent marches, units per sample, processes,
    seconds).  Processes are spawned, never forked (the parent may already
    hold a CUDA context)."""
    import multiprocessing as mp
    nproc = nproc or len(os.sched_getaffinity(0))
    ctx = mp.get_context("spawn")
    barrier = ctx.Barrier(nproc + 1)
    out = ctx.Queue()
    procs = [ctx.Process(target=_oracle_worker,
                         args=(workload, size, 7919 * (k + 1), warmup, steps,
                               barrier, out)) for k in range(nproc)]
    for p in procs:
        p.start()
    barrier.wait()
    t0 = time.perf_counter()
    res = [out.get() for _ in procs]
    t1 = time.perf_counter()
    for p in procs:
        p.join()
    units = res[0][0]
    return sum(c for c, _ in res) * steps / (t1 - t0), units, nproc, t1 - t0


def cpu_nside(workload, steps):
    """Sample resolution giving about 30 s of oracle work per process."""
    if workload == "tube1d":
        return int(min(1000001, 16e6 * 30.0 / max(steps, 1))) | 1
    if workload == "spacetime":
        return int(min(4000000, 40e6 * 30.0 / max(steps, 1)))
    w = WORKLOADS[workload]
    if w["ndim"] == 2:
        cells = 0.35e6 * 30.0 / max(steps, 1)
        return int(max(20, min(400, round((cells / 2.0) ** 0.5))))
    cells = 0.17e6 * 30.0 / max(steps, 1)
    return int(max(4, min(40, round((cells / 6.0) ** (1.0 / 3.0)))))


def pin_device(local):
    """One GPU per rank: the local rank's device, as the only visible one
    (the local-th entry when a device list is already set)."""
    seen = os.environ.get("CUDA_VISIBLE_DEVICES")
    if seen is None:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
        return
    devs = [d for d in seen.split(",") if d.strip()]
    if len(devs) > 1 and local < len(devs):
        os.environ["CUDA_VISIBLE_DEVICES"] = devs[local].strip()


def free_port():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch_ranks(n, argv):
    """Run this command as n ranks under torch.distributed.run (one process
    per GPU, rendezvous on 127.0.0.1) and return its exit status: used when
    ``--gpus n`` is given and no launcher set WORLD_SIZE."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
           "--nproc-per-node", str(n), "--master-addr", "127.0.0.1",
           "--master-port", str(free_port()),
           os.path.abspath(__file__)] + list(argv)
    return subprocess.call(cmd)


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local, dist


def reduce_max(dist, value):
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


LINE_WORKLOADS = {
    "tube1d": ("point-steps/s", 20000001,
               "1D Euler CESE march (Euler1DCore.march_alpha2) of a Sod-type "
               "tube on [-1, 1], %d points, gamma 1.4, CFL 0.8, FP64"),
    "spacetime": ("point-steps/s", 20000000,
                  "spacetime linear-scalar CESE march (march_alpha2) of "
                  "sin(x) on [0, 2 pi], %d conservation elements (a point "
                  "is a solution element of either plane), CFL 0.8, FP64"),
}

# Algorithmic HBM bytes per point-step of the 1D marches (FP64): Euler1DCore
# reads so0, so1, coord, gamma and writes so0, so1, cfl (120 B); the linear
# scalar reads so0, so1, x and writes so0, so1, cfl (48 B).
LINE_ALG_BYTES = {"tube1d": 120, "spacetime": 48}


def run_reference(args, world, rank, dist):
    if rank != 0:
        return
    size = args.cpu_nside or cpu_nside(args.workload, args.steps + args.warmup)
    value, units, nproc, secs = oracle_throughput(args.workload, size,
                                                  args.steps, args.warmup)
    if args.workload in LINE_WORKLOADS:
        unit, _, desc = LINE_WORKLOADS[args.workload]
        desc = desc % (args.nside or LINE_WORKLOADS[args.workload][1])
        what = "%d-point" % units
    else:
        unit = "cell-steps/s"
        desc = _desc(WORKLOADS[args.workload])
        what = "%d-cell" % units
    sample = ("%d processes (one per host core), each marching its own "
              "%s seeded sample of the %s workload (same generator, "
              "size %d) for %d steps after %d warm-up steps; the reference "
              "march is serial, so a core runs one sample"
              % (nproc, what, args.workload, size, args.steps, args.warmup))
    line = {
        "metric": unit, "value": value, "unit": unit,
        "impl": "reference", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": secs * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": "%s (%s)" % (args.workload, desc),
                   "sample_units": units, "precision": "fp64"},
        "cpu_baseline": {"value": value, "unit": unit,
                         "cores": nproc, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": unit,
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_line(args, world, rank, dist):
    """The 1D marches (Euler1DCore, spacetime linear scalar): point-steps/s
    with the state resident (CUDA events on the solver's stream around K
    steps replayed from the solver's CUDA graph), e2e through the C ABI with
    so0/so1 copied from and back to pinned host memory every step, the
    roofline on the algorithmic bytes, and the oracle on every host core."""
    from solvcon_gb300._lib import check, launch_count, lib
    unit, default, desc = LINE_WORKLOADS[args.workload]
    n = args.nside or default
    if args.workload == "tube1d":
        from solvcon_gb300 import onedim
        n |= 1
        x, so0, dt = tube_state(n, 2026 + rank)
        core = onedim.Euler1DCore(n, dt, precision=args.precision or "fp64")
        core.coord[...] = x
        core.so0[...] = so0
        core.so1.fill(0.0)
        core.gamma.fill(1.4)
        core.cfl.fill(0.0)
        core.setup_march()
        core.release_views()
        h, l1 = core._h, onedim.lib
        march = lambda k: check(l1.scg_e1d_march(h, 2, k))  # noqa: E731
        sync = lambda: check(l1.scg_e1d_sync(h))  # noqa: E731
        stream = ctypes.c_void_p()
        check(l1.scg_e1d_stream(h, ctypes.byref(stream)))
        points = n
        io = [(0, onedim._IDS["so0"], 3 * n), (0, onedim._IDS["so1"], 3 * n)]
        get = lambda i, b, c: check(l1.scg_e1d_get(h, i, b, c))  # noqa: E731
        put = lambda i, b, c: check(l1.scg_e1d_set(h, i, b, c))  # noqa: E731
    else:
        from solvcon_gb300 import spacetime as st
        grid, so0, so1, dt = scalar_state(n)
        svr = st.LinearScalarSolver(grid, dt)
        sz = grid.xsize
        for name, val in (("so0", so0), ("so1", so1)):
            buf = np.ascontiguousarray(val, dtype="float64")
            check(st.lib.scg_st_set(svr._h, svr._IDS[name],
                                    buf.ctypes.data, sz))
        svr.setup_march()
        h, l1 = svr._h, st.lib
        march = lambda k: check(l1.scg_st_march(h, 2, k))  # noqa: E731
        sync = lambda: check(l1.scg_st_sync(h))  # noqa: E731
        stream = ctypes.c_void_p()
        check(l1.scg_st_stream(h, ctypes.byref(stream)))
        points = grid.xsize - 4  # both planes: 2 ncelm + 1 solution points
        io = [(0, svr._IDS["so0"], sz), (0, svr._IDS["so1"], sz)]
        get = lambda i, b, c: check(l1.scg_st_get(h, i, b, c))  # noqa: E731
        put = lambda i, b, c: check(l1.scg_st_set(h, i, b, c))  # noqa: E731
    march(args.warmup)
    sync()
    e0, e1 = ctypes.c_void_p(), ctypes.c_void_p()
    check(lib.scg_event_create(ctypes.byref(e0)))
    check(lib.scg_event_create(ctypes.byref(e1)))
    barrier(dist)
    n0 = launch_count()
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clocks:
        check(lib.scg_event_record(e0, stream))
        march(args.steps)
        check(lib.scg_event_record(e1, stream))
        sync()
    launches = launch_count() - n0
    ms = ctypes.c_double()
    check(lib.scg_event_elapsed(e0, e1, ctypes.byref(ms)))
    check(lib.scg_event_destroy(e0))
    check(lib.scg_event_destroy(e1))
    barrier(dist)
    ms_max = reduce_max(dist, ms.value)
    value = world * points * args.steps / (ms_max * 1e-3)

    # e2e: host state in, one step, host state out, every step.
    e2e_steps = args.e2e_steps or 5
    bufs = []
    for _, i, c in io:
        p = ctypes.c_void_p()
        check(lib.scg_host_alloc(c * 8, ctypes.byref(p)))
        bufs.append((i, p, c))
        get(i, p, c)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for i, p, c in bufs:
            put(i, p, c)
        march(1)
        for i, p, c in bufs:
            get(i, p, c)
    e2e_s = time.perf_counter() - t0
    nbytes = sum(c * 8 for _, _, c in bufs)
    for _, p, _ in bufs:
        check(lib.scg_host_free(p))
    e2e_value = world * points * e2e_steps / reduce_max(dist, e2e_s)

    hbm_peak, peak_kind = peaks()
    alg = LINE_ALG_BYTES[args.workload]
    if args.workload == "tube1d" and args.precision == "fp32":
        alg = 64  # so0, so1, gamma, cfl in FP32 (56 B), coord FP64 (8 B)
    achieved = alg * points * args.steps / (ms.value * 1e-3) / 1e9
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        size = args.cpu_nside or cpu_nside(args.workload, args.cpu_steps)
        rate, units, nproc, secs = oracle_throughput(args.workload, size,
                                                     args.cpu_steps)
        cpu = {"value": rate, "unit": unit, "cores": nproc, "kind": "port",
               "sample": "%d processes (one per host core), each marching "
                         "its own %d-point sample for %d steps; %.1f s"
                         % (nproc, units, args.cpu_steps, secs)}
    line = {
        "metric": unit, "value": value, "unit": unit, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision == "fp32" else "f64",
        "data": "synthetic",
        "config": {"workload": "%s (%s)" % (
                       args.workload, (desc % n).replace(
                           "FP64", "FP32 state, FP64 coordinates")
                       if args.precision == "fp32" else desc % n),
                   "points": points, "dt": dt,
                   "l2": "state larger than L2 (no flush needed)"
                   if points * LINE_ALG_BYTES[args.workload] > 2e8 else
                   "state fits in L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak,
                     "traffic": None,
                     "alg_bytes_per_point_step": alg,
                     "kernel": "one march step (two fused half-step kernels)",
                     "step_ms": ms.value / args.steps,
                     "peak_source": peak_kind},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": unit,
                "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                "steps": e2e_steps},
        "gpu_launches": launches, "clocks": clocks.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def _batch_params(nmesh, seed, lo, hi):
    rng = np.random.Generator(np.random.PCG64(seed))
    ncells = np.exp(rng.uniform(np.log(lo), np.log(hi), nmesh))
    gammas = rng.uniform(1.1, 1.67, nmesh)
    return ncells, gammas


def batch_mesh(k, ncell, gamma, seed, order="native"):
    """Mesh k of the batched workload: a jittered triangulated square of
    about ``ncell`` cells, its four-quadrant state, slip-wall faces and
    gamma.  ``order="morton"`` numbers its cells along a Z-order curve of
    their node averages (the same mesh and state, renumbered)."""
    from solvcon_gb300 import meshgen
    from solvcon_gb300.batch import morton_order, node_average
    nside = max(2, int(round(np.sqrt(ncell / 2.0))))
    x, t, c = meshgen.tri_square(nside, 0.2, seed + 1 + k)
    if order == "morton":
        p = morton_order(node_average(x, c))
        t, c = np.asarray(t)[p], np.asarray(c)[p]
    elif order != "native":
        raise ValueError("unknown cell order %r" % order)
    mesh = meshgen.build_mesh(2, x, t, c)
    clcnd = np.asarray(mesh.clcnd.ndarray)[mesh.ngstcell:]
    state = meshgen.quadrant_state(clcnd, seed + 1 + k, gamma)
    faces = np.asarray(mesh.bndfcs.ndarray[:, 0]).copy()
    return mesh, state, faces, float(gamma)


def batch_meshes(nmesh, seed=2026, lo=2000, hi=200000, order="native",
                 only=None):
    """The batched workload: nmesh jittered triangulated squares with cell
    counts log-uniform in [lo, hi], per-mesh four-quadrant states and gamma
    in [1.1, 1.67], slip walls (``only``: the indices to build)."""
    ncells, gammas = _batch_params(nmesh, seed, lo, hi)
    ks = range(nmesh) if only is None else only
    return [batch_mesh(k, ncells[k], gammas[k], seed, order) for k in ks]


def setup_core_g(mesh, state, faces, dt, precision, gamma):
    import solvcon_gb300 as sg
    core = sg.EulerCore(mesh, dt, precision=precision)
    core.init_solution(gamma, 1.0, [0.0] * mesh.ndim, 1.0)
    core.add_slipwall(faces)
    core.so0n[0:] = state
    core.bc_soln()
    core.bc_dsoln()
    core.release_views()
    return core


def dt_for_cfl_g(mesh, state, cfl, gamma):
    import solvcon_gb300 as sg
    probe = sg.EulerCore(mesh, 1.0)
    probe.init_solution(gamma, 1.0, [0.0] * mesh.ndim, 1.0)
    probe.so0n[0:] = state
    probe.calc_cfl()
    cmax = probe.cfl_range()[1]
    del probe
    return cfl / cmax


def measure_batch(nmesh, seed, prec, steps, warmup, dist=None, world=1,
                  tune=True, accuracy=True, local=0):
    """One FP32 batched march of nmesh meshes of the batched distribution
    (tile, grid policy and cell ordering autotuned, or Morton order with
    one block of 128 per tile), CUDA graph per step, against the same
    meshes marched one after the other in plain FP64.  Returns the figures
    of the batched workload's line."""
    from solvcon_gb300._lib import launch_count
    from solvcon_gb300.batch import EulerBatch, autotune

    t_tune = time.perf_counter()
    if tune:
        # Autotune tile, grid policy and cell ordering on scratch cores of
        # a subset of the meshes, each built in both cell orders.
        sub = list(range(0, nmesh, max(1, nmesh // 32)))
        cand = {}
        for order in ("native", "morton"):
            cand[order] = [setup_core_g(m, s, f, dt_for_cfl_g(m, s, 0.8, g),
                                        prec, g)
                           for m, s, f, g in batch_meshes(nmesh, seed,
                                                          order=order,
                                                          only=sub)]
        best, table = autotune(cand["native"], steps=2, repeat=2,
                               orderings={"morton": cand["morton"]})
        del cand
    else:
        best = {"ordering": "morton", "block": 128, "persistent": False}
        table = None
    t_tune = time.perf_counter() - t_tune

    t_setup = time.perf_counter()
    data = batch_meshes(nmesh, seed, order=best["ordering"])
    dts = [dt_for_cfl_g(m, s, 0.8, g) for m, s, f, g in data]
    fast = [setup_core_g(m, s, f, dt, prec, g)
            for (m, s, f, g), dt in zip(data, dts)]
    plain = [setup_core_g(m, s, f, dt, "fp64", g)
             for (m, s, f, g), dt in zip(data, dts)]
    t_setup = time.perf_counter() - t_setup
    ncell = sum(c.ncell for c in fast)
    batch = EulerBatch(fast, block=best["block"],
                       persistent=best["persistent"])
    batch.march(warmup)
    barrier(dist)
    n0 = launch_count()
    with ClockSampler(local) as clocks:
        batch.march(steps)
        ms = batch.last_ms
    launches = launch_count() - n0
    barrier(dist)
    ms_max = reduce_max(dist, ms)
    value = world * ncell * steps / (ms_max * 1e-3)

    # Plain FP64, one mesh after the other, same steps.
    for c in plain:
        c.march(warmup)
    for c in plain:
        c.sync()
    t0 = time.perf_counter()
    for c in plain:
        c.march_async(steps)
    for c in plain:
        c.sync()
    seq_ms = (time.perf_counter() - t0) * 1e3
    seq_value = ncell * steps / (seq_ms * 1e-3)

    acc = None
    if accuracy:
        # Accuracy of the FP32 batch against the FP64 marches (same step
        # count), beside the problem's own sensitivity: the FP64 marches
        # restarted from states perturbed by 1e-15 relative.
        rng = np.random.default_rng(7)
        pert = [setup_core_g(m, s * (1 + 1e-15 * rng.uniform(-1, 1, s.shape)),
                             f, dt, "fp64", g)
                for (m, s, f, g), dt in zip(data, dts)]
        for c in pert:
            c.march(warmup + steps)
        ref = [_body(c) for c in plain]
        vols = [np.array(m.clvol.ndarray)[m.ngstcell:] for m, *_ in data]

        def rel_l1(cores):
            num, den, worst = np.zeros(4), np.zeros(4), np.zeros(4)
            for c, r, v in zip(cores, ref, vols):
                d = (np.abs(_body(c) - r) * v[:, None]).sum(0)
                a = (np.abs(r) * v[:, None]).sum(0)
                num += d
                den += a
                worst = np.maximum(worst, d / a)
            return {"rel_l1_aggregate": [float(x) for x in num / den],
                    "rel_l1_worst_mesh": [float(x) for x in worst]}
        acc = {"steps": warmup + steps, "fp32_vs_fp64": rel_l1(fast),
               "floor_fp64_perturbed_1e-15_vs_fp64": rel_l1(pert)}
        del pert

    hbm_peak, peak_kind = peaks()
    per_launch_ms = ms / (2 * steps)
    alg = ALG_BYTES[("tri2d", prec)] * ncell
    achieved = alg / (per_launch_ms * 1e-3) / 1e9
    return {
        "value": value, "ms_per_step": ms_max / steps, "ncell": ncell,
        "best": best, "table": table, "t_tune": t_tune, "t_setup": t_setup,
        "seq_value": seq_value, "accuracy": acc, "launches": launches,
        "clocks": clocks.summary(),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                     "unit": "GB/s", "frac": achieved / hbm_peak,
                     "traffic": None, "kernel": "k_fused_batch",
                     "alg_bytes_per_cell_substep": ALG_BYTES[("tri2d", prec)],
                     "launch_ms": per_launch_ms,
                     "peak_source": peak_kind},
    }


def run_batch(args, world, rank, dist):
    """The batched workload: one FP32 batched march of many meshes
    (autotuned tile, grid policy and cell ordering, CUDA graph per step)
    against the same meshes marched one after the other in plain FP64."""
    nmesh = args.nmesh
    prec = args.precision or "fp32"
    r = measure_batch(nmesh, 2026 + 1000 * rank, prec, args.steps,
                      args.warmup, dist, world,
                      local=int(os.environ.get("LOCAL_RANK", "0")))
    line = {
        "metric": "cell-steps/s", "value": r["value"], "unit": "cell-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if prec != "fp64" else "f64", "data": "synthetic",
        "config": {"workload": "batch%d (%d 2D jittered-triangle meshes, "
                               "cells log-uniform in [2k, 200k], per-mesh "
                               "quadrant states, gamma in [1.1, 1.67], CFL "
                               "0.8, slip walls)" % (nmesh, nmesh),
                   "cells": r["ncell"], "meshes": nmesh, "precision": prec,
                   "autotune": r["best"], "autotune_table": r["table"],
                   "autotune_s": r["t_tune"],
                   "l2": "state larger than L2 (no flush needed)",
                   "setup_s": r["t_setup"]},
        "baseline_plain_fp64_sequential": {
            "value": r["seq_value"], "unit": "cell-steps/s",
            "speedup_of_batch": r["value"] / r["seq_value"]},
        "accuracy_vs_fp64": r["accuracy"],
        "roofline": r["roofline"],
        "gpu_launches": r["launches"], "clocks": r["clocks"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def measure_serve(nmesh, nreq, rates, max_chunk, precision, seed=4242):
    """The served workload at the given Poisson arrival rates (one warm-up
    pass first, which creates every slot and captures the graphs), and the
    same requests each marched alone with the plain FP64 march.  Returns
    (stats per rate, alone-FP64 cell-steps/s, alone seconds)."""
    from solvcon_gb300 import serving
    data = batch_meshes(nmesh, seed=seed)
    srv = serving.Server(hbm_budget=120 * 2 ** 30, max_chunk=max_chunk,
                         precision=precision)
    for k, (m, s, f, g) in enumerate(data):
        srv.add_mesh(k, m, s, f, g, dt_for_cfl_g(m, s, 0.8, g))
    keys = list(range(len(data)))
    srv.run(serving.make_requests(nreq, 1e6, keys, seed=7))
    per_rate = []
    for rate in rates:
        reqs = serving.make_requests(nreq, rate, keys, seed=7)
        done = srv.run(reqs)
        st = serving.stats(done, srv.makespan)
        st["rate_req_per_s"] = rate
        st["rejected"] = len(srv.rejected)
        st["peak_resident"] = srv.peak_resident
        st["ticks"] = srv.ticks
        st["batch_rebuilds"] = srv.rebuilds
        st["seconds_rebuild_march_tubes_load_result"] = [
            srv.t_rebuild, srv.t_batch, srv.t_tubes, srv.t_load,
            srv.t_result]
        per_rate.append(st)
    # Each request alone with the plain FP64 march (the same request set).
    reqs = serving.make_requests(nreq, 1.0, keys, seed=7)
    alone_s = 0.0
    work = 0
    for r in reqs:
        _, secs = serving.alone(srv, r, "fp64")
        alone_s += secs
        cells = srv.meshes[r.mesh_key].mesh.ncell if r.kind == "2d" \
            else r.ncoord
        work += cells * r.steps
    return per_rate, work / alone_s, alone_s


def run_serve(args, world, rank, dist):
    """The served workload: Poisson arrivals of mixed 1D tubes (30%) and 2D
    meshes (70%, the batched workload's distribution), 200-2000 steps each,
    served with continuous batching under a 120 GB HBM budget; p50/p99
    latency and aggregate cell-steps/s per arrival rate, against each
    request marched alone with the plain FP64 march."""
    nreq = args.nreq
    rates = [float(r) for r in args.rates.split(",")]
    per_rate, alone_rate, alone_s = measure_serve(
        args.nmesh, nreq, rates, args.max_chunk, args.precision or "fp32",
        seed=4242 + 1000 * rank)
    best = max(per_rate, key=lambda s: s["cell_steps_per_s"])
    line = {
        "metric": "cell-steps/s", "value": best["cell_steps_per_s"],
        "unit": "cell-steps/s", "n_gpus": world, "steps": None,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "serve (%d requests per rate: 30%% 1D Sod-type "
                               "tubes of 1k-100k points, 70%% 2D meshes of "
                               "the batched distribution, 200-2000 steps; "
                               "HBM budget 120 GB; continuous batching)"
                               % nreq, "rates": rates,
                   "max_chunk": args.max_chunk},
        "per_rate": per_rate,
        "baseline_alone_plain_fp64": {"value": alone_rate,
                                      "unit": "cell-steps/s",
                                      "seconds": alone_s},
        "speedup_vs_alone_fp64": best["cell_steps_per_s"] / alone_rate,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def _rel_l1_linf(got, ref, vol):
    d = np.abs(got - ref)
    l1 = (d * vol[:, None]).sum(0) / (np.abs(ref) * vol[:, None]).sum(0)
    linf = d.max(0) / np.abs(ref).max(0)
    return [float(x) for x in l1], [float(x) for x in linf]


def _body(core):
    return np.array(core.so0n[...])[core.ngstcell:]


FP32_FORMS = ("fp32", "fp32-geom32")

# Gradient magnitude, relative to the equation's largest, above which a
# (cell, equation) pair's W-3/4 firing decision is not round-off: in a cell
# whose state is still uniform the per-element gradients are noise, their
# inverse-magnitude weights scatter by O(1) and the cap binds at random (the
# reference itself flips those bits under a 1e-15 input perturbation).
RESOLVED_GRADIENT = 1e-10


def _totals_rel(got, ref_q):
    """Relative difference of totals against sum(ref_q) per variable; a
    total that cancels is measured against the magnitudes it sums."""
    tref = ref_q.sum(0)
    scale = np.maximum(np.abs(tref), np.abs(ref_q).sum(0))
    return [float(x) for x in np.abs(np.asarray(got) - tref) / scale]


def _limiter_hamming(mask, ref_mask, ref_so1n, neq):
    """Hamming fraction of two W-3/4 firing masks over (cell, equation)
    pairs: over all pairs, and over the pairs whose gradient is resolved."""
    bits = lambda m: np.unpackbits(  # noqa: E731
        np.asarray(m, dtype=np.uint8)[:, None], axis=1,
        bitorder="little")[:, :neq].astype(bool)
    diff = bits(mask) != bits(ref_mask)
    grad = np.linalg.norm(ref_so1n, axis=2)
    res = grad > RESOLVED_GRADIENT * grad.max(axis=0)[None, :]
    return {"all": float(diff.mean()),
            "resolved": float(diff[res].mean()) if res.any() else 0.0,
            "resolved_fraction": float(res.mean()),
            "fired_fraction": float(bits(ref_mask).mean())}


def run_accuracy(args, world, rank, dist):
    """Accuracy of the GPU marches, beside the problem's own sensitivity (the
    FP64 march from an initial state perturbed by 1e-15 relative):

    * ``oracle2d``: a sample of the 2D four-quadrant workload (300 x 300 x 2
      triangles, CFL 0.8, 500 steps) against the CPU oracle itself;
    * ``oracle3d``: the 3D spherical blast at 40^3 x 6 = 384,000 tetrahedra
      (CFL 0.7, 200 steps) against the CPU oracle itself;
      both report per conserved variable the relative L1/Linf, the totals
      sum(so0n * clvol) against the oracle's, and the W-3/4 firing pattern's
      Hamming fraction (all pairs, and resolved pairs), for FP64, FP64 from
      the perturbed state, and both FP32 forms;
    * ``blast3d``: the 3D blast at full size (160^3 x 6 tetrahedra, 200
      steps): both FP32 forms and perturbed FP64 against FP64, with the
      totals' difference every 20 steps;
    * ``batch``: the batched distribution (64 meshes, CFL 0.8, 1000 steps):
      aggregate and worst-mesh relative L1 per variable of the FP32 forms
      (batched) and of perturbed FP64 against FP64; meshes on which the FP64
      march itself becomes non-finite (the fixed dt outgrows the CFL limit;
      the oracle fails on the same meshes at the same steps) are left out.

    At full size the FP64 GPU march stands in for the oracle (the oracle
    would take hours); the oracle cases and the parity tests pin it.  The
    oracle runs on every host core (its per-cell loops are threaded; the
    results do not depend on the thread count).  ``--cases`` picks a subset
    (default all)."""
    from oracle import oracle as ora
    if rank != 0:
        return
    ora.set_threads(len(os.sched_getaffinity(0)))
    out = {"metric": "accuracy", "data": "synthetic"}
    rng = np.random.default_rng(1)
    allc = ("oracle2d", "oracle3d", "blast3d", "batch")
    cases = set((args.cases or ",".join(allc)).split(","))
    unknown = cases - set(allc)
    if unknown:
        raise SystemExit("--cases: unknown %s" % sorted(unknown))
    for c in allc:
        if c in cases:
            t0 = time.perf_counter()
            {"oracle2d": _accuracy_oracle2d, "oracle3d": _accuracy_oracle3d,
             "blast3d": _accuracy_blast3d, "batch": _accuracy_batch}[c](
                 args, out, rng, ora)
            out[c]["seconds"] = time.perf_counter() - t0
            print(json.dumps({c: out[c]}), file=sys.stderr, flush=True)
    print(json.dumps(out), flush=True)


def _against_oracle(workload, nside, steps, rng, ora):
    w, mesh, state, faces = make_workload(workload, nside=nside)
    nd, ng = mesh.ndim, mesh.ngstcell
    dt = dt_for_cfl(mesh, state, faces, w["cfl"])
    vol = np.array(mesh.clvol.ndarray)[ng:]
    o = ora.OracleEuler(mesh, dt)
    o.init_solution(1.4, 1.0, [0.0] * nd, 1.0)
    o.so0n[ng:] = state
    o.add_slipwall(faces)
    o.call("bc_soln")
    o.call("bc_dsoln")
    t0 = time.perf_counter()
    o.march(steps)
    oracle_s = time.perf_counter() - t0
    want = np.array(o.so0n)[ng:]
    so1n = np.array(o.so1n)[ng:]
    q = want * vol[:, None]
    res = {"cells": mesh.ncell, "steps": steps, "cfl": w["cfl"],
           "oracle_s": oracle_s,
           "oracle_totals_change": _totals_rel(q.sum(0),
                                               state * vol[:, None])}
    pert = state * (1 + 1e-15 * rng.uniform(-1, 1, state.shape))
    for name, prec, st in (("gpu_fp64", "fp64", state),
                           ("gpu_fp64_perturbed", "fp64", pert)) + tuple(
                               ("gpu_" + f.replace("-", "_"), f, state)
                               for f in FP32_FORMS):
        c = setup_core(mesh, st, faces, dt, prec)
        c.march(steps)
        l1, linf = _rel_l1_linf(_body(c), want, vol)
        res[name + "_vs_oracle"] = {
            "rel_l1": l1, "rel_linf": linf,
            "totals_rel": _totals_rel(c.totals(), q),
            "limiter_hamming": _limiter_hamming(c.limiter_mask(), o.limiter[
                :mesh.ncell], so1n, nd + 2)}
        del c
    return res


def _accuracy_oracle2d(args, out, rng, ora):
    """A sample of the 2D four-quadrant workload against the CPU oracle."""
    out["oracle2d"] = _against_oracle("tri2d", 300, 500, rng, ora)


def _accuracy_oracle3d(args, out, rng, ora):
    """The 3D blast at 40^3 x 6 tetrahedra against the CPU oracle."""
    out["oracle3d"] = _against_oracle("tet3d", 40, 200, rng, ora)


def _accuracy_blast3d(args, out, rng, ora=None):
    """The 3D spherical blast at full size: the FP32 forms and perturbed
    FP64 against FP64, totals every 20 steps."""
    nside = args.nside or 160
    t0 = time.perf_counter()
    w, mesh, state, faces = make_workload("tet3d", nside=nside)
    build_s = time.perf_counter() - t0
    dt = dt_for_cfl(mesh, state, faces, 0.7)
    vol = np.array(mesh.clvol.ndarray)[mesh.ngstcell:]
    pert = state * (1 + 1e-15 * rng.uniform(-1, 1, state.shape))
    res = {"cells": mesh.ncell, "steps": 200, "cfl": 0.7, "build_s": build_s}
    finals, tots = {}, {}
    for name, prec, st in (("fp64", "fp64", state),
                           ("fp64_perturbed", "fp64", pert)) + tuple(
                               (f.replace("-", "_"), f, state)
                               for f in FP32_FORMS):
        c = setup_core(mesh, st, faces, dt, prec)
        series = [np.array(c.totals())]
        for _ in range(10):
            c.march(20)
            series.append(np.array(c.totals()))
        tots[name] = np.array(series)
        finals[name] = _body(c)
        del c
    t64 = tots["fp64"]
    res["fp64_mass_energy_change"] = [
        float(x) for x in ((t64[-1] - t64[0]) / np.abs(t64[0]))[[0, 4]]]
    for name in finals:
        if name == "fp64":
            continue
        l1, linf = _rel_l1_linf(finals[name], finals["fp64"], vol)
        res[name + "_vs_fp64"] = {
            "rel_l1": l1, "rel_linf": linf,
            "mass_energy_totals_every_20_steps": [
                [float(x) for x in col] for col in
                ((tots[name] - t64) / np.abs(t64))[:, [0, 4]].T]}
    out["blast3d"] = res
    del finals


def _accuracy_batch(args, out, rng, ora=None):
    """The batched distribution, 1000 steps: the FP32 forms (batched) and
    perturbed FP64 against FP64."""
    from solvcon_gb300.batch import EulerBatch
    nmesh = args.nmesh
    data = batch_meshes(nmesh)
    dts = [dt_for_cfl_g(m, s, 0.8, g) for m, s, f, g in data]
    finals = {}
    for name, prec in (("fp64", "fp64"), ("fp64_perturbed", "fp64")) + tuple(
            (f.replace("-", "_"), f) for f in FP32_FORMS):
        cs = []
        for (m, s, f, g), dtk in zip(data, dts):
            st = s * (1 + 1e-15 * rng.uniform(-1, 1, s.shape)) \
                if name == "fp64_perturbed" else s
            cs.append(setup_core_g(m, st, f, dtk, prec, g))
        if prec != "fp64":
            EulerBatch(cs, block=64, persistent=True).march(1000)
        else:
            for c in cs:
                c.march(1000)
        finals[name] = [_body(c) for c in cs]
        del cs
    ok = [k for k in range(nmesh) if np.isfinite(finals["fp64"][k]).all()]
    res = {"meshes": nmesh, "steps": 1000, "cfl": 0.8,
           "fp64_nonfinite_meshes": [k for k in range(nmesh) if k not in ok]}
    for name in finals:
        if name == "fp64":
            continue
        res[name + "_nonfinite_meshes"] = [
            k for k in range(nmesh) if not np.isfinite(finals[name][k]).all()]
        num = np.zeros(4)
        den = np.zeros(4)
        worst = np.zeros(4)
        for k in ok:
            v = np.array(data[k][0].clvol.ndarray)[data[k][0].ngstcell:]
            d = (np.abs(finals[name][k] - finals["fp64"][k]) *
                 v[:, None]).sum(0)
            a = (np.abs(finals["fp64"][k]) * v[:, None]).sum(0)
            num += d
            den += a
            worst = np.maximum(worst, d / a)
        res[name + "_vs_fp64"] = {"rel_l1_aggregate": [float(x) for x in
                                                       num / den],
                                  "rel_l1_worst_mesh": [float(x) for x in
                                                        worst]}
    out["batch"] = res
    del finals


def run_meshbuild(args, world, rank, dist):
    """Time to first step of the 3D workload's mesh (160^3 x 6 tetrahedra by
    default): StaticMesh build_interior + build_boundary + build_ghost on the
    host and with build_interior on the GPU (tables compared), then the GPU
    core's set-up (upload, prepare_ce, compaction) on the built mesh.  The
    node and cell arrays are generated before the clock starts."""
    import solvcon_gb300 as sg
    from solvcon_gb300 import meshgen
    if rank != 0:
        return
    nside = args.nside or 160
    x, t, c = meshgen.tet_cube(nside, 0.15, 2026)
    out = {"metric": "mesh build s", "unit": "s", "higher_is_better": False,
           "config": {"workload": "tet3d mesh, %d^3 x 6 = %d tetrahedra" %
                      (nside, len(t))}, "data": "synthetic"}
    meshes = {}
    for name, device in (("host", False), ("device", True)):
        t0 = time.perf_counter()
        m = sg.StaticMesh(ndim=3, nnode=len(x), nface=0, ncell=len(t))
        m.ndcrd[:, :] = x
        m.cltpn[:] = t
        m.clnds[:, :c.shape[1]] = c
        t1 = time.perf_counter()
        m.build_interior(do_metric=True, build_edge=False, device=device)
        t2 = time.perf_counter()
        m.build_boundary()
        m.build_ghost()
        t3 = time.perf_counter()
        out[name] = {"fill_s": t1 - t0, "build_interior_s": t2 - t1,
                     "boundary_ghost_s": t3 - t2, "total_s": t3 - t0}
        meshes[name] = m
    same = all(np.array_equal(np.asarray(getattr(meshes["host"], a).ndarray),
                              np.asarray(getattr(meshes["device"], a).ndarray))
               for a in ("fccls", "fcnds", "clfcs", "fccnd", "fcnml", "clvol",
                         "clcnd", "ndcrd"))
    out["tables_equal"] = bool(same)
    m = meshes.pop("device")
    meshes.clear()
    t0 = time.perf_counter()
    core = sg.EulerCore(m, 1e-4, precision="fp32")
    core.sync()
    out["core_setup_s"] = time.perf_counter() - t0
    out["value"] = out["device"]["total_s"]
    out["speedup_build_interior"] = (out["host"]["build_interior_s"] /
                                     out["device"]["build_interior_s"])
    print(json.dumps(out), flush=True)


def _desc(w):
    if w["ndim"] == 2:
        return ("2D Euler, unit square %dx%d quads x 2 triangles = %d cells, "
                "jitter %.2fh, four-quadrant Riemann state, slip walls, "
                "CFL %.1f" % (w["nside"], w["nside"], 2 * w["nside"] ** 2,
                              w["jitter"], w["cfl"]))
    return ("3D Euler, unit cube %d^3 hexes x 6 tetrahedra = %d cells, jitter "
            "%.2fh, spherical blast, slip walls, CFL %.1f" %
            (w["nside"], 6 * w["nside"] ** 3, w["jitter"], w["cfl"]))


def headline_figures(local):
    """The batched and served forms of the march, measured compactly beside
    the default line so that its record carries them: 512 meshes of the
    batched distribution in one FP32 batched march (Morton cell order, one
    block of 128 per tile, no autotuning or accuracy pass) against the same
    meshes in sequential plain FP64; and the served mix at 2000 req/s (64
    requests after a warm-up pass) against each request alone in plain
    FP64.  A failure is recorded in place of the figures."""
    out = {}
    try:
        steps, warmup = 20, 3
        r = measure_batch(512, 2026, "fp32", steps, warmup, tune=False,
                          accuracy=False, local=local)
        out["batched"] = {
            "metric": "cell-steps/s", "value": r["value"],
            "unit": "cell-steps/s",
            "workload": "batch512 (512 2D jittered-triangle meshes, cells "
                        "log-uniform in [2k, 200k], per-mesh quadrant "
                        "states, gamma in [1.1, 1.67], CFL 0.8, slip walls)",
            "cells": r["ncell"],
            "precision": "fp32 (FP32 state and flux, FP64 geometry)",
            "steps": steps, "warmup": warmup,
            "ms_per_step": r["ms_per_step"], "tiles": r["best"],
            "plain_fp64_sequential": r["seq_value"],
            "speedup_vs_plain_fp64_sequential": r["value"] / r["seq_value"],
            "roofline": r["roofline"], "gpu_launches": r["launches"],
            "clocks": r["clocks"], "setup_s": r["t_setup"]}
    except Exception as e:  # recorded, the default line still prints
        out["batched"] = {"error": "%s: %s" % (type(e).__name__, e)}
    try:
        nreq, rate = 64, 2000.0
        per_rate, alone_rate, alone_s = measure_serve(64, nreq, [rate], 32,
                                                      "fp32")
        st = per_rate[0]
        out["served"] = {
            "metric": "cell-steps/s", "value": st["cell_steps_per_s"],
            "unit": "cell-steps/s",
            "workload": "serve (%d requests at %g req/s: 30%% 1D Sod-type "
                        "tubes of 1k-100k points, 70%% 2D meshes of the "
                        "batched distribution, 200-2000 steps; HBM budget "
                        "120 GB; continuous batching, ticks of at most 32 "
                        "steps)" % (nreq, rate),
            "precision": "fp32 (FP32 state and flux, FP64 geometry; FP32 "
                         "tubes)",
            "p50_latency_s": st["p50_latency_s"],
            "p99_latency_s": st["p99_latency_s"],
            "makespan_s": st["makespan_s"],
            "alone_plain_fp64": alone_rate, "alone_seconds": alone_s,
            "speedup_vs_alone_plain_fp64": st["cell_steps_per_s"] / alone_rate}
    except Exception as e:
        out["served"] = {"error": "%s: %s" % (type(e).__name__, e)}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="tri2d",
                    choices=sorted(WORKLOADS) + ["batch", "serve",
                                                 "accuracy", "meshbuild"] +
                    sorted(LINE_WORKLOADS))
    ap.add_argument("--precision", default=None,
                    choices=["fp64", "fp32", "fp32-geom64", "fp32-geom32"],
                    help="fp32: FP32 state and flux with FP64 geometry "
                    "tables (fp32-geom64 is the same); fp32-geom32 also "
                    "stores the geometry in FP32")
    ap.add_argument("--nside", type=int, default=None)
    ap.add_argument("--cpu-nside", type=int, default=None)
    ap.add_argument("--cpu-steps", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-headline", action="store_true",
                    help="default line (the plain 2M-triangle workload): skip "
                         "the batched and served figures")
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--cases", default=None,
                    help="accuracy workload: comma-separated subset of "
                    "oracle2d, oracle3d, blast3d, batch")
    ap.add_argument("--nmesh", type=int, default=None)
    ap.add_argument("--nreq", type=int, default=64)
    ap.add_argument("--rates", default="50,200,1000,2000")
    ap.add_argument("--max-chunk", type=int, default=32,
                    help="serve: most steps one serving tick advances")
    args = ap.parse_args()
    if args.nmesh is None:
        args.nmesh = 512 if args.workload == "batch" else 64
    if args.warmup < 3:
        ap.error("--warmup must be at least 3 (untimed warm-up steps)")
    if args.gpus < 1:
        ap.error("--gpus must be at least 1")
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(launch_ranks(args.gpus, sys.argv[1:]))
    world, rank, local, dist = dist_setup(args)
    if world != args.gpus:
        ap.error("--gpus %d but the launcher started %d ranks" %
                 (args.gpus, world))
    if args.impl == "reference":
        run_reference(args, world, rank, dist)
        return
    if args.workload in ("batch", "serve", "accuracy", "meshbuild") or (
            args.workload in LINE_WORKLOADS and args.impl != "reference"):
        pin_device(local)
        import solvcon_gb300  # noqa: F401
        {"batch": run_batch, "serve": run_serve, "accuracy": run_accuracy,
         "meshbuild": run_meshbuild,
         "tube1d": run_line, "spacetime": run_line}[args.workload](
             args, world, rank, dist)
        if dist is not None:
            dist.destroy_process_group()
        return
    precision = args.precision or ("fp64" if args.workload == "tri2d"
                                   else "fp32")

    pin_device(local)
    import solvcon_gb300  # noqa: F401  (fails loudly without libscg.so)
    from solvcon_gb300._lib import check, lib

    t_setup = time.perf_counter()
    w, mesh, state, faces = make_workload(args.workload, args.nside,
                                          seed_offset=rank)
    dt = dt_for_cfl(mesh, state, faces, w["cfl"], precision)
    core = setup_core(mesh, state, faces, dt, precision)
    t_setup = time.perf_counter() - t_setup
    ncell = core.ncell

    core.march(args.warmup)
    fp64_peak = ctypes.c_double()
    check(lib.scg_fma_peak(0, 4000, ctypes.byref(fp64_peak)))
    barrier(dist)
    with ClockSampler(local) as clocks:
        ms, launches, kms, kn = time_resident(core, args.steps)
    barrier(dist)
    ms_max = reduce_max(dist, ms)
    value = world * ncell * args.steps / (ms_max * 1e-3)

    e2e_steps = args.e2e_steps or max(3, min(args.steps, 20))
    e2e_ms, h2d, d2h = time_e2e(core, e2e_steps)
    e2e_ms = reduce_max(dist, e2e_ms)
    e2e_value = world * ncell * e2e_steps / (e2e_ms * 1e-3)
    finite = bool(np.all(np.isfinite(np.array(core.so0n.ndarray))))
    lo, hi = core.cfl_range()

    hbm_peak, peak_kind = peaks()
    per_launch_ms = kms / max(kn, 1)
    key = (args.workload, precision)
    alg = ALG_BYTES[key] * ncell
    achieved = alg / (per_launch_ms * 1e-3) / 1e9
    traffic = NCU_TRAFFIC_PER_CELL.get(key)
    dp_flops = NCU_DP_FLOPS_PER_CELL.get(key)
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": hbm_peak,
        "unit": "GB/s", "frac": achieved / hbm_peak,
        "traffic": traffic * ncell if traffic else None,
        "kernel": "k_fused (one CESE substep)",
        "alg_bytes_per_cell_substep": ALG_BYTES[key],
        "launch_ms": per_launch_ms, "launches_timed": kn,
        "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind
        if peak_kind == "measured" else "fallback 6.8 TB/s",
        "fp64": {"peak_tflops": fp64_peak.value,
                 "peak_source": "measured live (scg_fma_peak FP64 FMA chain)",
                 "flops_per_cell_substep": dp_flops,
                 "achieved_tflops": (dp_flops * ncell /
                                     (per_launch_ms * 1e-3) / 1e12
                                     if dp_flops else None),
                 "frac": (dp_flops * ncell / (per_launch_ms * 1e-3) / 1e12 /
                          fp64_peak.value if dp_flops else None)},
    }

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        nside = args.cpu_nside or cpu_nside(args.workload, args.cpu_steps)
        rate, ncpu, nproc, secs = oracle_throughput(args.workload, nside,
                                                    args.cpu_steps)
        cpu = {"value": rate, "unit": "cell-steps/s", "cores": nproc,
               "kind": "port",
               "sample": "%d processes (one per host core), each marching "
                         "its own %d-cell seeded sample (same generator, "
                         "nside=%d) for %d steps; %.1f s" % (
                             nproc, ncpu, nside, args.cpu_steps, secs)}

    headline = {}
    if (rank == 0 and world == 1 and args.workload == "tri2d"
            and args.precision is None and args.nside is None
            and not args.no_headline):
        del core
        headline = headline_figures(local)

    line = {
        "metric": "cell-steps/s", "value": value, "unit": "cell-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if precision == "fp64" else "f32",
        "data": "synthetic",
        "config": {"workload": "%s (%s)" % (args.workload, _desc(w)),
                   "cells": ncell, "precision": precision, "dt": dt,
                   "l2": "state larger than L2 (no flush needed)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "setup_s": t_setup},
        "roofline": roofline, "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "cell-steps/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps},
        "gpu_launches": launches, "clocks": clocks.summary(),
        "check": {"finite": finite, "cflo_range": [lo, hi]},
    }
    line.update(headline)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
