"""bench.py's host-side parts on the CPU: the oracle's all-core throughput
run, the sizes of its samples, and the reference arm's JSON line for the
multidim and the spacetime workloads (the GPU arm is exercised on the GPU)."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpu_sample_sizes():
    sys.path.insert(0, ROOT)
    import bench
    for wl in ("tri2d", "tet3d", "tube1d", "spacetime"):
        big, small = bench.cpu_nside(wl, 10), bench.cpu_nside(wl, 1000)
        assert big >= small > 0
    assert bench.cpu_nside("tube1d", 5) % 2 == 1


def test_oracle_throughput_all_processes():
    sys.path.insert(0, ROOT)
    import bench
    rate, units, nproc, secs = bench.oracle_throughput("tri2d", 8, 2,
                                                       warmup=1, nproc=2)
    assert nproc == 2 and units == 2 * 8 * 8 and rate > 0 and secs > 0


def _reference_line(*extra):
    run = subprocess.run([sys.executable, "bench.py", "--impl", "reference",
                          "--steps", "3", "--warmup", "3"] + list(extra),
                         cwd=ROOT, capture_output=True, text=True,
                         timeout=600)
    assert run.returncode == 0, run.stderr[-2000:]
    lines = [json.loads(x) for x in run.stdout.splitlines()
             if x.startswith("{")]
    assert len(lines) == 1
    return lines[0]


def test_reference_arm_line_multidim():
    line = _reference_line("--workload", "tri2d", "--cpu-nside", "10")
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup",
                "ms_per_step", "higher_is_better", "scaling", "vs_baseline",
                "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == "cell-steps/s"
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["value"] == line["value"]


def test_reference_arm_line_spacetime():
    line = _reference_line("--workload", "spacetime", "--cpu-nside", "500")
    assert line["metric"] == "point-steps/s" and line["value"] > 0
    assert line["config"]["sample_units"] == 2 * 500 + 1


def test_batch_mesh_morton_is_a_renumbering():
    """The batched workload's Morton cell order renumbers the same mesh: the
    same cells (as node lists), the same state per cell."""
    sys.path.insert(0, ROOT)
    import numpy as np
    import bench
    a = bench.batch_mesh(3, 900, 1.3, 2026, "native")
    b = bench.batch_mesh(3, 900, 1.3, 2026, "morton")
    ma, mb = a[0], b[0]
    assert ma.ncell == mb.ncell and ma.nface == mb.nface
    ca = np.array(ma.clnds.ndarray)[ma.ngstcell:, :4]
    cb = np.array(mb.clnds.ndarray)[mb.ngstcell:, :4]
    key = {tuple(r): i for i, r in enumerate(ca.tolist())}
    perm = np.array([key[tuple(r)] for r in cb.tolist()])
    assert sorted(perm.tolist()) == list(range(ma.ncell))
    assert not np.array_equal(perm, np.arange(ma.ncell))
    np.testing.assert_array_equal(b[1], a[1][perm])
    assert a[3] == b[3] and len(a[2]) == len(b[2])


def test_pin_device_one_gpu_per_rank(monkeypatch):
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.delenv("CUDA_VISIBLE_DEVICES", raising=False)
    bench.pin_device(3)
    assert os.environ["CUDA_VISIBLE_DEVICES"] == "3"
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "4,5,6,7")
    bench.pin_device(2)
    assert os.environ["CUDA_VISIBLE_DEVICES"] == "6"
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", "5")
    bench.pin_device(0)
    assert os.environ["CUDA_VISIBLE_DEVICES"] == "5"


def test_cpu_arm_loads_nothing_of_the_library():
    """The CPU arms build their samples with the plain-numpy generators and
    the oracle's own mesh build: neither the package nor libscg.so is
    loaded in the process that marches."""
    code = (
        "import sys, numpy as np\n"
        "sys.path.insert(0, %r)\n"
        "import bench\n"
        "for wl, n in (('tri2d', 12), ('tet3d', 3), ('tube1d', 101),\n"
        "              ('spacetime', 64)):\n"
        "    units, march = bench._oracle_setup(wl, n, 0)\n"
        "    march(1)\n"
        "assert not [m for m in sys.modules if m.startswith('solvcon_gb300')]\n"
        "assert 'libscg' not in open('/proc/self/maps').read()\n"
        "print('ok')\n" % ROOT)
    run = subprocess.run([sys.executable, "-c", code], cwd=ROOT,
                         capture_output=True, text=True, timeout=300)
    assert run.returncode == 0 and "ok" in run.stdout, run.stderr[-2000:]


def test_cpu_sample_equals_the_gpu_workload_sample():
    """The CPU arm's sample of the 2D workload is the GPU arm's workload at
    the same size and seed: same mesh tables, same state."""
    sys.path.insert(0, ROOT)
    import numpy as np
    import bench
    from oracle import oracle as ora
    w, mesh, state, faces = bench.make_workload("tri2d", nside=20,
                                                seed_offset=3)
    sy = bench.synth()
    m = ora.OracleMesh(2, *sy.tri_square(20, w["jitter"], w["seed"] + 3))
    for name in ("fcnds", "fccls", "clfcs", "clcnd", "clvol", "ndcrd"):
        np.testing.assert_array_equal(
            np.asarray(getattr(m, name)).ravel(),
            np.asarray(getattr(mesh, name).ndarray).ravel(), name)
    np.testing.assert_array_equal(
        sy.quadrant_state(m.clcnd[m.ngstcell:], seed=w["seed"] + 3), state)
    np.testing.assert_array_equal(m.bndfcs[:, 0], faces)
