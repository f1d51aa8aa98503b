"""Serving loop: continuous batching of 2D and 1D solves.

Each request's result must be the same served in a mix as marched alone
(bit-identical: the batched 2D march is per-core exact and a reused slot is
reset to a fresh solver's tables); the HBM budget must bound the resident
set; requests that arrive while others run must be admitted and finish.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _server(budget=1 << 34, max_chunk=16):
    from solvcon_gb300 import meshgen
    from solvcon_gb300.serving import Server
    srv = Server(hbm_budget=budget, max_chunk=max_chunk, precision="fp32")
    for key, (n, g, seed) in enumerate([(6, 1.4, 1), (11, 1.2, 2),
                                        (17, 1.6, 3)]):
        x, t, c = meshgen.tri_square(n, 0.2, seed)
        mesh = meshgen.build_mesh(2, x, t, c)
        clcnd = np.asarray(mesh.clcnd.ndarray)[mesh.ngstcell:]
        state = meshgen.quadrant_state(clcnd, seed, g)
        faces = np.asarray(mesh.bndfcs.ndarray[:, 0]).copy()
        srv.add_mesh(key, mesh, state, faces, g, 1e-3 * (1 + key))
    return srv


def _requests():
    from solvcon_gb300.serving import Request
    # Staggered arrivals: later requests arrive while earlier ones run.
    return [Request(0, "2d", 40, 0.000, mesh_key=0),
            Request(1, "1d", 37, 0.000, ncoord=1001, seed=5),
            Request(2, "2d", 23, 0.002, mesh_key=1),
            Request(3, "2d", 51, 0.004, mesh_key=2),
            Request(4, "1d", 19, 0.005, ncoord=3001, seed=6),
            Request(5, "2d", 33, 0.006, mesh_key=0),
            Request(6, "2d", 17, 0.008, mesh_key=1)]


def test_results_same_alone_and_in_the_mix():
    from solvcon_gb300.serving import alone
    srv = _server()
    reqs = _requests()
    done = srv.run(reqs)
    assert sorted(r.rid for r in done) == list(range(len(reqs)))
    assert srv.peak_resident >= 2
    for r in done:
        ref, _ = alone(srv, r, "fp32")
        np.testing.assert_array_equal(r.result, ref, "request %d" % r.rid)
        assert r.latency >= 0 and r.t_admit >= r.arrival - 1e-9


def _jump_clock():
    """A clock that advances one second per reading: every request has
    arrived by the first tick, so admission depends on the budget alone and
    not on how fast the device runs."""
    import itertools
    return itertools.count(0.0, 1.0).__next__


def test_budget_limits_resident_set():
    from solvcon_gb300.serving import alone
    budget = 1200000
    srv = _server(budget=budget, max_chunk=8)
    reqs = _requests()
    done = srv.run(reqs, clock=_jump_clock())
    assert len(done) + len(srv.rejected) == len(reqs)
    assert not srv.rejected
    assert srv.peak_held <= budget
    big = _server(budget=1 << 34, max_chunk=8)
    big.run(_requests(), clock=_jump_clock())
    assert big.peak_resident == len(reqs)
    assert 1 <= srv.peak_resident <= big.peak_resident
    for r in done:
        ref, _ = alone(srv, r, "fp32")
        np.testing.assert_array_equal(r.result, ref, "request %d" % r.rid)


def test_results_same_alone_in_a_long_mixed_run():
    """The served workload's mix at a reduced scale: ticks of up to 32 steps
    (the 1D tubes then replay their captured 32-step graphs while the 2D
    batch runs), one batch re-pointed at member sets that grow and shrink
    from tick to tick, and the 1k-100k point tubes.  Every request must
    still equal its march alone bit for bit."""
    from solvcon_gb300 import meshgen
    from solvcon_gb300.serving import Server, alone, make_requests
    srv = Server(hbm_budget=1 << 34, max_chunk=32, precision="fp32")
    for key, (n, g, seed) in enumerate([(6, 1.4, 1), (13, 1.2, 2),
                                        (21, 1.6, 3), (34, 1.3, 4),
                                        (9, 1.5, 5), (27, 1.1, 6)]):
        x, t, c = meshgen.tri_square(n, 0.2, seed)
        mesh = meshgen.build_mesh(2, x, t, c)
        clcnd = np.asarray(mesh.clcnd.ndarray)[mesh.ngstcell:]
        state = meshgen.quadrant_state(clcnd, seed, g)
        faces = np.asarray(mesh.bndfcs.ndarray[:, 0]).copy()
        srv.add_mesh(key, mesh, state, faces, g, 2e-4 * (1 + key))
    reqs = make_requests(32, 2000.0, list(range(6)), seed=11,
                         steps=(33, 140))
    done = srv.run(reqs)
    assert sorted(r.rid for r in done) == list(range(len(reqs)))
    assert srv.rebuilds > 4 and srv.peak_resident >= 4
    assert any(r.kind == "1d" and r.steps >= 32 for r in done)
    for r in done:
        ref, _ = alone(srv, r, "fp32")
        np.testing.assert_array_equal(r.result, ref, "request %d" % r.rid)


def test_oversized_request_is_rejected():
    from solvcon_gb300.serving import Request
    srv = _server(budget=100000)
    done = srv.run([Request(0, "2d", 5, 0.0, mesh_key=2),
                    Request(1, "1d", 5, 0.0, ncoord=1001, seed=1)])
    assert [r.rid for r in srv.rejected] == [0]
    assert [r.rid for r in done] == [1]
