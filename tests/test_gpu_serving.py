"""Serving loop (continuous batching of independent KMC systems): each
system's result is the same alone and in the mix, admission respects the
slot and memory limits, and every request completes."""
import numpy as np
import pytest

from coulomb_kmc_gb300.serving import Request, Server, build_system, estimate_bytes

pytestmark = pytest.mark.gpu


def reqs():
    return [Request(rid=0, kind="lattice", bc="pbc", n=1500, rounds=7, seed=11, arrival=0.0),
            Request(rid=1, kind="offlattice", bc="free_space", n=2500, rounds=9, seed=12, arrival=0.0),
            Request(rid=2, kind="lattice", bc="pbc", n=900, rounds=5, seed=13, arrival=0.01),
            Request(rid=3, kind="offlattice", bc="free_space", n=1200, rounds=6, seed=14, arrival=0.02)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_same_alone_and_in_the_mix(precision):
    rs = reqs()
    alone = {}
    for r in rs:
        k, d = build_system(r, precision)
        d.launch(r.rounds)
        alone[r.rid] = (k.energy, d.stats(), k.state()["positions"])
        d.free()
        k.free()
    srv = Server(precision=precision, n_workers=3, keep_results=True)
    st = srv.serve(rs, realtime=True)
    assert st["requests"] == len(rs)
    for r in rs:
        got = srv.results[r.rid]
        e, stats, pos = alone[r.rid]
        assert got["energy"] == e
        assert got["stats"] == stats
        assert np.array_equal(got["positions"], pos)


def test_admission_limits():
    rs = reqs()
    srv = Server(precision="mixed", max_active=1, n_workers=2)
    st = srv.serve(rs, realtime=False)
    assert st["requests"] == len(rs) and srv.peak_active == 1
    # a budget that fits only the largest request on its own
    big = max(estimate_bytes(r.n, r.kind, r.L, 3) for r in rs)
    srv2 = Server(precision="mixed", hbm_budget=big * 1.01, n_workers=2)
    st2 = srv2.serve(rs, realtime=False)
    assert st2["requests"] == len(rs) and srv2.peak_active <= 2
    assert st2["round_ms_p99"] >= st2["round_ms_p50"] > 0.0


def test_dedicated_streams_are_distinct():
    """Drivers and the server run on dedicated streams: torch.cuda.Stream() takes
    streams from a fixed pool round-robin, so a few dozen of them alias, and a
    step captured on one stream while another thread launches on its alias fails
    (cudaErrorStreamCaptureIsolation)."""
    import torch
    from coulomb_kmc_gb300 import _native
    own = [_native.DedicatedStream() for _ in range(48)]
    assert len({d.cuda_stream for d in own}) == 48
    assert len({torch.cuda.Stream().cuda_stream for _ in range(48)}) < 48
    for d in own:
        d.close()


def test_concurrent_admission_many_systems():
    """Many small systems admitted by several threads while rounds run (the
    case that aliased pooled streams broke): every request completes."""
    rs = [Request(rid=i, kind="lattice" if i % 2 else "offlattice", bc="pbc" if i % 2 else "free_space",
                  n=800 + 37 * i, rounds=3 + i % 4, seed=100 + i, arrival=0.002 * i) for i in range(40)]
    srv = Server(precision="mixed", n_workers=16, max_active=24, n_admit=4)
    st = srv.serve(rs, realtime=True)
    assert st["requests"] == len(rs)


def test_over_budget_request_is_rejected_and_the_rest_served():
    rs = reqs()
    rs.append(Request(rid=9, kind="offlattice", bc="free_space", n=200000, rounds=3, seed=19, arrival=0.0))
    budget = 2.0 * max(estimate_bytes(r.n, r.kind, r.L, 3) for r in rs[:-1])
    srv = Server(precision="mixed", hbm_budget=budget, n_workers=2)
    st = srv.serve(rs, realtime=False)
    assert st["requests"] == len(rs) - 1 and st["ended_without_running"] == 1
    assert srv.status[9].startswith("rejected")
    assert all(srv.status[r.rid] == "done" for r in rs[:-1])


def test_cancelled_requests_end_and_the_rest_match_alone():
    import threading
    rs = reqs()
    rs.append(Request(rid=7, kind="lattice", bc="pbc", n=1500, rounds=100000, seed=17, arrival=0.0))
    rs.append(Request(rid=8, kind="offlattice", bc="free_space", n=1500, rounds=5, seed=18, arrival=0.05))
    srv = Server(precision="mixed", n_workers=3, keep_results=True)
    srv.cancel(8)  # before it arrives: never admitted
    t = threading.Timer(0.5, srv.cancel, args=(7,))  # while it runs
    t.start()
    st = srv.serve(rs, realtime=True)
    t.join()
    assert srv.status[7] == "cancelled" and srv.status[8] == "cancelled"
    assert st["requests"] == len(rs) - 2
    for r in rs[:4]:
        k, d = build_system(r, "mixed")
        d.launch(r.rounds)
        assert srv.results[r.rid]["energy"] == k.energy
        assert np.array_equal(srv.results[r.rid]["positions"], k.state()["positions"])
        d.free()
        k.free()


def test_failed_round_launch_ends_the_run_with_an_error():
    """A round whose launch reports an error code (a fake of the call, on the host)
    ends serve() with that error promptly: no hang, admission threads joined, every
    system released."""
    srv = Server(precision="mixed", n_workers=2)
    real = srv._launch
    calls = []

    def fake(*a):
        calls.append(1)
        return -2 if len(calls) >= 3 else real(*a)

    srv._launch = fake
    with pytest.raises(RuntimeError, match="kmc_drivers_launch"):
        srv.serve(reqs(), realtime=False)
    assert len(calls) == 3
    assert srv.active == [] and srv.reserved == 0


def test_device_error_status_fails_only_that_request():
    """A system whose kernels counted an invalid move (here: the allocation-free entry
    point given an id outside the system, a bounds check on the device) retires with
    an error status; the others complete."""
    import torch
    from coulomb_kmc_gb300 import _native
    srv = Server(precision="mixed", n_workers=2, keep_results=True)
    orig = srv.admit

    def admit(r, stream=None):
        s = orig(r, stream)
        if r.rid == 1:
            ids = torch.tensor([10 ** 9], dtype=torch.int64, device="cuda")
            es = torch.tensor([0, 1], dtype=torch.int64, device="cuda")
            pos = torch.zeros(3, dtype=torch.float64, device="cuda")
            out = torch.zeros(1, dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            _native.check(_native.lib().kmc_propose_moves_noalloc(s.kmc._handle, 1, 1, ids.data_ptr(),
                                                                  es.data_ptr(), pos.data_ptr(), out.data_ptr()),
                          "noalloc")
            torch.cuda.synchronize()
        return s

    srv.admit = admit
    st = srv.serve(reqs(), realtime=False)
    assert st["requests"] == 4
    assert srv.status[1].startswith("error")
    assert all(srv.status[r] == "done" for r in (0, 2, 3))
