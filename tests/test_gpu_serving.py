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
