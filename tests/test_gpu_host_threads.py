"""Host-path calls from worker threads, each on a CUDA stream of its own.

A caller serving many systems through the reference-facing API runs them from
several host threads (the library calls and numpy's bulk work release the GIL,
so one system's host work overlaps another's device work).  The same calls made
from four threads on four dedicated streams must give, bit for bit, what they
give one after another on the caller's stream: propose_with_dats through the
pinned host arrays, a Metropolis accept, three rounds.  Afterwards the systems'
page-locked arrays are released, the streams destroyed and the systems freed,
and the process carries on.
"""
import threading

import numpy as np
import pytest

from conftest import neutral_charges
from coulomb_kmc_gb300 import KMCFMM, _native
from coulomb_kmc_gb300.dats import make_state

pytestmark = pytest.mark.gpu
NSYS, ROUNDS, E = 4, 3, 9.0


def _systems():
    out = []
    for i in range(NSYS):
        rng = np.random.default_rng(100 + i)
        n = 500 + 150 * i
        P = rng.uniform(-0.5 * E, 0.5 * E, (n, 3))
        st = make_state(P, neutral_charges(n), E)
        k = KMCFMM(st.P, st.Q, st.domain, r=3, l=8, boundary_condition="pbc" if i % 2 else "free_space",
                   max_move=1.0, precision="mixed_fp64_accept")
        k.initialise()
        out.append(k)
    return out


def _moves():
    """Per system and round: proposals (one per charge), the charge tried, the uniform draw."""
    rng = np.random.default_rng(7)
    moves = []
    for i in range(NSYS):
        n = 500 + 150 * i
        moves.append([(rng.uniform(-0.45, 0.45, (n, 3)), int(rng.integers(0, n)), float(rng.uniform()))
                      for _ in range(ROUNDS)])
    return moves


def _run_system(k, mv, log):
    hb = k.host_buffers(1)
    hb["current_sites"][:] = 0
    hb["prop_masks"][:] = 1
    smc = np.array([1], np.int64)
    for step, pid, u in mv:
        pos = k.state()["positions"]
        prop = np.clip(pos + step, -0.5 * E, 0.5 * E)
        hb["prop_positions"][:] = prop
        k.propose_with_dats(smc, hb["current_sites"], hb["prop_positions"], hb["prop_masks"],
                            hb["prop_energy_diffs"])
        de = hb["prop_energy_diffs"][:, 0].copy()
        log.append(de)
        if u < np.exp(-de[pid]):
            k.accept((pid, prop[pid].copy()))
    log.append(k.energy)


def test_threaded_host_path_matches_sequential_and_streams_can_go():
    import torch
    moves = _moves()
    seq = _systems()
    logs_seq = [[] for _ in range(NSYS)]
    for k, mv, lg in zip(seq, moves, logs_seq):
        _run_system(k, mv, lg)
    torch.cuda.synchronize()

    thr = _systems()
    logs_thr = [[] for _ in range(NSYS)]
    streams = [_native.DedicatedStream() for _ in range(NSYS)]
    dev = torch.cuda.current_device()
    errors = []

    def work(i):
        try:
            torch.cuda.set_device(dev)
            with torch.cuda.stream(streams[i].stream):
                _run_system(thr[i], moves[i], logs_thr[i])
                streams[i].stream.synchronize()
        except Exception as e:  # reported below, on the test's thread
            errors.append(e)

    ts = [threading.Thread(target=work, args=(i,)) for i in range(NSYS)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert not errors, errors
    for a, b in zip(logs_seq, logs_thr):
        for x, y in zip(a, b):
            assert np.array_equal(np.asarray(x), np.asarray(y))

    # release the staging arrays while the streams exist, then end the streams
    for k in thr:
        k.release_host_buffers()
        k._set_stream()
    torch.cuda.synchronize()
    for st in streams:
        st.close()
    for k in thr + seq:
        k.free()
    # the process carries on: pinned and device allocations, a copy, a sync
    h = torch.empty(1 << 20, dtype=torch.float64, pin_memory=True)
    d = torch.ones(1 << 20, dtype=torch.float64, device="cuda")
    h.copy_(d, non_blocking=True)
    torch.cuda.synchronize()
    assert float(h[0]) == 1.0
    del h, d
    torch.cuda.synchronize()
