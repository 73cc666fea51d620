"""Launch-shape tuning and size-bucket launches change no result.

* Every candidate of the keys the autotuners search (blocks per cell of the
  mixed near field, proposals per block of the per-proposal lattice kernels,
  cells per block and blocks per SM of the FP64 accept kernel, with 16 source
  groups for pbc and 2 for free space) gives
  the same selections, positions, energy and expansions, bit for bit, as the
  built-in choice, over a chain of device-driven KMC steps; so does whatever
  kmc_autotune picks.
* A round launched as size-bucket graphs (one graph per bucket holding every
  member's captured step) leaves every system exactly as the per-system stream
  launches do.
"""
import numpy as np
import pytest

from coulomb_kmc_gb300 import KMCFMM, _native
from coulomb_kmc_gb300.dats import make_state
from coulomb_kmc_gb300.driver import KMCDriver
from coulomb_kmc_gb300.serving import Request, Server, Slot, build_system
from coulomb_kmc_gb300.workloads import LatticeHopSystem

pytestmark = pytest.mark.gpu


def _run(tune=None, autotune=False, steps=12):
    hs = LatticeHopSystem(side=24, occupancy=0.25, seed=5)
    st = make_state(hs.positions(), hs.charges(), hs.extent)
    # R = 3: 4^3 cells of 216 sites, ~54 charges and many more proposals per cell, so the
    # near field's cells take several rounds of items (the case blocks per cell changes)
    k = KMCFMM(st.P, st.Q, st.domain, r=3, l=12, boundary_condition="pbc", max_move=1.0,
               precision="mixed_fp64_accept")
    k.initialise()
    d = KMCDriver(k, "lattice", 2.0, seed=31, lattice_side=hs.side, lattice_sites=hs.site_of, log_capacity=64)
    d.step(1)
    chosen = None
    if autotune:
        chosen = k.autotune(reps=3)
    for key, val in (tune or {}).items():
        k.set_tuning(key, val)
    d.capture()
    d.launch(steps)
    out = (d.log(), k.energy, k.state())
    d.free()
    k.free()
    return out, chosen


def _run_free(tune=None, steps=12):
    rng = np.random.default_rng(8)
    N, E = 3000, 22.0
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    Q = np.where(np.arange(N) % 2 == 0, 1.0, -1.0)
    st = make_state(P, Q, E)
    k = KMCFMM(st.P, st.Q, st.domain, r=4, l=12, boundary_condition="free_space", max_move=1.0,
               precision="mixed_fp64_accept")
    k.initialise()
    d = KMCDriver(k, "offlattice", 1.0, seed=12, step=0.5, log_capacity=64)
    for key, val in (tune or {}).items():
        k.set_tuning(key, val)
    d.capture()
    d.launch(steps)
    out = (d.log(), k.energy, k.state())
    d.free()
    k.free()
    return out, None


def _same(a, b):
    (la, ea, sa), (lb, eb, sb) = a, b
    for x, y in zip(la, lb):
        assert np.array_equal(x, y)
    assert ea == eb
    assert np.array_equal(sa["positions"], sb["positions"])
    assert np.array_equal(sa["local_expansions"], sb["local_expansions"])


def test_every_tuning_candidate_is_bit_identical():
    ref, _ = _run()
    for val in (64, 256):
        got, _ = _run({_native.KMC_TUNE_LR_THREADS: val})
        _same(ref, got)
    for val in (4, 8):
        got, _ = _run({_native.KMC_TUNE_P2L64_CELLS: val})
        _same(ref, got)
    for val in (2, 4):
        got, _ = _run({_native.KMC_TUNE_NEAR_SPLIT: val})
        _same(ref, got)
    for val in (1, 2):
        got, _ = _run({_native.KMC_TUNE_P2L64_PER_SM: val})
        _same(ref, got)
    got, _ = _run({_native.KMC_TUNE_NEAR_PRIORITY: 1})
    _same(ref, got)


def test_fp64_accept_shapes_bit_identical_in_free_space():
    ref, _ = _run_free()
    for tune in ({_native.KMC_TUNE_P2L64_CELLS: 4}, {_native.KMC_TUNE_P2L64_CELLS: 8},
                 {_native.KMC_TUNE_P2L64_PER_SM: 1}):
        got, _ = _run_free(tune)
        _same(ref, got)


def test_autotuned_choice_is_bit_identical():
    ref, _ = _run()
    got, chosen = _run(autotune=True)
    assert chosen[_native.KMC_TUNE_LR_THREADS] in (0, 64, 256)
    assert chosen[_native.KMC_TUNE_P2L64_CELLS] in (0, 4, 8)
    _same(ref, got)


def test_bucket_rounds_equal_stream_rounds():
    reqs = [Request(rid=i, kind="offlattice" if i % 2 else "lattice", bc="free_space" if i % 2 else "pbc",
                    n=1200 + 300 * (i % 3), rounds=6, seed=40 + i) for i in range(8)]
    res = {}
    for mode in ("streams", "buckets"):
        srv = Server(precision="mixed_fp64_accept", n_workers=4, launch=mode)
        slots = []
        for r in reqs:
            k, d = build_system(r, "mixed_fp64_accept")
            slots.append(Slot(req=r, kmc=k, drv=d, nbytes=0, admitted=0.0))
        for _ in range(6):
            srv.round(slots)
        res[mode] = [(sl.kmc.energy, sl.drv.stats(), sl.kmc.state()["positions"]) for sl in slots]
        srv.free_buckets()
        for sl in slots:
            sl.drv.free()
            sl.kmc.free()
    for a, b in zip(res["streams"], res["buckets"]):
        assert a[0] == b[0] and a[1] == b[1]
        assert np.array_equal(a[2], b[2])


def test_round_tuner_keeps_results_and_each_systems_own_values():
    """Server.autotune_keys over combinations of the FP64 accept's cells per block and
    residency: the rounds it times are real rounds, the systems end as untuned ones
    do after the same number of rounds, and a candidate that leaves a key out keeps
    every system's own value."""
    reqs = [Request(rid=i, kind="offlattice", bc="pbc" if i % 2 else "free_space", n=1500 + 400 * i, rounds=8,
                    seed=60 + i) for i in range(4)]
    kc, ks = _native.KMC_TUNE_P2L64_CELLS, _native.KMC_TUNE_P2L64_PER_SM
    res = {}
    for tuned in (False, True):
        srv = Server(precision="mixed_fp64_accept", n_workers=4)
        slots = []
        for r in reqs:
            k, d = build_system(r, "mixed_fp64_accept")
            k.set_tuning(kc, 4)  # each system's own value, kept by the empty candidate
            slots.append(Slot(req=r, kmc=k, drv=d, nbytes=0, admitted=0.0))
        n_rounds = 0
        if tuned:
            combos = [{}, {ks: 1}, {kc: 2, ks: 3}]
            best, ms = srv.autotune_keys(slots, combos, rounds=1)
            assert len(ms) == 3 and 0 <= best < 3
            n_rounds = 3 * 2
            want = {kc: 4, ks: 0}
            want.update(combos[best])
            for sl in slots:
                assert sl.kmc.get_tuning(kc) == want[kc] and sl.kmc.get_tuning(ks) == want[ks]
        for _ in range(8 - n_rounds):
            srv.round(slots)
        res[tuned] = [(sl.kmc.energy, sl.drv.stats(), sl.kmc.state()["positions"]) for sl in slots]
        srv.free_buckets()
        for sl in slots:
            sl.drv.free()
            sl.kmc.free()
    for a, b in zip(res[False], res[True]):
        assert a[0] == b[0] and a[1] == b[1]
        assert np.array_equal(a[2], b[2])
