"""GPU FP64 path against the CPU oracle at the benchmark configurations' own sizes,
against the golden fixtures, and against an Ewald sum.

* Plain FP64 free space: N = 1,000 charges in a box of edge 12, R = 3, L = 12,
  10 steps of one proposal per charge (uniform in [-0.5, 0.5]^3, re-drawn
  inside the box) and a Metropolis accept at beta = 1: every difference within
  1e-10 relative (denominator max(|dE|, 1)), the energy within 1e-10 and the
  occupancy bit-exact after the chain.
* pbc lattice hopping on 48^3 sites (27,648 charges, R = 5, L = 12): one full
  step's ~124.5k proposals within 1e-10, then 10 rejection-free accepts with
  bit-exact occupancy and cells, and a second full step within 1e-10.  The
  initial local expansions come from the GPU's FMM solve (as the reference's
  come from ppmd's FMM); the oracle is fed the same expansions.
* pbc lattice hopping on 64^3 sites (65,536 charges, R = 6), L = 8, 12, 16: one
  full step's ~295k proposals within 1e-10 each.
* The golden fixtures (the reference tests' own RandomState streams,
  tests/golden/make_golden.py) through the GPU: total energies of proposed
  moves within the reference tests' 1e-5 of the direct sums.
* 1,024 sampled proposals of the 48^3 lattice workload against the Ewald sum
  (the reference's PBCDirect/Ewald pin, tests/host/test_propose_dat_setup.py:
  564-705 and tests/host/test_common.py:106-182): the proposed total energy
  within the reference's 1e-5 relative, and the RMS difference error within
  1e-4 (denominator max(|dE|, 1)); max and RMS are printed.  The error is the
  expansion truncation of the L = 12 FMM state, as in the reference.
"""
import numpy as np
import pytest

from conftest import load_golden, rel_err
from oracle import kmc_oracle as ko
from coulomb_kmc_gb300 import KMCFMM
from coulomb_kmc_gb300.dats import make_state
from coulomb_kmc_gb300.lattice import lattice_operator
from coulomb_kmc_gb300.workloads import LatticeHopSystem, OffLatticeSystem

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _dats_step(k, ppos, masks):
    n, M = masks.shape
    d = np.zeros((n, M))
    k.propose_with_dats(np.array([M], np.int64), np.zeros((n, 1), np.int64), ppos, masks, d)
    return d


def test_free_space_n1000_metropolis_chain():
    hs = OffLatticeSystem(1000, 12.0, seed=0, step=0.5)
    P, Q = hs.positions(), hs.charges()
    st = make_state(P, Q, 12.0)
    g = KMCFMM(st.P, st.Q, st.domain, r=3, l=12, boundary_condition="free_space")
    g.initialise()
    o = ko.OracleKMC(P.copy(), Q, 12.0, 3, 12, "free_space")
    o.initialise()
    assert rel_err(g.energy, o.energy) < TOL
    rng = np.random.default_rng(100)
    ones = np.ones((hs.n, 1), np.int64)
    for _ in range(10):
        prop = hs.proposals(rng)
        dg, do = _dats_step(g, prop, ones), _dats_step(o, prop, ones)
        assert np.max(rel_err(dg, do)) < TOL
        pid = int(rng.integers(0, hs.n))
        if rng.uniform() < np.exp(-1.0 * do[pid, 0]):
            g.accept((pid, prop[pid].copy()))
            o.accept((pid, prop[pid].copy()))
            hs.pos[pid] = prop[pid]
        assert rel_err(g.energy, o.energy) < TOL
    s = g.state()
    assert np.array_equal(s["occupancy"], o.cell_occupancy())
    assert np.array_equal(s["cells"], o.fmm_cells)
    assert np.array_equal(s["positions"], o.positions)
    g.free()


def _lattice_pair(side, R, L, seed):
    hs = LatticeHopSystem(side, 0.25, seed=seed)
    st = make_state(hs.positions(), hs.charges(), hs.extent)
    g = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition="pbc", max_move=1.0)
    g.initialise()
    o = ko.OracleKMC(hs.positions(), hs.charges(), hs.extent, R, L, "pbc", max_move=1.0,
                     lr_operator=lattice_operator(L, hs.extent))
    o.initialise(local_expansions=g.state()["local_expansions"])
    return hs, g, o


def test_lattice48_full_step_and_accept_chain():
    hs, g, o = _lattice_pair(48, 5, 12, seed=1)
    assert rel_err(g.energy, o.energy) < TOL
    ppos, masks, tsite = hs.proposals()
    assert masks.sum() > 120000
    dg, do = _dats_step(g, ppos, masks), _dats_step(o, ppos, masks)
    act = masks > 0
    assert np.max(rel_err(dg[act], do[act])) < TOL
    rng = np.random.default_rng(7)
    for _ in range(10):
        ppos, masks, tsite = hs.proposals()
        do = _dats_step(o, ppos, masks)
        pid, h = hs.select(do, masks, rng, 2.0)
        mv = ppos[pid, 3 * h:3 * h + 3].copy()
        g.accept((pid, mv))
        o.accept((pid, mv))
        hs._commit(pid, int(hs.site_of[pid]), int(tsite[pid, h]))
        assert rel_err(g.energy, o.energy) < TOL
    s = g.state()
    assert np.array_equal(s["occupancy"], o.cell_occupancy())
    assert np.array_equal(s["cells"], o.fmm_cells)
    assert np.array_equal(s["positions"], o.positions)
    b = o.primary_local_expansions()
    assert np.max(np.abs(s["local_expansions"] - b)) <= TOL * np.max(np.abs(b))
    ppos, masks, _ = hs.proposals()
    dg, do = _dats_step(g, ppos, masks), _dats_step(o, ppos, masks)
    act = masks > 0
    assert np.max(rel_err(dg[act], do[act])) < TOL
    g.free()


@pytest.mark.parametrize("L", [8, 12, 16])
def test_lattice64_full_step(L):
    hs, g, o = _lattice_pair(64, 6, L, seed=2)
    assert rel_err(g.energy, o.energy) < TOL
    ppos, masks, _ = hs.proposals()
    assert masks.sum() > 280000
    dg, do = _dats_step(g, ppos, masks), _dats_step(o, ppos, masks)
    act = masks > 0
    assert np.max(rel_err(dg[act], do[act])) < TOL
    g.free()


@pytest.mark.parametrize("name,bc", [("free_space_1", "free_space"), ("nearest27_1", "27"), ("pbc_1", "pbc")])
def test_golden_fixtures_on_gpu(name, bc):
    gd = load_golden(name)
    E = float(gd["E"])
    st = make_state(gd["P"].copy(), gd["Q"], E)
    g = KMCFMM(st.P, st.Q, st.domain, r=3, l=12, boundary_condition=bc)
    g.initialise()
    assert rel_err(g.energy, gd["e0"]) < 1e-5
    moves = tuple((int(p), np.asarray(m).reshape(1, 3)) for p, m in zip(gd["pids"], gd["moves"]))
    got = np.concatenate(g.propose(moves))
    assert np.max(np.abs(got - gd["energies"]) / np.abs(gd["energies"])) < 1e-5
    g.free()


def test_golden_multi_move_fixture_on_gpu():
    gd = load_golden("free_space_2")
    st = make_state(gd["P"].copy(), gd["Q"], float(gd["E"]))
    g = KMCFMM(st.P, st.Q, st.domain, r=3, l=12, boundary_condition="free_space")
    g.initialise()
    moves, k = [], 0
    for pid, c in zip(gd["pids"], gd["counts"]):
        moves.append((int(pid), gd["moves"][k:k + c]))
        k += c
    got = np.concatenate(g.propose(moves))
    assert np.max(np.abs(got - gd["energies"]) / np.abs(gd["energies"])) < 1e-5
    g.free()


@pytest.mark.parametrize("precision", ["fp64", "mixed_fp64_accept"])
def test_lattice48_sampled_proposals_vs_ewald(precision):
    from oracle.ewald import ewald_move_differences
    hs = LatticeHopSystem(48, 0.25, seed=1)
    st = make_state(hs.positions(), hs.charges(), hs.extent)
    g = KMCFMM(st.P, st.Q, st.domain, r=5, l=12, boundary_condition="pbc", max_move=1.0, precision=precision)
    g.initialise()
    ppos, masks, _ = hs.proposals()
    d = _dats_step(g, ppos, masks)
    rng = np.random.default_rng(1024)
    act = np.argwhere(masks > 0)
    sel = act[rng.choice(len(act), 1024, replace=False)]
    ref = ewald_move_differences(hs.positions(), hs.charges(), hs.extent, sel[:, 0],
                                 np.stack([ppos[p, 3 * h:3 * h + 3] for p, h in sel]))
    got = d[sel[:, 0], sel[:, 1]]
    err = rel_err(got, ref)
    # the reference's criterion: the proposed total energy E + dE against the direct
    # (Ewald) total within 1e-5 relative (test_propose_dat_setup.py:697-705); the
    # difference's share of that error is |dE - dE_ewald| / |E|
    tot = np.abs(got - ref) / abs(g.energy)
    print(f"\n{precision}: 1,024 sampled 48^3 proposals vs Ewald: dE error (denominator max(|dE|, 1)) max "
          f"{err.max():.3e} RMS {np.sqrt(np.mean(err * err)):.3e}; relative to the total energy max {tot.max():.3e}")
    assert tot.max() < 1e-5
    assert np.sqrt(np.mean(err * err)) < 1e-4
    g.free()
