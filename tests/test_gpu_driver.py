"""Device-side KMC driver (generation, selection, occupancy on the GPU) against
the host restatement of the same bookkeeping with the same Philox draws:
the sequence of selected moves and the final occupancy / positions are
identical, energies agree within 1e-10 (FP64 path)."""
import numpy as np
import pytest

from conftest import neutral_charges, rel_err
from oracle.kmc_driver_ref import LatticeRef, OffLatticeRef
from coulomb_kmc_gb300 import KMCFMM
from coulomb_kmc_gb300.dats import make_state
from coulomb_kmc_gb300.driver import KMCDriver
from coulomb_kmc_gb300.workloads import LatticeHopSystem

pytestmark = pytest.mark.gpu


def lattice_pair(bc, side=16, seed=3, precision="fp64", R=3, L=8):
    hs = LatticeHopSystem(side=side, occupancy=0.25, seed=seed)
    out = []
    for _ in range(2):
        st = make_state(hs.positions(), hs.charges(), hs.extent)
        k = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition=bc, max_move=1.0, precision=precision)
        k.initialise()
        out.append(k)
    return hs, out


@pytest.mark.parametrize("bc", ["pbc", "free_space"])
def test_lattice_driver_matches_host(bc):
    nsteps, seed, beta = 12, 77, 2.0
    hs, (kd, kh) = lattice_pair(bc)
    drv = KMCDriver(kd, "lattice", beta, seed=seed, lattice_side=hs.side, lattice_sites=hs.site_of,
                    log_capacity=64)
    drv.step(nsteps)
    pid_d, tgt_d, de_d = drv.log()
    ref = LatticeRef(hs.side, hs.extent, hs.site_of, bc != "free_space", beta, seed)
    pids, tgts, des = [], [], []
    for _ in range(nsteps):
        ppos, masks, tsite = ref.proposals()
        diffs = np.zeros((hs.n, 6))
        kh.propose_with_dats(np.array([6], np.int64), np.zeros((hs.n, 1), np.int64), ppos, masks, diffs)
        idx = ref.select(diffs, masks)
        pid, h = idx // 6, idx % 6
        newp = ppos[pid, 3 * h:3 * h + 3].copy()
        pid, ns = ref.commit(idx, tsite)
        kh.accept((pid, newp))
        pids.append(pid)
        tgts.append(ns)
        des.append(diffs.ravel()[idx])
    assert np.array_equal(pid_d, pids)
    assert np.array_equal(tgt_d, tgts)
    assert np.max(rel_err(de_d, np.array(des))) < 1e-10
    assert np.array_equal(drv.sites(), ref.site_of)
    assert drv.counters() == (nsteps, nsteps)
    assert rel_err(kd.energy, kh.energy) < 1e-10
    sd, sh = kd.state(), kh.state()
    assert np.array_equal(sd["positions"], sh["positions"])
    assert np.array_equal(sd["occupancy"], sh["occupancy"])
    drv.free()
    kd.free()
    kh.free()


def test_offlattice_driver_matches_host():
    N, E, nsteps, seed, beta, stepw = 500, 10.0, 20, 5, 1.0, 0.5
    rng = np.random.default_rng(2)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    Q = neutral_charges(N)
    ks = []
    for _ in range(2):
        st = make_state(P, Q, E)
        k = KMCFMM(st.P, st.Q, st.domain, r=3, l=8, boundary_condition="free_space", max_move=1.0)
        k.initialise()
        ks.append(k)
    kd, kh = ks
    drv = KMCDriver(kd, "offlattice", beta, seed=seed, step=stepw, log_capacity=64)
    drv.step(nsteps)
    pid_d, tgt_d, de_d = drv.log()
    ref = OffLatticeRef(P, E, stepw, beta, seed)
    pids, chosen, acc_n = [], [], 0
    for _ in range(nsteps):
        prop = ref.proposals()
        diffs = np.zeros((N, 1))
        kh.propose_with_dats(np.array([1], np.int64), np.zeros((N, 1), np.int64), prop, np.ones((N, 1), np.int64),
                             diffs)
        i, acc = ref.select(diffs[:, 0])
        if acc:
            kh.accept((i, prop[i].copy()))
            acc_n += 1
        ref.commit(i, acc, prop)
        pids.append(i if acc else -1)
        chosen.append(i)
    assert np.array_equal(pid_d, pids)
    assert np.array_equal(tgt_d, chosen)
    assert drv.counters() == (nsteps, acc_n)
    assert np.array_equal(kd.state()["positions"], ref.pos)
    assert rel_err(kd.energy, kh.energy) < 1e-10
    drv.free()
    kd.free()
    kh.free()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_replay_equals_steps(precision):
    hs, (ka, kb) = lattice_pair("pbc", precision=precision)
    da = KMCDriver(ka, "lattice", 2.0, seed=9, lattice_side=hs.side, lattice_sites=hs.site_of, log_capacity=32)
    db = KMCDriver(kb, "lattice", 2.0, seed=9, lattice_side=hs.side, lattice_sites=hs.site_of, log_capacity=32)
    da.step(10)
    db.capture()
    db.launch(10)
    la, lb = da.log(), db.log()
    for x, y in zip(la, lb):
        assert np.array_equal(x, y)
    assert ka.energy == kb.energy
    assert np.array_equal(ka.state()["local_expansions"], kb.state()["local_expansions"])
    for o in (da, db, ka, kb):
        o.free()


def test_driver_rejects_bad_setup():
    hs, (k, k2) = lattice_pair("pbc")
    bad = hs.site_of.copy()
    bad[0] = bad[1]
    with pytest.raises(RuntimeError):
        KMCDriver(k, "lattice", 2.0, lattice_side=hs.side, lattice_sites=bad)
    with pytest.raises(RuntimeError):
        KMCDriver(k, "offlattice", 1.0, step=2.0)  # beyond max_move = 1
    with pytest.raises(ValueError):
        KMCDriver(k, "hop", 1.0)
    k.free()
    k2.free()
