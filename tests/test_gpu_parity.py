"""GPU FP64 path against the CPU oracle (same inputs, same initial state
definition): energies and differences within 1e-10 relative (denominator
max(|x|, 1)), local expansions within 1e-10 of their scale, occupancy after
accept chains bit-exact."""
import numpy as np
import pytest

from conftest import neutral_charges, rel_err
from oracle import kmc_oracle as ko
from coulomb_kmc_gb300 import KMCFMM
from coulomb_kmc_gb300.dats import Domain, make_state
from coulomb_kmc_gb300.lattice import lattice_operator

pytestmark = pytest.mark.gpu
TOL = 1e-10


def pair(bc, N=200, E=4.0, R=3, L=12, seed=8657, max_move=None, P=None, Q=None):
    rng = np.random.RandomState(seed=seed)
    if P is None:
        P = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(N, 3))
    if Q is None:
        Q = neutral_charges(len(P))
    st = make_state(P, Q, E)
    g = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition=bc, max_move=max_move)
    g.initialise()
    lr = lattice_operator(L, E) if bc == "pbc" else None
    o = ko.OracleKMC(P.copy(), Q, E, R, L, bc, max_move=max_move, lr_operator=lr)
    o.initialise()
    return g, o, rng, st


def assert_state_equal(g, o, tol=TOL):
    s = g.state()
    a, b = s["local_expansions"], o.primary_local_expansions()
    assert np.max(np.abs(a - b)) <= tol * max(1.0, np.max(np.abs(b)))
    assert np.array_equal(s["occupancy"], o.cell_occupancy())
    assert np.array_equal(s["cells"], o.fmm_cells)
    assert np.array_equal(s["positions"], o.positions)
    if o.bc == "pbc":
        assert np.max(np.abs(s["multipole"] - o.multipole_exp)) <= tol * max(1, np.max(np.abs(o.multipole_exp)))
    assert rel_err(g.energy, o.energy) < tol


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
@pytest.mark.parametrize("R", [3, 4])
def test_initial_state(bc, R):
    g, o, _, _ = pair(bc, R=R)
    assert_state_equal(g, o)
    g.free()


@pytest.mark.parametrize("L", [4, 10, 16])
def test_initial_state_other_orders(L):
    g, o, _, _ = pair("pbc", L=L, N=100)
    assert_state_equal(g, o)
    g.free()


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
def test_propose_moves(bc):
    """propose(moves): 1-7 moves per charge for every charge (test_free_space_1.py:235-336)."""
    g, o, rng, _ = pair(bc, N=100)
    E = 4.0
    order = rng.permutation(range(100))
    moves = [(int(order[i]), rng.uniform(low=-0.5 * E, high=0.5 * E, size=(rng.randint(1, 8), 3)))
             for i in range(100)]
    a = np.concatenate(g.propose(moves))
    b = np.concatenate(o.propose(moves))
    assert np.max(rel_err(a - g.energy, b - o.energy)) < TOL
    assert np.max(rel_err(a, b)) < TOL
    g.free()


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
@pytest.mark.parametrize("R", [3, 5])
def test_propose_with_dats(bc, R):
    """propose_with_dats with site types and masks (test_propose_dat_setup.py:564-735)."""
    N, E, M = 200, 4.0, 4
    g, o, rng, _ = pair(bc, N=N, R=R)
    smc = rng.randint(0, 10, size=8).astype(np.int64)
    sites = rng.randint(0, 8, size=(N, 1)).astype(np.int64)
    masks = np.zeros((N, M), np.int64)
    for px in range(N):
        mk = np.zeros(M)
        mk[:smc[sites[px, 0]]] = 1
        masks[px] = rng.permutation(mk)
    ppos = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(N, 3 * M))
    dg = np.full((N, M), 123.0)
    do = np.full((N, M), 123.0)
    g.propose_with_dats(smc, sites, ppos, masks, dg)
    o.propose_with_dats(smc, sites, ppos, masks, do)
    assert np.array_equal(dg == 123.0, do == 123.0)
    assert np.max(rel_err(dg, do)) < TOL
    g.free()


def test_propose_with_dats_device_tensors_match_host():
    import torch
    N, E, M = 150, 4.0, 3
    g, o, rng, _ = pair("pbc", N=N)
    smc = np.array([3, 1], np.int64)
    sites = rng.randint(0, 2, size=(N, 1)).astype(np.int64)
    masks = rng.randint(0, 2, size=(N, M)).astype(np.int64)
    ppos = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(N, 3 * M))
    dh = np.zeros((N, M))
    g.propose_with_dats(smc, sites, ppos, masks, dh)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    dd = t(np.zeros((N, M)))
    g.propose_with_dats(t(smc), t(sites), t(ppos), t(masks), dd)
    assert np.array_equal(dd.cpu().numpy(), dh)
    g.free()


def test_prop_charges():
    N, E, M = 100, 4.0, 2
    g, o, rng, _ = pair("27", N=N)
    smc = np.array([2], np.int64)
    sites = np.zeros((N, 1), np.int64)
    masks = np.ones((N, M), np.int64)
    ppos = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(N, 3 * M))
    pq = rng.uniform(-1, 1, size=(N, M))
    dg, do = np.zeros((N, M)), np.zeros((N, M))
    g.propose_with_dats(smc, sites, ppos, masks, dg, prop_charges=pq)
    o.propose_with_dats(smc, sites, ppos, masks, do, prop_charges=pq)
    assert np.max(rel_err(dg, do)) < TOL
    g.free()


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
def test_accept_chain(bc):
    """20 accepts: energy, expansions, multipole, positions, cells, occupancy match the oracle."""
    N, E = 200, 4.0
    g, o, rng, st = pair(bc, N=N)
    for step in range(20):
        pid = rng.randint(0, N - 1)
        mv = rng.uniform(low=-0.5 * E, high=0.5 * E, size=3)
        g.accept((pid, mv))
        o.accept((pid, mv))
        assert rel_err(g.energy, o.energy) < TOL
    assert np.array_equal(st.P.data, o.positions)
    assert_state_equal(g, o)
    g.free()


def test_store_growth_and_edges():
    """Drive many charges into one cell (store capacity growth), moves onto cell
    boundaries and onto the box faces."""
    N, E = 64, 4.0
    g, o, rng, _ = pair("pbc", N=N, R=3)
    cw = E / 4
    targets = [np.array([0.1 + 0.01 * i, 0.2, -0.3]) for i in range(40)]
    targets += [np.array([-2.0, 0.0, cw]), np.array([2.0, 2.0, -2.0]), np.array([0.0, -cw, 1.0])]
    for i, t in enumerate(targets):
        g.accept((i, t))
        o.accept((i, t))
    assert g.state()["capacity"] >= 41
    assert_state_equal(g, o)
    g.free()


def test_empty_and_bad_proposals():
    N, E, M = 50, 4.0, 3
    g, o, rng, _ = pair("free_space", N=N, max_move=0.5)
    smc = np.array([3], np.int64)
    sites = np.zeros((N, 1), np.int64)
    d = np.full((N, M), 5.0)
    g.propose_with_dats(smc, sites, np.zeros((N, 3 * M)), np.zeros((N, M), np.int64), d)
    assert np.all(d == 5.0)
    pos = g.state()["positions"]
    bad = np.tile(pos, (1, M))
    bad[3, 0] += 0.75  # beyond max_move
    masks = np.zeros((N, M), np.int64)
    masks[3, 0] = 1
    with pytest.raises(RuntimeError):
        g.propose_with_dats(smc, sites, bad, masks, d)
    with pytest.raises(RuntimeError):
        g.propose(((0, pos[0] + np.array([0.0, 0.0, 0.6])),))
    with pytest.raises(RuntimeError):
        g.accept((0, np.array([2.1, 0.0, 0.0])))
    # still usable after the errors
    g.accept((1, pos[1] + 0.1))
    o.accept((1, pos[1] + 0.1))
    assert rel_err(g.energy, o.energy) < TOL
    g.free()


def test_uninitialised_raises():
    st = make_state(np.zeros((4, 3)), np.zeros(4), 4.0)
    g = KMCFMM(st.P, st.Q, st.domain, r=2, l=4, boundary_condition="free_space")
    with pytest.raises(RuntimeError):
        g.propose(((0, np.zeros(3)),))
    g.free()


def test_lattice_hopping_chain():
    """Rejection-free lattice-hop KMC on a small pbc lattice: the GPU and the
    oracle pick the same moves for the same random stream (same occupancy)."""
    from coulomb_kmc_gb300.workloads import LatticeHopSystem
    sysg = LatticeHopSystem(side=12, occupancy=0.25, seed=5)
    syso = LatticeHopSystem(side=12, occupancy=0.25, seed=5)
    E, R, L = sysg.extent, 3, 12
    st = make_state(sysg.positions(), sysg.charges(), E)
    g = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition="pbc", max_move=1.0)
    g.initialise()
    o = ko.OracleKMC(syso.positions(), syso.charges(), E, R, L, "pbc", max_move=1.0,
                     lr_operator=lattice_operator(L, E))
    o.initialise()
    rg, ro = np.random.default_rng(11), np.random.default_rng(11)
    for step in range(12):
        mg = sysg.step(g, rg, beta=2.0)
        mo = syso.step(o, ro, beta=2.0)
        assert mg == mo
    assert_state_equal(g, o)
    g.free()


def test_propose_with_dats_host_buffers_in_place():
    """The library's pinned host arrays, filled in place, give the same differences as
    ordinary numpy arrays (the copies through the staging buffers are skipped)."""
    N, E, M = 150, 4.0, 3
    g, o, rng, _ = pair("pbc", N=N)
    smc = np.array([M], np.int64)
    ppos = rng.uniform(-0.5 * E, 0.5 * E, (N, 3 * M))
    masks = (rng.uniform(size=(N, M)) < 0.7).astype(np.int64)
    ref = np.zeros((N, M))
    g.propose_with_dats(smc, np.zeros((N, 1), np.int64), ppos, masks, ref)
    hb = g.host_buffers(M)
    hb["prop_positions"][:] = ppos
    hb["prop_masks"][:] = masks
    hb["current_sites"][:] = 0
    hb["prop_energy_diffs"][:] = 0.0
    g.propose_with_dats(smc, hb["current_sites"], hb["prop_positions"], hb["prop_masks"], hb["prop_energy_diffs"])
    assert np.array_equal(hb["prop_energy_diffs"], ref)
    g.free()
