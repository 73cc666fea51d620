"""Mixed-precision propose path against the plain FP64 GPU path (same state):
energy differences within 1e-6 relative (denominator max(|dE|,1)); the total
energy and all expansions stay identical to the FP64 path through accepts."""
import numpy as np
import pytest
import torch

from conftest import neutral_charges, rel_err
from coulomb_kmc_gb300 import KMCFMM
from coulomb_kmc_gb300.dats import make_state
from coulomb_kmc_gb300.workloads import LatticeHopSystem

pytestmark = pytest.mark.gpu
MIXED_TOL = 1e-6


def both(P, Q, E, bc, R, L, max_move=None, mixed="mixed"):
    out = []
    for prec in ("fp64", mixed):
        st = make_state(P, Q, E)
        k = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition=bc, max_move=max_move, precision=prec)
        k.initialise()
        out.append((k, st))
    return out


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
@pytest.mark.parametrize("L", [8, 12])
def test_mixed_offlattice(bc, L):
    N, E, M = 400, 8.0, 4
    rng = np.random.default_rng(3)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    Q = neutral_charges(N)
    (g64, _), (g32, _) = both(P, Q, E, bc, 3, L)
    smc = np.array([M], np.int64)
    sites = np.zeros((N, 1), np.int64)
    masks = rng.integers(0, 2, (N, M)).astype(np.int64)
    ppos = np.clip(np.repeat(P, M, axis=0).reshape(N, 3 * M) + rng.uniform(-0.5, 0.5, (N, 3 * M)),
                   -0.5 * E, 0.5 * E)
    d64, d32 = np.zeros((N, M)), np.zeros((N, M))
    g64.propose_with_dats(smc, sites, ppos, masks, d64)
    g32.propose_with_dats(smc, sites, ppos, masks, d32)
    act = masks > 0
    err = rel_err(d32[act], d64[act])
    assert err.max() < MIXED_TOL, err.max()
    assert np.array_equal(d32[~act], d64[~act])
    g64.free()
    g32.free()


@pytest.mark.parametrize("bc", ["free_space", "pbc"])
def test_mixed_large_box_high_order(bc):
    """Box edge 64 and L = 16: the FP32 lattice quantities stay in range (box units)."""
    N, E, M = 600, 64.0, 2
    rng = np.random.default_rng(8)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    Q = neutral_charges(N)
    (g64, _), (g32, _) = both(P, Q, E, bc, 3, 16, max_move=1.0)
    smc = np.array([M], np.int64)
    sites = np.zeros((N, 1), np.int64)
    masks = np.ones((N, M), np.int64)
    ppos = np.clip(np.repeat(P, M, axis=0).reshape(N, 3 * M) + rng.uniform(-1.0, 1.0, (N, 3 * M)),
                   -0.5 * E, 0.5 * E)
    d64, d32 = np.zeros((N, M)), np.zeros((N, M))
    g64.propose_with_dats(smc, sites, ppos, masks, d64)
    g32.propose_with_dats(smc, sites, ppos, masks, d32)
    assert np.all(np.isfinite(d32))
    assert rel_err(d32, d64).max() < MIXED_TOL
    g64.free()
    g32.free()


@pytest.mark.parametrize("mode", ["mixed", "mixed_fp64_accept"])
def test_mixed_lattice_and_accepts(mode):
    """pbc lattice hops: mixed differences within 1e-6; after accepting the same
    moves the mixed instance's energy and state match the FP64 instance's
    (bit-identical with FP64 accept contributions, 1e-12 with double-FP32 ones)."""
    hs = LatticeHopSystem(side=24, occupancy=0.25, seed=9)
    (g64, s64), (g32, s32) = both(hs.positions(), hs.charges(), hs.extent, "pbc", 4, 12, max_move=1.0,
                                  mixed=mode)
    rng = np.random.default_rng(1)
    worst = 0.0
    for step in range(6):
        ppos, masks, tsite = hs.proposals()
        smc = np.array([6], np.int64)
        sites = np.zeros((hs.n, 1), np.int64)
        d64, d32 = np.zeros((hs.n, 6)), np.zeros((hs.n, 6))
        g64.propose_with_dats(smc, sites, ppos, masks, d64)
        g32.propose_with_dats(smc, sites, ppos, masks, d32)
        act = masks > 0
        worst = max(worst, rel_err(d32[act], d64[act]).max())
        pid, h = hs.select(d64, masks, rng, 2.0)
        mv = ppos[pid, 3 * h:3 * h + 3].copy()
        g64.accept((pid, mv))
        g32.accept((pid, mv))
        hs.occ[hs.site_of[pid]] = -1
        hs.occ[tsite[pid, h]] = pid
        hs.site_of[pid] = tsite[pid, h]
    assert worst < MIXED_TOL, worst
    a, b = g32.state(), g64.state()
    assert np.array_equal(a["occupancy"], b["occupancy"])
    if mode == "mixed_fp64_accept":
        assert g32.energy == g64.energy
        assert np.array_equal(a["local_expansions"], b["local_expansions"])
    else:
        la, lb = a["local_expansions"], b["local_expansions"]
        assert np.max(np.abs(la - lb)) < 1e-12 * np.max(np.abs(lb))
        assert rel_err(g32.energy, g64.energy) < 1e-12
    g64.free()
    g32.free()


def test_mixed_device_accept_energy_is_fp64():
    """accept_device in mixed mode advances the energy by the FP64 difference."""
    hs = LatticeHopSystem(side=16, occupancy=0.25, seed=4)
    (g64, _), (g32, _) = both(hs.positions(), hs.charges(), hs.extent, "pbc", 3, 10, max_move=1.0)
    ppos, masks, _ = hs.proposals()
    pid = int(np.nonzero(masks.sum(axis=1))[0][0])
    h = int(np.nonzero(masks[pid])[0][0])
    mv = ppos[pid, 3 * h:3 * h + 3].copy()
    d = torch.zeros(1, dtype=torch.float64, device="cuda")  # deliberately wrong dE: ignored in mixed mode
    g32.accept_device(torch.tensor([pid], device="cuda"), torch.from_numpy(mv).cuda(), d)
    g64.accept((pid, mv))
    assert rel_err(g32.energy, g64.energy) < 1e-12
    g64.free()
    g32.free()


@pytest.mark.parametrize("fused", [0, 1])
@pytest.mark.parametrize("groups", [1, 2, 3])
@pytest.mark.parametrize("fp32_from", [0, 4, 99])
@pytest.mark.parametrize("pair", [0, 1])
def test_mixed_kernel_variants(fused, groups, fp32_from, pair):
    """Launch-shape and precision variants (fused or split lattice kernels, source
    groups of the double-FP32 accept, first accept order in FP32: default, 4, none;
    the column-pair or per-column accept kernel at the default split) give the same
    differences within the mixed tolerance and the same state within 1e-12 after
    accepts."""
    from coulomb_kmc_gb300 import _native
    hs = LatticeHopSystem(side=16, occupancy=0.25, seed=5)
    (g64, _), (g32, _) = both(hs.positions(), hs.charges(), hs.extent, "pbc", 3, 12, max_move=1.0)
    lib = _native.lib()
    assert lib.kmc_set_tuning(g32._handle, 1, fused) == 0
    assert lib.kmc_set_tuning(g32._handle, 0, groups) == 0
    assert lib.kmc_set_tuning(g32._handle, 6, fp32_from) == 0
    assert lib.kmc_set_tuning(g32._handle, 9, pair) == 0
    rng = np.random.default_rng(3)
    for _ in range(3):
        ppos, masks, tsite = hs.proposals()
        smc = np.array([6], np.int64)
        sites = np.zeros((hs.n, 1), np.int64)
        d64, d32 = np.zeros((hs.n, 6)), np.zeros((hs.n, 6))
        g64.propose_with_dats(smc, sites, ppos, masks, d64)
        g32.propose_with_dats(smc, sites, ppos, masks, d32)
        act = masks > 0
        assert rel_err(d32[act], d64[act]).max() < MIXED_TOL
        pid, h = hs.select(d64, masks, rng, 2.0)
        mv = ppos[pid, 3 * h:3 * h + 3].copy()
        g64.accept((pid, mv))
        g32.accept((pid, mv))
        hs.occ[hs.site_of[pid]] = -1
        hs.occ[tsite[pid, h]] = pid
        hs.site_of[pid] = tsite[pid, h]
    # FP32 accept orders from l = 4 (not the default) reach the nearest
    # well-separated cells of this 4^3-cell box with ~1e-7 relative increments
    tol = 1e-10 if fp32_from == 4 else 1e-12
    la, lb = g32.state()["local_expansions"], g64.state()["local_expansions"]
    assert np.max(np.abs(la - lb)) < tol * np.max(np.abs(lb))
    assert rel_err(g32.energy, g64.energy) < tol
    g64.free()
    g32.free()


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
@pytest.mark.parametrize("R", [2, 3])
def test_mixed_near_packed_and_scalar(bc, R):
    """The near field summed two neighbours per packed FP32 instruction (default)
    and one at a time give the same differences to double-FP32 rounding, and both
    stay within the mixed tolerance of FP64.  Off-lattice charges give odd
    neighbour counts (a padded pair) and, at R = 2 with periodic images, cells
    that appear more than once in a neighbourhood."""
    from coulomb_kmc_gb300 import _native
    N, E, M = 300, 8.0, 3
    rng = np.random.default_rng(11 + R)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    Q = neutral_charges(N)
    (g64, _), (g32, _) = both(P, Q, E, bc, R, 10)
    smc = np.array([M], np.int64)
    sites = np.zeros((N, 1), np.int64)
    masks = rng.integers(0, 2, (N, M)).astype(np.int64)
    ppos = np.clip(np.repeat(P, M, axis=0).reshape(N, 3 * M) + rng.uniform(-0.5, 0.5, (N, 3 * M)),
                   -0.5 * E, 0.5 * E)
    lib = _native.lib()
    d64, dp, ds = np.zeros((N, M)), np.zeros((N, M)), np.zeros((N, M))
    g64.propose_with_dats(smc, sites, ppos, masks, d64)
    assert lib.kmc_set_tuning(g32._handle, 3, 0) == 0
    g32.propose_with_dats(smc, sites, ppos, masks, dp)
    assert lib.kmc_set_tuning(g32._handle, 3, 1) == 0
    g32.propose_with_dats(smc, sites, ppos, masks, ds)
    assert lib.kmc_set_tuning(g32._handle, 3, 2) != 0
    assert lib.kmc_set_tuning(g32._handle, 4, 1) == 0
    dc = np.zeros((N, M))
    g32.propose_with_dats(smc, sites, ppos, masks, dc)
    assert rel_err(dc[masks > 0], ds[masks > 0]).max() < 1e-11
    act = masks > 0
    assert rel_err(dp[act], ds[act]).max() < 1e-11
    assert rel_err(dp[act], d64[act]).max() < MIXED_TOL
    assert rel_err(ds[act], d64[act]).max() < MIXED_TOL
    g64.free()
    g32.free()


def test_mixed_lattice_cache_through_accepts():
    """The per-charge far-lattice cache (h = A b kept between moves, the accepted
    charge's entry refreshed by the accept) gives the same differences as
    recomputing h every propose (to FP32 rounding of b.g), through device-side
    accepts, and both stay within the mixed tolerance of FP64."""
    from coulomb_kmc_gb300 import _native
    hs = LatticeHopSystem(side=16, occupancy=0.25, seed=9)
    (g64, _), (g32, _) = both(hs.positions(), hs.charges(), hs.extent, "pbc", 3, 12, max_move=1.0)
    lib = _native.lib()
    rng = np.random.default_rng(4)
    for _ in range(4):
        ppos, masks, tsite = hs.proposals()
        smc = np.array([6], np.int64)
        sites = np.zeros((hs.n, 1), np.int64)
        d64, dc, dn = np.zeros((hs.n, 6)), np.zeros((hs.n, 6)), np.zeros((hs.n, 6))
        g64.propose_with_dats(smc, sites, ppos, masks, d64)
        assert lib.kmc_set_tuning(g32._handle, 5, 0) == 0
        g32.propose_with_dats(smc, sites, ppos, masks, dc)
        assert lib.kmc_set_tuning(g32._handle, 5, 1) == 0
        g32.propose_with_dats(smc, sites, ppos, masks, dn)
        assert lib.kmc_set_tuning(g32._handle, 5, 0) == 0
        act = masks > 0
        # the two kernels sum the FP32 part of b.g (l >= 3) in different orders
        assert rel_err(dc[act], dn[act]).max() < 1e-7
        assert rel_err(dc[act], d64[act]).max() < MIXED_TOL
        pid, h = hs.select(d64, masks, rng, 2.0)
        mv = ppos[pid, 3 * h:3 * h + 3].copy()
        g64.accept((pid, mv))
        g32.accept_device(torch.tensor([pid], device="cuda"), torch.from_numpy(mv).cuda(),
                          torch.zeros(1, dtype=torch.float64, device="cuda"))
        hs.occ[hs.site_of[pid]] = -1
        hs.occ[tsite[pid, h]] = pid
        hs.site_of[pid] = tsite[pid, h]
    g64.free()
    g32.free()


@pytest.mark.parametrize("side,cached", [(16, 0), (16, 1), (10, 0)])
def test_mixed_self_term_evaluators(side, cached):
    """The unrolled L = 12 cubic-lattice evaluator of the far-lattice self term F(x)
    and the general program interpreter agree to FP32 rounding (a different
    evaluation order, so not bit-identical), with and without the per-charge
    lattice cache, and both stay within the mixed tolerance of FP64."""
    from coulomb_kmc_gb300 import _native
    hs = LatticeHopSystem(side=side, occupancy=0.25, seed=5)
    (g64, _), (g32, _) = both(hs.positions(), hs.charges(), hs.extent, "pbc", 3, 12, max_move=1.0)
    lib = _native.lib()
    assert lib.kmc_set_tuning(g32._handle, 5, 1 - cached) == 0
    ppos, masks, _ = hs.proposals()
    smc = np.array([6], np.int64)
    sites = np.zeros((hs.n, 1), np.int64)
    d64, dc, dg = np.zeros((hs.n, 6)), np.zeros((hs.n, 6)), np.zeros((hs.n, 6))
    g64.propose_with_dats(smc, sites, ppos, masks, d64)
    g32.propose_with_dats(smc, sites, ppos, masks, dc)
    assert lib.kmc_set_tuning(g32._handle, 8, 1) == 0
    g32.propose_with_dats(smc, sites, ppos, masks, dg)
    assert lib.kmc_set_tuning(g32._handle, 8, 2) != 0
    act = masks > 0
    assert not np.array_equal(dc[act], dg[act])
    assert rel_err(dc[act], dg[act]).max() < 1e-7
    assert rel_err(dc[act], d64[act]).max() < MIXED_TOL
    assert rel_err(dg[act], d64[act]).max() < MIXED_TOL
    g64.free()
    g32.free()


@pytest.mark.parametrize("bc", ["free_space", "pbc"])
def test_mixed_shared_targets(bc):
    """Many proposals to the same positions (the near field and cell expansion are
    computed once per distinct position in a cell, the self term per proposal):
    within the mixed tolerance of FP64, and a charge's two proposals to one
    position give identical differences."""
    N, E, M = 300, 8.0, 4
    rng = np.random.default_rng(21)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    Q = neutral_charges(N)
    (g64, _), (g32, _) = both(P, Q, E, bc, 3, 12)
    pool = rng.uniform(-0.5 * E, 0.5 * E, (40, 3))
    pick = rng.integers(0, len(pool), (N, M))
    pick[:, 1] = pick[:, 0]  # a duplicate within each charge's own moves
    ppos = pool[pick].reshape(N, 3 * M)
    masks = np.ones((N, M), np.int64)
    smc = np.array([M], np.int64)
    sites = np.zeros((N, 1), np.int64)
    d64, d32 = np.zeros((N, M)), np.zeros((N, M))
    g64.propose_with_dats(smc, sites, ppos, masks, d64)
    g32.propose_with_dats(smc, sites, ppos, masks, d32)
    assert rel_err(d32, d64).max() < MIXED_TOL
    assert np.array_equal(d32[:, 0], d32[:, 1])
    g64.free()
    g32.free()
