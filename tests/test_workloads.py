"""Host-side lattice workload: the proposals step() keeps current across its own
accepts equal a fresh build, including after the occupancy is changed by hand."""
import numpy as np

from coulomb_kmc_gb300.workloads import LatticeHopSystem


class _Stub:
    """Stands in for KMCFMM: random differences, accept is a no-op."""

    def __init__(self, seed):
        self.rng = np.random.default_rng(seed)

    def propose_with_dats(self, smc, sites, ppos, masks, diffs):
        diffs[...] = self.rng.normal(size=diffs.shape)

    def accept(self, move):
        pass


def test_step_proposals_match_fresh_build():
    for side in (2, 3, 8):
        hs = LatticeHopSystem(side, 0.25 if side > 2 else 0.5, seed=side)
        k, rng = _Stub(1), np.random.default_rng(2)
        for i in range(300):
            before = int(hs.proposals()[1].sum())
            hs.step(k, rng, 2.0)
            assert hs.last_active == before
            a, b = hs._step_proposals(), hs.proposals()
            for x, y in zip(a, b):
                assert np.array_equal(x, y)
            if i == 150:  # a move made outside step(): the kept proposals are rebuilt
                pid = 0
                free = np.nonzero(hs.occ < 0)[0][0]
                hs.occ[hs.site_of[pid]] = -1
                hs.occ[free] = pid
                hs.site_of[pid] = free


def test_select_matches_dense_rates():
    hs = LatticeHopSystem(8, 0.25, seed=3)
    ppos, masks, _ = hs.proposals()
    d = np.random.default_rng(4).normal(size=masks.shape)
    for s in range(20):
        r1, r2 = np.random.default_rng(s), np.random.default_rng(s)
        rates = np.where(masks > 0, np.exp(-0.5 * 2.0 * d), 0.0).ravel()
        c = np.cumsum(rates)
        idx = min(int(np.searchsorted(c, r1.uniform(0.0, c[-1]), side="right")), len(c) - 1)
        while rates[idx] == 0.0:
            idx -= 1
        assert hs.select(d, masks, r2, 2.0) == (idx // 6, idx % 6)
