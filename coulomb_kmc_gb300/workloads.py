"""KMC drivers around the KMCFMM interface (host-side bookkeeping).

These follow the reference's example driver (examples/propose_with_dats_example.py:
218-446): build proposals, mask occupied targets, call ``propose_with_dats``,
turn energy differences into rates, select one move and ``accept`` it.  They
work with any object exposing that interface (the GPU ``KMCFMM`` or the CPU
oracle), which is how the tests check that both choose the same moves.
"""
import numpy as np

HOPS = np.array([(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)], dtype=np.int64)


class LatticeHopSystem:
    """Simple-cubic lattice of side^3 sites (spacing 1), a fraction occupied by
    +-1 charges in equal numbers; every charge proposes a hop to each vacant
    nearest-neighbour site (periodic wrap); rejection-free selection with rate
    exp(-beta dE / 2)."""

    def __init__(self, side, occupancy=0.25, seed=1):
        self.side = int(side)
        self.extent = float(side)
        rng = np.random.default_rng(seed)
        nsites = self.side ** 3
        n = int(round(occupancy * nsites))
        n -= n % 2
        self.n = n
        self.site_of = rng.choice(nsites, size=n, replace=False).astype(np.int64)
        q = np.ones(n)
        q[: n // 2] = -1.0
        rng.shuffle(q)
        self.q = q
        self.occ = np.full(nsites, -1, dtype=np.int64)
        self.occ[self.site_of] = np.arange(n)
        self.M = 6
        # per site: the six neighbour sites in HOPS order (periodic) and every site's centre
        xyz = self.site_xyz(np.arange(nsites))
        tgt = (xyz[:, None, :] + HOPS[None, :, :]) % self.side
        self._nb = tgt[..., 0] + self.side * (tgt[..., 1] + self.side * tgt[..., 2])
        self._centre = xyz.astype(np.float64) - 0.5 * self.extent + 0.5
        self.last_active = 0
        self._cache = None  # step(): [ppos, masks, tsite, site_of copy], updated per accepted hop

    def site_xyz(self, s):
        s = np.asarray(s, dtype=np.int64)
        k = self.side
        return np.stack([s % k, (s // k) % k, s // (k * k)], axis=-1)

    def site_pos(self, s):
        # site centres are offset by half a spacing so no charge sits on a cell face
        return self.site_xyz(s).astype(np.float64) - 0.5 * self.extent + 0.5

    def positions(self):
        return self.site_pos(self.site_of)

    def charges(self):
        return self.q.copy()

    def proposals(self):
        """(prop_positions [n, 18], prop_masks [n, 6], target sites [n, 6])."""
        tsite = self._nb[self.site_of]
        masks = (self.occ[tsite] < 0).astype(np.int64)
        ppos = self._centre[tsite].reshape(self.n, 3 * self.M)
        return ppos, masks, tsite

    def _step_proposals(self):
        """proposals() kept current across step()'s own accepts (one hop changes one
        charge's targets and the masks of the two sites' neighbours); rebuilt when
        anything else changed the occupancy."""
        c = self._cache
        if c is None or not np.array_equal(c[3], self.site_of):
            ppos, masks, tsite = self.proposals()
            self._cache = c = [ppos, masks, tsite, self.site_of.copy()]
        return c[0], c[1], c[2]

    def _commit(self, pid, old, new):
        self.occ[old] = -1
        self.occ[new] = pid
        self.site_of[pid] = new
        c = self._cache
        if c is None:
            return
        ppos, masks, tsite, sites = c
        for h in range(self.M):  # hop h ^ 1 of the charge at nb[s][h] leads back to s
            j = self.occ[self._nb[old, h]]
            if j >= 0:
                masks[j, h ^ 1] = 1
            j = self.occ[self._nb[new, h]]
            if j >= 0:
                masks[j, h ^ 1] = 0
        t = self._nb[new]
        tsite[pid] = t
        masks[pid] = self.occ[t] < 0
        ppos[pid] = self._centre[t].reshape(-1)
        sites[pid] = new

    def select(self, diffs, masks, rng, beta):
        rates = np.zeros(masks.size)
        np.exp(-0.5 * beta * diffs.ravel(), out=rates, where=masks.ravel() > 0)
        c = np.cumsum(rates)
        u = rng.uniform(0.0, c[-1])
        idx = int(np.searchsorted(c, u, side="right"))
        idx = min(idx, len(c) - 1)
        while rates[idx] == 0.0:
            idx -= 1
        return idx // self.M, idx % self.M

    def step(self, kmc, rng, beta=2.0):
        ppos, masks, tsite = self._step_proposals()
        diffs = np.zeros((self.n, self.M))
        smc = np.array([self.M], dtype=np.int64)
        sites = np.zeros((self.n, 1), dtype=np.int64)
        kmc.propose_with_dats(smc, sites, ppos, masks, diffs)
        self.last_active = int(masks.sum())
        pid, h = self.select(diffs, masks, rng, beta)
        newp = ppos[pid, 3 * h:3 * h + 3].copy()
        kmc.accept((pid, newp))
        old, new = int(self.site_of[pid]), int(tsite[pid, h])
        self._commit(pid, old, new)
        return int(pid), new


class OffLatticeSystem:
    """N charges uniform in a cube, +-1 balanced; every charge proposes one move
    displaced uniformly in [-0.5, 0.5]^3 (re-drawn if it leaves the box); one
    random charge's proposal is accepted by Metropolis at inverse temperature beta."""

    def __init__(self, n, extent, seed=0, step=0.5):
        rng = np.random.default_rng(seed)
        self.n = int(n)
        self.extent = float(extent)
        self.step_size = float(step)
        self.pos = rng.uniform(-0.5 * extent, 0.5 * extent, size=(n, 3))
        q = np.ones(n)
        q[: n // 2] = -1.0
        rng.shuffle(q)
        self.q = q

    def positions(self):
        return self.pos.copy()

    def charges(self):
        return self.q.copy()

    def proposals(self, rng):
        h = 0.5 * self.extent
        prop = self.pos + rng.uniform(-self.step_size, self.step_size, size=self.pos.shape)
        bad = np.any(np.abs(prop) > h, axis=1)
        while np.any(bad):
            prop[bad] = self.pos[bad] + rng.uniform(-self.step_size, self.step_size, size=(int(bad.sum()), 3))
            bad = np.any(np.abs(prop) > h, axis=1)
        return prop

    def step(self, kmc, rng, beta=1.0):
        prop = self.proposals(rng)
        diffs = np.zeros((self.n, 1))
        kmc.propose_with_dats(np.array([1], np.int64), np.zeros((self.n, 1), np.int64), prop,
                              np.ones((self.n, 1), np.int64), diffs)
        pid = int(rng.integers(0, self.n))
        u = rng.uniform()
        if u < np.exp(-beta * diffs[pid, 0]):
            kmc.accept((pid, prop[pid].copy()))
            self.pos[pid] = prop[pid]
            return pid, True
        return pid, False


def uniform_displacements(pos, extent, step, seed, round_, out=None, threads=1):
    """One proposal per charge for the host path: pos + a uniform displacement in
    [-step, step]^3, drawn again while it leaves the box (kmc_host_displacements: the
    device driver's draws for (seed, round, index), native threads, the GIL released).
    pos: (N, 3) float64; out: an (N, 3) float64 array to write into (for instance the
    pinned array of KMCFMM.host_buffers)."""
    import ctypes
    from . import _native
    pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    if out is None:
        out = np.empty_like(pos)
    if out.shape != pos.shape or out.dtype != np.float64 or not out.flags.c_contiguous:
        raise ValueError("out must be a C-contiguous float64 array shaped like pos")
    _native.check(_native.lib().kmc_host_displacements(pos.shape[0], pos.ctypes.data, float(extent), float(step),
                                                       ctypes.c_uint64(int(seed)), int(round_), out.ctypes.data,
                                                       int(threads)), "kmc_host_displacements")
    return out
