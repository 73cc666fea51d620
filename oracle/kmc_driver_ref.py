"""Host restatement of the device-side KMC driver's bookkeeping -- TEST
INFRASTRUCTURE ONLY (used by tests/ to check the GPU driver draw for draw).

The bookkeeping follows the reference's example driver
(examples/propose_with_dats_example.py:218-330: proposals at fixed hop
offsets, occupied targets masked, per-proposal rates and a cumulative-sum
pick) and the Metropolis loop of its tests (tests/host/test_free_space_1.py),
with the selection rules the GPU driver uses:

* lattice: hops +x, -x, +y, -y, +z, -z to the six nearest sites (wrapped when
  periodic, masked when a free-space lattice would be left), rate
  exp(-beta dE / 2) on unmasked proposals, pick the first proposal whose
  running sum exceeds u * total;
* off-lattice: displacement (2u - 1) * step per axis, re-drawn (at most 32
  times) while it leaves the box; one charge chosen as floor(u1 * N),
  accepted when dE <= 0 or u2 < exp(-beta dE).

Random numbers: Philox4x32-10 (Salmon, Moraes, Dror and Shaw, SC11) with key
(seed low, seed high) and counter (step low, step high, index,
attempt << 4 | tag), 53-bit uniforms from two words.
"""
import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK32 = np.uint64(0xFFFFFFFF)
TAG_DISP_XY, TAG_DISP_Z, TAG_SELECT = 1, 2, 3
MAX_ATTEMPTS = 32
HOPS = [(0, 1), (0, -1), (1, 1), (1, -1), (2, 1), (2, -1)]


def philox(c0, c1, c2, c3, seed):
    """Philox4x32-10 on arrays of counter words (broadcast); returns four uint64 arrays of 32-bit words."""
    c = [np.asarray(x, dtype=np.uint64) & MASK32 for x in (c0, c1, c2, c3)]
    c = list(np.broadcast_arrays(*c))
    c = [x.copy() for x in c]
    k0, k1 = seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF
    for _ in range(10):
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        n0 = (p1 >> np.uint64(32)) ^ c[1] ^ np.uint64(k0)
        n2 = (p0 >> np.uint64(32)) ^ c[3] ^ np.uint64(k1)
        c = [n0 & MASK32, p1 & MASK32, n2 & MASK32, p0 & MASK32]
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return c


def u53(a, b):
    return ((a >> np.uint64(5)).astype(np.float64) * 67108864.0 + (b >> np.uint64(6)).astype(np.float64)) * (
        1.0 / 9007199254740992.0)


def draw(seed, step, index, word3):
    return philox(step & 0xFFFFFFFF, (step >> 32) & 0xFFFFFFFF, index, word3, seed)


class LatticeRef:
    """Lattice hopping on the host with the GPU driver's draws."""

    def __init__(self, side, extent, sites, periodic, beta, seed):
        self.side, self.extent = int(side), float(extent)
        self.spacing = self.extent / self.side
        self.site_of = np.asarray(sites, dtype=np.int64).copy()
        self.occ = np.full(self.side ** 3, -1, np.int64)
        self.occ[self.site_of] = np.arange(len(self.site_of))
        self.periodic, self.beta, self.seed = periodic, float(beta), int(seed)
        self.step_no = 0

    def site_pos(self, s):
        k = self.side
        xyz = np.stack([s % k, (s // k) % k, s // (k * k)], axis=-1).astype(np.float64)
        return (xyz * self.spacing - 0.5 * self.extent) + 0.5 * self.spacing

    def proposals(self):
        k, n = self.side, len(self.site_of)
        s = self.site_of
        xyz = np.stack([s % k, (s // k) % k, s // (k * k)], axis=-1)
        tsite = np.zeros((n, 6), np.int64)
        masks = np.zeros((n, 6), np.int64)
        for h, (ax, d) in enumerate(HOPS):
            t = xyz.copy()
            t[:, ax] += d
            out = (t[:, ax] < 0) | (t[:, ax] >= k)
            if self.periodic:
                t[:, ax] %= k
                ok = np.ones(n, bool)
            else:
                ok = ~out
            ts = np.where(ok, t[:, 0] + k * (t[:, 1] + k * t[:, 2]), s)
            tsite[:, h] = ts
            masks[:, h] = (ok & (self.occ[ts] < 0)).astype(np.int64)
        ppos = self.site_pos(tsite).reshape(n, 18)
        return ppos, masks, tsite

    def select(self, diffs, masks):
        rates = np.where(masks.ravel() > 0, np.exp(-0.5 * self.beta * diffs.ravel()), 0.0)
        c = np.cumsum(rates)
        r = draw(self.seed, self.step_no, 0, TAG_SELECT)
        target = u53(r[0], r[1]) * c[-1]
        idx = int(np.searchsorted(c, target, side="right"))
        idx = min(idx, len(c) - 1)
        while rates[idx] == 0.0:
            idx -= 1
        return idx

    def commit(self, idx, tsite):
        pid, h = idx // 6, idx % 6
        ns = int(tsite[pid, h])
        self.occ[self.site_of[pid]] = -1
        self.occ[ns] = pid
        self.site_of[pid] = ns
        self.step_no += 1
        return pid, ns


class OffLatticeRef:
    """Off-lattice Metropolis on the host with the GPU driver's draws."""

    def __init__(self, positions, extent, step, beta, seed):
        self.pos = np.asarray(positions, dtype=np.float64).copy()
        self.extent, self.step, self.beta, self.seed = float(extent), float(step), float(beta), int(seed)
        self.step_no = 0

    def proposals(self):
        n = len(self.pos)
        h = 0.5 * self.extent
        idx = np.arange(n)
        out = self.pos.copy()
        todo = np.ones(n, bool)
        for a in range(MAX_ATTEMPTS):
            A = draw(self.seed, self.step_no, idx, (a << 4) | TAG_DISP_XY)
            B = draw(self.seed, self.step_no, idx, (a << 4) | TAG_DISP_Z)
            t = np.stack([self.pos[:, 0] + (2.0 * u53(A[0], A[1]) - 1.0) * self.step,
                          self.pos[:, 1] + (2.0 * u53(A[2], A[3]) - 1.0) * self.step,
                          self.pos[:, 2] + (2.0 * u53(B[0], B[1]) - 1.0) * self.step], axis=1)
            ok = todo & np.all(np.abs(t) <= h, axis=1)
            out[ok] = t[ok]
            todo &= ~ok
            if not todo.any():
                break
        return out

    def select(self, diffs):
        n = len(self.pos)
        r = draw(self.seed, self.step_no, 0, TAG_SELECT)
        i = min(int(u53(r[0], r[1]) * n), n - 1)
        de = float(diffs[i])
        acc = de <= 0.0 or float(u53(r[2], r[3])) < np.exp(-self.beta * de)
        return i, acc

    def commit(self, i, acc, prop):
        if acc:
            self.pos[i] = prop[i]
        self.step_no += 1
