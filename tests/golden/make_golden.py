"""Generate the golden fixtures under tests/golden/ (run once; outputs are committed).

The reference's own tests store no expected values: each test draws its
inputs from numpy's legacy ``RandomState`` with a fixed seed and compares
KMCFMM against a direct Coulomb sum computed in the same run.  These fixtures
replay exactly those input streams and store the direct-sum answers, computed
here with plain numpy (independent of the C oracle and of the GPU library):

* free_space_1   tests/host/test_free_space_1.py:143-232  (seed 1234, N=50, E=4, 2N moves)
* nearest27_1    tests/host/test_nearest_27_1.py:32-133   (seed 1234, N=50, E=4, N moves)
* free_space_2   tests/host/test_free_space_1.py:235-336  (seed 8657, 1-7 moves per charge)
* pbc_1          tests/host/test_pbc_1.py:247-367         (seed 1234, N=50, E=4, 3 moves per step)

The periodic oracle (ppmd's Ewald / full-pbc FMM) is not available; pbc_1
stores energies from oracle/ewald.py (tin-foil Ewald, converged to ~1e-15).

Usage:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle.ewald import ewald_energy  # noqa: E402


def direct_free(P, Q):
    """FreeSpaceDirect (tests/host/test_common.py:24-55): sum_{i<j} q_i q_j / r_ij."""
    d = P[:, None, :] - P[None, :, :]
    r = np.sqrt(np.sum(d * d, axis=2))
    iu = np.triu_indices(len(Q), 1)
    return float(np.sum((Q[:, None] * Q[None, :])[iu] / r[iu]))


def direct_27(P, Q, E):
    """NearestDirect (tests/host/test_common.py:61-103)."""
    e = direct_free(P, Q)
    for a in (-1, 0, 1):
        for b in (-1, 0, 1):
            for c in (-1, 0, 1):
                if a == b == c == 0:
                    continue
                d = P[None, :, :] - P[:, None, :] + E * np.array([a, b, c])
                r = np.sqrt(np.sum(d * d, axis=2))
                e += 0.5 * float(np.sum(Q[:, None] * Q[None, :] / r))
    return e


def charges(N):
    Q = np.array([(-1.0) ** (px + 1) for px in range(N)])
    return Q - np.sum(Q) / N


def single_moves(seed, N, E, nmoves, energy):
    rng = np.random.RandomState(seed=seed)
    P = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(N, 3))
    Q = charges(N)
    pids, pos, ens = [], [], []
    for _ in range(nmoves):
        pid = rng.randint(0, N - 1)
        p = rng.uniform(low=-0.5 * E, high=0.5 * E, size=3)
        PP = P.copy()
        PP[pid] = p
        pids.append(pid)
        pos.append(p)
        ens.append(energy(PP, Q))
    return dict(P=P, Q=Q, E=E, pids=np.array(pids), moves=np.array(pos), energies=np.array(ens),
                e0=energy(P, Q))


def multi_moves(seed, N, E):
    rng = np.random.RandomState(seed=seed)
    P = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(N, 3))
    Q = charges(N)
    order = rng.permutation(range(N))
    pids, counts, moves, ens = [], [], [], []
    for px in range(N):
        k = rng.randint(1, 8)
        mv = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(k, 3))
        pids.append(order[px])
        counts.append(k)
        for m in mv:
            PP = P.copy()
            PP[order[px]] = m
            moves.append(m)
            ens.append(direct_free(PP, Q))
    return dict(P=P, Q=Q, E=E, pids=np.array(pids), counts=np.array(counts), moves=np.array(moves),
                energies=np.array(ens), e0=direct_free(P, Q))


def pbc_moves(seed, N, E, steps, M):
    rng = np.random.RandomState(seed=seed)
    P = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(N, 3))
    Q = charges(N)
    pids, moves, ens = [], [], []
    for _ in range(steps):
        pid = rng.randint(0, N - 1)
        pos = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(M, 3))
        for m in pos:
            PP = P.copy()
            PP[pid] = m
            pids.append(pid)
            moves.append(m)
            ens.append(ewald_energy(PP, Q, E))
    return dict(P=P, Q=Q, E=E, pids=np.array(pids), moves=np.array(moves), energies=np.array(ens),
                e0=ewald_energy(P, Q, E))


def main():
    E = 4.0
    cases = {
        "free_space_1": single_moves(1234, 50, E, 100, direct_free),
        "nearest27_1": single_moves(1234, 50, E, 50, lambda P, Q: direct_27(P, Q, E)),
        "free_space_2": multi_moves(8657, 50, E),
        "pbc_1": pbc_moves(1234, 50, E, 8, 3),
    }
    for name, d in cases.items():
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **d)
        print(name, {k: np.shape(v) for k, v in d.items()})


if __name__ == "__main__":
    main()
