"""Ewald sum for cubic periodic boxes with tin-foil boundary conditions
(TEST INFRASTRUCTURE ONLY).

The reference pins its periodic energies against ppmd's ``EwaldOrthoganalHalf``
(tests/host/test_common.py:106-182, tests/host/test_propose_dat_setup.py:583-615),
which is not available.  This is an independent restatement of the standard
Ewald decomposition:

    U = 1/2 sum_{i,j,n}' q_i q_j erfc(a r)/r
      + (2 pi / V) sum_{k != 0} exp(-k^2/4a^2)/k^2 |S(k)|^2
      - a/sqrt(pi) sum_i q_i^2

for a neutral system.  Parameters are chosen generously so that the result is
converged well below the 1e-7 level used by the tests.
"""
import numpy as np
from scipy.special import erfc


def ewald_energy(positions, charges, E, alpha_e=3.2, nreal=3, nrecip=10):
    P = np.asarray(positions, dtype=np.float64)
    Q = np.ravel(np.asarray(charges, dtype=np.float64))
    E = float(E)
    V = E ** 3
    a = alpha_e / E
    g = np.arange(-nreal, nreal + 1)
    shifts = np.array([(x, y, z) for x in g for y in g for z in g], dtype=np.float64) * E
    d = P[None, :, :] - P[:, None, :]  # d[i,j] = P_j - P_i
    er = 0.0
    for s in shifts:
        r = np.linalg.norm(d + s[None, None, :], axis=2)
        if not s.any():
            np.fill_diagonal(r, np.inf)
        er += 0.5 * np.sum(Q[:, None] * Q[None, :] * erfc(a * r) / r)
    h = np.arange(-nrecip, nrecip + 1)
    ks = np.array([(x, y, z) for x in h for y in h for z in h if (x, y, z) != (0, 0, 0)], dtype=np.float64)
    ks *= 2 * np.pi / E
    k2 = np.sum(ks * ks, axis=1)
    Sk = np.exp(1j * (P @ ks.T)).T @ Q
    ek = 2 * np.pi / V * np.sum(np.exp(-k2 / (4 * a * a)) / k2 * np.abs(Sk) ** 2)
    es = -a / np.sqrt(np.pi) * np.sum(Q * Q)
    return er + ek + es
