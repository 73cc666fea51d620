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


def ewald_move_differences(positions, charges, E, pids, new_positions, alpha=None, tol=1e-13):
    """Energy change of moving charge pids[k] to new_positions[k] (one move at a
    time, the others fixed) in the periodic box with tin-foil boundary
    conditions, by Ewald summation: q_i [Phi_i(x_new) - Phi_i(x_old)], with Phi_i
    the periodic potential of every charge but i.  The interaction of the moved
    charge with its own images does not depend on its position, and neither does
    the Ewald constant, so both cancel.  This is the quantity the reference's
    periodic tests pin against ppmd's Ewald solver
    (tests/host/test_propose_dat_setup.py:583-650, tol 1e-4 on totals).

    The real-space cut-off is half the box (nearest image only), alpha is chosen
    so that the real-space tail is below ``tol`` there and the reciprocal sum
    runs over every k with exp(-k^2 / 4 alpha^2) above ``tol``; the reciprocal
    sums use separable exp(i k x) tables and BLAS products.
    """
    P = np.ascontiguousarray(positions, dtype=np.float64)
    Q = np.ravel(np.asarray(charges, dtype=np.float64))
    pids = np.asarray(pids, dtype=np.int64)
    X = np.ascontiguousarray(new_positions, dtype=np.float64).reshape(-1, 3)
    E = float(E)
    V = E ** 3
    rc = 0.5 * E
    if alpha is None:
        a = 1.0
        while erfc(a * rc) / rc > tol:
            a *= 1.05
        alpha = a
    a = float(alpha)
    kcut2 = -4 * a * a * np.log(tol)
    nmax = int(np.ceil(np.sqrt(kcut2) * E / (2 * np.pi)))
    n = np.arange(-nmax, nmax + 1)
    kk = 2 * np.pi / E * n
    # S(k) = sum_j q_j exp(i k.x_j) on the (2 nmax + 1)^3 grid
    ex = np.exp(1j * P[:, 0:1] * kk[None, :])
    ey = np.exp(1j * P[:, 1:2] * kk[None, :])
    ez = np.exp(1j * P[:, 2:3] * kk[None, :])
    S = np.empty((len(n), len(n), len(n)), dtype=np.complex128)
    for iz in range(len(n)):
        B = (Q * ez[:, iz])[:, None] * ey
        S[:, :, iz] = ex.T @ B
    KX, KY, KZ = np.meshgrid(kk, kk, kk, indexing="ij")
    K2 = KX ** 2 + KY ** 2 + KZ ** 2
    with np.errstate(divide="ignore"):
        C = np.where((K2 > 0) & (K2 <= kcut2), 4 * np.pi / V * np.exp(-K2 / (4 * a * a)) / K2, 0.0)

    def recip(pts):
        """sum_k C_k Re(exp(i k.x) conj S(k)) at every point."""
        px = np.exp(1j * pts[:, 0:1] * kk[None, :])
        py = np.exp(1j * pts[:, 1:2] * kk[None, :])
        pz = np.exp(1j * pts[:, 2:3] * kk[None, :])
        out = np.zeros(len(pts))
        for iz in range(len(n)):
            G = C[:, :, iz] * np.conj(S[:, :, iz])
            out += np.real(np.sum((px @ G) * py, axis=1) * pz[:, iz])
        return out

    def self_recip(d):
        """sum_k C_k cos(k.d) for displacement vectors d (the moved charge's own term)."""
        cx = np.exp(1j * d[:, 0:1] * kk[None, :])
        cy = np.exp(1j * d[:, 1:2] * kk[None, :])
        cz = np.exp(1j * d[:, 2:3] * kk[None, :])
        out = np.zeros(len(d))
        for iz in range(len(n)):
            out += np.real(np.sum((cx @ C[:, :, iz]) * cy, axis=1) * cz[:, iz])
        return out

    def real(pts, excl):
        """sum_{j != excl} q_j erfc(a r)/r over nearest images."""
        out = np.zeros(len(pts))
        for k0 in range(0, len(pts), 64):
            d = P[None, :, :] - pts[k0:k0 + 64, None, :]
            d -= E * np.round(d / E)
            r = np.sqrt(np.sum(d * d, axis=2))
            idx = np.arange(len(d))
            r[idx, excl[k0:k0 + 64]] = np.inf
            out[k0:k0 + 64] = np.sum(Q[None, :] * erfc(a * r) / r, axis=1)
        return out

    xo = P[pids]
    qi = Q[pids]
    zero = np.zeros_like(xo)
    phi_new = real(X, pids) + recip(X) - qi * self_recip(X - xo)
    phi_old = real(xo, pids) + recip(xo) - qi * self_recip(zero)
    return qi * (phi_new - phi_old)
