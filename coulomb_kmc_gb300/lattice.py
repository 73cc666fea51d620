"""Far-field lattice operator for fully periodic cubic boxes.

This is the operator the reference takes from ppmd's ``LongRangeMTL``
(coulomb_kmc/kmc_full_long_range.py:40, used at :172,:186-188): a real
L^2 x L^2 matrix ``R`` that maps the level-0 multipole expansion M of the
primary box (about its centre) to the local expansion, about the same centre,
of every periodic image outside the 3x3x3 block, applied identically to the
real and imaginary blocks, plus a dipole correction (S_x, S_y, S_z).  The
periodic energy is then

    U_pbc = U_27 + 1/2 [ (R ReM).ReE + (R ImM).ImE + dip(M, E) ].

ppmd is not available, so the operator is derived here from the mathematics:

* Expansion convention (the reference's): Y_l^m = sqrt((l-|m|)!/(l+|m|)!)
  P_l^{|m|}(cos theta) e^{i m phi} (Condon-Shortley phase),
  M_n^m = sum q r^n Y_n^{-m}, local L_j^k evaluated as sum r^j Re(L Y_j^k).
* Multipole-to-local translation for a multipole about d:
  L_j^k = sum_{n,m} A(j,k,n,m) M_n^m Y_{j+n}^{m-k}(d) / |d|^{j+n+1}
  with A given by ``_a_coeff`` (scaled solid-harmonic addition theorem,
  checked numerically against particle-to-local sums).
* Lattice sums S_l^mu = sum_{d in E Z^3, |n|_inf >= 2} Y_l^mu(d)/|d|^{l+1}
  are Ewald-split sums of irregular solid harmonics (Hobson's theorem turns
  I_l^mu into a derivative of 1/r).  Cubic symmetry leaves only even l >= 4
  and mu = 0 mod 4; l <= 2 entries are set to zero (spherical summation
  order; the l = 2 block vanishes by symmetry and l = 0 only multiplies the
  total charge).
* The dipole correction converts the spherical-summation result to tin-foil
  (Ewald) boundary conditions: dip(M, M) = -(4 pi / 3V) |D|^2 with
  (S_x, S_y, S_z) = (-4pi/3V, +4pi/3V, -4pi/3V) in the reference's
  ``apply_dipole_correction_split`` form (kmc_full_long_range.py:521-540).

For neutral systems U_pbc agrees with an Ewald sum to the expansion's
truncation error (about 1e-7 relative at L = 12).
"""
from functools import lru_cache
from math import factorial, pi, sqrt

import numpy as np
from scipy.special import erfc

__all__ = ["lattice_operator", "dense_operator", "lattice_sums"]


def _norm_legendre(lmax, x):
    """sqrt((l-m)!/(l+m)!) P_l^m(x) for 0<=m<=l<lmax over an array x (CS phase)."""
    x = np.asarray(x, dtype=np.float64)
    s = np.sqrt(np.maximum(0.0, 1.0 - x * x))
    N = np.zeros((lmax, lmax) + x.shape)
    N[0, 0] = 1.0
    for m in range(1, lmax):
        N[m, m] = -np.sqrt((2 * m - 1) / (2 * m)) * s * N[m - 1, m - 1]
    for m in range(lmax - 1):
        N[m + 1, m] = np.sqrt(2 * m + 1) * x * N[m, m]
    for m in range(lmax):
        for l in range(m + 2, lmax):
            N[l, m] = ((2 * l - 1) * x * N[l - 1, m] - np.sqrt((l - 1) ** 2 - m * m) * N[l - 2, m]) / np.sqrt(
                l * l - m * m)
    return N


def _ylm_points(lmax, pts):
    """r, and Y[l, m+lmax] (complex) for an array of points (n,3)."""
    pts = np.asarray(pts, dtype=np.float64)
    r = np.linalg.norm(pts, axis=1)
    ct = pts[:, 2] / r
    ph = np.arctan2(pts[:, 1], pts[:, 0])
    N = _norm_legendre(lmax, ct)
    Y = np.zeros((lmax, 2 * lmax + 1, len(r)), dtype=np.complex128)
    for l in range(lmax):
        for m in range(-l, l + 1):
            Y[l, m + lmax] = N[l, abs(m)] * np.exp(1j * m * ph)
    return r, Y


def _s(m):
    """Y_l^m = s(m) C_l^m (Racah-normalised harmonic)."""
    return 1.0 if m >= 0 else (-1.0) ** m


def _dfact(n):
    r = 1.0
    while n > 1:
        r *= n
        n -= 2
    return r


@lru_cache(maxsize=64)
def lattice_sums(lmax, E, alpha_e=2.5, nreal=6, nrecip=9):
    """S[l, mu+lmax] = sum over lattice vectors outside the 3x3x3 block of
    Y_l^mu(d) / |d|^(l+1) for the cubic lattice of edge E, l < lmax."""
    E = float(E)
    V = E ** 3
    alpha = alpha_e / E
    g = np.arange(-nreal, nreal + 1)
    real = np.array([(a, b, c) for a in g for b in g for c in g if (a, b, c) != (0, 0, 0)], dtype=np.float64) * E
    near = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)
                     if (a, b, c) != (0, 0, 0)], dtype=np.float64) * E
    h = np.arange(-nrecip, nrecip + 1)
    recip = np.array([(a, b, c) for a in h for b in h for c in h if (a, b, c) != (0, 0, 0)],
                     dtype=np.float64) * (2 * pi / E)
    rr, Yr = _ylm_points(lmax, real)
    rk, Yk = _ylm_points(lmax, recip)
    rn, Yn = _ylm_points(lmax, near)
    # B_l(r) = ((1/r d/dr)^l erfc(alpha r)/r) * (-1)^l
    B = erfc(alpha * rr) / rr
    gauss = np.exp(-alpha * alpha * rr * rr)
    Bl = [B]
    for l in range(1, lmax):
        B = ((2 * l - 1) * B + (2 * alpha * alpha) ** l / (alpha * sqrt(pi)) * gauss) / (rr * rr)
        Bl.append(B)
    wk = np.exp(-rk * rk / (4 * alpha * alpha)) / (rk * rk)
    S = np.zeros((lmax, 2 * lmax + 1))
    for l in range(4, lmax, 2):
        for mu in range(-l, l + 1):
            if mu % 4 != 0:
                continue
            # C_l^mu = Y_l^mu / s(mu); real-space and reciprocal Ewald parts of sum I_l^mu
            c_real = np.sum(rr ** l * Yr[l, mu + lmax] * Bl[l]) / _s(mu) / _dfact(2 * l - 1)
            c_rec = (1j ** l) * ((-1.0) ** l) / _dfact(2 * l - 1) * 4 * pi / V * np.sum(
                rk ** l * Yk[l, mu + lmax] * wk) / _s(mu)
            val = _s(mu) * (c_real + c_rec) - np.sum(Yn[l, mu + lmax] / rn ** (l + 1))
            S[l, mu + lmax] = val.real
    return S


def _a_coeff(j, k, n, m):
    """Multipole-to-local coefficient A(j,k,n,m) in the reference's normalisation."""
    l = j + n
    mu = m - k
    c = (-1.0) ** n * (-1.0) ** m * _s(-m) * _s(-k)
    c /= sqrt(factorial(n - m) * factorial(n + m)) * sqrt(factorial(j - k) * factorial(j + k))
    c *= sqrt(factorial(l - mu) * factorial(l + mu)) / _s(mu)
    return c


@lru_cache(maxsize=64)
def dense_operator(L, E):
    """Dense R (L^2 x L^2), row = l(l+1)+k of the local expansion, col = n(n+1)+m.

    The lattice sums are homogeneous in the edge, S_l(E) = S_l(1) E^-(l+1), so R is
    built once per L for E = 1 and scaled: R(E)[jk, nm] = R(1)[jk, nm] E^-(j+n+1)."""
    R1 = _unit_operator(int(L))
    deg = np.array([j for j in range(L) for _ in range(2 * j + 1)], dtype=np.float64)
    scale = float(E) ** (-(deg[:, None] + deg[None, :] + 1.0))
    R = R1 * scale
    R = 0.5 * (R + R.T)
    R.setflags(write=False)
    return R


@lru_cache(maxsize=8)
def _unit_operator(L):
    lmax = 2 * L - 1
    S = lattice_sums(lmax, 1.0)
    R = np.zeros((L * L, L * L))
    for j in range(L):
        for k in range(-j, j + 1):
            for n in range(L):
                for m in range(-n, n + 1):
                    l, mu = j + n, m - k
                    if l < 4 or l % 2 or mu % 4:
                        continue
                    s = S[l, mu + lmax]
                    if s != 0.0:
                        R[j * j + j + k, n * n + n + m] = _a_coeff(j, k, n, m) * s
    R = 0.5 * (R + R.T)  # exactly symmetric by construction; remove rounding asymmetry
    R.setflags(write=False)
    return R


def lattice_operator(L, E):
    """(data, indptr, indices, dipole) in CSR form, the reference's LongRangeMTL
    interface (linop_data / linop_indptr / linop_indices, dipole_correction)."""
    R = dense_operator(int(L), float(E))
    nz = R != 0.0
    indptr = np.zeros(L * L + 1, dtype=np.int64)
    indptr[1:] = np.cumsum(nz.sum(axis=1))
    rows, cols = np.nonzero(nz)
    data = R[rows, cols].astype(np.float64)
    c = -4.0 * pi / (3.0 * float(E) ** 3)
    dipole = np.array([c, -c, c], dtype=np.float64)
    return data, indptr, cols.astype(np.int64), dipole
