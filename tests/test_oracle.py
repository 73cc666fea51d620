"""CPU oracle pinned against the golden fixtures and the reference's own
known-answer relations (direct sums, scipy-lpmv harmonics, Ewald)."""
from math import cos, factorial, sin, sqrt

import numpy as np
import pytest
from scipy.special import lpmv

from conftest import load_golden, neutral_charges, rel_err
from oracle import kmc_oracle as ko
from oracle.ewald import ewald_energy
from coulomb_kmc_gb300.lattice import lattice_operator


# --- harmonics: restatements of kmc_expansion_tools.py:384-491 with scipy lpmv ---
def py_multipole_exp(L, sph, charge):
    arr = np.zeros(2 * L * L)
    for lx in range(L):
        p = lpmv(range(lx + 1), lx, cos(sph[1]))
        for mx in range(-lx, lx + 1):
            coeff = charge * sph[0] ** lx * sqrt(factorial(lx - abs(mx)) / factorial(lx + abs(mx))) * p[abs(mx)]
            arr[lx * lx + lx + mx] += cos(-mx * sph[2]) * coeff
            arr[L * L + lx * lx + lx + mx] += sin(-mx * sph[2]) * coeff
    return arr


def py_phi_local(L, moments, sph):
    phi = 0.0
    for lx in range(L):
        p = lpmv(range(lx + 1), lx, cos(sph[1]))
        for mx in range(-lx, lx + 1):
            val = sqrt(factorial(lx - abs(mx)) / factorial(lx + abs(mx))) * p[abs(mx)] * sph[0] ** lx
            re, im = cos(mx * sph[2]) * val, sin(mx * sph[2]) * val
            phi += re * moments[lx * lx + lx + mx] - im * moments[L * L + lx * lx + lx + mx]
    return phi


@pytest.mark.parametrize("L", [12, 26])
def test_harmonics_vs_lpmv(L):
    """tests/host/test_pbc_1.py:38-87 (C multipole / local eval vs the scipy restatement, 1e-12)."""
    rng = np.random.RandomState(seed=1234)
    for _ in range(10):
        p = rng.uniform(-1.0, 1.0, 3)
        sph = ko.spherical(p)
        q = rng.uniform(-1, 1)
        c = np.zeros(2 * L * L)
        ko.multipole_exp(L, sph, q, c)
        ref = py_multipole_exp(L, sph, q)
        assert np.max(np.abs(c - ref)) < 1e-12 * max(1.0, np.max(np.abs(ref)))
        d = np.zeros(2 * L * L)
        ko.dot_vec(L, sph, q, d)
        assert np.array_equal(c, d)  # multipole and dot vector coincide for a single charge
        mom = rng.uniform(-1, 1, 2 * L * L)
        a, b = ko.local_eval(L, sph, mom), py_phi_local(L, mom, sph)
        assert abs(a - b) < 1e-12 * max(1.0, abs(b))


def test_local_exp_addition_theorem():
    """local_exp then local_eval reproduces q/|x - s| (truncation-limited)."""
    L = 26
    s = np.array([1.7, -2.1, 2.9])
    lexp = np.zeros(2 * L * L)
    ko.local_exp(L, ko.spherical(s), 0.7, lexp)
    for x in ([0.1, 0.2, -0.3], [-0.4, 0.05, 0.2]):
        x = np.array(x)
        assert abs(ko.local_eval(L, ko.spherical(x), lexp) - 0.7 / np.linalg.norm(x - s)) < 1e-13


@pytest.mark.parametrize("R", [3, 4, 5])
def test_golden_free_space_1(R):
    g = load_golden("free_space_1")
    P = g["P"].copy()
    o = ko.OracleKMC(P, g["Q"], float(g["E"]), R, 12, "free_space")
    o.initialise()
    assert rel_err(o.energy, g["e0"]) < 1e-5
    for pid, mv, ref in zip(g["pids"], g["moves"], g["energies"]):
        e = o.propose(((int(pid), mv),))[0][0]
        assert abs(e - ref) / abs(ref) < 1e-5


def test_golden_nearest27_1():
    g = load_golden("nearest27_1")
    o = ko.OracleKMC(g["P"].copy(), g["Q"], float(g["E"]), 3, 12, "27")
    o.initialise()
    assert rel_err(o.energy, g["e0"]) < 1e-5
    for pid, mv, ref in zip(g["pids"], g["moves"], g["energies"]):
        e = o.propose(((int(pid), mv),))[0][0]
        assert abs(e - ref) / abs(ref) < 1e-5


def test_golden_free_space_2_multi():
    g = load_golden("free_space_2")
    o = ko.OracleKMC(g["P"].copy(), g["Q"], float(g["E"]), 3, 12, "free_space")
    o.initialise()
    moves, k = [], 0
    for pid, c in zip(g["pids"], g["counts"]):
        moves.append((int(pid), g["moves"][k:k + c]))
        k += c
    got = np.concatenate(o.propose(moves))
    assert np.max(np.abs(got - g["energies"]) / np.abs(g["energies"])) < 1e-5


def test_golden_pbc_1():
    g = load_golden("pbc_1")
    E = float(g["E"])
    o = ko.OracleKMC(g["P"].copy(), g["Q"], E, 3, 12, "pbc", lr_operator=lattice_operator(12, E))
    o.initialise()
    assert rel_err(o.energy, g["e0"]) < 1e-5
    for pid, mv, ref in zip(g["pids"], g["moves"], g["energies"]):
        e = o.propose(((int(pid), mv),))[0][0]
        assert abs(e - ref) / abs(ref) < 1e-5


@pytest.mark.parametrize("E,L,tol", [(1.0, 12, 1e-6), (4.0, 16, 5e-8)])
def test_lattice_operator_vs_ewald(E, L, tol):
    """E_27 + 1/2 M^T R M + dipole = Ewald (tin-foil) for neutral systems."""
    rng = np.random.default_rng(7)
    N = 12
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    Q = neutral_charges(N)
    d, ip, ix, dip = lattice_operator(L, E)
    M = np.zeros(2 * L * L)
    for i in range(N):
        ko.multipole_exp(L, ko.spherical(P[i]), Q[i], M)
    lr = ko.lib().orc_lr_energy(ko.c_int64(L), ko._p(d), ko._p(ip), ko._p(ix), ko._p(dip), ko._p(M), ko._p(M))
    e = ko.direct_energy("27", E, P, Q) + lr
    assert abs(e - ewald_energy(P, Q, E)) / abs(ewald_energy(P, Q, E)) < tol


def test_lattice_operator_structure():
    from coulomb_kmc_gb300.lattice import dense_operator
    R = dense_operator(12, 3.0)
    assert np.array_equal(R, R.T)
    rows, cols = np.nonzero(R)
    for r, c in zip(rows, cols):
        j = int(np.floor(np.sqrt(r)))
        n = int(np.floor(np.sqrt(c)))
        k, m = r - j * j - j, c - n * n - n
        assert (j + n) % 2 == 0 and (m - k) % 4 == 0 and j + n >= 4


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
def test_accept_chain_vs_reinit(bc):
    """Incremental accept equals re-initialisation (test_free_space_1.py:450-542 pattern).

    The expansions and occupancy agree to rounding.  The energies agree to the
    expansion truncation error only (the re-initialised energy averages each
    far pair over both partners), hence the reference's 1e-6 tolerance."""
    E, N, L, R = 4.0, 200, 12, 3
    rng = np.random.RandomState(seed=8657)
    P = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(N, 3))
    Q = neutral_charges(N)
    lr = lattice_operator(L, E) if bc == "pbc" else None
    o = ko.OracleKMC(P.copy(), Q, E, R, L, bc, lr_operator=lr)
    o.initialise()
    for _ in range(6):
        pid = rng.randint(0, N - 1)
        mv = rng.uniform(low=-0.5 * E, high=0.5 * E, size=3)
        o.accept((pid, mv))
    r = ko.OracleKMC(o.positions.copy(), Q, E, R, L, bc, lr_operator=lr)
    r.initialise()
    assert rel_err(o.energy, r.energy) < 1e-6
    a, b = o.primary_local_expansions(), r.primary_local_expansions()
    assert np.max(np.abs(a - b)) < 1e-10 * max(1.0, np.max(np.abs(b)))
    assert np.array_equal(o.cell_occupancy(), r.cell_occupancy())


def test_propose_with_dats_matches_propose():
    """setup_propose_with_dats and setup_propose give the same energies (test_propose_dat_setup.py:32-208)."""
    E, N, L, R, M = 4.0, 100, 10, 3, 4
    rng = np.random.RandomState(seed=12413)
    P = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(N, 3))
    Q = neutral_charges(N)
    o = ko.OracleKMC(P.copy(), Q, E, R, L, "free_space")
    o.initialise()
    smc = rng.randint(0, 5, size=4).astype(np.int64)
    sites = rng.randint(0, 4, size=(N, 1)).astype(np.int64)
    masks = rng.randint(0, 2, size=(N, M)).astype(np.int64)
    ppos = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(N, 3 * M))
    diffs = np.full((N, M), -7.0)
    o.propose_with_dats(smc, sites, ppos, masks, diffs)
    for px in range(N):
        found = 0
        for mv in range(M):
            if masks[px, mv] > 0 and found < smc[sites[px, 0]]:
                e = o.propose(((px, ppos[px, 3 * mv:3 * mv + 3]),))[0][0]
                assert abs((o.energy + diffs[px, mv]) - e) < 1e-10 * max(1, abs(e))
                found += 1
            else:
                assert diffs[px, mv] == -7.0


def test_bad_moves_raise():
    E = 4.0
    P = np.random.RandomState(1).uniform(-1.9, 1.9, (20, 3))
    o = ko.OracleKMC(P.copy(), neutral_charges(20), E, 3, 8, "free_space", max_move=0.5)
    o.initialise()
    with pytest.raises(RuntimeError):
        o.propose(((0, P[0] + np.array([0.6, 0, 0])),))
    with pytest.raises(RuntimeError):
        o.propose(((0, np.array([2.5, 0, 0])),))
