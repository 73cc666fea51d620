"""Insertion / removal energies of the oracle (CPU) against direct sums, as the
reference's own tests check them (tests/host/test_extract.py:50-156,
tests/host/test_inject.py:50-170: RandomState(3251), N=20, E=2*3.1416, r=3,
L=12, alternating unit charges): direct sums for free_space and '27', this
project's Ewald sum for pbc (neutral groups)."""
import numpy as np
import pytest

from oracle import kmc_oracle as ko
from oracle.ewald import ewald_energy
from coulomb_kmc_gb300.lattice import lattice_operator


def direct(bc, P, Q, E):
    d = P[:, None, :] - P[None, :, :]
    if bc == "pbc":
        return ewald_energy(P, Q, E)
    shifts = [np.zeros(3)] if bc == "free_space" else [
        np.array([a, b, c]) * E for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)]
    e = 0.0
    for s in shifts:
        r = np.sqrt(np.sum((d + s) ** 2, axis=2))
        if not s.any():
            np.fill_diagonal(r, np.inf)
        e += 0.5 * np.sum(Q[:, None] * Q[None, :] / r)
    return e


def setup(bc):
    rng = np.random.RandomState(3251)
    N, E = 20, 2 * 3.1416
    P = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(N, 3))
    Q = np.array([(-1.0) ** i for i in range(N)])
    o = ko.OracleKMC(P.copy(), Q, E, 3, 12, bc, max_move=1.0,
                     lr_operator=lattice_operator(12, E) if bc == "pbc" else None)
    o.initialise()
    return o, P, Q, E, rng


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
def test_compute_energy_is_the_direct_energy(bc):
    o, P, Q, E, _ = setup(bc)
    ref = direct(bc, P, Q, E)
    assert abs(o.compute_energy(P, Q) - ref) < 1e-6 * abs(ref)
    assert abs(o.energy - ref) < 1e-5 * abs(ref)


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
def test_propose_extract_against_direct(bc):
    o, P, Q, E, rng = setup(bc)
    e0 = direct(bc, P, Q, E)
    for _ in range(5):
        k = rng.randint(1, 5)
        plus = rng.choice(np.nonzero(Q > 0)[0], k, replace=False)
        minus = rng.choice(np.nonzero(Q < 0)[0], k, replace=False)
        rem = np.concatenate([plus, minus])
        keep = np.setdiff1d(np.arange(len(Q)), rem)
        ref = direct(bc, P[keep], Q[keep], E) - e0
        de = o.propose_extract(rem)
        assert abs(de[0] - ref) < 1e-5 * abs(ref) or abs(de[0] - ref) < 1e-5
        two = o.propose_extract(np.vstack([rem, rem]))
        assert abs(two[0] - de[0]) < 1e-12 and abs(two[1] - de[0]) < 1e-12


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
def test_propose_inject_against_direct(bc):
    o, P, Q, E, rng = setup(bc)
    e0 = direct(bc, P, Q, E)
    for _ in range(5):
        newp = rng.uniform(-0.5 * E, 0.5 * E, (2, 3))
        newq = np.array([1.0, -1.0])
        ref = direct(bc, np.vstack([P, newp]), np.concatenate([Q, newq]), E) - e0
        de = o.propose_inject(newp, newq)
        assert abs(de - ref) < 1e-5 * abs(ref) or abs(de - ref) < 1e-5


def test_get_energy_sums_groups():
    o, P, Q, E, _ = setup("27")
    single = o.get_energy(np.arange(6).reshape(6, 1))
    pairs = o.get_energy(np.arange(6).reshape(3, 2))
    assert np.allclose(pairs, single.reshape(3, 2).sum(axis=1), rtol=0, atol=1e-13)
