"""Insertion and removal of charges on the GPU (kmc_inject_extract.py) against
the oracle on the same state (1e-10), and the state after extract / inject
against a fresh initial solve of the resulting charges: expansions within
1e-10 of their scale, positions equal, energy within the reference's
tolerance for its incremental energy (tests/host/test_extract.py:250-256)."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import kmc_oracle as ko
from coulomb_kmc_gb300 import KMCFMM
from coulomb_kmc_gb300.dats import make_state
from coulomb_kmc_gb300.lattice import lattice_operator

pytestmark = pytest.mark.gpu


def system(bc, precision="fp64", N=200, E=6.0, seed=3251):
    rng = np.random.RandomState(seed)
    P = rng.uniform(low=-0.5 * E, high=0.5 * E, size=(N, 3))
    Q = np.array([(-1.0) ** i for i in range(N)])
    st = make_state(P, Q, E)
    k = KMCFMM(st.P, st.Q, st.domain, r=3, l=12, max_move=1.0, boundary_condition=bc, precision=precision,
               initial_solve="exact")
    k.initialise()
    return k, st, P, Q, E, rng


def oracle(bc, P, Q, E):
    o = ko.OracleKMC(P.copy(), Q, E, 3, 12, bc, max_move=1.0,
                     lr_operator=lattice_operator(12, E) if bc == "pbc" else None)
    o.initialise()
    return o


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
def test_energies_match_oracle(bc):
    k, st, P, Q, E, rng = system(bc)
    o = oracle(bc, P, Q, E)
    ids = rng.permutation(len(Q))[:12].reshape(6, 2)
    assert np.max(rel_err(k.get_energy(ids), o.get_energy(ids))) < 1e-10
    assert rel_err(k.compute_energy(P[:9], Q[:9]), o.compute_energy(P[:9], Q[:9])) < 1e-10
    rem = np.array([0, 5, 8, 13])
    assert np.max(rel_err(k.propose_extract(rem), o.propose_extract(rem))) < 1e-10
    newp = rng.uniform(-0.5 * E, 0.5 * E, (3, 3))
    newq = np.array([1.0, -1.0, 1.0])
    assert rel_err(k.propose_inject(newp, newq), o.propose_inject(newp, newq)) < 1e-10
    energy = np.zeros((len(Q), 1))
    masks = np.zeros((len(Q), 1), np.int64)
    masks[[1, 4, 9]] = 1
    k.get_energy_with_dats(masks, energy)
    assert np.max(rel_err(energy[[1, 4, 9], 0], o.get_energy(np.array([[1], [4], [9]])))) < 1e-10
    k.free()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
def test_extract_then_inject(bc, precision):
    k, st, P, Q, E, rng = system(bc, precision)
    e0 = k.energy
    rem = np.array([2, 3, 10, 11, 40, 41])
    de = k.propose_extract(rem)[0]
    k.extract(rem)
    keep = np.setdiff1d(np.arange(len(Q)), rem)
    st2 = make_state(P[keep], Q[keep], E)
    fresh = KMCFMM(st2.P, st2.Q, st2.domain, r=3, l=12, max_move=1.0, boundary_condition=bc,
                   precision=precision, initial_solve="exact")
    fresh.initialise()
    a, b = k.state(), fresh.state()
    assert k.N == len(keep) and np.array_equal(a["positions"], P[keep])
    assert np.array_equal(a["occupancy"], b["occupancy"])
    scale = np.max(np.abs(b["local_expansions"]))
    assert np.max(np.abs(a["local_expansions"] - b["local_expansions"])) < 1e-10 * scale
    assert abs(k.energy - (e0 + de)) < 1e-12 * abs(e0)
    assert abs(k.energy - fresh.energy) < 1e-5 * abs(fresh.energy)
    # proposals on the shrunk system equal those of the fresh one
    mv = tuple((i, np.clip(P[keep][i] + 0.3, -0.5 * E, 0.5 * E).reshape(1, 3)) for i in range(0, len(keep), 17))
    d1 = np.concatenate(k.propose(mv)) - k.energy
    d2 = np.concatenate(fresh.propose(mv)) - fresh.energy
    assert np.max(rel_err(d1, d2)) < (1e-9 if precision == "fp64" else 1e-6)
    # inject two charges back
    newp = rng.uniform(-0.5 * E, 0.5 * E, (2, 3))
    newq = np.array([1.0, -1.0])
    di = k.propose_inject(newp, newq)
    e1 = k.energy
    k.inject((newp, newq))
    assert k.N == len(keep) + 2
    assert abs(k.energy - (e1 + di)) < 1e-12 * abs(e1)
    P3 = np.vstack([P[keep], newp])
    Q3 = np.concatenate([Q[keep], newq])
    st3 = make_state(P3, Q3, E)
    f3 = KMCFMM(st3.P, st3.Q, st3.domain, r=3, l=12, max_move=1.0, boundary_condition=bc, precision=precision,
                initial_solve="exact")
    f3.initialise()
    a, b = k.state(), f3.state()
    assert np.array_equal(a["positions"], P3)
    scale = np.max(np.abs(b["local_expansions"]))
    assert np.max(np.abs(a["local_expansions"] - b["local_expansions"])) < 1e-10 * scale
    assert abs(k.energy - f3.energy) < 1e-5 * abs(f3.energy)
    for x in (k, fresh, f3):
        x.free()


def test_bad_extract_and_inject():
    k, st, P, Q, E, rng = system("free_space", N=40)
    with pytest.raises(RuntimeError):
        k.extract([1, 1])
    with pytest.raises(RuntimeError):
        k.inject((np.array([[0.0, 0.0, 10.0 * E]]), np.array([1.0])))
    k.free()
