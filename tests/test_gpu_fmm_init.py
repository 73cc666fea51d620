"""FMM initial solve (P2M, M2M, M2L, L2L on the GPU; the reference builds its
initial local expansions with ppmd's FMM, kmc_fmm.py:956-959).

* Against the exact particle-to-local initial solve: the initial energy and
  the proposed total energies agree to the FMM truncation error, within the
  reference's own criterion for its FMM-built state (total energy of a
  proposed move within 1e-5 relative at L=12, test_free_space_1.py:150-230),
  and the error falls as L grows.
* Against the oracle fed with the GPU's FMM expansions: the initial energy
  and every difference agree within 1e-10, as for the exact initial state."""
import numpy as np
import pytest

from conftest import neutral_charges, rel_err
from oracle import kmc_oracle as ko
from coulomb_kmc_gb300 import KMCFMM
from coulomb_kmc_gb300.dats import make_state
from coulomb_kmc_gb300.lattice import lattice_operator

pytestmark = pytest.mark.gpu


def system(N, E, seed):
    rng = np.random.default_rng(seed)
    return rng.uniform(-0.5 * E, 0.5 * E, (N, 3)), neutral_charges(N), rng


def make(P, Q, E, bc, R, L, how):
    st = make_state(P, Q, E)
    k = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition=bc, initial_solve=how)
    k.initialise()
    return k


def moves(P, E, rng, n=300):
    ids = rng.choice(len(P), size=n, replace=False)
    new = np.clip(P[ids] + rng.uniform(-0.5, 0.5, (n, 3)), -0.5 * E + 1e-9, 0.5 * E - 1e-9)
    return tuple((int(i), new[j:j + 1]) for j, i in enumerate(ids))


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
@pytest.mark.parametrize("R", [3, 4])
def test_fmm_matches_exact(bc, R):
    N, E, L = 600, 8.0, 12
    P, Q, rng = system(N, E, 11 + R)
    kx = make(P, Q, E, bc, R, L, "exact")
    kf = make(P, Q, E, bc, R, L, "fmm")
    assert abs(kf.energy - kx.energy) < 1e-5 * abs(kx.energy)
    mv = moves(P, E, rng)
    ex = np.concatenate(kx.propose(mv))
    ef = np.concatenate(kf.propose(mv))
    assert np.max(np.abs(ef - ex) / np.abs(ex)) < 1e-5
    kx.free()
    kf.free()


def test_fmm_error_falls_with_order():
    N, E = 600, 8.0
    P, Q, rng = system(N, E, 5)
    mv = moves(P, E, rng)
    errs = []
    for L in (6, 10, 16):
        kx = make(P, Q, E, "pbc", 4, L, "exact")
        kf = make(P, Q, E, "pbc", 4, L, "fmm")
        ex = np.concatenate(kx.propose(mv)) - kx.energy
        ef = np.concatenate(kf.propose(mv)) - kf.energy
        errs.append(float(np.max(rel_err(ef, ex))))
        kx.free()
        kf.free()
    assert errs[0] > errs[1] > errs[2], errs


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
def test_fmm_state_parity_with_oracle(bc):
    """Same initial expansions in both: the GPU energy and differences match the oracle at 1e-10."""
    N, E, R, L = 400, 8.0, 3, 12
    P, Q, rng = system(N, E, 21)
    kf = make(P, Q, E, bc, R, L, "fmm")
    lexp = kf.state()["local_expansions"]
    lr = lattice_operator(L, E) if bc == "pbc" else None
    o = ko.OracleKMC(P.copy(), Q, E, R, L, bc, lr_operator=lr)
    o.initialise(local_expansions=lexp)
    assert rel_err(kf.energy, o.energy) < 1e-10
    mv = moves(P, E, rng, 200)
    a = np.concatenate(kf.propose(mv))
    b = np.concatenate(o.propose(mv))
    assert np.max(rel_err(a, b)) < 1e-10
    kf.free()


def test_initial_solve_argument():
    P, Q, _ = system(50, 4.0, 1)
    st = make_state(P, Q, 4.0)
    with pytest.raises(ValueError):
        KMCFMM(st.P, st.Q, st.domain, r=2, l=8, boundary_condition="free_space", initial_solve="tree")
