"""eval_field (kmc_fmm.py:544-567) on the GPU against the oracle on the same
state (1e-10 relative, denominator max(|phi|, 1)), before and after accepts,
and against direct sums (free space, '27') at the reference's FMM tolerance."""
import numpy as np
import pytest
import torch

from conftest import neutral_charges, rel_err
from oracle import kmc_oracle as ko
from coulomb_kmc_gb300 import KMCFMM
from coulomb_kmc_gb300.dats import make_state
from coulomb_kmc_gb300.lattice import lattice_operator

pytestmark = pytest.mark.gpu


def pair(bc, N=300, E=6.0, R=3, L=12, seed=4):
    rng = np.random.default_rng(seed)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    Q = neutral_charges(N)
    st = make_state(P, Q, E)
    g = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition=bc, initial_solve="exact")
    g.initialise()
    o = ko.OracleKMC(P.copy(), Q, E, R, L, bc, lr_operator=lattice_operator(L, E) if bc == "pbc" else None)
    o.initialise()
    return g, o, rng, P, Q, E


@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
def test_eval_field_matches_oracle(bc):
    g, o, rng, P, Q, E = pair(bc)
    pts = rng.uniform(-0.5 * E, 0.5 * E, (200, 3))
    assert np.max(rel_err(g.eval_field(pts), o.eval_field(pts))) < 1e-10
    for _ in range(5):
        pid = int(rng.integers(0, len(P)))
        new = np.clip(P[pid] + rng.uniform(-0.4, 0.4, 3), -0.5 * E, 0.5 * E)
        g.accept((pid, new))
        o.accept((pid, new))
        P[pid] = new
    assert np.max(rel_err(g.eval_field(pts), o.eval_field(pts))) < 1e-10
    dev = torch.from_numpy(pts).cuda()
    out = g.eval_field(dev)
    assert out.is_cuda and np.max(rel_err(out.cpu().numpy(), o.eval_field(pts))) < 1e-10
    g.free()


@pytest.mark.parametrize("bc", ["free_space", "27"])
def test_eval_field_matches_direct_sums(bc):
    g, o, rng, P, Q, E = pair(bc, N=400, R=3, L=12)
    pts = rng.uniform(-0.5 * E, 0.5 * E, (50, 3))
    if bc == "free_space":
        ref = np.array([np.sum(Q / np.linalg.norm(P - p, axis=1)) for p in pts])
    else:
        shifts = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)]) * E
        ref = np.array([sum(np.sum(Q / np.linalg.norm(P + s - p, axis=1)) for s in shifts) for p in pts])
    got = g.eval_field(pts)
    assert np.max(rel_err(got, ref)) < 1e-4
    g.free()
