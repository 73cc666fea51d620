"""Near-field potentials kept between moves.

The reference sums every moving charge's near field afresh on each propose
(direct_old, kmc_local.py:956-1019).  Here each charge's near-field potential is
kept on the device (KMC_TUNE_NEAR_OLD = 0, the default) and every accept updates
the charges around the moved one (k_phin_move); a propose then evaluates only the
cell expansion for the moving charges.  After chains of host and device-selected
accepts -- moves across cells, within one cell, a null move, a move across a
periodic face -- and after extract and inject, a full propose_with_dats must give:

* FP64: the oracle's differences at 1e-10 (the parity tier) and the afresh sums'
  (KMC_TUNE_NEAR_OLD = 1) at 1e-11;
* mixed: the afresh sums' within 1e-8 (the afresh near sums are double-FP32,
  about 1e-10 relative in the differences and up to 2e-9; the kept potentials are
  FP64).
"""
import numpy as np
import pytest

from conftest import neutral_charges, rel_err
from oracle import kmc_oracle as ko
from coulomb_kmc_gb300 import KMCFMM, _native
from coulomb_kmc_gb300.dats import make_state
from coulomb_kmc_gb300.lattice import lattice_operator

pytestmark = pytest.mark.gpu
TOL = 1e-10
N, E, R, L, M = 300, 5.0, 3, 8, 2


def _device_accept(k, pid, pos):
    import torch
    de = float(k.propose(((pid, np.asarray(pos).reshape(1, 3)),))[0][0] - k.energy)
    d_pid = torch.tensor([pid], dtype=torch.int64, device="cuda")
    d_pos = torch.tensor(np.asarray(pos, dtype=np.float64).reshape(3), device="cuda")
    d_de = torch.tensor([de], dtype=torch.float64, device="cuda")
    k.accept_device(d_pid, d_pos, d_de)
    torch.cuda.synchronize()


def _moves(rng, pos):
    """(pid, new position) pairs covering the cases the update must handle."""
    w = E / 2 ** (R - 1)
    out = []
    for step in range(24):
        pid = int(rng.integers(0, pos.shape[0]))
        if step == 5:
            new = pos[pid].copy()                                     # null move
        elif step == 9:
            c = np.floor((pos[pid] + 0.5 * E) / w)
            new = -0.5 * E + (c + 0.5) * w + rng.uniform(-0.2, 0.2, 3) * w  # within its cell
        elif step == 13:
            new = np.array([0.5 * E - 1e-3, pos[pid][1], -0.5 * E + 1e-3])  # at two faces
        else:
            new = rng.uniform(-0.5 * E, 0.5 * E, 3)
        out.append((pid, new))
        pos[pid] = new
    return out


def _propose(k, rng_seed):
    rng = np.random.default_rng(rng_seed)
    smc = np.array([M], np.int64)
    sites = np.zeros((k.N, 1), np.int64)
    masks = np.ones((k.N, M), np.int64)
    ppos = rng.uniform(-0.5 * E, 0.5 * E, size=(k.N, 3 * M))
    out = {}
    for kept in (0, 1):
        k.set_tuning(_native.KMC_TUNE_NEAR_OLD, 1 - kept)
        d = np.zeros((k.N, M))
        k.propose_with_dats(smc, sites, ppos, masks, d)
        out[kept] = d
    k.set_tuning(_native.KMC_TUNE_NEAR_OLD, 0)
    return out, (smc, sites, ppos, masks)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("bc", ["free_space", "27", "pbc"])
def test_kept_potentials_after_accept_chains(bc, precision):
    rng = np.random.default_rng(17)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    Q = neutral_charges(N)
    st = make_state(P, Q, E)
    k = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition=bc, precision=precision)
    k.initialise()
    o = None
    if precision == "fp64":
        o = ko.OracleKMC(P.copy(), Q, E, R, L, bc, lr_operator=lattice_operator(L, E) if bc == "pbc" else None)
        o.initialise()
    for i, (pid, new) in enumerate(_moves(rng, P.copy())):
        if i % 2:
            _device_accept(k, pid, new)
        else:
            k.accept((pid, new.copy()))
        if o is not None:
            o.accept((pid, new.copy()))
    assert k.error_counts() == (0, 0)
    d, args = _propose(k, 3)
    if precision == "fp64":
        assert np.max(rel_err(d[1], d[0])) < 1e-11
        do = np.zeros_like(d[0])
        o.propose_with_dats(*args, do)
        assert np.max(rel_err(d[0], do)) < TOL
    else:
        assert np.max(rel_err(d[1], d[0])) < 1e-8
    k.free()


def test_kept_potentials_after_extract_and_inject():
    rng = np.random.default_rng(4)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    Q = neutral_charges(N)
    st = make_state(P, Q, E)
    k = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition="pbc")
    k.initialise()
    for pid, new in _moves(rng, P.copy())[:6]:
        k.accept((pid, new.copy()))
    k.extract([3, 40, 41])
    k.inject((rng.uniform(-0.5 * E, 0.5 * E, (2, 3)), np.array([1.0, -1.0])))
    for pid, new in _moves(rng, k.state()["positions"].copy())[:6]:
        k.accept((pid, new.copy()))
    d, _ = _propose(k, 5)
    assert np.max(rel_err(d[1], d[0])) < 1e-11
    k.free()


@pytest.mark.parametrize("bc", ["pbc", "27"])
def test_kept_potentials_two_cells_per_side(bc):
    """R = 2: every neighbour cell appears twice among a periodic cell's 27 (one image
    on each side), so the update must take each of them once per image."""
    n, Rr = 120, 2
    rng = np.random.default_rng(9)
    P = rng.uniform(-0.5 * E, 0.5 * E, (n, 3))
    Q = neutral_charges(n)
    st = make_state(P, Q, E)
    k = KMCFMM(st.P, st.Q, st.domain, r=Rr, l=L, boundary_condition=bc)
    k.initialise()
    o = ko.OracleKMC(P.copy(), Q, E, Rr, L, bc, lr_operator=lattice_operator(L, E) if bc == "pbc" else None)
    o.initialise()
    for i, (pid, new) in enumerate(_moves(rng, P.copy())[:12]):
        if i % 2:
            _device_accept(k, pid, new)
        else:
            k.accept((pid, new.copy()))
        o.accept((pid, new.copy()))
    d, args = _propose(k, 6)
    assert np.max(rel_err(d[1], d[0])) < 1e-11
    do = np.zeros_like(d[0])
    o.propose_with_dats(*args, do)
    assert np.max(rel_err(d[0], do)) < TOL
    k.free()

