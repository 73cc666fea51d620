"""A full cell store under device-selected accepts.

The reference grows a cell's particle store when an accepted move fills it
(kmc_local.py:318-326, 558-580).  A device-selected accept cannot reallocate
inside a captured step, so:

* an accept whose new cell is full leaves the whole state as it was, is
  counted as an overflow, and is kept; every later device-selected accept is
  refused the same way and a host accept reports the overflow;
  kmc_resolve_overflow grows the store and applies the kept move, after which
  the state equals the oracle's with that move applied (1e-10, occupancy
  bit-exact);
* the device driver never gets there: it reads the occupancy before a cell can
  fill and grows the store first (captured steps are captured again), so a
  run from a store with no free slot gives the same moves, positions and
  energy as a run from a roomy store, with no overflow counted.

No fault is involved: the store's slots are checked before they are written.
"""
import numpy as np
import pytest

from conftest import neutral_charges, rel_err
from oracle import kmc_oracle as ko
from coulomb_kmc_gb300 import KMCFMM
from coulomb_kmc_gb300.dats import make_state
from coulomb_kmc_gb300.driver import KMCDriver
from coulomb_kmc_gb300.workloads import LatticeHopSystem

pytestmark = pytest.mark.gpu
TOL = 1e-10


def _device_accept(k, pid, pos):
    import torch
    de = float(k.propose(((pid, np.asarray(pos).reshape(1, 3)),))[0][0] - k.energy)
    d_pid = torch.tensor([pid], dtype=torch.int64, device="cuda")
    d_pos = torch.tensor(np.asarray(pos, dtype=np.float64).reshape(3), device="cuda")
    d_de = torch.tensor([de], dtype=torch.float64, device="cuda")
    k.accept_device(d_pid, d_pos, d_de)
    torch.cuda.synchronize()


def _same_state(k, o):
    s = k.state()
    assert np.array_equal(s["occupancy"], o.cell_occupancy())
    assert np.array_equal(s["cells"], o.fmm_cells)
    assert np.array_equal(s["positions"], o.positions)
    b = o.primary_local_expansions()
    assert np.max(np.abs(s["local_expansions"] - b)) <= TOL * max(1.0, np.max(np.abs(b)))
    assert rel_err(k.energy, o.energy) < TOL


@pytest.mark.parametrize("bc", ["free_space", "pbc"])
def test_device_accept_into_full_cell_is_refused_then_resolved(bc):
    from coulomb_kmc_gb300.lattice import lattice_operator
    N, E, R, L = 200, 6.0, 3, 8
    rng = np.random.default_rng(5)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    Q = neutral_charges(N)
    st = make_state(P, Q, E)
    k = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition=bc)
    k.initialise()
    o = ko.OracleKMC(P.copy(), Q, E, R, L, bc, lr_operator=lattice_operator(L, E) if bc == "pbc" else None)
    o.initialise()
    mx, cap = k.max_occupancy()
    cap = k.reserve_store(0)  # tightest store: the largest occupancy rounded up to 4 slots
    assert cap == ((mx + 3) // 4) * 4
    # fill the fullest cell: charges from other cells moved to points inside it
    n = 2 ** (R - 1)
    w = E / n
    occ = k.state()["occupancy"]
    target = int(np.argmax(occ))
    tc = np.array([target % n, (target // n) % n, target // (n * n)])
    centre = -0.5 * E + (tc + 0.5) * w
    movers = [i for i in range(N) if o.fmm_cells[i] != target]
    for j in range(cap - int(occ[target])):
        pid = movers[j]
        pos = centre + rng.uniform(-0.3 * w, 0.3 * w, 3)
        _device_accept(k, pid, pos)
        o.accept((pid, pos.copy()))
    assert k.error_counts() == (0, 0)
    _same_state(k, o)
    # the cell is full: the next move into it is refused and kept, the state unchanged
    pid_a = movers[cap]
    pos_a = centre + rng.uniform(-0.3 * w, 0.3 * w, 3)
    _device_accept(k, pid_a, pos_a)
    assert k.error_counts() == (0, 1)
    _same_state(k, o)
    # later device-selected accepts are refused too, and a host accept reports it
    _device_accept(k, movers[cap + 1], np.zeros(3))
    assert k.error_counts() == (0, 1)
    _same_state(k, o)
    with pytest.raises(RuntimeError, match="overflow"):
        k.accept((movers[cap + 2], np.zeros(3)))
    # resolve: the store grows and the kept move is applied
    assert k.resolve_overflow()
    o.accept((pid_a, pos_a.copy()))
    _same_state(k, o)
    assert k.max_occupancy()[1] > cap
    assert not k.resolve_overflow()
    # and the system carries on
    _device_accept(k, movers[cap + 1], np.zeros(3))
    o.accept((movers[cap + 1], np.zeros(3)))
    _same_state(k, o)
    assert k.error_counts() == (0, 0)
    k.free()


def _offlattice_system(reserve):
    N, E = 500, 10.0
    rng = np.random.default_rng(2)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    st = make_state(P, neutral_charges(N), E)
    k = KMCFMM(st.P, st.Q, st.domain, r=3, l=8, boundary_condition="free_space", max_move=1.0)
    k.initialise()
    k.reserve_store(reserve)
    return k


@pytest.mark.parametrize("captured", [False, True])
def test_offlattice_driver_grows_tight_store_ahead(captured):
    roomy = _offlattice_system(256)
    tight = _offlattice_system(0)
    cap0 = tight.max_occupancy()[1]
    da = KMCDriver(roomy, "offlattice", 1.0, seed=5, step=0.5, log_capacity=256)
    db = KMCDriver(tight, "offlattice", 1.0, seed=5, step=0.5, log_capacity=256)
    da.step(200)
    if captured:
        db.capture()            # captured against the tight store; re-captured after it grows
        for _ in range(4):
            db.launch(50)
    else:
        for _ in range(4):
            db.step(50)
    for x, y in zip(da.log(), db.log()):
        assert np.array_equal(x, y)
    assert da.counters() == db.counters()
    assert np.array_equal(roomy.state()["positions"], tight.state()["positions"])
    assert rel_err(tight.energy, roomy.energy) < 1e-12
    assert tight.error_counts() == (0, 0)
    assert tight.max_occupancy()[1] > cap0
    for x in (da, db, roomy, tight):
        x.free()


def test_lattice_driver_reserves_a_slot_per_site():
    hs = LatticeHopSystem(side=16, occupancy=0.25, seed=3)
    st = make_state(hs.positions(), hs.charges(), hs.extent)
    k = KMCFMM(st.P, st.Q, st.domain, r=3, l=8, boundary_condition="pbc", max_move=1.0)
    k.initialise()
    k.reserve_store(0)
    d = KMCDriver(k, "lattice", 2.0, seed=1, lattice_side=hs.side, lattice_sites=hs.site_of)
    assert k.max_occupancy()[1] >= (16 // 4) ** 3  # 64 sites per cell
    d.free()
    k.free()
