"""Mixed modes at high order in large periodic boxes.

The double-FP32 accept updates the multipole and the lattice vector g = A M on the
FP32 pipe.  In position units the operator's entries scale as E^-(l + l' + 1) and
the multipole's as |x|^l, which leave the FP32 range at high orders in large boxes
(E = 64, l + l' = 30: ~1e-56); the update works in box units instead.  After a
chain of accepts in pbc boxes of edge 64 and 400 at L = 16, every proposal's
difference in both mixed modes must stay within the 1e-6 bar of the FP64 path on
identical states (relative, denominator max(|dE|, 1)).
"""
import numpy as np
import pytest

from conftest import neutral_charges
from coulomb_kmc_gb300 import KMCFMM
from coulomb_kmc_gb300.dats import make_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("E", [64.0, 400.0])
@pytest.mark.parametrize("precision", ["mixed", "mixed_fp64_accept"])
def test_high_order_large_box_accept_chain(E, precision):
    N, L, R = 2000, 16, 3
    rng = np.random.default_rng(12)
    P = rng.uniform(-0.5 * E, 0.5 * E, (N, 3))
    Q = neutral_charges(N)
    ks = {}
    for name, prec in (("fp64", "fp64"), ("mixed", precision)):
        st = make_state(P.copy(), Q, E)
        ks[name] = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition="pbc", precision=prec)
        ks[name].initialise()
    smc = np.array([1], np.int64)
    sites = np.zeros((N, 1), np.int64)
    masks = np.ones((N, 1), np.int64)
    worst = 0.0
    pos = P.copy()
    for step in range(4):
        prop = np.clip(pos + rng.uniform(-0.5, 0.5, (N, 3)), -0.5 * E, 0.5 * E)
        d = {}
        for name, k in ks.items():
            d[name] = np.zeros((N, 1))
            k.propose_with_dats(smc, sites, prop, masks, d[name])
        err = np.abs(d["mixed"] - d["fp64"]) / np.maximum(np.abs(d["fp64"]), 1.0)
        worst = max(worst, float(err.max()))
        # a charge moved across the box (large multipole change) and one displaced
        for pid, new in ((int(rng.integers(0, N)), rng.uniform(-0.5 * E, 0.5 * E, 3)),
                         (int(rng.integers(0, N)), None)):
            if new is None:
                new = prop[pid].copy()
            for k in ks.values():
                k.accept((pid, new.copy()))
            pos[pid] = new
    assert worst < 1e-6, worst
    for k in ks.values():
        k.free()
