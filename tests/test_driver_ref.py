"""Host restatement of the device KMC driver (CPU): Philox4x32-10 against the
published known-answer vectors of its authors' Random123 distribution, and the
lattice bookkeeping against the host workload used by the other tests."""
import numpy as np

from oracle.kmc_driver_ref import LatticeRef, OffLatticeRef, philox, u53
from coulomb_kmc_gb300.workloads import LatticeHopSystem


def test_philox_known_answers():
    r = philox(0, 0, 0, 0, 0)
    assert [int(x) for x in r] == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    r = philox(0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFF, 0xFFFFFFFFFFFFFFFF)
    assert [int(x) for x in r] == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]


def test_uniforms_in_range():
    r = philox(np.arange(10000), 0, 0, 0, 123)
    u = u53(r[0], r[1])
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.02


def test_lattice_ref_matches_workload():
    hs = LatticeHopSystem(side=10, occupancy=0.25, seed=4)
    ref = LatticeRef(hs.side, hs.extent, hs.site_of, True, 2.0, 1)
    a = ref.proposals()
    b = hs.proposals()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert np.array_equal(ref.site_pos(hs.site_of), hs.positions())


def test_free_space_lattice_masks_outward_hops():
    hs = LatticeHopSystem(side=6, occupancy=0.25, seed=2)
    ref = LatticeRef(hs.side, hs.extent, hs.site_of, False, 2.0, 1)
    ppos, masks, tsite = ref.proposals()
    k = hs.side
    xyz = np.stack([hs.site_of % k, (hs.site_of // k) % k, hs.site_of // (k * k)], axis=-1)
    for h, (ax, d) in enumerate([(0, 1), (0, -1), (1, 1), (1, -1), (2, 1), (2, -1)]):
        leaving = (xyz[:, ax] + d < 0) | (xyz[:, ax] + d >= k)
        assert np.all(masks[leaving, h] == 0)
    assert np.all(np.abs(ppos) <= 0.5 * hs.extent)


def test_offlattice_ref_stays_in_box():
    rng = np.random.default_rng(0)
    P = rng.uniform(-2.0, 2.0, (300, 3))
    ref = OffLatticeRef(P, 4.0, 0.5, 1.0, 9)
    prop = ref.proposals()
    assert np.all(np.abs(prop) <= 2.0)
    assert np.all(np.abs(prop - P) <= 0.5)
