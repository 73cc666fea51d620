"""kmc_host_displacements (the host path's proposal generator, no GPU involved):
every proposal inside the box and within `step` of its charge on every axis, the
draws uniform, the result a pure function of (seed, round, index) whatever the
number of threads, different rounds and seeds giving different draws, and
aliasing or bad arguments rejected."""
import numpy as np
import pytest

from coulomb_kmc_gb300 import _native
from coulomb_kmc_gb300.workloads import uniform_displacements


def test_in_box_within_step_and_thread_independent():
    E, step, n = 20.0, 0.5, 50_000
    pos = np.random.default_rng(1).uniform(-0.5 * E, 0.5 * E, (n, 3))
    pos[:100] = 0.5 * E - 0.05          # charges at a corner: draws leave the box and are redrawn
    a = uniform_displacements(pos, E, step, seed=7, round_=3, threads=1)
    for t in (2, 5, 16):
        assert np.array_equal(a, uniform_displacements(pos, E, step, seed=7, round_=3, threads=t))
    assert np.all(np.abs(a) <= 0.5 * E)
    d = a - pos
    assert np.all(np.abs(d) <= step)
    # the displacements of charges far from the faces are uniform: mean 0, variance step^2 / 3
    far = np.all(np.abs(pos) < 0.5 * E - step, axis=1)
    assert abs(d[far].mean()) < 0.01
    assert abs(d[far].var() / (step * step / 3.0) - 1.0) < 0.02
    assert not np.array_equal(a, uniform_displacements(pos, E, step, seed=7, round_=4))
    assert not np.array_equal(a, uniform_displacements(pos, E, step, seed=8, round_=3))


def test_bad_arguments_rejected():
    pos = np.zeros((10, 3))
    with pytest.raises(RuntimeError):
        uniform_displacements(pos, -1.0, 0.5, 1, 0)
    with pytest.raises(RuntimeError):
        _native.check(_native.lib().kmc_host_displacements(10, pos.ctypes.data, 10.0, 0.5, 1, 0, pos.ctypes.data, 1),
                      "kmc_host_displacements")
    with pytest.raises(ValueError):
        uniform_displacements(pos, 10.0, 0.5, 1, 0, out=np.zeros((10, 2)))
