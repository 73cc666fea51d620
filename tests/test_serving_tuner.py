"""The round tuner's bookkeeping (Server.autotune_keys), with the systems and the
round stubbed: every candidate is set on every system (a key it leaves out keeps
each system's own value), the steps are captured again, one untimed and `rounds`
timed rounds run per candidate, and the fastest candidate is applied at the end."""
from coulomb_kmc_gb300.serving import Server


class _Kmc:
    def __init__(self, own):
        self.t = dict(own)

    def get_tuning(self, key):
        return self.t.get(key, 0)

    def set_tuning(self, key, value):
        self.t[key] = value


class _Drv:
    def __init__(self):
        self.captures = 0

    def capture(self):
        self.captures += 1


class _Slot:
    def __init__(self, own):
        self.kmc = _Kmc(own)
        self.drv = _Drv()


def test_candidates_applied_timed_and_the_fastest_kept():
    slots = [_Slot({11: 4}), _Slot({11: 8})]
    srv = object.__new__(Server)  # no device: only the tuner's bookkeeping runs
    srv._buckets = {}
    times = iter([9.0, 5.0, 5.0, 9.0, 3.0, 4.0, 9.0, 6.0, 6.0])
    seen = []

    def fake_round(sl):
        seen.append(tuple((s.kmc.get_tuning(11), s.kmc.get_tuning(15)) for s in sl))
        return next(times)

    srv.round = fake_round
    combos = [{}, {15: 1}, {11: 2, 15: 3}]
    best, ms = srv.autotune_keys(slots, combos, rounds=2)
    assert best == 1
    assert ms == [5.0, 3.5, 6.0]
    assert seen[0] == ((4, 0), (8, 0))   # the empty candidate: each system's own values
    assert seen[3] == ((4, 1), (8, 1))
    assert seen[6] == ((2, 3), (2, 3))
    assert [(s.kmc.get_tuning(11), s.kmc.get_tuning(15)) for s in slots] == [(4, 1), (8, 1)]
    assert all(s.drv.captures == 4 for s in slots)  # once per candidate, once for the choice
