"""Device-side KMC driver: proposal generation, selection and lattice occupancy
on the GPU around one ``KMCFMM`` (C ABI ``kmc_driver_*``).

A step is generate -> ``propose_with_dats`` -> select -> ``accept`` with no host
round trip, so steps can be enqueued back to back or captured once as a CUDA
graph and replayed.  Two kinds, as in the reference's example driver
(examples/propose_with_dats_example.py:218-446) and its tests:

* ``lattice``: every charge proposes hops to its six nearest-neighbour sites,
  occupied targets masked; rejection-free selection with rate exp(-beta dE / 2).
* ``offlattice``: every charge proposes one displacement uniform in
  [-step, step]^3 (re-drawn while it leaves the box); one uniformly chosen
  charge's proposal is accepted with probability min(1, exp(-beta dE)).

Random numbers are Philox4x32-10 draws keyed by ``seed`` and counted by
(step, index), so a run is reproducible independently of launch shapes and of
whatever else runs on the GPU.
"""
from ctypes import POINTER, byref, c_int64, c_void_p

import numpy as np

from . import _native


class KMCDriver:
    def __init__(self, kmc, kind, beta, seed=0, lattice_side=None, lattice_sites=None, step=0.5, log_capacity=0):
        if kind not in _native.KMC_DRIVE:
            raise ValueError("kind must be one of %s" % sorted(_native.KMC_DRIVE))
        self.kmc = kmc
        self.kind = kind
        self.n = kmc.N
        self.M = 6 if kind == "lattice" else 1
        prm = _native.KmcDriverParams()
        prm.kind = _native.KMC_DRIVE[kind]
        prm.beta = float(beta)
        prm.step = float(step)
        prm.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        prm.log_capacity = int(log_capacity)
        sites = None
        if kind == "lattice":
            if lattice_side is None or lattice_sites is None:
                raise ValueError("a lattice driver needs lattice_side and lattice_sites")
            sites = np.ascontiguousarray(lattice_sites, dtype=np.int64)
            if sites.shape != (self.n,):
                raise ValueError("lattice_sites must hold one site per charge")
            prm.lattice_side = int(lattice_side)
            prm.lattice_sites = sites.ctypes.data_as(POINTER(c_int64))
        self._handle = c_void_p()
        kmc._set_stream()  # set-up work on the caller's current stream
        _native.check(_native.lib().kmc_driver_create(kmc._handle, byref(prm), byref(self._handle)),
                      "kmc_driver_create")
        self.log_capacity = int(log_capacity)
        kmc._energy_valid = False
        # the driver's work runs on its own stream (capturable), ordered after and
        # before the caller's current stream; a dedicated stream, not one from
        # torch's pool (pooled streams alias each other)
        self._ds = _native.DedicatedStream()
        self.stream = self._ds.stream

    def _enter(self):
        import torch
        self.stream.wait_stream(torch.cuda.current_stream())
        _native.lib().kmc_set_stream(self.kmc._handle, c_void_p(self.stream.cuda_stream))

    def _leave(self):
        import torch
        cur = torch.cuda.current_stream()
        cur.wait_stream(self.stream)
        # bind the system back to the caller's stream: the driver's stream is destroyed
        # with the driver, and the system may outlive it
        if self.kmc._handle is not None:
            _native.lib().kmc_set_stream(self.kmc._handle, c_void_p(cur.cuda_stream))
        self.kmc._energy_valid = False

    def step(self, n=1):
        """Enqueue n KMC steps (asynchronous)."""
        self._enter()
        try:
            _native.check(_native.lib().kmc_driver_step(self._handle, int(n)), "kmc_driver_step")
        finally:
            self._leave()

    def capture(self):
        """Capture one step as a CUDA graph (no step is run)."""
        self._enter()
        try:
            _native.check(_native.lib().kmc_driver_capture(self._handle), "kmc_driver_capture")
        finally:
            self._leave()

    def launch(self, n=1, stream=None):
        """Replay the captured step n times on ``stream`` (default: the driver's stream)."""
        if stream is None:
            self._enter()
            try:
                _native.check(_native.lib().kmc_driver_launch(self._handle, int(n), None), "kmc_driver_launch")
            finally:
                self._leave()
        else:
            s = c_void_p(int(getattr(stream, "cuda_stream", stream)))
            _native.check(_native.lib().kmc_driver_launch(self._handle, int(n), s), "kmc_driver_launch")
            self.kmc._energy_valid = False

    def counters(self):
        """(steps done, moves accepted); synchronises the device."""
        return self.stats()[:2]

    def stats(self):
        """(steps done, moves accepted, proposals evaluated); synchronises the device."""
        a, b, c = c_int64(), c_int64(), c_int64()
        _native.check(_native.lib().kmc_driver_counters(self._handle, byref(a), byref(b), byref(c)),
                      "kmc_driver_counters")
        return a.value, b.value, c.value

    def log(self):
        """Selection log, oldest first: (pid [-1 = rejected], target site or charge, dE)."""
        cap = self.log_capacity
        pid = np.zeros(cap, np.int64)
        tgt = np.zeros(cap, np.int64)
        de = np.zeros(cap)
        n = c_int64()
        _native.check(_native.lib().kmc_driver_log(self._handle, cap, pid.ctypes.data, tgt.ctypes.data,
                                                   de.ctypes.data, byref(n)), "kmc_driver_log")
        k = n.value
        return pid[:k], tgt[:k], de[:k]

    def sites(self):
        out = np.zeros(self.n, np.int64)
        _native.check(_native.lib().kmc_driver_sites(self._handle, out.ctypes.data), "kmc_driver_sites")
        return out

    def free(self):
        if self._handle is not None and self._handle.value:
            _native.lib().kmc_driver_free(self._handle)
        self._handle = None
        ds = getattr(self, "_ds", None)
        if ds is not None:
            ds.close()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass
