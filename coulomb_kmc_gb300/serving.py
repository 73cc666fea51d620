"""Continuous batching of independent KMC systems on one GPU.

A request asks for K propose/accept rounds of one KMC system (lattice hopping
or off-lattice moves).  The server

* admits requests as slots and HBM budget free up: admission threads build
  systems (charges, initial solve, device driver, captured step graph), each
  on its own CUDA stream, while the GPU keeps running the live systems' rounds;
* runs rounds: every live system advances one KMC step per round, all of them
  in one host call (``kmc_drivers_launch``: each system's captured step graph
  on one of a pool of worker streams, so small systems overlap on the device);
* retires a system after its K rounds and frees its memory.

State (positions, charges, cell stores, expansions, proposal buffers) stays on
the device for a system's whole life.  The per-round latency (all live
systems advancing one step) is timed with CUDA events.  Nothing here changes
results: a system evolves identically alone or in any mix (deterministic
kernels, per-system Philox streams).
"""
import ctypes
import math
import queue
import threading
import time
from ctypes import c_int64, c_void_p
from dataclasses import dataclass, field

import numpy as np

from . import _native
from .dats import make_state
from .driver import KMCDriver
from .kmc_fmm import KMCFMM


@dataclass
class Request:
    rid: int
    kind: str           # 'lattice' (pbc lattice hopping) or 'offlattice'
    bc: str             # boundary condition
    n: int              # charges requested
    rounds: int
    seed: int
    arrival: float = 0.0
    L: int = 12
    density: float = 0.25
    beta: float = 1.0


def default_r(n):
    """FMM levels for n charges: max(2, ceil(log8(n / 8)))."""
    return max(2, int(math.ceil(math.log(max(n / 8.0, 1.0), 8) - 1e-12)))


def system_inputs(req):
    """Positions, charges, box edge and (lattice) sites of a request, from its seed."""
    rng = np.random.default_rng(req.seed)
    if req.kind == "lattice":
        side = max(4, int(round((req.n / req.density) ** (1.0 / 3.0))))
        nsites = side ** 3
        n = int(round(req.density * nsites))
        n -= n % 2
        sites = rng.choice(nsites, size=n, replace=False).astype(np.int64)
        xyz = np.stack([sites % side, (sites // side) % side, sites // (side * side)], axis=-1)
        pos = (xyz.astype(np.float64) - 0.5 * side) + 0.5
        E = float(side)
    else:
        n = req.n - req.n % 2
        E = (n / req.density) ** (1.0 / 3.0)
        pos = rng.uniform(-0.5 * E, 0.5 * E, size=(n, 3))
        sites, side = None, None
    q = np.ones(n)
    q[: n // 2] = -1.0
    rng.shuffle(q)
    return pos, q, E, sites, side


def estimate_bytes(n, kind, L, R):
    """Device memory of one system (store, expansions, FP32 copies, proposal and
    driver buffers), with margin; used for admission against the HBM budget."""
    M = 6 if kind == "lattice" else 1
    ncell = 8 ** (R - 1)
    nh = L * (L + 1) // 2
    per_prop = 3 * 8 + 8 + 8 + 4 + 64      # proposal position, mask, difference, target, propose scratch
    per_charge = 3 * 8 + 8 + 16 + 2 * 32 + 64
    cells = ncell * nh * (16 + 16) * 2      # FP64 + FP32 copies, and the FMM levels during the initial solve
    return int(1.5 * (n * M * per_prop + n * per_charge + cells) + (8 << 20))


@dataclass
class Slot:
    req: Request
    kmc: KMCFMM
    drv: KMCDriver
    nbytes: int
    admitted: float
    done: int = 0
    proposals_per_step: float = 0.0
    finished: float = field(default=0.0)


def build_system(req, precision, stream=None):
    """Create, initialise and capture one system (on ``stream`` if given)."""
    import torch
    pos, q, E, sites, side = system_inputs(req)
    ctx = torch.cuda.stream(stream) if stream is not None else _null()
    with ctx:
        st = make_state(pos, q, E)
        max_move = 1.0 if req.kind == "lattice" else 0.5
        k = KMCFMM(st.P, st.Q, st.domain, r=default_r(len(q)), l=req.L, boundary_condition=req.bc,
                   max_move=max_move, precision=precision)
        k.initialise()
        if req.kind == "lattice":
            d = KMCDriver(k, "lattice", req.beta, seed=req.seed, lattice_side=side, lattice_sites=sites)
        else:
            d = KMCDriver(k, "offlattice", req.beta, seed=req.seed, step=0.5)
        d.capture()
        torch.cuda.current_stream().synchronize()
    return k, d


class _null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False


class Server:
    def __init__(self, precision="mixed", hbm_budget=150e9, max_active=64, n_workers=16, keep_results=False,
                 n_admit=4, launch="streams"):
        import torch
        if launch not in ("streams", "buckets"):
            raise ValueError("launch must be 'streams' or 'buckets'")
        self.precision = precision
        # how a round is launched: "streams" -- every system's captured step graph on one of
        # the worker streams; "buckets" -- one graph per size bucket holding the steps of
        # all its systems (kmc_bucket_*), the buckets spread over the worker streams.
        # Results are the same either way (the same step graphs run); autotune_launch()
        # times both and keeps the faster.
        self.launch = launch
        self._buckets = {}  # bucket key -> (driver handles, kmc_bucket handle)
        self.keep_results = bool(keep_results)
        self.results = {}
        self.peak_active = 0
        self.budget = float(hbm_budget)
        self.max_active = int(max_active)
        # dedicated streams (torch.cuda.Stream() reuses a fixed pool, whose members
        # would alias the drivers' capture streams)
        self._owned = [_native.DedicatedStream() for _ in range(int(n_workers) + 1 + max(1, int(n_admit)))]
        self.workers = [d.stream for d in self._owned[:int(n_workers)]]
        self.main = self._owned[int(n_workers)].stream
        # admission threads, each building systems on its own stream
        self.admit_streams = [d.stream for d in self._owned[int(n_workers) + 1:]]
        self.build_s = []
        self.used = 0.0
        self.reserved = 0  # slots taken by systems being built, waiting or running
        self.active = []
        self._cv = threading.Condition()
        self._worker_ptrs = (c_void_p * len(self.workers))(*[s.cuda_stream for s in self.workers])
        # request id -> "done", "cancelled", "rejected: ..." or "error: ..." (every served request)
        self.status = {}
        self._cancel = set()
        # the round's launch call (kmc_drivers_launch); an attribute so that a test can put a
        # fake in its place that returns an error code, which ends the run with an error
        self._launch = _native.lib().kmc_drivers_launch
        # round timing events, created once (before any system captures its step)
        self._e0 = torch.cuda.Event(enable_timing=True)
        self._e1 = torch.cuda.Event(enable_timing=True)

    # -- one round over the given slots ------------------------------------
    @staticmethod
    def bucket_key(slot):
        """Size bucket of a system: the same FMM depth, order, boundary condition and
        kind of driver (the same kernels and launch shapes)."""
        return (slot.kmc.R, slot.kmc.L, str(slot.req.bc), slot.req.kind)

    def _bucket_handles(self, slots):
        """One kmc_bucket per size bucket of `slots` (kept while its members stay)."""
        groups = {}
        for sl in slots:
            groups.setdefault(self.bucket_key(sl), []).append(sl.drv._handle.value)
        out = []
        for key, members in sorted(groups.items()):
            members = tuple(members)
            have = self._buckets.get(key)
            if have is None or have[0] != members:
                if have is not None:
                    _native.lib().kmc_bucket_free(have[1])
                arr = (c_void_p * len(members))(*members)
                h = c_void_p()
                _native.check(_native.lib().kmc_bucket_create(arr, len(members), ctypes.byref(h)),
                              "kmc_bucket_create")
                self._buckets[key] = (members, h)
            out.append(self._buckets[key][1])
        for key in [k for k in self._buckets if k not in groups]:
            _native.lib().kmc_bucket_free(self._buckets.pop(key)[1])
        return out

    def free_buckets(self):
        for _, h in self._buckets.values():
            _native.lib().kmc_bucket_free(h)
        self._buckets = {}

    def round(self, slots):
        """Advance every slot one step; returns the round's device time in ms."""
        import torch
        if not slots:
            return 0.0
        e0, e1 = self._e0, self._e1
        if self.launch == "buckets":
            hs = self._bucket_handles(slots)
            e0.record(self.main)
            for i, h in enumerate(hs):
                w = self.workers[i % len(self.workers)]
                w.wait_event(e0)
                _native.check(_native.lib().kmc_bucket_launch(h, 1, c_void_p(w.cuda_stream)), "kmc_bucket_launch")
            for w in self.workers[:len(hs)]:
                self.main.wait_stream(w)
        else:
            arr = (c_void_p * len(slots))(*[s.drv._handle.value for s in slots])
            e0.record(self.main)
            _native.check(self._launch(arr, len(slots), 1, c_void_p(self.main.cuda_stream), self._worker_ptrs,
                                       len(self.workers)), "kmc_drivers_launch")
        e1.record(self.main)
        e1.synchronize()
        for s in slots:
            s.done += 1
        return e0.elapsed_time(e1)

    def autotune_keys(self, slots, candidates, rounds=2):
        """autotune_key for combinations: each candidate maps keys to values, a key it
        leaves out keeps every system's own value (an empty candidate: the systems as
        they are).  Returns (the best candidate's index, [median round ms per candidate])."""
        keys = sorted({k for c in candidates for k in c})
        base = [{k: sl.kmc.get_tuning(k) for k in keys} for sl in slots]

        def apply(c):
            for sl, b in zip(slots, base):
                for k in keys:
                    sl.kmc.set_tuning(k, c.get(k, b[k]))
                sl.drv.capture()
            self.free_buckets()

        timing = []
        for c in candidates:
            apply(c)
            self.round(slots)
            timing.append(float(np.median([self.round(slots) for _ in range(rounds)])))
        best = int(np.argmin(timing))
        apply(candidates[best])
        return best, timing

    def autotune_key(self, slots, key, candidates, rounds=2):
        """Tune one launch-shape key whose variants give bit-identical results on whole
        rounds of `slots` (the device full, as in service): each candidate is set on
        every system, the steps captured again and `rounds` rounds timed (real rounds:
        the systems advance identically under every candidate); the fastest is kept.
        Returns (value, {value: median round ms})."""
        timing = {}

        def apply(v):
            for sl in slots:
                sl.kmc.set_tuning(key, v)
                sl.drv.capture()
            self.free_buckets()

        for v in candidates:
            apply(v)
            self.round(slots)
            timing[v] = float(np.median([self.round(slots) for _ in range(rounds)]))
        best = min(timing, key=timing.get)
        apply(best)
        return best, timing

    def autotune_launch(self, slots, rounds=3):
        """Time `rounds` rounds with each launch structure and keep the faster (the
        rounds are real rounds: every system advances, identically in either mode)."""
        best = None
        timing = {}
        for mode in ("streams", "buckets"):
            self.launch = mode
            self.round(slots)  # the first round of a mode builds its graphs
            ms = float(np.median([self.round(slots) for _ in range(rounds)]))
            timing[mode] = ms
            if best is None or ms < timing[best]:
                best = mode
        self.launch = best
        if best != "buckets":
            self.free_buckets()
        return best, timing

    def admit(self, req, stream=None):
        t0 = time.perf_counter()
        k, d = build_system(req, self.precision, stream if stream is not None else self.admit_streams[0])
        self.build_s.append(time.perf_counter() - t0)
        nb = estimate_bytes(k.N, req.kind, req.L, k.R)
        return Slot(req=req, kmc=k, drv=d, nbytes=nb, admitted=time.perf_counter())

    def cancel(self, rid):
        """Cancel a request (any thread): dropped if not yet admitted, otherwise
        retired at the next round boundary with status "cancelled"."""
        with self._cv:
            self._cancel.add(int(rid))

    def retire(self, slot, free=True, status=None):
        # the round's work is complete on the main stream: read the system there, not on
        # the admission stream it was built on (which may be building another system)
        _native.lib().kmc_set_stream(slot.kmc._handle, c_void_p(self.main.cuda_stream))
        st = slot.drv.stats()
        slot.proposals_per_step = st[2] / max(st[0], 1)
        if status is None:
            # the system's device error counters (invalid moves, store overflows): a
            # kernel-reported error fails the request instead of passing on a wrong state
            bad, ovf = slot.kmc.error_counts()
            status = "done" if bad == 0 and ovf == 0 else \
                "error: device reported %d invalid moves and %d store overflows" % (bad, ovf)
        self.status[slot.req.rid] = status
        if self.keep_results:
            self.results[slot.req.rid] = {"energy": slot.kmc.energy, "stats": st,
                                          "positions": slot.kmc.state()["positions"], "status": status}
        if free:
            Server.release(slot)
        return st

    @staticmethod
    def release(slot):
        slot.drv.free()
        slot.kmc.free()

    # -- continuous batching over a timed request stream ---------------------
    def serve(self, requests, realtime=True):
        """Serve requests arriving at ``req.arrival`` seconds (relative to the
        start); returns the statistics of the run."""
        import torch
        reqs = sorted(requests, key=lambda r: r.arrival)
        todo = queue.Queue()
        ready = queue.Queue()
        stop = threading.Event()
        errors = []

        graveyard = queue.Queue()
        closed = queue.Queue()  # (rid, status) of requests that end without running

        def bury():
            # memory is released here, off the round loop (freeing may wait for the device)
            while True:
                try:
                    s = graveyard.get_nowait()
                except queue.Empty:
                    return
                self.release(s)
                with self._cv:
                    self.used -= s.nbytes
                    self._cv.notify_all()

        def admission(stream):
            torch.cuda.set_device(torch.cuda.current_device())
            while not stop.is_set():
                bury()
                try:
                    r = todo.get(timeout=0.01)
                except queue.Empty:
                    continue
                need = estimate_bytes(r.n, r.kind, r.L, default_r(r.n))
                with self._cv:
                    cancelled = r.rid in self._cancel
                if cancelled:
                    closed.put((r.rid, "cancelled"))
                    continue
                if need > self.budget:
                    closed.put((r.rid, "rejected: needs %.3g bytes, above the %.3g byte budget" % (need, self.budget)))
                    continue
                with self._cv:
                    while not stop.is_set() and (self.used + need > self.budget or self.reserved >= self.max_active):
                        self._cv.wait(timeout=0.01)
                        self._cv.release()
                        try:
                            bury()
                        finally:
                            self._cv.acquire()
                    self.used += need
                    self.reserved += 1
                try:
                    s = self.admit(r, stream)
                    s.nbytes = need
                    ready.put(s)
                except Exception as e:  # surfaced in the main loop
                    errors.append(e)
                    with self._cv:
                        self.used -= need
                        self.reserved -= 1

        threads = [threading.Thread(target=admission, args=(st,), daemon=True) for st in self.admit_streams]
        t0 = time.perf_counter()
        for th in threads:
            th.start()
        pending = list(reqs)
        round_ms, round_wall, finished = [], [], []
        proposals = 0.0
        busy_t0 = None
        ended = 0  # requests rejected or cancelled before they ran
        ok = False
        try:
            while len(finished) + ended < len(reqs):
                if errors:
                    raise errors[0]
                while True:
                    try:
                        rid, why = closed.get_nowait()
                    except queue.Empty:
                        break
                    self.status[rid] = why
                    ended += 1
                now = time.perf_counter() - t0
                while pending and (not realtime or pending[0].arrival <= now):
                    todo.put(pending.pop(0))
                while True:
                    try:
                        s = ready.get_nowait()
                    except queue.Empty:
                        break
                    with self._cv:
                        self.active.append(s)
                        self.peak_active = max(self.peak_active, len(self.active))
                with self._cv:
                    cut = [s for s in self.active if s.req.rid in self._cancel]
                    if cut:
                        self.active = [s for s in self.active if s.req.rid not in self._cancel]
                        self.reserved -= len(cut)
                        self._cv.notify_all()
                for s in cut:
                    self.retire(s, free=False, status="cancelled")
                    ended += 1
                    graveyard.put(s)
                if not self.active:
                    time.sleep(0.0005)
                    continue
                if busy_t0 is None:
                    busy_t0 = time.perf_counter()
                w0 = time.perf_counter()
                ms = self.round(self.active)
                round_wall.append((time.perf_counter() - w0) * 1e3)
                round_ms.append(ms)
                done = [s for s in self.active if s.done >= s.req.rounds]
                if done:
                    with self._cv:
                        self.active = [s for s in self.active if s.done < s.req.rounds]
                        self.reserved -= len(done)
                        self._cv.notify_all()
                    for s in done:
                        st = self.retire(s, free=False)
                        proposals += st[2]
                        s.finished = time.perf_counter() - t0
                        finished.append(s)
                        graveyard.put(s)
            ok = True
        finally:
            self.free_buckets()
            stop.set()
            for th in threads:
                th.join(timeout=60)
            if not ok:
                # an error ends the run: every system still held is released
                with self._cv:
                    held, self.active = self.active, []
                while True:
                    try:
                        held.append(ready.get_nowait())
                    except queue.Empty:
                        break
                for s in held:
                    try:
                        self.release(s)
                    except Exception:
                        pass
                    self.used -= s.nbytes
                self.reserved = 0
            bury()
        wall = time.perf_counter() - (busy_t0 if busy_t0 else t0)
        lat = np.array([s.finished - s.req.arrival for s in finished])
        rm = np.array(round_ms)
        return {
            "requests": len(finished), "ended_without_running": ended, "rounds": len(rm), "proposals": proposals,
            "proposals_per_s": proposals / wall if wall > 0 else 0.0, "wall_s": wall,
            "round_ms_p50": float(np.percentile(rm, 50)) if len(rm) else 0.0,
            "round_ms_p99": float(np.percentile(rm, 99)) if len(rm) else 0.0,
            "round_wall_ms_p99": float(np.percentile(round_wall, 99)) if round_wall else 0.0,
            "request_latency_s_p50": float(np.percentile(lat, 50)) if len(lat) else 0.0,
            "request_latency_s_p99": float(np.percentile(lat, 99)) if len(lat) else 0.0,
            "build_s_p50": float(np.percentile(self.build_s, 50)) if self.build_s else 0.0,
            "build_s_p99": float(np.percentile(self.build_s, 99)) if self.build_s else 0.0,
            "admission_threads": len(self.admit_streams),
        }


def one_at_a_time(requests, precision="fp64"):
    """Baseline: each request alone, in arrival order, its K steps as one
    captured-graph replay; returns (proposals, device seconds of the steps,
    wall seconds including each system's build)."""
    import torch
    total_p, total_s = 0.0, 0.0
    w0 = time.perf_counter()
    for r in sorted(requests, key=lambda r: r.arrival):
        k, d = build_system(r, precision)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(d.stream)
        _native.check(_native.lib().kmc_driver_launch(d._handle, r.rounds, c_void_p(d.stream.cuda_stream)),
                      "kmc_driver_launch")
        e1.record(d.stream)
        e1.synchronize()
        total_s += e0.elapsed_time(e1) * 1e-3
        total_p += d.stats()[2]
        d.free()
        k.free()
    return total_p, total_s, time.perf_counter() - w0


def poisson_requests(count, rate, seed, n_range=(1000, 262144), k_range=(10, 1000), L=12):
    """Request stream: Poisson arrivals at ``rate``/s, N log-uniform in n_range,
    lattice hopping (pbc) or off-lattice (free_space) with probability 1/2, K
    uniform in k_range."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=count))
    out = []
    for i in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_range[0]), math.log(n_range[1])))))
        lat = rng.uniform() < 0.5
        out.append(Request(rid=i, kind="lattice" if lat else "offlattice", bc="pbc" if lat else "free_space",
                           n=n, rounds=int(rng.integers(k_range[0], k_range[1] + 1)),
                           seed=int(rng.integers(1, 2 ** 31)), arrival=float(t[i]), L=L))
    return out
