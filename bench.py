"""Benchmark: proposal energy differences per second, batched mixed precision against
plain FP64 (the metric's own configuration).

Default workload (--workload batched): 256 independent off-lattice KMC systems, N
log-uniform in [2,000, 131,072] (seed 3), half free space and half pbc, 0.25 charges
per unit volume, R = max(2, ceil(log8(N/8))), L = 12.  One step = one round: every
system advances one KMC step -- every charge proposes a displacement uniform in
[-0.5, 0.5]^3, all differences are computed, one random charge's proposal is accepted
by Metropolis at beta = 1 -- all systems' captured step graphs launched together.
Precision: the mixed mode with FP64 accept contributions (near field and harmonic
evaluation in FP32 / double-FP32; accept increments, the lattice operator, the energy
and the final difference in FP64).

Timed arms and keys:
  value  : device resident rounds (CUDA events per round on the server's main stream);
           the systems' state (~1 GB) is far above the 129 MB L2.
  e2e    : the reference-facing API with host (numpy) buffers, exactly as the
           reference's driver uses it: host proposals, propose_with_dats with host <->
           device copies, host Metropolis, accept -- every system every round.
  fp64   : the same systems on the plain FP64 path; mixed_vs_fp64 the ratio.
  mixed_error : mixed vs FP64 differences and Metropolis decisions on sampled systems.
  config1 / config2 : free space N=1,000 (R=3, L=12, Metropolis, 100 steps) and the
           48^3 pbc lattice-hop workload (27,648 charges, R=5, L=12, rejection-free).
  cpu_baseline / --impl reference : the reference's CPU path as restated by the oracle
           (ppmd/coulomb_kmc cannot be built here), all host threads, on a bounded sample.

Other workloads (--workload; each prints its own JSON line):
  lattice48       : the 48^3 lattice-hop workload as the headline line.
  precision_split : 64^3 lattice, 65,536 charges, R=6, L in {8, 12, 16}: mixed vs
                    FP64 error (max / RMS relative dE, Metropolis agreement) and
                    throughput of both paths.
  batched_streams : the batched workload through per-system graph launches on a pool
                    of worker streams, --systems/--rounds, mixed (double-FP32 accept)
                    vs FP64.
  serving         : Poisson request stream through the continuous-batching
                    server, p50/p99 round latency and throughput, against FP64
                    one system at a time.
  single          : one system (--case) stepped by its driver, for profiler captures.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload ...]
Multi-GPU (torchrun): independent replicas, no collective on the data path; value =
proposals over all ranks / max rank time.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "proposal ΔE/sec, batched mixed-precision vs plain FP64 at ≤1e-6 rel err; p99"
UNIT = "proposals/s"
SIDE, OCC, R, L, BETA = 48, 0.25, 5, 12, 2.0


def workload_config(side, precision):
    n = int(round(OCC * side ** 3))
    return {"workload": f"pbc lattice-hop {side}^3 sites, {n - n % 2} charges (25% occupied, +-1), "
                        f"R={R}, L={L}, rejection-free KMC beta={BETA}, hops to vacant nearest neighbours",
            "boundary_condition": "pbc", "R": R, "L": L, "sites_per_side": side, "precision": precision,
            "l2": "state < L2; a 256 MiB buffer is written between timed steps (L2 flush)"}


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm = [float(r[1]) for r in rows if len(r) >= 9 and r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) >= 9 and r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 9:
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() in ("active", "1"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# ---------------------------------------------------------------------------
def flop_model(kmc, host_sys, lr_nnz_folded):
    """Algorithmic FP64 flops per launch of the step's kernels (add/mul = 1,
    FMA = 2, rsqrt = 1), from this step's
    proposals and cell occupancy."""
    st = kmc.state()
    n = 2 ** (R - 1)
    occ = st["occupancy"].reshape(n, n, n)
    nb = np.zeros_like(occ)  # charges in the 27 neighbour cells of each cell (periodic)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                nb += np.roll(occ, shift=(dz, dy, dx), axis=(0, 1, 2))
    nb = nb.reshape(-1)
    ppos, masks, _ = host_sys.proposals()
    act = masks.reshape(-1) > 0
    pp = ppos.reshape(-1, 3)[act]
    inv_w = n / host_sys.extent
    c = np.minimum(((pp + 0.5 * host_sys.extent) * inv_w).astype(np.int64), n - 1)
    pcell = c[:, 0] + n * (c[:, 1] + n * c[:, 2])
    nh = L * (L + 1) // 2
    far = 12 * nh + 6 * L          # solid-harmonic recurrence + coefficient products
    mpole = 10 * nh + 6 * L        # multipole of one point
    nprop = int(act.sum())
    movers = np.nonzero(masks.sum(axis=1) > 0)[0]
    # the moved pair's self term (27 images) sits in the near-field kernel of the FP64
    # path and, under pbc, in the per-proposal lattice kernel of the mixed path
    self_t = 27 * 11 + 4
    self_in_lr = kmc.precision != "fp64"
    near_new = float(np.sum(11 * nb[pcell])) + nprop * (far + (0 if self_in_lr else self_t))
    near_old = float(np.sum(11 * nb[st["cells"][movers]])) + len(movers) * (far + 2)
    lr_new = nprop * (mpole + 4 * nh + lr_nnz_folded + 6 + (self_t if self_in_lr else 0))  # a, a.(g-h), a^T U a
    # old side with h = A b kept per charge (mixed path): b and b.g per moving charge;
    # the FP64 path recomputes h every step
    lr_old = len(movers) * (mpole + 4 * nh + (0 if kmc.precision != "fp64" else 2 * 2 * lr_nnz_folded + 4 * nh))
    ncell = n ** 3
    p2l = ncell * 54 * (12 * nh + 6 * L + 15)
    return {"near_far_cell": near_new + near_old, "far_lattice": lr_new, "far_lattice_old": lr_old,
            "accept_p2l": p2l, "proposals": nprop, "mean_neighbours": float(np.mean(nb[pcell]))}


# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of the lattice
# workload's kernels from an earlier ncu capture of the same kernels: not measured by this
# program, and stale once a kernel changes; the line says so beside the figure.
NCU_TRAFFIC = {"near_far_cell": 12.921088e6}
NCU_TRAFFIC_MIXED = {"near_far_cell": 12.378624e6, "accept_p2l": 5.167360e6, "far_lattice": 23.233024e6,
                     "far_lattice_old": 1.251584e6}
# warp instructions per launch (smsp__inst_executed.sum) from the same earlier capture, for
# the issue-slot fraction of the mixed kernels (4 warp instructions per SM per clock)
NCU_INST_MIXED = {"near_far_cell": 40.433271e6, "accept_p2l": 23.066700e6, "far_lattice": 11.877886e6,
                  "far_lattice_old": 1.332936e6}
NCU_SOURCE = "earlier ncu capture of the same kernels on this workload, not measured in this run"


def issue_fracs(per_launch_ms, clk):
    """Issue-slot fraction of the mixed kernels: ncu warp instructions per launch over
    the live launch time, against 4 warp instructions per SM per clock at the
    sampled SM clock."""
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = (clk or {}).get("sm_mhz") or 2070.0
    out = {}
    for k, inst in NCU_INST_MIXED.items():
        if k in per_launch_ms:
            out[k] = round(inst / (per_launch_ms[k] * 1e-3) / (sms * 4 * mhz * 1e6), 4)
    return out


def kernel_times(kmc):
    from ctypes import c_int64
    from coulomb_kmc_gb300 import _native
    lib = _native.lib()
    ms = np.zeros(_native.NKERNELS)
    cnt = np.zeros(_native.NKERNELS, np.int64)
    launches = c_int64()
    _native.check(lib.kmc_profile_read(kmc._handle, 1, ms.ctypes.data, cnt.ctypes.data, launches), "profile")
    names = [lib.kmc_kernel_name(i).decode() for i in range(_native.NKERNELS)]
    return {nm: (float(m), int(c)) for nm, m, c in zip(names, ms, cnt)}, launches.value


def fma_peak(fp64=True):
    from ctypes import c_double, byref
    from coulomb_kmc_gb300 import _native
    v = c_double()
    _native.check(_native.lib().kmc_diag_fma_rate(1 if fp64 else 0, 20000 if fp64 else 200000, byref(v)), "diag")
    return v.value


def folded_nnz():
    """Non-zeros of the folded lattice quadratic form (A_re + A_im), as the library builds it."""
    from coulomb_kmc_gb300.lattice import dense_operator
    Rm = dense_operator(L, float(SIDE))
    nh = L * (L + 1) // 2
    Ar = np.zeros((nh, nh))
    Ai = np.zeros((nh, nh))
    for j in range(L):
        for k in range(-j, j + 1):
            for nn in range(L):
                for m in range(-nn, nn + 1):
                    v = Rm[j * j + j + k, nn * nn + nn + m]
                    if v == 0.0:
                        continue
                    hr, hc = j * (j + 1) // 2 + abs(k), nn * (nn + 1) // 2 + abs(m)
                    Ar[hr, hc] += v
                    Ai[hr, hc] += np.sign(k) * np.sign(m) * v
    return int(np.count_nonzero(Ar) + np.count_nonzero(Ai) + 3)


# ---------------------------------------------------------------------------
def cpu_reference(steps, warmup, side, with_gpu_state=None):
    """The reference's CPU path (oracle restatement, OpenMP on all host cores)."""
    from oracle import kmc_oracle as ko
    from coulomb_kmc_gb300.lattice import lattice_operator
    from coulomb_kmc_gb300.workloads import LatticeHopSystem
    hs = LatticeHopSystem(side, OCC, seed=1)
    o = ko.OracleKMC(hs.positions(), hs.charges(), hs.extent, R, L, "pbc", max_move=1.0,
                     lr_operator=lattice_operator(L, hs.extent))
    ncell = (2 ** (R - 1)) ** 3
    lexp = with_gpu_state if with_gpu_state is not None else np.zeros((ncell, 2 * L * L))
    o.initialise(local_expansions=lexp)
    rng = np.random.default_rng(3)
    for _ in range(warmup):
        hs.step(o, rng, BETA)
    t0 = time.perf_counter()
    nprop = 0
    for _ in range(steps):
        hs.step(o, rng, BETA)
        nprop += hs.last_active
    dt = time.perf_counter() - t0
    return nprop / dt, dt, nprop


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    steps = max(1, args.steps)
    v, dt, nprop = cpu_reference(steps, args.warmup, SIDE)
    sample = (f"{steps} KMC steps of the {SIDE}^3 lattice-hop workload ({nprop} proposals), oracle restatement "
              f"of the reference's generated C (ppmd is unavailable), OpenMP {cores} threads; "
              f"initial expansions zero (the operation count does not depend on their values)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(SIDE, "fp64"),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
def make_system(side, rank, precision, local):
    from coulomb_kmc_gb300 import KMCFMM
    from coulomb_kmc_gb300.dats import make_state
    from coulomb_kmc_gb300.driver import KMCDriver
    from coulomb_kmc_gb300.workloads import LatticeHopSystem
    hs = LatticeHopSystem(side, OCC, seed=1 + rank)
    st = make_state(hs.positions(), hs.charges(), hs.extent)
    kmc = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition="pbc", max_move=1.0, precision=precision)
    t0 = time.perf_counter()
    kmc.initialise()
    init_s = time.perf_counter() - t0
    drv = KMCDriver(kmc, "lattice", BETA, seed=1234 + rank, lattice_side=hs.side, lattice_sites=hs.site_of)
    return hs, kmc, drv, init_s


DRIVER_KERNELS_PER_STEP = 2  # proposal generation, rate sums + pick (one launch)


def timed_loop(kmc, drv, steps, warmup, flush, sampler=None, graph=True):
    """Warm up, capture one KMC step (generate, propose, select, accept) as a CUDA
    graph, then time `steps` replays with CUDA events on the driver's stream,
    writing a 256 MiB buffer (L2 flush) before each timed step."""
    import torch
    drv.step(max(warmup, 1))
    torch.cuda.synchronize()
    kmc.check_errors()
    _, l0 = kernel_times(kmc)
    drv.step(1)
    torch.cuda.synchronize()
    _, l1 = kernel_times(kmc)
    per_step_launches = l1 + DRIVER_KERNELS_PER_STEP
    if graph:
        drv.capture()
        drv.launch(2)
    torch.cuda.synchronize()
    kmc.check_errors()
    s0 = drv.stats()
    if sampler:
        sampler.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    with torch.cuda.stream(drv.stream):
        for i in range(steps):
            flush.fill_(float(i))
            ev[i][0].record()
            if graph:
                drv.launch(1, stream=drv.stream)
            else:
                drv.step(1)
            ev[i][1].record()
    torch.cuda.synchronize()
    clk = sampler.stop() if sampler else None
    per_step = np.array([a.elapsed_time(b) for a, b in ev])
    s1 = drv.stats()
    nprop = s1[2] - s0[2]
    kmc.check_errors()
    return per_step, nprop, per_step_launches * steps, clk


def mixed_error_stats(side, local, nsteps=3, seed=11, precision="mixed"):
    """Mixed vs FP64 on identical states: relative dE error (denominator max(|dE|,1))
    and Metropolis-decision agreement (u < exp(-beta dE) with shared u)."""
    from coulomb_kmc_gb300 import KMCFMM
    from coulomb_kmc_gb300.dats import make_state
    from coulomb_kmc_gb300.workloads import LatticeHopSystem
    hs = LatticeHopSystem(side, OCC, seed=seed)
    ks = {}
    for name, prec in (("fp64", "fp64"), ("mixed", precision)):
        st = make_state(hs.positions(), hs.charges(), hs.extent)
        ks[name] = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition="pbc", max_move=1.0, precision=prec)
        ks[name].initialise()
    rng = np.random.default_rng(5)
    errs, agree, total, sel_agree = [], 0, 0, 0
    for _ in range(nsteps):
        ppos, masks, tsite = hs.proposals()
        smc = np.array([6], np.int64)
        sites = np.zeros((hs.n, 1), np.int64)
        d = {}
        for prec, k in ks.items():
            d[prec] = np.zeros((hs.n, 6))
            k.propose_with_dats(smc, sites, ppos, masks, d[prec])
        act = masks > 0
        a, b = d["mixed"][act], d["fp64"][act]
        errs.append(np.abs(a - b) / np.maximum(np.abs(b), 1.0))
        u = rng.uniform(size=a.shape)
        agree += int(np.sum((u < np.exp(-BETA * a)) == (u < np.exp(-BETA * b))))
        total += a.size
        r1 = np.random.default_rng(total)
        r2 = np.random.default_rng(total)
        s1 = hs.select(d["mixed"], masks, r1, BETA)
        s2 = hs.select(d["fp64"], masks, r2, BETA)
        sel_agree += int(s1 == s2)
        pid, h = s2
        mv = ppos[pid, 3 * h:3 * h + 3].copy()
        for k in ks.values():
            k.accept((pid, mv))
        hs.occ[hs.site_of[pid]] = -1
        hs.occ[tsite[pid, h]] = pid
        hs.site_of[pid] = tsite[pid, h]
    e = np.concatenate(errs)
    for k in ks.values():
        k.free()
    return {"max_rel": float(e.max()), "rms_rel": float(np.sqrt(np.mean(e * e))), "proposals": int(e.size),
            "metropolis_decision_agreement": agree / total, "rejection_free_selection_agreement":
                f"{sel_agree}/{nsteps}", "tolerance": 1e-6}


# ---------------------------------------------------------------------------
def bench_precision_split(args):
    """64^3 lattice, 65,536 charges (seed 2), R=6, L in {8, 12, 16}."""
    import torch
    side, r6 = 64, 6
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    out = {}
    for Lx in args.orders:
        res = {}
        for prec in (args.precision, "fp64"):
            from coulomb_kmc_gb300 import KMCFMM
            from coulomb_kmc_gb300.dats import make_state
            from coulomb_kmc_gb300.driver import KMCDriver
            from coulomb_kmc_gb300.workloads import LatticeHopSystem
            hs = LatticeHopSystem(side, OCC, seed=2)
            st = make_state(hs.positions(), hs.charges(), hs.extent)
            k = KMCFMM(st.P, st.Q, st.domain, r=r6, l=Lx, boundary_condition="pbc", max_move=1.0, precision=prec)
            t0 = time.perf_counter()
            k.initialise()
            init_s = time.perf_counter() - t0
            d = KMCDriver(k, "lattice", BETA, seed=99, lattice_side=side, lattice_sites=hs.site_of)
            d.step(1)
            tuned = {str(key): v for key, v in k.autotune(reps=3).items() if v}  # bit-identical shapes, per arm
            ps, npr, _, _ = timed_loop(k, d, args.steps, args.warmup, flush)
            res[prec] = {"value": npr / (ps.sum() * 1e-3), "ms_per_step": float(ps.mean()), "init_s": init_s,
                         "p99_ms": float(np.percentile(ps, 99)), "tuned": tuned}
            d.free()
            k.free()
        err = error_stats(side, r6, Lx, seed=2, nsteps=args.error_steps, precision=args.precision)
        out[f"L{Lx}"] = {"mixed": res[args.precision], "fp64": res["fp64"], "precision": args.precision,
                         "mixed_vs_fp64": res[args.precision]["value"] / res["fp64"]["value"], "error": err}
        print(json.dumps({"L": Lx, **out[f"L{Lx}"]}), file=sys.stderr)
    line = {"metric": METRIC, "workload": "precision_split", "unit": UNIT,
            "config": {"workload": "pbc lattice-hop 64^3 sites, 65,536 charges (seed 2), R=6, L swept",
                       "orders": list(args.orders), "steps": args.steps, "warmup": args.warmup},
            "results": out}
    print(json.dumps(line))


def error_stats(side, r, Lx, seed, nsteps, precision="mixed"):
    """Mixed vs FP64 differences on identical states along an FP64-selected chain."""
    global R, L
    saved = (R, L)
    R, L = r, Lx
    try:
        return mixed_error_stats(side, 0, nsteps=nsteps, seed=seed, precision=precision)
    finally:
        R, L = saved


def bench_batched(args):
    """Independent off-lattice systems advanced together, one step each per round."""
    import torch
    from coulomb_kmc_gb300.serving import Request, Server, Slot, build_system
    rng = np.random.default_rng(3)
    reqs = []
    for i in range(args.systems):
        n = int(round(np.exp(rng.uniform(np.log(2000), np.log(131072)))))
        bc = "free_space" if i % 2 == 0 else "pbc"
        reqs.append(Request(rid=i, kind="offlattice", bc=bc, n=n, rounds=args.rounds,
                            seed=int(rng.integers(1, 2 ** 31)), L=12))
    res = {}
    for prec in ("mixed", "fp64"):
        srv = Server(precision=prec, n_workers=args.workers)
        t0 = time.perf_counter()
        slots = []
        for r in reqs:
            k, d = build_system(r, prec)
            slots.append(Slot(req=r, kmc=k, drv=d, nbytes=0, admitted=0.0))
        build_s = time.perf_counter() - t0
        for _ in range(2):
            srv.round(slots)
        s0 = sum(sl.drv.stats()[2] for sl in slots)
        torch.cuda.synchronize()
        ms = [srv.round(slots) for _ in range(args.rounds)]
        s1 = sum(sl.drv.stats()[2] for sl in slots)
        ms = np.array(ms)
        res[prec] = {"value": (s1 - s0) / (ms.sum() * 1e-3), "round_ms_p50": float(np.percentile(ms, 50)),
                     "round_ms_p99": float(np.percentile(ms, 99)), "build_s": build_s,
                     "proposals_per_round": (s1 - s0) / len(ms)}
        for sl in slots:
            sl.drv.free()
            sl.kmc.free()
        print(json.dumps({prec: res[prec]}), file=sys.stderr)
    line = {"metric": METRIC, "workload": "batched", "unit": UNIT, "value": res["mixed"]["value"],
            "fp64": res["fp64"], "mixed": res["mixed"], "mixed_vs_fp64": res["mixed"]["value"] / res["fp64"]["value"],
            "config": {"workload": f"{args.systems} independent off-lattice systems, N log-uniform in "
                                   f"[2000, 131072] (seed 3), half free_space / half pbc, density 0.25, L=12, "
                                   f"R=max(2, ceil(log8(N/8))), one proposal per charge per round, Metropolis "
                                   f"beta=1", "rounds": args.rounds, "worker_streams": args.workers,
                       "total_charges": int(sum(r.n for r in reqs))}}
    print(json.dumps(line))


def bench_drift(args):
    """Mixed vs FP64 after long chains of accepts on the 48^3 lattice: the mixed
    driver runs and logs its selections, the same moves are accepted on an FP64
    system, then both evaluate the proposals of the common state."""
    import torch
    from coulomb_kmc_gb300 import KMCFMM, _native
    from coulomb_kmc_gb300.dats import make_state
    from coulomb_kmc_gb300.driver import KMCDriver
    from coulomb_kmc_gb300.workloads import LatticeHopSystem
    hs = LatticeHopSystem(SIDE, OCC, seed=1)
    ks = {}
    for prec in ("fp64", "mixed"):
        st = make_state(hs.positions(), hs.charges(), hs.extent)
        ks[prec] = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition="pbc", max_move=1.0, precision=prec)
        ks[prec].initialise()
    if args.fp32_from is not None:
        assert _native.lib().kmc_set_tuning(ks["mixed"]._handle, 6, args.fp32_from) == 0
    chunk = 10000
    drv = KMCDriver(ks["mixed"], "lattice", BETA, seed=77, lattice_side=hs.side, lattice_sites=hs.site_of,
                    log_capacity=chunk)
    out, done = [], 0
    for target in args.accepts:
        while done < target:
            k = min(chunk, target - done)
            drv.step(k)
            torch.cuda.synchronize()
            pid, tgt, _ = drv.log()
            for p_, t_ in zip(pid[-k:], tgt[-k:]):
                if p_ < 0:
                    continue
                ks["fp64"].accept((int(p_), hs.site_pos(int(t_))))
                hs.occ[hs.site_of[p_]] = -1
                hs.occ[t_] = p_
                hs.site_of[p_] = t_
            done += k
        assert np.array_equal(drv.sites(), hs.site_of)
        ppos, masks, _ = hs.proposals()
        smc = np.array([6], np.int64)
        sites = np.zeros((hs.n, 1), np.int64)
        d = {}
        for prec, kk in ks.items():
            d[prec] = np.zeros((hs.n, 6))
            kk.propose_with_dats(smc, sites, ppos, masks, d[prec])
        act = masks > 0
        e = np.abs(d["mixed"][act] - d["fp64"][act]) / np.maximum(np.abs(d["fp64"][act]), 1.0)
        le = np.max(np.abs(ks["mixed"].state()["local_expansions"] - ks["fp64"].state()["local_expansions"]))
        out.append({"accepts": done, "max_rel": float(e.max()), "rms_rel": float(np.sqrt(np.mean(e * e))),
                    "energy_rel": abs(ks["mixed"].energy - ks["fp64"].energy) / abs(ks["fp64"].energy),
                    "expansions_max_abs_diff": float(le)})
    drv.free()
    for kk in ks.values():
        kk.free()
    print(json.dumps({"workload": "drift", "config": {"workload": "pbc lattice-hop 48^3 sites, mixed driver "
                      "selections replayed on FP64", "fp32_from": args.fp32_from}, "results": out}))


def bench_serving(args):
    """Poisson request stream through the continuous-batching server."""
    from coulomb_kmc_gb300.serving import Server, one_at_a_time, poisson_requests
    out = {}
    for rate in args.rates:
        reqs = poisson_requests(args.requests, rate, seed=4, n_range=(1000, args.max_n),
                                k_range=(10, args.max_k))
        srv = Server(precision=args.precision, hbm_budget=150e9, max_active=args.max_active,
                     n_workers=args.workers)
        st = srv.serve(reqs, realtime=True)
        st["peak_active"] = srv.peak_active
        out[str(rate)] = st
        print(json.dumps({"rate": rate, **st}), file=sys.stderr)
    reqs = poisson_requests(args.requests, args.rates[0], seed=4, n_range=(1000, args.max_n),
                            k_range=(10, args.max_k))
    p64, s64, w64 = one_at_a_time(reqs, "fp64")
    base = p64 / s64
    line = {"metric": METRIC, "workload": "serving", "unit": UNIT,
            "value": max(v["proposals_per_s"] for v in out.values()),
            "fp64_one_at_a_time": base,
            "fp64_one_at_a_time_with_builds": p64 / w64,
            "mixed_vs_fp64": max(v["proposals_per_s"] for v in out.values()) / base,
            "mixed_vs_fp64_with_builds": max(v["proposals_per_s"] for v in out.values()) / (p64 / w64),
            "per_rate": out, "precision": args.precision,
            "config": {"workload": f"{args.requests} requests (seed 4), Poisson arrivals, N log-uniform in "
                                   f"[1000, {args.max_n}], lattice-hop pbc or off-lattice free_space with "
                                   f"probability 1/2, L=12, K uniform in [10, {args.max_k}], 150 GB budget",
                       "rates_per_s": list(args.rates), "max_active": args.max_active,
                       "worker_streams": args.workers}}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# Batched replicas (the metric's own configuration): 256 independent off-lattice
# systems, N log-uniform in [2,000, 131,072] (seed 3), half free space and half
# pbc, density 0.25, R = max(2, ceil(log8(N/8))), L = 12; one proposal per charge
# per round (uniform displacement in [-0.5, 0.5]^3, re-drawn inside the box) and a
# Metropolis accept (beta = 1) of one random charge's proposal, every system every
# round.
# ---------------------------------------------------------------------------
C4_BETA, C4_STEP = 1.0, 0.5


def config4_requests(n_systems, seed=3):
    from coulomb_kmc_gb300.serving import Request
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(n_systems):
        n = int(round(np.exp(rng.uniform(np.log(2000), np.log(131072)))))
        bc = "free_space" if i % 2 == 0 else "pbc"
        reqs.append(Request(rid=i, kind="offlattice", bc=bc, n=n, rounds=0, seed=int(rng.integers(1, 2 ** 31)),
                            L=12, beta=C4_BETA))
    return reqs


def config4_workload(n_systems):
    return (f"{n_systems} independent off-lattice systems, N log-uniform in [2000, 131072] (seed 3), half "
            f"free_space / half pbc, density 0.25, R=max(2, ceil(log8(N/8))), L=12, one proposal per charge per "
            f"round (uniform in [-0.5, 0.5]^3), Metropolis beta=1 on one random charge per system per round")


def build_kmcs(reqs, precision, threads=4):
    """Create and initialise every system (no driver yet), on `threads` host threads,
    each with its own CUDA stream.  Returns [(KMCFMM, extent)] in request order."""
    import torch
    from concurrent.futures import ThreadPoolExecutor
    from coulomb_kmc_gb300 import KMCFMM, _native
    from coulomb_kmc_gb300.dats import make_state
    from coulomb_kmc_gb300.serving import default_r, system_inputs
    streams = [_native.DedicatedStream() for _ in range(threads)]
    dev = torch.cuda.current_device()

    def one(i):
        r = reqs[i]
        torch.cuda.set_device(dev)
        st_ = streams[i % threads]
        with torch.cuda.stream(st_.stream):
            pos, q, E, _, _ = system_inputs(r)
            st = make_state(pos, q, E)
            k = KMCFMM(st.P, st.Q, st.domain, r=default_r(len(q)), l=r.L, boundary_condition=r.bc,
                       max_move=C4_STEP, precision=precision)
            k.initialise()
            st_.stream.synchronize()
        return k, E

    with ThreadPoolExecutor(threads) as ex:
        out = list(ex.map(one, range(len(reqs))))
    torch.cuda.synchronize()
    for k, _ in out:
        k._set_stream()  # off the build streams, which end here
    for st_ in streams:
        st_.close()
    return out


def combine_ranks(t_ms, nprop, device):
    """Across the replicas (one per rank, no exchange in the timed work): the slowest
    rank's timed milliseconds and the proposals of all ranks, so that the whole-job value
    is all proposals over the slowest rank's time."""
    import torch
    import torch.distributed as dist
    tot = torch.tensor([t_ms, float(nprop)], dtype=torch.float64, device=device)
    tmax = tot[0:1].clone()
    nsum = tot[1:2].clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(nsum, op=dist.ReduceOp.SUM)
    return float(tmax[0]), float(nsum[0])


def apply_tune(k, args):
    """Launch-shape keys given on the command line (--tune KEY=VALUE ...), set on a system
    before its steps are captured."""
    for kv in args.tune:
        key, val = kv.split("=")
        k.set_tuning(int(key), int(val))


def offlattice_proposals(pos, E, rng, out=None):
    """One displacement per charge, uniform in [-step, step]^3, re-drawn (the same draws
    in the same order) for the rows that left the box; only those rows are re-checked.
    `out`: an (N, 3) array to write into."""
    h = 0.5 * E
    prop = np.add(pos, rng.uniform(-C4_STEP, C4_STEP, size=pos.shape), out=out)
    bad = np.flatnonzero(np.any(np.abs(prop) > h, axis=1))
    while bad.size:
        prop[bad] = pos[bad] + rng.uniform(-C4_STEP, C4_STEP, size=(bad.size, 3))
        bad = bad[np.any(np.abs(prop[bad]) > h, axis=1)]
    return prop


class HostRound:
    """One Metropolis round of every system through the reference-facing API with host
    (numpy) buffers, as a caller serving many systems would run it: worker threads,
    each with its own CUDA stream and random generator, take the systems in turn;
    per system, proposals generated on the host into the library's pinned arrays,
    propose_with_dats (host -> device copies of the proposals, device -> host copy
    of the differences; it returns when they are on the host), Metropolis on the
    host, accept.  The library calls and numpy's bulk work release the GIL, so the
    systems' host work and device work overlap across workers.  Buffers per system
    are allocated once."""

    def __init__(self, kmcs, seed=7, workers=16):
        import torch
        from concurrent.futures import ThreadPoolExecutor
        from coulomb_kmc_gb300._native import DedicatedStream
        self.kmcs = kmcs
        self.workers = max(1, min(workers, len(kmcs)))
        self.rngs = [np.random.default_rng(sq) for sq in np.random.SeedSequence(seed).spawn(self.workers)]
        self.streams = [DedicatedStream() for _ in range(self.workers)]
        self.pool = ThreadPoolExecutor(self.workers)
        self.device = torch.cuda.current_device()
        self.buf = []
        for k, E in kmcs:
            # the library's pinned host arrays, filled in place (no staging copies)
            hb = k.host_buffers(1)
            hb["current_sites"][:] = 0
            hb["prop_masks"][:] = 1
            self.buf.append((np.array([1], np.int64), hb["current_sites"], hb["prop_masks"],
                             hb["prop_energy_diffs"], hb["prop_positions"]))
        self.proposals = 0
        self.h2d = 0
        self.d2h = 0
        self.round_no = 0
        # thread-seconds summed over the workers (they overlap in time)
        self.phase = {"host_proposals": 0.0, "propose_with_dats": 0.0, "select_accept": 0.0}

    def close(self):
        """Free the page-locked arrays, bind every system back to the caller's stream, then
        end the workers' streams."""
        import gc
        import torch
        self.pool.shutdown()
        self.buf = []
        for k, _ in self.kmcs:
            k.release_host_buffers()
        gc.collect()
        torch.cuda.synchronize()
        for k, _ in self.kmcs:
            k._set_stream()
        for st in self.streams:
            st.close()

    def _work(self, w):
        import torch
        from coulomb_kmc_gb300.workloads import uniform_displacements
        torch.cuda.set_device(self.device)
        pc = time.perf_counter
        rng = self.rngs[w]
        ph = {key: 0.0 for key in self.phase}
        nprop = h2d = d2h = 0
        with torch.cuda.stream(self.streams[w].stream):
            for j in range(w, len(self.kmcs), self.workers):
                (k, E), (smc, sites, masks, diffs, prop) = self.kmcs[j], self.buf[j]
                t0 = pc()
                pos = k.positions if isinstance(k.positions, np.ndarray) else np.asarray(k._positions_host())
                # native generator (the GIL released): the workers draw their systems' proposals at once
                uniform_displacements(np.asarray(pos, dtype=np.float64).reshape(-1, 3), E, C4_STEP, seed=1000 + j,
                                      round_=self.round_no, out=prop, threads=1)
                t1 = pc()
                k.propose_with_dats(smc, sites, prop, masks, diffs)
                t2 = pc()
                pid = int(rng.integers(0, k.N))
                if rng.uniform() < np.exp(-C4_BETA * diffs[pid, 0]):
                    k.accept((pid, prop[pid].copy()))
                t3 = pc()
                ph["host_proposals"] += t1 - t0
                ph["propose_with_dats"] += t2 - t1
                ph["select_accept"] += t3 - t2
                nprop += k.N
                h2d += smc.nbytes + sites.nbytes + prop.nbytes + masks.nbytes + diffs.nbytes
                d2h += diffs.nbytes + 16
            self.streams[w].stream.synchronize()  # the last accept
        return ph, nprop, h2d, d2h

    def run(self):
        self.round_no += 1
        for ph, nprop, h2d, d2h in self.pool.map(self._work, range(self.workers)):
            for key in ph:
                self.phase[key] += ph[key]
            self.proposals += nprop
            self.h2d += h2d
            self.d2h += d2h


def make_slots(reqs, kmcs, autotune=False):
    """A device driver per system; with `autotune`, the launch shapes of each size
    bucket (depth, order, boundary condition) are tuned on its largest system
    (kmc_autotune: only variants that leave every result bit-identical) and applied
    to all its systems; then every step is captured.  Returns (slots, choices)."""
    import torch
    from coulomb_kmc_gb300.driver import KMCDriver
    from coulomb_kmc_gb300.serving import Server, Slot
    slots = []
    for r, (k, E) in zip(reqs, kmcs):
        d = KMCDriver(k, "offlattice", C4_BETA, seed=r.seed, step=C4_STEP)
        slots.append(Slot(req=r, kmc=k, drv=d, nbytes=0, admitted=0.0))
    choices = {}
    if autotune:
        buckets = {}
        for sl in slots:
            buckets.setdefault(Server.bucket_key(sl), []).append(sl)
        for key, members in sorted(buckets.items()):
            big = max(members, key=lambda sl: sl.kmc.N)
            big.drv.step(1)  # a proposal set-up for the lattice kernels to run on
            torch.cuda.synchronize()
            with torch.cuda.stream(big.drv.stream):
                tuned = big.kmc.autotune(reps=5)
            torch.cuda.synchronize()
            big.kmc._set_stream()
            picked = {k: v for k, v in tuned.items() if v}
            for sl in members:
                for k, v in picked.items():
                    sl.kmc.set_tuning(k, v)
            choices["R=%d L=%d %s %s" % key] = picked
    for sl in slots:
        sl.drv.capture()
    torch.cuda.synchronize()
    return slots, choices


def timed_rounds(srv, slots, steps, warmup, sampler=None):
    """W untimed rounds, then exactly `steps` rounds, each timed with CUDA events on the
    server's main stream (every system one KMC step per round)."""
    import torch
    for _ in range(warmup):
        srv.round(slots)
    torch.cuda.synchronize()
    p0 = sum(sl.drv.stats()[2] for sl in slots)
    if sampler:
        sampler.start()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed_rounds")  # lets a profiler take exactly these launches
    ms = np.array([srv.round(slots) for _ in range(steps)])
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    clk = sampler.stop() if sampler else None
    p1 = sum(sl.drv.stats()[2] for sl in slots)
    return ms, p1 - p0, clk


def free_slots(slots):
    for sl in slots:
        sl.drv.free()
        sl.kmc.free()


def config4_error_stats(reqs, nsys=6, rounds=2, seed=11):
    """Mixed (FP64 accept) vs plain FP64 on identical states for a sample of the
    systems (smallest and largest of each boundary condition, two in between): relative
    difference error (denominator max(|dE|, 1)) and Metropolis-decision agreement with
    shared uniforms; both take the FP64 decision so the states stay identical."""
    idx = sorted(range(len(reqs)), key=lambda i: reqs[i].n)
    fs = [i for i in idx if reqs[i].bc == "free_space"]
    pb = [i for i in idx if reqs[i].bc == "pbc"]
    pick = sorted(set([fs[0], fs[-1], pb[0], pb[-1], fs[len(fs) // 2], pb[len(pb) // 2]]))[:nsys]
    sub = [reqs[i] for i in pick]
    mx = build_kmcs(sub, "mixed_fp64_accept", threads=2)
    f64 = build_kmcs(sub, "fp64", threads=2)
    rng = np.random.default_rng(seed)
    errs, agree, total = [], 0, 0
    per = {}
    for (km, E), (kf, _), r in zip(mx, f64, sub):
        e_sys = []
        for _ in range(rounds):
            pos = np.asarray(kf._positions_host(), dtype=np.float64).reshape(-1, 3)
            prop = offlattice_proposals(pos, E, rng)
            n = kf.N
            d = {}
            for name, k in (("m", km), ("f", kf)):
                d[name] = np.zeros((n, 1))
                k.propose_with_dats(np.array([1], np.int64), np.zeros((n, 1), np.int64), prop,
                                    np.ones((n, 1), np.int64), d[name])
            e = np.abs(d["m"] - d["f"]) / np.maximum(np.abs(d["f"]), 1.0)
            e_sys.append(e.ravel())
            u = rng.uniform(size=n)
            agree += int(np.sum((u < np.exp(-C4_BETA * d["m"][:, 0])) == (u < np.exp(-C4_BETA * d["f"][:, 0]))))
            total += n
            pid = int(rng.integers(0, n))
            if u[pid] < np.exp(-C4_BETA * d["f"][pid, 0]):
                for k in (km, kf):
                    k.accept((pid, prop[pid].copy()))
        es = np.concatenate(e_sys)
        errs.append(es)
        per[f"{r.bc} N={r.n}"] = {"max_rel": float(es.max()), "rms_rel": float(np.sqrt(np.mean(es * es)))}
        km.free()
        kf.free()
    e = np.concatenate(errs)
    return {"max_rel": float(e.max()), "rms_rel": float(np.sqrt(np.mean(e * e))), "proposals": int(e.size),
            "metropolis_decision_agreement": agree / total, "tolerance": 1e-6, "per_system": per,
            "sample": f"{len(sub)} systems x {rounds} rounds (smallest, middle and largest of each boundary condition)"}


def launches_per_step(slots):
    """Kernel launches of one step of each system (the library's own launch counter over
    one eager step, plus the driver's generation and selection kernels)."""
    import torch
    total = 0
    for sl in slots:
        kernel_times(sl.kmc)  # reads and resets the handle's launch counter
        sl.drv.step(1)
        torch.cuda.synchronize()
        _, l1 = kernel_times(sl.kmc)
        total += l1 + DRIVER_KERNELS_PER_STEP
    return total


def offlattice_flop_model(kmc, L_):
    """Algorithmic flops of one launch of the mixed near-field kernel (near_far_cell) on an
    off-lattice system: every charge's proposal (new side) and old position (old side)
    against its 27 neighbour cells, plus the cell-expansion evaluation (counting
    convention: add/mul 1, FMA 2, rsqrt 1)."""
    st = kmc.state()
    n = round(len(st["occupancy"]) ** (1 / 3))
    occ = st["occupancy"].reshape(n, n, n)
    nb = np.zeros_like(occ)
    from coulomb_kmc_gb300.common import BCType
    per = kmc.boundary_condition != BCType.FREE_SPACE
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                sh = np.roll(occ, shift=(dz, dy, dx), axis=(0, 1, 2))
                if not per:
                    if dz:
                        sh[0 if dz > 0 else -1, :, :] = 0
                    if dy:
                        sh[:, 0 if dy > 0 else -1, :] = 0
                    if dx:
                        sh[:, :, 0 if dx > 0 else -1] = 0
                nb += sh
    nb = nb.reshape(-1)
    nh = L_ * (L_ + 1) // 2
    far = 12 * nh + 6 * L_
    cells = st["cells"]
    # a proposal lands in its own cell or a neighbour: the old cell's neighbour count
    # stands for both sides (displacements are at most 0.5 of a ~5-wide cell)
    pair = float(np.sum(11 * nb[cells]))
    return 2 * pair + 2 * len(cells) * far, float(np.mean(nb[cells]))


def offlattice_flops_executed(kmc, L_):
    """The part of offlattice_flop_model the kernel executes with the moving charges'
    near-field potentials kept between moves: the new side's pair terms, both sides'
    cell-expansion evaluations."""
    total, mnb = offlattice_flop_model(kmc, L_)
    nh = L_ * (L_ + 1) // 2
    far = 12 * nh + 6 * L_
    n = kmc.N
    return 0.5 * (total - 2 * n * far) + 2 * n * far


def bench_config4(args, rank, world, local):
    """The headline: batched replicas of the metric's configuration (see config4_requests)."""
    import torch
    from coulomb_kmc_gb300 import _native
    from coulomb_kmc_gb300.serving import Server
    reqs = config4_requests(args.systems)
    prec = args.precision
    t0 = time.perf_counter()
    kmcs = build_kmcs(reqs, prec, threads=args.build_threads)
    for k, _ in kmcs:
        apply_tune(k, args)
    build_s = time.perf_counter() - t0
    extras = {}
    # e2e: the reference-facing API with host buffers (before the device drivers exist)
    if not args.no_extras:
        hr = HostRound(kmcs)
        hr.run()
        torch.cuda.synchronize()
        p0, b0, c0 = hr.proposals, hr.h2d, hr.d2h
        ph0 = dict(hr.phase)
        t1 = time.perf_counter()
        for _ in range(args.e2e_steps):
            hr.run()
        torch.cuda.synchronize()
        e2e_dt = time.perf_counter() - t1
        nr = max(args.e2e_steps, 1)
        hr.close()
        extras["e2e"] = {"value": (hr.proposals - p0) / e2e_dt, "unit": UNIT,
                         "h2d_bytes_per_step": int((hr.h2d - b0) / nr), "d2h_bytes_per_step": int((hr.d2h - c0) / nr),
                         "steps": args.e2e_steps,
                         "round_s": e2e_dt / nr,
                         "phases_thread_s_per_round": {k: (hr.phase[k] - ph0[k]) / nr for k in hr.phase},
                         "workers": hr.workers,
                         "path": "KMCFMM.propose_with_dats with numpy buffers (pinned staging, H2D of every "
                                 "proposal array, D2H of the differences) + host Metropolis + KMCFMM.accept, "
                                 "every system every round, systems taken in turn by 16 worker threads (own "
                                 "CUDA stream and generator each)"}
    slots, tuned = make_slots(reqs, kmcs, autotune=True)
    launches = launches_per_step(slots) if not args.no_extras else None
    srv = Server(precision=prec, n_workers=args.workers)
    # the round's launch structure (per-system graphs on worker streams, or one graph per
    # size bucket): both timed over a few rounds (untimed warm-up rounds), the faster kept
    # blocks per cell of the near field repeat each cell's set-up per block: tuned on whole
    # rounds (bit-identical candidates; the rounds are untimed warm-up rounds)
    split, split_ms = srv.autotune_key(slots, _native.KMC_TUNE_NEAR_SPLIT, (1, 2), rounds=2)
    # the near field's scheduling priority (default, or the device's highest)
    prio, prio_ms = srv.autotune_key(slots, _native.KMC_TUNE_NEAR_PRIORITY, (0, 1), rounds=2)
    # so are the FP64 accept kernel's cells per block and residency (blocks per SM), which
    # decide how much of each SM the other systems' near-field kernels find free ({}: each
    # size bucket's own kmc_autotune choice, no residency limit)
    k_c, k_s = _native.KMC_TUNE_P2L64_CELLS, _native.KMC_TUNE_P2L64_PER_SM
    combos = [{}, {k_s: 1}, {k_c: 2, k_s: 2}, {k_c: 2, k_s: 3}]
    best, combo_ms = srv.autotune_keys(slots, combos, rounds=2)
    per_sm = {str(k): v for k, v in combos[best].items()}
    per_sm_ms = {json.dumps({str(k): v for k, v in c.items()}): t for c, t in zip(combos, combo_ms)}
    mode, mode_ms = srv.autotune_launch(slots, rounds=3)
    extras["autotune"] = {"kernel_launch_shapes": tuned, "near_blocks_per_cell": split,
                          "round_ms_by_near_blocks_per_cell": split_ms,
                          "near_priority": prio, "round_ms_by_near_priority": prio_ms,
                          "fp64_accept_shape": per_sm, "round_ms_by_fp64_accept_shape": per_sm_ms,
                          "round_launch": mode, "round_ms_by_launch": mode_ms}
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    ms, nprop, clk = timed_rounds(srv, slots, args.steps, args.warmup, ClockSampler(local))
    t_ms = float(ms.sum())
    value = nprop / (t_ms * 1e-3)
    print(json.dumps({"stage": "timed rounds", "value": value, "round_ms_p50": float(np.percentile(ms, 50)),
                      "round_ms_p99": float(np.percentile(ms, 99)), "build_s": build_s,
                      "e2e": extras.get("e2e", {}).get("value")}), file=sys.stderr, flush=True)
    if world > 1:
        t_ms, nprop = combine_ranks(t_ms, nprop, "cuda")
        value = nprop / (t_ms * 1e-3)
    if not args.no_extras:
        # per-kernel times of the largest system of each boundary condition (separate pass)
        big = {}
        for bc in ("pbc", "free_space"):
            i = max((j for j in range(len(reqs)) if reqs[j].bc == bc), key=lambda j: reqs[j].n)
            sl = slots[i]
            _native.lib().kmc_profile(sl.kmc._handle, 1)
            kernel_times(sl.kmc)
            sl.drv.step(5)
            torch.cuda.synchronize()
            kt, _ = kernel_times(sl.kmc)
            _native.lib().kmc_profile(sl.kmc._handle, 0)
            per_launch = {k: v[0] / max(v[1], 1) for k, v in kt.items() if v[1] > 0}
            fl, mnb = offlattice_flop_model(sl.kmc, 12)
            big[bc] = {"n": reqs[i].n, "per_kernel_ms": {k: round(v, 5) for k, v in per_launch.items()},
                       "near_flops": fl, "near_flops_executed": offlattice_flops_executed(sl.kmc, 12),
                       "mean_neighbours": mnb}
        srv.free_buckets()
        free_slots(slots)
        peak64, peak32 = fma_peak(True), fma_peak(False)
        b = big["pbc"]
        nf_ms = b["per_kernel_ms"].get("near_far_cell")
        ach = b["near_flops"] / (nf_ms * 1e-3) / 1e12 if nf_ms else None
        extras["roofline"] = {
            "bound": "fp32", "kernel": "near_far_cell", "achieved": ach, "peak": peak32, "unit": "TFLOP/s",
            "frac": ach / peak32 if ach else None, "traffic": None,
            "kernel_workload": f"largest pbc system (N={b['n']}), 5 steps, CUDA events per launch",
            "peak_source": "measured in this run with kmc_diag_fma_rate (FMA issue rate of the FP32 pipe); "
                           "MEASURED_PEAKS.json holds HBM and bf16 only, and the kernel is arithmetic bound",
            "peaks_measured": {"fp64_tflops": peak64, "fp32_tflops": peak32},
            "flops_convention": "algorithmic flops of the FP64 algorithm (add/mul 1, FMA 2, rsqrt 1); the mixed "
                                "kernel spends several FP32 instructions per algorithmic flop",
            "flops_per_launch": b["near_flops"], "mean_neighbours_per_proposal": b["mean_neighbours"],
            "flops_executed_per_launch": b["near_flops_executed"],
            "frac_executed": (b["near_flops_executed"] / (nf_ms * 1e-3) / 1e12 / peak32) if nf_ms else None,
            "executed_note": "the algorithmic count takes every moving charge's old-side pair terms; "
                             "with the near-field potentials kept between moves the kernel executes the new "
                             "side's pair terms and both sides' cell-expansion evaluations only",
            "per_kernel_ms_largest": {k: v["per_kernel_ms"] for k, v in big.items()},
            "traffic_note": "not captured in this run; the ncu captures summarised with the profiles give the "
                            "DRAM bytes per launch"}
        # the plain FP64 path on the same systems
        k64 = build_kmcs(reqs, "fp64", threads=args.build_threads)
        s64, _ = make_slots(reqs, k64)
        srv64 = Server(precision="fp64", n_workers=args.workers)
        mode64, _ = srv64.autotune_launch(s64, rounds=1)
        ms64, np64, _ = timed_rounds(srv64, s64, max(2, args.fp64_rounds), 0)
        srv64.free_buckets()
        free_slots(s64)
        extras["fp64"] = {"value": np64 / (ms64.sum() * 1e-3), "round_ms_p50": float(np.percentile(ms64, 50)),
                          "round_ms_p99": float(np.percentile(ms64, 99)), "rounds": len(ms64),
                          "round_launch": mode64}
        extras["mixed_vs_fp64"] = value / extras["fp64"]["value"]
        print(json.dumps({"stage": "fp64", **extras["fp64"]}), file=sys.stderr, flush=True)
        extras["mixed_error"] = config4_error_stats(reqs)
        if rank == 0:
            cores = os.cpu_count()
            v, dt, npc, smp = cpu_config4(reqs, args.cpu_rounds, 1)
            extras["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": smp}
        extras["config1"] = bench_config1(args)
        extras["config2"] = bench_config2_extra(args, rank, local)
    else:
        srv.free_buckets()
        free_slots(slots)
    return value, t_ms, nprop, ms, clk, launches, build_s, extras


def cpu_config4(reqs, rounds, warmup, sample=None):
    """The reference's CPU path (oracle restatement, OpenMP on all host cores) on a
    bounded sample of the batched workload: `rounds` Metropolis rounds of each sampled
    system (one proposal per charge, one accept).  Initial expansions zero: the
    operation count does not depend on their values."""
    from oracle import kmc_oracle as ko
    from coulomb_kmc_gb300.lattice import lattice_operator
    from coulomb_kmc_gb300.serving import default_r, system_inputs
    from coulomb_kmc_gb300.workloads import uniform_displacements
    cores = os.cpu_count() or 1
    if sample is None:
        # the systems at the 30th and 70th percentile of N of each boundary condition
        sample = []
        for bc in ("free_space", "pbc"):
            idx = sorted((i for i in range(len(reqs)) if reqs[i].bc == bc), key=lambda i: reqs[i].n)
            sample += [idx[(3 * len(idx)) // 10], idx[(7 * len(idx)) // 10]]
    systems = []
    for i in sample:
        r = reqs[i]
        pos, q, E, _, _ = system_inputs(r)
        R_ = default_r(len(q))
        o = ko.OracleKMC(pos.copy(), q, E, R_, r.L, r.bc, max_move=C4_STEP,
                         lr_operator=lattice_operator(r.L, E) if r.bc == "pbc" else None)
        o.initialise(local_expansions=np.zeros(((2 ** (R_ - 1)) ** 3, 2 * r.L * r.L)))
        systems.append((o, E))
    rng = np.random.default_rng(5)

    rnd = [0]

    def one_round():
        n_tot = 0
        rnd[0] += 1
        for si, (o, E) in enumerate(systems):
            n = o.N
            prop = uniform_displacements(o.positions, E, C4_STEP, seed=1000 + si, round_=rnd[0], threads=cores)
            d = np.zeros((n, 1))
            o.propose_with_dats(np.array([1], np.int64), np.zeros((n, 1), np.int64), prop,
                                np.ones((n, 1), np.int64), d)
            pid = int(rng.integers(0, n))
            if rng.uniform() < np.exp(-C4_BETA * d[pid, 0]):
                o.accept((pid, prop[pid].copy()))
            n_tot += n
        return n_tot

    for _ in range(warmup):
        one_round()
    t0 = time.perf_counter()
    nprop = sum(one_round() for _ in range(rounds))
    dt = time.perf_counter() - t0
    desc = (f"{rounds} Metropolis rounds of {len(sample)} of the {len(reqs)} systems (N = "
            f"{', '.join(str(reqs[i].n) + ' ' + reqs[i].bc for i in sample)}; {nprop} proposals) on the oracle "
            f"(restated reference CPU path, OpenMP {os.cpu_count()} threads; initial expansions zero, which does "
            f"not change the operation count)")
    return nprop / dt, dt, nprop, desc


def bench_config1(args):
    """Plain FP64 free space: N=1,000 charges in a box of edge 12 (seed 0), R=3, L=12;
    every charge proposes one move per step (uniform in [-0.5, 0.5]^3), one random
    charge's move accepted by Metropolis at beta = 1; 100 steps, device driver with a
    captured step graph.  Also the mixed mode with FP64 accept contributions."""
    import torch
    from coulomb_kmc_gb300 import KMCFMM
    from coulomb_kmc_gb300.dats import make_state
    from coulomb_kmc_gb300.driver import KMCDriver
    from coulomb_kmc_gb300.workloads import OffLatticeSystem
    out = {}
    for prec in ("fp64", "mixed_fp64_accept"):
        hs = OffLatticeSystem(1000, 12.0, seed=0, step=0.5)
        st = make_state(hs.positions(), hs.charges(), 12.0)
        k = KMCFMM(st.P, st.Q, st.domain, r=3, l=12, boundary_condition="free_space", max_move=0.5,
                   precision=prec)
        k.initialise()
        d = KMCDriver(k, "offlattice", 1.0, seed=1, step=0.5)
        d.step(3)
        d.capture()
        torch.cuda.synchronize()
        s0 = d.stats()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(d.stream)
        d.launch(100, stream=d.stream)
        e1.record(d.stream)
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        s1 = d.stats()
        out[prec] = {"value": (s1[2] - s0[2]) / (ms * 1e-3), "ms_per_step": ms / 100, "steps": 100,
                     "accepted": s1[1] - s0[1]}
        d.free()
        k.free()
    out["workload"] = ("free_space N=1000, box 12, seed 0, R=3, L=12, one proposal per charge per step, "
                       "Metropolis beta=1, 100 steps")
    return out


def bench_config2_extra(args, rank, local):
    """pbc lattice hopping on 48^3 sites (27,648 charges, R=5, L=12, rejection-free,
    beta=2): the mixed mode with FP64 accept contributions, plain FP64 and the mixed mode
    with double-FP32 accept contributions; errors against FP64."""
    import torch
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    out = {}
    for prec, nsteps in (("mixed_fp64_accept", args.steps), ("fp64", max(5, args.steps // 3)),
                         ("mixed", args.steps)):
        _, k, d, _ = make_system(SIDE, rank, prec, local)
        # launch shapes tuned on the handle (bit-identical variants), for every arm
        d.step(1)
        tuned = {str(key): v for key, v in k.autotune(reps=5).items() if v}
        ps, npr, _, _ = timed_loop(k, d, nsteps, 3, flush)
        out[prec] = {"value": npr / (ps.sum() * 1e-3), "ms_per_step": float(ps.mean()),
                     "p50_ms": float(np.percentile(ps, 50)), "p99_ms": float(np.percentile(ps, 99)),
                     "steps": len(ps), "tuned": tuned}
        d.free()
        k.free()
    out["mixed_fp64_accept"]["vs_fp64"] = out["mixed_fp64_accept"]["value"] / out["fp64"]["value"]
    out["mixed"]["vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["error_mixed_fp64_accept"] = mixed_error_stats(SIDE, local, precision="mixed_fp64_accept")
    out["error_mixed"] = mixed_error_stats(SIDE, local, precision="mixed")
    out["workload"] = workload_config(SIDE, "mixed_fp64_accept")["workload"]
    return out


def bench_single(args):
    """One system of a named case stepped by its device driver, for profiler captures of
    single kernels (small enough for a full metric set): 'c4pbc' / 'c4free', the largest
    pbc / free-space system of the batched workload; 'lattice48', the 48^3 lattice-hop
    workload.  Prints the mean step time; the steps sit in an NVTX range 'steps'."""
    import torch
    from coulomb_kmc_gb300.driver import KMCDriver
    if args.case in ("c4pbc", "c4free"):
        reqs = config4_requests(args.systems)
        bc = "pbc" if args.case == "c4pbc" else "free_space"
        big = max((r for r in reqs if r.bc == bc), key=lambda r: r.n)
        (k, E), = build_kmcs([big], args.precision, threads=1)
        apply_tune(k, args)
        d = KMCDriver(k, "offlattice", C4_BETA, seed=big.seed, step=C4_STEP)
        what = f"{bc} off-lattice N={big.n}"
    else:
        _, k, d, _ = make_system(SIDE, 0, args.precision, 0)
        apply_tune(k, args)
        what = f"pbc lattice-hop {SIDE}^3"
    d.step(2)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("steps")
    e0.record(d.stream)
    d.step(args.steps)
    e1.record(d.stream)
    e1.synchronize()
    torch.cuda.nvtx.range_pop()
    print(json.dumps({"workload": "single", "case": what, "precision": args.precision,
                      "ms_per_step": e0.elapsed_time(e1) / max(args.steps, 1), "steps": args.steps}))
    d.free()
    k.free()


def run_reference_config4(args):
    """--impl reference on the headline workload: the oracle restatement of the
    reference's CPU path, each step one Metropolis round of a fixed sample of the
    systems (bounded so that --steps K --warmup W ends within minutes)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count()
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    reqs = config4_requests(args.systems)
    v, dt, nprop, smp = cpu_config4(reqs, args.steps, args.warmup)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config4_config(args, "fp64"),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "sample": smp},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def config4_config(args, precision):
    return {"workload": config4_workload(args.systems), "systems": args.systems, "L": 12, "precision": precision,
            "rounds": args.steps, "l2": "inputs larger than L2: the systems' state (~1 GB over 256 systems) is "
                                       "far above the 129 MB L2, no flush between rounds"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed_fp64_accept", choices=["mixed", "mixed_fp64_accept", "fp64"])
    ap.add_argument("--side", type=int, default=SIDE)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-steps", type=int, default=5)
    ap.add_argument("--cpu-rounds", type=int, default=2)
    ap.add_argument("--fp64-rounds", type=int, default=3)
    ap.add_argument("--build-threads", type=int, default=4)
    ap.add_argument("--ref-steps", type=int, default=10)
    ap.add_argument("--no-extras", action="store_true", help="timed loop only (for profiler runs)")
    ap.add_argument("--tune", nargs="*", default=[], metavar="KEY=VALUE",
                    help="launch-shape tuning keys (include/kmc_gb300.h KMC_TUNE_*) set on every system")
    ap.add_argument("--no-graph", action="store_true", help="launch the step eagerly instead of a CUDA graph")
    ap.add_argument("--workload", default="batched",
                    choices=["batched", "lattice48", "precision_split", "batched_streams", "serving", "drift",
                             "single"])
    ap.add_argument("--case", default="c4pbc", choices=["c4pbc", "c4free", "lattice48"],
                    help="single: the system to step")
    ap.add_argument("--accepts", type=int, nargs="+", default=[0, 2000, 10000, 30000])
    ap.add_argument("--fp32-from", type=int, default=None, help="drift: first accept order in FP32 (tuning key 6)")
    ap.add_argument("--orders", type=int, nargs="+", default=[8, 12, 16])
    ap.add_argument("--error-steps", type=int, default=3)
    ap.add_argument("--systems", type=int, default=256)
    ap.add_argument("--rounds", type=int, default=20)
    ap.add_argument("--workers", type=int, default=16)
    ap.add_argument("--requests", type=int, default=16)
    ap.add_argument("--rates", type=float, nargs="+", default=[50.0, 2000.0])
    ap.add_argument("--max-n", type=int, default=262144)
    ap.add_argument("--max-k", type=int, default=1000)
    ap.add_argument("--max-active", type=int, default=64)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    if args.impl == "reference":
        if args.workload == "batched":
            run_reference_config4(args)
        else:
            run_reference(args)
        return
    if args.workload in ("precision_split", "batched_streams", "serving", "drift", "single"):
        import torch
        torch.cuda.set_device(0)
        {"precision_split": bench_precision_split, "batched_streams": bench_batched, "serving": bench_serving,
         "drift": bench_drift, "single": bench_single}[args.workload](args)
        return

    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if args.workload == "lattice48":
        main_lattice48(args, world, rank, local)
    else:
        value, t_ms, nprop, ms, clk, launches, build_s, extras = bench_config4(args, rank, world, local)
        if rank == 0:
            dtype = {"fp64": "f64",
                     "mixed": "f32+df32 (f64 master state, energy, lattice operator g, final difference)",
                     "mixed_fp64_accept": "f32+df32 near field and harmonic evaluation; f64 accept increments, "
                                          "lattice operator (g = A M, h = A b), energy and final difference"}[
                args.precision]
            line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                    "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
                    "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
                    "config": dict(config4_config(args, args.precision), proposals_per_round=nprop / args.steps,
                                   replicas=world, build_s=build_s),
                    "p50_ms": float(np.percentile(ms, 50)), "p99_ms": float(np.percentile(ms, 99)),
                    "clocks": clk, "gpu_launches": int(launches * args.steps) if launches else None,
                    "cuda_graph": True}
            line.update(extras)
            print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def main_lattice48(args, world, rank, local):
    import torch
    import torch.distributed as dist
    from coulomb_kmc_gb300 import KMCFMM, _native
    from coulomb_kmc_gb300.dats import make_state
    from coulomb_kmc_gb300.workloads import LatticeHopSystem

    side = args.side
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    hs, kmc, drv, init_s = make_system(side, rank, args.precision, local)
    drv.step(1)
    kmc.autotune(reps=5)  # bit-identical launch-shape variants, the fastest kept
    if world > 1:
        dist.barrier()
    per_step, nprop, launches, clk = timed_loop(kmc, drv, args.steps, args.warmup, flush, ClockSampler(local),
                                                graph=not args.no_graph)
    if world > 1:
        dist.barrier()
    t_ms = float(per_step.sum())
    nprop_all = float(nprop)
    if world > 1:
        t_ms, nprop_all = combine_ranks(t_ms, nprop, "cuda")
    value = nprop_all / (t_ms * 1e-3)

    extras = {}
    if not args.no_extras:
        # per-kernel durations with CUDA events (separate pass, the timed loop is not perturbed)
        _native.lib().kmc_profile(kmc._handle, 1)
        kernel_times(kmc)
        snap = LatticeHopSystem(side, OCC, seed=1 + rank)
        snap.site_of = drv.sites()
        snap.occ[:] = -1
        snap.occ[snap.site_of] = np.arange(snap.n)
        fm = flop_model(kmc, snap, folded_nnz())
        for i in range(5):
            flush.fill_(float(i))
            drv.step(1)
        kt, _ = kernel_times(kmc)
        _native.lib().kmc_profile(kmc._handle, 0)
        peak64, peak32 = fma_peak(True), fma_peak(False)
        per_launch = {k: (v[0] / max(v[1], 1)) for k, v in kt.items() if v[1] > 0}
        top = max(per_launch, key=lambda k: kt[k][0])
        ach = {k: fm[k] / (per_launch[k] * 1e-3) / 1e12 for k in ("near_far_cell", "far_lattice",
                                                                   "far_lattice_old", "accept_p2l")
               if k in per_launch}
        fp32_kernels = {"near_far_cell", "far_lattice"} if args.precision == "mixed" else set()
        bound = "fp32" if top in fp32_kernels else "fp64"
        peak = peak32 if bound == "fp32" else peak64
        extras["roofline"] = {
            "bound": bound, "kernel": top, "achieved": ach.get(top), "peak": peak, "unit": "TFLOP/s",
            "frac": (ach.get(top) / peak) if ach.get(top) else None,
            "traffic": NCU_TRAFFIC.get(top) if args.precision == "fp64" else NCU_TRAFFIC_MIXED.get(top),
            "traffic_source": NCU_SOURCE, "issue_frac_source": NCU_SOURCE,
            "peak_source": "measured in this run with kmc_diag_fma_rate (FMA issue rate of the FP64 / FP32 "
                           "pipe); MEASURED_PEAKS.json holds HBM and bf16 only, and these kernels are "
                           "arithmetic bound with an L2-resident state",
            "peaks_measured": {"fp64_tflops": peak64, "fp32_tflops": peak32},
            "flops_convention": "algorithmic flops (add/mul 1, FMA 2, rsqrt 1) of the FP64 algorithm; "
                                "the mixed kernels spend several FP32 instructions per algorithmic flop "
                                "(double-FP32 pair terms)",
            "flops_per_launch": fm.get(top),
            "per_kernel_ms": {k: round(v, 5) for k, v in per_launch.items()},
            "per_kernel_tflops": {k: round(v, 4) for k, v in ach.items()},
            "issue_frac": issue_fracs(per_launch, clk) if args.precision == "mixed" else None,
            "mean_neighbours_per_proposal": fm["mean_neighbours"]}
        drv.free()
        kmc.free()
        # the plain FP64 path on the same workload, for the mixed/FP64 ratio
        if args.precision == "mixed":
            _, k64, d64, _ = make_system(side, rank, "fp64", local)
            ps64, np64, _, _ = timed_loop(k64, d64, max(5, args.steps // 3), 2, flush, graph=not args.no_graph)
            d64.free()
            extras["fp64"] = {"value": np64 / (ps64.sum() * 1e-3), "ms_per_step": float(ps64.mean()),
                              "steps": len(ps64)}
            extras["mixed_vs_fp64"] = value / extras["fp64"]["value"]
            k64.free()
            # mixed propose with the accept contributions kept in FP64
            _, kmf, dmf, _ = make_system(side, rank, "mixed_fp64_accept", local)
            psm, npm, _, _ = timed_loop(kmf, dmf, max(5, args.steps // 3), 2, flush, graph=not args.no_graph)
            dmf.free()
            extras["mixed_fp64_accept"] = {"value": npm / (psm.sum() * 1e-3), "ms_per_step": float(psm.mean()),
                                           "steps": len(psm),
                                           "vs_fp64": (npm / (psm.sum() * 1e-3)) / extras["fp64"]["value"]}
            kmf.free()
            extras["mixed_error"] = mixed_error_stats(side, local)

        # e2e through the public API with host buffers
        e2e_sys = LatticeHopSystem(side, OCC, seed=1 + rank)
        st2 = make_state(e2e_sys.positions(), e2e_sys.charges(), e2e_sys.extent)
        k2 = KMCFMM(st2.P, st2.Q, st2.domain, r=R, l=L, boundary_condition="pbc", max_move=1.0,
                    precision=args.precision)
        k2.initialise()
        rng = np.random.default_rng(7)
        for _ in range(2):
            e2e_sys.step(k2, rng, BETA)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        n2 = 0
        for _ in range(args.e2e_steps):
            e2e_sys.step(k2, rng, BETA)
            n2 += e2e_sys.last_active
        torch.cuda.synchronize()
        e2e_dt = time.perf_counter() - t0
        n = e2e_sys.n
        h2d = 8 + n * 8 + n * 18 * 8 + n * 6 * 8 + n * 6 * 8
        d2h = n * 6 * 8 + 16
        extras["e2e"] = {"value": n2 / e2e_dt, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}
        k2.free()
        if rank == 0:
            cores = os.cpu_count()
            v, dt, npc = cpu_reference(args.cpu_steps, 1, side, None)
            extras["cpu_baseline"] = {
                "value": v, "unit": UNIT, "cores": cores, "kind": "port",
                "sample": f"{args.cpu_steps} KMC steps ({npc} proposals) of the same workload on the oracle "
                          f"(restated reference CPU path, OpenMP {cores} threads; initial expansions zero, "
                          f"which does not change the operation count)"}
    else:
        drv.free()
        kmc.free()
    if rank == 0:
        dtype = {"fp64": "f64",
                 "mixed": "f32+df32 (f64 master state, energy, lattice operator, final difference)",
                 "mixed_fp64_accept": "f32+df32 (f64 accept, energy, lattice operator, final difference)"}[
            args.precision]
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic",
                "config": dict(workload_config(side, args.precision), proposals_per_step=nprop / args.steps,
                               replicas=world),
                "p50_ms": float(np.percentile(per_step, 50)), "p99_ms": float(np.percentile(per_step, 99)),
                "clocks": clk, "gpu_launches": int(launches), "init_s": init_s,
                "cuda_graph": not args.no_graph}
        line.update(extras)
        print(json.dumps(line))




if __name__ == "__main__":
    main()
