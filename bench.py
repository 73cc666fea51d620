"""Benchmark: proposal energy differences per second on the pbc lattice-hop workload.

Workload (one system per GPU): simple-cubic lattice of 48^3 sites (spacing 1,
box edge 48, periodic), 27,648 charges (25 % occupancy, +-1 balanced, seed 1),
FMM depth R=5 (16^3 cells), L=12.  One step = one rejection-free KMC step:
every charge proposes a hop to each vacant nearest-neighbour site (~124k
proposals), all proposal energy differences are computed, one move is chosen
with rate exp(-beta dE / 2), beta = 2, and accepted.

Timed arms:
  value : device resident -- the library's device-side KMC driver (proposal
          generation, rejection-free selection and occupancy kernels) around its
          propose and accept kernels, one captured CUDA graph per step; L2 flushed
          (256 MiB write) between timed steps.
  e2e   : the reference-facing API with host (numpy) buffers, exactly as the
          reference's driver uses it: host bookkeeping, propose_with_dats with
          host<->device copies, host selection, accept.
  --impl reference : the reference's CPU path as restated by the oracle
          (ppmd/coulomb_kmc cannot be built here), all host threads.

Other workloads (--workload; each prints its own JSON line):
  precision_split : 64^3 lattice, 65,536 charges, R=6, L in {8, 12, 16}: mixed vs
                    FP64 error (max / RMS relative dE, Metropolis agreement) and
                    throughput of both paths.
  batched         : independent off-lattice systems (N log-uniform in
                    [2,000, 131,072], half free_space, half pbc, density 0.25,
                    L=12), one step of every system per round through one
                    multi-stream launch of their captured step graphs; mixed vs FP64.
  serving         : Poisson request stream through the continuous-batching
                    server, p50/p99 round latency and throughput, against FP64
                    one system at a time.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload ...]
Multi-GPU (torchrun): independent replicas, one system per rank, no collective
on the data path; value = proposals over all ranks / max rank time.
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
    FMA = 2, rsqrt = 1; the counting convention of the survey), from this step's
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


# DRAM traffic per launch of the dominant kernel, from the ncu capture summarised in
# profiles/fp64_step_lattice48_launch_list.md (dram__bytes_read.sum + dram__bytes_write.sum)
NCU_TRAFFIC = {"near_far_cell": 12.921088e6}
# mixed path: profiles/k_near_cell_mixed_lattice48.md, k_p2l_pair_lattice48.md, k_lr_mixed_lattice48.md
NCU_TRAFFIC_MIXED = {"near_far_cell": 12.378624e6, "accept_p2l": 5.167360e6, "far_lattice": 23.233024e6,
                     "far_lattice_old": 1.251584e6}
# warp instructions per launch from the same ncu capture (smsp__inst_executed.sum), for the
# issue-slot fraction of the mixed kernels (4 warp instructions per SM per clock)
NCU_INST_MIXED = {"near_far_cell": 40.433271e6, "accept_p2l": 23.066700e6, "far_lattice": 11.877886e6,
                  "far_lattice_old": 1.332936e6}


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
    steps = max(1, min(args.steps, args.ref_steps))
    v, dt, nprop = cpu_reference(steps, min(args.warmup, 1), SIDE)
    sample = (f"{steps} KMC steps of the {SIDE}^3 lattice-hop workload ({nprop} proposals), oracle restatement "
              f"of the reference's generated C (ppmd is unavailable), OpenMP {cores} threads; "
              f"initial expansions zero (the operation count does not depend on their values)")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
            "warmup": min(args.warmup, 1), "ms_per_step": 1e3 * dt / steps, "higher_is_better": True,
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


def mixed_error_stats(side, local, nsteps=3, seed=11):
    """Mixed vs FP64 on identical states: relative dE error (denominator max(|dE|,1))
    and Metropolis-decision agreement (u < exp(-beta dE) with shared u)."""
    from coulomb_kmc_gb300 import KMCFMM
    from coulomb_kmc_gb300.dats import make_state
    from coulomb_kmc_gb300.workloads import LatticeHopSystem
    hs = LatticeHopSystem(side, OCC, seed=seed)
    ks = {}
    for prec in ("fp64", "mixed"):
        st = make_state(hs.positions(), hs.charges(), hs.extent)
        ks[prec] = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition="pbc", max_move=1.0, precision=prec)
        ks[prec].initialise()
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
        for prec in ("mixed", "fp64"):
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
            ps, npr, _, _ = timed_loop(k, d, args.steps, args.warmup, flush)
            res[prec] = {"value": npr / (ps.sum() * 1e-3), "ms_per_step": float(ps.mean()), "init_s": init_s,
                         "p99_ms": float(np.percentile(ps, 99))}
            d.free()
            k.free()
        err = error_stats(side, r6, Lx, seed=2, nsteps=args.error_steps)
        out[f"L{Lx}"] = {"mixed": res["mixed"], "fp64": res["fp64"],
                         "mixed_vs_fp64": res["mixed"]["value"] / res["fp64"]["value"], "error": err}
        print(json.dumps({"L": Lx, **out[f"L{Lx}"]}), file=sys.stderr)
    line = {"metric": METRIC, "workload": "precision_split", "unit": UNIT,
            "config": {"workload": "pbc lattice-hop 64^3 sites, 65,536 charges (seed 2), R=6, L swept",
                       "orders": list(args.orders), "steps": args.steps, "warmup": args.warmup},
            "results": out}
    print(json.dumps(line))


def error_stats(side, r, Lx, seed, nsteps):
    """Mixed vs FP64 differences on identical states along an FP64-selected chain."""
    global R, L
    saved = (R, L)
    R, L = r, Lx
    try:
        return mixed_error_stats(side, 0, nsteps=nsteps, seed=seed)
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
        srv = Server(precision="mixed", hbm_budget=150e9, max_active=args.max_active, n_workers=args.workers)
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
            "per_rate": out,
            "config": {"workload": f"{args.requests} requests (seed 4), Poisson arrivals, N log-uniform in "
                                   f"[1000, {args.max_n}], lattice-hop pbc or off-lattice free_space with "
                                   f"probability 1/2, L=12, K uniform in [10, {args.max_k}], 150 GB budget",
                       "rates_per_s": list(args.rates), "max_active": args.max_active,
                       "worker_streams": args.workers}}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "mixed_fp64_accept", "fp64"])
    ap.add_argument("--side", type=int, default=SIDE)
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-steps", type=int, default=5)
    ap.add_argument("--ref-steps", type=int, default=10)
    ap.add_argument("--no-extras", action="store_true", help="timed loop only (for profiler runs)")
    ap.add_argument("--no-graph", action="store_true", help="launch the step eagerly instead of a CUDA graph")
    ap.add_argument("--workload", default="lattice48",
                    choices=["lattice48", "precision_split", "batched", "serving", "drift"])
    ap.add_argument("--accepts", type=int, nargs="+", default=[0, 2000, 10000, 30000])
    ap.add_argument("--fp32-from", type=int, default=None, help="drift: first accept order in FP32 (tuning key 6)")
    ap.add_argument("--orders", type=int, nargs="+", default=[8, 12, 16])
    ap.add_argument("--error-steps", type=int, default=3)
    ap.add_argument("--systems", type=int, default=64)
    ap.add_argument("--rounds", type=int, default=20)
    ap.add_argument("--workers", type=int, default=16)
    ap.add_argument("--requests", type=int, default=16)
    ap.add_argument("--rates", type=float, nargs="+", default=[50.0, 2000.0])
    ap.add_argument("--max-n", type=int, default=262144)
    ap.add_argument("--max-k", type=int, default=1000)
    ap.add_argument("--max-active", type=int, default=64)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)
    if args.workload != "lattice48" and args.impl == "ours":
        import torch
        torch.cuda.set_device(0)
        {"precision_split": bench_precision_split, "batched": bench_batched, "serving": bench_serving,
         "drift": bench_drift}[
            args.workload](args)
        return

    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from coulomb_kmc_gb300 import KMCFMM, _native
    from coulomb_kmc_gb300.dats import make_state
    from coulomb_kmc_gb300.workloads import LatticeHopSystem

    side = args.side
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    hs, kmc, drv, init_s = make_system(side, rank, args.precision, local)
    if world > 1:
        dist.barrier()
    per_step, nprop, launches, clk = timed_loop(kmc, drv, args.steps, args.warmup, flush, ClockSampler(local),
                                                graph=not args.no_graph)
    if world > 1:
        dist.barrier()
    t_ms = float(per_step.sum())
    tot = torch.tensor([t_ms, float(nprop)], dtype=torch.float64, device="cuda")
    if world > 1:
        tmax = tot[0:1].clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.all_reduce(tot[1:2], op=dist.ReduceOp.SUM)
        tot[0] = tmax[0]
    t_ms, nprop_all = float(tot[0]), float(tot[1])
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
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
