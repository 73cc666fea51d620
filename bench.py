"""Benchmark: proposal energy differences per second on the pbc lattice-hop workload.

Workload (one system per GPU): simple-cubic lattice of 48^3 sites (spacing 1,
box edge 48, periodic), 27,648 charges (25 % occupancy, +-1 balanced, seed 1),
FMM depth R=5 (16^3 cells), L=12.  One step = one rejection-free KMC step:
every charge proposes a hop to each vacant nearest-neighbour site (~124k
proposals), all proposal energy differences are computed, one move is chosen
with rate exp(-beta dE / 2), beta = 2, and accepted.

Timed arms:
  value : device resident -- proposals, masks, selection and bookkeeping on the
          GPU (torch ops on device tensors) around the library's propose and
          accept kernels; L2 flushed (256 MiB write) between timed steps.
  e2e   : the reference-facing API with host (numpy) buffers, exactly as the
          reference's driver uses it: host bookkeeping, propose_with_dats with
          host<->device copies, host selection, accept.
  --impl reference : the reference's CPU path as restated by the oracle
          (ppmd/coulomb_kmc cannot be built here), all host threads.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
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
class DeviceLattice:
    """Lattice-hop bookkeeping on the device (torch), feeding the library's
    device-resident propose_with_dats / accept_device."""

    def __init__(self, host_sys, device):
        import torch
        self.t = torch
        self.k = host_sys.side
        self.E = host_sys.extent
        self.n = host_sys.n
        self.M = 6
        self.site_of = torch.from_numpy(host_sys.site_of.copy()).to(device)
        occ = np.full(self.k ** 3, -1, np.int64)
        occ[host_sys.site_of] = np.arange(self.n)
        self.occ = torch.from_numpy(occ).to(device)
        self.hops = torch.tensor([(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)],
                                 dtype=torch.int64, device=device)
        self.smc = torch.tensor([6], dtype=torch.int64, device=device)
        self.sites = torch.zeros((self.n, 1), dtype=torch.int64, device=device)
        self.diffs = torch.zeros((self.n, self.M), dtype=torch.float64, device=device)
        torch.cuda.manual_seed(1234)

    def build(self):
        t, k = self.t, self.k
        s = self.site_of
        xyz = torch_stack = t.stack((s % k, (s // k) % k, s // (k * k)), dim=1)
        tgt = (torch_stack[:, None, :] + self.hops[None, :, :]) % k
        self.tsite = tgt[..., 0] + k * (tgt[..., 1] + k * tgt[..., 2])
        self.masks = (self.occ[self.tsite] < 0).to(t.int64)
        self.ppos = (tgt.to(t.float64) - 0.5 * self.E + 0.5).reshape(self.n, 3 * self.M).contiguous()
        del xyz

    def select(self, beta):
        t = self.t
        rates = t.where(self.masks > 0, t.exp(-0.5 * beta * self.diffs), t.zeros_like(self.diffs)).reshape(-1)
        c = t.cumsum(rates, 0)
        u = t.rand(1, device=c.device, dtype=t.float64) * c[-1]
        idx = t.searchsorted(c, u, right=True).clamp_(max=c.numel() - 1)
        pid = idx // self.M
        h = idx % self.M
        self.d_pid = pid.contiguous()
        self.d_new = self.ppos.view(self.n, self.M, 3)[pid, h].reshape(3).contiguous()
        self.d_de = self.diffs.view(-1)[idx].contiguous()
        self.new_site = self.tsite[pid, h]

    def commit(self):
        # device-only index updates (capturable in a CUDA graph)
        pid = self.d_pid.view(-1)
        ns = self.new_site.view(-1)
        self.occ.index_fill_(0, self.site_of.index_select(0, pid), -1)
        self.occ.index_copy_(0, ns, pid)
        self.site_of.index_copy_(0, pid, ns)

    def step(self, kmc, beta):
        self.build()
        kmc.propose_with_dats(self.smc, self.sites, self.ppos, self.masks, self.diffs, sync=False)
        self.select(beta)
        kmc.accept_device(self.d_pid, self.d_new, self.d_de)
        self.commit()
        return self.n


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
    near_new = float(np.sum(11 * nb[pcell])) + nprop * (far + 27 * 11 + 4)
    near_old = float(np.sum(11 * nb[st["cells"][movers]])) + len(movers) * (far + 2)
    lr_new = nprop * (mpole + 4 * nh + lr_nnz_folded + 6)   # a, a.(g-h), a^T U a
    lr_old = len(movers) * (mpole + 2 * 2 * lr_nnz_folded + 8 * nh)
    ncell = n ** 3
    p2l = ncell * 54 * (12 * nh + 6 * L + 15)
    return {"near_far_cell": near_new + near_old, "far_lattice": lr_new, "far_lattice_old": lr_old,
            "accept_p2l": p2l, "proposals": nprop, "mean_neighbours": float(np.mean(nb[pcell]))}


# DRAM traffic per launch of the dominant kernel, from the ncu capture summarised in
# profiles/near_far_cell_fp64_lattice48.md (dram__bytes_read.sum + dram__bytes_write.sum)
NCU_TRAFFIC = {"near_far_cell": 12.921088e6}
NCU_TRAFFIC_MIXED = {}


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
        _, masks, _ = hs.proposals()
        nprop += int(masks.sum())
        hs.step(o, rng, BETA)
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
    import torch
    from coulomb_kmc_gb300 import KMCFMM
    from coulomb_kmc_gb300.dats import make_state
    from coulomb_kmc_gb300.workloads import LatticeHopSystem
    hs = LatticeHopSystem(side, OCC, seed=1 + rank)
    st = make_state(hs.positions(), hs.charges(), hs.extent)
    kmc = KMCFMM(st.P, st.Q, st.domain, r=R, l=L, boundary_condition="pbc", max_move=1.0, precision=precision)
    t0 = time.perf_counter()
    kmc.initialise()
    init_s = time.perf_counter() - t0
    dev = DeviceLattice(hs, torch.device("cuda", local))
    return hs, kmc, dev, init_s


def capture_step(kmc, dev, warmup):
    """Warm up on a side stream, then capture one full KMC step in a CUDA graph.
    Returns the graph and the number of library kernel launches per step."""
    import torch
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(max(warmup, 2)):
            dev.step(kmc, BETA)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    kmc.check_errors()
    _, l0 = kernel_times(kmc)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        dev.step(kmc, BETA)
    _, l1 = kernel_times(kmc)
    return g, l1


def timed_loop(kmc, dev, steps, warmup, flush, sampler=None, graph=True):
    import torch
    g, per_step_launches = None, None
    if graph:
        g, per_step_launches = capture_step(kmc, dev, warmup)
        for _ in range(2):
            g.replay()
    else:
        for _ in range(warmup):
            dev.step(kmc, BETA)
    torch.cuda.synchronize()
    kmc.check_errors()
    kernel_times(kmc)  # reset counters
    if sampler:
        sampler.start()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    counts = []
    torch.cuda.synchronize()
    for i in range(steps):
        flush.fill_(float(i))
        ev[i][0].record()
        if g is not None:
            g.replay()
        else:
            dev.step(kmc, BETA)
        ev[i][1].record()
        counts.append(dev.masks.sum())
    torch.cuda.synchronize()
    clk = sampler.stop() if sampler else None
    per_step = np.array([a.elapsed_time(b) for a, b in ev])
    nprop = int(torch.stack(counts).sum().item())
    _, launches = kernel_times(kmc)
    if g is not None:
        launches = per_step_launches * steps
    kmc.check_errors()
    return per_step, nprop, launches, clk


def mixed_error_stats(side, local, nsteps=3):
    """Mixed vs FP64 on identical states: relative dE error (denominator max(|dE|,1))
    and Metropolis-decision agreement (u < exp(-beta dE) with shared u)."""
    from coulomb_kmc_gb300 import KMCFMM
    from coulomb_kmc_gb300.dats import make_state
    from coulomb_kmc_gb300.workloads import LatticeHopSystem
    hs = LatticeHopSystem(side, OCC, seed=11)
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
    args = ap.parse_args()
    args.warmup = max(args.warmup, 0)

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
    hs, kmc, dev, init_s = make_system(side, rank, args.precision, local)
    if world > 1:
        dist.barrier()
    per_step, nprop, launches, clk = timed_loop(kmc, dev, args.steps, args.warmup, flush, ClockSampler(local),
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
        snap.site_of = dev.site_of.cpu().numpy()
        snap.occ[:] = -1
        snap.occ[snap.site_of] = np.arange(snap.n)
        fm = flop_model(kmc, snap, folded_nnz())
        for i in range(5):
            flush.fill_(float(i))
            dev.step(kmc, BETA)
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
            "mean_neighbours_per_proposal": fm["mean_neighbours"]}
        kmc.free()
        # the plain FP64 path on the same workload, for the mixed/FP64 ratio
        if args.precision == "mixed":
            _, k64, d64, _ = make_system(side, rank, "fp64", local)
            ps64, np64, _, _ = timed_loop(k64, d64, max(5, args.steps // 3), 2, flush, graph=not args.no_graph)
            extras["fp64"] = {"value": np64 / (ps64.sum() * 1e-3), "ms_per_step": float(ps64.mean()),
                              "steps": len(ps64)}
            extras["mixed_vs_fp64"] = value / extras["fp64"]["value"]
            k64.free()
            # mixed propose with the accept contributions kept in FP64
            _, kmf, dmf, _ = make_system(side, rank, "mixed_fp64_accept", local)
            psm, npm, _, _ = timed_loop(kmf, dmf, max(5, args.steps // 3), 2, flush, graph=not args.no_graph)
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
            _, m2, _ = e2e_sys.proposals()
            n2 += int(m2.sum())
            e2e_sys.step(k2, rng, BETA)
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
