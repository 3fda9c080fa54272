#!/usr/bin/env python
"""HMC link-updates/s at 32^4 on GB300: mixed FP32/FP64 (headline) and plain FP64.

One bench step is one full HMC trajectory of HybridMonteCarloDiagnostic on
LatticeStateDefault<4>: momentum refresh N(0, 0.5/beta) on the device, Gauss projection,
20 leap-frog steps of dt = 0.005, both Hamiltonians and the accept/reject -- D = 4, 32^4
sites, beta = 2.0, size 1000, links from random_su3 drawn on the device (seed 1).
value = links * md_steps * trajectories / device time of the timed trajectories.

--impl reference times the CPU oracle (a C++ restatement of the reference's
SymplecticEulerRayon + HybridMonteCarloDiagnostic, OpenMP over all host threads) on a
bounded sample of the same workload: the same trajectory on an 8^4 sublattice.
Under torchrun every rank runs an independent replica on its own GPU ("replicas only").
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "lattice-qcd-rs_gb300")
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "HMC link-updates/s at 32^4: mixed FP32/FP64 vs plain FP64 GPU at equal plaquette error"
UNIT = "link-updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--dim", type=int, default=4)
    ap.add_argument("--L", type=int, default=32)
    ap.add_argument("--beta", type=float, default=2.0)
    ap.add_argument("--dt", type=float, default=0.005)
    ap.add_argument("--md-steps", type=int, default=20)
    ap.add_argument("--size", type=float, default=1000.0)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "f32", "f64"])
    ap.add_argument("--fp64-steps", type=int, default=2, help="timed FP64 trajectories for the comparison leg")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-sample-L", type=int, default=8)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--projection", default="graph", choices=["graph", "host"],
                    help="Gauss projection loop of the headline state: one graph launch with a device-side test "
                         "(default) or host-driven launches (profilers do not see kernels inside graphs with "
                         "conditional nodes)")
    ap.add_argument("--batch-traj", type=int, default=50,
                    help="timed trajectories of the batched-ensembles leg, the configuration's 50 (0: skip it)")
    ap.add_argument("--batch-gap-traj", type=int, default=10,
                    help="trajectories of the batch leg's graph-gap measurement (0: skip it)")
    ap.add_argument("--host-driver-traj", type=int, default=10,
                    help="timed trajectories of the C++ HybridMonteCarloDiagnostic leg (0: skip it)")
    return ap.parse_args()


def run_host_driver(args, prec):
    """The C++ host interface's HybridMonteCarloDiagnostic (lattice-qcd-rs_gb300/host) driving a
    device-resident state in its own process: compiled here against the in-tree library, timed by the
    host clock.  None when the compiler or the run fails (the line says why)."""
    import lqgpu

    pkg = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lattice-qcd-rs_gb300")
    lib_dir = os.path.dirname(lqgpu.LIB_PATH)
    exe = os.path.join(lib_dir, "hmc_driver_timing")
    src = os.path.join(pkg, "host", "hmc_driver_timing.cpp")
    inc = os.path.join(os.path.dirname(pkg), "include")
    cmd = ["g++", "-std=c++17", "-O2", "-I", inc, "-I", os.path.join(pkg, "host"), src, "-o", exe, "-L", lib_dir,
           "-llqgpu", "-Wl,-rpath," + lib_dir]
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
        if r.returncode != 0:
            return {"unavailable": "g++ failed: " + r.stderr.strip()[-200:]}
        r = subprocess.run([exe, str(args.L), str(args.host_driver_traj), "3", str(prec), str(args.md_steps),
                            repr(args.dt), repr(args.beta)], capture_output=True, text=True, timeout=600)
        if r.returncode != 0:
            return {"unavailable": "run failed: " + (r.stderr or r.stdout).strip()[-200:]}
        out = json.loads(r.stdout.strip().splitlines()[-1])
    except (OSError, subprocess.SubprocessError, ValueError) as e:
        return {"unavailable": "%s: %s" % (type(e).__name__, e)}
    out["path"] = ("C++ HybridMonteCarloDiagnostic<4>::next_element per trajectory (new_random_e_state with device "
                   "momenta keyed by the driver's Xoshiro256++, lq_hmc_propose, the host's accept draw, "
                   "lq_hmc_decide), a separate process, host clock, D=4 %d^4 as the headline" % args.L)
    return out


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm_sorted = sorted(sm)
        return {"sm_mhz": sm_sorted[len(sm_sorted) // 2], "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "power_w_max": max(power), "samples": len(sm)}


def smi_index():
    """nvidia-smi index of this process's GPU (CUDA_VISIBLE_DEVICES when it is a plain index)."""
    v = os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0].strip()
    return int(v) if v.isdigit() else 0


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ------------------------------------------------------------------ CPU baseline (oracle)
def cpu_trajectory_rate(dim, L, beta, dt, md_steps, size, seconds, min_traj=2):
    """Times full oracle trajectories (refresh on the host + projection + MD + accept)."""
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    rng = O.Rng(1)
    links = O.links_random(dim, L, rng)
    n_links = L ** dim * dim
    # one untimed trajectory (warm-up)
    e_raw = O.efield_normal(dim, L, rng, 0.5 / beta)
    links = O.hmc_trajectory(dim, L, size, beta, links, e_raw, dt, md_steps, rng.uniform(0, 1))["links"]
    t_total, n = 0.0, 0
    while n < min_traj or t_total < seconds:
        t0 = time.perf_counter()
        e_raw = O.efield_normal(dim, L, rng, 0.5 / beta)
        r = O.hmc_trajectory(dim, L, size, beta, links, e_raw, dt, md_steps, rng.uniform(0, 1))
        t_total += time.perf_counter() - t0
        links = r["links"]
        n += 1
        if n >= 50:
            break
    return n_links * md_steps * n / t_total, threads, n, t_total


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O

    threads = os.cpu_count() or 1
    O.set_threads(threads)
    dim, L = args.dim, args.cpu_sample_L
    rng = O.Rng(1)
    links = O.links_random(dim, L, rng)
    n_links = L ** dim * dim

    def one():
        e_raw = O.efield_normal(dim, L, rng, 0.5 / args.beta)
        return O.hmc_trajectory(dim, L, args.size, args.beta, links, e_raw, args.dt, args.md_steps,
                                rng.uniform(0, 1))["links"]

    for _ in range(args.warmup):
        links = one()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        links = one()
    elapsed = time.perf_counter() - t0
    value = n_links * args.md_steps * args.steps / elapsed
    sample = ("full HMC trajectories (host momentum draw, Gauss projection, %d leap-frog steps, both Hamiltonians, "
              "accept) on a %d^%d sublattice of the %d^%d workload, beta %g, dt %g" %
              (args.md_steps, L, dim, args.L, dim, args.beta, args.dt))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "HMC trajectory D=%d %d^%d (CPU sample %d^%d), beta %g, %d leap-frog steps dt %g, "
                               "size %g" % (dim, args.L, dim, L, dim, args.beta, args.md_steps, args.dt, args.size),
                   "implementation": "CPU oracle: C++ restatement of SymplecticEulerRayon + "
                                     "HybridMonteCarloDiagnostic (the Rust reference cannot be built here)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ GPU arm
# DRAM bytes (read + write) per link of one kick+drift launch of the MD kernel (k_md_site), from one
# ncu capture of the mixed kernel at 28^4 (1050.5 MB for 2,458,624 links, with the L2 prefetch of the
# update data); traffic scales with the links of a launch, so the full-size value is this times the links.
NCU_MD_TRAFFIC_PER_LINK = {"mixed": 1050.5e6 / 2458624}
MD_KERNEL = "k_md_site (fused force + kick + drift, one thread per site)"


# FP64 operations per unit of the FP64 form's kernels (D = 4): FLOP with a multiply-add as 2; the dfma,
# dmul, dadd instruction counts per unit in parentheses are ncu's at 16^4.
#   MD kick+drift per link: a quarter of k_md_plaq's site (6 plaquettes, each formed once and projected
#     for its 4 links: 3528 dfma, 720 dmul, 240 dadd per site) and k_md_update (the 4 force parts
#     summed, two kicks, E U, the drift: 108, 28, 24); the final kick-only launch's update (8, 2, 24)
#   k_gauss_step_adj per link: H = U G U^dag through the link's transport table, the d-symbol
#     contraction 2 Re Tr(T^a H G(x+mu)) and the update (154, 29, 0)
#   k_gauss_adj per site: D transports U^dag E U through the tables, the accumulation of G and the
#     residual (292, 1, 45.5)
# The compiler contracts some products and sums into multiply-adds.
_PLAQ_PER_LINK = (2 * 3528 + 720 + 240) / 4.0
FP64_FLOPS = {"md_kick_drift": _PLAQ_PER_LINK + 2 * 108 + 28 + 24, "md_kick": _PLAQ_PER_LINK + 2 * 8 + 2 + 24,
              "gauss_step": 2 * 154 + 29, "gauss": 2 * 292 + 1 + 45.5}


def fp64_roofline(prof64, n_links, n_sites, md_steps, trajectories, peak):
    """achieved FP64 FLOP/s of the FP64 form's kernel classes over the timed trajectories, against the
    measured multiply-add peak (lq_fma_peak): those kernels are bound by the FP64 pipe, not by HBM"""
    md_n, md_ms = prof64["md"]
    st_n, st_ms = prof64["gauss_sweep"]  # the FP64 projection's step launches
    ga_n, ga_ms = prof64["gauss"]
    md_flops = n_links * (md_steps * FP64_FLOPS["md_kick_drift"] + FP64_FLOPS["md_kick"]) * trajectories
    out = {"peak_tflops": peak / 1e12, "peak_kind": "measured: lq_fma_peak, FP64 multiply-add chains on every SM",
           "flop_counts": "ncu FP64 instruction counts at 16^4 (2 FLOP per dfma), per link or site: " +
                          json.dumps(FP64_FLOPS),
           "pass": "one trajectory with the host-driven projection loop (per-kernel events)"}
    for name, flops, ms, n in (("k_md_plaq + k_md_update", md_flops, md_ms, md_n),
                               ("k_gauss_step_adj", st_n * n_links * FP64_FLOPS["gauss_step"], st_ms, st_n),
                               ("k_gauss_adj", ga_n * n_sites * FP64_FLOPS["gauss"], ga_ms, ga_n)):
        if ms > 0 and n > 0:
            achieved = flops / (ms / 1000.0)
            out[name] = {"launches": n, "ms_per_launch": ms / n, "achieved_tflops": achieved / 1e12,
                         "frac": achieved / peak}
    return out


def algorithmic_md_bytes(n_links, md_steps, real_bytes, compensated=False):
    """Bytes moved by the fused MD kernels of one trajectory at ideal neighbour reuse.
    kick+drift launch: read U (18 reals) + E (8) + write E (8) + U' (18) = 52 reals per link;
    final kick-only launch: read U (18) + E (8) + write E (8) = 34 reals per link, where the
    compensated (mixed) form reads the link's hi half only (9 pair-sized units): 25.
    real_bytes is the stored size of one real: 8 for FP64 and for the compensated FP32 pairs
    of the mixed form, 4 for plain FP32 storage."""
    return n_links * real_bytes * (52 * md_steps + (25 if compensated else 34))


def rank_reducers(pg, device):
    """(barrier, max_over_ranks, sum_over_ranks) for the replicas; identities without a group."""
    import torch

    def barrier():
        if pg is not None:
            pg.barrier()

    def reduce(x, op):
        if pg is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device=device)
        pg.all_reduce(t, op=op)
        return float(t.item())

    return (barrier, lambda x: reduce(x, pg.ReduceOp.MAX if pg else None),
            lambda x: reduce(x, pg.ReduceOp.SUM if pg else None))


def replica_value(units, ms, max_over_ranks, sum_over_ranks):
    """whole-job throughput: every rank's units over the slowest rank's time"""
    return sum_over_ranks(units) / (max_over_ranks(ms) / 1000.0)


def counted_batch_link_updates(status, side_lengths, dim, md_steps):
    """Link updates of the ensemble trajectories whose Gauss projection succeeded (status 0), from the
    per-trajectory, per-ensemble status array [trajectories, ensembles]: at the smallest betas the
    reference's projection diverges (its step is quadratic in the Gauss law) and its HMC refresh
    panics, so the work done on those ensembles is not counted.  Also returns, per failing ensemble,
    how many of its trajectories failed."""
    import numpy as np

    ok = np.asarray(status) == 0
    ens_links = np.asarray(side_lengths, dtype=np.int64) ** dim * dim
    counted = int((ok * ens_links[None, :]).sum()) * md_steps
    failed = {int(e): int((~ok[:, e]).sum()) for e in np.nonzero(~ok.all(axis=0))[0]}
    return counted, failed


def batch_leg(args, stream, peak):
    """The parameter-scan workload: 64 ensembles, D = 4, side lengths drawn from {8, 10, 12, 16, 20}
    (seed 3), beta linearly spaced 0.5 .. 3.5, size 1000, mixed, 10 leap-frog steps dt 0.01; every
    kernel one launch over all ensembles, one CUDA-graph launch per trajectory, autotuned shapes."""
    import numpy as np
    import torch

    import lqgpu

    n_ens, dt, nmd = 64, 0.01, 10
    Ls = np.random.default_rng(3).choice([8, 10, 12, 16, 20], size=n_ens)
    betas = np.linspace(0.5, 3.5, n_ens)
    b = lqgpu.Batch(4, Ls, [1000.0] * n_ens, betas, lqgpu.PRECISION_MIXED)
    links = b.info()["total_links"]
    b.set_links_random(3)
    b.set_seed(3, 0)
    tuning = b.autotune(dt, 3)
    b.set_stream(stream.cuda_stream)
    b.hmc_run(dt, nmd, 3)  # graph capture + warm-up
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = b.graph_launches()
    ev0.record(stream)
    b.hmc_run(dt, nmd, args.batch_traj)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    r = b.hmc_results()
    launches = b.graph_launches() - launches0
    gap = batch_graph_gap(b, stream, dt, nmd, args.batch_gap_traj, 3 + args.batch_traj) if args.batch_gap_traj else None
    b.close()
    md_bytes = links * 52 * 8
    ok = r["status"] == 0
    counted, failed = counted_batch_link_updates(r["status"], Ls, 4, nmd)
    return {"workload": "64 ensembles D=4, L from {8,10,12,16,20} (seed 3), beta 0.5..3.5, size 1000, mixed, "
                        "10 leap-frog steps dt 0.01; one launch per kernel over all ensembles, one CUDA graph "
                        "per trajectory", "total_links": links, "trajectories": args.batch_traj,
            "value": counted / (ms / 1000.0), "unit": UNIT,
            "counted": "link updates of ensemble trajectories whose Gauss projection succeeded",
            "value_all_ensembles": links * nmd * args.batch_traj / (ms / 1000.0),
            "ms_per_trajectory": ms / args.batch_traj, "graph_launches": launches, "md_launch_ms": tuning["md"]["ms"],
            "md_hbm_frac": md_bytes / (tuning["md"]["ms"] / 1000.0) / 1e9 / peak,
            "tuning": {k: [v["grid"], v["order"]] for k, v in tuning.items()},
            "projection_failures": int((~ok).sum()),
            "projection_failures_by_ensemble": [{"ensemble": e, "L": int(Ls[e]), "beta": round(float(betas[e]), 4),
                                                 "trajectories": c} for e, c in failed.items()],
            "projection_failure_cause": "NaN residual (LQ_ERR_GAUSS_PROJECTION): the reference's projection step is "
                                        "quadratic in the Gauss law and diverges for momenta of standard deviation "
                                        "0.5/beta near 1; the ensemble keeps its links",
            "acceptance": float(r["accepted"][ok].mean()) if ok.any() else None,
            "graph_gap": gap}


def batch_graph_gap(b, stream, dt, nmd, n_traj, counter):
    """The graph's cost between its kernel nodes: the same n_traj trajectories (links and Philox
    counters restored in between, results checked equal) run once as graph launches, timed by CUDA
    events around them, and once as eager launches with every kernel bracketed by CUDA events
    (lq_batch_profile_*); gap = 1 - summed kernel time / graph time."""
    import numpy as np
    import torch

    # both runs start from the same links as written back from their FP64 image (a compensated pair read
    # out and written back is re-split, which need not reproduce the pair the trajectories left behind)
    links = [b.link_matrix(e) for e in range(b.n)]
    for e, x in enumerate(links):
        b.set_link_matrix(e, x)
    b.set_seed(3, counter)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    ev0.record(stream)
    b.hmc_run(dt, nmd, n_traj)
    ev1.record(stream)
    torch.cuda.synchronize()
    graph_ms = ev0.elapsed_time(ev1)
    rg = b.hmc_results()
    for e, x in enumerate(links):
        b.set_link_matrix(e, x)
    b.set_seed(3, counter)
    b.profile_enable(True)
    b.profile_read(reset=True)
    b.hmc_run(dt, nmd, n_traj, graph=False)
    n_kernels, kernel_ms = b.profile_read(reset=True)
    b.profile_enable(False)
    re_ = b.hmc_results()
    # failed projections record NaN: equal NaNs count as equal
    same = all(np.array_equal(rg[k], re_[k], equal_nan=(k == "delta_h")) for k in ("delta_h", "accepted", "gauss_steps"))
    return {"trajectories": n_traj, "graph_ms_per_trajectory": graph_ms / n_traj,
            "kernel_ms_per_trajectory": kernel_ms / n_traj, "kernels_per_trajectory": n_kernels / n_traj,
            "gap_fraction": 1.0 - kernel_ms / graph_ms, "same_results": bool(same),
            "method": "the same trajectories (links and counters restored) as graph launches timed by events around "
                      "them and as eager launches with an event pair around every kernel"}


def run_ours(args):
    rank, world, local_rank = dist_env()
    if world > 1:
        # one GPU per replica: make the rank's GPU device 0 before CUDA initialises
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local_rank)
    import numpy as np
    import torch

    import lqgpu

    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    torch.cuda.synchronize()
    stream = torch.cuda.Stream(device=dev)

    dim, L, beta, dt, nmd, size = args.dim, args.L, args.beta, args.dt, args.md_steps, args.size
    n_links = L ** dim * dim
    prec = {"mixed": lqgpu.PRECISION_MIXED, "f32": lqgpu.PRECISION_F32, "f64": lqgpu.PRECISION_F64}[args.precision]
    real_bytes = 4 if prec == lqgpu.PRECISION_F32 else 8
    uni = np.random.default_rng(1000 + rank)

    barrier, max_over_ranks, sum_over_ranks = rank_reducers(pg, dev)

    def timed_trajectories(state, k_warm, k_timed, seed, sample_clocks=False):
        results = []
        for k in range(k_warm):
            state.hmc_trajectory(dt, nmd, seed, 10_000 + k, float(uni.uniform()))
        state.profile_read(reset=True)
        sampler = ClockSampler(smi_index()) if sample_clocks else None
        if sampler:
            sampler.start()
            time.sleep(0.5)
        barrier()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        t0 = time.perf_counter()
        for k in range(k_timed):
            results.append(state.hmc_trajectory(dt, nmd, seed, k, float(uni.uniform())))
        ev1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        barrier()
        clocks = sampler.stop() if sampler else None
        ms = ev0.elapsed_time(ev1)
        prof = state.profile_read(reset=True)
        return ms, wall, prof, results, clocks

    # ---- headline precision
    s = lqgpu.State(dim, L, size, beta, prec)
    s.set_stream(stream.cuda_stream)
    s.set_projection_graph(args.projection == "graph")
    s.set_links_random(1 + rank)
    # inside the timed region only the MD launches carry CUDA events (the roofline's kernel time);
    # the other classes run without them
    s.profile_enable(True)
    s.profile_classes(["md"])
    ms, wall, prof, res, clocks = timed_trajectories(s, args.warmup, args.steps, 77 + rank, sample_clocks=True)
    ms_max = max_over_ranks(ms)
    value = replica_value(n_links * nmd * args.steps, ms, max_over_ranks, sum_over_ranks)
    md_launches, md_ms = prof["md"]
    # every class timed on a few more trajectories of the same state: the kernel breakdown and the
    # launches of a trajectory (the same launches every trajectory but for its projection's sweeps)
    s.profile_classes(None)
    k_all = 3
    _, _, prof_all, res_all, _ = timed_trajectories(s, 0, k_all, 177 + rank)
    s.profile_enable(False)
    sweeps_all = sum(r["gauss_steps"] for r in res_all)
    sweeps_timed = sum(r["gauss_steps"] for r in res)
    per_sweep = prof_all["gauss_sweep"][0] / max(1, sweeps_all)  # sweep-loop launches per sweep (graph nodes)
    launches_fixed = (sum(v[0] for v in prof_all.values()) - prof_all["gauss_sweep"][0]) / k_all
    launches = int(round(launches_fixed * args.steps + per_sweep * sweeps_timed))
    md_bytes = algorithmic_md_bytes(n_links, nmd, real_bytes, prec == lqgpu.PRECISION_MIXED) * args.steps
    peak, peak_kind = measured_peaks()
    achieved = md_bytes / (md_ms / 1000.0) / 1e9 if md_ms > 0 else 0.0
    gauss_steps = [r["gauss_steps"] for r in res]
    acc_rate = sum(r["accepted"] for r in res) / max(1, len(res))

    # ---- e2e: momenta from pinned host memory through the C ABI test-mode entry, results back
    e2e = None
    if args.e2e_steps > 0:
        shape = (L ** dim, dim, 8)
        host_bufs = []
        for j in range(2):
            t = torch.empty(shape, dtype=torch.float64, pin_memory=True)
            t.normal_(0.0, 0.5 / beta, generator=torch.Generator().manual_seed(5 + j))
            host_bufs.append(t.numpy())
        s.efield_prefetch(host_bufs[0])  # warm the prefetch buffer and copy stream
        s.hmc_refresh_prefetched()
        s.hmc_propose(dt, nmd)
        s.hmc_decide(True)
        barrier()
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        d2h = 0
        # momenta of trajectory k + 1 are copied while trajectory k runs (lq_efield_prefetch)
        s.efield_prefetch(host_bufs[0])
        for k in range(args.e2e_steps):
            steps = s.hmc_refresh_prefetched()
            if k + 1 < args.e2e_steps:
                s.efield_prefetch(host_bufs[(k + 1) % 2])
            p, h0, h1 = s.hmc_propose(dt, nmd)
            s.hmc_decide(p >= 1.0 or float(uni.uniform()) < p)
            plaq = s.average_trace_plaquette()
            # the projection's reads (graph: sweeps and status, 2 ints; host loop: one double per test)
            # + 8 doubles (proposal) + 3 (plaquette)
            proj_d2h = 8 if args.projection == "graph" else 8 * ((steps - 1) // 4 + 1)
            d2h += proj_d2h + 8 * 8 + 8 * 3
        ev1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = max_over_ranks(ev0.elapsed_time(ev1))
        e2e = {"value": sum_over_ranks(n_links * nmd * args.e2e_steps) / (e2e_ms / 1000.0), "unit": UNIT,
               "h2d_bytes_per_step": int(np.prod(shape) * 8), "d2h_bytes_per_step": int(d2h / args.e2e_steps),
               "path": "lq_efield_prefetch + lq_hmc_refresh_prefetched + lq_hmc_propose + lq_hmc_decide + "
                       "lq_average_trace_plaquette, momenta (f64, reference layout) from pinned host memory each "
                       "trajectory, the next trajectory's copy overlapping the current one",
               "scope": "the C ABI called from Python (ctypes) as the reference's HMC driver would call it; the "
                        "links stay resident on the device (the state is device-resident), only the momenta and "
                        "the scalar results cross the bus"}
    plaq_mixed = s.average_trace_plaquette()
    s.close()

    # ---- the C++ host interface's HMC driver on the same workload (N = 1 only: its own process)
    host_driver = None
    if args.host_driver_traj > 0 and world == 1 and args.dim == 4:
        torch.cuda.synchronize()
        host_driver = run_host_driver(args, prec)

    # ---- FP64 leg (the plain GPU form), the plain-FP32-storage leg, and accuracy at equal inputs
    fp64 = None
    f32 = None
    accuracy = None
    if prec != lqgpu.PRECISION_F64 and args.fp64_steps > 0:
        s64 = lqgpu.State(dim, L, size, beta, lqgpu.PRECISION_F64)
        s64.set_stream(stream.cuda_stream)
        s64.set_links_random(1 + rank)
        s64.profile_enable(True)
        s64.profile_classes(["md"])
        ms64, _, prof64, res64, _ = timed_trajectories(s64, 1, args.fp64_steps, 77 + rank)
        # the projection runs as one graph launch: its kernels' FP64 rates come from one more
        # trajectory with the host-driven loop, which the profile sees kernel by kernel
        s64.profile_classes(None)
        s64.set_projection_graph(False)
        _, _, prof64k, _, _ = timed_trajectories(s64, 0, 1, 78 + rank)
        s64.profile_enable(False)
        ms64 = max_over_ranks(ms64)
        v64 = sum_over_ranks(n_links * nmd * args.fp64_steps) / (ms64 / 1000.0)
        md64_n, md64_ms = prof64["md"]
        fp64 = {"value": v64, "unit": UNIT, "ms_per_step": ms64 / args.fp64_steps,
                "headline_over_fp64": value / v64,
                "md_kernel_ms": md64_ms / max(1, md64_n),
                "gauss_steps": [r["gauss_steps"] for r in res64],
                "kernel_ms": {k: {"launches": v[0], "ms": round(v[1], 3)} for k, v in prof64k.items()},
                "roofline_fp64": fp64_roofline(prof64k, n_links, L ** dim, nmd, 1,
                                               lqgpu.fma_peak(lqgpu.PRECISION_F64))}
        other = lqgpu.PRECISION_F32 if prec == lqgpu.PRECISION_MIXED else lqgpu.PRECISION_MIXED
        so = lqgpu.State(dim, L, size, beta, other)
        so.set_stream(stream.cuda_stream)
        so.set_links_random(1 + rank)
        so.profile_enable(True)
        so.profile_classes(["md"])
        mso, _, profo, reso, _ = timed_trajectories(so, 1, max(2, args.fp64_steps), 77 + rank)
        so.profile_enable(False)
        mso = max_over_ranks(mso)
        vo = sum_over_ranks(n_links * nmd * max(2, args.fp64_steps)) / (mso / 1000.0)
        f32 = {"precision": "f32" if other == lqgpu.PRECISION_F32 else "mixed", "value": vo, "unit": UNIT,
               "ms_per_step": mso / max(2, args.fp64_steps),
               "md_kernel_ms": profo["md"][1] / max(1, profo["md"][0])}
        if not args.no_accuracy:
            # identical links, momenta (host draw) and uniforms into every precision
            sm = lqgpu.State(dim, L, size, beta, lqgpu.PRECISION_MIXED)
            sf = lqgpu.State(dim, L, size, beta, lqgpu.PRECISION_F32)
            states = {"f64": s64, "mixed": sm, "f32": sf}
            for st in states.values():
                st.set_links_random(5)
            rngacc = np.random.default_rng(9)
            acc_out = {k: [] for k in states}
            # Gauss-law residual gauss_sum_div of each form's projected momenta, evaluated in FP64 on
            # that form's own links (an FP64 state loaded with them): the FP32 forms stop their
            # projection at f32 eps * V * 320, the FP64 form at the reference's f64 eps * V * 320
            residual = {k: [] for k in states}
            chk = lqgpu.State(dim, L, size, beta, lqgpu.PRECISION_F64)
            chk.set_stream(stream.cuda_stream)
            for k in range(2):
                e_raw = rngacc.normal(0.0, 0.5 / beta, size=(L ** dim, dim, 8))
                u = float(rngacc.uniform())
                for name, st in states.items():
                    st.hmc_refresh_upload(e_raw)
                    if name == "f64":
                        residual[name].append(st.gauss_sum_div())
                    else:
                        chk.set_link_matrix(st.link_matrix())
                        chk.set_e_field(st.e_field())
                        residual[name].append(chk.gauss_sum_div())
                    p, h0, h1 = st.hmc_propose(dt, nmd)
                    st.hmc_decide(p >= 1.0 or u < p)
                    acc_out[name].append((h1 - h0, st.average_trace_plaquette().real / 3.0))
            chk.close()
            n_sites = L ** dim
            accuracy = {"trajectories": 2, "fp64_delta_h": [x[0] for x in acc_out["f64"]],
                        "note": "every precision vs FP64 GPU from identical links, momenta and uniforms",
                        "fp64": {"gauss_residual": max(residual["f64"]),
                                 "gauss_threshold": 2.220446049250313e-16 * n_sites * 320},
                        "gauss_residual_note": "gauss_sum_div (sum over sites of |Tr((sum_a T^a) G(x))|) of the "
                                               "projected start momenta, evaluated in FP64 on the form's own links"}
            for name in ("mixed", "f32"):
                accuracy[name] = {
                    "max_abs_delta_h_error": max(abs(a[0] - b[0]) for a, b in zip(acc_out[name], acc_out["f64"])),
                    "max_abs_plaquette_error": max(abs(a[1] - b[1]) for a, b in zip(acc_out[name], acc_out["f64"])),
                    "gauss_residual": max(residual[name]),
                    "gauss_threshold": 1.1920928955078125e-07 * n_sites * 320,
                    "gauss_residual_over_fp64": max(residual[name]) / max(max(residual["f64"]), 1e-300)}
            sm.close()
            sf.close()
        so.close()
        s64.close()

    batch = batch_leg(args, stream, peak) if args.batch_traj > 0 else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, threads, n, t = cpu_trajectory_rate(dim, args.cpu_sample_L, beta, dt, nmd, size, args.cpu_seconds)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d full HMC trajectories (%d leap-frog steps, host momentum draw, Gauss projection, both "
                         "Hamiltonians) on a %d^%d sublattice, %.1f s, OpenMP over all host threads" %
                         (n, nmd, args.cpu_sample_L, dim, t)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": {lqgpu.PRECISION_MIXED: "f32 (compensated f32 pairs stored) + f64 sums",
                                           lqgpu.PRECISION_F32: "f32 + f64 sums",
                                           lqgpu.PRECISION_F64: "f64"}[prec], "data": "synthetic",
            "config": {"workload": "HMC trajectory D=%d %d^%d, beta %g, %d leap-frog steps dt %g, size %g, "
                                   "random_su3 start, device momenta N(0,0.5/beta) + Gauss projection"
                                   % (dim, L, dim, beta, nmd, dt, size),
                       "precision": args.precision, "parallelism": "replicas" if world > 1 else "single GPU",
                       "projection_loop": args.projection,
                       "l2": "inputs larger than L2 (links %.0f MB)" % (n_links * 18 * real_bytes / 1e6)},
            "roofline": {"bound": "hbm", "kernel": MD_KERNEL, "achieved": achieved,
                         "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                         "traffic": (NCU_MD_TRAFFIC_PER_LINK[args.precision] * n_links
                                     if args.precision in NCU_MD_TRAFFIC_PER_LINK else None),
                         "traffic_source": "ncu dram bytes per link at 28^4 scaled to 32^4",
                         "algorithmic_bytes_per_link": 52 * real_bytes,
                         "md_launch_ms": md_ms / max(1, md_launches)},
            "kernel_ms": {k: {"launches": v[0], "ms": round(v[1], 3)} for k, v in prof_all.items()},
            "kernel_ms_pass": "%d further trajectories of the same state with every launch timed (in the timed "
                              "region only the MD launches carry events)" % k_all,
            "gpu_launches": launches,
            "gpu_launches_count": "the launches of each trajectory of the timed region: per trajectory those of the "
                                  "fully timed pass, the projection's launches per sweep times the sweeps each timed "
                                  "trajectory made",
            "gauss_steps": gauss_steps, "acceptance": acc_rate, "plaquette": plaq_mixed.real / 3.0,
            "wall_ms_per_step": 1000.0 * wall / args.steps,
            "clocks": clocks, "e2e": e2e, "host_driver": host_driver, "fp64": fp64, "other_precision": f32,
            "accuracy": accuracy,
            "batch": batch, "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    if pg is not None:
        pg.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
