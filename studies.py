#!/usr/bin/env python
"""Accuracy and scale studies of the HMC path on one GPU (the precision and scale-sweep
workloads), printing one JSON object per study.  --size sets the states' size parameter of the
precision and scale studies (default 1000; "L" for size = side length).

precision : D = 4, 32^4, beta in {0.5, 1, 2, 4}, random_su3 start (seed 1), 20 leap-frog steps
            dt 0.005, N trajectories per beta.  The FP64 form and each FP32-arithmetic form
            run trajectory by trajectory from identical links, momenta (host draws, injected
            through lq_hmc_refresh_upload) and accept uniforms; reported per beta: max |Delta H
            error|, max |Delta <P>/3|, acceptance of each form, and the forward/backward
            reversibility of one trajectory (momenta flipped at the end, integrated back).
            Every form reprojects its links onto SU(3) every 10 trajectories.  Where the Gauss projection
            of the momenta fails (the reference's relaxation diverges to NaN for momentum
            standard deviations near 1, i.e. beta = 0.5), the beta records the failure.
scale     : D = 4 at 24^4, 32^4, 48^4, 64^4 and D = 3 at 128^3, 256^3, beta 2, seed 4, 20 steps
            dt 0.005: link-updates/s of FP64 and mixed (device time of K trajectories), the
            MD kernel's (k_md_site) achieved HBM bandwidth, and the Delta H / plaquette error of mixed.

batch     : 64 ensembles of uneven side length and beta advanced together (one launch per kernel
            over every ensemble, a CUDA graph per trajectory), against the same ensembles run
            one after another as single states.

adjoint   : d<plaq>/dbeta through a 50-step leap-frog at 48^4 by the checkpointed reverse-mode
            adjoint, FP32 and FP64, each against its central difference in beta.

distribution: HMC and checkerboard Metropolis on the same lattice and beta give the same average
            plaquette within statistical errors (both sample the Wilson measure).

tour      : every kernel once at --L (for an ncu launch list: gpu__time_duration.sum alone at full size;
            captures with more counters on one kernel of a small lattice, --L 12 .. 20).

run       : N HMC trajectories of one state (device momenta, graph-driven projection), one JSON line per
            trajectory in --log (TrajectoryLog): Delta H, the acceptance probability and decision, the
            average plaquette, the projection's sweep count and the trajectory's wall time.

usage: python studies.py precision [--traj N] [--size L] [--log F] | scale [--traj K] [--size L] | tour [--L 32]
       | batch [--traj N] | adjoint [--L 48] | distribution [--therm N --meas M]
       | run [--L 16] [--traj N] [--precision mixed] [--log F]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "lattice-qcd-rs_gb300"))

import lqgpu  # noqa: E402
from bench import counted_batch_link_updates  # noqa: E402

PREC_NAMES = {lqgpu.PRECISION_F64: "f64", lqgpu.PRECISION_MIXED: "mixed", lqgpu.PRECISION_F32: "f32"}


class TrajectoryLog:
    """Per-trajectory diagnostics as JSON lines.  HybridMonteCarloDiagnostic keeps the last
    trajectory's acceptance probability and decision (prob_replace_last, has_replace_last;
    src/simulation/monte_carlo/hybrid_monte_carlo.rs:402-410); this log keeps every trajectory's,
    with Delta H, the average plaquette Re Tr P / 3, the Gauss projection's sweep count and the
    wall time of the trajectory in milliseconds.  A path of None logs nothing."""

    KEYS = ("trajectory", "form", "beta", "delta_h", "prob", "accepted", "plaquette", "gauss_steps", "ms")

    def __init__(self, path):
        self.f = open(path, "a") if path else None

    def write(self, **rec):
        if self.f is None:
            return
        missing = [k for k in self.KEYS if k not in rec]
        if missing:
            raise ValueError("trajectory record without %s" % ", ".join(missing))
        rec["accepted"] = bool(rec["accepted"])
        self.f.write(json.dumps({k: rec[k] for k in self.KEYS}) + "\n")
        self.f.flush()

    def close(self):
        if self.f is not None:
            self.f.close()
            self.f = None


def hbm_peak():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


def study_size(args, L):
    """The `size` parameter of the states: a number, or "L" for size = side length (the links and
    momenta then move L times farther per step than at the default size 1000 / L)."""
    return float(L) if args.size == "L" else float(args.size)


def precision_study(args):
    log = TrajectoryLog(args.log)
    dim, L, dt, nmd = 4, args.L, 0.005, 20
    size = study_size(args, L)
    out = {"study": "precision", "dim": dim, "L": L, "size": size, "dt": dt, "md_steps": nmd,
           "trajectories_per_beta": args.traj, "betas": {}}
    forms = [lqgpu.PRECISION_F64, lqgpu.PRECISION_MIXED, lqgpu.PRECISION_F32]
    for beta in args.betas:
        rng = np.random.default_rng(1000 + int(beta * 10))
        states = {p: lqgpu.State(dim, L, size, beta, p) for p in forms}
        ref = states[lqgpu.PRECISION_F64]
        ref.set_links_random(1)
        links = ref.link_matrix()
        for p in forms[1:]:
            states[p].set_link_matrix(links)
        acc = {p: 0 for p in forms}
        err_dh = {p: 0.0 for p in forms[1:]}
        err_pl = {p: 0.0 for p in forms[1:]}
        dh_ref = []
        t0 = time.time()
        failure = None
        for k in range(args.traj):
            e_raw = rng.normal(0.0, 0.5 / beta, size=(L ** dim, dim, 8))
            u = float(rng.uniform())
            res = {}
            for p, s in states.items():
                t_start = time.perf_counter()
                try:
                    steps = s.hmc_refresh_upload(e_raw)
                except lqgpu.LqError as err:
                    # the reference's projection (K = 0.12 relaxation) diverges for large momenta
                    failure = {"trajectory": k, "form": PREC_NAMES[p], "error": str(err)}
                    break
                prob, h0, h1 = s.hmc_propose(dt, nmd)
                a = prob >= 1.0 or u < prob
                s.hmc_decide(a)
                acc[p] += a
                res[p] = (h1 - h0, s.average_trace_plaquette().real / 3.0)
                log.write(trajectory=k, form=PREC_NAMES[p], beta=beta, delta_h=h1 - h0, prob=prob, accepted=a,
                          plaquette=res[p][1], gauss_steps=steps, ms=1000.0 * (time.perf_counter() - t_start))
                if (k + 1) % 10 == 0:
                    s.normalize_link_matrices()
            if failure:
                break
            dh_ref.append(res[lqgpu.PRECISION_F64][0])
            for p in forms[1:]:
                err_dh[p] = max(err_dh[p], abs(res[p][0] - res[lqgpu.PRECISION_F64][0]))
                err_pl[p] = max(err_pl[p], abs(res[p][1] - res[lqgpu.PRECISION_F64][1]))
        if failure:
            out["betas"][str(beta)] = {"seconds": round(time.time() - t0, 1), "momentum_std_dev": 0.5 / beta,
                                       "gauss_projection_failed": failure}
            for s in states.values():
                s.close()
            print(json.dumps({"beta": beta, **out["betas"][str(beta)]}), flush=True)
            continue
        # forward/backward reversibility of one trajectory of each form
        rev = {}
        for p, s in states.items():
            s.hmc_refresh_upload(rng.normal(0.0, 0.5 / beta, size=(L ** dim, dim, 8)))
            u0, e0 = s.link_matrix(), s.e_field()
            s.integrate(lqgpu.SYMPLECTIC, dt, nmd)
            s.set_e_field(-s.e_field())
            s.integrate(lqgpu.SYMPLECTIC, dt, nmd)
            rev[PREC_NAMES[p]] = {"links": float(np.abs(s.link_matrix() - u0).max()),
                                  "efield": float(np.abs(-s.e_field() - e0).max())}
        out["betas"][str(beta)] = {
            "seconds": round(time.time() - t0, 1),
            "fp64_delta_h_mean_abs": float(np.mean(np.abs(dh_ref))),
            "acceptance": {PREC_NAMES[p]: acc[p] / args.traj for p in forms},
            "max_abs_delta_h_error": {PREC_NAMES[p]: err_dh[p] for p in forms[1:]},
            "max_abs_plaquette_error": {PREC_NAMES[p]: err_pl[p] for p in forms[1:]},
            "reversibility_max_abs": rev,
        }
        for s in states.values():
            s.close()
        print(json.dumps({"beta": beta, **out["betas"][str(beta)]}), flush=True)
    log.close()
    return out


def run_study(args):
    """N trajectories of one state through the device path, each logged by TrajectoryLog"""
    prec = {"f64": lqgpu.PRECISION_F64, "mixed": lqgpu.PRECISION_MIXED, "f32": lqgpu.PRECISION_F32}[args.precision]
    dim, L, beta, dt, nmd = 4, args.L, args.betas[0] if args.betas else 2.0, 0.005, 20
    log = TrajectoryLog(args.log)
    uni = np.random.default_rng(7)
    out = {"study": "run", "dim": dim, "L": L, "beta": beta, "precision": args.precision, "trajectories": args.traj}
    with lqgpu.State(dim, L, study_size(args, L), beta, prec) as s:
        s.set_links_random(1)
        accepted, dh = 0, []
        for k in range(args.traj):
            t_start = time.perf_counter()
            r = s.hmc_trajectory(dt, nmd, 17, k, float(uni.uniform()))
            plaq = s.average_trace_plaquette().real / 3.0
            ms = 1000.0 * (time.perf_counter() - t_start)
            log.write(trajectory=k, form=args.precision, beta=beta, delta_h=r["delta_h"], prob=r["prob"],
                      accepted=r["accepted"], plaquette=plaq, gauss_steps=r["gauss_steps"], ms=ms)
            accepted += r["accepted"]
            dh.append(r["delta_h"])
        out.update(acceptance=accepted / max(1, args.traj), mean_abs_delta_h=float(np.mean(np.abs(dh))),
                   plaquette=plaq)
    log.close()
    return out


def time_trajectories(state, k, dt, nmd, warm=1):
    import torch

    stream = torch.cuda.Stream()
    state.set_stream(stream.cuda_stream)
    state.profile_enable(True)
    for i in range(warm):
        state.hmc_trajectory(dt, nmd, 3, 1000 + i, 0.5)
    state.profile_read(reset=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    steps = []
    for i in range(k):
        steps.append(state.hmc_trajectory(dt, nmd, 3, i, 0.5)["gauss_steps"])
    e1.record(stream)
    torch.cuda.synchronize()
    prof = state.profile_read(reset=True)
    return e0.elapsed_time(e1), prof, steps


def scale_study(args):
    dt, nmd, beta = 0.005, 20, 2.0
    peak = hbm_peak()
    out = {"study": "scale", "beta": beta, "dt": dt, "md_steps": nmd, "trajectories": args.traj,
           "size": args.size, "lattices": []}
    for dim, L in ((4, 24), (4, 32), (4, 48), (4, 64), (3, 128), (3, 256)):
        size = study_size(args, L)
        n_links = L ** dim * dim
        row = {"dim": dim, "L": L, "links": n_links, "size": size}
        for p in (lqgpu.PRECISION_MIXED, lqgpu.PRECISION_F64):
            k = args.traj if p != lqgpu.PRECISION_F64 else max(1, args.traj // 5)
            s = lqgpu.State(dim, L, size, beta, p)
            s.set_links_random(4)
            ms, prof, steps = time_trajectories(s, k, dt, nmd)
            md_n, md_ms = prof["md"]
            real = 8
            # kick+drift launches 52 reals per link; the final kick 34, 25 in the mixed form (link hi only)
            md_bytes = n_links * real * (52 * nmd + (25 if p == lqgpu.PRECISION_MIXED else 34)) * k
            row[PREC_NAMES[p]] = {"link_updates_per_s": n_links * nmd * k / (ms / 1e3), "ms_per_trajectory": ms / k,
                                  "gauss_steps": steps[0], "md_ms": md_ms / max(1, md_n),
                                  "md_hbm_gbs": md_bytes / (md_ms / 1e3) / 1e9 if md_ms else None,
                                  "md_hbm_frac": md_bytes / (md_ms / 1e3) / 1e9 / peak if md_ms else None}
            s.close()
        # accuracy of mixed against FP64 on two trajectories from identical inputs
        rng = np.random.default_rng(4)
        states = [lqgpu.State(dim, L, size, beta, p) for p in (lqgpu.PRECISION_F64, lqgpu.PRECISION_MIXED)]
        states[0].set_links_random(4)
        states[1].set_link_matrix(states[0].link_matrix())
        edh, epl = 0.0, 0.0
        for _ in range(2):
            e_raw = rng.normal(0.0, 0.5 / beta, size=(L ** dim, dim, 8))
            r = []
            for s in states:
                s.hmc_refresh_upload(e_raw)
                prob, h0, h1 = s.hmc_propose(dt, nmd)
                s.hmc_decide(True)
                r.append((h1 - h0, s.average_trace_plaquette().real / 3.0))
            edh = max(edh, abs(r[1][0] - r[0][0]))
            epl = max(epl, abs(r[1][1] - r[0][1]))
        for s in states:
            s.close()
        row["mixed"]["max_abs_delta_h_error"] = edh
        row["mixed"]["max_abs_plaquette_error"] = epl
        row["mixed_over_f64"] = row["mixed"]["link_updates_per_s"] / row["f64"]["link_updates_per_s"]
        out["lattices"].append(row)
        print(json.dumps(row), flush=True)
    return out


def batch_study(args):
    """64 independent ensembles, D = 4, side lengths drawn from {8, 10, 12, 16, 20} (seed 3),
    beta linearly spaced 0.5 .. 3.5, random_su3 starts, mixed form, 10 leap-frog steps
    dt 0.01, N trajectories each: batched (one launch per kernel over every ensemble, one graph
    launch per trajectory, autotuned launch shapes) against the same ensembles run one after
    another as single states (two trajectories each, scaled)."""
    import torch

    n_ens, dt, nmd, size = args.ensembles, 0.01, 10, 1000.0
    Ls = np.random.default_rng(3).choice([8, 10, 12, 16, 20], size=n_ens)
    betas = np.linspace(0.5, 3.5, n_ens)
    peak = hbm_peak()
    b = lqgpu.Batch(4, Ls, [size] * n_ens, betas, lqgpu.PRECISION_MIXED)
    info = b.info()
    b.set_links_random(3)
    b.set_seed(3, 0)
    t0 = time.time()
    tuning = b.autotune(dt, 3)
    tune_s = time.time() - t0
    stream = torch.cuda.Stream()
    b.set_stream(stream.cuda_stream)
    graph = not args.eager
    b.hmc_run(dt, nmd, 2, graph=graph)  # capture + warm-up
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    w0 = time.time()
    e0.record(stream)
    b.hmc_run(dt, nmd, args.traj, measure_plaquette=True, graph=graph)
    e1.record(stream)
    torch.cuda.synchronize()
    wall = time.time() - w0
    ms = e0.elapsed_time(e1)
    r = b.hmc_results()
    links = info["total_links"]
    md_ms = tuning["md"]["ms"]
    md_bytes = links * 4 * 52 * 2  # compensated FP32: 52 reals of (hi, lo) per link
    ok = r["status"] == 0
    out = {"study": "batch", "ensembles": n_ens, "dim": 4, "L_counts": {int(L): int((Ls == L).sum()) for L in (8, 10, 12, 16, 20)},
           "beta": [0.5, 3.5], "dt": dt, "md_steps": nmd, "trajectories": args.traj, "total_links": links,
           "device_bytes": info["device_bytes"], "autotune_seconds": round(tune_s, 2), "tuning": tuning,
           "ms_per_trajectory": ms / args.traj, "wall_s": wall,
           # trajectories whose projection failed (the reference's HMC refresh panics there) are not counted
           "link_updates_per_s": counted_batch_link_updates(r["status"], Ls, 4, nmd)[0] / (ms / 1e3),
           "link_updates_per_s_all_ensembles": links * nmd * args.traj / (ms / 1e3),
           "md_launch_ms": md_ms, "md_hbm_gbs": md_bytes / (md_ms / 1e3) / 1e9,
           "md_hbm_frac": md_bytes / (md_ms / 1e3) / 1e9 / peak,
           "graph_launches": b.graph_launches(),
           "projection_failures": int((~ok).sum()),
           "failed_ensembles_beta": sorted(set(float(round(betas[e], 3)) for e in np.nonzero(~ok.all(axis=0))[0])),
           "acceptance_mean": float(r["accepted"][ok].mean()) if ok.any() else None,
           "max_abs_delta_h": float(np.abs(r["delta_h"][ok]).max()) if ok.any() else None,
           "gauss_steps_range": [int(r["gauss_steps"][ok].min()), int(r["gauss_steps"][ok].max())] if ok.any() else None}
    b.close()
    if args.quick:
        print(json.dumps(out), flush=True)
        return out
    # the same ensembles one after another (the reference's way of scanning), 2 trajectories each
    seq_ms, seq_links = 0.0, 0
    for e in range(n_ens):
        s = lqgpu.State(4, int(Ls[e]), size, float(betas[e]), lqgpu.PRECISION_MIXED)
        s.set_links_random(3 + e)
        s.set_stream(stream.cuda_stream)
        try:
            s.hmc_trajectory(dt, nmd, 3 + e, 0, 0.5)
        except lqgpu.LqError:
            pass
        torch.cuda.synchronize()
        e0.record(stream)
        for k in range(2):
            try:
                s.hmc_trajectory(dt, nmd, 3 + e, 1 + k, 0.5)
                seq_links += int(Ls[e]) ** 4 * 4 * nmd
            except lqgpu.LqError:
                pass
        e1.record(stream)
        torch.cuda.synchronize()
        seq_ms += e0.elapsed_time(e1)
        s.close()
    out["sequential_link_updates_per_s"] = seq_links / (seq_ms / 1e3)
    out["batched_over_sequential"] = out["link_updates_per_s"] / out["sequential_link_updates_per_s"]
    print(json.dumps(out), flush=True)
    return out


def adjoint_study(args):
    """d<plaq>/dbeta through a 50-step dt 0.01 leap-frog by the reverse-mode adjoint with
    sqrt(n) checkpointing: D = 4, 48^4, beta 2, size 1, random links (seed 2), momenta
    N(0, 0.5/beta) (numpy seed 2); the FP32 form against the FP64 form and against the
    central difference in beta (delta beta 1e-4) of each form."""
    import torch

    dim, L, beta, size, dt, n, db = 4, args.L, 2.0, 1.0, 0.01, 50, 1e-4
    e_raw = np.random.default_rng(2).normal(0.0, 0.5 / beta, size=(L ** dim, dim, 8))
    out = {"study": "adjoint", "dim": dim, "L": L, "beta": beta, "size": size, "dt": dt, "steps": n, "forms": {}}
    for p in (lqgpu.PRECISION_F32, lqgpu.PRECISION_F64):
        s = lqgpu.State(dim, L, size, beta, p)
        s.set_links_random(2)
        s.set_e_field(e_raw)
        links, e0 = s.link_matrix(), s.e_field()
        torch.cuda.synchronize()
        t0 = time.time()
        r = s.leapfrog_adjoint(dt, n, grads=False)
        t_adj = time.time() - t0

        def objective(e):
            s.set_link_matrix(links)
            s.set_e_field(e)
            s.integrate(lqgpu.SYMPLECTIC, dt, n)
            return s.average_trace_plaquette().real / 3.0

        t0 = time.time()
        fd = (objective(e0 * beta / (beta + db)) - objective(e0 * beta / (beta - db))) / (2 * db)
        t_fd = time.time() - t0
        state_bytes = s.device_bytes()
        n_ck = -(-n // int(np.ceil(np.sqrt(n))))
        one = (L ** dim * dim) * (18 + 8) * (8 if p == lqgpu.PRECISION_F64 else 4)
        out["forms"][PREC_NAMES[p]] = {
            "objective": r["objective"], "d_objective_d_beta": r["d_objective_d_beta"],
            "central_difference": fd, "relative_difference_to_fd": abs(r["d_objective_d_beta"] - fd) / abs(fd),
            "adjoint_seconds": round(t_adj, 2), "fd_seconds_two_trajectories": round(t_fd, 2),
            "work_bytes_checkpointed": r["work_bytes"], "checkpoints": n_ck,
            "work_bytes_all_steps_stored": (n + 1) * one, "state_bytes": state_bytes}
        s.close()
        print(json.dumps({PREC_NAMES[p]: out["forms"][PREC_NAMES[p]]}), flush=True)
    f32, f64 = out["forms"]["f32"], out["forms"]["f64"]
    out["f32_vs_f64_relative"] = abs(f32["d_objective_d_beta"] - f64["d_objective_d_beta"]) / abs(f64["d_objective_d_beta"])
    print(json.dumps(out), flush=True)
    return out


def distribution_study(args):
    """Samplers of the Wilson measure exp(-beta sum (1 - Re Tr P / 3)) on the device: checkerboard
    Metropolis; the reference's HMC (momenta N(0, 0.5/beta) projected to the Gauss law, here with the
    exponential link update); and standard HMC with momenta from the kinetic term of the reference's
    own H, exp(-beta sum e^2 / 2), unprojected.  D = 4, 8^4, beta 2 and 4 (smaller betas give
    momenta for which the reference's Gauss projection diverges), random start; the average
    plaquette <Re Tr P>/3 over the measured part of each chain, with its error from 40 blocks."""
    dim, L = 4, 8
    out = {"study": "distribution", "dim": dim, "L": L, "betas": {}}

    def mean_err(x, block=None):
        x = np.asarray(x)
        block = block or max(20, len(x) // 40)  # 40 blocks
        nb = len(x) // block
        b = x[: nb * block].reshape(nb, block).mean(axis=1)
        return float(x.mean()), float(b.std(ddof=1) / np.sqrt(nb))

    for beta in (2.0, 4.0):
        row = {}
        s = lqgpu.State(dim, L, 1.0, beta, lqgpu.PRECISION_F64)
        s.set_links_random(11)
        # the exponential link update keeps the links in SU(3) and the leap-frog reversible; the
        # reference's first-order update drifts off the group at these step sizes, after which the
        # Gauss projection fails
        s.set_link_update(lqgpu.LINK_UPDATE_EXP)
        uni = np.random.default_rng(int(beta * 100))
        failed = 0

        def traj(k, dt, n):
            nonlocal failed
            try:
                return s.hmc_trajectory(dt, n, 13, k, float(uni.uniform()), max_gauss_steps=2001)["accepted"]
            except lqgpu.LqError:  # the projection diverged or stalled: no proposal
                failed += 1
                return False
        # the largest step (trajectory length 0.5) accepting >= 60% of 20 trial trajectories
        k = 0
        for dt in (0.04, 0.02, 0.01, 0.005):
            n = int(round(0.5 / dt))
            trial = [traj(k + i, dt, n) for i in range(20)]
            k += 20
            if np.mean(trial) >= 0.6:
                break
        plaq, acc = [], 0
        for i in range(args.therm + args.meas):
            a = traj(k, dt, n)
            k += 1
            if i >= args.therm:
                plaq.append(s.average_trace_plaquette().real / 3.0)
                acc += a
        m, e = mean_err(plaq)
        row["hmc"] = {"plaquette": m, "error": e, "acceptance": acc / args.meas, "dt": dt, "md_steps": n,
                      "size": 1.0, "link_update": "exp", "trajectories": k, "failed_projections": failed,
                      "finite": bool(np.isfinite(plaq).all())}
        s.close()
        # standard HMC: momenta from exp(-beta sum e^2 / 2), the kinetic term of the reference's H
        # (std 1/sqrt(beta), not the 0.5/beta of new_random_e_state), no Gauss projection
        s = lqgpu.State(dim, L, 1.0, beta, lqgpu.PRECISION_F64)
        s.set_links_random(11)
        s.set_link_update(lqgpu.LINK_UPDATE_EXP)
        rng = np.random.default_rng(int(beta * 1000))
        plaq, acc = [], 0
        for i in range(args.therm + args.meas):
            s.set_e_field(rng.normal(0.0, 1.0 / np.sqrt(beta), size=(L ** dim, dim, 8)))
            p, h0, h1 = s.hmc_propose(dt, n)
            a = p >= 1.0 or rng.uniform() < p
            s.hmc_decide(a)
            if i >= args.therm:
                plaq.append(s.average_trace_plaquette().real / 3.0)
                acc += a
        m, e = mean_err(plaq)
        row["hmc_standard_momenta"] = {"plaquette": m, "error": e, "acceptance": acc / args.meas, "dt": dt,
                                       "md_steps": n, "momentum_std_dev": 1.0 / np.sqrt(beta)}
        s.close()
        s = lqgpu.State(dim, L, 1.0, beta, lqgpu.PRECISION_F64)
        s.set_links_random(11)
        plaq, pm = [], []
        for k in range(args.therm + args.meas):
            a, p = s.metropolis_sweep(4, 0.3, 17, k)
            if k >= args.therm:
                plaq.append(s.average_trace_plaquette().real / 3.0)
                pm.append(p)
        m, e = mean_err(plaq)
        row["metropolis"] = {"plaquette": m, "error": e, "mean_acceptance_probability": float(np.mean(pm)),
                             "sweeps": args.therm + args.meas, "n_update": 4, "spread": 0.3}
        s.close()
        for name in ("hmc", "hmc_standard_momenta"):
            d = row[name]["plaquette"] - row["metropolis"]["plaquette"]
            row[name]["vs_metropolis_sigma"] = d / np.hypot(row[name]["error"], row["metropolis"]["error"])
        out["betas"][str(beta)] = row
        print(json.dumps({"beta": beta, **row}), flush=True)
    print(json.dumps(out), flush=True)
    return out


def tour_study(args):
    """Every kernel of the library launched at least once, for a per-kernel profile (a launch list with
    DRAM bytes under ncu): D = 4 states at L^4 (default 32^4: links and momenta above L2) in FP64,
    mixed and f32 -- conversions, momentum draws, Gauss law, projection (host-driven loop, so that
    profilers see its kernels), the MD modes and the exponential update, the HMC proposal, the action and
    its backward, a link rotation, normalisation, clover fields, Metropolis, heat-bath and overrelaxation sweeps
    and the trajectory adjoint -- a D = 3 (128^3) and a D = 2 (2048^2) trajectory, the allocation-free plaquette
    sums, and a batch of 8 uneven ensembles (L 16 .. 28, 9.4 M links) run eagerly."""
    import ctypes

    import torch

    L, dt = args.L, 0.005
    done = []
    for prec in (lqgpu.PRECISION_F64, lqgpu.PRECISION_MIXED, lqgpu.PRECISION_F32):
        with lqgpu.State(4, L, 1000.0, 2.0, prec) as s:
            s.set_projection_graph(False)
            s.set_links_cold()
            s.set_links_random(1)
            links = s.link_matrix()
            s.set_link_matrix(links)
            s.set_e_field_normal(2, 0, 0.25)
            e = s.e_field()
            s.set_e_field(e)
            s.gauss()
            s.gauss_sum_div()
            s.project_to_gauss()
            s.hamiltonian_links()
            s.hamiltonian_efield()
            s.average_trace_plaquette()
            for mode in (lqgpu.SYNC_SYNC, lqgpu.SYNC_LEAP, lqgpu.LEAP_LEAP, lqgpu.LEAP_SYNC):
                s.integrate(mode, dt, 1)
            s.integrate(lqgpu.SYMPLECTIC, dt, 2)
            s.integrate(lqgpu.SYMPLECTIC_EXP, dt, 1)
            s.integrate(lqgpu.SYMPLECTIC_EXP_REUNITARIZE, dt, 1)
            s.normalize_link_matrices()
            s.hmc_trajectory(dt, 3, 5, 0, 0.5)
            s.wilson_action()
            s.wilson_action_backward()
            s.link_rotate(7, 3, 1e-3)
            s.field_strength()
            s.magnetic_field()
            s.metropolis_sweep(1, 0.1, 3, 0)
            s.heat_bath_sweep(3, 1)
            s.overrelaxation_sweep(lqgpu.OVERRELAX_ROTATION)
            s.overrelaxation_sweep(lqgpu.OVERRELAX_REVERSE)
            s.leapfrog_adjoint(dt, 4)
        done.append(PREC_NAMES[prec])
    for dim, Ld in ((3, 128), (2, 2048)):
        with lqgpu.State(dim, Ld, 1000.0, 2.0, lqgpu.PRECISION_MIXED) as s:
            s.set_projection_graph(False)
            s.set_links_random(1)
            s.hmc_trajectory(dt, 3, 5, 0, 0.5)
        done.append("mixed D=%d" % dim)
    lib = lqgpu.load()
    dev = torch.device("cuda:0")
    with lqgpu.State(4, L, 1000.0, 2.0, lqgpu.PRECISION_F64) as s:
        s.set_links_random(3)
        d_links = torch.from_numpy(s.link_matrix()).to(dev)
    d_out = torch.zeros(3, dtype=torch.float64, device=dev)
    rc = lib.lq_plaquette_sums_noalloc(4, L, ctypes.c_void_p(d_links.data_ptr()), ctypes.c_void_p(d_out.data_ptr()),
                                       ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    torch.cuda.synchronize(dev)
    if rc != lqgpu.LQ_OK:
        raise lqgpu.LqError(rc, "lq_plaquette_sums_noalloc")
    done.append("noalloc plaquette sums")
    Ls = [16, 20, 24, 28, 16, 20, 24, 28]
    with lqgpu.Batch(4, Ls, [1000.0] * len(Ls), np.linspace(1.0, 3.0, len(Ls)), lqgpu.PRECISION_MIXED) as b:
        b.set_links_random(3)
        b.set_seed(3, 0)
        b.hmc_run(0.01, 3, 1, graph=False, measure_plaquette=True)
        b.normalize_link_matrices()
        b.average_trace_plaquette()
    done.append("batch (eager)")
    out = {"study": "tour", "L": L, "done": done}
    print(json.dumps(out), flush=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["precision", "scale", "batch", "adjoint", "distribution", "tour", "run"])
    ap.add_argument("--log", default=None, help="precision, run: per-trajectory JSON lines appended to this file")
    ap.add_argument("--precision", default="mixed", choices=["f64", "mixed", "f32"], help="run: the state's form")
    ap.add_argument("--traj", type=int, default=None)
    ap.add_argument("--L", type=int, default=32)
    ap.add_argument("--betas", type=float, nargs="*", default=[0.5, 1.0, 2.0, 4.0])
    ap.add_argument("--size", default="1000",
                    help="precision, scale: the states' size parameter, a number or L for size = side length")
    ap.add_argument("--quick", action="store_true", help="batch: skip the one-after-another comparison")
    ap.add_argument("--ensembles", type=int, default=64, help="batch: number of ensembles (the first n draws)")
    ap.add_argument("--therm", type=int, default=200, help="distribution: thermalisation steps")
    ap.add_argument("--meas", type=int, default=800, help="distribution: measured steps")
    ap.add_argument("--eager", action="store_true",
                    help="batch: launch the kernels one by one instead of the captured graph (for profilers, "
                         "which do not see kernels of graphs with conditional nodes)")
    args = ap.parse_args()
    if args.study == "precision":
        args.traj = args.traj or 100
        res = precision_study(args)
    elif args.study == "scale":
        args.traj = args.traj or 10
        res = scale_study(args)
    elif args.study == "batch":
        args.traj = args.traj or 50
        res = batch_study(args)
    elif args.study == "distribution":
        res = distribution_study(args)
    elif args.study == "tour":
        res = tour_study(args)
    elif args.study == "run":
        args.traj = args.traj or 20
        if args.L == 32:
            args.L = 16
        args.betas = args.betas if len(args.betas) == 1 else [2.0]
        res = run_study(args)
    else:
        if args.L == 32:
            args.L = 48
        res = adjoint_study(args)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
