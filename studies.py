#!/usr/bin/env python
"""Accuracy and scale studies of the HMC path on one GPU (the brief's precision and
scale-sweep configurations), printing one JSON object per study.

precision : D = 4, 32^4, beta in {0.5, 1, 2, 4}, random_su3 start (seed 1), 20 leap-frog steps
            dt 0.005, N trajectories per beta.  The FP64 form and each FP32-arithmetic form
            run trajectory by trajectory from identical links, momenta (host draws, injected
            through lq_hmc_refresh_upload) and accept uniforms; reported per beta: max |Delta H
            error|, max |Delta <P>/3|, acceptance of each form, and the forward/backward
            reversibility of one trajectory (momenta flipped at the end, integrated back).
            Mixed reprojects its links (FP64) every 10 trajectories.
scale     : D = 4 at 24^4, 32^4, 48^4, 64^4 and D = 3 at 128^3, 256^3, beta 2, seed 4, 20 steps
            dt 0.005: link-updates/s of FP64 and mixed (device time of K trajectories), the
            k_md kernel's achieved HBM bandwidth, and the Delta H / plaquette error of mixed.

usage: python studies.py precision [--traj N] | scale [--traj K]
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

PREC_NAMES = {lqgpu.PRECISION_F64: "f64", lqgpu.PRECISION_MIXED: "mixed", lqgpu.PRECISION_F32: "f32"}


def hbm_peak():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


def precision_study(args):
    dim, L, size, dt, nmd = 4, args.L, 1000.0, 0.005, 20
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
        for k in range(args.traj):
            e_raw = rng.normal(0.0, 0.5 / beta, size=(L ** dim, dim, 8))
            u = float(rng.uniform())
            res = {}
            for p, s in states.items():
                s.hmc_refresh_upload(e_raw)
                prob, h0, h1 = s.hmc_propose(dt, nmd)
                a = prob >= 1.0 or u < prob
                s.hmc_decide(a)
                acc[p] += a
                res[p] = (h1 - h0, s.average_trace_plaquette().real / 3.0)
                if p == lqgpu.PRECISION_MIXED and (k + 1) % 10 == 0:
                    s.normalize_link_matrices()
            dh_ref.append(res[lqgpu.PRECISION_F64][0])
            for p in forms[1:]:
                err_dh[p] = max(err_dh[p], abs(res[p][0] - res[lqgpu.PRECISION_F64][0]))
                err_pl[p] = max(err_pl[p], abs(res[p][1] - res[lqgpu.PRECISION_F64][1]))
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
    dt, nmd, beta, size = 0.005, 20, 2.0, 1000.0
    peak = hbm_peak()
    out = {"study": "scale", "beta": beta, "dt": dt, "md_steps": nmd, "trajectories": args.traj, "lattices": []}
    for dim, L in ((4, 24), (4, 32), (4, 48), (4, 64), (3, 128), (3, 256)):
        n_links = L ** dim * dim
        row = {"dim": dim, "L": L, "links": n_links}
        for p in (lqgpu.PRECISION_MIXED, lqgpu.PRECISION_F64):
            k = args.traj if p != lqgpu.PRECISION_F64 else max(1, args.traj // 5)
            s = lqgpu.State(dim, L, size, beta, p)
            s.set_links_random(4)
            ms, prof, steps = time_trajectories(s, k, dt, nmd)
            md_n, md_ms = prof["md"]
            real = 8
            md_bytes = n_links * real * (52 * nmd + 34) * k
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("study", choices=["precision", "scale"])
    ap.add_argument("--traj", type=int, default=None)
    ap.add_argument("--L", type=int, default=32)
    ap.add_argument("--betas", type=float, nargs="*", default=[0.5, 1.0, 2.0, 4.0])
    args = ap.parse_args()
    if args.study == "precision":
        args.traj = args.traj or 100
        res = precision_study(args)
    else:
        args.traj = args.traj or 10
        res = scale_study(args)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
