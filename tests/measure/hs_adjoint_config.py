#!/usr/bin/env python
"""Adjoint of Held-Suarez T42L20 over a one-day window, with recomputation checkpoints.

72 steps of dt = 1200 s from the seeded initial state (isothermal 264 K at rest, ps = 1e5 Pa, the
reference's vorticity seed, N(0, 0.1^2) K grid noise: Spectral_Initialize_Fields!), a checkpoint
every 8 steps.  Loss J = sum_{i,j,k} w_j (T - T_target)^2 / (2 nlon nd) of the final grid
temperature against a seeded target (the initial T plus N(0, 1) K noise).  Gradient with respect to
the initial spectral temperature and to k_f, k_a, k_s, dT_y, dtheta_z.

Reported:
  * the FP64 GPU gradient against central finite differences of the FP64 GPU forward model
    (eps = 1e-6, relative for the parameters, and 1e-4 and 1e-3 where the difference at 1e-6 is at
    the rounding level of the loss; one seeded direction for T0, row N+1 left out: that row is zero in
    every analysed field and not part of the control);
  * the FP64 GPU gradient against the FP64 oracle's gradient (the C restatement, every state kept);
  * the mixed-precision (FP32) gradient against the FP64 gradient;
  * wall-clock of one gradient (forward sweep + loss + reverse sweep with recomputation).

  python tests/measure/hs_adjoint_config.py [--steps 72] [--checkpoint 8] [--no-oracle] [--out adj.json]
  python tests/measure/hs_adjoint_config.py --profile fp32 --steps 8      (two gradients only, for ncu)
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [os.path.join(ROOT, "idealizedspectralgcm.jl_gb300"), os.path.join(ROOT, "oracle"), ROOT]

import numpy as np  # noqa: E402

NAME = "hs_t42l20"


def t0_direction(mesh, seed=3):
    rng = np.random.default_rng(seed)
    N1, S1 = mesh.num_fourier + 1, mesh.num_spherical + 1
    d = rng.standard_normal((N1, S1, mesh.nd)) + 1j * rng.standard_normal((N1, S1, mesh.nd))
    for m in range(N1):
        d[m, :m, :] = 0
    d[0] = d[0].real
    d /= (1.0 + np.arange(S1))[None, :, None] ** 2
    d[:, -1, :] = 0  # row N+1: zero in every analysed field (not part of the control)
    return np.asfortranarray(d)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=72)
    ap.add_argument("--checkpoint", type=int, default=8)
    ap.add_argument("--eps", type=float, default=1e-6)
    ap.add_argument("--no-oracle", action="store_true")
    ap.add_argument("--out", default=None)
    ap.add_argument("--profile", default=None, metavar="PRECISION",
                    help="only two gradients in this precision (a short launch sequence for ncu)")
    args = ap.parse_args()
    import __graft_entry__

    __graft_entry__.build()
    import jgcm
    from jgcm import configs

    if args.profile:
        mesh = configs.make_mesh(jgcm, NAME, precision=args.profile)
        md = jgcm.Model(mesh, configs.PARAMS[NAME])
        configs.init_held_suarez(jgcm, mesh, md)
        S0 = {k: md.get(k) for k in jgcm.STATE_FIELDS}
        tgt = np.asfortranarray(S0["grid_t_c"] + np.random.default_rng(5).standard_normal(S0["grid_t_c"].shape))
        for _ in range(2):
            for k in jgcm.STATE_FIELDS:
                md.set(k, S0[k])
            md.set_init_step(True)
            loss, _, _ = jgcm.HS_Gradient(md, args.steps, tgt, checkpoint_every=args.checkpoint)
        print(json.dumps({"profile": NAME, "precision": args.profile, "steps": args.steps, "loss": loss}))
        return

    nsteps, ck = args.steps, args.checkpoint
    rep = {"workload": f"Held-Suarez T42L20, {nsteps} steps of dt 1200 s, checkpoint every {ck}; loss = area-weighted "
                       "mean squared difference of the final grid T from a seeded target (initial T + N(0,1) K)",
           "steps": nsteps, "checkpoint_every": ck}
    ref = None
    grads = {}
    for prec in ("fp64", "fp32"):
        mesh = configs.make_mesh(jgcm, NAME, precision=prec)
        md = jgcm.Model(mesh, configs.PARAMS[NAME])
        configs.init_held_suarez(jgcm, mesh, md)
        S0 = {k: md.get(k) for k in jgcm.STATE_FIELDS}
        if ref is None:
            ref = S0
        tgt = np.asfortranarray(ref["grid_t_c"] + np.random.default_rng(5).standard_normal(ref["grid_t_c"].shape))

        def reset(model, fields):
            for k in jgcm.STATE_FIELDS:
                model.set(k, fields[k])
            model.set_init_step(True)

        reset(md, ref)
        loss, gT, gp = jgcm.HS_Gradient(md, nsteps, tgt, checkpoint_every=ck)  # warm-up (graphs, allocations)
        times = []
        for _ in range(3):
            reset(md, ref)
            jgcm.lib().jgcm_mesh_synchronize(mesh._h)
            t0 = time.perf_counter()
            loss, gT, gp = jgcm.HS_Gradient(md, nsteps, tgt, checkpoint_every=ck)
            times.append(time.perf_counter() - t0)
        reset(md, ref)
        jgcm.lib().jgcm_mesh_synchronize(mesh._h)
        t0 = time.perf_counter()
        md.step(nsteps)
        jgcm.lib().jgcm_mesh_synchronize(mesh._h)
        t_fwd = time.perf_counter() - t0
        grads[prec] = (loss, gT, gp)
        rep[prec] = {"loss": loss, "grad_params": dict(zip(jgcm.HS_PARAMS, map(float, gp))),
                     "gradient_wall_ms": 1e3 * min(times), "forward_wall_ms": 1e3 * t_fwd}
        print(prec, json.dumps(rep[prec]), file=sys.stderr, flush=True)
        if prec == "fp64":
            d = t0_direction(mesh)
            gd = mesh.grid(mesh.nd)
            jgcm.Trans_Spherical_To_Grid(mesh, d, gd)
            w = mesh.wts[None, :, None]

            def loss_of(fields, params=None):
                m2 = md if params is None else jgcm.Model(mesh, params)
                reset(m2, fields)
                m2.step(nsteps)
                diff = m2.get("grid_t_c") - tgt
                return float(np.sum(w * diff * diff) / (2.0 * mesh.nlon * mesh.nd))

            eps = args.eps
            fp_, fm_ = dict(ref), dict(ref)
            for k in ("spe_t_c", "spe_t_p"):
                fp_[k] = np.asfortranarray(ref[k] + eps * d)
                fm_[k] = np.asfortranarray(ref[k] - eps * d)
            for k in ("grid_t_c", "grid_t_p"):
                fp_[k] = np.asfortranarray(ref[k] + eps * gd)
                fm_[k] = np.asfortranarray(ref[k] - eps * gd)
            fd = (loss_of(fp_) - loss_of(fm_)) / (2 * eps)
            ad = float(np.sum((gT.conj() * d).real))
            fdrep = {"T0_direction": {"fd": fd, "adjoint": ad, "rel_err": abs(fd - ad) / abs(ad)}}
            for i, p in enumerate(jgcm.HS_PARAMS):
                fdrep[p] = {"adjoint": float(gp[i])}
                for e in (eps, 1e-4, 1e-3):  # larger steps: truncation O(e^2) still far below, rounding smaller
                    h = e * configs.PARAMS[NAME][p]
                    vals = []
                    for sg in (1, -1):
                        P = dict(configs.PARAMS[NAME])
                        P[p] += sg * h
                        vals.append(loss_of(ref, P))
                    f = (vals[0] - vals[1]) / (2 * h)
                    fdrep[p][f"fd_eps_{e:g}"] = f
                    fdrep[p][f"rel_err_eps_{e:g}"] = abs(f - gp[i]) / max(abs(gp[i]), 1e-300)
            rep["fp64_vs_central_differences"] = fdrep
            print("fd", json.dumps(fdrep), file=sys.stderr, flush=True)
    l64, g64, p64 = grads["fp64"]
    l32, g32, p32 = grads["fp32"]
    rep["fp32_vs_fp64"] = {"loss_rel": abs(l32 - l64) / l64,
                           "grad_T0_rel_l2": float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64)),
                           "grad_params_rel": {p: abs(p32[i] - p64[i]) / max(abs(p64[i]), 1e-300)
                                               for i, p in enumerate(jgcm.HS_PARAMS)}}
    if not args.no_oracle:
        import oracle

        om = configs.make_mesh(oracle, NAME)
        omd = oracle.Model(om, configs.PARAMS[NAME])
        for k in oracle.STATE_FIELDS:
            omd.set(k, ref[k])
        oracle.set_state(omd, (oracle.get_state(omd)[0], True))
        t0 = time.perf_counter()
        lo, go, po = oracle.HS_Gradient(omd, nsteps, tgt)
        rep["oracle_fp64"] = {"loss": lo, "wall_s": time.perf_counter() - t0,
                              "gpu_fp64_loss_rel": abs(l64 - lo) / lo,
                              "gpu_fp64_grad_T0_rel_l2": float(np.linalg.norm(g64 - go) / np.linalg.norm(go)),
                              "gpu_fp64_grad_params_rel": {p: abs(p64[i] - po[i]) / max(abs(po[i]), 1e-300)
                                                           for i, p in enumerate(jgcm.HS_PARAMS)},
                              "gpu_fp32_grad_T0_rel_l2": float(np.linalg.norm(g32 - go) / np.linalg.norm(go))}
    txt = json.dumps(rep, indent=1)
    print(txt)
    if args.out:
        with open(args.out, "w") as f:
            f.write(txt)


if __name__ == "__main__":
    main()
