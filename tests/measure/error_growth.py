#!/usr/bin/env python
"""Error growth of the GPU paths against the FP64 oracle: Held-Suarez T42L20 at 1, 10 and 100 days.

Runs the same seeded initial state (Spectral_Initialize_Fields! with the reference's vorticity seed
plus N(0, 0.1^2) K grid noise on T) through three models:
  oracle   the FP64 C restatement of the reference on the host cores,
  gpu64    the FP64 GPU path,
  gpu32    the mixed-precision GPU path (FP32 state/transforms, FP64 wave-matrix solve and sums),
and prints, per checkpoint day, the relative L2 difference of every prognostic grid field
(T, u, v, ps) and of the zonal means of T and u (a climatological measure that stays meaningful
after the flow becomes chaotic).  Writes one JSON document to stdout (and to --out if given).

  python tests/measure/error_growth.py --days 1 10 100 [--out results.json] [--threads N]
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

FIELDS = {"T": "grid_t_c", "u": "grid_u_c", "v": "grid_v_c", "ps": "grid_ps_c"}


def rel(a, b):
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return float(d / n) if n > 0 else float(d)


def snapshot(model):
    return {k: np.array(model.get(v)) for k, v in FIELDS.items()}


def compare(a, b):
    out = {k: rel(a[k], b[k]) for k in FIELDS}
    out["T_zonal_mean"] = rel(a["T"].mean(axis=0), b["T"].mean(axis=0))
    out["u_zonal_mean"] = rel(a["u"].mean(axis=0), b["u"].mean(axis=0))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--days", type=int, nargs="+", default=[1, 10, 100])
    ap.add_argument("--workload", default="hs_t42l20")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()

    import __graft_entry__

    __graft_entry__.build()
    import jgcm
    import oracle
    from jgcm import configs

    oracle.set_threads(args.threads)
    name = args.workload
    spd = configs.STEPS_PER_DAY[name]
    models = {}
    meshes = {}
    for key, backend, prec in (("oracle", oracle, None), ("gpu64", jgcm, "fp64"), ("gpu32", jgcm, "fp32")):
        mesh = configs.make_mesh(backend, name, precision=prec) if prec else configs.make_mesh(backend, name)
        md = backend.Model(mesh, configs.PARAMS[name])
        configs.init_held_suarez(backend, mesh, md)
        meshes[key], models[key] = mesh, md
    report = {"workload": name, "steps_per_day": spd, "initial_state": "Spectral_Initialize_Fields! with its "
              "vorticity seed + N(0,0.1^2) K grid noise on T, seed 20261203", "checkpoints": []}
    done = 0
    wall = {k: 0.0 for k in models}
    for day in sorted(args.days):
        steps = day * spd - done
        for k, md in models.items():
            t0 = time.perf_counter()
            md.step(steps)
            if k != "oracle":
                jgcm.lib().jgcm_mesh_synchronize(meshes[k]._h)
            wall[k] += time.perf_counter() - t0
        done = day * spd
        snap = {k: snapshot(md) for k, md in models.items()}
        row = {"day": day, "gpu64_vs_oracle": compare(snap["gpu64"], snap["oracle"]),
               "gpu32_vs_oracle": compare(snap["gpu32"], snap["oracle"]),
               "gpu32_vs_gpu64": compare(snap["gpu32"], snap["gpu64"]),
               "max_abs_u_oracle": float(np.abs(snap["oracle"]["u"]).max())}
        report["checkpoints"].append(row)
        print(json.dumps(row), file=sys.stderr, flush=True)
    report["wall_seconds"] = wall
    report["oracle_threads"] = args.threads
    txt = json.dumps(report, indent=1)
    print(txt)
    if args.out:
        with open(args.out, "w") as f:
            f.write(txt)


if __name__ == "__main__":
    main()
