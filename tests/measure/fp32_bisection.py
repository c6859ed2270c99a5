#!/usr/bin/env python
"""Which stage of the mixed-precision Held-Suarez step owns its error against the FP64 oracle.

The oracle (FP64) can run any stage of the step in FP32 arithmetic (oracle.set_f32: the forward FFT,
the analysis Legendre sums, the synthesis Legendre sums, the inverse FFT) or round the outputs of the
grid stage (the column computations: tendencies, energy, grid state) or of the spectral stage (the
analysed tendencies and the state after the semi-implicit leapfrog) to FP32.  "+ T anomaly" cases
compute the geopotential from the temperature synthesised without its level means, the GPU's FP32
formulation, instead of from grid T stored in FP32.  Each stage alone, all
of them together, and -- with --gpu -- the GPU's mixed path itself are stepped from the same seeded
initial state (HS T42L20, the bench state) and compared with the all-FP64 oracle run: relative L2 of
the grid T, u, v, ps and of the spectral vorticity and divergence after --days simulated days.

  python tests/measure/fp32_bisection.py [--days 1] [--threads N] [--gpu] [--out bisect.json]
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

FIELDS = {"T": "grid_t_c", "u": "grid_u_c", "v": "grid_v_c", "ps": "grid_ps_c", "vor": "spe_vor_c",
          "div": "spe_div_c"}
WORKLOAD = "hs_t42l20"


def rel(a, b):
    n = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / n) if n > 0 else float(np.linalg.norm(a.ravel()))


def run_oracle(oracle, configs, mask, nsteps):
    m = configs.make_mesh(oracle, WORKLOAD)
    md = oracle.Model(m, configs.PARAMS[WORKLOAD])
    oracle.set_f32(0)
    configs.init_held_suarez(oracle, m, md)
    oracle.set_f32(mask)
    try:
        md.step(nsteps)
    finally:
        oracle.set_f32(0)
    return {k: md.get(f) for k, f in FIELDS.items()}


def run_gpu(oracle, configs, nsteps, precision):
    import jgcm

    m = configs.make_mesh(oracle, WORKLOAD)
    om = oracle.Model(m, configs.PARAMS[WORKLOAD])
    configs.init_held_suarez(oracle, m, om)
    gm = configs.make_mesh(jgcm, WORKLOAD, precision=precision)
    md = jgcm.Model(gm, configs.PARAMS[WORKLOAD])
    configs.copy_state(om, md, "held_suarez")
    md.step(nsteps)
    return {k: md.get(f) for k, f in FIELDS.items()}


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--days", type=float, default=1.0)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    ap.add_argument("--gpu", action="store_true", help="also step the GPU's fp32 path (needs libjgcm and a GPU)")
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    import oracle
    from jgcm import configs

    oracle.set_threads(args.threads)
    nsteps = int(round(args.days * configs.STEPS_PER_DAY[WORKLOAD]))
    st = oracle.F32_STAGES
    cases = [("fp64 (reference run)", 0)] + [(k, v) for k, v in st.items()]
    allm = sum(st.values())
    cases += [("all stages", allm), ("all but grid", allm - st["grid"]),
              ("transforms only", st["fft_fwd"] | st["analysis"] | st["synthesis"] | st["fft_inv"]),
              ("all + T anomaly", allm | oracle.F32_TANOM),
              ("synthesis + T anomaly", st["synthesis"] | oracle.F32_TANOM),
              ("inverse FFT + T anomaly", st["fft_inv"] | oracle.F32_TANOM)]
    t0 = time.perf_counter()
    ref = None
    rows = {}
    for name, mask in cases:
        out = run_oracle(oracle, configs, mask, nsteps)
        if ref is None:
            ref = out
            continue
        rows[name] = {k: rel(out[k], ref[k]) for k in FIELDS}
        print(f"{name:>18s}: " + "  ".join(f"{k} {v:.1e}" for k, v in rows[name].items()), flush=True)
    if args.gpu:
        out = run_gpu(oracle, configs, nsteps, "fp32")
        rows["GPU mixed (fp32)"] = {k: rel(out[k], ref[k]) for k in FIELDS}
        print(f"{'GPU mixed (fp32)':>18s}: " + "  ".join(f"{k} {v:.1e}" for k, v in rows["GPU mixed (fp32)"].items()))
    doc = {"workload": f"HS T42L20 from the bench state, {nsteps} steps ({args.days} days)",
           "stage_masks": st, "relative_l2_vs_fp64_oracle": rows, "seconds": time.perf_counter() - t0}
    if args.out:
        with open(args.out, "w") as f:
            json.dump(doc, f, indent=1)
    print(json.dumps(doc))


if __name__ == "__main__":
    main()
