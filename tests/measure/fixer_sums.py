#!/usr/bin/env python
"""The effect of the precision of the column energy integrals on the Held-Suarez energy fixer.

Compute_Corrections! (Spectral_Dynamics.jl:5-68) sums each column's energy integral sum_k E_k dp_k
(E = |u|^2/2 + c_p T) and folds the columns into the global mean.  The oracle runs HS T42L20 from the
bench state three times -- its FP64 column integrals; the same integrals in FP32 (oracle.F32_FIXER);
and with only their kinetic part in FP32 (oracle.F32_FIXER_KE, the GPU's arithmetic: c_p T summed in
FP64) -- and reports the difference of the temperature correction (K) per step and, after --days, the
relative L2 difference of T, u, v, ps.

  python tests/measure/fixer_sums.py [--days 1] [--threads N]
"""
from __future__ import annotations

import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [os.path.join(ROOT, "idealizedspectralgcm.jl_gb300"), os.path.join(ROOT, "oracle"), ROOT]

import numpy as np  # noqa: E402

WORKLOAD = "hs_t42l20"


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--days", type=float, default=1.0)
    ap.add_argument("--threads", type=int, default=os.cpu_count())
    args = ap.parse_args()
    import oracle
    from jgcm import configs

    oracle.set_threads(args.threads)
    nsteps = int(round(args.days * configs.STEPS_PER_DAY[WORKLOAD]))
    runs = {}
    for name, mask in (("fp64", 0), ("fp32_column_sums", oracle.F32_FIXER), ("fp32_kinetic_part", oracle.F32_FIXER_KE)):
        m = configs.make_mesh(oracle, WORKLOAD)
        md = oracle.Model(m, configs.PARAMS[WORKLOAD])
        configs.init_held_suarez(oracle, m, md)
        corr = []
        oracle.set_f32(mask)
        try:
            for _ in range(nsteps):
                md.step(1)
                corr.append(md.fixer_scalars()[5])
        finally:
            oracle.set_f32(0)
        runs[name] = (np.array(corr), {k: md.get(f) for k, f in (("T", "grid_t_c"), ("u", "grid_u_c"),
                                                                    ("v", "grid_v_c"), ("ps", "grid_ps_c"))})
    c64, s64 = runs["fp64"]
    doc = {"workload": f"HS T42L20 from the bench state, {nsteps} steps",
           "mean_abs_temperature_correction_K": float(np.mean(np.abs(c64)))}
    for name in ("fp32_column_sums", "fp32_kinetic_part"):
        c32, s32 = runs[name]
        d = np.abs(c32 - c64)
        doc[name] = {"temperature_correction_K": {"max_abs_difference": float(d.max()),
                                                  "mean_abs_difference": float(d.mean()),
                                                  "difference_summed_over_steps": float(np.sum(c32 - c64))},
                     "state_relative_l2_after": {k: float(np.linalg.norm((s32[k] - s64[k]).ravel())
                                                          / np.linalg.norm(s64[k].ravel())) for k in s64}}
    print(json.dumps(doc, indent=1))


if __name__ == "__main__":
    main()
