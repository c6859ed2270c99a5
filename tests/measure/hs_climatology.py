#!/usr/bin/env python
"""Held-Suarez T42L20 climatology from the reference's own initial condition, on the GPU.

The reference's HS experiment (exp/HSt42/Run_HS.jl:6-14) runs 1200 days with 200 days of spin-up
from Spectral_Initialize_Fields! (isothermal 264 K at rest, its deterministic vorticity seed) and
plots the time-mean zonal means (exp/HSt42/Contourf_{U,T}.png).  This script runs the same
experiment with the library's on-device diagnostics (the reductions of Output_Manager.jl:81-145),
in the mixed (FP32) and FP64 paths, and reports the features the reference's figures show: the
zonal-mean jet maximum and where it sits, the near-surface equatorial temperature and the
equatorial tropopause minimum, plus the relative L2 difference between the two paths' climatologies.

  python tests/measure/hs_climatology.py [--days 1200] [--spinup 200] [--out clim.json]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [os.path.join(ROOT, "idealizedspectralgcm.jl_gb300"), ROOT]

import numpy as np  # noqa: E402


def features(mesh, u, t):
    lat = np.degrees(np.arcsin(mesh.sinth))
    nd = u.shape[1]
    sigma = (np.arange(nd) + 0.5) / nd  # even sigma: full levels between the half levels k/nd
    j, k = np.unravel_index(np.argmax(u), u.shape)
    eq = np.argsort(np.abs(lat))[:2]  # the two latitudes next to the equator
    trop = t[eq, :].mean(axis=0)
    return {"u_jet_max_m_s": float(u[j, k]), "u_jet_lat_deg": float(lat[j]), "u_jet_sigma": float(sigma[k]),
            "u_jet_max_other_hemisphere_m_s": float(u[(lat < 0) if lat[j] > 0 else (lat > 0), :].max()),
            "t_surface_equator_K": float(trop[-1]), "t_min_equator_K": float(trop.min()),
            "t_min_equator_sigma": float(sigma[int(np.argmin(trop))])}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--days", type=int, default=1200)
    ap.add_argument("--spinup", type=int, default=200)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    import __graft_entry__

    __graft_entry__.build()
    import jgcm
    from jgcm import configs

    name = "hs_t42l20"
    spd = configs.STEPS_PER_DAY[name]
    report = {"workload": "Held-Suarez T42L20, dt 1200 s, reference initial condition (isothermal 264 K at rest, "
                          "ps 1e5 Pa, the reference's vorticity seed, no noise)",
              "days": args.days, "spinup_days": args.spinup,
              "reference_figure": {"u_jet": "about 30-36 m/s near +-45 deg, sigma about 0.2-0.3",
                                   "t_surface_equator": "about 300-315 K",
                                   "t_tropopause_equator": "about 180-195 K"}}
    clim = {}
    for prec in ("fp32", "fp64"):
        mesh = configs.make_mesh(jgcm, name, precision=prec)
        md = jgcm.Model(mesh, configs.PARAMS[name])
        md.spectral_initialize_fields(None, True)
        t0 = time.perf_counter()
        md.step(spd * args.spinup)
        md.diagnostics(True)
        md.step(spd * (args.days - args.spinup))
        jgcm.lib().jgcm_mesh_synchronize(mesh._h)
        wall = time.perf_counter() - t0
        u, steps = md.read_diagnostics("u_zonal_mean")
        t, _ = md.read_diagnostics("t_zonal_mean")
        clim[prec] = (u, t)
        report[prec] = {"wall_seconds": wall, "sim_days_per_s": args.days / wall, "steps_averaged": steps,
                        **features(mesh, u, t)}
        print(prec, json.dumps(report[prec]), file=sys.stderr, flush=True)
    (u32, t32), (u64, t64) = clim["fp32"], clim["fp64"]
    report["fp32_vs_fp64_climatology_rel_l2"] = {
        "u_zonal_mean": float(np.linalg.norm(u32 - u64) / np.linalg.norm(u64)),
        "t_zonal_mean": float(np.linalg.norm(t32 - t64) / np.linalg.norm(t64))}
    txt = json.dumps(report, indent=1)
    print(txt)
    if args.out:
        with open(args.out, "w") as f:
            f.write(txt)


if __name__ == "__main__":
    main()
