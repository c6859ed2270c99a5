#!/usr/bin/env python
"""Held-Suarez T42L20 throughput on GB300: mixed precision vs the FP64 GPU path, at stated error.

One bench "step" is one simulated day (72 model steps of dt = 1200 s) of the Held-Suarez T42L20
dry dynamical core (128 x 64 Gaussian grid, 20 sigma levels), the reference's headline experiment
(exp/HSt42/HS.jl).  The initial state is the reference's Spectral_Initialize_Fields! (isothermal
264 K at rest, ps = 1e5 Pa, its vorticity seed) plus seeded N(0, 0.1^2) K white noise on the grid
(synthetic input; there is no dataset).

value      sim-days/s of the mixed-precision path (FP32 state, transforms and tendencies; FP64 wave-
           matrix solve and global sums), device-resident, CUDA-event timed over K sim-days, L2 flushed
           (256 MiB write) before every timed sim-day.
e2e        the same through the C ABI with host (pinned) buffers: per sim-day the whole state (one packed
           FP64 buffer of the 18 state arrays, reference layout) is uploaded, 72 steps run, and the
           state is read back into the same buffer; wall-clock.  fp64.e2e: the FP64 path the same way.
fp64       the FP64 GPU path on the same workload, same timing; error_vs_fp64 = relative L2 of
           T, u, v, ps of a mixed-precision twin against an FP64 twin stepped the same days from
           the same state (tensor_core_modes: the same for TF32x3 / BF16x3, with their speed).
tiles      both timed paths run the tiles the library's autotuner picks at start-up.
roofline   the dominant kernel of the mixed step (largest summed CUDA-event time), its algorithmic
           bytes per launch / its mean launch time, against the measured HBM copy bandwidth.
adjoint    the one-day gradient (HS T42L20, 72 steps, checkpoint every 8) in both paths: ms per
           gradient and the mixed gradient's error against the FP64 one.
config1    Barotropic T42 (128x64, 1 level) in FP64, 480 steps of 1800 s (10 days) from the Rossby-Haurwitz
           wave 4 + seeded noise: sim-days/s, whole-step roofline, end-state error against the FP64 oracle.
config2    Shallow water T85 (256x128), 864 steps of 600 s (6 days) from the unstable jet + seeded bump, in
           FP32 and split-BF16 (BF16x3): sim-days/s, whole-step roofline, per-field error against the FP64
           oracle at day 6.
config4    The batched ensemble as stated: 128 x HS T21L20, 32 x HS T42L20, 8 x SW T85 in split-BF16 with
           tiles from the autotuner, 30 simulated days per member in one graph launch per 24 windows:
           ensemble sim-days/s, and the first and last member of each truncation against the FP64 oracle
           (and against an FP64 GPU twin) after the 30 days.
headline   the last key: the headline figures in one short object (a truncated log keeps the end of stdout).
cpu_baseline  the FP64 C oracle (a restatement of the reference on the host) timed on a bounded sample.
--impl reference  times that oracle on all host threads on the same workload (the reference itself is
           Julia and Julia is not installed on the GPU hosts).
Multi-GPU: replicas only (independent members, different seeds), value = sum of sim-days / max time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "idealizedspectralgcm.jl_gb300")
sys.path[:0] = [PKG]

WORKLOAD = "hs_t42l20"
METRIC = "Held-Suarez T42L20 sim-days/s: mixed-precision vs FP64 GPU at stated error"
STATE_FIELDS = ["spe_vor_c", "spe_vor_p", "spe_div_c", "spe_div_p", "spe_lnps_c", "spe_lnps_p", "spe_t_c",
                "spe_t_p", "grid_u_c", "grid_u_p", "grid_v_c", "grid_v_p", "grid_ps_c", "grid_ps_p", "grid_t_c",
                "grid_t_p", "grid_vor", "grid_div"]


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def max_over_ranks(x: float, world: int) -> float:
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world: int):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# ------------------------------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
            time.sleep(0.4)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.f.name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        load = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


class L2Flush:
    """Writes a 256 MiB device buffer (> 129 MB L2) between timed iterations."""

    def __init__(self, device: int):
        self.buf = None
        try:
            import torch

            self.torch = torch
            self.buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{device}")
        except Exception as e:  # torch without CUDA
            log("L2 flush unavailable:", e)

    def __call__(self):
        if self.buf is not None:
            self.buf.fill_(1.0)
            self.torch.cuda.synchronize()


def pinned_like(arr):
    try:
        import torch

        t = torch.empty(arr.size, dtype=torch.float64 if arr.dtype.kind == "f" else torch.complex128,
                        pin_memory=True)
        out = t.numpy().reshape(arr.shape, order="F")
        out[...] = arr
        return out, t
    except Exception:
        return arr.copy(order="F"), None


# ------------------------------------------------------------------------------------------------
def algorithmic_bytes(name: str, N: int, nlat: int, nlon: int, nd: int, esize: int) -> float:
    """Bytes a kernel of the HS step must move per launch (each input read once, each output
    written once), for state element size `esize` (4 FP32, 8 FP64)."""
    G = nlon * nlat                     # grid points per level
    S = (N + 1) * (N + 4) // 2          # spectral modes n >= m per level (complex)
    F = (N + 1) * nlat                  # Fourier coefficients per column (complex)
    c = 2 * esize                       # complex element
    table = {
        "hs_column": (10 * nd + 5) * G * esize + (5 * nd + 1) * G * esize,
        "fft(tendencies)": (4 * nd + 1) * G * esize + (4 * nd + 1) * F * c,
        "g2s_legendre(vor,div,T,lnps)": (4 * nd + 1) * F * c + (3 * nd + 1) * S * c,
        "hs_implicit": (9 * nd + 3) * S * c + (6 * nd + 2) * S * c + (N + 1) * nd * nd * 8,
        # the new level (vor, div, u, v, T, ln ps) and the next step's gradients of ln ps and T, from
        # the same spectra; the FP32 path also writes T less its level means
        "s2g_legendre(vor,div,u,v,T,lnps,grad lnps,grad T)": (3 * nd + 1) * S * c + (7 * nd + 3) * F * c,
        "ifft(vor,div,u,v,T,lnps,grad lnps,grad T)": (7 * nd + 3) * F * c
        + ((7 * nd + 4) + (nd if esize == 4 else 0)) * G * esize,
        "hs_corr_reduce": (3 * nd + 1) * G * esize,
        "hs_corr_apply": 2 * (nd + 1) * G * esize,
    }
    return float(table[name])


def step_roofline(kt, N, nlat, nlon, nd, esize, s_per_step, peak):
    """The whole model step against the HBM roofline: the algorithmic bytes of its launches (one of
    each kernel of the step, the table of algorithmic_bytes) per measured step time."""
    alg = sum(algorithmic_bytes(k, N, nlat, nlon, nd, esize) for k in kt)
    ach = alg / s_per_step / 1e9
    return {"algorithmic_bytes": alg, "ms_per_step": 1e3 * s_per_step, "achieved": ach, "unit": "GB/s",
            "frac": ach / peak}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if one exists."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(p) as f:
            return json.load(f).get(kernel)
    except Exception:
        return None


def step_bytes(kind: str, N: int, nlat: int, nlon: int, nd: int, esize: int) -> float:
    """Algorithmic bytes of one model step from its transform counts: every transform reads its input
    and writes its output once, (#S2G + #G2S)(G + 2S) + #alpha (2G + 2S) reals of esize bytes per level
    (G = nlon nlat grid points, S = (N+1)(N+2) spectral reals).  Barotropic_Dynamics!: 3 S2G (vorticity,
    u, v) and the alpha pair of Vor_Div_From_Grid_UV!; Shallow_Water_Dynamics!: 7 S2G (two gradients,
    vor, div, h, u, v), 2 G2S (kinetic energy, h tendency) and the alpha pair."""
    G, S = nlon * nlat, (N + 1) * (N + 2)
    n_s2g, n_g2s, n_alpha = {"barotropic": (3, 0, 2), "shallow_water": (7, 2, 2)}[kind]
    return float(esize * nd * ((n_s2g + n_g2s) * (G + 2 * S) + n_alpha * (2 * G + 2 * S)))


def oracle_job(job):
    """One FP64 oracle run in a worker process (started with the spawn method): build the workload's
    initial state exactly as the GPU side does for it (configs.init_*), step it, return the prognostic
    fields.  job = (workload, init, seed, nsteps, threads)."""
    name, init, seed, nsteps, threads = job
    for pth in (PKG, os.path.join(ROOT, "oracle")):
        if pth not in sys.path:
            sys.path.insert(0, pth)
    import oracle
    from jgcm import configs

    oracle.set_threads(threads)
    m = configs.make_mesh(oracle, name)
    md = oracle.Model(m, configs.PARAMS[name])
    if init == "rh4":
        configs.init_barotropic_rh4(oracle, m, md, seed=seed)
    elif init == "jet":
        configs.init_shallow_water_jet(oracle, m, md, seed=seed)
    else:
        configs.init_held_suarez(oracle, m, md, seed=seed)
    t0 = time.perf_counter()
    md.step(nsteps)
    kind = configs.PARAMS[name]["kind"]
    return {"fields": {f: md.get(f) for f in configs.PROGNOSTIC[kind]}, "seconds": time.perf_counter() - t0}


def field_errors(gpu, ref, kind):
    """Relative L2 error per prognostic field (vorticity and divergence against the scale of the pair, a
    wind component against the wind), as the parity tests measure it."""
    import numpy as np

    scale = {"spe_div_c": ("spe_vor_c", "spe_div_c"), "spe_vor_c": ("spe_vor_c", "spe_div_c"),
             "grid_div": ("grid_vor", "grid_div"), "grid_vor": ("grid_vor", "grid_div"),
             "grid_u_c": ("grid_u_c", "grid_v_c"), "grid_v_c": ("grid_u_c", "grid_v_c")}
    out = {}
    for f, b in ref.items():
        den = np.linalg.norm(b.ravel())
        if f in scale and all(g in ref for g in scale[f]):
            den = max(den, math.sqrt(sum(np.linalg.norm(ref[g].ravel()) ** 2 for g in scale[f])))
        out[f] = float(np.linalg.norm((gpu[f] - b).ravel()) / (den if den > 0 else 1.0))
    return out


def whole_step_roofline(kind, name, prec, ms_per_step, kt):
    """Whole-step HBM roofline of a one-layer model (step_bytes / step time) and its longest kernel."""
    from jgcm import configs

    g = configs.GRIDS[name]
    alg = step_bytes(kind, g["num_fourier"], g["nlat"], g["nlon"], g["nd"], 8 if prec == "fp64" else 4)
    peak, pk = measured_peaks()
    ach = alg / (ms_per_step * 1e-3) / 1e9
    dom = max(kt, key=kt.get)
    return {"bound": "hbm", "kernel": "whole step", "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "peak_kind": pk, "algorithmic_bytes_per_step": alg,
            "longest_kernel": dom, "longest_kernel_share": kt[dom] / sum(kt.values())}


def one_layer_bench(jgcm, configs, name, init, prec, nsteps, engine=None):
    """A one-layer workload (barotropic or shallow water) on the GPU: the final prognostic fields of
    exactly nsteps steps from the seeded initial state (the first is the reference's forward step),
    and, on a twin with the autotuner's tiles, the CUDA-event time of nsteps - 1 steady steps (graph
    capture before timing steps the twin further), its per-kernel times and the whole-step roofline.
    engine="tcgen05" keeps a tensor-core mode's Legendre contractions on the tensor cores whatever the
    autotuner's engine choice (the mesh's knob, so the exact run uses it too)."""
    params = configs.PARAMS[name]
    kind = params["kind"]
    init_fn = configs.init_barotropic_rh4 if init == "rh4" else configs.init_shallow_water_jet
    m = configs.make_mesh(jgcm, name, precision=prec)
    tm = jgcm.Model(m, params)
    init_fn(jgcm, m, tm)
    tm.step(1)
    tuned = jgcm.autotune(tm, nsteps=24)["tuning"]
    if engine == "tcgen05":
        jgcm.set_tuning(tm, dict(tuned, simt_legendre=0))
        tuned = dict(jgcm.get_tuning(tm), autotuner_engine="simt" if tuned["simt_legendre"] else "tcgen05")
    ms = tm.time_steps(nsteps - 1)
    kt = tm.kernel_times(8)
    tm.close()
    md = jgcm.Model(m, params)
    init_fn(jgcm, m, md)
    md.step(nsteps)
    fields = {f: md.get(f) for f in configs.PROGNOSTIC[kind]}
    md.close()
    per_step = ms / (nsteps - 1)
    spd = configs.DAY / params["dt"]
    out = {"precision": prec, "steps": nsteps, "sim_days": nsteps * params["dt"] / configs.DAY,
           "sim_days_per_s": 1000.0 / (per_step * spd), "ms_per_step": per_step, "tuning": tuned,
           "roofline": whole_step_roofline(kind, name, prec, per_step, kt)}
    return out, fields


# ------------------------------------------------------------------------------------------------
def cpu_baseline(seconds_target: float = 12.0):
    """The FP64 C oracle on the host cores: bounded sample of the same workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from jgcm import configs

    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    m = configs.make_mesh(oracle, WORKLOAD)
    md = oracle.Model(m, configs.PARAMS[WORKLOAD])
    configs.init_held_suarez(oracle, m, md)
    md.step(1)  # init step
    t0 = time.perf_counter()
    md.step(2)
    per = (time.perf_counter() - t0) / 2
    n = max(2, min(720, int(seconds_target / max(per, 1e-6))))
    t0 = time.perf_counter()
    md.step(n)
    el = time.perf_counter() - t0
    spd = configs.STEPS_PER_DAY[WORKLOAD]
    return {"value": (n / spd) / el, "unit": "sim-days/s", "cores": threads, "kind": "port",
            "sample": f"{n} steady steps ({n / spd:.2f} sim-days) of HS T42L20 in FP64 on the C oracle, "
                      f"{threads} OpenMP threads, {el:.1f} s"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from jgcm import configs

    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    m = configs.make_mesh(oracle, WORKLOAD)
    md = oracle.Model(m, configs.PARAMS[WORKLOAD])
    configs.init_held_suarez(oracle, m, md)
    spd = configs.STEPS_PER_DAY[WORKLOAD]
    md.step(1)
    for _ in range(args.warmup):
        md.step(spd)
    t0 = time.perf_counter()
    md.step(spd * args.steps)
    el = time.perf_counter() - t0
    v = args.steps / el
    line = {"metric": METRIC, "value": v, "unit": "sim-days/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": "Held-Suarez T42L20 (128x64x20), dt 1200 s, 1 step = 1 sim-day",
                       "implementation": "FP64 C oracle restating the reference (Julia absent on the host)"},
            "cpu_baseline": {"value": v, "unit": "sim-days/s", "cores": threads, "kind": "port",
                             "sample": f"{args.steps} sim-days after {args.warmup} warm-up sim-days"},
            "e2e": {"value": v, "unit": "sim-days/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------------------
ENSEMBLE = [("hs_t21l20", 128), ("hs_t42l20", 32), ("sw_t85", 8)]  # the batched-ensemble configuration


def ensemble_bench(jgcm, configs, precisions, days=2):
    """Member-batched ensembles (one set of kernels advances every member of a truncation): HS
    T21L20 x128, HS T42L20 x32, SW T85 x8, each member with its own seeded initial state.  Reports,
    per truncation, member-sim-days/s stepped alone (CUDA events over `days` simulated days), and
    the whole ensemble advanced by 1200 s windows, one CUDA-graph launch per window whose branches
    step the three truncations concurrently (ensemble sim-days/s: every member advanced one day)."""
    out = {"members": {n: e for n, e in ENSEMBLE}, "days": days, "window_seconds": 1200}
    for prec in precisions:
        per, models, owned = {}, [], []
        for name, E in ENSEMBLE:
            params = configs.PARAMS[name]
            m = configs.make_mesh(jgcm, name, precision=prec)
            ens = jgcm.Model(m, params, members=E)
            one = jgcm.Model(m, params)
            for e in range(E):
                if params["kind"] == "held_suarez":
                    configs.init_held_suarez(jgcm, m, one, seed=configs.BASE_SEED + e)
                else:
                    configs.init_shallow_water_jet(jgcm, m, one, seed=configs.BASE_SEED + e)
                ens.copy_member(e, one)
            one.close()
            spd = configs.STEPS_PER_DAY[name]
            ens.step(spd)
            tuned = jgcm.autotune(ens, nsteps=8)["tuning"]
            t = sum(ens.time_steps(spd) for _ in range(days)) / 1000.0
            per[name] = {"member_sim_days_per_s": E * days / t, "ms_per_step": 1000.0 * t / (days * spd),
                         "tuning": tuned}
            if params["kind"] == "held_suarez":
                # the dominant kernel at ensemble scale: E members' algorithmic bytes per launch over
                # its CUDA-event launch time (eager steps), against the measured HBM copy bandwidth
                kt = ens.kernel_times(spd)
                dom = max(kt, key=kt.get)
                g = configs.GRIDS[name]
                alg = E * algorithmic_bytes(dom, g["num_fourier"], g["nlat"], g["nlon"], g["nd"],
                                            8 if prec == "fp64" else 4)
                peak, kind = measured_peaks()
                ach = alg / (kt[dom] * 1e-3) / 1e9
                per[name]["roofline"] = {"bound": "hbm", "kernel": dom, "achieved": ach, "peak": peak,
                                         "unit": "GB/s", "frac": ach / peak, "peak_kind": kind,
                                         "algorithmic_bytes": alg, "launch_ms": kt[dom]}
            models.append(ens)
            owned.append(m)
        group = jgcm.Ensemble(models, 1200)
        wpd = 86400 // 1200
        group.step(3)
        ms = group.time_windows(wpd * days)
        group.close()
        out[prec] = {"ensemble_sim_days_per_s": days / (ms / 1000.0), "ms_per_window": ms / (wpd * days),
                     "per_truncation_alone": per}
        for md in models:
            md.close()
    return out


def config4_bench(jgcm, configs, prec="bf16x3", days=30):
    """The batched-ensemble configuration as stated: 128 x HS T21L20, 32 x HS T42L20 and 8 x SW T85 (each
    member seeded base + e), Legendre contractions in split-BF16 (prec), tiles from the autotuner, `days`
    simulated days per member.  Every model takes its first window's steps on its own (the first step is
    the reference's forward step), then all three advance together by 1200 s windows, 24 windows per
    graph launch, CUDA-event timed.  The first and last member of each truncation start from the FP64 GPU
    initial state (equal to the oracle's to 1e-12) and are returned with an FP64 GPU twin stepped the same
    days, for the comparison against the FP64 oracle.  Returns (result, {(name, e): (member, fp64 twin)})."""
    win = 1200
    wpd = configs.DAY // win
    nwin = wpd * days
    chunk = 24
    pre = chunk  # windows each model takes on its own first: the first step and the rest of one chunk
    out = {"precision": prec, "members": {n: e for n, e in ENSEMBLE}, "days": days, "window_seconds": win,
           "windows_per_graph_launch": chunk}
    models, meshes, twins, per = [], [], {}, {}
    for name, E in ENSEMBLE:
        params = configs.PARAMS[name]
        kind = params["kind"]
        init = configs.init_held_suarez if kind == "held_suarez" else configs.init_shallow_water_jet
        steps_per_win = win // params["dt"]
        m = configs.make_mesh(jgcm, name, precision=prec)
        m64 = configs.make_mesh(jgcm, name, precision="fp64")
        ens = jgcm.Model(m, params, members=E)
        one = jgcm.Model(m, params)
        for e in range(E):
            if e in (0, E - 1):
                ref = jgcm.Model(m64, params)
                init(jgcm, m64, ref, seed=configs.BASE_SEED + e)
                configs.copy_state(ref, one, kind)
                twins[(name, e)] = ref
            else:
                init(jgcm, m, one, seed=configs.BASE_SEED + e)
            ens.copy_member(e, one)
        one.close()
        ens.step(1)
        per[name] = {"tuning": jgcm.autotune(ens, nsteps=8)["tuning"]}
        ens.step(pre * steps_per_win - 1)
        models.append(ens)
        meshes += [m, m64]
    group = jgcm.Ensemble(models, win)
    ms = group.time_windows(nwin - pre)
    group.close()
    timed_days = (nwin - pre) * win / configs.DAY
    out.update({"ensemble_sim_days_per_s": timed_days / (ms / 1000.0), "ms_per_window": ms / (nwin - pre),
                "timed_sim_days": timed_days, "per_truncation": per})
    states = {}
    for (name, E), ens in zip(ENSEMBLE, models):
        params = configs.PARAMS[name]
        kind = params["kind"]
        reader = jgcm.Model(ens.mesh, params)
        for e in (0, E - 1):
            reader.copy_member(0, ens, e)
            twin = twins[(name, e)]
            twin.step(days * configs.DAY // params["dt"])
            states[(name, e)] = ({f: reader.get(f) for f in configs.PROGNOSTIC[kind]},
                                 {f: twin.get(f) for f in configs.PROGNOSTIC[kind]})
            twin.close()
        reader.close()
        ens.close()
    return out, states


def precision_modes(jgcm, configs, days, timed=("tf32x3", "bf16x3")):
    """HS T42L20 in each mixed mode (FP32 SIMT; TF32x3 and BF16x3: the Legendre contractions on the
    tensor cores): the relative L2 error against an FP64 GPU twin stepped the same days from the same
    state, and for the tensor-core modes their tuned sim-days/s."""
    out = {}
    spd = configs.STEPS_PER_DAY[WORKLOAD]
    params = configs.PARAMS[WORKLOAD]
    m64 = configs.make_mesh(jgcm, WORKLOAD, precision="fp64")
    ref = jgcm.Model(m64, params)
    configs.init_held_suarez(jgcm, m64, ref)
    ref.step(spd * days)
    for prec in ("fp32",) + tuple(timed):
        m = configs.make_mesh(jgcm, WORKLOAD, precision=prec)
        md = jgcm.Model(m, params)
        configs.init_held_suarez(jgcm, m, md)
        md.step(spd * days)
        err = {k: configs.rel_l2(md.get(f), ref.get(f))
               for k, f in (("T", "grid_t_c"), ("u", "grid_u_c"), ("v", "grid_v_c"), ("ps", "grid_ps_c"))}
        out[prec] = {"after_sim_days": days, "error_vs_fp64": err}
        if prec in timed:
            tuned = jgcm.autotune(md, nsteps=spd)["tuning"]
            out[prec].update({"value": 1000.0 / md.time_steps(spd), "unit": "sim-days/s", "tuning": tuned})
            if tuned.get("simt_legendre"):  # the autotuner took the SIMT kernels: time tcgen05 too
                jgcm.set_tuning(md, dict(tuned, simt_legendre=0))
                out[prec]["value_tcgen05_legendre"] = 1000.0 / md.time_steps(spd)
    return out


def adjoint_bench(jgcm, configs, nsteps=72, checkpoint=8):
    """Gradient of the one-day loss (the adjoint configuration: HS T42L20, 72 steps, a checkpoint every
    8) in the mixed and FP64 paths: wall-clock per gradient (forward sweep, loss, recomputation and
    reverse sweep, host-timed after a warm-up) and the mixed gradient's error against the FP64 one."""
    import numpy as np

    out = {"workload": f"HS T42L20, {nsteps} steps from the seeded initial state, checkpoint every {checkpoint}; "
                       "loss = area-weighted mean squared difference of the final grid T from a seeded target",
           "gradient_of": "initial spectral T and k_f, k_a, k_s, dT_y, dtheta_z"}
    grads, ref = {}, None
    for prec in ("fp64", "fp32"):
        m = configs.make_mesh(jgcm, WORKLOAD, precision=prec)
        md = jgcm.Model(m, configs.PARAMS[WORKLOAD])
        configs.init_held_suarez(jgcm, m, md)
        if ref is None:
            ref = {k: md.get(k) for k in jgcm.STATE_FIELDS}
            tgt = np.asfortranarray(ref["grid_t_c"] + np.random.default_rng(5).standard_normal(ref["grid_t_c"].shape))
        times = []
        for i in range(4):
            for k in jgcm.STATE_FIELDS:
                md.set(k, ref[k])
            md.set_init_step(True)
            jgcm.lib().jgcm_mesh_synchronize(m._h)
            t0 = time.perf_counter()
            grads[prec] = jgcm.HS_Gradient(md, nsteps, tgt, checkpoint_every=checkpoint)
            if i:
                times.append(time.perf_counter() - t0)
        out[prec] = {"ms_per_gradient": 1e3 * min(times), "loss": grads[prec][0]}
        md.close()
    (l64, g64, p64), (l32, g32, p32) = grads["fp64"], grads["fp32"]
    out["fp32_vs_fp64"] = {"loss_rel": abs(l32 - l64) / l64,
                           "grad_T0_rel_l2": float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64)),
                           "grad_params_max_rel": float(np.max(np.abs(p32 - p64) / np.abs(p64)))}
    return out


def e2e_days(jgcm, mesh, params, tiles, init_state, ndays, flush):
    """End-to-end sim-days through the C ABI with host buffers: per sim-day, upload the whole state
    (jgcm_model_set_state: one pinned FP64 buffer of the 18 state arrays, reference layout), run 72
    steps, read it back into the same buffer (jgcm_model_get_state); wall-clock.  The first step (the
    reference's forward step) runs untimed; every timed day restarts from the host state."""
    spd = configs_steps_per_day(params)
    md = jgcm.Model(mesh, params)
    jgcm.set_tuning(md, tiles)
    buf, _keep = pinned_like(jgcm.pack_state(mesh, {f: init_state[f] for f in jgcm.STATE_FIELDS}))
    md.set_state(buf)
    md.step(1)
    md.get_state(out=buf)
    t = 0.0
    for _ in range(ndays):
        flush()
        t0 = time.perf_counter()
        md.set_state(buf)
        md.step(spd)
        md.get_state(out=buf)
        t += time.perf_counter() - t0
    md.close()
    return t, ndays, buf.nbytes


def configs_steps_per_day(params):
    return 86400 // params["dt"]


def oracle_checks(jobs, log_prefix="oracle checks"):
    """Run the FP64 oracle jobs (the reference values of the error figures) in spawned worker processes after
    the GPU work, on the host's cores; returns {job: result}."""
    import multiprocessing as mp

    cores = os.cpu_count() or 1
    workers = max(1, min(len(jobs), 4, cores))
    threads = max(1, cores // workers)
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(workers) as pool:
        res = pool.map(oracle_job, [j + (threads,) for j in jobs], chunksize=1)
    log(f"{log_prefix}: {len(jobs)} runs on {workers} x {threads} threads in {time.perf_counter() - t0:.1f} s")
    return dict(zip(jobs, res))


def run_jgcm(args):
    import numpy as np

    import jgcm
    from jgcm import configs

    rank, world, local = dist_env()
    jgcm.set_device(local)
    K, W = args.steps, args.warmup
    spd = configs.STEPS_PER_DAY[WORKLOAD]
    params = configs.PARAMS[WORKLOAD]
    g = configs.GRIDS[WORKLOAD]
    N, nlat, nlon, nd = g["num_fourier"], g["nlat"], g["nlon"], g["nd"]
    seed = configs.BASE_SEED + rank

    m64 = configs.make_mesh(jgcm, WORKLOAD, precision="fp64")
    mod64 = jgcm.Model(m64, params)
    configs.init_held_suarez(jgcm, m64, mod64, seed=seed)
    mmx = configs.make_mesh(jgcm, WORKLOAD, precision=args.precision)
    modmx = jgcm.Model(mmx, params)
    configs.copy_state(mod64, modmx, "held_suarez")  # identical start (FP64 init, rounded)
    init_state = {f: mod64.get(f) for f in STATE_FIELDS}

    flush = L2Flush(local)
    for mdl in (modmx, mod64):
        mdl.step(spd * W)  # warm-up sim-days (the first step is the reference's init step)
    # tiles chosen by the library's autotuner (timed on scratch copies; the models' states are untouched)
    tiles = {"mixed": jgcm.autotune(modmx, nsteps=spd)["tuning"], "fp64": jgcm.autotune(mod64, nsteps=spd)["tuning"]}
    # ---- timed: mixed precision
    clocks = ClockSampler(local)
    barrier(world)
    clocks.start()
    ms_mx = []
    for _ in range(K):
        flush()
        ms_mx.append(modmx.time_steps(spd))
    clk = clocks.stop()
    barrier(world)
    # ---- FP64 GPU path, same timing
    ms_64 = []
    for _ in range(K):
        flush()
        ms_64.append(mod64.time_steps(spd))
    days_done = W + K
    modes = precision_modes(jgcm, configs, days_done, timed=() if (args.no_ensemble or world > 1)
                            else ("tf32x3", "bf16x3"))
    err = modes["fp32"]["error_vs_fp64"]
    # ---- end to end through host buffers: the whole state in one pinned FP64 buffer (reference layout)
    t_e2e, ne2e, bytes_io = e2e_days(jgcm, mmx, params, tiles["mixed"], init_state, max(1, K), flush)
    t_e2e64, _, _ = e2e_days(jgcm, m64, params, tiles["fp64"], init_state, max(1, K), flush)
    # ---- per-kernel times and the roofline of the dominant kernel
    kt = modmx.kernel_times(spd)
    esize = 8 if args.precision == "fp64" else 4
    dom = max(kt, key=kt.get)
    alg = algorithmic_bytes(dom, N, nlat, nlon, nd, esize)
    peak, peak_kind = measured_peaks()
    achieved = alg / (kt[dom] * 1e-3) / 1e9
    # ---- aggregate over ranks
    t_mx = max_over_ranks(sum(ms_mx) / 1000.0, world)
    t_64 = max_over_ranks(sum(ms_64) / 1000.0, world)
    t_e2e = max_over_ranks(t_e2e, world)
    value = world * K / t_mx
    value64 = world * K / t_64
    if rank != 0:
        return 0
    base = None
    if not args.no_cpu_baseline and world == 1:
        try:
            base = cpu_baseline()
        except Exception as e:  # an oracle failure must not take the GPU result down
            base = {"value": None, "unit": "sim-days/s", "cores": os.cpu_count(), "kind": "port",
                    "sample": f"failed: {e}"}
    launches = modmx.launches_per_step()
    extra = {}
    if not args.no_ensemble and world == 1:
        try:
            # error of the tensor-core modes after the same W + K days as the FP64 run
            extra["tensor_core_modes"] = {k: v for k, v in modes.items() if k != "fp32"}
            extra["ensemble"] = ensemble_bench(jgcm, configs, ["fp32", "tf32x3"])
        except Exception as e:
            extra["ensemble_error"] = str(e)
    if not args.no_adjoint and world == 1:
        try:
            extra["adjoint"] = adjoint_bench(jgcm, configs)
        except Exception as e:
            extra["adjoint_error"] = str(e)
    if not args.no_configs and world == 1:
        try:
            extra.update(config_legs(jgcm, configs, args))
        except Exception as e:
            extra["configs_error"] = f"{type(e).__name__}: {e}"
    line = {
        "metric": METRIC, "value": value, "unit": "sim-days/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": 1000.0 * t_mx / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.precision != "fp64" else "f64", "data": "synthetic",
        "config": {"workload": "Held-Suarez T42L20 (128x64 Gaussian, 20 sigma levels), dt 1200 s; 1 step = 1 "
                               "sim-day = 72 model steps",
                   "precision": f"{args.precision} state/transforms/tendencies, fp64 semi-implicit solve and "
                                f"global mass/energy sums",
                   "initial_state": "isothermal 264 K at rest, ps 1e5 Pa, reference vorticity seed, seeded "
                                    "N(0,0.1^2) K grid noise",
                   "l2": "flushed (256 MiB write) before every timed sim-day; working set ~20 MB is otherwise "
                         "L2-resident within a day", "parallelism": f"replicas x{world}",
                   "ms_per_model_step": 1000.0 * t_mx / (K * spd),
                   "tiles": {"chosen_by": "jgcm.autotune (coordinate search, CUDA-event timed)", **tiles}},
        "fp64": {"value": value64, "unit": "sim-days/s", "ms_per_step": 1000.0 * t_64 / K,
                 "e2e": {"value": world * ne2e / t_e2e64, "unit": "sim-days/s", "h2d_bytes_per_step": bytes_io,
                         "d2h_bytes_per_step": bytes_io}},
        "speedup_vs_fp64": value / value64,
        "error_vs_fp64": {"after_sim_days": round(days_done, 3), **{k: v for k, v in err.items()}},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind, "algorithmic_bytes": alg,
                     "launch_ms": kt[dom], "traffic": profile_traffic(dom),
                     "step_kernels_ms": {k: round(v, 5) for k, v in kt.items()},
                     "whole_step": step_roofline(kt, N, nlat, nlon, nd, esize, t_mx / (K * spd), peak)},
        "cpu_baseline": base,
        "e2e": {"value": world * ne2e / t_e2e, "unit": "sim-days/s", "h2d_bytes_per_step": bytes_io,
                "d2h_bytes_per_step": bytes_io},
        "gpu_launches": launches * spd * K,
        "clocks": clk,
        **extra,
    }
    line["headline"] = headline_summary(line)
    print(json.dumps(line), flush=True)
    return 0


def headline_summary(line):
    """The headline figures in one short object, printed last (the end of stdout is what survives in a
    truncated log): mixed vs FP64 sim-days/s and their errors, e2e, tensor-core modes, configs 1, 2, 4."""
    r = lambda x, n=4: None if x is None else float(f"{x:.{n}g}")  # noqa: E731
    ns = {"mixed_sim_days_per_s": r(line["value"]), "fp64_sim_days_per_s": r(line["fp64"]["value"]),
          "speedup_vs_fp64": r(line["speedup_vs_fp64"], 3),
          "error_vs_fp64": {k: r(v, 2) for k, v in line["error_vs_fp64"].items()},
          "e2e_mixed": r(line["e2e"]["value"]), "e2e_fp64": r(line["fp64"]["e2e"]["value"]),
          "roofline_frac": r(line["roofline"]["frac"], 3),
          "whole_step_roofline_frac": r(line["roofline"]["whole_step"]["frac"], 3)}
    tc = line.get("tensor_core_modes") or {}
    ns["tensor_core_sim_days_per_s"] = {k: r(v.get("value")) for k, v in tc.items()}
    c1 = line.get("config1")
    if c1:
        ns["config1_barotropic_t42_fp64"] = {"sim_days_per_s": r(c1["sim_days_per_s"]),
                                             "max_error_vs_oracle": r(c1.get("max_error_vs_oracle"), 2)}
    c2 = line.get("config2")
    if c2:
        ns["config2_sw_t85"] = {p: {"sim_days_per_s": r(v["sim_days_per_s"]),
                                    "max_error_vs_oracle": r(v.get("max_error_vs_oracle"), 2)}
                                for p, v in c2.items() if isinstance(v, dict) and "sim_days_per_s" in v}
    c4 = line.get("config4")
    if c4:
        ns["config4_ensemble_bf16x3"] = {"ensemble_sim_days_per_s": r(c4["ensemble_sim_days_per_s"]),
                                         "days": c4["days"]}
    adj = line.get("adjoint")
    if adj:
        ns["adjoint_ms_per_gradient"] = {"fp32": r(adj["fp32"]["ms_per_gradient"]),
                                         "fp64": r(adj["fp64"]["ms_per_gradient"])}
    return ns


def config_legs(jgcm, configs, args):
    """Configs 1, 2 and 4 on the GPU, then their errors against the FP64 oracle (run in
    worker processes after the GPU work)."""
    base = configs.BASE_SEED
    out = {}
    c1, f1 = one_layer_bench(jgcm, configs, "barotropic_t42", "rh4", "fp64", 480)
    out["config1"] = dict(c1, workload="Barotropic T42 (128x64, 1 level), RH wave 4 + seeded noise, dt 1800 s, "
                                       "480 steps (10 days), FP64")
    c2 = {"workload": "Shallow water T85 (256x128), unstable jet + seeded bump, dt 600 s, 864 steps (6 days)"}
    f2 = {}
    for prec in ("fp32", "bf16x3"):  # split-BF16 as stated: the Legendre contractions on tcgen05
        c2[prec], f2[prec] = one_layer_bench(jgcm, configs, "sw_t85", "jet", prec, 864,
                                             engine="tcgen05" if prec == "bf16x3" else None)
    out["config2"] = c2
    c4, st4 = config4_bench(jgcm, configs, days=args.ensemble_days)
    out["config4"] = c4
    if args.no_oracle_checks:
        return out
    jobs = [("barotropic_t42", "rh4", base, 480), ("sw_t85", "jet", base, 864)]
    for (name, e) in st4:
        kind = configs.PARAMS[name]["kind"]
        jobs.append((name, "hs" if kind == "held_suarez" else "jet", base + e,
                     args.ensemble_days * configs.DAY // configs.PARAMS[name]["dt"]))
    jobs.sort(key=lambda j: -j[3] * (20 if j[0] == "hs_t42l20" else 4 if j[0] == "hs_t21l20" else 1))
    res = oracle_checks(jobs)
    ref = res[("barotropic_t42", "rh4", base, 480)]["fields"]
    e1 = field_errors(f1, ref, "barotropic")
    out["config1"]["error_vs_oracle"] = e1
    out["config1"]["max_error_vs_oracle"] = max(e1.values())
    ref = res[("sw_t85", "jet", base, 864)]["fields"]
    for prec in ("fp32", "bf16x3"):
        e2 = field_errors(f2[prec], ref, "shallow_water")
        c2[prec]["error_vs_oracle_day6"] = e2
        c2[prec]["max_error_vs_oracle"] = max(e2.values())
    errs = {}
    for (name, e), (member, twin) in st4.items():
        kind = configs.PARAMS[name]["kind"]
        job = next(j for j in jobs if j[0] == name and j[2] == base + e)
        ref = res[job]["fields"]
        errs[f"{name}[{e}]"] = {"bf16x3_vs_oracle": field_errors(member, ref, kind),
                               "fp64_gpu_vs_oracle": field_errors(twin, ref, kind),
                               "bf16x3_vs_fp64_gpu": field_errors(member, twin, kind)}
    c4["errors_after_days"] = {"days": args.ensemble_days, "members": errs}
    out["oracle_check_seconds"] = {f"{j[0]}:{j[2]}": round(v["seconds"], 2) for j, v in res.items()}
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5, help="timed sim-days")
    ap.add_argument("--warmup", type=int, default=3, help="warm-up sim-days")
    ap.add_argument("--impl", default="jgcm", choices=["jgcm", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64", "tf32x3", "bf16x3"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the ensemble and tensor-core side runs")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the one-day gradient timing")
    ap.add_argument("--no-configs", action="store_true", help="skip configs 1, 2 and 4 (barotropic T42, SW T85, "
                                                              "the 30-day split-BF16 ensemble)")
    ap.add_argument("--no-oracle-checks", action="store_true",
                    help="configs 1, 2, 4 without their errors against the FP64 oracle")
    ap.add_argument("--ensemble-days", type=int, default=30, help="simulated days per member of config 4")
    ap.add_argument("--profile", action="store_true",
                    help="only the mixed-precision headline model: --warmup then --steps sim-days with the tiles of "
                         "--tiles (no autotuning, no other model), a short launch sequence for ncu")
    ap.add_argument("--tiles", default="4,4,4,0",
                    help="lanes per column, S2G, G2S, FFT columns per block, or 'auto' for the autotuner (--profile)")
    ap.add_argument("--profile-members", type=int, default=1, metavar="E",
                    help="--profile: E member-batched members (seeds base + e); after the timing, one eager "
                         "step runs inside a CUDA profiler range (ncu --profile-from-start off captures it)")
    ap.add_argument("--ensemble-only", default=None, metavar="PRECISIONS",
                    help="run only the batched-ensemble measurement for these precisions (comma list, e.g. "
                         "fp32,tf32x3) over --steps days and print its JSON (for profiling the ensemble kernels)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world, _ = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    try:
        if args.impl == "reference":
            return run_reference(args)
        if args.profile:
            import jgcm
            from jgcm import configs

            jgcm.set_device(int(os.environ.get("LOCAL_RANK", 0)))
            name = WORKLOAD if args.profile_members == 1 else "hs_t21l20"
            spd = configs.STEPS_PER_DAY[name]
            m = configs.make_mesh(jgcm, name, precision=args.precision)
            E = args.profile_members
            md = jgcm.Model(m, configs.PARAMS[name], members=E)
            if E == 1:
                configs.init_held_suarez(jgcm, m, md)
            else:
                one = jgcm.Model(m, configs.PARAMS[name])
                for e in range(E):
                    configs.init_held_suarez(jgcm, m, one, seed=configs.BASE_SEED + e)
                    md.copy_member(e, one)
                one.close()
            md.step(1)
            if args.tiles == "auto":
                jgcm.autotune(md, nsteps=8)
            else:
                jgcm.set_tuning(md, dict(zip(jgcm.TUNING_KNOBS, [int(x) for x in args.tiles.split(",")])))
            md.step(spd * args.warmup)
            ms = [md.time_steps(spd) for _ in range(args.steps)]
            import ctypes

            cuda = ctypes.CDLL("libcuda.so.1")
            cuda.cuProfilerStart()
            kt = md.kernel_times(1)  # one eager step, its kernels serialised
            cuda.cuProfilerStop()
            print(json.dumps({"profile": name, "members": E, "precision": args.precision,
                              "tuning": jgcm.get_tuning(md), "ms_per_sim_day": ms, "kernel_ms": kt}), flush=True)
            return 0
        if args.ensemble_only:
            import jgcm
            from jgcm import configs

            jgcm.set_device(int(os.environ.get("LOCAL_RANK", 0)))
            res = ensemble_bench(jgcm, configs, args.ensemble_only.split(","), days=max(1, args.steps))
            print(json.dumps({"ensemble": res}), flush=True)
            return 0
        return run_jgcm(args)
    finally:
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
