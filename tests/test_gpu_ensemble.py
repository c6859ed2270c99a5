"""Ensembles: members advanced together by the same kernels must match one-member runs.

Each member gets its own seeded initial state (one-member models initialised through the
reference's Spectral_Initialize_Fields! / the SW jet / the RH4 wave, then copied in).  After the
same number of steps, every member copied back out must equal the one-member model stepped alone:
the per-column arithmetic is identical and the global sums of the fixers are per member and fold in
the same order, so the tolerance is 1e-12 (FP64) / 1e-6 (FP32 and tensor-core modes, whose tile
boundaries move with the column count).
"""
import numpy as np
import pytest

from jgcm import configs
from test_gpu_models import MIXED_TOL, _compare

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-6, "tf32x3": 1e-6, "bf16x3": 1e-6}


def _init(jg, kind, mesh, model, seed):
    if kind == "held_suarez":
        configs.init_held_suarez(jg, mesh, model, seed=seed)
    elif kind == "shallow_water":
        configs.init_shallow_water_jet(jg, mesh, model, seed=seed)
    else:
        configs.init_barotropic_rh4(jg, mesh, model, seed=seed)


@pytest.mark.parametrize("name,prec,members,steps", [
    ("hs_t21l20", "fp64", 3, 5), ("hs_t21l20", "fp32", 5, 7), ("hs_t42l20", "tf32x3", 3, 4),
    ("hs_t21l20", "bf16x3", 4, 4), ("sw_t85", "fp32", 3, 5), ("sw_t85", "tf32x3", 2, 4),
    ("barotropic_t42", "fp64", 4, 6)])
def test_ensemble_matches_members(jg, name, prec, members, steps):
    params = configs.PARAMS[name]
    kind = params["kind"]
    mesh = configs.make_mesh(jg, name, precision=prec)
    ens = jg.Model(mesh, params, members=members)
    singles = []
    for e in range(members):
        md = jg.Model(mesh, params)
        _init(jg, kind, mesh, md, configs.BASE_SEED + e)
        ens.copy_member(e, md)
        singles.append(md)
    ens.step(steps)
    for md in singles:
        md.step(steps)
    out = jg.Model(mesh, params)
    worst = 0.0
    for e, md in enumerate(singles):
        out.copy_member(0, ens, e)
        for f in configs.PROGNOSTIC[kind]:
            err = configs.rel_l2(out.get(f), md.get(f))
            worst = max(worst, err)
            assert err < TOL[prec], (e, f, err)
    # members with different seeds really differ
    a, b = jg.Model(mesh, params), jg.Model(mesh, params)
    a.copy_member(0, ens, 0)
    b.copy_member(0, ens, members - 1)
    f = "grid_t_c" if kind == "held_suarez" else "grid_vor"
    assert configs.rel_l2(a.get(f), b.get(f)) > 1e-12
    print(name, prec, members, "worst", worst)


@pytest.mark.parametrize("name,members", [("hs_t21l20", 24), ("hs_t42l20", 8)])
def test_large_fp32_ensemble_matches_oracle(jg, orc, name, members):
    """Member-batched FP32 steps at scale: enough members that the analysis runs one lane per
    output (k_g2s_legendre<T, 1>) and, at T21, every zonal FFT one row per thread (k_fft_rows /
    k_ifft_rows).  The first and last members, stepped from a developed flow, equal the oracle's
    steps (the FP32 step tolerance of the single-member parity tests)."""
    params = configs.PARAMS[name]
    gm, om = configs.make_mesh(jg, name, precision="fp32"), configs.make_mesh(orc, name)
    ens = jg.Model(gm, params, members=members)
    refs = {}
    for e in range(members):
        omod = orc.Model(om, params)
        configs.init_held_suarez(orc, om, omod, seed=configs.BASE_SEED + e)
        configs.add_hs_flow(orc, om, omod)
        one = jg.Model(gm, params)
        configs.copy_state(omod, one, "held_suarez")
        ens.copy_member(e, one)
        if e in (0, members - 1):
            refs[e] = omod
    ens.step(1)
    ens.step(3)
    for omod in refs.values():
        omod.step(4)
    out = jg.Model(gm, params)
    for e, omod in refs.items():
        out.copy_member(0, ens, e)
        _compare(out, omod, "held_suarez", MIXED_TOL["fp32"])


def test_ensemble_rejects_direct_field_access(jg):
    params = configs.PARAMS["hs_t21l20"]
    mesh = configs.make_mesh(jg, "hs_t21l20", precision="fp32")
    ens = jg.Model(mesh, params, members=2)
    with pytest.raises(AssertionError):
        ens.get("grid_t_c")
    md = jg.Model(mesh, params)
    with pytest.raises(AssertionError):
        md.copy_member(1, ens, 0)  # member out of range


def _ready(jg, name, prec, members, seed0):
    params = configs.PARAMS[name]
    mesh = configs.make_mesh(jg, name, precision=prec)
    ens = jg.Model(mesh, params, members=members)
    one = jg.Model(mesh, params)
    for e in range(members):
        _init(jg, params["kind"], mesh, one, seed0 + e)
        ens.copy_member(e, one)
    ens.step(1)  # the first (init) step runs eagerly
    return mesh, ens


def test_uneven_ensemble_one_graph_per_window(jg):
    """HS T21L20 x3, HS T42L20 x2 and SW T85 x2 (dt 600 s, two steps per 1200 s window) advanced by
    ensemble windows equal the same models advanced one by one."""
    specs = [("hs_t21l20", "fp32", 3), ("hs_t42l20", "fp32", 2), ("sw_t85", "fp32", 2)]
    a = [_ready(jg, n, p, e, configs.BASE_SEED + 10 * i) for i, (n, p, e) in enumerate(specs)]
    b = [_ready(jg, n, p, e, configs.BASE_SEED + 10 * i) for i, (n, p, e) in enumerate(specs)]
    ens = jg.Ensemble([m for _, m in a], 1200)
    windows = 4
    ens.step(windows - 1)
    ms = ens.time_windows(1)
    assert ms > 0
    for (name, _, _), (_, md) in zip(specs, b):
        md.step(windows * 1200 // configs.PARAMS[name]["dt"])
    for (name, prec, E), (mesh_a, ma), (mesh_b, mb) in zip(specs, a, b):
        kind = configs.PARAMS[name]["kind"]
        x, y = jg.Model(mesh_a, configs.PARAMS[name]), jg.Model(mesh_b, configs.PARAMS[name])
        for e in range(E):
            x.copy_member(0, ma, e)
            y.copy_member(0, mb, e)
            for f in configs.PROGNOSTIC[kind]:
                assert configs.rel_l2(x.get(f), y.get(f)) < 1e-12, (name, e, f)
    ens.close()


def test_uneven_ensemble_rejects_bad_windows(jg):
    mesh, md = _ready(jg, "hs_t21l20", "fp32", 1, configs.BASE_SEED)
    with pytest.raises(AssertionError):
        jg.Ensemble([md], 1000)  # not a multiple of dt = 1200 s
    fresh = jg.Model(mesh, configs.PARAMS["hs_t21l20"])
    with pytest.raises(AssertionError):
        jg.Ensemble([fresh], 1200)  # still in its first step


def test_autotuner_keeps_results_and_caches(jg, tmp_path):
    """The autotuner only changes tiles: the tuned model steps to the same state as an untuned twin
    (FP64: identical arithmetic per column; the tile sizes only regroup the same sums), and a second
    call is served from the JSON cache."""
    name = "hs_t21l20"
    params = configs.PARAMS[name]
    mesh_a = configs.make_mesh(jg, name, precision="fp64")
    mesh_b = configs.make_mesh(jg, name, precision="fp64")
    a, b = jg.Model(mesh_a, params, members=2), jg.Model(mesh_b, params, members=2)
    one = jg.Model(mesh_a, params)
    for e in range(2):
        configs.init_held_suarez(jg, mesh_a, one, seed=configs.BASE_SEED + e)
        a.copy_member(e, one)
    two = jg.Model(mesh_b, params)
    for e in range(2):
        configs.init_held_suarez(jg, mesh_b, two, seed=configs.BASE_SEED + e)
        b.copy_member(e, two)
    a.step(2)
    b.step(2)
    cache = str(tmp_path / "tiles.json")
    first = jg.autotune(a, nsteps=4, cache=cache)
    assert set(first["tuning"]) == set(jg.TUNING_KNOBS) and first["ms_per_step"] > 0
    again = jg.autotune(a, nsteps=4, cache=cache)
    assert again == first
    assert jg.get_tuning(a)["lanes_per_column"] in (1, 2, 4, 8)
    a.step(6)
    b.step(6)
    x, y = jg.Model(mesh_a, params), jg.Model(mesh_b, params)
    for e in range(2):
        x.copy_member(0, a, e)
        y.copy_member(0, b, e)
        for f in configs.PROGNOSTIC["held_suarez"]:
            assert configs.rel_l2(x.get(f), y.get(f)) < 1e-10, (e, f)
    with pytest.raises(AssertionError):
        jg.set_tuning(a, {"lanes_per_column": 3})
    # the C ABI writes no more knobs than the caller's buffer holds (n = 4 of the 5)
    import ctypes as C
    buf = (C.c_int * 6)(*([-7] * 6))
    ms = C.c_float()
    assert jg.lib().jgcm_model_autotune(a._h, 2, buf, 4, C.byref(ms)) == 0
    assert list(buf)[4:] == [-7, -7] and ms.value > 0
    assert list(buf)[:4] == [jg.get_tuning(a)[k] for k in jg.TUNING_KNOBS[:4]]
    assert jg.lib().jgcm_model_autotune(a._h, 2, buf, 3, C.byref(ms)) == -1  # fewer than 4: refused


@pytest.mark.gpu
def test_legendre_engine_knob(jg):
    """A tensor-core mesh can run its Legendre contractions on the FP32 SIMT kernels (the autotuner's
    fifth knob): the step then equals the FP32 mesh's step, and switching back reproduces the
    tensor-core result; on an FP32 mesh the knob has nothing to switch and stays 0."""
    name = "hs_t21l20"
    params = configs.PARAMS[name]
    m32 = configs.make_mesh(jg, name, precision="fp32")
    mtc = configs.make_mesh(jg, name, precision="tf32x3")
    r32, rtc = jg.Model(m32, params), jg.Model(mtc, params)
    configs.init_held_suarez(jg, m32, r32)
    start = {f: r32.get(f) for f in jg.STATE_FIELDS}  # everything a step reads
    for f, v in start.items():
        rtc.set(f, v)
    r32.step(4)
    rtc.step(4)
    tc_result = rtc.get("grid_t_c")
    simt = jg.Model(mtc, params)
    for f, v in start.items():
        simt.set(f, v)
    jg.set_tuning(simt, {"simt_legendre": 1})
    assert jg.get_tuning(simt)["simt_legendre"] == 1
    simt.step(4)
    assert configs.rel_l2(simt.get("grid_t_c"), r32.get("grid_t_c")) < 1e-12
    back = jg.Model(mtc, params)
    for f, v in start.items():
        back.set(f, v)
    jg.set_tuning(back, {"simt_legendre": 0})
    back.step(4)
    assert configs.rel_l2(back.get("grid_t_c"), tc_result) < 1e-12
    jg.set_tuning(r32, {"simt_legendre": 1})
    assert jg.get_tuning(r32)["simt_legendre"] == 0
