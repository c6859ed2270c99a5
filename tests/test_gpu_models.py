"""GPU model steps vs the FP64 oracle from identical states, through the C ABI.

The GPU model is loaded with the oracle's state (copy_state), both advance the same steps,
and every prognostic field is compared by relative L2.  Tolerances: FP64 path 1e-10 after a
few steps (summation order differs; HS's chaotic growth is slow over a few steps); the one-layer
models' FP32 path 5e-5; Held-Suarez's mixed modes per field (MIXED_TOL).  The barotropic T42
workload runs its full 480 steps (10 days) in FP64.
"""
import numpy as np
import pytest

from jgcm import configs

pytestmark = pytest.mark.gpu


def _pair(jg, orc, name, prec):
    params = configs.PARAMS[name]
    gm = configs.make_mesh(jg, name, precision=prec)
    om = configs.make_mesh(orc, name)
    return gm, om, jg.Model(gm, params), orc.Model(om, params)


# divergence (or vorticity) can be pure roundoff or just being born (a resting, non-divergent or purely
# divergent start), so each is measured against the scale of the pair (vorticity, divergence) -- the
# size of the velocity gradient -- and a wind component against the wind (u, v)
_SCALE = {"spe_div_c": ("spe_vor_c", "spe_div_c"), "spe_vor_c": ("spe_vor_c", "spe_div_c"),
          "spe_div_p": ("spe_vor_p", "spe_div_p"), "spe_vor_p": ("spe_vor_p", "spe_div_p"),
          "grid_div": ("grid_vor", "grid_div"), "grid_vor": ("grid_vor", "grid_div"),
          "grid_u_c": ("grid_u_c", "grid_v_c"), "grid_v_c": ("grid_u_c", "grid_v_c")}

# Per-field step tolerances of the mixed modes after a few steps from a developed flow (relative L2).
# Thermodynamic fields (T, ln ps / ps, the shallow-water height) are transformed and stepped with no
# cancellation and stay near FP32 rounding (measured <= 1e-6); the dynamics (vorticity, divergence,
# winds) carry the FP32 conditioning of the divergence tendency, a Laplacian of an energy whose
# dynamically active part is ~1e-3 of its size (measured <= 5e-5).  BF16x3 splits each operand into
# two 8-bit-mantissa halves (~16 bits kept, against FP32's 24), so its bounds are wider.
_THERMO = ("spe_t_c", "spe_t_p", "grid_t_c", "grid_t_p", "spe_lnps_c", "grid_ps_c", "grid_ps_p")
MIXED_TOL = {"fp32": {"default": 2e-4, **{f: 5e-6 for f in _THERMO}},
             "tf32x3": {"default": 2e-4, **{f: 5e-6 for f in _THERMO}},
             "bf16x3": {"default": 5e-4, **{f: 2e-5 for f in _THERMO}}}


def _compare(gmod, omod, kind, tol):
    """Relative L2 error of every prognostic field; `tol` is a bound for all of them or a dict of
    per-field bounds with a "default"."""
    errs = {}
    names = set(configs.PROGNOSTIC[kind]) | {"spe_div_p"}
    for f in configs.PROGNOSTIC[kind]:
        a, b = gmod.get(f), omod.get(f)
        den = np.linalg.norm(b.ravel())
        if f in _SCALE and all(g in names for g in _SCALE[f]):
            den = max(den, np.sqrt(sum(np.linalg.norm(omod.get(g).ravel()) ** 2 for g in _SCALE[f])))
        errs[f] = float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
    print(kind, {k: f"{v:.2e}" for k, v in errs.items()})
    bound = (lambda f: tol.get(f, tol["default"])) if isinstance(tol, dict) else (lambda f: tol)
    bad = {k: (v, bound(k)) for k, v in errs.items() if not v < bound(k)}
    assert not bad, f"fields above their bounds (error, bound): {bad}"
    return errs


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("fp32", 5e-5)])
def test_barotropic_steps(jg, orc, prec, tol):
    gm, om, gmod, omod = _pair(jg, orc, "barotropic_t42", prec)
    configs.init_barotropic_rh4(orc, om, omod)
    configs.copy_state(omod, gmod, "barotropic")
    for n in (1, 1, 5):
        gmod.step(n)
        omod.step(n)
        _compare(gmod, omod, "barotropic", tol)
    assert not gmod.init_step and not omod.init_step


def test_barotropic_10_days_fp64(jg, orc):
    gm, om, gmod, omod = _pair(jg, orc, "barotropic_t42", "fp64")
    configs.init_barotropic_rh4(orc, om, omod)
    configs.copy_state(omod, gmod, "barotropic")
    gmod.step(480)
    omod.step(480)
    _compare(gmod, omod, "barotropic", 1e-9)


def test_barotropic_init_parity(jg, orc):
    """The IC driver run on the GPU library reproduces the oracle's."""
    gm, om, gmod, omod = _pair(jg, orc, "barotropic_t42", "fp64")
    configs.init_barotropic_rh4(orc, om, omod)
    configs.init_barotropic_rh4(jg, gm, gmod)
    _compare(gmod, omod, "barotropic", 1e-12)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("fp32", 5e-5)])
def test_shallow_water_steps(jg, orc, prec, tol):
    gm, om, gmod, omod = _pair(jg, orc, "sw_t85", prec)
    configs.init_shallow_water_jet(orc, om, omod)
    configs.copy_state(omod, gmod, "shallow_water")
    for n in (1, 1, 4):
        gmod.step(n)
        omod.step(n)
        _compare(gmod, omod, "shallow_water", tol)


@pytest.mark.parametrize("name", ["hs_t21l10", "hs_t42l20"])
def test_held_suarez_init_parity(jg, orc, name):
    gm, om, gmod, omod = _pair(jg, orc, name, "fp64")
    noise = configs.hs_temperature_noise(om)
    omod.spectral_initialize_fields(noise, True)
    gmod.spectral_initialize_fields(noise, True)
    _compare(gmod, omod, "held_suarez", 1e-12)


def _hs_developed(jg, orc, name, prec):
    gm, om, gmod, omod = _pair(jg, orc, name, prec)
    omod.spectral_initialize_fields(configs.hs_temperature_noise(om), True)
    configs.add_hs_flow(orc, om, omod)
    configs.copy_state(omod, gmod, "held_suarez")
    return gm, om, gmod, omod


@pytest.mark.parametrize("name,prec,tol", [("hs_t21l10", "fp64", 1e-10), ("hs_t42l20", "fp64", 1e-10),
                                           ("hs_t21l10", "fp32", MIXED_TOL["fp32"]),
                                           ("hs_t42l20", "fp32", MIXED_TOL["fp32"])])
def test_held_suarez_steps(jg, orc, name, prec, tol):
    """FP32 tolerances (MIXED_TOL): the divergence tendency is the Laplacian of an energy field of
    ~1e5 m^2/s^2 whose dynamically active part is ~1e2, so FP32 bounds the divergence (and the
    divergent wind) near 1e-5..1e-4 relative; T and ps stay near 1e-7 (printed by _compare)."""
    gm, om, gmod, omod = _hs_developed(jg, orc, name, prec)
    for n in (1, 1, 2):
        gmod.step(n)
        omod.step(n)
        _compare(gmod, omod, "held_suarez", tol)
    for f in ("grid_t_eq", "grid_p_full", "grid_p_half", "grid_z_full"):
        assert configs.rel_l2(gmod.get(f), omod.get(f)) < (tol if prec == "fp64" else 1e-5), f


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 2e-5)])
@pytest.mark.parametrize("name,members", [("hs_t42l20", 1), ("hs_t21l20", 3), ("hs_t21l20", 4)])
def test_held_suarez_analysis_kernel_matches_general(jg, orc, name, members, prec, tol):
    """The Held-Suarez analysis kernel (one thread per (m, level) and one total wavenumber, or two of
    one parity from 4 members on; m pairs; tuning knob hs_analysis_levels) gives the general analysis
    kernel's steps (knob -1) at every levels-per-block setting, for one member and for ensembles.  The two sum the same products in a
    different order, so they agree to rounding (FP64 1e-12, FP32 2e-5 relative L2 after 3 steps;
    the FP32 bound is the dynamics' conditioning, as in MIXED_TOL)."""
    params = configs.PARAMS[name]
    om = configs.make_mesh(orc, name)
    omod = orc.Model(om, params)
    omod.spectral_initialize_fields(configs.hs_temperature_noise(om), True)
    configs.add_hs_flow(orc, om, omod)

    def run(levels):
        gm = configs.make_mesh(jg, name, precision=prec)
        one = jg.Model(gm, params)
        configs.copy_state(omod, one, "held_suarez")
        md = jg.Model(gm, params, members=members)
        for e in range(members):
            md.copy_member(e, one, 0)
        jg.set_tuning(md, dict(jg.get_tuning(md), hs_analysis_levels=levels))
        assert jg.get_tuning(md)["hs_analysis_levels"] == levels
        md.step(3)
        out = jg.Model(gm, params)
        fields = {}
        for e in range(members):
            out.copy_member(0, md, e)
            fields[e] = {f: out.get(f) for f in ("spe_vor_c", "spe_div_c", "spe_t_c", "spe_lnps_c", "grid_u_c")}
        return fields

    ref = run(-1)
    for levels in (0, 1, 2, 5):
        got = run(levels)
        for e in range(members):
            for f, a in got[e].items():
                err = configs.rel_l2(a, ref[e][f])
                assert err < tol, (levels, e, f, err)
    if members > 1:  # identical members stay identical
        for f, a in got[1].items():
            assert np.array_equal(a, got[0][f]), f


@pytest.mark.parametrize("name,option", configs.VERT_COORD_CASES)
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("fp32", MIXED_TOL["fp32"])])
def test_held_suarez_vert_coords(jg, orc, name, option, prec, tol):
    """Held-Suarez on Vert_Coordinate's other sigma options (mcm, v197, uneven_sigma): the
    semi-implicit matrices and the steps from a developed state equal the oracle's."""
    params = configs.PARAMS[name]
    gm, om = configs.make_mesh(jg, name, precision=prec), configs.make_mesh(orc, name)
    gmod, omod = jg.Model(gm, params, vert_coord=option), orc.Model(om, params, vert_coord=option)
    assert np.array_equal(gmod.bk, omod.bk)
    if prec == "fp64":
        assert configs.rel_l2(gmod.semi_implicit("div_mat"), omod.semi_implicit("div_mat")) < 1e-13
        assert configs.rel_l2(gmod.semi_implicit("wave_matrix"), omod.semi_implicit("wave_matrix")) < 1e-12
    omod.spectral_initialize_fields(configs.hs_temperature_noise(om), True)
    configs.add_hs_flow(orc, om, omod)
    configs.copy_state(omod, gmod, "held_suarez")
    for n in (1, 1, 2):
        gmod.step(n)
        omod.step(n)
        _compare(gmod, omod, "held_suarez", tol)
    for f in ("grid_t_eq", "grid_p_full", "grid_p_half"):
        assert configs.rel_l2(gmod.get(f), omod.get(f)) < (tol if prec == "fp64" else 1e-5), f


def test_held_suarez_vertical_coordinate_checks(jg):
    """Model creation refuses coefficients without a zero top, without the surface at the bottom or
    with half-level pressures that do not increase downwards; hybrid models refuse the step adjoint
    (its reverse column kernel reads the sigma coordinates' per-level constants)."""
    gm = configs.make_mesh(jg, "hs_t21l10", precision="fp32")
    params = configs.PARAMS["hs_t21l10"]
    ak, bk = np.linspace(0.0, 1.0e3, 11), np.linspace(0.0, 1.0, 11)
    with pytest.raises(AssertionError):
        jg.Model(gm, params, vert_coord=(ak, bk))  # a_nd != 0: the bottom is not the surface
    ak, bk = np.zeros(11), np.linspace(0.0, 1.0, 11)
    bk[5], bk[6] = bk[6], bk[5]
    with pytest.raises(AssertionError):
        jg.Model(gm, params, vert_coord=(ak, bk))  # not increasing
    hy = jg.Model(gm, params, vert_coord="hybrid")
    configs.init_held_suarez(jg, gm, hy)
    hy.step(2)
    bars = {f: np.zeros_like(hy.get(f)) for f in jg.STATE_FIELDS}
    with pytest.raises(AssertionError):
        jg.HS_Step_Adjoint(hy, bars)


def test_held_suarez_restart_steady_step(jg, orc):
    """A state saved after the init step continues identically once Update_Init_Step! is applied."""
    gm, om, gmod, omod = _hs_developed(jg, orc, "hs_t42l20", "fp64")
    omod.step(2)
    configs.copy_state(omod, gmod, "held_suarez")
    gmod.update_init_step()
    assert not gmod.init_step
    with pytest.raises(AssertionError):
        gmod.update_init_step()
    gmod.step(3)
    omod.step(3)
    _compare(gmod, omod, "held_suarez", 1e-11)


def test_held_suarez_semi_implicit_matrices(jg, orc):
    gm, om, gmod, omod = _pair(jg, orc, "hs_t42l20", "fp64")
    assert configs.rel_l2(gmod.semi_implicit("div_mat"), omod.semi_implicit("div_mat")) < 1e-13
    assert configs.rel_l2(gmod.semi_implicit("h"), omod.semi_implicit("h")) < 1e-13
    assert configs.rel_l2(gmod.semi_implicit("wave_matrix"), omod.semi_implicit("wave_matrix")) < 1e-12


def test_held_suarez_conservation(jg, orc):
    """The mass fixer keeps the area-mean surface pressure at its previous value."""
    gm, om, gmod, omod = _pair(jg, orc, "hs_t42l20", "fp32")
    gmod.spectral_initialize_fields(configs.hs_temperature_noise(gm), True)
    ps0 = jg.Area_Weighted_Global_Mean(gm, gmod.get("grid_ps_c"))
    gmod.step(10)
    ps1 = jg.Area_Weighted_Global_Mean(gm, gmod.get("grid_ps_c"))
    assert abs(ps1 - ps0) / ps0 < 1e-6
    assert np.isfinite(gmod.get("grid_t_c")).all()


def _hs_forcing_inputs(mesh, seed=11):
    """Grid inputs of HS_Forcing! on even-sigma levels: winds ~20 m/s, T ~ 220-300 K,
    ps ~ 1e5 Pa +- 2 %, p_half = b_k ps, p_full between the half levels."""
    rng = np.random.default_rng(seed)
    nlon, nlat, nd = mesh.nlon, mesh.nlat, mesh.nd
    u = np.asfortranarray(20.0 * rng.standard_normal((nlon, nlat, nd)))
    v = np.asfortranarray(10.0 * rng.standard_normal((nlon, nlat, nd)))
    t = np.asfortranarray(220.0 + 80.0 * rng.random((nlon, nlat, nd)))
    ps = 1.0e5 * (1.0 + 0.02 * rng.standard_normal((nlon, nlat)))
    b = np.linspace(0.0, 1.0, nd + 1)
    p_half = np.asfortranarray(ps[:, :, None] * b[None, None, :])
    p_full = np.asfortranarray(0.5 * (p_half[:, :, :-1] + p_half[:, :, 1:]))
    return u, v, p_half, p_full, t


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("fp32", 2e-5)])
def test_hs_forcing_entry_point(jg, orc, prec, tol):
    """HS_Forcing! (HS_Forcing.jl:1-130) through its own entry point, against the oracle."""
    gm, om, gmod, omod = _pair(jg, orc, "hs_t21l20", prec)
    ins = _hs_forcing_inputs(gm)
    outs = {}
    for key, backend, model in (("gpu", jg, gmod), ("orc", orc, omod)):
        o = [np.zeros_like(ins[0]) for _ in range(4)]
        backend.HS_Forcing(model, 2400, *ins, *o)
        outs[key] = o
    for name, a, b in zip(("du", "dv", "t_eq", "dt"), outs["gpu"], outs["orc"]):
        assert np.isfinite(a).all()
        assert configs.rel_l2(a, b) < tol, (name, configs.rel_l2(a, b))
    with pytest.raises(AssertionError):
        jg.HS_Forcing(gmod, 0, *ins, *[np.zeros_like(ins[0]) for _ in range(4)])


@pytest.mark.parametrize("members", [1, 2])
def test_on_device_zonal_mean_diagnostics(jg, members, tmp_path):
    """Update_Output! (Output_Manager.jl:81-107) as on-device FP64 sums: the means over the steps
    equal the zonal means of the fields read back after every step."""
    name = "hs_t21l10"
    gm = configs.make_mesh(jg, name, precision="fp64")
    params = configs.PARAMS[name]
    md = jg.Model(gm, params, members=members)
    one = jg.Model(gm, params)
    for e in range(members):
        configs.init_held_suarez(jg, gm, one, seed=configs.BASE_SEED + e)
        md.copy_member(e, one)
    md.step(2)
    md.diagnostics(True)
    want = {k: 0.0 for k in ("t_zonal_mean", "t_eq_zonal_mean", "u_zonal_mean", "v_zonal_mean", "ps_mean")}
    nsteps = 6
    reader = jg.Model(gm, params)
    for _ in range(nsteps):
        md.step(1)
        for e in range(members):
            reader.copy_member(0, md, e)
            for key, field in (("t_zonal_mean", "grid_t_c"), ("t_eq_zonal_mean", "grid_t_eq"),
                               ("u_zonal_mean", "grid_u_c"), ("v_zonal_mean", "grid_v_c")):
                z = reader.get(field).mean(axis=0)
                want[key] = want[key] + (z if members == 1 else np.stack([z if i == e else 0 * z
                                                                          for i in range(members)], -1))
            ps = reader.get("grid_ps_c")[:, :, 0]
            want["ps_mean"] = want["ps_mean"] + (ps if members == 1 else np.stack([ps if i == e else 0 * ps
                                                                                  for i in range(members)], -1))
    for key, w in want.items():
        got, steps = md.read_diagnostics(key)
        assert steps == nsteps
        assert configs.rel_l2(got, w / nsteps) < 1e-12, key
    # the file dump (raw FP64 + JSON header) holds the same means
    path = str(tmp_path / "diag.bin")
    head = md.write_diagnostics(path)
    back, _ = jg.read_arrays(path)
    assert head["steps"] == nsteps
    for key in want:
        assert np.array_equal(back[key], md.read_diagnostics(key)[0]), key


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_packed_state_transfer(jg, prec):
    """jgcm_model_get_state / set_state move the 18 state arrays in one buffer: the packed read equals
    the per-field reads, and a model loaded from it steps exactly like one loaded field by field."""
    name = "hs_t21l10"
    mesh = configs.make_mesh(jg, name, precision=prec)
    a = jg.Model(mesh, configs.PARAMS[name])
    configs.init_held_suarez(jg, mesh, a)
    a.step(2)
    fields = {k: a.get(k) for k in jg.STATE_FIELDS}
    packed = a.get_state()
    assert packed.size == a.state_size()
    back = jg.unpack_state(mesh, packed)
    for k in jg.STATE_FIELDS:
        assert np.array_equal(back[k], fields[k]), k
    assert np.array_equal(jg.pack_state(mesh, fields), packed)
    b, c = jg.Model(mesh, configs.PARAMS[name]), jg.Model(mesh, configs.PARAMS[name])
    b.set_state(packed)
    for k in jg.STATE_FIELDS:
        c.set(k, fields[k])
    for mdl in (b, c):
        mdl.update_init_step()
        mdl.step(3)
    for k in jg.STATE_FIELDS:
        assert np.array_equal(b.get(k), c.get(k)), k


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_gpu_rh4_phase_speed_and_steady_zonal_flow(jg, prec):
    """The analytic checks of the oracle on the library: the Rossby-Haurwitz wave 4 moves at the
    analytic speed (Barotropic T42), and Williamson test case 2 stays steady (shallow water T42)."""
    from test_oracle import (SW_TC2, init_sw_steady_zonal_flow, rh4_analytic_speed, rh4_phase_speed,
                             sw_tc2_params)

    name = "barotropic_t42"
    M = configs.make_mesh(jg, name, precision=prec)
    md = jg.Model(M, configs.PARAMS[name])
    nu = rh4_phase_speed(jg, M, md)
    ref = rh4_analytic_speed(configs.PARAMS[name]["omega"])
    assert abs(nu - ref) / ref < 1e-3, (nu, ref)
    g = SW_TC2
    M2 = jg.Spectral_Spherical_Mesh(g["num_fourier"], g["num_fourier"] + 1, g["nlat"], g["nlon"], 1, g["radius"],
                                    precision=prec)
    sw = jg.Model(M2, sw_tc2_params())
    h0 = init_sw_steady_zonal_flow(jg, M2, sw)
    u0 = sw.get("grid_u_c")
    sw.step(72)
    tol = 1e-8 if prec == "fp64" else 1e-4
    assert np.abs(sw.get("grid_ps_c") - h0).max() / (h0.max() - h0.min()) < tol
    assert np.abs(sw.get("grid_u_c") - u0).max() / np.abs(u0).max() < tol
