"""Passive tracers (Dyn_Data's spe_tracers_* / grid_tracers_*, Dyn_Data.jl:36-39,63-66) on the GPU
against the FP64 oracle, through the C ABI.

The reference allocates the tracers and rotates them in Time_Advance! but never steps them
(Spectral_Dynamics.jl:235 keeps "grid_q = grid_t" as a todo); both implementations advect them like
T: Vert_Advection! with the step's mass flux, Add_Horizontal_Advection! of spe_tracers_c, the
analysis, T's spectral damping and filtered leapfrog, the synthesis of the new level.
Tolerances: FP64 1e-10 after 4 steps (as the other FP64 step tests); the mixed path 1e-5 (a tracer
is transformed and stepped like T, whose mixed-path bound is 5e-6 per field; the tracers' tendency
has no forcing to damp the advective rounding).
"""
import numpy as np
import pytest

from jgcm import configs

pytestmark = pytest.mark.gpu

NAME = "hs_t21l10"


def _tracer_fields(om, omod):
    """Two tracers from the developed state: T itself, and a smooth field of its own (a seeded
    spectral field of the lowest modes), each with its grid synthesised from its spectrum."""
    spe_t = omod.get("spe_t_c")
    rng = np.random.default_rng(configs.BASE_SEED)
    s2 = np.zeros_like(spe_t)
    s2[:6, :7, :] = rng.standard_normal(s2[:6, :7, :].shape) + 1j * rng.standard_normal(s2[:6, :7, :].shape)
    s2[0, :, :] = s2[0, :, :].real  # m = 0 modes of a real field
    for m in range(s2.shape[0]):
        s2[m, :m, :] = 0.0  # n >= m only
    s2[0, 0, :] = 5.0
    spe = np.stack([spe_t, s2], axis=3)
    return spe


def _synth(orc, om, spe):
    """grid_tracers from spe_tracers, one tracer (nd levels) at a time."""
    out = []
    for i in range(spe.shape[3]):
        grid = om.grid(spe.shape[2])
        orc.Trans_Spherical_To_Grid(om, np.asfortranarray(spe[..., i]), grid)
        out.append(grid)
    return np.stack(out, axis=3)


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_tracers_match_the_oracle(jg, orc, prec, tol):
    params = configs.PARAMS[NAME]
    gm, om = configs.make_mesh(jg, NAME, precision=prec), configs.make_mesh(orc, NAME)
    gmod, omod = jg.Model(gm, params, num_tracers=2), orc.Model(om, params, num_tracers=2)
    omod.spectral_initialize_fields(configs.hs_temperature_noise(om), True)
    configs.add_hs_flow(orc, om, omod)
    configs.copy_state(omod, gmod, "held_suarez")
    spe = _tracer_fields(om, omod)
    grid = _synth(orc, om, spe)
    for md in (gmod, omod):
        md.set("spe_tracers_c", spe)
        md.set("spe_tracers_p", spe)
        md.set("grid_tracers_c", grid)
    assert np.allclose(gmod.get("spe_tracers_c"), spe, rtol=0, atol=1e-5 * np.abs(spe).max())
    for n in (1, 1, 2):
        gmod.step(n)
        omod.step(n)
        for f in ("spe_tracers_c", "spe_tracers_p", "grid_tracers_c", "grid_tracers_p"):
            a, b = gmod.get(f), omod.get(f)
            for i in range(2):
                err = configs.rel_l2(a[..., i], b[..., i])
                assert err < tol, (n, f, i, err)
        # the tracer that started as T has moved away from T (forcing, the energy conversion and the
        # semi-implicit terms act on T alone): the tracers are stepped, not copied
        t = omod.get("spe_t_c")
        assert configs.rel_l2(omod.get("spe_tracers_c")[..., 0], t) > 1e-6
    # the other prognostic fields are unchanged by the tracers
    ref = orc.Model(om, params)
    ref.spectral_initialize_fields(configs.hs_temperature_noise(om), True)
    configs.add_hs_flow(orc, om, ref)
    ref.step(4)
    assert configs.rel_l2(omod.get("spe_vor_c"), ref.get("spe_vor_c")) == 0.0


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_a_uniform_tracer_stays_uniform(jg, prec, tol):
    """q = 1 everywhere: its gradients vanish, the centred vertical flux form gives
    q (M_{k-1/2} - M_{k+1/2}) + q (M_{k+1/2} - M_{k-1/2}) = 0, and the (0,0) mode is not damped."""
    params = configs.PARAMS[NAME]
    gm = configs.make_mesh(jg, NAME, precision=prec)
    md = jg.Model(gm, params, num_tracers=1)
    configs.init_held_suarez(jg, gm, md)
    spe = np.zeros(md.get("spe_tracers_c").shape, dtype=np.complex128)
    spe[0, 0, :, :] = 1.0  # P_00 = 1
    md.set("spe_tracers_c", spe)
    md.set("spe_tracers_p", spe)
    md.set("grid_tracers_c", np.ones(md.get("grid_tracers_c").shape))
    md.step(30)
    q = md.get("grid_tracers_c")
    assert np.abs(q - 1.0).max() < tol, np.abs(q - 1.0).max()


def test_tracers_in_a_member_ensemble(jg, orc):
    """Members with tracers equal one-member models stepped alone (FP64, to rounding of the
    member-batched sums)."""
    params = configs.PARAMS[NAME]
    gm, om = configs.make_mesh(jg, NAME, precision="fp64"), configs.make_mesh(orc, NAME)
    ens = jg.Model(gm, params, members=2, num_tracers=2)
    singles = []
    for e in range(2):
        omod = orc.Model(om, params)
        configs.init_held_suarez(orc, om, omod, seed=configs.BASE_SEED + e)
        configs.add_hs_flow(orc, om, omod)
        one = jg.Model(gm, params, num_tracers=2)
        configs.copy_state(omod, one, "held_suarez")
        spe = _tracer_fields(om, omod) * (1 + e)
        one.set("spe_tracers_c", spe)
        one.set("spe_tracers_p", spe)
        one.set("grid_tracers_c", _synth(orc, om, spe))
        ens.copy_member(e, one)
        singles.append(one)
    ens.step(3)
    out = jg.Model(gm, params, num_tracers=2)
    for e, one in enumerate(singles):
        one.step(3)
        out.copy_member(0, ens, e)
        for f in ("spe_tracers_c", "grid_tracers_c", "spe_t_c"):
            assert configs.rel_l2(out.get(f), one.get(f)) < 1e-12, (e, f)


def test_tracer_arguments(jg):
    import ctypes as C

    params = configs.PARAMS[NAME]
    gm = configs.make_mesh(jg, NAME, precision="fp64")
    md = jg.Model(gm, params, num_tracers=3)
    n = C.c_int()
    assert jg.lib().jgcm_model_num_tracers(md._h, C.byref(n)) == 0 and n.value == 3
    assert md.get("spe_tracers_n").shape == (22, 23, 10, 3)
    assert md.get("grid_tracers_p").shape == (64, 32, 10, 3)
    assert jg.lib().jgcm_model_add_tracers(md._h, 1) == -1  # once per model
    plain = jg.Model(gm, params)
    assert jg.lib().jgcm_model_add_tracers(plain._h, 0) == -1
    with pytest.raises(AssertionError):
        plain.copy_member(0, md, 0)  # tracer counts differ
    with pytest.raises(AssertionError):
        plain.get("spe_tracers_c")  # no tracers: no such field
    bmesh = configs.make_mesh(jg, "barotropic_t42", precision="fp64")
    with pytest.raises(AssertionError):
        jg.Model(bmesh, configs.PARAMS["barotropic_t42"], num_tracers=1)
