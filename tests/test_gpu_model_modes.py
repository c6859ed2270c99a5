"""Model steps in the tensor-core precision modes, and from the reference experiments' own initial
conditions, against the FP64 oracle through the C ABI.

The tensor-core modes (TF32x3, BF16x3: the Legendre contractions on tcgen05 with 3-term split
operands and FP32 accumulation) are the mixed path with another Legendre engine, so their steps are
held to the FP32 step tolerances of test_gpu_models.py.  The reference initial conditions are the
ones exp/Barotropic/Barotropic.jl:43-62 and exp/Shallow_Water/SW.jl:57-80 build (the shallow-water
one with its relaxation forcing on and its h seeded into grid_lnps, so the first step sees h = 0).
"""
import numpy as np
import pytest

from jgcm import configs
from test_gpu_models import MIXED_TOL, _compare

pytestmark = pytest.mark.gpu


def _pair(jg, orc, name, prec):
    params = configs.PARAMS[name]
    gm = configs.make_mesh(jg, name, precision=prec)
    om = configs.make_mesh(orc, name)
    gmod, omod = jg.Model(gm, params), orc.Model(om, params)
    if prec in ("tf32x3", "bf16x3"):
        assert jg.get_tuning(gmod)["simt_legendre"] == 0  # the tcgen05 engine is the one stepped
    return gm, om, gmod, omod


@pytest.mark.parametrize("prec", ["tf32x3", "bf16x3"])
@pytest.mark.parametrize("name", ["hs_t21l20", "hs_t42l20"])
def test_tensor_core_held_suarez_steps(jg, orc, name, prec):
    gm, om, gmod, omod = _pair(jg, orc, name, prec)
    omod.spectral_initialize_fields(configs.hs_temperature_noise(om), True)
    configs.add_hs_flow(orc, om, omod)
    configs.copy_state(omod, gmod, "held_suarez")
    for n in (1, 1, 2):
        gmod.step(n)
        omod.step(n)
        _compare(gmod, omod, "held_suarez", MIXED_TOL[prec])


@pytest.mark.parametrize("prec", ["tf32x3", "bf16x3"])
def test_tensor_core_shallow_water_steps(jg, orc, prec):
    gm, om, gmod, omod = _pair(jg, orc, "sw_t85", prec)
    configs.init_shallow_water_jet(orc, om, omod)
    configs.copy_state(omod, gmod, "shallow_water")
    for n in (1, 1, 4):
        gmod.step(n)
        omod.step(n)
        _compare(gmod, omod, "shallow_water", MIXED_TOL[prec])


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("fp32", MIXED_TOL["fp32"]), ("tf32x3", MIXED_TOL["tf32x3"])])
def test_barotropic_reference_initial_condition(jg, orc, prec, tol):
    """exp/Barotropic/Barotropic.jl:43-62 (T85, the perturbed upper-tropospheric jet) built on each
    backend by the reference's own sequence, then stepped."""
    name = "barotropic_t85_ref"
    gm, om, gmod, omod = _pair(jg, orc, name, prec)
    configs.init_barotropic_reference(orc, om, omod)
    configs.init_barotropic_reference(jg, gm, gmod)
    _compare(gmod, omod, "barotropic", 1e-12 if prec == "fp64" else 1e-5)
    for n in (1, 1, 6):
        gmod.step(n)
        omod.step(n)
        _compare(gmod, omod, "barotropic", tol)


def test_barotropic_reference_one_day_fp64(jg, orc):
    name = "barotropic_t85_ref"
    gm, om, gmod, omod = _pair(jg, orc, name, "fp64")
    configs.init_barotropic_reference(orc, om, omod)
    configs.copy_state(omod, gmod, "barotropic")
    n = configs.STEPS_PER_DAY[name]
    gmod.step(n)
    omod.step(n)
    _compare(gmod, omod, "barotropic", 1e-9)


@pytest.mark.parametrize("prec", ["fp64", "fp32", "bf16x3"])
def test_shallow_water_reference_initial_condition(jg, orc, prec):
    """exp/Shallow_Water/SW.jl:57-80 with Shallow_Water_Physics! on (kappa_m = 1/20 days, kappa_t =
    1/10 days, the h_eq mound and ITCZ ridge).  The first step reads h = 0 from grid_ps_c (the
    reference seeds grid_lnps), relaxes it towards h_eq and advects nothing; every step after runs
    the full forced dynamics.  The FP64 path builds the initial state itself; the mixed modes start
    from the oracle's: their analysis of the constant h_0 = 3e4 field would leave FP32 rounding
    (~1e-3 m^2/s^2) in every n > 0 mode where the reference has none, a height anomaly the
    semi-implicit step then answers with gravity waves (divergence error 2e-4 at the second step,
    against 2e-7 from the oracle's state)."""
    tol = 1e-10 if prec == "fp64" else MIXED_TOL[prec]
    name = "sw_t85_ref"
    gm, om, gmod, omod = _pair(jg, orc, name, prec)
    configs.init_shallow_water_reference(orc, om, omod)
    if prec == "fp64":
        configs.init_shallow_water_reference(jg, gm, gmod)
    else:
        configs.copy_state(omod, gmod, "shallow_water")
    assert np.all(gmod.get("grid_ps_c") == 0) and np.all(omod.get("grid_ps_c") == 0)
    assert configs.rel_l2(gmod.get("grid_h_eq"), omod.get("grid_h_eq")) < (1e-15 if prec == "fp64" else 1e-7)
    for n in (1, 1, 4):
        gmod.step(n)
        omod.step(n)
        _compare(gmod, omod, "shallow_water", tol)
    # the forcing moved the fluid: the state is no longer at rest
    assert np.abs(omod.get("grid_u_c")).max() > 1e-3


def test_shallow_water_reference_one_day_fp64(jg, orc):
    name = "sw_t85_ref"
    gm, om, gmod, omod = _pair(jg, orc, name, "fp64")
    configs.init_shallow_water_reference(orc, om, omod)
    configs.init_shallow_water_reference(jg, gm, gmod)
    n = configs.STEPS_PER_DAY[name]
    gmod.step(n)
    omod.step(n)
    _compare(gmod, omod, "shallow_water", 1e-9)
