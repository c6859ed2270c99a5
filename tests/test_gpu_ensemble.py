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


def test_ensemble_rejects_direct_field_access(jg):
    params = configs.PARAMS["hs_t21l20"]
    mesh = configs.make_mesh(jg, "hs_t21l20", precision="fp32")
    ens = jg.Model(mesh, params, members=2)
    with pytest.raises(AssertionError):
        ens.get("grid_t_c")
    md = jg.Model(mesh, params)
    with pytest.raises(AssertionError):
        md.copy_member(1, ens, 0)  # member out of range
