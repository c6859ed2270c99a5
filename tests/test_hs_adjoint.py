"""Reverse mode of the Held-Suarez step and the gradient of a loss over many steps.

The reference has no adjoint; the checks are the ones a discrete adjoint must pass:
  * the oracle's step adjoint (oracle/jgcm_oracle_adjoint.inc) against central finite differences
    of the oracle's forward step, in random directions over all 18 state fields, for the
    init step (Δt) and a leapfrog step (2Δt);
  * the oracle's gradient of J = sum w_j (T_final - T_target)^2 / (2 nlon nd) with respect to the
    initial spectral temperature and the five HS parameters against central differences;
  * (GPU) the library's step adjoint equals the oracle's; the library's checkpointed gradient
    equals the oracle's (FP64) and central differences of the library's own FP64 forward model.
"""
import numpy as np
import pytest

from jgcm import configs

NAME = "hs_t21l10"


def _rand_like(rng, a, scale):
    if np.iscomplexobj(a):
        r = rng.standard_normal(a.shape) + 1j * rng.standard_normal(a.shape)
        for m in range(a.shape[0]):
            r[m, :m, :] = 0
        r[0] = r[0].real
    else:
        r = rng.standard_normal(a.shape)
    return np.asfortranarray(r * scale)


def _rms(a):
    return float(np.sqrt(np.mean(np.abs(a) ** 2))) or 1.0


def _dot(a, b):
    return sum(float(np.sum((a[k].conj() * b[k]).real)) for k in a)


def _developed_state(orc, steps=3):
    mesh = configs.make_mesh(orc, NAME)
    md = orc.Model(mesh, configs.PARAMS[NAME])
    configs.init_held_suarez(orc, mesh, md)
    configs.add_hs_flow(orc, mesh, md)
    orc.set_state(md, orc.get_state(md))
    md.step(steps)
    return mesh, md


@pytest.mark.parametrize("init", [False, True])
def test_oracle_step_adjoint_matches_finite_differences(orc, init):
    mesh, md = _developed_state(orc)
    fields, _ = orc.get_state(md)
    X = (fields, init)
    rng = np.random.default_rng(11 + int(init))
    dX = {k: _rand_like(rng, v, _rms(v)) for k, v in fields.items()}
    ybar = {k: _rand_like(rng, v, 1.0 / _rms(v)) for k, v in fields.items()}
    orc.set_state(md, X)
    xb, _ = orc.HS_Step_Adjoint(md, ybar)
    ad = _dot(xb, dX)
    eps = 1e-5
    outs = []
    for sg in (1.0, -1.0):
        orc.set_state(md, ({k: np.asfortranarray(fields[k] + sg * eps * dX[k]) for k in fields}, init))
        md.step(1)
        outs.append(orc.get_state(md)[0])
    fd = _dot(ybar, {k: (outs[0][k] - outs[1][k]) / (2 * eps) for k in fields})
    assert abs(fd - ad) <= 1e-7 * abs(ad), (fd, ad)


def _gradient_case(orc, nsteps=6):
    mesh = configs.make_mesh(orc, NAME)
    md = orc.Model(mesh, configs.PARAMS[NAME])
    configs.init_held_suarez(orc, mesh, md)
    configs.add_hs_flow(orc, mesh, md)
    orc.set_state(md, orc.get_state(md))
    S0 = orc.get_state(md)
    tgt = np.asfortranarray(S0[0]["grid_t_c"] + np.random.default_rng(5).standard_normal(S0[0]["grid_t_c"].shape))
    return mesh, md, S0, tgt


def _t0_direction(mesh, orc_or_jg, seed=3):
    rng = np.random.default_rng(seed)
    N1, S1 = mesh.num_fourier + 1, mesh.num_spherical + 1
    d = rng.standard_normal((N1, S1, mesh.nd)) + 1j * rng.standard_normal((N1, S1, mesh.nd))
    for m in range(N1):
        d[m, :m, :] = 0
    d[0] = d[0].real
    d /= (1.0 + np.arange(S1))[None, :, None] ** 2
    d[:, -1, :] = 0  # row N+1: zero in every analysed field (not part of the control)
    return np.asfortranarray(d)


def test_oracle_gradient_matches_finite_differences(orc):
    nsteps = 6
    mesh, md, S0, tgt = _gradient_case(orc)
    loss, gT, gp = orc.HS_Gradient(md, nsteps, tgt)
    d = _t0_direction(mesh, orc)
    gd = mesh.grid(mesh.nd)
    orc.Trans_Spherical_To_Grid(mesh, d, gd)

    def loss_t0(eps):
        f, init = S0
        st = dict(f)
        for lev in ("c", "p"):
            st[f"spe_t_{lev}"] = np.asfortranarray(f[f"spe_t_{lev}"] + eps * d)
            st[f"grid_t_{lev}"] = np.asfortranarray(f[f"grid_t_{lev}"] + eps * gd)
        orc.set_state(md, (st, init))
        md.step(nsteps)
        return orc.hs_loss(mesh, md.get("grid_t_c"), tgt)[0]

    assert abs(loss_t0(0.0) - loss) <= 1e-14 * loss
    eps = 1e-4
    fd = (loss_t0(eps) - loss_t0(-eps)) / (2 * eps)
    ad = float(np.sum((gT.conj() * d).real))
    assert abs(fd - ad) <= 1e-7 * abs(ad), (fd, ad)
    for i, p in enumerate(orc.HS_PARAMS):
        vals = []
        h = 1e-4 * configs.PARAMS[NAME][p]
        for sg in (1, -1):
            P = dict(configs.PARAMS[NAME])
            P[p] = P[p] + sg * h
            m2 = orc.Model(mesh, P)
            orc.set_state(m2, S0)
            m2.step(nsteps)
            vals.append(orc.hs_loss(mesh, m2.get("grid_t_c"), tgt)[0])
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(fd - gp[i]) <= 1e-6 * abs(gp[i]), (p, fd, gp[i])


# ---- GPU ----------------------------------------------------------------------------------------
def _gpu_twin(jg, orc, prec, fields, init):
    gm = configs.make_mesh(jg, NAME, precision=prec)
    gmod = jg.Model(gm, configs.PARAMS[NAME])
    for k in orc.STATE_FIELDS:
        gmod.set(k, fields[k])
    if not init:
        gmod.update_init_step()
    return gm, gmod


@pytest.mark.gpu
@pytest.mark.parametrize("init", [False, True])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("fp32", 2e-4)])
def test_gpu_step_adjoint_matches_oracle(jg, orc, init, prec, tol):
    mesh, md = _developed_state(orc)
    fields, _ = orc.get_state(md)
    orc.set_state(md, (fields, init))
    rng = np.random.default_rng(21)
    ybar = {k: _rand_like(rng, v, 1.0 / _rms(v)) for k, v in fields.items()}
    xb_o, pb_o = orc.HS_Step_Adjoint(md, ybar)
    gm, gmod = _gpu_twin(jg, orc, prec, fields, init)
    xb_g, pb_g = jg.HS_Step_Adjoint(gmod, ybar)
    for k in orc.STATE_FIELDS:
        err = configs.rel_l2(xb_g[k], xb_o[k])
        assert err < tol, (k, err)
    for i, p in enumerate(orc.HS_PARAMS):
        assert abs(pb_g[i] - pb_o[i]) <= tol * abs(pb_o[i]) + 1e-30, (p, pb_g[i], pb_o[i])
    # the model is left at X_s: the step adjoint again gives the same cotangents
    xb_g2, _ = jg.HS_Step_Adjoint(gmod, ybar)
    for k in orc.STATE_FIELDS:
        assert configs.rel_l2(xb_g2[k], xb_g[k]) < 1e-12, k


def _gpu_loss_t0(jg, gmod, S0, d, gd, eps, nsteps, tgt, init=True):
    f = S0
    for k in jg.STATE_FIELDS:
        v = f[k]
        if k in ("spe_t_c", "spe_t_p"):
            v = v + eps * d
        elif k in ("grid_t_c", "grid_t_p"):
            v = v + eps * gd
        gmod.set(k, np.asfortranarray(v))
    gmod.set_init_step(init)
    gmod.step(nsteps)
    w = gmod.mesh.wts[None, :, None]
    diff = gmod.get("grid_t_c") - tgt
    return float(np.sum(w * diff * diff) / (2.0 * gmod.mesh.nlon * gmod.mesh.nd))


@pytest.mark.gpu
def test_gpu_gradient_matches_oracle_and_finite_differences(jg, orc):
    """8 steps with a checkpoint every 3 (segments of 3, 3, 2), FP64: the library's gradient equals
    the oracle's, and central differences of the library's own forward model."""
    nsteps, ck = 8, 3
    mesh, md, S0, tgt = _gradient_case(orc)
    loss_o, gT_o, gp_o = orc.HS_Gradient(md, nsteps, tgt)
    gm, gmod = _gpu_twin(jg, orc, "fp64", S0[0], True)
    loss_g, gT_g, gp_g = jg.HS_Gradient(gmod, nsteps, tgt, checkpoint_every=ck)
    assert abs(loss_g - loss_o) <= 1e-11 * loss_o, (loss_g, loss_o)
    assert configs.rel_l2(gT_g, gT_o) < 1e-9, configs.rel_l2(gT_g, gT_o)
    for i, p in enumerate(orc.HS_PARAMS):
        assert abs(gp_g[i] - gp_o[i]) <= 1e-9 * abs(gp_o[i]), (p, gp_g[i], gp_o[i])
    # the model was left at the final state
    assert configs.rel_l2(gmod.get("grid_t_c"), md.get("grid_t_c")) < 1e-11
    d = _t0_direction(mesh, orc)
    gd = mesh.grid(mesh.nd)
    orc.Trans_Spherical_To_Grid(mesh, d, gd)
    eps = 1e-4
    fd = (_gpu_loss_t0(jg, gmod, S0[0], d, gd, eps, nsteps, tgt)
          - _gpu_loss_t0(jg, gmod, S0[0], d, gd, -eps, nsteps, tgt)) / (2 * eps)
    ad = float(np.sum((gT_g.conj() * d).real))
    assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


@pytest.mark.gpu
def test_gpu_gradient_on_v197_levels_matches_oracle(jg, orc):
    """The gradient on Vert_Coordinate's 18-level v197 sigma table (6 steps, checkpoint every 4)
    equals the oracle's: the reverse column, fixers and semi-implicit transposes take the level
    coefficients from the model."""
    name, nsteps, ck = "hs_t21l18", 6, 4
    mesh = configs.make_mesh(orc, name)
    md = orc.Model(mesh, configs.PARAMS[name], vert_coord="v197")
    configs.init_held_suarez(orc, mesh, md)
    configs.add_hs_flow(orc, mesh, md)
    orc.set_state(md, orc.get_state(md))
    S0 = orc.get_state(md)[0]
    tgt = np.asfortranarray(S0["grid_t_c"] + np.random.default_rng(5).standard_normal(S0["grid_t_c"].shape))
    loss_o, gT_o, gp_o = orc.HS_Gradient(md, nsteps, tgt)
    gm = configs.make_mesh(jg, name, precision="fp64")
    gmod = jg.Model(gm, configs.PARAMS[name], vert_coord="v197")
    for k in orc.STATE_FIELDS:
        gmod.set(k, S0[k])
    gmod.set_init_step(True)
    loss_g, gT_g, gp_g = jg.HS_Gradient(gmod, nsteps, tgt, checkpoint_every=ck)
    assert abs(loss_g - loss_o) <= 1e-11 * loss_o, (loss_g, loss_o)
    assert configs.rel_l2(gT_g, gT_o) < 1e-9, configs.rel_l2(gT_g, gT_o)
    for i, p in enumerate(orc.HS_PARAMS):
        assert abs(gp_g[i] - gp_o[i]) <= 1e-9 * abs(gp_o[i]), (p, gp_g[i], gp_o[i])


@pytest.mark.gpu
def test_gpu_gradient_one_day_t42l20():
    """The configuration of the adjoint benchmark: Held-Suarez T42L20, 72 steps from the seeded
    initial state, a checkpoint every 8.  FP64 against central differences (T0 direction and the five
    parameters, eps 1e-4 relative); the mixed-precision gradient against the FP64 one."""
    import jgcm

    name, nsteps = "hs_t42l20", 72
    grads = {}
    for prec in ("fp64", "fp32"):
        mesh = configs.make_mesh(jgcm, name, precision=prec)
        md = jgcm.Model(mesh, configs.PARAMS[name])
        configs.init_held_suarez(jgcm, mesh, md)
        if prec == "fp64":
            ref = {k: md.get(k) for k in jgcm.STATE_FIELDS}
            tgt = np.asfortranarray(ref["grid_t_c"] + np.random.default_rng(5).standard_normal(ref["grid_t_c"].shape))
        for k in jgcm.STATE_FIELDS:
            md.set(k, ref[k])
        md.set_init_step(True)
        grads[prec] = jgcm.HS_Gradient(md, nsteps, tgt, checkpoint_every=8)
        if prec != "fp64":
            continue
        loss, gT, gp = grads[prec]
        d = _t0_direction(mesh, None)
        gd = mesh.grid(mesh.nd)
        jgcm.Trans_Spherical_To_Grid(mesh, d, gd)
        eps = 1e-4
        fd = (_gpu_loss_t0(jgcm, md, ref, d, gd, eps, nsteps, tgt)
              - _gpu_loss_t0(jgcm, md, ref, d, gd, -eps, nsteps, tgt)) / (2 * eps)
        ad = float(np.sum((gT.conj() * d).real))
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)
        # the parameters by central differences at 1e-3 relative: k_f's cotangent is ~1e-5 of k_a's, so
        # at 1e-4 its difference (~1e-7 of a loss of 5.5) sits within reach of the loss's rounding,
        # while the truncation error at 1e-3 stays far below 1e-6 for all five
        for i, p in enumerate(jgcm.HS_PARAMS):
            h = 1e-3 * configs.PARAMS[name][p]
            vals = []
            for sg in (1, -1):
                P = dict(configs.PARAMS[name])
                P[p] += sg * h
                m2 = jgcm.Model(mesh, P)
                vals.append(_gpu_loss_t0(jgcm, m2, ref, d, gd, 0.0, nsteps, tgt))
            f = (vals[0] - vals[1]) / (2 * h)
            assert abs(f - gp[i]) <= 1e-6 * abs(gp[i]), (p, f, gp[i])
    (l64, g64, p64), (l32, g32, p32) = grads["fp64"], grads["fp32"]
    assert abs(l32 - l64) <= 1e-4 * l64
    assert configs.rel_l2(g32, g64) < 1e-3, configs.rel_l2(g32, g64)
    assert np.all(np.abs(p32 - p64) <= 1e-3 * np.abs(p64))


def test_packed_state_layout_round_trip():
    """pack_state / unpack_state (host side of jgcm_model_set_state / get_state): the 18 arrays back
    to back in STATE_FIELDS order, each in the reference layout; no GPU needed."""
    import types

    import jgcm

    mesh = types.SimpleNamespace(num_fourier=5, num_spherical=6, nlon=16, nlat=8, nd=3)
    rng = np.random.default_rng(0)
    fields = {}
    for k in jgcm.STATE_FIELDS:
        nlev = 1 if k in ("spe_lnps_c", "spe_lnps_p", "grid_ps_c", "grid_ps_p") else 3
        if k.startswith("spe_"):
            fields[k] = np.asfortranarray(rng.standard_normal((6, 7, nlev)) + 1j * rng.standard_normal((6, 7, nlev)))
        else:
            fields[k] = np.asfortranarray(rng.standard_normal((16, 8, nlev)))
    packed = jgcm.pack_state(mesh, fields)
    assert packed.size == 2 * 6 * 7 * (3 * 6 + 2) + 16 * 8 * (3 * 8 + 2)
    assert np.array_equal(packed[:2 * 6 * 7 * 3].view(np.complex128), fields["spe_vor_c"].ravel(order="F"))
    back = jgcm.unpack_state(mesh, packed)
    for k in jgcm.STATE_FIELDS:
        assert np.array_equal(back[k], fields[k]), k


def test_raw_array_dump_round_trip(tmp_path):
    """write_arrays / read_arrays (the diagnostics dump): Fortran-order FP64 arrays back to back."""
    import jgcm

    rng = np.random.default_rng(1)
    arrays = {"t_zonal_mean": rng.standard_normal((8, 3)), "ps_mean": rng.standard_normal((16, 8))}
    path = str(tmp_path / "diag.bin")
    head = jgcm.write_arrays(path, arrays, {"steps": 12})
    back, head2 = jgcm.read_arrays(path)
    assert head2 == head and head["steps"] == 12
    for k, v in arrays.items():
        assert np.array_equal(back[k], v)
    raw = np.fromfile(path, dtype="<f8")
    assert np.array_equal(raw[:24], arrays["t_zonal_mean"].ravel(order="F"))
