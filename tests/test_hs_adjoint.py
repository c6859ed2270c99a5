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
