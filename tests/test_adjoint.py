"""Adjoints of the spectral transforms (the transposed quadrature).

The inner products are the Euclidean ones of the reference-layout arrays: grid values, and the
(re, im) pairs of the spectral entries n >= m.  Checks:
  * the oracle's adjoints (written from the forward definitions on every latitude, without parity
    folding or FFT) pass the dot-product test against the oracle's forward transforms (CPU);
  * the GPU adjoints equal the oracle's (FP64 1e-12, FP32 5e-6) and pass the dot-product test;
  * central finite differences of a scalar loss through the forward transform reproduce the
    gradient the adjoint returns (the transforms are linear: FD is exact up to rounding).
"""
import numpy as np
import pytest

from jgcm import configs

CASES = [(21, 32, 64, 3), (42, 64, 128, 2)]


def _spec(m, nlev, seed):
    rng = np.random.default_rng(seed)
    N1, S1 = m.num_fourier + 1, m.num_spherical + 1
    s = rng.standard_normal((N1, S1, nlev)) + 1j * rng.standard_normal((N1, S1, nlev))
    s /= (1.0 + np.arange(S1))[None, :, None] ** 1.0
    for mm in range(N1):
        s[mm, :mm, :] = 0
    return np.asfortranarray(s)


def _grid(m, nlev, seed):
    return np.asfortranarray(np.random.default_rng(seed).standard_normal((m.nlon, m.nlat, nlev)))


def _sdot(a, b):
    return float(np.sum(a.real * b.real + a.imag * b.imag))


def _check_dot(backend, m, nlev, tol):
    s, g = _spec(m, nlev, 1), _grid(m, nlev, 2)
    Ss = m.grid(nlev)
    backend.Trans_Spherical_To_Grid(m, s, Ss)
    Stg = m.spectral(nlev)
    backend.Trans_Spherical_To_Grid_Adjoint(m, g, Stg)
    lhs, rhs = float(np.sum(Ss * g)), _sdot(s, Stg)
    assert abs(lhs - rhs) <= tol * (abs(lhs) + abs(rhs)), (lhs, rhs)
    Gg = m.spectral(nlev)
    backend.Trans_Grid_To_Spherical(m, g, Gg)
    Gts = m.grid(nlev)
    backend.Trans_Grid_To_Spherical_Adjoint(m, s, Gts)
    lhs, rhs = _sdot(Gg, s), float(np.sum(g * Gts))
    assert abs(lhs - rhs) <= tol * (abs(lhs) + abs(rhs)), (lhs, rhs)


@pytest.mark.parametrize("case", CASES)
def test_oracle_adjoint_dot_products(orc, case):
    N, nlat, nlon, nd = case
    m = orc.Spectral_Spherical_Mesh(N, N + 1, nlat, nlon, nd, 6371.0e3)
    _check_dot(orc, m, nd, 1e-12)


def test_oracle_adjoint_finite_differences(orc):
    """Gradient of J(s) = sum_g c * S2G(s) by central differences vs S2G^T c (a few entries)."""
    m = orc.Spectral_Spherical_Mesh(10, 11, 16, 32, 1, 1.0)
    c = _grid(m, 1, 3)
    s = _spec(m, 1, 4)
    gbar = m.spectral(1)
    orc.Trans_Spherical_To_Grid_Adjoint(m, c, gbar)
    eps = 1e-6
    for (mm, n, part) in [(0, 0, 0), (0, 3, 0), (2, 5, 0), (2, 5, 1), (7, 11, 1), (10, 10, 0)]:
        d = np.zeros_like(s)
        d[mm, n, 0] = eps if part == 0 else 1j * eps
        gp, gm = m.grid(1), m.grid(1)
        orc.Trans_Spherical_To_Grid(m, np.asfortranarray(s + d), gp)
        orc.Trans_Spherical_To_Grid(m, np.asfortranarray(s - d), gm)
        fd = float(np.sum(c * (gp - gm))) / (2 * eps)
        ad = gbar[mm, n, 0].real if part == 0 else gbar[mm, n, 0].imag
        assert abs(fd - ad) <= 1e-6 * max(1.0, abs(ad)), (mm, n, part, fd, ad)


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 5e-6), ("tf32x3", 1e-5)])
@pytest.mark.parametrize("case", CASES)
def test_gpu_adjoints(jg, orc, case, prec, tol):
    N, nlat, nlon, nd = case
    gm = jg.Spectral_Spherical_Mesh(N, N + 1, nlat, nlon, nd, 6371.0e3, precision=prec)
    om = orc.Spectral_Spherical_Mesh(N, N + 1, nlat, nlon, nd, 6371.0e3)
    for nlev in sorted({nd, 1}):
        g, s = _grid(om, nlev, 5 + nlev), _spec(om, nlev, 7 + nlev)
        a, b = gm.spectral(nlev), om.spectral(nlev)
        jg.Trans_Spherical_To_Grid_Adjoint(gm, g, a)
        orc.Trans_Spherical_To_Grid_Adjoint(om, g, b)
        assert configs.rel_l2(a, b) < tol
        a, b = gm.grid(nlev), om.grid(nlev)
        jg.Trans_Grid_To_Spherical_Adjoint(gm, s, a)
        orc.Trans_Grid_To_Spherical_Adjoint(om, s, b)
        assert configs.rel_l2(a, b) < tol
    _check_dot(jg, gm, nd, 1e-12 if prec == "fp64" else 1e-5)


# ---- one semi-implicit step (implicit correction + damping + filtered leapfrog) ------------------
_SCALE = {"dvor": 1e-10, "ddiv": 1e-10, "dt": 1e-5, "dlnps": 1e-9, "vor_p": 1e-5, "vor_c": 1e-5, "div_p": 1e-6,
          "div_c": 1e-6, "t_p": 1.0, "t_c": 1.0, "lnps_p": 1e-3, "lnps_c": 1e-3}


def _si_inputs(mesh, names, seed, scale=None):
    rng = np.random.default_rng(seed)
    out = {}
    for i, k in enumerate(names):
        nlev = 1 if k.startswith("lnps") or k == "dlnps" else mesh.nd
        a = _spec(mesh, nlev, seed * 100 + i)
        out[k] = np.asfortranarray(a * (scale[k] if scale else 1.0))
    del rng
    return out


def _si_dot(a, b):
    return sum(_sdot(a[k], b[k]) for k in a)


@pytest.mark.gpu
@pytest.mark.parametrize("init", [True, False])
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 2e-5)])
def test_gpu_semi_implicit_step_matches_oracle(jg, orc, init, prec, tol):
    name = "hs_t21l10"
    gm, om = configs.make_mesh(jg, name, precision=prec), configs.make_mesh(orc, name)
    gmod, omod = jg.Model(gm, configs.PARAMS[name]), orc.Model(om, configs.PARAMS[name])
    if not init:
        gmod.update_init_step()
        omod.update_init_step()
    x = _si_inputs(om, jg.SI_IN, 3, _SCALE)
    a, b = jg.Semi_Implicit_Step(gmod, x), orc.Semi_Implicit_Step(omod, x)
    for k in jg.SI_OUT:
        assert configs.rel_l2(a[k], b[k]) < tol, (k, configs.rel_l2(a[k], b[k]))


@pytest.mark.gpu
@pytest.mark.parametrize("init", [True, False])
def test_gpu_semi_implicit_step_adjoint(jg, init):
    """<J x, y> = <x, J^T y> for the step's linear map J (FP64), and J^T y reproduces a central
    finite difference of x -> <J x, y> in a few directions."""
    name = "hs_t21l10"
    gm = configs.make_mesh(jg, name, precision="fp64")
    md = jg.Model(gm, configs.PARAMS[name])
    if not init:
        md.update_init_step()
    x = _si_inputs(gm, jg.SI_IN, 5, _SCALE)
    y = _si_inputs(gm, jg.SI_OUT, 6)
    Jx = jg.Semi_Implicit_Step(md, x)
    JTy = jg.Semi_Implicit_Step_Adjoint(md, y)
    lhs, rhs = _si_dot(Jx, y), _si_dot(x, JTy)
    assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + abs(rhs)), (lhs, rhs)
    for k, (mm, n, lev) in [("ddiv", (1, 3, 2)), ("t_p", (0, 2, 5)), ("lnps_c", (2, 4, 0)), ("div_p", (4, 9, 7))]:
        d = {kk: np.zeros_like(v) for kk, v in x.items()}
        eps = 1e-3 * max(_SCALE[k], 1e-12)
        d[k][mm, n, lev] = eps
        plus = jg.Semi_Implicit_Step(md, {kk: x[kk] + d[kk] for kk in x})
        minus = jg.Semi_Implicit_Step(md, {kk: x[kk] - d[kk] for kk in x})
        fd = (_si_dot(plus, y) - _si_dot(minus, y)) / (2 * eps)
        ad = JTy[k][mm, n, lev].real
        assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-30) + 1e-12 * abs(lhs) / eps, (k, fd, ad)
