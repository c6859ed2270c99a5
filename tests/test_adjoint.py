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
