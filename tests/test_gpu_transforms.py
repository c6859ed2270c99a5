"""GPU transforms vs the FP64 oracle, through the C ABI (ctypes).

Tolerances (relative L2 over the whole array): FP64 path 1e-12 (the oracle and the GPU sum in
different orders); FP32 path 5e-6 for single transforms; the tensor-core modes as stated at TOL.
"""
import numpy as np
import pytest

from jgcm import configs

pytestmark = pytest.mark.gpu

CASES = [(21, 32, 64, 3), (42, 64, 128, 20), (85, 128, 256, 2)]
# tf32x3 / bf16x3: the Legendre contraction on the tensor cores with 3-term split operands
# (hi*hi + hi*lo + lo*hi, FP32 accumulation); TF32 pairs carry ~21 bits, BF16 pairs ~16
TOL = {"fp64": 1e-12, "fp32": 5e-6, "tf32x3": 1e-5, "bf16x3": 1e-4}
PRECS = ["fp64", "fp32", "tf32x3", "bf16x3"]


def _meshes(jg, orc, N, nlat, nlon, nd, prec, radius=6371.0e3):
    return (jg.Spectral_Spherical_Mesh(N, N + 1, nlat, nlon, nd, radius, precision=prec),
            orc.Spectral_Spherical_Mesh(N, N + 1, nlat, nlon, nd, radius))


def _grid(m, nlev, seed):
    return np.asfortranarray(configs.normal(seed, m.nlon * m.nlat * nlev).reshape((m.nlon, m.nlat, nlev), order="F"))


def _spec(m, nlev, seed, lower=True):
    N1, S1 = m.num_fourier + 1, m.num_spherical + 1
    z = configs.normal(seed, 2 * N1 * S1 * nlev)
    s = (z[0::2] + 1j * z[1::2]).reshape((N1, S1, nlev), order="F")
    # decay with n like a smooth field
    n = np.arange(S1)[None, :, None]
    s = s / (1.0 + n) ** 1.5
    if not lower:
        for mm in range(N1):
            s[mm, :mm, :] = 0
    return np.asfortranarray(s)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("case", CASES)
def test_tables(jg, orc, case, prec):
    N, nlat, nlon, nd = case
    gm, om = _meshes(jg, orc, N, nlat, nlon, nd, prec)
    assert np.max(np.abs(gm.sinth - om.sinth)) < 2e-15
    assert np.max(np.abs(gm.wts - om.wts) / om.wts) < 1e-13
    assert configs.rel_l2(gm.qnm, om.qnm) < 1e-14
    assert configs.rel_l2(gm.dqnm, om.dqnm) < 1e-12
    for name in ("epsilon", "coef_uvm", "coef_uvc", "coef_uvp", "coef_dlam", "coef_dthm", "coef_dthp",
                 "laplacian_eig", "coef_alp_a", "coef_alp_b", "qwg"):
        assert configs.rel_l2(getattr(gm, name), getattr(om, name)) < 1e-13, name


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("case", CASES)
def test_spherical_to_grid(jg, orc, case, prec):
    N, nlat, nlon, nd = case
    gm, om = _meshes(jg, orc, N, nlat, nlon, nd, prec)
    for nlev in sorted({nd, 1}):
        s = _spec(om, nlev, 11 + nlev)  # includes junk below the diagonal: ignored by both
        a, b = gm.grid(nlev), om.grid(nlev)
        jg.Trans_Spherical_To_Grid(gm, s, a)
        orc.Trans_Spherical_To_Grid(om, s, b)
        assert configs.rel_l2(a, b) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("case", CASES)
def test_grid_to_spherical(jg, orc, case, prec):
    N, nlat, nlon, nd = case
    gm, om = _meshes(jg, orc, N, nlat, nlon, nd, prec)
    for nlev in sorted({nd, 1}):
        g = _grid(om, nlev, 5 + nlev)
        a, b = gm.spectral(nlev), om.spectral(nlev)
        jg.Trans_Grid_To_Spherical(gm, g, a)
        orc.Trans_Grid_To_Spherical(om, g, b)
        assert configs.rel_l2(a, b) < TOL[prec]
        assert np.all(a[:, N + 1, :] == 0)  # the extra total wavenumber is zeroed (:290)
        for mm in range(N + 1):
            assert np.all(a[mm, :mm, :] == 0)


@pytest.mark.parametrize("prec", ["fp32", "tf32x3"])
@pytest.mark.parametrize("name", ["hs_t21l20", "hs_t42l20"])
def test_row_per_thread_ffts(jg, orc, name, prec):
    """The row-per-thread FFT kernels (k_fft_rows / k_ifft_rows, nlon 64 and 128; chosen by size for
    member ensembles) forced on through the FFT tile knob of a model on the mesh."""
    g = configs.GRIDS[name]
    N, nlat, nlon, nd = g["num_fourier"], g["nlat"], g["nlon"], g["nd"]
    gm, om = _meshes(jg, orc, N, nlat, nlon, nd, prec)
    md = jg.Model(gm, configs.PARAMS[name])
    jg.set_tuning(md, dict(jg.get_tuning(md), fft_columns=-1))
    s = _spec(om, nd, 17)
    a, b = gm.grid(nd), om.grid(nd)
    jg.Trans_Spherical_To_Grid(gm, s, a)
    orc.Trans_Spherical_To_Grid(om, s, b)
    assert configs.rel_l2(a, b) < TOL[prec]
    gr = _grid(om, nd, 19)
    a, b = gm.spectral(nd), om.spectral(nd)
    jg.Trans_Grid_To_Spherical(gm, gr, a)
    orc.Trans_Grid_To_Spherical(om, gr, b)
    assert configs.rel_l2(a, b) < TOL[prec]
    err = (np.linalg.norm((a - b)[:, :N + 1].reshape(-1, nd), axis=0)
           / np.linalg.norm(b[:, :N + 1].reshape(-1, nd), axis=0))
    assert err.max() < 4 * TOL[prec], err.max()  # every level, not only the whole


# the zonal FFT runs in the mesh's arithmetic (FP32 in every mixed mode; no tensor cores)
FOURIER_TOL = {"fp64": 1e-13, "fp32": 2e-6, "tf32x3": 2e-6, "bf16x3": 2e-6}


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("case", CASES)
def test_grid_to_fourier(jg, orc, case, prec):
    """Trans_Grid_To_Fourier! fills the reference-shaped fourier_g [nλ, nθ, L] (every mode of
    fft/nλ, Spectral_Spherical_Mesh.jl:295-330): every element against the oracle's."""
    N, nlat, nlon, nd = case
    gm, om = _meshes(jg, orc, N, nlat, nlon, nd, prec)
    for nlev in sorted({nd, 1}):
        g = _grid(om, nlev, 3 + nlev)
        f = np.full((nlon, nlat, nlev), np.nan + 1j * np.nan, dtype=np.complex128, order="F")
        jg.Trans_Grid_To_Fourier(gm, g, f)
        ref = np.zeros((nlon, nlat, nlev), dtype=np.complex128, order="F")
        orc.Trans_Grid_To_Fourier(om, g, ref)
        assert np.isfinite(f).all()
        scale = np.abs(ref).max()
        assert np.abs(f - ref).max() <= FOURIER_TOL[prec] * scale, np.abs(f - ref).max() / scale
        assert configs.rel_l2(f, ref) < FOURIER_TOL[prec]
        # a real row: Hermitian spectrum, real mean and Nyquist modes
        assert np.array_equal(f[1:], np.conj(f[:0:-1]))
        assert np.all(f[0].imag == 0) and np.all(f[nlon // 2].imag == 0)
    with pytest.raises(AssertionError):  # the reference's shape, not modes 0..N only
        jg.Trans_Grid_To_Fourier(gm, _grid(om, nd, 3), np.zeros((N + 1, nlat, nd), dtype=np.complex128, order="F"))


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("case", CASES)
def test_vor_div_uv(jg, orc, case, prec):
    N, nlat, nlon, nd = case
    gm, om = _meshes(jg, orc, N, nlat, nlon, nd, prec)
    u, v = _grid(om, nd, 21), _grid(om, nd, 22)
    vg, dg, vr, dr = gm.spectral(nd), gm.spectral(nd), om.spectral(nd), om.spectral(nd)
    jg.Vor_Div_From_Grid_UV(gm, u, v, vg, dg)
    orc.Vor_Div_From_Grid_UV(om, u, v, vr, dr)
    assert configs.rel_l2(vg, vr) < TOL[prec] and configs.rel_l2(dg, dr) < TOL[prec]
    s1, s2 = _spec(om, nd, 31, lower=False), _spec(om, nd, 32, lower=False)
    ug, vgg, ur, vrr = gm.grid(nd), gm.grid(nd), om.grid(nd), om.grid(nd)
    jg.UV_Grid_From_Vor_Div(gm, s1, s2, ug, vgg)
    orc.UV_Grid_From_Vor_Div(om, s1, s2, ur, vrr)
    assert configs.rel_l2(ug, ur) < TOL[prec] and configs.rel_l2(vgg, vrr) < TOL[prec]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("case", CASES)
def test_gradients_advection_laplacian(jg, orc, case, prec):
    N, nlat, nlon, nd = case
    gm, om = _meshes(jg, orc, N, nlat, nlon, nd, prec)
    s = _spec(om, nd, 41, lower=False)
    a1, a2, b1, b2 = gm.grid(nd), gm.grid(nd), om.grid(nd), om.grid(nd)
    jg.Compute_Gradients(gm, s, a1, a2)
    orc.Compute_Gradients(om, s, b1, b2)
    assert configs.rel_l2(a1, b1) < TOL[prec] and configs.rel_l2(a2, b2) < TOL[prec]
    u, v, dh = _grid(om, nd, 42), _grid(om, nd, 43), _grid(om, nd, 44)
    dg, dr = dh.copy(order="F"), dh.copy(order="F")
    jg.Add_Horizontal_Advection(gm, s, u, v, dg)
    orc.Add_Horizontal_Advection(om, s, u, v, dr)
    assert configs.rel_l2(dg - dh, dr - dh) < 10 * TOL[prec]
    lg, lr = s.copy(order="F"), s.copy(order="F")
    jg.Apply_Laplacian(gm, lg)
    orc.Apply_Laplacian(om, lr)
    assert configs.rel_l2(lg, lr) < TOL[prec]
    g1 = _grid(om, 1, 45) + 3.0
    assert abs(jg.Area_Weighted_Global_Mean(gm, g1) - orc.Area_Weighted_Global_Mean(om, g1)) < 10 * TOL[prec] * 3


def test_shape_errors(jg):
    gm = jg.Spectral_Spherical_Mesh(21, 22, 32, 64, 3, 1.0)
    with pytest.raises(AssertionError):
        jg.Trans_Spherical_To_Grid(gm, gm.spectral(2), gm.grid(2))  # third dim must be nd or 1
    with pytest.raises(AssertionError):
        jg.Spectral_Spherical_Mesh(21, 23, 32, 64, 3, 1.0)  # num_spherical must be N+1
    with pytest.raises(AssertionError):
        jg.Spectral_Spherical_Mesh(21, 22, 31, 64, 3, 1.0)  # odd nlat (reference @assert)
