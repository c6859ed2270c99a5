"""The FP64 oracle against every known answer the reference's own tests hold (CPU only).

The reference ships no fixtures: its checks are analytic (Gauss_And_Legendre.jl:120-169 test();
Spectral_Spherical_Mesh.jl:763-1022 test_fourier, velocity_profile, test_derivative,
test_advection).  Each is restated here with the tolerance the algorithm achieves, plus
scipy's Gauss-Legendre nodes, numpy.fft for the FFT boundary (FFTW.jl, unpinned) and an
independent numpy restatement of the transforms.
"""
import numpy as np
import pytest
from scipy.special import roots_legendre

from jgcm import configs


@pytest.mark.parametrize("nlat", [32, 64, 128])
def test_gaussian_nodes(orc, nlat):
    s, w = orc.compute_gaussian(nlat)
    x, wx = roots_legendre(nlat)
    assert np.all(np.diff(s) > 0)  # south -> north (Gauss_And_Legendre.jl:113)
    assert np.max(np.abs(s - x)) < 5e-16
    # the weight uses P'_n at the pre-update Newton iterate (Gauss_And_Legendre.jl:102-114), which
    # costs ~n^2 * 1e-15 relative accuracy at the polar nodes
    assert np.max(np.abs(w - wx) / wx) < 1e-14 * nlat ** 2
    assert abs(w.sum() - 2.0) < 1e-14


def test_legendre_closed_forms(orc):
    """Gauss_And_Legendre.jl:132-156 (T21, nθ = 32): P and dP/dμ against closed forms."""
    s, _ = orc.compute_gaussian(32)
    q, dq = orc.compute_legendre(21, 22, s, 32)
    c = np.sqrt(1 - s ** 2)
    P = {(3, 3): np.sqrt(35) / 4 * c ** 3, (2, 3): np.sqrt(105 / 8) * (s - s ** 3),
         (0, 2): np.sqrt(5) / 2 * (3 * s ** 2 - 1), (0, 3): np.sqrt(7) / 2 * (5 * s ** 3 - 3 * s),
         (1, 3): np.sqrt(21) / 4 * (5 * s ** 2 - 1) * c}
    dP = {(3, 3): np.sqrt(35) / 4 * c * 1.5 * (-2 * s), (2, 3): np.sqrt(105 / 8) * (1 - 3 * s ** 2),
          (0, 2): np.sqrt(5) / 2 * 6 * s, (0, 3): np.sqrt(7) / 2 * (15 * s ** 2 - 3),
          (1, 3): np.sqrt(21) / 4 * 10 * s * c + np.sqrt(21) / 4 * (5 * s ** 2 - 1) / c * 0.5 * (-2 * s)}
    for (m, n), ref in P.items():
        assert np.linalg.norm(q[m, n] - ref) < 1e-13, (m, n)
    for (m, n), ref in dP.items():
        # dP/dμ is recovered from (1-μ²) dP/dμ by a division by cos²: ~1e-12 near the poles
        assert np.linalg.norm(dq[m, n] - ref) < 5e-12, (m, n)


@pytest.mark.parametrize("N,nlat", [(21, 32), (42, 64)])
def test_orthonormality(orc, N, nlat):
    """Gauss_And_Legendre.jl:158-168 (with the abs the reference's @assert lacks)."""
    s, w = orc.compute_gaussian(nlat)
    q, _ = orc.compute_legendre(N, N + 1, s, nlat)
    worst = 0.0
    for m in range(N + 1):
        G = 0.5 * np.einsum("aj,bj,j->ab", q[m, m:], q[m, m:], w)
        worst = max(worst, np.max(np.abs(G - np.eye(G.shape[0]))))
    assert worst < 1e-12


def test_fft_boundary(orc):
    M = orc.Spectral_Spherical_Mesh(31, 32, 48, 96, 2, 1.0)
    g = np.asfortranarray(np.random.default_rng(0).random((96, 48, 2)))
    f = np.zeros((96, 48, 2), dtype=np.complex128, order="F")
    orc.Trans_Grid_To_Fourier(M, g, f)
    assert np.max(np.abs(f - np.fft.fft(g, axis=0) / 96)) < 1e-15


def test_round_trip_idempotence(orc):
    """test_fourier (Spectral_Spherical_Mesh.jl:763-787): G2S∘S2G is a projection."""
    M = orc.Spectral_Spherical_Mesh(31, 32, 48, 96, 2, 1.0)
    p0 = np.asfortranarray(np.random.default_rng(1).random((96, 48, 2)))
    s0, s1, p1, p2 = M.spectral(2), M.spectral(2), M.grid(2), M.grid(2)
    orc.Trans_Grid_To_Spherical(M, p0, s0)
    orc.Trans_Spherical_To_Grid(M, s0, p1)
    orc.Trans_Grid_To_Spherical(M, p1, s1)
    orc.Trans_Spherical_To_Grid(M, s1, p2)
    assert np.linalg.norm(s0 - s1) < 1e-13
    assert np.linalg.norm(p1 - p2) < 1e-11
    assert np.all(s0[:, 32, :] == 0)


def _velocity_profile(M, IC):
    """velocity_profile (Spectral_Spherical_Mesh.jl:804-910) at T85, nθ = 128, nd = 3, radius 5."""
    nlon, nlat, nd, a = M.nlon, M.nlat, M.nd, M.radius
    c, s, lam = M.costh, M.sinth, M.lonc
    u, v, vor, div = (np.zeros((nlon, nlat, nd), order="F") for _ in range(4))
    U, b = 2 * np.pi / 256.0, np.pi / 2.0
    for k in range(nd):
        ic = IC if IC != "mix" else ["rigid_rotation", "random_1", "random_2"][k]
        if ic == "rigid_rotation":
            u[:, :, k] = U * (np.cos(b) * c[None, :] + np.sin(b) * np.cos(lam)[:, None] * s[None, :])
            v[:, :, k] = -U * np.sin(b) * np.sin(lam)[:, None] * np.ones(nlat)[None, :]
            vor[:, :, k] = 2 * U / a * (np.cos(b) * s[None, :] - np.sin(b) * np.cos(lam)[:, None] * c[None, :])
        elif ic == "random_1":
            u[:, :, k] = (c ** 2)[None, :]
            vor[:, :, k] = (3 * s * c / a)[None, :]
        else:
            u[:, :, k] = (25 * c - 30 * c ** 3 + 300 * s ** 2 * c ** 6)[None, :]
            vor[:, :, k] = (-(-50 * s + 120 * c ** 2 * s + 300 * (2 * c ** 7 * s - 7 * c ** 5 * s ** 3)) / a)[None, :]
    return u, v, vor, div


# truncation error of each analytic field (cos θ is poorly represented on the harmonics)
_DERIV_TOL = {"rigid_rotation": 1e-10, "random_1": 1e-3, "random_2": 1e-6, "mix": 1e-4}


@pytest.fixture(scope="module")
def t85(orc):
    return orc.Spectral_Spherical_Mesh(85, 86, 128, 256, 3, 5.0)


@pytest.mark.parametrize("IC", ["rigid_rotation", "random_1", "random_2", "mix"])
def test_derivative(orc, t85, IC):
    """test_derivative (Spectral_Spherical_Mesh.jl:916-943)."""
    M = t85
    u, v, vor0, div0 = _velocity_profile(M, IC)
    sv, sd = M.spectral(3), M.spectral(3)
    orc.Vor_Div_From_Grid_UV(M, u, v, sv, sd)
    gd, gv = M.grid(3), M.grid(3)
    orc.Trans_Spherical_To_Grid(M, sd, gd)
    orc.Trans_Spherical_To_Grid(M, sv, gv)
    assert np.linalg.norm(gd - div0) < 1e-10
    assert np.linalg.norm(gv - vor0) / np.linalg.norm(vor0) < _DERIV_TOL[IC]
    u1, v1 = M.grid(3), M.grid(3)
    orc.UV_Grid_From_Vor_Div(M, sv, sd, u1, v1)
    assert np.linalg.norm(u1 - u) / np.linalg.norm(u) < _DERIV_TOL[IC]
    assert np.linalg.norm(v1 - v) < 1e-10 + _DERIV_TOL[IC] * np.linalg.norm(v)


@pytest.mark.parametrize("IC,tol", [("rigid_rotation", 5e-2), ("random_1", 1e-9), ("random_2", 1e-8),
                                    ("mix", 1e-4)])
def test_advection(orc, t85, IC, tol):
    """test_advection (Spectral_Spherical_Mesh.jl:945-1008): -v·∇h against the analytic gradient.
    h contains 25 cos θ, which is not band-limited; where v is non-zero at the poles (rigid
    rotation about an equatorial axis) its truncated gradient leaves a ~2% error."""
    M = t85
    u, v, _, _ = _velocity_profile(M, IC)
    c, s, lam, a = M.costh, M.sinth, M.lonc, M.radius
    C, S, L = c[None, :], s[None, :], lam[:, None]
    h = 25 * C - 30 * C ** 3 + 300 * S ** 2 * C ** 6 * np.sin(L)
    gl = 300 * S ** 2 * C ** 5 * np.cos(L) / a
    gt = (-25 * S + 90 * C ** 2 * S + 600 * S * C ** 7 * np.sin(L) - 1800 * S ** 3 * C ** 5 * np.sin(L)) / a
    hs = np.asfortranarray(np.repeat(h[:, :, None], 3, axis=2))
    sh = M.spectral(3)
    orc.Trans_Grid_To_Spherical(M, hs, sh)
    dh = M.grid(3)
    orc.Add_Horizontal_Advection(M, sh, u, v, dh)
    ref = -(gl[:, :, None] * u + gt[:, :, None] * v)
    assert np.linalg.norm(dh - ref) / np.linalg.norm(ref) < tol


def _numpy_transforms(M):
    """Independent numpy restatement (direct sums over all latitudes, numpy.fft)."""
    N, nlat, nlon = M.num_fourier, M.nlat, M.nlon
    q, w = M.qnm, M.wts

    def s2g(snm):
        g = np.einsum("mnj,mnk->mjk", np.where(np.arange(N + 2)[None, :] >= np.arange(N + 1)[:, None], 1.0, 0.0)[
            :, :, None] * q, snm)
        full = np.zeros((nlon, nlat, snm.shape[2]), dtype=complex)
        full[: N + 1] = g
        full[0] = full[0].real
        out = np.real(full[0])[None] + 2 * np.real(np.fft.ifft(np.concatenate([0 * full[:1], full[1:]]), axis=0) * nlon)
        return out

    def g2s(grid):
        f = np.fft.fft(grid, axis=0) / nlon
        s = 0.5 * np.einsum("mnj,mjk->mnk", q * w[None, None, :], f[: N + 1])
        mask = np.arange(N + 2)[None, :] >= np.arange(N + 1)[:, None]
        s = s * mask[:, :, None]
        s[:, N + 1, :] = 0
        return s

    return s2g, g2s


@pytest.mark.parametrize("N,nlat,nlon", [(10, 16, 32), (21, 32, 64)])
def test_numpy_restatement(orc, N, nlat, nlon):
    M = orc.Spectral_Spherical_Mesh(N, N + 1, nlat, nlon, 2, 6371.0e3)
    s2g, g2s = _numpy_transforms(M)
    rng = np.random.default_rng(3)
    g = np.asfortranarray(rng.standard_normal((nlon, nlat, 2)))
    s = M.spectral(2)
    orc.Trans_Grid_To_Spherical(M, g, s)
    assert configs.rel_l2(s, g2s(g)) < 1e-13
    sn = np.asfortranarray(rng.standard_normal((N + 1, N + 2, 2)) + 1j * rng.standard_normal((N + 1, N + 2, 2)))
    for m in range(N + 1):
        sn[m, :m] = 0
    out = M.grid(2)
    orc.Trans_Spherical_To_Grid(M, sn, out)
    assert configs.rel_l2(out, s2g(sn)) < 1e-13


def test_hs_mass_fixer_and_step_finite(orc):
    """Compute_Corrections! keeps the area-mean surface pressure of the previous level."""
    name = "hs_t21l10"
    M = configs.make_mesh(orc, name)
    md = orc.Model(M, configs.PARAMS[name])
    md.spectral_initialize_fields(configs.hs_temperature_noise(M), True)
    ps0 = orc.Area_Weighted_Global_Mean(M, md.get("grid_ps_c"))
    md.step(6)
    assert not md.init_step
    ps1 = orc.Area_Weighted_Global_Mean(M, md.get("grid_ps_c"))
    assert abs(ps1 - ps0) / ps0 < 1e-13
    assert np.isfinite(md.get("grid_t_c")).all()


def test_oracle_tracers_advect_linearly_and_keep_a_uniform_field(orc):
    """Passive tracers (Dyn_Data's spe_tracers_*, advected like T): the step is linear in them
    (twice the tracer gives twice the result), a uniform tracer stays uniform, and the other
    prognostic fields do not see them."""
    name = "hs_t21l10"
    M = configs.make_mesh(orc, name)
    md = orc.Model(M, configs.PARAMS[name], num_tracers=3)
    ref = orc.Model(M, configs.PARAMS[name])
    for m in (md, ref):
        m.spectral_initialize_fields(configs.hs_temperature_noise(M), True)
    t, g = md.get("spe_t_c"), md.get("grid_t_c")
    spe = np.stack([t, 2 * t, np.zeros_like(t)], axis=3)
    spe[0, 0, :, 2] = 1.0
    grid = np.stack([g, 2 * g, np.ones_like(g)], axis=3)
    for f, v in (("spe_tracers_c", spe), ("spe_tracers_p", spe), ("grid_tracers_c", grid)):
        md.set(f, v)
    md.step(5)
    ref.step(5)
    q = md.get("spe_tracers_c")
    assert np.abs(q[..., 1] - 2 * q[..., 0]).max() <= 1e-12 * np.abs(q[..., 1]).max()
    assert np.abs(md.get("grid_tracers_c")[..., 2] - 1.0).max() < 1e-12
    assert configs.rel_l2(q[..., 0], md.get("spe_t_c")) > 1e-6  # stepped, not copied from T
    assert np.array_equal(md.get("spe_vor_c"), ref.get("spe_vor_c"))
    with pytest.raises(AssertionError):  # tracers belong to the Held-Suarez model
        orc.Model(configs.make_mesh(orc, "barotropic_t42"), configs.PARAMS["barotropic_t42"], num_tracers=1)


def test_vert_coord_tables(orc):
    """Compute_Vert_Coord (Vert_Coordinate.jl:61-87), zero top: even_sigma is LinRange(0, 1);
    uneven_sigma with surf_res = 1 is exp(-scale_heights (1 - k/nd)) inside, and with surf_res < 1
    stays increasing; the v197 table is symmetric about 1/2 (b_k + b_{nd-k} = 1 to its 7 printed decimals); mcm and v197 need
    their own level counts.  hybrid (a branch that does not run in the reference, built as its code
    means it): a zero top, pure pressure levels (b = 0, a = 101325 s) above s = 0.1, pure sigma
    levels (a = 0) below s = 0.3, and half-level pressures increasing for ps near 1e5 Pa."""
    ak, bk = orc.Compute_Vert_Coord(20, "even_sigma")
    assert np.all(ak == 0) and np.allclose(bk, np.linspace(0, 1, 21), rtol=0, atol=1e-15)
    ak, bk = orc.Compute_Vert_Coord(20, "uneven_sigma")
    k = np.arange(1, 20)
    assert np.all(ak == 0) and bk[0] == 0 and bk[20] == 1
    assert np.allclose(bk[1:20], np.exp(-4.0 * (1.0 - k / 20.0)), rtol=1e-15, atol=0)
    _, bk = orc.Compute_Vert_Coord(24, "uneven_sigma", scale_heights=5.0, surf_res=0.2, exponent=2.0)
    assert np.all(np.diff(bk) > 0) and bk[0] == 0 and bk[24] == 1
    _, b197 = orc.Compute_Vert_Coord(18, "v197")
    assert np.allclose(b197 + b197[::-1], 1.0, rtol=0, atol=1.5e-7) and np.all(np.diff(b197) > 0)
    _, bmcm = orc.Compute_Vert_Coord(14, "mcm")
    assert bmcm[0] == 0 and bmcm[14] == 1 and np.all(np.diff(bmcm) > 0)
    ah, bh = orc.Compute_Vert_Coord(20, "hybrid")
    _, s = orc.Compute_Vert_Coord(20, "uneven_sigma")
    assert ah[0] == 0 and bh[0] == 0 and ah[20] == 0 and bh[20] == 1
    upper, lower = (s > 0) & (s <= 0.1), s >= 0.3
    assert np.all(bh[upper] == 0) and np.allclose(ah[upper], 101325.0 * s[upper], rtol=1e-15, atol=0)
    assert np.all(ah[lower] == 0) and np.allclose(bh[lower], s[lower], rtol=1e-15, atol=0)
    for ps in (0.9e5, 1.0e5, 1.1e5):
        assert np.all(np.diff(ah + bh * ps) > 0)
    for nd, opt in ((20, "mcm"), (20, "v197"), (20, "sigma")):
        with pytest.raises(AssertionError):
            orc.Compute_Vert_Coord(nd, opt)


@pytest.mark.parametrize("name,option", configs.VERT_COORD_CASES)
def test_hs_vert_coords_mass_fixer_and_step_finite(orc, name, option):
    """Held-Suarez on the other vertical coordinates: the mass fixer holds the area-mean surface
    pressure and the state stays finite; the half-level pressures are a_k + b_k ps."""
    M = configs.make_mesh(orc, name)
    md = orc.Model(M, configs.PARAMS[name], vert_coord=option)
    md.spectral_initialize_fields(configs.hs_temperature_noise(M), True)
    ps0 = orc.Area_Weighted_Global_Mean(M, md.get("grid_ps_c"))
    md.step(6)
    ps1 = orc.Area_Weighted_Global_Mean(M, md.get("grid_ps_c"))
    assert abs(ps1 - ps0) / ps0 < 1e-13
    assert np.isfinite(md.get("grid_t_c")).all() and np.isfinite(md.get("spe_div_c")).all()
    ph = md.get("grid_p_half")
    ps = md.get("grid_ps_c")
    assert np.allclose(ph, md.ak[None, None, :] + ps[:, :, :1] * md.bk[None, None, :], rtol=1e-14, atol=0)


def test_barotropic_rh4_is_steady_pattern(orc):
    """The Rossby-Haurwitz wave 4 keeps its shape (it is an exact solution of the barotropic
    vorticity equation; damping and noise perturb it only slightly over 2 days)."""
    name = "barotropic_t42"
    M = configs.make_mesh(orc, name)
    md = orc.Model(M, configs.PARAMS[name])
    spe0 = configs.init_barotropic_rh4(orc, M, md)
    md.step(96)
    amp0 = np.abs(spe0[4, 5, 0])
    amp1 = np.abs(md.get("spe_vor_c")[4, 5, 0])
    assert abs(amp1 - amp0) / amp0 < 0.02


def test_generator_is_reproducible():
    a = configs.normal(configs.BASE_SEED, 1001)
    b = configs.normal(configs.BASE_SEED, 1001)
    assert np.array_equal(a, b)
    assert abs(a.mean()) < 0.1 and abs(a.std() - 1) < 0.1
    assert configs.splitmix64(0, 1)[0] == np.uint64(0xE220A8397B1DCDAF)  # published SplitMix64(0) output


def test_hs_forcing_restatement(orc):
    """The oracle's HS_Forcing! against a numpy restatement of HS_Forcing.jl:1-130."""
    from jgcm import configs as cf

    name = "hs_t21l10"
    mesh = cf.make_mesh(orc, name)
    md = orc.Model(mesh, cf.PARAMS[name])
    P = cf.PARAMS[name]
    rng = np.random.default_rng(3)
    nlon, nlat, nd = mesh.nlon, mesh.nlat, mesh.nd
    u, v = 20.0 * rng.standard_normal((3, nlon, nlat, nd))[:2]
    t = 220.0 + 80.0 * rng.random((nlon, nlat, nd))
    ps = 1.0e5 * (1.0 + 0.02 * rng.standard_normal((nlon, nlat)))
    p_half = ps[:, :, None] * np.linspace(0.0, 1.0, nd + 1)[None, None, :]
    p_full = 0.5 * (p_half[:, :, :-1] + p_half[:, :, 1:])
    u, v, t, p_half, p_full = (np.asfortranarray(a) for a in (u, v, t, p_half, p_full))
    outs = [np.zeros_like(u, order="F") for _ in range(4)]
    Dt = 2400
    orc.HS_Forcing(md, Dt, u, v, p_half, p_full, t, *outs)
    day, sb = 86400.0, P["sigma_b"]
    sigma = p_full / p_half[:, :, -1:]
    smax = np.maximum(0.0, sigma - sb)
    k_v = P["k_f"] / day / (1.0 - sb) * smax
    du, dv = -k_v * u, -k_v * v
    cp = P["rdgas"] / P["kappa"]
    dt = -((u + 0.5 * du * Dt) * du + (v + 0.5 * dv * Dt) * dv) / cp
    s, _ = orc.compute_gaussian(nlat)
    s2 = (s * s)[None, :, None]
    c2 = 1.0 - s2
    pn = p_full / 1.0e5
    teq = np.maximum(200.0, (315.0 - P["dT_y"] * s2 - P["dtheta_z"] * c2 * np.log(pn)) * pn ** P["kappa"])
    ka, ks = P["k_a"] / day, P["k_s"] / day
    dt = dt - (ka + (ks - ka) / (1.0 - sb) * smax * c2 * c2) * (t - teq)
    for a, b in zip(outs, (du, dv, teq, dt)):
        assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))


def rh4_phase_speed(backend, mesh, model, days=2):
    """Angular phase speed of the (m, n) = (4, 5) vorticity coefficient over `days` (Barotropic T42),
    from the pure wave (the seeded noise of the benchmark state is left out: its 1e-7 on every mode
    is comparable to this coefficient and shifts its phase by a few per cent)."""
    spe0 = configs.init_barotropic_rh4(backend, mesh, model, noise=0.0)
    steps = days * configs.STEPS_PER_DAY["barotropic_t42"]
    model.step(steps)
    spe1 = model.get("spe_vor_c")
    dphase = np.angle(spe1[4, 5, 0] / spe0[4, 5, 0])
    return -dphase / (4 * days * 86400.0)


def rh4_analytic_speed(omega_earth=7.292e-5, omega=7.848e-6, R=4):
    """Williamson et al. (1992) test case 6 for the non-divergent barotropic vorticity equation: the
    wave moves eastward at nu = (R (3 + R) omega - 2 Omega) / ((1 + R)(2 + R))."""
    return (R * (3 + R) * omega - 2 * omega_earth) / ((1 + R) * (2 + R))


def test_barotropic_rh4_phase_speed(orc):
    name = "barotropic_t42"
    M = configs.make_mesh(orc, name)
    md = orc.Model(M, configs.PARAMS[name])
    nu = rh4_phase_speed(orc, M, md)
    ref = rh4_analytic_speed(configs.PARAMS[name]["omega"])
    assert abs(nu - ref) / ref < 1e-3, (nu, ref)  # measured 2.8e-4 (leapfrog + Robert filter at dt 1800)


SW_TC2 = dict(num_fourier=42, nlat=64, nlon=128, nd=1, radius=6371.22e3)


def init_sw_steady_zonal_flow(backend, mesh, model, grav=9.80616, omega=7.292e-5, gh0=2.94e4):
    """Williamson et al. (1992) test case 2, steady nonlinear zonal geostrophic flow: u = u0 cos(lat),
    v = 0, geopotential gh0 - (a Omega u0 + u0^2 / 2) sin^2(lat), u0 = 2 pi a / 12 days.  Every time
    level holds the same state; returns the geopotential grid."""
    a = mesh.radius
    u0 = 2 * np.pi * a / (12 * 86400.0)
    lat = np.arcsin(mesh.sinth)
    u = np.asfortranarray(np.broadcast_to((u0 * np.cos(lat))[None, :], (mesh.nlon, mesh.nlat))[:, :, None].copy())
    h = np.asfortranarray(np.broadcast_to((gh0 - (a * omega * u0 + 0.5 * u0 * u0) * np.sin(lat) ** 2)[None, :],
                                          (mesh.nlon, mesh.nlat))[:, :, None].copy())
    v = mesh.grid(1)
    vor, div, sh = mesh.spectral(1), mesh.spectral(1), mesh.spectral(1)
    backend.Vor_Div_From_Grid_UV(mesh, u, v, vor, div)
    backend.Trans_Grid_To_Spherical(mesh, h, sh)
    gvor, gdiv, gh, gu, gv = (mesh.grid(1) for _ in range(5))
    backend.Trans_Spherical_To_Grid(mesh, vor, gvor)
    backend.Trans_Spherical_To_Grid(mesh, div, gdiv)
    backend.Trans_Spherical_To_Grid(mesh, sh, gh)
    backend.UV_Grid_From_Vor_Div(mesh, vor, div, gu, gv)
    for lev in ("c", "p"):
        model.set(f"spe_vor_{lev}", vor)
        model.set(f"spe_div_{lev}", div)
        model.set(f"spe_lnps_{lev}", sh)
        model.set(f"grid_u_{lev}", gu)
        model.set(f"grid_v_{lev}", gv)
        model.set(f"grid_ps_{lev}", gh)
    model.set("grid_vor", gvor)
    model.set("grid_div", gdiv)
    model.set("grid_lnps", gh)
    return gh


def sw_tc2_params(gh0=2.94e4):
    p = dict(configs.PARAMS["sw_t85"])
    p.update(grav=9.80616, h0=gh0, dt=1200)
    return p


def test_shallow_water_steady_zonal_flow(orc):
    """Williamson test case 2 stays steady: after one day the geopotential and the zonal wind differ
    from the initial state by a small fraction of their meridional variation."""
    g = SW_TC2
    M = orc.Spectral_Spherical_Mesh(g["num_fourier"], g["num_fourier"] + 1, g["nlat"], g["nlon"], 1, g["radius"])
    md = orc.Model(M, sw_tc2_params())
    h0 = init_sw_steady_zonal_flow(orc, M, md)
    u0 = md.get("grid_u_c")
    md.step(72)
    h1, u1 = md.get("grid_ps_c"), md.get("grid_u_c")
    # measured 6.5e-10 after one day (3.2e-9 after five)
    assert np.abs(h1 - h0).max() / (h0.max() - h0.min()) < 1e-8
    assert np.abs(u1 - u0).max() / np.abs(u0).max() < 1e-8
    assert np.abs(md.get("grid_v_c")).max() / np.abs(u0).max() < 1e-8
