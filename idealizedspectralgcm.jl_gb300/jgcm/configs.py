"""Workload definitions: run parameters, seeded inputs and initial conditions.

The drivers below only call the reference-named API (``Spectral_Spherical_Mesh``,
``Trans_Grid_To_Spherical``, ``Model``...), so the same code initialises a model on the GPU
library (``jgcm``) or on any object exposing that API.

Workloads (sizes as in the reference experiments, exp/*):
  barotropic_t42   T42 (128x64), 1 level, FP64; Rossby-Haurwitz wave 4 (omega = K = 7.848e-6 /s,
                   Williamson et al. 1992 test 6) + N(0, 1e-7^2) noise on spectral vorticity n <= 42;
                   dt 1800 s, nabla^8 damping 1e-4, Robert 0.04 (exp/Barotropic/Barotropic.jl:25-33)
  sw_t85           T85 (256x128), shallow water; barotropically unstable jet, u_max 80 m/s at 45N,
                   mean depth 10 km, seeded 120 m height bump; semi-implicit, dt 600 s
  hs_t42l20        T42L20 Held-Suarez (exp/HSt42/HS.jl:8-54, Run_HS.jl:12): isothermal 264 K,
                   ps 1e5 Pa, N(0, 0.1^2) K white noise on the grid, the reference vorticity seed,
                   dt 1200 s
  hs_t21l20        T21L20 Held-Suarez, same physics (ensemble member size)
Seeded inputs come from one counter-based generator (SplitMix64 -> uniform -> Box-Muller),
base seed 20261203, member i uses seed + i.
"""
from __future__ import annotations

import math

import numpy as np

BASE_SEED = 20261203
DAY = 86400

GRIDS = {
    "barotropic_t42": dict(num_fourier=42, nlat=64, nlon=128, nd=1, radius=6371.2e3),
    "sw_t85": dict(num_fourier=85, nlat=128, nlon=256, nd=1, radius=6371.0e3),
    "hs_t42l20": dict(num_fourier=42, nlat=64, nlon=128, nd=20, radius=6371000.0),
    "hs_t21l20": dict(num_fourier=21, nlat=32, nlon=64, nd=20, radius=6371000.0),
    "hs_t21l10": dict(num_fourier=21, nlat=32, nlon=64, nd=10, radius=6371000.0),
    # the reference experiments' own grids (exp/Barotropic/Barotropic.jl:7-11, exp/Shallow_Water/SW.jl:7-12)
    "barotropic_t85_ref": dict(num_fourier=85, nlat=128, nlon=256, nd=1, radius=6371.2e3),
    "sw_t85_ref": dict(num_fourier=85, nlat=128, nlon=256, nd=1, radius=6371.0e3),
    # the level counts of Vert_Coordinate's fixed sigma tables (mcm: 14, v197: 18)
    "hs_t21l14": dict(num_fourier=21, nlat=32, nlon=64, nd=14, radius=6371000.0),
    "hs_t21l18": dict(num_fourier=21, nlat=32, nlon=64, nd=18, radius=6371000.0),
}

_COMMON = dict(robert_coef=0.04, damping_order=4, omega=7.292e-5, grav=9.80, rdgas=287.04, kappa=2.0 / 7.0,
               do_mass_correction=0, do_energy_correction=0, h0=0.0, kappa_m=0.0, kappa_t=0.0,
               sigma_b=0.7, k_f=1.0, k_a=1.0 / 40.0, k_s=1.0 / 4.0, dT_y=60.0, dtheta_z=10.0,
               ps_ref=1.0e5, t_ref=300.0, sea_level_ps_ref=1.0e5, init_t=264.0)

PARAMS = {
    "barotropic_t42": dict(_COMMON, kind="barotropic", damping_coef=1.0e-4, implicit_coef=0.0, dt=1800),
    "sw_t85": dict(_COMMON, kind="shallow_water", damping_coef=1.0e-4, implicit_coef=0.5, dt=600,
                   h0=9.80 * 1.0e4),
    "hs_t42l20": dict(_COMMON, kind="held_suarez", damping_coef=1.15741e-4, implicit_coef=0.5, dt=1200,
                      do_mass_correction=1, do_energy_correction=1),
}
# exp/Barotropic/Barotropic.jl:26-35 and exp/Shallow_Water/SW.jl:13-25,41-50 (h_0 = 3e4, friction and
# thermal relaxation times 20 and 10 days)
PARAMS["barotropic_t85_ref"] = dict(PARAMS["barotropic_t42"])
PARAMS["sw_t85_ref"] = dict(_COMMON, kind="shallow_water", damping_coef=1.0e-4, implicit_coef=0.5, dt=1200,
                            h0=3.0e4, kappa_m=1.0 / (20.0 * DAY), kappa_t=1.0 / (10.0 * DAY))
PARAMS["hs_t21l20"] = dict(PARAMS["hs_t42l20"])
PARAMS["hs_t21l10"] = dict(PARAMS["hs_t42l20"])
PARAMS["hs_t21l14"] = dict(PARAMS["hs_t42l20"])
PARAMS["hs_t21l18"] = dict(PARAMS["hs_t42l20"])

# Vert_Coordinate options with the grid whose level count each one needs
VERT_COORD_CASES = [("hs_t21l14", "mcm"), ("hs_t21l18", "v197"), ("hs_t21l20", "uneven_sigma"),
                    ("hs_t21l20", "hybrid")]

STEPS_PER_DAY = {k: DAY // v["dt"] for k, v in PARAMS.items()}


# ---- seeded generator -----------------------------------------------------------------------
_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n consecutive SplitMix64 outputs starting from state `seed` (uint64 array)."""
    with np.errstate(over="ignore"):
        z = np.uint64(seed % (1 << 64)) + (np.arange(1, n + 1, dtype=np.uint64) * _GOLDEN)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def normal(seed: int, n: int) -> np.ndarray:
    """n standard normal deviates: SplitMix64 -> 53-bit uniforms in (0,1) -> Box-Muller."""
    m = (n + 1) // 2
    z = splitmix64(seed, 2 * m)
    u = ((z >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)
    u1, u2 = u[0::2], u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    out = np.empty(2 * m)
    out[0::2] = r * np.cos(2.0 * math.pi * u2)
    out[1::2] = r * np.sin(2.0 * math.pi * u2)
    return out[:n]


# ---- builders -----------------------------------------------------------------------------
def make_mesh(backend, name: str, precision=None):
    g = GRIDS[name]
    N = g["num_fourier"]
    kw = {} if precision is None else {"precision": precision}
    return backend.Spectral_Spherical_Mesh(N, N + 1, g["nlat"], g["nlon"], g["nd"], g["radius"], **kw)


def init_barotropic_rh4(backend, mesh, model, seed=BASE_SEED, noise=1.0e-7):
    """Rossby-Haurwitz wave 4 vorticity + seeded spectral noise, then the reference barotropic
    driver's sequence (exp/Barotropic/Barotropic.jl:43-62): spectral vorticity, grid u, v, vor."""
    omega = K = 7.848e-6
    R = 4
    mu = mesh.sinth
    lat = np.arcsin(mu)
    lon = 2 * np.pi * np.arange(mesh.nlon) / mesh.nlon
    LAT, LON = np.meshgrid(lat, lon)  # [nlon, nlat]
    vor = 2 * omega * np.sin(LAT) - K * np.sin(LAT) * np.cos(LAT) ** R * (R * R + 3 * R + 2) * np.cos(R * LON)
    grid_vor = np.asfortranarray(vor[:, :, None])
    spe = mesh.spectral(1)
    backend.Trans_Grid_To_Spherical(mesh, grid_vor, spe)
    N = mesh.num_fourier
    nz = normal(seed, 2 * (N + 1) * (N + 2))
    idx = 0
    for m in range(N + 1):
        for n in range(m, N + 1):
            re, im = nz[idx], nz[idx + 1]
            idx += 2
            spe[m, n, 0] += noise * re + (1j * noise * im if m > 0 else 0.0)
    u, v, gv = mesh.grid(1), mesh.grid(1), mesh.grid(1)
    backend.Trans_Spherical_To_Grid(mesh, spe, gv)
    backend.UV_Grid_From_Vor_Div(mesh, spe, mesh.spectral(1), u, v)
    model.set("spe_vor_c", spe)
    model.set("spe_vor_p", spe)
    model.set("grid_vor", gv)
    model.set("grid_u_c", u)
    model.set("grid_v_c", v)
    model.set("grid_u_p", u)
    model.set("grid_v_p", v)
    return spe


def galewsky_fields(mesh, grav=9.80, omega=7.292e-5, u_max=80.0, depth=1.0e4, bump=120.0, lon_c=0.0):
    """Barotropically unstable mid-latitude jet (Galewsky et al. 2004 profile, centred at 45N)
    in gradient-wind balance, plus a localised height bump; returns (u, h) with h as geopotential
    (the reference stores geopotential in its h slot, exp/Shallow_Water/SW.jl:17)."""
    a = mesh.radius
    phi0, phi1 = np.pi / 7.0, np.pi / 2.0 - np.pi / 7.0
    en = np.exp(-4.0 / (phi1 - phi0) ** 2)

    def ujet(phi):
        out = np.zeros_like(phi)
        inside = (phi > phi0) & (phi < phi1)
        p = phi[inside]
        out[inside] = u_max / en * np.exp(1.0 / ((p - phi0) * (p - phi1)))
        return out

    # balanced geopotential: dΦ/dφ = -a u (f + u tanφ / a), integrated from the south pole
    fine = np.linspace(-np.pi / 2, np.pi / 2, 20001)
    uf = ujet(fine)
    integrand = -a * uf * (2 * omega * np.sin(fine) + uf * np.tan(np.clip(fine, -1.5707, 1.5707)) / a)
    cum = np.concatenate([[0.0], np.cumsum(0.5 * (integrand[1:] + integrand[:-1]) * np.diff(fine))])
    lat = np.arcsin(mesh.sinth)
    phi_bal = np.interp(lat, fine, cum)
    # shift so the area mean equals g * depth
    w = mesh.wts
    phi_bal = phi_bal - np.sum(phi_bal * w) / 2.0 + grav * depth
    lon = 2 * np.pi * np.arange(mesh.nlon) / mesh.nlon
    LAT, LON = np.meshgrid(lat, lon)
    dl = np.angle(np.exp(1j * (LON - lon_c)))
    hb = bump * np.cos(LAT) * np.exp(-(dl / (1.0 / 3.0)) ** 2) * np.exp(-((np.pi / 4 - LAT) / (1.0 / 15.0)) ** 2)
    u = np.asfortranarray(np.broadcast_to(ujet(lat)[None, :], (mesh.nlon, mesh.nlat))[:, :, None].copy())
    h = np.asfortranarray((phi_bal[None, :] + grav * hb)[:, :, None])
    return u, h


def init_shallow_water_jet(backend, mesh, model, seed=BASE_SEED, grav=9.80):
    """Unstable jet + seeded bump (bump longitude drawn from the seeded generator)."""
    z = splitmix64(seed, 1)[0]
    lon_c = 2 * np.pi * float(z >> np.uint64(11)) / 9007199254740992.0
    u, h = galewsky_fields(mesh, grav=grav, lon_c=lon_c)
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
    model.set("grid_lnps", h)


def init_barotropic_reference(backend, mesh, model):
    """The reference barotropic experiment's initial state (exp/Barotropic/Barotropic.jl:43-62): the
    zonal wind u = 25 cosθ - 30 cos³θ + 300 sin²θ cos⁶θ, v = 0, its vorticity and divergence (spectral
    and on the grid), then an m = 4 vorticity bump A/2 cosθ exp(-((θ-θ0)/θw)²) cos(4λ) (A = 8e-5,
    θ0 = 45°, θw = 15°) added on the grid and analysed back into the spectral vorticity.  As in the
    reference, grid u, v keep the unperturbed wind and every other field starts at zero."""
    cos, sin = mesh.costh, mesh.sinth
    lat, lon = mesh.latc, mesh.lonc
    u = mesh.grid(1)
    u[:, :, 0] = (25.0 * cos - 30.0 * cos ** 3 + 300.0 * sin ** 2 * cos ** 6)[None, :]
    v = mesh.grid(1)
    vor, div = mesh.spectral(1), mesh.spectral(1)
    backend.Vor_Div_From_Grid_UV(mesh, u, v, vor, div)
    gvor, gdiv = mesh.grid(1), mesh.grid(1)
    backend.Trans_Spherical_To_Grid(mesh, vor, gvor)
    backend.Trans_Spherical_To_Grid(mesh, div, gdiv)
    m, th0, thw, A = 4.0, 45.0 * math.pi / 180.0, 15.0 * math.pi / 180.0, 8.0e-5
    gvor[:, :, 0] += (A / 2.0 * cos[None, :] * np.exp(-((lat[None, :] - th0) / thw) ** 2)
                      * np.cos(m * lon[:, None]))
    backend.Trans_Grid_To_Spherical(mesh, gvor, vor)
    model.set("grid_u_c", u)
    model.set("grid_v_c", v)
    model.set("spe_vor_c", vor)
    model.set("grid_vor", gvor)
    return vor


def sw_reference_h_eq(mesh, h_0=3.0e4, h_amp=2.0e4, h_lon=math.pi / 2, h_lat=25.0 * math.pi / 180.0,
                      h_width=15.0 * math.pi / 180.0, h_itcz=1.0e5, itcz_width=4.0 * math.pi / 180.0):
    """The relaxation height of the reference shallow-water experiment (exp/Shallow_Water/SW.jl:69-80):
    h_0 + a Gaussian mound at (90°E, 25°N) + an equatorial ITCZ ridge, [nλ, nθ, 1]."""
    lat, lon = mesh.latc, mesh.lonc
    d2 = (lat / itcz_width) ** 2
    x2 = ((lon[:, None] - h_lon) / (2.0 * h_width)) ** 2
    y2 = ((lat[None, :] - h_lat) / h_width) ** 2
    return np.asfortranarray((h_0 + h_amp * np.exp(-(x2 + y2)) + h_itcz * np.exp(-d2)[None, :])[:, :, None])


def init_shallow_water_reference(backend, mesh, model, h_0=3.0e4):
    """The reference shallow-water experiment's initial state (exp/Shallow_Water/SW.jl:57-80): at rest,
    h = h_0 seeded into grid_lnps and analysed into spe_lnps_c, h_eq for Shallow_Water_Physics!.  The
    dynamics read h from grid_ps_c, which stays zero (and spe_lnps_p stays zero), so the first step
    sees h = 0 on the grid: the reference's own quirk, kept."""
    u, v = mesh.grid(1), mesh.grid(1)
    vor, div = mesh.spectral(1), mesh.spectral(1)
    backend.Vor_Div_From_Grid_UV(mesh, u, v, vor, div)
    gvor, gdiv = mesh.grid(1), mesh.grid(1)
    backend.Trans_Spherical_To_Grid(mesh, vor, gvor)
    backend.Trans_Spherical_To_Grid(mesh, div, gdiv)
    gh = np.asfortranarray(np.full((mesh.nlon, mesh.nlat, 1), h_0))
    sh = mesh.spectral(1)
    backend.Trans_Grid_To_Spherical(mesh, gh, sh)
    model.set("grid_u_c", u)
    model.set("grid_v_c", v)
    model.set("spe_vor_c", vor)
    model.set("spe_div_c", div)
    model.set("grid_vor", gvor)
    model.set("grid_div", gdiv)
    model.set("grid_lnps", gh)
    model.set("spe_lnps_c", sh)
    model.set("grid_h_eq", sw_reference_h_eq(mesh, h_0=h_0))


def hs_temperature_noise(mesh, seed=BASE_SEED, amplitude=0.1):
    n = mesh.nlon * mesh.nlat * mesh.nd
    return np.asfortranarray(amplitude * normal(seed, n).reshape((mesh.nlon, mesh.nlat, mesh.nd), order="F"))


def init_held_suarez(backend, mesh, model, seed=BASE_SEED, amplitude=0.1, vorticity_seed=True):
    """Spectral_Initialize_Fields! (Spectral_Dynamics.jl:372-449) with seeded grid noise on T."""
    model.spectral_initialize_fields(hs_temperature_noise(mesh, seed, amplitude), vorticity_seed)


def add_hs_flow(backend, mesh, model, u0=20.0, wave=2.0e-6):
    """Superpose a solid-body zonal flow u0 cos(lat) and a wave-4 vorticity pattern on both time
    levels of a Held-Suarez state (a developed-flow start for parity checks: from rest,
    vorticity and divergence are at the roundoff level of the 1e5 m^2/s^2 geopotential)."""
    nd = mesh.nd
    for lev in ("c", "p"):
        vor = model.get(f"spe_vor_{lev}")
        div = model.get(f"spe_div_{lev}")
        vor[0, 1, :] += 2.0 * u0 / (mesh.radius * math.sqrt(3.0))  # 2 u0 sin(lat) / a = c P_1^0
        vor[4, 5, :] += wave * (1.0 + 0.5j) * np.linspace(0.5, 1.5, nd)
        vor[2, 7, :] += 0.5 * wave * np.linspace(1.5, 0.5, nd)
        model.set(f"spe_vor_{lev}", vor)
        u, v, gv = mesh.grid(nd), mesh.grid(nd), mesh.grid(nd)
        backend.UV_Grid_From_Vor_Div(mesh, vor, div, u, v)
        model.set(f"grid_u_{lev}", u)
        model.set(f"grid_v_{lev}", v)
        if lev == "c":
            backend.Trans_Spherical_To_Grid(mesh, vor, gv)
            model.set("grid_vor", gv)


PROGNOSTIC = {
    "barotropic": ["spe_vor_c", "spe_vor_p", "grid_u_c", "grid_v_c", "grid_vor"],
    "shallow_water": ["spe_vor_c", "spe_div_c", "spe_lnps_c", "grid_u_c", "grid_v_c", "grid_ps_c", "grid_vor",
                      "grid_div"],
    "held_suarez": ["spe_vor_c", "spe_div_c", "spe_t_c", "spe_lnps_c", "grid_u_c", "grid_v_c", "grid_t_c",
                    "grid_ps_c", "spe_vor_p", "spe_t_p", "grid_t_p", "grid_ps_p"],
}


def copy_state(src_model, dst_model, kind):
    """Copy every field the next step reads from one model to another (any backends)."""
    names = {
        "barotropic": ["spe_vor_c", "spe_vor_p", "grid_u_c", "grid_v_c", "grid_u_p", "grid_v_p", "grid_vor"],
        "shallow_water": ["spe_vor_c", "spe_vor_p", "spe_div_c", "spe_div_p", "spe_lnps_c", "spe_lnps_p",
                          "spe_lnps_n", "grid_u_c", "grid_v_c", "grid_ps_c", "grid_u_p", "grid_v_p", "grid_ps_p",
                          "grid_vor", "grid_div", "grid_h_eq"],
        "held_suarez": ["spe_vor_c", "spe_vor_p", "spe_div_c", "spe_div_p", "spe_lnps_c", "spe_lnps_p", "spe_t_c",
                        "spe_t_p", "grid_u_c", "grid_u_p", "grid_v_c", "grid_v_p", "grid_ps_c", "grid_ps_p",
                        "grid_t_c", "grid_t_p", "grid_vor", "grid_div", "grid_geopots"],
    }[kind]
    for n in names:
        dst_model.set(n, src_model.get(n))


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
