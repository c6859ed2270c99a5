"""FP64 CPU oracle for the JGCM spectral dynamical core -- TEST INFRASTRUCTURE ONLY.

ctypes front end of ``jgcm_oracle.c``, a line-by-line FP64 restatement of the reference
(CliMA/IdealizedSpectralGCM.jl).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this module; the
product path (``jgcm``) never does.

The Python surface mirrors the reference names (``Trans_Spherical_To_Grid`` for
``Trans_Spherical_To_Grid!`` and so on, mutating their output argument) so the same
driver code runs against the oracle and against the GPU library.  Arrays use the
reference's Julia layout: numpy Fortran order, grid ``float64[nlon, nlat, nlev]``,
spectral ``complex128[N+1, N+2, nlev]``.

Parity pins (no golden vectors exist upstream): the analytic known-answer checks of
``Gauss_And_Legendre.jl:120-169`` and ``Spectral_Spherical_Mesh.jl:763-1022``, scipy's
Gauss-Legendre nodes and numpy.fft, all exercised by ``tests/test_oracle.py``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libjgcm_oracle.so")
_SOURCES = ["jgcm_oracle.c", "jgcm_oracle_models.inc", "jgcm_oracle_adjoint.inc", "jgcm_oracle.h"]


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (-ffp-contract=off keeps x86 and Arm bitwise alike)."""
    os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
    newest = max(os.path.getmtime(os.path.join(_HERE, s)) for s in _SOURCES)
    if not force and os.path.exists(_LIB_PATH) and os.path.getmtime(_LIB_PATH) >= newest:
        return _LIB_PATH
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-o", tmp,
           os.path.join(_HERE, "jgcm_oracle.c"), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        P, I, D, L = C.c_void_p, C.c_int, C.c_double, C.c_long
        sig = {
            "om_compute_gaussian": (I, [I, P, P]),
            "om_compute_legendre": (I, [I, I, P, I, P, P]),
            "om_mesh_create": (P, [I, I, I, I, I, D]),
            "om_mesh_destroy": (None, [P]),
            "om_mesh_table": (L, [P, C.c_char_p, P, L]),
            "om_set_threads": (None, [I]),
            "om_set_f32": (None, [I]),
            "om_trans_spherical_to_grid": (None, [P, P, I, P]),
            "om_trans_grid_to_spherical": (None, [P, P, I, P]),
            "om_trans_grid_to_fourier": (None, [P, P, I, P]),
            "om_vor_div_from_grid_uv": (None, [P, P, P, I, P, P]),
            "om_uv_grid_from_vor_div": (None, [P, P, P, I, P, P]),
            "om_compute_gradients": (None, [P, P, I, P, P]),
            "om_add_horizontal_advection": (None, [P, P, P, P, I, P]),
            "om_apply_laplacian": (None, [P, P, I]),
            "om_area_weighted_global_mean": (D, [P, P]),
            "om_model_create": (P, [P, P]),
            "om_model_create_vert": (P, [P, P, P, P]),
            "om_vert_coord": (I, [I, C.c_char_p, D, D, D, P, P]),
            "om_model_destroy": (None, [P]),
            "om_model_add_tracers": (I, [P, I]),
            "om_model_field": (L, [P, C.c_char_p, P, L, I]),
            "om_model_init_step": (I, [P]),
            "om_model_update_init_step": (I, [P]),
            "om_model_step": (I, [P, I]),
            "om_model_fixer_scalars": (None, [P, P]),
            "om_spectral_initialize_fields": (I, [P, P, I]),
            "om_model_semi_implicit": (L, [P, C.c_char_p, P, L]),
            "om_hs_forcing": (None, [P, I, P, P, P, P, P, P, P, P, P]),
            "om_semi_implicit_step": (None, [P, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
            "om_trans_spherical_to_grid_adjoint": (None, [P, P, I, P]),
            "om_trans_grid_to_spherical_adjoint": (None, [P, P, I, P]),
            "om_model_sync_pressure": (None, [P]),
            "om_model_set_init_step": (I, [P, I]),
            "om_vor_div_from_grid_uv_adjoint": (None, [P, P, P, I, P, P]),
            "om_uv_grid_from_vor_div_adjoint": (None, [P, P, P, I, P, P]),
            "om_compute_gradients_adjoint": (None, [P, P, P, I, P]),
            "om_hs_step_adjoint": (I, [P, C.POINTER(C.c_void_p), P]),
        }
        for name, (res, args) in sig.items():
            f = getattr(_lib, name)
            f.restype = res
            f.argtypes = args
    return _lib


def set_threads(n: int) -> None:
    lib().om_set_threads(int(n))


# FP32 emulation switches for error bisection (jgcm_oracle.h); 0 = the FP64 restatement
F32_STAGES = {"fft_fwd": 1, "analysis": 2, "synthesis": 4, "fft_inv": 8, "grid": 16, "spectral": 32}
F32_TANOM = 64  # the geopotential on T synthesised without its level means (the GPU's FP32 formulation)
F32_FIXER = 128  # the fixers' column energy integrals in FP32, the global fold in FP64
F32_FIXER_KE = 256  # only their kinetic part in FP32, c_p T and the sums in FP64 (the GPU's FP32 path)


def set_f32(mask: int) -> None:
    lib().om_set_f32(int(mask))


def _ptr(a: np.ndarray):
    assert a.flags.f_contiguous, "arrays must be Fortran-ordered (Julia layout)"
    return a.ctypes.data_as(C.c_void_p)


def compute_gaussian(n: int):
    """Gauss_And_Legendre.jl:69-118 Compute_Gaussian!(n) -> (sinθ, wts)."""
    s = np.zeros(n)
    w = np.zeros(n)
    lib().om_compute_gaussian(n, _ptr(s), _ptr(w))
    return s, w


def compute_legendre(num_fourier, num_spherical, sinth, nlat):
    """Gauss_And_Legendre.jl:4-66 Compute_Legendre! -> (qnm, dqnm), each [N+1, ns+1, nlat]."""
    sinth = np.asfortranarray(sinth, dtype=np.float64)
    q = np.zeros((num_fourier + 1, num_spherical + 1, nlat), order="F")
    dq = np.zeros_like(q)
    lib().om_compute_legendre(num_fourier, num_spherical, _ptr(sinth), nlat, _ptr(q), _ptr(dq))
    return q, dq


class Spectral_Spherical_Mesh:
    """Spectral_Spherical_Mesh.jl:69-139 (argument order num_fourier, num_spherical, nθ, nλ, nd, radius)."""

    _TABLES3 = ("qnm", "dqnm", "qwg", "coef_alp_a", "coef_alp_b")
    _TABLES2 = ("epsilon", "coef_uvm", "coef_uvc", "coef_uvp", "coef_dlam", "coef_dthm", "coef_dthp",
                "laplacian_eig")

    def __init__(self, num_fourier, num_spherical, nlat, nlon, nd, radius):
        self.num_fourier, self.num_spherical = int(num_fourier), int(num_spherical)
        self.nlat, self.nlon, self.nd, self.radius = int(nlat), int(nlon), int(nd), float(radius)
        h = lib().om_mesh_create(self.num_fourier, self.num_spherical, self.nlat, self.nlon, self.nd, self.radius)
        if not h:
            raise AssertionError("invalid mesh dimensions")
        self._h = h
        for name in ("sinth", "costh", "wts", "lonc", "latc") + self._TABLES3 + self._TABLES2:
            setattr(self, name, self._table(name))

    def _table(self, name):
        n = lib().om_mesh_table(self._h, name.encode(), None, 0)
        out = np.zeros(n)
        lib().om_mesh_table(self._h, name.encode(), _ptr(out), n)
        N1, S1 = self.num_fourier + 1, self.num_spherical + 1
        if name in self._TABLES3:
            return out.reshape((N1, S1, self.nlat), order="F")
        if name in self._TABLES2:
            return out.reshape((N1, S1), order="F")
        return out

    def __del__(self):
        if getattr(self, "_h", None):
            lib().om_mesh_destroy(self._h)
            self._h = None

    # layout helpers
    def spectral(self, nlev):
        return np.zeros((self.num_fourier + 1, self.num_spherical + 1, nlev), dtype=np.complex128, order="F")

    def grid(self, nlev):
        return np.zeros((self.nlon, self.nlat, nlev), order="F")


def _nlev_spec(mesh, a):
    assert a.dtype == np.complex128 and a.shape[:2] == (mesh.num_fourier + 1, mesh.num_spherical + 1)
    assert a.shape[2] in (mesh.nd, 1)
    return a.shape[2]


def _nlev_grid(mesh, a):
    assert a.dtype == np.float64 and a.shape[:2] == (mesh.nlon, mesh.nlat)
    assert a.shape[2] in (mesh.nd, 1)
    return a.shape[2]


def Trans_Spherical_To_Grid(mesh, snm, pfield):
    n = _nlev_spec(mesh, snm)
    assert _nlev_grid(mesh, pfield) == n
    lib().om_trans_spherical_to_grid(mesh._h, _ptr(snm), n, _ptr(pfield))


def Trans_Grid_To_Spherical(mesh, pfield, snm):
    n = _nlev_grid(mesh, pfield)
    assert _nlev_spec(mesh, snm) == n
    lib().om_trans_grid_to_spherical(mesh._h, _ptr(pfield), n, _ptr(snm))


def Trans_Grid_To_Fourier(mesh, pfield, fourier):
    n = _nlev_grid(mesh, pfield)
    assert fourier.dtype == np.complex128 and fourier.shape == pfield.shape
    lib().om_trans_grid_to_fourier(mesh._h, _ptr(pfield), n, _ptr(fourier))


def Vor_Div_From_Grid_UV(mesh, grid_u, grid_v, vor, div):
    n = _nlev_grid(mesh, grid_u)
    lib().om_vor_div_from_grid_uv(mesh._h, _ptr(grid_u), _ptr(grid_v), n, _ptr(vor), _ptr(div))


def UV_Grid_From_Vor_Div(mesh, vor, div, grid_u, grid_v):
    n = _nlev_spec(mesh, vor)
    lib().om_uv_grid_from_vor_div(mesh._h, _ptr(vor), _ptr(div), n, _ptr(grid_u), _ptr(grid_v))


def Compute_Gradients(mesh, spe_hs, grid_dlam_hs, grid_dth_hs):
    n = _nlev_spec(mesh, spe_hs)
    lib().om_compute_gradients(mesh._h, _ptr(spe_hs), n, _ptr(grid_dlam_hs), _ptr(grid_dth_hs))


def Add_Horizontal_Advection(mesh, spe_hs, grid_u, grid_v, grid_dhs):
    n = _nlev_spec(mesh, spe_hs)
    lib().om_add_horizontal_advection(mesh._h, _ptr(spe_hs), _ptr(grid_u), _ptr(grid_v), n, _ptr(grid_dhs))


def Apply_Laplacian(mesh, spe):
    lib().om_apply_laplacian(mesh._h, _ptr(spe), _nlev_spec(mesh, spe))


def Area_Weighted_Global_Mean(mesh, grid):
    _nlev_grid(mesh, grid)
    return lib().om_area_weighted_global_mean(mesh._h, _ptr(grid))


class _Params(C.Structure):
    _fields_ = [("kind", C.c_int), ("robert_coef", C.c_double), ("damping_order", C.c_int),
                ("damping_coef", C.c_double), ("implicit_coef", C.c_double), ("dt", C.c_int),
                ("omega", C.c_double), ("grav", C.c_double), ("rdgas", C.c_double), ("kappa", C.c_double),
                ("do_mass_correction", C.c_int), ("do_energy_correction", C.c_int),
                ("h0", C.c_double), ("kappa_m", C.c_double), ("kappa_t", C.c_double),
                ("sigma_b", C.c_double), ("k_f", C.c_double), ("k_a", C.c_double), ("k_s", C.c_double),
                ("dT_y", C.c_double), ("dtheta_z", C.c_double), ("ps_ref", C.c_double), ("t_ref", C.c_double),
                ("sea_level_ps_ref", C.c_double), ("init_t", C.c_double)]


KINDS = {"barotropic": 0, "shallow_water": 1, "held_suarez": 2}


def Compute_Vert_Coord(nd, vert_coord_option, scale_heights=4.0, surf_res=1.0, exponent=2.5):
    """Vert_Coordinate.jl:61-87 (zero top): (ak, bk), nd+1 each."""
    ak, bk = np.zeros(nd + 1), np.zeros(nd + 1)
    if lib().om_vert_coord(int(nd), vert_coord_option.encode(), float(scale_heights), float(surf_res),
                           float(exponent), ak.ctypes.data_as(C.c_void_p), bk.ctypes.data_as(C.c_void_p)):
        raise AssertionError(f"Compute_Vert_Coord: {vert_coord_option!r} with nd = {nd} is not supported")
    return ak, bk


class Model:
    """Dyn_Data + Filtered_Leapfrog (+ Semi_Implicit_Solver for Held-Suarez) on the oracle.

    ``vert_coord``: a Vert_Coordinate option (see ``Compute_Vert_Coord``) or a pair (ak, bk).
    ``num_tracers``: passive tracers (Dyn_Data's spe_tracers_* / grid_tracers_*, [.., nd, nq]) advected
    like T (Held-Suarez only)."""

    def __init__(self, mesh, params: dict, vert_coord="even_sigma", num_tracers=0, **vert_options):
        self.mesh = mesh
        self.params = dict(params)
        if isinstance(vert_coord, str):
            vert_coord = Compute_Vert_Coord(mesh.nd, vert_coord, **vert_options)
        self.ak, self.bk = (np.ascontiguousarray(x, dtype=np.float64) for x in vert_coord)
        p = _Params()
        for name, _ in _Params._fields_:
            if name == "kind":
                p.kind = KINDS[params["kind"]]
            elif name in params:
                setattr(p, name, params[name])
        self._p = p
        self._h = lib().om_model_create_vert(mesh._h, C.byref(p), self.ak.ctypes.data_as(C.c_void_p),
                                             self.bk.ctypes.data_as(C.c_void_p))
        if not self._h:
            raise AssertionError("model creation failed")
        self.num_tracers = int(num_tracers)
        if self.num_tracers and lib().om_model_add_tracers(self._h, self.num_tracers) != 0:
            raise AssertionError("tracers need a Held-Suarez model and num_tracers >= 1")

    def __del__(self):
        if getattr(self, "_h", None):
            lib().om_model_destroy(self._h)
            self._h = None

    def _shape(self, name, n):
        m = self.mesh
        N1, S1 = m.num_fourier + 1, m.num_spherical + 1
        if name.startswith("spe_"):
            shape, dt = (N1, S1, n // (2 * N1 * S1)), np.complex128
        else:
            shape, dt = (m.nlon, m.nlat, n // (m.nlon * m.nlat)), np.float64
        if "tracers" in name:  # [.., nd, nq]
            shape = shape[:2] + (m.nd, self.num_tracers)
        return shape, dt

    def get(self, name):
        n = lib().om_model_field(self._h, name.encode(), None, 0, 0)
        if n < 0:
            raise KeyError(name)
        shape, dt = self._shape(name, n)
        out = np.zeros(shape, dtype=dt, order="F")
        lib().om_model_field(self._h, name.encode(), _ptr(out), n, 0)
        return out

    def set(self, name, arr):
        n = lib().om_model_field(self._h, name.encode(), None, 0, 0)
        if n < 0:
            raise KeyError(name)
        shape, dt = self._shape(name, n)
        a = np.asfortranarray(np.asarray(arr, dtype=dt).reshape(shape, order="F"))
        lib().om_model_field(self._h, name.encode(), _ptr(a), n, 1)

    @property
    def init_step(self):
        return bool(lib().om_model_init_step(self._h))

    def step(self, nsteps=1):
        lib().om_model_step(self._h, int(nsteps))

    def fixer_scalars(self):
        """The last Held-Suarez step's mean_ps_p, mean_energy_p, mean_ps_n, factor, mean_energy_n and
        temperature correction (Compute_Corrections!)."""
        out = np.zeros(6)
        lib().om_model_fixer_scalars(self._h, _ptr(out))
        return out

    def update_init_step(self):
        assert lib().om_model_update_init_step(self._h) == 0, "Update_Init_Step!: not in the init step"

    def spectral_initialize_fields(self, grid_t_pert=None, vorticity_seed=True):
        if grid_t_pert is not None:
            g = np.asfortranarray(grid_t_pert, dtype=np.float64)
            lib().om_spectral_initialize_fields(self._h, _ptr(g), int(vorticity_seed))
        else:
            lib().om_spectral_initialize_fields(self._h, None, int(vorticity_seed))

    def semi_implicit(self, name):
        n = lib().om_model_semi_implicit(self._h, name.encode(), None, 0)
        out = np.zeros(n)
        lib().om_model_semi_implicit(self._h, name.encode(), _ptr(out), n)
        nd = self.mesh.nd
        if name == "div_mat":
            return out.reshape((nd, nd), order="F")
        if name == "wave_matrix":
            return out.reshape((nd, nd, -1), order="F")
        return out


def HS_Forcing(model, dt, grid_u, grid_v, grid_p_half, grid_p_full, grid_t, grid_du, grid_dv, grid_t_eq, grid_dt):
    """HS_Forcing! (HS_Forcing.jl:1-130); the physics parameters come from the model."""
    ins = [np.asfortranarray(a, dtype=np.float64) for a in (grid_u, grid_v, grid_p_half, grid_p_full, grid_t)]
    for a in (grid_du, grid_dv, grid_t_eq, grid_dt):
        _ptr(a)
    lib().om_hs_forcing(model._h, int(dt), *[_ptr(a) for a in ins], _ptr(grid_du), _ptr(grid_dv), _ptr(grid_t_eq),
                        _ptr(grid_dt))


def Trans_Spherical_To_Grid_Adjoint(mesh, grid_bar, spec_bar):
    """Adjoint of Trans_Spherical_To_Grid!: spec_bar = S2G^T grid_bar."""
    nlev = _nlev_grid(mesh, grid_bar)
    lib().om_trans_spherical_to_grid_adjoint(mesh._h, _ptr(np.asfortranarray(grid_bar)), nlev, _ptr(spec_bar))


def Trans_Grid_To_Spherical_Adjoint(mesh, spec_bar, grid_bar):
    """Adjoint of Trans_Grid_To_Spherical!: grid_bar = G2S^T spec_bar."""
    nlev = _nlev_spec(mesh, spec_bar)
    lib().om_trans_grid_to_spherical_adjoint(mesh._h, _ptr(np.asfortranarray(spec_bar)), nlev, _ptr(grid_bar))


SI_IN = ("dvor", "ddiv", "dt", "dlnps", "vor_p", "vor_c", "div_p", "div_c", "t_p", "t_c", "lnps_p", "lnps_c")
SI_OUT = ("vor_n", "vor_c", "div_n", "div_c", "t_n", "t_c", "lnps_n", "lnps_c")


def Semi_Implicit_Step(model, inputs):
    """One semi-implicit step (implicit correction + damping + filtered leapfrog): dict of the 12
    SI_IN spectral arrays -> dict of the 8 SI_OUT arrays."""
    ins = [np.asfortranarray(inputs[k], dtype=np.complex128) for k in SI_IN]
    nd = model.mesh.nd
    outs = [model.mesh.spectral(1 if k.startswith("lnps") else nd) for k in SI_OUT]
    pin = (C.c_void_p * 12)(*[a.ctypes.data for a in ins])
    pout = (C.c_void_p * 8)(*[a.ctypes.data for a in outs])
    lib().om_semi_implicit_step(model._h, pin, pout)
    return dict(zip(SI_OUT, outs))


# ---- reverse mode of the Held-Suarez step (the reference has none) --------------------------------
STATE_FIELDS = ("spe_vor_c", "spe_vor_p", "spe_div_c", "spe_div_p", "spe_lnps_c", "spe_lnps_p", "spe_t_c",
                "spe_t_p", "grid_u_c", "grid_u_p", "grid_v_c", "grid_v_p", "grid_ps_c", "grid_ps_p", "grid_t_c",
                "grid_t_p", "grid_vor", "grid_div")
HS_PARAMS = ("k_f", "k_a", "k_s", "dT_y", "dtheta_z")


def get_state(model):
    """The 18 fields one Held-Suarez step reads and writes, with the init-step flag."""
    return {k: model.get(k) for k in STATE_FIELDS}, model.init_step


def set_state(model, state):
    fields, init = state
    for k in STATE_FIELDS:
        model.set(k, fields[k])
    lib().om_model_sync_pressure(model._h)
    if model.init_step != init:
        lib().om_model_set_init_step(model._h, int(init))


def set_init_step(model, flag):
    lib().om_model_set_init_step(model._h, int(flag))


def HS_Step_Adjoint(model, xbar, pbar=None):
    """Cotangents of X_{s+1} (dict over STATE_FIELDS) -> cotangents of X_s (the model's state) and
    of the HS parameters (array over HS_PARAMS, accumulated into `pbar`)."""
    arrs = [np.array(xbar[k], dtype=model.get(k).dtype, order="F", copy=True) for k in STATE_FIELDS]
    pb = np.zeros(5) if pbar is None else pbar
    ptrs = (C.c_void_p * 18)(*[a.ctypes.data for a in arrs])
    assert lib().om_hs_step_adjoint(model._h, ptrs, _ptr(pb)) == 0
    return dict(zip(STATE_FIELDS, arrs)), pb


def Vor_Div_From_Grid_UV_Adjoint(mesh, vor_bar, div_bar, u_bar, v_bar):
    n = _nlev_spec(mesh, vor_bar)
    lib().om_vor_div_from_grid_uv_adjoint(mesh._h, _ptr(np.asfortranarray(vor_bar)), _ptr(np.asfortranarray(div_bar)),
                                          n, _ptr(u_bar), _ptr(v_bar))


def UV_Grid_From_Vor_Div_Adjoint(mesh, u_bar, v_bar, vor_bar, div_bar):
    n = _nlev_grid(mesh, u_bar)
    lib().om_uv_grid_from_vor_div_adjoint(mesh._h, _ptr(np.asfortranarray(u_bar)), _ptr(np.asfortranarray(v_bar)),
                                          n, _ptr(vor_bar), _ptr(div_bar))


def Compute_Gradients_Adjoint(mesh, dlam_bar, dth_bar, hs_bar):
    n = _nlev_grid(mesh, dlam_bar)
    lib().om_compute_gradients_adjoint(mesh._h, _ptr(np.asfortranarray(dlam_bar)), _ptr(np.asfortranarray(dth_bar)),
                                       n, _ptr(hs_bar))


def hs_loss(mesh, grid_t, t_target):
    """sum_{i,j,k} w_j (T - T_target)^2 / (2 nlon nd): the area-weighted mean squared difference
    (sum_j w_j = 2), and its gradient with respect to grid T."""
    w = mesh.wts[None, :, None]
    d = grid_t - t_target
    norm = 2.0 * mesh.nlon * grid_t.shape[2]
    return float(np.sum(w * d * d) / norm), np.asfortranarray(2.0 * w * d / norm)


def HS_Gradient(model, nsteps, t_target):
    """Loss of the grid temperature after `nsteps` Held-Suarez steps from the model's state, and its
    gradient with respect to the initial spectral temperature T0 (the state's spe_t_c = spe_t_p = T0,
    grid_t_c = grid_t_p = S2G(T0), as Spectral_Initialize_Fields! leaves them, row N+1 = 0) and the five HS
    parameters, by the step adjoint over all steps (every state kept: the CPU check needs no
    checkpointing).  The model is left at the final state."""
    states = []
    for _ in range(nsteps):
        states.append(get_state(model))
        model.step(1)
    loss, tbar = hs_loss(model.mesh, model.get("grid_t_c"), t_target)
    final = get_state(model)
    xbar = {k: np.zeros_like(v) for k, v in final[0].items()}
    xbar["grid_t_c"] = tbar
    pbar = np.zeros(5)
    for st in reversed(states):
        set_state(model, st)
        xbar, pbar = HS_Step_Adjoint(model, xbar, pbar)
    set_state(model, final)
    m = model.mesh
    g = np.asfortranarray(xbar["grid_t_c"] + xbar["grid_t_p"])
    s = m.spectral(m.nd)
    Trans_Spherical_To_Grid_Adjoint(m, g, s)
    g = np.asfortranarray(xbar["spe_t_c"] + xbar["spe_t_p"] + s)
    g[:, -1, :] = 0  # T0 has row N+1 = 0 (an analysis output); that row is not part of the control
    return loss, g, pbar
