"""jgcm -- Python host interface of libjgcm, the GB300-native JGCM spectral dynamical core.

Mirrors the reference's ``Atmos_Spectral`` call surface (CliMA/IdealizedSpectralGCM.jl,
module JGCM) through the C ABI declared in ``include/jgcm.h``:

* ``Spectral_Spherical_Mesh(num_fourier, num_spherical, nθ, nλ, nd, radius)``
  (Spectral_Spherical_Mesh.jl:69-139) plus a ``precision`` keyword;
* ``Trans_Spherical_To_Grid``, ``Trans_Grid_To_Spherical``, ``Trans_Grid_To_Fourier``,
  ``Vor_Div_From_Grid_UV``, ``UV_Grid_From_Vor_Div``, ``Compute_Gradients``,
  ``Add_Horizontal_Advection``, ``Apply_Laplacian``, ``Area_Weighted_Global_Mean`` -- the
  reference methods without the ``!``, mutating their output arguments as the reference does;
* ``Model`` -- Dyn_Data + Filtered_Leapfrog (+ Semi_Implicit_Solver) resident on the GPU,
  stepping Barotropic_Dynamics!, Shallow_Water_Dynamics! or Atmosphere_Update!.

Arrays follow the reference's Julia layout: numpy Fortran order, grid ``float64[nλ, nθ, nlev]``,
spectral ``complex128[N+1, N+2, nlev]``.  Shape errors raise ``AssertionError`` like the
reference's ``@assert``; library failures raise ``JGCMError`` with the library's message.
There is no CPU fallback: importing this package without a built ``libjgcm.so`` or calling
it without a CUDA device raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

__all__ = [
    "FP64", "FP32", "TF32X3", "BF16X3", "JGCMError", "Spectral_Spherical_Mesh", "Trans_Spherical_To_Grid",
    "Trans_Grid_To_Spherical", "Trans_Grid_To_Fourier", "Vor_Div_From_Grid_UV", "UV_Grid_From_Vor_Div",
    "Compute_Gradients", "Add_Horizontal_Advection", "Apply_Laplacian", "Area_Weighted_Global_Mean", "Model",
    "Compute_Vert_Coord", "lib", "lib_path",
]

FP64, FP32, TF32X3, BF16X3 = 0, 1, 2, 3
PRECISIONS = {"fp64": FP64, "fp32": FP32, "tf32x3": TF32X3, "bf16x3": BF16X3}

_HERE = os.path.dirname(os.path.abspath(__file__))


def lib_path() -> str:
    return os.path.join(_HERE, "libjgcm.so")


class JGCMError(RuntimeError):
    pass


_lib = None


def lib():
    """Load libjgcm.so (built by ``build_lib.py``); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not os.path.exists(path):
        raise JGCMError(f"libjgcm.so not built ({path}); run __graft_entry__.build()")
    L = C.CDLL(path)
    P, I, D, Lg = C.c_void_p, C.c_int, C.c_double, C.c_long
    PP = C.POINTER(C.c_void_p)
    sig = {
        "jgcm_last_error": (C.c_char_p, []),
        "jgcm_version": (I, []),
        "jgcm_device_info": (I, [C.POINTER(I), C.POINTER(I), C.POINTER(I)]),
        "jgcm_mesh_create": (I, [I, I, I, I, I, D, I, PP]),
        "jgcm_mesh_destroy": (I, [P]),
        "jgcm_mesh_precision": (I, [P]),
        "jgcm_mesh_table": (I, [P, C.c_char_p, P, Lg, C.POINTER(Lg)]),
        "jgcm_mesh_synchronize": (I, [P]),
        "jgcm_trans_spherical_to_grid": (I, [P, P, I, P]),
        "jgcm_trans_grid_to_spherical": (I, [P, P, I, P]),
        "jgcm_trans_grid_to_fourier": (I, [P, P, I, P]),
        "jgcm_trans_spherical_to_grid_adjoint": (I, [P, P, I, P]),
        "jgcm_trans_grid_to_spherical_adjoint": (I, [P, P, I, P]),
        "jgcm_vor_div_from_grid_uv": (I, [P, P, P, I, P, P]),
        "jgcm_uv_grid_from_vor_div": (I, [P, P, P, I, P, P]),
        "jgcm_compute_gradients": (I, [P, P, I, P, P]),
        "jgcm_add_horizontal_advection": (I, [P, P, P, P, I, P]),
        "jgcm_apply_laplacian": (I, [P, P, I]),
        "jgcm_area_weighted_global_mean": (I, [P, P, C.POINTER(D)]),
        "jgcm_model_create": (I, [P, P, PP]),
        "jgcm_model_create_members": (I, [P, P, I, PP]),
        "jgcm_vert_coord": (I, [I, C.c_char_p, D, D, D, P, P]),
        "jgcm_model_create_vert": (I, [P, P, I, P, P, PP]),
        "jgcm_model_members": (I, [P, C.POINTER(I)]),
        "jgcm_model_copy_member": (I, [P, I, P, I]),
        "jgcm_model_semi_implicit_step": (I, [P, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
        "jgcm_model_semi_implicit_step_adjoint": (I, [P, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
        "jgcm_model_state_size": (I, [P, C.POINTER(Lg)]),
        "jgcm_model_set_state": (I, [P, P]),
        "jgcm_model_get_state": (I, [P, P]),
        "jgcm_model_step_adjoint": (I, [P, C.POINTER(C.c_void_p), P]),
        "jgcm_model_hs_gradient": (I, [P, I, I, P, P, P, P]),
        "jgcm_model_diagnostics": (I, [P, I]),
        "jgcm_model_read_diagnostics": (I, [P, C.c_char_p, P, Lg, C.POINTER(Lg), C.POINTER(Lg)]),
        "jgcm_model_get_tuning": (I, [P, C.POINTER(I), I]),
        "jgcm_model_add_tracers": (I, [P, I]),
        "jgcm_model_num_tracers": (I, [P, C.POINTER(I)]),
        "jgcm_model_set_tuning": (I, [P, C.POINTER(I), I]),
        "jgcm_model_autotune": (I, [P, I, C.POINTER(I), I, C.POINTER(C.c_float)]),
        "jgcm_ensemble_create": (I, [C.POINTER(P), I, I, PP]),
        "jgcm_ensemble_step": (I, [P, I]),
        "jgcm_ensemble_time": (I, [P, I, C.POINTER(C.c_float)]),
        "jgcm_ensemble_destroy": (I, [P]),
        "jgcm_model_destroy": (I, [P]),
        "jgcm_model_get_field": (I, [P, C.c_char_p, P, Lg, C.POINTER(Lg)]),
        "jgcm_model_set_field": (I, [P, C.c_char_p, P, Lg]),
        "jgcm_model_step": (I, [P, I]),
        "jgcm_model_init_step": (I, [P, C.POINTER(I)]),
        "jgcm_model_update_init_step": (I, [P]),
        "jgcm_model_set_init_step": (I, [P, I]),
        "jgcm_spectral_initialize_fields": (I, [P, P, I]),
        "jgcm_model_semi_implicit": (I, [P, C.c_char_p, P, Lg, C.POINTER(Lg)]),
        "jgcm_hs_forcing": (I, [P, I, P, P, P, P, P, P, P, P, P]),
        "jgcm_model_time_steps": (I, [P, I, C.POINTER(C.c_float)]),
        "jgcm_model_launches_per_step": (I, [P, C.POINTER(I)]),
        "jgcm_model_kernel_times": (I, [P, I, C.POINTER(C.c_float), I, C.POINTER(I)]),
        "jgcm_model_kernel_name": (I, [P, I, C.c_char_p, I]),
        "jgcm_set_device": (I, [I]),
        "jgcm_selftest_bounded_wait": (I, [P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(status: int) -> None:
    if status != 0:
        msg = lib().jgcm_last_error().decode(errors="replace")
        if status == -1:
            raise AssertionError(msg)
        raise JGCMError(f"libjgcm status {status}: {msg}")


def _ptr(a: np.ndarray):
    assert a.flags.f_contiguous, "arrays must be Fortran-ordered (Julia layout)"
    return a.ctypes.data_as(C.c_void_p)


def device_info():
    sm, ma, mi = C.c_int(), C.c_int(), C.c_int()
    _check(lib().jgcm_device_info(C.byref(sm), C.byref(ma), C.byref(mi)))
    return {"sm_count": sm.value, "cc": (ma.value, mi.value)}


class Spectral_Spherical_Mesh:
    """Spectral_Spherical_Mesh.jl:69-139, device-resident; tables generated on the GPU in FP64."""

    _TABLES3 = ("qnm", "dqnm", "qwg", "coef_alp_a", "coef_alp_b")
    _TABLES2 = ("epsilon", "coef_uvm", "coef_uvc", "coef_uvp", "coef_dlam", "coef_dthm", "coef_dthp",
                "laplacian_eig")

    def __init__(self, num_fourier, num_spherical, nlat, nlon, nd, radius, precision="fp64"):
        if isinstance(precision, str):
            precision = PRECISIONS[precision]
        self.num_fourier, self.num_spherical = int(num_fourier), int(num_spherical)
        self.nlat, self.nlon, self.nd, self.radius = int(nlat), int(nlon), int(nd), float(radius)
        self.precision = int(precision)
        h = C.c_void_p()
        _check(lib().jgcm_mesh_create(self.num_fourier, self.num_spherical, self.nlat, self.nlon, self.nd,
                                      self.radius, self.precision, C.byref(h)))
        self._h = h
        self._cache = {}

    def __getattr__(self, name):
        if name.startswith("_"):
            raise AttributeError(name)
        if name in ("sinth", "costh", "wts", "lonc", "latc") + self._TABLES3 + self._TABLES2:
            if name not in self._cache:
                self._cache[name] = self._table(name)
            return self._cache[name]
        raise AttributeError(name)

    def _table(self, name):
        n = C.c_long()
        _check(lib().jgcm_mesh_table(self._h, name.encode(), None, 0, C.byref(n)))
        out = np.zeros(n.value)
        _check(lib().jgcm_mesh_table(self._h, name.encode(), _ptr(out), n.value, C.byref(n)))
        N1, S1 = self.num_fourier + 1, self.num_spherical + 1
        if name in self._TABLES3:
            return out.reshape((N1, S1, self.nlat), order="F")
        if name in self._TABLES2:
            return out.reshape((N1, S1), order="F")
        return out

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().jgcm_mesh_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def spectral(self, nlev):
        return np.zeros((self.num_fourier + 1, self.num_spherical + 1, nlev), dtype=np.complex128, order="F")

    def grid(self, nlev):
        return np.zeros((self.nlon, self.nlat, nlev), order="F")


def _nlev_spec(mesh, a):
    assert isinstance(a, np.ndarray) and a.dtype == np.complex128
    assert a.ndim == 3 and a.shape[:2] == (mesh.num_fourier + 1, mesh.num_spherical + 1)
    assert a.shape[2] in (mesh.nd, 1)
    return a.shape[2]


def _nlev_grid(mesh, a):
    assert isinstance(a, np.ndarray) and a.dtype == np.float64
    assert a.ndim == 3 and a.shape[:2] == (mesh.nlon, mesh.nlat)
    assert a.shape[2] in (mesh.nd, 1)
    return a.shape[2]


def Trans_Spherical_To_Grid(mesh, snm, pfield):
    """Spectral_Spherical_Mesh.jl:143-217 (sums total wavenumbers m..N+1)."""
    n = _nlev_spec(mesh, snm)
    assert _nlev_grid(mesh, pfield) == n
    _check(lib().jgcm_trans_spherical_to_grid(mesh._h, _ptr(snm), n, _ptr(pfield)))


def Trans_Grid_To_Spherical(mesh, pfield, snm):
    """Spectral_Spherical_Mesh.jl:221-293 (row N+1 set to zero)."""
    n = _nlev_grid(mesh, pfield)
    assert _nlev_spec(mesh, snm) == n
    _check(lib().jgcm_trans_grid_to_spherical(mesh._h, _ptr(pfield), n, _ptr(snm)))


def Trans_Spherical_To_Grid_Adjoint(mesh, grid_bar, spec_bar):
    """Adjoint of Trans_Spherical_To_Grid!: spec_bar = S2G^T grid_bar (row N+1 included)."""
    nlev = _nlev_grid(mesh, grid_bar)
    assert _nlev_spec(mesh, spec_bar) == nlev
    _check(lib().jgcm_trans_spherical_to_grid_adjoint(mesh._h, _ptr(np.asfortranarray(grid_bar)), nlev,
                                                      _ptr(spec_bar)))


def Trans_Grid_To_Spherical_Adjoint(mesh, spec_bar, grid_bar):
    """Adjoint of Trans_Grid_To_Spherical!: grid_bar = G2S^T spec_bar (row N+1 ignored)."""
    nlev = _nlev_spec(mesh, spec_bar)
    assert _nlev_grid(mesh, grid_bar) == nlev
    _check(lib().jgcm_trans_grid_to_spherical_adjoint(mesh._h, _ptr(np.asfortranarray(spec_bar)), nlev,
                                                      _ptr(grid_bar)))


def Trans_Grid_To_Fourier(mesh, pfield, fourier):
    """Spectral_Spherical_Mesh.jl:295-330: ``fourier`` (complex128[nλ, nθ, nlev], the reference's
    ``fourier_g``) receives fft(pfield, 1) / nλ, every mode."""
    n = _nlev_grid(mesh, pfield)
    assert fourier.dtype == np.complex128 and fourier.shape == (mesh.nlon, mesh.nlat, n)
    assert fourier.flags.f_contiguous
    _check(lib().jgcm_trans_grid_to_fourier(mesh._h, _ptr(pfield), n, _ptr(fourier)))


def Vor_Div_From_Grid_UV(mesh, grid_u, grid_v, vor, div):
    """Spectral_Spherical_Mesh.jl:349-393."""
    n = _nlev_grid(mesh, grid_u)
    assert _nlev_grid(mesh, grid_v) == n and _nlev_spec(mesh, vor) == n and _nlev_spec(mesh, div) == n
    _check(lib().jgcm_vor_div_from_grid_uv(mesh._h, _ptr(grid_u), _ptr(grid_v), n, _ptr(vor), _ptr(div)))


def UV_Grid_From_Vor_Div(mesh, vor, div, grid_u, grid_v):
    """Spectral_Spherical_Mesh.jl:462-482."""
    n = _nlev_spec(mesh, vor)
    assert _nlev_spec(mesh, div) == n and _nlev_grid(mesh, grid_u) == n and _nlev_grid(mesh, grid_v) == n
    _check(lib().jgcm_uv_grid_from_vor_div(mesh._h, _ptr(vor), _ptr(div), n, _ptr(grid_u), _ptr(grid_v)))


def Compute_Gradients(mesh, spe_hs, grid_dlam_hs, grid_dth_hs):
    """Spectral_Spherical_Mesh.jl:721-741."""
    n = _nlev_spec(mesh, spe_hs)
    assert _nlev_grid(mesh, grid_dlam_hs) == n and _nlev_grid(mesh, grid_dth_hs) == n
    _check(lib().jgcm_compute_gradients(mesh._h, _ptr(spe_hs), n, _ptr(grid_dlam_hs), _ptr(grid_dth_hs)))


def Add_Horizontal_Advection(mesh, spe_hs, grid_u, grid_v, grid_dhs):
    """Spectral_Spherical_Mesh.jl:694-718 (grid_dhs -= u ∂λhs + v ∂θhs)."""
    n = _nlev_spec(mesh, spe_hs)
    assert _nlev_grid(mesh, grid_u) == n and _nlev_grid(mesh, grid_v) == n and _nlev_grid(mesh, grid_dhs) == n
    _check(lib().jgcm_add_horizontal_advection(mesh._h, _ptr(spe_hs), _ptr(grid_u), _ptr(grid_v), n,
                                               _ptr(grid_dhs)))


def Apply_Laplacian(mesh, spe):
    """Spectral_Spherical_Mesh.jl:614-621."""
    _check(lib().jgcm_apply_laplacian(mesh._h, _ptr(spe), _nlev_spec(mesh, spe)))


def Area_Weighted_Global_Mean(mesh, grid):
    """Spectral_Spherical_Mesh.jl:746-760 (level 1)."""
    _nlev_grid(mesh, grid)
    out = C.c_double()
    _check(lib().jgcm_area_weighted_global_mean(mesh._h, _ptr(grid), C.byref(out)))
    return out.value


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
    """Vert_Coordinate.jl:61-87: the half-level coefficients (ak, bk), nd+1 each, top first, zero top.

    Options: "even_sigma", "uneven_sigma" (built as Compute_Uneven_Sigma's docstring states; the
    reference's own branch does not run), "mcm" (nd 14), "v197" (nd 18), "hybrid" (pressure levels
    above sigma 0.1, sigma levels below 0.3, Transition's sin^2 blend between; built as the reference's
    code means it, its branch does not run).  Hybrid models step forward; their step adjoint is refused."""
    ak, bk = np.zeros(nd + 1), np.zeros(nd + 1)
    _check(lib().jgcm_vert_coord(int(nd), vert_coord_option.encode(), float(scale_heights), float(surf_res),
                                 float(exponent), _ptr(ak), _ptr(bk)))
    return ak, bk


class Model:
    """Dyn_Data + Filtered_Leapfrog (+ Semi_Implicit_Solver) on the GPU.

    ``params`` is a dict with the fields of ``jgcm_params`` (see jgcm.configs).  Fields are
    read and written by their Dyn_Data names with δ spelled ``d`` (``spe_vor_c``,
    ``grid_u_p``, ``grid_t_eq``, ...).  ``step(n)`` runs n Barotropic_Dynamics! /
    Shallow_Water_Physics!+Shallow_Water_Dynamics! / Atmosphere_Update! steps, the first one
    being the reference drivers' init step followed by Update_Init_Step!.

    ``members`` > 1 makes an ensemble: that many independent members advanced together by the
    same kernels.  Members are loaded and read with ``copy_member`` through one-member models.

    ``vert_coord`` is Vert_Coordinate's option (``"even_sigma"``, the reference drivers' choice,
    ``"uneven_sigma"``, ``"mcm"``, ``"v197"``; see ``Compute_Vert_Coord``) or a pair (ak, bk) of
    sigma half-level coefficients.
    """

    def __init__(self, mesh: Spectral_Spherical_Mesh, params: dict, members: int = 1,
                 vert_coord="even_sigma", num_tracers: int = 0, **vert_options):
        self.mesh = mesh
        self.params = dict(params)
        self.members = int(members)
        if isinstance(vert_coord, str):
            ak, bk = Compute_Vert_Coord(mesh.nd, vert_coord, **vert_options)
        else:
            ak, bk = (np.ascontiguousarray(x, dtype=np.float64) for x in vert_coord)
            if ak.shape != (mesh.nd + 1,) or bk.shape != (mesh.nd + 1,):
                raise ValueError("ak and bk need nd + 1 values each")
        self.ak, self.bk = ak, bk
        p = _Params()
        for name, _ in _Params._fields_:
            if name == "kind":
                p.kind = KINDS[params["kind"]]
            elif name in params:
                setattr(p, name, params[name])
        self._p = p
        h = C.c_void_p()
        _check(lib().jgcm_model_create_vert(mesh._h, C.byref(p), self.members, _ptr(ak), _ptr(bk), C.byref(h)))
        self._h = h
        self.num_tracers = int(num_tracers)
        if self.num_tracers:
            _check(lib().jgcm_model_add_tracers(self._h, self.num_tracers))

    def diagnostics(self, on=True):
        """Start (zeroing the sums) or stop the on-device diagnostics (Held-Suarez): after every step
        the zonal means of T, T_eq, u, v and the ps field are added to FP64 sums."""
        _check(lib().jgcm_model_diagnostics(self._h, int(bool(on))))

    def read_diagnostics(self, name):
        """Mean over the summed steps of 't_zonal_mean', 't_eq_zonal_mean', 'u_zonal_mean',
        'v_zonal_mean' ([nθ, nd] per member) or 'ps_mean' ([nλ, nθ] per member), and the step count."""
        n, steps = C.c_long(), C.c_long()
        _check(lib().jgcm_model_read_diagnostics(self._h, name.encode(), None, 0, C.byref(n), C.byref(steps)))
        out = np.zeros(n.value)
        _check(lib().jgcm_model_read_diagnostics(self._h, name.encode(), _ptr(out), n.value, C.byref(n),
                                                 C.byref(steps)))
        m = self.mesh
        shape = (m.nlon, m.nlat, self.members) if name == "ps_mean" else (m.nlat, m.nd, self.members)
        out = out.reshape(shape, order="F")
        return (out[..., 0] if self.members == 1 else out), int(steps.value)

    DIAGNOSTICS = ("t_zonal_mean", "t_eq_zonal_mean", "u_zonal_mean", "v_zonal_mean", "ps_mean")

    def write_diagnostics(self, path):
        """Write the current diagnostic means to ``path`` (raw little-endian FP64, the arrays back to
        back in Julia column-major order: read in Julia with ``read!(io, Array{Float64}(undef,
        shape...))``) and ``path + ".json"`` (names, shapes, byte offsets, steps summed, mesh), the
        output of Output_Manager.jl:81-145 without its plots."""
        return write_arrays(path, {k: self.read_diagnostics(k)[0] for k in self.DIAGNOSTICS},
                            {"steps": self.read_diagnostics("ps_mean")[1], "members": self.members,
                             "mesh": {"num_fourier": self.mesh.num_fourier, "nlat": self.mesh.nlat,
                                      "nlon": self.mesh.nlon, "nd": self.mesh.nd},
                             "latitudes_deg": [float(x) for x in np.degrees(np.arcsin(self.mesh.sinth))]})

    def copy_member(self, member: int, src: "Model", src_member: int = 0):
        """Member `member` of this model <- member `src_member` of `src` (same mesh and kind)."""
        _check(lib().jgcm_model_copy_member(self._h, int(member), src._h, int(src_member)))

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().jgcm_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _shape(self, name, n):
        m = self.mesh
        N1, S1 = m.num_fourier + 1, m.num_spherical + 1
        if name.startswith("spe_"):
            shape, dt = (N1, S1, n // (2 * N1 * S1)), np.complex128
        else:
            shape, dt = (m.nlon, m.nlat, n // (m.nlon * m.nlat)), np.float64
        if "tracers" in name:  # Dyn_Data's [.., nd, num_tracers]
            shape = shape[:2] + (m.nd, self.num_tracers)
        return shape, dt

    def get(self, name):
        n = C.c_long()
        _check(lib().jgcm_model_get_field(self._h, name.encode(), None, 0, C.byref(n)))
        shape, dt = self._shape(name, n.value)
        out = np.zeros(shape, dtype=dt, order="F")
        _check(lib().jgcm_model_get_field(self._h, name.encode(), _ptr(out), n.value, C.byref(n)))
        return out

    def set(self, name, arr):
        n = C.c_long()
        _check(lib().jgcm_model_get_field(self._h, name.encode(), None, 0, C.byref(n)))
        shape, dt = self._shape(name, n.value)
        a = np.asfortranarray(np.asarray(arr, dtype=dt).reshape(shape, order="F"))
        _check(lib().jgcm_model_set_field(self._h, name.encode(), _ptr(a), n.value))

    @property
    def init_step(self):
        v = C.c_int()
        _check(lib().jgcm_model_init_step(self._h, C.byref(v)))
        return bool(v.value)

    def step(self, nsteps=1):
        _check(lib().jgcm_model_step(self._h, int(nsteps)))

    # ---- the whole state of a Held-Suarez step in one transfer (STATE_FIELDS, packed) ----
    def state_size(self):
        n = C.c_long()
        _check(lib().jgcm_model_state_size(self._h, C.byref(n)))
        return int(n.value)

    def set_state(self, packed):
        """Load the 18 STATE_FIELDS from one FP64 buffer (``pack_state``); pinned memory makes the
        host-to-device copy fastest."""
        a = np.asarray(packed)
        assert a.dtype == np.float64 and a.size == self.state_size() and a.flags.c_contiguous
        _check(lib().jgcm_model_set_state(self._h, a.ctypes.data_as(C.c_void_p)))

    def get_state(self, out=None):
        """The 18 STATE_FIELDS in one FP64 buffer (``unpack_state`` splits it)."""
        n = self.state_size()
        a = np.empty(n) if out is None else out
        assert a.dtype == np.float64 and a.size == n and a.flags.c_contiguous
        _check(lib().jgcm_model_get_state(self._h, a.ctypes.data_as(C.c_void_p)))
        return a

    def set_init_step(self, flag=True):
        """Make the next step a first step (Δt) or a leapfrog step (2Δt)."""
        _check(lib().jgcm_model_set_init_step(self._h, int(bool(flag))))

    def update_init_step(self):
        """Update_Init_Step! (Time_Integrator.jl:40-43): leave the forward init-step mode."""
        _check(lib().jgcm_model_update_init_step(self._h))

    def spectral_initialize_fields(self, grid_t_pert=None, vorticity_seed=True):
        """Spectral_Dynamics.jl:372-449 on the device."""
        if grid_t_pert is not None:
            g = np.asfortranarray(grid_t_pert, dtype=np.float64)
            _check(lib().jgcm_spectral_initialize_fields(self._h, _ptr(g), int(vorticity_seed)))
        else:
            _check(lib().jgcm_spectral_initialize_fields(self._h, None, int(vorticity_seed)))

    def semi_implicit(self, name):
        n = C.c_long()
        _check(lib().jgcm_model_semi_implicit(self._h, name.encode(), None, 0, C.byref(n)))
        out = np.zeros(n.value)
        _check(lib().jgcm_model_semi_implicit(self._h, name.encode(), _ptr(out), n.value, C.byref(n)))
        nd = self.mesh.nd
        if name == "div_mat":
            return out.reshape((nd, nd), order="F")
        if name == "wave_matrix":
            return out.reshape((nd, nd, -1), order="F")
        return out

    def time_steps(self, nsteps):
        """Advance nsteps steady steps (CUDA graphs) and return the CUDA-event time in ms."""
        ms = C.c_float()
        _check(lib().jgcm_model_time_steps(self._h, int(nsteps), C.byref(ms)))
        return float(ms.value)

    def launches_per_step(self):
        v = C.c_int()
        _check(lib().jgcm_model_launches_per_step(self._h, C.byref(v)))
        return v.value

    def kernel_times(self, nsteps):
        """{launch slot name: mean CUDA-event ms} over nsteps eager steady steps (advances the model)."""
        L = self.launches_per_step()
        arr = (C.c_float * L)()
        cnt = C.c_int()
        _check(lib().jgcm_model_kernel_times(self._h, int(nsteps), arr, L, C.byref(cnt)))
        out = {}
        buf = C.create_string_buffer(128)
        for s in range(cnt.value):
            _check(lib().jgcm_model_kernel_name(self._h, s, buf, 128))
            out[buf.value.decode()] = float(arr[s])
        return out


def set_device(device: int) -> None:
    _check(lib().jgcm_set_device(int(device)))


def HS_Forcing(model, dt, grid_u, grid_v, grid_p_half, grid_p_full, grid_t, grid_du, grid_dv, grid_t_eq, grid_dt):
    """HS_Forcing! (HS_Forcing.jl:1-130) on host arrays; the physics parameters (the reference's
    physics Dict) and c_p (Atmo_Data) come from the model.  Outputs are written in place."""
    ins = [np.asfortranarray(a, dtype=np.float64) for a in (grid_u, grid_v, grid_p_half, grid_p_full, grid_t)]
    assert ins[0].shape == ins[1].shape == ins[3].shape == ins[4].shape, "u, v, p_full, t shapes differ"
    assert ins[2].shape == ins[0].shape[:2] + (ins[0].shape[2] + 1,), "p_half must have nd+1 levels"
    for a in (grid_du, grid_dv, grid_t_eq, grid_dt):
        assert a.shape == ins[0].shape and a.dtype == np.float64, "output shape/dtype"
    _check(lib().jgcm_hs_forcing(model._h, int(dt), *[_ptr(a) for a in ins], _ptr(grid_du), _ptr(grid_dv),
                                 _ptr(grid_t_eq), _ptr(grid_dt)))


class Ensemble:
    """Models of uneven truncations / kinds advanced together: each window of `window_seconds` is
    one CUDA-graph launch whose branches step every model concurrently (window_seconds a multiple
    of every model's dt; every model past its first step)."""

    def __init__(self, models, window_seconds):
        self.models = list(models)
        arr = (C.c_void_p * len(self.models))(*[m._h.value for m in self.models])
        h = C.c_void_p()
        _check(lib().jgcm_ensemble_create(arr, len(self.models), int(window_seconds), C.byref(h)))
        self._h = h

    def step(self, nwindows=1):
        _check(lib().jgcm_ensemble_step(self._h, int(nwindows)))

    def time_windows(self, nwindows):
        """Advance nwindows windows and return their CUDA-event time in ms."""
        ms = C.c_float()
        _check(lib().jgcm_ensemble_time(self._h, int(nwindows), C.byref(ms)))
        return float(ms.value)

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().jgcm_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


TUNING_KNOBS = ("lanes_per_column", "s2g_columns", "g2s_columns", "fft_columns", "simt_legendre", "hs_analysis_levels")


def write_arrays(path, arrays, meta=None):
    """Raw FP64 dump: ``path`` holds the arrays back to back (Fortran order, little-endian),
    ``path + ".json"`` their names, shapes and byte offsets plus ``meta``.  Returns the header."""
    import json

    header = {"format": "raw float64 little-endian, column-major arrays back to back", "arrays": []}
    off = 0
    with open(path, "wb") as f:
        for name, a in arrays.items():
            a = np.asarray(a, dtype="<f8")
            f.write(np.asfortranarray(a).tobytes(order="F"))
            header["arrays"].append({"name": name, "shape": list(a.shape), "offset_bytes": off})
            off += a.nbytes
    header.update(meta or {})
    with open(path + ".json", "w") as f:
        json.dump(header, f, indent=1)
    return header


def read_arrays(path):
    """Inverse of write_arrays: dict name -> array, and the header."""
    import json

    with open(path + ".json") as f:
        header = json.load(f)
    raw = np.fromfile(path, dtype="<f8")
    out = {}
    for e in header["arrays"]:
        n = int(np.prod(e["shape"]))
        o = e["offset_bytes"] // 8
        out[e["name"]] = raw[o:o + n].reshape(e["shape"], order="F")
    return out, header


def get_tuning(model):
    k = (C.c_int * 6)()
    _check(lib().jgcm_model_get_tuning(model._h, k, 6))
    return dict(zip(TUNING_KNOBS, list(k)))


def set_tuning(model, tuning):
    k = (C.c_int * 6)(*[int(tuning.get(n, 0)) for n in TUNING_KNOBS])
    _check(lib().jgcm_model_set_tuning(model._h, k, 6))


def autotune(model, nsteps=24, cache=None):
    """Pick the tiles of `model` (and its mesh) by timing candidates on a scratch copy; with a
    `cache` path, results are stored in (and reused from) that JSON file, keyed by the workload
    and the device."""
    import json

    m = model.mesh
    dev = device_info()
    key = (f"{model.params.get('kind')}:N{m.num_fourier}:{m.nlat}x{m.nlon}x{m.nd}:members{model.members}:"
           f"prec{m.precision}:sm{dev['sm_count']}:cc{dev['cc'][0]}{dev['cc'][1]}")
    table = {}
    if cache and os.path.exists(cache):
        with open(cache) as f:
            table = json.load(f)
    if key in table:
        set_tuning(model, table[key]["tuning"])
        return table[key]
    k = (C.c_int * 6)()
    ms = C.c_float()
    _check(lib().jgcm_model_autotune(model._h, int(nsteps), k, 6, C.byref(ms)))
    entry = {"tuning": dict(zip(TUNING_KNOBS, list(k))), "ms_per_step": float(ms.value) / nsteps}
    if cache:
        table[key] = entry
        with open(cache, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
    return entry


SI_IN = ("dvor", "ddiv", "dt", "dlnps", "vor_p", "vor_c", "div_p", "div_c", "t_p", "t_c", "lnps_p", "lnps_c")
SI_OUT = ("vor_n", "vor_c", "div_n", "div_c", "t_n", "t_c", "lnps_n", "lnps_c")


def _si_arrays(model, names, source=None):
    nd = model.mesh.nd
    if source is None:
        return [model.mesh.spectral(1 if k.startswith("lnps") or k == "dlnps" else nd) for k in names]
    return [np.asfortranarray(source[k], dtype=np.complex128) for k in names]


def Semi_Implicit_Step(model, inputs):
    """One semi-implicit step on its own (Implicit_Correction! + Compute_Spectral_Damping! +
    Filtered_Leapfrog! for the model's current step): dict of the SI_IN spectral arrays -> dict of
    the SI_OUT arrays."""
    ins, outs = _si_arrays(model, SI_IN, inputs), _si_arrays(model, SI_OUT)
    pin = (C.c_void_p * 12)(*[a.ctypes.data for a in ins])
    pout = (C.c_void_p * 8)(*[a.ctypes.data for a in outs])
    _check(lib().jgcm_model_semi_implicit_step(model._h, pin, pout))
    return dict(zip(SI_OUT, outs))


def Semi_Implicit_Step_Adjoint(model, out_bar):
    """Adjoint of Semi_Implicit_Step: cotangents of the SI_OUT arrays -> cotangents of SI_IN."""
    obs, ibs = _si_arrays(model, SI_OUT, out_bar), _si_arrays(model, SI_IN)
    pob = (C.c_void_p * 8)(*[a.ctypes.data for a in obs])
    pib = (C.c_void_p * 12)(*[a.ctypes.data for a in ibs])
    _check(lib().jgcm_model_semi_implicit_step_adjoint(model._h, pob, pib))
    return dict(zip(SI_IN, ibs))


# ---- reverse mode of the Held-Suarez step -------------------------------------------------------
STATE_FIELDS = ("spe_vor_c", "spe_vor_p", "spe_div_c", "spe_div_p", "spe_lnps_c", "spe_lnps_p", "spe_t_c",
                "spe_t_p", "grid_u_c", "grid_u_p", "grid_v_c", "grid_v_p", "grid_ps_c", "grid_ps_p", "grid_t_c",
                "grid_t_p", "grid_vor", "grid_div")
HS_PARAMS = ("k_f", "k_a", "k_s", "dT_y", "dtheta_z")


def _state_shapes(mesh):
    N1, S1 = mesh.num_fourier + 1, mesh.num_spherical + 1
    out = []
    for k in STATE_FIELDS:
        nlev = 1 if k in ("spe_lnps_c", "spe_lnps_p", "grid_ps_c", "grid_ps_p") else mesh.nd
        out.append((k, (N1, S1, nlev), np.complex128) if k.startswith("spe_") else
                   (k, (mesh.nlon, mesh.nlat, nlev), np.float64))
    return out


def pack_state(mesh, fields, out=None):
    """dict over STATE_FIELDS (reference layout) -> one FP64 buffer for Model.set_state."""
    parts = [np.asarray(fields[k], dtype=dt).reshape(shp, order="F").ravel(order="F")
             for k, shp, dt in _state_shapes(mesh)]
    flat = [p.view(np.float64) if p.dtype == np.complex128 else p for p in parts]
    if out is None:
        return np.concatenate(flat)
    np.concatenate(flat, out=out)
    return out


def unpack_state(mesh, packed):
    """One FP64 buffer from Model.get_state -> dict over STATE_FIELDS (reference layout)."""
    out, off = {}, 0
    for k, shp, dt in _state_shapes(mesh):
        n = int(np.prod(shp)) * (2 if dt == np.complex128 else 1)
        v = np.asarray(packed[off:off + n])
        out[k] = np.asfortranarray((v.view(np.complex128) if dt == np.complex128 else v).reshape(shp, order="F"))
        off += n
    return out


def HS_Step_Adjoint(model, xbar, pbar=None):
    """Adjoint of one Held-Suarez step from the model's current state X_s: cotangents of X_{s+1}
    (dict over STATE_FIELDS, reference layout) -> cotangents of X_s, and the cotangents of the
    HS parameters (HS_PARAMS order) accumulated into ``pbar``.  The model stays at X_s."""
    m = model.mesh
    arrs = []
    for k in STATE_FIELDS:
        nlev = 1 if k in ("spe_lnps_c", "spe_lnps_p", "grid_ps_c", "grid_ps_p") else m.nd
        if k.startswith("spe_"):
            a = np.array(xbar[k], dtype=np.complex128, order="F", copy=True).reshape(
                (m.num_fourier + 1, m.num_spherical + 1, nlev), order="F")
        else:
            a = np.array(xbar[k], dtype=np.float64, order="F", copy=True).reshape((m.nlon, m.nlat, nlev), order="F")
        arrs.append(np.asfortranarray(a))
    pb = np.zeros(5) if pbar is None else pbar
    ptrs = (C.c_void_p * 18)(*[a.ctypes.data for a in arrs])
    _check(lib().jgcm_model_step_adjoint(model._h, ptrs, _ptr(pb)))
    return dict(zip(STATE_FIELDS, arrs)), pb


def HS_Gradient(model, nsteps, t_target, checkpoint_every=8):
    """Loss sum w_j (T - t_target)^2 / (2 nlon nd) of the grid temperature after ``nsteps`` steps from
    the model's state, with its gradient with respect to the initial spectral temperature (array
    [N+1, N+2, nd]; row N+1, zero in every analysed field, is not part of the control and returns 0)
    and the HS parameters (HS_PARAMS order): the discrete adjoint run backwards
    with a recomputation checkpoint every ``checkpoint_every`` steps.  The model ends at the final
    state."""
    m = model.mesh
    tgt = np.asfortranarray(t_target, dtype=np.float64)
    assert tgt.shape == (m.nlon, m.nlat, m.nd)
    loss = C.c_double()
    g = m.spectral(m.nd)
    gp = np.zeros(5)
    _check(lib().jgcm_model_hs_gradient(model._h, int(nsteps), int(checkpoint_every), _ptr(tgt), C.byref(loss),
                                        _ptr(g), _ptr(gp)))
    return loss.value, g, gp

