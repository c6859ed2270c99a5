"""The C ABI library builds, loads and exports every entry point include/jgcm.h declares (CPU)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "jgcm.h")


def declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(jgcm_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_the_reference_surface():
    names = declared()
    for n in ["jgcm_mesh_create", "jgcm_trans_spherical_to_grid", "jgcm_trans_grid_to_spherical",
              "jgcm_trans_grid_to_fourier", "jgcm_vor_div_from_grid_uv", "jgcm_uv_grid_from_vor_div",
              "jgcm_compute_gradients", "jgcm_add_horizontal_advection", "jgcm_apply_laplacian",
              "jgcm_area_weighted_global_mean", "jgcm_model_step", "jgcm_spectral_initialize_fields",
              "jgcm_model_update_init_step"]:
        assert n in names


def test_library_exports_every_declared_symbol(jg):
    path = jg.lib_path()
    assert os.path.exists(path)
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (jgcm_[a-z0-9_]+)", out))
    missing = [n for n in declared() if n not in exported]
    assert not missing, missing
    lib = ctypes.CDLL(path)
    for n in declared():
        assert hasattr(lib, n)


def _has_gpu(jg):
    try:
        jg.device_info()
        return True
    except Exception:
        return False


def test_fails_loudly_without_a_gpu(jg):
    if _has_gpu(jg):
        pytest.skip("a CUDA device is present")
    with pytest.raises(jg.JGCMError):
        jg.Spectral_Spherical_Mesh(21, 22, 32, 64, 3, 1.0)


def test_argument_errors_are_assertions(jg):
    # argument checks run before any CUDA call, so they hold with or without a device
    with pytest.raises(AssertionError):
        jg.Spectral_Spherical_Mesh(21, 23, 32, 64, 3, 1.0)
    with pytest.raises(AssertionError):
        jg.Spectral_Spherical_Mesh(21, 22, 31, 64, 3, 1.0)
    with pytest.raises(AssertionError):
        jg.Spectral_Spherical_Mesh(21, 22, 32, 40, 3, 1.0)  # nlon not a power of two


def test_vert_coord_tables_match_the_oracle(jg, orc):
    """jgcm_vert_coord is host code: it runs without a device and equals the oracle's tables."""
    for nd, opt, kw in ((20, "even_sigma", {}), (20, "uneven_sigma", {}), (14, "mcm", {}), (18, "v197", {}),
                        (24, "uneven_sigma", dict(scale_heights=5.0, surf_res=0.2, exponent=2.0)),
                        (20, "hybrid", {}), (30, "hybrid", dict(scale_heights=5.0, surf_res=0.5))):
        ag, bg = jg.Compute_Vert_Coord(nd, opt, **kw)
        ao, bo = orc.Compute_Vert_Coord(nd, opt, **kw)
        assert np.allclose(ag, ao, rtol=1e-15, atol=0) and np.allclose(bg, bo, rtol=1e-15, atol=0), opt
    for nd, opt in ((20, "mcm"), (20, "sigma")):
        with pytest.raises(AssertionError):
            jg.Compute_Vert_Coord(nd, opt)
