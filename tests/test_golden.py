"""The committed golden fixtures (tests/golden/, written by tests/golden/make_golden.py).

analytic_t21.npz pins the oracle's tables to the reference's own known answers; oracle_t21.npz pins
the transform entry points: the oracle must reproduce it (regression of the oracle itself) and the
GPU library must match it (FP64 1e-12, FP32 5e-6 relative L2, the transform-test tolerances).
"""
import os

import numpy as np
import pytest

from jgcm import configs

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLD, name)))


def test_oracle_tables_match_analytic_fixture(orc):
    g = load("analytic_t21.npz")
    s, w = orc.compute_gaussian(32)
    assert np.max(np.abs(s - g["sinth"])) < 5e-16
    assert np.max(np.abs(w - g["wts"]) / g["wts"]) < 1e-14 * 32 ** 2
    q, dq = orc.compute_legendre(21, 22, g["sinth"], 32)
    for (m, n), P, dP in zip(g["mn"], g["P"], g["dP"]):
        assert np.linalg.norm(q[m, n] - P) < 1e-13
        assert np.linalg.norm(dq[m, n] - dP) < 5e-12


def _run_transforms(backend, g, precision=None):
    N, nlat, nlon, nd, a = int(g["N"]), int(g["nlat"]), int(g["nlon"]), int(g["nd"]), float(g["radius"])
    kw = {} if precision is None else {"precision": precision}
    mesh = backend.Spectral_Spherical_Mesh(N, N + 1, nlat, nlon, nd, a, **kw)
    out = {}
    out["grid_out"] = mesh.grid(nd)
    backend.Trans_Spherical_To_Grid(mesh, g["spec_in"], out["grid_out"])
    out["spec_out"] = mesh.spectral(nd)
    backend.Trans_Grid_To_Spherical(mesh, np.asfortranarray(g["grid_in"]), out["spec_out"])
    out["vor_out"], out["div_out"] = mesh.spectral(nd), mesh.spectral(nd)
    backend.Vor_Div_From_Grid_UV(mesh, np.asfortranarray(g["u_in"]), np.asfortranarray(g["v_in"]), out["vor_out"],
                                 out["div_out"])
    out["u_out"], out["v_out"] = mesh.grid(nd), mesh.grid(nd)
    backend.UV_Grid_From_Vor_Div(mesh, np.asfortranarray(g["vor_in"]), np.asfortranarray(g["div_in"]), out["u_out"],
                                 out["v_out"])
    return out


def test_oracle_reproduces_transform_fixture(orc):
    g = load("oracle_t21.npz")
    out = _run_transforms(orc, g)
    for k, v in out.items():
        assert configs.rel_l2(v, g[k]) < 1e-14, k


@pytest.mark.gpu
@pytest.mark.parametrize("prec,tol", [("fp64", 1e-12), ("fp32", 5e-6)])
def test_gpu_matches_transform_fixture(jg, prec, tol):
    g = load("oracle_t21.npz")
    out = _run_transforms(jg, g, prec)
    for k, v in out.items():
        assert configs.rel_l2(v, g[k]) < tol, (k, configs.rel_l2(v, g[k]))
