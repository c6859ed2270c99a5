#!/usr/bin/env python
"""Generates the golden fixtures in this folder (run from the repository root):

  python tests/golden/make_golden.py

analytic_t21.npz   the reference's own known answers at T21, nθ = 32 (Gauss_And_Legendre.jl:120-169):
                   Gauss-Legendre nodes (south -> north) and weights from scipy, and the closed-form
                   P_{n,m}(μ) and dP/dμ the reference's test() compares against (:132-156), computed
                   here with numpy, independently of the oracle.
oracle_t21.npz     seeded inputs and the FP64 oracle's outputs of the transform entry points at T21
                   (nθ = 32, nλ = 64, 2 levels, radius 6371 km): Trans_Spherical_To_Grid!,
                   Trans_Grid_To_Spherical!, Vor_Div_From_Grid_UV!, UV_Grid_From_Vor_Div!.
                   The oracle is pinned by analytic_t21.npz and by the reference's analytic tests.
"""
import os
import sys

import numpy as np
from scipy.special import roots_legendre

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path[:0] = [os.path.join(ROOT, "oracle"), os.path.join(ROOT, "idealizedspectralgcm.jl_gb300")]


def closed_forms(s):
    """(m, n) -> (P, dP/dμ) for the five cases of Gauss_And_Legendre.jl:132-156."""
    c = np.sqrt(1 - s ** 2)
    return {
        (3, 3): (np.sqrt(35) / 4 * c ** 3, np.sqrt(35) / 4 * c * 1.5 * (-2 * s)),
        (2, 3): (np.sqrt(105 / 8) * (s - s ** 3), np.sqrt(105 / 8) * (1 - 3 * s ** 2)),
        (0, 2): (np.sqrt(5) / 2 * (3 * s ** 2 - 1), np.sqrt(5) / 2 * 6 * s),
        (0, 3): (np.sqrt(7) / 2 * (5 * s ** 3 - 3 * s), np.sqrt(7) / 2 * (15 * s ** 2 - 3)),
        (1, 3): (np.sqrt(21) / 4 * (5 * s ** 2 - 1) * c,
                 np.sqrt(21) / 4 * 10 * s * c + np.sqrt(21) / 4 * (5 * s ** 2 - 1) / c * 0.5 * (-2 * s)),
    }


def seeded_spectral(rng, N, nd):
    s = rng.standard_normal((N + 1, N + 2, nd)) + 1j * rng.standard_normal((N + 1, N + 2, nd))
    s /= (1.0 + np.arange(N + 2))[None, :, None] ** 1.5
    for m in range(N + 1):
        s[m, :m, :] = 0
    s[0, :, :] = s[0, :, :].real  # m = 0 modes of a real field are real
    return np.asfortranarray(s)


def main():
    s, w = roots_legendre(32)
    cf = closed_forms(s)
    keys = sorted(cf)
    np.savez(os.path.join(HERE, "analytic_t21.npz"), sinth=s, wts=w, mn=np.array(keys, dtype=np.int64),
             P=np.stack([cf[k][0] for k in keys]), dP=np.stack([cf[k][1] for k in keys]))

    import oracle

    N, nlat, nlon, nd, a = 21, 32, 64, 2, 6371.0e3
    mesh = oracle.Spectral_Spherical_Mesh(N, N + 1, nlat, nlon, nd, a)
    rng = np.random.default_rng(20261203)
    spec_in = seeded_spectral(rng, N, nd)
    grid_out = mesh.grid(nd)
    oracle.Trans_Spherical_To_Grid(mesh, spec_in, grid_out)
    grid_in = np.asfortranarray(rng.standard_normal((nlon, nlat, nd)))
    spec_out = mesh.spectral(nd)
    oracle.Trans_Grid_To_Spherical(mesh, grid_in, spec_out)
    u_in = np.asfortranarray(20.0 * rng.standard_normal((nlon, nlat, nd)))
    v_in = np.asfortranarray(20.0 * rng.standard_normal((nlon, nlat, nd)))
    vor_out, div_out = mesh.spectral(nd), mesh.spectral(nd)
    oracle.Vor_Div_From_Grid_UV(mesh, u_in, v_in, vor_out, div_out)
    vor_in = seeded_spectral(rng, N, nd) * 1e-5
    div_in = seeded_spectral(rng, N, nd) * 1e-6
    vor_in[0, 0, :] = 0
    div_in[0, 0, :] = 0
    u_out, v_out = mesh.grid(nd), mesh.grid(nd)
    oracle.UV_Grid_From_Vor_Div(mesh, vor_in, div_in, u_out, v_out)
    np.savez(os.path.join(HERE, "oracle_t21.npz"), N=N, nlat=nlat, nlon=nlon, nd=nd, radius=a,
             spec_in=spec_in, grid_out=grid_out, grid_in=grid_in, spec_out=spec_out, u_in=u_in, v_in=v_in,
             vor_out=vor_out, div_out=div_out, vor_in=vor_in, div_in=div_in, u_out=u_out, v_out=v_out)
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
