/*
 * jgcm_oracle.h -- FP64 CPU oracle for the JGCM spectral-transform dynamical core.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a line-by-line FP64 restatement of the
 * reference's hot path (CliMA/IdealizedSpectralGCM.jl, module JGCM).  It is used by
 * tests/ as the parity checker and by bench.py as the timed CPU baseline.  The
 * product (libjgcm) never links, loads or calls it.
 *
 * Parity pins: the reference ships no golden vectors or fixtures, only analytic
 * known-answer checks (src/Atmos_Spectral/Gauss_And_Legendre.jl:120-169,
 * src/Atmos_Spectral/Spectral_Spherical_Mesh.jl:763-1022).  The oracle is pinned
 * against every one of those (tests/test_oracle.py) and against an independent
 * numpy/scipy restatement; the FFT boundary (FFTW.jl, unpinned, no Manifest) is
 * pinned against numpy.fft.  The reference itself cannot run here (no Julia).
 *
 * Array conventions follow the reference exactly (Julia column-major, here 0-based):
 *   grid      g[i + nlon*(j + nlat*k)]                 (lon fastest, lat south->north)
 *   spectral  s[2*(m + (N+1)*(n + (ns+1)*k)) + {0,1}]  (complex interleaved, m fastest)
 *   tables    q[m + (N+1)*(n + (ns+1)*j)]
 * with N = num_fourier, ns = num_spherical (= N+1).
 */
#ifndef JGCM_ORACLE_H
#define JGCM_ORACLE_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct om_mesh om_mesh;
typedef struct om_model om_model;

/* Gauss_And_Legendre.jl:69-118 */
int om_compute_gaussian(int n, double* sinth, double* wts);
/* Gauss_And_Legendre.jl:4-66 ; qnm, dqnm: (N+1)*(ns+1)*nlat */
int om_compute_legendre(int num_fourier, int num_spherical, const double* sinth, int nlat,
                        double* qnm, double* dqnm);

/* Spectral_Spherical_Mesh.jl:69-139 */
om_mesh* om_mesh_create(int num_fourier, int num_spherical, int nlat, int nlon, int nd, double radius);
void om_mesh_destroy(om_mesh* m);
/* copy out a named mesh table ("sinth","costh","wts","lonc","latc","qnm","dqnm","qwg",
 * "epsilon","coef_alp_a","coef_alp_b","coef_uvm","coef_uvc","coef_uvp","coef_dlam",
 * "coef_dthm","coef_dthp","laplacian_eig"); returns element count or -1 */
long om_mesh_table(const om_mesh* m, const char* name, double* out, long cap);
void om_set_threads(int nthreads);
/* FP32 emulation for error bisection (all off by default: the oracle is FP64).  Each bit runs one
 * stage of the mixed-precision GPU path in FP32 arithmetic (every operation rounded to float, the
 * Legendre sums as fused multiply-adds) or rounds one stage's outputs to float:
 *   1 forward FFT, 2 analysis Legendre sums (grid->spectral, alpha operator), 4 synthesis Legendre
 *   sums (spectral->grid), 8 inverse FFT, 16 Held-Suarez grid stage (the column computations'
 *   outputs: tendencies and the energy field, and the grid state), 32 Held-Suarez spectral stage
 *   (the analysed tendencies and the state after the semi-implicit leapfrog).  With any bit set the
 *   energy field is analysed relative to each level's first point, as the GPU sums its geopotential
 *   on T - T0_k (a per-level constant the Laplacian annihilates). */
#define OM_F32_FFT_FWD 1
#define OM_F32_ANALYSIS 2
#define OM_F32_SYNTHESIS 4
#define OM_F32_FFT_INV 8
#define OM_F32_GRID 16
#define OM_F32_SPECTRAL 32
/* 64: the geopotential reads the temperature synthesised without its (0,0) modes, with the level
 * constants added back exactly (the GPU's FP32 formulation), instead of grid T (stored in FP32) */
#define OM_F32_TANOM 64
/* 128: the fixers' column energy integrals in FP32 (summands and the sum over levels; the global
 * fold stays FP64); 256: only the kinetic part of those energies in FP32, the c_p T part and the sums
 * in FP64 (the GPU's FP32 path) */
#define OM_F32_FIXER 128
#define OM_F32_FIXER_KE 256
void om_set_f32(int mask);

/* Spectral_Spherical_Mesh.jl transforms; nlev = third dimension (nd or 1) */
void om_trans_spherical_to_grid(om_mesh* m, const double* snm, int nlev, double* grid);
void om_trans_grid_to_spherical(om_mesh* m, const double* grid, int nlev, double* snm);
/* fourier: complex [nlon, nlat, nlev] */
void om_trans_grid_to_fourier(om_mesh* m, const double* grid, int nlev, double* fourier);
void om_vor_div_from_grid_uv(om_mesh* m, const double* u, const double* v, int nlev, double* vor, double* div);
void om_uv_grid_from_vor_div(om_mesh* m, const double* vor, const double* div, int nlev, double* u, double* v);
void om_compute_ucos_vcos_from_vor_div(om_mesh* m, const double* vor, const double* div, int nlev,
                                       double* ucos, double* vcos);
void om_compute_gradient_cos(om_mesh* m, const double* hs, int nlev, double* dlam, double* dth);
void om_compute_gradients(om_mesh* m, const double* hs, int nlev, double* dlam, double* dth);
void om_add_horizontal_advection(om_mesh* m, const double* hs, const double* u, const double* v, int nlev,
                                 double* dh);
void om_apply_laplacian(om_mesh* m, double* spe, int nlev);
/* adjoints of Trans_Spherical_To_Grid! and Trans_Grid_To_Spherical! (Euclidean inner products) */
void om_trans_spherical_to_grid_adjoint(om_mesh* m, const double* grid_bar, int nlev, double* spec_bar);
void om_trans_grid_to_spherical_adjoint(om_mesh* m, const double* spec_bar, int nlev, double* grid_bar);
double om_area_weighted_global_mean(om_mesh* m, const double* grid);

/* ---- models (Barotropic_Dynamics.jl, Shallow_Water_Dynamics.jl, Spectral_Dynamics.jl) ---- */
enum { OM_BAROTROPIC = 0, OM_SHALLOW_WATER = 1, OM_HELD_SUAREZ = 2 };

typedef struct {
  int kind;
  /* Filtered_Leapfrog (Time_Integrator.jl:20-38) */
  double robert_coef;
  int damping_order;
  double damping_coef;
  double implicit_coef;
  int dt;                 /* seconds (Int64 in the reference) */
  /* Atmo_Data (Atmo_Data.jl:34-55) */
  double omega, grav, rdgas, kappa;
  int do_mass_correction, do_energy_correction;
  /* shallow water (Shallow_Water_Dynamics.jl) */
  double h0, kappa_m, kappa_t;
  /* Held-Suarez (HS_Forcing.jl, exp/HSt42/Run_HS.jl:12) */
  double sigma_b, k_f, k_a, k_s, dT_y, dtheta_z;
  /* semi-implicit reference state (exp/HSt42/HS.jl:50-54) */
  double ps_ref, t_ref;
  double sea_level_ps_ref, init_t;
} om_params;

om_model* om_model_create(om_mesh* mesh, const om_params* p);
om_model* om_model_create_vert(om_mesh* mesh, const om_params* p, const double* ak, const double* bk);
int om_vert_coord(int nd, const char* option, double scale_heights, double surf_res, double exponent, double* ak,
                  double* bk);
void om_semi_implicit_step(om_model* md, const double* const* in, double* const* out);
void om_hs_forcing(om_model* md, int Dt, const double* u, const double* v, const double* p_half,
                   const double* p_full, const double* t, double* du, double* dv, double* t_eq, double* dtt);
void om_model_destroy(om_model* md);
/* nq passive tracers advected like T on a Held-Suarez model (once, before the first step) */
int om_model_add_tracers(om_model* md, int nq);
/* named Dyn_Data fields ("spe_vor_c", "grid_u_p", ... , "grid_h_eq"); returns element count
 * (doubles) or -1 */
long om_model_field(om_model* md, const char* name, double* host, long cap, int set);
int om_model_init_step(const om_model* md);
int om_model_update_init_step(om_model* md);
/* one Barotropic_Dynamics! / Shallow_Water_Physics!+Shallow_Water_Dynamics! /
 * Atmosphere_Update! followed by the driver's Update_Init_Step! after the first step */
int om_model_step(om_model* md, int nsteps);
/* the last Held-Suarez step's fixer scalars: mean_ps_p, mean_energy_p, mean_ps_n, factor,
 * mean_energy_n, temperature correction (out[6]) */
void om_model_fixer_scalars(const om_model* md, double* out);
/* Spectral_Dynamics.jl:372-449; grid_t_pert (nullable) is added to grid_t before filtering */
int om_spectral_initialize_fields(om_model* md, const double* grid_t_pert, int vorticity_seed);
/* Semi_Implicit.jl: copy out "div_mat" (nd*nd), "h" (nd), "wave_matrix" (nd*nd*(N+1)) */
long om_model_semi_implicit(om_model* md, const char* name, double* out, long cap);

/* ---- reverse mode (the reference has none; test infrastructure for the adjoint kernels) ---- */
/* pressure variables of grid_ps_c (call after setting grid_ps_c by om_model_field) */
void om_model_sync_pressure(om_model* md);
/* set the init-step flag and rebuild the wave matrices for it */
int om_model_set_init_step(om_model* md, int flag);
/* adjoints of Vor_Div_From_Grid_UV!, UV_Grid_From_Vor_Div!, Compute_Gradients! (outputs overwritten) */
void om_vor_div_from_grid_uv_adjoint(om_mesh* m, const double* vor_bar, const double* div_bar, int nlev,
                                     double* u_bar, double* v_bar);
void om_uv_grid_from_vor_div_adjoint(om_mesh* m, const double* u_bar, const double* v_bar, int nlev,
                                     double* vor_bar, double* div_bar);
void om_compute_gradients_adjoint(om_mesh* m, const double* dlam_bar, const double* dth_bar, int nlev,
                                  double* hs_bar);
/* adjoint of one Held-Suarez step from the model's state X_s: xbar[18] (cotangents of X_{s+1} in,
 * of X_s out; order spe_vor_c spe_vor_p spe_div_c spe_div_p spe_lnps_c spe_lnps_p spe_t_c spe_t_p
 * grid_u_c grid_u_p grid_v_c grid_v_p grid_ps_c grid_ps_p grid_t_c grid_t_p grid_vor grid_div);
 * pbar[5] += cotangents of k_f, k_a, k_s, dT_y, dtheta_z */
int om_hs_step_adjoint(om_model* md, double* const* xbar, double* pbar);

#ifdef __cplusplus
}
#endif
#endif
