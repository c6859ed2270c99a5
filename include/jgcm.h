/*
 * jgcm.h -- C ABI of libjgcm, the GB300-native (sm_103a) spectral-transform dynamical core.
 *
 * Drop-in for the Atmos_Spectral hot path of CliMA/IdealizedSpectralGCM.jl (module JGCM).
 * Every entry point below replaces one Julia method of the reference; the comment above
 * each cites the file:line of the method it replaces.  A Julia host binds these with
 * `ccall`; the tests bind them with ctypes.
 *
 * Conventions
 *  - Every function returns an int status: JGCM_OK (0) or a negative JGCM_E_* code.
 *    jgcm_last_error() returns a message for the calling thread's last failure.
 *    Nothing aborts, traps or throws across the ABI.
 *  - Host arrays use the reference's Julia layout (column-major, 1-based in Julia,
 *    0-based here):  grid  double[nlev][nlat][nlon]   (Array{Float64,3}(nlon,nlat,nlev))
 *                    spec  double[nlev][N+2][N+1][2]  (Array{ComplexF64,3}(N+1,N+2,nlev),
 *                                                       re/im interleaved, m fastest)
 *    with N = num_fourier, num_spherical = N+1, latitudes south->north (Gaussian).
 *    nlev is the array's third dimension and must be nd or 1, as in the reference.
 *  - Host arrays are always FP64; the device computes in the mesh's precision mode.
 *  - A mesh owns one CUDA stream, its device tables and its transform workspace.  Calls on
 *    one mesh (and the models built on it) are not re-entrant, matching the reference,
 *    whose mesh owns shared scratch buffers (Spectral_Spherical_Mesh.jl:51-64).
 */
#ifndef JGCM_H
#define JGCM_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
#if defined(__GNUC__)
#pragma GCC visibility push(default) /* the library builds with -fvisibility=hidden */
#endif

#define JGCM_OK 0
#define JGCM_E_ARG -1      /* bad argument / shape (reference: AssertionError) */
#define JGCM_E_CUDA -2     /* CUDA runtime failure */
#define JGCM_E_NOMEM -3    /* device allocation failed */
#define JGCM_E_STATE -4    /* call not valid in this state */
#define JGCM_E_NUMERIC -5  /* non-finite value detected by a device check */

/* Precision modes (jgcm_mesh_create). */
#define JGCM_FP64 0       /* all device arithmetic FP64 (the FP64 GPU path) */
#define JGCM_FP32 1       /* FP32 state/transforms, FP64 tables, implicit solve and sums */
#define JGCM_TF32X3 2     /* as FP32, Legendre contraction on tcgen05 tensor cores, 3xTF32 split */
#define JGCM_BF16X3 3     /* as FP32, Legendre contraction on tcgen05, 3-term split-BF16 */

typedef struct jgcm_mesh jgcm_mesh;
typedef struct jgcm_model jgcm_model;

const char* jgcm_last_error(void);
int jgcm_version(void);
/* Device properties of the current device: SM count, compute capability. */
int jgcm_device_info(int* sm_count, int* cc_major, int* cc_minor);

/* Spectral_Spherical_Mesh constructor, Spectral_Spherical_Mesh.jl:69-139 (argument order
 * num_fourier, num_spherical, nθ, nλ, nd, radius as in the reference).  Gaussian nodes
 * (Gauss_And_Legendre.jl:69-118) and Legendre tables (:4-66) are generated on the GPU
 * in FP64. */
int jgcm_mesh_create(int num_fourier, int num_spherical, int nlat, int nlon, int nd, double radius,
                     int precision, jgcm_mesh** out);
int jgcm_mesh_destroy(jgcm_mesh* mesh);
int jgcm_mesh_precision(const jgcm_mesh* mesh);
/* Copy a mesh table to the host, FP64, reference layout: "sinth","costh","wts","lonc","latc"
 * ([nlat] or [nlon]), "qnm","dqnm","qwg","coef_alp_a","coef_alp_b" ([nlat][N+2][N+1]),
 * "epsilon","coef_uvm","coef_uvc","coef_uvp","coef_dlam","coef_dthm","coef_dthp",
 * "laplacian_eig" ([N+2][N+1]).  Writes *count = element count; out may be NULL to query. */
int jgcm_mesh_table(jgcm_mesh* mesh, const char* name, double* out, long cap, long* count);
/* Block until all work queued on the mesh stream is done.  On a tensor-core mesh (JGCM_TF32X3,
 * JGCM_BF16X3) it also reports a Legendre kernel whose bounded wait gave up since the last check
 * (JGCM_E_CUDA, message in jgcm_last_error; the status is cleared): the only report the
 * asynchronous entry points (jgcm_trans_spherical_to_grid_noalloc) give of that failure. */
int jgcm_mesh_synchronize(jgcm_mesh* mesh);

/* Trans_Spherical_To_Grid!  Spectral_Spherical_Mesh.jl:143-217 */
int jgcm_trans_spherical_to_grid(jgcm_mesh* mesh, const double* snm, int nlev, double* pfield);
/* Trans_Grid_To_Spherical!  Spectral_Spherical_Mesh.jl:221-293 */
int jgcm_trans_grid_to_spherical(jgcm_mesh* mesh, const double* pfield, int nlev, double* snm);
/* Adjoints of the two transforms (no counterpart in the reference; the differentiation pattern
 * of the dynamical core): for the Euclidean inner products of the host arrays (complex entries as
 * (re, im) pairs, entries n < m excluded), <S2G s, g> = <s, S2G^T g> and <G2S g, s> = <g, G2S^T s>.
 * S2G^T is the transposed quadrature: forward DFT, then the unweighted Legendre sum c_m nlon
 * sum_j P_n^m(mu_j) G_m(mu_j) (c_0 = 1, c_m = 2), row N+1 included; G2S^T synthesises the
 * spectral cotangent (m >= 1 halved, row N+1 dropped) and scales each latitude by w_j / (2 nlon). */
int jgcm_trans_spherical_to_grid_adjoint(jgcm_mesh* mesh, const double* grid_bar, int nlev, double* spec_bar);
int jgcm_trans_grid_to_spherical_adjoint(jgcm_mesh* mesh, const double* spec_bar, int nlev, double* grid_bar);
/* Trans_Grid_To_Fourier!  Spectral_Spherical_Mesh.jl:295-330; fourier is the reference's
 * fourier_g, Array{ComplexF64,3}(nλ, nθ, nlev): fft(pfield, 1) / nλ, every mode m = 0..nλ-1
 * (complex double[nlev][nlat][nlon], re/im interleaved, m fastest; modes above nλ/2 are the complex
 * conjugates of modes nλ - m, as for any real row). */
int jgcm_trans_grid_to_fourier(jgcm_mesh* mesh, const double* pfield, int nlev, double* fourier);
/* Vor_Div_From_Grid_UV!  Spectral_Spherical_Mesh.jl:349-393 (+ Compute_Alpha_Operator! :424-459) */
int jgcm_vor_div_from_grid_uv(jgcm_mesh* mesh, const double* grid_u, const double* grid_v, int nlev,
                              double* vor, double* div);
/* UV_Grid_From_Vor_Div!  Spectral_Spherical_Mesh.jl:462-482 (+ :517-580) */
int jgcm_uv_grid_from_vor_div(jgcm_mesh* mesh, const double* vor, const double* div, int nlev,
                              double* grid_u, double* grid_v);
/* Compute_Gradients!  Spectral_Spherical_Mesh.jl:721-741 (+ Compute_Gradient_Cos! :655-692) */
int jgcm_compute_gradients(jgcm_mesh* mesh, const double* spe_hs, int nlev, double* grid_dlam_hs,
                           double* grid_dth_hs);
/* Add_Horizontal_Advection!  Spectral_Spherical_Mesh.jl:694-718 (grid_dhs updated in place) */
int jgcm_add_horizontal_advection(jgcm_mesh* mesh, const double* spe_hs, const double* grid_u,
                                  const double* grid_v, int nlev, double* grid_dhs);
/* Apply_Laplacian!  Spectral_Spherical_Mesh.jl:614-621 (in place) */
int jgcm_apply_laplacian(jgcm_mesh* mesh, double* spe, int nlev);
/* Area_Weighted_Global_Mean  Spectral_Spherical_Mesh.jl:746-760 (level 1; FP64 sum) */
int jgcm_area_weighted_global_mean(jgcm_mesh* mesh, const double* grid, double* out);

/* Spectral -> grid transform that allocates nothing.  No counterpart in the reference: it is an
 * addition for callers that cannot allocate device memory where they transform -- code running
 * while a stream is captured into a CUDA graph, hosts whose device memory belongs to their own
 * pool allocator, and loops that forbid allocation after start-up.
 *   d_snm   device array, mesh precision, library layout: complex [m][n][k] (N+1 x N+2 x nlev,
 *           levels innermost; entries n < m are ignored)
 *   d_grid  device array, mesh precision: [k][nlat][nlon]
 *   stream  cudaStream_t to run on, or NULL for the mesh's stream; the call is asynchronous.
 * Same result as jgcm_trans_spherical_to_grid.  The Fourier coefficients are staged in a static
 * 8 MiB device array owned by the library (every GPU that loads it holds it until exit), so
 * (N+1) * nlat * nlev complex values must fit: larger sizes return JGCM_E_ARG with a message.
 * The first call on a device resolves that array's address (set-up), so make it before any
 * stream capture.  All calls share the array: calls that overlap on the GPU (different streams,
 * meshes or threads without ordering) race.  A successful call writes every scratch element it
 * reads, so nothing needs clearing between calls.  On a tensor-core mesh a Legendre kernel whose
 * bounded wait gave up leaves the scratch (and so d_grid) stale; the call, being asynchronous,
 * cannot say so: jgcm_mesh_synchronize on the mesh reports it. */
int jgcm_trans_spherical_to_grid_noalloc(jgcm_mesh* mesh, const void* d_snm, int nlev, void* d_grid,
                                         void* stream);

/* ---- models: Dyn_Data + Filtered_Leapfrog (+ Semi_Implicit_Solver) kept on the device ---- */
#define JGCM_BAROTROPIC 0     /* Barotropic_Dynamics!  Barotropic_Dynamics.jl:2-46 */
#define JGCM_SHALLOW_WATER 1  /* Shallow_Water_Physics! + Shallow_Water_Dynamics!
                                 Shallow_Water_Dynamics.jl:7-179 */
#define JGCM_HELD_SUAREZ 2    /* Atmosphere_Update!  Spectral_Dynamics.jl:470-490 */

/* Run parameters.  Mirrors the arguments of Filtered_Leapfrog (Time_Integrator.jl:20-38),
 * Atmo_Data (Atmo_Data.jl:34-55), Semi_Implicit_Solver (Semi_Implicit.jl:40-97), the SW
 * driver (exp/Shallow_Water/SW.jl:12-25) and the HS physics Dict (exp/HSt42/Run_HS.jl:12). */
typedef struct {
  int kind;
  double robert_coef;
  int damping_order;
  double damping_coef;
  double implicit_coef;
  int dt; /* seconds */
  double omega, grav, rdgas, kappa;
  int do_mass_correction, do_energy_correction;
  double h0, kappa_m, kappa_t;
  double sigma_b, k_f, k_a, k_s, dT_y, dtheta_z;
  double ps_ref, t_ref;
  double sea_level_ps_ref, init_t;
} jgcm_params;

int jgcm_model_create(jgcm_mesh* mesh, const jgcm_params* params, jgcm_model** out);
/* Ensembles (no counterpart in the reference, whose drivers run one member): `members`
 * independent members of one mesh and parameter set, advanced together by the same kernels
 * (every field holds all members, member-major).  Members are initialised as one-member models
 * and copied in; their fields are read by copying a member out into a one-member model. */
int jgcm_model_create_members(jgcm_mesh* mesh, const jgcm_params* params, int members, jgcm_model** out);
int jgcm_model_members(jgcm_model* model, int* members);
/* Vert_Coordinate's Compute_Vert_Coord (Atmos_Spectral/Vert_Coordinate.jl:61-87), host FP64:
 * half-level coefficients ak[nd+1], bk[nd+1] (p_{k+1/2} = ak + bk ps, top first) for option
 * "even_sigma", "uneven_sigma" (scale_heights, surf_res, exponent: the reference's defaults are
 * 4, 1, 2.5; built as Compute_Uneven_Sigma's docstring states, :120-141 — the reference's code
 * for that branch does not run), "mcm" (nd 14), "v197" (nd 18) or "hybrid" (:71-76 as its code means
 * it -- the reference's branch does not run: uneven sigma levels s_k serve as pressure levels
 * 101325 s_k above s = 0.1 and as sigma levels below s = 0.3, blended by Transition's sin^2,
 * :93-110); always zero top (the constructor's default, :44). */
int jgcm_vert_coord(int nd, const char* option, double scale_heights, double surf_res, double exponent,
                    double* ak, double* bk);
/* jgcm_model_create_members on the vertical coordinate ak, bk (each nd+1; NULL, NULL = even_sigma,
 * the reference drivers' choice, Spectral_Dynamics.jl:513): a zero top (ak[0] = bk[0] = 0), the
 * surface at the bottom (ak[nd] = 0, bk[nd] = 1) and half-level pressures ak + bk ps increasing
 * downwards for ps within 10 % of ps_ref, else JGCM_E_ARG.  Hybrid coordinates (ak != 0) run the
 * forward model; jgcm_model_step_adjoint and jgcm_model_hs_gradient need sigma coordinates. */
int jgcm_model_create_vert(jgcm_mesh* mesh, const jgcm_params* params, int members, const double* ak,
                           const double* bk, jgcm_model** out);
/* Passive tracers (Dyn_Data's spe_tracers_{n,c,p} [N+1, N+2, nd, nq] and grid_tracers_{n,c,p}
 * [nλ, nθ, nd, nq], Dyn_Data.jl:36-39,63-66, rotated by Time_Advance! :341-342, 360-361): num_tracers
 * per member on a Held-Suarez model, every level zero, read and written by those names.  The
 * reference allocates them and never steps them (Spectral_Dynamics.jl:235 has "grid_q = grid_t" as
 * a todo); here every step advects them like T: Vert_Advection! with the step's mass flux and
 * Add_Horizontal_Advection! of spe_tracers_c, Trans_Grid_To_Spherical!, T's spectral damping and
 * filtered leapfrog, no forcing and no semi-implicit term, then Trans_Spherical_To_Grid! of the new
 * level.  Once per model, num_tracers in [1, 64]; the step adjoint refuses models with tracers. */
int jgcm_model_add_tracers(jgcm_model* model, int num_tracers);
int jgcm_model_num_tracers(jgcm_model* model, int* num_tracers);
/* Copy member src_member of src into member dst_member of dst (same mesh and model kind): every
 * time level of the prognostic state and the grid diagnostics.  A one-member dst also takes the
 * source's time-step state (init step); an ensemble dst must already share it. */
int jgcm_model_copy_member(jgcm_model* dst, int dst_member, jgcm_model* src, int src_member);
/* One semi-implicit step on its own and its adjoint (Held-Suarez; no counterpart in the reference):
 * Adjust_δlnps_δt_δdiv! + Implicit_Correction! (Semi_Implicit.jl:360-513) + Compute_Spectral_Damping!
 * + Filtered_Leapfrog! (Time_Integrator.jl:58-101) for the model's current step (init step or not),
 * a linear map.  in[12]: δvor, δdiv, δT, δlnps, vor_p, vor_c, div_p, div_c, T_p, T_c, lnps_p,
 * lnps_c; out[8]: vor_n, vor_c (filtered), div_n, div_c, T_n, T_c, lnps_n, lnps_c.  Spectral host
 * arrays [N+1, N+2, nd] (lnps: 1 level).  The adjoint maps cotangents of out to cotangents of in. */
int jgcm_model_semi_implicit_step(jgcm_model* model, const double* const* in, double* const* out);
int jgcm_model_semi_implicit_step_adjoint(jgcm_model* model, const double* const* out_bar, double* const* in_bar);
/* The whole state of a Held-Suarez step in one transfer (no counterpart in the reference, which keeps
 * Dyn_Data on the host): the 18 arrays in the order of jgcm_model_step_adjoint below, each in the
 * reference host layout (FP64; spectral complex interleaved), back to back in one host buffer of
 * *ndoubles doubles.  One host<->device copy and one layout-conversion launch each way; a restart
 * from host state, or a read-out of it, costs one call instead of one per field.  One-member models. */
int jgcm_model_state_size(jgcm_model* model, long* ndoubles);
int jgcm_model_set_state(jgcm_model* model, const double* packed);
int jgcm_model_get_state(jgcm_model* model, double* packed);
/* Reverse mode of one whole Held-Suarez step (Atmosphere_Update!, Spectral_Dynamics.jl:206-365 +
 * 452-490 with HS_Forcing.jl and Compute_Corrections!; no counterpart in the reference) from the
 * model's current state X_s.  state_bar[18] holds host arrays (reference layout) of the cotangents
 * of X_{s+1} on entry and receives those of X_s, in the order spe_vor_c, spe_vor_p, spe_div_c,
 * spe_div_p, spe_lnps_c, spe_lnps_p, spe_t_c, spe_t_p, grid_u_c, grid_u_p, grid_v_c, grid_v_p,
 * grid_ps_c, grid_ps_p, grid_t_c, grid_t_p, grid_vor, grid_div; param_bar[5] (nullable) is
 * incremented by the cotangents of k_f, k_a, k_s, dT_y, dtheta_z.  The model is left at X_s.
 * One-member models, nd <= 32, diagnostics off. */
int jgcm_model_step_adjoint(jgcm_model* model, double* const* state_bar, double* param_bar);
/* Loss J = sum_{i,j,k} w_j (T - t_target)^2 / (2 nlon nd) of the grid temperature after nsteps
 * steps from the model's current state, and its gradient with respect to the initial spectral
 * temperature T0 (the state's spe_t_c = spe_t_p = T0 and grid_t_c = grid_t_p = S2G(T0), as
 * Spectral_Initialize_Fields! leaves them; host array [N+1, N+2, nd]; T0 has row N+1 = 0 like every
 * analysis output, so that row of the gradient is returned as 0) and to k_f, k_a, k_s, dT_y,
 * dtheta_z (grad_params[5]).  The reverse sweep recomputes each segment of checkpoint_every steps
 * from its stored state.  t_target: host grid [nlon, nlat, nd].  Outputs are nullable.  The
 * model is left at the final state. */
int jgcm_model_hs_gradient(jgcm_model* model, int nsteps, int checkpoint_every, const double* t_target,
                           double* loss, double* grad_spe_t0, double* grad_params);
/* On-device diagnostics (Held-Suarez): the reductions of Update_Output! (Output_Manager.jl:81-107)
 * as FP64 sums after every step — zonal means of T, T_eq, u, v and the ps field.  on = 1 zeroes
 * the sums and starts; on = 0 stops.  read returns the mean over the summed steps of
 * "t_zonal_mean", "t_eq_zonal_mean", "u_zonal_mean", "v_zonal_mean" ([nθ, nd, members]) or
 * "ps_mean" ([nλ, nθ, members]) and, in *steps, how many steps were summed. */
int jgcm_model_diagnostics(jgcm_model* model, int on);
int jgcm_model_read_diagnostics(jgcm_model* model, const char* name, double* out, long cap, long* count,
                                long* steps);
/* Tiles (no counterpart in the reference).  knobs[0]: lanes per column of the Held-Suarez column
 * kernel (1, 2, 4, 8; this model); knobs[1..3]: S2G, G2S and FFT columns per block of the SIMT
 * transform kernels (the mesh: shared by its models).  0 = default; knobs[3] = -1 puts FP32 rows of
 * nlon 64 or 128 one per thread whatever their number (by default from 19456 rows on: nlon 64, and the inverse at nlon 128).  knobs[4] (read and written when
 * n >= 5): the Legendre engine of a tensor-core precision mode (0 tcgen05, 1 the FP32 SIMT
 * kernels; the mesh).  knobs[5] (n >= 6): levels per block of the Held-Suarez analysis kernel (the
 * mesh; 0 = default, -1 = the general analysis kernel instead).  The autotuner times candidates on a scratch copy of the model (coordinate
 * search, nsteps captured steps each), applies the fastest, writes it to knobs (nullable; the first
 * min(n, 6) knobs, n >= 4, like jgcm_model_get_tuning) and its time per nsteps to ms (nullable). */
int jgcm_model_get_tuning(jgcm_model* model, int* knobs, int n);
int jgcm_model_set_tuning(jgcm_model* model, const int* knobs, int n);
int jgcm_model_autotune(jgcm_model* model, int nsteps, int* knobs, int n, float* ms);
/* Uneven ensembles (no counterpart in the reference): several (member-batched) models of
 * different truncations or kinds advanced together, window_seconds of simulated time per window,
 * each window one graph launch whose branches step the models concurrently (window_seconds a
 * multiple of every model's dt; every model past its first step).  The models stay usable on
 * their own between windows. */
typedef struct jgcm_ensemble jgcm_ensemble;
int jgcm_ensemble_create(jgcm_model* const* models, int nmodels, int window_seconds, jgcm_ensemble** out);
int jgcm_ensemble_step(jgcm_ensemble* ensemble, int nwindows);
int jgcm_ensemble_time(jgcm_ensemble* ensemble, int nwindows, float* ms); /* CUDA-event ms of nwindows */
int jgcm_ensemble_destroy(jgcm_ensemble* ensemble);
int jgcm_model_destroy(jgcm_model* model);
/* Read / write one Dyn_Data field (Dyn_Data.jl:4-156) by its reference name with the
 * δ spelled "d": "spe_vor_c", "grid_u_p", "spe_dt", "grid_t_eq", "grid_p_full",
 * "grid_z_full", "grid_h_eq", ...  Layout as above; *count = doubles in the field. */
int jgcm_model_get_field(jgcm_model* model, const char* name, double* host, long cap, long* count);
int jgcm_model_set_field(jgcm_model* model, const char* name, const double* host, long count);
/* Advance nsteps model steps.  The first step of a fresh model is the forward (init) step
 * and is followed by Update_Init_Step! (Time_Integrator.jl:40-43, Semi_Implicit.jl:182-188),
 * exactly as the reference drivers do (exp/HSt42/HS.jl:73-81).  Steady-state steps run as
 * captured CUDA graphs. */
int jgcm_model_step(jgcm_model* model, int nsteps);
int jgcm_model_init_step(jgcm_model* model, int* init_step);
/* Update_Init_Step!  Time_Integrator.jl:40-43 / Semi_Implicit.jl:182-188: leave the forward
 * init-step mode without stepping (e.g. when restarting from a saved leapfrog state). */
int jgcm_model_update_init_step(jgcm_model* model);
/* Set the init-step flag (1: the next step is a first step with Δt, Time_Integrator.jl:40-56), e.g.
 * to restart from a stored first state.  No counterpart in the reference. */
int jgcm_model_set_init_step(jgcm_model* model, int init_step);
/* HS_Forcing!  HS_Forcing.jl:1-130 (Rayleigh_Damping! :101-130, energy-conserving heating :21-26,
 * Newtonian_Damping! :37-97) on host arrays in the reference layout: u, v, t, p_full, du, dv,
 * t_eq, dt are [nλ,nθ,nd], p_half is [nλ,nθ,nd+1]; Δt in seconds as Get_Δt returns it.  The
 * physics parameters and c_p come from the model (the reference's physics Dict and Atmo_Data);
 * computed in the mesh precision. */
int jgcm_hs_forcing(jgcm_model* model, int dt, const double* grid_u, const double* grid_v,
                    const double* grid_p_half, const double* grid_p_full, const double* grid_t, double* grid_du,
                    double* grid_dv, double* grid_t_eq, double* grid_dt);
/* Spectral_Initialize_Fields!  Spectral_Dynamics.jl:372-449.  grid_t_pert (nullable,
 * grid[nd]) is added to the isothermal init_t before the spectral filtering;
 * vorticity_seed != 0 keeps the reference's deterministic vorticity seed (:401-409). */
int jgcm_spectral_initialize_fields(jgcm_model* model, const double* grid_t_pert, int vorticity_seed);
/* Semi_Implicit_Solver internals: "div_mat" (nd*nd), "h" (nd), "wave_matrix"
 * (nd*nd*(N+1)), column-major as in Semi_Implicit.jl:112-180. */
int jgcm_model_semi_implicit(jgcm_model* model, const char* name, double* out, long cap, long* count);
/* Time nsteps steady-state steps with CUDA events on the model stream (milliseconds). */
int jgcm_model_time_steps(jgcm_model* model, int nsteps, float* ms);
/* Number of kernel launches one steady-state step issues. */
int jgcm_model_launches_per_step(jgcm_model* model, int* launches);
/* Per-kernel CUDA-event times of nsteps steady steps (eager launches): ms[slot] is the mean
 * device time of launch `slot` of a step; *count = launches per step.  Advances the model. */
int jgcm_model_kernel_times(jgcm_model* model, int nsteps, float* ms, int cap, int* count);
int jgcm_model_kernel_name(jgcm_model* model, int slot, char* buf, int cap);
/* Select the CUDA device used by subsequently created meshes on this thread. */
int jgcm_set_device(int device);
/* Failure-path self-test (no counterpart in the reference): a kernel waits, with a short poll
 * bound, on a barrier phase nothing completes, sets the mesh's status bit and
 * returns; the call then reports it like a Legendre kernel that gave up (JGCM_E_CUDA with a message)
 * and clears it.  The mesh stays usable. */
int jgcm_selftest_bounded_wait(jgcm_mesh* mesh);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif
#ifdef __cplusplus
}
#endif
#endif
