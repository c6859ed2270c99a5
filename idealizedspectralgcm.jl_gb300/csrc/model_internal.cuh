// model_internal.cuh -- the device-resident model (Dyn_Data + Semi_Implicit_Solver state) shared by
// the time stepping (models.cu) and the reverse sweep (hs_adjoint.cu).
#pragma once
#include "jgcm_internal.cuh"

namespace jgcm {
constexpr unsigned FULL = 0xffffffffu;
constexpr double kLnPsRef = 11.512925464970229;  // ln 1e5

struct VertCoef {  // Vert_Coordinate (even_sigma) and the semi-implicit reference column
  double ak[JGCM_MAX_ND + 1], bk[JGCM_MAX_ND + 1], dak[JGCM_MAX_ND], dbk[JGCM_MAX_ND];
  double dp_ref[JGCM_MAX_ND], rdp_ref[JGCM_MAX_ND], lnph_ref[JGCM_MAX_ND + 1], lnpf_ref[JGCM_MAX_ND],
      t_ref[JGCM_MAX_ND], h[JGCM_MAX_ND];
  // sigma coordinates (a_k = 0): with p = b ps, ln p_{k+1/2} = lb[k+1] + ln ps and
  // ln p_k = cf[k] + ln ps (Simmons-Burridge, Press_And_Geopot.jl:46-60, zero top), so every
  // log-pressure difference is a per-level constant and p_k = sf[k] ps
  int hybrid;                  // some a_k != 0: the log pressures vary per column (the sigma tables below unused)
  double lb[JGCM_MAX_ND + 1];  // ln b_k (k >= 1)
  double cf[JGCM_MAX_ND];      // ln p_k - ln ps
  double sf[JGCM_MAX_ND];      // exp(cf) = p_k / ps
  double dlp_p[JGCM_MAX_ND];   // ln p_{k+1/2} - ln p_k
  double dlp_m[JGCM_MAX_ND];   // ln p_k - ln p_{k-1/2}   (k >= 1)
  double dlp[JGCM_MAX_ND];     // ln p_{k+1/2} - ln p_{k-1/2}   (k >= 1)
  // Δa_k, Δb_k as FP32 pairs hi + lo (hi the FP32 rounding, lo that of the remainder): the FP32
  // path forms the column sums of T_k Δa_k, T_k Δb_k to FP64 accuracy from them
  float dak_hi[JGCM_MAX_ND], dak_lo[JGCM_MAX_ND], dbk_hi[JGCM_MAX_ND], dbk_lo[JGCM_MAX_ND];
};
}  // namespace jgcm

struct jgcm_model {
  jgcm_mesh* mesh;
  jgcm_params P;
  int nd, init_step, rot, sw_adv_from_n, steps_done;
  // ensemble members advanced together: every field holds ne members, member-major (grid level
  // index e*nd + k, spectral innermost index e*nd + k), so a transform sees L = ne*nd columns
  int ne, L;
  void* fbuf;  // Fourier buffer of fcap columns
  int fcap;
  int hs_lanes;  // lanes per column of the Held-Suarez column kernel (1, 2 or 4)
  int graph_gen;  // the mesh's tile generation the captured graphs were built with
  // half-level coefficients a_k, b_k given at creation (Vert_Coordinate's ak, bk); empty = even_sigma
  std::vector<double> vert_ak, vert_bk;
  // Held-Suarez: the gradients of ln ps and T of the current level are already in g_dlps ...
  // g_dtT (synthesised by the previous step together with its new level)
  int grad_ready;
  // on-device diagnostics (Output_Manager.jl:81-107): FP64 sums after every step of the zonal means
  // of T, T_eq, u, v ([4][ne][nd][nlat]) and of ps ([ne][nlat][nlon]), and the number of steps summed
  double* diag;
  int diag_on;
  long diag_steps;
  double cp_air;
  // time-levelled state (index by rotation)
  void *spe_vor[3], *spe_div[3], *spe_lnps[3], *spe_t[3];
  void *grid_u[3], *grid_v[3], *grid_ps[3], *grid_t[3];
  // single-level state and diagnostics
  void *grid_vor, *grid_div, *grid_lnps, *grid_t_eq, *grid_geopots, *grid_h_eq, *spe_zero;
  // tendencies and scratch
  void *spe_dvor, *spe_ddiv, *spe_dlnps, *spe_dt;
  void *g_dlps, *g_dtps, *g_dlT, *g_dtT, *g_ducos, *g_dvcos, *g_dt, *g_energy, *g_dlnps, *g_diag;
  void* g_tdev;  // FP32 path: the temperature of the level the next column kernel reads, less its level
                 // means (synthesised from spectral T without its (0,0) modes; written with the gradients)
  void *coriolis, *damping;  // [nlat], [m][n] in T
  void* dfac[2];             // [m][n] in T: 1/(1 + Δt d) (init step), 1/(1 + 2Δt d) (afterwards)
  // FP64 semi-implicit data
  jgcm::VertCoef vc;
  jgcm::VertCoef* d_vc;  // device copy read by the column and semi-implicit kernels
  double* div_mat;  // host nd*nd column-major
  double* d_W;      // device [2][N+1][nd][nd] (transposed: [c][r])
  int2* d_pairs;    // (m, n) pairs with n >= m
  int npairs;
  double *d_partials, *d_scalars;
  unsigned* d_counter;
  double* state_stage;  // FP64 staging of the packed host state (jgcm_model_set_state / get_state)
  // passive tracers (jgcm_model_add_tracers; Dyn_Data.jl:36-39,63-66), advected like T: nq per
  // member, columns member-major, then tracer, then level ((e nq + i) nd + k), LQ = ne nq nd
  int nq, LQ;
  void *spe_q[3], *grid_q[3];
  void *spe_dq, *g_dq, *g_dlq, *g_dtq;  // tendency (spectral, grid), gradients of the c level (÷ cos)
  void* g_mhalf;                        // the column kernel's mass flux M_{k+1/2} at level index k
  double* q_stage;                      // FP64 staging of one tracer field (get / set by name)
  void* adj;            // workspace of jgcm_model_hs_gradient, kept between calls (hs_adjoint.cu)
  cudaGraphExec_t graph[3];   // one steady step, per rotation phase
  cudaGraphExec_t graph3[3];  // three steady steps (a whole rotation), per starting phase
  cudaGraphExec_t graph24[3]; // twenty-four steady steps (eight rotations), per starting phase
  cudaEvent_t ev0, ev1;
};


namespace jgcm {
inline int lvl(const jgcm_model* md, int which) { return (md->rot + which) % 3; }  // 0 = p, 1 = c, 2 = n

// state.cu: the 18 arrays one Held-Suarez step reads and writes, in this order:
//   0 spe_vor_c, 1 spe_vor_p, 2 spe_div_c, 3 spe_div_p, 4 spe_lnps_c, 5 spe_lnps_p, 6 spe_t_c,
//   7 spe_t_p, 8 grid_u_c, 9 grid_u_p, 10 grid_v_c, 11 grid_v_p, 12 grid_ps_c, 13 grid_ps_p,
//   14 grid_t_c, 15 grid_t_p, 16 grid_vor, 17 grid_div
constexpr int NSTATE = 18;
struct StateBuf {  // a device copy of the state
  void* f[NSTATE];
  void* base;
  int init;  // the init-step flag of the copied state
};
bool st_spec(int i);
int st_levels(const jgcm_model* md, int i);
size_t st_bytes(const jgcm_model* md, int i);
void* model_slot(jgcm_model* md, int i);  // field i of the model's current state
int state_alloc(jgcm_model* md, StateBuf* b);
int state_save(jgcm_model* md, StateBuf* b, cudaStream_t st);        // model -> b (one launch)
int state_load(jgcm_model* md, const StateBuf* b, cudaStream_t st);  // b -> model (one launch)
int state_zero(jgcm_model* md, StateBuf* b, cudaStream_t st);
int copy_fields(jgcm_model* md, void* const* dst, const void* const* src, cudaStream_t st);

void adj_context_free(jgcm_model* md);  // hs_adjoint.cu: the cached gradient workspace

// models.cu services used by the reverse sweep
int dev_alloc(void** p, size_t bytes);  // cudaMalloc + zero fill
int hs_grad(jgcm_model* md, int lev, cudaStream_t st);  // gradients of ln ps and T of level `lev`
int model_step_async(jgcm_model* md);  // one step enqueued on the mesh stream, no synchronisation
// transposed semi-implicit step (Semi_Implicit.jl:360-513 + Time_Integrator.jl:58-101) on device
// buffers: obar[8] = cotangents of vor_n, vor_c', div_n, div_c', T_n, T_c', lnps_n, lnps_c';
// ibar[12] = cotangents of dvor, ddiv, dT, dlnps, vor_p, vor_c, div_p, div_c, T_p, T_c, lnps_p,
// lnps_c (written for n >= m); `mats` from si_adjoint_mats (freed by the caller with cudaFree);
// init: the step's init flag (Δt or 2Δt coefficients)
int si_adjoint_mats(jgcm_model* md, double** mats);
int si_adjoint_launch(jgcm_model* md, const void* const* obar, void* const* ibar, const double* mats, int init,
                      cudaStream_t st);
}  // namespace jgcm
