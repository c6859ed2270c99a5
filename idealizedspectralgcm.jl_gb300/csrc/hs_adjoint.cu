// hs_adjoint.cu -- reverse mode of the Held-Suarez step (the differentiation pattern; the reference
// has no adjoint) and the gradient of a loss over many steps with recomputation checkpoints.
//
// One step maps the state X_s (18 fields: spectral vor, div, ln ps, T at the c and p levels; grid
// u, v, ps, T at the c and p levels; grid vor, div) to X_{s+1} (Atmosphere_Update!,
// Spectral_Dynamics.jl:206-365 + 452-490 with HS_Forcing.jl:1-130 and Compute_Corrections!
// :30-68).  Its adjoint runs the stages backwards:
//   fixers (energy, then mass)            3 column kernels + 2 single-block FP64 folds
//   syntheses of the new level            one batched analysis-type launch (S2G^T)
//   implicit correction + leapfrog        the transposed semi-implicit kernel (models.cu)
//   analyses of the tendencies            one synthesis-type launch (G2S^T) + the transposed alpha
//                                         operator (k_alpha_adjoint + inverse FFT)
//   column physics and dynamics           k_hs_column_adjoint: a warp per column, lanes over
//                                         levels (Four_In_One!, Vert_Advection!, geopotential,
//                                         HS_Forcing!, the p-level energy), FP64 arithmetic
//   gradients of ln ps and T              one S2G^T launch + k_grad_adjoint
// In sigma coordinates (a_k = 0) every log-pressure difference is a per-level constant, so the
// dynamics depend on ps only through grad ln ps; only the Newtonian relaxation (T_eq(p)) and the
// fixers see ps itself.  FP64 folds of block partials keep every global sum deterministic.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "model_internal.cuh"
#include "transform_ops.cuh"

using namespace jgcm;

namespace {

// ---- deterministic FP64 reductions --------------------------------------------------------------
// Sum over the block in a fixed order; the result is valid in thread 0.
__device__ double block_sum(double v) {
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)((blockDim.x + 31) >> 5); w++) t += red[w];
  return t;
}

// fixed-order sum of nb block partials (one block of 256 threads): valid in thread 0
__device__ double fold_partials(const double* part, int nb) {
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) s += part[b];
  return block_sum(s);
}

// scalar slots (FP64, device)
enum {
  SC_MPS_P = 0,   // forward: mean_ps_p
  SC_EP = 1,      //          mean_energy_p
  SC_FACTOR = 2,  //          mass-fixer factor
  SC_CORR = 3,    //          temperature correction
  SC_EP_BAR = 4,
  SC_MPSP_BAR = 5,
  SC_EN_BAR = 6,
  SC_MN_BAR = 7,
  SC_LOSS = 8,
  SC_N = 16
};

struct FixArgs {
  const void *u_n, *v_n, *t_n2, *ps_n2;  // X_{s+1} grid fields
  void *bu, *bv, *bt, *bps;              // cotangents of X_{s+1} grid u_c, v_c, t_c, ps_c (updated in place)
  const void *bt_spec, *bl_spec;         // cotangents of X_{s+1} spe_t_c, spe_lnps_c
  void *g_lnps, *g_uc, *g_vc;            // outputs: ln ps cotangent, u and v cotangents / cos
  const double* wts;
  const void* cosj;
  double* sc;
  double* part;
  const VertCoef* vc;
  int nd, nlat, nlon, do_mass, do_energy;
  double cp, grav;
  double inv_2n, ig;  // 1 / (2 nlon) (exact: nlon is a power of two), 1 / grav
  float cpf, igf;     // cp and 1 / grav rounded to FP32 on the host
};

// one thread per grid point: block partials of the sum of the grid temperature cotangent
template <typename T>
__global__ void __launch_bounds__(256) k_fix1(FixArgs a) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  const size_t n = (size_t)a.nlat * a.nlon * a.nd, i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double s = i < n ? (double)((const T*)a.bt)[i] : 0.0;
  s = block_sum(s);
  if (threadIdx.x == 0) a.part[blockIdx.x] = s;
}

template <typename T>
__global__ void __launch_bounds__(256) k_fold1(FixArgs a, int nb) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using V = V2<T>;
  double s = fold_partials(a.part, nb);
  if (threadIdx.x == 0) {
    for (int k = 0; k < a.nd; k++) s += (double)((const V*)a.bt_spec)[k].x;  // mode (0,0) of every level
    double* sc = a.sc;
    const double mps_p = sc[SC_MPS_P], corr = sc[SC_CORR];
    sc[SC_EP_BAR] = sc[SC_MPSP_BAR] = sc[SC_EN_BAR] = sc[SC_MN_BAR] = 0.0;
    if (a.do_energy) {
      const double f = a.grav / (a.cp * mps_p);
      sc[SC_EN_BAR] = -f * s;
      sc[SC_EP_BAR] = f * s;
      sc[SC_MPSP_BAR] = -corr / mps_p * s;
    }
  }
}

// energy fixer reversed: en_n = |u_n|^2/2 + cp T_n weighted by dp(ps_n2).  Block = 32 consecutive
// columns of one latitude row x 8 level groups (warp g takes levels g, g+8, ...: every read and write
// a coalesced row), arithmetic in the state precision with the layer coefficients staged per block;
// the column sums fold over the level groups in a fixed order; block partials of ps_n2_bar ps_n in
// FP64.
template <typename T>
__global__ void __launch_bounds__(256) k_fix2(FixArgs a) {
  using R = T;
  constexpr int KS = 8;
  __shared__ R s_dak[JGCM_MAX_ND], s_dbk[JGCM_MAX_ND], s_acc[KS][32];
  for (int q = threadIdx.x; q < a.nd; q += blockDim.x) {
    s_dak[q] = (R)a.vc->dak[q];
    s_dbk[q] = (R)a.vc->dbk[q];
  }
  __syncthreads();
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  const int G = a.nlat * a.nlon, lane = threadIdx.x & 31, ks = threadIdx.x >> 5, j = blockIdx.y;
  const int i = blockIdx.x * 32 + lane;
  const bool act = i < a.nlon;
  const int c = j * a.nlon + (act ? i : 0);
  const R factor = (R)a.sc[SC_FACTOR], corr = (R)a.sc[SC_CORR], En_bar = (R)a.sc[SC_EN_BAR];
  const R Wc = (R)(a.wts[j] * a.inv_2n), cp = pick<R>(a.cp, a.cpf), ig = pick<R>(a.ig, a.igf);
  const R ps2 = act ? (R)((const T*)a.ps_n2)[c] : (R)0;
  R acc = 0;
  if (act && a.do_energy) {
#pragma unroll 4  // nd <= 32: every level's loads in flight together
    for (int k = ks; k < a.nd; k += KS) {
      const size_t x = c + (size_t)G * k;
      const R u = ((const T*)a.u_n)[x], v = ((const T*)a.v_n)[x], t = ((const T*)a.t_n2)[x] - corr;
      const R dbk = s_dbk[k];
      const R en = (R)0.5 * (u * u + v * v) + cp * t;
      const R eb = En_bar * Wc * (s_dak[k] + dbk * ps2) * ig;
      ((T*)a.bu)[x] = ((T*)a.bu)[x] + eb * u;
      ((T*)a.bv)[x] = ((T*)a.bv)[x] + eb * v;
      ((T*)a.bt)[x] = ((T*)a.bt)[x] + cp * eb;
      acc += en * dbk;
    }
  }
  s_acc[ks][lane] = acc;
  __syncthreads();
  double s = 0.0;
  if (ks == 0 && act) {
    R tot = 0;
    for (int q = 0; q < KS; q++) tot += s_acc[q][lane];
    R bps = ((T*)a.bps)[c];
    if (a.do_energy) {
      bps += En_bar * Wc * ig * tot;
      ((T*)a.bps)[c] = bps;
    }
    s = (double)bps * ((double)ps2 / (double)factor);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) a.part[blockIdx.y * gridDim.x + blockIdx.x] = s;
}

template <typename T>
__global__ void __launch_bounds__(256) k_fold2(FixArgs a, int nb) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using V = V2<T>;
  double s = fold_partials(a.part, nb);
  if (threadIdx.x == 0) {
    double* sc = a.sc;
    sc[SC_MN_BAR] = 0.0;
    if (a.do_mass) {
      const double factor = sc[SC_FACTOR], mps_n = sc[SC_MPS_P] / factor;
      const double fb = s + (double)((const V*)a.bl_spec)[0].x / factor;
      sc[SC_MPSP_BAR] += fb / mps_n;
      sc[SC_MN_BAR] = -fb * factor / mps_n;
    }
  }
}

// mass fixer reversed and exp(ln ps); u, v cotangents divided by cos (inputs of S2G^T of ucos,
// vcos); one thread per grid point
template <typename T>
__global__ void __launch_bounds__(256) k_fix3(FixArgs a) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  const int G = a.nlat * a.nlon;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)G * a.nd) return;
  const int c = (int)(i % G), j = c / a.nlon;
  const T cj = ((const T*)a.cosj)[j];
  ((T*)a.g_uc)[i] = ((const T*)a.bu)[i] / cj;
  ((T*)a.g_vc)[i] = ((const T*)a.bv)[i] / cj;
  if (i < (size_t)G) {
    const double factor = a.sc[SC_FACTOR];
    const double ps_n = (double)((const T*)a.ps_n2)[c] / factor;
    double bps = (double)((const T*)a.bps)[c];
    if (a.do_mass) bps = bps * factor + a.sc[SC_MN_BAR] * a.wts[j] * a.inv_2n;
    ((T*)a.g_lnps)[c] = (T)(bps * ps_n);
  }
}

// ---- spectral pieces ----------------------------------------------------------------------------
// cotangents of the new level: direct + S2G^T parts, and UV_Grid_From_Vor_Div! transposed (the
// ucos/vcos recurrence of Spectral_Spherical_Mesh.jl:517-580 read backwards)
template <typename T>
struct NbarArgs {
  const V2<T>*in_vor, *in_div, *in_t, *in_l;             // cotangents of X_{s+1} spe_*_c
  const V2<T>*a_vor, *a_div, *a_t, *a_l, *a_uc, *a_vc;   // S2G^T results
  V2<T>*nb_vor, *nb_div, *nb_t, *nb_l;
  int N, ns, nd;
};

template <typename T>
__global__ void __launch_bounds__(256) k_nbar(NbarArgs<T> a, Tables<T> tb) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using V = V2<T>;
  const size_t total = (size_t)(a.N + 1) * (a.ns + 1) * a.nd;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const int k = (int)(idx % a.nd);
  const size_t mn = idx / a.nd;
  const int m = (int)(mn / (a.ns + 1)), n = (int)(mn % (a.ns + 1));
  const size_t row = (size_t)m * (a.ns + 1);
  V z;
  z.x = z.y = 0;
  if (n < m) {
    a.nb_vor[idx] = z;
    a.nb_div[idx] = z;
    a.nb_t[idx] = z;
    if (k == 0) a.nb_l[mn] = z;
    return;
  }
  V vor = a.in_vor[idx], dv = a.in_div[idx];
  V av = a.a_vor[idx], ad = a.a_div[idx];
  vor.x += av.x;
  vor.y += av.y;
  dv.x += ad.x;
  dv.y += ad.y;
  const T c0 = tb.uvc[row + n];
  const V au = a.a_uc[idx], aw = a.a_vc[idx];
  dv.x += c0 * au.y;  // ucos = uvc (i div) + ...
  dv.y -= c0 * au.x;
  vor.x += c0 * aw.y;  // vcos = uvc (i vor) + ...
  vor.y -= c0 * aw.x;
  if (n + 1 <= a.ns) {  // row n+1 read vor_n / div_n through uvm_{n+1}
    const T cm = tb.uvm[row + n + 1];
    const V u1 = a.a_uc[idx + a.nd], w1 = a.a_vc[idx + a.nd];
    vor.x -= cm * u1.x;
    vor.y -= cm * u1.y;
    dv.x += cm * w1.x;
    dv.y += cm * w1.y;
  }
  if (n - 1 >= m) {  // row n-1 read them through uvp_{n-1}
    const T cp = tb.uvp[row + n - 1];
    const V u1 = a.a_uc[idx - a.nd], w1 = a.a_vc[idx - a.nd];
    vor.x -= cp * u1.x;
    vor.y -= cp * u1.y;
    dv.x += cp * w1.x;
    dv.y += cp * w1.y;
  }
  a.nb_vor[idx] = vor;
  a.nb_div[idx] = dv;
  V t = a.in_t[idx], at = a.a_t[idx];
  t.x += at.x;
  t.y += at.y;
  a.nb_t[idx] = t;
  if (k == 0) {
    V l = a.in_l[mn], al = a.a_l[mn];
    l.x += al.x;
    l.y += al.y;
    a.nb_l[mn] = l;
  }
}

// E = -eig ddiv_bar (the -Laplacian of the energy analysis, transposed)
template <typename T>
__global__ void k_neg_lap(const V2<T>* __restrict__ in, V2<T>* __restrict__ out, Tables<T> tb, int N, int ns, int L) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  const size_t total = (size_t)(N + 1) * (ns + 1) * L;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const T e = -tb.eig[idx / L];
  V2<T> v = in[idx];
  v.x *= e;
  v.y *= e;
  out[idx] = v;
}

// Compute_Gradient_Cos! (:655-692) transposed: out += DLAM^T sl + DTH^T st (n >= m)
template <typename T>
__global__ void k_grad_adjoint(const V2<T>* __restrict__ sl, const V2<T>* __restrict__ stt, V2<T>* __restrict__ out,
                               Tables<T> tb, int N, int ns, int L) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using V = V2<T>;
  const size_t total = (size_t)(N + 1) * (ns + 1) * L;
  const size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= total) return;
  const size_t mn = idx / L;
  const int m = (int)(mn / (ns + 1)), n = (int)(mn % (ns + 1));
  if (n < m) return;
  const size_t row = (size_t)m * (ns + 1);
  const T cl = tb.dlam[row + n];
  const V x = sl[idx];
  V h = out[idx];
  h.x += cl * x.y;  // dl = coef_dlam (i h)
  h.y -= cl * x.x;
  if (n - 1 >= m) {  // row n-1 read h_n through dthp_{n-1}
    const T cp = tb.dthp[row + n - 1];
    const V y = stt[idx - L];
    h.x += cp * y.x;
    h.y += cp * y.y;
  }
  if (n + 1 <= ns) {  // row n+1 read h_n through dthm_{n+1}
    const T cm = tb.dthm[row + n + 1];
    const V y = stt[idx + L];
    h.x += cm * y.x;
    h.y += cm * y.y;
  }
  out[idx] = h;
}

// Vor_Div_From_Grid_UV!'s alpha operators (Compute_Alpha_Operator!, :424-459) transposed, as a
// synthesis: vor = i CA F(v cos) - CB F(u cos), div = i CA F(u cos) + CB F(v cos) over n = m..N,
// so F_bar(u cos) = -i CA div_bar - CB vor_bar and F_bar(v cos) = -i CA vor_bar + CB div_bar, summed
// over n with CA(-mu) = (-1)^(n-m) CA(mu), CB(-mu) = -(-1)^(n-m) CB(mu).  The inverse FFT that
// follows weights m >= 1 twice and the grid cotangent of fft/nlon is (1/nlon) sum_m Re(F_bar e^{im
// lam}), so the coefficients are stored x cos_j / (c_m nlon) (c_0 = 1, c_m = 2): the grid result is
// then the cotangent of u and v themselves.  Fourier columns [0, nd) u, [nd, 2 nd) v.
// grid (ceil(nh*nd/256), N+1), 256 threads: one (latitude pair, level) per thread.
template <typename T>
__global__ void __launch_bounds__(256) k_alpha_adjoint(const V2<T>* __restrict__ bvor, const V2<T>* __restrict__ bdiv,
                                                       V2<T>* __restrict__ F, Tables<T> tb, int N, int ns, int nlat,
                                                       int nlon, int nd) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using V = V2<T>;
  const int m = blockIdx.y, nh = nlat >> 1;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nh * nd) return;
  const int k = i % nd, jh = i / nd;
  const size_t row = (size_t)m * (ns + 1);
  // even / odd (n - m) partial sums of the CA terms and of the CB terms, u and v
  T uae[2] = {0, 0}, uao[2] = {0, 0}, ube[2] = {0, 0}, ubo[2] = {0, 0};
  T vae[2] = {0, 0}, vao[2] = {0, 0}, vbe[2] = {0, 0}, vbo[2] = {0, 0};
  for (int n = m; n <= ns - 1; n++) {
    const T ca = tb.CA[(row + n) * nh + jh], cb = tb.CB[(row + n) * nh + jh];
    const V vb = bvor[(row + n) * nd + k], db = bdiv[(row + n) * nd + k];
    const bool odd = (n - m) & 1;
    T* ua = odd ? uao : uae;
    T* ub = odd ? ubo : ube;
    T* va = odd ? vao : vae;
    T* vbb = odd ? vbo : vbe;
    ua[0] += ca * db.y;  // -i CA div_bar
    ua[1] -= ca * db.x;
    ub[0] -= cb * vb.x;  // -CB vor_bar
    ub[1] -= cb * vb.y;
    va[0] += ca * vb.y;  // -i CA vor_bar
    va[1] -= ca * vb.x;
    vbb[0] += cb * db.x;  // +CB div_bar
    vbb[1] += cb * db.y;
  }
  const T sc = tb.cosj[jh] / ((m == 0 ? (T)1 : (T)2) * (T)nlon);  // exact in T: no FP64 per thread
  const int C = 2 * nd;
  const int jn = nlat - 1 - jh;
  V us, un, vs, vn;
  us.x = (uae[0] + uao[0] + ube[0] + ubo[0]) * sc;
  us.y = (uae[1] + uao[1] + ube[1] + ubo[1]) * sc;
  un.x = (uae[0] - uao[0] - ube[0] + ubo[0]) * sc;
  un.y = (uae[1] - uao[1] - ube[1] + ubo[1]) * sc;
  vs.x = (vae[0] + vao[0] + vbe[0] + vbo[0]) * sc;
  vs.y = (vae[1] + vao[1] + vbe[1] + vbo[1]) * sc;
  vn.x = (vae[0] - vao[0] - vbe[0] + vbo[0]) * sc;
  vn.y = (vae[1] - vao[1] - vbe[1] + vbo[1]) * sc;
  F[((size_t)m * nlat + jh) * C + k] = us;
  F[((size_t)m * nlat + jn) * C + k] = un;
  F[((size_t)m * nlat + jh) * C + nd + k] = vs;
  F[((size_t)m * nlat + jn) * C + nd + k] = vn;
}

// ---- the column kernel --------------------------------------------------------------------------
// Arithmetic in the state precision R = T (the mixed path's FP32 column, as its forward column
// kernel; FP64 on the FP64 path); per-column sums of the parameter cotangents go to FP64 block
// partials.  Divisions by constants are host-side reciprocals, and T_eq's power and logarithm come
// from one ln ps per column: ln(p_k / p0) = cf_k + ln ps - ln p0, (p_k/p0)^kappa = exp(kappa ln).
template <typename T>
struct ColAdjArgs {
  const T *u, *v, *t, *vor, *div, *up, *vp, *tp, *ps, *psp;  // X_s
  const T *gl, *gt, *tl, *tt;                                // grad ln ps, grad T (Compute_Gradients!)
  const T *DU, *DV, *DT, *EN, *DLN;                          // cotangents of du, dv, dT, energy, dlnps
  const T *seed_u, *seed_v, *seed_t, *seed_ps;               // cotangents of X_{s+1} grid_*_p
  T *bu, *bv, *bt, *bps, *bup, *bvp, *btp, *bpsp, *bvor, *bdiv;  // cotangents of X_s
  T *btl, *btt, *bgl, *bgt;                                  // cotangents of the gradients, / cos
  const T *coriolis, *sinj, *cosj;
  const double* wts;
  const double* sc;
  double* ppart;  // [5][nblocks]
  int nd, nlat, nlon, Dt;
  // HS_Forcing.jl constants (per second): k_v = kvc max(0, sigma - sigma_b),
  // k_t = ka + ktc max(0, sigma - sigma_b) cos^4
  double sigma_b, kvc, ka, ktc, inv_1msb, inv_day, dT_y, dtheta_z, kappa, ln_p0;
  double rdgas, cp, inv_cp, inv_grav;
  double inv_2n;  // 1 / (2 nlon), exact (nlon is a power of two)
  // the same constants rounded to T on the host (an FP64 -> FP32 conversion per thread would run on
  // the FP64 pipe)
  T sigma_b_t, kvc_t, ka_t, ktc_t, inv_1msb_t, inv_day_t, dT_y_t, dtheta_z_t, kappa_t, ln_p0_t;
  T rdgas_t, cp_t, inv_cp_t, inv_grav_t;
};

template <typename T>
void col_adj_consts(ColAdjArgs<T>& a) {
  a.sigma_b_t = (T)a.sigma_b; a.kvc_t = (T)a.kvc; a.ka_t = (T)a.ka; a.ktc_t = (T)a.ktc;
  a.inv_1msb_t = (T)a.inv_1msb; a.inv_day_t = (T)a.inv_day; a.dT_y_t = (T)a.dT_y;
  a.dtheta_z_t = (T)a.dtheta_z; a.kappa_t = (T)a.kappa; a.ln_p0_t = (T)a.ln_p0;
  a.rdgas_t = (T)a.rdgas; a.cp_t = (T)a.cp; a.inv_cp_t = (T)a.inv_cp; a.inv_grav_t = (T)a.inv_grav;
  a.inv_2n = 0.5 / a.nlon;
}

template <typename R>
__device__ __forceinline__ R up1(R x, int lane) {  // value of lane - 1 (0 for lane 0)
  R y = __shfl_up_sync(FULL, x, 1);
  return lane == 0 ? (R)0 : y;
}
template <typename R>
__device__ __forceinline__ R dn1(R x, int lane) {  // value of lane + 1 (0 for lane 31)
  R y = __shfl_down_sync(FULL, x, 1);
  return lane == 31 ? (R)0 : y;
}
template <typename R>
__device__ __forceinline__ R wsum(R x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
  return x;
}
template <typename R>
__device__ __forceinline__ R scan_excl(R x, int lane) {  // sum over lanes < lane
  R s = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    R y = __shfl_up_sync(FULL, s, o);
    if (lane >= o) s += y;
  }
  return s - x;
}
template <typename R>
__device__ __forceinline__ R rscan_excl(R x, int lane) {  // sum over lanes > lane
  R s = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    R y = __shfl_down_sync(FULL, s, o);
    if (lane + o < 32) s += y;
  }
  return s - x;
}

template <typename T>
__global__ void __launch_bounds__(256) k_hs_column_adjoint(ColAdjArgs<T> a, const VertCoef* __restrict__ vcp) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using R = T;
  __shared__ double pw[8][5];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int G = a.nlat * a.nlon, nd = a.nd;
  const int col = blockIdx.x * 8 + wid;
  const bool colv = col < G;
  const int k = lane;
  const bool act = colv && k < nd;
  const VertCoef& vc = *vcp;
  const int j = colv ? col / a.nlon : 0;
  const size_t x = (size_t)(colv ? col : 0) + (size_t)G * (act ? k : 0);
  auto ld = [&](const T* p) -> R { return act ? (R)p[x] : (R)0; };
  const R u = ld(a.u), v = ld(a.v), t = ld(a.t), vor = ld(a.vor), div = ld(a.div);
  const R tl = ld(a.tl), tt = ld(a.tt), up = ld(a.up), vp = ld(a.vp), tp = ld(a.tp);
  const R DU = ld(a.DU), DV = ld(a.DV), DT = ld(a.DT), EN = ld(a.EN);
  const size_t c1 = colv ? col : 0;
  const R ps = a.ps[c1], psp = a.psp[c1], gl = a.gl[c1], gt = a.gt[c1];
  const R DLN = colv ? (R)a.DLN[c1] : (R)0;
  const R Rg = (R)a.rdgas_t, kap = (R)a.kappa_t;
  // vertical constants; lanes >= nd carry zeros (dbk = 1 keeps the divisions finite)
  const R bk = act ? (R)vc.bk[k] : (R)0, bk1 = act ? (R)vc.bk[k + 1] : (R)0, dbk = act ? (R)vc.dbk[k] : (R)1;
  const R rdbk = (R)1 / dbk;
  const R dlp_p = act ? (R)vc.dlp_p[k] : (R)0, dlp_m = (act && k >= 1) ? (R)vc.dlp_m[k] : (R)0;
  const R dlp = (act && k >= 1) ? (R)vc.dlp[k] : (R)0, sf = act ? (R)vc.sf[k] : (R)1;
  const R cf = act ? (R)vc.cf[k] : (R)0;
  const R X1 = (bk * dlp_m + bk1 * dlp_p) * rdbk;  // x1 ps (Four_In_One!)
  // ---- forward of the column: Four_In_One! with the mass fluxes scaled by 1/ps ----
  const R gu = u * gl + v * gt;
  const R q = act ? dbk * (div + gu) : (R)0;  // dmean / ps
  const R Tex = scan_excl(q, lane);           // dmean_tot before level k, / ps
  const R Ttot = wsum(q);
  const R x5 = -(Tex * dlp + q * dlp_p) * rdbk + X1 * gu;
  const R Mt = (act && k >= 1) ? (-Tex + Ttot * bk) : (R)0;  // M_half[k] / ps (k = 1..nd-1)
  const R Mn = dn1(Mt, lane);                                 // every lane takes part in the shuffle
  const R Mb = (k + 1 < nd) ? Mn : (R)0;                      // M_half[k+1] / ps
  const R dbk_m1 = up1(dbk, lane);
  const R al = (act && k >= 1) ? dbk_m1 / (dbk_m1 + dbk) : (R)0;
  // ---- cotangents ----
  R bu = act ? (R)a.seed_u[x] : (R)0, bv = act ? (R)a.seed_v[x] : (R)0;
  R bt = act ? (R)a.seed_t[x] : (R)0;
  // absolute-vorticity fluxes: du += (vor + f) v, dv -= (vor + f) u
  const R av = vor + (R)a.coriolis[j];
  const R bvor = DU * v - DV * u;
  bv += DU * av;
  bu -= DV * av;
  // horizontal advection of T: dT -= u dT/dlam + v dT/dth
  bu -= DT * tl;
  bv -= DT * tt;
  const R btl = -DT * u, btt = -DT * v;
  // vertical advection (Vert_Advection!, dz = dp = dbk ps, w = M_half): flux_k = w_k r_int_k
  R Mbar = 0;
  auto vadv = [&](R r, R Rb, R& rb) {
    const R r_m1 = up1(r, lane);
    const R rint = (k >= 1) ? r_m1 + (r - r_m1) * al : (R)0;
    const R qq = Rb * rdbk;
    const R qq_m1 = up1(qq, lane);
    const R fb = (act && k >= 1) ? qq - qq_m1 : (R)0;  // flux_k enters rdt_k (+) and rdt_{k-1} (-)
    rb += qq * (Mb - Mt);
    Mbar += -qq * r + ((k >= 1) ? qq_m1 * r_m1 : (R)0);
    Mbar += fb * rint;
    rb += fb * Mt * al;
    rb += dn1(fb * Mt * ((R)1 - al), lane);  // r_{k-1} share of flux_k, from lane k + 1's view
  };
  vadv(u, DU, bu);
  vadv(v, DV, bv);
  vadv(t, DT, bt);
  // dlnps = dps / ps = -dmean_tot / ps
  R Tbar_tot = -DLN;
  // energy = geopotential + |u|^2 / 2: Phi_k = R (t_k dlp_p_k + sum_{l > k} t_l dlp_l)
  bu += EN * u;
  bv += EN * v;
  bt += Rg * (EN * dlp_p + dlp * scan_excl(EN, lane));
  // Four_In_One! reversed: M_half[k] = -tot_k + tot_nd b_k
  R Tbar = (act && k >= 1) ? -Mbar : (R)0;
  Tbar_tot += wsum((act && k >= 1) ? Mbar * bk : (R)0);
  bt += kap * x5 * DT;
  const R bx5 = kap * t * DT;
  if (k >= 1) Tbar -= bx5 * dlp * rdbk;
  R qbar = -bx5 * dlp_p * rdbk;
  R gub = bx5 * X1;
  bt -= Rg * X1 * (gl * DU + gt * DV);
  R glb = -Rg * t * X1 * DU, gtb = -Rg * t * X1 * DV;
  qbar += rscan_excl(act ? Tbar : (R)0, lane) + Tbar_tot;  // tot_k = sum_{l < k} dmean_l
  const R bdiv = qbar * dbk;
  gub += qbar * dbk;
  bu += gub * gl;
  bv += gub * gt;
  glb += gub * u;
  gtb += gub * v;
  // ---- HS_Forcing! of the p level and the energy integral of Compute_Corrections_Init ----
  const R t_zero = 315, t_strat = 200, sb = (R)a.sigma_b_t;
  const R sj = a.sinj[j], s2 = sj * sj, c2 = (R)1 - s2, c4 = c2 * c2;
  const R Ep_bar = (R)a.sc[SC_EP_BAR], Wc = (R)(a.wts[j] * a.inv_2n);
  const R Dt = (R)a.Dt, icp = (R)a.inv_cp_t, ig = (R)a.inv_grav_t;
  const R lps = log(ps) - (R)a.ln_p0_t;  // one logarithm per column
  R bup = 0, bvp = 0, btp = 0, bps_l = 0, bpsp_l = 0;
  R pb0 = 0, pb1 = 0, pb2 = 0, pb3 = 0, pb4 = 0;
  if (act) {
    const R s = sf - sb, sp = s > (R)0 ? s : (R)0;  // sigma = p_k / ps
    const R kv = (R)a.kvc_t * sp;
    const R duf = -kv * up, dvf = -kv * vp;
    const R lpn = cf + lps;                  // ln(p_k / p0)
    const R pk = exp(kap * lpn);             // (p_k / p0)^kappa
    const R pn = sf * ps * (R)1.0e-5;        // p_k / p0
    const R tpot = t_zero - (R)a.dT_y_t * s2 - (R)a.dtheta_z_t * c2 * lpn;
    const R te = tpot * pk;
    const R teq = te > t_strat ? te : t_strat;
    const R kt = (R)a.ka_t + (R)a.ktc_t * sp * c4;
    const R fr = -((up + (R)0.5 * duf * Dt) * duf + (vp + (R)0.5 * dvf * Dt) * dvf) * icp;
    const R dTf = fr - kt * (tp - teq);
    const R aa = up + Dt * duf, bb = vp + Dt * dvf;
    const R enp = (R)0.5 * (aa * aa + bb * bb) + (R)a.cp_t * (tp + Dt * dTf);
    bpsp_l = Ep_bar * Wc * ig * enp * dbk;
    const R eb = Ep_bar * Wc * ((R)vc.dak[k] + dbk * psp) * ig;
    const R ba = eb * aa, bbv = eb * bb;
    btp += (R)a.cp_t * eb;
    R bdTf = DT + (R)a.cp_t * Dt * eb;
    R bduf = DU + Dt * ba;
    R bdvf = DV + Dt * bbv;
    bup += ba;
    bvp += bbv;
    const R bkt = -bdTf * (tp - teq);
    btp -= kt * bdTf;
    const R bteq = kt * bdTf;
    bduf -= bdTf * (up + duf * Dt) * icp;
    bup -= bdTf * duf * icp;
    bdvf -= bdTf * (vp + dvf * Dt) * icp;
    bvp -= bdTf * dvf * icp;
    const R bkv = -bduf * up - bdvf * vp;
    bup -= kv * bduf;
    bvp -= kv * bdvf;
    const R spn = sp * (R)a.inv_1msb_t;
    pb0 = bkv * spn * (R)a.inv_day_t;
    pb1 = bkt * ((R)1 - spn * c4) * (R)a.inv_day_t;
    pb2 = bkt * spn * c4 * (R)a.inv_day_t;
    const R bte = te > t_strat ? bteq : (R)0;
    pb3 = -s2 * pk * bte;
    pb4 = -c2 * lpn * pk * bte;
    // d te / d pn = (pk / pn) (kappa tpot - dtheta_z cos^2); pn = sf ps / p0
    const R dte = pk / pn * (kap * tpot - (R)a.dtheta_z_t * c2);
    bps_l = bte * dte * sf * (R)1.0e-5;
  }
  const R glb_c = wsum(act ? glb : (R)0), gtb_c = wsum(act ? gtb : (R)0);
  const R bps_c = wsum(bps_l), bpsp_c = wsum(bpsp_l);
  const R p0 = wsum(pb0), p1 = wsum(pb1), p2 = wsum(pb2), p3 = wsum(pb3), p4 = wsum(pb4);
  if (act) {
    const R rc = (R)1 / (R)a.cosj[j];
    a.bu[x] = (T)bu;
    a.bv[x] = (T)bv;
    a.bt[x] = (T)bt;
    a.bup[x] = (T)bup;
    a.bvp[x] = (T)bvp;
    a.btp[x] = (T)btp;
    a.bvor[x] = (T)bvor;
    a.bdiv[x] = (T)bdiv;
    a.btl[x] = (T)(btl * rc);
    a.btt[x] = (T)(btt * rc);
  }
  if (colv && lane == 0) {
    const R rc = (R)1 / (R)a.cosj[j];
    a.bps[col] = (T)((R)a.seed_ps[col] + bps_c);
    a.bpsp[col] = (T)(bpsp_c + (R)a.sc[SC_MPSP_BAR] * Wc);
    a.bgl[col] = (T)(glb_c * rc);
    a.bgt[col] = (T)(gtb_c * rc);
  }
  if (lane == 0) {
    pw[wid][0] = colv ? (double)p0 : 0.0;
    pw[wid][1] = colv ? (double)p1 : 0.0;
    pw[wid][2] = colv ? (double)p2 : 0.0;
    pw[wid][3] = colv ? (double)p3 : 0.0;
    pw[wid][4] = colv ? (double)p4 : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < 5) {
    double sum = 0.0;
    for (int w = 0; w < 8; w++) sum += pw[w][threadIdx.x];
    a.ppart[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = sum;
  }
}

// one block per parameter
__global__ void k_fold_params(const double* __restrict__ part, int nb, double* __restrict__ pbar) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  const int v = blockIdx.x;
  double s = fold_partials(part + (size_t)v * nb, nb);
  if (threadIdx.x == 0) pbar[v] += s;
}

// loss = sum w_j (T - T_target)^2 / (2 nlon nd) and its grid cotangent
template <typename T>
__global__ void __launch_bounds__(256) k_loss(const T* __restrict__ t, const double* __restrict__ tgt, T* __restrict__ bar,
                                              const double* __restrict__ wts, int nlat, int nlon, int nd,
                                              double* __restrict__ part) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  const size_t n = (size_t)nlat * nlon * nd;
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double s = 0.0;
  if (i < n) {
    const int j = (int)((i / nlon) % nlat);
    const double norm = 2.0 * nlon * nd;
    const double d = (double)t[i] - tgt[i];
    s = wts[j] * d * d / norm;
    bar[i] = (T)(2.0 * wts[j] * d / norm);
  }
  s = block_sum(s);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_fold_scalar(const double* __restrict__ part, int nb, double* __restrict__ out) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  double s = fold_partials(part, nb);
  if (threadIdx.x == 0) *out = s;
}

template <typename T>
__global__ void k_add2(const T* __restrict__ a, const T* __restrict__ b, T* __restrict__ out, size_t n) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = a[i] + b[i];
}

// ---- workspace --------------------------------------------------------------------------------
struct AdjWork {
  void* base;
  // grid (T): lnps bar, u/cos, v/cos, du, dv, dT, energy, dlnps, gl, gt, tl, tt
  void *g_l, *g_uc, *g_vc, *g_du, *g_dv, *g_dT, *g_en, *g_dln, *g_gl, *g_gt, *g_tl, *g_tt;
  // grid (T): the gradients of ln ps and T of X_s (forward values: Compute_Gradients!)
  void *x_gl, *x_gt, *x_tl, *x_tt;
  // spectral (T2): S2G^T results, new-level cotangents, tendency cotangents, E, gradient S2G^T
  void *a_l, *a_t, *a_vor, *a_div, *a_uc, *a_vc, *nb_vor, *nb_div, *nb_t, *nb_l;
  void *b_dvor, *b_ddiv, *b_dt, *b_dl, *e_spec, *s_gl, *s_gt, *s_tl, *s_tt;
  double* mats;  // transposed vertical operators of the semi-implicit step
  double* sc;    // scalars
  double* part;  // block partials
  double* ppart; // parameter partials [5][nblocks]
  double* pbar;  // parameter cotangents (accumulated)
  int nb_col, nb_adj;
};

int work_alloc(jgcm_model* md, AdjWork* w) {
  jgcm_mesh* m = md->mesh;
  const int nd = md->nd;
  const size_t ts = tsize(m), G1 = grid_elems(m, 1) * ts, GL = grid_elems(m, nd) * ts;
  const size_t S1 = spec_elems(m, 1) * 2 * ts, SL = spec_elems(m, nd) * 2 * ts;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const int G = m->nlat * m->nlon;
  w->nb_col = (int)((grid_elems(m, nd) + 255) / 256);  // block partials: a thread per grid point
  w->nb_adj = (G + 7) / 8;      // one warp per column
  const size_t gtot = 6 * al(G1) + 10 * al(GL);
  const size_t stot = 4 * al(S1) + 15 * al(SL);
  const size_t dtot = al(SC_N * 8) + al((size_t)(std::max(w->nb_col, w->nb_adj) + 8) * 8) +
                      al((size_t)5 * w->nb_adj * 8) + al(5 * 8);
  JG_TRY(dev_alloc(&w->base, gtot + stot + dtot));
  char* p = (char*)w->base;
  auto take = [&](size_t b) {
    void* r = p;
    p += al(b);
    return r;
  };
  w->g_l = take(G1);
  w->g_dln = take(G1);
  w->g_gl = take(G1);
  w->g_gt = take(G1);
  w->g_uc = take(GL);
  w->g_vc = take(GL);
  w->g_du = take(GL);
  w->g_dv = take(GL);
  w->g_dT = take(GL);
  w->g_en = take(GL);
  w->g_tl = take(GL);
  w->g_tt = take(GL);
  w->x_gl = take(G1);
  w->x_gt = take(G1);
  w->x_tl = take(GL);
  w->x_tt = take(GL);
  w->a_l = take(S1);
  w->nb_l = take(S1);
  w->b_dl = take(S1);
  w->s_gl = take(S1);
  w->a_t = take(SL);
  w->a_vor = take(SL);
  w->a_div = take(SL);
  w->a_uc = take(SL);
  w->a_vc = take(SL);
  w->nb_vor = take(SL);
  w->nb_div = take(SL);
  w->nb_t = take(SL);
  w->b_dvor = take(SL);
  w->b_ddiv = take(SL);
  w->b_dt = take(SL);
  w->e_spec = take(SL);
  w->s_gt = take(S1 > SL ? S1 : SL);  // one level used
  w->s_tl = take(SL);
  w->s_tt = take(SL);
  w->sc = (double*)take(SC_N * 8);
  w->part = (double*)take((size_t)(std::max(w->nb_col, w->nb_adj) + 8) * 8);
  w->ppart = (double*)take((size_t)5 * w->nb_adj * 8);
  w->pbar = (double*)take(5 * 8);
  JG_TRY(si_adjoint_mats(md, &w->mats));
  return JGCM_OK;
}

void work_free(AdjWork* w) {
  cudaFree(w->base);
  cudaFree(w->mats);
}

GridInGroup gin(const void* src, int L, int col0) {
  GridInGroup g;
  memset(&g, 0, sizeof(g));
  g.src = src;
  g.pro = PRO_NONE;
  g.L = L;
  g.col0 = col0;
  return g;
}
SpecOutGroup sadj(void* dst, int L, int col0, double nlon) {  // S2G^T output group
  SpecOutGroup g;
  memset(&g, 0, sizeof(g));
  g.dst = dst;
  g.op = G2S_ADJ_S2G;
  g.L = L;
  g.col0 = col0;
  g.scale = nlon;
  g.colA = col0;
  g.colB = g.colE = g.colH = -1;
  return g;
}
S2GGroup sin_adj(const void* a, int L, int col0) {  // G2S^T input group
  S2GGroup g;
  memset(&g, 0, sizeof(g));
  g.a = a;
  g.op = S2G_ADJ_G2S;
  g.L = L;
  g.col0 = col0;
  return g;
}
GridOutGroup gout(int epi, void* dst, int L, int col0) {
  GridOutGroup g;
  memset(&g, 0, sizeof(g));
  g.dst = dst;
  g.epi = epi;
  g.L = L;
  g.col0 = col0;
  return g;
}

// One adjoint step.  x0 is X_s (init: the step's init flag, Δt or 2Δt), x1 is X_{s+1}; w->sc holds
// the step's forward scalars; xin holds the cotangents of X_{s+1} (its grid u_c, v_c, t_c, ps_c are
// updated in place), xout receives those of X_s; w->pbar accumulates.  Reads no model state slot,
// so a step is capturable once per (segment slot, buffer parity) and replayed.
template <typename T>
int adjoint_step(jgcm_model* md, AdjWork* w, const StateBuf* x0, const StateBuf* x1, StateBuf* xin, StateBuf* xout,
                 int init) {
  using V = V2<T>;
  jgcm_mesh* m = md->mesh;
  cudaStream_t st = m->stream;
  const int nd = md->nd, N = m->N, ns = m->ns, nlat = m->nlat, nlon = m->nlon, G = nlat * nlon;
  Tables<T> tb = tables<T>(m);
  // 1. fixers reversed
  FixArgs fa;
  memset(&fa, 0, sizeof(fa));
  fa.u_n = x1->f[8];
  fa.v_n = x1->f[10];
  fa.t_n2 = x1->f[14];
  fa.ps_n2 = x1->f[12];
  fa.bu = xin->f[8];
  fa.bv = xin->f[10];
  fa.bt = xin->f[14];
  fa.bps = xin->f[12];
  fa.bt_spec = xin->f[6];
  fa.bl_spec = xin->f[4];
  fa.g_lnps = w->g_l;
  fa.g_uc = w->g_uc;
  fa.g_vc = w->g_vc;
  fa.wts = m->d_wts;
  fa.cosj = tb.cosj;
  fa.sc = w->sc;
  fa.part = w->part;
  fa.vc = md->d_vc;
  fa.nd = nd;
  fa.nlat = nlat;
  fa.nlon = nlon;
  fa.do_mass = md->P.do_mass_correction;
  fa.do_energy = md->P.do_energy_correction;
  fa.cp = md->cp_air;
  fa.grav = md->P.grav;
  fa.inv_2n = 0.5 / nlon;
  fa.ig = 1.0 / md->P.grav;
  fa.cpf = (float)md->cp_air;
  fa.igf = (float)(1.0 / md->P.grav);
  const int nbp = (int)((grid_elems(m, nd) + 255) / 256);  // a thread per grid point
  const dim3 gf2((nlon + 31) / 32, nlat);                   // 32 columns x 8 level groups
  JG_CUDA(launch_pdl(k_fix1<T>, nbp, 256, 0, st, fa));
  JG_CUDA(launch_pdl(k_fold1<T>, 1, 256, 0, st, fa, nbp));
  JG_CUDA(launch_pdl(k_fix2<T>, gf2, 256, 0, st, fa));
  JG_CUDA(launch_pdl(k_fold2<T>, 1, 256, 0, st, fa, (int)(gf2.x * gf2.y)));
  JG_CUDA(launch_pdl(k_fix3<T>, nbp, 256, 0, st, fa));
  JG_CUDA(cudaGetLastError());
  // 2. syntheses of the new level reversed: ln ps, T, vor, div, u cos, v cos
  {
    FFTPlan fp;
    memset(&fp, 0, sizeof(fp));
    G2SPlan gp;
    memset(&gp, 0, sizeof(gp));
    fp.ng = gp.ng = 6;
    fp.C = gp.C = 5 * nd + 1;
    const void* src[6] = {w->g_l, xin->f[14], xin->f[16], xin->f[17], w->g_uc, w->g_vc};
    void* dst[6] = {w->a_l, w->a_t, w->a_vor, w->a_div, w->a_uc, w->a_vc};
    for (int i = 0, col = 0; i < 6; i++) {
      const int L = i == 0 ? 1 : nd;
      fp.g[i] = gin(src[i], L, col);
      gp.g[i] = sadj(dst[i], L, col, (double)nlon);
      col += L;
    }
    JG_TRY(launch_g2s<T>(m, fp, gp, st, md->fbuf, md->fcap));
  }
  NbarArgs<T> na;
  na.in_vor = (const V*)xin->f[0];
  na.in_div = (const V*)xin->f[2];
  na.in_t = (const V*)xin->f[6];
  na.in_l = (const V*)xin->f[4];
  na.a_vor = (const V*)w->a_vor;
  na.a_div = (const V*)w->a_div;
  na.a_t = (const V*)w->a_t;
  na.a_l = (const V*)w->a_l;
  na.a_uc = (const V*)w->a_uc;
  na.a_vc = (const V*)w->a_vc;
  na.nb_vor = (V*)w->nb_vor;
  na.nb_div = (V*)w->nb_div;
  na.nb_t = (V*)w->nb_t;
  na.nb_l = (V*)w->nb_l;
  na.N = N;
  na.ns = ns;
  na.nd = nd;
  const size_t SL = spec_elems(m, nd);
  const int nbs = (int)((SL + 255) / 256);
  JG_CUDA(launch_pdl(k_nbar<T>, nbs, 256, 0, st, na, tb));
  JG_CUDA(cudaGetLastError());
  // 3. implicit correction + damping + filtered leapfrog reversed
  {
    const void* ob[8] = {w->nb_vor, xin->f[1], w->nb_div, xin->f[3], w->nb_t, xin->f[7], w->nb_l, xin->f[5]};
    void* ib[12] = {w->b_dvor, w->b_ddiv, w->b_dt, w->b_dl, xout->f[1], xout->f[0],
                    xout->f[3], xout->f[2], xout->f[7], xout->f[6], xout->f[5], xout->f[4]};
    JG_TRY(si_adjoint_launch(md, ob, ib, w->mats, init, st));
  }
  // 4. analyses of the tendencies reversed: dT, dlnps, energy (-eig ddiv_bar) ...
  JG_CUDA(launch_pdl(k_neg_lap<T>, nbs, 256, 0, st, (const V*)w->b_ddiv, (V*)w->e_spec, tb, N, ns, nd));
  JG_CUDA(cudaGetLastError());
  {
    S2GPlan sp;
    memset(&sp, 0, sizeof(sp));
    IFFTPlan ip;
    memset(&ip, 0, sizeof(ip));
    sp.ng = ip.ng = 3;
    sp.C = ip.C = 2 * nd + 1;
    sp.g[0] = sin_adj(w->b_dt, nd, 0);
    sp.g[1] = sin_adj(w->e_spec, nd, nd);
    sp.g[2] = sin_adj(w->b_dl, 1, 2 * nd);
    ip.g[0] = gout(EPI_ADJ_G2S, w->g_dT, nd, 0);
    ip.g[1] = gout(EPI_ADJ_G2S, w->g_en, nd, nd);
    ip.g[2] = gout(EPI_ADJ_G2S, w->g_dln, 1, 2 * nd);
    JG_TRY(launch_s2g<T>(m, sp, ip, st, md->fbuf, md->fcap));
  }
  // ... and the alpha operators (vor, div from u cos, v cos) -> du, dv
  {
    dim3 ga((m->nh * nd + 255) / 256, N + 1);
    JG_CUDA(launch_pdl(k_alpha_adjoint<T>, ga, 256, 0, st, (const V*)w->b_dvor, (const V*)w->b_ddiv, (V*)md->fbuf, tb, N, ns, nlat,
                                            nlon, nd));
    JG_CUDA(cudaGetLastError());
    IFFTPlan ip;
    memset(&ip, 0, sizeof(ip));
    ip.ng = 2;
    ip.C = 2 * nd;
    ip.g[0] = gout(EPI_NONE, w->g_du, nd, 0);
    ip.g[1] = gout(EPI_NONE, w->g_dv, nd, nd);
    JG_TRY(launch_ifft_only<T>(m, ip, st, md->fbuf, md->fcap));
  }
  // 5. columns: the gradients of ln ps and T of X_s first (Compute_Gradients!: DLAM / DTH prologues,
  //    / cos epilogue)
  {
    S2GPlan sp;
    memset(&sp, 0, sizeof(sp));
    IFFTPlan ip;
    memset(&ip, 0, sizeof(ip));
    sp.ng = ip.ng = 4;
    sp.C = ip.C = 2 + 2 * nd;
    const int ops[4] = {S2G_DLAM, S2G_DTH, S2G_DLAM, S2G_DTH};
    const void* src[4] = {x0->f[4], x0->f[4], x0->f[6], x0->f[6]};
    void* dst[4] = {w->x_gl, w->x_gt, w->x_tl, w->x_tt};
    for (int i = 0, col = 0; i < 4; i++) {
      const int L = i < 2 ? 1 : nd;
      memset(&sp.g[i], 0, sizeof(sp.g[i]));
      sp.g[i].a = src[i];
      sp.g[i].op = ops[i];
      sp.g[i].L = L;
      sp.g[i].col0 = col;
      ip.g[i] = gout(EPI_DIVCOS, dst[i], L, col);
      col += L;
    }
    JG_TRY(launch_s2g<T>(m, sp, ip, st, md->fbuf, md->fcap));
  }
  ColAdjArgs<T> ca;
  memset(&ca, 0, sizeof(ca));
  ca.u = (const T*)x0->f[8];
  ca.v = (const T*)x0->f[10];
  ca.t = (const T*)x0->f[14];
  ca.vor = (const T*)x0->f[16];
  ca.div = (const T*)x0->f[17];
  ca.up = (const T*)x0->f[9];
  ca.vp = (const T*)x0->f[11];
  ca.tp = (const T*)x0->f[15];
  ca.ps = (const T*)x0->f[12];
  ca.psp = (const T*)x0->f[13];
  ca.gl = (const T*)w->x_gl;
  ca.gt = (const T*)w->x_gt;
  ca.tl = (const T*)w->x_tl;
  ca.tt = (const T*)w->x_tt;
  ca.DU = (const T*)w->g_du;
  ca.DV = (const T*)w->g_dv;
  ca.DT = (const T*)w->g_dT;
  ca.EN = (const T*)w->g_en;
  ca.DLN = (const T*)w->g_dln;
  ca.seed_u = (const T*)xin->f[9];
  ca.seed_v = (const T*)xin->f[11];
  ca.seed_t = (const T*)xin->f[15];
  ca.seed_ps = (const T*)xin->f[13];
  ca.bu = (T*)xout->f[8];
  ca.bup = (T*)xout->f[9];
  ca.bv = (T*)xout->f[10];
  ca.bvp = (T*)xout->f[11];
  ca.bps = (T*)xout->f[12];
  ca.bpsp = (T*)xout->f[13];
  ca.bt = (T*)xout->f[14];
  ca.btp = (T*)xout->f[15];
  ca.bvor = (T*)xout->f[16];
  ca.bdiv = (T*)xout->f[17];
  ca.btl = (T*)w->g_tl;
  ca.btt = (T*)w->g_tt;
  ca.bgl = (T*)w->g_gl;
  ca.bgt = (T*)w->g_gt;
  ca.coriolis = (const T*)md->coriolis;
  ca.sinj = tb.sinj;
  ca.cosj = tb.cosj;
  ca.wts = m->d_wts;
  ca.sc = w->sc;
  ca.ppart = w->ppart;
  ca.nd = nd;
  ca.nlat = nlat;
  ca.nlon = nlon;
  ca.Dt = init ? md->P.dt : 2 * md->P.dt;
  {
    const double day = 86400.0, sb = md->P.sigma_b;
    ca.sigma_b = sb;
    ca.kvc = md->P.k_f / day / (1.0 - sb);
    ca.ka = md->P.k_a / day;
    ca.ktc = (md->P.k_s - md->P.k_a) / day / (1.0 - sb);
    ca.inv_1msb = 1.0 / (1.0 - sb);
    ca.inv_day = 1.0 / day;
    ca.dT_y = md->P.dT_y;
    ca.dtheta_z = md->P.dtheta_z;
    ca.kappa = md->P.kappa;
    ca.ln_p0 = std::log(1.0e5);
    ca.rdgas = md->P.rdgas;
    ca.cp = md->cp_air;
    ca.inv_cp = 1.0 / md->cp_air;
    ca.inv_grav = 1.0 / md->P.grav;
    col_adj_consts<T>(ca);
  }
  k_hs_column_adjoint<T><<<w->nb_adj, 256, 0, st>>>(ca, md->d_vc);
  JG_CUDA(launch_pdl(k_fold_params, 5, 256, 0, st, w->ppart, w->nb_adj, w->pbar));
  JG_CUDA(cudaGetLastError());
  // 6. the gradients' syntheses reversed, then Compute_Gradient_Cos! transposed
  {
    FFTPlan fp;
    memset(&fp, 0, sizeof(fp));
    G2SPlan gp;
    memset(&gp, 0, sizeof(gp));
    fp.ng = gp.ng = 4;
    fp.C = gp.C = 2 * nd + 2;
    fp.g[0] = gin(w->g_gl, 1, 0);
    fp.g[1] = gin(w->g_gt, 1, 1);
    fp.g[2] = gin(w->g_tl, nd, 2);
    fp.g[3] = gin(w->g_tt, nd, 2 + nd);
    gp.g[0] = sadj(w->s_gl, 1, 0, (double)nlon);
    gp.g[1] = sadj(w->s_gt, 1, 1, (double)nlon);
    gp.g[2] = sadj(w->s_tl, nd, 2, (double)nlon);
    gp.g[3] = sadj(w->s_tt, nd, 2 + nd, (double)nlon);
    JG_TRY(launch_g2s<T>(m, fp, gp, st, md->fbuf, md->fcap));
  }
  const size_t S1 = spec_elems(m, 1);
  JG_CUDA(launch_pdl(k_grad_adjoint<T>, (int)((S1 + 255) / 256), 256, 0, st, (const V*)w->s_gl, (const V*)w->s_gt, (V*)xout->f[4], tb,
                                                             N, ns, 1));
  JG_CUDA(launch_pdl(k_grad_adjoint<T>, nbs, 256, 0, st, (const V*)w->s_tl, (const V*)w->s_tt, (V*)xout->f[6], tb, N, ns, nd));
  JG_CUDA(cudaGetLastError());
  (void)G;
  return JGCM_OK;
}

int adjoint_step_any(jgcm_model* md, AdjWork* w, const StateBuf* x0, const StateBuf* x1, StateBuf* xin,
                     StateBuf* xout, int init) {
  return is_fp64(md->mesh) ? adjoint_step<double>(md, w, x0, x1, xin, xout, init)
                           : adjoint_step<float>(md, w, x0, x1, xin, xout, init);
}

// forward scalars of the step just taken: mean_ps_p, mean_energy_p, factor, correction
int save_scalars(jgcm_model* md, double* dst, cudaStream_t st) {
  return cudaMemcpyAsync(dst, md->d_scalars, 4 * sizeof(double), cudaMemcpyDeviceToDevice, st) == cudaSuccess
             ? JGCM_OK
             : JGCM_E_CUDA;
}

int check_model(jgcm_model* md) {
  JG_ARG(md, "NULL model");
  JG_ARG(md->P.kind == JGCM_HELD_SUAREZ, "the step adjoint exists for Held-Suarez models");
  JG_ARG(md->ne == 1, "one-member models only");
  JG_ARG(md->nd <= 32, "the column adjoint holds one level per lane: nd <= 32");
  JG_ARG(!md->diag_on, "switch the on-device diagnostics off before differentiating");
  // the reverse column kernel reads the sigma coordinates' per-level log-pressure constants
  JG_ARG(!md->vc.hybrid, "the step adjoint is built for sigma coordinates (a_k = 0), not hybrid ones");
  JG_ARG(md->nq == 0, "the step adjoint does not differentiate passive tracers: a model without tracers");
  return JGCM_OK;
}

// host (reference layout, FP64) <-> device state cotangents
int bars_h2d(jgcm_model* md, const double* const* host, StateBuf* b) {
  jgcm_mesh* m = md->mesh;
  cudaStream_t st = m->stream;
  for (int i = 0; i < NSTATE; i++) {
    const int L = st_levels(md, i);
    const size_t n = st_spec(i) ? 2 * spec_elems(m, L) : grid_elems(m, L);
    JG_CUDA(cudaMemcpyAsync(m->d_stage, host[i], n * 8, cudaMemcpyHostToDevice, st));
    if (st_spec(i)) JG_TRY(spec_host_to_dev(m, m->d_stage, b->f[i], L, st));
    else JG_TRY(grid_host_to_dev(m, m->d_stage, b->f[i], n, st));
    JG_CUDA(cudaStreamSynchronize(st));
  }
  return JGCM_OK;
}

int bars_d2h(jgcm_model* md, const StateBuf* b, double* const* host) {
  jgcm_mesh* m = md->mesh;
  cudaStream_t st = m->stream;
  for (int i = 0; i < NSTATE; i++) {
    const int L = st_levels(md, i);
    const size_t n = st_spec(i) ? 2 * spec_elems(m, L) : grid_elems(m, L);
    if (st_spec(i)) JG_TRY(spec_dev_to_host(m, b->f[i], m->d_stage, L, st));
    else JG_TRY(grid_dev_to_host(m, b->f[i], m->d_stage, n, st));
    JG_CUDA(cudaMemcpyAsync(host[i], m->d_stage, n * 8, cudaMemcpyDeviceToHost, st));
    JG_CUDA(cudaStreamSynchronize(st));
  }
  return JGCM_OK;
}

struct Scope {  // frees device allocations on every return path (holds copies of the handles)
  std::vector<void*> p;
  std::vector<AdjWork> w;
  ~Scope() {
    for (void* q : p) cudaFree(q);
    for (AdjWork& a : w) work_free(&a);
  }
};

}  // namespace

extern "C" int jgcm_model_step_adjoint(jgcm_model* md, double* const* state_bar, double* param_bar) {
  JG_TRY(check_model(md));
  JG_ARG(state_bar, "NULL cotangent array");
  for (int i = 0; i < NSTATE; i++) JG_ARG(state_bar[i], "cotangent %d is NULL", i);
  jgcm_mesh* m = md->mesh;
  cudaStream_t st = m->stream;
  Scope sc;
  StateBuf x0, x1, bi, bo;
  for (StateBuf* b : {&x0, &x1, &bi, &bo}) {
    JG_TRY(state_alloc(md, b));
    sc.p.push_back(b->base);
  }
  AdjWork w;
  JG_TRY(work_alloc(md, &w));
  sc.w.push_back(w);
  JG_TRY(state_save(md, &x0, st));
  JG_TRY(jgcm_model_step(md, 1));
  JG_TRY(state_save(md, &x1, st));
  JG_TRY(save_scalars(md, w.sc, st));
  JG_TRY(state_load(md, &x0, st));
  JG_TRY(bars_h2d(md, state_bar, &bi));
  JG_TRY(state_zero(md, &bo, st));
  JG_CUDA(cudaMemsetAsync(w.pbar, 0, 5 * 8, st));
  JG_TRY(adjoint_step_any(md, &w, &x0, &x1, &bi, &bo, x0.init));
  JG_TRY(bars_d2h(md, &bo, state_bar));
  double pb[5];
  JG_CUDA(cudaMemcpyAsync(pb, w.pbar, sizeof(pb), cudaMemcpyDeviceToHost, st));
  JG_CUDA(cudaStreamSynchronize(st));
  if (param_bar)
    for (int i = 0; i < 5; i++) param_bar[i] += pb[i];
  if (m->tc.on) JG_TRY(tc_status(m));
  return JGCM_OK;
}

namespace {
// The workspace of the checkpointed gradient, kept in the model between calls with the same step
// count and checkpoint interval (allocation, and the host build of the transposed vertical
// operators, would otherwise dominate short windows).
struct AdjContext {
  int nsteps = 0, K = 0, nbl = 0, tune_gen = -1;
  std::vector<std::pair<int, cudaGraphExec_t>> graphs;  // reverse steps: key (slot, init, parity)
  std::vector<StateBuf> ck, seg;
  StateBuf fin{}, bi{}, bo{};
  AdjWork w{};
  bool has_w = false;
  std::vector<void*> bufs;  // every StateBuf base and scratch array
  double *d_tgt = nullptr, *d_scal = nullptr, *part = nullptr;
};

void ctx_free(AdjContext* c) {
  if (!c) return;
  for (auto& kv : c->graphs)
    if (kv.second) cudaGraphExecDestroy(kv.second);
  for (void* p : c->bufs) cudaFree(p);
  if (c->has_w) work_free(&c->w);
  delete c;
}

int ctx_create(jgcm_model* md, int nsteps, int K, AdjContext** out) {
  jgcm_mesh* m = md->mesh;
  AdjContext* c = new AdjContext();
  c->nsteps = nsteps;
  c->K = K;
  const int nseg = (nsteps + K - 1) / K, segl = K < nsteps ? K : nsteps;
  c->ck.resize(nseg);
  c->seg.resize(segl + 1);
  auto fail = [&](int st) {
    ctx_free(c);
    return st;
  };
  auto nb = [&](StateBuf* b) -> int {
    const int st = state_alloc(md, b);
    if (st == JGCM_OK) c->bufs.push_back(b->base);
    return st;
  };
  for (auto& b : c->ck)
    if (int st = nb(&b)) return fail(st);
  for (auto& b : c->seg)
    if (int st = nb(&b)) return fail(st);
  for (StateBuf* b : {&c->fin, &c->bi, &c->bo})
    if (int st = nb(b)) return fail(st);
  if (int st = work_alloc(md, &c->w)) return fail(st);
  c->has_w = true;
  const size_t GL = grid_elems(m, md->nd);
  c->nbl = (int)((GL + 255) / 256);
  void** scratch[] = {(void**)&c->d_tgt, (void**)&c->d_scal, (void**)&c->part};
  const size_t bytes[] = {GL * 8, (size_t)segl * 4 * 8, (size_t)c->nbl * 8};
  for (int i = 0; i < 3; i++) {
    if (int st = dev_alloc(scratch[i], bytes[i])) return fail(st);
    c->bufs.push_back(*scratch[i]);
  }
  *out = c;
  return JGCM_OK;
}
// The reverse step of segment slot j: the step's forward scalars copied into the work scalars, then
// adjoint_step from seg[j] (X_s) and seg[j+1] (X_{s+1}) between the two cotangent buffers (bi -> bo
// when in_bi, else bo -> bi), captured once and replayed in every segment.
int ctx_step_graph(jgcm_model* md, AdjContext* c, int j, int init, bool in_bi, cudaGraphExec_t* out) {
  const int key = (j * 2 + (init ? 1 : 0)) * 2 + (in_bi ? 1 : 0);
  for (auto& kv : c->graphs)
    if (kv.first == key) {
      *out = kv.second;
      return JGCM_OK;
    }
  cudaStream_t st = md->mesh->stream;
  StateBuf* xin = in_bi ? &c->bi : &c->bo;
  StateBuf* xout = in_bi ? &c->bo : &c->bi;
  cudaGraph_t g;
  JG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  cudaError_t e = cudaMemcpyAsync(c->w.sc, c->d_scal + 4 * j, 4 * 8, cudaMemcpyDeviceToDevice, st);
  int s = e == cudaSuccess ? adjoint_step_any(md, &c->w, &c->seg[j], &c->seg[j + 1], xin, xout, init) : JGCM_OK;
  cudaError_t e2 = cudaStreamEndCapture(st, &g);
  if (s != JGCM_OK || e != cudaSuccess || e2 != cudaSuccess) {
    if (e2 == cudaSuccess) cudaGraphDestroy(g);
    if (s != JGCM_OK) return s;
    JG_CUDA(e != cudaSuccess ? e : e2);
  }
  cudaGraphExec_t ge = nullptr;
  cudaError_t e3 = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  JG_CUDA(e3);
  c->graphs.push_back({key, ge});
  *out = ge;
  return JGCM_OK;
}
}  // namespace

void jgcm::adj_context_free(jgcm_model* md) {
  ctx_free((AdjContext*)md->adj);
  md->adj = nullptr;
}

extern "C" int jgcm_model_hs_gradient(jgcm_model* md, int nsteps, int checkpoint_every, const double* t_target,
                                      double* loss, double* grad_spe_t0, double* grad_params) {
  JG_TRY(check_model(md));
  JG_ARG(nsteps >= 1 && checkpoint_every >= 1, "nsteps and checkpoint_every must be positive");
  JG_ARG(t_target, "NULL target");
  jgcm_mesh* m = md->mesh;
  cudaStream_t st = m->stream;
  const int nd = md->nd, K = checkpoint_every, nseg = (nsteps + K - 1) / K;
  AdjContext* ctx = (AdjContext*)md->adj;
  if (!ctx || ctx->nsteps != nsteps || ctx->K != K) {
    jgcm::adj_context_free(md);
    JG_TRY(ctx_create(md, nsteps, K, &ctx));
    md->adj = ctx;
  }
  if (ctx->tune_gen != m->tune_gen) {  // tiles or Legendre engine changed since the capture
    for (auto& kv : ctx->graphs)
      if (kv.second) cudaGraphExecDestroy(kv.second);
    ctx->graphs.clear();
    ctx->tune_gen = m->tune_gen;
  }
  std::vector<StateBuf>& ck = ctx->ck;
  std::vector<StateBuf>& seg = ctx->seg;
  StateBuf &fin = ctx->fin, &bi = ctx->bi, &bo = ctx->bo;
  AdjWork& w = ctx->w;
  double *d_tgt = ctx->d_tgt, *d_scal = ctx->d_scal;
  const size_t GL = grid_elems(m, nd);
  // the target, FP64: the reference layout [i][j][k] (i fastest) is the device grid layout [k][j][i]
  JG_CUDA(cudaMemcpyAsync(d_tgt, t_target, GL * 8, cudaMemcpyHostToDevice, st));
  // forward sweep with checkpoints
  for (int s = 0; s < nsteps; s++) {
    if (s % K == 0) JG_TRY(state_save(md, &ck[s / K], st));
    JG_TRY(model_step_async(md));
  }
  JG_TRY(state_save(md, &fin, st));
  // loss and the cotangent of the final grid temperature
  JG_TRY(state_zero(md, &bi, st));
  JG_TRY(state_zero(md, &bo, st));
  JG_CUDA(cudaMemsetAsync(w.pbar, 0, 5 * 8, st));
  {
    const int nbl = ctx->nbl;
    double* part = ctx->part;
    if (is_fp64(m))
      JG_CUDA(launch_pdl(k_loss<double>, nbl, 256, 0, st, (const double*)fin.f[14], d_tgt, (double*)bi.f[14], m->d_wts, m->nlat,
                                          m->nlon, nd, part));
    else
      JG_CUDA(launch_pdl(k_loss<float>, nbl, 256, 0, st, (const float*)fin.f[14], d_tgt, (float*)bi.f[14], m->d_wts, m->nlat,
                                         m->nlon, nd, part));
    JG_CUDA(launch_pdl(k_fold_scalar, 1, 256, 0, st, part, nbl, w.sc + SC_LOSS));
    JG_CUDA(cudaGetLastError());
    if (loss) {  // the mesh stream does not synchronise with the legacy default stream
      JG_CUDA(cudaMemcpyAsync(loss, w.sc + SC_LOSS, 8, cudaMemcpyDeviceToHost, st));
      JG_CUDA(cudaStreamSynchronize(st));
    }
  }
  // reverse sweep: each segment is recomputed from its checkpoint, then reversed step by step
  StateBuf* xin = &bi;
  StateBuf* xout = &bo;
  for (int g = nseg - 1; g >= 0; g--) {
    const int s0 = g * K, s1 = (s0 + K < nsteps) ? s0 + K : nsteps;
    JG_TRY(state_load(md, &ck[g], st));
    for (int s = s0; s < s1; s++) {
      JG_TRY(state_save(md, &seg[s - s0], st));
      JG_TRY(model_step_async(md));
      JG_TRY(save_scalars(md, d_scal + 4 * (s - s0), st));
    }
    JG_TRY(state_save(md, &seg[s1 - s0], st));
    for (int s = s1 - 1; s >= s0; s--) {  // one captured graph per (slot, init flag, buffer parity)
      const int j = s - s0;
      cudaGraphExec_t ge = nullptr;
      JG_TRY(ctx_step_graph(md, ctx, j, seg[j].init, xin == &bi, &ge));
      JG_CUDA(cudaGraphLaunch(ge, st));
      StateBuf* t = xin;
      xin = xout;
      xout = t;
    }
  }
  // d loss / d T0 with spe_t_c = spe_t_p = T0 and grid_t_c = grid_t_p = S2G(T0)
  if (grad_spe_t0) {
    const size_t ts = tsize(m);
    void* gsum = w.g_du;  // free scratch: nd grid levels
    const int nbl = (int)((GL + 255) / 256);
    if (is_fp64(m))
      JG_CUDA(launch_pdl(k_add2<double>, nbl, 256, 0, st, (const double*)xin->f[14], (const double*)xin->f[15], (double*)gsum, GL));
    else
      JG_CUDA(launch_pdl(k_add2<float>, nbl, 256, 0, st, (const float*)xin->f[14], (const float*)xin->f[15], (float*)gsum, GL));
    FFTPlan fp;
    memset(&fp, 0, sizeof(fp));
    G2SPlan gp;
    memset(&gp, 0, sizeof(gp));
    fp.ng = gp.ng = 1;
    fp.C = gp.C = nd;
    fp.g[0] = gin(gsum, nd, 0);
    gp.g[0] = sadj(w.a_t, nd, 0, (double)m->nlon);
    if (is_fp64(m)) JG_TRY(launch_g2s<double>(m, fp, gp, st, md->fbuf, md->fcap));
    else JG_TRY(launch_g2s<float>(m, fp, gp, st, md->fbuf, md->fcap));
    const size_t SLn = spec_elems(m, nd) * 2;  // reals
    const int nbs = (int)((SLn + 255) / 256);
    if (is_fp64(m)) {
      JG_CUDA(launch_pdl(k_add2<double>, nbs, 256, 0, st, (const double*)xin->f[6], (const double*)xin->f[7], (double*)w.nb_t, SLn));
      JG_CUDA(launch_pdl(k_add2<double>, nbs, 256, 0, st, (const double*)w.nb_t, (const double*)w.a_t, (double*)w.nb_t, SLn));
    } else {
      JG_CUDA(launch_pdl(k_add2<float>, nbs, 256, 0, st, (const float*)xin->f[6], (const float*)xin->f[7], (float*)w.nb_t, SLn));
      JG_CUDA(launch_pdl(k_add2<float>, nbs, 256, 0, st, (const float*)w.nb_t, (const float*)w.a_t, (float*)w.nb_t, SLn));
    }
    JG_CUDA(cudaGetLastError());
    JG_TRY(spec_dev_to_host(m, w.nb_t, m->d_stage, nd, st));
    JG_CUDA(cudaMemcpyAsync(grad_spe_t0, m->d_stage, SLn * 8, cudaMemcpyDeviceToHost, st));
    JG_CUDA(cudaStreamSynchronize(st));
    // T0 lives where the analysis puts it: row N+1 zero (Trans_Grid_To_Spherical!).  That row is
    // outside the semi-implicit solve (n > N skips W_n) and an explicit gravity-wave mode of the
    // step grows there by orders of magnitude per step; it is not part of the control.
    for (int k = 0; k < nd; k++)
      for (int mm = 0; mm <= m->N; mm++) {
        const size_t h = 2 * ((size_t)mm + (size_t)(m->N + 1) * ((size_t)m->ns + (size_t)(m->ns + 1) * k));
        grad_spe_t0[h] = grad_spe_t0[h + 1] = 0.0;
      }
    (void)ts;
  }
  if (grad_params) JG_CUDA(cudaMemcpyAsync(grad_params, w.pbar, 5 * 8, cudaMemcpyDeviceToHost, st));
  // leave the model at the final state
  JG_TRY(state_load(md, &fin, st));
  md->init_step = 0;
  JG_CUDA(cudaStreamSynchronize(st));
  if (m->tc.on) JG_TRY(tc_status(m));
  return JGCM_OK;
}
