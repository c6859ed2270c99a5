// models.cu -- device-resident time stepping of the three JGCM models.
//
//   Barotropic_Dynamics!        Barotropic_Dynamics.jl:2-46                 4 launches / step
//   Shallow_Water_Dynamics!     Shallow_Water_Dynamics.jl:7-179             6 launches / step
//   Atmosphere_Update! (HS)     Spectral_Dynamics.jl:206-365, 452-490,
//                               HS_Forcing.jl:1-130, Semi_Implicit.jl        8 launches / step
//
// Dyn_Data lives on the device in the model's precision.  Time levels p/c/n rotate by
// pointer (Time_Advance!, Dyn_Data.jl:326-364, copies instead); steady steps are captured
// once per rotation phase as CUDA graphs and replayed.  The semi-implicit wave matrices
// (Semi_Implicit.jl:165-180) are inverted on the device in FP64, the per-(m,n) vertical
// solve runs in FP64 (one warp per spectral mode, lanes over levels) and the mass/energy
// fixers (Spectral_Dynamics.jl:5-68) use deterministic FP64 reductions.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cooperative_groups.h>

#include "jgcm_internal.cuh"

using namespace jgcm;
namespace cg = cooperative_groups;

#include "model_internal.cuh"

namespace {
template <typename T>
using V2 = typename C2<T>::t;
}  // namespace

namespace {

// ------------------------------------------------------------------------------------------
// warp scans over levels (lanes >= nd hold zero)
template <typename R>
__device__ __forceinline__ R scan_incl(R x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    R y = __shfl_up_sync(FULL, x, o);
    if (lane >= o) x += y;
  }
  return x;
}
template <typename R>
__device__ __forceinline__ R rscan_incl(R x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    R y = __shfl_down_sync(FULL, x, o);
    if (lane + o < 32) x += y;
  }
  return x;
}
template <typename R>
__device__ __forceinline__ R warp_sum_t(R x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
  return x;
}
__device__ __forceinline__ double warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(FULL, x, o);
  return x;
}
template <typename T>
__device__ __forceinline__ T shfl_up1(T x, int lane, T fill) {
  T y = __shfl_up_sync(FULL, x, 1);
  return lane == 0 ? fill : y;
}
template <typename T>
__device__ __forceinline__ T shfl_dn1(T x, int lane, int nd, T fill) {
  T y = __shfl_down_sync(FULL, x, 1);
  return lane + 1 >= nd ? fill : y;
}

// Deterministic two-level grid reduction of FP64 block values (the fixers' global sums).  FP64
// issues at 2 lanes per cycle per SM here (a warp instruction holds its sub-partition's FP64 pipe
// for ~64 cycles), so the folds are laid out to keep few FP64 warp instructions on the critical
// path and to spread them over the four sub-partitions: one warp per value, lanes over partials,
// a fixed butterfly.  The first level's units are either thread-block clusters (up to 8 blocks on
// one GPC, folding their values through distributed shared memory at the cluster barrier) or,
// when the grid takes more than one wave of blocks (where a cluster barrier would hold SM slots),
// groups of CORR_GS consecutive blocks whose last block to arrive (atomic ticket) folds them.
// Each unit publishes its values, and the last unit to arrive folds the units' values.
constexpr int CORR_GS = 16;  // blocks per group
constexpr int CORR_CL = 8;   // blocks per cluster at most (the portable cluster size)

__host__ __device__ inline int corr_groups(int nb) { return (nb + CORR_GS - 1) / CORR_GS; }

// The fixer reduction's cluster shape over its (gx = nlon/32) x nlat grid: powers of two that
// divide the grid, x first (the blocks of one latitude row), at most CORR_CL blocks
inline void corr_cluster(int gx, int nlat, int& cx, int& cy) {
  cx = 1;
  while (cx * 2 <= CORR_CL && gx % (cx * 2) == 0) cx *= 2;
  cy = 1;
  while (cx * cy * 2 <= CORR_CL && nlat % (cy * 2) == 0) cy *= 2;
}

// sum of the n consecutive values at p: lane-strided in a fixed order, then the butterfly; every
// lane of the warp returns the same total
__device__ __forceinline__ double warp_fold(const double* p, int n, int lane) {
  double s = 0.0;
  for (int q = lane; q < n; q += 32) s += __ldcg(p + q);
  return warp_sum(s);
}

// Publishes this block's arrival after its writes (made by any of its threads before the call)
// and returns, in every thread, whether it was the last of the `n` arrivals on `counter`; the last
// one resets the counter for the next launch.  The block barrier orders the writes before thread 0's
// arrival, which is an acquire-release atomic at GPU scope: it releases them to the block that
// arrives last and, in that block, acquires every earlier block's released writes (no full fences).
__device__ __forceinline__ bool ticket_last(unsigned* counter, unsigned n) {
  __shared__ bool last;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned t;
    asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], 1;" : "=r"(t) : "l"(counter) : "memory");
    last = (t == n - 1);
    if (last) *counter = 0u;
  }
  __syncthreads();
  return last;
}

// Error-free transformations in FP32: the pair hi + lo carries a sum to ~2^-48 relative (FP64-class
// accuracy from FP32 instructions: an FP64 instruction holds a sub-partition ~64 cycles on this part,
// an FP32 one ~1).  The _rn intrinsics are never contracted into a multiply-add, which would break
// the exactness of the two-sum.
__device__ __forceinline__ void ds_add(float& hi, float& lo, float x) {
  const float s = __fadd_rn(hi, x), bb = __fsub_rn(s, hi);
  lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb)));
  hi = s;
}
// hi + lo += t (ch + cl): the product t ch as its rounding plus its exact error, t cl added to lo
__device__ __forceinline__ void ds_add_prod(float& hi, float& lo, float t, float ch, float cl) {
  const float p = __fmul_rn(t, ch);
  const float pe = __fmaf_rn(t, ch, -p);
  ds_add(hi, lo, p);
  lo = __fadd_rn(lo, __fmaf_rn(t, cl, pe));
}

// Mercator series of log(1 + d) for |d| <= 2^-12: the remainder after the d^5 term is below
// |d|^6 / 6 < 2^-62 |d|, under half an ulp of the sum; larger |d| take the library's log
__device__ __forceinline__ double log_near_one(double f) {
  const double d = f - 1.0;  // exact for f in [1/2, 2] (Sterbenz)
  if (fabs(d) > 0x1p-12) return log(f);
  const double c3 = 1.0 / 3.0, c5 = 1.0 / 5.0;
  double r = fma(-d, c5, 0.25);   // 1/4 - d/5
  r = fma(-d, r, c3);             // 1/3 - d (1/4 - d/5)
  r = fma(-d, r, 0.5);            // 1/2 - ...
  r = fma(-d, r, 1.0);            // 1 - d (1/2 - ...)
  return d * r;
}

// ------------------------------------------------------------------------------------------
// Held-Suarez: physics (HS_Forcing!, previous time level) + corrections-init sums +
// Four_In_One! + Compute_Geopotential! + Vert_Advection! x3 + horizontal advection of T +
// absolute-vorticity fluxes + energy, fused.  One thread per grid column (consecutive threads,
// consecutive longitudes: every level read and write is a coalesced row), levels walked in two
// passes: bottom-up for the hydrostatic geopotential (Compute_Geopotential!) and the column
// divergence sum, then top-down for everything else (the mass-flux prefix sum of Four_In_One!
// and the centred vertical advection, whose flux at k+1/2 is carried to the next level).
// Sigma coordinates: one log per column, one exp per level (ln p = const_k + ln ps).
constexpr int HS_CT = 64;  // columns (threads) per block

template <typename T>
struct HSColArgs {
  const T *u_p, *v_p, *t_p, *ps_p, *ps_c, *u_c, *v_c, *t_c, *div, *vor, *dlps, *dtps, *dlT, *dtT, *geopots, *coriolis,
      *sinj, *cosj;
  const T* tdev;  // T_c less its level means, synthesised as such (FP32 path); NULL: T_c - T0_k here
  int has_dak;    // some a_k differs between levels (hybrid coordinates): the energy sums need sum_k T_k Δa_k
  T *ducos, *dvcos, *dtg, *energy, *dlnps, *t_eq;
  T* m_half;            // tracers: M_{k+1/2} at level index k (NULL: not stored)
  const V2<T>* t_spec;  // spe_t_c: its (0,0) modes are the level means of T
  const double* wts;
  double* partials;  // per member: partials + e * pstride (the block partials of mean ps_p, energy_p)
  size_t pstride;
  int nd, nlat, nlon, Dt;
  double sigma_b, k_f, k_a, k_s, dT_y, dtheta_z, kappa, rdgas, cp, grav;
  double inv_2n;  // 1 / (2 nlon), exact (nlon is a power of two)
  // the physics constants in T, formed on the host with the kernel's own T arithmetic (no FP64 ->
  // FP32 conversion per thread: those run on the FP64 pipe)
  T sb, R, kap, cp_t, kv0, ka, ks, kt0, dTy, dthz, kappa_t;
};

template <typename T>
void hs_col_consts(HSColArgs<T>& a) {
  const T day = (T)86400;
  a.sb = (T)a.sigma_b;
  a.R = (T)a.rdgas;
  a.cp_t = (T)a.cp;
  a.kap = a.R / a.cp_t;
  a.kv0 = ((T)a.k_f / day) / ((T)1.0 - a.sb);
  a.ka = (T)a.k_a / day;
  a.ks = (T)a.k_s / day;
  a.kt0 = (a.ks - a.ka) / ((T)1.0 - a.sb);
  a.dTy = (T)a.dT_y;
  a.dthz = (T)a.dtheta_z;
  a.kappa_t = (T)a.kappa;
}

// S lanes per column (S = 1, 2, 4): lane s walks levels [s*len, s*len + len), len = ceil(nd/S); the
// running sums that couple the levels (the geopotential from below, the mass-divergence prefix and
// column total) are completed across the S lanes with shuffles, so a column's chain of dependent
// work is nd/S levels long.  Small grids run S = 4 for latency, large ensembles S = 1.
template <int S, typename R>
__device__ __forceinline__ R seg_sum(R x) {  // sum over the S lanes of this column
#pragma unroll
  for (int o = 1; o < S; o <<= 1) x += __shfl_xor_sync(FULL, x, o, S);
  return x;
}
template <int S, typename R>
__device__ __forceinline__ R seg_excl_prefix(R x, int s) {  // sum over the lanes s' < s
  R incl = x;
#pragma unroll
  for (int o = 1; o < S; o <<= 1) {
    R y = __shfl_up_sync(FULL, incl, o, S);
    if (s >= o) incl += y;
  }
  return incl - x;
}
template <int S, typename R>
__device__ __forceinline__ R seg_excl_suffix(R x, int s) {  // sum over the lanes s' > s
  R incl = x;
#pragma unroll
  for (int o = 1; o < S; o <<= 1) {
    R y = __shfl_down_sync(FULL, incl, o, S);
    if (s + o < S) incl += y;
  }
  return incl - x;
}

// FP32, one lane per column (member ensembles): at most 72 registers (14 blocks of 64 threads per SM):
// at that scale the kernel streams and its time follows occupancy (at 77 registers, allocated as 80,
// 12 blocks: 97 -> 109 us, measured).  Several lanes per column (small grids, a few blocks per SM):
// registers up to 6 blocks per SM, the level loops' values held without spills
// HYB (hybrid coordinates, a_k != 0): the log pressures of Pressure_Variables! (Press_And_Geopot.jl:
// 36-67, Simmons-Burridge, zero top) are formed per column and level from p_{k+1/2} = a_k + b_k ps:
// D_k = ln(p_{k+1/2} / p_{k-1/2}) = log1p(Δp_k / p_{k-1/2}) (no difference of two large logarithms),
// ln p_{k+1/2} - ln p_k = 1 - p_{k-1/2} D_k / Δp_k, ln p_k - ln p_{k-1/2} = D_k - that; the top level
// has ln p_1 = ln p_{3/2} - 1.  Sigma coordinates read the same quantities as per-level constants.
template <typename T, int S, bool HYB>
__global__ void __launch_bounds__(HS_CT, (sizeof(T) == 4 && S == 1) ? 14 : sizeof(T) == 4 ? 6 : 1)
    k_hs_column(HSColArgs<T> a, const VertCoef* __restrict__ vcp) {
  const VertCoef& vc = *vcp;
  __shared__ double red[2][HS_CT / 32];
  // the vertical coefficients in the state precision, staged once per block (constants: staged
  // before the dependency wait; on the FP32 path this also keeps the FP64 -> FP32 conversions out of
  // the level loops)
  __shared__ T s_dak[JGCM_MAX_ND], s_dbk[JGCM_MAX_ND], s_bk[JGCM_MAX_ND + 1], s_cf[JGCM_MAX_ND],
      s_dlpp[JGCM_MAX_ND], s_dlpm[JGCM_MAX_ND], s_dlp[JGCM_MAX_ND], s_sf[JGCM_MAX_ND];
  __shared__ T s_lb1;
  __shared__ T s_ak[JGCM_MAX_ND + 1];  // hybrid coordinates: a_k in the state precision
  __shared__ double s_dak64[JGCM_MAX_ND], s_dbk64[JGCM_MAX_ND];  // FP64 layer coefficients: the energy integral
  __shared__ float s_dah[JGCM_MAX_ND], s_dal[JGCM_MAX_ND], s_dbh[JGCM_MAX_ND], s_dbl[JGCM_MAX_ND];  // as FP32 pairs
  const int nd = a.nd, nlon = a.nlon, nlat = a.nlat;
  for (int q = threadIdx.x; q <= nd; q += blockDim.x) {
    s_bk[q] = (T)vc.bk[q];
    s_ak[q] = (T)vc.ak[q];
    if (q < nd) {
      s_dak64[q] = vc.dak[q];
      s_dbk64[q] = vc.dbk[q];
      s_dah[q] = vc.dak_hi[q];
      s_dal[q] = vc.dak_lo[q];
      s_dbh[q] = vc.dbk_hi[q];
      s_dbl[q] = vc.dbk_lo[q];
      s_dak[q] = (T)vc.dak[q];
      s_dbk[q] = (T)vc.dbk[q];
      s_cf[q] = (T)vc.cf[q];
      s_dlpp[q] = (T)vc.dlp_p[q];
      s_dlpm[q] = (T)vc.dlp_m[q];
      s_dlp[q] = (T)vc.dlp[q];
      s_sf[q] = (T)vc.sf[q];
    }
  }
  if (threadIdx.x == 0) s_lb1 = (T)vc.lb[1];
  __syncthreads();
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  const int seg = threadIdx.x % S, i = blockIdx.x * (HS_CT / S) + threadIdx.x / S, j = blockIdx.y, e = blockIdx.z;
  const int len = (nd + S - 1) / S, k0 = min(nd, seg * len), k1 = min(nd, k0 + len);
  const bool act = i < nlon;
  const size_t G = (size_t)nlat * nlon;
  // member e: its nd levels start at level e*nd, its single-level fields at level e
  const size_t col = (size_t)j * nlon + (act ? i : 0), c1 = (size_t)e * G + col, cL = (size_t)e * nd * G + col;
  const T* __restrict__ u_c = a.u_c + cL;
  const T* __restrict__ v_c = a.v_c + cL;
  const T* __restrict__ t_c = a.t_c + cL;
  const T* __restrict__ dvgp = a.div + cL;
  const T sj = a.sinj[j], s2 = sj * sj, c2 = (T)1.0 - s2, c4 = c2 * c2, cj = a.cosj[j], fj = a.coriolis[j];
  const T sb = a.sb, R = a.R, kap = a.kap, cp = a.cp_t;
  const T kv0 = a.kv0, ka = a.ka, kt0 = a.kt0;
  const T ln_pref = (T)11.512925464970229;  // ln 1e5 (HS_Forcing.jl:49 p_ref)
  const T tDt = (T)a.Dt;
  const T ps = act ? a.ps_c[c1] : (T)1, psp = act ? a.ps_p[c1] : (T)0;
  // ∇ps / cos θ = (∇ ln ps / cos θ) ps (Spectral_Dynamics.jl:259-264)
  const T dlps = act ? a.dlps[c1] * ps : (T)0, dtps = act ? a.dtps[c1] * ps : (T)0;
  const T gs = act ? a.geopots[c1] : (T)0;
  // ---- pressure variables from ps_c (Pressure_Variables!, Press_And_Geopot.jl:36-67)
  const T lnps = log(ps);
  // the level's log-pressure differences: dlnp = ln p_{k+1/2} - ln p_{k-1/2} (k = 0: ln p_{3/2}),
  // dlpp = ln p_{k+1/2} - ln p_k, dlpm = ln p_k - ln p_{k-1/2} (k = 0: ln p_1), lnpf = ln p_k
  auto logs = [&](int k, T& dlnp, T& dlpp, T& dlpm, T& lnpf) {
    if constexpr (HYB) {
      const T plo = s_ak[k] + s_bk[k] * ps, phi = s_ak[k + 1] + s_bk[k + 1] * ps, dpk = phi - plo;
      const T lph = log(phi);
      if (k == 0) {
        dlnp = lph;
        dlpp = (T)1;
        lnpf = lph - (T)1;
        dlpm = lnpf;
      } else {
        dlnp = log1p(dpk / plo);
        dlpp = (T)1 - plo * dlnp / dpk;
        dlpm = dlnp - dlpp;
        lnpf = lph - dlpp;
      }
    } else {
      dlnp = k == 0 ? s_lb1 + lnps : s_dlp[k];
      dlpp = s_dlpp[k];
      lnpf = s_cf[k] + lnps;
      dlpm = k == 0 ? lnpf : s_dlpm[k];
    }
  };
  // ---- pass 1: Compute_Geopotential! (Press_And_Geopot.jl:71-111) on T - T0_k with T0_k the level's
  // area mean (spectral mode (0,0)): the T0 part is a per-level constant (dlnp_r, r >= 1, and dlnp_p
  // do not vary horizontally), so it only moves the (0,0) mode of the energy, which the Laplacian
  // annihilates, while the rounding of the sum shrinks with |T - T0|.  On the FP32 path T - T0_k is
  // read as synthesised without the (0,0) modes (a.tdev): T itself, stored in FP32 at ~264 K, keeps
  // only ~3e-5 K of it, and that rounding, through the Laplacian of the energy, set the divergence's
  // error (day-1 u, v errors against the FP64 oracle 8e-5, 5e-4 with T_c - T0_k formed here).  Also
  // the column sum of the mass divergence D_k.
  // Hybrid coordinates: dlnp_k and dlpp_k follow ps, so the T0 part is no per-level constant there;
  // it is summed on its own (rs0) and added back, keeping the anomaly sum's conditioning.
  const T* __restrict__ tdev = a.tdev ? a.tdev + cL : nullptr;
  T termS = 0, term0S = 0, dmeanS = 0;
  if (act)
    for (int k = k0; k < k1; k++) {
      const size_t x = (size_t)k * G;
      const T u = u_c[x], v = v_c[x], dvg = dvgp[x];
      const T t0 = (T)a.t_spec[e * nd + k].x;
      const T td = tdev ? tdev[x] : t_c[x] - t0;
      T dlnp, dlpp, dlpm, lnpf;
      logs(k, dlnp, dlpp, dlpm, lnpf);
      termS += R * td * dlnp;
      if constexpr (HYB) term0S += R * t0 * dlnp;
      dmeanS += dvg * (s_dak[k] + s_dbk[k] * ps) + s_dbk[k] * (u * dlps + v * dtps);
    }
  const T tot = seg_sum<S>(dmeanS);
  T rs = seg_excl_suffix<S>(termS, seg);  // sum_{r >= k1} R (T_r - T0_r) dlnp_r
  T rs0 = (T)0;
  if constexpr (HYB) rs0 = seg_excl_suffix<S>(term0S, seg);  // sum_{r >= k1} R T0_r dlnp_r
  const T incl0 = seg_excl_prefix<S>(dmeanS, seg);  // sum_{r < k0} D_r
  if (act)
    for (int k = k1 - 1; k >= k0; k--) {  // the energy Φ + |u|^2/2, bottom-up within the segment
      const size_t x = (size_t)k * G;
      const T u = u_c[x], v = v_c[x];
      const T t0 = (T)a.t_spec[e * nd + k].x;
      const T td = tdev ? tdev[x] : t_c[x] - t0;
      T dlnp, dlpp, dlpm, lnpf;
      logs(k, dlnp, dlpp, dlpm, lnpf);
      T en = gs + rs + R * td * dlpp + (T)0.5 * (u * u + v * v);
      if constexpr (HYB) {
        en += rs0 + R * t0 * dlpp;
        rs0 += R * t0 * dlnp;
      }
      a.energy[cL + x] = en;
      rs += R * td * dlnp;
    }
  // ---- pass 2, top-down within the segment
  // the column's energy integral (Compute_Corrections_Init): its kinetic part in the state precision,
  // its c_p T part (~99 % of it) to FP64 accuracy (on the FP32 path the state precision's rounding of
  // c_p T, the same at nearly every point of a near-uniform temperature, biased the energy correction
  // by up to 1e-6 K per step): FP64 sums of T_k Δa_k and T_k Δb_k on the FP64 path, the same sums as
  // FP32 pairs (error-free products and additions, ds_add_prod) on the FP32 path
  T col_e = 0;
  double col_ta = 0, col_tb = 0;
  float ah = 0, al = 0, bh = 0, bl = 0;
  if (act && k0 < k1) {
    T incl = incl0, Mlo = 0, flu = 0, flv = 0, flt = 0;  // M and the advective fluxes at k0-1/2
    T u = u_c[(size_t)k0 * G], v = v_c[(size_t)k0 * G], t = t_c[(size_t)k0 * G];
    T dp = s_dak[k0] + s_dbk[k0] * ps;
    if (k0 > 0) {  // the level above the segment: M_{k0-1/2} and its fluxes
      const size_t x = (size_t)(k0 - 1) * G;
      const T um = u_c[x], vm = v_c[x], tm = t_c[x], dpm = s_dak[k0 - 1] + s_dbk[k0 - 1] * ps;
      Mlo = -incl0 + tot * s_bk[k0];
      const T w = dpm / (dpm + dp);
      flu = Mlo * (um + (u - um) * w);
      flv = Mlo * (vm + (v - vm) * w);
      flt = Mlo * (tm + (t - tm) * w);
    }
    // the column's inputs and outputs through restrict-qualified pointers: no store of a level can
    // alias a load of the next, so the next level's loads may be issued before this level's stores
    const T* __restrict__ upp = a.u_p + cL;
    const T* __restrict__ vpp = a.v_p + cL;
    const T* __restrict__ tpp = a.t_p + cL;
    const T* __restrict__ vorp = a.vor + cL;
    const T* __restrict__ dlTp = a.dlT + cL;
    const T* __restrict__ dtTp = a.dtT + cL;
    T* __restrict__ o_du = a.ducos + cL;
    T* __restrict__ o_dv = a.dvcos + cL;
    T* __restrict__ o_dt = a.dtg + cL;
    T* __restrict__ o_teq = a.t_eq + cL;
    T* __restrict__ o_mh = a.m_half ? a.m_half + cL : nullptr;
    for (int k = k0; k < k1; k++) {
      const size_t x = (size_t)k * G;
      const T up = upp[x], vp = vpp[x], tp = tpp[x], dvg = dvgp[x], vor = vorp[x], dlT = dlTp[x], dtT = dtTp[x];
      const bool below = k + 1 < nd;
      T u1 = 0, v1 = 0, t1 = 0, dp1 = 1;
      if (below) {
        u1 = u_c[x + G];
        v1 = v_c[x + G];
        t1 = t_c[x + G];
        dp1 = s_dak[k + 1] + s_dbk[k + 1] * ps;
      }
      const T rdp = (T)1 / dp;
      T dlnp, dlnp_p, dlnp_m, lnpf;  // ln p_{k+1/2} - ln p_k, ln p_k - ln p_{k-1/2} (ln p_{1/2} = 0)
      logs(k, dlnp, dlnp_p, dlnp_m, lnpf);
      // HS_Forcing! on the previous level (sigma = p_k / ps: sf[k] in sigma coordinates)
      T sg;
      if constexpr (HYB) sg = exp(lnpf) / ps - sb;
      else sg = s_sf[k] - sb;
      const T smax = sg > (T)0 ? sg : (T)0;
      const T k_v = kv0 * smax;
      T du = -k_v * up, dv = -k_v * vp;
      T dt = -((up + (T)0.5 * du * tDt) * du + (vp + (T)0.5 * dv * tDt) * dv) / cp;
      const T lpn = lnpf - ln_pref;  // ln(p / p_ref)
      T teq = ((T)315.0 - a.dTy * s2 - a.dthz * c2 * lpn) * exp(a.kappa_t * lpn);
      teq = teq > (T)200.0 ? teq : (T)200.0;
      dt = dt - (ka + kt0 * smax * c4) * (tp - teq);
      // Compute_Corrections_Init: column energy integral with ps_p
      {
        const T ua = up + tDt * du, va = vp + tDt * dv;
        const T te = tp + tDt * dt;
        col_e += ((T)0.5 * (ua * ua + va * va)) * (s_dak[k] + s_dbk[k] * psp);
        if constexpr (std::is_same<T, float>::value) {
          if constexpr (HYB) ds_add_prod(ah, al, te, s_dah[k], s_dal[k]);  // Δa_k = 0 on sigma levels
          ds_add_prod(bh, bl, te, s_dbh[k], s_dbl[k]);
        } else {
          const double ted = (double)te;
          if (a.has_dak) col_ta += ted * s_dak64[k];
          col_tb += ted * s_dbk64[k];
        }
      }
      // Four_In_One! (Spectral_Dynamics.jl:88-183)
      const T x1 = (s_bk[k] * dlnp_m + s_bk[k + 1] * dlnp_p) * rdp;
      const T dlnp_dl = x1 * dlps, dlnp_dt = x1 * dtps;
      du = du - R * t * dlnp_dl;
      dv = dv - R * t * dlnp_dt;
      const T dmean = dvg * dp + s_dbk[k] * (u * dlps + v * dtps);
      const T excl = incl;
      incl += dmean;
      const T x5 = -(excl * dlnp + dmean * dlnp_p) * rdp + u * dlnp_dl + v * dlnp_dt;
      dt = dt + kap * t * x5;
      // M_{k+1/2} = -sum_{r<=k} D_r + B_{k+1/2} sum_r D_r, zero at the surface
      const T Mhi = below ? -incl + tot * s_bk[k + 1] : (T)0;
      if (o_mh) o_mh[x] = Mhi;
      // Vert_Advection! (second_centered_wts): flux at k+1/2 with weight dp_k / (dp_k + dp_{k+1})
      const T w1 = dp / (dp + dp1);
      const T fhu = below ? Mhi * (u + (u1 - u) * w1) : (T)0;
      const T fhv = below ? Mhi * (v + (v1 - v) * w1) : (T)0;
      const T fht = below ? Mhi * (t + (t1 - t) * w1) : (T)0;
      du = du + (flu - fhu + u * (Mhi - Mlo)) * rdp;
      dv = dv + (flv - fhv + v * (Mhi - Mlo)) * rdp;
      dt = dt + (flt - fht + t * (Mhi - Mlo)) * rdp;
      // Add_Horizontal_Advection!(spe_t_c), Compute_Abs_Vor! fluxes
      dt = dt - (u * dlT + v * dtT);
      const T absvor = vor + fj;
      du = du + absvor * v;
      dv = dv - absvor * u;
      o_du[x] = du * cj;
      o_dv[x] = dv * cj;
      o_dt[x] = dt;
      o_teq[x] = teq;
      Mlo = Mhi;
      flu = fhu;
      flv = fhv;
      flt = fht;
      u = u1;
      v = v1;
      t = t1;
      dp = dp1;
    }
  }
  if constexpr (std::is_same<T, float>::value) {
    col_ta = (double)ah + (double)al;
    col_tb = (double)bh + (double)bl;
  }
  double col_ed = (double)col_e + a.cp * (col_ta + col_tb * (double)psp);
  col_ed = seg_sum<S>(col_ed);
  double accp = 0.0, acce = 0.0;
  if (act && seg == 0) {
    a.dlnps[c1] = (-tot) / ps;  // grid_δlnps = grid_δps / ps (Spectral_Dynamics.jl:279)
    accp = (double)psp;
    acce = col_ed;
  }
  // ---- block partials for mean_ps_p and mean_energy_p (fixed order), then the member's fold;
  // only lanes with seg = 0 hold values, so the butterfly stops at offset S (the skipped levels
  // would add exact zeros)
#pragma unroll
  for (int o = 16; o >= S; o >>= 1) {
    accp += __shfl_xor_sync(FULL, accp, o);
    acce += __shfl_xor_sync(FULL, acce, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = accp;
    red[1][threadIdx.x >> 5] = acce;
  }
  __syncthreads();
  double vals[2] = {0, 0};
  if (threadIdx.x == 0)
    for (int q = 0; q < HS_CT / 32; q++) {
      vals[0] += red[0][q];
      vals[1] += red[1][q];
    }
  // the block partials only: the fixer reduction, their one consumer, folds them (its last block), so
  // no grid-wide fold sits at this kernel's end
  if (threadIdx.x == 0) {
    const int nb = gridDim.x * gridDim.y, bid = blockIdx.y * gridDim.x + blockIdx.x;
    double* p = a.partials + e * a.pstride;
    p[bid] = vals[0];
    p[(size_t)nb + bid] = vals[1];
  }
}

// Passive tracers, advected like T (the reference keeps spe_tracers / grid_tracers in Dyn_Data,
// Dyn_Data.jl:36-39,63-66, and rotates them, but its Spectral_Dynamics! leaves "grid_q = grid_t" as
// a todo, :235): per column and tracer, top-down, Vert_Advection! (second_centered_wts,
// Vert_Coordinate.jl:171-210) with the column kernel's mass flux M_{k+1/2}, the flux at k+1/2
// carried to the next level as for T, then Add_Horizontal_Advection! (Spectral_Spherical_Mesh.jl:
// 694-718) with the synthesised gradients.  No forcing, no semi-implicit term.
template <typename T>
struct TracerArgs {
  const T *u_c, *v_c, *ps_c, *q_c, *dlq, *dtq, *m_half;
  T* dq;
  int nd, nq, nlat, nlon;
};

template <typename T>
__global__ void __launch_bounds__(128) k_hs_tracers(TracerArgs<T> a, const VertCoef* __restrict__ vcp) {
  const VertCoef& vc = *vcp;
  __shared__ T s_dak[JGCM_MAX_ND], s_dbk[JGCM_MAX_ND];
  const int nd = a.nd;
  for (int q = threadIdx.x; q < nd; q += blockDim.x) {
    s_dak[q] = (T)vc.dak[q];
    s_dbk[q] = (T)vc.dbk[q];
  }
  __syncthreads();
  pdl_wait();  // programmatic dependent launch: the column kernel's mass flux is complete
  const int i = blockIdx.x * blockDim.x + threadIdx.x, j = blockIdx.y, e = blockIdx.z;
  if (i >= a.nlon) return;
  const size_t G = (size_t)a.nlat * a.nlon, col = (size_t)j * a.nlon + i, cL = (size_t)e * nd * G + col;
  const T ps = a.ps_c[(size_t)e * G + col];
  for (int iq = 0; iq < a.nq; iq++) {
    const size_t cQ = (size_t)(e * a.nq + iq) * nd * G + col;
    T Mlo = 0, flq = 0, q = a.q_c[cQ], dp = s_dak[0] + s_dbk[0] * ps;
    for (int k = 0; k < nd; k++) {
      const size_t x = (size_t)k * G;
      const bool below = k + 1 < nd;
      T q1 = 0, dp1 = 1;
      if (below) {
        q1 = a.q_c[cQ + x + G];
        dp1 = s_dak[k + 1] + s_dbk[k + 1] * ps;
      }
      const T rdp = (T)1 / dp;
      const T Mhi = below ? a.m_half[cL + x] : (T)0;
      const T w1 = dp / (dp + dp1);
      const T fhq = below ? Mhi * (q + (q1 - q) * w1) : (T)0;
      T d = (flq - fhq + q * (Mhi - Mlo)) * rdp;
      d = d - (a.u_c[cL + x] * a.dlq[cQ + x] + a.v_c[cL + x] * a.dtq[cQ + x]);
      a.dq[cQ + x] = d;
      Mlo = Mhi;
      flq = fhq;
      q = q1;
      dp = dp1;
    }
  }
}

// lanes per column for a launch: S = 4 for small grids (latency), 1 for large ensembles; the
// autotuner may pick 8
inline int hs_lanes(const jgcm_mesh* m, int ne, int nd) {
  const size_t cols = (size_t)ne * m->nlat * m->nlon;
  int S = cols >= 65536 ? 1 : cols >= 32768 ? 2 : 4;
  while (S > 1 && (nd + S - 1) / S < 2) S >>= 1;
  return S;
}

template <typename T, bool HYB>
int launch_hs_column_v(const HSColArgs<T>& a, const jgcm_mesh* m, int ne, int S, const VertCoef* vc, cudaStream_t st) {
  const int cpb = HS_CT / S;  // columns per block
  dim3 g((m->nlon + cpb - 1) / cpb, m->nlat, ne);
  if (S == 1) JG_CUDA(launch_pdl(k_hs_column<T, 1, HYB>, g, HS_CT, 0, st, a, vc));
  else if (S == 2) JG_CUDA(launch_pdl(k_hs_column<T, 2, HYB>, g, HS_CT, 0, st, a, vc));
  else if (S == 4) JG_CUDA(launch_pdl(k_hs_column<T, 4, HYB>, g, HS_CT, 0, st, a, vc));
  else JG_CUDA(launch_pdl(k_hs_column<T, 8, HYB>, g, HS_CT, 0, st, a, vc));
  return JGCM_OK;
}
template <typename T>
int launch_hs_column(const HSColArgs<T>& a, const jgcm_mesh* m, int ne, int S, const VertCoef* vc, bool hybrid,
                     cudaStream_t st) {
  return hybrid ? launch_hs_column_v<T, true>(a, m, ne, S, vc, st) : launch_hs_column_v<T, false>(a, m, ne, S, vc, st);
}

// ------------------------------------------------------------------------------------------
// Semi-implicit correction (Adjust_δlnps_δt_δdiv! + Implicit_Correction!, Semi_Implicit.jl:
// 271-513) followed by Compute_Spectral_Damping! and Filtered_Leapfrog! for vor, div, T, lnps
// (Spectral_Dynamics.jl:313-327).  One warp per spectral mode (m,n), lane = level.  The
// per-n solve with W_n = (I - ξ² ∇²_n D)^{-1} runs in FP64; the linearised vertical operators
// and the time filter run in the state precision T (FP64 on the FP64 path).
template <typename T>
struct ImplArgs {
  const V2<T>*dvor, *ddiv, *dtend, *dlnps;  // spectral tendencies from the analysis
  V2<T> *vor_p, *vor_c, *vor_n, *div_p, *div_c, *div_n, *t_p, *t_c, *t_n, *lnps_p, *lnps_c, *lnps_n;
  const T *damping, *dfac;  // [m][n]: damping, 1/(1 + Δt' damping) for this step
  const double* eig64;      // [m][n]: -n(n+1)/a², FP64
  const double* W;                // [N+1][c][r]
  const int2* pairs;
  int npairs, nd, L, ne, ns, N, init_step, dt;  // spectral innermost index e*nd + k of L = ne*nd
  double xi, ps_ref, kappa, rdgas, robert;
  // the same scalars rounded to T on the host (no FP64 division or conversion per thread), and the
  // Laplacian eigenvalues in T
  const T* eig_t;
  T xi_t, rpsr_t, xipsr_t, kap_t, rg_t, rob_t;
  // passive tracers: tendency, p/c/n levels (innermost index (e nq + i) nd + k of LQ = ne nq nd)
  const V2<T>* dq;
  V2<T> *q_p, *q_c, *q_n;
  int nq, LQ;
};

template <typename T>
void impl_consts(ImplArgs<T>& a, const T* eig_t) {
  a.eig_t = eig_t;
  a.xi_t = (T)a.xi;
  a.rpsr_t = (T)(1.0 / a.ps_ref);
  a.xipsr_t = (T)(a.xi / a.ps_ref);
  a.kap_t = (T)a.kappa;
  a.rg_t = (T)a.rdgas;
  a.rob_t = (T)a.robert;
}

template <typename R>
struct CX {
  R x, y;
};

// Linear_Ps_T_δdiv! (Semi_Implicit.jl:271-341) for one (m,n) column held one level per lane.
// The semi-implicit kernel's per-level reference-column constants in the vertical-algebra precision R,
// staged once per block (the same FP64 expressions, rounded once instead of in every warp)
template <typename R>
struct VertR {
  R dpr[JGCM_MAX_ND], rdpr[JGCM_MAX_ND], dlnp[JGCM_MAX_ND], dlnpp[JGCM_MAX_ND], tref[JGCM_MAX_ND],
      bk1[JGCM_MAX_ND], tdh[JGCM_MAX_ND], dh[JGCM_MAX_ND], df[JGCM_MAX_ND], hk[JGCM_MAX_ND];
};

template <typename R>
__device__ __forceinline__ void stage_vert(const VertCoef& vc, int nd, double ps_ref, VertR<R>& v) {
  for (int k = threadIdx.x; k < nd; k += blockDim.x) {
    v.dpr[k] = (R)vc.dp_ref[k];
    v.rdpr[k] = (R)vc.rdp_ref[k];
    v.dlnp[k] = (R)(vc.lnph_ref[k + 1] - vc.lnph_ref[k]);
    v.dlnpp[k] = (R)(vc.lnph_ref[k + 1] - vc.lnpf_ref[k]);
    v.tref[k] = (R)vc.t_ref[k];
    v.bk1[k] = (R)vc.bk[k + 1];
    v.tdh[k] = k + 1 <= nd - 1 ? (R)(vc.t_ref[k + 1] - vc.t_ref[k]) : (R)0;
    v.dh[k] = (R)(vc.lnph_ref[k + 1] - vc.lnph_ref[k]);
    v.df[k] = (R)(vc.lnph_ref[k + 1] - vc.lnpf_ref[k]);
    v.hk[k] = (R)(vc.h[k] * ps_ref);
  }
}

template <typename R>
__device__ __forceinline__ void linear_ps_t(const VertR<R>& vr, int lane, int nd, R kappa, CX<R> d, CX<R>& dps,
                                            CX<R>& dtt) {
  const bool act = lane < nd;
  const int k = act ? lane : 0;
  const R dpr = vr.dpr[k], rdpr = vr.rdpr[k];
  CX<R> dm = {act ? d.x * dpr : (R)0, act ? d.y * dpr : (R)0};
  R ix = scan_incl<R>(dm.x, lane), iy = scan_incl<R>(dm.y, lane);
  R tx = __shfl_sync(FULL, ix, nd - 1), ty = __shfl_sync(FULL, iy, nd - 1);
  R ex = shfl_up1(ix, lane, (R)0), ey = shfl_up1(iy, lane, (R)0);
  R dlnp = vr.dlnp[k], dlnp_p = vr.dlnpp[k];
  R c = -kappa * vr.tref[k];
  dtt.x = c * (ex * dlnp + dm.x * dlnp_p) * rdpr;
  dtt.y = c * (ey * dlnp + dm.y * dlnp_p) * rdpr;
  // M_{k+1/2} (k <= nd-2) and the centred vertical-advection term with (t_ref[k] - t_ref[k-1])
  const bool inner = lane + 1 <= nd - 1;
  R bk1 = vr.bk1[k];
  R mhx = inner ? -ix + tx * bk1 : (R)0, mhy = inner ? -iy + ty * bk1 : (R)0;
  R tdh = inner ? vr.tdh[k] : (R)0;
  R mdhx = mhx * tdh, mdhy = mhy * tdh;  // Mdt_{k+1/2}
  R mdlx = shfl_up1(mdhx, lane, (R)0), mdly = shfl_up1(mdhy, lane, (R)0);
  dtt.x = dtt.x - (R)0.5 * (mdhx + mdlx) * rdpr;
  dtt.y = dtt.y - (R)0.5 * (mdhy + mdly) * rdpr;
  dps.x = -tx;
  dps.y = -ty;
}

// Compute_Spectral_Damping! + Filtered_Leapfrog! (Time_Integrator.jl:58-101); f = 1/(1 + Δt' d).
template <typename R>
__device__ __forceinline__ void lf(int init, int Dt, R rob, R d, R f, R& dq, R qp, R& qc, R& qn) {
  if (init) {
    dq = (dq - qc * d) * f;
    qn = qc + (R)Dt * dq;
    qc = qc + rob * ((R)-1.0 * qc + qn);
  } else {
    dq = (dq - qp * d) * f;
    qc = qc + rob * (qp - (R)2 * qc);
    qn = qp + (R)(2 * Dt) * dq;
    qc = qc + rob * qn;
  }
}

// R is the precision of the vertical algebra (FP64 on the FP64 path; selectable on the FP32 path).
// DENSE: the FP64 wave-matrix products of the block's modes are spread over all its threads, one
// (mode, component, row) output each, instead of one mode per warp, whose 32 - nd idle lanes the
// FP64 pipe executes all the same (for launches with many modes: member ensembles).
template <typename T, typename R, bool DENSE = false>
__global__ void __launch_bounds__(256) k_hs_implicit(ImplArgs<T> a, const VertCoef* __restrict__ vcp) {
  const VertCoef& vc = *vcp;
  __shared__ VertR<R> vr;
  stage_vert<R>(vc, a.nd, a.ps_ref, vr);  // constants: staged before the dependency wait
  __syncthreads();
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using C = CX<R>;
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const int pid = blockIdx.x * nw + w;  // one (m, n) mode per warp
  const bool live = pid < a.npairs;     // warp-uniform
  if (!DENSE && !live) return;          // whole warp exits together (no block barrier follows)
  const int2 mn = live ? a.pairs[pid] : make_int2(0, 0);  // DENSE: a spare warp only meets the barriers
  const int m = mn.x, n = mn.y, nd = a.nd, e = blockIdx.y;
  const bool act = lane < nd;
  const int k = act ? lane : 0;
  const size_t row = (size_t)m * (a.ns + 1) + n;
  const size_t s = row * a.L + (size_t)e * nd + k, s1 = row * a.ne + e;  // nd-level and single-level index
  auto ld = [&](const V2<T>* p) -> C {
    if (!act) return C{0, 0};
    V2<T> v = p[s];
    return C{(R)v.x, (R)v.y};
  };
  C ddiv = ld(a.ddiv), dtt = ld(a.dtend), dvor = ld(a.dvor);
  C divp = ld(a.div_p), divc = ld(a.div_c), tp = ld(a.t_p), tc = ld(a.t_c), vorp = ld(a.vor_p), vorc = ld(a.vor_c);
  V2<T> l0 = a.dlnps[s1], lp0 = a.lnps_p[s1], lc0 = a.lnps_c[s1];
  C dl = {(R)l0.x, (R)l0.y}, lp = {(R)lp0.x, (R)lp0.y}, lc = {(R)lc0.x, (R)lc0.y};
  const R xi = (R)a.xi_t, rpsr = (R)a.rpsr_t, xipsr = (R)a.xipsr_t, eig = (R)a.eig_t[row];
  const R kap = (R)a.kap_t, Rg = (R)a.rg_t;
  // Adjust_δlnps_δt_δdiv! :360-404
  C dps, dtmp;
  linear_ps_t<R>(vr, lane, nd, kap, C{divp.x - divc.x, divp.y - divc.y}, dps, dtmp);
  dtt.x = dtt.x + dtmp.x;
  dtt.y = dtt.y + dtmp.y;
  dl.x = dl.x + dps.x * rpsr;
  dl.y = dl.y + dps.y * rpsr;
  C t2 = {tp.x - tc.x + xi * dtt.x, tp.y - tc.y + xi * dtt.y};
  C l2 = {lp.x - lc.x + xi * dl.x, lp.y - lc.y + xi * dl.y};
  // Linear_Geopot_δt! :213-241
  R dh = vr.dh[k];
  R tmx = act ? Rg * (t2.x * dh) : (R)0, tmy = act ? Rg * (t2.y * dh) : (R)0;
  R rx = rscan_incl<R>(tmx, lane), ry = rscan_incl<R>(tmy, lane);
  R hx = shfl_dn1(rx, lane, nd, (R)0), hy = shfl_dn1(ry, lane, nd, (R)0);  // Φ_{k+1/2}
  R df = vr.df[k];
  R gx = hx + Rg * (t2.x * df), gy = hy + Rg * (t2.y * df);
  R hk = vr.hk[k];
  ddiv.x = ddiv.x - eig * (gx + hk * l2.x);
  ddiv.y = ddiv.y - eig * (gy + hk * l2.y);
  // wave-matrix solve in FP64, n <= N only (Implicit_Correction! :486-497)
  if (DENSE) {
    __shared__ double s_b[8][2][JGCM_MAX_ND], s_o[8][2][JGCM_MAX_ND];
    if (act) {
      s_b[w][0][k] = (double)ddiv.x;
      s_b[w][1][k] = (double)ddiv.y;
    }
    __syncthreads();
    // outputs o = (mode, component, row); the block's first output rotates with the block so that
    // the remainder past a multiple of the block size falls on every warp in turn
    const int nout = nw * 2 * nd, o0 = (int)((blockIdx.x * 32u) % (unsigned)blockDim.x);
    for (int t = threadIdx.x; t < nout; t += blockDim.x) {
      const int o = (t + o0) % nout;
      const int wq = o / (2 * nd), rem = o - wq * 2 * nd, cq = rem / nd, rw = rem - cq * nd;
      const int pq = blockIdx.x * nw + wq;
      if (pq < a.npairs) {
        const int nq = a.pairs[pq].y;
        if (nq <= a.N) {
          const double* W = a.W + (size_t)nq * nd * nd;
          double acc = 0;  // the same products in the same order as the per-warp form below
#pragma unroll 4
          for (int c = 0; c < nd; c++) acc = acc + W[(size_t)c * nd + rw] * s_b[wq][cq][c];
          s_o[wq][cq][rw] = acc;
        }
      }
    }
    __syncthreads();
    if (n <= a.N) {
      ddiv.x = act ? (R)s_o[w][0][k] : (R)0;
      ddiv.y = act ? (R)s_o[w][1][k] : (R)0;
    }
  } else if (n <= a.N) {
    const double* W = a.W + (size_t)n * nd * nd;
    const double bxl = (double)ddiv.x, byl = (double)ddiv.y;
    double sx = 0, sy = 0;
    // row k of W_n in chunks of 8 (8 loads in flight; the whole row would hold 64 registers and
    // cost the kernel occupancy it needs to overlap its FP32 scans with other warps' FP64 products)
    for (int c0 = 0; c0 < nd; c0 += 8) {  // nd is warp-uniform
      double wv[8];
#pragma unroll
      for (int cc = 0; cc < 8; cc++) wv[cc] = (act && c0 + cc < nd) ? W[(size_t)(c0 + cc) * nd + k] : 0.0;
#pragma unroll
      for (int cc = 0; cc < 8; cc++) {
        if (c0 + cc < nd) {
          double bx = __shfl_sync(FULL, bxl, c0 + cc), by = __shfl_sync(FULL, byl, c0 + cc);
          sx = sx + wv[cc] * bx;
          sy = sy + wv[cc] * by;
        }
      }
    }
    ddiv.x = act ? (R)sx : (R)0;
    ddiv.y = act ? (R)sy : (R)0;
  }
  linear_ps_t<R>(vr, lane, nd, kap, ddiv, dps, dtmp);
  dtt.x = dtt.x + xi * dtmp.x;
  dtt.y = dtt.y + xi * dtmp.y;
  dl.x = dl.x + xipsr * dps.x;
  dl.y = dl.y + xipsr * dps.y;
  // damping + leapfrog
  const R d = (R)a.damping[row], f = (R)a.dfac[row], rob = (R)a.rob_t;
  const int ini = a.init_step, Dt = a.dt;
  if (live && act) {
    C vn, dn, tn;
    lf<R>(ini, Dt, rob, d, f, dvor.x, vorp.x, vorc.x, vn.x);
    lf<R>(ini, Dt, rob, d, f, dvor.y, vorp.y, vorc.y, vn.y);
    lf<R>(ini, Dt, rob, d, f, ddiv.x, divp.x, divc.x, dn.x);
    lf<R>(ini, Dt, rob, d, f, ddiv.y, divp.y, divc.y, dn.y);
    lf<R>(ini, Dt, rob, d, f, dtt.x, tp.x, tc.x, tn.x);
    lf<R>(ini, Dt, rob, d, f, dtt.y, tp.y, tc.y, tn.y);
    V2<T> o;
    o.x = (T)vn.x; o.y = (T)vn.y; a.vor_n[s] = o;
    o.x = (T)vorc.x; o.y = (T)vorc.y; a.vor_c[s] = o;
    o.x = (T)dn.x; o.y = (T)dn.y; a.div_n[s] = o;
    o.x = (T)divc.x; o.y = (T)divc.y; a.div_c[s] = o;
    o.x = (T)tn.x; o.y = (T)tn.y; a.t_n[s] = o;
    o.x = (T)tc.x; o.y = (T)tc.y; a.t_c[s] = o;
  }
  if (live && lane == 0) {  // lnps: leapfrog without damping (d = 0, f = 1)
    C ln;
    lf<R>(ini, Dt, rob, (R)0, (R)1, dl.x, lp.x, lc.x, ln.x);
    lf<R>(ini, Dt, rob, (R)0, (R)1, dl.y, lp.y, lc.y, ln.y);
    V2<T> o;
    o.x = (T)ln.x; o.y = (T)ln.y; a.lnps_n[s1] = o;
    o.x = (T)lc.x; o.y = (T)lc.y; a.lnps_c[s1] = o;
  }
  // passive tracers: damping and the filtered leapfrog of T (Time_Integrator.jl:58-101)
  if (live && act)
    for (int iq = 0; iq < a.nq; iq++) {
      const size_t sq = row * a.LQ + (size_t)(e * a.nq + iq) * nd + k;
      const V2<T> g = a.dq[sq], qp0 = a.q_p[sq], qc0 = a.q_c[sq];
      C dq = {(R)g.x, (R)g.y}, qp = {(R)qp0.x, (R)qp0.y}, qc = {(R)qc0.x, (R)qc0.y}, qn;
      lf<R>(ini, Dt, rob, d, f, dq.x, qp.x, qc.x, qn.x);
      lf<R>(ini, Dt, rob, d, f, dq.y, qp.y, qc.y, qn.y);
      V2<T> o;
      o.x = (T)qn.x; o.y = (T)qn.y; a.q_n[sq] = o;
      o.x = (T)qc.x; o.y = (T)qc.y; a.q_c[sq] = o;
    }
}

// ------------------------------------------------------------------------------------------
// Compute_Corrections! (Spectral_Dynamics.jl:30-68): FP64 sums of ps_n and of the column
// energy (split into the Δa and Δb·ps parts so the mass correction can be applied after the
// sum), then the spectral (m,n)=(0,0) fixes in the last block.  k_hs_corr_apply follows.
template <typename T>
struct CorrArgs {
  const T *u_n, *v_n, *t_n, *ps_n;
  V2<T>*lnps_n, *t_spec_n;
  const double* wts;
  double *partials, *scalars;  // per member: partials + e * pstride, scalars + 4 e
  T* scal_t;                   // per member: factor and correction rounded to T (for k_hs_corr_apply)
  unsigned* counter;           // per member: corr_groups(nb) + 1 tickets
  size_t pstride;
  // the column kernel's block partials (ps_p and the column energy of the previous level) at the
  // start of the member's region, its grid (col_gx x nlat blocks); this kernel's block values at
  // col_off (3 x nb, the group form), the first level's units' values after them (5 x the units)
  int col_gx, col_nb;
  size_t col_off;
  int nd, nlat, nlon, do_mass, do_energy;
  int has_dak;  // some a_k differs between levels: the energy sums need sum_k T_k Δa_k
  double cp, grav;
  double inv_2n;  // 1 / (2 nlon), exact (nlon is a power of two)
  T cp_t;         // cp rounded to T on the host
  float cp_hi, cp_lo;  // cp as an FP32 pair (hi its rounding, lo that of the remainder)
};

// The sums, every one weighted by the Gaussian weight of its latitude row:
//   S0 = Σ ps_n,  S1 = Σ Σ_k E_k Δa_k,  S2 = Σ ps_n Σ_k E_k Δb_k  (E = |u|²/2 + c_p T of level n)
//   S3 = Σ ps_p,  S4 = Σ Σ_k E_k Δp_k of level p  (the column kernel's partials)
// mean_ps = S / (2 nlon) (Area_Weighted_Global_Mean), mean_energy = S / (2 nlon g)
// (Mass_Weighted_Global_Integral); factor = mean_ps_p / mean_ps_n = S3 / S0, and with Δp_k =
// Δa_k + Δb_k factor ps_n the correction grav (mean_energy_p - mean_energy_n) / (c_p mean_ps_p)
// = (S4 - S1 - factor S2) / (c_p S3).
// Unit u's share (of nu) of the column kernel's block partials of sum v (0: ps_p, 1: the column
// energy of level p), each weighted by its row; every lane returns the share
template <typename T>
__device__ __forceinline__ double corr_col_share(const CorrArgs<T>& a, const double* pe, int v, int u, int nu,
                                                 int lane) {
  const int per = (a.col_nb + nu - 1) / nu, q0 = u * per, q1 = min(a.col_nb, q0 + per);
  const double* cp_ = pe + (size_t)v * a.col_nb;
  double s = 0.0;
  for (int q = q0 + lane; q < q1; q += 32) s += __ldcg(cp_ + q) * a.wts[q / a.col_gx];
  return warp_sum(s);
}

// CL: the first fold level in thread-block clusters (launched with a cluster shape), else in
// groups of CORR_GS blocks
template <typename T, bool CL>
__global__ void __launch_bounds__(256) k_hs_corr_reduce(CorrArgs<T> a, const VertCoef* __restrict__ vcp) {
  const VertCoef& vc = *vcp;
  // block = 32 consecutive columns of one latitude row x 8 level groups: warp ks reads levels
  // ks, ks + 8, ... of the 32 columns (coalesced rows)
  constexpr int KS = 8;
  __shared__ T s_dak[JGCM_MAX_ND], s_dbk[JGCM_MAX_ND];  // the layer coefficients in the state precision
  __shared__ double s_dak64[JGCM_MAX_ND], s_dbk64[JGCM_MAX_ND];  // and in FP64 (the c_p T sums)
  __shared__ float s_dah[JGCM_MAX_ND], s_dal[JGCM_MAX_ND], s_dbh[JGCM_MAX_ND], s_dbl[JGCM_MAX_ND];  // FP32 pairs
  for (int q = threadIdx.x; q < a.nd; q += blockDim.x) {
    s_dak[q] = (T)vc.dak[q];
    s_dbk[q] = (T)vc.dbk[q];
    s_dak64[q] = vc.dak[q];
    s_dbk64[q] = vc.dbk[q];
    s_dah[q] = vc.dak_hi[q];
    s_dal[q] = vc.dak_lo[q];
    s_dbh[q] = vc.dbk_hi[q];
    s_dbl[q] = vc.dbk_lo[q];
  }
  __syncthreads();
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  const int lane = threadIdx.x & 31, ks = threadIdx.x >> 5, j = blockIdx.y, nd = a.nd;
  const int i = blockIdx.x * 32 + lane, e = blockIdx.z;  // e: member
  const bool act = i < a.nlon;
  const size_t G = (size_t)a.nlat * a.nlon, col = (size_t)j * a.nlon + (act ? i : 0);
  const size_t offL = (size_t)e * nd * G, off1 = (size_t)e * G;
  // the energy integrals sum_k E_k Δa_k, sum_k E_k Δb_k (E = |u|²/2 + c_p T): the kinetic part in
  // the state precision, the c_p T part (~99 %) to FP64 accuracy (the state precision's rounding of
  // c_p T biased the energy correction by up to 1e-6 K per step): FP64 sums of the products T_k Δa_k,
  // T_k Δb_k on the FP64 path; on the FP32 path the same sums as FP32 pairs (error-free products
  // against Δ_hi + Δ_lo, error-free additions), each column's pair converted to FP64 once
  __shared__ double part[2][KS][32];
  __shared__ float pk[2][KS][32], ph[2][KS][32], pl[2][KS][32];  // FP32 path: kinetic; c_p T part as hi + lo
  if constexpr (std::is_same<T, float>::value) {
    float ea = 0, eb = 0, ah = 0, al = 0, bh = 0, bl = 0;
    if (act) {
#pragma unroll 4  // nd <= 32: every level's loads in flight together
      for (int k = ks; k < nd; k += KS) {
        const size_t x = offL + (size_t)k * G + col;
        const float u = a.u_n[x], v = a.v_n[x], t = a.t_n[x];
        const float K = 0.5f * (u * u + v * v);
        ea += K * s_dak[k];
        eb += K * s_dbk[k];
        if (a.has_dak) ds_add_prod(ah, al, t, s_dah[k], s_dal[k]);
        ds_add_prod(bh, bl, t, s_dbh[k], s_dbl[k]);
      }
    }
    pk[0][ks][lane] = ea;
    pk[1][ks][lane] = eb;
    ph[0][ks][lane] = ah;
    pl[0][ks][lane] = al;
    ph[1][ks][lane] = bh;
    pl[1][ks][lane] = bl;
    __syncthreads();
    if (ks == 1 || ks == 2) {  // the level groups of this lane's column, in order, then FP64 once
      const int w = ks - 1;
      float kh = 0, kl = 0, th = 0, tl = 0;
      for (int q = 0; q < KS; q++) {
        ds_add(kh, kl, pk[w][q][lane]);
        ds_add(th, tl, ph[w][q][lane]);
        tl = __fadd_rn(tl, pl[w][q][lane]);
      }
      // E = K + c_p T as a pair: c_p (th + tl) with c_p = cp_hi + cp_lo, the product th cp_hi
      // error-free, the small cross terms rounded
      const float p = __fmul_rn(th, a.cp_hi), pe = __fmaf_rn(th, a.cp_hi, -p);
      float eh = kh, el = kl;
      ds_add(eh, el, p);
      el = __fadd_rn(el, __fadd_rn(pe, __fmaf_rn(th, a.cp_lo, __fmul_rn(tl, a.cp_hi))));
      ph[w][0][lane] = eh;  // this warp's own row of the staging arrays, read back below
      pl[w][0][lane] = el;
    }
  } else {
    T ea = 0, eb = 0;
    double ta = 0, tb = 0;
    if (act) {
#pragma unroll 4
      for (int k = ks; k < nd; k += KS) {
        const size_t x = offL + (size_t)k * G + col;
        const T u = a.u_n[x], v = a.v_n[x];
        const double t = (double)a.t_n[x];
        const T K = (T)0.5 * (u * u + v * v);
        ea += K * s_dak[k];
        eb += K * s_dbk[k];
        if (a.has_dak) ta += t * s_dak64[k];
        tb += t * s_dbk64[k];
      }
    }
    part[0][ks][lane] = (double)ea + a.cp * ta;
    part[1][ks][lane] = (double)eb + a.cp * tb;
    __syncthreads();
    if (ks == 1 || ks == 2) {  // the level groups of this lane's column (each lane its own column)
      double sq = 0;
      for (int q = 0; q < KS; q++) sq += part[ks - 1][q][lane];
      part[ks - 1][0][lane] = sq;
    }
  }
  // block values S0, S1, S2 (one warp each, on three sub-partitions): the level groups of each
  // column, the butterfly over the columns, the row's weight
  const int nb = gridDim.x * gridDim.y, bid = blockIdx.y * gridDim.x + blockIdx.x, ng = corr_groups(nb);
  double* const pe = a.partials + e * a.pstride;
  unsigned* const ctr = a.counter + (size_t)e * (ng + 1);
  int rank = 0, nu, u;  // the first level's units (clusters or groups) and this block's unit
  if constexpr (CL) {
    const dim3 cd = cg::this_cluster().dim_blocks();
    rank = (int)cg::this_cluster().block_rank();
    const int gcx = gridDim.x / cd.x;
    nu = gcx * (gridDim.y / cd.y);
    u = (blockIdx.y / cd.y) * gcx + blockIdx.x / cd.x;
  } else {
    nu = ng;
    u = bid / CORR_GS;
  }
  double* const bpart = pe + a.col_off;           // [3][nb] (groups)
  double* const upart = bpart + (size_t)3 * nb;  // [5][nu]
  __shared__ double s_bv[3];                      // this block's values (clusters)
  double x = 0.0;
  if (ks < 3) {
    const T ps = act ? a.ps_n[off1 + col] : (T)0;
    if constexpr (std::is_same<T, float>::value) {
      // the butterfly over the block's 32 columns on FP32 pairs (error-free additions), one FP64
      // conversion per block value
      float h = ps, l = 0.f;
      if (ks > 0) {
        h = ph[ks - 1][0][lane];
        l = pl[ks - 1][0][lane];
        if (ks == 2) {  // (h + l) ps, the product h ps error-free
          const float p = __fmul_rn(h, ps), pe = __fmaf_rn(h, ps, -p);
          l = __fadd_rn(pe, __fmul_rn(l, ps));
          h = p;
        }
      }
#pragma unroll
      for (int o = 16; o >= 1; o >>= 1) {
        const float h2 = __shfl_xor_sync(FULL, h, o), l2 = __shfl_xor_sync(FULL, l, o);
        ds_add(h, l, h2);
        l = __fadd_rn(l, l2);
      }
      x = (double)h + (double)l;
    } else {
      const double colsum = ks > 0 ? part[ks - 1][0][lane] : 0.0;  // written by this warp above
      x = ks == 0 ? (double)ps : ks == 1 ? colsum : colsum * (double)ps;
      x = warp_sum(x);
    }
    x *= a.wts[j];
    if (lane == 0) {
      if constexpr (CL)
        s_bv[ks] = x;
      else
        __stcg(bpart + (size_t)ks * nb + bid, x);  // released by ticket_last
    }
  } else if (CL && ks < 5 && rank == 0) {
    x = corr_col_share(a, pe, ks - 3, u, nu, lane);  // the leader's share, while the others finish
  }
  // first level
  if constexpr (CL) {
    // every thread of every block of the cluster reaches both cluster barriers (no return before
    // them): the first releases the blocks' values to the leader, the second keeps the blocks
    // resident until the leader has read them
    cg::cluster_group cl = cg::this_cluster();
    cl.sync();
    if (rank == 0 && ks < 3) {  // the cluster's blocks in rank order, the fixed butterfly
      const double v = lane < (int)cl.num_blocks() ? *cl.map_shared_rank(&s_bv[ks], lane) : 0.0;
      x = warp_sum(v);
    }
    cl.sync();
    if (rank != 0) return;
  } else {
    // the group's last block folds the group's block values and its share of the column kernel's
    const int g0 = u * CORR_GS, gn = min(CORR_GS, nb - g0);
    if (!ticket_last(ctr + u, (unsigned)gn)) return;
    if (ks < 3)
      x = warp_fold(bpart + (size_t)ks * nb + g0, gn, lane);
    else if (ks < 5)
      x = corr_col_share(a, pe, ks - 3, u, nu, lane);
  }
  if (ks < 5 && lane == 0) __stcg(upart + (size_t)ks * nu + u, x);  // released by ticket_last
  // second level: the last unit to arrive folds the units' values and applies the fixes
  if (!ticket_last(ctr + ng, (unsigned)nu)) return;
  __shared__ double S[5];
  if (ks < 5) {
    const double x = warp_fold(upart + (size_t)ks * nu, nu, lane);
    if (lane == 0) S[ks] = x;
  }
  __syncthreads();
  double* scal = a.scalars + 4 * e;
  __shared__ double s_corr;
  // warp 0: the mass factor and spe_lnps_n(0,0) += log(factor); warp 1 (another sub-partition):
  // the same factor and the energy correction; warp 2: the two means, off the critical path
  if (ks == 0 && lane == 0) {
    const double factor = a.do_mass ? S[3] / S[0] : 1.0;
    scal[2] = factor;
    a.scal_t[2 * e] = (T)factor;
    if (a.do_mass) {
      V2<T> l = a.lnps_n[e];  // spe_lnps_n[1,1,1] += log(factor)  (P_00 = 1)
      l.x = (T)((double)l.x + log_near_one(factor));
      a.lnps_n[e] = l;
    }
  } else if (ks == 1 && lane == 0) {
    double corr = 0.0;
    if (a.do_energy)  // one division on this warp's chain: factor S2 = S3 S2 / S0
      corr = a.do_mass ? fma(-S[3], S[2], S[0] * (S[4] - S[1])) / ((a.cp * S[3]) * S[0])
                       : (S[4] - S[1] - S[2]) / (a.cp * S[3]);
    scal[3] = corr;
    a.scal_t[2 * e + 1] = (T)corr;
    s_corr = corr;
  } else if (ks == 2 && lane == 0) {
    scal[0] = S[3] * a.inv_2n;           // mean_ps_p   (Area_Weighted_Global_Mean)
    scal[1] = S[4] * a.inv_2n / a.grav;  // mean_energy_p (Mass_Weighted_Global_Integral)
  }
  __syncthreads();
  if (a.do_energy && (int)threadIdx.x < nd) {  // spe_t_n[1,1,:] .+= temperature_correction
    V2<T> tt = a.t_spec_n[e * nd + threadIdx.x];
    tt.x = (T)((double)tt.x + s_corr);
    a.t_spec_n[e * nd + threadIdx.x] = tt;
  }
}

template <typename T>
__global__ void k_hs_corr_apply(T* t_n, T* ps_n, const T* scal_t, size_t memL, size_t mem1) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  const int e = blockIdx.y;  // member: ps *= factor, T += correction
  const T factor = scal_t[2 * e], corr = scal_t[2 * e + 1];
  T* t = t_n + (size_t)e * memL;
  T* ps = ps_n + (size_t)e * mem1;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < memL; q += (size_t)gridDim.x * blockDim.x) {
    t[q] = t[q] + corr;
    if (q < mem1) ps[q] = ps[q] * factor;
  }
}

// Pressure variables and heights on demand (Compute_Pressures_And_Heights!, Press_And_Geopot.jl:3-19).
// out: [0]=p_half (nd+1) [1]=lnp_half (nd+1) [2]=dp (nd) [3]=p_full (nd) [4]=lnp_full (nd)
//      [5]=z_full (nd) [6]=z_half (nd+1), each stored at its own offset in `diag`.
template <typename T>
__global__ void k_pressure_heights(const T* ps_c, const T* t_c, const T* geopots, double* diag, const VertCoef* __restrict__ vcp, int nd,
                                   size_t G, double rdgas, double grav) {
  const VertCoef& vc = *vcp;
  size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (c >= G) return;
  double* ph = diag;
  double* lph = ph + G * (nd + 1);
  double* dpp = lph + G * (nd + 1);
  double* pf = dpp + G * nd;
  double* lpf = pf + G * nd;
  double* zf = lpf + G * nd;
  double* zh = zf + G * nd;
  double ps = ps_c[c];
  for (int k = 0; k <= nd; k++) ph[c + G * k] = vc.ak[k] + vc.bk[k] * ps;
  for (int k = 0; k < nd; k++) dpp[c + G * k] = ph[c + G * (k + 1)] - ph[c + G * k];
  for (int k = 1; k <= nd; k++) lph[c + G * k] = log(ph[c + G * k]);
  for (int k = 1; k < nd; k++)
    lpf[c + G * k] = lph[c + G * (k + 1)] + ph[c + G * k] * (lph[c + G * (k + 1)] - lph[c + G * k]) / dpp[c + G * k] - 1.0;
  lph[c] = 0.0;
  lpf[c] = lph[c + G] - 1.0;
  for (int k = 0; k < nd; k++) pf[c + G * k] = exp(lpf[c + G * k]);
  zh[c + G * nd] = (double)geopots[c];
  zh[c] = 0.0;
  for (int k = nd - 1; k >= 1; k--)
    zh[c + G * k] = zh[c + G * (k + 1)] + rdgas * (double)t_c[c + G * k] * (lph[c + G * (k + 1)] - lph[c + G * k]);
  for (int k = 0; k < nd; k++)
    zf[c + G * k] = zh[c + G * (k + 1)] + rdgas * (double)t_c[c + G * k] * (lph[c + G * (k + 1)] - lpf[c + G * k]);
  for (int k = 0; k < nd; k++) zf[c + G * k] /= grav;
  for (int k = 0; k <= nd; k++) zh[c + G * k] /= grav;
}

// Build_Wave_Matrices (Semi_Implicit.jl:165-180): W_n = (I - ξ² eig_n div_mat)^{-1}, one
// block per n, Gauss-Jordan with partial pivoting in shared memory, FP64.  Output [n][c][r].
__global__ void k_wave_matrices(const double* div_mat, const double* eig0, double xi, int nd, int N, double* W,
                                int* status) {
  extern __shared__ double sh[];
  double* A = sh;            // [nd][nd] column-major
  double* B = sh + nd * nd;  // inverse
  __shared__ int piv;
  const int n = blockIdx.x;
  double factor = xi * xi * eig0[n];
  for (int q = threadIdx.x; q < nd * nd; q += blockDim.x) {
    int r = q % nd, c = q / nd;
    A[q] = (r == c ? 1.0 : 0.0) - factor * div_mat[q];
    B[q] = (r == c) ? 1.0 : 0.0;
  }
  __syncthreads();
  for (int c = 0; c < nd; c++) {
    if (threadIdx.x == 0) {
      int p = c;
      for (int r = c + 1; r < nd; r++)
        if (fabs(A[r + nd * c]) > fabs(A[p + nd * c])) p = r;
      piv = p;
      if (A[p + nd * c] == 0.0) atomicExch(status, 1);
    }
    __syncthreads();
    int p = piv;
    if (p != c)
      for (int q = threadIdx.x; q < nd; q += blockDim.x) {
        double t = A[c + nd * q]; A[c + nd * q] = A[p + nd * q]; A[p + nd * q] = t;
        t = B[c + nd * q]; B[c + nd * q] = B[p + nd * q]; B[p + nd * q] = t;
      }
    __syncthreads();
    double pv = A[c + nd * c];
    __syncthreads();
    for (int q = threadIdx.x; q < nd; q += blockDim.x) {
      A[c + nd * q] /= pv;
      B[c + nd * q] /= pv;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < nd * nd; q += blockDim.x) {
      int r = q % nd, cc = q / nd;
      if (r == c) continue;
      double f = A[r + nd * c];
      if (cc != c) {
        A[r + nd * cc] -= f * A[c + nd * cc];
      }
      B[r + nd * cc] -= f * B[c + nd * cc];
    }
    __syncthreads();
    for (int r = threadIdx.x; r < nd; r += blockDim.x)
      if (r != c) A[r + nd * c] = 0.0;
    __syncthreads();
  }
  for (int q = threadIdx.x; q < nd * nd; q += blockDim.x) {
    int r = q % nd, c = q / nd;
    W[(size_t)n * nd * nd + (size_t)c * nd + r] = B[r + nd * c];
  }
}

// ------------------------------------------------------------------------------------------
// host-side vertical setup: Vert_Coordinate (even_sigma), reference pressures and
// Build_Implicit_Matrices (Semi_Implicit.jl:40-160), FP64.
void press_vars_col(const VertCoef& vc, int nd, double ps, double* ph, double* dp, double* lph, double* pf, double* lpf) {
  for (int k = 0; k <= nd; k++) ph[k] = vc.ak[k] + vc.bk[k] * ps;
  for (int k = 0; k < nd; k++) dp[k] = ph[k + 1] - ph[k];
  for (int k = 1; k <= nd; k++) lph[k] = std::log(ph[k]);
  for (int k = 1; k < nd; k++) lpf[k] = lph[k + 1] + ph[k] * (lph[k + 1] - lph[k]) / dp[k] - 1.0;
  lph[0] = 0.0;
  lpf[0] = lph[1] - 1.0;
  for (int k = 0; k < nd; k++) pf[k] = std::exp(lpf[k]);
}

void lin_ps_t_col(const VertCoef& vc, int nd, double kappa, const double* d, double* dps, double* dtt) {
  std::vector<double> Mh(nd + 1, 0.0), Mdt(nd + 1, 0.0);
  double tot = 0.0;
  for (int k = 0; k < nd; k++) {
    double dlnp_p = vc.lnph_ref[k + 1] - vc.lnpf_ref[k], dlnp = vc.lnph_ref[k + 1] - vc.lnph_ref[k];
    double dmean = d[k] * vc.dp_ref[k];
    dtt[k] = -kappa * vc.t_ref[k] * (tot * dlnp + dmean * dlnp_p) / vc.dp_ref[k];
    tot = tot + dmean;
    Mh[k + 1] = -tot;
  }
  *dps = -tot;
  for (int k = 0; k < nd - 1; k++) Mh[k + 1] = Mh[k + 1] + tot * vc.bk[k + 1];
  Mh[0] = Mh[nd] = 0.0;
  for (int k = 1; k < nd; k++) Mdt[k] = Mh[k] * (vc.t_ref[k] - vc.t_ref[k - 1]);
  for (int k = 0; k < nd; k++) dtt[k] = dtt[k] - 0.5 * (Mdt[k + 1] + Mdt[k]) / vc.dp_ref[k];
}

void lin_geo_col(const VertCoef& vc, int nd, double R, const double* dtt, double* geo) {
  std::vector<double> gh(nd + 1, 0.0);
  for (int k = nd - 1; k >= 1; k--) gh[k] = gh[k + 1] + R * (dtt[k] * (vc.lnph_ref[k + 1] - vc.lnph_ref[k]));
  for (int k = 0; k < nd; k++) geo[k] = gh[k + 1] + R * (dtt[k] * (vc.lnph_ref[k + 1] - vc.lnpf_ref[k]));
}

// Compute_Vert_Coord (Vert_Coordinate.jl:61-87) for the sigma options, zero top (the constructor's
// default, :44): a_k = 0 and b_k from
//   even_sigma    LinRange(0, 1, nd+1)                                    (Compute_Even_Sigma, :112-117)
//   uneven_sigma  b = exp(-(surf_res z + (1 - surf_res) z^exponent) scale_heights), z = 1 - k/nd,
//                 b_nd = 1, b_0 = 0 (Compute_Uneven_Sigma, :120-141, following its docstring: the
//                 reference's branch (:69-70) passes undefined a, b and its code flips the sign of
//                 the exponent, which gives b > 1 above the surface)
//   mcm, v197     the fixed 14- and 18-level tables of Compute_Old_Model_Sigma / Compute_V197_Sigma
//                 (:143-165)
//   hybrid        (:71-76, built as its code means it: the branch does not run in the reference,
//                 Compute_Uneven_Sigma and Transition being called without nd) uneven sigma levels s_k
//                 (zero_top false) serve as pressure levels p_ref s_k above s = p_press and as sigma
//                 levels below s = p_sigma, blended by Transition (:93-110, sin^2 between):
//                 a_k = p_ref s_k (1 - trans_k), b_k = s_k trans_k, with the constructor's defaults
//                 p_ref = 101325, p_press = 0.1, p_sigma = 0.3 (:44-46); top half level zero, as the
//                 zero_top pressure variables assume
int vert_coord_table(int nd, const std::string& opt, double scale_heights, double surf_res, double exponent,
                     double* ak, double* bk) {
  static const double kMcm[15] = {0.0, 0.03, 0.0707, 0.1311, 0.2102, 0.3036, 0.4062, 0.5138,
                                  0.6226, 0.7284, 0.8255, 0.9066, 0.9640, 0.9933, 1.0};
  static const double kV197[19] = {0.0, 0.0089163, 0.0342936, 0.0740741, 0.1262002, 0.1886145, 0.2592592,
                                   0.3360768, 0.4170096, 0.5000000, 0.5829904, 0.6639231, 0.7407407,
                                   0.8113854, 0.8737997, 0.9259259, 0.9657064, 0.9910837, 1.0};
  for (int k = 0; k <= nd; k++) ak[k] = 0.0;
  if (opt == "even_sigma") {
    for (int k = 0; k <= nd; k++) {
      double t = (double)k / (double)nd;
      bk[k] = (1 - t) * 0.0 + t * 1.0;
    }
  } else if (opt == "uneven_sigma") {
    for (int k = 0; k <= nd; k++) {
      double t = (double)k / (double)nd, z = (1 - t) * 1.0 + t * 0.0;  // LinRange(1, 0, nd+1)
      bk[k] = std::exp(-(surf_res * z + (1.0 - surf_res) * std::pow(z, exponent)) * scale_heights);
    }
    bk[nd] = 1.0;
    bk[0] = 0.0;
  } else if (opt == "mcm" || opt == "v197") {
    const int need = opt == "mcm" ? 14 : 18;
    if (nd != need) {
      set_error("%s has %d levels", opt.c_str(), need);
      return JGCM_E_ARG;
    }
    memcpy(bk, opt == "mcm" ? kMcm : kV197, (size_t)(nd + 1) * sizeof(double));
  } else if (opt == "hybrid") {
    const double p_ref = 101325.0, p_press = 0.1, p_sigma = 0.3, pi = 3.14159265358979323846;
    for (int k = 0; k <= nd; k++) {
      double t = (double)k / (double)nd, z = (1 - t) * 1.0 + t * 0.0;  // LinRange(1, 0, nd+1)
      double sg = k == nd ? 1.0 : std::exp(-(surf_res * z + (1.0 - surf_res) * std::pow(z, exponent)) * scale_heights);
      double tr = sg <= p_press ? 0.0 : sg >= p_sigma ? 1.0 : std::pow(std::sin(0.5 * pi * (sg - p_press) / (p_sigma - p_press)), 2);
      ak[k] = p_ref * sg * (1.0 - tr);
      bk[k] = sg * tr;
    }
    ak[0] = bk[0] = 0.0;
  } else {
    set_error("Compute_Vert_Coord: %s is not a valid value for option", opt.c_str());
    return JGCM_E_ARG;
  }
  return JGCM_OK;
}

void vertical_setup(jgcm_model* md) {
  int nd = md->nd;
  VertCoef& vc = md->vc;
  memset(&vc, 0, sizeof(vc));
  for (int k = 0; k <= nd; k++) {
    double t = (double)k / (double)nd;
    vc.ak[k] = md->vert_ak.empty() ? 0.0 : md->vert_ak[k];
    vc.bk[k] = md->vert_bk.empty() ? (1 - t) * 0.0 + t * 1.0 : md->vert_bk[k];
    if (vc.ak[k] != 0.0) vc.hybrid = 1;
  }
  for (int k = 0; k < nd; k++) {
    vc.dak[k] = vc.ak[k + 1] - vc.ak[k];
    vc.dbk[k] = vc.bk[k + 1] - vc.bk[k];
    vc.dak_hi[k] = (float)vc.dak[k];
    vc.dak_lo[k] = (float)(vc.dak[k] - (double)vc.dak_hi[k]);
    vc.dbk_hi[k] = (float)vc.dbk[k];
    vc.dbk_lo[k] = (float)(vc.dbk[k] - (double)vc.dbk_hi[k]);
  }
  // sigma coordinates: every log-pressure difference is a per-level constant (formed here in FP64)
  for (int k = 1; k <= nd && !vc.hybrid; k++) vc.lb[k] = std::log(vc.bk[k]);
  for (int k = 0; k < nd && !vc.hybrid; k++) {
    vc.cf[k] = (k == 0) ? vc.lb[1] - 1.0
                        : vc.lb[k + 1] + vc.bk[k] * (vc.lb[k + 1] - vc.lb[k]) / vc.dbk[k] - 1.0;
    vc.sf[k] = std::exp(vc.cf[k]);
    vc.dlp_p[k] = vc.lb[k + 1] - vc.cf[k];
    vc.dlp_m[k] = (k == 0) ? 0.0 : vc.cf[k] - vc.lb[k];
    vc.dlp[k] = (k == 0) ? 0.0 : vc.lb[k + 1] - vc.lb[k];
  }
  if (md->P.kind != JGCM_HELD_SUAREZ) return;
  std::vector<double> ph(nd + 1), pf(nd), dlh(nd + 1), dlf(nd);
  double lph[JGCM_MAX_ND + 1], lpf[JGCM_MAX_ND];
  press_vars_col(vc, nd, md->P.ps_ref, ph.data(), vc.dp_ref, lph, pf.data(), lpf);
  for (int k = 0; k <= nd; k++) vc.lnph_ref[k] = lph[k];
  for (int k = 0; k < nd; k++) vc.lnpf_ref[k] = lpf[k];
  for (int k = 0; k < nd; k++) vc.t_ref[k] = md->P.t_ref;
  for (int k = 0; k < nd; k++) vc.rdp_ref[k] = 1.0 / vc.dp_ref[k];
  for (int k = 0; k <= nd; k++) dlh[k] = vc.bk[k] / ph[k];
  for (int k = 0; k < nd; k++)
    dlf[k] = (vc.bk[k + 1] * (vc.lnph_ref[k + 1] - vc.lnpf_ref[k]) + vc.bk[k] * (vc.lnpf_ref[k] - vc.lnph_ref[k])) /
             vc.dp_ref[k];
  std::vector<double> tau(nd * nd), gamma(nd * nd), nu(nd), e(nd), dtt(nd), geo(nd);
  for (int k = 0; k < nd; k++) {
    std::fill(e.begin(), e.end(), 0.0);
    e[k] = 1.0;
    double dps;
    lin_ps_t_col(vc, nd, md->P.kappa, e.data(), &dps, dtt.data());
    nu[k] = -dps;
    for (int r = 0; r < nd; r++) tau[r + nd * k] = -dtt[r];
    lin_geo_col(vc, nd, md->P.rdgas, e.data(), geo.data());
    for (int r = 0; r < nd; r++) gamma[r + nd * k] = geo[r];
  }
  double R = md->P.rdgas;
  std::vector<double> h1(nd), h2(nd), gh2(nd + 1, 0.0);
  for (int k = 0; k < nd; k++)
    h1[k] = R * vc.t_ref[k] *
            (vc.bk[k + 1] * (vc.lnph_ref[k + 1] - vc.lnpf_ref[k]) + vc.bk[k] * (vc.lnpf_ref[k] - vc.lnph_ref[k])) /
            vc.dp_ref[k];
  for (int k = nd - 1; k >= 1; k--) gh2[k] = gh2[k + 1] + R * (vc.t_ref[k] * (dlh[k + 1] - dlh[k]));
  for (int k = 0; k < nd; k++) h2[k] = gh2[k + 1] + R * (vc.t_ref[k] * (dlh[k + 1] - dlf[k]));
  for (int k = 0; k < nd; k++) vc.h[k] = h1[k] + h2[k];
  for (int r = 0; r < nd; r++)
    for (int c = 0; c < nd; c++) {
      double s = 0.0;
      for (int q = 0; q < nd; q++) s += gamma[r + nd * q] * tau[q + nd * c];
      md->div_mat[r + nd * c] = vc.h[r] * nu[c] + s;
    }
}

// ------------------------------------------------------------------------------------------
template <typename T>
__global__ void k_fill_damping(const double* eig, T* out, int N, int ns, double coef, int order, double dt_eff) {
  // Time_Integrator.jl:31: damping = coef (eig / eig[1, num_spherical])^order; with dt_eff > 0
  // the implicit damping factor 1/(1 + dt_eff damping) of Compute_Spectral_Damping! (:76-80)
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (N + 1) * (ns + 1)) return;
  double e0 = eig[0 * (ns + 1) + (ns - 1)];
  double d = coef * pow(eig[t] / e0, (double)order);
  out[t] = (T)(dt_eff > 0.0 ? 1.0 / (1.0 + dt_eff * d) : d);
}
template <typename T>
__global__ void k_fill_coriolis(const double* sinth, T* f, int nlat, double omega) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nlat) f[t] = (T)(2 * omega * sinth[t]);
}

int alloc(void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    set_error("cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
    return JGCM_E_NOMEM;
  }
  e = cudaMemset(*p, 0, bytes);
  if (e != cudaSuccess) {
    set_error("cudaMemset: %s", cudaGetErrorString(e));
    return JGCM_E_CUDA;
  }
  return JGCM_OK;
}

void model_free(jgcm_model* md) {
  if (!md) return;
  adj_context_free(md);
  if (md->state_stage) cudaFree(md->state_stage);
  for (int i = 0; i < 3; i++) {
    void* ps[] = {md->spe_vor[i], md->spe_div[i], md->spe_lnps[i], md->spe_t[i],
                  md->grid_u[i], md->grid_v[i], md->grid_ps[i], md->grid_t[i]};
    for (auto p : ps)
      if (p) cudaFree(p);
    if (md->graph[i]) cudaGraphExecDestroy(md->graph[i]);
    if (md->graph3[i]) cudaGraphExecDestroy(md->graph3[i]);
    if (md->graph24[i]) cudaGraphExecDestroy(md->graph24[i]);
  }
  for (int i = 0; i < 3; i++) {
    if (md->spe_q[i]) cudaFree(md->spe_q[i]);
    if (md->grid_q[i]) cudaFree(md->grid_q[i]);
  }
  for (void* p : {md->spe_dq, md->g_dq, md->g_dlq, md->g_dtq, md->g_mhalf, (void*)md->q_stage})
    if (p) cudaFree(p);
  void* ps[] = {md->grid_vor, md->grid_div, md->grid_lnps, md->grid_t_eq, md->grid_geopots, md->grid_h_eq,
                md->spe_zero, md->spe_dvor, md->spe_ddiv, md->spe_dlnps, md->spe_dt, md->g_dlps, md->g_dtps,
                md->g_dlT, md->g_dtT, md->g_ducos, md->g_dvcos, md->g_dt, md->g_energy, md->g_dlnps, md->g_diag,
                md->g_tdev, md->coriolis, md->damping, md->dfac[0], md->dfac[1], md->d_W, md->d_pairs, md->d_partials,
                md->d_scalars, md->d_counter, md->d_vc, md->fbuf, md->diag};
  for (auto p : ps)
    if (p) cudaFree(p);
  delete[] md->div_mat;
  if (md->ev0) cudaEventDestroy(md->ev0);
  if (md->ev1) cudaEventDestroy(md->ev1);
  delete md;
}

int build_wave(jgcm_model* md) {
  jgcm_mesh* m = md->mesh;
  int nd = md->nd, N = m->N;
  double *d_div = nullptr, *d_eig0 = nullptr;
  int* d_status = nullptr;
  JG_TRY(alloc((void**)&d_div, nd * nd * 8));
  JG_TRY(alloc((void**)&d_eig0, (N + 1) * 8));
  JG_TRY(alloc((void**)&d_status, 4));
  std::vector<double> eig0(N + 1);
  for (int n = 0; n <= N; n++) eig0[n] = (double)(-n * (n + 1)) / (m->radius * m->radius);
  JG_CUDA(cudaMemcpy(d_div, md->div_mat, nd * nd * 8, cudaMemcpyHostToDevice));
  JG_CUDA(cudaMemcpy(d_eig0, eig0.data(), (N + 1) * 8, cudaMemcpyHostToDevice));
  const double a = md->P.implicit_coef;
  double xis[2] = {md->P.dt * a, (2 * md->P.dt) * a};  // Get_ξ for the init step and afterwards
  for (int s = 0; s < 2; s++) {
    k_wave_matrices<<<N + 1, 128, 2 * nd * nd * 8, m->stream>>>(d_div, d_eig0, xis[s], nd, N,
                                                                 md->d_W + (size_t)s * (N + 1) * nd * nd, d_status);
    JG_CUDA(cudaGetLastError());
  }
  int st = 0;
  JG_CUDA(cudaMemcpyAsync(&st, d_status, 4, cudaMemcpyDeviceToHost, m->stream));
  JG_CUDA(cudaStreamSynchronize(m->stream));
  cudaFree(d_div);
  cudaFree(d_eig0);
  cudaFree(d_status);
  if (st) {
    set_error("singular semi-implicit wave matrix");
    return JGCM_E_NUMERIC;
  }
  return JGCM_OK;
}

// FP64 block partials per member: the column kernel's 2 sums over its (nlon/(64/S)) x nlat blocks
// (S <= 8) first, then the fixer kernel's 3 sums over (nlon/32) x nlat blocks (both live until the
// fixer's last block has folded them)
size_t col_partials(const jgcm_mesh* m) { return (size_t)2 * ((m->nlon + HS_CT / 8 - 1) / (HS_CT / 8)) * m->nlat; }
size_t partial_stride(const jgcm_mesh* m) {
  const int nb = ((m->nlon + 31) / 32) * m->nlat;  // the fixer reduction's blocks per member
  return col_partials(m) + (size_t)3 * nb + (size_t)5 * nb;  // its block values, its units' (<= nb)
}
// the fixer reduction's tickets per member
inline size_t corr_tickets(const jgcm_mesh* m) { return (size_t)corr_groups(((m->nlon + 31) / 32) * m->nlat) + 1; }

int model_alloc(jgcm_model* md) {
  jgcm_mesh* m = md->mesh;
  const int nd = md->nd, N = m->N, ns = m->ns, ne = md->ne, L = md->L;
  const size_t ts = tsize(m);
  const size_t S = spec_elems(m, L) * 2 * ts, S1 = spec_elems(m, ne) * 2 * ts;
  const size_t G = grid_elems(m, L) * ts, G1 = grid_elems(m, ne) * ts;
  // the widest plan: Held-Suarez's synthesis of vor, div, u, v, T, ln ps and the next step's
  // gradients of ln ps and T (7 nd + 3 columns per member)
  md->fcap = (7 * nd + 3) * ne;
  JG_TRY(alloc(&md->fbuf, (size_t)(N + 1) * m->nlat * md->fcap * 2 * ts));
  for (int i = 0; i < 3; i++) {
    JG_TRY(alloc(&md->spe_vor[i], S));
    JG_TRY(alloc(&md->spe_div[i], S));
    JG_TRY(alloc(&md->spe_lnps[i], S1));
    JG_TRY(alloc(&md->spe_t[i], S));
    JG_TRY(alloc(&md->grid_u[i], G));
    JG_TRY(alloc(&md->grid_v[i], G));
    JG_TRY(alloc(&md->grid_ps[i], G1));
    JG_TRY(alloc(&md->grid_t[i], G));
  }
  void** gnd[] = {&md->grid_vor, &md->grid_div, &md->grid_t_eq, &md->g_dlT, &md->g_dtT, &md->g_ducos, &md->g_dvcos,
                  &md->g_dt, &md->g_energy, &md->g_tdev};
  for (auto p : gnd) JG_TRY(alloc(p, G));
  void** g1[] = {&md->grid_lnps, &md->grid_geopots, &md->grid_h_eq, &md->g_dlps, &md->g_dtps, &md->g_dlnps};
  for (auto p : g1) JG_TRY(alloc(p, G1));
  void** snd[] = {&md->spe_zero, &md->spe_dvor, &md->spe_ddiv, &md->spe_dt};
  for (auto p : snd) JG_TRY(alloc(p, S));
  JG_TRY(alloc(&md->spe_dlnps, S1));
  JG_TRY(alloc(&md->g_diag, grid_elems(m, 1) * (7 * (size_t)nd + 3) * 8));
  JG_TRY(alloc(&md->coriolis, (size_t)m->nlat * ts));
  JG_TRY(alloc(&md->damping, (size_t)(N + 1) * (ns + 1) * ts));
  JG_TRY(alloc((void**)&md->d_W, 2 * (size_t)(N + 1) * nd * nd * 8));
  std::vector<int2> pairs;
  for (int mm = 0; mm <= N; mm++)
    for (int n = mm; n <= ns; n++) pairs.push_back(make_int2(mm, n));
  md->npairs = (int)pairs.size();
  JG_TRY(alloc((void**)&md->d_pairs, pairs.size() * sizeof(int2)));
  JG_CUDA(cudaMemcpy(md->d_pairs, pairs.data(), pairs.size() * sizeof(int2), cudaMemcpyHostToDevice));
  JG_TRY(alloc((void**)&md->d_partials, (size_t)ne * partial_stride(m) * 8));
  // 4 FP64 scalars per member, then each member's factor and correction in the state precision
  JG_TRY(alloc((void**)&md->d_scalars, (size_t)6 * ne * 8));
  JG_TRY(alloc((void**)&md->d_counter, (size_t)ne * corr_tickets(m) * sizeof(unsigned)));
  int nt = (N + 1) * (ns + 1);
  JG_TRY(alloc(&md->dfac[0], (size_t)nt * ts));
  JG_TRY(alloc(&md->dfac[1], (size_t)nt * ts));
  const double cf = md->P.damping_coef, dt1 = md->P.dt, dt2 = 2.0 * md->P.dt;
  const int od = md->P.damping_order, nb = (nt + 127) / 128;
  if (is_fp64(m)) {
    k_fill_damping<double><<<nb, 128, 0, m->stream>>>(m->t64.eig, (double*)md->damping, N, ns, cf, od, 0.0);
    k_fill_damping<double><<<nb, 128, 0, m->stream>>>(m->t64.eig, (double*)md->dfac[0], N, ns, cf, od, dt1);
    k_fill_damping<double><<<nb, 128, 0, m->stream>>>(m->t64.eig, (double*)md->dfac[1], N, ns, cf, od, dt2);
    k_fill_coriolis<double><<<(m->nlat + 127) / 128, 128, 0, m->stream>>>(m->d_sinth, (double*)md->coriolis, m->nlat,
                                                                          md->P.omega);
  } else {
    k_fill_damping<float><<<nb, 128, 0, m->stream>>>(m->t64.eig, (float*)md->damping, N, ns, cf, od, 0.0);
    k_fill_damping<float><<<nb, 128, 0, m->stream>>>(m->t64.eig, (float*)md->dfac[0], N, ns, cf, od, dt1);
    k_fill_damping<float><<<nb, 128, 0, m->stream>>>(m->t64.eig, (float*)md->dfac[1], N, ns, cf, od, dt2);
    k_fill_coriolis<float><<<(m->nlat + 127) / 128, 128, 0, m->stream>>>(m->d_sinth, (float*)md->coriolis, m->nlat,
                                                                         md->P.omega);
  }
  JG_CUDA(cudaGetLastError());
  JG_CUDA(cudaEventCreate(&md->ev0));
  JG_CUDA(cudaEventCreate(&md->ev1));
  md->div_mat = new double[nd * nd]();
  vertical_setup(md);
  JG_TRY(alloc((void**)&md->d_vc, sizeof(VertCoef)));
  JG_CUDA(cudaMemcpy(md->d_vc, &md->vc, sizeof(VertCoef), cudaMemcpyHostToDevice));
  if (md->P.kind == JGCM_HELD_SUAREZ) JG_TRY(build_wave(md));
  JG_CUDA(cudaStreamSynchronize(m->stream));
  return JGCM_OK;
}

// ------------------------------------------------------------------------------------------
// plan builders
S2GGroup sg(int op, const void* a, const void* b, int L, int col0) {
  S2GGroup g;
  memset(&g, 0, sizeof(g));
  g.op = op; g.a = a; g.b = b; g.L = L; g.col0 = col0;
  return g;
}
GridOutGroup og(int epi, void* dst, int L, int col0, void* dst2 = nullptr, const void* ps = nullptr) {
  GridOutGroup g;
  memset(&g, 0, sizeof(g));
  g.epi = epi; g.dst = dst; g.dst2 = dst2; g.ps = ps; g.L = L; g.col0 = col0;
  return g;
}
GridInGroup ig(int pro, const void* src, int L, int col0) {
  GridInGroup g;
  memset(&g, 0, sizeof(g));
  g.pro = pro; g.src = src; g.L = L; g.col0 = col0;
  return g;
}
SpecOutGroup og2(int op, void* dst, int L, int col0, int colA, int colB, int colE, int colH = -1) {
  SpecOutGroup g;
  memset(&g, 0, sizeof(g));
  g.op = op; g.dst = dst; g.L = L; g.col0 = col0; g.colA = colA; g.colB = colB; g.colE = colE; g.colH = colH;
  return g;
}

StepParams step_params(const jgcm_model* md) {
  StepParams sp;
  memset(&sp, 0, sizeof(sp));
  sp.init_step = md->init_step;
  sp.dt = md->P.dt;
  sp.robert = md->P.robert_coef;
  sp.implicit_coef = md->P.implicit_coef;
  sp.h0 = md->P.h0;
  sp.damping = md->damping;
  return sp;
}

template <typename T>
int s2g_final_uv(jgcm_model* md, int lev_n, cudaStream_t st);

// Barotropic_Dynamics! (Barotropic_Dynamics.jl:2-46)
template <typename T>
int step_barotropic(jgcm_model* md, cudaStream_t st) {
  jgcm_mesh* m = md->mesh;
  const int nd = md->L, p = lvl(md, 0), c = lvl(md, 1), n = lvl(md, 2);
  FFTPlan fp;
  memset(&fp, 0, sizeof(fp));
  fp.ng = 2;
  fp.C = 2 * nd;
  fp.kappa_m = 0.0;
  fp.coriolis = md->coriolis;
  fp.g[0] = ig(PRO_FLUXU, md->grid_u[c], nd, 0);
  fp.g[0].s1 = md->grid_v[c];
  fp.g[0].s2 = md->grid_vor;
  fp.g[1] = ig(PRO_FLUXV, md->grid_u[c], nd, nd);
  fp.g[1].s1 = md->grid_v[c];
  fp.g[1].s2 = md->grid_vor;
  G2SPlan gp;
  memset(&gp, 0, sizeof(gp));
  gp.ng = 1;
  gp.C = nd;
  gp.sp = step_params(md);
  gp.g[0] = og2(G2S_BARO, md->spe_vor[n], nd, 0, nd, 0, -1);  // A = δv cos, B = δu cos
  gp.g[0].qc[0] = md->spe_vor[c];
  gp.g[0].qp[0] = md->spe_vor[p];
  JG_TRY(launch_g2s<T>(m, fp, gp, st, md->fbuf, md->fcap));
  S2GPlan sp;
  memset(&sp, 0, sizeof(sp));
  sp.ng = 3;
  sp.C = 3 * nd;
  sp.g[0] = sg(S2G_PLAIN, md->spe_vor[n], nullptr, nd, 0);
  sp.g[1] = sg(S2G_UCOS, md->spe_vor[n], md->spe_zero, nd, nd);
  sp.g[2] = sg(S2G_VCOS, md->spe_vor[n], md->spe_zero, nd, 2 * nd);
  IFFTPlan ip;
  memset(&ip, 0, sizeof(ip));
  ip.ng = 3;
  ip.C = 3 * nd;
  ip.g[0] = og(EPI_NONE, md->grid_vor, nd, 0);
  ip.g[1] = og(EPI_DIVCOS, md->grid_u[n], nd, nd);
  ip.g[2] = og(EPI_DIVCOS, md->grid_v[n], nd, 2 * nd);
  JG_TRY(launch_s2g<T>(m, sp, ip, st, md->fbuf, md->fcap));
  return JGCM_OK;
}

// Shallow_Water_Physics! + Shallow_Water_Dynamics! (Shallow_Water_Dynamics.jl:7-179).
// h lives in the lnps/ps slots; the advected height is spe_h_n, which equals spe_h_c after the
// first Time_Advance! (Shallow_Water_Dynamics.jl:147).
template <typename T>
int step_shallow_water(jgcm_model* md, cudaStream_t st) {
  jgcm_mesh* m = md->mesh;
  const int p = lvl(md, 0), c = lvl(md, 1), n = lvl(md, 2), E = md->ne;
  const void* h_adv = md->sw_adv_from_n ? md->spe_lnps[n] : md->spe_lnps[c];
  S2GPlan sp;
  memset(&sp, 0, sizeof(sp));
  sp.ng = 2;
  sp.C = 2 * E;
  sp.g[0] = sg(S2G_DLAM, h_adv, nullptr, E, 0 * E);
  sp.g[1] = sg(S2G_DTH, h_adv, nullptr, E, 1 * E);
  IFFTPlan ip;
  memset(&ip, 0, sizeof(ip));
  ip.ng = 2;
  ip.C = 2 * E;
  ip.g[0] = og(EPI_DIVCOS, md->g_dlps, E, 0 * E);
  ip.g[1] = og(EPI_DIVCOS, md->g_dtps, E, 1 * E);
  JG_TRY(launch_s2g<T>(m, sp, ip, st, md->fbuf, md->fcap));
  FFTPlan fp;
  memset(&fp, 0, sizeof(fp));
  fp.ng = 4;
  fp.C = 4 * E;
  fp.kappa_m = md->P.kappa_m;
  fp.kappa_t = md->P.kappa_t;
  fp.coriolis = md->coriolis;
  fp.g[0] = ig(PRO_FLUXU, md->grid_u[c], E, 0 * E);
  fp.g[0].s1 = md->grid_v[c];
  fp.g[0].s2 = md->grid_vor;
  fp.g[1] = ig(PRO_FLUXV, md->grid_u[c], E, 1 * E);
  fp.g[1].s1 = md->grid_v[c];
  fp.g[1].s2 = md->grid_vor;
  fp.g[2] = ig(PRO_KIN, md->grid_u[c], E, 2 * E);
  fp.g[2].s1 = md->grid_v[c];
  fp.g[3] = ig(PRO_SWH, md->grid_ps[c], E, 3 * E);
  fp.g[3].s1 = md->grid_u[c];
  fp.g[3].s2 = md->grid_v[c];
  fp.g[3].s3 = md->g_dlps;
  fp.g[3].s4 = md->g_dtps;
  fp.g[3].s5 = md->grid_div;
  fp.g[3].s6 = md->grid_h_eq;
  G2SPlan gp;
  memset(&gp, 0, sizeof(gp));
  gp.ng = 1;
  gp.C = E;
  gp.sp = step_params(md);
  gp.g[0] = og2(G2S_SW, md->spe_vor[n], E, 0, 0, E, 2 * E, 3 * E);
  gp.g[0].dst2 = md->spe_div[n];
  gp.g[0].dst3 = md->spe_lnps[n];
  gp.g[0].qc[0] = md->spe_vor[c];
  gp.g[0].qc[1] = md->spe_div[c];
  gp.g[0].qc[2] = md->spe_lnps[c];
  gp.g[0].qp[0] = md->spe_vor[p];
  gp.g[0].qp[1] = md->spe_div[p];
  gp.g[0].qp[2] = md->spe_lnps[p];
  JG_TRY(launch_g2s<T>(m, fp, gp, st, md->fbuf, md->fcap));
  S2GPlan sp2;
  memset(&sp2, 0, sizeof(sp2));
  sp2.ng = 5;
  sp2.C = 5 * E;
  sp2.g[0] = sg(S2G_PLAIN, md->spe_vor[n], nullptr, E, 0 * E);
  sp2.g[1] = sg(S2G_PLAIN, md->spe_div[n], nullptr, E, 1 * E);
  sp2.g[2] = sg(S2G_PLAIN, md->spe_lnps[n], nullptr, E, 2 * E);
  sp2.g[3] = sg(S2G_UCOS, md->spe_vor[n], md->spe_div[n], E, 3 * E);
  sp2.g[4] = sg(S2G_VCOS, md->spe_vor[n], md->spe_div[n], E, 4 * E);
  IFFTPlan ip2;
  memset(&ip2, 0, sizeof(ip2));
  ip2.ng = 5;
  ip2.C = 5 * E;
  ip2.g[0] = og(EPI_NONE, md->grid_vor, E, 0 * E);
  ip2.g[1] = og(EPI_NONE, md->grid_div, E, 1 * E);
  ip2.g[2] = og(EPI_NONE, md->grid_ps[n], E, 2 * E);
  ip2.g[3] = og(EPI_DIVCOS, md->grid_u[n], E, 3 * E);
  ip2.g[4] = og(EPI_DIVCOS, md->grid_v[n], E, 4 * E);
  JG_TRY(launch_s2g<T>(m, sp2, ip2, st, md->fbuf, md->fcap));
  return JGCM_OK;
}

// Atmosphere_Update! (Spectral_Dynamics.jl:470-490) for Held-Suarez.
// Zonal means of T, T_eq, u, v added to the FP64 sums (Zonal_Mean, Output_Manager.jl:81-107):
// block (latitude j, level k, member e), threads over longitude, fixed-order FP64 reduction.
template <typename T>
__global__ void k_diag_zonal(const T* t, const T* t_eq, const T* u, const T* v, double* sums, int nd, int nlat,
                             int nlon, int ne) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  const int j = blockIdx.x, k = blockIdx.y, e = blockIdx.z;
  const size_t G = (size_t)nlat * nlon, row = ((size_t)e * nd + k) * G + (size_t)j * nlon;
  __shared__ double red[4][4];
  double acc[4] = {0, 0, 0, 0};
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    acc[0] += (double)t[row + i];
    acc[1] += (double)t_eq[row + i];
    acc[2] += (double)u[row + i];
    acc[3] += (double)v[row + i];
  }
  for (int f = 0; f < 4; f++) acc[f] = warp_sum(acc[f]);
  if ((threadIdx.x & 31) == 0)
    for (int f = 0; f < 4; f++) red[f][threadIdx.x >> 5] = acc[f];
  __syncthreads();
  if (threadIdx.x < 4) {
    const int f = threadIdx.x;
    double tot = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += red[f][w];
    sums[(((size_t)f * ne + e) * nd + k) * nlat + j] += tot / nlon;
  }
}
template <typename T>
__global__ void k_diag_ps(const T* ps, double* sums, size_t n) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    sums[q] += (double)ps[q];
}

template <typename T>
int issue_diag(jgcm_model* md, int lev, cudaStream_t st) {
  jgcm_mesh* m = md->mesh;
  const int nd = md->nd, E = md->ne;
  JG_CUDA(launch_pdl(k_diag_zonal<T>, dim3(m->nlat, nd, E), 128, 0, st, (const T*)md->grid_t[lev], (const T*)md->grid_t_eq,
                                                         (const T*)md->grid_u[lev], (const T*)md->grid_v[lev],
                                                         md->diag, nd, m->nlat, m->nlon, E));
  JG_CUDA(cudaGetLastError());
  const size_t nps = grid_elems(m, E);
  JG_CUDA(launch_pdl(k_diag_ps<T>, (int)std::min<size_t>((nps + 255) / 256, 1024), 256, 0, st, 
      (const T*)md->grid_ps[lev], md->diag + (size_t)4 * E * nd * m->nlat, nps));
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}

// Gradients (cos θ ∇ / cos θ) of ln ps and T of time level `lev` into g_dlps, g_dtps, g_dlT, g_dtT
// (Compute_Gradients!, Spectral_Spherical_Mesh.jl:721-741), and on the FP32 path T less its level
// means (g_tdev, the column kernel's geopotential), for a state that no step synthesised (the
// first step from a state set on the host; a step's own synthesis writes them for the next one).
template <typename T>
int issue_hs_grad(jgcm_model* md, int lev, cudaStream_t st) {
  const int L = md->L, E = md->ne;
  S2GPlan sp;
  memset(&sp, 0, sizeof(sp));
  const bool anom = std::is_same<T, float>::value;
  sp.ng = anom ? 5 : 4;
  sp.C = 2 * E + (anom ? 3 : 2) * L;
  sp.g[0] = sg(S2G_DLAM, md->spe_lnps[lev], nullptr, E, 0);
  sp.g[1] = sg(S2G_DTH, md->spe_lnps[lev], nullptr, E, E);
  sp.g[2] = sg(S2G_DLAM, md->spe_t[lev], nullptr, L, 2 * E);
  sp.g[3] = sg(S2G_DTH, md->spe_t[lev], nullptr, L, 2 * E + L);
  if (anom) sp.g[4] = sg(S2G_ANOM, md->spe_t[lev], nullptr, L, 2 * E + 2 * L);
  IFFTPlan ip;
  memset(&ip, 0, sizeof(ip));
  ip.ng = sp.ng;
  ip.C = sp.C;
  ip.g[0] = og(EPI_DIVCOS, md->g_dlps, E, 0);
  ip.g[1] = og(EPI_DIVCOS, md->g_dtps, E, E);
  ip.g[2] = og(EPI_DIVCOS, md->g_dlT, L, 2 * E);
  ip.g[3] = og(EPI_DIVCOS, md->g_dtT, L, 2 * E + L);
  if (anom) ip.g[4] = og(EPI_NONE, md->g_tdev, L, 2 * E + 2 * L);
  if (md->nq) {  // and those of the tracers
    const int LQ = md->LQ, c0 = sp.C;
    sp.g[sp.ng] = sg(S2G_DLAM, md->spe_q[lev], nullptr, LQ, c0);
    ip.g[sp.ng++] = og(EPI_DIVCOS, md->g_dlq, LQ, c0);
    sp.g[sp.ng] = sg(S2G_DTH, md->spe_q[lev], nullptr, LQ, c0 + LQ);
    ip.g[sp.ng++] = og(EPI_DIVCOS, md->g_dtq, LQ, c0 + LQ);
    sp.C += 2 * LQ;
    ip.ng = sp.ng;
    ip.C = sp.C;
  }
  return launch_s2g<T>(md->mesh, sp, ip, st, md->fbuf, md->fcap);
}

// whether the vertical coordinate has Δa_k != 0 (hybrid): the energy integrals then need sum_k T_k Δa_k
inline int has_dak(const jgcm_model* md) {
  for (int k = 0; k < md->nd; k++)
    if (md->vc.dak[k] != 0.0) return 1;
  return 0;
}

template <typename T>
int step_held_suarez(jgcm_model* md, cudaStream_t st) {
  jgcm_mesh* m = md->mesh;
  const int nd = md->nd, L = md->L, E = md->ne, p = lvl(md, 0), c = lvl(md, 1), n = lvl(md, 2);
  const int Dt = md->init_step ? md->P.dt : 2 * md->P.dt;
  // 1. gradients of lnps_c and T_c, unless the previous step left them (∇ps = ∇lnps ps is formed in
  //    the column kernel)
  if (!md->grad_ready) JG_TRY(issue_hs_grad<T>(md, c, st));
  // 2. physics + grid dynamics (one warp per column)
  Tables<T> tb = tables<T>(m);
  HSColArgs<T> a;
  memset(&a, 0, sizeof(a));
  a.u_p = (const T*)md->grid_u[p];
  a.v_p = (const T*)md->grid_v[p];
  a.t_p = (const T*)md->grid_t[p];
  a.ps_p = (const T*)md->grid_ps[p];
  a.ps_c = (const T*)md->grid_ps[c];
  a.u_c = (const T*)md->grid_u[c];
  a.v_c = (const T*)md->grid_v[c];
  a.t_c = (const T*)md->grid_t[c];
  a.tdev = std::is_same<T, float>::value ? (const T*)md->g_tdev : nullptr;
  a.has_dak = has_dak(md);
  a.div = (const T*)md->grid_div;
  a.vor = (const T*)md->grid_vor;
  a.dlps = (const T*)md->g_dlps;
  a.dtps = (const T*)md->g_dtps;
  a.dlT = (const T*)md->g_dlT;
  a.dtT = (const T*)md->g_dtT;
  a.geopots = (const T*)md->grid_geopots;
  a.coriolis = (const T*)md->coriolis;
  a.sinj = tb.sinj;
  a.cosj = tb.cosj;
  a.ducos = (T*)md->g_ducos;
  a.dvcos = (T*)md->g_dvcos;
  a.dtg = (T*)md->g_dt;
  a.energy = (T*)md->g_energy;
  a.dlnps = (T*)md->g_dlnps;
  a.t_eq = (T*)md->grid_t_eq;
  a.t_spec = (const V2<T>*)md->spe_t[c];
  a.m_half = md->nq ? (T*)md->g_mhalf : nullptr;
  a.wts = m->d_wts;
  a.partials = md->d_partials;
  a.nd = nd;
  a.nlat = m->nlat;
  a.nlon = m->nlon;
  a.Dt = Dt;
  a.sigma_b = md->P.sigma_b;
  a.k_f = md->P.k_f;
  a.k_a = md->P.k_a;
  a.k_s = md->P.k_s;
  a.dT_y = md->P.dT_y;
  a.dtheta_z = md->P.dtheta_z;
  a.kappa = md->P.kappa;
  a.rdgas = md->P.rdgas;
  a.cp = md->cp_air;
  a.grav = md->P.grav;
  a.inv_2n = 0.5 / m->nlon;
  a.pstride = partial_stride(m);
  hs_col_consts<T>(a);
  JG_TRY(launch_hs_column<T>(a, m, E, md->hs_lanes, md->d_vc, md->vc.hybrid, st));
  mark(st);
  JG_CUDA(cudaGetLastError());
  if (md->nq) {  // 2'. the tracers' tendencies
    TracerArgs<T> ta;
    ta.u_c = (const T*)md->grid_u[c];
    ta.v_c = (const T*)md->grid_v[c];
    ta.ps_c = (const T*)md->grid_ps[c];
    ta.q_c = (const T*)md->grid_q[c];
    ta.dlq = (const T*)md->g_dlq;
    ta.dtq = (const T*)md->g_dtq;
    ta.m_half = (const T*)md->g_mhalf;
    ta.dq = (T*)md->g_dq;
    ta.nd = nd;
    ta.nq = md->nq;
    ta.nlat = m->nlat;
    ta.nlon = m->nlon;
    JG_CUDA(launch_pdl(k_hs_tracers<T>, dim3((m->nlon + 127) / 128, m->nlat, E), 128, 0, st, ta, md->d_vc));
    mark(st);
    JG_CUDA(cudaGetLastError());
  }
  // 3. forward transforms: δu cos, δv cos, δT, energy, δlnps -> vor/div tendencies (alpha
  //    operator, δdiv -= ∇²E), δT, δlnps
  FFTPlan fp;
  memset(&fp, 0, sizeof(fp));
  fp.ng = 5;
  fp.C = 4 * L + E;
  fp.g[0] = ig(PRO_NONE, md->g_ducos, L, 0);
  fp.g[1] = ig(PRO_NONE, md->g_dvcos, L, L);
  fp.g[2] = ig(PRO_NONE, md->g_dt, L, 2 * L);
  fp.g[3] = ig(PRO_NONE, md->g_energy, L, 3 * L);
  fp.g[4] = ig(PRO_NONE, md->g_dlnps, E, 4 * L);
  G2SPlan gp;
  memset(&gp, 0, sizeof(gp));
  gp.ng = 4;
  gp.C = 3 * L + E;
  gp.g[0] = og2(G2S_VOR, md->spe_dvor, L, 0, L, 0, -1);
  gp.g[1] = og2(G2S_DIV, md->spe_ddiv, L, L, 0, L, 3 * L);
  gp.g[2] = og2(G2S_PLAIN, md->spe_dt, L, 2 * L, 2 * L, -1, -1);
  gp.g[3] = og2(G2S_PLAIN, md->spe_dlnps, E, 3 * L, 4 * L, -1, -1);
  if (hs_analysis_fits(m, nd, E))  // the same outputs, one thread per (m, n, level)
    JG_TRY(launch_hs_analysis<T>(m, fp, 0, L, 3 * L, 2 * L, 4 * L, nd, E, md->spe_dvor, md->spe_ddiv, md->spe_dt,
                                 md->spe_dlnps, st, md->fbuf, md->fcap));
  else
    JG_TRY(launch_g2s<T>(m, fp, gp, st, md->fbuf, md->fcap));
  if (md->nq) {  // 3'. the tracers' tendencies to spectral space
    FFTPlan fq;
    memset(&fq, 0, sizeof(fq));
    fq.ng = 1;
    fq.C = md->LQ;
    fq.g[0] = ig(PRO_NONE, md->g_dq, md->LQ, 0);
    G2SPlan gq;
    memset(&gq, 0, sizeof(gq));
    gq.ng = 1;
    gq.C = md->LQ;
    gq.g[0] = og2(G2S_PLAIN, md->spe_dq, md->LQ, 0, 0, -1, -1);
    JG_TRY(launch_g2s<T>(m, fq, gq, st, md->fbuf, md->fcap));
  }
  // 4. semi-implicit correction, damping, leapfrog (FP64, warp per mode)
  ImplArgs<T> ia;
  memset(&ia, 0, sizeof(ia));
  using V = V2<T>;
  ia.dvor = (const V*)md->spe_dvor;
  ia.ddiv = (const V*)md->spe_ddiv;
  ia.dtend = (const V*)md->spe_dt;
  ia.dlnps = (const V*)md->spe_dlnps;
  ia.vor_p = (V*)md->spe_vor[p]; ia.vor_c = (V*)md->spe_vor[c]; ia.vor_n = (V*)md->spe_vor[n];
  ia.div_p = (V*)md->spe_div[p]; ia.div_c = (V*)md->spe_div[c]; ia.div_n = (V*)md->spe_div[n];
  ia.t_p = (V*)md->spe_t[p]; ia.t_c = (V*)md->spe_t[c]; ia.t_n = (V*)md->spe_t[n];
  ia.lnps_p = (V*)md->spe_lnps[p]; ia.lnps_c = (V*)md->spe_lnps[c]; ia.lnps_n = (V*)md->spe_lnps[n];
  ia.eig64 = m->t64.eig;
  ia.damping = (const T*)md->damping;
  ia.dfac = (const T*)md->dfac[md->init_step ? 0 : 1];
  ia.W = md->d_W + (md->init_step ? 0 : (size_t)(m->N + 1) * nd * nd);
  ia.pairs = md->d_pairs;
  ia.npairs = md->npairs;
  ia.nd = nd;
  ia.L = L;
  ia.ne = E;
  ia.ns = m->ns;
  ia.N = m->N;
  ia.init_step = md->init_step;
  ia.dt = md->P.dt;
  ia.xi = md->init_step ? md->P.dt * md->P.implicit_coef : (2 * md->P.dt) * md->P.implicit_coef;
  ia.ps_ref = md->P.ps_ref;
  ia.kappa = md->P.kappa;
  ia.rdgas = md->P.rdgas;
  ia.robert = md->P.robert_coef;
  impl_consts<T>(ia, tables<T>(md->mesh).eig);
  ia.nq = md->nq;
  ia.LQ = md->LQ;
  if (md->nq) {
    ia.dq = (const V*)md->spe_dq;
    ia.q_p = (V*)md->spe_q[p];
    ia.q_c = (V*)md->spe_q[c];
    ia.q_n = (V*)md->spe_q[n];
  }
  // vertical algebra in the state precision (FP64 algebra on the FP32 path measured no more
  // accurate: its error is set by FP32 storage); the wave-matrix solve is FP64 in both
  // 4 modes per block: (N+1)(N+2)/2 + N+1 modes at T42 make 248 blocks, every SM's FP64 units busy;
  // member ensembles (from 4 members) spread the FP64 products densely over each block
  if (E >= 4)
    JG_CUDA(launch_pdl(k_hs_implicit<T, T, true>, dim3((md->npairs + 3) / 4, E), 128, 0, st, ia, md->d_vc));
  else
    JG_CUDA(launch_pdl(k_hs_implicit<T, T>, dim3((md->npairs + 3) / 4, E), 128, 0, st, ia, md->d_vc));
  mark(st);
  JG_CUDA(cudaGetLastError());
  // 5. back to the grid: vor, div, u, v, T, lnps (+ ps = exp(lnps)), and the next step's gradients
  //    of ln ps and T (Compute_Gradients!, Spectral_Spherical_Mesh.jl:721-741): they read no (0,0)
  //    mode (its coefficients m/a and (n-1) ε_n/a vanish), so the fixers' later shifts of those
  //    modes leave them unchanged
  S2GPlan s2;
  memset(&s2, 0, sizeof(s2));
  s2.ng = 10;
  s2.C = 7 * L + 3 * E;
  s2.g[0] = sg(S2G_PLAIN, md->spe_vor[n], nullptr, L, 0);
  s2.g[1] = sg(S2G_PLAIN, md->spe_div[n], nullptr, L, L);
  s2.g[2] = sg(S2G_UCOS, md->spe_vor[n], md->spe_div[n], L, 2 * L);
  s2.g[3] = sg(S2G_VCOS, md->spe_vor[n], md->spe_div[n], L, 3 * L);
  // FP32: T synthesised without its level means; the epilogue writes grid T (+ the means) and the
  // anomaly itself for the next step's geopotential (the fixer's shift of T leaves it unchanged)
  const bool anom = std::is_same<T, float>::value;
  s2.g[4] = sg(anom ? S2G_ANOM : S2G_PLAIN, md->spe_t[n], nullptr, L, 4 * L);
  // ln ps is synthesised as ln ps - ln 1e5 (mode (0,0) shifted; P_00 = 1) and shifted back in the
  // epilogue, so its rounding scales with |ln(ps / 1e5)| ~ 0.02 instead of ln ps ~ 11.5
  s2.g[5] = sg(S2G_PLAIN, md->spe_lnps[n], nullptr, E, 5 * L);
  s2.g[5].shift = kLnPsRef;
  s2.g[6] = sg(S2G_DLAM, md->spe_lnps[n], nullptr, E, 5 * L + E);
  s2.g[7] = sg(S2G_DTH, md->spe_lnps[n], nullptr, E, 5 * L + 2 * E);
  s2.g[8] = sg(S2G_DLAM, md->spe_t[n], nullptr, L, 5 * L + 3 * E);
  s2.g[9] = sg(S2G_DTH, md->spe_t[n], nullptr, L, 6 * L + 3 * E);
  IFFTPlan i2;
  memset(&i2, 0, sizeof(i2));
  i2.ng = s2.ng;
  i2.C = s2.C;
  i2.g[0] = og(EPI_NONE, md->grid_vor, L, 0);
  i2.g[1] = og(EPI_NONE, md->grid_div, L, L);
  i2.g[2] = og(EPI_DIVCOS, md->grid_u[n], L, 2 * L);
  i2.g[3] = og(EPI_DIVCOS, md->grid_v[n], L, 3 * L);
  i2.g[4] = og(anom ? EPI_ANOM : EPI_NONE, md->grid_t[n], L, 4 * L, anom ? md->g_tdev : nullptr);
  i2.g[4].ps = anom ? md->spe_t[n] : nullptr;
  i2.g[5] = og(EPI_EXP2, md->grid_lnps, E, 5 * L, md->grid_ps[n]);
  i2.g[5].shift = kLnPsRef;
  i2.g[6] = og(EPI_DIVCOS, md->g_dlps, E, 5 * L + E);
  i2.g[7] = og(EPI_DIVCOS, md->g_dtps, E, 5 * L + 2 * E);
  i2.g[8] = og(EPI_DIVCOS, md->g_dlT, L, 5 * L + 3 * E);
  i2.g[9] = og(EPI_DIVCOS, md->g_dtT, L, 6 * L + 3 * E);
  if (md->nq) {  // the tracers' new level and its gradients
    const int LQ = md->LQ, c0 = s2.C;
    s2.g[10] = sg(S2G_PLAIN, md->spe_q[n], nullptr, LQ, c0);
    s2.g[11] = sg(S2G_DLAM, md->spe_q[n], nullptr, LQ, c0 + LQ);
    s2.g[12] = sg(S2G_DTH, md->spe_q[n], nullptr, LQ, c0 + 2 * LQ);
    i2.g[10] = og(EPI_NONE, md->grid_q[n], LQ, c0);
    i2.g[11] = og(EPI_DIVCOS, md->g_dlq, LQ, c0 + LQ);
    i2.g[12] = og(EPI_DIVCOS, md->g_dtq, LQ, c0 + 2 * LQ);
    s2.ng = i2.ng = 13;
    s2.C = i2.C = c0 + 3 * LQ;
  }
  JG_TRY(launch_s2g<T>(m, s2, i2, st, md->fbuf, md->fcap));
  // 6. mass and energy fixers
  CorrArgs<T> ca;
  memset(&ca, 0, sizeof(ca));
  ca.u_n = (const T*)md->grid_u[n];
  ca.v_n = (const T*)md->grid_v[n];
  ca.t_n = (const T*)md->grid_t[n];
  ca.ps_n = (const T*)md->grid_ps[n];
  ca.lnps_n = (V*)md->spe_lnps[n];
  ca.t_spec_n = (V*)md->spe_t[n];
  ca.wts = m->d_wts;
  ca.partials = md->d_partials;
  ca.scalars = md->d_scalars;
  ca.scal_t = (T*)(md->d_scalars + 4 * E);
  ca.counter = md->d_counter;
  ca.nd = nd;
  ca.pstride = partial_stride(m);
  ca.col_gx = (m->nlon + HS_CT / md->hs_lanes - 1) / (HS_CT / md->hs_lanes);
  ca.col_nb = ca.col_gx * m->nlat;
  ca.col_off = col_partials(m);
  ca.nlat = m->nlat;
  ca.nlon = m->nlon;
  ca.do_mass = md->P.do_mass_correction;
  ca.do_energy = md->P.do_energy_correction;
  ca.cp = md->cp_air;
  ca.grav = md->P.grav;
  ca.inv_2n = 0.5 / m->nlon;
  ca.cp_t = (T)md->cp_air;
  ca.cp_hi = (float)md->cp_air;
  ca.cp_lo = (float)(md->cp_air - (double)ca.cp_hi);
  ca.has_dak = has_dak(md);
  {
    // clusters when the grid is one wave of blocks (8 of these per SM), groups otherwise
    const int gx = (m->nlon + 31) / 32;
    if ((size_t)gx * m->nlat * E <= (size_t)8 * m->sm_count) {
      int cx, cy;
      corr_cluster(gx, m->nlat, cx, cy);
      JG_CUDA(launch_pdl_cluster(k_hs_corr_reduce<T, true>, dim3(gx, m->nlat, E), 256, 0, st, dim3(cx, cy, 1), ca,
                                 md->d_vc));
    } else {
      JG_CUDA(launch_pdl(k_hs_corr_reduce<T, false>, dim3(gx, m->nlat, E), 256, 0, st, ca, md->d_vc));
    }
  }
  mark(st);
  JG_CUDA(cudaGetLastError());
  const size_t G1 = grid_elems(m, 1);
  int nb = (int)(((size_t)nd * G1 + 255) / 256);
  if (nb * E > 8 * m->sm_count) nb = (8 * m->sm_count + E - 1) / E;
  JG_CUDA(launch_pdl(k_hs_corr_apply<T>, dim3(nb, E), 256, 0, st, (T*)md->grid_t[n], (T*)md->grid_ps[n],
                     (const T*)(md->d_scalars + 4 * E), (size_t)nd * G1, G1));
  mark(st);
  JG_CUDA(cudaGetLastError());
  if (md->diag_on && g_marker == nullptr) JG_TRY(issue_diag<T>(md, n, st));  // the new state, after the fixers
  return JGCM_OK;
}

template <typename T>
int issue_step(jgcm_model* md, cudaStream_t st) {
  switch (md->P.kind) {
    case JGCM_BAROTROPIC:
      return step_barotropic<T>(md, st);
    case JGCM_SHALLOW_WATER:
      return step_shallow_water<T>(md, st);
    default:
      return step_held_suarez<T>(md, st);
  }
}

int issue(jgcm_model* md, cudaStream_t st) {
  return is_fp64(md->mesh) ? issue_step<double>(md, st) : issue_step<float>(md, st);
}

void after_step(jgcm_model* md) {
  md->grad_ready = md->P.kind == JGCM_HELD_SUAREZ;
  if (md->diag_on) md->diag_steps++;
  md->rot = (md->rot + 1) % 3;
  md->init_step = 0;
  md->sw_adv_from_n = 0;
  md->steps_done++;
}

// One steady step through a CUDA graph captured for the current rotation phase.
void drop_graphs(jgcm_model* md) {
  for (auto& g : md->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  for (auto& g : md->graph3)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
  for (auto& g : md->graph24)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

int graph_step(jgcm_model* md) {
  jgcm_mesh* m = md->mesh;
  if (md->graph_gen != m->tune_gen) {  // tiles changed since the capture
    drop_graphs(md);
    md->graph_gen = m->tune_gen;
  }
  int ph = md->rot;
  if (!md->graph[ph]) {
    cudaGraph_t g;
    JG_CUDA(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
    int s = issue(md, m->stream);
    cudaError_t e = cudaStreamEndCapture(m->stream, &g);
    if (s != JGCM_OK) {
      if (e == cudaSuccess) cudaGraphDestroy(g);
      return s;
    }
    JG_CUDA(e);
    cudaError_t e2 = cudaGraphInstantiate(&md->graph[ph], g, 0);
    cudaGraphDestroy(g);
    JG_CUDA(e2);
  }
  JG_CUDA(cudaGraphLaunch(md->graph[ph], m->stream));
  after_step(md);
  return JGCM_OK;
}

// K steady steps through one CUDA graph (K a multiple of 3: whole time-level rotations): fewer graph
// launches, and the step boundaries inside become ordinary (programmatic) kernel edges.
bool steady(const jgcm_model* md) {
  return !(md->init_step || md->sw_adv_from_n || (md->P.kind == JGCM_HELD_SUAREZ && !md->grad_ready));
}

int graph_steps(jgcm_model* md, int K, cudaGraphExec_t* slots) {
  jgcm_mesh* m = md->mesh;
  if (md->graph_gen != m->tune_gen) {
    drop_graphs(md);
    md->graph_gen = m->tune_gen;
  }
  const int ph = md->rot;
  if (!slots[ph]) {
    // capture: the host-side bookkeeping of the three steps is replayed below, so restore it after
    const int rot = md->rot, gr = md->grad_ready, init = md->init_step, adv = md->sw_adv_from_n;
    const int done = md->steps_done;
    const long dsteps = md->diag_steps;
    cudaGraph_t g;
    JG_CUDA(cudaStreamBeginCapture(m->stream, cudaStreamCaptureModeThreadLocal));
    int s = JGCM_OK;
    for (int k = 0; k < K && s == JGCM_OK; k++) {
      s = issue(md, m->stream);
      after_step(md);
    }
    cudaError_t e = cudaStreamEndCapture(m->stream, &g);
    md->rot = rot;
    md->grad_ready = gr;
    md->init_step = init;
    md->sw_adv_from_n = adv;
    md->steps_done = done;
    md->diag_steps = dsteps;
    if (s != JGCM_OK) {
      if (e == cudaSuccess) cudaGraphDestroy(g);
      return s;
    }
    JG_CUDA(e);
    cudaError_t e2 = cudaGraphInstantiate(&slots[ph], g, 0);
    cudaGraphDestroy(g);
    JG_CUDA(e2);
  }
  JG_CUDA(cudaGraphLaunch(slots[ph], m->stream));
  for (int k = 0; k < K; k++) after_step(md);
  return JGCM_OK;
}
int graph_step3(jgcm_model* md) { return graph_steps(md, 3, md->graph3); }
int graph_step24(jgcm_model* md) { return graph_steps(md, 24, md->graph24); }

int model_step(jgcm_model* md) {
  if (md->init_step || md->sw_adv_from_n || (md->P.kind == JGCM_HELD_SUAREZ && !md->grad_ready)) {
    JG_TRY(issue(md, md->mesh->stream));
    after_step(md);
    return JGCM_OK;
  }
  return graph_step(md);
}

// ------------------------------------------------------------------------------------------
struct FieldRef {
  void* ptr;
  int L;        // levels
  bool spec;    // spectral (complex) vs grid
  bool derived; // computed on demand, FP64 in g_diag at `off`
  size_t off;
  bool state;   // writable
};

bool lookup(jgcm_model* md, const std::string& nm, FieldRef* f) {
  const int nd = md->nd;
  const size_t G = grid_elems(md->mesh, 1);
  auto lev = [&](const std::string& suf) -> int {
    if (suf == "p") return lvl(md, 0);
    if (suf == "c") return lvl(md, 1);
    if (suf == "n") return lvl(md, 2);
    return -1;
  };
  *f = FieldRef{nullptr, 0, false, false, 0, true};
  auto tl = [&](const char* base, void* const* arr, int L, bool spec) -> bool {
    std::string b(base);
    if (nm.size() == b.size() + 2 && nm.compare(0, b.size(), b) == 0 && nm[b.size()] == '_') {
      int l = lev(nm.substr(b.size() + 1));
      if (l < 0) return false;
      *f = FieldRef{arr[l], L, spec, false, 0, true};
      return true;
    }
    return false;
  };
  if (md->nq && (tl("spe_tracers", md->spe_q, nd * md->nq, true) || tl("grid_tracers", md->grid_q, nd * md->nq, false)))
    return true;
  if (tl("spe_vor", md->spe_vor, nd, true) || tl("spe_div", md->spe_div, nd, true) ||
      tl("spe_lnps", md->spe_lnps, 1, true) || tl("spe_t", md->spe_t, nd, true) || tl("grid_u", md->grid_u, nd, false) ||
      tl("grid_v", md->grid_v, nd, false) || tl("grid_ps", md->grid_ps, 1, false) || tl("grid_t", md->grid_t, nd, false))
    return true;
  struct {
    const char* n;
    void* p;
    int L;
    bool spec;
  } single[] = {{"grid_vor", md->grid_vor, nd, false},   {"grid_div", md->grid_div, nd, false},
                {"grid_lnps", md->grid_lnps, 1, false},  {"grid_t_eq", md->grid_t_eq, nd, false},
                {"grid_geopots", md->grid_geopots, 1, false}, {"grid_h_eq", md->grid_h_eq, 1, false}};
  for (auto& s : single)
    if (nm == s.n) {
      *f = FieldRef{s.p, s.L, s.spec, false, 0, true};
      return true;
    }
  struct {
    const char* n;
    int L;
    size_t off;
  } der[] = {{"grid_p_half", nd + 1, 0},
             {"grid_lnp_half", nd + 1, G * (nd + 1)},
             {"grid_dp", nd, 2 * G * (nd + 1)},
             {"grid_p_full", nd, 2 * G * (nd + 1) + G * nd},
             {"grid_lnp_full", nd, 2 * G * (nd + 1) + 2 * G * nd},
             {"grid_z_full", nd, 2 * G * (nd + 1) + 3 * G * nd},
             {"grid_z_half", nd + 1, 2 * G * (nd + 1) + 4 * G * nd}};
  for (auto& d : der)
    if (nm == d.n) {
      *f = FieldRef{nullptr, d.L, false, true, d.off, false};
      return true;
    }
  return false;
}

}  // namespace

// ------------------------------------------------------------------------------------------
extern "C" int jgcm_model_create(jgcm_mesh* mesh, const jgcm_params* params, jgcm_model** out) {
  return jgcm_model_create_members(mesh, params, 1, out);
}

extern "C" int jgcm_model_create_members(jgcm_mesh* mesh, const jgcm_params* params, int members,
                                         jgcm_model** out) {
  return jgcm_model_create_vert(mesh, params, members, nullptr, nullptr, out);
}

extern "C" int jgcm_vert_coord(int nd, const char* option, double scale_heights, double surf_res, double exponent,
                               double* ak, double* bk) {
  JG_ARG(option && ak && bk, "NULL argument");
  JG_ARG(nd >= 1 && nd <= JGCM_MAX_ND, "nd out of range");
  return vert_coord_table(nd, option, scale_heights, surf_res, exponent, ak, bk);
}

extern "C" int jgcm_model_create_vert(jgcm_mesh* mesh, const jgcm_params* params, int members, const double* ak,
                                      const double* bk, jgcm_model** out) {
  JG_ARG(mesh && params && out, "NULL argument");
  JG_ARG((ak == nullptr) == (bk == nullptr), "ak and bk are given together");
  if (bk) {
    const int nd = mesh->nd;
    JG_ARG(ak[0] == 0.0 && bk[0] == 0.0, "the top half level must be zero (a_0 = b_0 = 0, zero_top)");
    JG_ARG(ak[nd] == 0.0 && bk[nd] == 1.0, "the bottom half level must be the surface (a_nd = 0, b_nd = 1)");
    for (int k = 0; k < nd; k++)
      for (double f : {0.9, 1.1}) {  // half-level pressures increase downwards around the reference ps
        const double ps = f * params->ps_ref;
        JG_ARG(ak[k + 1] + bk[k + 1] * ps > ak[k] + bk[k] * ps, "a_k + b_k ps must increase downwards (k = %d)", k);
      }
  }
  *out = nullptr;
  JG_ARG(members >= 1 && members <= 65535, "members must be in [1, 65535]");
  JG_ARG(params->kind >= JGCM_BAROTROPIC && params->kind <= JGCM_HELD_SUAREZ, "unknown model kind");
  JG_ARG(params->dt > 0, "dt must be positive");
  JG_ARG(params->damping_order % 2 == 0, "damping_order must be even (Time_Integrator.jl:24)");
  if (params->kind != JGCM_HELD_SUAREZ) JG_ARG(mesh->nd == 1 || params->kind == JGCM_BAROTROPIC, "shallow water needs nd = 1");
  if (params->kind == JGCM_SHALLOW_WATER) JG_ARG(mesh->nd == 1, "shallow water needs nd = 1");
  if (params->kind == JGCM_HELD_SUAREZ) JG_ARG(mesh->nd <= 32, "Held-Suarez supports nd <= 32 (one warp per column)");
  jgcm_model* md = new jgcm_model();
  md->mesh = mesh;
  md->P = *params;
  md->nd = mesh->nd;
  md->ne = members;
  md->L = members * mesh->nd;
  md->hs_lanes = hs_lanes(mesh, members, mesh->nd);
  md->init_step = 1;
  md->sw_adv_from_n = 1;
  md->cp_air = params->rdgas / params->kappa;
  if (bk) {
    md->vert_bk.assign(bk, bk + mesh->nd + 1);
    md->vert_ak.assign(ak, ak + mesh->nd + 1);
  }
  int s = model_alloc(md);
  if (s != JGCM_OK) {
    model_free(md);
    return s;
  }
  mesh_retain(mesh);
  *out = md;
  return JGCM_OK;
}

// Passive tracers on a Held-Suarez model: nq per member, every time level zero, advected like T
// by every later step (k_hs_tracers, the tracers' analysis, their leapfrog in k_hs_implicit, their
// synthesis with the new level).  Once per model; drops the captured graphs.
extern "C" int jgcm_model_add_tracers(jgcm_model* md, int num_tracers) {
  JG_ARG(md, "NULL model");
  JG_ARG(md->P.kind == JGCM_HELD_SUAREZ, "tracers are advected by the Held-Suarez model only");
  JG_ARG(md->nq == 0, "the model already has %d tracers", md->nq);
  JG_ARG(num_tracers >= 1 && num_tracers <= 64, "num_tracers must be in [1, 64]");
  jgcm_mesh* m = md->mesh;
  JG_CUDA(cudaStreamSynchronize(m->stream));
  const int nd = md->nd, ne = md->ne, LQ = num_tracers * nd * ne;
  const size_t ts = tsize(m), S = spec_elems(m, LQ) * 2 * ts, G = grid_elems(m, LQ) * ts;
  auto zalloc = [&](void** p, size_t bytes) -> int {
    JG_CUDA(cudaMalloc(p, bytes));
    JG_CUDA(cudaMemsetAsync(*p, 0, bytes, m->stream));
    return JGCM_OK;
  };
  for (int i = 0; i < 3; i++) {
    JG_TRY(zalloc(&md->spe_q[i], S));
    JG_TRY(zalloc(&md->grid_q[i], G));
  }
  JG_TRY(zalloc(&md->spe_dq, S));
  JG_TRY(zalloc(&md->g_dq, G));
  JG_TRY(zalloc(&md->g_dlq, G));
  JG_TRY(zalloc(&md->g_dtq, G));
  JG_TRY(zalloc(&md->g_mhalf, grid_elems(m, md->L) * ts));
  const size_t nstage = std::max(grid_elems(m, num_tracers * nd), 2 * spec_elems(m, num_tracers * nd));
  JG_TRY(zalloc((void**)&md->q_stage, nstage * 8));
  // the Fourier buffer holds the widest plan: the step's synthesis with the tracers' 3 LQ columns
  const int fcap = (7 * nd + 3) * ne + 3 * LQ;
  void* fbuf = nullptr;
  JG_TRY(zalloc(&fbuf, (size_t)(m->N + 1) * m->nlat * fcap * 2 * ts));
  JG_CUDA(cudaFree(md->fbuf));
  md->fbuf = fbuf;
  md->fcap = fcap;
  md->nq = num_tracers;
  md->LQ = LQ;
  md->grad_ready = 0;
  drop_graphs(md);
  JG_CUDA(cudaStreamSynchronize(m->stream));
  return JGCM_OK;
}

extern "C" int jgcm_model_num_tracers(jgcm_model* md, int* num_tracers) {
  JG_ARG(md && num_tracers, "NULL argument");
  *num_tracers = md->nq;
  return JGCM_OK;
}

extern "C" int jgcm_model_destroy(jgcm_model* md) {
  if (!md) return JGCM_OK;
  jgcm_mesh* m = md->mesh;
  cudaStreamSynchronize(m->stream);
  model_free(md);
  mesh_release(m);
  return JGCM_OK;
}

extern "C" int jgcm_model_step(jgcm_model* md, int nsteps) {
  JG_ARG(md && nsteps >= 0, "bad arguments");
  for (int s = 0; s < nsteps;) {
    if (nsteps - s >= 24 && steady(md)) {
      JG_TRY(graph_step24(md));
      s += 24;
    } else if (nsteps - s >= 3 && steady(md)) {
      JG_TRY(graph_step3(md));
      s += 3;
    } else {
      JG_TRY(model_step(md));
      s++;
    }
  }
  JG_CUDA(cudaStreamSynchronize(md->mesh->stream));
  if (md->mesh->tc.on) JG_TRY(tc_status(md->mesh));  // a tensor-core kernel whose bounded wait gave up
  return JGCM_OK;
}

extern "C" int jgcm_model_init_step(jgcm_model* md, int* init_step) {
  JG_ARG(md && init_step, "NULL argument");
  *init_step = md->init_step;
  return JGCM_OK;
}

// Sets the init-step flag (Get_Δt: Δt on the first step, 2Δt afterwards): restarting a run from a
// stored first state.  The device holds the wave matrices of both flags.
extern "C" int jgcm_model_set_init_step(jgcm_model* md, int init_step) {
  JG_ARG(md, "NULL model");
  JG_CUDA(cudaStreamSynchronize(md->mesh->stream));
  md->init_step = init_step != 0;
  md->grad_ready = 0;
  return JGCM_OK;
}

extern "C" int jgcm_model_update_init_step(jgcm_model* md) {
  JG_ARG(md, "NULL argument");
  JG_ARG(md->init_step, "Update_Init_Step!: the model is not in its init step (@assert(integrator.init_step))");
  md->init_step = 0;  // the steady wave matrices are already built; the next step selects them
  return JGCM_OK;
}

static int launches_per_step(const jgcm_model* md) {
  return md->P.kind == JGCM_BAROTROPIC ? 4 : md->P.kind == JGCM_SHALLOW_WATER ? 6 : md->nq ? 11 : 8;
}

extern "C" int jgcm_model_launches_per_step(jgcm_model* md, int* launches) {
  JG_ARG(md && launches, "NULL argument");
  *launches = launches_per_step(md);
  return JGCM_OK;
}

extern "C" int jgcm_model_kernel_name(jgcm_model* md, int slot, char* buf, int cap) {
  JG_ARG(md && buf && cap > 0, "bad arguments");
  static const char* hs[] = {"hs_column", "fft(tendencies)", "g2s_legendre(vor,div,T,lnps)", "hs_implicit",
                             "s2g_legendre(vor,div,u,v,T,lnps,grad lnps,grad T)",
                             "ifft(vor,div,u,v,T,lnps,grad lnps,grad T)", "hs_corr_reduce", "hs_corr_apply"};
  static const char* bt[] = {"fft(flux)", "g2s_legendre(vor+leapfrog)", "s2g_legendre(vor,u,v)", "ifft(vor,u,v)"};
  static const char* sw[] = {"s2g_legendre(grad h)", "ifft(grad h)", "fft(fluxes,kin,dh)",
                             "g2s_legendre(vor,div,h+implicit+leapfrog)", "s2g_legendre(vor,div,h,u,v)",
                             "ifft(vor,div,h,u,v)"};
  static const char* hsq[] = {"hs_column", "hs_tracers", "fft(tendencies)", "g2s_legendre(vor,div,T,lnps)",
                              "fft(tracers)", "g2s_legendre(tracers)", "hs_implicit",
                              "s2g_legendre(vor,div,u,v,T,lnps,grad lnps,grad T,tracers)",
                              "ifft(vor,div,u,v,T,lnps,grad lnps,grad T,tracers)", "hs_corr_reduce", "hs_corr_apply"};
  const char** names = md->P.kind == JGCM_HELD_SUAREZ ? (md->nq ? hsq : hs) : md->P.kind == JGCM_BAROTROPIC ? bt : sw;
  JG_ARG(slot >= 0 && slot < launches_per_step(md), "slot out of range");
  snprintf(buf, cap, "%s", names[slot]);
  return JGCM_OK;
}

// Holds the stream for a fixed number of SM clock cycles (bounded: no flag, no external wait), so
// the launches queued behind it run back to back and their events time the device alone.
__global__ void k_hold(long long cycles) {
  const long long t0 = clock64();
  while (clock64() - t0 < cycles) {
  }
}

// Per-kernel device times of steady steps: every launch is followed by an event (eager launches
// queued behind k_hold, events on the model stream), ms[slot] = mean over nsteps of
// event(slot) - event(slot - 1).
extern "C" int jgcm_model_kernel_times(jgcm_model* md, int nsteps, float* ms, int cap, int* count) {
  JG_ARG(md && ms && count && nsteps > 0, "bad arguments");
  jgcm_mesh* m = md->mesh;
  const int L = launches_per_step(md);
  JG_ARG(cap >= L, "buffer too small");
  if (md->init_step || (md->P.kind == JGCM_HELD_SUAREZ && !md->grad_ready)) JG_TRY(model_step(md));
  struct DiagOff {  // the timed steps run without the diagnostics' reductions (and are not summed)
    jgcm_model* md;
    int saved;
    ~DiagOff() { md->diag_on = saved; }
  } diag_off{md, md->diag_on};
  md->diag_on = 0;
  std::vector<cudaEvent_t> ev((size_t)nsteps * L + 1);
  for (auto& e : ev) JG_CUDA(cudaEventCreate(&e));
  Marker mk{ev.data() + 1, 0, nsteps * L};
  JG_CUDA(cudaStreamSynchronize(m->stream));
  // ~1 ms + ~6 us per queued launch at 2 GHz (capped at ~20 ms): the host queues every launch
  // before the first one starts
  long long hold = 2000000LL + (long long)nsteps * L * 12000LL;
  k_hold<<<1, 1, 0, m->stream>>>(hold < 40000000LL ? hold : 40000000LL);
  JG_CUDA(cudaGetLastError());
  JG_CUDA(cudaEventRecord(ev[0], m->stream));
  g_marker = &mk;
  int st = JGCM_OK;
  for (int s = 0; s < nsteps && st == JGCM_OK; s++) {
    st = issue(md, m->stream);
    if (st == JGCM_OK) after_step(md);
  }
  g_marker = nullptr;
  if (st == JGCM_OK) {
    cudaError_t e = cudaEventSynchronize(ev.back());
    if (e != cudaSuccess) {
      set_error("kernel timing: %s", cudaGetErrorString(e));
      st = JGCM_E_CUDA;
    }
  }
  if (st == JGCM_OK && mk.n != nsteps * L) {
    set_error("kernel timing: %d launches recorded, %d expected", mk.n, nsteps * L);
    st = JGCM_E_STATE;
  }
  if (st == JGCM_OK) {
    for (int k = 0; k < L; k++) ms[k] = 0.0f;
    for (int s = 0; s < nsteps; s++)
      for (int k = 0; k < L; k++) {
        float t = 0.0f;
        cudaEventElapsedTime(&t, ev[(size_t)s * L + k], ev[(size_t)s * L + k + 1]);
        ms[k] += t / nsteps;
      }
    *count = L;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return st;
}

extern "C" int jgcm_model_time_steps(jgcm_model* md, int nsteps, float* ms) {
  JG_ARG(md && ms && nsteps > 0, "bad arguments");
  jgcm_mesh* m = md->mesh;
  while (md->init_step || md->sw_adv_from_n || (md->P.kind == JGCM_HELD_SUAREZ && !md->grad_ready))
    JG_TRY(model_step(md));
  // capture every rotation phase before timing (after a tile change the graphs are rebuilt)
  auto captured = [&]() {
    if (md->graph_gen != m->tune_gen) return false;
    for (auto g : md->graph)
      if (!g) return false;
    for (auto g : md->graph3)
      if (!g) return false;
    if (nsteps >= 24)
      for (auto g : md->graph24)
        if (!g) return false;
    return true;
  };
  for (int s = 0; s < 3 && !captured(); s++) {
    JG_TRY(graph_step(md));
    JG_TRY(graph_step3(md));
    if (nsteps >= 24) JG_TRY(graph_step24(md));
  }
  JG_CUDA(cudaStreamSynchronize(m->stream));
  JG_CUDA(cudaEventRecord(md->ev0, m->stream));
  for (int s = 0; s < nsteps;) {
    if (nsteps - s >= 24) {
      JG_TRY(graph_step24(md));
      s += 24;
    } else if (nsteps - s >= 3) {
      JG_TRY(graph_step3(md));
      s += 3;
    } else {
      JG_TRY(graph_step(md));
      s++;
    }
  }
  JG_CUDA(cudaEventRecord(md->ev1, m->stream));
  JG_CUDA(cudaEventSynchronize(md->ev1));
  JG_CUDA(cudaEventElapsedTime(ms, md->ev0, md->ev1));
  return JGCM_OK;
}

extern "C" int jgcm_model_get_field(jgcm_model* md, const char* name, double* host, long cap, long* count) {
  JG_ARG(md && name, "NULL argument");
  JG_ARG(md->ne == 1, "an ensemble's fields are read through jgcm_model_copy_member into a one-member model");
  FieldRef f;
  JG_ARG(lookup(md, name, &f), "unknown field '%s'", name);
  jgcm_mesh* m = md->mesh;
  size_t n = f.spec ? 2 * spec_elems(m, f.L) : grid_elems(m, f.L);
  if (count) *count = (long)n;
  if (!host) return JGCM_OK;
  JG_ARG(cap >= (long)n, "buffer too small for '%s'", name);
  cudaStream_t st = m->stream;
  double* stage = n <= 4 * m->stage_slot ? m->d_stage : md->q_stage;  // tracer fields may need their own
  if (f.derived) {
    size_t G = grid_elems(m, 1);
    int nb = (int)((G + 127) / 128);
    int c = lvl(md, 1);
    if (is_fp64(m))
      k_pressure_heights<double><<<nb, 128, 0, st>>>((const double*)md->grid_ps[c], (const double*)md->grid_t[c],
                                                     (const double*)md->grid_geopots, (double*)md->g_diag, md->d_vc,
                                                     md->nd, G, md->P.rdgas, md->P.grav);
    else
      k_pressure_heights<float><<<nb, 128, 0, st>>>((const float*)md->grid_ps[c], (const float*)md->grid_t[c],
                                                    (const float*)md->grid_geopots, (double*)md->g_diag, md->d_vc,
                                                    md->nd, G, md->P.rdgas, md->P.grav);
    JG_CUDA(cudaGetLastError());
    JG_CUDA(cudaMemcpyAsync(host, (double*)md->g_diag + f.off, n * 8, cudaMemcpyDeviceToHost, st));
  } else if (f.spec) {
    JG_TRY(spec_dev_to_host(m, f.ptr, stage, f.L, st));
    JG_CUDA(cudaMemcpyAsync(host, stage, n * 8, cudaMemcpyDeviceToHost, st));
  } else {
    JG_TRY(grid_dev_to_host(m, f.ptr, stage, n, st));
    JG_CUDA(cudaMemcpyAsync(host, stage, n * 8, cudaMemcpyDeviceToHost, st));
  }
  JG_CUDA(cudaStreamSynchronize(st));
  return JGCM_OK;
}

extern "C" int jgcm_model_set_field(jgcm_model* md, const char* name, const double* host, long count) {
  JG_ARG(md && name && host, "NULL argument");
  JG_ARG(md->ne == 1, "an ensemble's fields are written through jgcm_model_copy_member from a one-member model");
  FieldRef f;
  JG_ARG(lookup(md, name, &f), "unknown field '%s'", name);
  JG_ARG(f.state, "field '%s' is derived and cannot be set", name);
  jgcm_mesh* m = md->mesh;
  size_t n = f.spec ? 2 * spec_elems(m, f.L) : grid_elems(m, f.L);
  JG_ARG(count == (long)n, "field '%s' needs %zu doubles, got %ld", name, n, count);
  cudaStream_t st = m->stream;
  double* stage = n <= 4 * m->stage_slot ? m->d_stage : md->q_stage;  // tracer fields may need their own
  JG_CUDA(cudaStreamSynchronize(st));
  JG_CUDA(cudaMemcpyAsync(stage, host, n * 8, cudaMemcpyHostToDevice, st));
  if (f.spec)
    JG_TRY(spec_host_to_dev(m, stage, f.ptr, f.L, st));
  else
    JG_TRY(grid_host_to_dev(m, stage, f.ptr, n, st));
  if (!strcmp(name, "spe_lnps_n")) md->sw_adv_from_n = 1;
  md->grad_ready = 0;  // the gradients of the current level are recomputed by the next step
  JG_CUDA(cudaStreamSynchronize(st));
  return JGCM_OK;
}

extern "C" int jgcm_model_semi_implicit(jgcm_model* md, const char* name, double* out, long cap, long* count) {
  JG_ARG(md && name, "NULL argument");
  JG_ARG(md->P.kind == JGCM_HELD_SUAREZ, "semi-implicit matrices exist for Held-Suarez only");
  const int nd = md->nd, N = md->mesh->N;
  std::string nm(name);
  std::vector<double> res;
  if (nm == "div_mat") res.assign(md->div_mat, md->div_mat + nd * nd);
  else if (nm == "h") res.assign(md->vc.h, md->vc.h + nd);
  else if (nm == "wave_matrix") {
    std::vector<double> w((size_t)(N + 1) * nd * nd);
    size_t off = md->init_step ? 0 : (size_t)(N + 1) * nd * nd;
    JG_CUDA(cudaMemcpy(w.data(), md->d_W + off, w.size() * 8, cudaMemcpyDeviceToHost));
    res.assign(w.size(), 0.0);
    for (int n = 0; n <= N; n++)
      for (int c = 0; c < nd; c++)
        for (int r = 0; r < nd; r++) res[(size_t)n * nd * nd + r + (size_t)nd * c] = w[(size_t)n * nd * nd + (size_t)c * nd + r];
  } else {
    set_error("unknown semi-implicit item '%s'", name);
    return JGCM_E_ARG;
  }
  if (count) *count = (long)res.size();
  if (out) {
    JG_ARG(cap >= (long)res.size(), "buffer too small");
    memcpy(out, res.data(), res.size() * 8);
  }
  return JGCM_OK;
}

// HS_Forcing! (HS_Forcing.jl:1-130) on caller arrays: Rayleigh_Damping! (:101-130), the
// energy-conserving frictional heating (:21-26) and Newtonian_Damping! (:37-97), elementwise over
// the [nλ, nθ, nd] grid in the model's precision.  sigma = p_full / ps with ps = p_half[:, :, nd+1],
// as the reference computes it (the fused step kernel uses the sigma levels of even_sigma instead).
namespace {
struct HSForcingArgs {
  const double *u, *v, *p_half, *p_full, *t, *sinth;
  double *du, *dv, *t_eq, *dt;
  int nlon, nlat, nd, Dt;
  double sigma_b, k_f, k_a, k_s, dT_y, dtheta_z, kappa, cp;
};

template <typename T>
__global__ void k_hs_forcing(HSForcingArgs a) {
  const size_t G = (size_t)a.nlon * a.nlat, n = G * a.nd;
  const T day = (T)86400, sb = (T)a.sigma_b, Dt = (T)a.Dt;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x) {
    const size_t k = x / G, c = x - k * G;
    const int j = (int)(c / a.nlon);
    const T sj = (T)a.sinth[j], s2 = sj * sj, c2 = (T)1 - s2, c4 = c2 * c2;
    const T pf = (T)a.p_full[x], ps = (T)a.p_half[c + G * a.nd];
    const T smax = fmax(pf / ps - sb, (T)0);
    const T k_v = ((T)a.k_f / day) / ((T)1 - sb) * smax;
    const T u = (T)a.u[x], v = (T)a.v[x];
    const T du = -k_v * u, dv = -k_v * v;
    T dt = -((u + (T)0.5 * du * Dt) * du + (v + (T)0.5 * dv * Dt) * dv) / (T)a.cp;
    const T pn = pf / (T)1.0e5;
    T teq = ((T)315 - (T)a.dT_y * s2 - (T)a.dtheta_z * c2 * log(pn)) * pow(pn, (T)a.kappa);
    teq = fmax(teq, (T)200);
    const T ka = (T)a.k_a / day, ks = (T)a.k_s / day;
    const T k_t = ka + (ks - ka) / ((T)1 - sb) * smax * c4;
    dt -= k_t * ((T)a.t[x] - teq);
    a.du[x] = (double)du;
    a.dv[x] = (double)dv;
    a.t_eq[x] = (double)teq;
    a.dt[x] = (double)dt;
  }
}
}  // namespace

extern "C" int jgcm_hs_forcing(jgcm_model* md, int Dt, const double* grid_u, const double* grid_v,
                               const double* grid_p_half, const double* grid_p_full, const double* grid_t,
                               double* grid_du, double* grid_dv, double* grid_t_eq, double* grid_dt) {
  JG_ARG(md, "NULL model");
  JG_ARG(md->P.kind == JGCM_HELD_SUAREZ, "HS_Forcing! needs a Held-Suarez model (its physics parameters)");
  JG_ARG(Dt > 0, "Δt must be positive");
  JG_ARG(grid_u && grid_v && grid_p_half && grid_p_full && grid_t && grid_du && grid_dv && grid_t_eq && grid_dt,
         "NULL array");
  jgcm_mesh* m = md->mesh;
  const size_t G = (size_t)m->nlon * m->nlat, n = G * md->nd, nh = G * (md->nd + 1);
  double* buf = nullptr;
  JG_CUDA(cudaMalloc(&buf, (8 * n + nh) * sizeof(double)));
  int st = JGCM_OK;
  auto cp = [&](cudaError_t e) {
    if (e != cudaSuccess && st == JGCM_OK) {
      set_error("HS_Forcing! staging: %s", cudaGetErrorString(e));
      st = JGCM_E_CUDA;
    }
  };
  HSForcingArgs a;
  double* d = buf;
  a.u = d;
  a.v = d + n;
  a.p_full = d + 2 * n;
  a.t = d + 3 * n;
  a.du = d + 4 * n;
  a.dv = d + 5 * n;
  a.t_eq = d + 6 * n;
  a.dt = d + 7 * n;
  a.p_half = d + 8 * n;
  a.sinth = m->d_sinth;
  cp(cudaMemcpyAsync((void*)a.u, grid_u, n * 8, cudaMemcpyHostToDevice, m->stream));
  cp(cudaMemcpyAsync((void*)a.v, grid_v, n * 8, cudaMemcpyHostToDevice, m->stream));
  cp(cudaMemcpyAsync((void*)a.p_full, grid_p_full, n * 8, cudaMemcpyHostToDevice, m->stream));
  cp(cudaMemcpyAsync((void*)a.t, grid_t, n * 8, cudaMemcpyHostToDevice, m->stream));
  cp(cudaMemcpyAsync((void*)a.p_half, grid_p_half, nh * 8, cudaMemcpyHostToDevice, m->stream));
  a.nlon = m->nlon;
  a.nlat = m->nlat;
  a.nd = md->nd;
  a.Dt = Dt;
  a.sigma_b = md->P.sigma_b;
  a.k_f = md->P.k_f;
  a.k_a = md->P.k_a;
  a.k_s = md->P.k_s;
  a.dT_y = md->P.dT_y;
  a.dtheta_z = md->P.dtheta_z;
  a.kappa = md->P.kappa;
  a.cp = md->cp_air;
  if (st == JGCM_OK) {
    int nb = (int)std::min<size_t>((n + 255) / 256, 4 * (size_t)m->sm_count);
    if (is_fp64(m)) k_hs_forcing<double><<<nb, 256, 0, m->stream>>>(a);
    else k_hs_forcing<float><<<nb, 256, 0, m->stream>>>(a);
    mark(m->stream);
    cp(cudaGetLastError());
  }
  cp(cudaMemcpyAsync(grid_du, a.du, n * 8, cudaMemcpyDeviceToHost, m->stream));
  cp(cudaMemcpyAsync(grid_dv, a.dv, n * 8, cudaMemcpyDeviceToHost, m->stream));
  cp(cudaMemcpyAsync(grid_t_eq, a.t_eq, n * 8, cudaMemcpyDeviceToHost, m->stream));
  cp(cudaMemcpyAsync(grid_dt, a.dt, n * 8, cudaMemcpyDeviceToHost, m->stream));
  cp(cudaStreamSynchronize(m->stream));
  cudaFree(buf);
  return st;
}

// Spectral_Initialize_Fields! (Spectral_Dynamics.jl:372-449) on the device.
namespace {
// The mixed precisions form the initial state in FP64 (a scratch FP64 mesh and one-member model of
// the same grid, coordinate and parameters) and round it into the model: an FP32 analysis of the
// isothermal 264 K temperature and of ln ps (~11.5) leaves their FP32 rounding (~1e-5 K) in every
// n > 0 mode, where the reference's state holds only the seeded perturbation (0.1 K noise, so a
// 1e-4 relative error before the first step).
int initialize_fields_fp64(jgcm_model* md, const double* grid_t_pert, int vorticity_seed) {
  jgcm_mesh* m = md->mesh;
  jgcm_mesh* m64 = nullptr;
  JG_TRY(jgcm_mesh_create(m->N, m->ns, m->nlat, m->nlon, m->nd, m->radius, JGCM_FP64, &m64));
  jgcm_model* t64 = nullptr;
  int st = jgcm_model_create_vert(m64, &md->P, 1, md->vc.ak, md->vc.bk, &t64);
  static const char* names[] = {"grid_t_c", "grid_t_p", "grid_lnps", "grid_ps_c", "grid_ps_p", "spe_vor_c",
                                "spe_vor_p", "spe_div_c", "spe_div_p", "spe_t_c", "spe_t_p", "spe_lnps_c",
                                "spe_lnps_p", "grid_u_c", "grid_u_p", "grid_v_c", "grid_v_p", "grid_vor", "grid_div"};
  std::vector<double> buf;
  auto move = [&](jgcm_model* dst, jgcm_model* src, const char* nm) -> int {
    long cnt = 0;
    JG_TRY(jgcm_model_get_field(src, nm, nullptr, 0, &cnt));
    buf.resize((size_t)cnt);
    JG_TRY(jgcm_model_get_field(src, nm, buf.data(), cnt, &cnt));
    return jgcm_model_set_field(dst, nm, buf.data(), cnt);
  };
  if (st == JGCM_OK) st = move(t64, md, "grid_geopots");  // the surface geopotential the init reads
  if (st == JGCM_OK) st = jgcm_spectral_initialize_fields(t64, grid_t_pert, vorticity_seed);
  for (const char* nm : names)
    if (st == JGCM_OK) st = move(md, t64, nm);
  if (t64) jgcm_model_destroy(t64);
  jgcm_mesh_destroy(m64);
  return st;
}
}  // namespace

extern "C" int jgcm_spectral_initialize_fields(jgcm_model* md, const double* grid_t_pert, int vorticity_seed) {
  JG_ARG(md, "NULL model");
  JG_ARG(md->ne == 1, "initialise one-member models and copy them into the ensemble (jgcm_model_copy_member)");
  jgcm_mesh* m = md->mesh;
  const int nd = md->nd, N = m->N, ns = m->ns;
  const size_t G = grid_elems(m, 1);
  JG_ARG(N >= 5 && ns >= 9 || !vorticity_seed, "the vorticity seed needs num_fourier >= 5");
  if (!is_fp64(m)) return initialize_fields_fp64(md, grid_t_pert, vorticity_seed);
  // host-side grid fields (FP64), uploaded through set_field
  std::vector<double> gt(G * nd), geo(G), lnps(G), ps(G), spv(2 * spec_elems(m, nd), 0.0);
  long cnt = 0;
  JG_TRY(jgcm_model_get_field(md, "grid_geopots", geo.data(), (long)geo.size(), &cnt));
  for (size_t x = 0; x < G * nd; x++) gt[x] = md->P.init_t + (grid_t_pert ? grid_t_pert[x] : 0.0);
  for (size_t x = 0; x < G; x++) lnps[x] = std::log(md->P.sea_level_ps_ref) - geo[x] / (md->P.rdgas * md->P.init_t);
  for (size_t x = 0; x < G; x++) ps[x] = std::exp(lnps[x]);
  if (vorticity_seed) {
    double ip = 1.0e-7 / std::sqrt(2.0);
    auto six = [&](int mm, int n, int k) { return 2 * ((size_t)mm + (size_t)(N + 1) * ((size_t)n + (size_t)(ns + 1) * k)); };
    for (int k = nd - 3; k < nd; k++) {
      if (k < 0) continue;
      spv[six(1, 4, k)] = ip;
      spv[six(5, 8, k)] = ip;
      spv[six(1, 3, k)] = ip;
      spv[six(5, 7, k)] = ip;
    }
  }
  std::vector<double> zero(spv.size(), 0.0);
  JG_TRY(jgcm_model_set_field(md, "grid_t_c", gt.data(), (long)gt.size()));
  JG_TRY(jgcm_model_set_field(md, "grid_lnps", lnps.data(), (long)lnps.size()));
  JG_TRY(jgcm_model_set_field(md, "grid_ps_c", ps.data(), (long)ps.size()));
  JG_TRY(jgcm_model_set_field(md, "spe_div_c", zero.data(), (long)zero.size()));
  JG_TRY(jgcm_model_set_field(md, "spe_vor_c", spv.data(), (long)spv.size()));
  const int c = lvl(md, 1), p = lvl(md, 0);
  cudaStream_t st = m->stream;
  auto run = [&](auto tag) -> int {
    using T = decltype(tag);
    // UV_Grid_From_Vor_Div!(vor_c, div_c) -> u_c, v_c
    auto uv = [&]() -> int {
      S2GPlan sp;
      memset(&sp, 0, sizeof(sp));
      sp.ng = 2; sp.C = 2 * nd;
      sp.g[0] = sg(S2G_UCOS, md->spe_vor[c], md->spe_div[c], nd, 0);
      sp.g[1] = sg(S2G_VCOS, md->spe_vor[c], md->spe_div[c], nd, nd);
      IFFTPlan ip;
      memset(&ip, 0, sizeof(ip));
      ip.ng = 2; ip.C = 2 * nd;
      ip.g[0] = og(EPI_DIVCOS, md->grid_u[c], nd, 0);
      ip.g[1] = og(EPI_DIVCOS, md->grid_v[c], nd, nd);
      return launch_s2g<T>(m, sp, ip, st);
    };
    auto g2s_plain = [&](const void* grid, void* spec, int L) -> int {
      FFTPlan fp;
      memset(&fp, 0, sizeof(fp));
      fp.ng = 1; fp.C = L;
      fp.g[0] = ig(PRO_NONE, grid, L, 0);
      G2SPlan gp;
      memset(&gp, 0, sizeof(gp));
      gp.ng = 1; gp.C = L;
      gp.g[0] = og2(G2S_PLAIN, spec, L, 0, 0, -1, -1);
      return launch_g2s<T>(m, fp, gp, st);
    };
    auto s2g_plain = [&](const void* spec, void* grid, int L, int epi, void* dst2) -> int {
      S2GPlan sp;
      memset(&sp, 0, sizeof(sp));
      sp.ng = 1; sp.C = L;
      sp.g[0] = sg(S2G_PLAIN, spec, nullptr, L, 0);
      IFFTPlan ip;
      memset(&ip, 0, sizeof(ip));
      ip.ng = 1; ip.C = L;
      ip.g[0] = og(epi, grid, L, 0, dst2);
      return launch_s2g<T>(m, sp, ip, st);
    };
    JG_TRY(uv());
    JG_TRY(g2s_plain(md->grid_t[c], md->spe_t[c], nd));
    JG_TRY(s2g_plain(md->spe_t[c], md->grid_t[c], nd, EPI_NONE, nullptr));
    JG_TRY(g2s_plain(md->grid_lnps, md->spe_lnps[c], 1));
    JG_TRY(s2g_plain(md->spe_lnps[c], md->grid_lnps, 1, EPI_EXP2, md->grid_ps[c]));
    {  // Vor_Div_From_Grid_UV!(u_c, v_c) -> vor_c, div_c
      FFTPlan fp;
      memset(&fp, 0, sizeof(fp));
      fp.ng = 2; fp.C = 2 * nd;
      fp.g[0] = ig(PRO_MULCOS, md->grid_u[c], nd, 0);
      fp.g[1] = ig(PRO_MULCOS, md->grid_v[c], nd, nd);
      G2SPlan gp;
      memset(&gp, 0, sizeof(gp));
      gp.ng = 2; gp.C = 2 * nd;
      gp.g[0] = og2(G2S_VOR, md->spe_vor[c], nd, 0, nd, 0, -1);
      gp.g[1] = og2(G2S_DIV, md->spe_div[c], nd, nd, 0, nd, -1);
      JG_TRY(launch_g2s<T>(m, fp, gp, st));
    }
    JG_TRY(uv());
    JG_TRY(s2g_plain(md->spe_vor[c], md->grid_vor, nd, EPI_NONE, nullptr));
    JG_TRY(s2g_plain(md->spe_div[c], md->grid_div, nd, EPI_NONE, nullptr));
    return JGCM_OK;
  };
  JG_TRY(is_fp64(m) ? run(double()) : run(float()));
  const size_t ts = tsize(m);
  const size_t S = spec_elems(m, nd) * 2 * ts, S1 = spec_elems(m, 1) * 2 * ts, Gb = grid_elems(m, nd) * ts,
               G1 = G * ts;
  JG_CUDA(cudaMemcpyAsync(md->spe_vor[p], md->spe_vor[c], S, cudaMemcpyDeviceToDevice, st));
  JG_CUDA(cudaMemcpyAsync(md->spe_div[p], md->spe_div[c], S, cudaMemcpyDeviceToDevice, st));
  JG_CUDA(cudaMemcpyAsync(md->spe_lnps[p], md->spe_lnps[c], S1, cudaMemcpyDeviceToDevice, st));
  JG_CUDA(cudaMemcpyAsync(md->spe_t[p], md->spe_t[c], S, cudaMemcpyDeviceToDevice, st));
  JG_CUDA(cudaMemcpyAsync(md->grid_u[p], md->grid_u[c], Gb, cudaMemcpyDeviceToDevice, st));
  JG_CUDA(cudaMemcpyAsync(md->grid_v[p], md->grid_v[c], Gb, cudaMemcpyDeviceToDevice, st));
  JG_CUDA(cudaMemcpyAsync(md->grid_ps[p], md->grid_ps[c], G1, cudaMemcpyDeviceToDevice, st));
  JG_CUDA(cudaMemcpyAsync(md->grid_t[p], md->grid_t[c], Gb, cudaMemcpyDeviceToDevice, st));
  JG_CUDA(cudaStreamSynchronize(st));
  return JGCM_OK;
}

// ------------------------------------------------------------------------------------------
// Member copies between models of one mesh and one parameter set (ensembles, member-major).
namespace {
// spectral [m][n][ne*L] member slices: dst member dm <- src member sm, L innermost levels each
template <typename V>
__global__ void k_spec_member_copy(V* dst, int dne, int dm, const V* src, int sne, int sm, size_t S, int L) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < S * L; q += (size_t)gridDim.x * blockDim.x) {
    const size_t r = q / L, k = q - r * L;
    dst[(r * dne + dm) * L + k] = src[(r * sne + sm) * L + k];
  }
}
}  // namespace

extern "C" int jgcm_model_members(jgcm_model* md, int* members) {
  JG_ARG(md && members, "NULL argument");
  *members = md->ne;
  return JGCM_OK;
}

extern "C" int jgcm_model_copy_member(jgcm_model* dst, int dst_member, jgcm_model* src, int src_member) {
  JG_ARG(dst && src, "NULL model");
  JG_ARG(dst->mesh == src->mesh, "members can only be copied between models of one mesh");
  JG_ARG(dst->P.kind == src->P.kind && dst->P.dt == src->P.dt, "members can only be copied between models of one kind and dt");
  JG_ARG(dst_member >= 0 && dst_member < dst->ne && src_member >= 0 && src_member < src->ne, "member out of range");
  JG_ARG(dst->nq == src->nq, "members can only be copied between models with the same number of tracers");
  if (dst->ne > 1 && dst != src)
    JG_ARG(dst->init_step == src->init_step && dst->sw_adv_from_n == src->sw_adv_from_n,
           "ensemble members must share the time-step state (init step) of the ensemble");
  jgcm_mesh* m = dst->mesh;
  cudaStream_t st = m->stream;
  const int nd = dst->nd;
  const size_t ts = tsize(m), G1 = grid_elems(m, 1), S = (size_t)(m->N + 1) * (m->ns + 1);
  auto grid = [&](void* d, const void* s_, int L) -> int {  // member slices are contiguous
    JG_CUDA(cudaMemcpyAsync((char*)d + (size_t)dst_member * L * G1 * ts, (const char*)s_ + (size_t)src_member * L * G1 * ts,
                            (size_t)L * G1 * ts, cudaMemcpyDeviceToDevice, st));
    return JGCM_OK;
  };
  auto spec = [&](void* d, const void* s_, int L) -> int {
    int nb = (int)std::min<size_t>((S * L + 255) / 256, 1024);
    if (is_fp64(m))
      k_spec_member_copy<double2><<<nb, 256, 0, st>>>((double2*)d, dst->ne, dst_member, (const double2*)s_, src->ne,
                                                      src_member, S, L);
    else
      k_spec_member_copy<float2><<<nb, 256, 0, st>>>((float2*)d, dst->ne, dst_member, (const float2*)s_, src->ne,
                                                     src_member, S, L);
    JG_CUDA(cudaGetLastError());
    return JGCM_OK;
  };
  for (int w = 0; w < 3; w++) {  // logical levels p, c, n
    const int ld = lvl(dst, w), ls = lvl(src, w);
    JG_TRY(spec(dst->spe_vor[ld], src->spe_vor[ls], nd));
    JG_TRY(spec(dst->spe_div[ld], src->spe_div[ls], nd));
    JG_TRY(spec(dst->spe_t[ld], src->spe_t[ls], nd));
    JG_TRY(spec(dst->spe_lnps[ld], src->spe_lnps[ls], 1));
    JG_TRY(grid(dst->grid_u[ld], src->grid_u[ls], nd));
    JG_TRY(grid(dst->grid_v[ld], src->grid_v[ls], nd));
    JG_TRY(grid(dst->grid_t[ld], src->grid_t[ls], nd));
    JG_TRY(grid(dst->grid_ps[ld], src->grid_ps[ls], 1));
    if (dst->nq) {
      JG_TRY(spec(dst->spe_q[ld], src->spe_q[ls], nd * dst->nq));
      JG_TRY(grid(dst->grid_q[ld], src->grid_q[ls], nd * dst->nq));
    }
  }
  JG_TRY(grid(dst->grid_vor, src->grid_vor, nd));
  JG_TRY(grid(dst->grid_div, src->grid_div, nd));
  JG_TRY(grid(dst->grid_t_eq, src->grid_t_eq, nd));
  JG_TRY(grid(dst->grid_lnps, src->grid_lnps, 1));
  JG_TRY(grid(dst->grid_geopots, src->grid_geopots, 1));
  JG_TRY(grid(dst->grid_h_eq, src->grid_h_eq, 1));
  dst->grad_ready = 0;
  if (dst->ne == 1) {  // a one-member model takes the source's time-step state
    dst->init_step = src->init_step;
    dst->sw_adv_from_n = src->sw_adv_from_n;
    dst->steps_done = src->steps_done;
  }
  JG_CUDA(cudaStreamSynchronize(st));
  return JGCM_OK;
}


// ------------------------------------------------------------------------------------------
// Ensembles of uneven truncations in one graph launch per time window: each member-batched model
// advances window / dt steady steps on its own branch of one captured CUDA graph (forked from and
// joined back into the ensemble's stream), so the truncations run concurrently and one launch
// advances them all.  A window graph is keyed by the models' time-level rotations at its start
// (which repeat with period 3), captured when first needed and replayed afterwards.
struct jgcm_ensemble {
  std::vector<jgcm_model*> models;
  std::vector<int> steps;  // steady steps per window of each model
  std::vector<cudaStream_t> side;
  cudaStream_t st;
  cudaEvent_t fork, t0, t1;
  std::vector<cudaEvent_t> join;
  std::vector<std::pair<std::vector<int>, cudaGraphExec_t>> graphs;  // (rotations at start, graph)
};

namespace {
// windows per graph launch when a run is long enough: independent members, so each truncation's
// branch runs its steps of all these windows back to back (a multiple of 3 steps for every member
// returns to the same rotation phase, and the same graph serves every launch)
constexpr int kEnsembleChunk = 24;

std::vector<int> ensemble_key(const jgcm_ensemble* en, int nwin) {  // rotations and tiles at the start
  std::vector<int> k{nwin};
  for (auto* md : en->models) {
    k.push_back(md->rot);
    k.push_back(md->mesh->tune_gen);
    k.push_back(md->hs_lanes);
  }
  return k;
}

int ensemble_capture(jgcm_ensemble* en, cudaGraphExec_t* out, int nwin) {
  struct Saved {
    int rot, init_step, sw_adv_from_n, steps_done, grad_ready;
  };
  std::vector<Saved> saved;
  for (auto* md : en->models)
    saved.push_back({md->rot, md->init_step, md->sw_adv_from_n, md->steps_done, md->grad_ready});
  cudaGraph_t g;
  JG_CUDA(cudaStreamBeginCapture(en->st, cudaStreamCaptureModeThreadLocal));
  int s = JGCM_OK;
  cudaError_t e = cudaEventRecord(en->fork, en->st);
  for (size_t i = 0; i < en->models.size() && s == JGCM_OK && e == cudaSuccess; i++) {
    e = cudaStreamWaitEvent(en->side[i], en->fork, 0);
    for (int k = 0; k < en->steps[i] * nwin && s == JGCM_OK && e == cudaSuccess; k++) {
      s = issue(en->models[i], en->side[i]);
      after_step(en->models[i]);
    }
    if (e == cudaSuccess) e = cudaEventRecord(en->join[i], en->side[i]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(en->st, en->join[i], 0);
  }
  cudaError_t e2 = cudaStreamEndCapture(en->st, &g);
  for (size_t i = 0; i < en->models.size(); i++) {  // the graph has not run yet
    en->models[i]->rot = saved[i].rot;
    en->models[i]->init_step = saved[i].init_step;
    en->models[i]->sw_adv_from_n = saved[i].sw_adv_from_n;
    en->models[i]->steps_done = saved[i].steps_done;
    en->models[i]->grad_ready = saved[i].grad_ready;
  }
  if (s != JGCM_OK || e != cudaSuccess || e2 != cudaSuccess) {
    if (e2 == cudaSuccess) cudaGraphDestroy(g);
    if (s != JGCM_OK) return s;
    JG_CUDA(e != cudaSuccess ? e : e2);
  }
  cudaError_t e3 = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  JG_CUDA(e3);
  return JGCM_OK;
}

int ensemble_graph(jgcm_ensemble* en, cudaGraphExec_t* out, int nwin) {
  const std::vector<int> key = ensemble_key(en, nwin);
  for (auto& kv : en->graphs)
    if (kv.first == key) {
      *out = kv.second;
      return JGCM_OK;
    }
  cudaGraphExec_t g = nullptr;
  JG_TRY(ensemble_capture(en, &g, nwin));
  en->graphs.push_back({key, g});
  *out = g;
  return JGCM_OK;
}

int ensemble_windows(jgcm_ensemble* en, int nwin) {
  for (auto* md : en->models)  // window graphs start from ready gradients
    if (md->P.kind == JGCM_HELD_SUAREZ && !md->grad_ready) {
      JG_TRY(is_fp64(md->mesh) ? issue_hs_grad<double>(md, lvl(md, 1), en->st)
                               : issue_hs_grad<float>(md, lvl(md, 1), en->st));
      md->grad_ready = 1;
    }
  cudaGraphExec_t g;
  JG_TRY(ensemble_graph(en, &g, nwin));
  JG_CUDA(cudaGraphLaunch(g, en->st));
  for (size_t i = 0; i < en->models.size(); i++)
    for (int k = 0; k < en->steps[i] * nwin; k++) after_step(en->models[i]);
  return JGCM_OK;
}

// nwindows windows: whole chunks when the count is a multiple of the chunk, single windows otherwise
int ensemble_run(jgcm_ensemble* en, int nwindows) {
  const int chunk = (nwindows % kEnsembleChunk == 0) ? kEnsembleChunk : 1;
  for (int w = 0; w < nwindows; w += chunk) JG_TRY(ensemble_windows(en, chunk));
  return JGCM_OK;
}

void ensemble_free(jgcm_ensemble* en) {
  if (!en) return;
  for (auto& kv : en->graphs)
    if (kv.second) cudaGraphExecDestroy(kv.second);
  for (auto s : en->side)
    if (s) cudaStreamDestroy(s);
  for (auto ev : en->join)
    if (ev) cudaEventDestroy(ev);
  if (en->fork) cudaEventDestroy(en->fork);
  if (en->t0) cudaEventDestroy(en->t0);
  if (en->t1) cudaEventDestroy(en->t1);
  if (en->st) cudaStreamDestroy(en->st);
  delete en;
}
}  // namespace

extern "C" int jgcm_ensemble_create(jgcm_model* const* models, int nmodels, int window_seconds,
                                    jgcm_ensemble** out) {
  JG_ARG(models && out && nmodels >= 1 && nmodels <= 64, "need 1..64 models");
  JG_ARG(window_seconds > 0, "window_seconds must be positive");
  *out = nullptr;
  for (int i = 0; i < nmodels; i++) {
    JG_ARG(models[i], "model %d is NULL", i);
    JG_ARG(window_seconds % models[i]->P.dt == 0, "window %d s is not a multiple of model %d's dt (%d s)",
           window_seconds, i, models[i]->P.dt);
    JG_ARG(!models[i]->init_step && !models[i]->sw_adv_from_n,
           "model %d is still in its first step: step every model once before grouping", i);
    for (int k = 0; k < i; k++) JG_ARG(models[k] != models[i], "model %d appears twice", i);
    JG_ARG(models[i]->mesh->device == models[0]->mesh->device, "all models must live on one device");
  }
  jgcm_ensemble* en = new jgcm_ensemble();
  auto fail = [&](cudaError_t e) -> int {
    set_error("ensemble: %s", cudaGetErrorString(e));
    ensemble_free(en);
    return JGCM_E_CUDA;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&en->st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&en->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreate(&en->t0);
  if (e == cudaSuccess) e = cudaEventCreate(&en->t1);
  if (e != cudaSuccess) return fail(e);
  for (int i = 0; i < nmodels; i++) {
    en->models.push_back(models[i]);
    en->steps.push_back(window_seconds / models[i]->P.dt);
    cudaStream_t s = nullptr;
    cudaEvent_t ev = nullptr;
    e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    en->side.push_back(s);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    en->join.push_back(ev);
    if (e != cudaSuccess) return fail(e);
  }
  // work already queued on the models' own streams comes first
  for (auto* md : en->models) {
    e = cudaStreamSynchronize(md->mesh->stream);
    if (e != cudaSuccess) return fail(e);
  }
  *out = en;
  return JGCM_OK;
}

extern "C" int jgcm_ensemble_step(jgcm_ensemble* en, int nwindows) {
  JG_ARG(en && nwindows >= 0, "bad arguments");
  for (auto* md : en->models) JG_CUDA(cudaStreamSynchronize(md->mesh->stream));  // work queued on a model alone
  JG_TRY(ensemble_run(en, nwindows));
  JG_CUDA(cudaStreamSynchronize(en->st));
  return JGCM_OK;
}

extern "C" int jgcm_ensemble_time(jgcm_ensemble* en, int nwindows, float* ms) {
  JG_ARG(en && ms && nwindows >= 1, "bad arguments");
  for (auto* md : en->models) JG_CUDA(cudaStreamSynchronize(md->mesh->stream));
  // capture the graphs the timed windows use before timing: the chunk graph (its key repeats), or the
  // single-window graph of every rotation phase (host bookkeeping advanced and restored; nothing runs)
  {
    const int nwin = (nwindows % kEnsembleChunk == 0) ? kEnsembleChunk : 1, count = nwin == 1 ? 3 : 1;
    struct Saved {
      int rot, init_step, sw_adv_from_n, steps_done, grad_ready;
      long diag_steps;
    };
    std::vector<Saved> saved;
    for (auto* md : en->models)
      saved.push_back({md->rot, md->init_step, md->sw_adv_from_n, md->steps_done, md->grad_ready, md->diag_steps});
    int st = JGCM_OK;
    for (int c = 0; c < count && st == JGCM_OK; c++) {
      bool ready = true;
      for (auto* md : en->models) ready = ready && !(md->P.kind == JGCM_HELD_SUAREZ && !md->grad_ready);
      if (!ready) break;  // the first window prepares the gradients; its graph is captured when it runs
      cudaGraphExec_t g;
      st = ensemble_graph(en, &g, nwin);
      for (size_t i = 0; i < en->models.size(); i++)
        for (int k = 0; k < en->steps[i] * nwin; k++) after_step(en->models[i]);
    }
    for (size_t i = 0; i < en->models.size(); i++) {
      jgcm_model* md = en->models[i];
      md->rot = saved[i].rot;
      md->init_step = saved[i].init_step;
      md->sw_adv_from_n = saved[i].sw_adv_from_n;
      md->steps_done = saved[i].steps_done;
      md->grad_ready = saved[i].grad_ready;
      md->diag_steps = saved[i].diag_steps;
    }
    JG_TRY(st);
  }
  JG_CUDA(cudaEventRecord(en->t0, en->st));
  JG_TRY(ensemble_run(en, nwindows));
  JG_CUDA(cudaEventRecord(en->t1, en->st));
  JG_CUDA(cudaEventSynchronize(en->t1));
  JG_CUDA(cudaEventElapsedTime(ms, en->t0, en->t1));
  return JGCM_OK;
}

extern "C" int jgcm_ensemble_destroy(jgcm_ensemble* en) {
  if (!en) return JGCM_OK;
  cudaStreamSynchronize(en->st);
  ensemble_free(en);
  return JGCM_OK;
}

// ------------------------------------------------------------------------------------------
// Tiles and their autotuner.  Knobs: [0] lanes per column of the Held-Suarez column kernel
// (model), [1] S2G columns, [2] G2S columns, [3] FFT columns per block of the SIMT transform
// kernels, [4] the Legendre engine of the tensor-core modes, [5] levels per block of the
// Held-Suarez analysis (mesh: shared by the models of the mesh).  0 keeps the default.
extern "C" int jgcm_model_get_tuning(jgcm_model* md, int* knobs, int n) {
  JG_ARG(md && knobs && n >= 4, "need 4 knobs");
  knobs[0] = md->hs_lanes;
  for (int i = 1; i < 4; i++) knobs[i] = md->mesh->tune[i];
  if (n >= 5) knobs[4] = md->mesh->simt_legendre;
  if (n >= 6) knobs[5] = md->mesh->hs_levels;
  return JGCM_OK;
}

extern "C" int jgcm_model_set_tuning(jgcm_model* md, const int* knobs, int n) {
  JG_ARG(md && knobs && n >= 4, "need 4 knobs");
  jgcm_mesh* m = md->mesh;
  const int lanes = knobs[0] > 0 ? knobs[0] : hs_lanes(m, md->ne, md->nd);
  JG_ARG(lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8, "lanes per column must be 1, 2, 4 or 8");
  for (int i = 1; i < 4; i++) JG_ARG(knobs[i] >= (i == 3 ? -1 : 0) && knobs[i] <= 256, "tile %d out of range", i);
  int t[4] = {0, knobs[1], knobs[2], knobs[3]};
  const int s2g = t[1] > 0 ? t[1] : (m->nh >= 256 ? 1 : 256 / m->nh);
  const int g2s = t[2] > 0 ? t[2] : (m->nh >= 64 ? 4 : m->nh >= 32 ? 8 : 16);
  const int fft = t[3] > 0 ? t[3] : (m->nlon >= 1024 ? 1 : 1024 / m->nlon);
  JG_ARG(g2s % 4 == 0 || t[2] == 0, "G2S columns per block must be a multiple of 4");
  JG_ARG(simt_smem_need(m, s2g, g2s, fft) <= kSmemBudget, "tiles need more than %zu bytes of shared memory",
         kSmemBudget);
  JG_CUDA(cudaStreamSynchronize(m->stream));
  if (lanes != md->hs_lanes) {
    md->hs_lanes = lanes;
    drop_graphs(md);
  }
  int simt = m->simt_legendre;
  if (n >= 5) {
    JG_ARG(knobs[4] == 0 || knobs[4] == 1, "Legendre engine knob must be 0 (tensor cores) or 1 (SIMT)");
    simt = m->tc.on ? knobs[4] : 0;  // meaningful for the tensor-core precision modes only
  }
  int hsl = m->hs_levels;
  if (n >= 6) {
    JG_ARG(knobs[5] >= -1 && knobs[5] <= 256, "analysis levels per block out of range");
    hsl = knobs[5];
  }
  bool changed = simt != m->simt_legendre || hsl != m->hs_levels;
  for (int i = 1; i < 4; i++) changed = changed || m->tune[i] != t[i];
  if (changed) {
    for (int i = 1; i < 4; i++) m->tune[i] = t[i];
    m->simt_legendre = simt;
    m->hs_levels = hsl;
    m->tune_gen++;
  }
  return JGCM_OK;
}

// Coordinate search over the knobs on a scratch copy of the model (its state is left untouched):
// each candidate is timed with CUDA events over `nsteps` captured steps (after one untimed step
// that captures the graphs); the fastest setting of each knob is kept before the next is tried.
extern "C" int jgcm_model_autotune(jgcm_model* md, int nsteps, int* knobs_out, int n, float* ms_out) {
  JG_ARG(md && nsteps >= 1, "bad arguments");
  JG_ARG(knobs_out == nullptr || n >= 4, "knobs_out holds %d ints, need at least 4", n);
  jgcm_mesh* m = md->mesh;
  jgcm_model* sc = nullptr;
  JG_TRY(jgcm_model_create_vert(m, &md->P, md->ne, md->vc.ak, md->vc.bk, &sc));
  struct Guard {
    jgcm_model* p;
    ~Guard() { jgcm_model_destroy(p); }
  } guard{sc};
  sc->init_step = md->init_step;  // the scratch ensemble takes the model's time-step state
  sc->sw_adv_from_n = md->sw_adv_from_n;
  for (int e = 0; e < md->ne; e++) JG_TRY(jgcm_model_copy_member(sc, e, md, e));
  if (sc->init_step || sc->sw_adv_from_n) JG_TRY(jgcm_model_step(sc, 1));
  int cur[6];
  JG_TRY(jgcm_model_get_tuning(md, cur, 6));
  auto timed = [&](const int* k, float* ms) -> int {
    JG_TRY(jgcm_model_set_tuning(sc, k, 6));
    JG_TRY(jgcm_model_step(sc, 3));  // captures the three rotation phases
    return jgcm_model_time_steps(sc, nsteps, ms);
  };
  float best = 0.f;
  JG_TRY(timed(cur, &best));
  const int d1 = m->nh >= 256 ? 1 : 256 / m->nh, d2 = m->nh >= 64 ? 4 : m->nh >= 32 ? 8 : 16,
            d3 = m->nlon >= 1024 ? 1 : 1024 / m->nlon;
  std::vector<std::vector<int>> cand = {
      {1, 2, 4, 8}, {std::max(1, d1 / 2), d1, 2 * d1, 4 * d1}, {4, 8, 16, 32}, {std::max(1, d3 / 2), d3, 2 * d3},
      {0, 1}, {}};
  if (md->P.kind != JGCM_HELD_SUAREZ) cand[0] = {cur[0]};
  if (!m->tc.on) cand[4] = {cur[4]};  // the Legendre engine: tensor cores or SIMT (tensor-core modes)
  // levels per block of the Held-Suarez analysis kernel: 0 (default) and 1 .. what a block holds
  if (md->P.kind == JGCM_HELD_SUAREZ)
    for (int v : {0, -1, 1, 2, 3, 4, 5, 6, 8, 10})
      if (v <= 256 / (m->N + 4)) cand[5].push_back(v);
  if (cand[5].empty()) cand[5] = {cur[5]};
  // the Legendre engine first: the SIMT tiles searched next only matter once the engine is known
  for (int knob : {4, 0, 1, 2, 3, 5})
    for (int v : cand[knob]) {
      int k[6] = {cur[0], cur[1], cur[2], cur[3], cur[4], cur[5]};
      k[knob] = v;
      if (knob == 1 && v == d1) k[1] = 0;
      if (knob == 2 && v == d2) k[2] = 0;
      if (knob == 3 && v == d3) k[3] = 0;
      if (k[knob] == cur[knob]) continue;
      const int s2g = k[1] ? k[1] : d1, g2s = k[2] ? k[2] : d2, fft = k[3] ? k[3] : d3;
      if (simt_smem_need(m, s2g, g2s, fft) > kSmemBudget) continue;
      if (knob == 0 && (md->nd + v - 1) / v < 2) continue;
      float ms = 0.f;
      if (timed(k, &ms) != JGCM_OK) continue;
      if (ms < best) {
        best = ms;
        for (int i = 0; i < 6; i++) cur[i] = k[i];
      }
    }
  JG_TRY(jgcm_model_set_tuning(md, cur, 6));
  if (knobs_out)
    for (int i = 0; i < std::min(n, 6); i++) knobs_out[i] = cur[i];
  if (ms_out) *ms_out = best;
  return JGCM_OK;
}


// ------------------------------------------------------------------------------------------
// One semi-implicit step on its own, and its adjoint (the differentiation pattern; no counterpart in
// the reference).  The step is Adjust_δlnps_δt_δdiv! + Implicit_Correction! (Semi_Implicit.jl:
// 360-513), Compute_Spectral_Damping! and Filtered_Leapfrog! (Time_Integrator.jl:58-101) for one
// model step: a linear map, per spectral mode (m,n), of the tendencies and the p and c time levels
// to the n level and the filtered c level.  The adjoint reverses it mode by mode with the transposed
// vertical operators, built once on the host in FP64 as matrices (Linear_Ps_T_δdiv!: d -> (δps,
// δT); Linear_Geopot_δt!: δT -> Φ) from the same column functions as the wave matrices, and W_n^T.
namespace {
struct AdjMats {  // vertical operators A, row-major (A[k][c] at k*nd + c); matT applies A^T
  double *Apt, *spt, *Ageo, *hk;  // FP64 (the FP64 path)
  float *Aptf, *sptf, *Ageof, *hkf;  // the same rounded to FP32 (the mixed path: no conversions per use)
};

// the operators of the state precision T within one allocation made by adj_mats
template <typename T>
struct AdjMatsT;
template <>
struct AdjMatsT<double> {
  static void get(const AdjMats& m, const double** Apt, const double** spt, const double** Ageo, const double** hk) {
    *Apt = m.Apt, *spt = m.spt, *Ageo = m.Ageo, *hk = m.hk;
  }
};
template <>
struct AdjMatsT<float> {
  static void get(const AdjMats& m, const float** Apt, const float** spt, const float** Ageo, const float** hk) {
    *Apt = m.Aptf, *spt = m.sptf, *Ageo = m.Ageof, *hk = m.hkf;
  }
};

AdjMats adj_mats_view(double* d, int nd) {  // the pointers of an adj_mats allocation
  AdjMats a;
  const size_t n2 = (size_t)nd * nd;
  a.Apt = d;
  a.Ageo = d + n2;
  a.spt = d + 2 * n2;
  a.hk = a.spt + nd;
  float* f = (float*)(d + 2 * n2 + 2 * nd);
  a.Aptf = f;
  a.Ageof = f + n2;
  a.sptf = f + 2 * n2;
  a.hkf = a.sptf + nd;
  return a;
}

int adj_mats(jgcm_model* md, AdjMats* out) {
  const int nd = md->nd;
  std::vector<double> Apt((size_t)nd * nd), spt(nd), Ageo((size_t)nd * nd), hk(nd), e(nd), dtt(nd), geo(nd);
  for (int c = 0; c < nd; c++) {
    std::fill(e.begin(), e.end(), 0.0);
    e[c] = 1.0;
    double dps = 0.0;
    lin_ps_t_col(md->vc, nd, md->P.kappa, e.data(), &dps, dtt.data());
    spt[c] = dps;
    // response of level k to a unit input at level c is A[k][c]; stored at [k][c] (row-major A), so
    // that lane k reading M[c*nd + k] over c walks column k of A, i.e. row k of A^T
    for (int k = 0; k < nd; k++) Apt[(size_t)k * nd + c] = dtt[k];
    lin_geo_col(md->vc, nd, md->P.rdgas, e.data(), geo.data());
    for (int k = 0; k < nd; k++) Ageo[(size_t)k * nd + c] = geo[k];
  }
  for (int k = 0; k < nd; k++) hk[k] = md->vc.h[k] * md->P.ps_ref;
  const size_t nall = 2 * (size_t)nd * nd + 2 * nd;
  std::vector<double> host(nall);
  std::copy(Apt.begin(), Apt.end(), host.begin());
  std::copy(Ageo.begin(), Ageo.end(), host.begin() + (size_t)nd * nd);
  std::copy(spt.begin(), spt.end(), host.begin() + 2 * (size_t)nd * nd);
  std::copy(hk.begin(), hk.end(), host.begin() + 2 * (size_t)nd * nd + nd);
  std::vector<float> hostf(nall);
  for (size_t i = 0; i < nall; i++) hostf[i] = (float)host[i];
  double* d = nullptr;
  JG_TRY(alloc((void**)&d, nall * 8 + nall * 4));
  *out = adj_mats_view(d, nd);
  JG_CUDA(cudaMemcpy(d, host.data(), nall * 8, cudaMemcpyHostToDevice));
  JG_CUDA(cudaMemcpy(out->Aptf, hostf.data(), nall * 4, cudaMemcpyHostToDevice));
  return JGCM_OK;
}

// cotangents of the step's outputs -> cotangents of its inputs; arrays MNK, nd levels (lnps: 1)
template <typename T>
struct AdjArgs {
  const V2<T>*vn_b, *vc_b, *dn_b, *dc_b, *tn_b, *tc_b, *ln_b, *lc_b;                 // outputs' cotangents
  V2<T>*dvor_b, *ddiv_b, *dt_b, *dl_b, *vp_b, *vcin_b, *dp_b, *dcin_b, *tp_b, *tcin_b, *lp_b, *lcin_b;  // inputs'
  const T *damping, *dfac;
  const double *eig64, *W;
  const T *Apt, *spt, *Ageo, *hk;  // vertical operators in the state precision
  const int2* pairs;
  int npairs, nd, ns, N, init_step, dt;
  double xi, ps_ref, robert;
  // the scalars rounded to T on the host (no FP64 division or conversion per thread) and the
  // Laplacian eigenvalues in T
  const T* eig_t;
  T xi_t, rpsr_t, xipsr_t, rob_t;
};

template <typename T>
void adj_consts(AdjArgs<T>& a, const T* eig_t) {
  a.eig_t = eig_t;
  a.xi_t = (T)a.xi;
  a.rpsr_t = (T)(1.0 / a.ps_ref);
  a.xipsr_t = (T)(a.xi / a.ps_ref);
  a.rob_t = (T)a.robert;
}

// y = M^T x for row-major M: y_k = sum_c M[c][k] x_c at the lane's level k; lanes >= nd return 0
template <typename R, typename E>
__device__ __forceinline__ R matT(const E* M, R x, int lane, int nd) {
  R y = 0;
  for (int c = 0; c < nd; c++) {
    R xc = __shfl_sync(FULL, x, c);
    if (lane < nd) y += (R)M[(size_t)c * nd + lane] * xc;
  }
  return y;
}

template <typename R>
__device__ __forceinline__ void lf_adj(int init, R Dt, R rob, R d, R f, R qnb, R qcb_out, R& dqb, R& qpb, R& qcb) {
  const R qnt = qnb + rob * qcb_out;  // q_n feeds the filtered q_c
  if (init) {  // dq' = (dq - qc d) f, qn = qc + Dt dq', qc' = (1 - r) qc + r qn
    const R dqp = Dt * qnt;
    dqb = f * dqp;
    qcb = ((R)1 - rob) * qcb_out + qnt - d * f * dqp;
    qpb = 0;
  } else {  // dq' = (dq - qp d) f, qc'' = (1 - 2r) qc + r qp, qn = qp + 2 Dt dq', qc' = qc'' + r qn
    const R dqp = (R)2 * Dt * qnt;
    dqb = f * dqp;
    qcb = ((R)1 - (R)2 * rob) * qcb_out;
    qpb = rob * qcb_out + qnt - d * f * dqp;
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_hs_implicit_adjoint(AdjArgs<T> a) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using R = T;
  const int lane = threadIdx.x & 31;
  const int pid = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (pid >= a.npairs) return;  // whole warp
  const int2 mn = a.pairs[pid];
  const int m = mn.x, n = mn.y, nd = a.nd;
  const bool act = lane < nd;
  const size_t row = (size_t)m * (a.ns + 1) + n, s = row * nd + (act ? lane : 0);
  auto ld = [&](const V2<T>* p, int comp) -> R { return act ? (R)(comp ? p[s].y : p[s].x) : (R)0; };
  const R rob = (R)a.rob_t, Dt = (R)a.dt, d = (R)a.damping[row], f = (R)a.dfac[row], xi = (R)a.xi_t;
  const R rpsr = (R)a.rpsr_t, xipsr = (R)a.xipsr_t, eig = (R)a.eig_t[row];
  for (int comp = 0; comp < 2; comp++) {  // real and imaginary parts are independent
    R dvb, vpb, vcb, ddb2, dpb, dcb, dtb2, tpb, tcb;
    lf_adj<R>(a.init_step, Dt, rob, d, f, ld(a.vn_b, comp), ld(a.vc_b, comp), dvb, vpb, vcb);
    lf_adj<R>(a.init_step, Dt, rob, d, f, ld(a.dn_b, comp), ld(a.dc_b, comp), ddb2, dpb, dcb);
    lf_adj<R>(a.init_step, Dt, rob, d, f, ld(a.tn_b, comp), ld(a.tc_b, comp), dtb2, tpb, tcb);
    R dlb2 = 0, lpb = 0, lcb = 0;
    {
      const R lnb = comp ? (R)a.ln_b[row].y : (R)a.ln_b[row].x, lcbo = comp ? (R)a.lc_b[row].y : (R)a.lc_b[row].x;
      lf_adj<R>(a.init_step, Dt, rob, (R)0, (R)1, lnb, lcbo, dlb2, lpb, lcb);
    }
    // dtt2 = dtt1 + xi dtmp_b, dl2 = dl1 + xi/ps_ref dps_b, (dps_b, dtmp_b) = LPT(ddiv2)
    R dtt1b = dtb2, dl1b = dlb2;
    const R dtmpb = xi * dtb2, dpsb = xipsr * dlb2;
    R ddiv2b = ddb2 + matT<R>(a.Apt, dtmpb, lane, nd) + (act ? (R)a.spt[lane] * dpsb : (R)0);
    // ddiv2 = W_n ddiv1 (n <= N)
    R ddiv1b = ddiv2b;
    if (n <= a.N) {
      const double* W = a.W + (size_t)n * nd * nd;  // W[k][c] at c*nd + k: W^T[k][c] = W[c][k] at k*nd + c
      R y = 0;
      for (int c = 0; c < nd; c++) {
        R xc = __shfl_sync(FULL, ddiv2b, c);
        if (act) y += (R)W[(size_t)lane * nd + c] * xc;
      }
      ddiv1b = act ? y : (R)0;
    }
    // ddiv1 = ddiv - eig (A_geo t2 + hk l2)
    const R gb = -eig * ddiv1b;
    const R t2b = matT<R>(a.Ageo, gb, lane, nd);
    R hdot = act ? (R)a.hk[lane] * ddiv1b : (R)0;
    for (int o = 16; o > 0; o >>= 1) hdot += __shfl_xor_sync(FULL, hdot, o);
    const R l2b = -eig * hdot;
    // t2 = tp - tc + xi dtt1, l2 = lp - lc + xi dl1
    tpb += t2b;
    tcb -= t2b;
    dtt1b += xi * t2b;
    lpb += l2b;
    lcb -= l2b;
    dl1b += xi * l2b;
    // dtt1 = dtt + dtmp_a, dl1 = dl + dps_a / ps_ref, (dps_a, dtmp_a) = LPT(div_p - div_c)
    const R qb = matT<R>(a.Apt, dtt1b, lane, nd) + (act ? (R)a.spt[lane] * (rpsr * dl1b) : (R)0);
    dpb += qb;
    dcb -= qb;
    auto st = [&](V2<T>* p, R v) {
      if (act) {
        if (comp) p[s].y = (T)v;
        else p[s].x = (T)v;
      }
    };
    st(a.dvor_b, dvb);
    st(a.ddiv_b, ddiv1b);
    st(a.dt_b, dtt1b);
    st(a.vp_b, vpb);
    st(a.vcin_b, vcb);
    st(a.dp_b, dpb);
    st(a.dcin_b, dcb);
    st(a.tp_b, tpb);
    st(a.tcin_b, tcb);
    if (lane == 0) {
      if (comp) {
        a.dl_b[row].y = (T)dl1b;
        a.lp_b[row].y = (T)lpb;
        a.lcin_b[row].y = (T)lcb;
      } else {
        a.dl_b[row].x = (T)dl1b;
        a.lp_b[row].x = (T)lpb;
        a.lcin_b[row].x = (T)lcb;
      }
    }
  }
}

// device buffers for the host-pointer entry points: 20 spectral fields (nd levels, lnps 1 level)
struct SIBuffers {
  void* f[20];
  void* base;
};
int si_alloc(jgcm_model* md, SIBuffers* b) {
  jgcm_mesh* m = md->mesh;
  const size_t ts = tsize(m), S = spec_elems(m, md->nd) * 2 * ts, S1 = spec_elems(m, 1) * 2 * ts;
  JG_TRY(alloc(&b->base, 20 * S));
  for (int i = 0; i < 20; i++) b->f[i] = (char*)b->base + (size_t)i * S;
  (void)S1;
  return JGCM_OK;
}
// level count of field i in the input (12) / output (8) orders: lnps slots have one level
int si_levels_in(const jgcm_model* md, int i) { return (i == 3 || i == 10 || i == 11) ? 1 : md->nd; }
int si_levels_out(const jgcm_model* md, int i) { return (i == 6 || i == 7) ? 1 : md->nd; }

template <typename T>
ImplArgs<T> si_args(jgcm_model* md, void* const* in, void* const* out) {
  using V = V2<T>;
  jgcm_mesh* m = md->mesh;
  ImplArgs<T> ia;
  memset(&ia, 0, sizeof(ia));
  ia.dvor = (const V*)in[0];
  ia.ddiv = (const V*)in[1];
  ia.dtend = (const V*)in[2];
  ia.dlnps = (const V*)in[3];
  ia.vor_p = (V*)in[4];
  ia.vor_c = (V*)out[1];  // c level: read from the copy in the output slot, filtered in place
  ia.vor_n = (V*)out[0];
  ia.div_p = (V*)in[6];
  ia.div_c = (V*)out[3];
  ia.div_n = (V*)out[2];
  ia.t_p = (V*)in[8];
  ia.t_c = (V*)out[5];
  ia.t_n = (V*)out[4];
  ia.lnps_p = (V*)in[10];
  ia.lnps_c = (V*)out[7];
  ia.lnps_n = (V*)out[6];
  ia.eig64 = m->t64.eig;
  ia.damping = (const T*)md->damping;
  ia.dfac = (const T*)md->dfac[md->init_step ? 0 : 1];
  ia.W = md->d_W + (md->init_step ? 0 : (size_t)(m->N + 1) * md->nd * md->nd);
  ia.pairs = md->d_pairs;
  ia.npairs = md->npairs;
  ia.nd = md->nd;
  ia.L = md->nd;
  ia.ne = 1;
  ia.ns = m->ns;
  ia.N = m->N;
  ia.init_step = md->init_step;
  ia.dt = md->P.dt;
  ia.xi = md->init_step ? md->P.dt * md->P.implicit_coef : (2 * md->P.dt) * md->P.implicit_coef;
  ia.ps_ref = md->P.ps_ref;
  ia.kappa = md->P.kappa;
  ia.rdgas = md->P.rdgas;
  ia.robert = md->P.robert_coef;
  impl_consts<T>(ia, tables<T>(md->mesh).eig);
  return ia;
}
}  // namespace

namespace jgcm {
int dev_alloc(void** p, size_t bytes) { return alloc(p, bytes); }

int model_step_async(jgcm_model* md) { return model_step(md); }

int hs_grad(jgcm_model* md, int lev, cudaStream_t st) {
  return is_fp64(md->mesh) ? issue_hs_grad<double>(md, lev, st) : issue_hs_grad<float>(md, lev, st);
}

int si_adjoint_mats(jgcm_model* md, double** mats) {
  AdjMats am;
  JG_TRY(adj_mats(md, &am));
  *mats = am.Apt;  // one allocation: Apt, Ageo, spt, hk
  return JGCM_OK;
}

int si_adjoint_launch(jgcm_model* md, const void* const* obar, void* const* ibar, const double* mats, int init,
                      cudaStream_t st) {
  jgcm_mesh* m = md->mesh;
  const int nd = md->nd;
  auto launch = [&](auto tag) -> cudaError_t {
    using T = decltype(tag);
    using V = V2<T>;
    AdjArgs<T> a;
    memset(&a, 0, sizeof(a));
    a.vn_b = (const V*)obar[0]; a.vc_b = (const V*)obar[1]; a.dn_b = (const V*)obar[2]; a.dc_b = (const V*)obar[3];
    a.tn_b = (const V*)obar[4]; a.tc_b = (const V*)obar[5]; a.ln_b = (const V*)obar[6]; a.lc_b = (const V*)obar[7];
    a.dvor_b = (V*)ibar[0]; a.ddiv_b = (V*)ibar[1]; a.dt_b = (V*)ibar[2]; a.dl_b = (V*)ibar[3];
    a.vp_b = (V*)ibar[4]; a.vcin_b = (V*)ibar[5]; a.dp_b = (V*)ibar[6]; a.dcin_b = (V*)ibar[7];
    a.tp_b = (V*)ibar[8]; a.tcin_b = (V*)ibar[9]; a.lp_b = (V*)ibar[10]; a.lcin_b = (V*)ibar[11];
    a.damping = (const T*)md->damping;
    a.dfac = (const T*)md->dfac[init ? 0 : 1];
    a.eig64 = m->t64.eig;
    a.W = md->d_W + (init ? 0 : (size_t)(m->N + 1) * nd * nd);
    AdjMatsT<T>::get(adj_mats_view(const_cast<double*>(mats), nd), &a.Apt, &a.spt, &a.Ageo, &a.hk);
    a.pairs = md->d_pairs;
    a.npairs = md->npairs;
    a.nd = nd;
    a.ns = m->ns;
    a.N = m->N;
    a.init_step = init;
    a.dt = md->P.dt;
    a.xi = init ? md->P.dt * md->P.implicit_coef : (2 * md->P.dt) * md->P.implicit_coef;
    a.ps_ref = md->P.ps_ref;
    a.robert = md->P.robert_coef;
    adj_consts<T>(a, tables<T>(m).eig);
    return launch_pdl(k_hs_implicit_adjoint<T>, dim3((md->npairs + 7) / 8), dim3(256), 0, st, a);
  };
  JG_CUDA(is_fp64(m) ? launch(double()) : launch(float()));
  mark(st);
  return JGCM_OK;
}
}  // namespace jgcm

extern "C" int jgcm_model_semi_implicit_step(jgcm_model* md, const double* const* in, double* const* out) {
  JG_ARG(md && in && out, "NULL argument");
  JG_ARG(md->P.kind == JGCM_HELD_SUAREZ, "the semi-implicit step exists for Held-Suarez only");
  JG_ARG(md->ne == 1, "one-member models only");
  for (int i = 0; i < 12; i++) JG_ARG(in[i], "input %d is NULL", i);
  for (int i = 0; i < 8; i++) JG_ARG(out[i], "output %d is NULL", i);
  jgcm_mesh* m = md->mesh;
  cudaStream_t st = m->stream;
  SIBuffers b;
  JG_TRY(si_alloc(md, &b));
  struct Free {
    void* p;
    ~Free() { cudaFree(p); }
  } fr{b.base};
  void* din[12];
  void* dout[8];
  for (int i = 0; i < 12; i++) din[i] = b.f[i];
  for (int i = 0; i < 8; i++) dout[i] = b.f[12 + i];
  for (int i = 0; i < 12; i++) {
    const size_t nn = 2 * spec_elems(m, si_levels_in(md, i));
    JG_CUDA(cudaMemcpyAsync(m->d_stage, in[i], nn * 8, cudaMemcpyHostToDevice, st));
    JG_TRY(spec_host_to_dev(m, m->d_stage, din[i], si_levels_in(md, i), st));
  }
  const size_t ts = tsize(m);
  JG_CUDA(cudaMemcpyAsync(dout[1], din[5], spec_elems(m, md->nd) * 2 * ts, cudaMemcpyDeviceToDevice, st));
  JG_CUDA(cudaMemcpyAsync(dout[3], din[7], spec_elems(m, md->nd) * 2 * ts, cudaMemcpyDeviceToDevice, st));
  JG_CUDA(cudaMemcpyAsync(dout[5], din[9], spec_elems(m, md->nd) * 2 * ts, cudaMemcpyDeviceToDevice, st));
  JG_CUDA(cudaMemcpyAsync(dout[7], din[11], spec_elems(m, 1) * 2 * ts, cudaMemcpyDeviceToDevice, st));
  if (is_fp64(m))
    k_hs_implicit<double, double><<<(md->npairs + 7) / 8, 256, 0, st>>>(si_args<double>(md, din, dout), md->d_vc);
  else
    k_hs_implicit<float, float><<<(md->npairs + 7) / 8, 256, 0, st>>>(si_args<float>(md, din, dout), md->d_vc);
  JG_CUDA(cudaGetLastError());
  for (int i = 0; i < 8; i++) {
    const size_t nn = 2 * spec_elems(m, si_levels_out(md, i));
    JG_TRY(spec_dev_to_host(m, dout[i], m->d_stage, si_levels_out(md, i), st));
    JG_CUDA(cudaMemcpyAsync(out[i], m->d_stage, nn * 8, cudaMemcpyDeviceToHost, st));
    JG_CUDA(cudaStreamSynchronize(st));
  }
  return JGCM_OK;
}

extern "C" int jgcm_model_semi_implicit_step_adjoint(jgcm_model* md, const double* const* out_bar,
                                                     double* const* in_bar) {
  JG_ARG(md && out_bar && in_bar, "NULL argument");
  JG_ARG(md->P.kind == JGCM_HELD_SUAREZ, "the semi-implicit step exists for Held-Suarez only");
  JG_ARG(md->ne == 1, "one-member models only");
  for (int i = 0; i < 8; i++) JG_ARG(out_bar[i], "output cotangent %d is NULL", i);
  for (int i = 0; i < 12; i++) JG_ARG(in_bar[i], "input cotangent %d is NULL", i);
  jgcm_mesh* m = md->mesh;
  cudaStream_t st = m->stream;
  SIBuffers b;
  JG_TRY(si_alloc(md, &b));
  AdjMats am;
  JG_TRY(adj_mats(md, &am));
  struct Free {
    void *p, *q;
    ~Free() {
      cudaFree(p);
      cudaFree(q);
    }
  } fr{b.base, am.Apt};
  void* dob[8];
  void* dib[12];
  for (int i = 0; i < 8; i++) dob[i] = b.f[i];
  for (int i = 0; i < 12; i++) dib[i] = b.f[8 + i];
  for (int i = 0; i < 8; i++) {
    const size_t nn = 2 * spec_elems(m, si_levels_out(md, i));
    JG_CUDA(cudaMemcpyAsync(m->d_stage, out_bar[i], nn * 8, cudaMemcpyHostToDevice, st));
    JG_TRY(spec_host_to_dev(m, m->d_stage, dob[i], si_levels_out(md, i), st));
  }
  auto launch = [&](auto tag) {
    using T = decltype(tag);
    using V = V2<T>;
    AdjArgs<T> a;
    memset(&a, 0, sizeof(a));
    a.vn_b = (const V*)dob[0]; a.vc_b = (const V*)dob[1]; a.dn_b = (const V*)dob[2]; a.dc_b = (const V*)dob[3];
    a.tn_b = (const V*)dob[4]; a.tc_b = (const V*)dob[5]; a.ln_b = (const V*)dob[6]; a.lc_b = (const V*)dob[7];
    a.dvor_b = (V*)dib[0]; a.ddiv_b = (V*)dib[1]; a.dt_b = (V*)dib[2]; a.dl_b = (V*)dib[3];
    a.vp_b = (V*)dib[4]; a.vcin_b = (V*)dib[5]; a.dp_b = (V*)dib[6]; a.dcin_b = (V*)dib[7];
    a.tp_b = (V*)dib[8]; a.tcin_b = (V*)dib[9]; a.lp_b = (V*)dib[10]; a.lcin_b = (V*)dib[11];
    a.damping = (const T*)md->damping;
    a.dfac = (const T*)md->dfac[md->init_step ? 0 : 1];
    a.eig64 = m->t64.eig;
    a.W = md->d_W + (md->init_step ? 0 : (size_t)(m->N + 1) * md->nd * md->nd);
    AdjMatsT<T>::get(am, &a.Apt, &a.spt, &a.Ageo, &a.hk);
    a.pairs = md->d_pairs;
    a.npairs = md->npairs;
    a.nd = md->nd;
    a.ns = m->ns;
    a.N = m->N;
    a.init_step = md->init_step;
    a.dt = md->P.dt;
    a.xi = md->init_step ? md->P.dt * md->P.implicit_coef : (2 * md->P.dt) * md->P.implicit_coef;
    a.ps_ref = md->P.ps_ref;
    a.robert = md->P.robert_coef;
    adj_consts<T>(a, tables<T>(m).eig);
    k_hs_implicit_adjoint<T><<<(md->npairs + 7) / 8, 256, 0, st>>>(a);
  };
  if (is_fp64(m)) launch(double());
  else launch(float());
  JG_CUDA(cudaGetLastError());
  for (int i = 0; i < 12; i++) {
    const size_t nn = 2 * spec_elems(m, si_levels_in(md, i));
    JG_TRY(spec_dev_to_host(m, dib[i], m->d_stage, si_levels_in(md, i), st));
    JG_CUDA(cudaMemcpyAsync(in_bar[i], m->d_stage, nn * 8, cudaMemcpyDeviceToHost, st));
    JG_CUDA(cudaStreamSynchronize(st));
  }
  return JGCM_OK;
}

// ------------------------------------------------------------------------------------------
// On-device diagnostics (the reductions of Output_Manager.jl:81-145; its file output and plots stay
// with the host).  Held-Suarez only.
extern "C" int jgcm_model_diagnostics(jgcm_model* md, int on) {
  JG_ARG(md, "NULL model");
  JG_ARG(md->P.kind == JGCM_HELD_SUAREZ, "diagnostics are kept for Held-Suarez models");
  jgcm_mesh* m = md->mesh;
  const size_t n = (size_t)4 * md->ne * md->nd * m->nlat + grid_elems(m, md->ne);
  JG_CUDA(cudaStreamSynchronize(m->stream));
  if (on) {
    if (!md->diag) JG_TRY(alloc((void**)&md->diag, n * 8));
    JG_CUDA(cudaMemset(md->diag, 0, n * 8));
    md->diag_steps = 0;
  }
  if ((on != 0) != (md->diag_on != 0)) drop_graphs(md);  // the step graphs gain / lose the reduction
  md->diag_on = on != 0;
  return JGCM_OK;
}

// Means over the steps summed since jgcm_model_diagnostics(model, 1): "t_zonal_mean",
// "t_eq_zonal_mean", "u_zonal_mean", "v_zonal_mean" ([nθ, nd, members], column-major) and
// "ps_mean" ([nλ, nθ, members]); `steps` returns the number of steps summed.
extern "C" int jgcm_model_read_diagnostics(jgcm_model* md, const char* name, double* out, long cap, long* count,
                                           long* steps) {
  JG_ARG(md && name, "NULL argument");
  JG_ARG(md->diag, "diagnostics were never started");
  jgcm_mesh* m = md->mesh;
  const std::string nm(name);
  const char* names[4] = {"t_zonal_mean", "t_eq_zonal_mean", "u_zonal_mean", "v_zonal_mean"};
  int f = -1;
  for (int i = 0; i < 4; i++)
    if (nm == names[i]) f = i;
  JG_ARG(f >= 0 || nm == "ps_mean", "unknown diagnostic '%s'", name);
  const size_t nz = (size_t)md->ne * md->nd * m->nlat;
  const size_t n = f >= 0 ? nz : grid_elems(m, md->ne);
  if (count) *count = (long)n;
  if (steps) *steps = md->diag_steps;
  if (!out) return JGCM_OK;
  JG_ARG(cap >= (long)n, "buffer too small");
  JG_CUDA(cudaStreamSynchronize(m->stream));
  const double* src = md->diag + (f >= 0 ? (size_t)f * nz : 4 * nz);
  JG_CUDA(cudaMemcpy(out, src, n * 8, cudaMemcpyDeviceToHost));  // [e][k][j] / [e][j][i]: Julia order
  const double sc = md->diag_steps > 0 ? 1.0 / (double)md->diag_steps : 0.0;
  for (size_t q = 0; q < n; q++) out[q] *= sc;
  return JGCM_OK;
}

