// transform_ops.cuh -- per-element pieces shared by the SIMT and the tensor-core Legendre
// kernels: the spectral prologues of the synthesis (the inputs built from neighbouring total
// wavenumbers) and the epilogues of the analysis (plain store, alpha operator, Laplacian of the
// energy, fused damping + leapfrog + Robert-Asselin filter, shallow-water implicit correction).
#pragma once
#include "jgcm_internal.cuh"

namespace jgcm {

template <typename T>
using V2 = typename C2<T>::t;

// Ampere-style asynchronous global -> shared copy of 16 bytes (both addresses 16-byte aligned):
// staged tables need no registers and every copy is in flight at once
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(sdst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <typename G>
__device__ __forceinline__ const G& group_of(const G* g, int ng, int c, int* k) {
  int i = 0;
  for (; i < ng - 1; i++)
    if (c < g[i].col0 + g[i].L) break;
  *k = c - g[i].col0;
  return g[i];
}

// Fused spectral time stepping used by the G2S epilogues (Time_Integrator.jl:58-101).
template <typename T>
__device__ __forceinline__ void damp_leapfrog(const StepParams& sp, T d, T& dq, T qp, T& qc, T& qn) {
  const T r = pick<T>(sp.robert, sp.robertf);
  const int Dt = sp.dt;
  if (sp.init_step) {
    dq = (dq - qc * d) / ((T)1.0 + (T)Dt * d);
    qn = qc + (T)Dt * dq;
    qc = qc + r * ((T)-1.0 * qc + qn);
  } else {
    dq = (dq - qp * d) / ((T)1.0 + (T)(2 * Dt) * d);
    qc = qc + r * (qp - (T)2 * qc);
    qn = qp + (T)(2 * Dt) * dq;
    qc = qc + r * qn;
  }
}

template <typename T>
__device__ __forceinline__ void leapfrog_c(const StepParams& sp, T d, V2<T>& dq, V2<T> qp, V2<T>& qc, V2<T>& qn,
                                           bool damp) {
  if (!damp) d = 0;
  damp_leapfrog<T>(sp, d, dq.x, qp.x, qc.x, qn.x);
  damp_leapfrog<T>(sp, d, dq.y, qp.y, qc.y, qn.y);
}


// Input of the synthesis for total wavenumber n (>= m) of column k of group g: the field itself,
// cos(lat) x its gradient (Compute_Gradient_Cos!, Spectral_Spherical_Mesh.jl:655-692) or ucos / vcos
// from vorticity and divergence (Compute_Ucos_Vcos_From_Vor_Div!, :517-580; these fill row N+1).
template <typename T>
__device__ __forceinline__ V2<T> s2g_input(const S2GGroup& g, const Tables<T>& tb, int m, int n, int ns, size_t mrow,
                                           int k) {
  using V = V2<T>;
  const int L = g.L;
  const V* a = (const V*)g.a;
  V x;
  x.x = 0;
  x.y = 0;
  switch (g.op) {
    case S2G_PLAIN:
      x = a[(mrow + n) * L + k];
      if (m == 0 && n == 0) x.x = x.x - pick<T>(g.shift, g.shiftf);
      break;
    case S2G_ANOM:
      x = a[(mrow + n) * L + k];
      if (m == 0 && n == 0) x.x = 0;
      break;
    case S2G_ADJ_G2S:  // the synthesis weights every m >= 1 twice; the analysis never sees row N+1
      if (n < ns) {
        x = a[(mrow + n) * L + k];
        if (m > 0) {
          x.x = x.x * (T)0.5;
          x.y = x.y * (T)0.5;
        }
      }
      break;
    case S2G_DLAM: {  // coef_dlam .* (i h)
      T cf = tb.dlam[mrow + n];
      V h = a[(mrow + n) * L + k];
      x.x = cf * (-h.y);
      x.y = cf * h.x;
    } break;
    case S2G_DTH: {  // coef_dthp h_{n+1} + coef_dthm h_{n-1}
      if (n <= ns - 1) {
        T cp = tb.dthp[mrow + n];
        V h = a[(mrow + n + 1) * L + k];
        x.x = cp * h.x;
        x.y = cp * h.y;
      }
      if (n - 1 >= m) {
        T cm = tb.dthm[mrow + n];
        V h = a[(mrow + n - 1) * L + k];
        x.x = x.x + cm * h.x;
        x.y = x.y + cm * h.y;
      }
    } break;
    case S2G_UCOS:
    case S2G_VCOS: {
      // ucos = uvc (i div) - uvm vor_{n-1} - uvp vor_{n+1}
      // vcos = uvc (i vor) + uvm div_{n-1} + uvp div_{n+1}
      const V* vor = a;
      const V* dv = (const V*)g.b;
      const bool u = g.op == S2G_UCOS;
      const V* ic = u ? dv : vor;  // term multiplied by i*uvc
      const V* nb = u ? vor : dv;  // neighbour terms
      T sg = u ? (T)-1 : (T)1;
      T cc = tb.uvc[mrow + n];
      V z = ic[(mrow + n) * L + k];
      x.x = cc * (-z.y);
      x.y = cc * z.x;
      if (n - 1 >= m) {
        T cm = tb.uvm[mrow + n];
        V h = nb[(mrow + n - 1) * L + k];
        x.x = x.x + sg * (cm * h.x);
        x.y = x.y + sg * (cm * h.y);
      }
      if (n + 1 <= ns) {
        T cp = tb.uvp[mrow + n];
        V h = nb[(mrow + n + 1) * L + k];
        x.x = x.x + sg * (cp * h.x);
        x.y = x.y + sg * (cp * h.y);
      }
    } break;
  }
  return x;
}

// Analysis epilogue for output (m, n) of column k of group g (sidx = its MNK index) from the
// contraction results r0..r3 of the group's slots.
template <typename T>
__device__ __forceinline__ void g2s_store(const G2SPlan& plan, const SpecOutGroup& g, const Tables<T>& tb, size_t mrow,
                                          int n, size_t sidx, V2<T> r0, V2<T> r1, V2<T> r2, V2<T> r3) {
  using V = V2<T>;
  const T eig = tb.eig[mrow + n];
  switch (g.op) {
    case G2S_PLAIN:
    case G2S_ADJ_S2G:
      ((V*)g.dst)[sidx] = r0;
      break;
    case G2S_VOR:
      ((V*)g.dst)[sidx] = r0;
      break;
    case G2S_DIV: {
      V v = r0;
      if (g.colE >= 0) {  // - laplacian(G2S(E) + extra)
        V e = r2;
        if (g.extra) {
          V x = ((const V*)g.extra)[sidx];
          e.x = e.x + x.x;
          e.y = e.y + x.y;
        }
        v.x = v.x - eig * e.x;
        v.y = v.y - eig * e.y;
      }
      ((V*)g.dst)[sidx] = v;
    } break;
    case G2S_BARO: {  // Barotropic_Dynamics.jl:31-36: vorticity tendency, damping, leapfrog
      V dq = r0;
      V* qc = (V*)g.qc[0];
      const V* qp = (const V*)g.qp[0];
      V c0 = qc[sidx], p0 = qp[sidx], n0;
      T d = ((const T*)plan.sp.damping)[mrow + n];
      leapfrog_c<T>(plan.sp, d, dq, p0, c0, n0, true);
      qc[sidx] = c0;
      ((V*)g.dst)[sidx] = n0;
    } break;
    case G2S_SW: {  // Shallow_Water_Dynamics.jl:133-165
      // slots: 0 = du cos, 1 = dv cos, 2 = kinetic energy, 3 = dh
      V dvor = r0;
      V ddiv = r1;
      V kin = r2;
      V dh = r3;
      const V* hc_p = (const V*)g.qc[2];
      V hc = hc_p[sidx], hp = ((const V*)g.qp[2])[sidx];
      V dc = ((const V*)g.qc[1])[sidx], dp = ((const V*)g.qp[1])[sidx];
      // spe_energy = (kin + h_c) * eig ; ddiv -= spe_energy
      ddiv.x = ddiv.x - eig * (kin.x + hc.x);
      ddiv.y = ddiv.y - eig * (kin.y + hc.y);
      // Implicit_Correction! (SW) :25-54
      const T h0 = pick<T>(plan.sp.h0, plan.sp.h0f);
      const T Dt = plan.sp.init_step ? (T)plan.sp.dt : (T)(2 * plan.sp.dt);
      ddiv.x = ddiv.x + eig * (hc.x - hp.x);
      ddiv.y = ddiv.y + eig * (hc.y - hp.y);
      dh.x = dh.x + h0 * (dc.x - dp.x);
      dh.y = dh.y + h0 * (dc.y - dp.y);
      const T mu = pick<T>(plan.sp.implicit_coef, plan.sp.implicit_coeff) * Dt, mu2 = mu * mu;
      const T den = (T)1.0 - mu2 * eig * h0;
      ddiv.x = (ddiv.x - mu * eig * dh.x) / den;
      ddiv.y = (ddiv.y - mu * eig * dh.y) / den;
      dh.x = dh.x - mu * h0 * ddiv.x;
      dh.y = dh.y - mu * h0 * ddiv.y;
      const T d = ((const T*)plan.sp.damping)[mrow + n];
      V vc = ((V*)g.qc[0])[sidx], vp = ((const V*)g.qp[0])[sidx], vn, dn, hn;
      leapfrog_c<T>(plan.sp, d, dvor, vp, vc, vn, true);
      leapfrog_c<T>(plan.sp, d, ddiv, dp, dc, dn, true);
      leapfrog_c<T>(plan.sp, d, dh, hp, hc, hn, true);
      ((V*)g.qc[0])[sidx] = vc;
      ((V*)g.qc[1])[sidx] = dc;
      ((V*)g.qc[2])[sidx] = hc;
      ((V*)g.dst)[sidx] = vn;
      ((V*)g.dst2)[sidx] = dn;
      ((V*)g.dst3)[sidx] = hn;
    } break;
  }
}

}  // namespace jgcm
