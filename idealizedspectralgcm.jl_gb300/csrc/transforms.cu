// transforms.cu -- spectral transforms of the JGCM dynamical core on sm_103a.
//
// spectral -> grid (Trans_Spherical_To_Grid!, Spectral_Spherical_Mesh.jl:143-217) runs as
//   k_s2g_legendre : per zonal wavenumber m, the even/odd-split Legendre synthesis
//                    F[m][j] = sum_n P_n^m(mu_j) s_n^m over n = m..N+1 (the reference's extra
//                    row N+1 included), a dense (nlat/2 x K) x (K x C) contraction per m,
//                    mirrored to the northern hemisphere by parity;
//   k_ifft         : inverse real zonal FFT of every (latitude, column) row as a half-length
//                    complex FFT, radix-2 in shared memory, fused epilogue (÷cos, exp, ×ps).
// grid -> spectral (Trans_Grid_To_Spherical!, :221-293; Vor_Div_From_Grid_UV!, :349-459) runs as
//   k_fft          : forward real zonal FFT (fft/nlon) with fused prologue (×cos, vorticity
//                    fluxes, kinetic energy, shallow-water height tendency);
//   k_g2s_legendre : per m, Gaussian quadrature over the hemisphere pairs, for plain analysis
//                    (row N+1 zeroed) and the alpha operator (vor/div from u cos, v cos), with
//                    fused epilogues (Laplacian of the energy, spectral damping, the leapfrog with
//                    Robert-Asselin filter and the shallow-water semi-implicit correction).
// Spectral prologues build the inputs of the synthesis on the fly from neighbouring total
// wavenumbers (gradient, Compute_Gradient_Cos! :655-692; ucos/vcos, :517-580).
#include <cstdlib>
#include <algorithm>
#include <cmath>
#include <mutex>
#include <type_traits>

#include "jgcm_internal.cuh"
#include "transform_ops.cuh"

namespace jgcm {

// programmatic dependent launch of the step kernels (JGCM_PDL=0 turns it off)
int g_pdl = [] {
  const char* e = std::getenv("JGCM_PDL");
  return (e && e[0] == '0') ? 0 : 1;
}();

__host__ __device__ __forceinline__ size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }
__device__ __forceinline__ int brev(int x, int logn) { return (int)(__brev((unsigned)x) >> (32 - logn)); }


// ------------------------------------------------------------------------------------------
// Complex radix-2 DIT stages over `nrow` rows of length h = nlon/2 held as (re, im) in shared
// memory (row stride h), input in bit-reversed order, output in natural order.  tw holds
// e^{2 pi i t / nlon} for t < nlon/2 (cos, sin interleaved).  SIGN = -1 forward, +1 backward.
template <typename T, int SIGN>
__device__ __forceinline__ void fft_stages(T* re, T* im, const T* tw, int nrow, int h, int logh) {
  const int hh = h >> 1;
  for (int s = 1; s <= logh; s++) {
    const int half = 1 << (s - 1);
    const int tshift = logh + 1 - s;  // e^{2 pi i k / 2^s} = tw[k * nlon / 2^s]
    for (int b = threadIdx.x; b < nrow * hh; b += blockDim.x) {
      int p = b / hh, bb = b - p * hh;
      int grp = bb >> (s - 1), k = bb & (half - 1);
      int i0 = p * h + (grp << s) + k, i1 = i0 + half;
      int ti = k << tshift;
      T wr = tw[2 * ti], wi = (T)SIGN * tw[2 * ti + 1];
      T xr = re[i1], xi = im[i1];
      T tr = xr * wr - xi * wi, tI = xr * wi + xi * wr;
      T ar = re[i0], ai = im[i0];
      re[i1] = ar - tr;
      im[i1] = ai - tI;
      re[i0] = ar + tr;
      im[i0] = ai + tI;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------------------------------------
// spectral -> Fourier: Legendre synthesis.  grid (ceil(C/CT), N+1), 256 threads.
template <typename T>
__global__ void __launch_bounds__(256) k_s2g_legendre(S2GPlan plan, Tables<T> tb, V2<T>* __restrict__ F, int ns,
                                                      int nlat, int CT) {
  using V = V2<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int m = blockIdx.y;
  const int nh = nlat >> 1;
  const int K = ns + 1 - m;
  T* Ps = (T*)smem;
  V* X = (V*)(smem + align16((size_t)(ns + 1) * nh * sizeof(T)));
  const int C = plan.C;
  const int cbase = blockIdx.x * CT;
  const size_t mrow = (size_t)m * (ns + 1);
  const T* Pm = tb.P + (mrow + m) * nh;
  // the m-block of P (constants, one contiguous run): staged before the dependency wait, by
  // asynchronous 16-byte copies when its rows are whole chunks
  const bool async_p = (nh * sizeof(T)) % 16 == 0;
  if (async_p) {
    constexpr int ce = 16 / (int)sizeof(T);
    for (int i = threadIdx.x; i < K * nh / ce; i += blockDim.x) cp_async16(Ps + i * ce, Pm + i * ce);
    cp_async_commit();
  } else {
    for (int i = threadIdx.x; i < K * nh; i += blockDim.x) Ps[i] = Pm[i];
  }
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  // CT divides the block (a power of two up to 256): a thread keeps one column, its group found
  // once, and walks rows r (and below latitudes j) in steps of blockDim / CT
  const bool fixed_col = blockDim.x % CT == 0;
  const int cl0 = threadIdx.x % CT, rstep = blockDim.x / CT;
  if (fixed_col) {
    const int c = cbase + cl0;
    if (c < C) {
      int k;
      const S2GGroup& g = group_of(plan.g, plan.ng, c, &k);
      for (int r = threadIdx.x / CT; r < K; r += rstep) X[r * CT + cl0] = s2g_input<T>(g, tb, m, m + r, ns, mrow, k);
    } else {
      for (int r = threadIdx.x / CT; r < K; r += rstep) X[r * CT + cl0] = V{0, 0};
    }
  } else {
    for (int i = threadIdx.x; i < K * CT; i += blockDim.x) {
      int r = i / CT, cl = i - r * CT, n = m + r, c = cbase + cl;
      V x;
      x.x = 0;
      x.y = 0;
      if (c < C) {
        int k;
        const S2GGroup& g = group_of(plan.g, plan.ng, c, &k);
        x = s2g_input<T>(g, tb, m, n, ns, mrow, k);
      }
      X[i] = x;
    }
  }
  if (async_p) cp_async_wait_all();
  __syncthreads();
  // two or more outputs per thread (large column tiles: member ensembles): a thread takes columns cl
  // and cl + CT/2 of one latitude, so each P weight loaded serves both (the kernel is
  // instruction-bound there); same products in the same order per output
  if (CT % 2 == 0 && nh * CT >= 2 * (int)blockDim.x) {
    const int CT2 = CT / 2;
    for (int i = threadIdx.x; i < nh * CT2; i += blockDim.x) {
      const int j = i / CT2, cl = i - j * CT2;
      T er0 = 0, ei0 = 0, or0 = 0, oi0 = 0, er1 = 0, ei1 = 0, or1 = 0, oi1 = 0;
      int r = 0;
      for (; r + 1 < K; r += 2) {
        const T p0 = Ps[r * nh + j], p1 = Ps[(r + 1) * nh + j];
        const V a0 = X[r * CT + cl], a1 = X[(r + 1) * CT + cl];
        const V b0 = X[r * CT + cl + CT2], b1 = X[(r + 1) * CT + cl + CT2];
        er0 += p0 * a0.x;
        ei0 += p0 * a0.y;
        or0 += p1 * a1.x;
        oi0 += p1 * a1.y;
        er1 += p0 * b0.x;
        ei1 += p0 * b0.y;
        or1 += p1 * b1.x;
        oi1 += p1 * b1.y;
      }
      if (r < K) {
        const T p0 = Ps[r * nh + j];
        const V a0 = X[r * CT + cl], b0 = X[r * CT + cl + CT2];
        er0 += p0 * a0.x;
        ei0 += p0 * a0.y;
        er1 += p0 * b0.x;
        ei1 += p0 * b0.y;
      }
      const size_t rn = ((size_t)m * nlat + j) * C, rs = ((size_t)m * nlat + (nlat - 1 - j)) * C;
      V s, nn;
      if (cbase + cl < C) {
        s.x = er0 + or0;
        s.y = ei0 + oi0;
        nn.x = er0 - or0;
        nn.y = ei0 - oi0;
        F[rn + cbase + cl] = s;
        F[rs + cbase + cl] = nn;
      }
      if (cbase + cl + CT2 < C) {
        s.x = er1 + or1;
        s.y = ei1 + oi1;
        nn.x = er1 - or1;
        nn.y = ei1 - oi1;
        F[rn + cbase + cl + CT2] = s;
        F[rs + cbase + cl + CT2] = nn;
      }
    }
    return;
  }
  for (int i = threadIdx.x, jf = threadIdx.x / CT; i < nh * CT; i += blockDim.x, jf += rstep) {
    const int j = fixed_col ? jf : i / CT, cl = fixed_col ? cl0 : i - j * CT, c = cbase + cl;
    T er = 0, ei = 0, orr = 0, oi = 0;
    int r = 0;
    for (; r + 1 < K; r += 2) {
      T p0 = Ps[r * nh + j], p1 = Ps[(r + 1) * nh + j];
      V x0 = X[r * CT + cl], x1 = X[(r + 1) * CT + cl];
      er += p0 * x0.x;
      ei += p0 * x0.y;
      orr += p1 * x1.x;
      oi += p1 * x1.y;
    }
    if (r < K) {
      T p0 = Ps[r * nh + j];
      V x0 = X[r * CT + cl];
      er += p0 * x0.x;
      ei += p0 * x0.y;
    }
    if (c < C) {
      V s, nn;
      s.x = er + orr;
      s.y = ei + oi;
      nn.x = er - orr;
      nn.y = ei - oi;
      F[((size_t)m * nlat + j) * C + c] = s;
      F[((size_t)m * nlat + (nlat - 1 - j)) * C + c] = nn;
    }
  }
}

// ------------------------------------------------------------------------------------------
// Per-element epilogue of the inverse FFT (value x at longitude t of latitude j, column k of
// group g) and prologue of the forward FFT (the grid value to transform).
template <typename T>
__device__ __forceinline__ void ifft_store(const GridOutGroup& g, const Tables<T>& tb, int k, int j, int t, int nlat,
                                           int nlon, T x) {
  size_t idx = ((size_t)k * nlat + j) * nlon + t;
  T* dst = (T*)g.dst;
  switch (g.epi) {
    case EPI_NONE:
      dst[idx] = x;
      break;
    case EPI_DIVCOS:
      dst[idx] = x / tb.cosj[j];
      break;
    case EPI_EXP2:
      dst[idx] = x + pick<T>(g.shift, g.shiftf);
      ((T*)g.dst2)[idx] = exp(x) * pick<T>(g.eshift, g.eshiftf);
      break;
    case EPI_DIVCOS_MULPS:
      dst[idx] = (x / tb.cosj[j]) * ((const T*)g.ps)[((size_t)k * nlat + j) * nlon + t];  // level k of ps
      break;
    case EPI_ADJ_G2S:
      dst[idx] = x * (tb.wts[j] / (T)(2 * nlon));
      break;
    case EPI_ANOM:
      dst[idx] = x + ((const V2<T>*)g.ps)[k].x;
      ((T*)g.dst2)[idx] = x;
      break;
  }
}

template <typename T>
__device__ __forceinline__ T fft_load(const FFTPlan& plan, const GridInGroup& g, int k, int j, int t, int nlat,
                                      int nlon, T cj) {
  T x = 0;
  size_t idx = ((size_t)k * nlat + j) * nlon + t;
  const T* s0 = (const T*)g.src;
  switch (g.pro) {
    case PRO_NONE:
      x = s0[idx];
      break;
    case PRO_MULCOS:
      x = s0[idx] * cj;
      break;
    case PRO_FLUXU: {  // (-kappa_m u + (vor + f) v) cos   (Shallow_Water_Dynamics.jl:129, Barotropic :28)
      T u = s0[idx], v = ((const T*)g.s1)[idx], vor = ((const T*)g.s2)[idx];
      T absvor = vor + ((const T*)plan.coriolis)[j];
      x = ((-pick<T>(plan.kappa_m, plan.kappa_mf)) * u + absvor * v) * cj;
    } break;
    case PRO_FLUXV: {  // (-kappa_m v + (-(vor + f)) u) cos
      T u = s0[idx], v = ((const T*)g.s1)[idx], vor = ((const T*)g.s2)[idx];
      T absvor = vor + ((const T*)plan.coriolis)[j];
      x = ((-pick<T>(plan.kappa_m, plan.kappa_mf)) * v + (-absvor) * u) * cj;
    } break;
    case PRO_KIN: {  // 0.5 (u^2 + v^2)
      T u = s0[idx], v = ((const T*)g.s1)[idx];
      x = (T)0.5 * (u * u + v * v);
    } break;
    case PRO_SWH: {  // -kappa_t (h - h_eq) - (u dlam_h + v dth_h) - h div
      T h = s0[idx], u = ((const T*)g.s1)[idx], v = ((const T*)g.s2)[idx];
      T dl = ((const T*)g.s3)[idx], dt = ((const T*)g.s4)[idx], dv = ((const T*)g.s5)[idx];
      T heq = ((const T*)g.s6)[idx];
      T d = (-pick<T>(plan.kappa_t, plan.kappa_tf)) * (h - heq);
      d = d - (u * dl + v * dt);
      x = d - h * dv;
    } break;
  }
  return x;
}

// Fourier -> grid: inverse real FFT, one column per half-length (h = nlon/2) complex transform,
// so rounding never leaks between columns of different magnitude.  grid (ceil(C/CT), nlat),
// 256 threads.  Row x(λ_t) = Re g_0 + 2 Re sum_{m=1}^{N} g_m e^{imλ_t}, i.e. 2 nλ Re(ifft(g)) with
// g_0 halved as in Spectral_Spherical_Mesh.jl:211-215.  With X the Hermitian spectrum,
// Z[m] = (X[m] + conj X[h-m]) + i e^{2πim/nλ} (X[m] - conj X[h-m]) and z = ifft_h(Z) give
// x[2k] = Re z[k], x[2k+1] = Im z[k].
template <typename T>
__global__ void __launch_bounds__(256) k_ifft(IFFTPlan plan, Tables<T> tb, const V2<T>* __restrict__ F, int N,
                                              int nlat, int nlon, int logh, int CT) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using V = V2<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int h = nlon >> 1;
  T* re = (T*)smem;
  T* im = re + CT * h;
  T* tw = im + CT * h;
  V* G = (V*)(smem + align16((size_t)(CT * nlon + nlon) * sizeof(T)));  // [N+1][CT]
  const int j = blockIdx.y;
  const int C = plan.C;
  const int cbase = blockIdx.x * CT;
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) tw[i] = tb.tw[i];
  for (int i = threadIdx.x; i < (N + 1) * CT; i += blockDim.x) {
    int mm = i / CT, cc = i - mm * CT, c = cbase + cc;
    V g;
    g.x = 0;
    g.y = 0;
    if (c < C) g = F[((size_t)mm * nlat + j) * C + c];
    if (mm == 0) g.y = 0;  // only Re g_0 reaches the grid
    G[i] = g;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < CT * h; i += blockDim.x) {
    int cc = i / h, mm = i - cc * h, q = h - mm;
    V x, y;
    x.x = x.y = y.x = y.y = 0;
    if (mm <= N) x = G[mm * CT + cc];
    if (mm >= 1 && q <= N) y = G[q * CT + cc];
    T er = x.x + y.x, ei = x.y - y.y;  // X[m] + conj X[h-m]
    T dr = x.x - y.x, di = x.y + y.y;  // X[m] - conj X[h-m]
    T c = tw[2 * mm], s = tw[2 * mm + 1];
    T orr = dr * c - di * s, oi = dr * s + di * c;
    int pos = brev(mm, logh);
    re[cc * h + pos] = er - oi;
    im[cc * h + pos] = ei + orr;
  }
  __syncthreads();
  fft_stages<T, 1>(re, im, tw, CT, h, logh);
  for (int i = threadIdx.x; i < CT * nlon; i += blockDim.x) {
    int cc = i / nlon, t = i - cc * nlon, c = cbase + cc;
    if (c >= C) continue;
    T x = (t & 1) ? im[cc * h + (t >> 1)] : re[cc * h + (t >> 1)];
    int k;
    const GridOutGroup& g = group_of(plan.g, plan.ng, c, &k);
    ifft_store<T>(g, tb, k, j, t, nlat, nlon, x);
  }
}

// Grid -> Fourier: forward real FFT (fft/nlon), modes 0..N, one column per half-length complex
// transform: z[k] = x[2k] + i x[2k+1], Z = fft_h(z), X[m] = E[m] + e^{-2πim/nλ} O[m] with
// E = (Z[m] + conj Z[h-m])/2, O = (Z[m] - conj Z[h-m])/(2i).  grid (ceil(C/CT), nlat).
template <typename T>
__global__ void __launch_bounds__(256) k_fft(FFTPlan plan, Tables<T> tb, V2<T>* __restrict__ F, int N, int nlat,
                                             int nlon, int logh, int CT) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using V = V2<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int h = nlon >> 1;
  T* re = (T*)smem;
  T* im = re + CT * h;
  T* tw = im + CT * h;
  const int j = blockIdx.y;
  const int C = plan.C;
  const int ncol = CT;
  const int cbase = blockIdx.x * ncol;
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) tw[i] = tb.tw[i];
  const T cj = tb.cosj[j];
  for (int i = threadIdx.x; i < ncol * nlon; i += blockDim.x) {
    int cc = i / nlon, t = i - cc * nlon, c = cbase + cc;
    T x = 0;
    if (c < C) {
      int k;
      const GridInGroup& g = group_of(plan.g, plan.ng, c, &k);
      x = fft_load<T>(plan, g, k, j, t, nlat, nlon, cj);
    }
    int pos = brev(t >> 1, logh);
    if (t & 1)
      im[cc * h + pos] = x;
    else
      re[cc * h + pos] = x;
  }
  __syncthreads();
  fft_stages<T, -1>(re, im, tw, CT, h, logh);
  const T scale = (T)0.5 / (T)nlon;  // nlon is a power of two: exact
  for (int i = threadIdx.x; i < (N + 1) * ncol; i += blockDim.x) {
    int mm = i / ncol, cc = i - mm * ncol, c = cbase + cc;
    if (c >= C) continue;
    int q = (h - mm) & (h - 1);
    T zr = re[cc * h + mm], zi = im[cc * h + mm], qr = re[cc * h + q], qi = im[cc * h + q];
    T er = zr + qr, ei = zi - qi;  // 2 E
    T orr = zi + qi, oi = qr - zr;  // 2 O
    T tc = tw[2 * mm], ts = tw[2 * mm + 1];  // e^{-2πim/nλ} = tc - i ts
    V o;
    o.x = (er + (tc * orr + ts * oi)) * scale;
    o.y = (ei + (tc * oi - ts * orr)) * scale;
    F[((size_t)mm * nlat + j) * C + c] = o;
  }
}

// Grid -> Fourier as Trans_Grid_To_Fourier! returns it (Spectral_Spherical_Mesh.jl:295-330): fft/nλ of
// every row, all nλ modes, written straight into the FP64 host layout out[k][j][i] (complex
// interleaved, i fastest: Julia's Array{ComplexF64,3}(nλ, nθ, L)).  Modes m < h as k_fft forms them,
// the Nyquist mode X[h] = Re Z[0] - Im Z[0], and the modes above h by the Hermitian symmetry of a
// real row, X[nλ - m] = conj X[m].  Same shared-memory transform and block shape as k_fft; this
// serves the entry point only (the model steps read modes m <= N from k_fft and its variants).
template <typename T>
__global__ void __launch_bounds__(256) k_fourier_full(const T* __restrict__ grid, Tables<T> tb,
                                                      double* __restrict__ out, int C, int nlat, int nlon,
                                                      int logh, int CT) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int h = nlon >> 1;
  T* re = (T*)smem;
  T* im = re + CT * h;
  T* tw = im + CT * h;
  const int j = blockIdx.y;
  const int cbase = blockIdx.x * CT;
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) tw[i] = tb.tw[i];
  for (int i = threadIdx.x; i < CT * nlon; i += blockDim.x) {
    int cc = i / nlon, t = i - cc * nlon, c = cbase + cc;
    T x = c < C ? grid[((size_t)c * nlat + j) * nlon + t] : (T)0;
    int pos = brev(t >> 1, logh);
    if (t & 1)
      im[cc * h + pos] = x;
    else
      re[cc * h + pos] = x;
  }
  __syncthreads();
  fft_stages<T, -1>(re, im, tw, CT, h, logh);
  const T scale = (T)0.5 / (T)nlon;  // nlon is a power of two: exact
  for (int i = threadIdx.x; i < CT * nlon; i += blockDim.x) {
    int cc = i / nlon, t = i - cc * nlon, c = cbase + cc;
    if (c >= C) continue;
    const int mm = t <= h ? t : nlon - t;
    T xr, xi;
    if (mm == h) {
      xr = (re[cc * h] - im[cc * h]) * (scale + scale);
      xi = 0;
    } else {
      int q = (h - mm) & (h - 1);
      T zr = re[cc * h + mm], zi = im[cc * h + mm], qr = re[cc * h + q], qi = im[cc * h + q];
      T er = zr + qr, ei = zi - qi;   // 2 E
      T orr = zi + qi, oi = qr - zr;  // 2 O
      T tc = tw[2 * mm], ts = tw[2 * mm + 1];
      xr = (er + (tc * orr + ts * oi)) * scale;
      xi = (ei + (tc * oi - ts * orr)) * scale;
    }
    if (t > h) xi = -xi;
    const size_t o = (((size_t)c * nlat + j) * nlon + t) * 2;
    out[o] = (double)xr;
    out[o + 1] = (double)xi;
  }
}

// ------------------------------------------------------------------------------------------
// Warp-register FFTs (nlon = 64 V, V = 1..16): one warp per (column, latitude) row, the H = 32 V
// complex points held V per lane (point i = lane + 32 r), radix-2 stages of half-size s >= 32
// within a lane and s < 32 across lanes by shuffles: no block barrier inside the transform.  A
// block stages the Fourier coefficients of its 8 columns once (coalesced) and its 8 warps transform
// one column each.  Same arithmetic as k_ifft / k_fft (half-length complex transform of a real row).
constexpr int FW_COLS = 8;  // columns (warps) per block

// twiddle e^{SIGN 2πi t / nlon}, t < nlon/2, from the cos/sin table
template <typename T, int SIGN>
__device__ __forceinline__ void twiddle(const T* tw, int t, T& c, T& s) {
  c = __ldg(tw + 2 * t);
  s = (T)SIGN * __ldg(tw + 2 * t + 1);
}

// inverse: DIT on bit-reversed input -> natural order, twiddles e^{+2πi j/(2s)} = tw[j H / s]
template <typename T, int V>
__device__ __forceinline__ void warp_fft_dit(T (&re)[V], T (&im)[V], const T* tw, int lane) {
  constexpr int H = 32 * V;
#pragma unroll
  for (int s = 1; s < 32; s <<= 1) {
    const bool upper = (lane & s) != 0;
    const int jj = lane & (s - 1);
    T c, sn;
    twiddle<T, 1>(tw, jj * (H / s), c, sn);
#pragma unroll
    for (int r = 0; r < V; r++) {
      const T pr = __shfl_xor_sync(0xffffffffu, re[r], s), pi = __shfl_xor_sync(0xffffffffu, im[r], s);
      // lower: a + w b (b = partner); upper: a' - w b' with a' = partner, b' = own
      const T br = upper ? re[r] : pr, bi = upper ? im[r] : pi;
      const T ar = upper ? pr : re[r], ai = upper ? pi : im[r];
      const T tr = br * c - bi * sn, ti = br * sn + bi * c;
      re[r] = upper ? ar - tr : ar + tr;
      im[r] = upper ? ai - ti : ai + ti;
    }
  }
#pragma unroll
  for (int s = 32; s < H; s <<= 1) {
    constexpr int dummy = 0;
    (void)dummy;
    const int sr = s / 32;
#pragma unroll
    for (int r = 0; r < V; r++) {
      if ((r & sr) == 0) {
        const int jj = (lane + 32 * r) & (s - 1);
        T c, sn;
        twiddle<T, 1>(tw, jj * (H / s), c, sn);
        const T br = re[r + sr], bi = im[r + sr];
        const T tr = br * c - bi * sn, ti = br * sn + bi * c;
        re[r + sr] = re[r] - tr;
        im[r + sr] = im[r] - ti;
        re[r] = re[r] + tr;
        im[r] = im[r] + ti;
      }
    }
  }
}

// forward: DIF on natural input -> bit-reversed order, twiddles e^{-2πi j/(2s)}
template <typename T, int V>
__device__ __forceinline__ void warp_fft_dif(T (&re)[V], T (&im)[V], const T* tw, int lane) {
  constexpr int H = 32 * V;
#pragma unroll
  for (int s = H / 2; s >= 32; s >>= 1) {
    const int sr = s / 32;
#pragma unroll
    for (int r = 0; r < V; r++) {
      if ((r & sr) == 0) {
        const int jj = (lane + 32 * r) & (s - 1);
        T c, sn;
        twiddle<T, -1>(tw, jj * (H / s), c, sn);
        const T ar = re[r], ai = im[r], br = re[r + sr], bi = im[r + sr];
        re[r] = ar + br;
        im[r] = ai + bi;
        const T dr = ar - br, di = ai - bi;
        re[r + sr] = dr * c - di * sn;
        im[r + sr] = dr * sn + di * c;
      }
    }
  }
#pragma unroll
  for (int s = 16; s >= 1; s >>= 1) {
    const bool upper = (lane & s) != 0;
    const int jj = lane & (s - 1);
    T c, sn;
    twiddle<T, -1>(tw, jj * (H / s), c, sn);
#pragma unroll
    for (int r = 0; r < V; r++) {
      const T pr = __shfl_xor_sync(0xffffffffu, re[r], s), pi = __shfl_xor_sync(0xffffffffu, im[r], s);
      // lower: a + b; upper: (a - b) w with a = partner, b = own
      const T dr = pr - re[r], di = pi - im[r];
      re[r] = upper ? dr * c - di * sn : re[r] + pr;
      im[r] = upper ? dr * sn + di * c : im[r] + pi;
    }
  }
}

// The epilogue of longitudes t, t+1 (t even) of row (k, j): one 8- or 16-byte store per output,
// ÷cos θ as a product with rc = 1/cos θ (within an ulp of the quotient)
template <typename T>
__device__ __forceinline__ void ifft_store_pair(const GridOutGroup& g, const Tables<T>& tb, int k, int j, int nlat,
                                                int nlon, int t, T a, T b, T rc) {
  using P = V2<T>;
  const size_t idx = ((size_t)k * nlat + j) * nlon + t;
  P v;
  switch (g.epi) {
    case EPI_NONE:
      v.x = a;
      v.y = b;
      break;
    case EPI_DIVCOS:
      v.x = a * rc;
      v.y = b * rc;
      break;
    case EPI_EXP2: {
      const T sh = pick<T>(g.shift, g.shiftf), es = pick<T>(g.eshift, g.eshiftf);
      v.x = a + sh;
      v.y = b + sh;
      P e;
      e.x = exp(a) * es;
      e.y = exp(b) * es;
      *reinterpret_cast<P*>((T*)g.dst2 + idx) = e;
    } break;
    case EPI_DIVCOS_MULPS: {  // level k of ps
      const P q = *reinterpret_cast<const P*>((const T*)g.ps + idx);
      v.x = (a * rc) * q.x;
      v.y = (b * rc) * q.y;
    } break;
    case EPI_ADJ_G2S: {
      const auto sc = tb.wts[j] / (T)(2 * nlon);
      v.x = (T)(a * sc);
      v.y = (T)(b * sc);
    } break;
    case EPI_ANOM: {
      const T mean = ((const V2<T>*)g.ps)[k].x;
      v.x = a + mean;
      v.y = b + mean;
      P d;
      d.x = a;
      d.y = b;
      *reinterpret_cast<P*>((T*)g.dst2 + idx) = d;
    } break;
  }
  *reinterpret_cast<P*>((T*)g.dst + idx) = v;
}

// The epilogue of one warp's row (k_ifft_w): x(λ_2i) = re[r], x(λ_2i+1) = im[r] for i = lane + 32 r,
// the group's epilogue chosen once per row and each pair of longitudes stored as one 8- or 16-byte
// word.  ÷cos θ as a product with 1/cos θ (within an ulp of the quotient).
template <typename T, int V>
__device__ __forceinline__ void ifft_store_row(const GridOutGroup& g, const Tables<T>& tb, int k, int j, int nlat,
                                               int nlon, const T (&re)[V], const T (&im)[V], int lane) {
  using P = V2<T>;
  const size_t row = ((size_t)k * nlat + j) * nlon;
  P* dst = reinterpret_cast<P*>((T*)g.dst + row);
  auto put = [](P* d, int i, T a, T b) {
    P v;
    v.x = a;
    v.y = b;
    d[i] = v;
  };
  switch (g.epi) {
    case EPI_NONE:
#pragma unroll
      for (int r = 0; r < V; r++) put(dst, lane + 32 * r, re[r], im[r]);
      break;
    case EPI_DIVCOS: {
      const T rc = (T)1 / tb.cosj[j];
#pragma unroll
      for (int r = 0; r < V; r++) put(dst, lane + 32 * r, re[r] * rc, im[r] * rc);
    } break;
    case EPI_EXP2: {
      const T sh = pick<T>(g.shift, g.shiftf), es = pick<T>(g.eshift, g.eshiftf);
      P* d2 = reinterpret_cast<P*>((T*)g.dst2 + row);
#pragma unroll
      for (int r = 0; r < V; r++) {
        put(dst, lane + 32 * r, re[r] + sh, im[r] + sh);
        put(d2, lane + 32 * r, exp(re[r]) * es, exp(im[r]) * es);
      }
    } break;
    case EPI_DIVCOS_MULPS: {  // level k of ps
      const T rc = (T)1 / tb.cosj[j];
      const P* ps = reinterpret_cast<const P*>((const T*)g.ps + row);
#pragma unroll
      for (int r = 0; r < V; r++) {
        const P q = ps[lane + 32 * r];
        put(dst, lane + 32 * r, (re[r] * rc) * q.x, (im[r] * rc) * q.y);
      }
    } break;
    case EPI_ADJ_G2S: {
      const auto sc = tb.wts[j] / (T)(2 * nlon);
#pragma unroll
      for (int r = 0; r < V; r++) put(dst, lane + 32 * r, (T)(re[r] * sc), (T)(im[r] * sc));
    } break;
    case EPI_ANOM: {
      const T mean = ((const V2<T>*)g.ps)[k].x;
      P* d2 = reinterpret_cast<P*>((T*)g.dst2 + row);
#pragma unroll
      for (int r = 0; r < V; r++) {
        put(dst, lane + 32 * r, re[r] + mean, im[r] + mean);
        put(d2, lane + 32 * r, re[r], im[r]);
      }
    } break;
  }
}

template <typename T, int V>
__global__ void __launch_bounds__(256) k_ifft_w(IFFTPlan plan, Tables<T> tb, const V2<T>* __restrict__ F, int N,
                                                int nlat, int nlon) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using Vc = V2<T>;
  constexpr int H = 32 * V, LOGH = (V == 1 ? 5 : V == 2 ? 6 : V == 4 ? 7 : V == 8 ? 8 : 9);
  extern __shared__ __align__(16) unsigned char smem[];
  Vc* G = (Vc*)smem;  // [N+1][FW_COLS]
  const int j = blockIdx.y, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int C = plan.C, cbase = blockIdx.x * FW_COLS, c = cbase + w;
  for (int i = threadIdx.x; i < (N + 1) * FW_COLS; i += blockDim.x) {
    const int mm = i / FW_COLS, cc = i - mm * FW_COLS;
    Vc g;
    g.x = g.y = 0;
    if (cbase + cc < C) g = F[((size_t)mm * nlat + j) * C + cbase + cc];
    if (mm == 0) g.y = 0;  // only Re g_0 reaches the grid
    G[i] = g;
  }
  __syncthreads();
  if (c >= C) return;  // whole warp
  T re[V], im[V];
#pragma unroll
  for (int r = 0; r < V; r++) {  // Z at bit-reversed position: element i holds Z[brev(i)]
    const int mm = brev(lane + 32 * r, LOGH), q = H - mm;
    Vc x, y;
    x.x = x.y = y.x = y.y = 0;
    if (mm <= N) x = G[mm * FW_COLS + w];
    if (mm >= 1 && q <= N) y = G[q * FW_COLS + w];
    const T er = x.x + y.x, ei = x.y - y.y;  // X[m] + conj X[h-m]
    const T dr = x.x - y.x, di = x.y + y.y;  // X[m] - conj X[h-m]
    T cs, sn;
    twiddle<T, 1>(tb.tw, mm, cs, sn);
    const T orr = dr * cs - di * sn, oi = dr * sn + di * cs;
    re[r] = er - oi;
    im[r] = ei + orr;
  }
  warp_fft_dit<T, V>(re, im, tb.tw, lane);
  int k;
  const GridOutGroup& g = group_of(plan.g, plan.ng, c, &k);
  ifft_store_row<T, V>(g, tb, k, j, nlat, nlon, re, im, lane);  // z[i] = x[2i] + i x[2i+1]
}

template <typename T, int V, bool PLAIN>
__global__ void __launch_bounds__(256) k_fft_w(FFTPlan plan, Tables<T> tb, V2<T>* __restrict__ F, int N, int nlat,
                                               int nlon) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using Vc = V2<T>;
  constexpr int H = 32 * V, LOGH = (V == 1 ? 5 : V == 2 ? 6 : V == 4 ? 7 : V == 8 ? 8 : 9);
  extern __shared__ __align__(16) unsigned char smem[];
  const int j = blockIdx.y, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  Vc* Z = (Vc*)smem + (size_t)w * H;  // this warp's spectrum, natural order
  Vc* X = (Vc*)smem + (size_t)FW_COLS * H;  // [N+1][FW_COLS] results of the block
  const int C = plan.C, cbase = blockIdx.x * FW_COLS, c = cbase + w;
  if (c < C) {
    int k;
    const GridInGroup& g = group_of(plan.g, plan.ng, c, &k);
    const T cj = tb.cosj[j];
    T re[V], im[V];
#pragma unroll
    for (int r = 0; r < V; r++) {  // z[i] = x[2i] + i x[2i+1], natural order
      const int i = lane + 32 * r;
      if (PLAIN) {  // every group reads its field as it is (k_fft_rows' PLAIN); a pair per load
        const Vc* src = reinterpret_cast<const Vc*>((const T*)g.src + ((size_t)k * nlat + j) * nlon);
        const Vc x = src[i];
        re[r] = x.x;
        im[r] = x.y;
      } else {
        re[r] = fft_load<T>(plan, g, k, j, 2 * i, nlat, nlon, cj);
        im[r] = fft_load<T>(plan, g, k, j, 2 * i + 1, nlat, nlon, cj);
      }
    }
    warp_fft_dif<T, V>(re, im, tb.tw, lane);
#pragma unroll
    for (int r = 0; r < V; r++) {
      Vc z;
      z.x = re[r];
      z.y = im[r];
      Z[brev(lane + 32 * r, LOGH)] = z;
    }
    __syncwarp();
    const T scale = (T)0.5 / (T)nlon;  // nlon is a power of two: exact
    for (int mm = lane; mm <= N; mm += 32) {
      const int q = (H - mm) & (H - 1);
      const Vc zm = Z[mm], zq = Z[q];
      const T er = zm.x + zq.x, ei = zm.y - zq.y;  // 2 E
      const T orr = zm.y + zq.y, oi = zq.x - zm.x;  // 2 O
      T tc, ts;
      twiddle<T, 1>(tb.tw, mm, tc, ts);  // e^{-2πim/nλ} = tc - i ts
      Vc o;
      o.x = (er + (tc * orr + ts * oi)) * scale;
      o.y = (ei + (tc * oi - ts * orr)) * scale;
      X[mm * FW_COLS + w] = o;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < (N + 1) * FW_COLS; i += blockDim.x) {  // rows of 8 columns per m
    const int mm = i / FW_COLS, cc = i - mm * FW_COLS;
    if (cbase + cc < C) F[((size_t)mm * nlat + j) * C + cbase + cc] = X[i];
  }
}

// ------------------------------------------------------------------------------------------
// Row-per-thread real FFTs (FP32, nlon = 64 or 128) for transforms with many (column, latitude) rows
// (member ensembles).  Each thread transforms one row in registers: the H = nlon/2 point complex
// transform as radix-2 stages unrolled at compile time, with the twiddles passed as a kernel
// parameter and read at compile-time indices (constant-bank operands: no loads, shuffles or block
// barriers in the transform).  A warp's 32 rows pass through padded shared memory, so that every
// global read and write is a coalesced row (grid) or a run of 32 consecutive columns (Fourier).
// Same arithmetic as k_fft_w / k_ifft_w: the half-length complex transform of the real row.
template <int NLON>
struct RowTwiddles {
  float c[NLON / 2], s[NLON / 2];  // cos, sin of 2π t / nlon
};
constexpr int RF_WARPS = 4;               // warps per block, 32 rows each
// rows from which the row-per-thread kernels are used: 128 per SM (4 warps), 19456 on GB300
static inline size_t rows_min(const jgcm_mesh* m) { return (size_t)m->sm_count * 4 * 32; }

__host__ __device__ constexpr int brev_c(int x, int bits) {
  int r = 0;
  for (int b = 0; b < bits; b++) r |= ((x >> b) & 1) << (bits - 1 - b);
  return r;
}

// PLAIN: every group of the plan reads its field as it is (PRO_NONE): the prologue switch, inlined
// for each of a warp's 32 rows, leaves the instruction stream
template <int NLON, bool PLAIN>
__global__ void __launch_bounds__(32 * RF_WARPS) k_fft_rows(FFTPlan plan, Tables<float> tb, RowTwiddles<NLON> tw,
                                                            float2* __restrict__ F, int N, int nlat) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  constexpr int H = NLON / 2, P = NLON + 1, LOGH = NLON == 64 ? 5 : 6;
  extern __shared__ float rsm[];
  const int j = blockIdx.y, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int C = plan.C, c0 = (blockIdx.x * RF_WARPS + w) * 32;
  if (c0 >= C) return;  // whole warp; no block barrier follows
  float* S = rsm + (size_t)w * 32 * P;
  const int nr = min(32, C - c0);
  const float cj = tb.cosj[j];
  // each lane finds the group of one row (its own column) once; the rows' groups are broadcast
  int gi = 0, gk = 0;
  if (lane < nr) {
    while (gi < plan.ng - 1 && c0 + lane >= plan.g[gi].col0 + plan.g[gi].L) gi++;
    gk = c0 + lane - plan.g[gi].col0;
  }
  // row r = column c0 + r, lanes along longitude (coalesced); 16 rows' loads are issued before any
  // of them is stored, so their latencies overlap
  constexpr int RB = 16;
#pragma unroll
  for (int rb = 0; rb < 32; rb += RB) {
    float v[RB][NLON / 32];
#pragma unroll
    for (int rr = 0; rr < RB; rr++) {
#pragma unroll
      for (int q = 0; q < NLON / 32; q++) v[rr][q] = 0.f;
      const int g_r = __shfl_sync(0xffffffffu, gi, rb + rr), k = __shfl_sync(0xffffffffu, gk, rb + rr);
      if (rb + rr < nr) {
        const GridInGroup& g = plan.g[g_r];
#pragma unroll
        for (int q = 0; q < NLON / 32; q++)
          v[rr][q] = PLAIN ? ((const float*)g.src)[((size_t)k * nlat + j) * NLON + lane + 32 * q]
                           : fft_load<float>(plan, g, k, j, lane + 32 * q, nlat, NLON, cj);
      }
    }
#pragma unroll
    for (int rr = 0; rr < RB; rr++)
#pragma unroll
      for (int q = 0; q < NLON / 32; q++) S[(rb + rr) * P + lane + 32 * q] = v[rr][q];
  }
  __syncwarp();
  if (lane >= nr) return;
  float re[H], im[H];  // z[i] = x[2i] + i x[2i+1], natural order
#pragma unroll
  for (int i = 0; i < H; i++) {
    re[i] = S[lane * P + 2 * i];
    im[i] = S[lane * P + 2 * i + 1];
  }
  // decimation in frequency, w = e^{-2πi jj/(2s)} = tw[jj nlon/(2s)]: bit-reversed output
#pragma unroll
  for (int s = H / 2; s >= 1; s >>= 1) {
#pragma unroll
    for (int b = 0; b < H; b += 2 * s) {
#pragma unroll
      for (int jj = 0; jj < s; jj++) {
        const int i0 = b + jj, i1 = i0 + s, t = jj * (NLON / (2 * s));
        const float ar = re[i0], ai = im[i0], br = re[i1], bi = im[i1];
        re[i0] = ar + br;
        im[i0] = ai + bi;
        const float dr = ar - br, di = ai - bi;
        re[i1] = dr * tw.c[t] + di * tw.s[t];
        im[i1] = di * tw.c[t] - dr * tw.s[t];
      }
    }
  }
  // X[m] = (E_m + e^{-2πim/nλ} O_m) / nλ for m <= N, from Z[m] and Z[H - m]
  const float scale = 0.5f / (float)NLON;
  const int c = c0 + lane;
#pragma unroll
  for (int mm = 0; mm < H; mm++) {
    if (mm <= N) {
      const int zi = brev_c(mm, LOGH), qi = brev_c((H - mm) & (H - 1), LOGH);
      const float er = re[zi] + re[qi], ei = im[zi] - im[qi];  // 2 E
      const float orr = im[zi] + im[qi], oi = re[qi] - re[zi];  // 2 O
      const float tc = tw.c[mm], ts = tw.s[mm];
      float2 o;
      o.x = (er + (tc * orr + ts * oi)) * scale;
      o.y = (ei + (tc * oi - ts * orr)) * scale;
      F[((size_t)mm * nlat + j) * C + c] = o;
    }
  }
}

template <int NLON>
__global__ void __launch_bounds__(32 * RF_WARPS, NLON == 64 ? 6 : 1) k_ifft_rows(IFFTPlan plan, Tables<float> tb, RowTwiddles<NLON> tw,
                                                             const float2* __restrict__ F, int N, int nlat) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  constexpr int H = NLON / 2, P = NLON + 1, LOGH = NLON == 64 ? 5 : 6;
  extern __shared__ float rsm[];
  const int j = blockIdx.y, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int C = plan.C, c0 = (blockIdx.x * RF_WARPS + w) * 32;
  if (c0 >= C) return;  // whole warp; no block barrier follows
  float* S = rsm + (size_t)w * 32 * P;
  const int nr = min(32, C - c0);
  if (lane < nr) {
    const int c = c0 + lane;
    auto X = [&](int mm) -> float2 {  // coefficient m of this column (Re only for m = 0), 0 above N
      float2 x = make_float2(0.f, 0.f);
      if (mm <= N) x = F[((size_t)mm * nlat + j) * C + c];
      if (mm == 0) x.y = 0.f;
      return x;
    };
    // Z[m] = (X[m] + conj X[H-m]) + i e^{2πim/nλ} (X[m] - conj X[H-m]), placed bit-reversed; Z[m]
    // and Z[H-m] from the same pair, each coefficient loaded once (short live ranges)
    float re[H], im[H];
    auto zput = [&](int mm, float2 x, float2 y) {
      const float er = x.x + y.x, ei = x.y - y.y, dr = x.x - y.x, di = x.y + y.y;
      const float cs = tw.c[mm], sn = tw.s[mm];
      const float orr = dr * cs - di * sn, oi = dr * sn + di * cs;
      re[brev_c(mm, LOGH)] = er - oi;
      im[brev_c(mm, LOGH)] = ei + orr;
    };
    zput(0, X(0), make_float2(0.f, 0.f));
#pragma unroll
    for (int mm = 1; mm <= H / 2; mm++) {
      const float2 a = X(mm), b = X(H - mm);
      zput(mm, a, b);
      if (mm < H / 2) zput(H - mm, b, a);
    }
    // decimation in time, w = e^{+2πi jj/(2s)}: natural output
#pragma unroll
    for (int s = 1; s < H; s <<= 1) {
#pragma unroll
      for (int b = 0; b < H; b += 2 * s) {
#pragma unroll
        for (int jj = 0; jj < s; jj++) {
          const int i0 = b + jj, i1 = i0 + s, t = jj * (NLON / (2 * s));
          const float br = re[i1], bi = im[i1];
          const float tr = br * tw.c[t] - bi * tw.s[t], ti = br * tw.s[t] + bi * tw.c[t];
          re[i1] = re[i0] - tr;
          im[i1] = im[i0] - ti;
          re[i0] = re[i0] + tr;
          im[i0] = im[i0] + ti;
        }
      }
    }
#pragma unroll
    for (int i = 0; i < H; i++) {  // x[2i] = Re z[i], x[2i+1] = Im z[i]
      S[lane * P + 2 * i] = re[i];
      S[lane * P + 2 * i + 1] = im[i];
    }
  }
  __syncwarp();
  // each lane finds the group of one row (its own column) once; the rows' groups are broadcast
  int gi = 0, gk = 0;
  if (lane < nr) {
    while (gi < plan.ng - 1 && c0 + lane >= plan.g[gi].col0 + plan.g[gi].L) gi++;
    gk = c0 + lane - plan.g[gi].col0;
  }
  const float rc = 1.f / tb.cosj[j];
#pragma unroll 1  // stores need no unrolling to overlap; one copy of the epilogue switch in the code
  for (int r = 0; r < nr; r++) {  // row r = column c0 + r: lane pairs along longitude (coalesced)
    const int g_r = __shfl_sync(0xffffffffu, gi, r), k = __shfl_sync(0xffffffffu, gk, r);
    const GridOutGroup& g = plan.g[g_r];
#pragma unroll
    for (int q = 0; q < NLON / 64; q++) {
      const int t = 2 * (lane + 32 * q);
      ifft_store_pair<float>(g, tb, k, j, nlat, NLON, t, S[r * P + t], S[r * P + t + 1], rc);
    }
  }
}

template <int NLON>
RowTwiddles<NLON> row_twiddles(const jgcm_mesh* m) {
  RowTwiddles<NLON> t;
  for (int q = 0; q < NLON / 2; q++) {
    t.c[q] = m->twf_host[2 * q];
    t.s[q] = m->twf_host[2 * q + 1];
  }
  return t;
}

// FFT tile knob: 0 = by size, from rows_min rows on: nlon 64 both ways, nlon 128 the inverse only
// (its thread holds 64 complex points in 158 registers and still beats the warp FFT, 135 -> 107 us
// at T42 x 32 members; the forward one at 165 registers does not, 80 -> 190 us, measured);
// -1 = rows per thread always (nlon 64 and 128)
static inline bool use_row_fft(const jgcm_mesh* m, int C, bool inverse = false) {
  if (m->tune[3] == -1) return m->nlon == 64 || m->nlon == 128;
  return m->tune[3] == 0 && (m->nlon == 64 || (inverse && m->nlon == 128)) && (size_t)C * m->nlat >= rows_min(m);
}
static inline size_t row_fft_smem(const jgcm_mesh* m) { return (size_t)RF_WARPS * 32 * (m->nlon + 1) * sizeof(float); }

// Fourier -> spectral: Gaussian quadrature per m.  grid (ceil(Cout/CT), N+1), 256 threads.
// Shared memory holds, for 4 input slots, the hemisphere-symmetric and -antisymmetric
// combinations g(mu_j) +/- g(-mu_j) of the tile's columns.
// four consecutive table weights in one 16-byte load (the address is 16-byte aligned: nh is a
// multiple of 4 and the tables start aligned)
__device__ __forceinline__ void ld4(const float* p, float (&w)[4]) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&w)[4]) {
  const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
  w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y;
}

// QL lanes per output (4: a quad splits the latitude sum and combines it with two shuffles, for
// launches too small to fill the device; 1: a lane sums its output alone, half the instructions per
// output, for launches with many outputs).
template <typename T, int QL>
__global__ void __launch_bounds__(256) k_g2s_legendre(G2SPlan plan, Tables<T> tb, const V2<T>* __restrict__ F,
                                                      int ns, int nlat, int Cin, int CT, int stage) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using V = V2<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int m = blockIdx.y;
  const int nh = nlat >> 1;
  const int K = ns + 1 - m;
  const int C = plan.C;
  const int cbase = blockIdx.x * CT;
  V* S = (V*)smem;              // [4][nh][CT] symmetric      (column fastest: no bank conflicts)
  V* A = S + 4 * CT * nh;       // [4][nh][CT] antisymmetric
  const size_t mrow = (size_t)m * (ns + 1);
  // quadrature rows n = m..ns of this m ([K][nh]); staged once per block when they fit
  const T* tPW = tb.PW + (mrow + m) * nh;
  const T* tCA = tb.CA + (mrow + m) * nh;
  const T* tCB = tb.CB + (mrow + m) * nh;
  if (stage) {
    T* sPW = (T*)(A + 4 * CT * nh);
    T* sCA = sPW + K * nh;
    T* sCB = sCA + K * nh;
    for (int i = threadIdx.x; i < K * nh; i += blockDim.x) {
      sPW[i] = tPW[i];
      sCA[i] = tCA[i];
      sCB[i] = tCB[i];
    }
    tPW = sPW;
    tCA = sCA;
    tCB = sCB;
  }
  for (int i = threadIdx.x; i < 4 * CT * nh; i += blockDim.x) {
    int slot = i / (CT * nh), rem = i - slot * CT * nh, jh = rem / CT, cl = rem - jh * CT, c = cbase + cl;
    V s, a;
    s.x = s.y = a.x = a.y = 0;
    if (c < C) {
      int k;
      const SpecOutGroup& g = group_of(plan.g, plan.ng, c, &k);
      int col = slot == 0 ? g.colA : slot == 1 ? g.colB : slot == 2 ? g.colE : g.colH;
      if (col >= 0) {
        col += k;
        V x = F[((size_t)m * nlat + jh) * Cin + col];
        V y = F[((size_t)m * nlat + (nlat - 1 - jh)) * Cin + col];
        s.x = x.x + y.x;
        s.y = x.y + y.y;
        a.x = x.x - y.x;
        a.y = x.y - y.y;
      }
    }
    S[(slot * nh + jh) * CT + cl] = s;
    A[(slot * nh + jh) * CT + cl] = a;
  }
  __syncthreads();
  // each output is summed by QL threads (latitudes jh = q, q+QL, ...), then combined with masked
  // shuffles; the QL lanes never straddle loop iterations (blockDim is a multiple of 4)
  const unsigned qmask = QL == 4 ? 0xFu << (threadIdx.x & 28) : 0u;
  auto qsum = [&](T& x) {
    if (QL == 4) {
      x += __shfl_xor_sync(qmask, x, 1);
      x += __shfl_xor_sync(qmask, x, 2);
    }
  };
  for (int i = threadIdx.x; i < K * CT * QL; i += blockDim.x) {
    const int q = i & (QL - 1), o = i / QL;
    int r = o / CT, cl = o - r * CT, n = m + r, c = cbase + cl;
    if (c >= C) continue;  // whole quad
    int k;
    const SpecOutGroup& g = group_of(plan.g, plan.ng, c, &k);
    const bool even = (r & 1) == 0;
    const T* pw = tPW + r * nh;
    const T* ca = tCA + r * nh;
    const T* cb = tCB + r * nh;
    const size_t sidx = (mrow + n) * g.L + k;
    auto plain = [&](int slot) -> V {
      const V* src = (even ? S : A) + slot * nh * CT + cl;
      T sr = 0, si = 0;
      if (QL == 1) {  // a lane walks every latitude: weights four at a time, same order of sums
        for (int jh = 0; jh < nh; jh += 4) {
          T w[4];
          ld4(pw + jh, w);
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const V x = src[(jh + u) * CT];
            sr += x.x * w[u];
            si += x.y * w[u];
          }
        }
      } else {
#pragma unroll 4
        for (int jh = q; jh < nh; jh += QL) {
          T w = pw[jh];
          V x = src[jh * CT];
          sr += x.x * w;
          si += x.y * w;
        }
      }
      qsum(sr);
      qsum(si);
      V o;
      o.x = (n == ns) ? (T)0 : sr * (T)0.5;
      o.y = (n == ns) ? (T)0 : si * (T)0.5;
      return o;
    };
    // alpha operator: i * sum CA (A) + sign * sum CB (B), all latitudes folded by parity
    auto alpha = [&](int slotA, int slotB, T sign) -> V {
      const V* sa = (even ? S : A) + slotA * nh * CT + cl;
      const V* sb = (even ? A : S) + slotB * nh * CT + cl;
      T ar = 0, ai = 0, br = 0, bi = 0;
      if (QL == 1) {  // weights four at a time, same order of sums
        for (int jh = 0; jh < nh; jh += 4) {
          T wa[4], wb[4];
          ld4(ca + jh, wa);
          ld4(cb + jh, wb);
#pragma unroll
          for (int u = 0; u < 4; u++) {
            const V xa = sa[(jh + u) * CT], xb = sb[(jh + u) * CT];
            ar += (-xa.y) * wa[u];
            ai += xa.x * wa[u];
            br += xb.x * wb[u];
            bi += xb.y * wb[u];
          }
        }
      } else {
#pragma unroll 4
        for (int jh = q; jh < nh; jh += QL) {
          T wa = ca[jh], wb = cb[jh];
          V xa = sa[jh * CT], xb = sb[jh * CT];
          ar += (-xa.y) * wa;
          ai += xa.x * wa;
          br += xb.x * wb;
          bi += xb.y * wb;
        }
      }
      T xr = ar + sign * br, xi = ai + sign * bi;
      qsum(xr);
      qsum(xi);
      V o;
      o.x = (n == ns) ? (T)0 : xr;
      o.y = (n == ns) ? (T)0 : xi;
      return o;
    };
    // adjoint of the synthesis: unweighted quadrature with P, c_m nlon, row N+1 kept
    auto plain_adj = [&]() -> V {
      const V* src = (even ? S : A) + cl;
      const T* p = tb.P + (mrow + n) * nh;
      T sr = 0, si = 0;
#pragma unroll 4
      for (int jh = q; jh < nh; jh += QL) {
        T w = p[jh];
        V x = src[jh * CT];
        sr += x.x * w;
        si += x.y * w;
      }
      qsum(sr);
      qsum(si);
      const T sc = (m == 0 ? (T)1 : (T)2) * pick<T>(g.scale, g.scalef);  // scale = nlon (the FFT returned fft / nlon)
      V o;
      o.x = sr * sc;
      o.y = si * sc;
      return o;
    };
    // every lane of the quad takes part in the sums; lane q = 0 applies the epilogue
    V r0, r1, r2, r3;
    r0.x = r0.y = r1.x = r1.y = r2.x = r2.y = r3.x = r3.y = 0;
    switch (g.op) {
      case G2S_PLAIN:
        r0 = plain(0);
        break;
      case G2S_ADJ_S2G:
        r0 = plain_adj();
        break;
      case G2S_VOR:
      case G2S_BARO:
        r0 = alpha(0, 1, (T)-1);
        break;
      case G2S_DIV:
        r0 = alpha(0, 1, (T)1);
        if (g.colE >= 0) r2 = plain(2);
        break;
      case G2S_SW:
        r0 = alpha(1, 0, (T)-1);
        r1 = alpha(0, 1, (T)1);
        r2 = plain(2);
        r3 = plain(3);
        break;
    }
    if (q != 0) continue;
    g2s_store<T>(plan, g, tb, mrow, n, sidx, r0, r1, r2, r3);
  }
}

// ------------------------------------------------------------------------------------------
static PerDeviceOnce g_smem_configured[2];  // [0] FP32 kernels, [1] FP64 kernels

template <typename T>
static int configure_smem() {
  const int idx = sizeof(T) == 8 ? 1 : 0;
  return g_smem_configured[idx].run([idx]() -> int {
    const int big = (int)kSmemBudget;
    JG_CUDA(cudaFuncSetAttribute(k_s2g_legendre<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    JG_CUDA(cudaFuncSetAttribute(k_ifft<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    JG_CUDA(cudaFuncSetAttribute(k_fft<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    JG_CUDA(cudaFuncSetAttribute(k_fourier_full<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    JG_CUDA(cudaFuncSetAttribute(k_g2s_legendre<T, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    JG_CUDA(cudaFuncSetAttribute(k_g2s_legendre<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    if (idx == 0) {
      JG_CUDA(cudaFuncSetAttribute(k_fft_rows<64, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
      JG_CUDA(cudaFuncSetAttribute(k_fft_rows<64, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
      JG_CUDA(cudaFuncSetAttribute(k_fft_rows<128, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
      JG_CUDA(cudaFuncSetAttribute(k_fft_rows<128, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
      JG_CUDA(cudaFuncSetAttribute(k_ifft_rows<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
      JG_CUDA(cudaFuncSetAttribute(k_ifft_rows<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, big));
    }
    return JGCM_OK;
  });
}

// column tiles per block; a tuned value (jgcm_model_set_tuning / the autotuner) overrides the default
static inline int s2g_ct(const jgcm_mesh* m) {
  return m->tune[1] > 0 ? m->tune[1] : m->nh >= 256 ? 1 : 256 / m->nh;
}
static inline int g2s_ct(const jgcm_mesh* m) {
  return m->tune[2] > 0 ? m->tune[2] : m->nh >= 64 ? 4 : m->nh >= 32 ? 8 : 16;
}
// columns per FFT block: CT * nlon/4 butterflies per stage = 256 threads by default
static inline int fft_ct(const jgcm_mesh* m) {
  return m->tune[3] > 0 ? m->tune[3] : m->nlon >= 1024 ? 1 : 1024 / m->nlon;
}

// The plans' FP32 copies of their FP64 scalars (pick<T> in the kernels), filled here so that
// every plan builder stays in FP64.
static S2GPlan with_f32(const S2GPlan& p) {
  S2GPlan q = p;
  for (int i = 0; i < q.ng; i++) q.g[i].shiftf = (float)q.g[i].shift;
  return q;
}
static IFFTPlan with_f32(const IFFTPlan& p) {
  IFFTPlan q = p;
  for (int i = 0; i < q.ng; i++) {
    q.g[i].eshift = std::exp(q.g[i].shift);
    q.g[i].shiftf = (float)q.g[i].shift;
    q.g[i].eshiftf = (float)q.g[i].eshift;
  }
  return q;
}
static FFTPlan with_f32(const FFTPlan& p) {
  FFTPlan q = p;
  q.kappa_mf = (float)q.kappa_m;
  q.kappa_tf = (float)q.kappa_t;
  return q;
}
static G2SPlan with_f32(const G2SPlan& p) {
  G2SPlan q = p;
  q.sp.robertf = (float)q.sp.robert;
  q.sp.implicit_coeff = (float)q.sp.implicit_coef;
  q.sp.h0f = (float)q.sp.h0;
  for (int i = 0; i < q.ng; i++) q.g[i].scalef = (float)q.g[i].scale;
  return q;
}

template <typename T>
static int launch_ifft_stage(jgcm_mesh* m, const IFFTPlan& ip, cudaStream_t st, V2<T>* fbuf);

// Legendre synthesis then inverse FFT, with the Fourier coefficients staged in `fbuf`
// ((N+1) x nlat x C complex T).
template <typename T>
static int launch_s2g_into(jgcm_mesh* m, const S2GPlan& sp0, const IFFTPlan& ip, cudaStream_t st, V2<T>* fbuf) {
  using V = V2<T>;
  const S2GPlan sp = with_f32(sp0);
  JG_TRY(configure_smem<T>());
  Tables<T> tb = tables<T>(m);
  const int nh = m->nh, ct = s2g_ct(m);
  if (std::is_same<T, float>::value && m->tc.on && !m->simt_legendre) {
    JG_TRY(launch_s2g_legendre_tc(m, sp, fbuf, st));
  } else {
    size_t sm1 = align16((size_t)(m->ns + 1) * nh * sizeof(T)) + (size_t)(m->ns + 1) * ct * sizeof(V);
    dim3 g1((sp.C + ct - 1) / ct, m->N + 1);
    JG_CUDA(launch_pdl(k_s2g_legendre<T>, g1, 256, sm1, st, sp, tb, fbuf, m->ns, m->nlat, ct));
    mark(st);
    JG_CUDA(cudaGetLastError());
  }
  return launch_ifft_stage<T>(m, ip, st, fbuf);
}

// The inverse FFT stage alone (Fourier coefficients already in `fbuf`).
template <typename T>
static int launch_ifft_stage(jgcm_mesh* m, const IFFTPlan& ip0, cudaStream_t st, V2<T>* fbuf) {
  using V = V2<T>;
  const IFFTPlan ip = with_f32(ip0);
  Tables<T> tb = tables<T>(m);
  const int fc = fft_ct(m);
  if (std::is_same<T, float>::value && use_row_fft(m, ip.C, true)) {  // many rows: a row per thread
    dim3 gr((ip.C + 32 * RF_WARPS - 1) / (32 * RF_WARPS), m->nlat);
    const Tables<float> tf = tables<float>(m);
    const float2* Ff = (const float2*)fbuf;
    if (m->nlon == 64)
      JG_CUDA(launch_pdl(k_ifft_rows<64>, gr, 32 * RF_WARPS, row_fft_smem(m), st, ip, tf, row_twiddles<64>(m), Ff, m->N, m->nlat));
    else
      JG_CUDA(launch_pdl(k_ifft_rows<128>, gr, 32 * RF_WARPS, row_fft_smem(m), st, ip, tf, row_twiddles<128>(m), Ff, m->N, m->nlat));
    mark(st);
    JG_CUDA(cudaGetLastError());
    return JGCM_OK;
  }
  // the warp-register FFT wins in FP32; in FP64 the shared-memory radix-2 kernel is faster (measured)
  if (std::is_same<T, float>::value && m->nlon >= 64 && m->nlon <= 1024 && m->tune[3] == 0) {
    const size_t smw = (size_t)(m->N + 1) * FW_COLS * sizeof(V);
    dim3 gw((ip.C + FW_COLS - 1) / FW_COLS, m->nlat);
    switch (m->nlon) {
      case 64: JG_CUDA(launch_pdl(k_ifft_w<T, 1>, gw, 256, smw, st, ip, tb, (const V*)fbuf, m->N, m->nlat, m->nlon)); break;
      case 128: JG_CUDA(launch_pdl(k_ifft_w<T, 2>, gw, 256, smw, st, ip, tb, (const V*)fbuf, m->N, m->nlat, m->nlon)); break;
      case 256: JG_CUDA(launch_pdl(k_ifft_w<T, 4>, gw, 256, smw, st, ip, tb, (const V*)fbuf, m->N, m->nlat, m->nlon)); break;
      case 512: JG_CUDA(launch_pdl(k_ifft_w<T, 8>, gw, 256, smw, st, ip, tb, (const V*)fbuf, m->N, m->nlat, m->nlon)); break;
      default: JG_CUDA(launch_pdl(k_ifft_w<T, 16>, gw, 256, smw, st, ip, tb, (const V*)fbuf, m->N, m->nlat, m->nlon)); break;
    }
    mark(st);
    JG_CUDA(cudaGetLastError());
    return JGCM_OK;
  }
  size_t sm2 = align16((size_t)(fc * m->nlon + m->nlon) * sizeof(T)) + (size_t)(m->N + 1) * fc * sizeof(V);
  dim3 g2((ip.C + fc - 1) / fc, m->nlat);
  JG_CUDA(launch_pdl(k_ifft<T>, g2, 256, sm2, st, ip, tb, (const V*)fbuf, m->N, m->nlat, m->nlon, m->logn - 1, fc));
  mark(st);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}

template <typename T>
int launch_s2g(jgcm_mesh* m, const S2GPlan& sp, const IFFTPlan& ip, cudaStream_t st, void* fbuf, int cap) {
  if (!fbuf) {
    fbuf = m->d_fbuf;
    cap = m->Cmax;
  }
  JG_ARG(sp.C == ip.C && sp.C <= cap && sp.C > 0, "bad S2G plan");
  return launch_s2g_into<T>(m, sp, ip, st, (V2<T>*)fbuf);
}

template <typename T>
int launch_ifft_only(jgcm_mesh* m, const IFFTPlan& ip, cudaStream_t st, void* fbuf, int cap) {
  JG_TRY(configure_smem<T>());
  if (!fbuf) {
    fbuf = m->d_fbuf;
    cap = m->Cmax;
  }
  JG_ARG(ip.C <= cap && ip.C > 0, "bad inverse FFT plan");
  return launch_ifft_stage<T>(m, ip, st, (V2<T>*)fbuf);
}

template <typename T>
int launch_fft_only(jgcm_mesh* m, const FFTPlan& fp0, cudaStream_t st, void* fbuf, int cap) {
  using V = V2<T>;
  const FFTPlan fp = with_f32(fp0);
  JG_TRY(configure_smem<T>());
  if (!fbuf) {
    fbuf = m->d_fbuf;
    cap = m->Cmax;
  }
  JG_ARG(fp.C <= cap && fp.C > 0, "bad FFT plan");
  Tables<T> tb = tables<T>(m);
  const int fc = fft_ct(m);
  if (std::is_same<T, float>::value && use_row_fft(m, fp.C)) {  // many rows: a row per thread
    dim3 gr((fp.C + 32 * RF_WARPS - 1) / (32 * RF_WARPS), m->nlat);
    const Tables<float> tf = tables<float>(m);
    float2* Ff = (float2*)fbuf;
    bool plain = true;
    for (int i = 0; i < fp.ng; i++) plain = plain && fp.g[i].pro == PRO_NONE;
    const size_t sm = row_fft_smem(m);
    if (m->nlon == 64 && plain)
      JG_CUDA(launch_pdl(k_fft_rows<64, true>, gr, 32 * RF_WARPS, sm, st, fp, tf, row_twiddles<64>(m), Ff, m->N, m->nlat));
    else if (m->nlon == 64)
      JG_CUDA(launch_pdl(k_fft_rows<64, false>, gr, 32 * RF_WARPS, sm, st, fp, tf, row_twiddles<64>(m), Ff, m->N, m->nlat));
    else if (plain)
      JG_CUDA(launch_pdl(k_fft_rows<128, true>, gr, 32 * RF_WARPS, sm, st, fp, tf, row_twiddles<128>(m), Ff, m->N, m->nlat));
    else
      JG_CUDA(launch_pdl(k_fft_rows<128, false>, gr, 32 * RF_WARPS, sm, st, fp, tf, row_twiddles<128>(m), Ff, m->N, m->nlat));
    mark(st);
    JG_CUDA(cudaGetLastError());
    return JGCM_OK;
  }
  // forward: the warp-register FFT wins in FP32 from nlon = 128 on (measured)
  if (std::is_same<T, float>::value && m->nlon >= 128 && m->nlon <= 1024 && m->tune[3] == 0) {
    const size_t smw = ((size_t)FW_COLS * (m->nlon / 2) + (size_t)(m->N + 1) * FW_COLS) * sizeof(V);
    dim3 gw((fp.C + FW_COLS - 1) / FW_COLS, m->nlat);
    bool plain = true;
    for (int i = 0; i < fp.ng; i++) plain = plain && fp.g[i].pro == PRO_NONE;
#define JG_FFT_W(VV)                                                                                               \
  (plain ? launch_pdl(k_fft_w<T, VV, true>, gw, 256, smw, st, fp, tb, (V*)fbuf, m->N, m->nlat, m->nlon)            \
         : launch_pdl(k_fft_w<T, VV, false>, gw, 256, smw, st, fp, tb, (V*)fbuf, m->N, m->nlat, m->nlon))
    switch (m->nlon) {
      case 64: JG_CUDA(JG_FFT_W(1)); break;
      case 128: JG_CUDA(JG_FFT_W(2)); break;
      case 256: JG_CUDA(JG_FFT_W(4)); break;
      case 512: JG_CUDA(JG_FFT_W(8)); break;
      default: JG_CUDA(JG_FFT_W(16)); break;
    }
#undef JG_FFT_W
    mark(st);
    JG_CUDA(cudaGetLastError());
    return JGCM_OK;
  }
  size_t sm = (size_t)(fc * m->nlon + m->nlon) * sizeof(T);
  dim3 g((fp.C + fc - 1) / fc, m->nlat);
  JG_CUDA(launch_pdl(k_fft<T>, g, 256, sm, st, fp, tb, (V*)fbuf, m->N, m->nlat, m->nlon, m->logn - 1, fc));
  mark(st);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}

template <typename T>
int launch_g2s(jgcm_mesh* m, const FFTPlan& fp, const G2SPlan& gp0, cudaStream_t st, void* fbuf, int cap) {
  using V = V2<T>;
  const G2SPlan gp = with_f32(gp0);
  if (!fbuf) {
    fbuf = m->d_fbuf;
    cap = m->Cmax;
  }
  JG_TRY(launch_fft_only<T>(m, fp, st, fbuf, cap));
  bool adj = false;
  for (int i = 0; i < gp.ng; i++) adj = adj || gp.g[i].op == G2S_ADJ_S2G;
  if (std::is_same<T, float>::value && m->tc.on && !adj && !m->simt_legendre)
    return launch_g2s_legendre_tc(m, gp, fp.C, st, fbuf);
  Tables<T> tb = tables<T>(m);
  const int nh = m->nh, ct = g2s_ct(m);
  size_t sm = (size_t)8 * ct * nh * sizeof(V);
  const size_t tab = (size_t)3 * (m->ns + 1) * nh * sizeof(T);
  const int stage = sm + tab <= kSmemBudget;
  if (stage) sm += tab;
  dim3 g((gp.C + ct - 1) / ct, m->N + 1);
  // one lane per output once the launch has outputs for every thread the device holds
  const size_t outputs = (size_t)gp.C * (m->N + 1) * (m->N + 2) / 2;
  if (outputs >= (size_t)m->sm_count * 2048 && nh % 4 == 0)
    JG_CUDA(launch_pdl(k_g2s_legendre<T, 1>, g, 256, sm, st, gp, tb, (const V*)fbuf, m->ns, m->nlat, fp.C, ct, stage));
  else
    JG_CUDA(launch_pdl(k_g2s_legendre<T, 4>, g, 256, sm, st, gp, tb, (const V*)fbuf, m->ns, m->nlat, fp.C, ct, stage));
  mark(st);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}

template int launch_s2g<float>(jgcm_mesh*, const S2GPlan&, const IFFTPlan&, cudaStream_t, void*, int);
template int launch_s2g<double>(jgcm_mesh*, const S2GPlan&, const IFFTPlan&, cudaStream_t, void*, int);
template int launch_g2s<float>(jgcm_mesh*, const FFTPlan&, const G2SPlan&, cudaStream_t, void*, int);
template int launch_g2s<double>(jgcm_mesh*, const FFTPlan&, const G2SPlan&, cudaStream_t, void*, int);
template int launch_ifft_only<float>(jgcm_mesh*, const IFFTPlan&, cudaStream_t, void*, int);
template int launch_ifft_only<double>(jgcm_mesh*, const IFFTPlan&, cudaStream_t, void*, int);
template int launch_fft_only<float>(jgcm_mesh*, const FFTPlan&, cudaStream_t, void*, int);
template int launch_fft_only<double>(jgcm_mesh*, const FFTPlan&, cudaStream_t, void*, int);

// ------------------------------------------------------------------------------------------
// Layout / precision conversion between the reference host layout (FP64) and device layout.
template <typename T>
__global__ void k_spec_h2d(const double* __restrict__ src, V2<T>* __restrict__ dst, int N, int ns, int L) {
  size_t total = (size_t)(N + 1) * (ns + 1) * L;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    int k = (int)(t % L);
    size_t mn = t / L;
    int n = (int)(mn % (ns + 1)), m = (int)(mn / (ns + 1));
    size_t h = 2 * ((size_t)m + (size_t)(N + 1) * ((size_t)n + (size_t)(ns + 1) * k));
    V2<T> v;
    v.x = (n >= m) ? (T)src[h] : (T)0;
    v.y = (n >= m) ? (T)src[h + 1] : (T)0;
    dst[t] = v;
  }
}
template <typename T>
__global__ void k_spec_d2h(const V2<T>* __restrict__ src, double* __restrict__ dst, int N, int ns, int L) {
  size_t total = (size_t)(N + 1) * (ns + 1) * L;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    int m = (int)(t % (N + 1));
    size_t r = t / (N + 1);
    int n = (int)(r % (ns + 1)), k = (int)(r / (ns + 1));
    V2<T> v = src[((size_t)m * (ns + 1) + n) * L + k];
    dst[2 * t] = (double)v.x;
    dst[2 * t + 1] = (double)v.y;
  }
}
template <typename A, typename B>
__global__ void k_cast(const A* __restrict__ src, B* __restrict__ dst, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    dst[t] = (B)src[t];
}
// Fourier buffer [m][j][c] -> host [c][j][m] (modes 0..N)
template <typename T>
__global__ void k_fourier_d2h(const V2<T>* __restrict__ F, double* __restrict__ dst, int N, int nlat, int L) {
  size_t total = (size_t)(N + 1) * nlat * L;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    int m = (int)(t % (N + 1));
    size_t r = t / (N + 1);
    int j = (int)(r % nlat), k = (int)(r / nlat);
    V2<T> v = F[((size_t)m * nlat + j) * L + k];
    dst[2 * t] = (double)v.x;
    dst[2 * t + 1] = (double)v.y;
  }
}

static inline int nblk(size_t n) {
  size_t b = (n + 255) / 256;
  return (int)(b > 1184 ? 1184 : (b < 1 ? 1 : b));
}

int spec_host_to_dev(jgcm_mesh* m, const double* src, void* dst, int L, cudaStream_t st) {
  size_t n = spec_elems(m, L);
  if (is_fp64(m))
    k_spec_h2d<double><<<nblk(n), 256, 0, st>>>(src, (double2*)dst, m->N, m->ns, L);
  else
    k_spec_h2d<float><<<nblk(n), 256, 0, st>>>(src, (float2*)dst, m->N, m->ns, L);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}
int spec_dev_to_host(jgcm_mesh* m, const void* src, double* dst, int L, cudaStream_t st) {
  size_t n = spec_elems(m, L);
  if (is_fp64(m))
    k_spec_d2h<double><<<nblk(n), 256, 0, st>>>((const double2*)src, dst, m->N, m->ns, L);
  else
    k_spec_d2h<float><<<nblk(n), 256, 0, st>>>((const float2*)src, dst, m->N, m->ns, L);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}
int grid_host_to_dev(jgcm_mesh* m, const double* src, void* dst, size_t n, cudaStream_t st) {
  if (is_fp64(m))
    JG_CUDA(cudaMemcpyAsync(dst, src, n * 8, cudaMemcpyDeviceToDevice, st));
  else
    k_cast<double, float><<<nblk(n), 256, 0, st>>>(src, (float*)dst, n);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}
int grid_dev_to_host(jgcm_mesh* m, const void* src, double* dst, size_t n, cudaStream_t st) {
  if (is_fp64(m))
    JG_CUDA(cudaMemcpyAsync(dst, src, n * 8, cudaMemcpyDeviceToDevice, st));
  else
    k_cast<float, double><<<nblk(n), 256, 0, st>>>((const float*)src, dst, n);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}
int fourier_dev_to_host(jgcm_mesh* m, int L, double* dst, cudaStream_t st) {
  size_t n = (size_t)(m->N + 1) * m->nlat * L;
  if (is_fp64(m))
    k_fourier_d2h<double><<<nblk(n), 256, 0, st>>>((const double2*)m->d_fbuf, dst, m->N, m->nlat, L);
  else
    k_fourier_d2h<float><<<nblk(n), 256, 0, st>>>((const float2*)m->d_fbuf, dst, m->N, m->nlat, L);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}

// Trans_Grid_To_Fourier!: every mode of fft/nλ of the L device grid levels at d_grid, FP64 host layout.
int fourier_full_to_host(jgcm_mesh* m, const void* d_grid, int L, double* d_dst, cudaStream_t st) {
  const int fc = fft_ct(m);
  const size_t sm = (size_t)(fc * m->nlon + m->nlon) * tsize(m);
  JG_ARG(sm <= kSmemBudget, "FFT tile needs %zu bytes of shared memory", sm);
  dim3 g((L + fc - 1) / fc, m->nlat);
  if (is_fp64(m)) {
    JG_TRY(configure_smem<double>());
    k_fourier_full<double><<<g, 256, sm, st>>>((const double*)d_grid, tables<double>(m), d_dst, L, m->nlat,
                                               m->nlon, m->logn - 1, fc);
  } else {
    JG_TRY(configure_smem<float>());
    k_fourier_full<float><<<g, 256, sm, st>>>((const float*)d_grid, tables<float>(m), d_dst, L, m->nlat, m->nlon,
                                              m->logn - 1, fc);
  }
  mark(st);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}

template <typename T>
__global__ void k_laplacian(V2<T>* s, const T* eig, int N, int ns, int L) {
  size_t total = (size_t)(N + 1) * (ns + 1) * L;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    T e = eig[t / L];
    V2<T> v = s[t];
    v.x = e * v.x;
    v.y = e * v.y;
    s[t] = v;
  }
}
int apply_laplacian(jgcm_mesh* m, void* d_spec, int L, cudaStream_t st) {
  size_t n = spec_elems(m, L);
  if (is_fp64(m))
    k_laplacian<double><<<nblk(n), 256, 0, st>>>((double2*)d_spec, m->t64.eig, m->N, m->ns, L);
  else
    k_laplacian<float><<<nblk(n), 256, 0, st>>>((float2*)d_spec, m->t32.eig, m->N, m->ns, L);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}

// Area_Weighted_Global_Mean (Spectral_Spherical_Mesh.jl:746-760): one block, FP64, fixed order.
template <typename T>
__global__ void k_area_mean(const T* __restrict__ g, const double* __restrict__ w, int nlat, int nlon, double* out) {
  __shared__ double red[256];
  double acc = 0.0;
  for (int i = threadIdx.x; i < nlon; i += blockDim.x) {
    double r = 0.0;
    for (int j = 0; j < nlat; j++) r += (double)g[(size_t)j * nlon + i] * w[j];
    acc += r;
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0] / (2.0 * nlon);
}
int area_mean(jgcm_mesh* m, const void* d_grid, double* d_out, cudaStream_t st) {
  if (is_fp64(m))
    k_area_mean<double><<<1, 256, 0, st>>>((const double*)d_grid, m->d_wts, m->nlat, m->nlon, d_out);
  else
    k_area_mean<float><<<1, 256, 0, st>>>((const float*)d_grid, m->d_wts, m->nlat, m->nlon, d_out);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}

}  // namespace jgcm

// ------------------------------------------------------------------------------------------
// Allocation-free spectral -> grid transform (jgcm_trans_spherical_to_grid_noalloc).
//
// Some callers cannot allocate device memory at the point where they transform: code that runs
// while a stream is being captured into a CUDA graph, hosts whose device memory is owned by their
// own pool allocator (so a stray cudaMalloc would break their accounting or fail under a memory
// cap), and real-time loops that forbid allocation after start-up.  This variant of
// Trans_Spherical_To_Grid! works on device buffers the caller already owns and stages its Fourier
// coefficients in a fixed-size scratch array that is part of the library image instead of in
// memory obtained at run time.  The array lives on every GPU that loads the library until the
// process exits; every call on a device shares it.
namespace {
constexpr size_t kNoAllocScratchBytes = 8u << 20;  // 8 MiB
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
void* g_noalloc_addr[64];  // device address of g_noalloc_scratch, per CUDA device
std::mutex g_noalloc_mu;

// Once per device, with that device current: resolve the device address of the scratch array
// (the host-side name is only a stand-in for it).
int noalloc_scratch_address(int dev, void** out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr) {
      jgcm::set_error("cudaGetSymbolAddress(g_noalloc_scratch) failed on device %d: %s", dev,
                      cudaGetErrorString(e));
      return JGCM_E_CUDA;
    }
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return JGCM_OK;
}
}  // namespace

extern "C" int jgcm_trans_spherical_to_grid_noalloc(jgcm_mesh* m, const void* d_snm, int nlev, void* d_grid,
                                                    void* stream) {
  using namespace jgcm;
  JG_ARG(m != nullptr && d_snm != nullptr && d_grid != nullptr, "NULL argument");
  JG_ARG(nlev == m->nd || nlev == 1, "third dimension must be nd=%d or 1 (got %d)", m->nd, nlev);
  const size_t need = (size_t)(m->N + 1) * m->nlat * nlev * 2 * tsize(m);
  JG_ARG(need <= kNoAllocScratchBytes,
         "jgcm_trans_spherical_to_grid_noalloc: needs %zu bytes of scratch for (N+1)=%d x nlat=%d x nlev=%d, the "
         "static scratch holds %zu bytes",
         need, m->N + 1, m->nlat, nlev, kNoAllocScratchBytes);
  int dev = -1;
  JG_CUDA(cudaGetDevice(&dev));
  JG_ARG(dev == m->device, "the mesh lives on device %d but device %d is current", m->device, dev);
  JG_ARG(dev >= 0 && dev < 64, "device index %d out of range", dev);
  void* scratch = nullptr;
  JG_TRY(noalloc_scratch_address(dev, &scratch));
  cudaStream_t st = stream ? (cudaStream_t)stream : m->stream;
  S2GPlan sp;
  memset(&sp, 0, sizeof(sp));
  sp.ng = 1;
  sp.C = nlev;
  sp.g[0].op = S2G_PLAIN;
  sp.g[0].a = d_snm;
  sp.g[0].L = nlev;
  IFFTPlan ip;
  memset(&ip, 0, sizeof(ip));
  ip.ng = 1;
  ip.C = nlev;
  ip.g[0].epi = EPI_NONE;
  ip.g[0].dst = d_grid;
  ip.g[0].L = nlev;
  // The synthesis writes every scratch element (all m <= N, all latitudes, all columns) before
  // the inverse FFT reads it, so nothing left by an earlier call needs clearing.
  return is_fp64(m) ? launch_s2g_into<double>(m, sp, ip, st, (double2*)scratch)
                    : launch_s2g_into<float>(m, sp, ip, st, (float2*)scratch);
}

namespace jgcm {
// shared memory of the SIMT transform kernels with tiles (s2g, g2s, fft); 0 = the mesh's current
size_t simt_smem_need(const jgcm_mesh* m, int s2g, int g2s, int fft) {
  const size_t ts = tsize(m), nh = m->nh, ns1 = m->ns + 1, nlon = m->nlon;
  const size_t a = align16(ns1 * nh * ts) + ns1 * (size_t)s2g * 2 * ts;
  const size_t b = 8 * (size_t)g2s * nh * 2 * ts;
  const size_t c = align16(((size_t)fft * nlon + nlon) * ts) + (size_t)(m->N + 1) * fft * 2 * ts;
  return std::max(a, std::max(b, c));
}
}  // namespace jgcm

