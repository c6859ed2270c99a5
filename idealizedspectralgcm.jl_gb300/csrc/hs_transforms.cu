// hs_transforms.cu -- the Held-Suarez step's Legendre analysis as one contraction per
// (zonal-wavenumber pair, level group, member).
//
// The general analysis kernel (k_g2s_legendre, transforms.cu) treats every output column on its
// own: a column tile per block, a group lookup and an input slot per column, the quadrature weights
// re-read for every column.  The Held-Suarez step always analyses the same four fields per level
// (δu cos, δv cos, the energy and δT, plus δ ln ps per member) into the same three outputs per level
// (the vorticity and divergence tendencies of the alpha operator, Vor_Div_From_Grid_UV! and
// Compute_Alpha_Operator!, Spectral_Spherical_Mesh.jl:349-459, with ∇² of the energy taken off the
// divergence, Spectral_Dynamics.jl:286-296, and the temperature tendency; Trans_Grid_To_Spherical!
// :221-293 for δ ln ps).  Here one thread owns one (m, n, level) and forms all of its outputs from
// the same weight rows (P w, the alpha operator's two rows) and the same folded inputs, so each
// weight load serves 12 multiply-adds instead of 2.  Blocks take the zonal wavenumbers in pairs
// (m, N - m), whose output counts K_m + K_{N-m} = N + 4 are the same for every pair, so the blocks
// carry equal work.  Sums run over the folded latitudes in order, four weights per load, as in the
// general kernel's one-lane form.
#include <algorithm>
#include <atomic>
#include <mutex>
#include <type_traits>

#include "jgcm_internal.cuh"
#include "transform_ops.cuh"

namespace jgcm {

namespace {

// one 16-byte load of four consecutive table weights (16-byte aligned rows)
__device__ __forceinline__ void ld4w(const float* p, float (&w)[4]) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  w[0] = v.x; w[1] = v.y; w[2] = v.z; w[3] = v.w;
}
__device__ __forceinline__ void ld4w(const double* p, double (&w)[4]) {
  const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
  w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y;
}

template <typename T>
struct HSAnaArgs {
  const V2<T>* F;                       // Fourier buffer [m][j][Cin]
  V2<T> *dvor, *ddiv, *dt, *dlnps;      // outputs, MNK: [m][n][L] (dlnps: [m][n][E])
  int Cin;                              // columns of the Fourier buffer
  int colU, colV, colE, colT, colP;     // base columns of δu cos, δv cos, energy, δT (L each), δ ln ps (E)
  int nd, L, E, N, ns, nlat, nh;
  int LG;                               // levels per block (the level nd of a member is δ ln ps)
};

// row pitch of the staged weight tables: one 16-byte pad per row, so that the rows read by the
// threads of a warp start in different shared-memory banks
template <typename T>
__host__ __device__ constexpr int wpitch(int nh) {
  return nh + 16 / (int)sizeof(T);
}

// grid (N/2 + 1 pairs, ceil((nd + 1) / LG) level groups, members), blockDim >= rows * LG with rows the
// largest per-pair thread count (N + 4 for NP = 1)
template <typename T, int NP>
__global__ void __launch_bounds__(256) k_hs_analysis(HSAnaArgs<T> a, Tables<T> tb) {
  using V = V2<T>;
  extern __shared__ __align__(16) unsigned char smem[];
  const int N = a.N, ns = a.ns, nh = a.nh, LG = a.LG, nd = a.nd, nlat = a.nlat;
  const int m1 = blockIdx.x, m2 = N - m1, g = blockIdx.y, e = blockIdx.z;
  const int nm = m2 != m1 ? 2 : 1;
  const int K1 = ns + 1 - m1, K2 = nm == 2 ? ns + 1 - m2 : 0;
  const int wp = wpitch<T>(nh);
  // weights: slot s (m1, m2) holds [3][K_s][wp]: P w, the alpha operator's i-term and its B-term
  T* W = (T*)smem;
  const size_t wsz = (size_t)3 * (K1 + K2) * wp;
  // folded inputs [f][jh][parity][slot][level]: the lanes of a warp that read one latitude of one
  // field read neighbouring words
  V* X = (V*)(smem + ((wsz * sizeof(T) + 15) & ~(size_t)15));
  // 1. the weight rows n = m..ns of both m (constants): asynchronous 16-byte copies, issued before
  //    the dependency wait and waited for once.  A row is nh * sizeof(T) / 16 chunks (a power of
  //    two): a warp pass copies 32 / chunks rows, or one row in passes of 32 chunks.
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  {
    constexpr int ce = 16 / (int)sizeof(T);  // weights per chunk
    const int nchunk = nh / ce, rpi = nchunk >= 32 ? 1 : 32 / nchunk;
    const int rsub = nchunk >= 32 ? 0 : lane / nchunk, c0 = nchunk >= 32 ? lane : lane - rsub * nchunk;
    for (int s = 0; s < nm; s++) {
      const int m = s ? m2 : m1, K = s ? K2 : K1;
      const size_t src = ((size_t)m * (ns + 1) + m) * nh;
      T* dst = W + (s ? (size_t)3 * K1 * wp : 0);
#pragma unroll
      for (int tbl = 0; tbl < 3; tbl++) {
        const T* from = (tbl == 0 ? tb.PW : tbl == 1 ? tb.CA : tb.CB) + src;
        T* to = dst + (size_t)tbl * K * wp;
        for (int r = warp * rpi + rsub; r < K; r += nw * rpi)
          for (int c = c0; c < nchunk; c += 32) cp_async16(to + (size_t)r * wp + c * ce, from + (size_t)r * nh + c * ce);
      }
    }
    cp_async_commit();
  }
  pdl_wait();  // programmatic dependent launch: the forward FFT's coefficients are complete
  // 2. hemisphere folds of the block's input columns: thread (l, jh) loads its latitude pair of all
  //    fields of both m first (up to 16 loads in flight), then folds them; consecutive threads take
  //    consecutive levels, i.e. neighbouring columns of the Fourier buffer
  for (int item = threadIdx.x; item < LG * nh; item += blockDim.x) {
    const int jh = item / LG, l = item - jh * LG, lv = g * LG + l;
    V x[2][4], y[2][4];
#pragma unroll
    for (int s = 0; s < 2; s++)
#pragma unroll
      for (int f = 0; f < 4; f++) {
        x[s][f].x = x[s][f].y = y[s][f].x = y[s][f].y = 0;
        int col = -1;
        if (lv < nd)
          col = (f == 0 ? a.colU : f == 1 ? a.colV : f == 2 ? a.colE : a.colT) + e * nd + lv;
        else if (lv == nd && f == 3)
          col = a.colP + e;
        if (s < nm && col >= 0) {
          const int m = s ? m2 : m1;
          x[s][f] = a.F[((size_t)m * nlat + jh) * a.Cin + col];
          y[s][f] = a.F[((size_t)m * nlat + (nlat - 1 - jh)) * a.Cin + col];
        }
      }
#pragma unroll
    for (int s = 0; s < 2; s++)
#pragma unroll
      for (int f = 0; f < 4; f++) {
        if (s >= nm) continue;
        V sv, av;
        sv.x = x[s][f].x + y[s][f].x;
        sv.y = x[s][f].y + y[s][f].y;
        av.x = x[s][f].x - y[s][f].x;
        av.y = x[s][f].y - y[s][f].y;
        const size_t base = ((size_t)(f * nh + jh) * 2) * nm * LG + (size_t)s * LG + l;
        X[base] = sv;
        X[base + (size_t)nm * LG] = av;
      }
  }
  cp_async_wait_all();
  __syncthreads();
  // 3. one thread per (m, level) and NP total wavenumbers of one parity, n and n + 2 (NP = 2:
  //    each folded input loaded from shared memory serves both; rows r = 4 i + b, b < 2)
  int q = threadIdx.x / LG;
  const int l = threadIdx.x - q * LG;
  const int Q1 = NP == 1 ? K1 : 2 * ((K1 + 3) / 4), Q2 = nm == 2 ? (NP == 1 ? K2 : 2 * ((K2 + 3) / 4)) : 0;
  if (q >= Q1 + Q2) return;
  const int s = q < Q1 ? 0 : 1;
  if (s) q -= Q1;
  const int m = s ? m2 : m1, K = s ? K2 : K1;
  const int r0 = NP == 1 ? q : 4 * (q >> 1) + (q & 1);
  if (r0 >= K) return;
  const int lv = g * LG + l;
  if (lv > nd) return;
  const bool even = (r0 & 1) == 0;  // P_n^m is symmetric about the equator for n - m even
  const T* wbase = W + (s ? (size_t)3 * K1 * wp : 0);
  const T* pw[NP];
  const T* ca[NP];
  const T* cb[NP];
  bool live[NP];
#pragma unroll
  for (int u = 0; u < NP; u++) {
    const int r = r0 + 2 * u;
    live[u] = r < K;
    const int rr = live[u] ? r : r0;  // a row past K reads row r0's weights and is not stored
    pw[u] = wbase + (size_t)rr * wp;
    ca[u] = wbase + ((size_t)K + rr) * wp;
    cb[u] = wbase + ((size_t)2 * K + rr) * wp;
  }
  // element (f, jh, parity) of this thread's column: X[((f nh + jh) 2 + par) nm LG + s LG + l]
  const size_t pstride = (size_t)nm * LG, jstride = 2 * pstride, fstride = (size_t)nh * jstride;
  const V* xcol = X + (size_t)s * LG + l;
  const size_t same = even ? 0 : pstride, other = even ? pstride : 0;
  const size_t mrow = (size_t)m * (ns + 1);
  if (lv == nd) {  // δ ln ps of member e: plain analysis
    const V* src = xcol + 3 * fstride + same;
    T sr[NP], si[NP];
#pragma unroll
    for (int u = 0; u < NP; u++) sr[u] = si[u] = 0;
    for (int jh = 0; jh < nh; jh += 4) {
      T w[NP][4];
#pragma unroll
      for (int u = 0; u < NP; u++) ld4w(pw[u] + jh, w[u]);
#pragma unroll
      for (int v = 0; v < 4; v++) {
        const V x = src[(size_t)(jh + v) * jstride];
#pragma unroll
        for (int u = 0; u < NP; u++) {
          sr[u] += x.x * w[u][v];
          si[u] += x.y * w[u][v];
        }
      }
    }
#pragma unroll
    for (int u = 0; u < NP; u++) {
      const int n = m + r0 + 2 * u;
      if (!live[u]) continue;
      V o;
      o.x = n == ns ? (T)0 : sr[u] * (T)0.5;
      o.y = n == ns ? (T)0 : si[u] * (T)0.5;
      a.dlnps[(mrow + n) * a.E + e] = o;
    }
    return;
  }
  const V* us = xcol + same;                 // δu cos, parity of n - m
  const V* uo = xcol + other;                // δu cos, the other parity
  const V* vs = xcol + fstride + same;       // δv cos
  const V* vo = xcol + fstride + other;
  const V* es = xcol + 2 * fstride + same;   // energy
  const V* ts = xcol + 3 * fstride + same;   // δT
  // vorticity: alpha operator of (A = δv cos, B = δu cos), i Σ CA A - Σ CB B
  // divergence: alpha operator of (A = δu cos, B = δv cos), i Σ CA A + Σ CB B, less ∇² of the energy
  T var[NP], vai[NP], vbr[NP], vbi[NP], dar[NP], dai[NP], dbr[NP], dbi[NP], er[NP], ei[NP], tr[NP], ti[NP];
#pragma unroll
  for (int u = 0; u < NP; u++)
    var[u] = vai[u] = vbr[u] = vbi[u] = dar[u] = dai[u] = dbr[u] = dbi[u] = er[u] = ei[u] = tr[u] = ti[u] = 0;
  for (int jh = 0; jh < nh; jh += 4) {
    T wP[NP][4], wA[NP][4], wB[NP][4];
#pragma unroll
    for (int u = 0; u < NP; u++) {
      ld4w(pw[u] + jh, wP[u]);
      ld4w(ca[u] + jh, wA[u]);
      ld4w(cb[u] + jh, wB[u]);
    }
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const size_t o = (size_t)(jh + v) * jstride;
      const V xu = us[o], yv = vo[o], xv = vs[o], yu = uo[o], xe = es[o], xt = ts[o];
#pragma unroll
      for (int u = 0; u < NP; u++) {
        var[u] += (-xv.y) * wA[u][v];
        vai[u] += xv.x * wA[u][v];
        vbr[u] += yu.x * wB[u][v];
        vbi[u] += yu.y * wB[u][v];
        dar[u] += (-xu.y) * wA[u][v];
        dai[u] += xu.x * wA[u][v];
        dbr[u] += yv.x * wB[u][v];
        dbi[u] += yv.y * wB[u][v];
        er[u] += xe.x * wP[u][v];
        ei[u] += xe.y * wP[u][v];
        tr[u] += xt.x * wP[u][v];
        ti[u] += xt.y * wP[u][v];
      }
    }
  }
#pragma unroll
  for (int u = 0; u < NP; u++) {
    if (!live[u]) continue;
    const int n = m + r0 + 2 * u;
    V ov, od, ot;
    if (n == ns) {  // row N+1 of the analysis is zero (Trans_Grid_To_Spherical!, :288-291)
      ov.x = ov.y = od.x = od.y = ot.x = ot.y = 0;
    } else {
      const T eig = tb.eig[mrow + n];
      ov.x = var[u] + (T)-1 * vbr[u];
      ov.y = vai[u] + (T)-1 * vbi[u];
      od.x = dar[u] + dbr[u];
      od.y = dai[u] + dbi[u];
      od.x = od.x - eig * (er[u] * (T)0.5);
      od.y = od.y - eig * (ei[u] * (T)0.5);
      ot.x = tr[u] * (T)0.5;
      ot.y = ti[u] * (T)0.5;
    }
    const size_t sidx = (mrow + n) * a.L + (size_t)e * nd + lv;
    a.dvor[sidx] = ov;
    a.ddiv[sidx] = od;
    a.dt[sidx] = ot;
  }
}

template <typename T>
size_t hs_analysis_smem(const jgcm_mesh* m, int LG) {
  const int N = m->N, nh = m->nh;
  const size_t w = (size_t)3 * (N + 4) * wpitch<T>(nh) * sizeof(T);
  return ((w + 15) & ~(size_t)15) + (size_t)4 * nh * 2 * 2 * LG * sizeof(V2<T>);
}

PerDeviceOnce g_hs_ana_smem[2];

}  // namespace

// total wavenumbers per thread: two of one parity for member ensembles (each folded input loaded
// from shared memory serves both: the analysis is shared-memory-bound at that scale), one otherwise
// (shorter chains for the latency-bound single member)
static int hs_analysis_np(int E) { return E >= 4 ? 2 : 1; }

// threads per level of a block: the largest row count of an m pair (rows r = 4 i + b, b < 2, for
// two rows per thread)
static int hs_analysis_rows(const jgcm_mesh* m, int np) {
  if (np == 1) return m->N + 4;
  int q = 0;
  for (int m1 = 0; m1 <= m->N / 2; m1++) {
    const int m2 = m->N - m1, K1 = m->ns + 1 - m1, K2 = m2 != m1 ? m->ns + 1 - m2 : 0;
    q = std::max(q, 2 * ((K1 + 3) / 4) + 2 * ((K2 + 3) / 4));
  }
  return q;
}

// levels per block of the Held-Suarez analysis: the tuned value when set (clamped to what a block
// of 256 threads holds), else as many as a block holds (HS T42L20, one member: 5 levels 5.5 us,
// 2 levels 7.1 us, 1 level 7.6 us per step in a captured graph)
int hs_analysis_levels(const jgcm_mesh* m, int nd, int E) {
  (void)nd;
  const int lg_max = 256 / hs_analysis_rows(m, hs_analysis_np(E));
  if (lg_max < 1) return 0;
  if (m->hs_levels > 0) return std::min(m->hs_levels, lg_max);
  return lg_max;
}

// The Held-Suarez analysis kernel serves this mesh: not tuned away (levels per block -1), SIMT
// Legendre path, weights in 16-byte rows, shared memory within the budget.
bool hs_analysis_fits(const jgcm_mesh* m, int nd, int E) {
  if (m->hs_levels < 0) return false;  // tuned to the general analysis kernel
  if (m->tc.on && !m->simt_legendre) return false;
  // weight rows of a power-of-two nh/4 16-byte chunks (at most 32: one warp pass per row or more)
  if (m->nh < 4 || m->nh > 128 || (m->nh & (m->nh - 1)) != 0) return false;
  const int LG = hs_analysis_levels(m, nd, E);
  if (LG < 1) return false;
  const size_t sm = is_fp64(m) ? hs_analysis_smem<double>(m, LG) : hs_analysis_smem<float>(m, LG);
  return sm <= kSmemBudget;
}

// Forward FFT of the step's tendency groups (the FFT plan's columns: δu cos, δv cos, δT, energy
// at colU, colV, colT, colE with L columns each, δ ln ps at colP with E), then the analysis.
template <typename T>
int launch_hs_analysis(jgcm_mesh* m, const FFTPlan& fp, int colU, int colV, int colE, int colT, int colP, int nd,
                       int E, void* dvor, void* ddiv, void* dt, void* dlnps, cudaStream_t st, void* fbuf, int cap) {
  JG_ARG(hs_analysis_fits(m, nd, E), "the Held-Suarez analysis kernel does not fit this mesh");
  JG_TRY(launch_fft_only<T>(m, fp, st, fbuf, cap));
  const int LG = hs_analysis_levels(m, nd, E);
  const size_t sm = hs_analysis_smem<T>(m, LG);
  JG_TRY(g_hs_ana_smem[sizeof(T) == 8 ? 1 : 0].run([]() -> int {
    JG_CUDA(cudaFuncSetAttribute(k_hs_analysis<T, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBudget));
    JG_CUDA(cudaFuncSetAttribute(k_hs_analysis<T, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBudget));
    return JGCM_OK;
  }));
  HSAnaArgs<T> a;
  a.F = (const V2<T>*)(fbuf ? fbuf : m->d_fbuf);
  a.dvor = (V2<T>*)dvor;
  a.ddiv = (V2<T>*)ddiv;
  a.dt = (V2<T>*)dt;
  a.dlnps = (V2<T>*)dlnps;
  a.Cin = fp.C;
  a.colU = colU;
  a.colV = colV;
  a.colE = colE;
  a.colT = colT;
  a.colP = colP;
  a.nd = nd;
  a.L = nd * E;
  a.E = E;
  a.N = m->N;
  a.ns = m->ns;
  a.nlat = m->nlat;
  a.nh = m->nh;
  a.LG = LG;
  const int np = hs_analysis_np(E);
  const int threads = (hs_analysis_rows(m, np) * LG + 31) / 32 * 32;
  dim3 grid(m->N / 2 + 1, (nd + 1 + LG - 1) / LG, E);
  if (np == 2)
    JG_CUDA(launch_pdl(k_hs_analysis<T, 2>, grid, threads, sm, st, a, tables<T>(m)));
  else
    JG_CUDA(launch_pdl(k_hs_analysis<T, 1>, grid, threads, sm, st, a, tables<T>(m)));
  mark(st);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}

template int launch_hs_analysis<float>(jgcm_mesh*, const FFTPlan&, int, int, int, int, int, int, int, void*, void*,
                                       void*, void*, cudaStream_t, void*, int);
template int launch_hs_analysis<double>(jgcm_mesh*, const FFTPlan&, int, int, int, int, int, int, int, void*, void*,
                                        void*, void*, cudaStream_t, void*, int);

}  // namespace jgcm
