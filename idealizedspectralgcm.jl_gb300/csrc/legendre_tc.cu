// legendre_tc.cu -- the Legendre contractions on the 5th-generation tensor cores (tcgen05).
//
// Precision modes JGCM_TF32X3 and JGCM_BF16X3 run the per-m Legendre contraction of the synthesis
// (Trans_Spherical_To_Grid!, Spectral_Spherical_Mesh.jl:143-217) and of the analysis
// (Trans_Grid_To_Spherical! :221-293, Compute_Alpha_Operator! :424-459) as MMAs with FP32
// accumulation in tensor memory.  Each FP32 operand x is split into a hi and a lo part of the
// operand type (TF32 or BF16), and D += A_hi B_hi + A_hi B_lo + A_lo B_hi (3-term compensated
// products; the lo x lo term is below FP32 rounding for TF32).
//
// One CTA owns 64 complex columns = 128 real rows (M = 128; row 2c + r is component r of column c):
//   synthesis  D[row][q]  = sum_n X[row][n] Pq[q][n], q < nh: P of even n - m, q >= nh: odd n - m,
//              so D holds the even and odd hemisphere sums E, O; F_south = E + O, F_north = E - O.
//   analysis   D_ch[row][n] = sum_kappa A_ch[row][kappa] B[n][kappa], kappa running over folded
//              latitudes (g(mu_j) +- g(-mu_j)): plain analysis (PW / 2) and the alpha operator
//              (CA, CB with the i of its first term folded into A's rows); up to four result
//              channels per column (the slots of the fused epilogues), each a TMEM column range.
// Operands live in shared memory in the no-swizzle K-major layout (core matrices of 8 rows x 16 B;
// K-adjacent core matrices 128 B apart, 8-row groups SBO apart).  The table operand of each m (or
// each (m, K chunk)) is one contiguous image in HBM, fetched by a bulk async copy completing on an
// mbarrier; the data operand is built by the CTA's threads (prologue: the spectral recurrences of
// the synthesis, the hemisphere folds of the analysis).  One thread issues the MMAs and commits
// them to an mbarrier; four warps read the accumulator back with tcgen05.ld for the epilogue.
// Every wait is bounded: a wait that gives up sets a bit in the mesh's status word and the CTA
// frees its tensor memory and returns.
#include <cuda_bf16.h>

#include <cstdint>
#include <vector>

#include "jgcm_internal.cuh"
#include "transform_ops.cuh"

namespace jgcm {

namespace tc {

// ---- operand types ------------------------------------------------------------------------
struct TF32x3 {
  using E = uint32_t;
  static constexpr int per = 4, kstep = 8;
  static constexpr uint32_t fmt = 2;  // instruction-descriptor operand format TF32 (kind::tf32)
  static __device__ __forceinline__ E rnd(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
  }
  static __device__ __forceinline__ float val(E e) { return __uint_as_float(e); }
};
struct BF16x3 {
  using E = uint16_t;
  static constexpr int per = 8, kstep = 16;
  static constexpr uint32_t fmt = 1;  // BF16 (kind::f16)
  static __device__ __forceinline__ E rnd(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
  static __device__ __forceinline__ float val(E e) { return __bfloat162float(__ushort_as_bfloat16(e)); }
};

template <class P>
__device__ __forceinline__ void split(float x, typename P::E& hi, typename P::E& lo) {
  hi = P::rnd(x);
  lo = P::rnd(x - P::val(hi));
}
template <class P>
__device__ __forceinline__ void split_d(double x, typename P::E& hi, typename P::E& lo) {
  hi = P::rnd((float)x);
  lo = P::rnd((float)(x - (double)P::val(hi)));
}

// byte offset of element (r, k) in a no-swizzle K-major operand with 8-row-group stride sbo
template <class P>
__host__ __device__ __forceinline__ uint32_t cm_off(int r, int k, uint32_t sbo) {
  return (uint32_t)(r >> 3) * sbo + (uint32_t)(k / P::per) * 128u + (uint32_t)(r & 7) * 16u +
         (uint32_t)(k % P::per) * (uint32_t)sizeof(typename P::E);
}

// ---- PTX wrappers ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t sbo) {
  uint64_t d = (uint64_t)((addr & 0x3FFFFu) >> 4);
  d |= (uint64_t)(128u >> 4) << 16;           // leading (K) byte offset between core matrices
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;  // stride byte offset between 8-row groups
  d |= (uint64_t)1 << 46;                     // descriptor version of tcgen05; no swizzle
  return d;
}

template <class P>
__device__ __forceinline__ uint32_t idesc(int M, int N) {
  return (1u << 4) | (P::fmt << 7) | (P::fmt << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

template <class P>
__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t acc);
template <>
__device__ __forceinline__ void mma<TF32x3>(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(id), "r"(acc));
}
template <>
__device__ __forceinline__ void mma<BF16x3>(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(id), "r"(acc));
}

__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void bar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(1));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// bounded wait for the phase with the given parity; true when it completed
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity, int max_polls = 1 << 20) {
  uint32_t done = 0;
  for (int it = 0; it < max_polls && !done; it++) {
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(su32(bar)), "r"(parity)
        : "memory");
  }
  return done != 0;
}
// one thread: expect `bytes` on bar and start the bulk copy global -> shared
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   su32(dst)),
               "l"(src), "r"(bytes), "r"(su32(bar))
               : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(slot)), "r"(ncols));
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tmem_free(uint32_t base, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(ncols));
}
// 8 consecutive FP32 columns of this thread's lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

__host__ __device__ __forceinline__ uint32_t tmem_cols(int n) {
  uint32_t c = 32;
  while ((int)c < n) c <<= 1;
  return c;
}
__host__ __device__ __forceinline__ int roundup(int x, int q) { return (x + q - 1) / q * q; }

enum : unsigned { ST_TABLE_WAIT = 1u, ST_MMA_WAIT = 2u };

// ---- table images ---------------------------------------------------------------------------
// synthesis, per m: B[q][r] (q < 2nh, r < Kp_m = roundup(ns + 1 - m, kstep)), hi image then lo image
template <class P>
__global__ void k_pack_s2g(const double* __restrict__ Pt, unsigned char* img, const long long* __restrict__ off,
                           int ns, int nh, int kstep) {
  const int m = blockIdx.x, K = ns + 1 - m, Kp = roundup(K, kstep), Nq = 2 * nh;
  const uint32_t sbo = (uint32_t)(Kp / P::per) * 128u;
  using E = typename P::E;
  unsigned char* hi = img + off[m];
  unsigned char* lo = hi + (size_t)Nq * Kp * sizeof(E);
  const size_t mrow = (size_t)m * (ns + 1);
  for (int i = threadIdx.x; i < Nq * Kp; i += blockDim.x) {
    const int q = i / Kp, r = i - q * Kp, jh = q % nh;
    double v = 0.0;
    if (r < K && ((r & 1) == (q >= nh ? 1 : 0))) v = Pt[(mrow + m + r) * nh + jh];
    E h, l;
    split_d<P>(v, h, l);
    *(E*)(hi + cm_off<P>(q, r, sbo)) = h;
    *(E*)(lo + cm_off<P>(q, r, sbo)) = l;
  }
}

// analysis, per (m, chunk): B[r][kappa] (r < Np_m = max(16, roundup(ns + 1 - m, 16)), kappa < KC of
// the chunk's folded latitudes); alpha = 0 plain (PW/2 on [sym | anti]), 1 alpha ([CA sym | CA anti |
// CB sym | CB anti] blocks, each matched to the parity of n - m).  Row n = ns is zero (the reference
// zeroes the extra total wavenumber of an analysis).
template <class P>
__global__ void k_pack_g2s(const double* __restrict__ PW, const double* __restrict__ CA, const double* __restrict__ CB,
                           unsigned char* img, const long long* __restrict__ off, int ns, int nh, int KC, int alpha) {
  const int m = blockIdx.x, K = ns + 1 - m, Np = roundup(K, 16) < 16 ? 16 : roundup(K, 16);
  const int Kf = (alpha ? 4 : 2) * nh, nch = (Kf + KC - 1) / KC;
  const uint32_t sbo = (uint32_t)(KC / P::per) * 128u;
  using E = typename P::E;
  const size_t mrow = (size_t)m * (ns + 1), chunk_bytes = (size_t)2 * Np * KC * sizeof(E);
  for (int i = threadIdx.x; i < nch * Np * KC; i += blockDim.x) {
    const int ch = i / (Np * KC), rem = i - ch * Np * KC, r = rem / KC, kl = rem - r * KC, kap = ch * KC + kl;
    double v = 0.0;
    const int n = m + r;
    if (r < K && n < ns && kap < Kf) {
      const int blk = kap / nh, jh = kap - blk * nh;
      const bool even = (r & 1) == 0;
      const size_t t = (mrow + n) * nh + jh;
      if (!alpha) {
        if ((blk == 0) == even) v = 0.5 * PW[t];
      } else {
        if (blk == 0 && even) v = CA[t];
        if (blk == 1 && !even) v = CA[t];
        if (blk == 2 && !even) v = CB[t];
        if (blk == 3 && even) v = CB[t];
      }
    }
    E h, l;
    split_d<P>(v, h, l);
    unsigned char* hi = img + off[m] + (size_t)ch * chunk_bytes;
    unsigned char* lo = hi + (size_t)Np * KC * sizeof(E);
    *(E*)(hi + cm_off<P>(r, kl, sbo)) = h;
    *(E*)(lo + cm_off<P>(r, kl, sbo)) = l;
  }
}

// ---- synthesis ------------------------------------------------------------------------------
template <class P>
__global__ void __launch_bounds__(256) k_s2g_tc(S2GPlan plan, Tables<float> tb, const unsigned char* __restrict__ timg,
                                                const long long* __restrict__ toff, float2* __restrict__ F, int ns,
                                                int nlat, unsigned* status) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using E = typename P::E;
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int issued;
  const int m = blockIdx.y, nh = nlat >> 1, Nq = 2 * nh;
  const int K = ns + 1 - m, Kp = roundup(K, P::kstep);
  const int C = plan.C;
  int gi = 0, tile = blockIdx.x;
  while (gi < plan.ng - 1 && tile >= (plan.g[gi].L + 63) / 64) {
    tile -= (plan.g[gi].L + 63) / 64;
    gi++;
  }
  const S2GGroup& g = plan.g[gi];
  const int k0 = tile * 64, ncl = min(64, g.L - k0), cbase = g.col0 + k0;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sboA = (uint32_t)(Kp / P::per) * 128u, sboB = sboA;
  const size_t opA = (size_t)128 * Kp * sizeof(E), opB = (size_t)Nq * Kp * sizeof(E);
  unsigned char* Ahi = smem;
  unsigned char* Alo = smem + opA;
  unsigned char* Bhi = smem + 2 * opA;
  unsigned char* Blo = Bhi + opB;
  const uint32_t ncols = tmem_cols(Nq);
  if (tid == 0) {
    bar_init(&bar[0]);
    bar_init(&bar[1]);
    issued = 0;
  }
  if (warp == 0) tmem_alloc(&tmem_slot, ncols);
  __syncthreads();
  if (tid == 0) bulk_load(Bhi, timg + toff[m], (uint32_t)(2 * opB), &bar[0]);
  // prologue: X[row][r] for n = m + r, split into hi / lo
  const size_t mrow = (size_t)m * (ns + 1);
  // U items per thread per pass: all their loads are issued before any shared-memory store
  constexpr int U = 4;
  for (int base = tid; base < Kp * 64; base += U * blockDim.x) {
    float2 x[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int i = base + u * blockDim.x, r = i >> 6, cl = i & 63;
      x[u] = make_float2(0.f, 0.f);
      if (i < Kp * 64 && r < K && cl < ncl) x[u] = s2g_input<float>(g, tb, m, m + r, ns, mrow, k0 + cl);
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int i = base + u * blockDim.x, r = i >> 6, cl = i & 63;
      if (i < Kp * 64) {
        E h, l;
        split<P>(x[u].x, h, l);
        *(E*)(Ahi + cm_off<P>(2 * cl, r, sboA)) = h;
        *(E*)(Alo + cm_off<P>(2 * cl, r, sboA)) = l;
        split<P>(x[u].y, h, l);
        *(E*)(Ahi + cm_off<P>(2 * cl + 1, r, sboA)) = h;
        *(E*)(Alo + cm_off<P>(2 * cl + 1, r, sboA)) = l;
      }
    }
  }
  fence_async_smem();
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;
  if (tid == 0) {
    if (bar_wait(&bar[0], 0)) {
      const uint32_t id = idesc<P>(128, Nq);
      const int steps = Kp / P::kstep;
      const uint32_t stepb = (uint32_t)(P::kstep / P::per) * 128u;
      for (int s = 0; s < steps; s++) {
        const uint32_t a_hi = su32(Ahi) + s * stepb, a_lo = su32(Alo) + s * stepb;
        const uint32_t b_hi = su32(Bhi) + s * stepb, b_lo = su32(Blo) + s * stepb;
        mma<P>(tmem, sdesc(a_lo, sboA), sdesc(b_hi, sboB), id, s > 0 ? 1u : 0u);
        mma<P>(tmem, sdesc(a_hi, sboA), sdesc(b_lo, sboB), id, 1u);
        mma<P>(tmem, sdesc(a_hi, sboA), sdesc(b_hi, sboB), id, 1u);
      }
      commit(&bar[1]);
      issued = 1;
    } else {
      atomicOr(status, ST_TABLE_WAIT);
    }
  }
  __syncthreads();
  bool ok = issued != 0;
  if (ok && !bar_wait(&bar[1], 0)) {
    ok = false;
    if (lane == 0) atomicOr(status, ST_MMA_WAIT);
  }
  ok = __syncthreads_and(ok);
  if (!ok && tid == 0) {  // let a copy or MMAs that may still be in flight finish before leaving
    bar_wait(&bar[0], 0);
    bar_wait(&bar[1], 0);
  }
  fence_after();
  if (ok && warp < 8) {
    const int q = warp & 3, half = warp >> 2;
    const int row = q * 32 + lane, cl = row >> 1, reim = row & 1, c = cbase + cl;
    const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16);
    float* Fs = (float*)F;
    for (int j0 = half * (nh >> 1); j0 < (half + 1) * (nh >> 1); j0 += 8) {
      float e[8], o[8];
      tmem_ld8(tl + (uint32_t)j0, e);
      tmem_ld8(tl + (uint32_t)(nh + j0), o);
      if (cl < ncl) {
#pragma unroll
        for (int t = 0; t < 8; t++) {
          const int j = j0 + t;
          Fs[2 * (((size_t)m * nlat + j) * C + c) + reim] = e[t] + o[t];
          Fs[2 * (((size_t)m * nlat + (nlat - 1 - j)) * C + c) + reim] = e[t] - o[t];
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0) tmem_free(tmem, ncols);
}

// ---- analysis -------------------------------------------------------------------------------
enum { KIND_PLAIN = 0, KIND_ALPHA = 1 };

// Which contraction a column of group g contributes to result channel ch (the slots r0..r3 of
// g2s_store); false when the group does not use the channel.
__device__ __forceinline__ bool chan_spec(const SpecOutGroup& g, int ch, int* kind, int* sa, int* sb, float* sign) {
  *sa = 0;
  *sb = 1;
  *sign = 1.f;
  switch (g.op) {
    case G2S_PLAIN:
      *kind = KIND_PLAIN;
      return ch == 0;
    case G2S_VOR:
    case G2S_BARO:
      *kind = KIND_ALPHA;
      *sign = -1.f;
      return ch == 0;
    case G2S_DIV:
      if (ch == 0) {
        *kind = KIND_ALPHA;
        return true;
      }
      if (ch == 2 && g.colE >= 0) {
        *kind = KIND_PLAIN;
        *sa = 2;
        return true;
      }
      return false;
    case G2S_SW:
      if (ch == 0) {
        *kind = KIND_ALPHA;
        *sa = 1;
        *sb = 0;
        *sign = -1.f;
        return true;
      }
      if (ch == 1) {
        *kind = KIND_ALPHA;
        return true;
      }
      *kind = KIND_PLAIN;
      *sa = ch;
      return ch <= 3;
  }
  return false;
}

__device__ __forceinline__ int slot_col(const SpecOutGroup& g, int slot) {
  return slot == 0 ? g.colA : slot == 1 ? g.colB : slot == 2 ? g.colE : g.colH;
}

template <class P>
__global__ void __launch_bounds__(256) k_g2s_tc(G2SPlan plan, Tables<float> tb, const unsigned char* __restrict__ img_p,
                                                const long long* __restrict__ off_p,
                                                const unsigned char* __restrict__ img_a,
                                                const long long* __restrict__ off_a, const float2* __restrict__ F,
                                                int ns, int nlat, int Cin, int KC, int NpM, int nchan,
                                                unsigned* status) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  using E = typename P::E;
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ int flag;
  const int m = blockIdx.y, nh = nlat >> 1;
  const int K = ns + 1 - m, Np = roundup(K, 16) < 16 ? 16 : roundup(K, 16);
  // tile = 64 consecutive columns of one group (uniform op and channels across the CTA)
  int gi = 0, tile = blockIdx.x;
  while (gi < plan.ng - 1 && tile >= (plan.g[gi].L + 63) / 64) {
    tile -= (plan.g[gi].L + 63) / 64;
    gi++;
  }
  const SpecOutGroup& g = plan.g[gi];
  const int k0 = tile * 64, ncl = min(64, g.L - k0);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t sbo = (uint32_t)(KC / P::per) * 128u;
  const size_t opA = (size_t)128 * KC * sizeof(E), opB = (size_t)Np * KC * sizeof(E);
  unsigned char* Ahi = smem;
  unsigned char* Alo = smem + opA;
  unsigned char* Bhi = smem + 2 * opA;
  unsigned char* Blo = Bhi + opB;
  const uint32_t ncols = tmem_cols(nchan * NpM);
  if (tid == 0) {
    bar_init(&bar[0]);
    bar_init(&bar[1]);
    flag = 1;
  }
  if (warp == 0) tmem_alloc(&tmem_slot, ncols);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = tmem_slot;
  const size_t mrow = (size_t)m * (ns + 1);
  uint32_t ph0 = 0, ph1 = 0;
  bool ok = true;
  for (int ch = 0; ch < 4 && ok; ch++) {
    int kind, sa, sb;
    float sg;
    if (!chan_spec(g, ch, &kind, &sa, &sb, &sg)) continue;
    const int Kf = (kind == KIND_ALPHA ? 4 : 2) * nh, nch = (Kf + KC - 1) / KC;
    const unsigned char* img = kind == KIND_ALPHA ? img_a + off_a[m] : img_p + off_p[m];
    const int colA = slot_col(g, sa) + k0, colB = slot_col(g, sb) + k0;
    for (int chunk = 0; chunk < nch && ok; chunk++) {
      if (tid == 0) bulk_load(Bhi, img + (size_t)chunk * 2 * opB, (uint32_t)(2 * opB), &bar[0]);
      // A[row][kappa]: the folded inputs of this channel's contraction
      constexpr int U = 8;  // items per thread per pass: loads first, then the stores
      for (int base = tid; base < KC * 64; base += U * blockDim.x) {
        float2 xs[U], ys[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
          const int i = base + u * blockDim.x, kl = i >> 6, cl = i & 63, kap = chunk * KC + kl;
          xs[u] = ys[u] = make_float2(0.f, 0.f);
          if (i < KC * 64 && cl < ncl && kap < Kf) {
            const int blk = kap / nh, jh = kap - blk * nh;
            const int col = ((kind == KIND_ALPHA && blk >= 2) ? colB : colA) + cl;
            xs[u] = __ldg(F + ((size_t)m * nlat + jh) * Cin + col);
            ys[u] = __ldg(F + ((size_t)m * nlat + (nlat - 1 - jh)) * Cin + col);
          }
        }
#pragma unroll
        for (int u = 0; u < U; u++) {
        const int i = base + u * blockDim.x, kl = i >> 6, cl = i & 63, kap = chunk * KC + kl;
        if (i >= KC * 64) continue;
        float v0 = 0.f, v1 = 0.f;
        if (cl < ncl && kap < Kf) {
          const int blk = kap / nh;
          const float2 x = xs[u], y = ys[u];
          const bool sym = (blk & 1) == 0;
          const float fx = sym ? x.x + y.x : x.x - y.x, fy = sym ? x.y + y.y : x.y - y.y;
          if (kind == KIND_PLAIN) {
            v0 = fx;
            v1 = fy;
          } else if (blk < 2) {  // i * CA-term: (re, im) <- (-im, re)
            v0 = -fy;
            v1 = fx;
          } else {
            v0 = sg * fx;
            v1 = sg * fy;
          }
        }
        E h, l;
        split<P>(v0, h, l);
        *(E*)(Ahi + cm_off<P>(2 * cl, kl, sbo)) = h;
        *(E*)(Alo + cm_off<P>(2 * cl, kl, sbo)) = l;
        split<P>(v1, h, l);
        *(E*)(Ahi + cm_off<P>(2 * cl + 1, kl, sbo)) = h;
        *(E*)(Alo + cm_off<P>(2 * cl + 1, kl, sbo)) = l;
        }
      }
      fence_async_smem();
      fence_before();
      __syncthreads();
      fence_after();
      if (tid == 0) {
        if (bar_wait(&bar[0], ph0)) {
          const uint32_t id = idesc<P>(128, Np);
          const uint32_t d = tmem + (uint32_t)(ch * NpM);
          const int steps = KC / P::kstep;
          const uint32_t stepb = (uint32_t)(P::kstep / P::per) * 128u;
          for (int s = 0; s < steps; s++) {
            const uint32_t a_hi = su32(Ahi) + s * stepb, a_lo = su32(Alo) + s * stepb;
            const uint32_t b_hi = su32(Bhi) + s * stepb, b_lo = su32(Blo) + s * stepb;
            mma<P>(d, sdesc(a_lo, sbo), sdesc(b_hi, sbo), id, (chunk > 0 || s > 0) ? 1u : 0u);
            mma<P>(d, sdesc(a_hi, sbo), sdesc(b_lo, sbo), id, 1u);
            mma<P>(d, sdesc(a_hi, sbo), sdesc(b_hi, sbo), id, 1u);
          }
          commit(&bar[1]);
        } else {
          atomicOr(status, ST_TABLE_WAIT);
          flag = 0;
        }
      }
      ph0 ^= 1u;
      __syncthreads();
      ok = flag != 0;
      if (ok && !bar_wait(&bar[1], ph1)) {
        ok = false;
        if (lane == 0) atomicOr(status, ST_MMA_WAIT);
      }
      ph1 ^= 1u;
      ok = __syncthreads_and(ok);
      fence_after();
    }
  }
  if (!ok && tid == 0) {  // let a copy or MMAs that may still be in flight finish before leaving
    bar_wait(&bar[0], ph0 ^ 1u);
    bar_wait(&bar[1], ph1 ^ 1u);
  }
  if (ok) {
    // epilogue: warps 0-3 own the 128 rows; lanes 2c, 2c + 1 hold the two components of column c
    if (warp < 4) {
      const int row = warp * 32 + lane, cl = row >> 1, reim = row & 1, k = k0 + cl;
      const uint32_t tl = tmem + ((uint32_t)(warp * 32) << 16);
      for (int n0 = 0; n0 < Np; n0 += 8) {
        float v[4][8];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          if (q < nchan) tmem_ld8(tl + (uint32_t)(q * NpM + n0), v[q]);
          else
#pragma unroll
            for (int t = 0; t < 8; t++) v[q][t] = 0.f;
        }
#pragma unroll
        for (int t = 0; t < 8; t++) {
          float2 r[4];
#pragma unroll
          for (int q = 0; q < 4; q++) {
            const float mine = v[q][t], other = __shfl_xor_sync(0xffffffffu, mine, 1);
            r[q] = reim ? make_float2(other, mine) : make_float2(mine, other);
          }
          const int n = m + n0 + t;
          if (cl < ncl && reim == 0 && n <= ns) {
            const size_t sidx = (mrow + n) * g.L + k;
            g2s_store<float>(plan, g, tb, mrow, n, sidx, r[0], r[1], r[2], r[3]);
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 0) tmem_free(tmem, ncols);
}

// ---- host -----------------------------------------------------------------------------------
struct Geom {
  int esz, per, kstep, KC, Nq, NpM;
  size_t smem_s2g, smem_g2s;
};

Geom geometry(int N, int ns, int nlat, int precision) {
  Geom g;
  const bool tf = precision == JGCM_TF32X3;
  g.esz = tf ? 4 : 2;
  g.per = tf ? 4 : 8;
  g.kstep = tf ? 8 : 16;
  const int nh = nlat / 2;
  g.KC = 2 * nh < 64 ? 2 * nh : 64;
  g.Nq = 2 * nh;
  g.NpM = roundup(ns + 1, 16);
  const int Kp0 = roundup(ns + 1, g.kstep);
  g.smem_s2g = (size_t)2 * (128 + g.Nq) * Kp0 * g.esz;
  g.smem_g2s = (size_t)2 * (128 + g.NpM) * g.KC * g.esz;
  (void)N;
  return g;
}

}  // namespace tc

int tc_check_mesh(int N, int ns, int nlat, int precision) {
  tc::Geom g = tc::geometry(N, ns, nlat, precision);
  JG_ARG(nlat % 32 == 0, "the tensor-core precision modes need nlat to be a multiple of 32 (got %d)", nlat);
  JG_ARG(g.Nq <= 256, "the tensor-core precision modes support nlat <= 256 (got %d)", nlat);
  JG_ARG(4 * g.NpM <= 512, "the tensor-core precision modes support num_spherical <= 128 (got %d)", ns);
  JG_ARG(g.smem_s2g <= kSmemBudget && g.smem_g2s <= kSmemBudget,
         "mesh too large for the tensor-core tiling (%zu / %zu bytes of shared memory)", g.smem_s2g, g.smem_g2s);
  return JGCM_OK;
}

void tc_tables_free(jgcm_mesh* m) {
  TcTables& t = m->tc;
  void* ps[] = {t.s2g, t.g2s_p, t.g2s_a, t.s2g_off, t.g2s_p_off, t.g2s_a_off};
  for (auto p : ps)
    if (p) cudaFree(p);
  t = TcTables();
}

int tc_tables_build(jgcm_mesh* m) {
  tc::Geom g = tc::geometry(m->N, m->ns, m->nlat, m->precision);
  TcTables& t = m->tc;
  t = TcTables();
  t.esz = g.esz;
  t.per = g.per;
  t.kstep = g.kstep;
  t.KC = g.KC;
  t.Nq = g.Nq;
  t.NpM = g.NpM;
  t.smem_s2g = g.smem_s2g;
  t.smem_g2s = g.smem_g2s;
  const int N = m->N, ns = m->ns, nh = m->nh;
  std::vector<long long> os(N + 1), op(N + 1), oa(N + 1);
  long long s_tot = 0, p_tot = 0, a_tot = 0;
  const int nchp = (2 * nh + g.KC - 1) / g.KC, ncha = (4 * nh + g.KC - 1) / g.KC;
  for (int mm = 0; mm <= N; mm++) {
    const int K = ns + 1 - mm, Kp = tc::roundup(K, g.kstep), Np = tc::roundup(K, 16) < 16 ? 16 : tc::roundup(K, 16);
    os[mm] = s_tot;
    s_tot += (long long)2 * g.Nq * Kp * g.esz;
    op[mm] = p_tot;
    p_tot += (long long)nchp * 2 * Np * g.KC * g.esz;
    oa[mm] = a_tot;
    a_tot += (long long)ncha * 2 * Np * g.KC * g.esz;
  }
  auto al = [&](void** p, size_t bytes) -> int {
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
      set_error("tensor-core tables: %s", cudaGetErrorString(e));
      return e == cudaErrorMemoryAllocation ? JGCM_E_NOMEM : JGCM_E_CUDA;
    }
    return JGCM_OK;
  };
  JG_TRY(al((void**)&t.s2g, (size_t)s_tot));
  JG_TRY(al((void**)&t.g2s_p, (size_t)p_tot));
  JG_TRY(al((void**)&t.g2s_a, (size_t)a_tot));
  JG_TRY(al((void**)&t.s2g_off, (N + 1) * sizeof(long long)));
  JG_TRY(al((void**)&t.g2s_p_off, (N + 1) * sizeof(long long)));
  JG_TRY(al((void**)&t.g2s_a_off, (N + 1) * sizeof(long long)));
  cudaStream_t st = m->stream;
  JG_CUDA(cudaMemcpyAsync(t.s2g_off, os.data(), (N + 1) * sizeof(long long), cudaMemcpyHostToDevice, st));
  JG_CUDA(cudaMemcpyAsync(t.g2s_p_off, op.data(), (N + 1) * sizeof(long long), cudaMemcpyHostToDevice, st));
  JG_CUDA(cudaMemcpyAsync(t.g2s_a_off, oa.data(), (N + 1) * sizeof(long long), cudaMemcpyHostToDevice, st));
  const TableStore<double>& d = m->t64;
  if (m->precision == JGCM_TF32X3) {
    tc::k_pack_s2g<tc::TF32x3><<<N + 1, 256, 0, st>>>(d.P, t.s2g, t.s2g_off, ns, nh, g.kstep);
    tc::k_pack_g2s<tc::TF32x3><<<N + 1, 256, 0, st>>>(d.PW, d.CA, d.CB, t.g2s_p, t.g2s_p_off, ns, nh, g.KC, 0);
    tc::k_pack_g2s<tc::TF32x3><<<N + 1, 256, 0, st>>>(d.PW, d.CA, d.CB, t.g2s_a, t.g2s_a_off, ns, nh, g.KC, 1);
  } else {
    tc::k_pack_s2g<tc::BF16x3><<<N + 1, 256, 0, st>>>(d.P, t.s2g, t.s2g_off, ns, nh, g.kstep);
    tc::k_pack_g2s<tc::BF16x3><<<N + 1, 256, 0, st>>>(d.PW, d.CA, d.CB, t.g2s_p, t.g2s_p_off, ns, nh, g.KC, 0);
    tc::k_pack_g2s<tc::BF16x3><<<N + 1, 256, 0, st>>>(d.PW, d.CA, d.CB, t.g2s_a, t.g2s_a_off, ns, nh, g.KC, 1);
  }
  JG_CUDA(cudaGetLastError());
  JG_CUDA(cudaStreamSynchronize(st));
  t.on = 1;
  return JGCM_OK;
}

static PerDeviceOnce g_tc_smem_set[2];  // [0] TF32x3, [1] BF16x3

template <class P>
static int tc_configure() {
  const int idx = sizeof(typename P::E) == 4 ? 0 : 1;
  return g_tc_smem_set[idx].run([]() -> int {
    JG_CUDA(cudaFuncSetAttribute(tc::k_s2g_tc<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBudget));
    JG_CUDA(cudaFuncSetAttribute(tc::k_g2s_tc<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBudget));
    return JGCM_OK;
  });
}

template <class P>
static int s2g_tc(jgcm_mesh* m, const S2GPlan& sp, void* fbuf, cudaStream_t st) {
  JG_TRY(tc_configure<P>());
  const TcTables& t = m->tc;
  int tiles = 0;
  for (int i = 0; i < sp.ng; i++) tiles += (sp.g[i].L + 63) / 64;
  dim3 g(tiles, m->N + 1);
  JG_CUDA(launch_pdl(tc::k_s2g_tc<P>, g, 256, t.smem_s2g, st, sp, tables<float>(m), t.s2g, t.s2g_off, (float2*)fbuf, m->ns, m->nlat,
                                              m->d_status));
  mark(st);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}

template <class P>
static int g2s_tc(jgcm_mesh* m, const G2SPlan& gp, int Cin, cudaStream_t st, void* fbuf) {
  JG_TRY(tc_configure<P>());
  const TcTables& t = m->tc;
  int nchan = 1;
  for (int i = 0; i < gp.ng; i++) {
    if (gp.g[i].op == G2S_SW) nchan = 4;
    else if (gp.g[i].op == G2S_DIV && gp.g[i].colE >= 0 && nchan < 3) nchan = 3;
  }
  int tiles = 0;
  for (int i = 0; i < gp.ng; i++) tiles += (gp.g[i].L + 63) / 64;
  dim3 g(tiles, m->N + 1);
  JG_CUDA(launch_pdl(tc::k_g2s_tc<P>, g, 256, t.smem_g2s, st, gp, tables<float>(m), t.g2s_p, t.g2s_p_off, t.g2s_a, t.g2s_a_off,
                                              (const float2*)fbuf, m->ns, m->nlat, Cin, t.KC, t.NpM, nchan,
                                              m->d_status));
  mark(st);
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}

int launch_s2g_legendre_tc(jgcm_mesh* m, const S2GPlan& sp, void* fbuf, cudaStream_t st) {
  return m->precision == JGCM_TF32X3 ? s2g_tc<tc::TF32x3>(m, sp, fbuf, st) : s2g_tc<tc::BF16x3>(m, sp, fbuf, st);
}

int launch_g2s_legendre_tc(jgcm_mesh* m, const G2SPlan& gp, int Cin, cudaStream_t st, void* fbuf) {
  return m->precision == JGCM_TF32X3 ? g2s_tc<tc::TF32x3>(m, gp, Cin, st, fbuf)
                                     : g2s_tc<tc::BF16x3>(m, gp, Cin, st, fbuf);
}

// Self-test of the failure path: one CTA waits (with a short poll bound) on an mbarrier phase that
// nothing completes, records the give-up in the status word exactly as the Legendre kernels do and
// returns; no copy or MMA is in flight, so the context stays usable.
namespace tc {
__global__ void k_bounded_wait_selftest(unsigned* status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    bar_init(&bar);
    if (!bar_wait(&bar, 0, 4096)) atomicOr(status, ST_TABLE_WAIT);  // phase 0 never completes
  }
}
}  // namespace tc

int tc_status(jgcm_mesh* m) {
  unsigned s = 0;
  JG_CUDA(cudaMemcpy(&s, m->d_status, sizeof(s), cudaMemcpyDeviceToHost));
  if (s) {
    JG_CUDA(cudaMemset(m->d_status, 0, sizeof(s)));
    set_error("tensor-core Legendre kernel gave up waiting (%s%s)", (s & 1u) ? "table copy " : "",
              (s & 2u) ? "MMA completion" : "");
    return JGCM_E_CUDA;
  }
  return JGCM_OK;
}

}  // namespace jgcm

extern "C" int jgcm_selftest_bounded_wait(jgcm_mesh* m) {
  JG_ARG(m, "mesh is NULL");
  jgcm::tc::k_bounded_wait_selftest<<<1, 32, 0, m->stream>>>(m->d_status);
  JG_CUDA(cudaGetLastError());
  // on a tensor-core mesh the give-up is reported the way an asynchronous call's is: by
  // jgcm_mesh_synchronize
  if (m->tc.on) return jgcm_mesh_synchronize(m);
  JG_CUDA(cudaStreamSynchronize(m->stream));
  return jgcm::tc_status(m);
}
