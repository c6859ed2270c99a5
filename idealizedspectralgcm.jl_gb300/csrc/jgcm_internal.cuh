// jgcm_internal.cuh -- shared definitions of libjgcm (GB300 / sm_103a).
//
// Device data layout (all fields resident in HBM, one allocation per field):
//   grid      T   g[k][j][i]         k < L, j < nlat (south->north), i < nlon   (= Julia layout)
//   spectral  T2  s[m][n][k]         m <= N, n <= N+1, k < L  ("MNK": levels innermost, so a
//                                      per-m Legendre block and a per-(m,n) vertical column both
//                                      read contiguous memory); entries n < m are kept at zero
//   fourier   T2  F[m][j][c]         m <= N, j < nlat, c < C (c = (field, level) column of a batch)
//   tables    T   P[m][n][jh]        jh < nlat/2 (southern hemisphere; the north follows by parity)
// T is double (JGCM_FP64) or float (the mixed-precision modes).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <string>
#include <vector>
#include <utility>

#include "jgcm.h"

#define JGCM_MAX_GROUPS 16
#define JGCM_MAX_ND 64
#define JGCM_MAX_DEVICES 64

namespace jgcm {

// Dynamic shared memory the transform kernels may use per block (the SM allows 227 KB).
constexpr size_t kSmemBudget = 200 * 1024;

// Largest dynamic shared memory the unconditional parts of the transform kernels need for a mesh
// whose tables hold `ts`-byte reals: the synthesis stages all P rows of one m plus one spectral
// column tile, the analysis four Fourier slots per hemisphere pair, the FFTs one line per column.
inline size_t transform_smem_need(int N, int ns, int nlat, int nlon, size_t ts) {
  const size_t nh = (size_t)nlat / 2;
  const size_t s2g_ct = nh >= 256 ? 1 : 256 / nh, g2s_ct = nh >= 64 ? 4 : nh >= 32 ? 8 : 16;
  const size_t fft_ct = nlon >= 1024 ? 1 : 1024 / nlon;
  size_t s2g = (((size_t)(ns + 1) * nh * ts + 15) & ~(size_t)15) + (size_t)(ns + 1) * s2g_ct * 2 * ts;
  size_t g2s = 8 * g2s_ct * nh * 2 * ts;
  size_t fft = (((fft_ct * nlon + nlon) * ts + 15) & ~(size_t)15) + (size_t)(N + 1) * fft_ct * 2 * ts;
  size_t r = s2g > g2s ? s2g : g2s;
  return r > fft ? r : fft;
}

void set_error(const char* fmt, ...);

#define JG_CUDA(expr)                                                                         \
  do {                                                                                        \
    cudaError_t e_ = (expr);                                                                  \
    if (e_ != cudaSuccess) {                                                                  \
      jgcm::set_error("%s:%d %s -> %s", __FILE__, __LINE__, #expr, cudaGetErrorString(e_)); \
      return JGCM_E_CUDA;                                                                     \
    }                                                                                         \
  } while (0)
#define JG_TRY(expr)          \
  do {                        \
    int s_ = (expr);          \
    if (s_ != JGCM_OK) return s_; \
  } while (0)
#define JG_ARG(cond, ...)               \
  do {                                  \
    if (!(cond)) {                      \
      jgcm::set_error(__VA_ARGS__);     \
      return JGCM_E_ARG;                \
    }                                   \
  } while (0)

// One-time set-up that has to be repeated on every CUDA device: cudaFuncSetAttribute (the dynamic
// shared-memory cap of a kernel) applies only to the device current when it is called.  run() calls
// `f` once per device, with that device current; callers on several threads serialise on the mutex,
// and a device already set up costs one atomic load.
struct PerDeviceOnce {
  std::atomic<bool> done[JGCM_MAX_DEVICES] = {};
  std::mutex mu;
  template <class F>
  int run(F&& f) {
    int dev = 0;
    JG_CUDA(cudaGetDevice(&dev));
    JG_ARG(dev >= 0 && dev < JGCM_MAX_DEVICES, "device index %d out of range", dev);
    if (done[dev].load(std::memory_order_acquire)) return JGCM_OK;
    std::lock_guard<std::mutex> lk(mu);
    if (done[dev].load(std::memory_order_relaxed)) return JGCM_OK;
    JG_TRY(f());
    done[dev].store(true, std::memory_order_release);
    return JGCM_OK;
  }
};

template <typename T>
struct C2;
template <>
struct C2<float> {
  using t = float2;
};
template <>
struct C2<double> {
  using t = double2;
};

// ------------------------------------------------------------------------------------------
// Tables used by the kernels, one set per arithmetic type.
template <typename T>
struct Tables {
  const T* P;     // [m][n][jh]  P_n^m(mu_j)                          (S2G)
  const T* PW;    // [m][n][jh]  P_n^m(mu_j) w_j                      (G2S, x0.5 applied after the sum)
  const T* CA;    // [m][n][jh]  m w P / cos^2 / (2a)                 (alpha operator, i*A term)
  const T* CB;    // [m][n][jh]  -w dP/dmu / (2a)                     (alpha operator, B term)
  const T* dlam;  // [m][n]  m/a
  const T* dthm;  // [m][n]  -(n-1) eps_n / a
  const T* dthp;  // [m][n]  (n+2) eps_{n+1} / a
  const T* uvm;   // [m][n]  a eps_n / n
  const T* uvc;   // [m][n]  -a m / (n(n+1))
  const T* uvp;   // [m][n]  -a eps_{n+1} / (n+1)
  const T* eig;   // [m][n]  -n(n+1)/a^2
  const T* cosj;  // [nlat]
  const T* sinj;  // [nlat]
  const T* tw;    // [nlon/2][2]  cos, sin of 2 pi k / nlon
  const double* wts;  // [nlat] FP64 Gaussian weights (for FP64 global sums)
};

template <typename T>
struct TableStore {
  T *P, *PW, *CA, *CB, *dlam, *dthm, *dthp, *uvm, *uvc, *uvp, *eig, *cosj, *sinj, *tw;
  Tables<T> view(const double* wts) const {
    return Tables<T>{P, PW, CA, CB, dlam, dthm, dthp, uvm, uvc, uvp, eig, cosj, sinj, tw, wts};
  }
};

// ------------------------------------------------------------------------------------------
// Transform plans.  A launch processes a batch of columns; each group maps a contiguous
// column range [col0, col0+L) to one field (one column per level).
// S2G_ADJ_G2S: input of the adjoint of the analysis (m >= 1 halved, row N+1 dropped)
// S2G_ANOM: the field without the real part of its (0,0) mode (P_00 = 1: each level's anomaly about
// its area mean), so its FP32 rounding scales with the anomaly, not with the mean
enum S2GOp { S2G_PLAIN = 0, S2G_DLAM = 1, S2G_DTH = 2, S2G_UCOS = 3, S2G_VCOS = 4, S2G_ADJ_G2S = 5, S2G_ANOM = 6 };
// A plan scalar in the kernel's precision: FP64 fields keep the host's values and FP32 kernels read
// the FP32 copies the launchers fill in (every FP64 -> FP32 conversion, like every FP64 operation,
// runs on the FP64 pipe, at 1/64 of the FP32 rate on this part).
template <typename T>
__host__ __device__ __forceinline__ T pick(double d, float f);
template <>
__host__ __device__ __forceinline__ float pick<float>(double, float f) {
  return f;
}
template <>
__host__ __device__ __forceinline__ double pick<double>(double d, float) {
  return d;
}

struct S2GGroup {
  const void* a;  // spectral field (MNK, L levels)
  const void* b;  // second field (UCOS/VCOS: divergence; a = vorticity)
  double shift;   // PLAIN: subtracted from the real part of mode (0,0) before the synthesis
  float shiftf;   // its FP32 copy (filled by the launchers, as every *f field below)
  int op, L, col0;
};
struct S2GPlan {
  int ng, C;
  S2GGroup g[JGCM_MAX_GROUPS];
};

// EPI_ADJ_G2S: x w_j / (2 nlon), the output scaling of the adjoint of the analysis
// EPI_ANOM: x synthesised from an S2G_ANOM group (the field less its level means): dst = x + the level
// mean (the real part of the group's spectral (0,0) mode, P_00 = 1), dst2 = x
enum GridEpi { EPI_NONE = 0, EPI_DIVCOS = 1, EPI_EXP2 = 2, EPI_DIVCOS_MULPS = 3, EPI_ADJ_G2S = 4, EPI_ANOM = 5 };
struct GridOutGroup {
  void* dst;
  void* dst2;      // EPI_EXP2: exp(x); EPI_ANOM: x
  const void* ps;  // EPI_DIVCOS_MULPS: surface pressure grid [nlat][nlon]; EPI_ANOM: the spectral field
  double shift;    // EPI_EXP2: x is ln(ps) - shift: dst = x + shift, dst2 = exp(x) exp(shift)
  double eshift;   // exp(shift)
  float shiftf, eshiftf;
  int epi, L, col0, pad;
};
struct IFFTPlan {
  int ng, C;
  GridOutGroup g[JGCM_MAX_GROUPS];
};

enum GridPro { PRO_NONE = 0, PRO_MULCOS = 1, PRO_FLUXU = 2, PRO_FLUXV = 3, PRO_KIN = 4, PRO_SWH = 5 };
struct GridInGroup {
  const void* src;  // NONE/MULCOS: field; FLUX*: u ; KIN: u ; SWH: h
  const void* s1;   // FLUX*: v ; KIN: v ; SWH: u
  const void* s2;   // FLUX*: vor ; SWH: v
  const void* s3;   // SWH: dlam_h
  const void* s4;   // SWH: dth_h
  const void* s5;   // SWH: div
  const void* s6;   // SWH: h_eq
  int pro, L, col0, pad;
};
struct FFTPlan {
  int ng, C;
  double kappa_m, kappa_t;
  float kappa_mf, kappa_tf;
  const void* coriolis;  // [nlat] in T
  GridInGroup g[JGCM_MAX_GROUPS];
};

// G2S_ADJ_S2G: adjoint of the synthesis, c_m nlon sum_j P F (unweighted quadrature, row N+1 kept)
enum G2SOp { G2S_PLAIN = 0, G2S_VOR = 1, G2S_DIV = 2, G2S_BARO = 3, G2S_SW = 4, G2S_ADJ_S2G = 5 };
// Fused time-stepping parameters for the G2S epilogues (barotropic / shallow water).
struct StepParams {
  int init_step;
  int dt;
  double robert, implicit_coef, h0;
  float robertf, implicit_coeff, h0f;
  const void* damping;  // [m][n] in T
};
struct SpecOutGroup {
  void* dst;          // PLAIN/VOR/DIV: output; BARO: vor_n; SW: vor_n
  void* dst2;         // SW: div_n
  void* dst3;         // SW: h_n
  const void* extra;  // DIV: spectral field added to G2S(E) before the Laplacian (SW: h_c), nullable
  const void* qc[3];  // BARO/SW: current level (vor, div, h) -- updated in place by the RA filter
  const void* qp[3];  // BARO/SW: previous level
  double scale;       // ADJ_S2G: nlon
  float scalef;
  int op, L, col0;
  int colA, colB, colE, colH;  // Fourier-buffer base columns of the input slots (-1 = unused)
};
struct G2SPlan {
  int ng, C;  // C = number of output columns
  StepParams sp;
  SpecOutGroup g[JGCM_MAX_GROUPS];
};

// Tensor-core (tcgen05) Legendre path of the TF32x3 / BF16x3 precision modes: the tables as
// hi + lo operand images in the no-swizzle K-major layout of the MMA, one block per m (synthesis)
// or per (m, K chunk) (analysis), fetched whole by bulk async copies.
struct TcTables {
  int on;                  // this mesh runs its Legendre contractions on the tensor cores
  int esz, per, kstep;     // operand bytes, elements per 16-byte row of a core matrix, MMA K
  int KC;                  // analysis K chunk (folded latitudes per pass)
  int Nq;                  // synthesis MMA N = 2 * nh (even | odd parity)
  int NpM;                 // analysis MMA N for m = 0: roundup(ns + 1, 16); channel stride in TMEM
  size_t smem_s2g, smem_g2s;
  unsigned char *s2g, *g2s_p, *g2s_a;          // images (synthesis P; analysis PW/2; alpha CA, CB)
  long long *s2g_off, *g2s_p_off, *g2s_a_off;  // device [N+1]: byte offset of each m's image
};

}  // namespace jgcm

// ------------------------------------------------------------------------------------------
struct jgcm_mesh {
  int N, ns, nlat, nlon, nd, nh, logn, precision;
  double radius;
  cudaStream_t stream;
  // FP64 reference-layout tables generated on the GPU
  double *d_sinth, *d_wts, *d_costh, *d_qnm, *d_dqnm;
  double* d_ref2;  // scratch for reference-layout 2-D tables on export
  jgcm::TableStore<double> t64;
  jgcm::TableStore<float> t32;
  jgcm::TcTables tc;
  unsigned int* d_status;  // device error bits of the tensor-core kernels (bounded waits that gave up)
  int tune[4];             // tile overrides: [1] S2G columns, [2] G2S columns, [3] FFT columns per block (0 = default)
  int tune_gen;            // bumped when the tiles change: captured graphs of the mesh's models are stale
  int simt_legendre;       // tensor-core precision modes: 1 = run the Legendre contractions on the FP32
                           // SIMT kernels instead (chosen by the autotuner where they are faster)
  int hs_levels;           // levels per block of the Held-Suarez analysis kernel (0 = default)
  // workspace
  int Cmax;
  void* d_fbuf;       // Fourier buffer [m][j][c] complex T, c < Cmax
  double* d_stage;    // FP64 host-layout staging, 4 slots of max(spec,grid) * nd
  size_t stage_slot;  // doubles per slot
  void* d_grid[4];    // native grid scratch (T), nd levels each
  void* d_spec[4];    // native spectral scratch (T2), nd levels each
  double* d_red;      // reduction scratch (FP64)
  unsigned int* d_counter;
  int refs;           // 1 for the caller's handle + 1 per live model built on the mesh
  int device;         // CUDA device the mesh lives on
  int sm_count;       // its SMs (152 on GB300): the size thresholds of the kernel choices
  std::string name;
  std::vector<float> twf_host;  // the FP32 twiddle table (cos, sin of 2π t / nlon, t < nlon/2) on the host
};

namespace jgcm {
// Per-launch CUDA-event markers for kernel timing (jgcm_model_kernel_times): while a Marker is
// installed on the calling thread, every kernel launch of the library records an event after it.
struct Marker {
  cudaEvent_t* ev;
  int n, cap;
};
extern thread_local Marker* g_marker;
inline void mark(cudaStream_t st) {
  if (g_marker && g_marker->n < g_marker->cap) cudaEventRecord(g_marker->ev[g_marker->n++], st);
}

// Programmatic dependent launch.  The kernels of a model step start with pdl_wait() (griddepcontrol.wait:
// returns once the preceding grid on the stream has completed and its writes are visible; a no-op
// for an ordinary launch), and launch_pdl() launches them with the programmatic-serialization
// attribute: the next grid is launched as the blocks of its predecessor exit, without waiting for
// the whole grid's completion, in streams and in captured graphs (HS T42L20 FP32 step: 78.3 -> 75.3
// us).  An explicit griddepcontrol.launch_dependents at the start of every block, which lets the
// next grid's blocks occupy the SMs while this one runs, measured 10 % slower and is not used.
// Set JGCM_PDL=0 to launch them ordinarily.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
extern int g_pdl;
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = g_pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}
// launch_pdl() in thread-block clusters of `cluster` blocks (each grid dimension a multiple of it)
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl_cluster(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                                      dim3 cluster, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[2];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = cluster.x;
  at[0].val.clusterDim.y = cluster.y;
  at[0].val.clusterDim.z = cluster.z;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = g_pdl ? 2 : 1;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

inline bool is_fp64(const jgcm_mesh* m) { return m->precision == JGCM_FP64; }
inline size_t spec_elems(const jgcm_mesh* m, int L) { return (size_t)(m->N + 1) * (m->ns + 1) * L; }
inline size_t grid_elems(const jgcm_mesh* m, int L) { return (size_t)m->nlon * m->nlat * L; }
inline size_t tsize(const jgcm_mesh* m) { return is_fp64(m) ? 8 : 4; }

// transforms.cu
// fbuf: Fourier buffer of `cap` columns ((N+1) x nlat x cap complex T); NULL = the mesh's own
template <typename T>
int launch_s2g(jgcm_mesh* m, const S2GPlan& sp, const IFFTPlan& ip, cudaStream_t st, void* fbuf = nullptr,
               int cap = 0);
template <typename T>
int launch_g2s(jgcm_mesh* m, const FFTPlan& fp, const G2SPlan& gp, cudaStream_t st, void* fbuf = nullptr,
               int cap = 0);
template <typename T>
int launch_fft_only(jgcm_mesh* m, const FFTPlan& fp, cudaStream_t st, void* fbuf = nullptr, int cap = 0);
// the inverse FFT of Fourier coefficients already staged in fbuf ((N+1) x nlat x ip.C)
template <typename T>
int launch_ifft_only(jgcm_mesh* m, const IFFTPlan& ip, cudaStream_t st, void* fbuf = nullptr, int cap = 0);
int spec_host_to_dev(jgcm_mesh* m, const double* d_host_layout, void* d_native, int L, cudaStream_t st);
int spec_dev_to_host(jgcm_mesh* m, const void* d_native, double* d_host_layout, int L, cudaStream_t st);
int grid_host_to_dev(jgcm_mesh* m, const double* d_src, void* d_native, size_t n, cudaStream_t st);
int grid_dev_to_host(jgcm_mesh* m, const void* d_native, double* d_dst, size_t n, cudaStream_t st);
int fourier_dev_to_host(jgcm_mesh* m, int L, double* d_dst, cudaStream_t st);
// all nλ modes of fft/nλ of L device grid levels, FP64 host layout [L][nlat][nlon] complex
int fourier_full_to_host(jgcm_mesh* m, const void* d_grid, int L, double* d_dst, cudaStream_t st);
int apply_laplacian(jgcm_mesh* m, void* d_spec, int L, cudaStream_t st);
int area_mean(jgcm_mesh* m, const void* d_grid, double* d_out, cudaStream_t st);
template <typename T>
Tables<T> tables(const jgcm_mesh* m);

// legendre_tc.cu
int tc_check_mesh(int N, int ns, int nlat, int precision);  // JGCM_OK if the tensor path fits
int tc_tables_build(jgcm_mesh* m);
void tc_tables_free(jgcm_mesh* m);
int launch_s2g_legendre_tc(jgcm_mesh* m, const S2GPlan& sp, void* fbuf, cudaStream_t st);
int launch_g2s_legendre_tc(jgcm_mesh* m, const G2SPlan& gp, int Cin, cudaStream_t st, void* fbuf);
int tc_status(jgcm_mesh* m);  // reads and clears the device error bits

size_t simt_smem_need(const jgcm_mesh* m, int s2g, int g2s, int fft);

// hs_transforms.cu: the Held-Suarez step's analysis as one contraction per (m pair, level group,
// member); the forward FFT of the plan first
bool hs_analysis_fits(const jgcm_mesh* m, int nd, int E);
int hs_analysis_levels(const jgcm_mesh* m, int nd, int E);
template <typename T>
int launch_hs_analysis(jgcm_mesh* m, const FFTPlan& fp, int colU, int colV, int colE, int colT, int colP, int nd,
                       int E, void* dvor, void* ddiv, void* dt, void* dlnps, cudaStream_t st, void* fbuf, int cap);

// mesh.cu
int mesh_build_tables(jgcm_mesh* m);
void mesh_retain(jgcm_mesh* m);
void mesh_release(jgcm_mesh* m);  // frees the mesh when the last reference goes
}  // namespace jgcm
