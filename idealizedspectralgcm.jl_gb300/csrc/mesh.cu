// mesh.cu -- Spectral_Spherical_Mesh on the GPU (Spectral_Spherical_Mesh.jl:69-139).
//
// The Gaussian nodes (Gauss_And_Legendre.jl:69-118) and the associated Legendre functions
// with their mu-derivatives (Gauss_And_Legendre.jl:4-66) are generated on the device in
// FP64, one thread per root / per (m, latitude), following the reference recurrences
// operation by operation.  The kernel tables (P, P*w, the alpha-operator coefficients and
// the (m,n) coefficient tables of :396-652) are then derived on the device in FP64 and
// stored in both FP64 and FP32 in the [m][n][jh] layout the transform kernels read.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "jgcm_internal.cuh"

namespace jgcm {

thread_local Marker* g_marker = nullptr;
static thread_local char g_err[1024] = "";
void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}
const char* last_error() { return g_err; }

// Gauss_And_Legendre.jl:69-118, one thread per root of the southern half.
__global__ void k_gauss(int n, double* sinth, double* wts, int* status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (i > n / 2) return;
  const int itermax = 10000;
  const double tol = 1.0e-15;
  double dp = 0.0;
  double z = cos(3.14159265358979323846 * (i - 0.25) / (n + 0.5));
  for (int iter = 1; iter <= itermax; iter++) {
    double p2 = 0.0, p1 = 1.0, p3;
    for (int j = 1; j <= n; j++) {
      p3 = p2;
      p2 = p1;
      p1 = __dsub_rn(__dmul_rn(__dmul_rn(2.0 * j - 1.0, z), p2), __dmul_rn(j - 1.0, p3)) / j;
    }
    dp = __dmul_rn((double)n, __dsub_rn(__dmul_rn(z, p1), p2)) / __dsub_rn(__dmul_rn(z, z), 1.0);
    double z1 = z;
    z = __dsub_rn(z1, p1 / dp);
    if (fabs(z - z1) <= tol) break;
    if (iter == itermax) atomicExch(status, 1);
  }
  sinth[i - 1] = -z;
  sinth[n - i] = z;
  double w = 2.0 / __dmul_rn(__dmul_rn(__dsub_rn(1.0, __dmul_rn(z, z)), dp), dp);
  wts[i - 1] = w;
  wts[n - i] = w;
}

__device__ __forceinline__ double eps_ml(int m, int l) {
  return sqrt((double)(l * l - m * m) / (double)(4 * l * l - 1));
}

// Gauss_And_Legendre.jl:4-66, one thread per (m, latitude); FMA contraction is disabled
// with explicit round-to-nearest intrinsics so the tables agree with the FP64 oracle to
// the last few ulps.  Outputs use the reference layout q[m + (N+1)(l + (ns+1) j)].
__global__ void k_legendre(int N, int ns, int nlat, const double* sinth, double* qnm, double* dqnm) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (N + 1) * nlat) return;
  int m = t % (N + 1), j = t / (N + 1);
  double s = sinth[j];
  double c = sqrt(__dsub_rn(1.0, __dmul_rn(s, s)));
  double c2 = __dmul_rn(c, c);
  double q = 1.0;
  for (int mm = 1; mm <= m; mm++) q = __dmul_rn(__dmul_rn(sqrt((2.0 * mm + 1) / (2.0 * mm)), c), q);
  // P_{m+1} = sqrt(2m+3) sin P_m
  double pl = __dmul_rn(__dmul_rn(sqrt((double)(2 * m + 3)), s), q);
  size_t base = (size_t)m + (size_t)(N + 1) * (size_t)(ns + 1) * (size_t)j;
  // walk l = m .. ns emitting P_l and dP_l (dP_l needs P_{l+1})
  // state at loop head: cur = P_l, nxt = P_{l+1}, prv = P_{l-1}
  double prv = 0.0, cur = q, nxt = pl;
  for (int l = m; l <= ns; l++) {
    qnm[base + (size_t)(N + 1) * l] = cur;
    double e1 = eps_ml(m, l + 1);
    double d;
    if (l == m)
      d = __dmul_rn(__dmul_rn((double)(-l), e1), nxt) / c2;
    else
      d = __dadd_rn(__dmul_rn(__dmul_rn((double)(-l), e1), nxt), __dmul_rn(__dmul_rn((double)(l + 1), eps_ml(m, l)), prv)) / c2;
    dqnm[base + (size_t)(N + 1) * l] = d;
    // advance: P_{l+2} = (s P_{l+1} - eps(m,l+1) P_l) / eps(m,l+2)
    double nn = (l + 2 <= ns + 1) ? __dsub_rn(__dmul_rn(s, nxt), __dmul_rn(e1, cur)) / eps_ml(m, l + 2) : 0.0;
    prv = cur;
    cur = nxt;
    nxt = nn;
  }
}

// Derived kernel tables (FP64 and FP32) in [m][n][jh] / [m][n] layout.
__global__ void k_derive3(int N, int ns, int nlat, double radius, const double* qnm, const double* dqnm,
                          const double* wts, const double* sinth, double* P, double* PW, double* CA, double* CB,
                          float* Pf, float* PWf, float* CAf, float* CBf) {
  int nh = nlat / 2;
  size_t total = (size_t)(N + 1) * (ns + 1) * nh;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    int jh = (int)(t % nh);
    size_t mn = t / nh;
    int n = (int)(mn % (ns + 1)), m = (int)(mn / (ns + 1));
    double p = 0, pw = 0, ca = 0, cb = 0;
    if (n >= m) {
      size_t r = (size_t)m + (size_t)(N + 1) * ((size_t)n + (size_t)(ns + 1) * jh);
      double q = qnm[r], dq = dqnm[r], w = wts[jh];
      double cth = sqrt(1 - sinth[jh] * sinth[jh]);
      double inv2a = 1 / (2 * radius);
      p = q;
      pw = q * w;
      ca = w * q / (cth * cth) * m * inv2a;
      cb = -w * dq * inv2a;
    }
    P[t] = p; PW[t] = pw; CA[t] = ca; CB[t] = cb;
    Pf[t] = (float)p; PWf[t] = (float)pw; CAf[t] = (float)ca; CBf[t] = (float)cb;
  }
}

struct Coef2Ptrs {
  double *dlam, *dthm, *dthp, *uvm, *uvc, *uvp, *eig;
  float *dlamf, *dthmf, *dthpf, *uvmf, *uvcf, *uvpf, *eigf;
};

// Spectral_Spherical_Mesh.jl:101-114, :485-515, :583-652 coefficient tables, [m][n] layout.
__global__ void k_derive2(int N, int ns, double radius, Coef2Ptrs o) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (N + 1) * (ns + 1)) return;
  int n = t % (ns + 1), m = t / (ns + 1);
  double dlam = 0, dthm = 0, dthp = 0, uvm = 0, uvc = 0, uvp = 0, eig = 0;
  if (n >= m) {
    double e_n = sqrt((double)(n * n - m * m) / (4.0 * n * n - 1.0));
    double e_n1 = (n + 1 <= ns) ? sqrt((double)((n + 1) * (n + 1) - m * m) / (4.0 * (n + 1) * (n + 1) - 1.0)) : 0.0;
    dlam = m / radius;
    dthm = -(n - 1) * e_n / radius;
    if (n <= ns - 1) dthp = (n + 2) * e_n1 / radius;
    if (n > 0) uvc = -radius * m / (double)(n * (n + 1));
    if (n > 0) uvm = radius * e_n / n;
    if (n <= ns - 1) uvp = -radius * e_n1 / (n + 1);
    eig = (double)(-n * (n + 1)) / (radius * radius);
  }
  o.dlam[t] = dlam; o.dthm[t] = dthm; o.dthp[t] = dthp; o.uvm[t] = uvm; o.uvc[t] = uvc; o.uvp[t] = uvp; o.eig[t] = eig;
  o.dlamf[t] = (float)dlam; o.dthmf[t] = (float)dthm; o.dthpf[t] = (float)dthp; o.uvmf[t] = (float)uvm;
  o.uvcf[t] = (float)uvc; o.uvpf[t] = (float)uvp; o.eigf[t] = (float)eig;
}

__global__ void k_derive1(int nlat, int nlon, const double* sinth, double* cosd, double* cosj, double* sinj,
                          double* tw, float* cosf, float* sinf, float* twf) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < nlat) {
    double s = sinth[t], c = sqrt(1 - s * s);
    cosd[t] = c; cosj[t] = c; sinj[t] = s; cosf[t] = (float)c; sinf[t] = (float)s;
  }
  if (t < nlon / 2) {
    double sn, cs;
    sincospi(2.0 * t / nlon, &sn, &cs);
    tw[2 * t] = cs; tw[2 * t + 1] = sn;
    twf[2 * t] = (float)cs; twf[2 * t + 1] = (float)sn;
  }
}

template <typename T>
static int alloc_store(TableStore<T>& s, int N, int ns, int nlat, int nlon) {
  size_t n3 = (size_t)(N + 1) * (ns + 1) * (nlat / 2), n2 = (size_t)(N + 1) * (ns + 1);
  T** p3[] = {&s.P, &s.PW, &s.CA, &s.CB};
  for (auto pp : p3) JG_CUDA(cudaMalloc(pp, n3 * sizeof(T)));
  T** p2[] = {&s.dlam, &s.dthm, &s.dthp, &s.uvm, &s.uvc, &s.uvp, &s.eig};
  for (auto pp : p2) JG_CUDA(cudaMalloc(pp, n2 * sizeof(T)));
  JG_CUDA(cudaMalloc(&s.cosj, nlat * sizeof(T)));
  JG_CUDA(cudaMalloc(&s.sinj, nlat * sizeof(T)));
  JG_CUDA(cudaMalloc(&s.tw, (size_t)nlon * sizeof(T)));
  return JGCM_OK;
}
template <typename T>
static void free_store(TableStore<T>& s) {
  T* ps[] = {s.P, s.PW, s.CA, s.CB, s.dlam, s.dthm, s.dthp, s.uvm, s.uvc, s.uvp, s.eig, s.cosj, s.sinj, s.tw};
  for (auto p : ps)
    if (p) cudaFree(p);
}

int mesh_build_tables(jgcm_mesh* m) {
  int N = m->N, ns = m->ns, nlat = m->nlat, nlon = m->nlon;
  cudaStream_t st = m->stream;
  int* d_status = nullptr;
  JG_CUDA(cudaMalloc(&d_status, sizeof(int)));
  JG_CUDA(cudaMemsetAsync(d_status, 0, sizeof(int), st));
  k_gauss<<<(nlat / 2 + 63) / 64, 64, 0, st>>>(nlat, m->d_sinth, m->d_wts, d_status);
  JG_CUDA(cudaGetLastError());
  int nt = (N + 1) * nlat;
  k_legendre<<<(nt + 127) / 128, 128, 0, st>>>(N, ns, nlat, m->d_sinth, m->d_qnm, m->d_dqnm);
  JG_CUDA(cudaGetLastError());
  k_derive3<<<256, 256, 0, st>>>(N, ns, nlat, m->radius, m->d_qnm, m->d_dqnm, m->d_wts, m->d_sinth, m->t64.P,
                                 m->t64.PW, m->t64.CA, m->t64.CB, m->t32.P, m->t32.PW, m->t32.CA, m->t32.CB);
  JG_CUDA(cudaGetLastError());
  Coef2Ptrs o{m->t64.dlam, m->t64.dthm, m->t64.dthp, m->t64.uvm, m->t64.uvc, m->t64.uvp, m->t64.eig,
              m->t32.dlam, m->t32.dthm, m->t32.dthp, m->t32.uvm, m->t32.uvc, m->t32.uvp, m->t32.eig};
  int n2 = (N + 1) * (ns + 1);
  k_derive2<<<(n2 + 127) / 128, 128, 0, st>>>(N, ns, m->radius, o);
  JG_CUDA(cudaGetLastError());
  int n1 = nlat > nlon / 2 ? nlat : nlon / 2;
  k_derive1<<<(n1 + 127) / 128, 128, 0, st>>>(nlat, nlon, m->d_sinth, m->d_costh, m->t64.cosj, m->t64.sinj, m->t64.tw,
                                              m->t32.cosj, m->t32.sinj, m->t32.tw);
  JG_CUDA(cudaGetLastError());
  m->twf_host.assign(nlon, 0.0f);
  JG_CUDA(cudaMemcpyAsync(m->twf_host.data(), m->t32.tw, (size_t)nlon * sizeof(float), cudaMemcpyDeviceToHost, st));
  int h_status = 0;
  JG_CUDA(cudaMemcpyAsync(&h_status, d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  JG_CUDA(cudaStreamSynchronize(st));
  cudaFree(d_status);
  if (h_status) {
    set_error("Compute_Gaussian! does not converge (nlat=%d)", nlat);
    return JGCM_E_NUMERIC;
  }
  return JGCM_OK;
}

template <>
Tables<double> tables<double>(const jgcm_mesh* m) {
  return m->t64.view(m->d_wts);
}
template <>
Tables<float> tables<float>(const jgcm_mesh* m) {
  return m->t32.view(m->d_wts);
}

}  // namespace jgcm

using namespace jgcm;

extern "C" const char* jgcm_last_error(void) { return jgcm::last_error(); }
extern "C" int jgcm_version(void) { return 1; }

extern "C" int jgcm_set_device(int device) {
  JG_CUDA(cudaSetDevice(device));
  return JGCM_OK;
}

extern "C" int jgcm_device_info(int* sm_count, int* cc_major, int* cc_minor) {
  int dev = 0;
  JG_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp p;
  JG_CUDA(cudaGetDeviceProperties(&p, dev));
  if (sm_count) *sm_count = p.multiProcessorCount;
  if (cc_major) *cc_major = p.major;
  if (cc_minor) *cc_minor = p.minor;
  return JGCM_OK;
}

static void mesh_free(jgcm_mesh* m) {
  if (!m) return;
  void* ps[] = {m->d_sinth, m->d_wts, m->d_costh, m->d_qnm, m->d_dqnm, m->d_ref2, m->d_fbuf, m->d_stage,
                m->d_grid[0], m->d_grid[1], m->d_grid[2], m->d_grid[3], m->d_spec[0], m->d_spec[1], m->d_spec[2],
                m->d_spec[3], m->d_red, m->d_counter, m->d_status};
  for (auto p : ps)
    if (p) cudaFree(p);
  tc_tables_free(m);
  free_store(m->t64);
  free_store(m->t32);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

extern "C" int jgcm_mesh_create(int num_fourier, int num_spherical, int nlat, int nlon, int nd, double radius,
                                int precision, jgcm_mesh** out) {
  JG_ARG(out != nullptr, "out is NULL");
  *out = nullptr;
  JG_ARG(num_fourier >= 1 && num_fourier <= 1023, "num_fourier out of range");
  JG_ARG(num_spherical == num_fourier + 1, "num_spherical must be num_fourier + 1");
  JG_ARG(nlat >= 4 && nlat % 2 == 0 && nlat <= 2048, "nlat must be even (reference @assert(nθ%%2 == 0))");
  JG_ARG(nlon >= 8 && nlon <= 1024 && (nlon & (nlon - 1)) == 0, "nlon must be a power of two in [8, 1024]");
  JG_ARG(nlon >= 2 * num_fourier + 2, "nlon must exceed 2*num_fourier+1 (alias-free zonal transform)");
  JG_ARG(nd >= 1 && nd <= JGCM_MAX_ND, "nd must be in [1, %d]", JGCM_MAX_ND);
  JG_ARG(radius > 0, "radius must be positive");
  JG_ARG(precision >= JGCM_FP64 && precision <= JGCM_BF16X3, "unknown precision mode");
  {
    const size_t need = transform_smem_need(num_fourier, num_spherical, nlat, nlon,
                                            precision == JGCM_FP64 ? sizeof(double) : sizeof(float));
    JG_ARG(need <= kSmemBudget, "mesh too large for the shared-memory tiling: %zu bytes > %zu per block", need,
           kSmemBudget);
    if (precision == JGCM_TF32X3 || precision == JGCM_BF16X3) {
      int st = tc_check_mesh(num_fourier, num_spherical, nlat, precision);
      if (st != JGCM_OK) return st;
    }
  }
  jgcm_mesh* m = new jgcm_mesh();  // value-initialised: all pointers start NULL
  m->N = num_fourier;
  m->ns = num_spherical;
  m->nlat = nlat;
  m->nlon = nlon;
  m->nd = nd;
  m->nh = nlat / 2;
  m->radius = radius;
  m->precision = precision;
  int lg = 0;
  while ((1 << lg) < nlon) lg++;
  m->logn = lg;
  int st = JGCM_OK;
#define MCHK(x)            \
  do {                     \
    st = (x);              \
    if (st != JGCM_OK) {   \
      mesh_free(m);        \
      return st;           \
    }                      \
  } while (0)
  auto cuda = [&](cudaError_t e, const char* what) -> int {
    if (e != cudaSuccess) {
      set_error("%s: %s", what, cudaGetErrorString(e));
      return e == cudaErrorMemoryAllocation ? JGCM_E_NOMEM : JGCM_E_CUDA;
    }
    return JGCM_OK;
  };
  MCHK(cuda(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking), "cudaStreamCreate"));
  int dev = 0;
  MCHK(cuda(cudaGetDevice(&dev), "cudaGetDevice"));
  MCHK(cuda(cudaDeviceGetAttribute(&m->sm_count, cudaDevAttrMultiProcessorCount, dev), "cudaDeviceGetAttribute"));
  size_t T3 = (size_t)(m->N + 1) * (m->ns + 1) * nlat;
  MCHK(cuda(cudaMalloc(&m->d_sinth, nlat * 8), "alloc"));
  MCHK(cuda(cudaMalloc(&m->d_wts, nlat * 8), "alloc"));
  MCHK(cuda(cudaMalloc(&m->d_costh, nlat * 8), "alloc"));
  MCHK(cuda(cudaMalloc(&m->d_qnm, T3 * 8), "alloc"));
  MCHK(cuda(cudaMalloc(&m->d_dqnm, T3 * 8), "alloc"));
  MCHK(cuda(cudaMemset(m->d_qnm, 0, T3 * 8), "memset"));
  MCHK(cuda(cudaMemset(m->d_dqnm, 0, T3 * 8), "memset"));
  MCHK(alloc_store(m->t64, m->N, m->ns, nlat, nlon));
  MCHK(alloc_store(m->t32, m->N, m->ns, nlat, nlon));
  MCHK(mesh_build_tables(m));
  // workspace
  m->Cmax = 5 * nd + 2;
  size_t ts = tsize(m);
  MCHK(cuda(cudaMalloc(&m->d_fbuf, (size_t)(m->N + 1) * nlat * m->Cmax * 2 * ts), "alloc fbuf"));
  size_t sg = grid_elems(m, nd), ss = 2 * spec_elems(m, nd);
  m->stage_slot = sg > ss ? sg : ss;
  MCHK(cuda(cudaMalloc(&m->d_stage, 4 * m->stage_slot * 8), "alloc stage"));
  for (int i = 0; i < 4; i++) {
    MCHK(cuda(cudaMalloc(&m->d_grid[i], sg * ts), "alloc grid scratch"));
    MCHK(cuda(cudaMalloc(&m->d_spec[i], spec_elems(m, nd) * 2 * ts), "alloc spec scratch"));
    MCHK(cuda(cudaMemset(m->d_spec[i], 0, spec_elems(m, nd) * 2 * ts), "memset"));
  }
  MCHK(cuda(cudaMalloc(&m->d_red, (size_t)(4 * nlat + 64) * 8), "alloc red"));
  MCHK(cuda(cudaMalloc(&m->d_counter, 64 * sizeof(unsigned int)), "alloc counter"));
  MCHK(cuda(cudaMemset(m->d_counter, 0, 64 * sizeof(unsigned int)), "memset"));
  MCHK(cuda(cudaMalloc(&m->d_ref2, T3 * 8), "alloc ref2"));
  MCHK(cuda(cudaMalloc(&m->d_status, sizeof(unsigned int)), "alloc status"));
  MCHK(cuda(cudaMemset(m->d_status, 0, sizeof(unsigned int)), "memset"));
  if (precision == JGCM_TF32X3 || precision == JGCM_BF16X3) MCHK(tc_tables_build(m));
#undef MCHK
  m->refs = 1;
  cudaGetDevice(&m->device);
  *out = m;
  return JGCM_OK;
}

namespace jgcm {
void mesh_retain(jgcm_mesh* m) { m->refs++; }
void mesh_release(jgcm_mesh* m) {
  if (--m->refs > 0) return;
  cudaStreamSynchronize(m->stream);
  mesh_free(m);
}
}  // namespace jgcm

// Models hold a reference, so a mesh released before its models stays alive until the
// last of them is destroyed (host garbage collectors may finalise in any order).
extern "C" int jgcm_mesh_destroy(jgcm_mesh* m) {
  if (!m) return JGCM_OK;
  mesh_release(m);
  return JGCM_OK;
}

extern "C" int jgcm_mesh_precision(const jgcm_mesh* m) { return m ? m->precision : JGCM_E_ARG; }

// Also reports what the asynchronous entry points cannot: a tensor-core Legendre kernel whose bounded
// wait gave up since the last check (its output is then not a transform; JGCM_E_CUDA with a message,
// and the status is cleared).
extern "C" int jgcm_mesh_synchronize(jgcm_mesh* m) {
  JG_ARG(m, "mesh is NULL");
  JG_CUDA(cudaStreamSynchronize(m->stream));
  if (m->tc.on) JG_TRY(jgcm::tc_status(m));
  return JGCM_OK;
}

// Export a table in the reference layout (FP64).
extern "C" int jgcm_mesh_table(jgcm_mesh* m, const char* name, double* out, long cap, long* count) {
  JG_ARG(m && name, "mesh or name is NULL");
  int N = m->N, ns = m->ns, nlat = m->nlat, nlon = m->nlon;
  long T3 = (long)(N + 1) * (ns + 1) * nlat, T2 = (long)(N + 1) * (ns + 1);
  std::string nm(name);
  std::vector<double> sinth(nlat), wts(nlat);
  JG_CUDA(cudaMemcpy(sinth.data(), m->d_sinth, nlat * 8, cudaMemcpyDeviceToHost));
  JG_CUDA(cudaMemcpy(wts.data(), m->d_wts, nlat * 8, cudaMemcpyDeviceToHost));
  std::vector<double> res;
  auto want3 = [&]() -> int {
    std::vector<double> q(T3), dq(T3);
    JG_CUDA(cudaMemcpy(q.data(), m->d_qnm, T3 * 8, cudaMemcpyDeviceToHost));
    JG_CUDA(cudaMemcpy(dq.data(), m->d_dqnm, T3 * 8, cudaMemcpyDeviceToHost));
    res.assign(T3, 0.0);
    for (int j = 0; j < nlat; j++) {
      double c = std::sqrt(1 - sinth[j] * sinth[j]);
      for (int n = 0; n <= ns; n++)
        for (int mm = 0; mm <= N; mm++) {
          long r = mm + (long)(N + 1) * (n + (long)(ns + 1) * j);
          if (nm == "qnm") res[r] = q[r];
          else if (nm == "dqnm") res[r] = dq[r];
          else if (nm == "qwg") res[r] = q[r] * wts[j];
          else if (nm == "coef_alp_a") res[r] = (n >= mm) ? wts[j] * q[r] / (c * c) * mm : 0.0;
          else if (nm == "coef_alp_b") res[r] = (n >= mm) ? -wts[j] * dq[r] : 0.0;
        }
    }
    return JGCM_OK;
  };
  auto want2 = [&](const double* dptr) -> int {
    std::vector<double> t(T2);
    JG_CUDA(cudaMemcpy(t.data(), dptr, T2 * 8, cudaMemcpyDeviceToHost));
    res.assign(T2, 0.0);
    for (int mm = 0; mm <= N; mm++)
      for (int n = 0; n <= ns; n++) res[mm + (long)(N + 1) * n] = t[(long)mm * (ns + 1) + n];
    return JGCM_OK;
  };
  if (nm == "sinth") res = sinth;
  else if (nm == "wts") res = wts;
  else if (nm == "costh") {
    res.resize(nlat);
    for (int j = 0; j < nlat; j++) res[j] = std::sqrt(1 - sinth[j] * sinth[j]);
  } else if (nm == "latc") {
    res.resize(nlat);
    for (int j = 0; j < nlat; j++) res[j] = std::asin(sinth[j]);
  } else if (nm == "lonc") {
    res.resize(nlon);
    for (int i = 0; i < nlon; i++) {
      double t = (double)i / (double)nlon;
      res[i] = (1 - t) * 0.0 + t * (2 * M_PI);
    }
  } else if (nm == "qnm" || nm == "dqnm" || nm == "qwg" || nm == "coef_alp_a" || nm == "coef_alp_b") {
    JG_TRY(want3());
  } else if (nm == "coef_dlam") JG_TRY(want2(m->t64.dlam));
  else if (nm == "coef_dthm") JG_TRY(want2(m->t64.dthm));
  else if (nm == "coef_dthp") JG_TRY(want2(m->t64.dthp));
  else if (nm == "coef_uvm") JG_TRY(want2(m->t64.uvm));
  else if (nm == "coef_uvc") JG_TRY(want2(m->t64.uvc));
  else if (nm == "coef_uvp") JG_TRY(want2(m->t64.uvp));
  else if (nm == "laplacian_eig") JG_TRY(want2(m->t64.eig));
  else if (nm == "epsilon") {
    res.assign(T2, 0.0);
    for (int mm = 0; mm <= N; mm++)
      for (int n = mm; n <= ns; n++)
        res[mm + (long)(N + 1) * n] = std::sqrt((double)(n * n - mm * mm) / (4.0 * n * n - 1.0));
  } else {
    set_error("unknown mesh table '%s'", name);
    return JGCM_E_ARG;
  }
  if (count) *count = (long)res.size();
  if (out) {
    JG_ARG(cap >= (long)res.size(), "buffer too small for table '%s'", name);
    memcpy(out, res.data(), res.size() * 8);
  }
  return JGCM_OK;
}
