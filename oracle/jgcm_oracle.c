/*
 * jgcm_oracle.c -- FP64 CPU oracle (TEST INFRASTRUCTURE ONLY; see jgcm_oracle.h).
 *
 * Every function below restates one reference function, cited by file:line inside
 * CliMA/IdealizedSpectralGCM.jl.  Operation order follows the reference expression by
 * expression (compiled with -ffp-contract=off so x86 and Arm agree) so that the
 * FP64 GPU path can be compared at rounding level.  The reference's quirks are kept:
 * the extra total wavenumber N+1 is summed by spectral->grid and zeroed by
 * grid->spectral; physics runs on the previous time level; the first step is a
 * forward step with wave matrices rebuilt afterwards.
 */
#include "jgcm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI 3.14159265358979323846

struct om_mesh {
  int N, ns, nlon, nlat, nd;
  double radius;
  double *sinth, *costh, *wts, *lonc, *latc;
  double *qnm, *dqnm, *qwg;   /* (N+1)*(ns+1)*nlat */
  double* epsilon;            /* (N+1)*(ns+1) */
  double *coef_alp_a, *coef_alp_b;
  double *coef_uvm, *coef_uvc, *coef_uvp;
  double *coef_dlam, *coef_dthm, *coef_dthp;
  double* laplacian_eig;
  /* FFT support */
  double* tw;   /* cos/sin of 2*pi*t/nlon, t < nlon */
  int* bitrev;
  int pow2;
};

static int g_threads = 0;
void om_set_threads(int n) { g_threads = n; }
#ifdef _OPENMP
#define OMP_THREADS (g_threads > 0 ? g_threads : omp_get_max_threads())
#endif

static double* zalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* FP32 emulation switches (jgcm_oracle.h); 0 = the FP64 restatement of the reference */
static int g_f32 = 0;
void om_set_f32(int mask) { g_f32 = mask; }
static inline double r32(double x) { return (double)(float)x; }
/* a + b c rounded once to float: b, c are floats, so their product is exact in double */
static inline double fma32(double a, double b, double c) { return r32(a + r32(b) * r32(c)); }
static void r32_arr(double* a, size_t n) {
  for (size_t i = 0; i < n; i++) a[i] = r32(a[i]);
}

#define TIX(m, n, j) ((size_t)(m) + (size_t)(N + 1) * ((size_t)(n) + (size_t)(ns + 1) * (size_t)(j)))
#define SIX(m, n, k) (2 * ((size_t)(m) + (size_t)(N + 1) * ((size_t)(n) + (size_t)(ns + 1) * (size_t)(k))))
#define GIX(i, j, k) ((size_t)(i) + (size_t)nlon * ((size_t)(j) + (size_t)nlat * (size_t)(k)))

/* ------------------------------------------------------------------------------------------ */
/* Gauss_And_Legendre.jl:69-118  Compute_Gaussian!                                             */
int om_compute_gaussian(int n, double* sinth, double* wts) {
  const int itermax = 10000;
  const double tol = 1.0e-15;
  int n_half = n / 2, ok = 0;
  for (int i = 1; i <= n_half; i++) {
    double dp = 0.0;
    double z = cos(PI * (i - 0.25) / (n + 0.5));
    for (int iter = 1; iter <= itermax; iter++) {
      double p2 = 0.0, p1 = 1.0, p3;
      for (int j = 1; j <= n; j++) {
        p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      dp = n * (z * p1 - p2) / (z * z - 1.0);
      double z1 = z;
      z = z1 - p1 / dp;
      if (fabs(z - z1) <= tol) break;
      if (iter == itermax) ok = -1; /* reference: @error("Compute_Gaussian! does not converge!") */
    }
    sinth[i - 1] = -z;
    sinth[n - i] = z;
    wts[i - 1] = wts[n - i] = 2.0 / ((1.0 - z * z) * dp * dp);
  }
  return ok;
}

/* Gauss_And_Legendre.jl:4-66  Compute_Legendre! ; qnm/dqnm are (N+1)*(ns+1)*nlat */
int om_compute_legendre(int N, int ns, const double* sinth, int nlat, double* qnm_out, double* dqnm) {
  int nsf = ns + 2; /* internal qnm has num_spherical+2 columns */
  double* q = zalloc((size_t)(N + 1) * nsf * nlat);
  double* eps = zalloc((size_t)(N + 1) * nsf);
  double* c = zalloc(nlat);
#define QF(m, l, j) q[(size_t)(m) + (size_t)(N + 1) * ((size_t)(l) + (size_t)nsf * (size_t)(j))]
#define EF(m, l) eps[(size_t)(m) + (size_t)(N + 1) * (size_t)(l)]
  for (int j = 0; j < nlat; j++) c[j] = sqrt(1 - sinth[j] * sinth[j]);
  for (int j = 0; j < nlat; j++) QF(0, 0, j) = 1.0;
  for (int m = 1; m <= N; m++)
    for (int j = 0; j < nlat; j++) QF(m, m, j) = sqrt((2.0 * m + 1) / (2.0 * m)) * c[j] * QF(m - 1, m - 1, j);
  for (int m1 = 1; m1 <= N + 1; m1++) /* qnm[m, m+1, :] = sqrt(2m+1) sin qnm[m,m,:] (1-based m) */
    for (int j = 0; j < nlat; j++) QF(m1 - 1, m1, j) = sqrt((double)(2 * m1 + 1)) * sinth[j] * QF(m1 - 1, m1 - 1, j);
  for (int m = 0; m <= N; m++)
    for (int l = m; l <= ns + 1; l++)
      EF(m, l) = sqrt((double)(l * l - m * m) / (double)(4 * l * l - 1));
  for (int m = 0; m <= N; m++)
    for (int l = m + 2; l <= ns + 1; l++)
      for (int j = 0; j < nlat; j++)
        QF(m, l, j) = (sinth[j] * QF(m, l - 1, j) - EF(m, l - 1) * QF(m, l - 2, j)) / EF(m, l);
  memset(dqnm, 0, sizeof(double) * (size_t)(N + 1) * (ns + 1) * nlat);
  for (int m = 0; m <= N; m++)
    for (int l = m; l <= ns; l++)
      for (int j = 0; j < nlat; j++) {
        double val;
        if (l == m)
          val = ((double)(-l) * EF(m, l + 1) * QF(m, l + 1, j)) / (c[j] * c[j]);
        else
          val = ((double)(-l) * EF(m, l + 1) * QF(m, l + 1, j) + (double)(l + 1) * EF(m, l) * QF(m, l - 1, j)) /
                (c[j] * c[j]);
        dqnm[TIX(m, l, j)] = val;
      }
  for (int j = 0; j < nlat; j++)
    for (int l = 0; l <= ns; l++)
      for (int m = 0; m <= N; m++) qnm_out[TIX(m, l, j)] = QF(m, l, j);
#undef QF
#undef EF
  free(q);
  free(eps);
  free(c);
  return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* FFT (stand-in for FFTW.jl fft/ifft, unpinned third-party boundary): radix-2 for powers of  */
/* two, plain DFT otherwise.  sign=-1 forward (fft), +1 backward (unnormalised ifft).         */
static void fft_inplace_f32(const om_mesh* M, double* re, double* im, int sign);
static void fft_inplace(const om_mesh* M, double* re, double* im, int sign) {
  int n = M->nlon;
  if (M->pow2 && (g_f32 & (sign < 0 ? OM_F32_FFT_FWD : OM_F32_FFT_INV))) {
    fft_inplace_f32(M, re, im, sign);
    return;
  }
  if (M->pow2) {
    for (int i = 0; i < n; i++) {
      int r = M->bitrev[i];
      if (r > i) {
        double t = re[i]; re[i] = re[r]; re[r] = t;
        t = im[i]; im[i] = im[r]; im[r] = t;
      }
    }
    for (int len = 2; len <= n; len <<= 1) {
      int half = len >> 1, step = n / len;
      for (int i = 0; i < n; i += len)
        for (int k = 0; k < half; k++) {
          double wr = M->tw[2 * (k * step)], wi = sign * M->tw[2 * (k * step) + 1];
          double xr = re[i + k + half], xi = im[i + k + half];
          double tr = xr * wr - xi * wi, ti = xr * wi + xi * wr;
          re[i + k + half] = re[i + k] - tr;
          im[i + k + half] = im[i + k] - ti;
          re[i + k] = re[i + k] + tr;
          im[i + k] = im[i + k] + ti;
        }
    }
  } else {
    double* ore = zalloc(n);
    double* oim = zalloc(n);
    for (int k = 0; k < n; k++) {
      double sr = 0, si = 0;
      for (int t = 0; t < n; t++) {
        int idx = (int)(((long)k * t) % n);
        double wr = M->tw[2 * idx], wi = sign * M->tw[2 * idx + 1];
        sr += re[t] * wr - im[t] * wi;
        si += re[t] * wi + im[t] * wr;
      }
      ore[k] = sr;
      oim[k] = si;
    }
    memcpy(re, ore, sizeof(double) * n);
    memcpy(im, oim, sizeof(double) * n);
    free(ore);
    free(oim);
  }
}

/* The radix-2 FFT above in FP32 arithmetic (FP32 emulation, not the reference's FP64). */
static void fft_inplace_f32(const om_mesh* M, double* re, double* im, int sign) {
  int n = M->nlon;
  float* a = (float*)calloc((size_t)n, sizeof(float));
  float* b = (float*)calloc((size_t)n, sizeof(float));
  for (int i = 0; i < n; i++) {
    a[M->bitrev[i]] = (float)re[i];
    b[M->bitrev[i]] = (float)im[i];
  }
  for (int len = 2; len <= n; len <<= 1) {
    int half = len >> 1, step = n / len;
    for (int i = 0; i < n; i += len)
      for (int k = 0; k < half; k++) {
        float wr = (float)M->tw[2 * (k * step)], wi = (float)(sign * M->tw[2 * (k * step) + 1]);
        float xr = a[i + k + half], xi = b[i + k + half];
        float tr = xr * wr - xi * wi, ti = xr * wi + xi * wr;
        a[i + k + half] = a[i + k] - tr;
        b[i + k + half] = b[i + k] - ti;
        a[i + k] = a[i + k] + tr;
        b[i + k] = b[i + k] + ti;
      }
  }
  for (int i = 0; i < n; i++) {
    re[i] = a[i];
    im[i] = b[i];
  }
  free(a);
  free(b);
}

/* ------------------------------------------------------------------------------------------ */
/* Spectral_Spherical_Mesh.jl:396-422 Compute_Alpha_Operator_Init                             */
static void alpha_init(om_mesh* M) {
  int N = M->N, ns = M->ns, nlat = M->nlat;
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= ns; n++)
      for (int j = 0; j < nlat; j++) {
        M->coef_alp_a[TIX(m, n, j)] = M->wts[j] * M->qnm[TIX(m, n, j)] / (M->costh[j] * M->costh[j]) * m;
        M->coef_alp_b[TIX(m, n, j)] = -M->wts[j] * M->dqnm[TIX(m, n, j)];
      }
}

/* Spectral_Spherical_Mesh.jl:69-139 mesh constructor (+ :485-515, :583-613, :625-652 inits) */
om_mesh* om_mesh_create(int N, int ns, int nlat, int nlon, int nd, double radius) {
  if (N < 0 || ns != N + 1 || nlat < 2 || (nlat % 2) || nlon < 2 * N + 1 || nd < 1) return NULL;
  om_mesh* M = (om_mesh*)calloc(1, sizeof(om_mesh));
  M->N = N; M->ns = ns; M->nlat = nlat; M->nlon = nlon; M->nd = nd; M->radius = radius;
  size_t T3 = (size_t)(N + 1) * (ns + 1) * nlat, T2 = (size_t)(N + 1) * (ns + 1);
  M->sinth = zalloc(nlat); M->costh = zalloc(nlat); M->wts = zalloc(nlat);
  M->lonc = zalloc(nlon); M->latc = zalloc(nlat);
  M->qnm = zalloc(T3); M->dqnm = zalloc(T3); M->qwg = zalloc(T3);
  M->coef_alp_a = zalloc(T3); M->coef_alp_b = zalloc(T3);
  M->epsilon = zalloc(T2);
  M->coef_uvm = zalloc(T2); M->coef_uvc = zalloc(T2); M->coef_uvp = zalloc(T2);
  M->coef_dlam = zalloc(T2); M->coef_dthm = zalloc(T2); M->coef_dthp = zalloc(T2);
  M->laplacian_eig = zalloc(T2);
  om_compute_gaussian(nlat, M->sinth, M->wts);
  om_compute_legendre(N, ns, M->sinth, nlat, M->qnm, M->dqnm);
  for (int j = 0; j < nlat; j++) M->costh[j] = sqrt(1 - M->sinth[j] * M->sinth[j]);
  for (int i = 0; i < nlon; i++) { /* LinRange(0, 2pi, nlon+1)[1:nlon] */
    double t = (double)i / (double)nlon;
    M->lonc[i] = (1 - t) * 0.0 + t * (2 * PI);
  }
  for (int j = 0; j < nlat; j++) M->latc[j] = asin(M->sinth[j]);
  for (int j = 0; j < nlat; j++)
    for (size_t mn = 0; mn < T2; mn++) M->qwg[mn + T2 * j] = M->qnm[mn + T2 * j] * M->wts[j];
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= ns; n++)
      M->epsilon[m + (N + 1) * n] = sqrt((double)(n * n - m * m) / (4.0 * n * n - 1.0));
  alpha_init(M);
  /* :485-515 Compute_Ucos_Vcos_From_Vor_Div_Init */
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= ns; n++)
      if (n > 0) M->coef_uvc[m + (N + 1) * n] = -radius * m / (double)(n * (n + 1));
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= ns; n++)
      if (n > 0) M->coef_uvm[m + (N + 1) * n] = radius * M->epsilon[m + (N + 1) * n] / n;
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= ns - 1; n++)
      M->coef_uvp[m + (N + 1) * n] = -radius * M->epsilon[m + (N + 1) * (n + 1)] / (n + 1);
  /* :625-652 Compute_Gradient_Cos_Init */
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= ns; n++) {
      M->coef_dlam[m + (N + 1) * n] = m / radius;
      M->coef_dthm[m + (N + 1) * n] = -(n - 1) * M->epsilon[m + (N + 1) * n] / radius;
    }
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= ns - 1; n++)
      M->coef_dthp[m + (N + 1) * n] = (n + 2) * M->epsilon[m + (N + 1) * (n + 1)] / radius;
  /* :599-613 Apply_Laplacian_Init */
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= ns; n++) M->laplacian_eig[m + (N + 1) * n] = (double)(-n * (n + 1)) / (radius * radius);
  /* FFT tables */
  M->tw = zalloc(2 * (size_t)nlon);
  for (int t = 0; t < nlon; t++) {
    M->tw[2 * t] = cos(2 * PI * t / nlon);
    M->tw[2 * t + 1] = sin(2 * PI * t / nlon);
  }
  M->pow2 = (nlon & (nlon - 1)) == 0;
  M->bitrev = (int*)calloc(nlon, sizeof(int));
  if (M->pow2) {
    int lg = 0;
    while ((1 << lg) < nlon) lg++;
    for (int i = 0; i < nlon; i++) {
      int r = 0;
      for (int b = 0; b < lg; b++)
        if (i & (1 << b)) r |= 1 << (lg - 1 - b);
      M->bitrev[i] = r;
    }
  }
  return M;
}

void om_mesh_destroy(om_mesh* M) {
  if (!M) return;
  double* ptrs[] = {M->sinth, M->costh, M->wts, M->lonc, M->latc, M->qnm, M->dqnm, M->qwg, M->epsilon,
                    M->coef_alp_a, M->coef_alp_b, M->coef_uvm, M->coef_uvc, M->coef_uvp, M->coef_dlam,
                    M->coef_dthm, M->coef_dthp, M->laplacian_eig, M->tw};
  for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); i++) free(ptrs[i]);
  free(M->bitrev);
  free(M);
}

long om_mesh_table(const om_mesh* M, const char* name, double* out, long cap) {
  long T3 = (long)(M->N + 1) * (M->ns + 1) * M->nlat, T2 = (long)(M->N + 1) * (M->ns + 1);
  struct { const char* nm; const double* p; long n; } tab[] = {
      {"sinth", M->sinth, M->nlat}, {"costh", M->costh, M->nlat}, {"wts", M->wts, M->nlat},
      {"lonc", M->lonc, M->nlon}, {"latc", M->latc, M->nlat}, {"qnm", M->qnm, T3},
      {"dqnm", M->dqnm, T3}, {"qwg", M->qwg, T3}, {"epsilon", M->epsilon, T2},
      {"coef_alp_a", M->coef_alp_a, T3}, {"coef_alp_b", M->coef_alp_b, T3},
      {"coef_uvm", M->coef_uvm, T2}, {"coef_uvc", M->coef_uvc, T2}, {"coef_uvp", M->coef_uvp, T2},
      {"coef_dlam", M->coef_dlam, T2}, {"coef_dthm", M->coef_dthm, T2}, {"coef_dthp", M->coef_dthp, T2},
      {"laplacian_eig", M->laplacian_eig, T2}};
  for (size_t i = 0; i < sizeof(tab) / sizeof(tab[0]); i++)
    if (!strcmp(tab[i].nm, name)) {
      if (out && cap >= tab[i].n) memcpy(out, tab[i].p, sizeof(double) * tab[i].n);
      return tab[i].n;
    }
  return -1;
}

/* ------------------------------------------------------------------------------------------ */
/* Spectral_Spherical_Mesh.jl:143-217 Trans_Spherical_To_Grid!                                */
void om_trans_spherical_to_grid(om_mesh* M, const double* snm, int nlev, double* pfield) {
  int N = M->N, ns = M->ns, nlat = M->nlat, nlon = M->nlon, nh = nlat / 2;
  /* fourier_g / fourier_s hold only m = 0..N (higher rows are zero in the reference) */
  double* g = zalloc(2 * (size_t)(N + 1) * nlat * nlev);
#define FG(m, j, k) g[2 * ((size_t)(m) + (size_t)(N + 1) * ((size_t)(j) + (size_t)nlat * (size_t)(k)))]
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic) num_threads(OMP_THREADS)
#endif
  for (int m = 0; m <= N; m++) {
    double* s = zalloc(2 * (size_t)nlat * nlev); /* fourier_s[m, :, :] */
    for (int n = m; n <= ns; n++) {
      int off = ((n - m) % 2 == 0) ? 0 : nh;
      for (int k = 0; k < nlev; k++) {
        double sr = snm[SIX(m, n, k)], si = snm[SIX(m, n, k) + 1];
        for (int j = 0; j < nh; j++) {
          double q = M->qnm[TIX(m, n, j)];
          double* d = &s[2 * ((size_t)(off + j) + (size_t)nlat * k)];
          if (g_f32 & OM_F32_SYNTHESIS) {
            d[0] = fma32(d[0], q, sr);
            d[1] = fma32(d[1], q, si);
          } else {
            d[0] = d[0] + q * sr;
            d[1] = d[1] + q * si;
          }
        }
      }
    }
    for (int k = 0; k < nlev; k++)
      for (int j = 0; j < nh; j++) {
        double* e = &s[2 * ((size_t)j + (size_t)nlat * k)];
        double* o = &s[2 * ((size_t)(nh + j) + (size_t)nlat * k)];
        (&FG(m, j, k))[0] = e[0] + o[0];
        (&FG(m, j, k))[1] = e[1] + o[1];
        (&FG(m, nlat - 1 - j, k))[0] = e[0] - o[0];
        (&FG(m, nlat - 1 - j, k))[1] = e[1] - o[1];
        if (g_f32 & OM_F32_SYNTHESIS) {
          r32_arr(&FG(m, j, k), 2);
          r32_arr(&FG(m, nlat - 1 - j, k), 2);
        }
      }
    free(s);
  }
  for (int k = 0; k < nlev; k++)
    for (int j = 0; j < nlat; j++) {
      (&FG(0, j, k))[0] /= 2.0;
      (&FG(0, j, k))[1] /= 2.0;
    }
#ifdef _OPENMP
#pragma omp parallel for num_threads(OMP_THREADS)
#endif
  for (int kj = 0; kj < nlev * nlat; kj++) {
    int k = kj / nlat, j = kj % nlat;
    double* re = zalloc(nlon);
    double* im = zalloc(nlon);
    for (int m = 0; m <= N; m++) {
      re[m] = (&FG(m, j, k))[0];
      im[m] = (&FG(m, j, k))[1];
    }
    fft_inplace(M, re, im, +1);
    for (int i = 0; i < nlon; i++) pfield[GIX(i, j, k)] = 2.0 * nlon * (re[i] / nlon);
    if (g_f32 & OM_F32_FFT_INV)
      for (int i = 0; i < nlon; i++) pfield[GIX(i, j, k)] = r32(pfield[GIX(i, j, k)]);
    free(re);
    free(im);
  }
#undef FG
  free(g);
}

/* Spectral_Spherical_Mesh.jl:295-330 Trans_Grid_To_Fourier! (fft/nlon over all nlon modes) */
void om_trans_grid_to_fourier(om_mesh* M, const double* pfield, int nlev, double* fourier) {
  int nlat = M->nlat, nlon = M->nlon;
#ifdef _OPENMP
#pragma omp parallel for num_threads(OMP_THREADS)
#endif
  for (int kj = 0; kj < nlev * nlat; kj++) {
    int k = kj / nlat, j = kj % nlat;
    double* re = zalloc(nlon);
    double* im = zalloc(nlon);
    for (int i = 0; i < nlon; i++) re[i] = pfield[GIX(i, j, k)];
    fft_inplace(M, re, im, -1);
    for (int i = 0; i < nlon; i++) {
      fourier[2 * GIX(i, j, k)] = re[i] / nlon;
      fourier[2 * GIX(i, j, k) + 1] = im[i] / nlon;
    }
    if (g_f32 & OM_F32_FFT_FWD)
      for (int i = 0; i < nlon; i++) r32_arr(&fourier[2 * GIX(i, j, k)], 2);
    free(re);
    free(im);
  }
}

/* Spectral_Spherical_Mesh.jl:221-293 Trans_Grid_To_Spherical! */
void om_trans_grid_to_spherical(om_mesh* M, const double* pfield, int nlev, double* snm) {
  int N = M->N, ns = M->ns, nlat = M->nlat, nlon = M->nlon, nh = nlat / 2;
  double* f = zalloc(2 * (size_t)nlon * nlat * nlev);
  om_trans_grid_to_fourier(M, pfield, nlev, f);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic) num_threads(OMP_THREADS)
#endif
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= ns - 1; n++) {
      int even = ((n - m) % 2 == 0);
      for (int k = 0; k < nlev; k++) {
        double sr = 0.0, si = 0.0;
        for (int j = 0; j < nh; j++) {
          const double* a = &f[2 * GIX(m, j, k)];
          const double* b = &f[2 * GIX(m, nlat - 1 - j, k)];
          double q = M->qwg[TIX(m, n, j)];
          double cr = even ? a[0] + b[0] : a[0] - b[0];
          double ci = even ? a[1] + b[1] : a[1] - b[1];
          if (g_f32 & OM_F32_ANALYSIS) {
            sr = fma32(sr, r32(cr), q);
            si = fma32(si, r32(ci), q);
          } else {
            sr = sr + cr * q;
            si = si + ci * q;
          }
        }
        snm[SIX(m, n, k)] = sr / 2.0;
        snm[SIX(m, n, k) + 1] = si / 2.0;
      }
    }
  for (int k = 0; k < nlev; k++)
    for (int m = 0; m <= N; m++) snm[SIX(m, ns, k)] = snm[SIX(m, ns, k) + 1] = 0.0;
  free(f);
}

/* Spectral_Spherical_Mesh.jl:424-459 Compute_Alpha_Operator! (all nlat latitudes, n = m..ns) */
static void alpha_operator(om_mesh* M, const double* fa, const double* fb, double isign, int nlev, double* alpha) {
  int N = M->N, ns = M->ns, nlat = M->nlat, nlon = M->nlon;
  double c = 1 / (2 * M->radius);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic) num_threads(OMP_THREADS)
#endif
  for (int m = 0; m <= N; m++)
    for (int n = m; n <= ns; n++)
      for (int k = 0; k < nlev; k++) {
        double ar = 0, ai = 0, br = 0, bi = 0;
        for (int j = 0; j < nlat; j++) {
          const double* A = &fa[2 * GIX(m, j, k)];
          const double* B = &fb[2 * GIX(m, j, k)];
          double ca = M->coef_alp_a[TIX(m, n, j)], cb = M->coef_alp_b[TIX(m, n, j)];
          /* (imag(A') + real(A') im) = i*A  */
          if (g_f32 & OM_F32_ANALYSIS) {
            ar = fma32(ar, -A[1], ca);
            ai = fma32(ai, A[0], ca);
            br = fma32(br, B[0], cb);
            bi = fma32(bi, B[1], cb);
          } else {
            ar = ar + (-A[1]) * ca;
            ai = ai + A[0] * ca;
            br = br + B[0] * cb;
            bi = bi + B[1] * cb;
          }
        }
        alpha[SIX(m, n, k)] = c * (ar + isign * br);
        alpha[SIX(m, n, k) + 1] = c * (ai + isign * bi);
        if (g_f32 & OM_F32_ANALYSIS) r32_arr(&alpha[SIX(m, n, k)], 2);
      }
}

/* Spectral_Spherical_Mesh.jl:349-393 Vor_Div_From_Grid_UV! */
void om_vor_div_from_grid_uv(om_mesh* M, const double* u, const double* v, int nlev, double* vor, double* div) {
  int N = M->N, ns = M->ns, nlat = M->nlat, nlon = M->nlon;
  size_t G = (size_t)nlon * nlat * nlev;
  double* uc = zalloc(G);
  double* vc = zalloc(G);
  double* fu = zalloc(2 * G);
  double* fv = zalloc(2 * G);
  for (int k = 0; k < nlev; k++)
    for (int j = 0; j < nlat; j++)
      for (int i = 0; i < nlon; i++) {
        uc[GIX(i, j, k)] = u[GIX(i, j, k)] * M->costh[j];
        vc[GIX(i, j, k)] = v[GIX(i, j, k)] * M->costh[j];
      }
  om_trans_grid_to_fourier(M, uc, nlev, fu);
  om_trans_grid_to_fourier(M, vc, nlev, fv);
  alpha_operator(M, fv, fu, -1.0, nlev, vor);
  alpha_operator(M, fu, fv, 1.0, nlev, div);
  for (int k = 0; k < nlev; k++)
    for (int m = 0; m <= N; m++) {
      vor[SIX(m, ns, k)] = vor[SIX(m, ns, k) + 1] = 0.0;
      div[SIX(m, ns, k)] = div[SIX(m, ns, k) + 1] = 0.0;
    }
  free(uc); free(vc); free(fu); free(fv);
}

/* Spectral_Spherical_Mesh.jl:517-580 Compute_Ucos_Vcos_From_Vor_Div! */
void om_compute_ucos_vcos_from_vor_div(om_mesh* M, const double* vor, const double* div, int nlev, double* ucos,
                                       double* vcos) {
  int N = M->N, ns = M->ns;
  for (int k = 0; k < nlev; k++)
    for (int n = 0; n <= ns; n++)
      for (int m = 0; m <= N; m++) {
        double c = M->coef_uvc[m + (N + 1) * n];
        size_t s = SIX(m, n, k);
        ucos[s] = c * (-div[s + 1] + 0.0);
        ucos[s + 1] = c * div[s];
        vcos[s] = c * (-vor[s + 1] + 0.0);
        vcos[s + 1] = c * vor[s];
      }
  for (int k = 0; k < nlev; k++) /* .-= coef_uvm[:,2:ns+1] .* vor[:,1:ns] */
    for (int n = 1; n <= ns; n++)
      for (int m = 0; m <= N; m++) {
        double c = M->coef_uvm[m + (N + 1) * n];
        size_t s = SIX(m, n, k), sm = SIX(m, n - 1, k);
        ucos[s] = ucos[s] - c * vor[sm];
        ucos[s + 1] = ucos[s + 1] - c * vor[sm + 1];
      }
  for (int k = 0; k < nlev; k++)
    for (int n = 0; n <= ns - 1; n++)
      for (int m = 0; m <= N; m++) {
        double c = M->coef_uvp[m + (N + 1) * n];
        size_t s = SIX(m, n, k), sp = SIX(m, n + 1, k);
        ucos[s] = ucos[s] - c * vor[sp];
        ucos[s + 1] = ucos[s + 1] - c * vor[sp + 1];
      }
  for (int k = 0; k < nlev; k++)
    for (int n = 1; n <= ns; n++)
      for (int m = 0; m <= N; m++) {
        double c = M->coef_uvm[m + (N + 1) * n];
        size_t s = SIX(m, n, k), sm = SIX(m, n - 1, k);
        vcos[s] = vcos[s] + c * div[sm];
        vcos[s + 1] = vcos[s + 1] + c * div[sm + 1];
      }
  for (int k = 0; k < nlev; k++)
    for (int n = 0; n <= ns - 1; n++)
      for (int m = 0; m <= N; m++) {
        double c = M->coef_uvp[m + (N + 1) * n];
        size_t s = SIX(m, n, k), sp = SIX(m, n + 1, k);
        vcos[s] = vcos[s] + c * div[sp];
        vcos[s + 1] = vcos[s + 1] + c * div[sp + 1];
      }
}

static void divide_by_cos(om_mesh* M, double* g, int nlev) { /* :333-339 */
  int nlat = M->nlat, nlon = M->nlon;
  for (int k = 0; k < nlev; k++)
    for (int j = 0; j < nlat; j++)
      for (int i = 0; i < nlon; i++) g[GIX(i, j, k)] /= M->costh[j];
}

/* Spectral_Spherical_Mesh.jl:462-482 UV_Grid_From_Vor_Div! */
void om_uv_grid_from_vor_div(om_mesh* M, const double* vor, const double* div, int nlev, double* u, double* v) {
  size_t S = 2 * (size_t)(M->N + 1) * (M->ns + 1) * nlev;
  double* uc = zalloc(S);
  double* vc = zalloc(S);
  om_compute_ucos_vcos_from_vor_div(M, vor, div, nlev, uc, vc);
  om_trans_spherical_to_grid(M, uc, nlev, u);
  om_trans_spherical_to_grid(M, vc, nlev, v);
  divide_by_cos(M, u, nlev);
  divide_by_cos(M, v, nlev);
  free(uc);
  free(vc);
}

/* Spectral_Spherical_Mesh.jl:655-692 Compute_Gradient_Cos! */
void om_compute_gradient_cos(om_mesh* M, const double* hs, int nlev, double* dl, double* dt) {
  int N = M->N, ns = M->ns;
  for (int k = 0; k < nlev; k++)
    for (int n = 0; n <= ns; n++)
      for (int m = 0; m <= N; m++) {
        double c = M->coef_dlam[m + (N + 1) * n];
        size_t s = SIX(m, n, k);
        dl[s] = c * (-hs[s + 1] + 0.0);
        dl[s + 1] = c * hs[s];
      }
  for (int k = 0; k < nlev; k++)
    for (int m = 0; m <= N; m++) dt[SIX(m, ns, k)] = dt[SIX(m, ns, k) + 1] = 0.0;
  for (int k = 0; k < nlev; k++)
    for (int n = 0; n <= ns - 1; n++)
      for (int m = 0; m <= N; m++) {
        double c = M->coef_dthp[m + (N + 1) * n];
        size_t s = SIX(m, n, k), sp = SIX(m, n + 1, k);
        dt[s] = c * hs[sp];
        dt[s + 1] = c * hs[sp + 1];
      }
  for (int k = 0; k < nlev; k++)
    for (int n = 1; n <= ns; n++)
      for (int m = 0; m <= N; m++) {
        double c = M->coef_dthm[m + (N + 1) * n];
        size_t s = SIX(m, n, k), sm = SIX(m, n - 1, k);
        dt[s] = dt[s] + c * hs[sm];
        dt[s + 1] = dt[s + 1] + c * hs[sm + 1];
      }
}

/* Spectral_Spherical_Mesh.jl:721-741 Compute_Gradients! */
void om_compute_gradients(om_mesh* M, const double* hs, int nlev, double* gdl, double* gdt) {
  size_t S = 2 * (size_t)(M->N + 1) * (M->ns + 1) * nlev;
  double* sl = zalloc(S);
  double* st = zalloc(S);
  om_compute_gradient_cos(M, hs, nlev, sl, st);
  om_trans_spherical_to_grid(M, sl, nlev, gdl);
  om_trans_spherical_to_grid(M, st, nlev, gdt);
  divide_by_cos(M, gdl, nlev);
  divide_by_cos(M, gdt, nlev);
  free(sl);
  free(st);
}

/* Spectral_Spherical_Mesh.jl:694-718 Add_Horizontal_Advection! */
void om_add_horizontal_advection(om_mesh* M, const double* hs, const double* u, const double* v, int nlev,
                                 double* dh) {
  size_t G = (size_t)M->nlon * M->nlat * nlev;
  double* gl = zalloc(G);
  double* gt = zalloc(G);
  om_compute_gradients(M, hs, nlev, gl, gt);
  for (size_t x = 0; x < G; x++) dh[x] = dh[x] - (u[x] * gl[x] + v[x] * gt[x]);
  free(gl);
  free(gt);
}

/* Spectral_Spherical_Mesh.jl:614-621 Apply_Laplacian! */
void om_apply_laplacian(om_mesh* M, double* spe, int nlev) {
  size_t T2 = (size_t)(M->N + 1) * (M->ns + 1);
  for (int k = 0; k < nlev; k++)
    for (size_t mn = 0; mn < T2; mn++) {
      spe[2 * (mn + T2 * k)] = M->laplacian_eig[mn] * spe[2 * (mn + T2 * k)];
      spe[2 * (mn + T2 * k) + 1] = M->laplacian_eig[mn] * spe[2 * (mn + T2 * k) + 1];
    }
}

/* Spectral_Spherical_Mesh.jl:746-760 Area_Weighted_Global_Mean (level 1 only) */
double om_area_weighted_global_mean(om_mesh* M, const double* g) {
  int nlat = M->nlat, nlon = M->nlon;
  double total = 0.0;
  for (int i = 0; i < nlon; i++) {
    double r = 0.0;
    for (int j = 0; j < nlat; j++) r = r + g[GIX(i, j, 0)] * M->wts[j];
    total = total + r;
  }
  return total / (2.0 * nlon);
}

#include "jgcm_oracle_models.inc"

/* ---- adjoints of the two transforms (test infrastructure for the differentiation pattern) ------
 * Written directly from the forward definitions on every latitude (no parity folding, no FFT):
 *   S2G: g(lam_t, mu_j) = sum_m c_m Re( sum_n s_mn P_n^m(mu_j) e^{i m lam_t} ),  c_0 = 1, c_m = 2,
 *        Im s_0n does not reach the grid (Spectral_Spherical_Mesh.jl:143-217);
 *   G2S: s_mn = 1/2 sum_j w_j P_n^m(mu_j) (1/nlon) sum_t g e^{-i m lam_t}, n <= N, row N+1 = 0
 *        (Spectral_Spherical_Mesh.jl:221-293). */
void om_trans_spherical_to_grid_adjoint(om_mesh* M, const double* gbar, int nlev, double* sbar) {
  int N = M->N, ns = M->ns, nlat = M->nlat, nlon = M->nlon;
  memset(sbar, 0, 2 * sizeof(double) * (size_t)(N + 1) * (ns + 1) * nlev);
#ifdef _OPENMP
#pragma omp parallel for num_threads(OMP_THREADS)
#endif
  for (int k = 0; k < nlev; k++) {
    double* Gc = zalloc((size_t)(N + 1) * nlat);
    double* Gs = zalloc((size_t)(N + 1) * nlat);
    for (int j = 0; j < nlat; j++)
      for (int m = 0; m <= N; m++) {
        double c = 0.0, sn = 0.0;
        for (int t = 0; t < nlon; t++) {
          double a = 6.283185307179586476925287 * (double)(((long)m * t) % nlon) / (double)nlon;
          double x = gbar[(size_t)t + (size_t)nlon * ((size_t)j + (size_t)nlat * k)];
          c += x * cos(a);
          sn += x * sin(a);
        }
        Gc[m + (size_t)(N + 1) * j] = c;
        Gs[m + (size_t)(N + 1) * j] = sn;
      }
    for (int m = 0; m <= N; m++) {
      double cm = m == 0 ? 1.0 : 2.0;
      for (int n = m; n <= ns; n++) {
        double re = 0.0, im = 0.0;
        for (int j = 0; j < nlat; j++) {
          double q = M->qnm[TIX(m, n, j)];
          re += q * Gc[m + (size_t)(N + 1) * j];
          im -= q * Gs[m + (size_t)(N + 1) * j];
        }
        sbar[SIX(m, n, k)] = cm * re;
        sbar[SIX(m, n, k) + 1] = m == 0 ? 0.0 : cm * im;
      }
    }
    free(Gc);
    free(Gs);
  }
}

void om_trans_grid_to_spherical_adjoint(om_mesh* M, const double* sbar, int nlev, double* gbar) {
  int N = M->N, ns = M->ns, nlat = M->nlat, nlon = M->nlon;
#ifdef _OPENMP
#pragma omp parallel for collapse(2) num_threads(OMP_THREADS)
#endif
  for (int k = 0; k < nlev; k++)
    for (int j = 0; j < nlat; j++) {
      double* a_re = zalloc(N + 1);
      double* a_im = zalloc(N + 1);
      for (int m = 0; m <= N; m++)
        for (int n = m; n <= N && n < ns; n++) {
          double q = M->qnm[TIX(m, n, j)];
          a_re[m] += q * sbar[SIX(m, n, k)];
          a_im[m] += q * sbar[SIX(m, n, k) + 1];
        }
      double sc = M->wts[j] / (2.0 * nlon);
      for (int t = 0; t < nlon; t++) {
        double g = 0.0;
        for (int m = 0; m <= N; m++) {
          double a = 6.283185307179586476925287 * (double)(((long)m * t) % nlon) / (double)nlon;
          g += a_re[m] * cos(a) - a_im[m] * sin(a);
        }
        gbar[(size_t)t + (size_t)nlon * ((size_t)j + (size_t)nlat * k)] = sc * g;
      }
      free(a_re);
      free(a_im);
    }
}

#include "jgcm_oracle_adjoint.inc"
