// capi_transforms.cu -- host-pointer C ABI of the mesh-level operators (jgcm.h).
//
// Each call copies its FP64 host arrays (reference layout) into the mesh's staging buffer,
// converts them to the device layout and precision, runs the transform kernels on the
// mesh stream and copies the results back, blocking until they are on the host.
#include <cstring>

#include "jgcm_internal.cuh"

using namespace jgcm;

namespace {

int check_nlev(const jgcm_mesh* m, int nlev) {
  JG_ARG(m != nullptr, "mesh is NULL");
  JG_ARG(nlev == m->nd || nlev == 1, "third dimension must be nd=%d or 1 (got %d)", m->nd, nlev);
  return JGCM_OK;
}

double* slot(jgcm_mesh* m, int i) { return m->d_stage + (size_t)i * m->stage_slot; }

int h2d(jgcm_mesh* m, double* dst, const double* src, size_t n) {
  JG_ARG(src != nullptr, "input array is NULL");
  JG_CUDA(cudaMemcpyAsync(dst, src, n * 8, cudaMemcpyHostToDevice, m->stream));
  return JGCM_OK;
}
int d2h(jgcm_mesh* m, double* dst, const double* src, size_t n) {
  JG_ARG(dst != nullptr, "output array is NULL");
  JG_CUDA(cudaMemcpyAsync(dst, src, n * 8, cudaMemcpyDeviceToHost, m->stream));
  return JGCM_OK;
}
int finish(jgcm_mesh* m) {
  JG_CUDA(cudaStreamSynchronize(m->stream));
  JG_CUDA(cudaGetLastError());
  if (m->tc.on) JG_TRY(tc_status(m));  // a tensor-core kernel whose bounded wait gave up
  return JGCM_OK;
}

template <typename T>
int s2g_run(jgcm_mesh* m, const S2GPlan& sp, const IFFTPlan& ip) {
  return launch_s2g<T>(m, sp, ip, m->stream);
}
int s2g(jgcm_mesh* m, const S2GPlan& sp, const IFFTPlan& ip) {
  return is_fp64(m) ? s2g_run<double>(m, sp, ip) : s2g_run<float>(m, sp, ip);
}
int g2s(jgcm_mesh* m, const FFTPlan& fp, const G2SPlan& gp) {
  return is_fp64(m) ? launch_g2s<double>(m, fp, gp, m->stream) : launch_g2s<float>(m, fp, gp, m->stream);
}

S2GGroup s2g_group(int op, const void* a, const void* b, int L, int col0) {
  S2GGroup g;
  memset(&g, 0, sizeof(g));
  g.op = op;
  g.a = a;
  g.b = b;
  g.L = L;
  g.col0 = col0;
  return g;
}
GridOutGroup out_group(int epi, void* dst, int L, int col0) {
  GridOutGroup g;
  memset(&g, 0, sizeof(g));
  g.epi = epi;
  g.dst = dst;
  g.L = L;
  g.col0 = col0;
  return g;
}
GridInGroup in_group(int pro, const void* src, int L, int col0) {
  GridInGroup g;
  memset(&g, 0, sizeof(g));
  g.pro = pro;
  g.src = src;
  g.L = L;
  g.col0 = col0;
  return g;
}
SpecOutGroup spec_group(int op, void* dst, int L, int col0, int colA, int colB, int colE) {
  SpecOutGroup g;
  memset(&g, 0, sizeof(g));
  g.op = op;
  g.dst = dst;
  g.L = L;
  g.col0 = col0;
  g.colA = colA;
  g.colB = colB;
  g.colE = colE;
  g.colH = -1;
  return g;
}

// spectral gradient -> two grid fields (device), used by compute_gradients / advection
int gradients_dev(jgcm_mesh* m, const void* d_spec, int nlev, void* d_gl, void* d_gt) {
  S2GPlan sp;
  memset(&sp, 0, sizeof(sp));
  sp.ng = 2;
  sp.C = 2 * nlev;
  sp.g[0] = s2g_group(S2G_DLAM, d_spec, nullptr, nlev, 0);
  sp.g[1] = s2g_group(S2G_DTH, d_spec, nullptr, nlev, nlev);
  IFFTPlan ip;
  memset(&ip, 0, sizeof(ip));
  ip.ng = 2;
  ip.C = 2 * nlev;
  ip.g[0] = out_group(EPI_DIVCOS, d_gl, nlev, 0);
  ip.g[1] = out_group(EPI_DIVCOS, d_gt, nlev, nlev);
  return s2g(m, sp, ip);
}

template <typename T>
__global__ void k_adv_update(const T* gl, const T* gt, const double* u, const double* v, double* dh, size_t n) {
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x)
    dh[t] = dh[t] - (u[t] * (double)gl[t] + v[t] * (double)gt[t]);
}

}  // namespace

extern "C" int jgcm_trans_spherical_to_grid(jgcm_mesh* m, const double* snm, int nlev, double* pfield) {
  JG_TRY(check_nlev(m, nlev));
  size_t ns = 2 * spec_elems(m, nlev), ng = grid_elems(m, nlev);
  JG_TRY(h2d(m, slot(m, 0), snm, ns));
  JG_TRY(spec_host_to_dev(m, slot(m, 0), m->d_spec[0], nlev, m->stream));
  S2GPlan sp;
  memset(&sp, 0, sizeof(sp));
  sp.ng = 1;
  sp.C = nlev;
  sp.g[0] = s2g_group(S2G_PLAIN, m->d_spec[0], nullptr, nlev, 0);
  IFFTPlan ip;
  memset(&ip, 0, sizeof(ip));
  ip.ng = 1;
  ip.C = nlev;
  ip.g[0] = out_group(EPI_NONE, m->d_grid[0], nlev, 0);
  JG_TRY(s2g(m, sp, ip));
  JG_TRY(grid_dev_to_host(m, m->d_grid[0], slot(m, 1), ng, m->stream));
  JG_TRY(d2h(m, pfield, slot(m, 1), ng));
  return finish(m);
}

extern "C" int jgcm_trans_grid_to_spherical(jgcm_mesh* m, const double* pfield, int nlev, double* snm) {
  JG_TRY(check_nlev(m, nlev));
  size_t ns = 2 * spec_elems(m, nlev), ng = grid_elems(m, nlev);
  JG_TRY(h2d(m, slot(m, 0), pfield, ng));
  JG_TRY(grid_host_to_dev(m, slot(m, 0), m->d_grid[0], ng, m->stream));
  FFTPlan fp;
  memset(&fp, 0, sizeof(fp));
  fp.ng = 1;
  fp.C = nlev;
  fp.g[0] = in_group(PRO_NONE, m->d_grid[0], nlev, 0);
  G2SPlan gp;
  memset(&gp, 0, sizeof(gp));
  gp.ng = 1;
  gp.C = nlev;
  gp.g[0] = spec_group(G2S_PLAIN, m->d_spec[0], nlev, 0, 0, -1, -1);
  JG_TRY(g2s(m, fp, gp));
  JG_TRY(spec_dev_to_host(m, m->d_spec[0], slot(m, 1), nlev, m->stream));
  JG_TRY(d2h(m, snm, slot(m, 1), ns));
  return finish(m);
}

// Adjoint of Trans_Spherical_To_Grid!: grid cotangent -> spectral cotangent (row N+1 included).
extern "C" int jgcm_trans_spherical_to_grid_adjoint(jgcm_mesh* m, const double* grid_bar, int nlev, double* spec_bar) {
  JG_TRY(check_nlev(m, nlev));
  size_t ns = 2 * spec_elems(m, nlev), ng = grid_elems(m, nlev);
  JG_TRY(h2d(m, slot(m, 0), grid_bar, ng));
  JG_TRY(grid_host_to_dev(m, slot(m, 0), m->d_grid[0], ng, m->stream));
  FFTPlan fp;
  memset(&fp, 0, sizeof(fp));
  fp.ng = 1;
  fp.C = nlev;
  fp.g[0] = in_group(PRO_NONE, m->d_grid[0], nlev, 0);
  G2SPlan gp;
  memset(&gp, 0, sizeof(gp));
  gp.ng = 1;
  gp.C = nlev;
  gp.g[0] = spec_group(G2S_ADJ_S2G, m->d_spec[0], nlev, 0, 0, -1, -1);
  gp.g[0].scale = m->nlon;
  JG_TRY(g2s(m, fp, gp));
  JG_TRY(spec_dev_to_host(m, m->d_spec[0], slot(m, 1), nlev, m->stream));
  JG_TRY(d2h(m, spec_bar, slot(m, 1), ns));
  return finish(m);
}

// Adjoint of Trans_Grid_To_Spherical!: spectral cotangent (row N+1 ignored) -> grid cotangent.
extern "C" int jgcm_trans_grid_to_spherical_adjoint(jgcm_mesh* m, const double* spec_bar, int nlev, double* grid_bar) {
  JG_TRY(check_nlev(m, nlev));
  size_t ns = 2 * spec_elems(m, nlev), ng = grid_elems(m, nlev);
  JG_TRY(h2d(m, slot(m, 0), spec_bar, ns));
  JG_TRY(spec_host_to_dev(m, slot(m, 0), m->d_spec[0], nlev, m->stream));
  S2GPlan sp;
  memset(&sp, 0, sizeof(sp));
  sp.ng = 1;
  sp.C = nlev;
  sp.g[0] = s2g_group(S2G_ADJ_G2S, m->d_spec[0], nullptr, nlev, 0);
  IFFTPlan ip;
  memset(&ip, 0, sizeof(ip));
  ip.ng = 1;
  ip.C = nlev;
  ip.g[0] = out_group(EPI_ADJ_G2S, m->d_grid[0], nlev, 0);
  JG_TRY(s2g(m, sp, ip));
  JG_TRY(grid_dev_to_host(m, m->d_grid[0], slot(m, 1), ng, m->stream));
  JG_TRY(d2h(m, grid_bar, slot(m, 1), ng));
  return finish(m);
}

extern "C" int jgcm_trans_grid_to_fourier(jgcm_mesh* m, const double* pfield, int nlev, double* fourier) {
  JG_TRY(check_nlev(m, nlev));
  size_t ng = grid_elems(m, nlev), nf = 2 * ng;  // complex [nlev][nlat][nlon]: staging slots 1 and 2
  JG_TRY(h2d(m, slot(m, 0), pfield, ng));
  JG_TRY(grid_host_to_dev(m, slot(m, 0), m->d_grid[0], ng, m->stream));
  JG_TRY(fourier_full_to_host(m, m->d_grid[0], nlev, slot(m, 1), m->stream));
  JG_TRY(d2h(m, fourier, slot(m, 1), nf));
  return finish(m);
}

extern "C" int jgcm_vor_div_from_grid_uv(jgcm_mesh* m, const double* u, const double* v, int nlev, double* vor,
                                         double* div) {
  JG_TRY(check_nlev(m, nlev));
  size_t ns = 2 * spec_elems(m, nlev), ng = grid_elems(m, nlev);
  JG_TRY(h2d(m, slot(m, 0), u, ng));
  JG_TRY(h2d(m, slot(m, 1), v, ng));
  JG_TRY(grid_host_to_dev(m, slot(m, 0), m->d_grid[0], ng, m->stream));
  JG_TRY(grid_host_to_dev(m, slot(m, 1), m->d_grid[1], ng, m->stream));
  FFTPlan fp;
  memset(&fp, 0, sizeof(fp));
  fp.ng = 2;
  fp.C = 2 * nlev;
  fp.g[0] = in_group(PRO_MULCOS, m->d_grid[0], nlev, 0);     // u cos
  fp.g[1] = in_group(PRO_MULCOS, m->d_grid[1], nlev, nlev);  // v cos
  G2SPlan gp;
  memset(&gp, 0, sizeof(gp));
  gp.ng = 2;
  gp.C = 2 * nlev;
  gp.g[0] = spec_group(G2S_VOR, m->d_spec[0], nlev, 0, nlev, 0, -1);     // A = v cos, B = u cos, sign -1
  gp.g[1] = spec_group(G2S_DIV, m->d_spec[1], nlev, nlev, 0, nlev, -1);  // A = u cos, B = v cos, sign +1
  JG_TRY(g2s(m, fp, gp));
  JG_TRY(spec_dev_to_host(m, m->d_spec[0], slot(m, 2), nlev, m->stream));
  JG_TRY(spec_dev_to_host(m, m->d_spec[1], slot(m, 3), nlev, m->stream));
  JG_TRY(d2h(m, vor, slot(m, 2), ns));
  JG_TRY(d2h(m, div, slot(m, 3), ns));
  return finish(m);
}

extern "C" int jgcm_uv_grid_from_vor_div(jgcm_mesh* m, const double* vor, const double* div, int nlev, double* u,
                                         double* v) {
  JG_TRY(check_nlev(m, nlev));
  size_t ns = 2 * spec_elems(m, nlev), ng = grid_elems(m, nlev);
  JG_TRY(h2d(m, slot(m, 0), vor, ns));
  JG_TRY(h2d(m, slot(m, 1), div, ns));
  JG_TRY(spec_host_to_dev(m, slot(m, 0), m->d_spec[0], nlev, m->stream));
  JG_TRY(spec_host_to_dev(m, slot(m, 1), m->d_spec[1], nlev, m->stream));
  S2GPlan sp;
  memset(&sp, 0, sizeof(sp));
  sp.ng = 2;
  sp.C = 2 * nlev;
  sp.g[0] = s2g_group(S2G_UCOS, m->d_spec[0], m->d_spec[1], nlev, 0);
  sp.g[1] = s2g_group(S2G_VCOS, m->d_spec[0], m->d_spec[1], nlev, nlev);
  IFFTPlan ip;
  memset(&ip, 0, sizeof(ip));
  ip.ng = 2;
  ip.C = 2 * nlev;
  ip.g[0] = out_group(EPI_DIVCOS, m->d_grid[0], nlev, 0);
  ip.g[1] = out_group(EPI_DIVCOS, m->d_grid[1], nlev, nlev);
  JG_TRY(s2g(m, sp, ip));
  JG_TRY(grid_dev_to_host(m, m->d_grid[0], slot(m, 2), ng, m->stream));
  JG_TRY(grid_dev_to_host(m, m->d_grid[1], slot(m, 3), ng, m->stream));
  JG_TRY(d2h(m, u, slot(m, 2), ng));
  JG_TRY(d2h(m, v, slot(m, 3), ng));
  return finish(m);
}

extern "C" int jgcm_compute_gradients(jgcm_mesh* m, const double* hs, int nlev, double* gdl, double* gdt) {
  JG_TRY(check_nlev(m, nlev));
  size_t ns = 2 * spec_elems(m, nlev), ng = grid_elems(m, nlev);
  JG_TRY(h2d(m, slot(m, 0), hs, ns));
  JG_TRY(spec_host_to_dev(m, slot(m, 0), m->d_spec[0], nlev, m->stream));
  JG_TRY(gradients_dev(m, m->d_spec[0], nlev, m->d_grid[0], m->d_grid[1]));
  JG_TRY(grid_dev_to_host(m, m->d_grid[0], slot(m, 2), ng, m->stream));
  JG_TRY(grid_dev_to_host(m, m->d_grid[1], slot(m, 3), ng, m->stream));
  JG_TRY(d2h(m, gdl, slot(m, 2), ng));
  JG_TRY(d2h(m, gdt, slot(m, 3), ng));
  return finish(m);
}

extern "C" int jgcm_add_horizontal_advection(jgcm_mesh* m, const double* hs, const double* u, const double* v,
                                             int nlev, double* dh) {
  JG_TRY(check_nlev(m, nlev));
  size_t ns = 2 * spec_elems(m, nlev), ng = grid_elems(m, nlev);
  JG_TRY(h2d(m, slot(m, 0), hs, ns));
  JG_TRY(spec_host_to_dev(m, slot(m, 0), m->d_spec[0], nlev, m->stream));
  JG_TRY(gradients_dev(m, m->d_spec[0], nlev, m->d_grid[0], m->d_grid[1]));
  JG_TRY(h2d(m, slot(m, 1), u, ng));
  JG_TRY(h2d(m, slot(m, 2), v, ng));
  JG_TRY(h2d(m, slot(m, 3), dh, ng));
  size_t nb = (ng + 255) / 256;
  if (nb > 1184) nb = 1184;
  if (is_fp64(m))
    k_adv_update<double><<<(int)nb, 256, 0, m->stream>>>((const double*)m->d_grid[0], (const double*)m->d_grid[1],
                                                          slot(m, 1), slot(m, 2), slot(m, 3), ng);
  else
    k_adv_update<float><<<(int)nb, 256, 0, m->stream>>>((const float*)m->d_grid[0], (const float*)m->d_grid[1],
                                                         slot(m, 1), slot(m, 2), slot(m, 3), ng);
  JG_CUDA(cudaGetLastError());
  JG_TRY(d2h(m, dh, slot(m, 3), ng));
  return finish(m);
}

extern "C" int jgcm_apply_laplacian(jgcm_mesh* m, double* spe, int nlev) {
  JG_TRY(check_nlev(m, nlev));
  size_t ns = 2 * spec_elems(m, nlev);
  JG_TRY(h2d(m, slot(m, 0), spe, ns));
  JG_TRY(spec_host_to_dev(m, slot(m, 0), m->d_spec[0], nlev, m->stream));
  JG_TRY(apply_laplacian(m, m->d_spec[0], nlev, m->stream));
  JG_TRY(spec_dev_to_host(m, m->d_spec[0], slot(m, 1), nlev, m->stream));
  JG_TRY(d2h(m, spe, slot(m, 1), ns));
  return finish(m);
}

extern "C" int jgcm_area_weighted_global_mean(jgcm_mesh* m, const double* grid, double* out) {
  JG_ARG(m && grid && out, "NULL argument");
  size_t ng = grid_elems(m, 1);
  JG_TRY(h2d(m, slot(m, 0), grid, ng));
  JG_TRY(grid_host_to_dev(m, slot(m, 0), m->d_grid[0], ng, m->stream));
  JG_TRY(area_mean(m, m->d_grid[0], m->d_red, m->stream));
  JG_CUDA(cudaMemcpyAsync(out, m->d_red, 8, cudaMemcpyDeviceToHost, m->stream));
  return finish(m);
}
