// state.cu -- the state of one Held-Suarez step as a unit: the 18 arrays one Atmosphere_Update!
// reads and writes (Dyn_Data.jl), whole-state device copies for the reverse sweep's checkpoints, and
// the batched host <-> device transfer of the C ABI (one copy and one layout-conversion launch each
// way instead of one call per field).
#include <algorithm>
#include <cstring>

#include "model_internal.cuh"
#include "transform_ops.cuh"

using namespace jgcm;

namespace {
// The 18 fields copied by one launch (a block row per field, 16-byte words; every field's size is
// a multiple of 16 bytes: 8-byte complex floats x an even count, or 4-byte reals x nlon (even)).
struct CopyList {
  const uint4* src[NSTATE];
  uint4* dst[NSTATE];
  size_t n16[NSTATE];
};

__global__ void __launch_bounds__(256) k_copy_fields(CopyList c) {
  pdl_wait();  // programmatic dependent launch: the predecessor's output is complete
  const int f = blockIdx.y;
  const uint4* __restrict__ s = c.src[f];
  uint4* __restrict__ d = c.dst[f];
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < c.n16[f]; i += (size_t)gridDim.x * blockDim.x)
    d[i] = s[i];
}


// Packed host state (reference layout, FP64, fields back to back) <-> device fields.
struct PackList {
  void* dev[NSTATE];
  size_t off[NSTATE];  // doubles from the start of the packed buffer
  int L[NSTATE];
  int spec[NSTATE];
};

template <typename T>
__global__ void __launch_bounds__(256) k_state_h2d(PackList p, const double* __restrict__ src, int N, int ns,
                                                   size_t G1) {
  const int f = blockIdx.y, L = p.L[f];
  const double* s = src + p.off[f];
  if (p.spec[f]) {
    V2<T>* d = (V2<T>*)p.dev[f];
    const size_t total = (size_t)(N + 1) * (ns + 1) * L;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
      const int k = (int)(t % L);
      const size_t mn = t / L;
      const int n = (int)(mn % (ns + 1)), m = (int)(mn / (ns + 1));
      const size_t h = 2 * ((size_t)m + (size_t)(N + 1) * ((size_t)n + (size_t)(ns + 1) * k));
      V2<T> v;
      v.x = (n >= m) ? (T)s[h] : (T)0;
      v.y = (n >= m) ? (T)s[h + 1] : (T)0;
      d[t] = v;
    }
  } else {
    T* d = (T*)p.dev[f];
    const size_t total = G1 * L;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x)
      d[t] = (T)s[t];
  }
}

template <typename T>
__global__ void __launch_bounds__(256) k_state_d2h(PackList p, double* __restrict__ dst, int N, int ns, size_t G1) {
  const int f = blockIdx.y, L = p.L[f];
  double* d = dst + p.off[f];
  if (p.spec[f]) {
    const V2<T>* s = (const V2<T>*)p.dev[f];
    const size_t total = (size_t)(N + 1) * (ns + 1) * L;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
      const int m = (int)(t % (N + 1));
      const size_t r = t / (N + 1);
      const int n = (int)(r % (ns + 1)), k = (int)(r / (ns + 1));
      const V2<T> v = s[((size_t)m * (ns + 1) + n) * L + k];
      d[2 * t] = (double)v.x;
      d[2 * t + 1] = (double)v.y;
    }
  } else {
    const T* s = (const T*)p.dev[f];
    const size_t total = G1 * L;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x)
      d[t] = (double)s[t];
  }
}

size_t packed_doubles(const jgcm_model* md, int i) {
  const jgcm_mesh* m = md->mesh;
  const int L = st_levels(md, i);
  return st_spec(i) ? 2 * spec_elems(m, L) : grid_elems(m, L);
}

int pack_list(jgcm_model* md, PackList* p, size_t* total) {
  size_t off = 0;
  for (int i = 0; i < NSTATE; i++) {
    p->dev[i] = model_slot(md, i);
    p->off[i] = off;
    p->L[i] = st_levels(md, i);
    p->spec[i] = st_spec(i);
    off += packed_doubles(md, i);
  }
  *total = off;
  if (!md->state_stage) JG_TRY(dev_alloc((void**)&md->state_stage, off * 8));
  return JGCM_OK;
}

int check_state_model(jgcm_model* md) {
  JG_ARG(md, "NULL model");
  JG_ARG(md->P.kind == JGCM_HELD_SUAREZ, "the packed state is defined for Held-Suarez models");
  JG_ARG(md->ne == 1, "one-member models only (ensembles load members with jgcm_model_copy_member)");
  return JGCM_OK;
}
}  // namespace

namespace jgcm {
// ---- state buffers ----------------------------------------------------------------------------
// field i of the state: 0 spe_vor_c, 1 spe_vor_p, 2 spe_div_c, 3 spe_div_p, 4 spe_lnps_c,
// 5 spe_lnps_p, 6 spe_t_c, 7 spe_t_p, 8 grid_u_c, 9 grid_u_p, 10 grid_v_c, 11 grid_v_p,
// 12 grid_ps_c, 13 grid_ps_p, 14 grid_t_c, 15 grid_t_p, 16 grid_vor, 17 grid_div
bool st_spec(int i) { return i < 8; }
int st_levels(const jgcm_model* md, int i) { return (i == 4 || i == 5 || i == 12 || i == 13) ? 1 : md->nd; }
size_t st_bytes(const jgcm_model* md, int i) {
  const jgcm_mesh* m = md->mesh;
  const size_t ts = tsize(m);
  return st_spec(i) ? spec_elems(m, st_levels(md, i)) * 2 * ts : grid_elems(m, st_levels(md, i)) * ts;
}
void* model_slot(jgcm_model* md, int i) {
  const int p = lvl(md, 0), c = lvl(md, 1);
  switch (i) {
    case 0: return md->spe_vor[c];
    case 1: return md->spe_vor[p];
    case 2: return md->spe_div[c];
    case 3: return md->spe_div[p];
    case 4: return md->spe_lnps[c];
    case 5: return md->spe_lnps[p];
    case 6: return md->spe_t[c];
    case 7: return md->spe_t[p];
    case 8: return md->grid_u[c];
    case 9: return md->grid_u[p];
    case 10: return md->grid_v[c];
    case 11: return md->grid_v[p];
    case 12: return md->grid_ps[c];
    case 13: return md->grid_ps[p];
    case 14: return md->grid_t[c];
    case 15: return md->grid_t[p];
    case 16: return md->grid_vor;
    default: return md->grid_div;
  }
}

int state_alloc(jgcm_model* md, StateBuf* b) {
  size_t tot = 0;
  for (int i = 0; i < NSTATE; i++) tot += (st_bytes(md, i) + 255) & ~(size_t)255;
  JG_TRY(dev_alloc(&b->base, tot));
  size_t off = 0;
  for (int i = 0; i < NSTATE; i++) {
    b->f[i] = (char*)b->base + off;
    off += (st_bytes(md, i) + 255) & ~(size_t)255;
  }
  b->init = 0;
  return JGCM_OK;
}

int copy_fields(jgcm_model* md, void* const* dst, const void* const* src, cudaStream_t st) {
  CopyList c;
  size_t mx = 0;
  for (int i = 0; i < NSTATE; i++) {
    const size_t b = st_bytes(md, i);
    JG_ARG(b % 16 == 0, "state field %d is not a whole number of 16-byte words", i);
    c.src[i] = (const uint4*)src[i];
    c.dst[i] = (uint4*)dst[i];
    c.n16[i] = b / 16;
    mx = c.n16[i] > mx ? c.n16[i] : mx;
  }
  const int bx = (int)std::min<size_t>((mx + 255) / 256, 64);
  JG_CUDA(launch_pdl(k_copy_fields, dim3(bx, NSTATE), 256, 0, st, c));
  JG_CUDA(cudaGetLastError());
  return JGCM_OK;
}

int state_save(jgcm_model* md, StateBuf* b, cudaStream_t st) {
  const void* src[NSTATE];
  for (int i = 0; i < NSTATE; i++) src[i] = model_slot(md, i);
  JG_TRY(copy_fields(md, b->f, src, st));
  b->init = md->init_step;
  return JGCM_OK;
}

int state_load(jgcm_model* md, const StateBuf* b, cudaStream_t st) {
  void* dst[NSTATE];
  for (int i = 0; i < NSTATE; i++) dst[i] = model_slot(md, i);
  JG_TRY(copy_fields(md, dst, b->f, st));
  md->init_step = b->init;
  md->grad_ready = 0;  // the next step recomputes the gradients of the loaded c level
  return JGCM_OK;
}

int state_zero(jgcm_model* md, StateBuf* b, cudaStream_t st) {
  for (int i = 0; i < NSTATE; i++) JG_CUDA(cudaMemsetAsync(b->f[i], 0, st_bytes(md, i), st));
  return JGCM_OK;
}

}  // namespace jgcm

extern "C" int jgcm_model_state_size(jgcm_model* md, long* ndoubles) {
  JG_TRY(check_state_model(md));
  JG_ARG(ndoubles, "NULL argument");
  size_t n = 0;
  for (int i = 0; i < NSTATE; i++) n += packed_doubles(md, i);
  *ndoubles = (long)n;
  return JGCM_OK;
}

extern "C" int jgcm_model_set_state(jgcm_model* md, const double* packed) {
  JG_TRY(check_state_model(md));
  JG_ARG(packed, "NULL state");
  jgcm_mesh* m = md->mesh;
  cudaStream_t st = m->stream;
  PackList p;
  size_t n = 0;
  JG_TRY(pack_list(md, &p, &n));
  JG_CUDA(cudaMemcpyAsync(md->state_stage, packed, n * 8, cudaMemcpyHostToDevice, st));
  const dim3 g(64, NSTATE);
  const size_t G1 = grid_elems(m, 1);
  if (is_fp64(m)) k_state_h2d<double><<<g, 256, 0, st>>>(p, md->state_stage, m->N, m->ns, G1);
  else k_state_h2d<float><<<g, 256, 0, st>>>(p, md->state_stage, m->N, m->ns, G1);
  JG_CUDA(cudaGetLastError());
  md->grad_ready = 0;  // the gradients of the new c level are recomputed by the next step
  JG_CUDA(cudaStreamSynchronize(st));
  return JGCM_OK;
}

extern "C" int jgcm_model_get_state(jgcm_model* md, double* packed) {
  JG_TRY(check_state_model(md));
  JG_ARG(packed, "NULL state");
  jgcm_mesh* m = md->mesh;
  cudaStream_t st = m->stream;
  PackList p;
  size_t n = 0;
  JG_TRY(pack_list(md, &p, &n));
  const dim3 g(64, NSTATE);
  const size_t G1 = grid_elems(m, 1);
  if (is_fp64(m)) k_state_d2h<double><<<g, 256, 0, st>>>(p, md->state_stage, m->N, m->ns, G1);
  else k_state_d2h<float><<<g, 256, 0, st>>>(p, md->state_stage, m->N, m->ns, G1);
  JG_CUDA(cudaGetLastError());
  JG_CUDA(cudaMemcpyAsync(packed, md->state_stage, n * 8, cudaMemcpyDeviceToHost, st));
  JG_CUDA(cudaStreamSynchronize(st));
  return JGCM_OK;
}
