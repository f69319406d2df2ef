// capi.cu -- the C ABI of librimu_gpu (declared in include/rimu_gpu.h): handles, host-side
// tables, capacity planning and the orchestration of one projector step.
#include <cuda_runtime.h>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <string>
#include <vector>
#include <algorithm>
#include "rimu_internal.h"

using namespace rimu;

// ---------------------------------------------------------------------------------------------
// Errors
// ---------------------------------------------------------------------------------------------
static thread_local std::string g_err;

void rimu_set_error(const std::string &msg) { g_err = msg; }

int rimu_cuda_check(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return RIMU_OK;
  g_err = std::string(what) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? RIMU_ERR_OOM : RIMU_ERR_CUDA;
}

static int bad(const std::string &msg) {
  g_err = msg;
  return RIMU_ERR_BADARG;
}

// launchers defined in hv.cu
int rimu_hv_grid(rimu_ctx *ctx, int64_t dim);
int rimu_launch_hv(rimu_ctx *ctx, const DevModel &h, const uint64_t *binom, int ntab,
                   const double *v, double *w, int64_t dim, const double *dtabH);
int rimu_launch_hv_adjoint(rimu_ctx *ctx, const DevModel &h, const uint64_t *binom, int ntab,
                           const double *v, const double *gw, double *gv, int64_t dim,
                           const double *dtabH, const double *dhdt, double *partial,
                           int grid, double *out2);

// model tables used by the basis products (kept with the model)
struct ModelExtra {
  uint64_t *binom = nullptr;
  int ntab = 0;
  double *dtabH = nullptr;
  double *dhdt = nullptr;
  double *partial = nullptr;
  int partial_n = 0;
  double *out2 = nullptr;
  double *h_out2 = nullptr;
};
static ModelExtra *extra_of(rimu_model *m);

extern "C" {

int rimu_version(void) { return 10000; }

int rimu_last_error(char *buf, size_t len) {
  if (!buf || len == 0) return RIMU_ERR_BADARG;
  std::snprintf(buf, len, "%s", g_err.c_str());
  return RIMU_OK;
}

// ---------------------------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------------------------
int rimu_ctx_create(int device, void *stream, rimu_ctx **out) {
  if (!out) return bad("rimu_ctx_create: out is NULL");
  int n = 0;
  RIMU_CUDA(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return bad("rimu_ctx_create: no such device");
  RIMU_CUDA(cudaSetDevice(device));
  rimu_ctx *c = new rimu_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  // NULL selects the CUDA default stream, so the caller's default-stream work (for
  // example a torch tensor initialised on it) is ordered with the library's kernels.
  c->stream = (cudaStream_t)stream;
  c->own_stream = false;
  // Keep freed stream-ordered allocations in the device's pool instead of returning them to
  // the system at every synchronization: steps, uploads and downloads reallocate buffers of
  // gigabytes, and mapping them again costs milliseconds each time.  rimu_ctx_destroy trims it.
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  *out = c;
  return RIMU_OK;
}

int rimu_ctx_destroy(rimu_ctx *ctx) {
  if (!ctx) return RIMU_OK;
  cudaStreamSynchronize(ctx->stream);
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
  if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return RIMU_OK;
}

int rimu_ctx_synchronize(rimu_ctx *ctx) {
  if (!ctx) return bad("rimu_ctx_synchronize: NULL context");
  RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
  return RIMU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------------
// Helpers
// ---------------------------------------------------------------------------------------------
static bool two_components(const rimu_model_desc &d) { return d.n_components >= 2; }

// Largest occupation product under the square root of an offdiagonal element (one table
// block; with several HubbardRealSpace components, of any component).
static int model_max_prod(const rimu_model_desc &d) {
  int N = d.n_particles;
  if (d.kind == RIMU_MODEL_MOM1D) return two_components(d) ? 4 : (N + 1) * (N + 1) * (N + 1) * (N + 1);
  if (two_components(d)) {
    int p = 1;
    for (int c = 0; c < d.n_components; ++c)
      if (!d.comp_fermion[c]) p = std::max(p, d.comp_particles[c] * (d.comp_particles[c] + 1));
    return p;
  }
  if (d.fermion) return 1;
  return N * (N + 1);
}

// Hamiltonian offdiagonal magnitude for occupation product p in table block c: -t sqrt(p)
// (HubbardReal1D.jl:59-62, HubbardRealSpace.jl:336, per component t[c]) or u/(2M) sqrt(p)
// (HubbardMom1D.jl:189-194; FermiFS2C's u/M is p = 4).
static double hoff_value(const rimu_model_desc &d, int c, int p) {
  const double s = std::sqrt((double)p);
  if (d.kind == RIMU_MODEL_MOM1D) return d.u / (2 * d.n_modes) * s;
  const double t = two_components(d) ? d.comp_t[c] : d.t;
  return -t * s;
}

static int64_t binomial_u(int n, int k, bool *ovf) {
  if (k < 0 || k > n) return 0;
  unsigned __int128 r = 1;
  for (int i = 1; i <= k; ++i) {
    r = r * (unsigned)(n - k + i) / (unsigned)i;
    if (r > (unsigned __int128)INT64_MAX) { *ovf = true; return 0; }
  }
  return (int64_t)r;
}

// ---------------------------------------------------------------------------------------------
// Models
// ---------------------------------------------------------------------------------------------
static std::vector<ModelExtra *> g_extras;   // parallel to models (simple registry)
static std::vector<rimu_model *> g_models;

static ModelExtra *extra_of(rimu_model *m) {
  for (size_t i = 0; i < g_models.size(); ++i) if (g_models[i] == m) return g_extras[i];
  return nullptr;
}

extern "C" int rimu_model_destroy(rimu_model *m);

extern "C" int rimu_model_create(rimu_ctx *ctx, const rimu_model_desc *d, rimu_model **out) {
  if (!ctx || !d || !out) return bad("rimu_model_create: NULL argument");
  if (d->kind < 1 || d->kind > 3) return bad("rimu_model_create: unknown model kind");
  if (d->n_particles < 0 || d->n_modes < 1 || d->n_modes > 128)
    return bad("rimu_model_create: need 1 <= n_modes <= 128");
  if (d->n_components < 0 || d->n_components > RIMU_MAX_COMPONENTS)
    return bad("rimu_model_create: n_components must be 0 .. RIMU_MAX_COMPONENTS");
  const bool two = two_components(*d);
  const int C = two ? d->n_components : 1;
  int nbits = d->fermion ? d->n_modes : d->n_particles + d->n_modes - 1;
  int cbits[RIMU_MAX_COMPONENTS] = {0, 0, 0, 0};
  if (two) {
    if (d->kind == RIMU_MODEL_REAL1D)
      return bad("rimu_model_create: HubbardReal1D takes a single-component BoseFS");
    if (d->kind == RIMU_MODEL_MOM1D && !(C == 2 && d->comp_fermion[0] && d->comp_fermion[1]))
      return bad("rimu_model_create: HubbardMom1D takes two components only as FermiFS2C");
    int nsum = 0;
    nbits = 0;
    for (int c = 0; c < C; ++c) {
      if (d->comp_particles[c] < 0) return bad("rimu_model_create: negative particle number");
      if (d->comp_fermion[c] && d->comp_particles[c] > d->n_modes)
        return bad("rimu_model_create: too many fermions in a component");
      cbits[c] = d->comp_fermion[c] ? d->n_modes : d->comp_particles[c] + d->n_modes - 1;
      nsum += d->comp_particles[c];
      nbits += cbits[c];
    }
    if (nsum != d->n_particles)
      return bad("rimu_model_create: n_particles must be the sum over the components");
  }
  if (nbits > 128) return bad("rimu_model_create: address does not fit 128 bits");
  if (two) {
    // a multi-component address takes one or two words, each component at most one word
    if (d->n_modes > 64) return bad("rimu_model_create: multi-component addresses take at most 64 modes");
    for (int c = 0; c < C; ++c)
      if (cbits[c] > 64) return bad("rimu_model_create: a component of more than 64 bits");
  }
  if (d->n_modes > 64 && d->kind == RIMU_MODEL_MOM1D)
    return bad("rimu_model_create: HubbardMom1D takes at most 64 modes");
  if (d->fermion && d->kind != RIMU_MODEL_REALSPACE)
    return bad("rimu_model_create: FermiFS is supported with HubbardRealSpace only");
  if (d->fermion && d->n_particles > d->n_modes) return bad("rimu_model_create: too many fermions");
  if (d->kind == RIMU_MODEL_MOM1D && !d->dispersion)
    return bad("rimu_model_create: HubbardMom1D needs the dispersion (h.kes)");
  if (d->kind == RIMU_MODEL_MOM1D && d->n_modes < 3)
    return bad("rimu_model_create: HubbardMom1D needs at least 3 modes");
  int ndim = d->kind == RIMU_MODEL_REALSPACE ? d->ndim : 1;
  if (ndim < 1 || ndim > 3) return bad("rimu_model_create: ndim must be 1..3");
  if (d->kind == RIMU_MODEL_REALSPACE) {
    int prod = 1;
    for (int i = 0; i < ndim; ++i) {
      if (d->dims[i] < 2) return bad("rimu_model_create: all dimensions must be at least 2");
      prod *= d->dims[i];
    }
    if (prod != d->n_modes) return bad("rimu_model_create: geometry does not match n_modes");
  }
  rimu_model *m = new rimu_model();
  m->ctx = ctx;
  m->desc = *d;
  m->desc.potential = nullptr;
  m->desc.dispersion = nullptr;
  DevModel &h = m->dm;
  h.kind = d->kind; h.fermion = two ? 0 : d->fermion; h.N = d->n_particles; h.M = d->n_modes;
  h.nbits = nbits; h.u = d->u; h.t = d->t;
  h.ncomp = C;
  {
    int off = 0;                          // the last component in the lowest bits
    for (int c = RIMU_MAX_COMPONENTS - 1; c >= 0; --c) {
      const bool in = two && c < C;
      h.cferm[c] = in ? (d->comp_fermion[c] != 0) : 0;
      h.cN[c] = in ? d->comp_particles[c] : 0;
      h.cbits[c] = in ? cbits[c] : 0;
      h.coff[c] = in ? off : 0;
      if (in) off += cbits[c];
      h.ct[c] = in ? d->comp_t[c] : d->t;
    }
  }
  h.u_nonzero = 0;
  for (int i = 0; i < RIMU_MAX_COMPONENTS * (RIMU_MAX_COMPONENTS + 1) / 2; ++i) {
    const bool in = two && i < C * (C + 1) / 2;
    h.cu[i] = in ? d->comp_u[i] : 0.0;
    if (in && d->comp_u[i] != 0.0) h.u_nonzero = 1;
  }
  h.ndim = ndim;
  for (int i = 0; i < 3; ++i) {
    h.dims[i] = d->kind == RIMU_MODEL_REALSPACE ? (i < ndim ? d->dims[i] : 1) : (i == 0 ? d->n_modes : 1);
    h.periodic[i] = d->kind == RIMU_MODEL_REALSPACE ? (i < ndim ? d->periodic[i] : 1) : 1;
  }
  int rc = RIMU_OK;
  int M = d->n_modes, N = d->n_particles;
  if (d->kind == RIMU_MODEL_MOM1D) {
    if ((rc = dalloc(ctx, &m->d_kes, M)) || (rc = h2d(ctx, m->d_kes, d->dispersion, M))) goto fail;
    h.kes = m->d_kes;
  }
  if (d->kind == RIMU_MODEL_REALSPACE && d->potential) {
    const int np = C * M;              // with several components: component 1's sites first
    if ((rc = dalloc(ctx, &m->d_pot, np)) || (rc = h2d(ctx, m->d_pot, d->potential, np))) goto fail;
    h.pot = m->d_pot;
  }
  {
    // 1/n and (double)n tables (host IEEE arithmetic) for the spawn amplitude factor
    const int nr = 4096;
    std::vector<double> rec(2 * nr);
    rec[0] = 0.0;
    for (int i = 1; i < nr; ++i) rec[i] = 1.0 / (double)i;
    for (int i = 0; i < nr; ++i) rec[nr + i] = (double)i;
    if ((rc = dalloc(ctx, &m->d_recip, 2 * nr)) || (rc = h2d(ctx, m->d_recip, rec.data(), 2 * nr))) goto fail;
    h.recip = m->d_recip;
    h.dint = m->d_recip + nr;
    h.recip_len = nr;
    // Hamiltonian offdiagonal magnitudes by occupation product, one block per component
    // with its own t for several HubbardRealSpace components
    const int pmax = model_max_prod(*d);
    const int blocks = (two && d->kind == RIMU_MODEL_REALSPACE) ? C : 1;
    const int len = blocks * (pmax + 1);
    m->aoff_len = len;
    h.cstride = blocks > 1 ? pmax + 1 : 0;
    std::vector<double> hoff(len);
    for (int c = 0; c < blocks; ++c)
      for (int p = 0; p <= pmax; ++p) hoff[c * (pmax + 1) + p] = hoff_value(*d, c, p);
    if ((rc = dalloc(ctx, &m->d_hoff, len)) || (rc = h2d(ctx, m->d_hoff, hoff.data(), len)))
      goto fail;
    if ((rc = dalloc(ctx, &m->d_aoff, len))) goto fail;
    h.hoff = m->d_hoff;
    h.aoff = m->d_aoff;
    h.aoff_len = len;
    m->aoff_dt = std::nan("");
    bool table_diag = !two && (d->kind == RIMU_MODEL_REAL1D ||
                               (d->kind == RIMU_MODEL_REALSPACE && !d->potential));
    m->ndiag = table_diag ? (d->fermion ? 1 : N * (N - 1) + 1) : 0;
    // max offdiagonals of a column (capacity planning)
    if (d->kind == RIMU_MODEL_MOM1D && two) {
      m->max_offdiag = d->comp_particles[0] * d->comp_particles[1] * (M - 1);
    } else if (d->kind == RIMU_MODEL_MOM1D) {
      int s = std::min(N, M);
      m->max_offdiag = s * (s - 1) * (M - 2) + s * (M - 1);
    } else if (two) {
      int s = 0;
      for (int c = 0; c < C; ++c) s += std::min(d->comp_particles[c], M);
      m->max_offdiag = s * 2 * ndim;
    } else {
      int s = std::min(N, M);
      m->max_offdiag = s * 2 * ndim;
    }
  }
  {
    ModelExtra *x = new ModelExtra();
    g_models.push_back(m);
    g_extras.push_back(x);
  }
  *out = m;
  return RIMU_OK;
fail:
  rimu_model_destroy(m);
  return rc;
}

extern "C" int rimu_model_destroy(rimu_model *m) {
  if (!m) return RIMU_OK;
  rimu_ctx *ctx = m->ctx;
  dfree(ctx, m->d_kes); dfree(ctx, m->d_pot); dfree(ctx, m->d_aoff); dfree(ctx, m->d_hoff);
  dfree(ctx, m->d_recip);
  for (size_t i = 0; i < g_models.size(); ++i) {
    if (g_models[i] == m) {
      ModelExtra *x = g_extras[i];
      dfree(ctx, x->binom); dfree(ctx, x->dtabH); dfree(ctx, x->dhdt); dfree(ctx, x->partial);
      dfree(ctx, x->out2);
      if (x->h_out2) cudaFreeHost(x->h_out2);
      delete x;
      g_models.erase(g_models.begin() + i);
      g_extras.erase(g_extras.begin() + i);
      break;
    }
  }
  cudaStreamSynchronize(ctx->stream);
  delete m;
  return RIMU_OK;
}

// transition offdiagonal table -H dt for the current dt (fciqmc.jl:109-112)
int ensure_aoff(rimu_model *m, double dt) {
  if (m->aoff_dt == dt) return RIMU_OK;
  const rimu_model_desc &d = m->desc;
  const int n = m->aoff_len, stride = m->dm.cstride ? m->dm.cstride : n;
  std::vector<double> a(n);
  for (int i = 0; i < n; ++i) a[i] = -hoff_value(d, i / stride, i % stride) * dt;
  int rc = h2d(m->ctx, m->d_aoff, a.data(), n);
  if (rc) return rc;
  RIMU_CUDA(cudaStreamSynchronize(m->ctx->stream));
  m->aoff_dt = dt;
  return RIMU_OK;
}

extern "C" int rimu_model_diagonal(rimu_model *m, const uint64_t *keys, int64_t n, double *out) {
  if (!m || (n > 0 && (!keys || !out))) return bad("rimu_model_diagonal: NULL argument");
  if (n == 0) return RIMU_OK;
  rimu_ctx *ctx = m->ctx;
  uint64_t *dk = nullptr;
  double *dv = nullptr;
  int rc;
  const int kw = m->dm.nbits > 64 ? 2 : 1;   // wide addresses come as (lo, hi) pairs
  if ((rc = dalloc(ctx, &dk, n * kw)) || (rc = dalloc(ctx, &dv, n))) return rc;
  if ((rc = h2d(ctx, dk, keys, n * kw)) || (rc = rimu_launch_diagonal(ctx, m->dm, dk, n, dv)) ||
      (rc = d2h(ctx, out, dv, n))) { dfree(ctx, dk); dfree(ctx, dv); return rc; }
  dfree(ctx, dk); dfree(ctx, dv);
  RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
  return RIMU_OK;
}

static int host_num_offdiagonals(const rimu_model *m, uint64_t key, uint64_t key_hi = 0) {
  const DevModel &h = m->dm;
  if (h.kind == MODEL_MOM1D && h.ncomp == 2) return h.cN[0] * h.cN[1] * (h.M - 1);
  if (h.nbits > 64 && h.kind == MODEL_MOM1D) {
    MomMap mm;
    mom_map(k128(key, key_hi), mm);
    return num_offdiagonals_mom(h, mm);
  }
  if (h.nbits > 64) return num_offdiagonals_real(h, k128(key, key_hi));
  if (h.kind == MODEL_MOM1D && h.ncomp == 2) return h.cN[0] * h.cN[1] * (h.M - 1);
  if (h.kind == MODEL_MOM1D) {
    MomMap mm;
    mom_map(key, mm);
    return num_offdiagonals_mom(h, mm);
  }
  return num_offdiagonals_real(h, key);
}

extern "C" int rimu_model_num_offdiagonals(rimu_model *m, uint64_t key, int *out) {
  if (!m || !out) return bad("rimu_model_num_offdiagonals: NULL argument");
  if (m->dm.nbits > 64) return bad("rimu_model_num_offdiagonals: use the _w form for wide addresses");
  *out = host_num_offdiagonals(m, key);
  return RIMU_OK;
}

extern "C" int rimu_model_num_offdiagonals_w(rimu_model *m, const uint64_t *key2, int *out) {
  if (!m || !key2 || !out) return bad("rimu_model_num_offdiagonals_w: NULL argument");
  *out = host_num_offdiagonals(m, key2[0], m->dm.nbits > 64 ? key2[1] : 0);
  return RIMU_OK;
}

static int model_offdiagonals(rimu_model *m, uint64_t key, uint64_t key_hi, uint64_t *keys,
                              double *vals, int cap, int *n) {
  if (!m || !n) return bad("rimu_model_offdiagonals: NULL argument");
  int noff = host_num_offdiagonals(m, key, key_hi);
  *n = noff;
  if (noff == 0) return RIMU_OK;
  if (cap < noff || !keys || !vals) return bad("rimu_model_offdiagonals: buffer too small");
  rimu_ctx *ctx = m->ctx;
  const int kw = m->dm.nbits > 64 ? 2 : 1;
  uint64_t *dk = nullptr;
  double *dv = nullptr;
  int rc;
  if ((rc = dalloc(ctx, &dk, noff * kw)) || (rc = dalloc(ctx, &dv, noff))) return rc;
  rc = rimu_launch_offdiagonals(ctx, m->dm, key, key_hi, noff, dk, dv);
  if (!rc) rc = d2h(ctx, keys, dk, noff * kw);
  if (!rc) rc = d2h(ctx, vals, dv, noff);
  dfree(ctx, dk); dfree(ctx, dv);
  if (rc) return rc;
  RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
  return RIMU_OK;
}

extern "C" int rimu_model_offdiagonals(rimu_model *m, uint64_t key, uint64_t *keys,
                                       double *vals, int cap, int *n) {
  if (m && m->dm.nbits > 64) return bad("rimu_model_offdiagonals: use the _w form for wide addresses");
  return model_offdiagonals(m, key, 0, keys, vals, cap, n);
}

extern "C" int rimu_model_offdiagonals_w(rimu_model *m, const uint64_t *key2, uint64_t *keys2,
                                         double *vals, int cap, int *n) {
  if (!m || !key2) return bad("rimu_model_offdiagonals_w: NULL argument");
  return model_offdiagonals(m, key2[0], m->dm.nbits > 64 ? key2[1] : 0, keys2, vals, cap, n);
}

// ---------------------------------------------------------------------------------------------
// Vectors
// ---------------------------------------------------------------------------------------------
static void vec_free(rimu_vec *v) {
  dfree(v->ctx, v->recs);
  dfree(v->ctx, v->count);
}

static int vec_alloc(rimu_vec *v, int nb_bits, uint32_t capv) {
  vec_free(v);
  size_t nb = (size_t)1 << nb_bits;
  int rc;
  if ((rc = dalloc(v->ctx, &v->recs, nb * capv * v->kw)) || (rc = dalloc(v->ctx, &v->count, nb))) return rc;
  RIMU_CUDA(cudaMemsetAsync(v->count, 0, nb * sizeof(uint32_t), v->ctx->stream));
  v->nb_bits = nb_bits;
  v->capv = capv;
  return RIMU_OK;
}

// Walkers per bucket when a list is sized from its length alone (upload, creation): a step
// with about as many spawns as walkers then sees about 1024 contributions per bucket.
static constexpr int64_t kWalkersPerBucket = 512;

static uint32_t capv_for(int64_t n, int nb_bits) {
  double mu = (double)n / (double)(1ull << nb_bits);
  uint64_t c = (uint64_t)(1.25 * mu + 8.0 * std::sqrt(mu) + 64.0);
  return round_up(c, 32);
}

extern "C" int rimu_vec_create_kw(rimu_ctx *ctx, int val_kind, int key_words,
                                  int64_t capacity_hint, rimu_vec **out) {
  if (!ctx || !out) return bad("rimu_vec_create: NULL argument");
  if (val_kind != RIMU_VAL_F64 && val_kind != RIMU_VAL_I64) return bad("rimu_vec_create: bad val_kind");
  if (key_words != 1 && key_words != 2) return bad("rimu_vec_create: key_words must be 1 or 2");
  rimu_vec *v = new rimu_vec();
  v->ctx = ctx;
  v->val_kind = val_kind;
  v->kw = key_words;
  int nb_bits = ceil_log2(std::max<int64_t>(1, capacity_hint / kWalkersPerBucket));
  int rc = vec_alloc(v, nb_bits, capv_for(capacity_hint, nb_bits));
  if (rc) { delete v; return rc; }
  *out = v;
  return RIMU_OK;
}

extern "C" int rimu_vec_create(rimu_ctx *ctx, int val_kind, int64_t capacity_hint, rimu_vec **out) {
  return rimu_vec_create_kw(ctx, val_kind, 1, capacity_hint, out);
}

extern "C" int rimu_vec_key_words(const rimu_vec *v, int *key_words) {
  if (!v || !key_words) return bad("rimu_vec_key_words: NULL argument");
  *key_words = v->kw;
  return RIMU_OK;
}

extern "C" int rimu_vec_destroy(rimu_vec *v) {
  if (!v) return RIMU_OK;
  vec_free(v);
  cudaStreamSynchronize(v->ctx->stream);
  delete v;
  return RIMU_OK;
}

extern "C" int rimu_vec_empty(rimu_vec *v) {
  if (!v) return bad("rimu_vec_empty: NULL vector");
  RIMU_CUDA(cudaMemsetAsync(v->count, 0, ((size_t)1 << v->nb_bits) * sizeof(uint32_t), v->ctx->stream));
  v->len = 0;
  v->norm = 0.0;
  return RIMU_OK;
}

extern "C" int rimu_vec_upload(rimu_vec *v, const uint64_t *keys, const void *vals, int64_t n) {
  if (!v || (n > 0 && (!keys || !vals))) return bad("rimu_vec_upload: NULL argument");
  rimu_ctx *ctx = v->ctx;
  int nb_bits = std::max(v->nb_bits, ceil_log2(std::max<int64_t>(1, n / kWalkersPerBucket)));
  uint32_t capv = std::max(v->capv, capv_for(n, nb_bits));
  uint64_t *dk = nullptr, *dv = nullptr;
  unsigned int *flag = nullptr;
  int rc;
  const int kw = v->kw;
  if ((rc = dalloc(ctx, &dk, n * kw)) || (rc = dalloc(ctx, &dv, n)) || (rc = dalloc(ctx, &flag, 1))) return rc;
  if ((rc = h2d(ctx, dk, keys, n * kw)) || (rc = h2d(ctx, dv, (const uint64_t *)vals, n))) goto done;
  for (int attempt = 0; attempt < 8; ++attempt) {
    if (nb_bits != v->nb_bits || capv != v->capv) {
      if ((rc = vec_alloc(v, nb_bits, capv))) goto done;
    } else {
      RIMU_CUDA(cudaMemsetAsync(v->count, 0, ((size_t)1 << nb_bits) * sizeof(uint32_t), ctx->stream));
    }
    unsigned int hflag = 0;
    RIMU_CUDA(cudaMemsetAsync(flag, 0, sizeof(unsigned), ctx->stream));
    if ((rc = rimu_launch_bucketize(ctx, dk, dv, n, nb_bits, capv, v->recs, v->count, flag, kw))) goto done;
    if ((rc = d2h(ctx, &hflag, flag, 1))) goto done;
    RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
    if (!hflag) {
      v->len = n;
      rc = RIMU_OK;
      goto done;
    }
    capv *= 2;
  }
  rc = RIMU_ERR_OVERFLOW;
  g_err = "rimu_vec_upload: bucket capacity overflow";
done:
  dfree(ctx, dk); dfree(ctx, dv); dfree(ctx, flag);
  if (!rc) {
    double norm;
    int64_t len;
    rc = rimu_vec_walkernumber_and_length(v, &norm, &len);
  }
  return rc;
}

extern "C" int rimu_vec_length(rimu_vec *v, int64_t *len) {
  if (!v || !len) return bad("rimu_vec_length: NULL argument");
  *len = v->len;
  return RIMU_OK;
}

extern "C" int rimu_vec_walkernumber_and_length(rimu_vec *v, double *norm, int64_t *len) {
  if (!v) return bad("rimu_vec_walkernumber_and_length: NULL vector");
  rimu_ctx *ctx = v->ctx;
  unsigned long long *acc = nullptr;
  unsigned long long h[3];
  int rc;
  if ((rc = dalloc(ctx, &acc, 3))) return rc;
  RIMU_CUDA(cudaMemsetAsync(acc, 0, 3 * sizeof(unsigned long long), ctx->stream));
  rc = rimu_launch_norm(ctx, v->recs, v->count, 1 << v->nb_bits, v->capv, v->val_kind, acc, v->kw);
  if (!rc) rc = d2h(ctx, h, acc, 3);
  dfree(ctx, acc);
  if (rc) return rc;
  RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
  v->norm = fixed_to_double(U128{h[0], h[1]});
  v->len = (int64_t)h[2];
  if (norm) *norm = v->norm;
  if (len) *len = v->len;
  return RIMU_OK;
}

extern "C" int rimu_vec_download(rimu_vec *v, uint64_t *keys, void *vals, int64_t cap, int64_t *n) {
  if (!v || !n) return bad("rimu_vec_download: NULL argument");
  rimu_ctx *ctx = v->ctx;
  int nb = 1 << v->nb_bits;
  std::vector<uint32_t> cnt(nb);
  int rc;
  if ((rc = d2h(ctx, cnt.data(), v->count, nb))) return rc;
  RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<uint64_t> off(nb);
  uint64_t tot = 0;
  for (int i = 0; i < nb; ++i) { off[i] = tot; tot += cnt[i]; }
  *n = (int64_t)tot;
  if (tot == 0) return RIMU_OK;
  if ((int64_t)tot > cap || !keys || !vals) return bad("rimu_vec_download: buffer too small");
  uint64_t *doff = nullptr, *dk = nullptr, *dv = nullptr;
  if ((rc = dalloc(ctx, &doff, nb)) || (rc = dalloc(ctx, &dk, tot * v->kw)) || (rc = dalloc(ctx, &dv, tot))) return rc;
  if (!(rc = h2d(ctx, doff, off.data(), nb)) &&
      !(rc = rimu_launch_compact(ctx, v->recs, v->count, nb, v->capv, doff, dk, dv, v->kw)) &&
      !(rc = d2h(ctx, keys, dk, tot * v->kw)))
    rc = d2h(ctx, (uint64_t *)vals, dv, tot);
  dfree(ctx, doff); dfree(ctx, dk); dfree(ctx, dv);
  if (rc) return rc;
  RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
  return RIMU_OK;
}

extern "C" int rimu_vec_lookup(rimu_vec *v, const uint64_t *keys, int64_t n, void *vals) {
  if (!v || (n > 0 && (!keys || !vals))) return bad("rimu_vec_lookup: NULL argument");
  if (n == 0) return RIMU_OK;
  rimu_ctx *ctx = v->ctx;
  uint64_t *dk = nullptr, *dv = nullptr;
  int *df = nullptr;
  int rc;
  if ((rc = dalloc(ctx, &dk, n * v->kw)) || (rc = dalloc(ctx, &dv, n)) || (rc = dalloc(ctx, &df, n))) return rc;
  if (!(rc = h2d(ctx, dk, keys, n * v->kw)) &&
      !(rc = rimu_launch_lookup(ctx, v->recs, v->count, v->nb_bits, v->capv, dk, n, dv, df, v->kw)))
    rc = d2h(ctx, (uint64_t *)vals, dv, n);
  dfree(ctx, dk); dfree(ctx, dv); dfree(ctx, df);
  if (rc) return rc;
  RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
  return RIMU_OK;
}

extern "C" int rimu_vec_copy(rimu_vec *dst, const rimu_vec *src) {
  if (!dst || !src) return bad("rimu_vec_copy: NULL argument");
  if (dst == src) return RIMU_OK;
  int rc;
  if (dst->nb_bits != src->nb_bits || dst->capv != src->capv || dst->kw != src->kw) {
    dst->kw = src->kw;
    if ((rc = vec_alloc(dst, src->nb_bits, src->capv))) return rc;
  }
  size_t nb = (size_t)1 << src->nb_bits;
  RIMU_CUDA(cudaMemcpyAsync(dst->recs, src->recs, nb * src->capv * sizeof(Rec) * src->kw,
                            cudaMemcpyDeviceToDevice, src->ctx->stream));
  RIMU_CUDA(cudaMemcpyAsync(dst->count, src->count, nb * sizeof(uint32_t),
                            cudaMemcpyDeviceToDevice, src->ctx->stream));
  dst->val_kind = src->val_kind;
  dst->len = src->len;
  dst->norm = src->norm;
  return RIMU_OK;
}

// Re-bucket v to nb_bits with capacity capv, keeping its contents.
static int vec_regrid(rimu_vec *v, int nb_bits, uint32_t capv) {
  rimu_ctx *ctx = v->ctx;
  Rec *old = v->recs;
  uint32_t *oldc = v->count;
  int old_bits = v->nb_bits;
  uint32_t old_capv = v->capv;
  unsigned int *flag = nullptr;
  int rc;
  for (int attempt = 0; attempt < 8; ++attempt) {
    Rec *nr = nullptr;
    uint32_t *nc = nullptr;
    size_t nb = (size_t)1 << nb_bits;
    if ((rc = dalloc(ctx, &nr, nb * capv * v->kw)) || (rc = dalloc(ctx, &nc, nb)) || (rc = dalloc(ctx, &flag, 1))) return rc;
    RIMU_CUDA(cudaMemsetAsync(nc, 0, nb * sizeof(uint32_t), ctx->stream));
    RIMU_CUDA(cudaMemsetAsync(flag, 0, sizeof(unsigned), ctx->stream));
    if ((rc = rimu_launch_rebucket(ctx, old, oldc, old_bits, old_capv, nr, nc, nb_bits, capv, flag, v->kw))) return rc;
    unsigned int hflag = 0;
    if ((rc = d2h(ctx, &hflag, flag, 1))) return rc;
    RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
    dfree(ctx, flag);
    if (!hflag) {
      dfree(ctx, old);
      dfree(ctx, oldc);
      v->recs = nr;
      v->count = nc;
      v->nb_bits = nb_bits;
      v->capv = capv;
      return RIMU_OK;
    }
    dfree(ctx, nr);
    dfree(ctx, nc);
    capv *= 2;
  }
  g_err = "vec_regrid: capacity overflow";
  return RIMU_ERR_OVERFLOW;
}

// ---------------------------------------------------------------------------------------------
// scale! and add! (VectorInterface on AbstractDVec, src/DictVectors/abstractdvec.jl:121-188)
// ---------------------------------------------------------------------------------------------
// An integer list takes only integer factors (Julia would throw InexactError storing a
// non-integer product into an Int64 list).
static bool int_factor(double x, long long *out) {
  if (!(std::fabs(x) <= 9007199254740992.0) || std::trunc(x) != x) return false;
  *out = (long long)x;
  return true;
}

extern "C" int rimu_vec_scale(rimu_vec *v, double alpha) {
  if (!v) return bad("rimu_vec_scale: NULL vector");
  long long ia = 0;
  if (v->val_kind == RIMU_VAL_I64 && !int_factor(alpha, &ia))
    return bad("rimu_vec_scale: an Int64 list takes integer factors only");
  if (alpha == 0.0) return rimu_vec_empty(v);     // scale!(v, 0) = zerovector!(v)
  if (alpha == 1.0) return RIMU_OK;               // scale!(v, one) leaves v as it is
  rimu_ctx *ctx = v->ctx;
  unsigned long long *removed = nullptr, h = 0;
  int rc;
  if ((rc = dalloc(ctx, &removed, 1))) return rc;
  RIMU_CUDA(cudaMemsetAsync(removed, 0, sizeof(unsigned long long), ctx->stream));
  rc = rimu_launch_vec_scale(ctx, v->recs, v->count, 1 << v->nb_bits, v->capv, v->val_kind, v->kw,
                             alpha, ia, removed);
  if (!rc) rc = d2h(ctx, &h, removed, 1);
  if (!rc) rc = rimu_cuda_check(cudaStreamSynchronize(ctx->stream), "rimu_vec_scale");
  dfree(ctx, removed);
  if (rc) return rc;
  return rimu_vec_walkernumber_and_length(v, nullptr, nullptr);
}

// w = beta*w + alpha*v for lists with the same bucket count, into new buckets of w;
// kCrowded when a bucket of v does not fit the kernel's shared memory.
constexpr int kCrowded = -1;
static int vec_axpby_same_layout(rimu_vec *w, const rimu_vec *v, double alpha, double beta,
                                 long long ia, long long ib, bool w_empty) {
  rimu_ctx *ctx = w->ctx;
  const int nb = 1 << w->nb_bits;
  const int64_t lw = w_empty ? 0 : w->len;
  uint32_t capo = std::max<uint32_t>(capv_for(lw + v->len, w->nb_bits), 64);
  int rc;
  for (int attempt = 0; attempt < 8; ++attempt) {
    Rec *ro = nullptr;
    uint32_t *co = nullptr;
    unsigned int *flag = nullptr;
    unsigned long long *total = nullptr;
    if ((rc = dalloc(ctx, &ro, (size_t)nb * capo * w->kw)) || (rc = dalloc(ctx, &co, nb)) ||
        (rc = dalloc(ctx, &flag, 1)) || (rc = dalloc(ctx, &total, 1)))
      return rc;
    RIMU_CUDA(cudaMemsetAsync(flag, 0, sizeof(unsigned), ctx->stream));
    RIMU_CUDA(cudaMemsetAsync(total, 0, sizeof(unsigned long long), ctx->stream));
    unsigned int hflag = 0;
    unsigned long long htot = 0;
    rc = rimu_launch_vec_axpby(ctx, w->recs, w->count, w->capv, v->recs, v->count, v->capv, ro, co,
                               capo, nb, w->val_kind, w->kw, alpha, beta, ia, ib, w_empty ? 1 : 0,
                               flag, total);
    if (!rc) rc = d2h(ctx, &hflag, flag, 1);
    if (!rc) rc = d2h(ctx, &htot, total, 1);
    if (!rc) rc = rimu_cuda_check(cudaStreamSynchronize(ctx->stream), "rimu_vec_add");
    dfree(ctx, flag);
    dfree(ctx, total);
    if (rc || hflag) {
      dfree(ctx, ro);
      dfree(ctx, co);
      if (rc) return rc;
      if (hflag & 1u) return kCrowded;               // the caller splits the buckets further
      capo *= 2;
      continue;
    }
    dfree(ctx, w->recs);
    dfree(ctx, w->count);
    w->recs = ro;
    w->count = co;
    w->capv = capo;
    w->len = (int64_t)htot;
    return RIMU_OK;
  }
  g_err = "rimu_vec_add: capacity overflow";
  return RIMU_ERR_OVERFLOW;
}

extern "C" int rimu_vec_add(rimu_vec *w, const rimu_vec *v, double alpha, double beta) {
  if (!w || !v) return bad("rimu_vec_add: NULL vector");
  if (w->ctx != v->ctx) return bad("rimu_vec_add: vectors of different contexts");
  if (w->kw != v->kw) return bad("rimu_vec_add: vectors of different address widths");
  if (w->val_kind == RIMU_VAL_I64 && v->val_kind != RIMU_VAL_I64)
    return bad("rimu_vec_add: an Int64 list cannot take Float64 values");
  long long ia = 0, ib = 0;
  if (w->val_kind == RIMU_VAL_I64 && (!int_factor(alpha, &ia) || !int_factor(beta, &ib)))
    return bad("rimu_vec_add: an Int64 list takes integer factors only");
  int rc;
  if (w == v) {
    // add!(w, w, alpha, beta): w is scaled first and the scaled w is what gets added
    if ((rc = rimu_vec_scale(w, beta))) return rc;
    rimu_vec tmp;
    tmp.ctx = w->ctx;
    rc = rimu_vec_copy(&tmp, w);
    if (!rc) rc = rimu_vec_add(w, &tmp, alpha, 1.0);
    vec_free(&tmp);
    return rc;
  }
  // v as a list of w's value type with at least w's bucket count, and both bucket counts at
  // least the one that puts about 128 entries of the two lists into a bucket
  rimu_vec tv;
  tv.ctx = v->ctx;
  const rimu_vec *src = v;
  if (v->val_kind != w->val_kind) {                 // Int64 values into a Float64 list
    if ((rc = rimu_vec_convert(&tv, v, w->val_kind))) { vec_free(&tv); return rc; }
    src = &tv;
  }
  const bool w_empty = beta == 0.0;                 // scale!(w, 0) empties w
  int nbits = std::max(std::max(w->nb_bits, src->nb_bits),
                       ceil_log2((uint64_t)((w_empty ? 0 : w->len) + src->len) / 128 + 1));
  for (int attempt = 0; attempt < 6; ++attempt, ++nbits) {
    if (nbits > 26) { rc = RIMU_ERR_OVERFLOW; g_err = "rimu_vec_add: too many buckets"; break; }
    if (src->nb_bits != nbits) {
      if (src != &tv) {
        if ((rc = rimu_vec_copy(&tv, src))) break;
        src = &tv;
      }
      if ((rc = vec_regrid(&tv, nbits, capv_for(tv.len, nbits)))) break;
    }
    if (w->nb_bits != nbits && (rc = vec_regrid(w, nbits, capv_for(w->len, nbits)))) break;
    rc = vec_axpby_same_layout(w, src, alpha, beta, ia, ib, w_empty);
    if (rc != kCrowded) break;                      // a crowded bucket: split further
  }
  if (rc == kCrowded) { rc = RIMU_ERR_OVERFLOW; g_err = "rimu_vec_add: buckets too crowded"; }
  vec_free(&tv);
  if (rc) return rc;
  return rimu_vec_walkernumber_and_length(w, nullptr, nullptr);
}

// ---------------------------------------------------------------------------------------------
// Working memory
// ---------------------------------------------------------------------------------------------
extern "C" int rimu_wm_create(rimu_ctx *ctx, rimu_wm **out) {
  if (!ctx || !out) return bad("rimu_wm_create: NULL argument");
  rimu_wm *w = new rimu_wm();
  w->ctx = ctx;
  *out = w;
  return RIMU_OK;
}

extern "C" int rimu_wm_destroy(rimu_wm *w) {
  if (!w) return RIMU_OK;
  rimu_ctx *ctx = w->ctx;
  dfree(ctx, w->spawn); dfree(ctx, w->scount); dfree(ctx, w->heavy); dfree(ctx, w->heavy_count);
  dfree(ctx, w->stats); dfree(ctx, w->dtab); dfree(ctx, w->d_shift);
  dfree(ctx, w->proj_keys); dfree(ctx, w->proj_v); dfree(ctx, w->proj_h);
  dfree(ctx, w->proj_out_v); dfree(ctx, w->proj_out_h);
  dfree(ctx, w->ann_list); dfree(ctx, w->ann_count);
  cudaStreamSynchronize(ctx->stream);
  for (int i = 0; i < 4; ++i) if (w->ev[i]) cudaEventDestroy(w->ev[i]);
  if (w->h_stats) cudaFreeHost(w->h_stats);
  if (w->h_proj_out) cudaFreeHost(w->h_proj_out);
  delete w;
  return RIMU_OK;
}

extern "C" int rimu_wm_set_timing(rimu_wm *w, int enable) {
  if (!w) return bad("rimu_wm_set_timing: NULL working memory");
  w->timing = enable != 0;
  for (int i = 0; i < 4; ++i) w->t_ms[i] = 0;
  for (int i = 0; i < 3; ++i) w->bytes[i] = 0;
  return RIMU_OK;
}

extern "C" int rimu_wm_set_annihilation(rimu_wm *w, int mode) {
  if (!w) return bad("rimu_wm_set_annihilation: NULL working memory");
  if (mode != RIMU_ANN_HASH && mode != RIMU_ANN_SORT)
    return bad("rimu_wm_set_annihilation: mode must be RIMU_ANN_HASH or RIMU_ANN_SORT");
  w->ann_mode = mode;
  return RIMU_OK;
}

extern "C" int rimu_wm_set_launch_shape(rimu_wm *w, int keys_per_bucket, int table_slots) {
  if (!w) return bad("rimu_wm_set_launch_shape: NULL working memory");
  if (keys_per_bucket < 16 || keys_per_bucket > 4096)
    return bad("rimu_wm_set_launch_shape: keys_per_bucket must be in 16..4096");
  if (table_slots != 0 &&
      (table_slots < 512 || table_slots > 4096 || (table_slots & (table_slots - 1))))
    return bad("rimu_wm_set_launch_shape: table_slots must be 0 or a power of two in 512..4096");
  w->keys_per_bucket = keys_per_bucket;
  w->table_slots = table_slots;
  w->shape_set = true;
  return RIMU_OK;
}

extern "C" int rimu_wm_timing(rimu_wm *w, double *out7) {
  if (!w || !out7) return bad("rimu_wm_timing: NULL argument");
  for (int i = 0; i < 4; ++i) out7[i] = w->t_ms[i];
  for (int i = 0; i < 3; ++i) out7[4 + i] = w->bytes[i];
  return RIMU_OK;
}

// Projector of kw-word addresses (keys: n addresses, kw words each, (lo, hi) for kw = 2).
static int wm_set_projector(rimu_wm *w, const uint64_t *keys, const double *pvals,
                            const double *hpvals, int n, int kw) {
  if (!w || n < 0 || (n > 0 && (!keys || !pvals || !hpvals))) return bad("rimu_wm_set_projector: bad argument");
  rimu_ctx *ctx = w->ctx;
  for (int i = 1; i < n; ++i) {
    const bool up = kw == 1 ? keys[i] > keys[i - 1]
                            : (keys[2 * i + 1] > keys[2 * i - 1] ||
                               (keys[2 * i + 1] == keys[2 * i - 1] && keys[2 * i] > keys[2 * i - 2]));
    if (!up) return bad("rimu_wm_set_projector: keys must be sorted and distinct");
  }
  w->proj_kw = kw;
  dfree(ctx, w->proj_keys); dfree(ctx, w->proj_v); dfree(ctx, w->proj_h);
  dfree(ctx, w->proj_out_v); dfree(ctx, w->proj_out_h);
  if (w->h_proj_out) { cudaStreamSynchronize(ctx->stream); cudaFreeHost(w->h_proj_out); w->h_proj_out = nullptr; }
  w->nproj = n;
  if (n == 0) return RIMU_OK;
  int rc;
  if ((rc = dalloc(ctx, &w->proj_keys, (size_t)n * kw)) || (rc = dalloc(ctx, &w->proj_v, n)) ||
      (rc = dalloc(ctx, &w->proj_h, n)) || (rc = dalloc(ctx, &w->proj_out_v, n)) ||
      (rc = dalloc(ctx, &w->proj_out_h, n)))
    return rc;
  if ((rc = h2d(ctx, w->proj_keys, keys, (size_t)n * kw)) || (rc = h2d(ctx, w->proj_v, pvals, n)) ||
      (rc = h2d(ctx, w->proj_h, hpvals, n)))
    return rc;
  RIMU_CUDA(cudaMallocHost((void **)&w->h_proj_out, 2 * n * sizeof(double)));
  RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
  return RIMU_OK;
}

extern "C" int rimu_wm_set_projector(rimu_wm *w, const uint64_t *keys, const double *pvals,
                                     const double *hpvals, int n) {
  return wm_set_projector(w, keys, pvals, hpvals, n, 1);
}

extern "C" int rimu_wm_set_projector_w(rimu_wm *w, const uint64_t *keys2, const double *pvals,
                                       const double *hpvals, int n) {
  return wm_set_projector(w, keys2, pvals, hpvals, n, 2);
}

static int wm_ensure(rimu_wm *w, int nb_total, uint32_t caps, uint32_t heavy_cap, int ndiag,
                     int kw) {
  rimu_ctx *ctx = w->ctx;
  int rc;
  if (w->nb_total != nb_total || w->caps != caps || w->kw != kw) {
    dfree(ctx, w->spawn);
    dfree(ctx, w->scount);
    dfree(ctx, w->ann_list);
    if ((rc = dalloc(ctx, &w->spawn, (size_t)nb_total * caps * kw)) || (rc = dalloc(ctx, &w->scount, nb_total)) ||
        (rc = dalloc(ctx, &w->ann_list, nb_total)))
      return rc;
    w->kw = kw;
    RIMU_CUDA(cudaMemsetAsync(w->scount, 0, (size_t)nb_total * sizeof(uint32_t), ctx->stream));
    w->nb_total = nb_total;
    w->caps = caps;
  }
  if (w->heavy_cap < heavy_cap) {
    dfree(ctx, w->heavy);
    if ((rc = dalloc(ctx, &w->heavy, heavy_cap))) return rc;
    w->heavy_cap = heavy_cap;
  }
  if (!w->heavy_count && (rc = dalloc(ctx, &w->heavy_count, 1))) return rc;
  if (!w->ann_count && (rc = dalloc(ctx, &w->ann_count, 1))) return rc;
  if (!w->stats) {
    if ((rc = dalloc(ctx, &w->stats, 1))) return rc;
    RIMU_CUDA(cudaMallocHost((void **)&w->h_stats, sizeof(DevStats)));
    w->stats_n = 1;
  }
  if (!w->d_shift && (rc = dalloc(ctx, &w->d_shift, 1))) return rc;
  if (ndiag > w->dtab_n) {
    dfree(ctx, w->dtab);
    if ((rc = dalloc(ctx, &w->dtab, ndiag))) return rc;
    w->dtab_n = ndiag;
  }
  return RIMU_OK;
}

// ---------------------------------------------------------------------------------------------
// The projector step
// ---------------------------------------------------------------------------------------------
extern "C" int rimu_apply_operator(rimu_model *m, rimu_wm *w, rimu_vec *target, const rimu_vec *source_c,
                                   const rimu_step_params *p, rimu_step_stats *out) {
  if (!m || !w || !target || !source_c || !p) return bad("rimu_apply_operator: NULL argument");
  if (target == source_c) return bad("rimu_apply_operator: target and source must differ");
  rimu_vec *source = const_cast<rimu_vec *>(source_c);
  rimu_ctx *ctx = m->ctx;
  if (w->ctx != ctx || target->ctx != ctx || source->ctx != ctx)
    return bad("rimu_apply_operator: handles belong to different contexts");
  if (p->style < 0 || p->style > 2) return bad("rimu_apply_operator: unknown style");
  if ((p->style == RIMU_STYLE_INTEGER) != (source->val_kind == RIMU_VAL_I64))
    return bad("rimu_apply_operator: IsStochasticInteger needs Int64 walkers, other styles Float64");
  if (p->style == RIMU_STYLE_INTEGER && (p->proj_threshold != 0 || p->compression != 0))
    return bad("rimu_apply_operator: thresholding not supported for integer walkers");
  if (p->initiator < RIMU_INIT_NONE || p->initiator > RIMU_INIT_COHERENT)
    return bad("rimu_apply_operator: unknown initiator rule");
  if (p->initiator != RIMU_INIT_NONE && (m->dm.nbits == 64 || m->dm.nbits > 127))
    return bad("rimu_apply_operator: initiator rules need addresses of at most 63 bits or of "
               "65-127 bits (a flag bit above the address)");
  if (!(p->boost > 0)) return bad("rimu_apply_operator: boost must be positive");
  {
    const int need_kw = m->dm.nbits > 64 ? 2 : 1;
    if (source->kw != need_kw)
      return bad("rimu_apply_operator: the vector's address width does not match the model's");
    if (w->nproj != 0 && w->proj_kw != need_kw)
      return bad("rimu_apply_operator: the projector's address width does not match the model's");
    if (target->kw != need_kw) {
      target->kw = need_kw;
      target->nb_bits = -1;                   // forces a new allocation below
    }
  }
  int rc;
  if (p->op == RIMU_OP_TRANSITION && (rc = ensure_aoff(m, p->dt))) return rc;

  // capacity planning: one annihilation CTA per bucket; the bucket count keeps the expected
  // number of contributions (source walkers plus spawns) per bucket between kKeys / 2 and kKeys
  const int64_t L = std::max<int64_t>(source->len, 1);
  const double norm = std::max(source->norm, 1.0);
  int64_t S_est;
  if (w->last_spawns >= 0) S_est = (int64_t)(1.3 * (double)w->last_spawns) + 256;
  else if (p->style == RIMU_STYLE_DETERMINISTIC) S_est = L * (int64_t)m->max_offdiag + 256;
  // about one spawn per attempt, and max(floor(|v| boost), 1) attempts per walker; an
  // underestimate only costs a re-run of this first step with larger slabs
  else S_est = std::max<int64_t>((int64_t)(norm * p->boost), L) + 256;
  // Buckets of one-word addresses without an initiator rule are annihilated one warp each
  // (up to AW_CAP contributions; by default 7/16 to 7/8 of that per bucket, the few fuller
  // buckets left to the CTA kernel); the others one CTA each, 512-1024 per bucket.
  const bool warp_ann = m->dm.nbits <= 64 && p->initiator == RIMU_INIT_NONE;
  double kKeys = (double)(w->shape_set ? w->keys_per_bucket : (warp_ann ? AW_DEFAULT_KPB : 1024));
  // An exact (deterministic) step gives each address all the contributions of its column's
  // length at once: buckets of about eight such lumps keep the fullest bucket, which sets the
  // slab capacity of all of them, within a small factor of the mean.
  if (!w->shape_set && p->style == RIMU_STYLE_DETERMINISTIC)
    kKeys = std::max(kKeys, 8.0 * (double)(m->max_offdiag + 1));
  int need_bits = ceil_log2((uint64_t)((double)(L + S_est) / kKeys) + 1);
  // A source with more than twice the buckets the step needs (a list uploaded or grown for a
  // larger load) is re-bucketed once to need_bits; otherwise buckets only grow.
  int nb_bits = source->nb_bits > need_bits + 1 ? need_bits : std::max(source->nb_bits, need_bits);
  uint32_t caps = 0, capv = 0;
  uint32_t heavy_cap = 0;
  int retries = 0;
  const int ndiag = m->ndiag;
  const uint32_t kMaxCaps = 16384;
  uint32_t min_caps = 0;   // raised after a spawn-slab overflow
  for (;;) {
    if (nb_bits > 26) { g_err = "rimu_apply_operator: too many buckets needed"; return RIMU_ERR_OVERFLOW; }
    if (nb_bits != source->nb_bits) {
      if ((rc = vec_regrid(source, nb_bits, capv_for(source->len, nb_bits)))) return rc;
    }
    const uint64_t nb = 1ull << nb_bits;
    double mu_s = (double)S_est / (double)nb;
    uint32_t want_caps = round_up((uint64_t)(mu_s + 6.0 * std::sqrt(mu_s) + 32.0), 32);
    if (want_caps > kMaxCaps) { nb_bits++; continue; }
    caps = std::min(kMaxCaps, std::max(std::max(caps, want_caps), min_caps));
    // reuse the allocated spawn slabs and target slabs when they are large enough, so
    // that steady-state steps do not reallocate (capacities only grow, with headroom)
    if (w->nb_total == (int)nb && w->caps >= caps && w->caps <= kMaxCaps) caps = w->caps;
    else if (caps < kMaxCaps) caps = std::min(kMaxCaps, round_up((uint64_t)caps * 5 / 4, 32));
    capv = std::max(capv, std::max(source->capv, capv_for((int64_t)(1.5 * L + 64), nb_bits)));
    if (target->nb_bits == nb_bits && target->capv >= capv) capv = target->capv;
    uint64_t work_bound = (uint64_t)(norm * p->boost) + (uint64_t)L * (uint64_t)m->max_offdiag;
    uint64_t hc = work_bound / HEAVY_CHUNK + std::min<uint64_t>((uint64_t)L, work_bound / HEAVY_LIMIT + 1) + 64;
    heavy_cap = std::max<uint32_t>(heavy_cap, (uint32_t)std::min<uint64_t>(hc, 1u << 28));
    heavy_cap = std::max<uint32_t>(heavy_cap, w->heavy_cap);
    if (target->nb_bits != nb_bits || target->capv != capv) {
      if ((rc = vec_alloc(target, nb_bits, capv))) return rc;
    }
    target->val_kind = source->val_kind;
    if ((rc = wm_ensure(w, (int)nb, caps, heavy_cap, ndiag, source->kw))) return rc;
    RIMU_CUDA(cudaMemsetAsync(w->stats, 0, sizeof(DevStats), ctx->stream));
    RIMU_CUDA(cudaMemsetAsync(w->heavy_count, 0, sizeof(uint32_t), ctx->stream));
    if (w->nproj) {
      RIMU_CUDA(cudaMemsetAsync(w->proj_out_v, 0, w->nproj * sizeof(double), ctx->stream));
      RIMU_CUDA(cudaMemsetAsync(w->proj_out_h, 0, w->nproj * sizeof(double), ctx->stream));
    }
    RIMU_CUDA(cudaMemcpyAsync(w->d_shift, &p->shift, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    if (ndiag > 0) {
      if ((rc = rimu_launch_diag_table(ctx, m->dm, p->op, p->dt, w->d_shift, 1, ndiag, w->dtab))) return rc;
    }
    StepArgs a{};
    a.h = m->dm;
    a.style = p->style; a.op = p->op; a.dt = p->dt;
    a.boost = p->boost; a.proj_threshold = p->proj_threshold; a.compression = p->compression;
    a.rel_threshold = p->rel_spawning_threshold; a.abs_threshold = p->abs_spawning_threshold;
    a.has_proj = p->proj_threshold > 0;
    a.comp_mode = p->compression > 0 ? (p->compression == 1.0 ? 1 : 2) : 0;
    a.boost_one = p->boost == 1.0 && p->rel_spawning_threshold == 1.0;
    a.has_abs_thr = std::isfinite(p->abs_spawning_threshold);
    a.init_rule = p->initiator;
    a.init_thr = p->initiator_threshold;
    a.seed = p->seed; a.step = (uint32_t)p->step; a.replica_base = p->replica;
    a.nrep = 1; a.nb_bits = nb_bits;
    a.capv_in = source->capv;
    a.capv = capv; a.caps = caps;
    // annihilation table: room for 5/4 of the expected contributions of a bucket plus one
    // round of insertions by all threads; fuller buckets are processed in several passes
    const double mu_k = (double)(L + S_est) / (double)nb;
    uint32_t T = 512;
    while ((double)T < 1.25 * mu_k + 256.0 && T < 4096) T <<= 1;
    a.tsize = w->table_slots ? (uint32_t)w->table_slots : T;
    if (warp_ann) {
      // the buckets the warps leave hold more than 512 contributions, and one address can
      // receive max_offdiag + 1 of them: the table leaves room for that plus one round
      uint32_t TL = std::max<uint32_t>(T, 2048);
      if ((uint32_t)m->max_offdiag + 1 > TL - 256) TL = 4096;
      a.ann_list = w->ann_list;
      a.ann_count = w->ann_count;
      a.tsize_list = w->table_slots ? (uint32_t)w->table_slots : TL;
      a.ann_sort = w->ann_mode == RIMU_ANN_SORT;
    }
    // spawn chunks of about 256 source walkers per warp
    const double mu_v = (double)L / (double)nb;
    int cb = 1;
    while (cb < 32 && (double)cb * mu_v < 256.0 && cb < (int)nb) cb <<= 1;
    a.spawn_cb = cb;
    a.kw = source->kw;
    a.v_in = source->recs; a.cnt_in = source->count;
    a.v_out = target->recs; a.cnt_out = target->count;
    a.spawn = w->spawn; a.scount = w->scount;
    a.heavy = w->heavy; a.heavy_cap = w->heavy_cap; a.heavy_count = w->heavy_count;
    a.stats = w->stats;
    a.dtab = ndiag > 0 ? w->dtab : nullptr; a.ndiag = ndiag;
    a.shift = w->d_shift;
    a.nproj = w->nproj;
    a.proj_keys = w->proj_keys; a.proj_v = w->proj_v; a.proj_h = w->proj_h;
    a.proj_out_v = w->proj_out_v; a.proj_out_h = w->proj_out_h;
    if (w->timing && !w->ev[0]) {
      for (int i = 0; i < 4; ++i) RIMU_CUDA(cudaEventCreate(&w->ev[i]));
    }
    if ((rc = rimu_launch_step(ctx, a, (int)nb, w->timing ? w->ev : nullptr))) return rc;
    if ((rc = d2h(ctx, w->h_stats, w->stats, 1))) return rc;
    if (w->nproj) {
      if ((rc = d2h(ctx, w->h_proj_out, w->proj_out_v, w->nproj)) ||
          (rc = d2h(ctx, w->h_proj_out + w->nproj, w->proj_out_h, w->nproj)))
        return rc;
    }
    RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
    const DevStats &st = *w->h_stats;
    if (st.flags & FLAG_TABLE) { g_err = "rimu_apply_operator: hash table overflow"; return RIMU_ERR_OVERFLOW; }
    if (st.flags == 0) break;
    if (++retries > 10) { g_err = "rimu_apply_operator: capacities could not be grown enough"; return RIMU_ERR_OVERFLOW; }
    if (st.flags & FLAG_SPAWN_OVERFLOW) {
      S_est = std::max<int64_t>(2 * S_est, (int64_t)st.max_spawn_bucket * (int64_t)nb);
      min_caps = round_up((uint64_t)st.max_spawn_bucket * 5 / 4 + 32, 32);
      if (min_caps > kMaxCaps) { nb_bits++; min_caps = 0; }
      caps = 0;
    }
    if (st.flags & FLAG_V_OVERFLOW) {
      uint64_t want = (uint64_t)st.max_v_bucket * 5 / 4 + 64;
      if (want > 65536) { nb_bits++; capv = 0; }
      else capv = std::max<uint32_t>(2 * capv, round_up(want, 32));
    }
    if (st.flags & FLAG_HEAVY_OVERFLOW) heavy_cap *= 2;
    if (st.flags & FLAG_VALUE_OVERFLOW) { g_err = "rimu_apply_operator: walker value overflow"; return RIMU_ERR_OVERFLOW; }
  }
  const DevStats &st = *w->h_stats;
  if (w->timing) {
    float ms[3];
    cudaEventElapsedTime(&ms[0], w->ev[0], w->ev[1]);
    cudaEventElapsedTime(&ms[1], w->ev[1], w->ev[2]);
    cudaEventElapsedTime(&ms[2], w->ev[2], w->ev[3]);
    for (int i = 0; i < 3; ++i) w->t_ms[i] += ms[i];
    w->t_ms[3] += 1;
    // algorithmic bytes: spawn reads the source and writes the spawns; annihilation reads
    // spawns and source and writes the target (16-byte records)
    const double r = (double)sizeof(Rec) * source->kw;   // record bytes
    w->bytes[0] += r * ((double)source->len + (double)st.spawn_records);
    w->bytes[1] += r * ((double)st.spawn_records + (double)source->len + (double)st.len);
    w->bytes[2] += 1;
  }
  target->len = st.len;
  target->norm = fixed_to_double(U128{st.norm_lo, st.norm_hi});
  w->last_spawns = st.spawn_records;
  if (out) {
    out->norm = target->norm;
    out->len = st.len;
    out->len_before = st.len_before;
    out->exact_steps = st.exact_steps;
    out->inexact_steps = st.inexact_steps;
    out->spawn_attempts = st.spawn_attempts;
    out->spawns = p->style == RIMU_STYLE_INTEGER ? (double)st.spawns_int
                                                 : fixed_to_double(U128{st.spawn_lo, st.spawn_hi});
    out->clones = st.clones; out->deaths = st.deaths; out->zombies = st.zombies;
    double vp = 0.0, hp = 0.0;
    for (int i = 0; i < w->nproj; ++i) { vp += w->h_proj_out[i]; hp += w->h_proj_out[w->nproj + i]; }
    out->vproj = vp;
    out->hproj = hp;
    out->spawn_records = st.spawn_records;
    out->retries = retries;
    out->nb_bits = nb_bits;
  }
  return RIMU_OK;
}

// ---------------------------------------------------------------------------------------------
// Full-basis products
// ---------------------------------------------------------------------------------------------
static int basis_dim(const rimu_model *m, int64_t *dim) {
  bool ovf = false;
  int B = m->dm.nbits, w = m->dm.N;
  if (m->dm.ncomp >= 2) { g_err = "basis: multi-component addresses are not supported"; return RIMU_ERR_BADARG; }
  if (B > 63) { g_err = "basis: address wider than 63 bits"; return RIMU_ERR_BADARG; }
  *dim = binomial_u(B, w, &ovf);
  if (ovf) { g_err = "basis: dimension does not fit int64"; return RIMU_ERR_BADARG; }
  return RIMU_OK;
}

static int ensure_basis_tables(rimu_model *m) {
  ModelExtra *x = extra_of(m);
  if (x->binom) return RIMU_OK;
  rimu_ctx *ctx = m->ctx;
  int B = m->dm.nbits, w = m->dm.N, N = w;
  int ntab = (B + 1) * (w + 1);
  std::vector<uint64_t> tab(ntab, 0);
  for (int p = 0; p <= B; ++p) {
    for (int i = 0; i <= w; ++i) {
      bool ovf = false;
      int64_t c = binomial_u(p, i, &ovf);
      tab[p * (w + 1) + i] = ovf ? ~0ull : (uint64_t)c;
    }
  }
  int rc;
  if ((rc = dalloc(ctx, &x->binom, ntab)) || (rc = h2d(ctx, x->binom, tab.data(), ntab))) return rc;
  x->ntab = ntab;
  int nd = N * (N > 0 ? N - 1 : 0) + 1;
  std::vector<double> dH(nd);
  for (int I = 0; I < nd; ++I) dH[I] = (m->desc.fermion ? 0.0 : m->desc.u * (double)I / 2);
  if ((rc = dalloc(ctx, &x->dtabH, nd)) || (rc = h2d(ctx, x->dtabH, dH.data(), nd))) return rc;
  int np = m->aoff_len;
  std::vector<double> dt(np);
  for (int p = 0; p < np; ++p) dt[p] = -std::sqrt((double)p);
  if ((rc = dalloc(ctx, &x->dhdt, np)) || (rc = h2d(ctx, x->dhdt, dt.data(), np))) return rc;
  if ((rc = dalloc(ctx, &x->out2, 2))) return rc;
  RIMU_CUDA(cudaMallocHost((void **)&x->h_out2, 2 * sizeof(double)));
  RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
  return RIMU_OK;
}

extern "C" int rimu_basis_dimension(rimu_model *m, int64_t *dim) {
  if (!m || !dim) return bad("rimu_basis_dimension: NULL argument");
  return basis_dim(m, dim);
}

extern "C" int rimu_basis_keys(rimu_model *m, int64_t start, int64_t n, uint64_t *keys) {
  if (!m || (n > 0 && !keys)) return bad("rimu_basis_keys: NULL argument");
  int64_t D;
  int rc = basis_dim(m, &D);
  if (rc) return rc;
  if (start < 0 || n < 0 || start + n > D) return bad("rimu_basis_keys: range outside the basis");
  if (n == 0) return RIMU_OK;
  int B = m->dm.nbits, w = m->dm.N;
  // unrank `start` (colex), then step with Gosper's hack
  uint64_t r = (uint64_t)start, key = 0;
  int i = w;
  for (int p = B - 1; p >= 0 && i > 0; --p) {
    bool ovf = false;
    uint64_t c = (uint64_t)binomial_u(p, i, &ovf);
    if (c <= r) { key |= 1ull << p; r -= c; --i; }
  }
  for (int64_t k = 0; k < n; ++k) {
    keys[k] = key;
    if (key == 0) break;
    uint64_t c = key & (~key + 1), s = key + c;
    key = (((s ^ key) >> 2) / c) | s;
  }
  return RIMU_OK;
}

extern "C" int rimu_hv_basis(rimu_model *m, const double *v, double *w, int64_t dim) {
  if (!m || !v || !w) return bad("rimu_hv_basis: NULL argument");
  int64_t D;
  int rc = basis_dim(m, &D);
  if (rc) return rc;
  if (dim != D) return bad("rimu_hv_basis: dim does not match the basis dimension");
  if ((rc = ensure_basis_tables(m))) return rc;
  ModelExtra *x = extra_of(m);
  return rimu_launch_hv(m->ctx, m->dm, x->binom, x->ntab, v, w, dim, x->dtabH);
}

extern "C" int rimu_hv_basis_adjoint(rimu_model *m, const double *v, const double *gw, double *gv,
                                     double *gu, double *gt, int64_t dim) {
  if (!m || !v || !gw || !gv || !gu || !gt) return bad("rimu_hv_basis_adjoint: NULL argument");
  if (!(m->dm.kind == MODEL_REAL1D || (m->dm.kind == MODEL_REALSPACE && !m->dm.fermion && !m->dm.pot)))
    return bad("rimu_hv_basis_adjoint: needs HubbardReal1D or bosonic HubbardRealSpace without trap");
  int64_t D;
  int rc = basis_dim(m, &D);
  if (rc) return rc;
  if (dim != D) return bad("rimu_hv_basis_adjoint: dim does not match the basis dimension");
  if ((rc = ensure_basis_tables(m))) return rc;
  ModelExtra *x = extra_of(m);
  int grid = rimu_hv_grid(m->ctx, dim);
  if (x->partial_n < grid) {
    dfree(m->ctx, x->partial);
    if ((rc = dalloc(m->ctx, &x->partial, 2 * (size_t)grid))) return rc;
    x->partial_n = grid;
  }
  if ((rc = rimu_launch_hv_adjoint(m->ctx, m->dm, x->binom, x->ntab, v, gw, gv, dim, x->dtabH,
                                   x->dhdt, x->partial, grid, x->out2)))
    return rc;
  if ((rc = d2h(m->ctx, x->h_out2, x->out2, 2))) return rc;
  RIMU_CUDA(cudaStreamSynchronize(m->ctx->stream));
  *gu = x->h_out2[0];
  *gt = x->h_out2[1];
  return RIMU_OK;
}
