// batch.cu -- many independent FCIQMC runs stepped together.
//
// The reference steps the replicas of a ProjectorMonteCarloProblem one after another
// (pmc_simulation.jl:288-290) and runs different Hamiltonians as separate simulations.  Here
// the replicas share one launch of each step kernel: replica r owns the buckets
// [off[r], off[r] + 2^bits[r]) of one bucket array, each replica with as many buckets as its own
// population needs, and its own diagonal table, shift, statistics and projector.  The shift
// update (DoubleLogUpdate, shiftstrategy.jl:174-181) and the step counter live on the device, so a
// segment of steps needs no host round trip and can be replayed as one CUDA graph.  Capacities
// are planned per segment with room for growth; a step that runs out of room sets a flag, and the
// segment is re-run from a snapshot with larger buffers (every step is a pure function of its
// source vector, shifts and the step number).
#include <cuda_runtime.h>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "rimu_internal.h"

using namespace rimu;

namespace {

struct BatchRecord { double shift, norm, vproj, hproj; };

// Diagonal of T per replica: 1 - dt ((u_r I)/2 - S_r), I = sum n(n-1) (the table of k_diag_table
// with the interaction of each replica).
__global__ void k_batch_diag(double dt, const double *u, const double *shift, int nrep, int ndiag,
                             double *dtab) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrep * ndiag) return;
  const int r = i / ndiag, I = i % ndiag;
  const double d = u[r] * (double)I / 2;
  dtab[i] = 1 - dt * (d - shift[r]);
}

// After a step: the new norm of each replica, DoubleLogUpdate of its shift
// S <- S - xi/dt ln(N/N_target) - zeta/dt ln(N/N_previous) (skipped for an empty vector, as in
// advance!, fciqmc.jl:146-160), the ProjectedEnergy sums, and the step counter.
__global__ void k_batch_after_step(const DevStats *st, int nrep, int update, double dt,
                                   double zeta, double xi, const double *target, double *shift,
                                   double *pnorm, int nproj, double *pov, double *poh,
                                   BatchRecord *rec, uint32_t *step) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r == 0) *step += 1;
  if (r >= nrep) return;
  const DevStats &s = st[r];
  const double N = fixed_to_double(U128{s.norm_lo, s.norm_hi});
  double S = shift[r];
  if (update && s.len > 0) {
    S -= xi / dt * log(N / target[r]) + zeta / dt * log(N / pnorm[r]);
    shift[r] = S;
    pnorm[r] = N;
  }
  double vp = 0.0, hp = 0.0;
  for (int i = 0; i < nproj; ++i) {
    const size_t o = (size_t)r * nproj + i;
    vp += pov[o];
    hp += poh[o];
    pov[o] = 0.0;
    poh[o] = 0.0;
  }
  rec[r] = BatchRecord{S, N, vp, hp};
}

int fail_arg(const std::string &msg) {
  rimu_set_error(msg);
  return RIMU_ERR_BADARG;
}

uint32_t capv_of(double mu) {
  return round_up((uint64_t)(1.25 * mu + 8.0 * std::sqrt(mu) + 64.0), 32);
}

}  // namespace

struct rimu_batch {
  rimu_ctx *ctx = nullptr;
  rimu_ctx bctx{};                    // the context with the batch's own stream
  int nrep = 0, val_kind = RIMU_VAL_F64;
  std::vector<rimu_model *> models;
  std::vector<double> u, shift0, target;
  std::vector<std::vector<uint64_t>> hkeys, hvals;   // start vectors until first use
  bool materialized = false;
  // layout
  std::vector<int> bits;
  std::vector<uint32_t> off;          // [nrep + 1]
  uint32_t capv = 0;
  Rec *recs[3] = {nullptr, nullptr, nullptr};        // two step buffers and a snapshot
  uint32_t *cnt[3] = {nullptr, nullptr, nullptr};
  int cur = 0;
  std::vector<int64_t> len, spawns_last;
  std::vector<double> norm, rate;     // rate: growth per step (log) seen in the last segment
  // device state
  uint32_t *d_off = nullptr;
  int *d_bits = nullptr;
  double *d_u = nullptr, *d_shift = nullptr, *d_pnorm = nullptr, *d_target = nullptr;
  double *s_shift = nullptr, *s_pnorm = nullptr;
  uint32_t *d_step = nullptr, *s_step = nullptr;
  double *dtab = nullptr;
  int ndiag = 0;
  // working memory
  Rec *spawn = nullptr;
  uint32_t *scount = nullptr;
  uint32_t *ann_list = nullptr, *ann_count = nullptr;   // buckets left to the CTA annihilation
  uint32_t caps = 0, sp_nb = 0;
  HeavyChunk *heavy = nullptr;
  uint32_t heavy_cap = 0;
  uint32_t *heavy_count = nullptr;
  DevStats *stats = nullptr, *h_stats = nullptr;
  BatchRecord *rec = nullptr, *h_rec = nullptr;
  int kcap = 0;
  // projector
  int nproj = 0;
  bool proj_dirty = false;
  std::vector<std::vector<uint64_t>> pkeys;
  std::vector<std::vector<double>> pvals, phvals;
  uint64_t *proj_keys = nullptr;
  double *proj_v = nullptr, *proj_h = nullptr, *proj_out_v = nullptr, *proj_out_h = nullptr;
  // launch shape and the captured segment
  int kpb = AW_DEFAULT_KPB, tslots = 0;
  int ann_mode = RIMU_ANN_HASH;
  bool tuned = false;
  uint32_t T = 512;
  int spawn_cb = 1;
  cudaGraphExec_t gexec = nullptr;
  int g_k = 0, g_cur = -1;
  uint64_t gen = 1, g_gen = 0;
  rimu_batch_params g_par{};
  // accounting
  int64_t graph_segments = 0, eager_segments = 0, retries = 0, steps_done = 0;
  double kernel_ms = 0.0;
};

static uint32_t nb_total_of(const rimu_batch *b) { return b->off.empty() ? 0 : b->off.back(); }

static void release_graph(rimu_batch *b) {
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  b->gexec = nullptr;
  b->g_gen = 0;
}

// Allocate a bucket array for `bits` and move the current vector into it.
static int regrid(rimu_batch *b, const std::vector<int> &nbits, uint32_t ncapv) {
  rimu_ctx *ctx = &b->bctx;
  std::vector<uint32_t> noff(b->nrep + 1, 0);
  for (int r = 0; r < b->nrep; ++r) noff[r + 1] = noff[r] + (1u << nbits[r]);
  const uint32_t nb = noff.back();
  for (int attempt = 0; attempt < 8; ++attempt) {
    Rec *nr[3] = {nullptr, nullptr, nullptr};
    uint32_t *nc[3] = {nullptr, nullptr, nullptr};
    unsigned int *flag = nullptr;
    int rc = 0;
    for (int i = 0; i < 3 && !rc; ++i)
      if (!(rc = dalloc(ctx, &nr[i], (size_t)nb * ncapv))) rc = dalloc(ctx, &nc[i], nb);
    if (!rc) rc = dalloc(ctx, &flag, 1);
    if (rc) return rc;
    for (int i = 0; i < 3; ++i)
      RIMU_CUDA(cudaMemsetAsync(nc[i], 0, (size_t)nb * sizeof(uint32_t), ctx->stream));
    RIMU_CUDA(cudaMemsetAsync(flag, 0, sizeof(unsigned), ctx->stream));
    if (b->materialized) {
      for (int r = 0; r < b->nrep && !rc; ++r)
        rc = rimu_launch_rebucket(ctx, b->recs[b->cur] + (size_t)b->off[r] * b->capv,
                                  b->cnt[b->cur] + b->off[r], b->bits[r], b->capv,
                                  nr[0] + (size_t)noff[r] * ncapv, nc[0] + noff[r], nbits[r], ncapv,
                                  flag, 1);
    } else {
      for (int r = 0; r < b->nrep && !rc; ++r) {
        const int64_t n = (int64_t)b->hkeys[r].size();
        if (n == 0) continue;
        uint64_t *dk = nullptr, *dv = nullptr;
        if (!(rc = dalloc(ctx, &dk, n)) && !(rc = dalloc(ctx, &dv, n)) &&
            !(rc = h2d(ctx, dk, b->hkeys[r].data(), n)) && !(rc = h2d(ctx, dv, b->hvals[r].data(), n)))
          rc = rimu_launch_bucketize(ctx, dk, dv, n, nbits[r], ncapv,
                                     nr[0] + (size_t)noff[r] * ncapv, nc[0] + noff[r], flag, 1);
        dfree(ctx, dk);
        dfree(ctx, dv);
      }
    }
    unsigned int hflag = 0;
    if (!rc) rc = d2h(ctx, &hflag, flag, 1);
    if (!rc) rc = rimu_cuda_check(cudaStreamSynchronize(ctx->stream), "batch regrid");
    dfree(ctx, flag);
    if (rc) return rc;
    if (hflag) {
      for (int i = 0; i < 3; ++i) { dfree(ctx, nr[i]); dfree(ctx, nc[i]); }
      ncapv *= 2;
      continue;
    }
    for (int i = 0; i < 3; ++i) { dfree(ctx, b->recs[i]); dfree(ctx, b->cnt[i]); b->recs[i] = nr[i]; b->cnt[i] = nc[i]; }
    b->cur = 0;
    b->bits = nbits;
    b->off = noff;
    b->capv = ncapv;
    b->materialized = true;
    b->hkeys.assign(b->nrep, {});
    b->hvals.assign(b->nrep, {});
    dfree(ctx, b->d_off);
    dfree(ctx, b->d_bits);
    if ((rc = dalloc(ctx, &b->d_off, b->nrep + 1)) || (rc = dalloc(ctx, &b->d_bits, b->nrep)) ||
        (rc = h2d(ctx, b->d_off, b->off.data(), b->nrep + 1)) ||
        (rc = h2d(ctx, b->d_bits, b->bits.data(), b->nrep)))
      return rc;
    b->gen++;
    return RIMU_OK;
  }
  rimu_set_error("rimu_batch: bucket capacity overflow while re-bucketing");
  return RIMU_ERR_OVERFLOW;
}

// Buckets, slab capacities and table size for the next segment of steps.
static int plan(rimu_batch *b, const rimu_batch_params *p, int ksteps, int min_caps, int min_capv,
                uint32_t heavy_min) {
  const rimu_model *m0 = b->models[0];
  std::vector<int> nbits(b->nrep);
  double mu_v = 0, mu_s = 0, tot_l = 0, tot_b = 0;
  double work = 0;
  const uint32_t kMaxCaps = 16384;
  for (int r = 0; r < b->nrep; ++r) {
    // room for the growth per step seen so far, over the steps of the next segment
    const double g = std::max(2.0, 1.5 * std::exp(std::min(b->rate[r] * ksteps, std::log(64.0))));
    const double L = (double)std::max<int64_t>(b->len[r], 1);
    double S;
    if (b->spawns_last[r] >= 0) S = 1.3 * (double)b->spawns_last[r] + 256;
    else if (p->style == RIMU_STYLE_DETERMINISTIC) S = L * m0->max_offdiag + 256;
    else S = std::max(b->norm[r], 1.0) * p->boost + 4 * L + 256;
    int need = ceil_log2((uint64_t)(g * (L + S) / b->kpb) + 1);
    // keep the layout unless the replica needs more buckets or has twice too many
    int nbr = b->materialized ? b->bits[r] : need;
    if (need > nbr || need < nbr - 1) nbr = need;
    while (g * S / (double)(1u << nbr) + 6 * std::sqrt(g * S / (double)(1u << nbr)) + 32 > kMaxCaps) ++nbr;
    if (nbr > 24) { rimu_set_error("rimu_batch: too many buckets needed"); return RIMU_ERR_OVERFLOW; }
    nbits[r] = nbr;
    const double nb = (double)(1u << nbr);
    mu_v = std::max(mu_v, g * L / nb);
    mu_s = std::max(mu_s, g * S / nb);
    tot_l += L;
    tot_b += nb;
    work += g * std::max(b->norm[r], 1.0) * p->boost + L * m0->max_offdiag;
  }
  uint32_t ncapv = std::max<uint32_t>(capv_of(mu_v), (uint32_t)min_capv);
  if (b->materialized && nbits == b->bits && ncapv <= b->capv) ncapv = b->capv;
  int rc;
  if (!b->materialized || nbits != b->bits || ncapv != b->capv) {
    if ((rc = regrid(b, nbits, ncapv))) return rc;
    release_graph(b);
  }
  const uint32_t nb_total = nb_total_of(b);
  uint32_t caps = round_up((uint64_t)(mu_s + 6 * std::sqrt(mu_s) + 32), 32);
  caps = std::min(kMaxCaps, std::max(caps, (uint32_t)min_caps));
  if (b->sp_nb == nb_total && b->caps >= caps) caps = b->caps;
  rimu_ctx *ctx = &b->bctx;
  if (b->sp_nb != nb_total || b->caps != caps) {
    dfree(ctx, b->spawn);
    dfree(ctx, b->scount);
    dfree(ctx, b->ann_list);
    if ((rc = dalloc(ctx, &b->spawn, (size_t)nb_total * caps)) || (rc = dalloc(ctx, &b->scount, nb_total)) ||
        (rc = dalloc(ctx, &b->ann_list, nb_total)))
      return rc;
    if (!b->ann_count && (rc = dalloc(ctx, &b->ann_count, 1))) return rc;
    RIMU_CUDA(cudaMemsetAsync(b->scount, 0, (size_t)nb_total * sizeof(uint32_t), ctx->stream));
    b->sp_nb = nb_total;
    b->caps = caps;
    release_graph(b);
  }
  uint64_t hc = (uint64_t)(work / HEAVY_CHUNK) + (uint64_t)std::min(tot_l, work / HEAVY_LIMIT + 1) + 64;
  hc = std::max<uint64_t>(hc, heavy_min);
  if (b->heavy_cap < hc) {
    dfree(ctx, b->heavy);
    const uint32_t cap = (uint32_t)std::min<uint64_t>(hc, 1u << 28);
    if ((rc = dalloc(ctx, &b->heavy, cap))) return rc;
    b->heavy_cap = cap;
    release_graph(b);
  }
  // annihilation table and spawn chunks (the rules of rimu_apply_operator)
  const double mu_k = mu_v + mu_s;
  uint32_t T = 512;
  while ((double)T < 1.25 * mu_k + 256.0 && T < 4096) T <<= 1;
  if (b->tslots) T = (uint32_t)b->tslots;
  int minbits = 31;
  for (int r = 0; r < b->nrep; ++r) minbits = std::min(minbits, b->bits[r]);
  const double mu_avg = tot_l / std::max(tot_b, 1.0);
  int cb = 1;
  while (cb < 32 && (double)cb * mu_avg < 256.0 && cb < (1 << minbits)) cb <<= 1;
  if (T != b->T || cb != b->spawn_cb) release_graph(b);
  b->T = T;
  b->spawn_cb = cb;
  return RIMU_OK;
}

static int ensure_records(rimu_batch *b, int k) {
  if (k <= b->kcap) return RIMU_OK;
  rimu_ctx *ctx = &b->bctx;
  dfree(ctx, b->stats);
  dfree(ctx, b->rec);
  if (b->h_stats) cudaFreeHost(b->h_stats);
  if (b->h_rec) cudaFreeHost(b->h_rec);
  b->h_stats = nullptr;
  b->h_rec = nullptr;
  const size_t n = (size_t)k * b->nrep;
  int rc;
  if ((rc = dalloc(ctx, &b->stats, n)) || (rc = dalloc(ctx, &b->rec, n))) return rc;
  RIMU_CUDA(cudaMallocHost((void **)&b->h_stats, n * sizeof(DevStats)));
  RIMU_CUDA(cudaMallocHost((void **)&b->h_rec, n * sizeof(BatchRecord)));
  b->kcap = k;
  release_graph(b);
  return RIMU_OK;
}

static int upload_projector(rimu_batch *b) {
  if (!b->proj_dirty) return RIMU_OK;
  rimu_ctx *ctx = &b->bctx;
  int np = 0;
  for (int r = 0; r < b->nrep; ++r) np = std::max(np, (int)b->pkeys[r].size());
  dfree(ctx, b->proj_keys);
  dfree(ctx, b->proj_v);
  dfree(ctx, b->proj_h);
  dfree(ctx, b->proj_out_v);
  dfree(ctx, b->proj_out_h);
  b->nproj = np;
  b->proj_dirty = false;
  release_graph(b);
  if (np == 0) return RIMU_OK;
  // per replica np sorted keys, padded with the largest key (never an address) and zeros
  std::vector<uint64_t> k((size_t)b->nrep * np, EMPTY_KEY);
  std::vector<double> pv((size_t)b->nrep * np, 0.0), ph((size_t)b->nrep * np, 0.0);
  for (int r = 0; r < b->nrep; ++r)
    for (size_t i = 0; i < b->pkeys[r].size(); ++i) {
      k[(size_t)r * np + i] = b->pkeys[r][i];
      pv[(size_t)r * np + i] = b->pvals[r][i];
      ph[(size_t)r * np + i] = b->phvals[r][i];
    }
  const size_t n = (size_t)b->nrep * np;
  int rc;
  if ((rc = dalloc(ctx, &b->proj_keys, n)) || (rc = dalloc(ctx, &b->proj_v, n)) ||
      (rc = dalloc(ctx, &b->proj_h, n)) || (rc = dalloc(ctx, &b->proj_out_v, n)) ||
      (rc = dalloc(ctx, &b->proj_out_h, n)) || (rc = h2d(ctx, b->proj_keys, k.data(), n)) ||
      (rc = h2d(ctx, b->proj_v, pv.data(), n)) || (rc = h2d(ctx, b->proj_h, ph.data(), n)))
    return rc;
  RIMU_CUDA(cudaMemsetAsync(b->proj_out_v, 0, n * sizeof(double), ctx->stream));
  RIMU_CUDA(cudaMemsetAsync(b->proj_out_h, 0, n * sizeof(double), ctx->stream));
  return RIMU_OK;
}

// Enqueue step j of a segment that starts from buffer b->cur.
static int enqueue_step(rimu_batch *b, const rimu_batch_params *p, int j) {
  rimu_ctx *ctx = &b->bctx;
  const rimu_model *m0 = b->models[0];
  RIMU_CUDA(cudaMemsetAsync(b->stats + (size_t)j * b->nrep, 0, b->nrep * sizeof(DevStats), ctx->stream));
  RIMU_CUDA(cudaMemsetAsync(b->heavy_count, 0, sizeof(uint32_t), ctx->stream));
  if (b->ndiag > 0) {
    const int n = b->nrep * b->ndiag;
    k_batch_diag<<<(n + 255) / 256, 256, 0, ctx->stream>>>(p->dt, b->d_u, b->d_shift, b->nrep,
                                                          b->ndiag, b->dtab);
    RIMU_CUDA(cudaGetLastError());
  }
  const int src = (b->cur + j) & 1, dst = (b->cur + j + 1) & 1;
  StepArgs a{};
  a.h = m0->dm;
  a.style = p->style;
  a.op = RIMU_OP_TRANSITION;
  a.dt = p->dt;
  a.boost = p->boost;
  a.proj_threshold = p->proj_threshold;
  a.compression = p->compression;
  a.rel_threshold = p->rel_spawning_threshold;
  a.abs_threshold = p->abs_spawning_threshold;
  a.has_proj = p->proj_threshold > 0;
  a.comp_mode = p->compression > 0 ? (p->compression == 1.0 ? 1 : 2) : 0;
  a.boost_one = p->boost == 1.0 && p->rel_spawning_threshold == 1.0;
  a.has_abs_thr = std::isfinite(p->abs_spawning_threshold);
  a.seed = p->seed;
  a.step = 0;
  a.step_dev = b->d_step;
  a.replica_base = 0;
  a.nrep = b->nrep;
  a.nb_bits = 0;
  a.rep_off = b->d_off;
  a.rep_bits = b->d_bits;
  a.capv_in = b->capv;
  a.capv = b->capv;
  a.caps = b->caps;
  a.tsize = b->T;
  // buckets of up to 512 contributions one warp each, the others one CTA each with room for
  // the largest number of contributions one address can receive
  a.ann_list = b->ann_list;
  a.ann_count = b->ann_count;
  {
    uint32_t TL = std::max<uint32_t>(b->T, 2048);
    if ((uint32_t)m0->max_offdiag + 1 > TL - 256) TL = 4096;
    a.tsize_list = b->tslots ? (uint32_t)b->tslots : TL;
  }
  a.ann_sort = b->ann_mode == RIMU_ANN_SORT;
  a.kw = 1;
  a.spawn_cb = b->spawn_cb;
  a.v_in = b->recs[src];
  a.cnt_in = b->cnt[src];
  a.v_out = b->recs[dst];
  a.cnt_out = b->cnt[dst];
  a.spawn = b->spawn;
  a.scount = b->scount;
  a.heavy = b->heavy;
  a.heavy_cap = b->heavy_cap;
  a.heavy_count = b->heavy_count;
  a.stats = b->stats + (size_t)j * b->nrep;
  a.dtab = b->ndiag > 0 ? b->dtab : nullptr;
  a.ndiag = b->ndiag;
  a.shift = b->d_shift;
  a.nproj = b->nproj;
  a.proj_keys = b->proj_keys;
  a.proj_v = b->proj_v;
  a.proj_h = b->proj_h;
  a.proj_out_v = b->proj_out_v;
  a.proj_out_h = b->proj_out_h;
  int rc;
  if ((rc = rimu_launch_step(ctx, a, (int)nb_total_of(b)))) return rc;
  k_batch_after_step<<<(b->nrep + 127) / 128, 128, 0, ctx->stream>>>(
      b->stats + (size_t)j * b->nrep, b->nrep, p->shift_update, p->dt, p->zeta, p->xi, b->d_target,
      b->d_shift, b->d_pnorm, b->nproj, b->proj_out_v, b->proj_out_h, b->rec + (size_t)j * b->nrep,
      b->d_step);
  return rimu_cuda_check(cudaGetLastError(), "k_batch_after_step");
}

static int snapshot(rimu_batch *b, bool restore) {
  rimu_ctx *ctx = &b->bctx;
  const size_t nb = nb_total_of(b);
  const int from = restore ? 2 : b->cur, to = restore ? b->cur : 2;
  RIMU_CUDA(cudaMemcpyAsync(b->recs[to], b->recs[from], nb * b->capv * sizeof(Rec),
                            cudaMemcpyDeviceToDevice, ctx->stream));
  RIMU_CUDA(cudaMemcpyAsync(b->cnt[to], b->cnt[from], nb * sizeof(uint32_t),
                            cudaMemcpyDeviceToDevice, ctx->stream));
  double *sh[2] = {b->d_shift, b->s_shift}, *pn[2] = {b->d_pnorm, b->s_pnorm};
  uint32_t *st[2] = {b->d_step, b->s_step};
  const int f = restore ? 1 : 0, t = restore ? 0 : 1;
  RIMU_CUDA(cudaMemcpyAsync(sh[t], sh[f], b->nrep * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  RIMU_CUDA(cudaMemcpyAsync(pn[t], pn[f], b->nrep * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  RIMU_CUDA(cudaMemcpyAsync(st[t], st[f], sizeof(uint32_t), cudaMemcpyDeviceToDevice, ctx->stream));
  if (restore && b->nproj) {
    const size_t n = (size_t)b->nrep * b->nproj;
    RIMU_CUDA(cudaMemsetAsync(b->proj_out_v, 0, n * sizeof(double), ctx->stream));
    RIMU_CUDA(cudaMemsetAsync(b->proj_out_h, 0, n * sizeof(double), ctx->stream));
  }
  return RIMU_OK;
}

// Run k steps from b->cur, as one captured graph when asked for and possible.
static int run_segment(rimu_batch *b, const rimu_batch_params *p, int k, bool graph, float *ms) {
  rimu_ctx *ctx = &b->bctx;
  cudaEvent_t e0, e1;
  RIMU_CUDA(cudaEventCreate(&e0));
  RIMU_CUDA(cudaEventCreate(&e1));
  int rc = RIMU_OK;
  const bool same = b->gexec && b->g_gen == b->gen && b->g_k == k && b->g_cur == b->cur &&
                    std::memcmp(&b->g_par, p, sizeof(*p)) == 0;
  if (graph && !same) {
    release_graph(b);
    cudaGraph_t gr = nullptr;
    rc = rimu_cuda_check(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal),
                         "cudaStreamBeginCapture");
    for (int j = 0; j < k && !rc; ++j) rc = enqueue_step(b, p, j);
    const int rc2 = rimu_cuda_check(cudaStreamEndCapture(ctx->stream, &gr), "cudaStreamEndCapture");
    if (!rc) rc = rc2;
    if (!rc) rc = rimu_cuda_check(cudaGraphInstantiate(&b->gexec, gr, 0), "cudaGraphInstantiate");
    if (gr) cudaGraphDestroy(gr);
    if (!rc) {
      b->g_gen = b->gen;
      b->g_k = k;
      b->g_cur = b->cur;
      b->g_par = *p;
    }
  }
  if (!rc) rc = rimu_cuda_check(cudaEventRecord(e0, ctx->stream), "cudaEventRecord");
  if (!rc) {
    if (graph) {
      rc = rimu_cuda_check(cudaGraphLaunch(b->gexec, ctx->stream), "cudaGraphLaunch");
      b->graph_segments++;
    } else {
      for (int j = 0; j < k && !rc; ++j) rc = enqueue_step(b, p, j);
      b->eager_segments++;
    }
  }
  if (!rc) rc = rimu_cuda_check(cudaEventRecord(e1, ctx->stream), "cudaEventRecord");
  if (!rc) rc = d2h(ctx, b->h_stats, b->stats, (size_t)k * b->nrep);
  if (!rc) rc = d2h(ctx, b->h_rec, b->rec, (size_t)k * b->nrep);
  if (!rc) rc = rimu_cuda_check(cudaStreamSynchronize(ctx->stream), "batch segment");
  if (!rc) rc = rimu_cuda_check(cudaEventElapsedTime(ms, e0, e1), "cudaEventElapsedTime");
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc;
}

extern "C" int rimu_batch_create(rimu_ctx *ctx, int nrep, int val_kind, rimu_batch **out) {
  if (!ctx || !out) return fail_arg("rimu_batch_create: NULL argument");
  if (nrep < 1 || nrep > 65536) return fail_arg("rimu_batch_create: nrep must be in 1..65536");
  if (val_kind != RIMU_VAL_F64 && val_kind != RIMU_VAL_I64) return fail_arg("rimu_batch_create: bad val_kind");
  rimu_batch *b = new rimu_batch();
  b->ctx = ctx;
  b->bctx = *ctx;
  b->bctx.own_stream = false;
  int rc = rimu_cuda_check(cudaSetDevice(ctx->device), "cudaSetDevice");
  if (!rc) rc = rimu_cuda_check(cudaStreamCreateWithFlags(&b->bctx.stream, cudaStreamNonBlocking),
                                "cudaStreamCreate");
  if (rc) { delete b; return rc; }
  b->nrep = nrep;
  b->val_kind = val_kind;
  b->models.assign(nrep, nullptr);
  b->u.assign(nrep, 0.0);
  b->shift0.assign(nrep, 0.0);
  b->target.assign(nrep, 1000.0);
  b->hkeys.assign(nrep, {});
  b->hvals.assign(nrep, {});
  b->bits.assign(nrep, 0);
  b->len.assign(nrep, 0);
  b->norm.assign(nrep, 0.0);
  b->spawns_last.assign(nrep, -1);
  b->rate.assign(nrep, 0.0);
  b->pkeys.assign(nrep, {});
  b->pvals.assign(nrep, {});
  b->phvals.assign(nrep, {});
  rimu_ctx *c = &b->bctx;
  if ((rc = dalloc(c, &b->d_u, nrep)) || (rc = dalloc(c, &b->d_shift, nrep)) ||
      (rc = dalloc(c, &b->d_pnorm, nrep)) || (rc = dalloc(c, &b->d_target, nrep)) ||
      (rc = dalloc(c, &b->s_shift, nrep)) || (rc = dalloc(c, &b->s_pnorm, nrep)) ||
      (rc = dalloc(c, &b->d_step, 1)) || (rc = dalloc(c, &b->s_step, 1)) ||
      (rc = dalloc(c, &b->heavy_count, 1))) {
    rimu_batch_destroy(b);
    return rc;
  }
  *out = b;
  return RIMU_OK;
}

extern "C" int rimu_batch_destroy(rimu_batch *b) {
  if (!b) return RIMU_OK;
  rimu_ctx *c = &b->bctx;
  release_graph(b);
  for (int i = 0; i < 3; ++i) { dfree(c, b->recs[i]); dfree(c, b->cnt[i]); }
  dfree(c, b->d_off); dfree(c, b->d_bits); dfree(c, b->d_u); dfree(c, b->d_shift);
  dfree(c, b->d_pnorm); dfree(c, b->d_target); dfree(c, b->s_shift); dfree(c, b->s_pnorm);
  dfree(c, b->d_step); dfree(c, b->s_step); dfree(c, b->dtab); dfree(c, b->spawn);
  dfree(c, b->scount); dfree(c, b->heavy); dfree(c, b->heavy_count); dfree(c, b->stats);
  dfree(c, b->ann_list); dfree(c, b->ann_count);
  dfree(c, b->rec); dfree(c, b->proj_keys); dfree(c, b->proj_v); dfree(c, b->proj_h);
  dfree(c, b->proj_out_v); dfree(c, b->proj_out_h);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (b->h_stats) cudaFreeHost(b->h_stats);
  if (b->h_rec) cudaFreeHost(b->h_rec);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete b;
  return RIMU_OK;
}

static bool same_lattice(const rimu_model_desc &a, const rimu_model_desc &c) {
  if (a.kind != c.kind || a.fermion != c.fermion || a.n_particles != c.n_particles ||
      a.n_modes != c.n_modes || a.t != c.t || a.ndim != c.ndim)
    return false;
  for (int i = 0; i < 3; ++i)
    if (a.dims[i] != c.dims[i] || a.periodic[i] != c.periodic[i]) return false;
  return true;
}

extern "C" int rimu_batch_set_replica(rimu_batch *b, int replica, rimu_model *m,
                                      const uint64_t *keys, const void *vals, int64_t n,
                                      double shift, double target_walkers) {
  if (!b || !m || (n > 0 && (!keys || !vals))) return fail_arg("rimu_batch_set_replica: NULL argument");
  if (replica < 0 || replica >= b->nrep) return fail_arg("rimu_batch_set_replica: replica out of range");
  if (m->ctx->device != b->ctx->device) return fail_arg("rimu_batch_set_replica: model on another device");
  if (!(target_walkers > 0)) return fail_arg("rimu_batch_set_replica: target_walkers must be positive");
  if (m->dm.nbits > 64) return fail_arg("rimu_batch_set_replica: batched runs take addresses of at most 64 bits");
  for (int r = 0; r < b->nrep; ++r) {
    const rimu_model *o = b->models[r];
    if (!o || r == replica) continue;
    if (!same_lattice(o->desc, m->desc))
      return fail_arg("rimu_batch_set_replica: replicas need the same lattice, particles and hopping");
    // interactions may differ only where the diagonal is tabulated
    if (o != m && (m->ndiag == 0 || o->ndiag == 0))
      return fail_arg("rimu_batch_set_replica: models without a diagonal table must be the same handle");
  }
  if (b->materialized) return fail_arg("rimu_batch_set_replica: the batch has already run");
  b->models[replica] = m;
  b->u[replica] = m->desc.u;
  b->shift0[replica] = shift;
  b->target[replica] = target_walkers;
  b->hkeys[replica].assign(keys, keys + n);
  const uint64_t *vb = (const uint64_t *)vals;
  b->hvals[replica].assign(vb, vb + n);
  // exact 1-norm and length of the start vector (walkernumber_and_length)
  U128 acc{0, 0};
  for (int64_t i = 0; i < n; ++i) {
    const double x = b->val_kind == RIMU_VAL_I64 ? (double)(int64_t)vb[i] : bitsd(vb[i]);
    acc = add128(acc, fixed_of(x < 0 ? -x : x));
  }
  b->norm[replica] = fixed_to_double(acc);
  b->len[replica] = n;
  return RIMU_OK;
}

extern "C" int rimu_batch_set_projector(rimu_batch *b, int replica, const uint64_t *keys,
                                        const double *pvals, const double *hpvals, int n) {
  if (!b || (n > 0 && (!keys || !pvals || !hpvals))) return fail_arg("rimu_batch_set_projector: NULL argument");
  if (replica < 0 || replica >= b->nrep) return fail_arg("rimu_batch_set_projector: replica out of range");
  std::vector<size_t> o(n);
  for (int i = 0; i < n; ++i) o[i] = i;
  std::sort(o.begin(), o.end(), [&](size_t x, size_t y) { return keys[x] < keys[y]; });
  b->pkeys[replica].clear();
  b->pvals[replica].clear();
  b->phvals[replica].clear();
  for (int i = 0; i < n; ++i) {
    if (i && keys[o[i]] == keys[o[i - 1]]) return fail_arg("rimu_batch_set_projector: repeated address");
    b->pkeys[replica].push_back(keys[o[i]]);
    b->pvals[replica].push_back(pvals[o[i]]);
    b->phvals[replica].push_back(hpvals[o[i]]);
  }
  b->proj_dirty = true;
  return RIMU_OK;
}

extern "C" int rimu_batch_set_launch_shape(rimu_batch *b, int keys_per_bucket, int table_slots) {
  if (!b) return fail_arg("rimu_batch_set_launch_shape: NULL batch");
  if (keys_per_bucket < 16 || keys_per_bucket > 4096)
    return fail_arg("rimu_batch_set_launch_shape: keys_per_bucket must be in 16..4096");
  if (table_slots != 0 && (table_slots < 512 || table_slots > 4096 || (table_slots & (table_slots - 1))))
    return fail_arg("rimu_batch_set_launch_shape: table_slots must be 0 or a power of two in 512..4096");
  b->kpb = keys_per_bucket;
  b->tslots = table_slots;
  b->tuned = true;
  return RIMU_OK;
}

extern "C" int rimu_batch_set_annihilation(rimu_batch *b, int mode) {
  if (!b) return fail_arg("rimu_batch_set_annihilation: NULL batch");
  if (mode != RIMU_ANN_HASH && mode != RIMU_ANN_SORT)
    return fail_arg("rimu_batch_set_annihilation: mode must be RIMU_ANN_HASH or RIMU_ANN_SORT");
  b->ann_mode = mode;
  b->tuned = true;
  return RIMU_OK;
}

extern "C" int rimu_batch_run(rimu_batch *b, const rimu_batch_params *pin, uint64_t first_step,
                              int nsteps, rimu_batch_stats *out) {
  if (!b || !pin) return fail_arg("rimu_batch_run: NULL argument");
  if (nsteps < 0 || (nsteps > 0 && !out)) return fail_arg("rimu_batch_run: bad nsteps or output");
  for (int r = 0; r < b->nrep; ++r)
    if (!b->models[r]) return fail_arg("rimu_batch_run: replica without a model");
  rimu_batch_params p = *pin;
  if (p.style < 0 || p.style > 2) return fail_arg("rimu_batch_run: unknown style");
  if ((p.style == RIMU_STYLE_INTEGER) != (b->val_kind == RIMU_VAL_I64))
    return fail_arg("rimu_batch_run: IsStochasticInteger needs Int64 walkers, other styles Float64");
  if (p.style == RIMU_STYLE_INTEGER && (p.proj_threshold != 0 || p.compression != 0))
    return fail_arg("rimu_batch_run: thresholding not supported for integer walkers");
  if (!(p.boost > 0)) return fail_arg("rimu_batch_run: boost must be positive");
  if (!(p.dt > 0)) return fail_arg("rimu_batch_run: dt must be positive");
  if (p.segment_steps <= 0) p.segment_steps = 64;
  p.segment_steps = (p.segment_steps + 1) & ~1;   // even: a captured segment ends in its start buffer
  rimu_ctx *ctx = &b->bctx;
  int rc;
  RIMU_CUDA(cudaSetDevice(ctx->device));
  rimu_model *m0 = b->models[0];
  if ((rc = ensure_aoff(m0, p.dt))) return rc;
  if (!b->materialized) {
    // device-side per-replica state
    b->ndiag = m0->ndiag;
    if (b->ndiag > 0 && (rc = dalloc(ctx, &b->dtab, (size_t)b->nrep * b->ndiag))) return rc;
    std::vector<double> pn(b->norm);
    if ((rc = h2d(ctx, b->d_u, b->u.data(), b->nrep)) ||
        (rc = h2d(ctx, b->d_shift, b->shift0.data(), b->nrep)) ||
        (rc = h2d(ctx, b->d_pnorm, pn.data(), b->nrep)) ||
        (rc = h2d(ctx, b->d_target, b->target.data(), b->nrep)))
      return rc;
  }
  if ((rc = upload_projector(b))) return rc;
  // the counter holds the number of the next step; k_batch_after_step advances it
  const uint32_t step0 = (uint32_t)(first_step + 1);
  if ((rc = h2d(ctx, b->d_step, &step0, 1))) return rc;
  // the first step of a run after new parameters always runs eagerly (it also sets kernel
  // attributes before any capture)
  int pos = 0;
  int min_caps = 0, min_capv = 0;
  uint32_t heavy_min = 0;
  int tries = 0;
  // segments start short and double up to segment_steps while they succeed; an overflow halves
  // them, so that the growth within one segment stays within the planned room
  int seg = b->steps_done == 0 ? std::min(p.segment_steps, 8) : p.segment_steps;
  std::vector<double> trial_cost;
  // bucket sizes: up to 512 contributions go to one warp each, larger buckets to one CTA
  // each; the warps hash the spawns, or sort them (the last shape)
  constexpr int kShapes = 5;
  const int shapes[kShapes] = {2048, 1024, AW_DEFAULT_KPB, AW_CAP / 2, AW_DEFAULT_KPB};
  const int modes[kShapes] = {RIMU_ANN_HASH, RIMU_ANN_HASH, RIMU_ANN_HASH, RIMU_ANN_HASH,
                              RIMU_ANN_SORT};
  int trial = -1;
  while (pos < nsteps) {
    int64_t tot_len = 0;
    for (int r = 0; r < b->nrep; ++r) tot_len += b->len[r];
    if (p.autotune && !b->tuned && tot_len >= (1 << 20) && trial < 0) trial = 0;
    if (trial >= 0) { b->kpb = shapes[trial]; b->ann_mode = modes[trial]; }
    if ((rc = plan(b, &p, seg, min_caps, min_capv, heavy_min))) return rc;
    int k = std::min(seg, nsteps - pos);
    if (trial >= 0) k = std::min(k, 4);
    if ((rc = ensure_records(b, p.segment_steps))) return rc;
    const bool graph = p.use_graph && trial < 0 && k == p.segment_steps && b->eager_segments > 0;
    if ((rc = snapshot(b, false))) return rc;
    float ms = 0.0f;
    if ((rc = run_segment(b, &p, k, graph, &ms))) return rc;
    unsigned flags = 0;
    uint32_t max_sp = 0, max_v = 0;
    for (int i = 0; i < k * b->nrep; ++i) {
      flags |= b->h_stats[i].flags;
      max_sp = std::max(max_sp, b->h_stats[i].max_spawn_bucket);
      max_v = std::max(max_v, b->h_stats[i].max_v_bucket);
    }
    if (flags & (FLAG_TABLE | FLAG_VALUE_OVERFLOW)) {
      rimu_set_error(flags & FLAG_TABLE ? "rimu_batch_run: annihilation table overflow"
                                        : "rimu_batch_run: walker value overflow");
      return RIMU_ERR_OVERFLOW;
    }
    if (flags) {
      // re-run the segment from the snapshot, shorter and with larger buffers; the steps before
      // the overflow show how far each replica grows
      if (++tries > 30) { rimu_set_error("rimu_batch_run: capacities could not be grown enough"); return RIMU_ERR_OVERFLOW; }
      if ((rc = snapshot(b, true))) return rc;
      RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
      b->retries++;
      for (int r = 0; r < b->nrep; ++r) {
        int64_t ml = 0, ms_ = 0;
        for (int j = 0; j < k; ++j) {
          ml = std::max<int64_t>(ml, b->h_stats[(size_t)j * b->nrep + r].len);
          ms_ = std::max<int64_t>(ms_, b->h_stats[(size_t)j * b->nrep + r].spawn_records);
        }
        const double f = std::max((double)ml / (double)std::max<int64_t>(b->len[r], 1),
                                  (double)ms_ / (double)std::max<int64_t>(b->spawns_last[r], 1));
        b->rate[r] = std::max(2 * b->rate[r], std::log(std::max(f, 1.0)) / k + 0.01);
        b->spawns_last[r] = std::max(b->spawns_last[r], ms_);
      }
      seg = std::max(2, seg / 2);
      if (flags & FLAG_SPAWN_OVERFLOW) min_caps = (int)round_up((uint64_t)max_sp * 5 / 4 + 32, 32);
      if (flags & FLAG_V_OVERFLOW) min_capv = (int)round_up((uint64_t)max_v * 5 / 4 + 64, 32);
      if (flags & FLAG_HEAVY_OVERFLOW) heavy_min = b->heavy_cap * 2;
      continue;
    }
    tries = 0;
    min_caps = min_capv = 0;
    b->kernel_ms += ms;
    b->steps_done += k;
    for (int r = 0; r < b->nrep; ++r) {
      const DevStats &s = b->h_stats[(size_t)(k - 1) * b->nrep + r];
      const double nl = (double)std::max<int64_t>(s.len, 1) / (double)std::max<int64_t>(b->len[r], 1);
      const double nn = b->h_rec[(size_t)(k - 1) * b->nrep + r].norm / std::max(b->norm[r], 1.0);
      b->rate[r] = std::log(std::max(1.0, std::max(nl, nn))) / k;
    }
    double contributions = 0;
    for (int j = 0; j < k; ++j) {
      for (int r = 0; r < b->nrep; ++r) {
        const DevStats &s = b->h_stats[(size_t)j * b->nrep + r];
        const BatchRecord &q = b->h_rec[(size_t)j * b->nrep + r];
        rimu_batch_stats &o = out[(size_t)(pos + j) * b->nrep + r];
        o.shift = q.shift;
        o.norm = q.norm;
        o.vproj = q.vproj;
        o.hproj = q.hproj;
        o.spawns = p.style == RIMU_STYLE_INTEGER ? (double)s.spawns_int
                                                 : fixed_to_double(U128{s.spawn_lo, s.spawn_hi});
        o.len = s.len;
        o.len_before = s.len_before;
        o.exact_steps = s.exact_steps;
        o.inexact_steps = s.inexact_steps;
        o.spawn_attempts = s.spawn_attempts;
        o.spawn_records = s.spawn_records;
        o.clones = s.clones;
        o.deaths = s.deaths;
        o.zombies = s.zombies;
        contributions += (double)s.len + (double)s.spawn_records;
        if (j == 0) b->spawns_last[r] = 0;
        b->spawns_last[r] = std::max<int64_t>(b->spawns_last[r], s.spawn_records);
        if (j == k - 1) { b->len[r] = s.len; b->norm[r] = q.norm; }
      }
    }
    b->cur ^= (k & 1);
    pos += k;
    if (trial < 0) seg = std::min(p.segment_steps, seg * 2);
    if (trial >= 0) {
      trial_cost.push_back(ms / std::max(contributions, 1.0));
      if (++trial == kShapes) {
        const int best = (int)(std::min_element(trial_cost.begin(), trial_cost.end()) - trial_cost.begin());
        b->kpb = shapes[best];
        b->ann_mode = modes[best];
        b->tuned = true;
        trial = -1;
      }
    }
  }
  return RIMU_OK;
}

extern "C" int rimu_batch_download(rimu_batch *b, int replica, uint64_t *keys, void *vals,
                                   int64_t cap, int64_t *n) {
  if (!b || !n) return fail_arg("rimu_batch_download: NULL argument");
  if (replica < 0 || replica >= b->nrep) return fail_arg("rimu_batch_download: replica out of range");
  if (!b->materialized) {
    const int64_t m = (int64_t)b->hkeys[replica].size();
    *n = m;
    if (m > cap || (m && (!keys || !vals))) return fail_arg("rimu_batch_download: buffer too small");
    std::copy(b->hkeys[replica].begin(), b->hkeys[replica].end(), keys);
    std::copy(b->hvals[replica].begin(), b->hvals[replica].end(), (uint64_t *)vals);
    return RIMU_OK;
  }
  rimu_ctx *ctx = &b->bctx;
  const int nb = 1 << b->bits[replica];
  const uint32_t o = b->off[replica];
  std::vector<uint32_t> c(nb);
  int rc;
  if ((rc = d2h(ctx, c.data(), b->cnt[b->cur] + o, nb))) return rc;
  RIMU_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<uint64_t> offs(nb);
  uint64_t tot = 0;
  for (int i = 0; i < nb; ++i) { offs[i] = tot; tot += std::min(c[i], b->capv); }
  *n = (int64_t)tot;
  if (tot == 0) return RIMU_OK;
  if ((int64_t)tot > cap || !keys || !vals) return fail_arg("rimu_batch_download: buffer too small");
  uint64_t *doff = nullptr, *dk = nullptr, *dv = nullptr;
  if ((rc = dalloc(ctx, &doff, nb)) || (rc = dalloc(ctx, &dk, tot)) || (rc = dalloc(ctx, &dv, tot))) return rc;
  if (!(rc = h2d(ctx, doff, offs.data(), nb)) &&
      !(rc = rimu_launch_compact(ctx, b->recs[b->cur] + (size_t)o * b->capv, b->cnt[b->cur] + o, nb,
                                 b->capv, doff, dk, dv, 1)) &&
      !(rc = d2h(ctx, keys, dk, tot)))
    rc = d2h(ctx, (uint64_t *)vals, dv, tot);
  dfree(ctx, doff);
  dfree(ctx, dk);
  dfree(ctx, dv);
  if (rc) return rc;
  return rimu_cuda_check(cudaStreamSynchronize(ctx->stream), "rimu_batch_download");
}

extern "C" int rimu_batch_annihilation(rimu_batch *b, int *mode) {
  if (!b || !mode) return fail_arg("rimu_batch_annihilation: NULL argument");
  *mode = b->ann_mode;
  return RIMU_OK;
}

extern "C" int rimu_batch_info(rimu_batch *b, double *out8) {
  if (!b || !out8) return fail_arg("rimu_batch_info: NULL argument");
  out8[0] = b->kpb;
  out8[1] = b->T;
  out8[2] = nb_total_of(b);
  out8[3] = (double)b->graph_segments;
  out8[4] = (double)b->eager_segments;
  out8[5] = (double)b->retries;
  out8[6] = b->kernel_ms;
  out8[7] = (double)b->steps_done;
  return RIMU_OK;
}
