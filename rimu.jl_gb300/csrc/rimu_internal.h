// rimu_internal.h -- structures shared by the CUDA translation units of librimu_gpu.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <string>
#include <vector>
#include "rimu_device.cuh"
#include "../../include/rimu_gpu.h"

namespace rimu {

// One walker: an address and its amplitude (double or int64 bit pattern).  16 bytes for
// addresses of up to 64 bits, 32 bytes (16-byte aligned) for two-word addresses.
template <class K> struct __align__(16) RecT { K key; uint64_t val; };
using Rec = RecT<uint64_t>;
using Rec2 = RecT<Key128>;

// A heavy column is split into chunks of at most HEAVY_CHUNK spawn attempts.
constexpr int HEAVY_CHUNK = 2048;
constexpr int HEAVY_LIMIT = 1024;   // columns with more work than this go to the heavy list

struct __align__(16) HeavyChunk {
  uint64_t key;      // address (low word)
  uint64_t key_hi;   // high word of a two-word address, else 0
  uint64_t val;      // amplitude bits
  double c;          // spawn coefficient
  int noff;
  int exact;
  uint32_t j0, cnt;
  uint32_t rep;
  uint32_t unsafe;   // 1: a non-initiator's column (initiator rules)
};

// Per-replica step accumulators (zeroed before each step).
struct DevStats {
  unsigned long long norm_lo, norm_hi;       // sum |v'| in 2^-64 fixed point
  unsigned long long spawn_lo, spawn_hi;     // sum |spawn| (float styles) in fixed point
  long long len, len_before;
  long long exact_steps, inexact_steps, spawn_attempts;
  long long spawns_int;
  long long clones, deaths, zombies;
  long long spawn_records;
  unsigned int max_spawn_bucket, max_v_bucket;
  unsigned int flags;
  unsigned int heavy_chunks;
};

enum Flags : unsigned int {
  FLAG_SPAWN_OVERFLOW = 1u, FLAG_V_OVERFLOW = 2u, FLAG_HEAVY_OVERFLOW = 4u,
  FLAG_VALUE_OVERFLOW = 8u, FLAG_TABLE = 16u
};

// Parameters of one launch of the step kernels.
// Warp-per-bucket annihilation: contributions (and table slots) one warp takes, and the
// default expected contributions per bucket of the steps that use it.
#ifndef RIMU_AW_CAP
#define RIMU_AW_CAP 512
#endif
constexpr int AW_CAP = RIMU_AW_CAP;
constexpr int AW_DEFAULT_KPB = AW_CAP * 7 / 8;

struct StepArgs {
  DevModel h;
  int style, op;
  double dt;
  double boost, proj_threshold, compression, rel_threshold, abs_threshold;
  int has_proj;      // proj_threshold > 0
  int comp_mode;     // 0: no compression, 1: threshold 1, 2: other threshold
  int boost_one;     // boost == 1 and rel_threshold == 1
  int has_abs_thr;   // abs_threshold finite
  int init_rule;     // RIMU_INIT_*: initiator rule (0: none)
  double init_thr;   // initiators have |value| > init_thr
  uint64_t seed;
  uint32_t step;
  uint32_t replica_base;
  int nrep;
  int nb_bits;
  uint32_t capv_in;           // slab capacity of the source list
  uint32_t capv, caps, tsize; // target slab, spawn slab, annihilation table slots
  int spawn_cb;               // buckets per warp chunk in k_spawn (power of two <= 32)
  // Replica layout: replica r owns the buckets [rep_off[r], rep_off[r] + 2^rep_bits[r]).
  // When rep_off is null every replica has 2^nb_bits buckets.
  const uint32_t *rep_off;    // [nrep + 1]
  const int *rep_bits;        // [nrep]
  const uint32_t *step_dev;   // when non-null, *step_dev is added to `step` (device counter)
  int kw;                     // address words: 1 (Rec records) or 2 (Rec2 records)
  const void *v_in;
  const uint32_t *cnt_in;
  void *v_out;
  uint32_t *cnt_out;
  void *spawn;
  uint32_t *scount;
  HeavyChunk *heavy;
  uint32_t heavy_cap;
  uint32_t *heavy_count;
  DevStats *stats;            // [nrep]
  const double *dtab;         // [nrep * ndiag] diagonal transition table or null
  int ndiag;
  const double *shift;        // [nrep] shifts (used when dtab == null)
  // ProjectedEnergy: per replica nproj sorted keys, projector values and (H'P) values
  int nproj;
  const uint64_t *proj_keys;  // [nrep * nproj]
  const double *proj_v;
  const double *proj_h;
  double *proj_out_v;         // [nrep * nproj]
  double *proj_out_h;
  // Annihilation kernels: when `ann_list` is set, buckets run first one warp each
  // (k_ann_warp); a bucket with more contributions than a warp's table holds is appended to
  // ann_list (count in *ann_count, reset by k_spawn) and annihilated by a CTA with a table of
  // tsize_list slots afterwards.  Null: every bucket by a CTA with tsize slots.
  uint32_t *ann_list;         // [number of buckets]
  uint32_t *ann_count;
  uint32_t tsize_list;
  int ann_sort;               // with ann_list: the warps sort the spawns (k_ann_sort) instead
                              // of hashing them (k_ann_warp)
};

}  // namespace rimu

struct rimu_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int num_sms = 0;
};

struct rimu_model {
  rimu_ctx *ctx = nullptr;
  rimu_model_desc desc{};
  rimu::DevModel dm{};
  double *d_kes = nullptr, *d_pot = nullptr, *d_aoff = nullptr, *d_hoff = nullptr;
  double *d_recip = nullptr;
  int aoff_len = 0;
  double aoff_dt = -1.0;    // dt of the transition table currently on the device
  int ndiag = 0;            // size of the diagonal table (0: diagonal computed per address)
  int max_offdiag = 0;
};

struct rimu_vec {
  rimu_ctx *ctx = nullptr;
  int val_kind = RIMU_VAL_F64;
  int nb_bits = 0;
  uint32_t capv = 0;
  int kw = 1;               // address words: records are Rec (1) or Rec2 (2, two Rec units)
  rimu::Rec *recs = nullptr;
  uint32_t *count = nullptr;
  int64_t len = 0;          // length after the last operation that changed it
  double norm = 0.0;
};

struct rimu_wm {
  rimu_ctx *ctx = nullptr;
  int nb_total = 0;         // buckets allocated (nrep * 2^nb_bits)
  uint32_t caps = 0;
  rimu::Rec *spawn = nullptr;
  uint32_t *scount = nullptr;
  rimu::HeavyChunk *heavy = nullptr;
  uint32_t heavy_cap = 0;
  uint32_t *heavy_count = nullptr;
  rimu::DevStats *stats = nullptr;
  rimu::DevStats *h_stats = nullptr;   // pinned host copy
  int stats_n = 0;
  double *dtab = nullptr;
  int dtab_n = 0;
  double *d_shift = nullptr;
  int64_t last_spawns = -1;
  int kw = 1;                           // address words of the spawn slabs
  int keys_per_bucket = 1024;           // expected contributions per bucket (launch shape)
  int table_slots = 0;                  // annihilation table slots per CTA (0: automatic)
  bool shape_set = false;               // launch shape chosen by the caller
  int ann_mode = 0;                     // RIMU_ANN_HASH or RIMU_ANN_SORT
  int proj_kw = 1;                      // projector address words: 1, or 2 ((lo, hi) pairs)
  uint32_t *ann_list = nullptr;         // [nb_total] buckets left to the CTA annihilation
  uint32_t *ann_count = nullptr;
  // projector
  int nproj = 0;
  uint64_t *proj_keys = nullptr;
  double *proj_v = nullptr, *proj_h = nullptr, *proj_out_v = nullptr, *proj_out_h = nullptr;
  double *h_proj_out = nullptr;         // pinned [2 * nproj]
  // optional per-kernel timing (CUDA events on the context stream)
  bool timing = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  double t_ms[4] = {0, 0, 0, 0};        // spawn, heavy, annihilate, steps timed
  double bytes[3] = {0, 0, 0};          // algorithmic bytes of spawn, annihilate; steps
};

// error reporting shared by the translation units
void rimu_set_error(const std::string &msg);
int rimu_cuda_check(cudaError_t e, const char *what);
#define RIMU_CUDA(call) do { int _rc = rimu_cuda_check((call), #call); if (_rc) return _rc; } while (0)

// allocation and copies on the context stream (stream-ordered allocator)
template <class T>
inline int dalloc(rimu_ctx *ctx, T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  return rimu_cuda_check(cudaMallocAsync((void **)p, n * sizeof(T), ctx->stream), "cudaMallocAsync");
}
template <class T>
inline void dfree(rimu_ctx *ctx, T *&p) {
  if (p) cudaFreeAsync(p, ctx->stream);
  p = nullptr;
}
template <class T>
inline int h2d(rimu_ctx *ctx, T *d, const T *h, size_t n) {
  if (n == 0) return RIMU_OK;
  return rimu_cuda_check(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream),
                         "cudaMemcpyAsync H2D");
}
template <class T>
inline int d2h(rimu_ctx *ctx, T *h, const T *d, size_t n) {
  if (n == 0) return RIMU_OK;
  return rimu_cuda_check(cudaMemcpyAsync(h, d, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream),
                         "cudaMemcpyAsync D2H");
}
inline int ceil_log2(uint64_t x) {
  int b = 0;
  while ((1ull << b) < x) ++b;
  return b;
}
inline uint32_t round_up(uint64_t x, uint32_t m) { return (uint32_t)((x + m - 1) / m * m); }

// transition-operator offdiagonal table of a model for time step dt (capi.cu)
int ensure_aoff(rimu_model *m, double dt);

// launchers (fciqmc.cu)
// ev (optional, 4 events): recorded before k_spawn, after k_spawn, after k_spawn_heavy and
// after k_annihilate on the context stream.
int rimu_launch_step(rimu_ctx *ctx, const rimu::StepArgs &a, int nb_total,
                     cudaEvent_t *ev = nullptr);
// Walker-list launchers; kw = address words (1: Rec records, 2: Rec2 records and (lo, hi) key
// pairs in the host-side key arrays).
int rimu_launch_bucketize(rimu_ctx *ctx, const uint64_t *keys, const uint64_t *vals, int64_t n,
                          int nb_bits, uint32_t capv, void *recs, uint32_t *count,
                          unsigned int *flag, int kw);
int rimu_launch_rebucket(rimu_ctx *ctx, const void *old_recs, const uint32_t *old_count,
                         int old_nb_bits, uint32_t old_capv, void *recs, uint32_t *count,
                         int nb_bits, uint32_t capv, unsigned int *flag, int kw);
int rimu_launch_compact(rimu_ctx *ctx, const void *recs, const uint32_t *count, int nb,
                        uint32_t capv, const uint64_t *offsets, uint64_t *keys, uint64_t *vals,
                        int kw);
// scale!/add! of walker lists (kw address words, kind RIMU_VAL_*)
int rimu_launch_vec_scale(rimu_ctx *ctx, void *recs, uint32_t *count, int nb, uint32_t capv,
                          int kind, int kw, double alpha, long long ialpha,
                          unsigned long long *removed);
int rimu_launch_vec_axpby(rimu_ctx *ctx, const void *rw, const uint32_t *cw, uint32_t capw,
                          const void *rv, const uint32_t *cv, uint32_t capv, void *ro, uint32_t *co,
                          uint32_t capo, int nb, int kind, int kw, double alpha, double beta,
                          long long ialpha, long long ibeta, int w_empty, unsigned int *flag,
                          unsigned long long *total);
int rimu_launch_norm(rimu_ctx *ctx, const void *recs, const uint32_t *count, int nb,
                     uint32_t capv, int val_kind, unsigned long long *acc3, int kw);
int rimu_launch_lookup(rimu_ctx *ctx, const void *recs, const uint32_t *count, int nb_bits,
                       uint32_t capv, const uint64_t *keys, int64_t n, uint64_t *vals,
                       int *found, int kw);
int rimu_launch_diag_table(rimu_ctx *ctx, const rimu::DevModel &h, int op, double dt,
                           const double *shift, int nrep, int ndiag, double *dtab);
int rimu_launch_diagonal(rimu_ctx *ctx, const rimu::DevModel &h, const uint64_t *keys,
                         int64_t n, double *out);
int rimu_launch_offdiagonals(rimu_ctx *ctx, const rimu::DevModel &h, uint64_t key_lo,
                             uint64_t key_hi, int noff, uint64_t *keys, double *vals);
