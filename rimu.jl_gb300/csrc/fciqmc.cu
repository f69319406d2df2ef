// fciqmc.cu -- kernels of one FCIQMC projector step on a bucketed, device-resident walker list.
//
// Layout in HBM.  A walker list is 2^nb_bits buckets per replica; bucket b holds the walkers
// whose address hashes (top nb_bits of mix64) to b, as 16-byte (address, amplitude) records
// in a fixed-capacity slab [b * capv, b * capv + count[b]).  The spawn buffer uses the same
// buckets with slabs of capacity caps.
//
// One step (apply_operator!, src/Interfaces/dictvectors.jl:112-140):
//   k_spawn      each warp lays the walkers of 32 consecutive buckets out as one list,
//                evaluates their columns and deals the spawn attempts out to its lanes in
//                work items of G units; every spawn is written straight into the slab of
//                its destination bucket (perform_spawns!, pdworkingmemory.jl:208-217).
//                Columns with more than HEAVY_LIMIT units are cut into chunks.
//   k_spawn_heavy  processes the chunks of heavy columns on all SMs.
//   k_annihilate one warp per bucket: the source walkers (after their diagonal step) and the
//                spawns go into a shared-memory table holding one exact 128-bit fixed-point
//                sum per address; the sums are rounded once, threshold compression applied,
//                statistics and the norm accumulated exactly, and the survivors written to
//                the target slab (collect_local!/move_and_compress!,
//                pdworkingmemory.jl:228-273; compression.jl:18-42).
#include <cuda_runtime.h>
#include <cstdio>
#include "rimu_internal.h"

namespace rimu {


// ------------------------------------------------------------------------------------------
// Model dispatch
// ------------------------------------------------------------------------------------------
template <int KIND>
__device__ __forceinline__ int column_noff(const DevModel &h, uint64_t key) {
  if (KIND == MODEL_MOM1D) {
    MomMap m;
    mom_map(key, m);
    return num_offdiagonals_mom(h, m);
  }
  return num_offdiagonals_real(h, key);
}

template <int KIND>
__device__ __forceinline__ Offdiag column_offdiag(const DevModel &h, uint64_t key, int chosen) {
  if (KIND == MODEL_REAL1D) return real1d_offdiag(h, key, chosen);
  if (KIND == MODEL_REALSPACE) return realspace_offdiag(h, key, chosen);
  MomMap m;
  mom_map(key, m);
  return mom1d_offdiag(h, key, m, chosen);
}

// sum_i n_i (n_i - 1) of a BoseFS key (bose_hubbard_interaction, bosefs.jl:415-428)
__device__ __forceinline__ int bose_interaction(uint64_t key) {
  uint64_t x = key;
  int acc = 0;
  while (x) {
    x = shr64(x, ctz64(x));
    int n = ctz64(~x);
    acc += n * (n - 1);
    x = shr64(x, n);
  }
  return acc;
}

// Hamiltonian diagonal computed per address (HubbardRealSpace with trap, HubbardMom1D).
template <int KIND>
__device__ double model_diagonal(const DevModel &h, uint64_t key) {
  if (KIND == MODEL_MOM1D) {
    // dot(h.kes, map) + u/(2M) * momentum_transfer_diagonal(map)  (HubbardMom1D.jl:174-177)
    uint64_t x = key;
    int mode = 1, s = 0;
    int occ[MAX_MODES];
    double kin = 0.0;
    while (x) {
      int z = ctz64(x);
      x = shr64(x, z); mode += z;
      int n = ctz64(~x);
      kin += h.kes[mode - 1] * (double)n;
      occ[s++] = n;
      x = shr64(x, n);
    }
    long long onp = 0;
    for (int i = 0; i < s; ++i) {
      onp += (long long)occ[i] * (occ[i] - 1);
      for (int j = 0; j < i; ++j) onp += 4LL * occ[i] * occ[j];
    }
    return kin + h.u / (2 * h.M) * (double)onp;
  }
  if (KIND == MODEL_REAL1D) return h.u * (double)bose_interaction(key) / 2;
  // HubbardRealSpace one component (HubbardRealSpace.jl:284-293)
  double in = 0.0;
  if (!h.fermion && h.u != 0.0) in = h.u * (double)bose_interaction(key) / 2;
  double pe = 0.0;
  if (h.pot) {
    if (h.fermion) {
      uint64_t x = key;
      while (x) { int b = ctz64(x); pe += 1.0 * h.pot[b]; x &= x - 1; }
    } else {
      uint64_t x = key;
      int mode = 1;
      while (x) {
        int z = ctz64(x);
        x = shr64(x, z); mode += z;
        int n = ctz64(~x);
        pe += (double)n * h.pot[mode - 1];
        x = shr64(x, n);
      }
    }
  }
  return in + pe;
}

// Diagonal element of the applied operator for replica r.
template <int KIND>
__device__ __forceinline__ double op_diagonal(const StepArgs &a, int r, uint64_t key) {
  if (a.dtab) {
    int I = a.h.fermion ? 0 : bose_interaction_fast(key);
    return a.dtab[(size_t)r * a.ndiag + I];
  }
  double d = model_diagonal<KIND>(a.h, key);
  return a.op == OP_TRANSITION ? 1 - a.dt * (d - a.shift[r]) : d;
}

// Offdiagonal element of the applied operator: -H_{new,key} dt (fciqmc.jl:109-112) or H.
__device__ __forceinline__ double op_offdiag(const StepArgs &a, const Offdiag &od) {
  const double *tab = a.op == OP_TRANSITION ? a.h.aoff : a.h.hoff;
  double v = tab[od.prod];
  return od.sign < 0 ? -v : v;
}

// ------------------------------------------------------------------------------------------
// Statistics
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ U128 shfl_down128(U128 v, int o) {
  U128 r;
  r.lo = __shfl_down_sync(0xffffffffu, v.lo, o);
  r.hi = __shfl_down_sync(0xffffffffu, v.hi, o);
  return r;
}
__device__ __forceinline__ long long warp_sum(long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ U128 warp_sum128(U128 v) {
  for (int o = 16; o > 0; o >>= 1) v = add128(v, shfl_down128(v, o));
  return v;
}
__device__ __forceinline__ void atomic_add128(unsigned long long *lo, unsigned long long *hi,
                                              U128 v) {
  if (v.lo == 0 && v.hi == 0) return;
  unsigned long long old = atomicAdd(lo, (unsigned long long)v.lo);
  unsigned long long carry = (old + v.lo < old) ? 1ull : 0ull;
  if (v.hi + carry) atomicAdd(hi, (unsigned long long)(v.hi + carry));
}
__device__ __forceinline__ void atomic_add_ll(long long *p, long long v) {
  if (v) atomicAdd((unsigned long long *)p, (unsigned long long)v);
}
__device__ __forceinline__ uint32_t lanemask_lt() {
  return (1u << (threadIdx.x & 31)) - 1u;
}

// ------------------------------------------------------------------------------------------
// Spawning: a warp spreads the walkers of CHUNK_BUCKETS consecutive buckets over its lanes
// ------------------------------------------------------------------------------------------
struct SpawnAcc {
  long long attempts, exact_n, inexact_n;
};

constexpr int WARPS = 8;            // warps per CTA in the step kernels
constexpr int G = 4;                // units (attempts or offdiagonals) per work item
constexpr int CHUNK_BUCKETS = 32;   // buckets whose walkers one warp processes together
constexpr int BATCH = 64;           // walkers whose work items are distributed together

__device__ __forceinline__ void emit_spawn(const StepArgs &a, int r, uint64_t nk, uint64_t vb) {
  const uint32_t b = ((uint32_t)r << a.nb_bits) | bucket_of(nk, a.nb_bits);
  const uint32_t pos = atomicAdd(&a.scount[b], 1u);
  if (pos < a.caps) a.spawn[(size_t)b * a.caps + pos] = Rec{nk, vb};
  else atomicOr(&a.stats[r].flags, (unsigned)FLAG_SPAWN_OVERFLOW);
}

template <int KIND>
__device__ __forceinline__ Offdiag step_offdiag(const DevModel &h, uint64_t key, int chosen) {
  if (KIND == MODEL_REAL1D) return real1d_offdiag_fast(key, h.nbits, chosen);
  return column_offdiag<KIND>(h, key, chosen);
}

// Units [j0, j1) of one column, j0 a multiple of G.  Exact columns deposit val * T_{new,key}
// for offdiagonals j+1 (spawning.jl:174-182); sampled columns draw a uniform offdiagonal per
// attempt and deposit c * T_{new,key} (spawning.jl:232-243).  With float walkers and no
// on-the-fly projection an attempt needs 32 random bits, so one Philox block serves the four
// attempts 4q..4q+3.
template <int KIND, int STYLE>
__device__ __forceinline__ void spawn_units(const StepArgs &a, int r, uint64_t key, uint64_t vb,
                                            double c, int noff, int exact, uint32_t j0,
                                            uint32_t j1) {
  const uint32_t rep = a.replica_base + (uint32_t)r;
  if (exact) {
    const double val = bitsd(vb);
    for (uint32_t j = j0; j < j1; ++j) {
      const Offdiag od = step_offdiag<KIND>(a.h, key, (int)j + 1);
      if (od.prod == 0) continue;
      double y = val * op_offdiag(a, od);
      if (STYLE == STYLE_DSS && a.has_proj) {
        const U4 rr = draw(a.seed, PURPOSE_SPAWN, rep, a.step, key, j);
        y = project_threshold(y, a.proj_threshold, u53_of(rr));
      }
      if (is_zero_d(y)) continue;
      emit_spawn(a, r, od.key, dbits(y));
    }
    return;
  }
  const bool grouped = STYLE != STYLE_INTEGER && !a.has_proj;
  U4 blk{0, 0, 0, 0};
  if (grouped) blk = draw(a.seed, PURPOSE_SPAWN, rep, a.step, key, j0 >> 2);
  for (uint32_t j = j0; j < j1; ++j) {
    U4 rr = blk;
    uint32_t word;
    if (grouped) {
      const uint32_t q = j & 3;
      word = q == 0 ? blk.x : q == 1 ? blk.y : q == 2 ? blk.z : blk.w;
    } else {
      rr = draw(a.seed, PURPOSE_SPAWN, rep, a.step, key, j);
      word = rr.x;
    }
    const int chosen = (int)uniform_index(word, (uint32_t)noff) + 1;
    const Offdiag od = step_offdiag<KIND>(a.h, key, chosen);
    if (od.prod == 0) continue;
    double y = c * op_offdiag(a, od);
    if (STYLE == STYLE_INTEGER) {
      const int64_t k = round_stochastic(y, u53_of(rr));
      if (k == 0) continue;
      emit_spawn(a, r, od.key, (uint64_t)k);
    } else {
      if (a.has_proj) y = project_threshold(y, a.proj_threshold, u53_of(rr));
      if (is_zero_d(y)) continue;
      emit_spawn(a, r, od.key, dbits(y));
    }
  }
}

__device__ __forceinline__ void flush_spawn_acc(const StepArgs &a, int r, SpawnAcc &acc) {
  const long long at = warp_sum(acc.attempts);
  const long long ex = warp_sum(acc.exact_n), ie = warp_sum(acc.inexact_n);
  if ((threadIdx.x & 31) == 0) {
    DevStats &st = a.stats[r];
    atomic_add_ll(&st.spawn_attempts, at);
    atomic_add_ll(&st.exact_steps, ex);
    atomic_add_ll(&st.inexact_steps, ie);
  }
  acc = SpawnAcc{};
}

__device__ __forceinline__ double dint_of(const DevModel &h, int n) {
  return n < h.recip_len ? h.dint[n] : (double)n;
}

// Work of one column: units (offdiagonals if exact, attempts otherwise) and the spawn
// coefficient c, without FP64 compares (DynamicSemistochastic, spawning.jl:364-378;
// WithReplacement attempts, spawning.jl:234-235).
template <int KIND, int STYLE>
__device__ __forceinline__ uint64_t column_work(const StepArgs &a, uint64_t key, uint64_t vb,
                                                int &noff, int &exact, double &c,
                                                SpawnAcc &acc) {
  noff = column_noff<KIND>(a.h, key);
  exact = 0;
  c = 0.0;
  uint64_t natt = 0;
  if (STYLE == STYLE_DETERMINISTIC) {
    exact = 1;
    acc.exact_n++;
  } else if (STYLE == STYLE_DSS) {
    const double val = bitsd(vb);
    const double amount = a.boost_one ? abs_d(val) : a.boost * abs_d(val) * a.rel_threshold;
    if (!a.has_abs_thr || a.abs_threshold >= (double)noff) exact = floor_abs(amount) >= (int64_t)noff;
    else exact = amount >= a.abs_threshold;
    if (exact) acc.exact_n++; else acc.inexact_n++;
    if (!exact) {
      natt = (uint64_t)floor_abs(a.boost_one ? val : abs_d(val) * a.boost);
      if (natt < 1) natt = 1;
      const double rc = natt < (uint64_t)a.h.recip_len ? a.h.recip[natt] : 1.0 / (double)natt;
      c = (natt == 1 ? val : val * rc) * dint_of(a.h, noff);
    }
  } else {  // IsStochasticInteger
    const int64_t iv = (int64_t)vb;
    const uint64_t av = (uint64_t)(iv < 0 ? -iv : iv);
    if (a.boost_one) {
      natt = av < 1 ? 1 : av;
      const double dn = dint_of(a.h, noff);
      c = iv < 0 ? bitsd(dbits(dn) ^ 0x8000000000000000ull) : dn;
    } else {
      natt = (uint64_t)floor_abs(i2d_exact(iv) * a.boost);
      if (natt < 1) natt = 1;
      const double rc = natt < (uint64_t)a.h.recip_len ? a.h.recip[natt] : 1.0 / (double)natt;
      c = (i2d_exact(iv) * rc) * dint_of(a.h, noff);
    }
  }
  return noff == 0 ? 0 : (exact ? (uint64_t)noff : natt);
}

// Cut a column with more than HEAVY_LIMIT units into chunks for k_spawn_heavy.
__device__ void push_heavy(const StepArgs &a, int r, const Rec &rec, double c, int noff,
                           int exact, uint64_t work) {
  const uint64_t nch = (work + HEAVY_CHUNK - 1) / HEAVY_CHUNK;
  const uint32_t idx = atomicAdd(a.heavy_count, (uint32_t)nch);
  for (uint64_t k = 0; k < nch; ++k) {
    if (idx + k >= a.heavy_cap) {
      atomicOr(&a.stats[r].flags, (unsigned)FLAG_HEAVY_OVERFLOW);
      break;
    }
    HeavyChunk ch;
    ch.key = rec.key; ch.val = rec.val; ch.c = c; ch.noff = noff; ch.exact = exact;
    ch.j0 = (uint32_t)(k * HEAVY_CHUNK);
    const uint64_t rem = work - k * HEAVY_CHUNK;
    ch.cnt = (uint32_t)(rem < (uint64_t)HEAVY_CHUNK ? rem : HEAVY_CHUNK);
    ch.rep = (uint32_t)r; ch.pad = 0;
    a.heavy[idx + k] = ch;
  }
}

// Each warp takes CHUNK_BUCKETS consecutive buckets of one replica, lays their walkers out
// as one flat list and works through it BATCH walkers at a time: every lane evaluates the
// column of one or two walkers, then the batch's work items (G units each) are dealt out to
// the lanes by an exclusive scan and a binary search.
template <int KIND, int STYLE>
__global__ void __launch_bounds__(WARPS * 32, 3) k_spawn(StepArgs a, int nb_total) {
  __shared__ uint32_t s_bpre[WARPS][CHUNK_BUCKETS + 1];
  __shared__ uint64_t s_key[WARPS][BATCH];
  __shared__ uint64_t s_val[WARPS][BATCH];
  __shared__ double s_c[WARPS][BATCH];
  __shared__ uint32_t s_units[WARPS][BATCH];
  __shared__ uint32_t s_excl[WARPS][BATCH];
  __shared__ uint32_t s_meta[WARPS][BATCH];   // noff | exact << 31
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int cb = a.nb_bits < 5 ? (1 << a.nb_bits) : CHUNK_BUCKETS;
  const int nchunks = nb_total / cb;
  SpawnAcc acc{};
  int cur_r = -1;
  for (int ch = blockIdx.x * WARPS + w; ch < nchunks; ch += gridDim.x * WARPS) {
    const int b0 = ch * cb;
    const int r = b0 >> a.nb_bits;
    if (r != cur_r) {
      if (cur_r >= 0) flush_spawn_acc(a, cur_r, acc);
      cur_r = r;
    }
    uint32_t n = 0;
    if (lane < cb) {
      n = a.cnt_in[b0 + lane];
      if (n > a.capv_in) n = a.capv_in;
    }
    uint32_t incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 0) s_bpre[w][0] = 0;
    s_bpre[w][lane + 1] = incl;
    const uint32_t E = __shfl_sync(0xffffffffu, incl, 31);
    __syncwarp();
    for (uint32_t e0 = 0; e0 < E; e0 += BATCH) {
      uint32_t items[2];
#pragma unroll
      for (int hh = 0; hh < 2; ++hh) {
        const uint32_t f = e0 + (uint32_t)(hh * 32 + lane);
        const int slot = hh * 32 + lane;
        uint32_t it = 0, units = 0;
        if (f < E) {
          int bi = 0;
#pragma unroll
          for (int st = 16; st >= 1; st >>= 1)
            if (bi + st < cb && s_bpre[w][bi + st] <= f) bi += st;
          const Rec rec = a.v_in[(size_t)(b0 + bi) * a.capv_in + (f - s_bpre[w][bi])];
          int noff, exact;
          double c;
          uint64_t work = column_work<KIND, STYLE>(a, rec.key, rec.val, noff, exact, c, acc);
          if (work > (1ull << 36)) {       // more attempts than any walker list can hold
            atomicOr(&a.stats[r].flags, (unsigned)FLAG_VALUE_OVERFLOW);
            work = 0;
          }
          acc.attempts += (long long)work;
          if (work > (uint64_t)HEAVY_LIMIT) {
            push_heavy(a, r, rec, c, noff, exact, work);
            work = 0;
          }
          s_key[w][slot] = rec.key;
          s_val[w][slot] = rec.val;
          s_c[w][slot] = c;
          s_meta[w][slot] = (uint32_t)noff | ((uint32_t)exact << 31);
          units = (uint32_t)work;
          it = (units + G - 1) / G;
        }
        s_units[w][slot] = units;
        items[hh] = it;
      }
      uint32_t in0 = items[0], in1 = items[1];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y0 = __shfl_up_sync(0xffffffffu, in0, o);
        const uint32_t y1 = __shfl_up_sync(0xffffffffu, in1, o);
        if (lane >= o) { in0 += y0; in1 += y1; }
      }
      const uint32_t tot0 = __shfl_sync(0xffffffffu, in0, 31);
      const uint32_t total = tot0 + __shfl_sync(0xffffffffu, in1, 31);
      s_excl[w][lane] = in0 - items[0];
      s_excl[w][32 + lane] = tot0 + in1 - items[1];
      __syncwarp();
      for (uint32_t it = lane; it < total; it += 32) {
        int lo = 0;
#pragma unroll
        for (int st = 32; st >= 1; st >>= 1)
          if (s_excl[w][lo + st] <= it) lo += st;
        const uint32_t j0 = (it - s_excl[w][lo]) * G;
        const uint32_t ju = s_units[w][lo];
        const uint32_t j1 = j0 + G < ju ? j0 + G : ju;
        const uint32_t meta = s_meta[w][lo];
        spawn_units<KIND, STYLE>(a, r, s_key[w][lo], s_val[w][lo], s_c[w][lo],
                                 (int)(meta & 0x7fffffffu), (int)(meta >> 31), j0, j1);
      }
      __syncwarp();
    }
  }
  if (cur_r >= 0) flush_spawn_acc(a, cur_r, acc);
}

template <int KIND, int STYLE>
__global__ void __launch_bounds__(256) k_spawn_heavy(StepArgs a) {
  uint32_t nch = *a.heavy_count;
  if (nch > a.heavy_cap) nch = a.heavy_cap;
  for (uint32_t ci = blockIdx.x; ci < nch; ci += gridDim.x) {
    HeavyChunk ch = a.heavy[ci];
    if (ch.cnt > (uint32_t)HEAVY_CHUNK || ch.rep >= (uint32_t)a.nrep || (ch.j0 & (G - 1))) {
      if (threadIdx.x == 0) atomicOr(&a.stats[0].flags, (unsigned)FLAG_TABLE);
      continue;
    }
    for (uint32_t t = threadIdx.x * G; t < ch.cnt; t += blockDim.x * G) {
      const uint32_t j1 = t + G < ch.cnt ? t + G : ch.cnt;
      spawn_units<KIND, STYLE>(a, (int)ch.rep, ch.key, ch.val, ch.c, ch.noff, ch.exact,
                               ch.j0 + t, ch.j0 + j1);
    }
  }
}

// ------------------------------------------------------------------------------------------
// Annihilation: one warp per bucket, exact fixed-point sums in a shared-memory table
// ------------------------------------------------------------------------------------------
// Summation rule (the oracle states the same): when every contribution to an address is a
// multiple of 2^-64 below 2^48 in magnitude, the address gets the exact sum rounded once to
// the nearest double, so the order of the contributions does not matter; otherwise the
// contributions are added in canonical order (the diagonal term, then the spawns by
// increasing value).  Integer walkers are summed as int64.
struct AnnAcc {
  U128 norm, spawn_fx;
  long long len, len_before, clones, deaths, zombies, spawns_i, records;
};

// Statistics of one pass over a bucket; kept only if the pass completes.
struct PassAcc {
  U128 spawn_fx;
  long long clones, deaths, zombies, spawns_i, records;
};

constexpr uint32_t INFO_INEXACT = 1u;   // tinfo bit 0; bits 1..31: 1 + source walker index
constexpr int MAX_SPLIT = 16;           // at most 2^MAX_SPLIT passes over one bucket

// Per-warp table of T slots: keys, 128-bit sums (lo, hi), info words, occupied-slot list.
__host__ __device__ inline size_t ann_warp_smem(uint32_t T) { return (size_t)T * 30; }

__device__ __forceinline__ U128 neg128(U128 x) {
  U128 r;
  r.lo = ~x.lo + 1;
  r.hi = ~x.hi + (x.lo == 0 ? 1 : 0);
  return r;
}

// x as a two's-complement multiple of 2^-64, if it is one and |x| < 2^48.
__device__ __forceinline__ bool fixed_exact(double x, U128 &out) {
  const uint64_t b = dbits(x);
  const uint64_t ab = b & 0x7fffffffffffffffull;
  out = U128{0, 0};
  if (ab == 0) return true;
  const int e = (int)(ab >> 52);
  if (e == 0 || e >= 1023 + 48) return false;
  const uint64_t mant = (ab & lowmask(52)) | (1ull << 52);
  const int sh = e - 1075 + 64;            // |x| = mant * 2^(sh - 64), sh <= 59
  U128 m;
  if (sh >= 0) {
    m.lo = mant << sh;
    m.hi = sh > 11 ? (mant >> (64 - sh)) : 0;
  } else {
    if (-sh >= 53 || (mant & lowmask(-sh))) return false;
    m.lo = mant >> (-sh);
    m.hi = 0;
  }
  out = (b >> 63) ? neg128(m) : m;
  return true;
}

__device__ __forceinline__ double signed_fixed_to_double(U128 x) {
  if (x.hi >> 63) return bitsd(dbits(fixed_to_double(neg128(x))) ^ 0x8000000000000000ull);
  return fixed_to_double(x);
}

__device__ __forceinline__ double from_ordered(uint64_t o) {
  return bitsd((o >> 63) ? (o & 0x7fffffffffffffffull) : ~o);
}

// Canonical-order sum for an address with an inexact contribution: `first` (the diagonal
// term, when `have`) followed by the spawns on `key` in increasing order of value.
__device__ double canonical_sum_scan(bool have, double first, uint64_t key, const Rec *sp,
                                     uint32_t ns, bool *bad) {
  double sum = first;
  constexpr int K = 8;
  uint64_t ob[K];
  int n = 0;
  bool more = false;
  for (uint32_t j = 0; j < ns; ++j) {
    if (sp[j].key != key) continue;
    if (n < K) ob[n++] = ordered_bits(bitsd(sp[j].val));
    else { more = true; break; }
  }
  if (!more) {
    for (int i = 1; i < n; ++i) {
      const uint64_t v = ob[i];
      int k = i - 1;
      while (k >= 0 && ob[k] > v) { ob[k + 1] = ob[k]; --k; }
      ob[k + 1] = v;
    }
    for (int i = 0; i < n; ++i) {
      const double v = from_ordered(ob[i]);
      sum = have ? sum + v : v;
      have = true;
    }
    return sum;
  }
  uint64_t last = 0;
  bool any_last = false;
  for (uint32_t round = 0; round <= ns; ++round) {
    uint64_t best = ~0ull;
    uint32_t cnt = 0;
    for (uint32_t j = 0; j < ns; ++j) {
      if (sp[j].key != key) continue;
      const uint64_t o = ordered_bits(bitsd(sp[j].val));
      if (any_last && o <= last) continue;
      if (o < best) { best = o; cnt = 1; } else if (o == best) ++cnt;
    }
    if (cnt == 0) return sum;
    const double v = from_ordered(best);
    for (uint32_t c = 0; c < cnt; ++c) { sum = have ? sum + v : v; have = true; }
    last = best;
    any_last = true;
  }
  *bad = true;
  return sum;
}

// Diagonal step of one walker (diagonal_step!, spawning.jl:73-77), float walkers.
template <int KIND>
__device__ __forceinline__ double diag_float(const StepArgs &a, int r, uint32_t rep,
                                             const Rec &rec) {
  double res = op_diagonal<KIND>(a, r, rec.key) * bitsd(rec.val);
  if (a.has_proj) {
    const U4 rr = draw(a.seed, PURPOSE_DIAG, rep, a.step, rec.key, 0);
    res = project_threshold(res, a.proj_threshold, u53_of(rr));
  }
  return res;
}

// Slot of `key` in the table, claimed if the key is new; -1 if the table is full.
__device__ __forceinline__ int table_insert(uint64_t *tkey, uint32_t T, uint64_t key,
                                            uint64_t hsh, bool &claimed) {
  uint32_t sl = (uint32_t)hsh & (T - 1);
  claimed = false;
  for (uint32_t p = 0; p < T; ++p) {
    const uint64_t k = *(volatile uint64_t *)&tkey[sl];
    if (k == key) return (int)sl;
    if (k == EMPTY_KEY) {
      const unsigned long long old = atomicCAS((unsigned long long *)&tkey[sl],
                                               (unsigned long long)EMPTY_KEY,
                                               (unsigned long long)key);
      if (old == EMPTY_KEY) { claimed = true; return (int)sl; }
      if (old == key) return (int)sl;
    }
    sl = (sl + 1) & (T - 1);
  }
  return -1;
}

// Final value of one address: threshold compression (compression.jl:18-42), statistics, the
// ProjectedEnergy dot products.  Returns whether the address is kept and its value bits.
template <int STYLE>
__device__ __forceinline__ bool finalize_entry(const StepArgs &a, int r, uint64_t key, double fv,
                                               int64_t iv, uint64_t &vb, AnnAcc &acc) {
  double dv;
  if (STYLE == STYLE_INTEGER) {
    if (iv == 0) return false;
    acc.len_before++;
    vb = (uint64_t)iv;
    const uint64_t mag = (uint64_t)(iv < 0 ? -iv : iv);
    acc.norm = add128(acc.norm, U128{0, mag});
    acc.len++;
    if (a.nproj == 0) return true;
    dv = i2d_exact(iv);
  } else {
    if (is_zero_d(fv)) return false;
    acc.len_before++;
    if (a.comp_mode != 0) {
      bool small;
      double prob;
      if (a.comp_mode == 1) { small = abs_lt_one(fv); prob = abs_d(fv); }
      else { prob = abs_d(fv) / a.compression; small = prob < 1; }
      if (small) {
        U4 rr = draw(a.seed, PURPOSE_COMPRESS, a.replica_base + (uint32_t)r, a.step, key, 0);
        if (!bernoulli53(u53_of(rr), prob)) return false;
        fv = signed_like(a.compression, fv);
      }
    }
    vb = dbits(fv);
    acc.norm = add128(acc.norm, fixed_of(abs_d(fv)));
    acc.len++;
    if (a.nproj == 0) return true;
    dv = fv;
  }
  const uint64_t *pk = a.proj_keys + (size_t)r * a.nproj;
  int lo = 0, hi = a.nproj - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    if (pk[mid] == key) {
      const size_t o = (size_t)r * a.nproj + mid;
      a.proj_out_v[o] = a.proj_v[o] * dv;
      a.proj_out_h[o] = a.proj_h[o] * dv;
      break;
    }
    if (pk[mid] < key) lo = mid + 1; else hi = mid - 1;
  }
  return true;
}

// Warp-synchronous append of the kept entries to the target slab of bucket gb.
__device__ __forceinline__ void warp_emit(const StepArgs &a, int gb, bool keep, uint64_t key,
                                          uint64_t vb, uint32_t &out) {
  const uint32_t m = __ballot_sync(0xffffffffu, keep);
  const uint32_t pos = out + __popc(m & lanemask_lt());
  if (keep && pos < a.capv) a.v_out[(size_t)gb * a.capv + pos] = Rec{key, vb};
  out += __popc(m);
}

__device__ __forceinline__ void flush_ann_acc(const StepArgs &a, int r, AnnAcc &acc) {
  const U128 nfx = warp_sum128(acc.norm), sfx = warp_sum128(acc.spawn_fx);
  const long long l = warp_sum(acc.len), lb = warp_sum(acc.len_before);
  const long long cl = warp_sum(acc.clones), de = warp_sum(acc.deaths), zo = warp_sum(acc.zombies);
  const long long si = warp_sum(acc.spawns_i), rc = warp_sum(acc.records);
  if ((threadIdx.x & 31) == 0) {
    DevStats &st = a.stats[r];
    atomic_add128(&st.norm_lo, &st.norm_hi, nfx);
    atomic_add128(&st.spawn_lo, &st.spawn_hi, sfx);
    atomic_add_ll(&st.len, l);
    atomic_add_ll(&st.len_before, lb);
    atomic_add_ll(&st.clones, cl);
    atomic_add_ll(&st.deaths, de);
    atomic_add_ll(&st.zombies, zo);
    atomic_add_ll(&st.spawns_int, si);
    atomic_add_ll(&st.spawn_records, rc);
  }
  acc = AnnAcc{};
}

// One warp per bucket.  The bucket's addresses go into a T-slot table: first the source
// walkers after their diagonal step, then the spawns, each contribution added exactly into
// the address's 128-bit fixed-point sum by shared-memory atomics.  The occupied slots are
// then finalized (rounding, compression, statistics) and appended to the target slab.  A
// bucket with more addresses than the table holds is processed in passes, each taking the
// addresses whose hash bits 16.. select it; a pass that still overflows is split in two.
template <int KIND, int STYLE>
__global__ void __launch_bounds__(WARPS * 32, 3) k_annihilate(StepArgs a, int nb_total) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t T = a.tsize;
  unsigned char *mine = smem + (size_t)w * ann_warp_smem(T);
  uint64_t *tkey = reinterpret_cast<uint64_t *>(mine);
  unsigned long long *tlo = reinterpret_cast<unsigned long long *>(tkey + T);
  unsigned long long *thi = tlo + T;
  uint32_t *tinfo = reinterpret_cast<uint32_t *>(thi + T);
  uint16_t *slist = reinterpret_cast<uint16_t *>(tinfo + T);
  const uint32_t lim = T - 32;      // a round of 32 insertions starts only below this fill
  AnnAcc acc{};
  int cur_r = -1;
  bool bad = false;
  for (int gb = blockIdx.x * WARPS + w; gb < nb_total; gb += gridDim.x * WARPS) {
    const int r = gb >> a.nb_bits;
    if (r != cur_r) {
      if (cur_r >= 0) flush_ann_acc(a, cur_r, acc);
      cur_r = r;
    }
    const uint32_t rep = a.replica_base + (uint32_t)r;
    const uint32_t nsp = a.scount[gb];
    const uint32_t ns = nsp < a.caps ? nsp : a.caps;
    const uint32_t nv0 = a.cnt_in[gb];
    const uint32_t nv = nv0 < a.capv_in ? nv0 : a.capv_in;
    const Rec *sp = a.spawn + (size_t)gb * a.caps;
    const Rec *vbase = a.v_in + (size_t)gb * a.capv_in;
    const uint32_t need = nv + ns;   // upper bound on the bucket's distinct addresses
    int lvl0 = 0;
    if (need > lim) {
      lvl0 = 1;
      while (lvl0 < MAX_SPLIT && need > ((lim * 3 / 4) << lvl0)) ++lvl0;
    }
    int lvl = lvl0;
    uint32_t sel = 0;
    uint32_t out = 0;
    for (;;) {
      const uint32_t mask = (1u << lvl) - 1u;
      for (uint32_t i = lane; i < T; i += 32) {
        tkey[i] = EMPTY_KEY; tlo[i] = 0; thi[i] = 0; tinfo[i] = 0;
      }
      __syncwarp();
      uint32_t nslots = 0;
      bool fail = false;
      PassAcc pa{};
      // source walkers: diagonal step; their keys are distinct, each claims its own slot
      for (uint32_t e0 = 0; e0 < nv; e0 += 32) {
        if (nslots > lim) { fail = true; break; }
        const uint32_t e = e0 + lane;
        bool claimed = false, lfail = false;
        int slot = -1;
        if (e < nv) {
          const Rec rec = vbase[e];
          const uint64_t hsh = mix64(rec.key);
          if (((uint32_t)(hsh >> 16) & mask) == sel) {
            slot = table_insert(tkey, T, rec.key, hsh, claimed);
            if (slot < 0) lfail = true;
            else if (!claimed) bad = true;          // an address listed twice in the source
            else if (STYLE == STYLE_INTEGER) {
              const int64_t v = (int64_t)rec.val;
              const double x = op_diagonal<KIND>(a, r, rec.key) * i2d_exact(v);
              const U4 rr = draw(a.seed, PURPOSE_DIAG, rep, a.step, rec.key, 0);
              const int64_t res = round_stochastic(x, u53_of(rr));
              // clones_deaths_zombies (spawning.jl:79-93)
              const int sr = (res > 0) - (res < 0), sv = (v > 0) - (v < 0);
              if (res > v) pa.clones += res - v;
              else if (sr != sv) { pa.deaths += v < 0 ? -v : v; pa.zombies += res < 0 ? -res : res; }
              else pa.deaths += (res - v) < 0 ? v - res : res - v;
              tlo[slot] = (unsigned long long)res;
            } else {
              const double res = diag_float<KIND>(a, r, rep, rec);
              U128 fx;
              uint32_t info = (e + 1) << 1;
              if (fixed_exact(res, fx)) { tlo[slot] = fx.lo; thi[slot] = fx.hi; }
              else info |= INFO_INEXACT;
              tinfo[slot] = info;
            }
          }
        }
        const uint32_t m = __ballot_sync(0xffffffffu, claimed);
        if (claimed) slist[nslots + __popc(m & lanemask_lt())] = (uint16_t)slot;
        nslots += __popc(m);
        if (__any_sync(0xffffffffu, lfail)) { fail = true; break; }
      }
      __syncwarp();
      // spawns: find or claim the slot, add the value
      if (!fail) {
        for (uint32_t j0 = 0; j0 < ns; j0 += 32) {
          if (nslots > lim) { fail = true; break; }
          const uint32_t j = j0 + lane;
          bool claimed = false, lfail = false;
          int slot = -1;
          if (j < ns) {
            const Rec s = sp[j];
            const uint64_t hsh = mix64(s.key);
            if (((uint32_t)(hsh >> 16) & mask) == sel) {
              slot = table_insert(tkey, T, s.key, hsh, claimed);
              if (slot < 0) {
                lfail = true;
              } else {
                pa.records++;
                if (STYLE == STYLE_INTEGER) {
                  const int64_t k = (int64_t)s.val;
                  pa.spawns_i += k < 0 ? -k : k;
                  atomicAdd(&tlo[slot], (unsigned long long)k);
                } else {
                  const double y = bitsd(s.val);
                  pa.spawn_fx = add128(pa.spawn_fx, fixed_of(abs_d(y)));
                  U128 fx;
                  if (fixed_exact(y, fx)) {
                    const unsigned long long old = atomicAdd(&tlo[slot], fx.lo);
                    const unsigned long long hadd = fx.hi + ((old + fx.lo < old) ? 1ull : 0ull);
                    if (hadd) atomicAdd(&thi[slot], hadd);
                  } else {
                    atomicOr(&tinfo[slot], INFO_INEXACT);
                  }
                }
              }
            }
          }
          const uint32_t m = __ballot_sync(0xffffffffu, claimed);
          if (claimed) slist[nslots + __popc(m & lanemask_lt())] = (uint16_t)slot;
          nslots += __popc(m);
          if (__any_sync(0xffffffffu, lfail)) { fail = true; break; }
        }
      }
      __syncwarp();
      if (fail) {
        if (lvl >= MAX_SPLIT) { bad = true; break; }
        ++lvl;                       // first half of this pass: hash bit lvl-1 clear
        continue;
      }
      // finalize the pass's addresses
      for (uint32_t i0 = 0; i0 < nslots; i0 += 32) {
        const uint32_t i = i0 + lane;
        bool keep = false;
        uint64_t key = 0, vb = 0;
        if (i < nslots) {
          const int slot = slist[i];
          key = tkey[slot];
          if (STYLE == STYLE_INTEGER) {
            keep = finalize_entry<STYLE>(a, r, key, 0.0, (int64_t)tlo[slot], vb, acc);
          } else {
            const uint32_t info = tinfo[slot];
            double fv;
            if (info & INFO_INEXACT) {
              bool have = false;
              double first = 0.0;
              const uint32_t src = info >> 1;
              if (src) {
                first = diag_float<KIND>(a, r, rep, vbase[src - 1]);
                have = !is_zero_d(first);
              }
              fv = canonical_sum_scan(have, first, key, sp, ns, &bad);
            } else {
              fv = signed_fixed_to_double(U128{tlo[slot], thi[slot]});
            }
            keep = finalize_entry<STYLE>(a, r, key, fv, 0, vb, acc);
          }
        }
        warp_emit(a, gb, keep, key, vb, out);
      }
      acc.spawn_fx = add128(acc.spawn_fx, pa.spawn_fx);
      acc.clones += pa.clones; acc.deaths += pa.deaths; acc.zombies += pa.zombies;
      acc.spawns_i += pa.spawns_i; acc.records += pa.records;
      __syncwarp();
      // next pass: depth first over the splits
      while (lvl > lvl0 && ((sel >> (lvl - 1)) & 1u)) { sel &= ~(1u << (lvl - 1)); --lvl; }
      if (lvl == lvl0) {
        if (++sel >= (1u << lvl0)) break;
      } else {
        sel |= 1u << (lvl - 1);
      }
    }
    if (lane == 0) {
      a.cnt_out[gb] = out < a.capv ? out : a.capv;
      if (out > a.capv) atomicOr(&a.stats[r].flags, (unsigned)FLAG_V_OVERFLOW);
      if (nsp > a.caps) atomicOr(&a.stats[r].flags, (unsigned)FLAG_SPAWN_OVERFLOW);
      atomicMax(&a.stats[r].max_v_bucket, out);
      atomicMax(&a.stats[r].max_spawn_bucket, nsp);
      a.scount[gb] = 0;
    }
    __syncwarp();
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0)
    atomicOr(&a.stats[cur_r < 0 ? 0 : cur_r].flags, (unsigned)FLAG_TABLE);
  if (cur_r >= 0) flush_ann_acc(a, cur_r, acc);
}

// ------------------------------------------------------------------------------------------
// Auxiliary kernels
// ------------------------------------------------------------------------------------------
__global__ void k_diag_table(DevModel h, int op, double dt, const double *shift, int nrep,
                             int ndiag, double *dtab) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrep * ndiag) return;
  int r = i / ndiag, I = i % ndiag;
  double d = h.u * (double)I / 2;
  dtab[i] = op == OP_TRANSITION ? 1 - dt * (d - shift[r]) : d;
}

__global__ void k_bucketize(const uint64_t *keys, const uint64_t *vals, int64_t n, int nb_bits,
                            uint32_t capv, Rec *recs, uint32_t *count, unsigned int *flag) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t k = keys[i];
  uint32_t b = bucket_of(k, nb_bits);
  uint32_t pos = atomicAdd(&count[b], 1u);
  if (pos < capv) recs[(size_t)b * capv + pos] = Rec{k, vals[i]};
  else atomicOr(flag, (unsigned)FLAG_V_OVERFLOW);
}

__global__ void k_rebucket(const Rec *old_recs, const uint32_t *old_count, int old_nb,
                           uint32_t old_capv, Rec *recs, uint32_t *count, int nb_bits,
                           uint32_t capv, unsigned int *flag) {
  for (int gb = blockIdx.x; gb < old_nb; gb += gridDim.x) {
    uint32_t n = old_count[gb];
    for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
      Rec rec = old_recs[(size_t)gb * old_capv + e];
      uint32_t b = bucket_of(rec.key, nb_bits);
      uint32_t pos = atomicAdd(&count[b], 1u);
      if (pos < capv) recs[(size_t)b * capv + pos] = rec;
      else atomicOr(flag, (unsigned)FLAG_V_OVERFLOW);
    }
  }
}

__global__ void k_compact(const Rec *recs, const uint32_t *count, int nb, uint32_t capv,
                          const uint64_t *offsets, uint64_t *keys, uint64_t *vals) {
  for (int gb = blockIdx.x; gb < nb; gb += gridDim.x) {
    uint32_t n = count[gb];
    uint64_t o = offsets[gb];
    for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
      Rec rec = recs[(size_t)gb * capv + e];
      keys[o + e] = rec.key;
      vals[o + e] = rec.val;
    }
  }
}

__global__ void k_norm(const Rec *recs, const uint32_t *count, int nb, uint32_t capv,
                       int val_kind, unsigned long long *acc3) {
  U128 fx{0, 0};
  long long len = 0;
  for (int gb = blockIdx.x; gb < nb; gb += gridDim.x) {
    uint32_t n = count[gb];
    for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
      Rec rec = recs[(size_t)gb * capv + e];
      double v = val_kind == RIMU_VAL_I64 ? (double)(int64_t)rec.val : bitsd(rec.val);
      fx = add128(fx, fixed_of(fabs(v)));
      len++;
    }
  }
  fx = warp_sum128(fx);
  len = warp_sum(len);
  if ((threadIdx.x & 31) == 0) {
    atomic_add128(&acc3[0], &acc3[1], fx);
    if (len) atomicAdd(&acc3[2], (unsigned long long)len);
  }
}

__global__ void k_lookup(const Rec *recs, const uint32_t *count, int nb_bits, uint32_t capv,
                         const uint64_t *keys, int64_t n, uint64_t *vals, int *found) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t k = keys[i];
  uint32_t b = bucket_of(k, nb_bits);
  uint32_t c = count[b];
  const Rec *base = recs + (size_t)b * capv;
  vals[i] = 0;
  found[i] = 0;
  for (uint32_t e = 0; e < c; ++e) {
    if (base[e].key == k) { vals[i] = base[e].val; found[i] = 1; break; }
  }
}

template <int KIND>
__global__ void k_diagonal(DevModel h, const uint64_t *keys, int64_t n, double *out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = model_diagonal<KIND>(h, keys[i]);
}

template <int KIND>
__global__ void k_offdiagonals(DevModel h, uint64_t key, int noff, uint64_t *keys, double *vals) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= noff) return;
  Offdiag od = column_offdiag<KIND>(h, key, c + 1);
  keys[c] = od.key;
  double v = od.prod == 0 ? 0.0 : h.hoff[od.prod];
  vals[c] = od.sign < 0 ? -v : v;
}

// ------------------------------------------------------------------------------------------
// Launchers
// ------------------------------------------------------------------------------------------
template <int KIND, int STYLE>
static int launch_step_t(rimu_ctx *ctx, const StepArgs &a, int nb_total, cudaEvent_t *ev) {
  cudaStream_t st = ctx->stream;
  const int cap = ctx->num_sms * 64;
  const int cb = a.nb_bits < 5 ? (1 << a.nb_bits) : CHUNK_BUCKETS;
  const int want_s = (nb_total / cb + WARPS - 1) / WARPS;
  const int grid_s = want_s < cap ? want_s : cap;
  const int want = (nb_total + WARPS - 1) / WARPS;
  const int grid = want < cap ? want : cap;
  if (ev) cudaEventRecord(ev[0], st);
  k_spawn<KIND, STYLE><<<grid_s, WARPS * 32, 0, st>>>(a, nb_total);
  if (ev) cudaEventRecord(ev[1], st);
  k_spawn_heavy<KIND, STYLE><<<ctx->num_sms * 4, 256, 0, st>>>(a);
  if (ev) cudaEventRecord(ev[2], st);
  const size_t smem = WARPS * ann_warp_smem(a.tsize);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_annihilate<KIND, STYLE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         200 * 1024);
    attr_set = true;
  }
  k_annihilate<KIND, STYLE><<<grid, WARPS * 32, smem, st>>>(a, nb_total);
  if (ev) cudaEventRecord(ev[3], st);
  return rimu_cuda_check(cudaGetLastError(), "step kernels");
}

template <int KIND>
static int launch_step_k(rimu_ctx *ctx, const StepArgs &a, int nb_total, cudaEvent_t *ev) {
  switch (a.style) {
    case STYLE_INTEGER: return launch_step_t<KIND, STYLE_INTEGER>(ctx, a, nb_total, ev);
    case STYLE_DETERMINISTIC: return launch_step_t<KIND, STYLE_DETERMINISTIC>(ctx, a, nb_total, ev);
    default: return launch_step_t<KIND, STYLE_DSS>(ctx, a, nb_total, ev);
  }
}

}  // namespace rimu

using namespace rimu;

int rimu_launch_step(rimu_ctx *ctx, const StepArgs &a, int nb_total, cudaEvent_t *ev) {
  switch (a.h.kind) {
    case MODEL_REAL1D: return launch_step_k<MODEL_REAL1D>(ctx, a, nb_total, ev);
    case MODEL_REALSPACE: return launch_step_k<MODEL_REALSPACE>(ctx, a, nb_total, ev);
    default: return launch_step_k<MODEL_MOM1D>(ctx, a, nb_total, ev);
  }
}

int rimu_launch_bucketize(rimu_ctx *ctx, const uint64_t *keys, const uint64_t *vals, int64_t n,
                          int nb_bits, uint32_t capv, Rec *recs, uint32_t *count,
                          unsigned int *flag) {
  if (n == 0) return 0;
  int64_t blocks = (n + 255) / 256;
  k_bucketize<<<(unsigned)blocks, 256, 0, ctx->stream>>>(keys, vals, n, nb_bits, capv, recs,
                                                         count, flag);
  return rimu_cuda_check(cudaGetLastError(), "k_bucketize");
}

int rimu_launch_rebucket(rimu_ctx *ctx, const Rec *old_recs, const uint32_t *old_count,
                         int old_nb_bits, uint32_t old_capv, Rec *recs, uint32_t *count,
                         int nb_bits, uint32_t capv, unsigned int *flag) {
  int old_nb = 1 << old_nb_bits;
  int grid = old_nb < 65536 ? old_nb : 65536;
  k_rebucket<<<grid, 256, 0, ctx->stream>>>(old_recs, old_count, old_nb, old_capv, recs, count,
                                            nb_bits, capv, flag);
  return rimu_cuda_check(cudaGetLastError(), "k_rebucket");
}

int rimu_launch_compact(rimu_ctx *ctx, const Rec *recs, const uint32_t *count, int nb,
                        uint32_t capv, const uint64_t *offsets, uint64_t *keys, uint64_t *vals) {
  int grid = nb < 65536 ? nb : 65536;
  k_compact<<<grid, 256, 0, ctx->stream>>>(recs, count, nb, capv, offsets, keys, vals);
  return rimu_cuda_check(cudaGetLastError(), "k_compact");
}

int rimu_launch_norm(rimu_ctx *ctx, const Rec *recs, const uint32_t *count, int nb,
                     uint32_t capv, int val_kind, unsigned long long *acc3) {
  int grid = nb < ctx->num_sms * 8 ? nb : ctx->num_sms * 8;
  k_norm<<<grid, 256, 0, ctx->stream>>>(recs, count, nb, capv, val_kind, acc3);
  return rimu_cuda_check(cudaGetLastError(), "k_norm");
}

int rimu_launch_lookup(rimu_ctx *ctx, const Rec *recs, const uint32_t *count, int nb_bits,
                       uint32_t capv, const uint64_t *keys, int64_t n, uint64_t *vals,
                       int *found) {
  if (n == 0) return 0;
  k_lookup<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(recs, count, nb_bits, capv,
                                                                 keys, n, vals, found);
  return rimu_cuda_check(cudaGetLastError(), "k_lookup");
}

int rimu_launch_diag_table(rimu_ctx *ctx, const DevModel &h, int op, double dt,
                           const double *shift, int nrep, int ndiag, double *dtab) {
  int n = nrep * ndiag;
  k_diag_table<<<(n + 255) / 256, 256, 0, ctx->stream>>>(h, op, dt, shift, nrep, ndiag, dtab);
  return rimu_cuda_check(cudaGetLastError(), "k_diag_table");
}

int rimu_launch_diagonal(rimu_ctx *ctx, const DevModel &h, const uint64_t *keys, int64_t n,
                         double *out) {
  if (n == 0) return 0;
  unsigned g = (unsigned)((n + 255) / 256);
  switch (h.kind) {
    case MODEL_REAL1D: k_diagonal<MODEL_REAL1D><<<g, 256, 0, ctx->stream>>>(h, keys, n, out); break;
    case MODEL_REALSPACE: k_diagonal<MODEL_REALSPACE><<<g, 256, 0, ctx->stream>>>(h, keys, n, out); break;
    default: k_diagonal<MODEL_MOM1D><<<g, 256, 0, ctx->stream>>>(h, keys, n, out); break;
  }
  return rimu_cuda_check(cudaGetLastError(), "k_diagonal");
}

int rimu_launch_offdiagonals(rimu_ctx *ctx, const DevModel &h, uint64_t key, int noff,
                             uint64_t *keys, double *vals) {
  if (noff == 0) return 0;
  unsigned g = (unsigned)((noff + 127) / 128);
  switch (h.kind) {
    case MODEL_REAL1D: k_offdiagonals<MODEL_REAL1D><<<g, 128, 0, ctx->stream>>>(h, key, noff, keys, vals); break;
    case MODEL_REALSPACE: k_offdiagonals<MODEL_REALSPACE><<<g, 128, 0, ctx->stream>>>(h, key, noff, keys, vals); break;
    default: k_offdiagonals<MODEL_MOM1D><<<g, 128, 0, ctx->stream>>>(h, key, noff, keys, vals); break;
  }
  return rimu_cuda_check(cudaGetLastError(), "k_offdiagonals");
}
