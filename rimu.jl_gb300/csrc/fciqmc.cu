// fciqmc.cu -- kernels of one FCIQMC projector step on a bucketed, device-resident walker list.
//
// Layout in HBM.  A walker list is 2^nb_bits buckets per replica; bucket b holds the walkers
// whose address hashes (top nb_bits of mix64) to b, as 16-byte (address, amplitude) records
// in a fixed-capacity slab [b * capv, b * capv + count[b]).  The spawn buffer uses the same
// buckets with slabs of capacity caps.
//
// One step (apply_operator!, src/Interfaces/dictvectors.jl:112-140):
//   k_spawn      reads the source slabs and writes every spawn straight into the slab of
//                its destination bucket (perform_spawns!, pdworkingmemory.jl:208-217).
//                Columns are balanced across the CTA by a block scan over their work;
//                columns with more than HEAVY_LIMIT attempts are cut into chunks.
//   k_spawn_heavy  processes the chunks of heavy columns on all SMs.
//   k_annihilate one CTA per bucket: spawns go into a shared-memory hash table, each source
//                walker takes its diagonal step and collects the spawns on its address, new
//                addresses are emitted, contributions summed in canonical order (diagonal
//                first, spawns by increasing value), threshold compression applied, and the
//                norm accumulated exactly (collect_local!/move_and_compress!,
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
struct Acc {
  U128 fx;                 // fixed-point sum (spawn magnitudes or norm)
  long long a0, a1, a2, a3, a4, a5;
};

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

// ------------------------------------------------------------------------------------------
// Spawning: one warp per bucket, no block barriers
// ------------------------------------------------------------------------------------------
struct SpawnAcc {
  U128 fx;           // sum |spawn| for float styles
  long long spawns_i;
  long long records;
  long long attempts, exact_n, inexact_n;
};

constexpr int WARPS = 8;           // warps per CTA in the step kernels
constexpr int G = 4;               // units (attempts or offdiagonals) per work item

__device__ __forceinline__ void emit_spawn(const StepArgs &a, int r, uint64_t nk, uint64_t vb,
                                           SpawnAcc &acc) {
  uint32_t b = ((uint32_t)r << a.nb_bits) | bucket_of(nk, a.nb_bits);
  uint32_t pos = atomicAdd(&a.scount[b], 1u);
  if (pos < a.caps) {
    a.spawn[(size_t)b * a.caps + pos] = Rec{nk, vb};
  } else {
    atomicOr(&a.stats[r].flags, (unsigned)FLAG_SPAWN_OVERFLOW);
  }
  acc.records++;
}

template <int KIND>
__device__ __forceinline__ Offdiag step_offdiag(const DevModel &h, uint64_t key, int chosen) {
  if (KIND == MODEL_REAL1D) return real1d_offdiag_fast(key, h.nbits, chosen);
  return column_offdiag<KIND>(h, key, chosen);
}

// Units [j0, j1) of one column.  Exact columns deposit val * T_{new,key} for offdiagonals
// j+1 (spawning.jl:174-182); sampled columns draw a uniform offdiagonal per attempt and
// deposit c * T_{new,key} (spawning.jl:232-243).  With float walkers and no on-the-fly
// projection an attempt needs 32 random bits, so one Philox block serves four attempts.
template <int KIND, int STYLE>
__device__ __forceinline__ void spawn_units(const StepArgs &a, int r, uint64_t key, uint64_t vb,
                                            double c, int noff, int exact, uint32_t j0,
                                            uint32_t j1, SpawnAcc &acc) {
  const uint32_t rep = a.replica_base + (uint32_t)r;
  if (exact) {
    const double val = bitsd(vb);
    for (uint32_t j = j0; j < j1; ++j) {
      Offdiag od = step_offdiag<KIND>(a.h, key, (int)j + 1);
      if (od.prod == 0) continue;
      double y = val * op_offdiag(a, od);
      if (STYLE == STYLE_DSS && a.has_proj) {
        U4 rr = draw(a.seed, PURPOSE_SPAWN, rep, a.step, key, j);
        y = project_threshold(y, a.proj_threshold, u53_of(rr));
      }
      if (is_zero_d(y)) continue;
      acc.fx = add128(acc.fx, fixed_of(abs_d(y)));
      emit_spawn(a, r, od.key, dbits(y), acc);
    }
    return;
  }
  const bool grouped = STYLE != STYLE_INTEGER && !a.has_proj;
  U4 blk{0, 0, 0, 0};
  uint32_t blk_id = 0xffffffffu;
  for (uint32_t j = j0; j < j1; ++j) {
    uint32_t word;
    U4 rr;
    if (grouped) {
      if ((j >> 2) != blk_id) { blk_id = j >> 2; blk = draw(a.seed, PURPOSE_SPAWN, rep, a.step, key, blk_id); }
      const uint32_t q = j & 3;
      word = q == 0 ? blk.x : q == 1 ? blk.y : q == 2 ? blk.z : blk.w;
      rr = blk;
    } else {
      rr = draw(a.seed, PURPOSE_SPAWN, rep, a.step, key, j);
      word = rr.x;
    }
    const int chosen = (int)uniform_index(word, (uint32_t)noff) + 1;
    Offdiag od = step_offdiag<KIND>(a.h, key, chosen);
    if (od.prod == 0) continue;
    double y = c * op_offdiag(a, od);
    if (STYLE == STYLE_INTEGER) {
      int64_t k = round_stochastic(y, u53_of(rr));
      if (k == 0) continue;
      acc.spawns_i += k < 0 ? -k : k;
      emit_spawn(a, r, od.key, (uint64_t)k, acc);
    } else {
      if (a.has_proj) y = project_threshold(y, a.proj_threshold, u53_of(rr));
      if (is_zero_d(y)) continue;
      acc.fx = add128(acc.fx, fixed_of(abs_d(y)));
      emit_spawn(a, r, od.key, dbits(y), acc);
    }
  }
}

__device__ __forceinline__ void flush_spawn_acc(const StepArgs &a, int r, SpawnAcc &acc) {
  U128 fx = warp_sum128(acc.fx);
  long long s = warp_sum(acc.spawns_i), rc = warp_sum(acc.records), at = warp_sum(acc.attempts);
  long long ex = warp_sum(acc.exact_n), ie = warp_sum(acc.inexact_n);
  if ((threadIdx.x & 31) == 0) {
    DevStats &st = a.stats[r];
    atomic_add128(&st.spawn_lo, &st.spawn_hi, fx);
    atomic_add_ll(&st.spawns_int, s);
    atomic_add_ll(&st.spawn_records, rc);
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

template <int KIND, int STYLE>
__global__ void __launch_bounds__(WARPS * 32) k_spawn(StepArgs a, int nb_total) {
  __shared__ uint64_t s_key[WARPS][32];
  __shared__ uint64_t s_val[WARPS][32];
  __shared__ double s_c[WARPS][32];
  __shared__ uint32_t s_units[WARPS][32];
  __shared__ uint32_t s_excl[WARPS][32];
  __shared__ int s_noff[WARPS][32];
  __shared__ int s_exact[WARPS][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  SpawnAcc acc{};
  int cur_r = -1;
  for (int gb = blockIdx.x * WARPS + w; gb < nb_total; gb += gridDim.x * WARPS) {
    const int r = gb >> a.nb_bits;
    if (r != cur_r) {
      if (cur_r >= 0) flush_spawn_acc(a, cur_r, acc);
      cur_r = r;
    }
    const uint32_t n0 = a.cnt_in[gb];
    const uint32_t n = n0 < a.capv_in ? n0 : a.capv_in;
    const Rec *base = a.v_in + (size_t)gb * a.capv_in;
    for (uint32_t c0 = 0; c0 < n; c0 += 32) {
      const uint32_t e = c0 + lane;
      uint32_t items = 0;
      if (e < n) {
        const Rec rec = base[e];
        int noff, exact;
        double c;
        uint64_t work = column_work<KIND, STYLE>(a, rec.key, rec.val, noff, exact, c, acc);
        if (work > (1ull << 36)) {       // more attempts than any walker list can hold
          atomicOr(&a.stats[r].flags, (unsigned)FLAG_VALUE_OVERFLOW);
          work = 0;
        }
        acc.attempts += (long long)work;
        if (work > (uint64_t)HEAVY_LIMIT) {
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
          work = 0;
        }
        s_key[w][lane] = rec.key; s_val[w][lane] = rec.val; s_c[w][lane] = c;
        s_noff[w][lane] = noff; s_exact[w][lane] = exact;
        s_units[w][lane] = (uint32_t)work;
        items = ((uint32_t)work + G - 1) / G;
      }
      // warp exclusive scan of the work items
      uint32_t incl = items;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
      s_excl[w][lane] = incl - items;
      __syncwarp();
      for (uint32_t it = lane; it < total; it += 32) {
        int lo = 0;
#pragma unroll
        for (int step = 16; step >= 1; step >>= 1)
          if (s_excl[w][lo + step] <= it) lo += step;
        const uint32_t j0 = (it - s_excl[w][lo]) * G;
        const uint32_t ju = s_units[w][lo];
        const uint32_t j1 = j0 + G < ju ? j0 + G : ju;
        spawn_units<KIND, STYLE>(a, r, s_key[w][lo], s_val[w][lo], s_c[w][lo], s_noff[w][lo],
                                 s_exact[w][lo], j0, j1, acc);
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
  SpawnAcc acc{};
  for (uint32_t ci = blockIdx.x; ci < nch; ci += gridDim.x) {
    HeavyChunk ch = a.heavy[ci];
    if (ch.cnt > (uint32_t)HEAVY_CHUNK || ch.rep >= (uint32_t)a.nrep) {
      if (threadIdx.x == 0) atomicOr(&a.stats[0].flags, (unsigned)FLAG_TABLE);
      ch.cnt = 0;
      ch.rep = 0;
    }
    for (uint32_t t = threadIdx.x * G; t < ch.cnt; t += blockDim.x * G) {
      const uint32_t j1 = t + G < ch.cnt ? t + G : ch.cnt;
      spawn_units<KIND, STYLE>(a, (int)ch.rep, ch.key, ch.val, ch.c, ch.noff, ch.exact,
                               ch.j0 + t, ch.j0 + j1, acc);
    }
    // attempts were counted when the chunk was created
    acc.attempts = 0;
    flush_spawn_acc(a, (int)ch.rep, acc);
  }
}

// ------------------------------------------------------------------------------------------
// Annihilation: one warp per bucket
// ------------------------------------------------------------------------------------------
struct AnnAcc {
  U128 norm;
  long long len, len_before, clones, deaths, zombies;
};

__device__ __forceinline__ double from_ordered(uint64_t o) {
  return bitsd((o >> 63) ? (o & 0x7fffffffffffffffull) : ~o);
}

// Sum of the spawn list starting at `head` in increasing order of value, after `first`.
// Lists hold at most `ns` entries; a longer walk means a corrupted list and is cut short.
__device__ double canonical_sum(bool have, double first, int head, const uint64_t *sval,
                                const int *snext, int ns, bool *bad) {
  double sum = first;
  constexpr int K = 8;
  uint64_t ob[K];
  int n = 0, idx = head;
  while (idx >= 0 && n < K) {
    if (idx >= ns) { *bad = true; return sum; }
    ob[n++] = ordered_bits(bitsd(sval[idx]));
    idx = snext[idx];
  }
  if (idx < 0) {
    for (int i = 1; i < n; ++i) {
      uint64_t v = ob[i];
      int k = i - 1;
      while (k >= 0 && ob[k] > v) { ob[k + 1] = ob[k]; --k; }
      ob[k + 1] = v;
    }
    for (int i = 0; i < n; ++i) {
      double v = from_ordered(ob[i]);
      sum = have ? sum + v : v;
      have = true;
    }
    return sum;
  }
  uint64_t last = 0;
  bool any_last = false;
  for (int round = 0; round <= ns; ++round) {
    uint64_t best = ~0ull;
    int cnt = 0, steps = 0;
    for (int i = head; i >= 0; i = snext[i]) {
      if (i >= ns || ++steps > ns) { *bad = true; return sum; }
      uint64_t o = ordered_bits(bitsd(sval[i]));
      if (any_last && o <= last) continue;
      if (o < best) { best = o; cnt = 1; } else if (o == best) ++cnt;
    }
    if (cnt == 0) return sum;
    double v = from_ordered(best);
    for (int c = 0; c < cnt; ++c) { sum = have ? sum + v : v; have = true; }
    last = best;
    any_last = true;
  }
  *bad = true;
  return sum;
}

__device__ __forceinline__ int64_t list_sum_int(int head, const uint64_t *sval, const int *snext,
                                                int ns, bool *bad) {
  int64_t tot = 0;
  int steps = 0;
  for (int i = head; i >= 0; i = snext[i]) {
    if (i >= ns || ++steps > ns) { *bad = true; break; }
    tot += (int64_t)sval[i];
  }
  return tot;
}

__device__ __forceinline__ int table_lookup(uint64_t key, const uint64_t *tkey, uint32_t T) {
  uint32_t slot = (uint32_t)mix64(key) & (T - 1);
  for (uint32_t p = 0; p < T; ++p) {
    uint64_t k = tkey[slot];
    if (k == key) return (int)slot;
    if (k == EMPTY_KEY) return -1;
    slot = (slot + 1) & (T - 1);
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
  const int lane = threadIdx.x & 31;
  const uint32_t m = __ballot_sync(0xffffffffu, keep);
  const uint32_t pos = out + __popc(m & ((1u << lane) - 1));
  if (keep && pos < a.capv) a.v_out[(size_t)gb * a.capv + pos] = Rec{key, vb};
  out += __popc(m);
}

__device__ __forceinline__ void flush_ann_acc(const StepArgs &a, int r, AnnAcc &acc) {
  U128 nfx = warp_sum128(acc.norm);
  long long l = warp_sum(acc.len), lb = warp_sum(acc.len_before);
  long long cl = warp_sum(acc.clones), de = warp_sum(acc.deaths), zo = warp_sum(acc.zombies);
  if ((threadIdx.x & 31) == 0) {
    DevStats &st = a.stats[r];
    atomic_add128(&st.norm_lo, &st.norm_hi, nfx);
    atomic_add_ll(&st.len, l);
    atomic_add_ll(&st.len_before, lb);
    atomic_add_ll(&st.clones, cl);
    atomic_add_ll(&st.deaths, de);
    atomic_add_ll(&st.zombies, zo);
  }
  acc = AnnAcc{};
}

// Per-warp shared memory: table keys [tmax], spawn values [caps], table heads [tmax],
// list links [caps], slots first claimed [caps].
__host__ __device__ inline size_t ann_warp_smem(uint32_t tmax, uint32_t caps) {
  return (size_t)tmax * 12 + (size_t)caps * 16;
}

template <int KIND, int STYLE>
__global__ void __launch_bounds__(WARPS * 32) k_annihilate(StepArgs a, int nb_total) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t caps = a.caps, tmax = a.tsize;
  unsigned char *mine = smem + (size_t)w * ann_warp_smem(tmax, caps);
  uint64_t *tkey = reinterpret_cast<uint64_t *>(mine);
  uint64_t *sval = tkey + tmax;
  int *thead = reinterpret_cast<int *>(sval + caps);
  int *snext = thead + tmax;
  int *snew = snext + caps;
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
    const uint32_t ns = nsp < caps ? nsp : caps;
    const uint32_t nv0 = a.cnt_in[gb];
    const uint32_t nv = nv0 < a.capv_in ? nv0 : a.capv_in;
    uint32_t T = 64;
    while (T < 2 * ns && T < tmax) T <<= 1;
    for (uint32_t i = lane; i < T; i += 32) { tkey[i] = EMPTY_KEY; thead[i] = -1; }
    __syncwarp();
    // spawns into the table; slots claimed first are listed in snew
    uint32_t nnew = 0;
    const Rec *sp = a.spawn + (size_t)gb * caps;
    for (uint32_t j0 = 0; j0 < ns; j0 += 32) {
      const uint32_t j = j0 + lane;
      bool first = false;
      int slot = -1;
      if (j < ns) {
        const Rec s = sp[j];
        sval[j] = s.val;
        uint32_t sl = (uint32_t)mix64(s.key) & (T - 1);
        for (uint32_t p = 0; p < T; ++p) {
          const unsigned long long old = atomicCAS((unsigned long long *)&tkey[sl],
                                                   (unsigned long long)EMPTY_KEY,
                                                   (unsigned long long)s.key);
          if (old == EMPTY_KEY || old == s.key) {
            first = old == EMPTY_KEY;
            slot = (int)sl;
            snext[j] = atomicExch(&thead[sl], (int)j);
            break;
          }
          sl = (sl + 1) & (T - 1);
        }
        if (slot < 0) bad = true;
      }
      const uint32_t m = __ballot_sync(0xffffffffu, first);
      if (first) snew[nnew + __popc(m & ((1u << lane) - 1))] = slot;
      nnew += __popc(m);
    }
    __syncwarp();
    uint32_t out = 0;
    // source walkers: diagonal step (diagonal_step!, spawning.jl:73-77) + spawns on them
    const Rec *vbase = a.v_in + (size_t)gb * a.capv_in;
    for (uint32_t e0 = 0; e0 < nv; e0 += 32) {
      const uint32_t e = e0 + lane;
      bool keep = false;
      uint64_t key = 0, vb = 0;
      if (e < nv) {
        const Rec rec = vbase[e];
        key = rec.key;
        const double dg = op_diagonal<KIND>(a, r, key);
        const int slot = ns ? table_lookup(key, tkey, T) : -1;
        int head = -1;
        if (slot >= 0) { head = thead[slot]; thead[slot] = -2; }
        if (STYLE == STYLE_INTEGER) {
          const int64_t v = (int64_t)rec.val;
          const double x = dg * i2d_exact(v);
          const U4 rr = draw(a.seed, PURPOSE_DIAG, rep, a.step, key, 0);
          const int64_t res = round_stochastic(x, u53_of(rr));
          // clones_deaths_zombies (spawning.jl:79-93)
          const int sr = (res > 0) - (res < 0), sv = (v > 0) - (v < 0);
          if (res > v) acc.clones += res - v;
          else if (sr != sv) { acc.deaths += v < 0 ? -v : v; acc.zombies += res < 0 ? -res : res; }
          else acc.deaths += (res - v) < 0 ? v - res : res - v;
          const int64_t tot = res + list_sum_int(head, sval, snext, (int)ns, &bad);
          keep = finalize_entry<STYLE>(a, r, key, 0.0, tot, vb, acc);
        } else {
          double res = dg * bitsd(rec.val);
          if (a.has_proj) {
            const U4 rr = draw(a.seed, PURPOSE_DIAG, rep, a.step, key, 0);
            res = project_threshold(res, a.proj_threshold, u53_of(rr));
          }
          const double tot =
              head >= 0 ? canonical_sum(!is_zero_d(res), res, head, sval, snext, (int)ns, &bad) : res;
          keep = finalize_entry<STYLE>(a, r, key, tot, 0, vb, acc);
        }
      }
      warp_emit(a, gb, keep, key, vb, out);
    }
    __syncwarp();
    // addresses reached only by spawns
    for (uint32_t i0 = 0; i0 < nnew; i0 += 32) {
      const uint32_t i = i0 + lane;
      bool keep = false;
      uint64_t key = 0, vb = 0;
      if (i < nnew) {
        const int slot = snew[i];
        const int head = thead[slot];
        key = tkey[slot];
        if (head >= 0) {
          if (STYLE == STYLE_INTEGER) {
            const int64_t tot = list_sum_int(head, sval, snext, (int)ns, &bad);
            keep = finalize_entry<STYLE>(a, r, key, 0.0, tot, vb, acc);
          } else {
            const double tot = canonical_sum(false, 0.0, head, sval, snext, (int)ns, &bad);
            keep = finalize_entry<STYLE>(a, r, key, tot, 0, vb, acc);
          }
        }
      }
      warp_emit(a, gb, keep, key, vb, out);
    }
    if (lane == 0) {
      a.cnt_out[gb] = out < a.capv ? out : a.capv;
      if (out > a.capv) atomicOr(&a.stats[r].flags, (unsigned)FLAG_V_OVERFLOW);
      if (nsp > caps) atomicOr(&a.stats[r].flags, (unsigned)FLAG_SPAWN_OVERFLOW);
      atomicMax(&a.stats[r].max_v_bucket, out);
      atomicMax(&a.stats[r].max_spawn_bucket, nsp);
      a.scount[gb] = 0;
    }
    __syncwarp();
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(&a.stats[cur_r < 0 ? 0 : cur_r].flags, (unsigned)FLAG_TABLE);
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
  const int want = (nb_total + WARPS - 1) / WARPS;
  const int cap = ctx->num_sms * 64;
  const int grid = want < cap ? want : cap;
  if (ev) cudaEventRecord(ev[0], st);
  k_spawn<KIND, STYLE><<<grid, WARPS * 32, 0, st>>>(a, nb_total);
  if (ev) cudaEventRecord(ev[1], st);
  k_spawn_heavy<KIND, STYLE><<<ctx->num_sms * 4, 256, 0, st>>>(a);
  if (ev) cudaEventRecord(ev[2], st);
  const size_t smem = WARPS * ann_warp_smem(a.tsize, a.caps);
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
