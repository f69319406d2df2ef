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

constexpr int SB = 256;   // spawn CTA
constexpr int AB = 256;   // annihilation CTA

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
    int I = a.h.fermion ? 0 : bose_interaction(key);
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
// Spawning
// ------------------------------------------------------------------------------------------
struct SpawnAcc {
  U128 fx;           // sum |spawn| for float styles
  long long spawns_i;
  long long records;
  long long attempts, exact_n, inexact_n;
};

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

template <int KIND, int STYLE>
__device__ __forceinline__ void spawn_item(const StepArgs &a, int r, uint64_t key, uint64_t vb,
                                           double c, int noff, int exact, uint32_t j,
                                           SpawnAcc &acc) {
  uint32_t rep = a.replica_base + (uint32_t)r;
  if (exact) {
    // Exact (spawning.jl:174-182): val * mat_elem for offdiagonal j+1
    Offdiag od = column_offdiag<KIND>(a.h, key, (int)j + 1);
    if (od.prod == 0) return;
    double y = bitsd(vb) * op_offdiag(a, od);
    if (STYLE == STYLE_DSS && a.proj_threshold > 0) {
      U4 rr = draw(a.seed, PURPOSE_SPAWN, rep, a.step, key, j);
      y = project_threshold(y, a.proj_threshold, u53_of(rr));
    }
    if (y == 0.0) return;
    acc.fx = add128(acc.fx, fixed_of(fabs(y)));
    emit_spawn(a, r, od.key, dbits(y), acc);
    return;
  }
  // WithReplacement attempt j (spawning.jl:232-243): uniform offdiagonal, amplitude c * elem
  U4 rr = draw(a.seed, PURPOSE_SPAWN, rep, a.step, key, j);
  int chosen = (int)uniform_index(rr.x, (uint32_t)noff) + 1;
  Offdiag od = column_offdiag<KIND>(a.h, key, chosen);
  if (od.prod == 0) return;
  double y = c * op_offdiag(a, od);
  if (STYLE == STYLE_INTEGER) {
    int64_t k = round_stochastic(y, u53_of(rr));
    if (k == 0) return;
    acc.spawns_i += k < 0 ? -k : k;
    emit_spawn(a, r, od.key, (uint64_t)k, acc);
  } else {
    if (a.proj_threshold > 0) y = project_threshold(y, a.proj_threshold, u53_of(rr));
    if (y == 0.0) return;
    acc.fx = add128(acc.fx, fixed_of(fabs(y)));
    emit_spawn(a, r, od.key, dbits(y), acc);
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

template <int KIND, int STYLE>
__global__ void __launch_bounds__(SB) k_spawn(StepArgs a, int nb_total) {
  __shared__ uint64_t s_key[SB];
  __shared__ uint64_t s_val[SB];
  __shared__ double s_c[SB];
  __shared__ int s_noff[SB];
  __shared__ int s_exact[SB];
  __shared__ uint32_t s_pref[SB];
  __shared__ uint32_t s_warp[SB / 32];
  __shared__ uint32_t s_tot;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  SpawnAcc acc{};
  for (int gb = blockIdx.x; gb < nb_total; gb += gridDim.x) {
    const int r = gb >> a.nb_bits;
    const uint32_t n0 = a.cnt_in[gb];
    const uint32_t n = n0 < a.capv_in ? n0 : a.capv_in;
    const Rec *base = a.v_in + (size_t)gb * a.capv_in;
    for (uint32_t c0 = 0; c0 < n; c0 += SB) {
      uint32_t e = c0 + tid;
      uint32_t w = 0;
      if (e < n) {
        Rec rec = base[e];
        uint64_t key = rec.key;
        int noff = column_noff<KIND>(a.h, key);
        int exact = 0;
        double c = 0.0;
        uint64_t natt = 0;
        if (STYLE == STYLE_DETERMINISTIC) {
          exact = 1;
          acc.exact_n++;
        } else if (STYLE == STYLE_DSS) {
          double val = bitsd(rec.val);
          double thresh = a.abs_threshold < (double)noff ? a.abs_threshold : (double)noff;
          double amount = (a.boost == 1.0 && a.rel_threshold == 1.0)
                              ? fabs(val) : a.boost * fabs(val) * a.rel_threshold;
          exact = amount >= thresh;
          if (exact) acc.exact_n++; else acc.inexact_n++;
          if (!exact) {
            double bv = a.boost == 1.0 ? fabs(val) : fabs(val) * a.boost;
            natt = (uint64_t)floor_abs(bv);
            if (natt < 1) natt = 1;
            double rc = natt < (uint64_t)a.h.recip_len ? a.h.recip[natt] : 1.0 / (double)natt;
            c = (natt == 1 ? val : val * rc) * (double)noff;
          }
        } else {  // IsStochasticInteger
          int64_t iv = (int64_t)rec.val;
          uint64_t av = (uint64_t)(iv < 0 ? -iv : iv);
          if (a.boost == 1.0) {
            natt = av < 1 ? 1 : av;
            c = (iv < 0 ? -1.0 : 1.0) * (double)noff;
          } else {
            natt = (uint64_t)floor_abs((double)iv * a.boost);
            if (natt < 1) natt = 1;
            double rc = natt < (uint64_t)a.h.recip_len ? a.h.recip[natt] : 1.0 / (double)natt;
            c = ((double)iv * rc) * (double)noff;
          }
        }
        uint64_t work = noff == 0 ? 0 : (exact ? (uint64_t)noff : natt);
        if (work > (1ull << 36)) {       // more attempts than any walker list can hold
          atomicOr(&a.stats[r].flags, (unsigned)FLAG_VALUE_OVERFLOW);
          work = 0;
        }
        acc.attempts += noff == 0 ? 0 : (long long)work;
        if (work > (uint64_t)HEAVY_LIMIT) {
          uint64_t nch = (work + HEAVY_CHUNK - 1) / HEAVY_CHUNK;
          uint32_t idx = atomicAdd(a.heavy_count, (uint32_t)nch);
          for (uint64_t k = 0; k < nch; ++k) {
            if (idx + k >= a.heavy_cap) {
              atomicOr(&a.stats[r].flags, (unsigned)FLAG_HEAVY_OVERFLOW);
              break;
            }
            {
              HeavyChunk ch;
              ch.key = key; ch.val = rec.val; ch.c = c; ch.noff = noff; ch.exact = exact;
              ch.j0 = (uint32_t)(k * HEAVY_CHUNK);
              uint64_t rem = work - k * HEAVY_CHUNK;
              ch.cnt = (uint32_t)(rem < (uint64_t)HEAVY_CHUNK ? rem : HEAVY_CHUNK);
              ch.rep = (uint32_t)r; ch.pad = 0;
              a.heavy[idx + k] = ch;
            }
          }
          work = 0;
        }
        w = (uint32_t)work;
        s_key[tid] = key; s_val[tid] = rec.val; s_c[tid] = c;
        s_noff[tid] = noff; s_exact[tid] = exact;
      }
      // block exclusive scan of w
      uint32_t x = w;
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) s_warp[wid] = x;
      __syncthreads();
      if (wid == 0) {
        uint32_t t = lane < SB / 32 ? s_warp[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
          uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
          if (lane >= o) t += y;
        }
        if (lane < SB / 32) s_warp[lane] = t;
        if (lane == SB / 32 - 1) s_tot = t;
      }
      __syncthreads();
      s_pref[tid] = x - w + (wid ? s_warp[wid - 1] : 0);
      __syncthreads();
      const uint32_t W = s_tot;
      for (uint32_t it = tid; it < W; it += SB) {
        int lo = 0, hi = SB - 1;
        while (lo < hi) {
          int mid = (lo + hi + 1) >> 1;
          if (s_pref[mid] <= it) lo = mid; else hi = mid - 1;
        }
        spawn_item<KIND, STYLE>(a, r, s_key[lo], s_val[lo], s_c[lo], s_noff[lo], s_exact[lo],
                                it - s_pref[lo], acc);
      }
      __syncthreads();
    }
    flush_spawn_acc(a, r, acc);
  }
}

template <int KIND, int STYLE>
__global__ void __launch_bounds__(SB) k_spawn_heavy(StepArgs a) {
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
    for (uint32_t t = threadIdx.x; t < ch.cnt; t += blockDim.x) {
      spawn_item<KIND, STYLE>(a, (int)ch.rep, ch.key, ch.val, ch.c, ch.noff, ch.exact, ch.j0 + t,
                              acc);
    }
    // attempts were counted when the chunk was created
    acc.attempts = 0;
    flush_spawn_acc(a, (int)ch.rep, acc);
  }
}

// ------------------------------------------------------------------------------------------
// Annihilation
// ------------------------------------------------------------------------------------------
struct AnnAcc {
  U128 norm;
  long long len, len_before, clones, deaths, zombies;
};

__device__ __forceinline__ double from_ordered(uint64_t o) {
  return bitsd((o >> 63) ? (o & 0x7fffffffffffffffull) : ~o);
}

// Sum of the spawn list starting at `head` in increasing order of value, after `first`.
// Lists hold at most `ns` entries; a longer walk means a corrupted list and is cut short
// (the caller's flag check reports it).
__device__ double canonical_sum(bool have, double first, int head, const uint64_t *sval,
                                const int *snext, int ns, bool *bad) {
  double sum = first;
  constexpr int K = 16;
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
  // long list: repeated minimum (ties of equal value are indistinguishable)
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

template <int STYLE>
__device__ __forceinline__ void finalize_entry(const StepArgs &a, int r, int gb, uint64_t key,
                                               double fv, int64_t iv, uint32_t *s_out,
                                               AnnAcc &acc) {
  uint64_t vb;
  double dv;
  if (STYLE == STYLE_INTEGER) {
    if (iv == 0) return;
    acc.len_before++;
    vb = (uint64_t)iv;
    dv = (double)iv;
  } else {
    if (fv == 0.0) return;
    acc.len_before++;
    if (a.compression > 0) {
      double at = fabs(fv);
      double prob = a.compression == 1.0 ? at : at / a.compression;
      if (prob < 1) {
        U4 rr = draw(a.seed, PURPOSE_COMPRESS, a.replica_base + (uint32_t)r, a.step, key, 0);
        fv = bernoulli53(u53_of(rr), prob) ? (fv < 0 ? -a.compression : a.compression) : 0.0;
      }
      if (fv == 0.0) return;
    }
    vb = dbits(fv);
    dv = fv;
  }
  uint32_t pos = atomicAdd(s_out, 1u);
  if (pos < a.capv) a.v_out[(size_t)gb * a.capv + pos] = Rec{key, vb};
  acc.norm = add128(acc.norm, fixed_of(fabs(dv)));
  acc.len++;
  if (a.nproj > 0) {
    const uint64_t *pk = a.proj_keys + (size_t)r * a.nproj;
    int lo = 0, hi = a.nproj - 1;
    while (lo <= hi) {
      int mid = (lo + hi) >> 1;
      if (pk[mid] == key) {
        size_t o = (size_t)r * a.nproj + mid;
        a.proj_out_v[o] = a.proj_v[o] * dv;
        a.proj_out_h[o] = a.proj_h[o] * dv;
        break;
      }
      if (pk[mid] < key) lo = mid + 1; else hi = mid - 1;
    }
  }
}

template <int KIND, int STYLE>
__global__ void __launch_bounds__(AB) k_annihilate(StepArgs a, int nb_total) {
  extern __shared__ __align__(16) unsigned char smem[];
  const uint32_t T = a.tsize, caps = a.caps;
  uint64_t *tkey = reinterpret_cast<uint64_t *>(smem);
  uint64_t *skey = tkey + T;
  uint64_t *sval = skey + caps;
  int *thead = reinterpret_cast<int *>(sval + caps);
  int *snext = thead + T;
  __shared__ uint32_t s_out;
  const int tid = threadIdx.x;
  AnnAcc acc{};
  for (int gb = blockIdx.x; gb < nb_total; gb += gridDim.x) {
    const int r = gb >> a.nb_bits;
    const uint32_t rep = a.replica_base + (uint32_t)r;
    const uint32_t nsp = a.scount[gb];
    const uint32_t ns = nsp < caps ? nsp : caps;
    const uint32_t nv0 = a.cnt_in[gb];
    const uint32_t nv = nv0 < a.capv_in ? nv0 : a.capv_in;
    bool bad = false;
    for (uint32_t i = tid; i < T; i += AB) { tkey[i] = EMPTY_KEY; thead[i] = -1; }
    if (tid == 0) s_out = 0;
    const Rec *sp = a.spawn + (size_t)gb * caps;
    for (uint32_t j = tid; j < ns; j += AB) {
      Rec s = sp[j];
      skey[j] = s.key;
      sval[j] = s.val;
    }
    __syncthreads();
    for (uint32_t j = tid; j < ns; j += AB) {
      uint64_t k = skey[j];
      uint32_t slot = (uint32_t)mix64(k) & (T - 1);
      uint32_t p = 0;
      for (; p < T; ++p) {
        unsigned long long old = atomicCAS((unsigned long long *)&tkey[slot],
                                           (unsigned long long)EMPTY_KEY, (unsigned long long)k);
        if (old == EMPTY_KEY || old == k) {
          snext[j] = atomicExch(&thead[slot], (int)j);
          break;
        }
        slot = (slot + 1) & (T - 1);
      }
      if (p == T) atomicOr(&a.stats[r].flags, (unsigned)FLAG_TABLE);
    }
    __syncthreads();
    // source walkers: diagonal step + spawns on the same address
    const Rec *vb = a.v_in + (size_t)gb * a.capv_in;
    for (uint32_t e = tid; e < nv; e += AB) {
      Rec rec = vb[e];
      const uint64_t key = rec.key;
      const double dg = op_diagonal<KIND>(a, r, key);
      const int slot = ns ? table_lookup(key, tkey, T) : -1;
      int head = -1;
      if (slot >= 0) { head = thead[slot]; thead[slot] = -2; }
      if (STYLE == STYLE_INTEGER) {
        const int64_t v = (int64_t)rec.val;
        const double x = dg * (double)v;
        U4 rr = draw(a.seed, PURPOSE_DIAG, rep, a.step, key, 0);
        const int64_t res = round_stochastic(x, u53_of(rr));
        // clones_deaths_zombies (spawning.jl:79-93)
        const int sr = (res > 0) - (res < 0), sv = (v > 0) - (v < 0);
        if (res > v) acc.clones += res - v;
        else if (sr != sv) { acc.deaths += v < 0 ? -v : v; acc.zombies += res < 0 ? -res : res; }
        else acc.deaths += (res - v) < 0 ? v - res : res - v;
        const int64_t tot = res + list_sum_int(head, sval, snext, (int)ns, &bad);
        finalize_entry<STYLE>(a, r, gb, key, 0.0, tot, &s_out, acc);
      } else {
        const double v = bitsd(rec.val);
        double res = dg * v;
        if (a.proj_threshold > 0) {
          U4 rr = draw(a.seed, PURPOSE_DIAG, rep, a.step, key, 0);
          res = project_threshold(res, a.proj_threshold, u53_of(rr));
        }
        const double tot =
            head >= 0 ? canonical_sum(res != 0.0, res, head, sval, snext, (int)ns, &bad) : res;
        finalize_entry<STYLE>(a, r, gb, key, tot, 0, &s_out, acc);
      }
    }
    __syncthreads();
    // addresses that received spawns but were not in the source
    for (uint32_t s = tid; s < T; s += AB) {
      const uint64_t key = tkey[s];
      const int head = thead[s];
      if (key == EMPTY_KEY || head < 0) continue;
      if (STYLE == STYLE_INTEGER) {
        const int64_t tot = list_sum_int(head, sval, snext, (int)ns, &bad);
        finalize_entry<STYLE>(a, r, gb, key, 0.0, tot, &s_out, acc);
      } else {
        const double tot = canonical_sum(false, 0.0, head, sval, snext, (int)ns, &bad);
        finalize_entry<STYLE>(a, r, gb, key, tot, 0, &s_out, acc);
      }
    }
    if (bad) atomicOr(&a.stats[r].flags, (unsigned)FLAG_TABLE);
    __syncthreads();
    if (tid == 0) {
      uint32_t no = s_out;
      a.cnt_out[gb] = no < a.capv ? no : a.capv;
      if (no > a.capv) atomicOr(&a.stats[r].flags, (unsigned)FLAG_V_OVERFLOW);
      if (nsp > caps) atomicOr(&a.stats[r].flags, (unsigned)FLAG_SPAWN_OVERFLOW);
      atomicMax(&a.stats[r].max_v_bucket, no);
      atomicMax(&a.stats[r].max_spawn_bucket, nsp);
      a.scount[gb] = 0;
    }
    // flush statistics of this bucket
    {
      U128 nfx = warp_sum128(acc.norm);
      long long l = warp_sum(acc.len), lb = warp_sum(acc.len_before);
      long long cl = warp_sum(acc.clones), de = warp_sum(acc.deaths), zo = warp_sum(acc.zombies);
      if ((tid & 31) == 0) {
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
    __syncthreads();
  }
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
  int grid = nb_total < (1 << 20) ? nb_total : (1 << 20);
  if (ev) cudaEventRecord(ev[0], st);
  k_spawn<KIND, STYLE><<<grid, SB, 0, st>>>(a, nb_total);
  if (ev) cudaEventRecord(ev[1], st);
  k_spawn_heavy<KIND, STYLE><<<ctx->num_sms * 4, SB, 0, st>>>(a);
  if (ev) cudaEventRecord(ev[2], st);
  size_t smem = (size_t)a.tsize * 12 + (size_t)a.caps * 20;
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_annihilate<KIND, STYLE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         200 * 1024);
    attr_set = true;
  }
  k_annihilate<KIND, STYLE><<<grid, AB, smem, st>>>(a, nb_total);
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
