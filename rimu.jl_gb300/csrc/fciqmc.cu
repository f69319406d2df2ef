// fciqmc.cu -- kernels of one FCIQMC projector step on a bucketed, device-resident walker list.
//
// Layout in HBM.  A walker list is 2^nb_bits buckets per replica; bucket b holds the walkers
// whose address hashes (top nb_bits of mix64) to b, as 16-byte (address, amplitude) records
// in a fixed-capacity slab [b * capv, b * capv + count[b]).  The spawn buffer uses the same
// buckets with slabs of capacity caps.  Every kernel is a template on the address type: one
// 64-bit word, or a Key128 (two words, 32-byte records) for addresses of 65-128 bits.
//
// One step (apply_operator!, src/Interfaces/dictvectors.jl:112-140):
//   k_spawn      each warp lays the walkers of 32 consecutive buckets out as one list,
//                evaluates their columns and deals the spawn attempts out to its lanes, one
//                attempt per lane; every spawn is written straight into the slab of
//                its destination bucket (perform_spawns!, pdworkingmemory.jl:208-217).
//                Columns with more than HEAVY_LIMIT units are cut into chunks.
//   k_spawn_heavy  processes the chunks of heavy columns on all SMs.
//   k_annihilate one CTA per bucket: the source walkers (after their diagonal step) and the
//                spawns are linked into per-address lists of a shared-memory table; each
//                address is summed exactly in 128-bit fixed point and rounded once, threshold
//                compression applied, statistics and the norm accumulated exactly, and the
//                survivors written to the target slab (collect_local!/move_and_compress!,
//                pdworkingmemory.jl:228-273; compression.jl:18-42).
#include <cuda_runtime.h>
#include <cstdio>
#include "rimu_internal.h"

namespace rimu {

// x / y out of line.  A division inlined next to a common path that does not need it (the
// compression threshold one, a tabulated reciprocal) was evaluated speculatively, and on
// GB300 its reciprocal iterations occupied the scarce FP64 pipe for every address.
__device__ __noinline__ double ratio_to_threshold(double x, double y) { return x / y; }


// ------------------------------------------------------------------------------------------
// Model dispatch
// ------------------------------------------------------------------------------------------
template <int KIND, class K>
__device__ __forceinline__ int column_noff(const DevModel &h, K key) {
  if constexpr (KIND == MODEL_MOM1D) {
    // FermiFS2C: N1 * N2 * (M - 1) (HubbardMom1D.jl:141-144)
    if (h.ncomp == 2) return h.cN[0] * h.cN[1] * (h.M - 1);
    MomMap m;
    mom_map(key, m);
    return num_offdiagonals_mom(h, m);
  } else if constexpr (KIND == MODEL_REAL1D) {
    return 2 * bose_num_occupied(key);       // HubbardReal1D.jl:51-53 (one BoseFS)
  }
  return num_offdiagonals_real(h, key);
}

template <int KIND, class K>
__device__ __forceinline__ OffdiagT<K> column_offdiag(const DevModel &h, K key, int chosen) {
  if constexpr (KIND == MODEL_REAL1D) {
    return real1d_offdiag(h, key, chosen);
  } else if constexpr (KIND == MODEL_REALSPACE) {
    return realspace_offdiag(h, key, chosen);
  } else {
    if (h.ncomp == 2) return mom2c_offdiag(h, key, chosen);
    MomMap m;
    mom_map(key, m);
    return mom1d_offdiag(h, key, m, chosen);
  }
}

// sum_i n_i (n_i - 1) of a BoseFS key (bose_hubbard_interaction, bosefs.jl:415-428)
template <class K>
__device__ __forceinline__ int bose_interaction(K key) {
  K x = key;
  int acc = 0;
  while (!kzero(x)) {
    x = kshr(x, kctz(x));
    int n = kctz(~x);
    acc += n * (n - 1);
    x = kshr(x, n);
  }
  return acc;
}

// external_potential of one component chunk: sum over occupied modes, in mode order, of
// n * pot[mode] (HubbardRealSpace.jl:90-97)
template <class K>
__device__ __forceinline__ double component_potential(K ck, int fermion, const double *pot) {
  double pe = 0.0;
  K x = ck;
  if (fermion) {
    while (!kzero(x)) { int b = kctz(x); pe += 1.0 * pot[b]; x = kclear_lowest(x); }
    return pe;
  }
  int mode = 1;
  while (!kzero(x)) {
    int z = kctz(x);
    x = kshr(x, z); mode += z;
    int n = kctz(~x);
    pe += (double)n * pot[mode - 1];
    x = kshr(x, n);
  }
  return pe;
}

// dot(h.kes, OccupiedModeMap(f)) of a FermiFS chunk (fockaddress.jl:316-322)
__device__ __forceinline__ double fermi_kinetic(uint64_t ck, const double *kes) {
  double kin = 0.0;
  uint64_t x = ck;
  while (x) { int b = ctz64(x); kin += kes[b] * 1.0; x &= x - 1; }
  return kin;
}

// FermiFS2C diagonal (one- or two-word address).
template <class K>
__device__ double mom2c_diagonal(const DevModel &h, K key) {
  // FermiFS2C: dot(kes, map_a) + dot(kes, map_b) + u/(2M) * 2 n_a n_b
  // (HubbardMom1D.jl:168-171, 182-187; excitations.jl:172-180)
  const uint64_t ka = component_of(h, key, 0), kb = component_of(h, key, 1);
  const long long nab = 2LL * popc64(ka) * popc64(kb);
  return fermi_kinetic(ka, h.kes) + fermi_kinetic(kb, h.kes) + h.u / (2 * h.M) * (double)nab;
}

// Multi-component HubbardRealSpace diagonal (one- or two-word address).
template <class K>
__device__ double composite_diagonal(const DevModel &h, K key) {
  // local_interaction of the components with the u matrix, then the trap
  // (HubbardRealSpace.jl:18-61, 100-107, 284-287), in the reference's order of operations:
  // _interactions((a_s, ...)) = (self_s + row_s) + _interactions((a_{s+1}, ...)), ending in
  // 0.0; row_s = li(a_s, a_{s+1}) + (li(a_s, a_{s+2}) + (... + 0)), ending in the integer 0;
  // the self-interaction of a FermiFS is the integer 0.  Adding an integer 0 to a double is
  // "+ 0.0" (it turns -0.0 into +0.0); integer + integer stays the integer 0.
  const int C = h.ncomp;
  double in = 0.0;
  if (h.u_nonzero) {
    double rest = 0.0;                         // _interactions of the empty tuple: 0.0
    for (int s = C - 1; s >= 0; --s) {
      const uint64_t ks = component_of(h, key, s);
      double row = 0.0;
      bool row_int = true;                     // the integer 0 closing _interaction_col
      for (int j = C - 1; j > s; --j) {
        const double li = h.cu[cu_index(C, s, j)] *
                          (double)component_overlap(h, ks, h.cferm[s], component_of(h, key, j),
                                                    h.cferm[j]);
        row = row_int ? li + 0.0 : li + row;
        row_int = false;
      }
      double first;
      bool first_int;
      if (h.cferm[s]) {                        // self + row with self the integer 0
        first = row_int ? 0.0 : row + 0.0;
        first_int = row_int;
      } else {
        const double self = h.cu[cu_index(C, s, s)] * (double)bose_interaction(ks) / 2;
        first = row_int ? self + 0.0 : self + row;
        first_int = false;
      }
      rest = first_int ? rest + 0.0 : first + rest;
    }
    in = rest;
  }
  double pe = 0.0;
  if (h.pot) {
    for (int c = 0; c < C; ++c)
      pe += component_potential(component_of(h, key, c), h.cferm[c], h.pot + c * h.M);
  }
  return in + pe;
}

template <int KIND>
__device__ double model_diagonal64(const DevModel &h, uint64_t key);

// Hamiltonian diagonal computed per address (HubbardRealSpace with trap, HubbardMom1D).
template <int KIND, class K>
__device__ double model_diagonal(const DevModel &h, K key) {
  if constexpr (KT<K>::BITS == 64) return model_diagonal64<KIND>(h, key);
  else if constexpr (KIND == MODEL_REAL1D) return h.u * (double)bose_interaction(key) / 2;
  else if (KIND == MODEL_MOM1D && h.ncomp == 2) return mom2c_diagonal(h, key);
  else if (KIND == MODEL_REALSPACE && h.ncomp >= 2) return composite_diagonal(h, key);
  else if constexpr (KIND == MODEL_MOM1D) {
    // dot(h.kes, map) + u/(2M) * momentum_transfer_diagonal(map) (HubbardMom1D.jl:174-177),
    // the same arithmetic as on one-word addresses
    K x = key;
    int mode = 1, s = 0;
    int occ[MAX_MODES];
    double kin = 0.0;
    while (!kzero(x)) {
      int z = kctz(x);
      x = kshr(x, z); mode += z;
      int n = kctz(~x);
      kin += h.kes[mode - 1] * (double)n;
      occ[s++] = n;
      x = kshr(x, n);
    }
    long long onp = 0;
    for (int i = 0; i < s; ++i) {
      onp += (long long)occ[i] * (occ[i] - 1);
      for (int j = 0; j < i; ++j) onp += 4LL * occ[i] * occ[j];
    }
    return kin + h.u / (2 * h.M) * (double)onp;
  } else {
    // HubbardRealSpace one component (HubbardRealSpace.jl:284-293)
    double in = 0.0;
    if (!h.fermion && h.u != 0.0) in = h.u * (double)bose_interaction(key) / 2;
    const double pe = h.pot ? component_potential(key, h.fermion, h.pot) : 0.0;
    return in + pe;
  }
}

// The same for 64-bit addresses, with the momentum-space and two-component models.
template <int KIND>
__device__ double model_diagonal64(const DevModel &h, uint64_t key) {
  if (KIND == MODEL_MOM1D && h.ncomp == 2) return mom2c_diagonal(h, key);
  if (KIND == MODEL_REALSPACE && h.ncomp >= 2) return composite_diagonal(h, key);
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
  const double pe = h.pot ? component_potential(key, h.fermion, h.pot) : 0.0;
  return in + pe;
}

// Diagonal element of the applied operator for replica r.
template <int KIND, class K>
__device__ __forceinline__ double op_diagonal(const StepArgs &a, int r, K key) {
  if (a.dtab) {
    int I = a.h.fermion ? 0 : bose_interaction_fast(key);
    return a.dtab[(size_t)r * a.ndiag + I];
  }
  double d = model_diagonal<KIND>(a.h, key);
  return a.op == OP_TRANSITION ? 1 - a.dt * (d - a.shift[r]) : d;
}

// Offdiagonal element of the applied operator: -H_{new,key} dt (fciqmc.jl:109-112) or H.
template <class K>
__device__ __forceinline__ double op_offdiag(const StepArgs &a, const OffdiagT<K> &od) {
  const double *tab = a.op == OP_TRANSITION ? a.h.aoff : a.h.hoff;
  // the sign by flipping the sign bit (an integer operation; the same value as -v)
  return bitsd(dbits(tab[od.prod]) ^ ((uint64_t)(od.sign < 0) << 63));
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

constexpr int WARPS = 8;            // warps per CTA in the spawn kernel
constexpr int CHUNK_BUCKETS = 32;   // most buckets whose walkers one warp processes together
constexpr int BATCH = 64;           // walkers whose work items are distributed together

// Bucket range of replica r and the replica of bucket gb.
struct RepLayout { uint32_t off; int bits; };
__device__ __forceinline__ RepLayout layout_of(const StepArgs &a, int r) {
  if (!a.rep_off) return RepLayout{(uint32_t)r << a.nb_bits, a.nb_bits};
  return RepLayout{a.rep_off[r], a.rep_bits[r]};
}
__device__ __forceinline__ int replica_of(const StepArgs &a, uint32_t gb) {
  if (!a.rep_off) return (int)(gb >> a.nb_bits);
  int lo = 0, hi = a.nrep - 1;       // the last replica whose range starts at or before gb
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (a.rep_off[mid] <= gb) lo = mid; else hi = mid - 1;
  }
  return lo;
}
__device__ __forceinline__ uint32_t step_of(const StepArgs &a) {
  return a.step_dev ? a.step + *a.step_dev : a.step;
}

// A spawn of a non-initiator parent carries bit 63 of its address's top word (initiator rules
// only; addresses then fit in 63 bits, or in 127 bits of two words); the bucket is that of the
// address itself.
constexpr uint64_t UNSAFE_BIT = 1ull << 63;
__device__ __forceinline__ uint64_t with_flag(uint64_t k, uint64_t flag) { return k | flag; }
__device__ __forceinline__ Key128 with_flag(Key128 k, uint64_t flag) { k.hi |= flag; return k; }
__device__ __forceinline__ bool has_flag(uint64_t k) { return (k & UNSAFE_BIT) != 0; }
__device__ __forceinline__ bool has_flag(Key128 k) { return (k.hi & UNSAFE_BIT) != 0; }
__device__ __forceinline__ uint64_t without_flag(uint64_t k) { return k & ~UNSAFE_BIT; }
__device__ __forceinline__ Key128 without_flag(Key128 k) { k.hi &= ~UNSAFE_BIT; return k; }

template <class K>
__device__ __forceinline__ void emit_spawn(const StepArgs &a, int r, RepLayout lay, K nk,
                                           uint64_t vb, uint64_t flag) {
  const uint32_t b = lay.off + bucket_of(nk, lay.bits);
  const uint32_t pos = atomicAdd(&a.scount[b], 1u);
  if (pos < a.caps) {
    RecT<K> *sp = static_cast<RecT<K> *>(a.spawn);
    sp[(size_t)b * a.caps + pos] = RecT<K>{with_flag(nk, flag), vb};
  } else {
    atomicOr(&a.stats[r].flags, (unsigned)FLAG_SPAWN_OVERFLOW);
  }
}

template <int KIND, class K>
__device__ __forceinline__ OffdiagT<K> step_offdiag(const DevModel &h, K key, int chosen) {
  if constexpr (KIND == MODEL_REAL1D) return real1d_offdiag_fast(key, h.nbits, chosen);
  else return column_offdiag<KIND>(h, key, chosen);
}

// Unit j of one column.  Exact columns deposit val * T_{new,key} for offdiagonal j+1
// (spawning.jl:174-182); sampled columns draw a uniform offdiagonal for attempt j and deposit
// c * T_{new,key} (spawning.jl:232-243).  With float walkers and no on-the-fly projection an
// attempt needs 32 random bits: attempt j takes word j % 4 of Philox block j / 4 (each lane
// evaluates the block of its own attempt; under SIMT this costs no extra issue slots).
template <int KIND, int STYLE, class K>
__device__ __forceinline__ void spawn_unit(const StepArgs &a, int r, RepLayout lay, uint32_t step,
                                           K key, uint64_t vb, double c, int noff,
                                           int exact, uint64_t flag, uint32_t j) {
  const uint32_t rep = a.replica_base + (uint32_t)r;
  if (exact) {
    const OffdiagT<K> od = step_offdiag<KIND>(a.h, key, (int)j + 1);
    if (od.prod == 0) return;
    double y = bitsd(vb) * op_offdiag(a, od);
    if (STYLE == STYLE_DSS && a.has_proj) {
      const U4 rr = draw(a.seed, PURPOSE_SPAWN, rep, step, kword(key), j);
      y = project_threshold(y, a.proj_threshold, u53_of(rr));
    }
    if (is_zero_d(y)) return;
    emit_spawn(a, r, lay, od.key, dbits(y), flag);
    return;
  }
  const bool grouped = STYLE != STYLE_INTEGER && !a.has_proj;
  const U4 rr = draw(a.seed, PURPOSE_SPAWN, rep, step, kword(key), grouped ? j >> 2 : j);
  uint32_t word = rr.x;
  if (grouped) {
    const uint32_t q = j & 3;
    word = q == 0 ? rr.x : q == 1 ? rr.y : q == 2 ? rr.z : rr.w;
  }
  const int chosen = (int)uniform_index(word, (uint32_t)noff) + 1;
  const OffdiagT<K> od = step_offdiag<KIND>(a.h, key, chosen);
  if (od.prod == 0) return;
  double y = c * op_offdiag(a, od);
  if (STYLE == STYLE_INTEGER) {
    const int64_t k = round_stochastic(y, u53_of(rr));
    if (k == 0) return;
    emit_spawn(a, r, lay, od.key, (uint64_t)k, flag);
  } else {
    if (a.has_proj) y = project_threshold(y, a.proj_threshold, u53_of(rr));
    if (is_zero_d(y)) return;
    emit_spawn(a, r, lay, od.key, dbits(y), flag);
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

// Whether a walker is a non-initiator under the initiator rule (|value| <= threshold,
// initiators.jl:142-157); always false without a rule.
template <int STYLE>
__device__ __forceinline__ int parent_unsafe(const StepArgs &a, uint64_t vb) {
  if (!a.init_rule) return 0;
  const double v = STYLE == STYLE_INTEGER ? i2d_exact((int64_t)vb) : bitsd(vb);
  return !(abs_d(v) > a.init_thr);
}

__device__ __forceinline__ double dint_of(const DevModel &h, int n) {
  return n < h.recip_len ? h.dint[n] : (double)n;
}
// 1/n from the host table (the division only beyond it)
__device__ __forceinline__ double recip_of(const DevModel &h, uint64_t n) {
  if (n < (uint64_t)h.recip_len) return h.recip[n];
  return ratio_to_threshold(1.0, (double)n);
}

// Work of one column: units (offdiagonals if exact, attempts otherwise) and the spawn
// coefficient c, without FP64 compares (DynamicSemistochastic, spawning.jl:364-378;
// WithReplacement attempts, spawning.jl:234-235).
template <int KIND, int STYLE, class K>
__device__ __forceinline__ uint64_t column_work(const StepArgs &a, K key, uint64_t vb,
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
    if (a.boost_one && !a.has_abs_thr) {
      // boost 1, rel_threshold 1, no absolute threshold: the amount is |val| and the column is
      // exact when floor(|val|) >= noff; only the spawn coefficient takes FP64 multiplies
      const int64_t fl = floor_abs(val);
      exact = fl >= (int64_t)noff;
      if (exact) acc.exact_n++; else acc.inexact_n++;
      if (!exact) {
        natt = fl < 1 ? 1 : (uint64_t)fl;
        double t = val;
        if (natt != 1) t = val * recip_of(a.h, natt);
        c = t * dint_of(a.h, noff);
      }
    } else {
      const double amount = a.boost_one ? abs_d(val) : a.boost * abs_d(val) * a.rel_threshold;
      if (!a.has_abs_thr || a.abs_threshold >= (double)noff) exact = floor_abs(amount) >= (int64_t)noff;
      else exact = amount >= a.abs_threshold;
      if (exact) acc.exact_n++; else acc.inexact_n++;
      if (!exact) {
        natt = (uint64_t)floor_abs(a.boost_one ? val : abs_d(val) * a.boost);
        if (natt < 1) natt = 1;
        c = (natt == 1 ? val : val * recip_of(a.h, natt)) * dint_of(a.h, noff);
      }
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
      c = (i2d_exact(iv) * recip_of(a.h, natt)) * dint_of(a.h, noff);
    }
  }
  return noff == 0 ? 0 : (exact ? (uint64_t)noff : natt);
}

// Cut a column with more than HEAVY_LIMIT units into chunks for k_spawn_heavy.
template <class K>
__device__ void push_heavy(const StepArgs &a, int r, const RecT<K> &rec, double c, int noff,
                           int exact, int unsafe, uint64_t work) {
  const uint64_t nch = (work + HEAVY_CHUNK - 1) / HEAVY_CHUNK;
  const uint32_t idx = atomicAdd(a.heavy_count, (uint32_t)nch);
  for (uint64_t k = 0; k < nch; ++k) {
    if (idx + k >= a.heavy_cap) {
      atomicOr(&a.stats[r].flags, (unsigned)FLAG_HEAVY_OVERFLOW);
      break;
    }
    HeavyChunk ch;
    ch.key = KT<K>::lo(rec.key); ch.key_hi = KT<K>::hi(rec.key);
    ch.val = rec.val; ch.c = c; ch.noff = noff; ch.exact = exact;
    ch.j0 = (uint32_t)(k * HEAVY_CHUNK);
    const uint64_t rem = work - k * HEAVY_CHUNK;
    ch.cnt = (uint32_t)(rem < (uint64_t)HEAVY_CHUNK ? rem : HEAVY_CHUNK);
    ch.rep = (uint32_t)r; ch.unsafe = (uint32_t)unsafe;
    a.heavy[idx + k] = ch;
  }
}

// Each warp takes spawn_cb (a power of two <= CHUNK_BUCKETS) consecutive buckets of one
// replica, lays their walkers out as one flat list and works through it BATCH walkers at a
// time: every lane evaluates the columns of two walkers, then the batch's units (spawn
// attempts, or offdiagonals of exact columns) are dealt out one per lane by an exclusive scan
// and a binary search.  Five CTAs per SM (at most 48 registers a thread, a few bytes spilled):
// the kernel waits mostly on memory, and 40 resident warps hide more of it than 32 (spawn 5 %
// faster than with four CTAs at 64 registers).
template <int KIND, int STYLE, class K>
__global__ void __launch_bounds__(WARPS * 32, 5) k_spawn(StepArgs a, int nb_total) {
  __shared__ uint32_t s_bpre[WARPS][CHUNK_BUCKETS + 1];
  __shared__ K s_key[WARPS][BATCH];
  __shared__ uint64_t s_val[WARPS][BATCH];
  __shared__ double s_c[WARPS][BATCH];
  __shared__ uint32_t s_excl[WARPS][BATCH];
  __shared__ uint32_t s_meta[WARPS][BATCH];   // noff | exact << 31
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (a.ann_count && blockIdx.x == 0 && threadIdx.x == 0) *a.ann_count = 0;
  const int cb = a.spawn_cb;
  const int nchunks = nb_total / cb;
  const uint32_t step = step_of(a);
  SpawnAcc acc{};
  int cur_r = -1;
  for (int ch = blockIdx.x * WARPS + w; ch < nchunks; ch += gridDim.x * WARPS) {
    const int b0 = ch * cb;
    const int r = replica_of(a, (uint32_t)b0);
    const RepLayout lay = layout_of(a, r);
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
        uint32_t units = 0;
        if (f < E) {
          int bi = 0;
#pragma unroll
          for (int st = 16; st >= 1; st >>= 1)
            if (bi + st < cb && s_bpre[w][bi + st] <= f) bi += st;
          const RecT<K> rec = static_cast<const RecT<K> *>(a.v_in)[(size_t)(b0 + bi) * a.capv_in +
                                                                  (f - s_bpre[w][bi])];
          int noff, exact;
          double c;
          uint64_t work = column_work<KIND, STYLE>(a, rec.key, rec.val, noff, exact, c, acc);
          if (work > (1ull << 36)) {       // more attempts than any walker list can hold
            atomicOr(&a.stats[r].flags, (unsigned)FLAG_VALUE_OVERFLOW);
            work = 0;
          }
          acc.attempts += (long long)work;
          if (work > (uint64_t)HEAVY_LIMIT) {
            push_heavy(a, r, rec, c, noff, exact, parent_unsafe<STYLE>(a, rec.val), work);
            work = 0;
          }
          s_key[w][slot] = rec.key;
          s_val[w][slot] = rec.val;
          s_c[w][slot] = c;
          s_meta[w][slot] = (uint32_t)noff | ((uint32_t)exact << 31) |
                            ((uint32_t)parent_unsafe<STYLE>(a, rec.val) << 30);
          units = (uint32_t)work;
        }
        items[hh] = units;
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
        const uint32_t meta = s_meta[w][lo];
        spawn_unit<KIND, STYLE>(a, r, lay, step, s_key[w][lo], s_val[w][lo], s_c[w][lo],
                                (int)(meta & 0x3fffffffu), (int)(meta >> 31),
                                ((meta >> 30) & 1u) ? UNSAFE_BIT : 0ull, it - s_excl[w][lo]);
      }
      __syncwarp();
    }
  }
  if (cur_r >= 0) flush_spawn_acc(a, cur_r, acc);
}

template <int KIND, int STYLE, class K>
__global__ void __launch_bounds__(256) k_spawn_heavy(StepArgs a) {
  const uint32_t step = step_of(a);
  uint32_t nch = *a.heavy_count;
  if (nch > a.heavy_cap) nch = a.heavy_cap;
  for (uint32_t ci = blockIdx.x; ci < nch; ci += gridDim.x) {
    HeavyChunk ch = a.heavy[ci];
    if (ch.cnt > (uint32_t)HEAVY_CHUNK || ch.rep >= (uint32_t)a.nrep) {
      if (threadIdx.x == 0) atomicOr(&a.stats[0].flags, (unsigned)FLAG_TABLE);
      continue;
    }
    const RepLayout lay = layout_of(a, (int)ch.rep);
    for (uint32_t t = threadIdx.x; t < ch.cnt; t += blockDim.x)
      spawn_unit<KIND, STYLE>(a, (int)ch.rep, lay, step, KT<K>::make(ch.key, ch.key_hi), ch.val,
                              ch.c, ch.noff, ch.exact, ch.unsafe ? UNSAFE_BIT : 0ull, ch.j0 + t);
  }
}

// ------------------------------------------------------------------------------------------
// Annihilation: one CTA per bucket, exact sums from per-address lists in a shared-memory table
// ------------------------------------------------------------------------------------------
// Summation rule (the oracle states the same): when every contribution to an address is a
// multiple of 2^-64 below 2^48 in magnitude, the address gets the exact sum rounded once to
// the nearest double, so the order of the contributions does not matter; otherwise the
// contributions are added in canonical order (the diagonal term, then the spawns by
// increasing value).  Integer walkers are summed as int64.
struct AnnAcc {
  U128 norm, spawn_fx;
  long long len, len_before, clones, deaths, zombies, spawns_i, records;
  long long ncomp;                      // survivors of compression draws (|value| = threshold)
};

// Integer-walker statistics of one pass over a bucket; kept only if the pass completes.
struct PassAcc {
  long long clones, deaths, zombies;
};

// A bucket whose contributions overflow the table is processed in passes: pass `sel` at depth
// `lvl` takes the addresses whose split word agrees with sel in its low lvl bits.  The split
// word is a bijection of the address word, so any two addresses are separated by depth 64.
constexpr int MAX_SPLIT = 64;
__device__ __forceinline__ uint64_t split_word(uint64_t kw) {
  return mix64(kw ^ 0x5851F42D4C957F2Dull);
}
__device__ __forceinline__ uint64_t split_mask(int lvl) {
  return lvl >= 64 ? ~0ull : (1ull << lvl) - 1ull;
}
constexpr uint32_t NIL = 0xffffffffu;   // end of a contribution list
constexpr int ANN_THREADS = 256;        // threads of one annihilation CTA
constexpr uint32_t PACK_FAIL = 0x80000000u;   // overflow bit of the packed insertion counter

// Shared memory of one annihilation CTA with T table slots and T contribution entries:
// keys [T] u64, contribution values [T] u64, list heads [T] u32, contribution link words
// [T] u16, occupied-slot list [T] u16, compression queue [T] u16: 26 bytes per slot, so that
// four CTAs with 2048 slots fit one SM.
// With two-word addresses the keys take 16 bytes: 34 bytes per slot.
template <class K = uint64_t>
__host__ __device__ inline size_t ann_smem(uint32_t T) { return (size_t)T * (sizeof(K) + 18); }


__device__ __forceinline__ U128 neg128(U128 x) {
  U128 r;
  r.lo = ~x.lo + 1;
  r.hi = ~x.hi + (x.lo == 0 ? 1 : 0);
  return r;
}

// |x| as a multiple of 2^-64, if it is one and |x| < 2^48 (then equal to fixed_of(|x|)).
__device__ __forceinline__ bool fixed_magnitude(double x, U128 &m) {
  const uint64_t ab = dbits(x) & 0x7fffffffffffffffull;
  m = U128{0, 0};
  if (ab == 0) return true;
  const int e = (int)(ab >> 52);
  if (e == 0 || e >= 1023 + 48) return false;
  const uint64_t mant = (ab & lowmask(52)) | (1ull << 52);
  const int sh = e - 1075 + 64;            // |x| = mant * 2^(sh - 64), sh <= 59
  if (sh >= 0) {
    m.lo = mant << sh;
    m.hi = sh > 11 ? (mant >> (64 - sh)) : 0;
  } else {
    if (-sh >= 53 || (mant & lowmask(-sh))) return false;
    m.lo = mant >> (-sh);
  }
  return true;
}

__device__ __forceinline__ double signed_fixed_to_double(U128 x) {
  if (x.hi >> 63) return bitsd(dbits(fixed_to_double(neg128(x))) ^ 0x8000000000000000ull);
  return fixed_to_double(x);
}

__device__ __forceinline__ double from_ordered(uint64_t o) {
  return bitsd((o >> 63) ? (o & 0x7fffffffffffffffull) : ~o);
}

// Contribution link word (16 bits): the index of the next contribution of the address's list
// (13 bits; LINK_END after the last), the contribution's class (2 bits, initiator rules) and
// whether it is the diagonal term of a source walker (1 bit).
constexpr uint32_t LINK_END = 0x1FFFu;
__device__ __forceinline__ uint32_t link_next(uint16_t w) {
  const uint32_t n = w & 0x1FFFu;
  return n == LINK_END ? NIL : n;
}
__device__ __forceinline__ int link_cls(uint16_t w) { return (w >> 13) & 3; }
__device__ __forceinline__ bool link_diag(uint16_t w) { return (w >> 15) != 0; }

// Whether contribution a comes before b in the canonical order: the diagonal term first,
// then by increasing value (order-preserving bits).
__device__ __forceinline__ bool canon_before(const uint64_t *cval, const uint16_t *clink,
                                             uint32_t a, uint32_t b) {
  const bool da = link_diag(clink[a]), db = link_diag(clink[b]);
  if (da != db) return da;
  return ordered_bits(bitsd(cval[a])) <= ordered_bits(bitsd(cval[b]));
}
__device__ __forceinline__ void link_set_next(uint16_t *clink, uint32_t c, uint32_t nxt) {
  clink[c] = (uint16_t)((clink[c] & ~LINK_END) | (nxt == NIL ? LINK_END : nxt));
}

// Sorts the list starting at `head` into canonical order by relinking it in place (bottom-up
// merge sort of a singly linked list: O(k log k) comparisons, no extra memory) and returns
// the new head.  Lists hold at most `n` entries; a longer walk means a corrupted list.
__device__ uint32_t sort_list(uint32_t head, const uint64_t *cval, uint16_t *clink, uint32_t n,
                              bool *bad) {
  uint32_t len = 0;
  for (uint32_t c = head; c != NIL; c = link_next(clink[c])) {
    if (c >= n || ++len > n) { *bad = true; return head; }
  }
  for (uint32_t width = 1; width < len; width <<= 1) {
    uint32_t new_head = NIL, tail = NIL, cur = head;
    while (cur != NIL) {
      uint32_t a = cur, na = 0;
      while (cur != NIL && na < width) { cur = link_next(clink[cur]); ++na; }
      uint32_t b = cur, nb = 0;
      while (cur != NIL && nb < width) { cur = link_next(clink[cur]); ++nb; }
      while (na > 0 || nb > 0) {
        uint32_t take;
        if (nb == 0 || (na > 0 && canon_before(cval, clink, a, b))) {
          take = a; a = link_next(clink[a]); --na;
        } else {
          take = b; b = link_next(clink[b]); --nb;
        }
        if (tail == NIL) new_head = take; else link_set_next(clink, tail, take);
        tail = take;
      }
    }
    link_set_next(clink, tail, NIL);
    head = new_head;
  }
  return head;
}

// Canonical-order sum for an address with an inexact contribution: `first` (the diagonal
// term, when `have`) followed by the spawns of the list starting at `head` (diagonal terms are
// skipped; with cls >= 0 only that class counts) in increasing order of value.  Lists of more
// than eight such spawns are sorted in place first (`head` is updated).  Lists hold at most
// `n` entries; a longer walk means a corrupted list and is cut short.
__device__ double canonical_sum_list(bool have, double first, uint32_t &head, const uint64_t *cval,
                                     uint16_t *clink, uint32_t n, bool *bad, int cls = -1) {
  double sum = first;
  constexpr int K = 8;
  uint64_t ob[K];
  int k = 0;
  bool more = false;
  uint32_t steps = 0;
  for (uint32_t c = head; c != NIL; c = link_next(clink[c])) {
    if (c >= n || ++steps > n) { *bad = true; return sum; }
    const uint16_t w = clink[c];
    if (link_diag(w) || (cls >= 0 && link_cls(w) != cls)) continue;
    if (k < K) ob[k++] = ordered_bits(bitsd(cval[c]));
    else { more = true; break; }
  }
  if (!more) {
    for (int i = 1; i < k; ++i) {
      const uint64_t v = ob[i];
      int j = i - 1;
      while (j >= 0 && ob[j] > v) { ob[j + 1] = ob[j]; --j; }
      ob[j + 1] = v;
    }
    for (int i = 0; i < k; ++i) {
      const double v = from_ordered(ob[i]);
      sum = have ? sum + v : v;
      have = true;
    }
    return sum;
  }
  head = sort_list(head, cval, clink, n, bad);
  steps = 0;
  for (uint32_t c = head; c != NIL; c = link_next(clink[c])) {
    if (c >= n || ++steps > n) { *bad = true; return sum; }
    const uint16_t w = clink[c];
    if (link_diag(w) || (cls >= 0 && link_cls(w) != cls)) continue;
    const double v = bitsd(cval[c]);
    sum = have ? sum + v : v;
    have = true;
  }
  return sum;
}

enum : uint8_t { CLS_SAFE = 0, CLS_UNSAFE = 1, CLS_INITIATOR = 2 };

// Value of an address from the sums of its three contribution classes by the initiator rule
// (from_initiator_value, initiators.jl:138-140, 181-183, 208-214).
__device__ __forceinline__ double initiator_value_f(int rule, double thr, double fs, double fu,
                                                    double fi) {
  if (rule == RIMU_INIT_INITIATOR) {          // safe + initiator + !iszero(initiator) * unsafe
    double s = fs + fi;
    if (!is_zero_d(fi)) s = s + fu;
    return s;
  }
  if (rule == RIMU_INIT_SIMPLE) return fs + fi;
  double s = fi + fs;                         // CoherentInitiator
  if (!is_zero_d(fi) || abs_d(fu) > thr) s = s + fu;
  return s;
}
__device__ __forceinline__ int64_t initiator_value_i(int rule, double thr, int64_t ns, int64_t nu,
                                                     int64_t ni) {
  if (rule == RIMU_INIT_INITIATOR) return ns + ni + (ni != 0 ? nu : 0);
  if (rule == RIMU_INIT_SIMPLE) return ns + ni;
  return ni + ns + ((ni != 0 || abs_d(i2d_exact(nu)) > thr) ? nu : 0);
}

// Sum of the contributions of one address under an initiator rule: each class summed by the
// summation rule (the diagonal term, when in that class, first in canonical order), then
// combined.  Also counts the spawn statistics.
__device__ double initiator_sum_f(const StepArgs &a, uint32_t head, const uint64_t *cval,
                                  uint16_t *clink, uint32_t ncon, AnnAcc &acc, bool *bad) {
  U128 sum[3] = {{0, 0}, {0, 0}, {0, 0}};
  bool exact[3] = {true, true, true};
  int cnt[3] = {0, 0, 0};
  int dcls = -1;                       // class of the diagonal term, if any
  double dval = 0.0;
  uint32_t steps = 0;
  for (uint32_t c = head; c != NIL; c = link_next(clink[c])) {
    if (c >= ncon || ++steps > ncon) { *bad = true; break; }
    const uint64_t v = cval[c];
    const uint16_t w = clink[c];
    const int k = link_cls(w) < 3 ? link_cls(w) : 0;
    U128 m;
    const bool ex = fixed_magnitude(bitsd(v), m);
    if (link_diag(w)) {
      dcls = k;
      dval = bitsd(v);
    } else {
      acc.records++;
      acc.spawn_fx = add128(acc.spawn_fx, ex ? m : fixed_of(abs_d(bitsd(v))));
    }
    exact[k] = exact[k] && ex;
    sum[k] = add128(sum[k], (v >> 63) ? neg128(m) : m);
    cnt[k]++;
  }
  double f[3];
  for (int k = 0; k < 3; ++k) {
    if (cnt[k] == 0) { f[k] = 0.0; continue; }
    if (exact[k]) { f[k] = signed_fixed_to_double(sum[k]); continue; }
    const bool dk = dcls == k;
    f[k] = canonical_sum_list(dk && !is_zero_d(dval), dk ? dval : 0.0, head, cval, clink, ncon,
                              bad, k);
  }
  return initiator_value_f(a.init_rule, a.init_thr, f[CLS_SAFE], f[CLS_UNSAFE], f[CLS_INITIATOR]);
}

// Diagonal step of one walker (diagonal_step!, spawning.jl:73-77), float walkers.
template <int KIND, class K>
__device__ __forceinline__ double diag_float(const StepArgs &a, int r, uint32_t rep, uint32_t step,
                                             const RecT<K> &rec) {
  double res = op_diagonal<KIND>(a, r, rec.key) * bitsd(rec.val);
  if (a.has_proj) {
    const U4 rr = draw(a.seed, PURPOSE_DIAG, rep, step, kword(rec.key), 0);
    res = project_threshold(res, a.proj_threshold, u53_of(rr));
  }
  return res;
}

// Slot of `key` in the table, claimed if the key is new; -1 if the table is full.  Probing
// starts at the top bits of a multiplicative hash of the key.
__device__ __forceinline__ int table_insert(Key128 *tkey, uint32_t T, int tbits, Key128 key,
                                            bool &claimed) {
  // two-word keys: every probe is a 16-byte compare-and-swap (no torn reads of a slot)
  uint32_t sl = (uint32_t)((kword(key) * 0x9E3779B97F4A7C15ull) >> (64 - tbits));
  claimed = false;
  const Key128 empty = KT<Key128>::empty();
  for (uint32_t p = 0; p < T; ++p) {
    const Key128 old = atomicCAS(&tkey[sl], empty, key);
    if (old == empty) { claimed = true; return (int)sl; }
    if (old == key) return (int)sl;
    sl = (sl + 1) & (T - 1);
  }
  return -1;
}
__device__ __forceinline__ int table_insert(uint64_t *tkey, uint32_t T, int tbits, uint64_t key,
                                            bool &claimed) {
  uint32_t sl = (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - tbits));
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

__device__ __forceinline__ void flush_ann_acc(const StepArgs &a, int r, AnnAcc &acc) {
  // each compression survivor adds fixed_of(threshold) to the norm
  const U128 th = fixed_of(abs_d(a.compression));
  const uint64_t nc = (uint64_t)acc.ncomp;
  acc.norm = add128(acc.norm, U128{th.lo * nc, __umul64hi(th.lo, nc) + th.hi * nc});
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

// Index for the lanes of a warp with `flag` set in a list whose length is *count: one
// shared-memory atomic per warp.
__device__ __forceinline__ uint32_t warp_append(uint32_t *count, bool flag) {
  const uint32_t m = __ballot_sync(0xffffffffu, flag);
  uint32_t base = 0;
  if ((threadIdx.x & 31) == 0 && m) base = atomicAdd(count, (uint32_t)__popc(m));
  base = __shfl_sync(0xffffffffu, base, 0);
  return base + __popc(m & lanemask_lt());
}

__device__ __forceinline__ bool below_threshold(const StepArgs &a, double fv) {
  if (a.comp_mode == 1) return abs_lt_one(fv);
  if (a.comp_mode == 2) return ratio_to_threshold(abs_d(fv), a.compression) < 1;
  return false;
}

// Compression draw (compression.jl:28-42) for an address whose |value| is below the
// threshold: kept at +-threshold with probability |value| / threshold.
template <int STYLE, class K>
__device__ __forceinline__ bool compress_draw(const StepArgs &a, int r, uint32_t step, K key,
                                              double &fv) {
  const double prob = a.comp_mode == 1 ? abs_d(fv) : ratio_to_threshold(abs_d(fv), a.compression);
  const U4 rr = draw(a.seed, PURPOSE_COMPRESS, a.replica_base + (uint32_t)r, step, kword(key), 0);
  if (!bernoulli53(u53_of(rr), prob)) return false;
  fv = signed_like(a.compression, fv);
  return true;
}

// Statistics and the ProjectedEnergy dot products of a kept address (its |value| in fixed
// point is added to the norm by the caller).
template <int STYLE, class K>
__device__ __forceinline__ void account_entry(const StepArgs &a, int r, K key, double dv,
                                              AnnAcc &acc) {
  acc.len++;
  if (a.nproj == 0) return;
  // the projector's addresses, sorted, in the words of K (Key128: (lo, hi) pairs)
  const K *pk = reinterpret_cast<const K *>(a.proj_keys) + (size_t)r * a.nproj;
  int lo = 0, hi = a.nproj - 1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    const K pm = pk[mid];
    if (pm == key) {
      const size_t o = (size_t)r * a.nproj + mid;
      a.proj_out_v[o] = a.proj_v[o] * dv;
      a.proj_out_h[o] = a.proj_h[o] * dv;
      break;
    }
    if (pm < key) lo = mid + 1; else hi = mid - 1;
  }
}
template <int STYLE, class K>
__device__ __forceinline__ void account_kept(const StepArgs &a, int r, K key, double dv,
                                             U128 mag, AnnAcc &acc) {
  acc.norm = add128(acc.norm, mag);
  account_entry<STYLE>(a, r, key, dv, acc);
}

// One CTA per bucket.  The bucket's contributions -- the source walkers after their
// diagonal step and the spawns -- are dealt out to all threads: each finds or claims the
// slot of its address in a shared-memory table and pushes itself onto the slot's list (one
// 32-bit atomic exchange).  Each occupied slot is then finalized by one thread, which walks
// its list adding the contributions exactly in 128-bit fixed point, rounds once, applies the
// compression threshold and appends the survivor to the target slab; addresses below the
// threshold are queued and drawn together afterwards, so that the random draws run on full
// warps, and float addresses with three or more contributions are finished after them, also
// by full warps.  A bucket with more contributions than the table holds is processed in
// passes, each taking the addresses whose hash bits 16.. select it; a pass that still
// overflows is split.
template <int KIND, int STYLE, class K>
__global__ void __launch_bounds__(ANN_THREADS, 4) k_annihilate(StepArgs a, int nb_total) {
  extern __shared__ __align__(16) unsigned char smem[];
  // per pass parity: packed insertion counter, compression queue length, second-list length
  __shared__ uint32_t s_cnt[2][4];
  __shared__ uint32_t s_out;            // entries written to the target slab of the bucket
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  const uint32_t T = a.ann_list ? a.tsize_list : a.tsize;
  K *tkey = reinterpret_cast<K *>(smem);
  uint64_t *cval = reinterpret_cast<uint64_t *>(tkey + T);
  uint32_t *thead = reinterpret_cast<uint32_t *>(cval + T);
  uint16_t *clink = reinterpret_cast<uint16_t *>(thead + T);
  uint16_t *slist = clink + T;
  uint16_t *qlist = slist + T;
  const uint32_t lim = T - ANN_THREADS;   // a warp starts a round of insertions only below this
  const int tbits = 31 - __clz((int)T);
  const K EMPTY = KT<K>::empty();
  for (uint32_t i = tid; i < T; i += ANN_THREADS) { tkey[i] = EMPTY; thead[i] = NIL; }
  if (tid < 8) s_cnt[tid >> 2][tid & 3] = 0;
  if (tid == 0) s_out = 0;
  __syncthreads();
  // Three barriers per pass: after the insertions, before the addresses with three or more
  // contributions and the compression draws (float walkers), and at the end.  Each thread clears the slots it finalizes, and the counters of a pass are zeroed
  // during the next pass (they alternate by pass parity).
  int par = 0;
  const uint32_t step = step_of(a);
  AnnAcc acc{};
  int cur_r = -1;
  bool bad = false;
  // every bucket, or (after k_ann_warp) the buckets it left in the list
  uint32_t nwork = (uint32_t)nb_total;
  if (a.ann_list) {
    const uint32_t n = *a.ann_count;
    nwork = n < nwork ? n : nwork;
  }
  for (uint32_t wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
    const int gb = a.ann_list ? (int)a.ann_list[wi] : (int)wi;
    const int r = replica_of(a, (uint32_t)gb);
    if (r != cur_r) {
      if (cur_r >= 0) flush_ann_acc(a, cur_r, acc);
      cur_r = r;
    }
    const uint32_t rep = a.replica_base + (uint32_t)r;
    const uint32_t nsp = a.scount[gb];
    const uint32_t ns = nsp < a.caps ? nsp : a.caps;
    const uint32_t nv0 = a.cnt_in[gb];
    const uint32_t nv = nv0 < a.capv_in ? nv0 : a.capv_in;
    const RecT<K> *sp = static_cast<const RecT<K> *>(a.spawn) + (size_t)gb * a.caps;
    const RecT<K> *vbase = static_cast<const RecT<K> *>(a.v_in) + (size_t)gb * a.capv_in;
    RecT<K> *vout = static_cast<RecT<K> *>(a.v_out) + (size_t)gb * a.capv;
    const uint32_t need = nv + ns;   // contributions: also an upper bound on the addresses
    int lvl0 = 0;
    if (need > lim) {
      lvl0 = 1;
      while (lvl0 < 30 && (uint64_t)need > ((uint64_t)(lim * 3 / 4) << lvl0)) ++lvl0;
    }
    int lvl = lvl0;
    uint64_t sel = 0;
    for (;;) {
      const uint64_t mask = split_mask(lvl);
      // s_pack: contribution entries (bits 0-15), occupied slots (bits 16-30), overflow (bit 31)
      uint32_t *const s_pack = &s_cnt[par][0], *const s_nq = &s_cnt[par][1];
      uint32_t *const s_nslow = &s_cnt[par][2];
      PassAcc pa{};
      // ---- every contribution of this pass onto the list of its address ----
      for (uint32_t f0 = (uint32_t)w * 32; f0 < need; f0 += ANN_THREADS) {
        const uint32_t pk = __shfl_sync(0xffffffffu, *(volatile uint32_t *)s_pack, 0);
        if (pk >> 31) break;
        if ((pk & 0xffffu) > lim || ((pk >> 16) & 0x7fffu) > lim) {
          if (lane == 0) atomicOr(s_pack, PACK_FAIL);
          break;
        }
        const uint32_t f = f0 + lane;
        bool add = false, claimed = false, lfail = false, src = false;
        int slot = -1;
        uint64_t vbits = 0;
        uint8_t cls = CLS_SAFE;
        if (f < need) {
          src = f < nv;
          RecT<K> rec = src ? vbase[f] : sp[f - nv];
          if (a.init_rule) {
            // classes of the initiator rules (initiators.jl:142-157): a spawn carries its
            // parent's class in bit 63 of the top word; a diagonal term is "initiator" for an
            // initiator
            if (src) cls = parent_unsafe<STYLE>(a, rec.val) ? CLS_SAFE : CLS_INITIATOR;
            else cls = has_flag(rec.key) ? CLS_UNSAFE : CLS_SAFE;
            rec.key = without_flag(rec.key);
          }
          if (lvl == 0 || (split_word(kword(rec.key)) & mask) == sel) {
            slot = table_insert(tkey, T, tbits, rec.key, claimed);
            if (slot < 0) {
              lfail = true;
            } else {
              add = true;
              vbits = rec.val;
              if (src) {
                // diagonal step of a source walker
                if (STYLE == STYLE_INTEGER) {
                  const int64_t v = (int64_t)rec.val;
                  const double x = op_diagonal<KIND>(a, r, rec.key) * i2d_exact(v);
                  const U4 rr = draw(a.seed, PURPOSE_DIAG, rep, step, kword(rec.key), 0);
                  const int64_t res = round_stochastic(x, u53_of(rr));
                  // clones_deaths_zombies (spawning.jl:79-93)
                  const int sr = (res > 0) - (res < 0), sv = (v > 0) - (v < 0);
                  if (res > v) pa.clones += res - v;
                  else if (sr != sv) { pa.deaths += v < 0 ? -v : v; pa.zombies += res < 0 ? -res : res; }
                  else pa.deaths += (res - v) < 0 ? v - res : res - v;
                  vbits = (uint64_t)res;
                } else {
                  vbits = dbits(diag_float<KIND>(a, r, rep, step, rec));
                }
              }
            }
          }
        }
        // one shared-memory atomic reserves the warp's contribution and occupied-slot entries
        const uint32_t madd = __ballot_sync(0xffffffffu, add);
        const uint32_t mcl = __ballot_sync(0xffffffffu, claimed);
        uint32_t base = 0;
        if (lane == 0 && (madd | mcl))
          base = atomicAdd(s_pack, (uint32_t)__popc(madd) | ((uint32_t)__popc(mcl) << 16));
        base = __shfl_sync(0xffffffffu, base, 0);
        const uint32_t lt = lanemask_lt();
        if (add) {
          const uint32_t c = (base & 0xffffu) + (uint32_t)__popc(madd & lt);
          if (c < T) {
            cval[c] = vbits;
            const uint32_t old = atomicExch(&thead[slot], c);
            clink[c] = (uint16_t)((old == NIL ? LINK_END : old) | ((uint32_t)cls << 13) |
                                  (src ? 0x8000u : 0u));
          } else {
            lfail = true;
          }
        }
        if (claimed) {
          const uint32_t pos = ((base >> 16) & 0x7fffu) + (uint32_t)__popc(mcl & lt);
          if (pos < T) slist[pos] = (uint16_t)slot;
        }
        if (__any_sync(0xffffffffu, lfail)) { if (lane == 0) atomicOr(s_pack, PACK_FAIL); break; }
      }
      __syncthreads();
      const uint32_t pk = *s_pack;
      const bool fail = (pk >> 31) != 0;
      const uint32_t nslots = ((pk >> 16) & 0x7fffu) < T ? ((pk >> 16) & 0x7fffu) : T;
      const uint32_t ncon = (pk & 0xffffu) < T ? (pk & 0xffffu) : T;
      // the other parity's counters were last read before the previous pass ended
      if (tid < 4) s_cnt[par ^ 1][tid] = 0;
      if (fail) {
        for (uint32_t i = tid; i < nslots; i += ANN_THREADS) {
          const int slot = slist[i];
          tkey[slot] = EMPTY; thead[slot] = NIL;
        }
      } else {
        // ---- finalize: exact sum, compression threshold, statistics, output ----
        // Float addresses with one or two contributions are finished here; the others (and
        // every address under an initiator rule) go to a second list, finished by full warps
        // after the next barrier, so that the short common case does not wait for them.
        for (uint32_t i0 = (uint32_t)w * 32; i0 < nslots; i0 += ANN_THREADS) {
          const uint32_t i = i0 + lane;
          bool keep = false, queue = false, slow = false;
          K key = KT<K>::from(0);
          uint64_t vb = 0;
          int slot = 0;
          uint32_t head = NIL;
          if (i < nslots) {
            slot = slist[i];
            key = tkey[slot];
            head = thead[slot];
            if (STYLE == STYLE_INTEGER) {
              uint32_t steps = 0;
              int64_t iv = 0, part[3] = {0, 0, 0};
              for (uint32_t c = head; c != NIL; c = link_next(clink[c])) {
                if (c >= ncon || ++steps > ncon) { bad = true; break; }
                const uint16_t lw = clink[c];
                const int64_t k = (int64_t)cval[c];
                iv += k;
                part[link_cls(lw) < 3 ? link_cls(lw) : 0] += k;
                if (!link_diag(lw)) { acc.records++; acc.spawns_i += k < 0 ? -k : k; }
              }
              if (a.init_rule)
                iv = initiator_value_i(a.init_rule, a.init_thr, part[CLS_SAFE], part[CLS_UNSAFE],
                                       part[CLS_INITIATOR]);
              if (iv != 0) {
                acc.len_before++;
                keep = true;
                vb = (uint64_t)iv;
                const uint64_t mag = (uint64_t)(iv < 0 ? -iv : iv);
                account_kept<STYLE>(a, r, key, i2d_exact(iv), U128{0, mag}, acc);
              }
            } else {
              const uint16_t w0 = head < ncon ? clink[head] : (uint16_t)LINK_END;
              const uint32_t c1 = link_next(w0);
              if (!a.init_rule && head < ncon && (c1 == NIL || (c1 < ncon && link_next(clink[c1]) == NIL))) {
                // One or two contributions: a single IEEE addition is correctly rounded, so
                // it equals both the exact fixed-point sum and the canonical-order sum.
                const double y0 = bitsd(cval[head]);
                if (!link_diag(w0)) { acc.records++; acc.spawn_fx = add128(acc.spawn_fx, fixed_of(abs_d(y0))); }
                double fv = y0;
                if (c1 != NIL) {
                  const double y1 = bitsd(cval[c1]);
                  if (!link_diag(clink[c1])) { acc.records++; acc.spawn_fx = add128(acc.spawn_fx, fixed_of(abs_d(y1))); }
                  fv = __dadd_rn(y0, y1);
                }
                vb = dbits(fv);
                if (!is_zero_d(fv)) {
                  acc.len_before++;
                  const bool small = below_threshold(a, fv);
                  if (small) {
                    queue = true;
                  } else {
                    keep = true;
                    account_kept<STYLE>(a, r, key, fv, fixed_of(abs_d(fv)), acc);
                  }
                }
              } else {
                slow = true;
              }
            }
          }
          const uint32_t pos = warp_append(&s_out, keep);
          if (keep && pos < a.capv) vout[pos] = RecT<K>{key, vb};
          if (STYLE != STYLE_INTEGER) {
            // compression queue from the bottom of qlist, second list from the top
            const uint32_t q = warp_append(s_nq, queue);
            if (queue) {
              qlist[q] = (uint16_t)slot;
              cval[head] = vb;          // the list was read above: its head keeps the value
            }
            const uint32_t sl = warp_append(s_nslow, slow);
            if (slow) qlist[T - 1 - sl] = (uint16_t)slot;
          }
          if (i < nslots && !queue && !slow) { tkey[slot] = EMPTY; thead[slot] = NIL; }
        }
        if (STYLE != STYLE_INTEGER) {
          __syncthreads();
          const uint32_t nq = *s_nq, nslow = *s_nslow;
          // ---- addresses with three or more contributions ----
          for (uint32_t i0 = (uint32_t)w * 32; i0 < nslow; i0 += ANN_THREADS) {
            const uint32_t i = i0 + lane;
            bool keep = false;
            K key = KT<K>::from(0);
            uint64_t vb = 0;
            if (i < nslow && nq + i < T) {
              const int slot = qlist[T - 1 - i];
              key = tkey[slot];
              uint32_t head = thead[slot];
              tkey[slot] = EMPTY; thead[slot] = NIL;
              double fv;
              if (a.init_rule) {
                fv = initiator_sum_f(a, head, cval, clink, ncon, acc, &bad);
              } else {
                U128 sum{0, 0};
                bool exact = true, have_d = false;
                double first = 0.0;
                uint32_t steps = 0;
                for (uint32_t c = head; c != NIL; c = link_next(clink[c])) {
                  if (c >= ncon || ++steps > ncon) { bad = true; break; }
                  const uint64_t v = cval[c];
                  U128 m;
                  const bool ex = fixed_magnitude(bitsd(v), m);
                  if (link_diag(clink[c])) {
                    have_d = true;
                    first = bitsd(v);
                  } else {
                    acc.records++;
                    acc.spawn_fx = add128(acc.spawn_fx, ex ? m : fixed_of(abs_d(bitsd(v))));
                  }
                  exact = exact && ex;
                  sum = add128(sum, (v >> 63) ? neg128(m) : m);
                }
                if (exact) {
                  fv = signed_fixed_to_double(sum);
                } else {
                  fv = canonical_sum_list(have_d && !is_zero_d(first), first, head, cval, clink,
                                          ncon, &bad);
                }
              }
              if (!is_zero_d(fv)) {
                acc.len_before++;
                const bool small = below_threshold(a, fv);
                if (small) {
                  keep = compress_draw<STYLE>(a, r, step, key, fv);
                  if (keep) { acc.ncomp++; account_entry<STYLE>(a, r, key, fv, acc); }
                } else {
                  keep = true;
                  account_kept<STYLE>(a, r, key, fv, fixed_of(abs_d(fv)), acc);
                }
              }
              vb = dbits(fv);
            }
            const uint32_t pos = warp_append(&s_out, keep);
            if (keep && pos < a.capv) vout[pos] = RecT<K>{key, vb};
          }
          // ---- compression draws of the queued addresses, on full warps ----
          for (uint32_t i0 = (uint32_t)w * 32; i0 < nq; i0 += ANN_THREADS) {
            const uint32_t i = i0 + lane;
            bool keep = false;
            K key = KT<K>::from(0);
            double fv = 0.0;
            if (i < nq) {
              const int slot = qlist[i];
              key = tkey[slot];
              fv = bitsd(cval[thead[slot]]);
              tkey[slot] = EMPTY; thead[slot] = NIL;
              keep = compress_draw<STYLE>(a, r, step, key, fv);
              if (keep) { acc.ncomp++; account_entry<STYLE>(a, r, key, fv, acc); }
            }
            const uint32_t pos = warp_append(&s_out, keep);
            if (keep && pos < a.capv) vout[pos] = RecT<K>{key, dbits(fv)};
          }
        }
        acc.clones += pa.clones; acc.deaths += pa.deaths; acc.zombies += pa.zombies;
      }
      __syncthreads();
      par ^= 1;
      if (fail) {
        if (lvl >= MAX_SPLIT) { bad = true; break; }
        ++lvl;                       // first half of this pass: split bit lvl-1 clear
        continue;
      }
      // next pass: depth first over the splits
      while (lvl > lvl0 && ((sel >> (lvl - 1)) & 1ull)) { sel &= ~(1ull << (lvl - 1)); --lvl; }
      if (lvl == lvl0) {
        if (++sel >= (1ull << lvl0)) break;
      } else {
        sel |= 1ull << (lvl - 1);
      }
    }
    if (tid == 0) {
      const uint32_t out = s_out;
      s_out = 0;                     // next used after the next bucket's first barrier
      a.cnt_out[gb] = out < a.capv ? out : a.capv;
      if (out > a.capv) atomicOr(&a.stats[r].flags, (unsigned)FLAG_V_OVERFLOW);
      if (nsp > a.caps) atomicOr(&a.stats[r].flags, (unsigned)FLAG_SPAWN_OVERFLOW);
      atomicMax(&a.stats[r].max_v_bucket, out);
      atomicMax(&a.stats[r].max_spawn_bucket, nsp);
      a.scount[gb] = 0;
    }
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0)
    atomicOr(&a.stats[cur_r < 0 ? 0 : cur_r].flags, (unsigned)FLAG_TABLE);
  if (cur_r >= 0) flush_ann_acc(a, cur_r, acc);
}

// ------------------------------------------------------------------------------------------
// Annihilation, one warp per bucket
// ------------------------------------------------------------------------------------------
// The common case.  One warp annihilates one bucket in a table of its own in shared memory,
// so no warp ever waits for another (k_annihilate's CTA barriers were its main stall).  Only
// the spawns go into the table: each address's spawns on a list.  The source walkers, whose
// addresses are distinct, then stream past it: each takes its diagonal step, looks its
// address up (a read, no atomics), adds the spawns found there and is written out, and the
// addresses that only spawns reached are finished last.  Same arithmetic as k_annihilate (the
// summation rule, compression, statistics, ProjectedEnergy terms), for one-word addresses
// without an initiator rule.  A bucket with more than AW_SCAP spawns is appended to ann_list
// and left to k_annihilate, launched after this kernel.
constexpr int AW_WARPS = 4;              // warps per CTA
constexpr int AW_SLOTS = AW_CAP;         // table slots per warp
constexpr int AW_SCAP = AW_CAP * 3 / 4;  // spawns per bucket
constexpr int AW_TBITS = AW_CAP == 256 ? 8 : AW_CAP == 512 ? 9 : 10;   // log2 of the table slots
static_assert((1 << AW_TBITS) == AW_SLOTS, "AW_CAP must be 256, 512 or 1024");
constexpr uint32_t AW_DONE = 0x80000000u;   // list head flag: a source walker took the slot
// per warp: keys [AW_SLOTS] u64, list heads [AW_SLOTS] u32, spawn values [AW_SCAP] u64, spawn
// links [AW_SCAP] u16 (the k_annihilate link word), occupied-slot list [AW_SCAP] u16
constexpr size_t AW_WARP_SMEM = (size_t)AW_SLOTS * (8 + 4) + (size_t)AW_SCAP * (8 + 2 + 2);
// resident CTAs per SM that the shared memory allows (at most 8)
constexpr int AW_MINB = (int)((220 * 1024) / (AW_WARPS * AW_WARP_SMEM)) > 8 ? 8
                        : (int)((220 * 1024) / (AW_WARPS * AW_WARP_SMEM));

__device__ __forceinline__ double warp_sum_long(uint32_t head, bool have_d, double dv,
                                                const uint64_t *cval, uint16_t *clink, uint32_t n,
                                                AnnAcc &acc, bool *bad);

// Sum of the spawns on the list at `head` (n entries at most) and of the diagonal term dv
// (when have_d) by the summation rule; counts the spawn statistics.
template <int STYLE>
__device__ __forceinline__ double warp_sum_float(uint32_t head, bool have_d, double dv,
                                                 const uint64_t *cval, uint16_t *clink,
                                                 uint32_t n, AnnAcc &acc, bool *bad) {
  const uint16_t w0 = clink[head];
  const uint32_t c1 = link_next(w0);
  const double y0 = bitsd(cval[head]);
  acc.records++;
  acc.spawn_fx = add128(acc.spawn_fx, fixed_of(abs_d(y0)));
  if (c1 == NIL && !have_d) return y0;
  if (c1 == NIL) return __dadd_rn(dv, y0);     // two terms: one correctly rounded addition
  const uint16_t w1 = clink[c1];
  if (!have_d && link_next(w1) == NIL) {
    const double y1 = bitsd(cval[c1]);
    acc.records++;
    acc.spawn_fx = add128(acc.spawn_fx, fixed_of(abs_d(y1)));
    return __dadd_rn(y0, y1);
  }
  return warp_sum_long(head, have_d, dv, cval, clink, n, acc, bad);
}

// Three or more terms: exact in fixed point when every term allows it, else canonical order.
__device__ __forceinline__ double warp_sum_long(uint32_t head, bool have_d, double dv,
                                                const uint64_t *cval, uint16_t *clink, uint32_t n,
                                                AnnAcc &acc, bool *bad) {
  U128 sum{0, 0}, m;
  bool exact = true;
  if (have_d) {
    exact = fixed_magnitude(dv, m);
    sum = is_neg_d(dv) ? neg128(m) : m;
  }
  uint32_t steps = 0;
  for (uint32_t c = head; c != NIL; c = link_next(clink[c])) {
    if (c >= n || ++steps > n) { *bad = true; break; }
    const uint64_t v = cval[c];
    const bool ex = fixed_magnitude(bitsd(v), m);
    if (c != head) {
      acc.records++;
      acc.spawn_fx = add128(acc.spawn_fx, ex ? m : fixed_of(abs_d(bitsd(v))));
    }
    exact = exact && ex;
    sum = add128(sum, (v >> 63) ? neg128(m) : m);
  }
  if (exact) return signed_fixed_to_double(sum);
  uint32_t h = head;
  return canonical_sum_list(have_d, dv, h, cval, clink, n, bad);
}

// Compression (compression.jl:18-42), statistics and ProjectedEnergy terms of one summed
// address; whether it is kept (fv then holds its value).
template <int STYLE>
__device__ __forceinline__ bool warp_settle_float(const StepArgs &a, int r, uint32_t step,
                                                  uint64_t key, double &fv, AnnAcc &acc) {
  if (is_zero_d(fv)) return false;
  acc.len_before++;
  if (below_threshold(a, fv)) {
    if (!compress_draw<STYLE>(a, r, step, key, fv)) return false;
    acc.ncomp++;
    account_entry<STYLE>(a, r, key, fv, acc);
    return true;
  }
  account_kept<STYLE>(a, r, key, fv, fixed_of(abs_d(fv)), acc);
  return true;
}

template <int KIND, int STYLE>
__global__ void __launch_bounds__(AW_WARPS * 32, AW_MINB) k_ann_warp(StepArgs a, int nb_total) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned char *base = smem + (size_t)w * AW_WARP_SMEM;
  uint64_t *tkey = reinterpret_cast<uint64_t *>(base);
  uint64_t *cval = tkey + AW_SLOTS;
  uint32_t *thead = reinterpret_cast<uint32_t *>(cval + AW_SCAP);
  uint16_t *clink = reinterpret_cast<uint16_t *>(thead + AW_SLOTS);
  uint16_t *slist = clink + AW_SCAP;
  for (int i = lane; i < AW_SLOTS; i += 32) { tkey[i] = EMPTY_KEY; thead[i] = NIL; }
  __syncwarp();
  const uint32_t lt = lanemask_lt();
  const uint32_t step = step_of(a);
  AnnAcc acc{};
  int cur_r = -1;
  bool bad = false;
  for (int gb = blockIdx.x * AW_WARPS + w; gb < nb_total; gb += gridDim.x * AW_WARPS) {
    const int r = replica_of(a, (uint32_t)gb);
    if (r != cur_r) {
      if (cur_r >= 0) flush_ann_acc(a, cur_r, acc);
      cur_r = r;
    }
    const uint32_t rep = a.replica_base + (uint32_t)r;
    const uint32_t nsp = a.scount[gb];
    const uint32_t ns = nsp < a.caps ? nsp : a.caps;
    const uint32_t nv0 = a.cnt_in[gb];
    const uint32_t nv = nv0 < a.capv_in ? nv0 : a.capv_in;
    if (ns > (uint32_t)AW_SCAP) {               // for k_annihilate
      if (lane == 0) {
        const uint32_t idx = atomicAdd(a.ann_count, 1u);
        if (idx < (uint32_t)nb_total) a.ann_list[idx] = (uint32_t)gb;
      }
      continue;
    }
    const Rec *sp = static_cast<const Rec *>(a.spawn) + (size_t)gb * a.caps;
    const Rec *vbase = static_cast<const Rec *>(a.v_in) + (size_t)gb * a.capv_in;
    Rec *vout = static_cast<Rec *>(a.v_out) + (size_t)gb * a.capv;
    // the first source records are loaded while the spawns go into the table, and each round
    // of spawns while the previous one is inserted
    Rec nxt{}, snxt{};
    if ((uint32_t)lane < nv) nxt = vbase[lane];
    if ((uint32_t)lane < ns) snxt = sp[lane];
    // ---- the spawns, each onto the list of its address ----
    uint32_t nsl = 0;
    for (uint32_t f0 = 0; f0 < ns; f0 += 32) {
      const uint32_t f = f0 + lane;
      const bool add = f < ns;
      const Rec rec = snxt;
      if (f + 32 < ns) snxt = sp[f + 32];
      int slot = -1;
      bool claimed = false;
      if (add) {
        uint32_t sl = (uint32_t)((rec.key * 0x9E3779B97F4A7C15ull) >> (64 - AW_TBITS));
        for (int p = 0; p < AW_SLOTS; ++p) {
          const uint64_t k = *(volatile uint64_t *)&tkey[sl];
          if (k == rec.key) { slot = (int)sl; break; }
          if (k == EMPTY_KEY) {
            const unsigned long long old = atomicCAS((unsigned long long *)&tkey[sl],
                                                     (unsigned long long)EMPTY_KEY,
                                                     (unsigned long long)rec.key);
            if (old == EMPTY_KEY) { slot = (int)sl; claimed = true; break; }
            if (old == rec.key) { slot = (int)sl; break; }
          }
          sl = (sl + 1) & (AW_SLOTS - 1);
        }
        if (slot < 0) bad = true;                // cannot happen: slots > spawns
        else {
          cval[f] = rec.val;
          const uint32_t old = atomicExch(&thead[slot], f);
          clink[f] = (uint16_t)(old == NIL ? LINK_END : old);
        }
      }
      const uint32_t mcl = __ballot_sync(0xffffffffu, claimed);
      if (claimed) slist[nsl + (uint32_t)__popc(mcl & lt)] = (uint16_t)slot;
      nsl += (uint32_t)__popc(mcl);
    }
    __syncwarp();
    // ---- the source walkers (diagonal step, lookup, the spawns found there), then the
    // addresses only spawns reached: one loop over both, so the summing and settling code
    // appears once in the kernel.  The slots start on a fresh round, after every source has
    // marked the slot it took.
    uint32_t out = 0;
    const uint32_t nvr = (nv + 31u) & ~31u;
    for (uint32_t f0 = 0; f0 < nvr + nsl; f0 += 32) {
      const uint32_t f = f0 + lane;
      const bool is_src = f0 < nvr;
      Rec rec{};
      if (is_src) {
        rec = nxt;
        if (f + 32 < nv) nxt = vbase[f + 32];
      }
      bool keep = false, item = false, have_d = false;
      uint64_t key = 0, vb = 0;
      uint32_t head = NIL;
      double dv = 0.0;
      int64_t iv = 0;
      if (is_src && f < nv) {
        item = true;
        key = rec.key;
        int slot = -1;
        if (ns) {
          uint32_t sl = (uint32_t)((key * 0x9E3779B97F4A7C15ull) >> (64 - AW_TBITS));
          for (int p = 0; p < AW_SLOTS; ++p) {
            const uint64_t k = tkey[sl];
            if (k == key) { slot = (int)sl; break; }
            if (k == EMPTY_KEY) break;
            sl = (sl + 1) & (AW_SLOTS - 1);
          }
        }
        if (slot >= 0) { head = thead[slot]; thead[slot] = head | AW_DONE; }
        if (STYLE == STYLE_INTEGER) {
          const int64_t v = (int64_t)rec.val;
          const double x = op_diagonal<KIND>(a, r, key) * i2d_exact(v);
          const U4 rr = draw(a.seed, PURPOSE_DIAG, rep, step, key, 0);
          iv = round_stochastic(x, u53_of(rr));
          // clones_deaths_zombies (spawning.jl:79-93)
          const int sr = (iv > 0) - (iv < 0), sv = (v > 0) - (v < 0);
          if (iv > v) acc.clones += iv - v;
          else if (sr != sv) { acc.deaths += v < 0 ? -v : v; acc.zombies += iv < 0 ? -iv : iv; }
          else acc.deaths += (iv - v) < 0 ? v - iv : iv - v;
        } else {
          dv = diag_float<KIND>(a, r, rep, step, rec);
          have_d = !is_zero_d(dv);
        }
      } else if (!is_src && f - nvr < nsl) {
        const int slot = slist[f - nvr];
        key = tkey[slot];
        head = thead[slot];
        tkey[slot] = EMPTY_KEY;
        thead[slot] = NIL;
        item = !(head & AW_DONE);
      }
      if (item) {
        if (STYLE == STYLE_INTEGER) {
          uint32_t steps = 0;
          for (uint32_t c = head; c != NIL; c = link_next(clink[c])) {
            if (c >= ns || ++steps > ns) { bad = true; break; }
            const int64_t k = (int64_t)cval[c];
            iv += k;
            acc.records++;
            acc.spawns_i += k < 0 ? -k : k;
          }
          if (iv != 0) {
            acc.len_before++;
            keep = true;
            vb = (uint64_t)iv;
            account_kept<STYLE>(a, r, key, i2d_exact(iv), U128{0, (uint64_t)(iv < 0 ? -iv : iv)}, acc);
          }
        } else {
          double fv = head == NIL ? dv
                                  : warp_sum_float<STYLE>(head, have_d, dv, cval, clink, ns, acc, &bad);
          keep = warp_settle_float<STYLE>(a, r, step, key, fv, acc);
          vb = dbits(fv);
        }
      }
      const uint32_t mk = __ballot_sync(0xffffffffu, keep);
      const uint32_t pos = out + (uint32_t)__popc(mk & lt);
      if (keep && pos < a.capv) vout[pos] = Rec{key, vb};
      out += (uint32_t)__popc(mk);
      if (f0 + 32 == nvr) __syncwarp();          // the sources' marks, before the slot rounds
    }
    __syncwarp();
    if (lane == 0) {
      a.cnt_out[gb] = out < a.capv ? out : a.capv;
      if (out > a.capv) atomicOr(&a.stats[r].flags, (unsigned)FLAG_V_OVERFLOW);
      if (nsp > a.caps) atomicOr(&a.stats[r].flags, (unsigned)FLAG_SPAWN_OVERFLOW);
      atomicMax(&a.stats[r].max_v_bucket, out);
      atomicMax(&a.stats[r].max_spawn_bucket, nsp);
      a.scount[gb] = 0;
    }
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0)
    atomicOr(&a.stats[cur_r < 0 ? 0 : cur_r].flags, (unsigned)FLAG_TABLE);
  if (cur_r >= 0) flush_ann_acc(a, cur_r, acc);
}

// ------------------------------------------------------------------------------------------
// Sorting instead of hashing: the work of k_ann_warp with the bucket's spawns ordered in
// shared memory by a bitonic network on (address, value) -- for float walkers the value's
// order-preserving bits, so that each address's spawns stand in the canonical summation order
// and no list is ever sorted.  The runs of equal addresses take the place of the table's
// lists: a source walker finds its run by binary search and marks it taken, and the runs no
// source took are finished in the second part of the same loop.  Same buckets, same results
// bit for bit; which of the two is faster is measured (rimu_wm_set_annihilation and the
// batched autotuner choose).
constexpr int AS_P = 512;                       // sort width: a power of two >= AW_SCAP
static_assert(AS_P >= AW_SCAP && (AS_P & (AS_P - 1)) == 0, "sort width");
// per warp: records [AS_P] 16 B (address, value bits), run heads [AW_SCAP] u16, taken flags
// [AS_P] u8
constexpr size_t AS_WARP_SMEM = (size_t)AS_P * 16 + (size_t)AW_SCAP * 2 + (size_t)AS_P;
constexpr int AS_MINB = (int)((220 * 1024) / (AW_WARPS * AS_WARP_SMEM)) > 8 ? 8
                        : (int)((220 * 1024) / (AW_WARPS * AS_WARP_SMEM));

// Sorts s[0, p) ascending by (x, y) (by x alone when !BY_VALUE), p a power of two >= 2: one
// warp, p / 64 compare-exchanges per lane and stage.
template <bool BY_VALUE>
__device__ __forceinline__ void warp_bitonic(ulonglong2 *s, uint32_t p, int lane) {
  for (uint32_t k = 2; k <= p; k <<= 1) {
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      for (uint32_t i = (uint32_t)lane; i < p / 2; i += 32) {
        const uint32_t lo = ((i & ~(j - 1)) << 1) | (i & (j - 1));
        const uint32_t hi = lo + j;
        const ulonglong2 x = s[lo], y = s[hi];
        const bool gt = x.x > y.x || (BY_VALUE && x.x == y.x && x.y > y.y);
        if (gt == ((lo & k) == 0)) { s[lo] = y; s[hi] = x; }
      }
      __syncwarp();
    }
  }
}

// Sum of the run of spawns at s[seg..] (address key, canonical order, order-preserving value
// bits) and of the diagonal term dv (when have_d) by the summation rule; counts the spawn
// statistics.  Three or more terms: exact in fixed point when every term allows it, else in
// the run's order after the diagonal term.
__device__ double run_sum_long(uint32_t seg, uint32_t ns, uint64_t key, bool have_d, double dv,
                               const ulonglong2 *s, AnnAcc &acc) {
  U128 sum{0, 0}, m;
  bool exact = true;
  if (have_d) {
    exact = fixed_magnitude(dv, m);
    sum = is_neg_d(dv) ? neg128(m) : m;
  }
  uint32_t c = seg;
  for (; c < ns && s[c].x == key; ++c) {
    const double v = from_ordered(s[c].y);
    const bool ex = fixed_magnitude(v, m);
    if (c != seg) {
      acc.records++;
      acc.spawn_fx = add128(acc.spawn_fx, ex ? m : fixed_of(abs_d(v)));
    }
    exact = exact && ex;
    sum = add128(sum, is_neg_d(v) ? neg128(m) : m);
  }
  if (exact) return signed_fixed_to_double(sum);
  double t = have_d ? dv : from_ordered(s[seg].y);
  for (uint32_t d = have_d ? seg : seg + 1; d < c; ++d) t = t + from_ordered(s[d].y);
  return t;
}
__device__ __forceinline__ double run_sum_float(uint32_t seg, uint32_t ns, uint64_t key,
                                                bool have_d, double dv, const ulonglong2 *s,
                                                AnnAcc &acc) {
  const double y0 = from_ordered(s[seg].y);
  acc.records++;
  acc.spawn_fx = add128(acc.spawn_fx, fixed_of(abs_d(y0)));
  const bool one = seg + 1 >= ns || s[seg + 1].x != key;
  if (one) return have_d ? __dadd_rn(dv, y0) : y0;
  if (!have_d && (seg + 2 >= ns || s[seg + 2].x != key)) {
    const double y1 = from_ordered(s[seg + 1].y);
    acc.records++;
    acc.spawn_fx = add128(acc.spawn_fx, fixed_of(abs_d(y1)));
    return __dadd_rn(y0, y1);
  }
  return run_sum_long(seg, ns, key, have_d, dv, s, acc);
}

template <int KIND, int STYLE>
__global__ void __launch_bounds__(AW_WARPS * 32, AS_MINB) k_ann_sort(StepArgs a, int nb_total) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned char *base = smem + (size_t)w * AS_WARP_SMEM;
  ulonglong2 *srec = reinterpret_cast<ulonglong2 *>(base);
  uint16_t *hlist = reinterpret_cast<uint16_t *>(srec + AS_P);
  uint8_t *taken = reinterpret_cast<uint8_t *>(hlist + AW_SCAP);
  const uint32_t lt = lanemask_lt();
  const uint32_t step = step_of(a);
  AnnAcc acc{};
  int cur_r = -1;
  for (int gb = blockIdx.x * AW_WARPS + w; gb < nb_total; gb += gridDim.x * AW_WARPS) {
    const int r = replica_of(a, (uint32_t)gb);
    if (r != cur_r) {
      if (cur_r >= 0) flush_ann_acc(a, cur_r, acc);
      cur_r = r;
    }
    const uint32_t rep = a.replica_base + (uint32_t)r;
    const uint32_t nsp = a.scount[gb];
    const uint32_t ns = nsp < a.caps ? nsp : a.caps;
    const uint32_t nv0 = a.cnt_in[gb];
    const uint32_t nv = nv0 < a.capv_in ? nv0 : a.capv_in;
    if (ns > (uint32_t)AW_SCAP) {               // for k_annihilate
      if (lane == 0) {
        const uint32_t idx = atomicAdd(a.ann_count, 1u);
        if (idx < (uint32_t)nb_total) a.ann_list[idx] = (uint32_t)gb;
      }
      continue;
    }
    const Rec *sp = static_cast<const Rec *>(a.spawn) + (size_t)gb * a.caps;
    const Rec *vbase = static_cast<const Rec *>(a.v_in) + (size_t)gb * a.capv_in;
    Rec *vout = static_cast<Rec *>(a.v_out) + (size_t)gb * a.capv;
    Rec nxt{};
    if ((uint32_t)lane < nv) nxt = vbase[lane];
    // ---- the spawns, padded to a power of two with keys that sort last, then sorted ----
    uint32_t p = 2;
    while (p < ns) p <<= 1;
    for (uint32_t f = (uint32_t)lane; f < p; f += 32) {
      ulonglong2 e{EMPTY_KEY, ~0ull};
      if (f < ns) {
        const Rec rec = sp[f];
        e.x = rec.key;
        e.y = STYLE == STYLE_INTEGER ? rec.val : ordered_bits(bitsd(rec.val));
      }
      srec[f] = e;
      taken[f] = 0;
    }
    __syncwarp();
    if (ns > 1) warp_bitonic<STYLE != STYLE_INTEGER>(srec, p, lane);
    // ---- run heads ----
    uint32_t nsl = 0;
    for (uint32_t f0 = 0; f0 < ns; f0 += 32) {
      const uint32_t f = f0 + (uint32_t)lane;
      const bool h = f < ns && (f == 0 || srec[f].x != srec[f - 1].x);
      const uint32_t m = __ballot_sync(0xffffffffu, h);
      if (h) hlist[nsl + (uint32_t)__popc(m & lt)] = (uint16_t)f;
      nsl += (uint32_t)__popc(m);
    }
    __syncwarp();
    // ---- the source walkers, then the runs no source took (as in k_ann_warp) ----
    uint32_t out = 0;
    const uint32_t nvr = (nv + 31u) & ~31u;
    for (uint32_t f0 = 0; f0 < nvr + nsl; f0 += 32) {
      const uint32_t f = f0 + (uint32_t)lane;
      const bool is_src = f0 < nvr;
      Rec rec{};
      if (is_src) {
        rec = nxt;
        if (f + 32 < nv) nxt = vbase[f + 32];
      }
      bool keep = false, item = false, have_d = false;
      uint64_t key = 0, vb = 0;
      uint32_t seg = NIL;
      double dv = 0.0;
      int64_t iv = 0;
      if (is_src && f < nv) {
        item = true;
        key = rec.key;
        if (ns) {
          uint32_t lo = 0, n = ns;               // lower bound of key among the spawns
          while (n > 0) {
            const uint32_t h = n >> 1;
            if (srec[lo + h].x < key) { lo += h + 1; n -= h + 1; }
            else n = h;
          }
          if (lo < ns && srec[lo].x == key) { seg = lo; taken[lo] = 1; }
        }
        if (STYLE == STYLE_INTEGER) {
          const int64_t v = (int64_t)rec.val;
          const double x = op_diagonal<KIND>(a, r, key) * i2d_exact(v);
          const U4 rr = draw(a.seed, PURPOSE_DIAG, rep, step, key, 0);
          iv = round_stochastic(x, u53_of(rr));
          // clones_deaths_zombies (spawning.jl:79-93)
          const int sr = (iv > 0) - (iv < 0), sv = (v > 0) - (v < 0);
          if (iv > v) acc.clones += iv - v;
          else if (sr != sv) { acc.deaths += v < 0 ? -v : v; acc.zombies += iv < 0 ? -iv : iv; }
          else acc.deaths += (iv - v) < 0 ? v - iv : iv - v;
        } else {
          dv = diag_float<KIND>(a, r, rep, step, rec);
          have_d = !is_zero_d(dv);
        }
      } else if (!is_src && f - nvr < nsl) {
        seg = hlist[f - nvr];
        key = srec[seg].x;
        item = !taken[seg];
      }
      if (item) {
        if (STYLE == STYLE_INTEGER) {
          for (uint32_t c = seg; c < ns && srec[c].x == key; ++c) {
            const int64_t k = (int64_t)srec[c].y;
            iv += k;
            acc.records++;
            acc.spawns_i += k < 0 ? -k : k;
          }
          if (iv != 0) {
            acc.len_before++;
            keep = true;
            vb = (uint64_t)iv;
            account_kept<STYLE>(a, r, key, i2d_exact(iv), U128{0, (uint64_t)(iv < 0 ? -iv : iv)}, acc);
          }
        } else {
          double fv = seg == NIL ? dv : run_sum_float(seg, ns, key, have_d, dv, srec, acc);
          keep = warp_settle_float<STYLE>(a, r, step, key, fv, acc);
          vb = dbits(fv);
        }
      }
      const uint32_t mk = __ballot_sync(0xffffffffu, keep);
      const uint32_t pos = out + (uint32_t)__popc(mk & lt);
      if (keep && pos < a.capv) vout[pos] = Rec{key, vb};
      out += (uint32_t)__popc(mk);
      if (f0 + 32 == nvr) __syncwarp();          // the sources' marks, before the run rounds
    }
    __syncwarp();
    if (lane == 0) {
      a.cnt_out[gb] = out < a.capv ? out : a.capv;
      if (out > a.capv) atomicOr(&a.stats[r].flags, (unsigned)FLAG_V_OVERFLOW);
      if (nsp > a.caps) atomicOr(&a.stats[r].flags, (unsigned)FLAG_SPAWN_OVERFLOW);
      atomicMax(&a.stats[r].max_v_bucket, out);
      atomicMax(&a.stats[r].max_spawn_bucket, nsp);
      a.scount[gb] = 0;
    }
  }
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

// Walker-list kernels, on Rec (one-word addresses) or Rec2 (two-word addresses, K = Key128,
// host key arrays of (lo, hi) pairs).
template <class K>
__global__ void k_bucketize(const K *keys, const uint64_t *vals, int64_t n, int nb_bits,
                            uint32_t capv, RecT<K> *recs, uint32_t *count, unsigned int *flag) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const K k = keys[i];
  uint32_t b = bucket_of(k, nb_bits);
  uint32_t pos = atomicAdd(&count[b], 1u);
  if (pos < capv) recs[(size_t)b * capv + pos] = RecT<K>{k, vals[i]};
  else atomicOr(flag, (unsigned)FLAG_V_OVERFLOW);
}

template <class K>
__global__ void k_rebucket(const RecT<K> *old_recs, const uint32_t *old_count, int old_nb,
                           uint32_t old_capv, RecT<K> *recs, uint32_t *count, int nb_bits,
                           uint32_t capv, unsigned int *flag) {
  for (int gb = blockIdx.x; gb < old_nb; gb += gridDim.x) {
    uint32_t n = old_count[gb];
    for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
      RecT<K> rec = old_recs[(size_t)gb * old_capv + e];
      uint32_t b = bucket_of(rec.key, nb_bits);
      uint32_t pos = atomicAdd(&count[b], 1u);
      if (pos < capv) recs[(size_t)b * capv + pos] = rec;
      else atomicOr(flag, (unsigned)FLAG_V_OVERFLOW);
    }
  }
}

template <class K>
__global__ void k_compact(const RecT<K> *recs, const uint32_t *count, int nb, uint32_t capv,
                          const uint64_t *offsets, K *keys, uint64_t *vals) {
  for (int gb = blockIdx.x; gb < nb; gb += gridDim.x) {
    uint32_t n = count[gb];
    uint64_t o = offsets[gb];
    for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
      RecT<K> rec = recs[(size_t)gb * capv + e];
      keys[o + e] = rec.key;
      vals[o + e] = rec.val;
    }
  }
}

template <class K>
__global__ void k_norm(const RecT<K> *recs, const uint32_t *count, int nb, uint32_t capv,
                       int val_kind, unsigned long long *acc3) {
  U128 fx{0, 0};
  long long len = 0;
  for (int gb = blockIdx.x; gb < nb; gb += gridDim.x) {
    uint32_t n = count[gb];
    for (uint32_t e = threadIdx.x; e < n; e += blockDim.x) {
      const uint64_t val = recs[(size_t)gb * capv + e].val;
      double v = val_kind == RIMU_VAL_I64 ? (double)(int64_t)val : bitsd(val);
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

template <class K>
__global__ void k_lookup(const RecT<K> *recs, const uint32_t *count, int nb_bits, uint32_t capv,
                         const K *keys, int64_t n, uint64_t *vals, int *found) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const K k = keys[i];
  uint32_t b = bucket_of(k, nb_bits);
  uint32_t c = count[b];
  const RecT<K> *base = recs + (size_t)b * capv;
  vals[i] = 0;
  found[i] = 0;
  for (uint32_t e = 0; e < c; ++e) {
    if (base[e].key == k) { vals[i] = base[e].val; found[i] = 1; break; }
  }
}

template <int KIND, class K>
__global__ void k_diagonal(DevModel h, const K *keys, int64_t n, double *out) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) out[i] = model_diagonal<KIND>(h, keys[i]);
}

template <int KIND, class K>
__global__ void k_offdiagonals(DevModel h, K key, int noff, K *keys, double *vals) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= noff) return;
  OffdiagT<K> od = column_offdiag<KIND>(h, key, c + 1);
  keys[c] = od.key;
  double v = od.prod == 0 ? 0.0 : h.hoff[od.prod];
  vals[c] = od.sign < 0 ? -v : v;
}

// ------------------------------------------------------------------------------------------
// Launchers
// ------------------------------------------------------------------------------------------
template <int KIND, int STYLE, class K>
static int launch_step_t(rimu_ctx *ctx, const StepArgs &a_in, int nb_total, cudaEvent_t *ev) {
  cudaStream_t st = ctx->stream;
  // the warp kernels take one-word addresses only: other steps annihilate every bucket in
  // the CTA kernel with a table of tsize slots (the size its shared memory is launched with)
  StepArgs a = a_in;
  if constexpr (KT<K>::BITS != 64) {
    a.ann_list = nullptr;
    a.ann_count = nullptr;
  }
  const int cap = ctx->num_sms * 64;
  const int want_s = (nb_total / a.spawn_cb + WARPS - 1) / WARPS;
  const int grid_s = want_s < cap ? want_s : cap;
  const int cap_a = ctx->num_sms * 4;                 // resident annihilation CTAs
  const int grid = nb_total < cap_a ? nb_total : cap_a;
  if (ev) cudaEventRecord(ev[0], st);
  k_spawn<KIND, STYLE, K><<<grid_s, WARPS * 32, 0, st>>>(a, nb_total);
  if (ev) cudaEventRecord(ev[1], st);
  k_spawn_heavy<KIND, STYLE, K><<<ctx->num_sms * 4, 256, 0, st>>>(a);
  if (ev) cudaEventRecord(ev[2], st);
  static bool attr_set = false;
  if (!attr_set) {
    cudaFuncSetAttribute(k_annihilate<KIND, STYLE, K>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         200 * 1024);
    if constexpr (KT<K>::BITS == 64) {
      cudaFuncSetAttribute(k_ann_warp<KIND, STYLE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(AW_WARPS * AW_WARP_SMEM));
      cudaFuncSetAttribute(k_ann_sort<KIND, STYLE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)(AW_WARPS * AS_WARP_SMEM));
    }
    attr_set = true;
  }
  if constexpr (KT<K>::BITS == 64) {
    if (a.ann_list) {
      const int want_w = (nb_total + AW_WARPS - 1) / AW_WARPS;
      if (a.ann_sort) {
        const int cap_w = ctx->num_sms * AS_MINB;
        k_ann_sort<KIND, STYLE><<<want_w < cap_w ? want_w : cap_w, AW_WARPS * 32,
                                  AW_WARPS * AS_WARP_SMEM, st>>>(a, nb_total);
      } else {
        const int cap_w = ctx->num_sms * AW_MINB;
        k_ann_warp<KIND, STYLE><<<want_w < cap_w ? want_w : cap_w, AW_WARPS * 32,
                                  AW_WARPS * AW_WARP_SMEM, st>>>(a, nb_total);
      }
      // the buckets the warps left: as many CTAs as can be resident
      k_annihilate<KIND, STYLE, K><<<cap_a, ANN_THREADS, ann_smem<K>(a.tsize_list), st>>>(a, nb_total);
      if (ev) cudaEventRecord(ev[3], st);
      return rimu_cuda_check(cudaGetLastError(), "step kernels");
    }
  }
  k_annihilate<KIND, STYLE, K><<<grid, ANN_THREADS, ann_smem<K>(a.tsize), st>>>(a, nb_total);
  if (ev) cudaEventRecord(ev[3], st);
  return rimu_cuda_check(cudaGetLastError(), "step kernels");
}

template <int KIND, class K>
static int launch_step_k(rimu_ctx *ctx, const StepArgs &a, int nb_total, cudaEvent_t *ev) {
  switch (a.style) {
    case STYLE_INTEGER: return launch_step_t<KIND, STYLE_INTEGER, K>(ctx, a, nb_total, ev);
    case STYLE_DETERMINISTIC: return launch_step_t<KIND, STYLE_DETERMINISTIC, K>(ctx, a, nb_total, ev);
    default: return launch_step_t<KIND, STYLE_DSS, K>(ctx, a, nb_total, ev);
  }
}

}  // namespace rimu

using namespace rimu;

int rimu_launch_step(rimu_ctx *ctx, const StepArgs &a, int nb_total, cudaEvent_t *ev) {
  if (a.kw == 2) {   // two-word addresses: one-component models
    switch (a.h.kind) {
      case MODEL_REAL1D: return launch_step_k<MODEL_REAL1D, Key128>(ctx, a, nb_total, ev);
      case MODEL_REALSPACE: return launch_step_k<MODEL_REALSPACE, Key128>(ctx, a, nb_total, ev);
      default: return launch_step_k<MODEL_MOM1D, Key128>(ctx, a, nb_total, ev);
    }
  }
  switch (a.h.kind) {
    case MODEL_REAL1D: return launch_step_k<MODEL_REAL1D, uint64_t>(ctx, a, nb_total, ev);
    case MODEL_REALSPACE: return launch_step_k<MODEL_REALSPACE, uint64_t>(ctx, a, nb_total, ev);
    default: return launch_step_k<MODEL_MOM1D, uint64_t>(ctx, a, nb_total, ev);
  }
}

int rimu_launch_bucketize(rimu_ctx *ctx, const uint64_t *keys, const uint64_t *vals, int64_t n,
                          int nb_bits, uint32_t capv, void *recs, uint32_t *count,
                          unsigned int *flag, int kw) {
  if (n == 0) return 0;
  unsigned blocks = (unsigned)((n + 255) / 256);
  if (kw == 2)
    k_bucketize<<<blocks, 256, 0, ctx->stream>>>(reinterpret_cast<const Key128 *>(keys), vals, n,
                                                 nb_bits, capv, static_cast<Rec2 *>(recs), count, flag);
  else
    k_bucketize<<<blocks, 256, 0, ctx->stream>>>(keys, vals, n, nb_bits, capv,
                                                 static_cast<Rec *>(recs), count, flag);
  return rimu_cuda_check(cudaGetLastError(), "k_bucketize");
}

int rimu_launch_rebucket(rimu_ctx *ctx, const void *old_recs, const uint32_t *old_count,
                         int old_nb_bits, uint32_t old_capv, void *recs, uint32_t *count,
                         int nb_bits, uint32_t capv, unsigned int *flag, int kw) {
  int old_nb = 1 << old_nb_bits;
  int grid = old_nb < 65536 ? old_nb : 65536;
  if (kw == 2)
    k_rebucket<<<grid, 256, 0, ctx->stream>>>(static_cast<const Rec2 *>(old_recs), old_count, old_nb,
                                              old_capv, static_cast<Rec2 *>(recs), count, nb_bits,
                                              capv, flag);
  else
    k_rebucket<<<grid, 256, 0, ctx->stream>>>(static_cast<const Rec *>(old_recs), old_count, old_nb,
                                              old_capv, static_cast<Rec *>(recs), count, nb_bits,
                                              capv, flag);
  return rimu_cuda_check(cudaGetLastError(), "k_rebucket");
}

int rimu_launch_compact(rimu_ctx *ctx, const void *recs, const uint32_t *count, int nb,
                        uint32_t capv, const uint64_t *offsets, uint64_t *keys, uint64_t *vals,
                        int kw) {
  int grid = nb < 65536 ? nb : 65536;
  if (kw == 2)
    k_compact<<<grid, 256, 0, ctx->stream>>>(static_cast<const Rec2 *>(recs), count, nb, capv,
                                             offsets, reinterpret_cast<Key128 *>(keys), vals);
  else
    k_compact<<<grid, 256, 0, ctx->stream>>>(static_cast<const Rec *>(recs), count, nb, capv,
                                             offsets, keys, vals);
  return rimu_cuda_check(cudaGetLastError(), "k_compact");
}

int rimu_launch_norm(rimu_ctx *ctx, const void *recs, const uint32_t *count, int nb,
                     uint32_t capv, int val_kind, unsigned long long *acc3, int kw) {
  int grid = nb < ctx->num_sms * 8 ? nb : ctx->num_sms * 8;
  if (kw == 2)
    k_norm<<<grid, 256, 0, ctx->stream>>>(static_cast<const Rec2 *>(recs), count, nb, capv,
                                          val_kind, acc3);
  else
    k_norm<<<grid, 256, 0, ctx->stream>>>(static_cast<const Rec *>(recs), count, nb, capv,
                                          val_kind, acc3);
  return rimu_cuda_check(cudaGetLastError(), "k_norm");
}

int rimu_launch_lookup(rimu_ctx *ctx, const void *recs, const uint32_t *count, int nb_bits,
                       uint32_t capv, const uint64_t *keys, int64_t n, uint64_t *vals,
                       int *found, int kw) {
  if (n == 0) return 0;
  const unsigned g = (unsigned)((n + 127) / 128);
  if (kw == 2)
    k_lookup<<<g, 128, 0, ctx->stream>>>(static_cast<const Rec2 *>(recs), count, nb_bits, capv,
                                         reinterpret_cast<const Key128 *>(keys), n, vals, found);
  else
    k_lookup<<<g, 128, 0, ctx->stream>>>(static_cast<const Rec *>(recs), count, nb_bits, capv,
                                         keys, n, vals, found);
  return rimu_cuda_check(cudaGetLastError(), "k_lookup");
}

int rimu_launch_diag_table(rimu_ctx *ctx, const DevModel &h, int op, double dt,
                           const double *shift, int nrep, int ndiag, double *dtab) {
  int n = nrep * ndiag;
  k_diag_table<<<(n + 255) / 256, 256, 0, ctx->stream>>>(h, op, dt, shift, nrep, ndiag, dtab);
  return rimu_cuda_check(cudaGetLastError(), "k_diag_table");
}

// Diagonal elements of n addresses; with an address wider than 64 bits (h.nbits > 64) the
// keys are (lo, hi) pairs, 2n words.
int rimu_launch_diagonal(rimu_ctx *ctx, const DevModel &h, const uint64_t *keys, int64_t n,
                         double *out) {
  if (n == 0) return 0;
  unsigned g = (unsigned)((n + 255) / 256);
  if (h.nbits > 64) {
    const Key128 *k2 = reinterpret_cast<const Key128 *>(keys);
    if (h.kind == MODEL_REAL1D) k_diagonal<MODEL_REAL1D><<<g, 256, 0, ctx->stream>>>(h, k2, n, out);
    else if (h.kind == MODEL_REALSPACE) k_diagonal<MODEL_REALSPACE><<<g, 256, 0, ctx->stream>>>(h, k2, n, out);
    else k_diagonal<MODEL_MOM1D><<<g, 256, 0, ctx->stream>>>(h, k2, n, out);
    return rimu_cuda_check(cudaGetLastError(), "k_diagonal");
  }
  switch (h.kind) {
    case MODEL_REAL1D: k_diagonal<MODEL_REAL1D><<<g, 256, 0, ctx->stream>>>(h, keys, n, out); break;
    case MODEL_REALSPACE: k_diagonal<MODEL_REALSPACE><<<g, 256, 0, ctx->stream>>>(h, keys, n, out); break;
    default: k_diagonal<MODEL_MOM1D><<<g, 256, 0, ctx->stream>>>(h, keys, n, out); break;
  }
  return rimu_cuda_check(cudaGetLastError(), "k_diagonal");
}

// All offdiagonals of the column of address (key_lo, key_hi); keys out as one word each, or
// as (lo, hi) pairs when h.nbits > 64.
int rimu_launch_offdiagonals(rimu_ctx *ctx, const DevModel &h, uint64_t key_lo, uint64_t key_hi,
                             int noff, uint64_t *keys, double *vals) {
  if (noff == 0) return 0;
  unsigned g = (unsigned)((noff + 127) / 128);
  if (h.nbits > 64) {
    const Key128 key = k128(key_lo, key_hi);
    Key128 *k2 = reinterpret_cast<Key128 *>(keys);
    if (h.kind == MODEL_REAL1D) k_offdiagonals<MODEL_REAL1D><<<g, 128, 0, ctx->stream>>>(h, key, noff, k2, vals);
    else if (h.kind == MODEL_REALSPACE) k_offdiagonals<MODEL_REALSPACE><<<g, 128, 0, ctx->stream>>>(h, key, noff, k2, vals);
    else k_offdiagonals<MODEL_MOM1D><<<g, 128, 0, ctx->stream>>>(h, key, noff, k2, vals);
    return rimu_cuda_check(cudaGetLastError(), "k_offdiagonals");
  }
  const uint64_t key = key_lo;
  switch (h.kind) {
    case MODEL_REAL1D: k_offdiagonals<MODEL_REAL1D><<<g, 128, 0, ctx->stream>>>(h, key, noff, keys, vals); break;
    case MODEL_REALSPACE: k_offdiagonals<MODEL_REALSPACE><<<g, 128, 0, ctx->stream>>>(h, key, noff, keys, vals); break;
    default: k_offdiagonals<MODEL_MOM1D><<<g, 128, 0, ctx->stream>>>(h, key, noff, keys, vals); break;
  }
  return rimu_cuda_check(cudaGetLastError(), "k_offdiagonals");
}
