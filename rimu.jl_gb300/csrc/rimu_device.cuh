// rimu_device.cuh -- device primitives for the GB300 FCIQMC step and matrix-free H*v.
//
// Addresses are single-chunk bit strings (up to 64 bits) with the Rimu.jl layout:
//   BoseFS: mode 1 at the least significant end, each mode written as n_i ones followed by
//           a zero separator (src/BitStringAddresses/bitstring.jl:464-472).
//   FermiFS: mode k <-> bit k-1 (bitstring.jl:713-723).
// The unsigned integer order of the key equals BitString isless (bitstring.jl:317-324).
//
// FP64 is scarce on GB300 (about 0.5 T FP64 instructions/s for the whole GPU), so the
// kernels use at most one FP64 multiply per spawn: matrix elements of the transition
// operator come from tables computed on the host with the reference's own expressions,
// and stochastic rounding / threshold projection decisions are evaluated with integer
// instructions on the IEEE bit patterns (exactly equivalent to comparing r < p with
// r = u53 * 2^-53).
#pragma once
#include <cstdint>

#ifndef RIMU_HD
#define RIMU_HD __host__ __device__ __forceinline__
#endif

namespace rimu {

enum ModelKind : int { MODEL_REAL1D = 1, MODEL_REALSPACE = 2, MODEL_MOM1D = 3 };
enum Style : int { STYLE_INTEGER = 0, STYLE_DETERMINISTIC = 1, STYLE_DSS = 2 };
enum OpKind : int { OP_TRANSITION = 0, OP_HAMILTONIAN = 1 };
enum Purpose : uint32_t { PURPOSE_SPAWN = 1, PURPOSE_DIAG = 2, PURPOSE_COMPRESS = 3 };

constexpr int MAX_MODES = 64;
constexpr uint64_t EMPTY_KEY = ~0ull;   // never a valid address: would need 64 particles in 1 mode

// ------------------------------------------------------------------------------------------
// Device model description (immutable during a step).
// ------------------------------------------------------------------------------------------
constexpr int MAXC = 4;   // components of a multi-component address

struct DevModel {
  int kind, fermion, N, M, nbits;
  int ndim, dims[3], periodic[3];
  double u, t;
  const double *kes;     // HubbardMom1D dispersion [M]
  const double *pot;     // HubbardRealSpace trap [M] or null
  const double *aoff;    // transition offdiagonal magnitudes, indexed by occupation product
  int aoff_len;
  const double *hoff;    // Hamiltonian offdiagonal magnitudes (no dt), same indexing
  const double *recip;   // recip[n] = 1.0 / n for n < recip_len
  int recip_len;
  const double *dint;    // dint[n] = (double)n for n < recip_len
  // Multi-component addresses (CompositeFS, FermiFS2C): component c in the bits
  // [coff[c], coff[c] + cbits[c]) of the key, the last component in the lowest bits.
  int ncomp;             // 1 .. MAXC
  int cferm[MAXC];       // per component: FermiFS (1) or BoseFS (0)
  int cN[MAXC];          // particles per component
  int cbits[MAXC];       // bits per component
  int coff[MAXC];        // lowest key bit of each component
  double ct[MAXC];       // HubbardRealSpace hopping t[c]
  double cu[MAXC * (MAXC + 1) / 2];   // HubbardRealSpace u, upper triangle row by row
  int u_nonzero;         // HubbardRealSpace: some interaction is nonzero
  int cstride;           // offdiagonal-table block size per component (HubbardRealSpace)
};

// ------------------------------------------------------------------------------------------
// Bits
// ------------------------------------------------------------------------------------------
RIMU_HD int ctz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return x ? __ffsll((long long)x) - 1 : 64;
#else
  return x ? __builtin_ctzll(x) : 64;
#endif
}
RIMU_HD int popc64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __popcll(x);
#else
  return __builtin_popcountll(x);
#endif
}
RIMU_HD int clz64_hd(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}
RIMU_HD uint64_t shr64(uint64_t x, int s) { return s >= 64 ? 0 : x >> s; }
RIMU_HD uint64_t shl64(uint64_t x, int s) { return s >= 64 ? 0 : x << s; }
RIMU_HD uint64_t lowmask(int n) { return n >= 64 ? ~0ull : ((1ull << n) - 1); }

// murmur3 fmix64 finalizer: spreads address bits for bucket and table placement.
RIMU_HD uint64_t mix64(uint64_t x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}
RIMU_HD uint32_t bucket_of(uint64_t key, int nb_bits) {
  return nb_bits == 0 ? 0u : (uint32_t)(mix64(key) >> (64 - nb_bits));
}

// ------------------------------------------------------------------------------------------
// Address words.  An address of at most 64 bits is one uint64_t; a two-chunk address (65-128
// bits, bitstring.jl:6-18) is a Key128 with the same bit positions across both words.  The
// generic helpers below let the BoseFS/FermiFS operations be written once for both.
// ------------------------------------------------------------------------------------------
struct __align__(16) Key128 { uint64_t lo, hi; };
RIMU_HD Key128 k128(uint64_t lo, uint64_t hi) { Key128 k; k.lo = lo; k.hi = hi; return k; }
RIMU_HD bool operator==(Key128 a, Key128 b) { return a.lo == b.lo && a.hi == b.hi; }
RIMU_HD bool operator!=(Key128 a, Key128 b) { return a.lo != b.lo || a.hi != b.hi; }
RIMU_HD bool operator<(Key128 a, Key128 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
RIMU_HD Key128 operator&(Key128 a, Key128 b) { return k128(a.lo & b.lo, a.hi & b.hi); }
RIMU_HD Key128 operator|(Key128 a, Key128 b) { return k128(a.lo | b.lo, a.hi | b.hi); }
RIMU_HD Key128 operator^(Key128 a, Key128 b) { return k128(a.lo ^ b.lo, a.hi ^ b.hi); }
RIMU_HD Key128 operator~(Key128 a) { return k128(~a.lo, ~a.hi); }

// shifts by any s >= 0 (0 beyond the width)
RIMU_HD uint64_t kshl(uint64_t a, int s) { return shl64(a, s); }
RIMU_HD uint64_t kshr(uint64_t a, int s) { return shr64(a, s); }
RIMU_HD Key128 kshl(Key128 a, int s) {
  if (s <= 0) return a;
  if (s >= 128) return k128(0, 0);
  if (s >= 64) return k128(0, a.lo << (s - 64));
  return k128(a.lo << s, (a.hi << s) | (a.lo >> (64 - s)));
}
RIMU_HD Key128 kshr(Key128 a, int s) {
  if (s <= 0) return a;
  if (s >= 128) return k128(0, 0);
  if (s >= 64) return k128(a.hi >> (s - 64), 0);
  return k128((a.lo >> s) | (a.hi << (64 - s)), a.hi >> s);
}
RIMU_HD int kctz(uint64_t x) { return ctz64(x); }
RIMU_HD int kctz(Key128 x) { return x.lo ? ctz64(x.lo) : 64 + ctz64(x.hi); }
RIMU_HD int kpopc(uint64_t x) { return popc64(x); }
RIMU_HD int kpopc(Key128 x) { return popc64(x.lo) + popc64(x.hi); }
RIMU_HD int kclz(uint64_t x) { return clz64_hd(x); }
RIMU_HD int kclz(Key128 x) { return x.hi ? clz64_hd(x.hi) : 64 + clz64_hd(x.lo); }
RIMU_HD bool kzero(uint64_t x) { return x == 0; }
RIMU_HD bool kzero(Key128 x) { return (x.lo | x.hi) == 0; }
RIMU_HD bool ktest(uint64_t x, int b) { return ((x >> b) & 1) != 0; }
RIMU_HD bool ktest(Key128 x, int b) { return b < 64 ? ((x.lo >> b) & 1) != 0 : ((x.hi >> (b - 64)) & 1) != 0; }
RIMU_HD uint64_t kclear_lowest(uint64_t x) { return x & (x - 1); }
RIMU_HD Key128 kclear_lowest(Key128 x) {
  return x.lo ? k128(x.lo & (x.lo - 1), x.hi) : k128(0, x.hi & (x.hi - 1));
}
// The 64-bit word that stands for an address in hashes and random-number counters: the
// address itself up to 64 bits, lo ^ mix64(hi) for two words (mix64(0) = 0).
RIMU_HD uint64_t kword(uint64_t k) { return k; }
RIMU_HD uint64_t kword(Key128 k) { return k.lo ^ mix64(k.hi); }
RIMU_HD uint32_t bucket_of(Key128 key, int nb_bits) { return bucket_of(kword(key), nb_bits); }

template <class K> struct KT;
template <> struct KT<uint64_t> {
  static constexpr int BITS = 64;
  RIMU_HD static uint64_t make(uint64_t lo, uint64_t) { return lo; }
  RIMU_HD static uint64_t lo(uint64_t k) { return k; }
  RIMU_HD static uint64_t hi(uint64_t) { return 0; }
  RIMU_HD static uint64_t mask(int n) { return lowmask(n); }            // low n bits
  RIMU_HD static uint64_t bit(int i) { return 1ull << i; }
  RIMU_HD static uint64_t from(uint64_t v) { return v; }
  RIMU_HD static uint64_t empty() { return ~0ull; }
};
template <> struct KT<Key128> {
  static constexpr int BITS = 128;
  RIMU_HD static Key128 make(uint64_t lo, uint64_t hi) { return k128(lo, hi); }
  RIMU_HD static uint64_t lo(Key128 k) { return k.lo; }
  RIMU_HD static uint64_t hi(Key128 k) { return k.hi; }
  RIMU_HD static Key128 mask(int n) {
    return n >= 128 ? k128(~0ull, ~0ull) : (n >= 64 ? k128(~0ull, lowmask(n - 64)) : k128(lowmask(n), 0));
  }
  RIMU_HD static Key128 bit(int i) { return i < 64 ? k128(1ull << i, 0) : k128(0, 1ull << (i - 64)); }
  RIMU_HD static Key128 from(uint64_t v) { return k128(v, 0); }
  RIMU_HD static Key128 empty() { return k128(~0ull, ~0ull); }
};

// ------------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as easy as 1, 2, 3",
// SC'11).  Counter (draw, step, address lo, address hi), key (seed lo, seed hi ^ purpose ^
// replica): a draw depends only on what it is for, never on the thread that makes it.
// ------------------------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };

RIMU_HD U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    // one 32 x 32 -> 64-bit product gives both halves (a single wide multiply on the GPU)
    const uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    U4 n;
    n.x = hi1 ^ c.y ^ k0; n.y = lo1; n.z = hi0 ^ c.w ^ k1; n.w = lo0;
    c = n;
  }
  return c;
}
RIMU_HD U4 draw(uint64_t seed, uint32_t purpose, uint32_t replica, uint32_t step,
                uint64_t addr, uint32_t j) {
  U4 c{j, step, (uint32_t)addr, (uint32_t)(addr >> 32)};
  return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32) ^ (purpose << 28) ^ replica);
}
RIMU_HD uint64_t u53_of(U4 r) { return ((uint64_t)r.y << 21) | (uint64_t)(r.z >> 11); }
RIMU_HD uint32_t uniform_index(uint32_t r, uint32_t n) {   // floor(r * n / 2^32)
  return (uint32_t)(((uint64_t)r * n) >> 32);
}

// ------------------------------------------------------------------------------------------
// Exact stochastic decisions with integer instructions.
// ------------------------------------------------------------------------------------------
RIMU_HD uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t u; __builtin_memcpy(&u, &x, 8); return u;
#endif
}
RIMU_HD double bitsd(uint64_t u) {
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x; __builtin_memcpy(&x, &u, 8); return x;
#endif
}

// u53 < p * 2^53 for finite p >= 0 (p >= 1 -> always true), i.e. r < p for r = u53 * 2^-53.
RIMU_HD bool bernoulli53(uint64_t u53, double p) {
  uint64_t b = dbits(p) & 0x7fffffffffffffffull;
  int e = (int)(b >> 52);
  if (e >= 1023) return true;                       // p >= 1
  uint64_t mant = b & lowmask(52);
  int s;
  if (e == 0) { s = 1074 - 53; }                    // subnormal: p = mant * 2^-1074
  else { mant |= 1ull << 52; s = 1075 - 53 - e; }   // p * 2^53 = mant * 2^-(s)
  // s >= 1 here because e <= 1022.
  if (s >= 64) return u53 == 0 && mant != 0;
  uint64_t q = mant >> s;
  uint64_t rem = mant & lowmask(s);
  return u53 < q + (rem != 0 ? 1u : 0u);
}

// floor(|x|) and the Bernoulli on frac(|x|): the integer stochastic rounding of
// spawning.jl:33-45, restated as floor(|x|) + [r < frac(|x|)].  |x| < 2^62 assumed.
RIMU_HD int64_t round_stochastic(double x, uint64_t u53) {
  uint64_t b = dbits(x);
  bool neg = (b >> 63) != 0;
  b &= 0x7fffffffffffffffull;
  int e = (int)(b >> 52);
  int64_t k;
  bool up;
  if (e < 1023) {                 // |x| < 1: k = 0, frac = |x|
    k = 0;
    up = bernoulli53(u53, bitsd(b));
  } else {
    uint64_t mant = (b & lowmask(52)) | (1ull << 52);
    int sh = e - 1075;            // |x| = mant * 2^sh
    if (sh >= 0) {                // integer already
      k = (int64_t)(mant << sh);
      up = false;
    } else {
      int s = -sh;                // 1..52
      k = (int64_t)(mant >> s);
      uint64_t fr = mant & lowmask(s);   // frac = fr * 2^-s ; compare u53 < fr * 2^(53-s)
      up = u53 < (fr << (53 - s)) ;      // exact: fr * 2^(53-s) is an integer < 2^53
    }
  }
  int64_t n = k + (up ? 1 : 0);
  return neg ? -n : n;
}

// Threshold projection of a float spawn (spawning.jl:13-31).  thresh > 0.
RIMU_HD double project_threshold(double x, double thresh, uint64_t u53) {
  double ax = fabs(x);
  if (ax < thresh) {
    double prob = (thresh == 1.0) ? ax : ax / thresh;
    if (bernoulli53(u53, prob)) return x < 0 ? -thresh : thresh;
    return 0.0;
  }
  return x;
}

// Integer part of |x| (x finite, |x| < 2^62) via the bit pattern.
RIMU_HD int64_t floor_abs(double x) {
  uint64_t b = dbits(x) & 0x7fffffffffffffffull;
  int e = (int)(b >> 52);
  if (e < 1023) return 0;
  uint64_t mant = (b & lowmask(52)) | (1ull << 52);
  int sh = e - 1075;
  return sh >= 0 ? (int64_t)(mant << sh) : (int64_t)(mant >> (-sh));
}

// Tests on IEEE bit patterns (GB300 issues FP64 compares on the slow FP64 pipe).
RIMU_HD uint64_t abs_bits(double x) { return dbits(x) & 0x7fffffffffffffffull; }
RIMU_HD bool is_zero_d(double x) { return abs_bits(x) == 0; }
RIMU_HD bool is_neg_d(double x) { return (dbits(x) >> 63) != 0; }
RIMU_HD bool abs_lt_one(double x) { return abs_bits(x) < 0x3FF0000000000000ull; }
RIMU_HD double abs_d(double x) { return bitsd(abs_bits(x)); }
RIMU_HD double signed_like(double mag, double s) {   // |mag| with the sign of s
  return bitsd(abs_bits(mag) | (dbits(s) & 0x8000000000000000ull));
}
// Exact int64 -> double for |v| < 2^53 with integer instructions.
RIMU_HD double i2d_exact(int64_t v) {
  if (v == 0) return 0.0;
  uint64_t sgn = v < 0 ? 0x8000000000000000ull : 0;
  uint64_t a = (uint64_t)(v < 0 ? -v : v);
  int p = 63 - clz64_hd(a);
  uint64_t mant = (p <= 52) ? (a << (52 - p)) : (a >> (p - 52));
  return bitsd(sgn | ((uint64_t)(1023 + p) << 52) | (mant & lowmask(52)));
}

// Order-preserving map of doubles to unsigned integers (for canonical summation order).
RIMU_HD uint64_t ordered_bits(double v) {
  uint64_t u = dbits(v);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// Unsigned 128-bit fixed point with 2^-64 resolution: |x| -> floor(|x| * 2^64).
struct U128 { uint64_t lo, hi; };
RIMU_HD U128 fixed_of_general(double ax);
// |x| in [2^-12, 2^52), the range of nearly every walker value, takes the short path: the
// 53-bit significand shifted left by sh = e - 1011 in [0, 64); other values the general one.
RIMU_HD U128 fixed_of(double ax) {
  const uint64_t b = dbits(ax) & 0x7fffffffffffffffull;
  const int sh = (int)(b >> 52) - 1011;
  if ((unsigned)sh < 64u) {
    const uint64_t mant = (b & lowmask(52)) | (1ull << 52);
    U128 r;
    r.lo = mant << sh;
    r.hi = sh ? mant >> (64 - sh) : 0;
    return r;
  }
  return fixed_of_general(ax);
}
RIMU_HD U128 fixed_of_general(double ax) {
  uint64_t b = dbits(ax) & 0x7fffffffffffffffull;
  int e = (int)(b >> 52);
  U128 r{0, 0};
  if (b == 0) return r;
  uint64_t mant = b & lowmask(52);
  int sh;
  if (e == 0) sh = -1074 + 64; else { mant |= 1ull << 52; sh = e - 1075 + 64; }
  if (sh >= 75) { r.lo = ~0ull; r.hi = ~0ull; return r; }
  if (sh >= 64) { r.hi = mant << (sh - 64); return r; }
  if (sh > 0) { r.lo = mant << sh; r.hi = (sh > 11) ? (mant >> (64 - sh)) : 0; return r; }
  if (sh == 0) { r.lo = mant; return r; }
  r.lo = (-sh >= 64) ? 0 : (mant >> (-sh));
  return r;
}
RIMU_HD U128 add128(U128 a, U128 b) {
  U128 r;
  r.lo = a.lo + b.lo;
  r.hi = a.hi + b.hi + (r.lo < a.lo ? 1 : 0);
  return r;
}
RIMU_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
  return __clzll((long long)x);
#else
  return x ? __builtin_clzll(x) : 64;
#endif
}
// Correctly rounded (nearest-even) value of (hi*2^64 + lo) * 2^-64.
RIMU_HD double fixed_to_double(U128 x) {
  if (x.hi == 0 && x.lo == 0) return 0.0;
  int top = x.hi ? 127 - clz64(x.hi) : 63 - clz64(x.lo);   // index of the leading one
  uint64_t m;
  if (top <= 52) {
    m = x.lo << (52 - top);
  } else {
    int drop = top - 52;                                      // 1..75
    m = drop >= 64 ? (x.hi >> (drop - 64)) : ((x.lo >> drop) | (x.hi << (64 - drop)));
    m &= lowmask(53);
    int rb = drop - 1;
    uint64_t rbit;
    bool sticky;
    if (rb >= 64) {
      rbit = (x.hi >> (rb - 64)) & 1;
      sticky = (x.lo != 0) || ((x.hi & lowmask(rb - 64)) != 0);
    } else {
      rbit = (x.lo >> rb) & 1;
      sticky = (x.lo & lowmask(rb)) != 0;
    }
    if (rbit && (sticky || (m & 1))) {
      m += 1;
      if (m >> 53) { m >>= 1; top += 1; }
    }
  }
  return bitsd(((uint64_t)(1023 + top - 64) << 52) | (m & lowmask(52)));
}

// ------------------------------------------------------------------------------------------
// BoseFS / FermiFS operations on a 64-bit key
// ------------------------------------------------------------------------------------------
// Occupied mode record (BoseFSIndex, fockaddress.jl:515-519): occupation, 1-based mode,
// bit offset of the first boson.
struct ModeIdx { int occ, mode, offset; };

// k-th occupied mode (1-based).  Also reports the previous occupied mode (mode 0 if none).
template <class K>
RIMU_HD ModeIdx bose_find_occupied(K key, int k, ModeIdx *prev) {
  K x = key;
  int mode = 1, bit = 0;
  ModeIdx p{0, 0, 0};
  while (!kzero(x)) {
    int z = kctz(x);
    x = kshr(x, z); mode += z; bit += z;
    int n = kctz(~x);
    ModeIdx cur{n, mode, bit};
    if (--k == 0) { if (prev) *prev = p; return cur; }
    p = cur;
    x = kshr(x, n); bit += n;
  }
  if (prev) *prev = p;
  return ModeIdx{0, 0, 0};
}

// find_mode (bosefs.jl:188-203): occupation and offset of a given 1-based mode.
template <class K>
RIMU_HD ModeIdx bose_find_mode(K key, int mode_wanted) {
  K x = key;
  int mode = 1, bit = 0, last_occ = 0, last_mode = 0, last_off = 0;
  while (!kzero(x)) {
    int z = kctz(x);
    x = kshr(x, z); mode += z; bit += z;
    int n = kctz(~x);
    int dist = mode_wanted - mode;
    if (dist == 0) return ModeIdx{n, mode_wanted, bit};
    if (dist < 0) return ModeIdx{0, mode_wanted, bit + dist};
    last_occ = n; last_mode = mode; last_off = bit;
    x = kshr(x, n); bit += n;
  }
  return ModeIdx{0, mode_wanted, last_off + last_occ + mode_wanted - last_mode};
}

template <class K>
RIMU_HD int bose_num_occupied(K key) {
  // number of runs of ones
  return kpopc(key & ~kshl(key, 1));
}

// partial_left_shift / partial_right_shift (bitstring.jl:342-375) on one 64-bit chunk.
template <class K>
RIMU_HD K partial_left_shift(K c, int i, int j) {
  const K mask = kshl(KT<K>::mask(j - i + 1), i);
  const K shifted = kshl(c & mask, 1) & mask;
  return shifted | (c & ~mask) | KT<K>::bit(i);
}
template <class K>
RIMU_HD K partial_right_shift(K c, int i, int j) {
  const K mask = kshl(KT<K>::mask(j - i + 1), i);
  const K shifted = kshr(c & mask, 1) & mask;
  return shifted | (c & ~mask) | KT<K>::bit(j);
}
// bose_move_particle (bitstring.jl:559-567): move one boson between bit offsets.
template <class K>
RIMU_HD K bose_move(K c, int from, int to) {
  if (to == from) return c;
  if (to < from) return partial_left_shift(c, to, from);
  return partial_right_shift(c, from, to - 1);
}

// ------------------------------------------------------------------------------------------
// Model offdiagonals.  Each returns the new key and the integer "occupation product" whose
// square root is the magnitude (index into the aoff/hoff tables), plus a sign.  prod == 0
// marks an illegal move (value 0.0, address unchanged).
// ------------------------------------------------------------------------------------------
template <class K> struct OffdiagT { K key; int prod; int sign; };
using Offdiag = OffdiagT<uint64_t>;

template <class K>
RIMU_HD int num_offdiagonals_real(const DevModel &h, K key) {
  if constexpr (KT<K>::BITS == 64) {
    if (h.ncomp >= 2) {   // every component's hops
      int s = 0;
      for (int c = 0; c < h.ncomp; ++c) {
        const uint64_t kc = shr64(key, h.coff[c]) & lowmask(h.cbits[c]);
        s += h.cferm[c] ? popc64(kc) : bose_num_occupied(kc);
      }
      return s * 2 * h.ndim;
    }
  } else {
    if (h.ncomp >= 2) {   // the same on a two-word address (each component one word)
      int s = 0;
      for (int c = 0; c < h.ncomp; ++c) {
        const uint64_t kc = kshr(key, h.coff[c]).lo & lowmask(h.cbits[c]);
        s += h.cferm[c] ? popc64(kc) : bose_num_occupied(kc);
      }
      return s * 2 * h.ndim;
    }
  }
  int s = h.fermion ? kpopc(key) : bose_num_occupied(key);
  return h.kind == MODEL_REAL1D ? 2 * s : s * 2 * h.ndim;
}

// HubbardReal1D.get_offdiagonal via hopnextneighbour (bosefs.jl:297-345).
template <class K>
RIMU_HD OffdiagT<K> real1d_offdiag(const DevModel &h, K key, int chosen) {
  int site = (chosen + 1) >> 1;
  ModeIdx prev;
  ModeIdx cur = bose_find_occupied(key, site, &prev);
  int M = h.M, B = h.nbits;
  OffdiagT<K> r;
  r.sign = 1;
  if (chosen & 1) {   // hop right
    if (cur.mode == M) {
      r.key = (kshl(key, 1) | KT<K>::from(1)) & KT<K>::mask(B);
      r.prod = cur.occ * (kctz(~key) + 1);
    } else {
      int after = cur.offset + cur.occ;          // separator after the site
      int next = kctz(~kshr(key, after + 1));    // occupation of mode+1
      r.key = key ^ kshl(KT<K>::from(3), after - 1);
      r.prod = cur.occ * (next + 1);
    }
  } else {            // hop left
    if (cur.mode == 1) {
      K nk = kshr(key, 1) | KT<K>::bit(B - 1);
      // leading ones of nk within B bits = occupation of mode M after the hop
      int lead = 0;
      for (int b = B - 1; b >= 0 && ktest(nk, b); --b) ++lead;
      r.key = nk;
      r.prod = kctz(~key) * lead;
    } else {
      int prev_occ = (prev.mode == cur.mode - 1) ? prev.occ : 0;
      r.key = key ^ kshl(KT<K>::from(3), cur.offset - 1);
      r.prod = cur.occ * (prev_occ + 1);
    }
  }
  return r;
}

// sum_i n_i (n_i - 1) of a BoseFS word: each run of n ones contributes n(n-1), and
// sum over runs of C(n, 2) = sum_{d >= 1} popcount(bits starting d+1 consecutive ones).
template <class K>
RIMU_HD int bose_interaction_fast(K x) {
  int acc = 0;
  K y = x & kshr(x, 1);
  while (!kzero(y)) { acc += kpopc(y); y = y & kshr(y, 1); }
  return 2 * acc;
}

// Position of the k-th (0-based) set bit (k < number of set bits): a binary search on
// popcounts of halves, constant time and without divergent loops.
RIMU_HD int select_bit(uint64_t x, int k) {
  int pos = 0;
  int c = popc64(x & 0xffffffffull);
  if (k >= c) { k -= c; x >>= 32; pos = 32; }
  uint32_t y = (uint32_t)x;
  c = popc64(y & 0xffffu);
  if (k >= c) { k -= c; y >>= 16; pos += 16; }
  c = popc64(y & 0xffu);
  if (k >= c) { k -= c; y >>= 8; pos += 8; }
  c = popc64(y & 0xfu);
  if (k >= c) { k -= c; y >>= 4; pos += 4; }
  c = popc64(y & 0x3u);
  if (k >= c) { k -= c; y >>= 2; pos += 2; }
  return pos + (k >= (int)(y & 1u) ? 1 : 0);
}
RIMU_HD int select_bit(Key128 x, int k) {
  const int c = popc64(x.lo);
  return k < c ? select_bit(x.lo, k) : 64 + select_bit(x.hi, k - c);
}

// HubbardReal1D offdiagonal with word operations only: the site-th occupied mode starts at
// the site-th run start (bits that are set and whose lower neighbour is not); same results
// as hopnextneighbour (bosefs.jl:297-345).
template <class K>
RIMU_HD OffdiagT<K> real1d_offdiag_fast(K key, int B, int chosen) {
  constexpr int W = KT<K>::BITS;
  const int site = (chosen + 1) >> 1;
  const K starts = key & ~kshl(key, 1);
  const int start = select_bit(starts, site - 1);
  const int n = kctz(~kshr(key, start));
  const int end = start + n;                 // separator after the mode, or B for mode M
  OffdiagT<K> r;
  r.sign = 1;
  if (chosen & 1) {                          // hop right
    if (end == B) {                          // from mode M to mode 1 (periodic wrap)
      r.key = (kshl(key, 1) | KT<K>::from(1)) & KT<K>::mask(B);
      r.prod = n * (kctz(~key) + 1);
    } else {
      const int next = kctz(~kshr(key, end + 1));
      r.key = key ^ kshl(KT<K>::from(3), end - 1);
      r.prod = n * (next + 1);
    }
  } else {                                   // hop left
    if (start == 0) {                        // from mode 1 to mode M
      const K nk = kshr(key, 1) | KT<K>::bit(B - 1);
      const int lead = kclz(~kshl(nk, W - B));
      r.key = nk;
      r.prod = n * lead;
    } else {
      const int prev = start >= 2 ? kclz(~kshl(key, W + 1 - start)) : 0;
      r.key = key ^ kshl(KT<K>::from(3), start - 1);
      r.prod = n * (prev + 1);
    }
  }
  return r;
}

// neighbor_site (geometry.jl:232-235): 1-based mode and direction, 0 if illegal.
RIMU_HD int neighbor_site(const DevModel &h, int mode, int chosen) {
  int D = h.ndim, x[3] = {0, 0, 0}, rem = mode - 1;
  for (int d = 0; d < D; ++d) { x[d] = rem % h.dims[d]; rem /= h.dims[d]; }
  int dir = chosen <= D ? chosen - 1 : chosen - D - 1;
  x[dir] += chosen <= D ? 1 : -1;
  if (x[dir] < 0 || x[dir] >= h.dims[dir]) {
    if (!h.periodic[dir]) return 0;
    x[dir] = (x[dir] + h.dims[dir]) % h.dims[dir];
  }
  int site = 0;
  for (int d = D - 1; d >= 0; --d) site = site * h.dims[d] + x[d];
  return site + 1;
}

// Fermionic single excitation a+_dst a_src on one FermiFS chunk (1-based modes; src occupied):
// false when dst is occupied; else the new chunk and the sign (-1)^(occupied modes below src,
// then below dst after the removal) (fermi_excitation, bitstring.jl:746-791).
template <class K>
RIMU_HD bool fermi_move(K key, int src, int dst, K &out, int &sign) {
  if (ktest(key, dst - 1)) return false;
  int count = kpopc(key & KT<K>::mask(src - 1));
  const K k1 = key ^ KT<K>::bit(src - 1);
  count += kpopc(k1 & KT<K>::mask(dst - 1));
  out = k1 | KT<K>::bit(dst - 1);
  sign = (count & 1) ? -1 : 1;
  return true;
}

// HubbardRealSpace offdiagonal `chosen` of one component's chunk (HubbardRealSpace.jl:325-338).
template <class K>
RIMU_HD OffdiagT<K> realspace_hop(const DevModel &h, K key, int chosen, bool fermion) {
  int nb = 2 * h.ndim;
  int particle = (chosen - 1) / nb + 1, neigh = (chosen - 1) % nb + 1;
  OffdiagT<K> r{key, 0, 1};
  if (fermion) {
    // particle-th set bit
    K x = key;
    for (int i = 1; i < particle; ++i) x = kclear_lowest(x);
    int src = kctz(x) + 1;
    int dst = neighbor_site(h, src, neigh);
    if (dst == 0) return r;
    K nk;
    int sign;
    if (!fermi_move(key, src, dst, nk, sign)) return r;   // Pauli blocked
    r.key = nk;
    r.prod = 1;
    r.sign = sign;
    return r;
  }
  ModeIdx src = bose_find_occupied(key, particle, nullptr);
  int dst_mode = neighbor_site(h, src.mode, neigh);
  if (dst_mode == 0) return r;
  ModeIdx dst = bose_find_mode(key, dst_mode);
  r.key = bose_move(key, src.offset, dst.offset);
  r.prod = src.occ * (dst.occ + 1);
  return r;
}

// ---- two-component addresses -------------------------------------------------------------
// A component has at most 64 bits; a multi-component address has one or two words.
RIMU_HD uint64_t component_of(const DevModel &h, uint64_t key, int c) {
  return shr64(key, h.coff[c]) & lowmask(h.cbits[c]);
}
RIMU_HD uint64_t with_component(const DevModel &h, uint64_t key, int c, uint64_t ck) {
  const uint64_t m = shl64(lowmask(h.cbits[c]), h.coff[c]);
  return (key & ~m) | shl64(ck, h.coff[c]);
}
RIMU_HD uint64_t component_of(const DevModel &h, Key128 key, int c) {
  return kshr(key, h.coff[c]).lo & lowmask(h.cbits[c]);
}
RIMU_HD Key128 with_component(const DevModel &h, Key128 key, int c, uint64_t ck) {
  const Key128 m = kshl(k128(lowmask(h.cbits[c]), 0), h.coff[c]);
  return (key & ~m) | kshl(k128(ck, 0), h.coff[c]);
}
// Position of u[i, j] (i <= j, 0-based) in the upper triangle of a C x C matrix, row by row.
RIMU_HD int cu_index(int C, int i, int j) { return i * C - i * (i - 1) / 2 + (j - i); }
RIMU_HD int component_occupied(uint64_t ck, int fermion) {
  return fermion ? popc64(ck) : bose_num_occupied(ck);
}
// Occupation number of every mode of one component chunk (0-based modes < M).
RIMU_HD void component_occupations(uint64_t ck, int fermion, int M, uint8_t *occ) {
  for (int i = 0; i < M; ++i) occ[i] = 0;
  uint64_t x = ck;
  if (fermion) {
    while (x) { occ[ctz64(x)] = 1; x &= x - 1; }
    return;
  }
  int mode = 0;
  while (x) {
    const int z = ctz64(x);
    x = shr64(x, z); mode += z;
    const int n = ctz64(~x);
    if (mode < M) occ[mode] = (uint8_t)n;
    x = shr64(x, n);
  }
}
// sum_i n_{a,i} n_{b,i} (dot of occupied modes, fockaddress.jl:692-717; two FermiFS chunks:
// the popcount of their intersection, bitstring.jl:833-838)
RIMU_HD int component_overlap(const DevModel &h, uint64_t a, int fa, uint64_t b, int fb) {
  if (fa && fb) return popc64(a & b);
  uint8_t oa[MAX_MODES], ob[MAX_MODES];
  component_occupations(a, fa, h.M, oa);
  component_occupations(b, fb, h.M, ob);
  int acc = 0;
  for (int i = 0; i < h.M; ++i) acc += (int)oa[i] * (int)ob[i];
  return acc;
}

// HubbardRealSpace offdiagonal: one component, or component 1's hops followed by component
// 2's, and so on (HubbardRealSpaceOffdiagonals, HubbardRealSpace.jl:344-391), each with its
// own t (table block c).
template <class K>
RIMU_HD OffdiagT<K> realspace_offdiag(const DevModel &h, K key, int chosen) {
  if (h.ncomp >= 2) {
    int c = 0;
    uint64_t kc = component_of(h, key, 0);
    for (;;) {
      const int nc = component_occupied(kc, h.cferm[c]) * 2 * h.ndim;
      if (chosen <= nc || c + 1 == h.ncomp) break;
      chosen -= nc;
      ++c;
      kc = component_of(h, key, c);
    }
    const Offdiag r = realspace_hop(h, kc, chosen, h.cferm[c] != 0);
    OffdiagT<K> out{key, r.prod, r.sign};
    if (r.prod == 0) return out;
    out.key = with_component(h, key, c, r.key);
    out.prod += c * h.cstride;
    return out;
  }
  return realspace_hop(h, key, chosen, h.fermion != 0);
}

// HubbardMom1D with FermiFS2C: momentum_transfer_excitation of two components with fold=true
// (excitations.jl:82-119) and element u/M * (sign_a * sign_b) (HubbardMom1D.jl:196-205).  The
// magnitude u/M = u/(2M) * sqrt(4) is entry 4 of the u/(2M) sqrt(p) table (exact: scaling by 2).
template <class K>
RIMU_HD OffdiagT<K> mom2c_offdiag(const DevModel &h, K key, int chosen) {
  const int M = h.M, nb = h.cN[1];
  const uint64_t ka = component_of(h, key, 0), kb = component_of(h, key, 1);
  const int per_a = (M - 1) * nb;
  const int src_a = (chosen - 1) / per_a + 1, rem = (chosen - 1) % per_a + 1;
  int dst_a = (rem - 1) / nb + 1;
  const int src_b = (rem - 1) % nb + 1;
  OffdiagT<K> r{key, 0, 1};
  if (src_a > popc64(ka) || src_b > popc64(kb)) return r;
  const int sa = select_bit(ka, src_a - 1) + 1, sb = select_bit(kb, src_b - 1) + 1;
  if (dst_a >= sa) dst_a += 1;               // skip the source mode
  const int mom = dst_a - sa;
  const int dst_b = ((sb - mom - 1) % M + M) % M + 1;
  uint64_t na, nbk;
  int ga, gb;
  if (!fermi_move(ka, sa, dst_a, na, ga) || !fermi_move(kb, sb, dst_b, nbk, gb)) return r;
  r.key = with_component(h, with_component(h, key, 0, na), 1, nbk);
  r.prod = 4;
  r.sign = ga * gb;
  return r;
}

// HubbardMom1D occupied mode map in registers (OccupiedModeMap, fockaddress.jl:258-281).
struct MomMap { int s, d; uint8_t mode[MAX_MODES]; uint8_t occ[MAX_MODES]; };
template <class K>
RIMU_HD void mom_map(K key, MomMap &m) {
  K x = key;
  int mode = 1;
  m.s = 0; m.d = 0;
  while (!kzero(x)) {
    int z = kctz(x);
    x = kshr(x, z); mode += z;
    int n = kctz(~x);
    m.mode[m.s] = (uint8_t)mode; m.occ[m.s] = (uint8_t)n; m.s++; m.d += n > 1;
    x = kshr(x, n);
  }
}
RIMU_HD int num_offdiagonals_mom(const DevModel &h, const MomMap &m) {
  return m.s * (m.s - 1) * (h.M - 2) + m.d * (h.M - 1);
}

// momentum_transfer_excitation with fold=true (excitations.jl:26-80), on one- or two-word
// addresses.
template <class K>
RIMU_HD OffdiagT<K> mom1d_offdiag(const DevModel &h, K key, const MomMap &m, int chosen) {
  int M = h.M, s = m.s;
  int dbl = chosen - s * (s - 1) * (M - 2);
  int p_idx, q_idx, mom;
  if (dbl > 0) {
    int which = (dbl - 1) / (M - 1) + 1;
    mom = (dbl - 1) % (M - 1) + 1;
    int idx = 0;
    for (int k = 0; k < s; ++k) {
      which -= m.occ[k] >= 2;
      if (which == 0) { idx = k; break; }
    }
    p_idx = q_idx = idx;
  } else {
    int pair = (chosen - 1) / (M - 2) + 1;
    mom = (chosen - 1) % (M - 2) + 1;
    int fst = (pair - 1) / (s - 1) + 1, snd = (pair - 1) % (s - 1) + 1;
    int fh, sh;
    if (snd < fst) { fh = snd; sh = fst; } else { fh = fst; sh = snd + 1; }
    p_idx = fh - 1; q_idx = sh - 1;
    if (mom >= m.mode[q_idx] - m.mode[p_idx]) mom += 1;
  }
  int src1 = m.mode[p_idx], src2 = m.mode[q_idx];
  int dst1 = ((src1 + mom - 1) % M + M) % M + 1;
  int dst2 = ((src2 - mom - 1) % M + M) % M + 1;
  // occupations before the move
  auto occ_of = [&](int mode) -> int {
    for (int k = 0; k < s; ++k) if (m.mode[k] == mode) return m.occ[k];
    return 0;
  };
  int o_s2 = occ_of(src2), o_s1 = occ_of(src1), o_d2 = occ_of(dst2), o_d1 = occ_of(dst1);
  // a_{src2}, a_{src1}, then a+_{dst2}, a+_{dst1}: sequential occupation factors
  int v = o_s2;
  int c_s1 = o_s1 - (src1 == src2);
  v *= c_s1;
  int c_d2 = o_d2 - (dst2 == src2) - (dst2 == src1);
  v *= c_d2 + 1;
  int c_d1 = o_d1 - (dst1 == src2) - (dst1 == src1) + (dst1 == dst2);
  v *= c_d1 + 1;
  OffdiagT<K> r{key, 0, 1};
  if (v == 0) return r;
  // apply the moves on the bit string: destroy at src offsets, create at dst offsets,
  // one particle at a time with fresh offsets each time
  K k1 = key;
  {
    ModeIdx a = bose_find_mode(k1, src2), b = bose_find_mode(k1, dst2);
    k1 = bose_move(k1, a.offset, b.offset);
    ModeIdx c = bose_find_mode(k1, src1), d = bose_find_mode(k1, dst1);
    k1 = bose_move(k1, c.offset, d.offset);
  }
  r.key = k1;
  r.prod = v;
  return r;
}

}  // namespace rimu
