/*
 * rimu_oracle.c -- CPU restatement of the Rimu.jl FCIQMC hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is compared
 * against; it is never linked into, loaded by, or called from the product library.
 * Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg use it.
 *
 * It restates, in plain C and on occupation-number arrays (ONR) rather than bit tricks,
 * the reference semantics of:
 *   - BoseFS / FermiFS bit-string encodings      src/BitStringAddresses/bitstring.jl:464-472,
 *                                                 511-520, 713-723, 746-791
 *   - HubbardReal1D                               src/Hamiltonians/HubbardReal1D.jl:51-62
 *   - HubbardRealSpace (one component)            src/Hamiltonians/HubbardRealSpace.jl:18,90-97,
 *                                                 279-338; geometry.jl:127-139,161-181,232-235
 *   - HubbardMom1D (BoseFS)                       src/Hamiltonians/HubbardMom1D.jl:49-65,131-194;
 *                                                 excitations.jl:26-80,126-137
 *   - two-component addresses (CompositeFS of     src/BitStringAddresses/multicomponent.jl:10-103
 *     two components, FermiFS2C) with
 *     HubbardRealSpace                            src/Hamiltonians/HubbardRealSpace.jl:18-61,
 *                                                 90-107,284-287,344-391
 *     and HubbardMom1D (FermiFS2C)                src/Hamiltonians/HubbardMom1D.jl:141-205;
 *                                                 excitations.jl:82-119,172-180
 *   - FirstOrderTransitionOperator                src/fciqmc.jl:78-112
 *   - the stochastic styles                       src/StochasticStyles/styles.jl:11-25,94-105,
 *                                                 175-214; spawning.jl:9-93,174-182,232-243,
 *                                                 364-378; compression.jl:18-42
 *   - one apply_operator! step                    src/Interfaces/dictvectors.jl:112-140
 *   - the matrix-free product                     src/DictVectors/abstractdvec.jl:275-284
 *
 * Random numbers.  The reference draws from Julia's task-local Xoshiro in dictionary
 * iteration order, which no parallel implementation can reproduce.  This restatement uses
 * the counter-based Philox4x32-10 generator (Salmon, Moraes, Dror, Shaw, SC'11), keyed on
 * (seed, purpose, replica) and counted by (draw index, step, address), so that any
 * evaluation order gives the same draws.  The GPU path uses the same stream definition, so
 * stochastic steps are compared bit for bit; agreement with the reference itself is
 * statistical (blocking analysis against exact energies).
 *
 * Arithmetic.  Floating-point operations follow the reference expressions except where a
 * different but equally valid rounding order was chosen for the GPU (documented at each
 * site).  Contributions to one address are summed in a canonical order: the diagonal
 * term first, then the spawned values in increasing numerical order.  Compile with
 * -ffp-contract=off so that no multiply-add is fused.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#define O_MAXM 128
#define O_MAXC 4      /* components of a CompositeFS */

/* Addresses are handled as 128-bit integers: a single 64-bit chunk has hi = 0, a two-chunk
 * address (65-128 bits, bitstring.jl:6-18) keeps the same bit positions across both words.
 * The exported 64-bit entry points convert; the *_w entry points take (lo, hi) word pairs. */
typedef unsigned __int128 okey;
#define OKEY_ONE ((okey)1)
static okey o_key_of(uint64_t lo, uint64_t hi) { return ((okey)hi << 64) | lo; }
static uint64_t o_lo(okey k) { return (uint64_t)k; }
static uint64_t o_hi(okey k) { return (uint64_t)(k >> 64); }

/* ------------------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon et al., "Parallel random numbers: as easy as 1, 2, 3", SC'11). */
/* ------------------------------------------------------------------------------------ */
void o_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; ++r) {
    if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

enum { O_PURPOSE_SPAWN = 1, O_PURPOSE_DIAG = 2, O_PURPOSE_COMPRESS = 3 };

/* One Philox block for (seed, purpose, replica) at counter (j, step, address). */
void o_draw(uint64_t seed, uint32_t purpose, uint32_t replica, uint32_t step, uint64_t addr,
            uint32_t j, uint32_t out[4]) {
  uint32_t ctr[4] = {j, step, (uint32_t)addr, (uint32_t)(addr >> 32)};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32) ^ (purpose << 28) ^ replica};
  o_philox4x32_10(ctr, key, out);
}
/* murmur3 fmix64 finalizer (mix64 of the device code); mix64(0) = 0. */
static uint64_t o_mix64(uint64_t x) {
  x ^= x >> 33; x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33; x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}
/* The 64-bit word that stands for an address in random-number counters: the chunk itself for
 * addresses of at most 64 bits, lo ^ mix64(hi) for two chunks. */
static uint64_t o_key_word(okey k) { return o_lo(k) ^ o_mix64(o_hi(k)); }
static void o_draw_k(uint64_t seed, uint32_t purpose, uint32_t replica, uint32_t step, okey addr,
                     uint32_t j, uint32_t out[4]) {
  o_draw(seed, purpose, replica, step, o_key_word(addr), j, out);
}
static inline uint64_t o_u53(const uint32_t r[4]) {
  return ((uint64_t)r[1] << 21) | (uint64_t)(r[2] >> 11);
}
/* r < p with r = u53 * 2^-53, evaluated exactly (p in [0, 1]). */
static inline int o_bernoulli(uint64_t u53, double p) {
  return (double)u53 < ldexp(p, 53);
}

/* ------------------------------------------------------------------------------------ */
/* Addresses                                                                             */
/* ------------------------------------------------------------------------------------ */
/* from_bose_onr, single chunk: bitstring.jl:464-472.  Mode 1 sits at the low end; each
 * mode contributes n_i ones followed by one zero (the last mode has no trailing zero). */
static okey o_bose_from_onr_k(const int *onr, int M) {
  okey result = 0;
  for (int i = M - 1; i >= 0; --i) {
    int n = onr[i];
    result = (n + 1 >= 128) ? 0 : (result << (n + 1));
    result |= (n >= 128) ? ~(okey)0 : ((OKEY_ONE << n) - 1);
  }
  return result;
}
/* to_bose_onr, one 128-bit word: bitstring.jl:511-520. */
static void o_bose_to_onr_k(okey key, int M, int *onr) {
  for (int i = 0; i < M; ++i) onr[i] = 0;
  for (int mode = 0; mode < M; ++mode) {
    int b = 0;
    while (b < 128 && ((key >> b) & 1)) ++b;
    onr[mode] = b;
    key = (b + 1 >= 128) ? 0 : key >> (b + 1);
    if (key == 0) break;
  }
}
/* from_fermi_onr: bitstring.jl:713-723 (mode k <-> bit k-1). */
static okey o_fermi_from_onr_k(const int *onr, int M) {
  okey r = 0;
  for (int k = 0; k < M; ++k) if (onr[k]) r |= OKEY_ONE << k;
  return r;
}
static void o_fermi_to_onr_k(okey key, int M, int *onr) {
  for (int k = 0; k < M; ++k) onr[k] = (int)((key >> k) & 1);
}
uint64_t o_bose_from_onr(const int *onr, int M) { return o_lo(o_bose_from_onr_k(onr, M)); }
void o_bose_to_onr(uint64_t key, int M, int *onr) { o_bose_to_onr_k(key, M, onr); }
uint64_t o_fermi_from_onr(const int *onr, int M) { return o_lo(o_fermi_from_onr_k(onr, M)); }
void o_fermi_to_onr(uint64_t key, int M, int *onr) { o_fermi_to_onr_k(key, M, onr); }

/* ------------------------------------------------------------------------------------ */
/* Models                                                                                */
/* ------------------------------------------------------------------------------------ */
enum { O_REAL1D = 1, O_REALSPACE = 2, O_MOM1D = 3 };

typedef struct {
  int kind;          /* O_REAL1D, O_REALSPACE, O_MOM1D */
  int fermion;       /* 1: FermiFS address (HubbardRealSpace only) */
  int N, M;
  double u, t;
  int ndim;          /* HubbardRealSpace geometry */
  int dims[3];
  int periodic[3];
  const double *pot; /* HubbardRealSpace trap energy per site (two components: 2M, component
                        1 first), or NULL */
  const double *kes; /* HubbardMom1D dispersion per mode */
  /* C = ncomp >= 2 components: the key holds the last component in its low bits, the one
   * before it above them, and so on (component 1 highest); the ONR of such an address is
   * component 1's M modes, then component 2's, and so on. */
  int ncomp;             /* 1 .. O_MAXC */
  int cferm[O_MAXC];     /* FermiFS (1) or BoseFS (0) per component */
  int cN[O_MAXC];        /* particles per component */
  double ct[O_MAXC];     /* HubbardRealSpace t per component */
  double cu[O_MAXC * (O_MAXC + 1) / 2];   /* HubbardRealSpace u, upper triangle row by row */
} o_model;

static int o_comp_bits(const o_model *h, int c) {
  return h->cferm[c] ? h->M : h->cN[c] + h->M - 1;
}
/* u[i, j] (0-based, i <= j) in the upper triangle of the C x C matrix, row by row */
static double o_cu(const o_model *h, int i, int j) {
  return h->cu[i * h->ncomp - i * (i - 1) / 2 + (j - i)];
}
static void o_to_onr(const o_model *h, okey key, int *onr) {
  if (h->ncomp >= 2) {
    for (int c = h->ncomp - 1; c >= 0; --c) {
      int b = o_comp_bits(h, c);
      okey kc = key & ((OKEY_ONE << b) - 1);
      key >>= b;
      if (h->cferm[c]) o_fermi_to_onr_k(kc, h->M, onr + c * h->M);
      else o_bose_to_onr_k(kc, h->M, onr + c * h->M);
    }
    return;
  }
  if (h->fermion) o_fermi_to_onr_k(key, h->M, onr); else o_bose_to_onr_k(key, h->M, onr);
}
static okey o_from_onr(const o_model *h, const int *onr) {
  if (h->ncomp >= 2) {
    okey key = 0;
    for (int c = 0; c < h->ncomp; ++c) {
      const int *oc = onr + c * h->M;
      okey kc = h->cferm[c] ? o_fermi_from_onr_k(oc, h->M) : o_bose_from_onr_k(oc, h->M);
      key = (key << o_comp_bits(h, c)) | kc;
    }
    return key;
  }
  return h->fermion ? o_fermi_from_onr_k(onr, h->M) : o_bose_from_onr_k(onr, h->M);
}
static int o_num_occupied(const int *onr, int M) {
  int c = 0;
  for (int i = 0; i < M; ++i) c += onr[i] > 0;
  return c;
}
/* k-th occupied mode (1-based k), returns 0-based mode index or -1
 * (find_occupied_mode, fockaddress.jl:115-125). */
static int o_find_occupied(const int *onr, int M, int k) {
  for (int i = 0; i < M; ++i) if (onr[i] > 0 && --k == 0) return i;
  return -1;
}

/* neighbor_site(geometry, mode, chosen): geometry.jl:127-139,161-181,232-235.
 * mode is 0-based here, chosen is 1-based; returns 0-based site or -1 if illegal. */
static int o_neighbor_site(const o_model *h, int mode, int chosen) {
  int D = h->ndim, x[3] = {0, 0, 0}, rem = mode;
  for (int d = 0; d < D; ++d) { x[d] = rem % h->dims[d]; rem /= h->dims[d]; }
  int dir = chosen <= D ? chosen - 1 : chosen - D - 1;
  int step = chosen <= D ? 1 : -1;
  x[dir] += step;
  if (x[dir] < 0 || x[dir] >= h->dims[dir]) {
    if (!h->periodic[dir]) return -1;
    x[dir] = (x[dir] + h->dims[dir]) % h->dims[dir];
  }
  int site = 0;
  for (int d = D - 1; d >= 0; --d) site = site * h->dims[d] + x[d];
  return site;
}

static int o_noff(const o_model *h, okey key) {
  int onr[O_MAXC * O_MAXM];
  o_to_onr(h, key, onr);
  if (h->ncomp >= 2) {
    if (h->kind == O_MOM1D) return h->cN[0] * h->cN[1] * (h->M - 1);   /* HubbardMom1D.jl:141-144 */
    /* each component's hops (HubbardRealSpace.jl:316-321, 366-371) */
    int s = 0;
    for (int c = 0; c < h->ncomp; ++c) s += o_num_occupied(onr + c * h->M, h->M);
    return s * 2 * h->ndim;
  }
  int s = o_num_occupied(onr, h->M);
  if (h->kind == O_REAL1D) return 2 * s;                        /* HubbardReal1D.jl:51-53 */
  if (h->kind == O_REALSPACE) return s * 2 * h->ndim;           /* HubbardRealSpace.jl:316-321 */
  int d = 0;                                                    /* HubbardMom1D.jl:103-140 */
  for (int i = 0; i < h->M; ++i) d += onr[i] > 1;
  return s * (s - 1) * (h->M - 2) + d * (h->M - 1);
}

/* Fermionic single excitation sign (fermi_excitation, bitstring.jl:746-791).
 * Returns 0 for an illegal move, else +1/-1; updates onr. */
static int o_fermi_hop(int *onr, int src, int dst) {
  if (!onr[src] || onr[dst]) return 0;
  int count = 0;
  for (int k = 0; k < src; ++k) count += onr[k];
  onr[src] = 0;
  for (int k = 0; k < dst; ++k) count += onr[k];
  onr[dst] = 1;
  return (count % 2 == 0) ? 1 : -1;
}

/* Hamiltonian matrix element of offdiagonal `chosen` (1-based) of column `key`:
 * returns the new address and H_{new,key}; *prod receives the integer under the square
 * root of the element (0 for an illegal move). */
/* One component's HubbardRealSpace hop on its ONR (HubbardRealSpace.jl:325-338): returns the
 * matrix element -t * excitation value and the product under the square root; onr updated. */
static double o_realspace_hop(const o_model *h, int *onr, int fermion, double t, int chosen,
                              long *prod) {
  int M = h->M, nb = 2 * h->ndim;
  int particle = (chosen - 1) / nb + 1, neigh = (chosen - 1) % nb + 1;
  int src = o_find_occupied(onr, M, particle);
  int dst = o_neighbor_site(h, src, neigh);
  *prod = 0;
  if (dst < 0) return 0.0;
  if (fermion) {
    int sgn = o_fermi_hop(onr, src, dst);
    if (!sgn) return 0.0;
    *prod = 1;
    return -t * (double)sgn;
  }
  int value = onr[src] * (onr[dst] + 1);   /* bose_excitation_value, fockaddress.jl:559-567 */
  *prod = value;
  onr[src] -= 1;
  onr[dst] += 1;
  return -t * sqrt((double)value);
}

static void o_offdiag_k(const o_model *h, okey key, int chosen, okey *nkey, double *val,
                        long *prod) {
  int onr[O_MAXC * O_MAXM];
  *prod = 0;
  o_to_onr(h, key, onr);
  int M = h->M;
  if (h->ncomp >= 2 && h->kind == O_REALSPACE) {
    /* component 1's hops, then component 2's, and so on (HubbardRealSpace.jl:344-391) */
    int c = 0;
    for (;;) {
      int nc = o_num_occupied(onr + c * M, M) * 2 * h->ndim;
      if (chosen <= nc || c + 1 == h->ncomp) break;
      chosen -= nc;
      ++c;
    }
    double v = o_realspace_hop(h, onr + c * M, h->cferm[c], h->ct[c], chosen, prod);
    if (*prod == 0) { *nkey = key; *val = 0.0; return; }
    *nkey = o_from_onr(h, onr);
    *val = v;
    return;
  }
  if (h->ncomp >= 2) {
    /* FermiFS2C: momentum_transfer_excitation of two components, fold=true
     * (excitations.jl:82-119); element u/M * (val_a * val_b) (HubbardMom1D.jl:196-205) */
    int *oa = onr, *ob = onr + M;
    int nbn = h->cN[1];
    int src_a, rem, dst_a, src_b;
    src_a = (chosen - 1) / ((M - 1) * nbn) + 1;          /* fldmod1(chosen, (M-1)*N_b) */
    rem = (chosen - 1) % ((M - 1) * nbn) + 1;
    dst_a = (rem - 1) / nbn + 1;                          /* fldmod1(rem, N_b) */
    src_b = (rem - 1) % nbn + 1;
    int sa = o_find_occupied(oa, M, src_a) + 1, sb = o_find_occupied(ob, M, src_b) + 1;
    if (dst_a >= sa) dst_a += 1;
    int mom = dst_a - sa;
    int dst_b = sb - mom;
    dst_a = ((dst_a - 1) % M + M) % M + 1;                /* mod1 */
    dst_b = ((dst_b - 1) % M + M) % M + 1;
    int ga = o_fermi_hop(oa, sa - 1, dst_a - 1);
    int gb = ga ? o_fermi_hop(ob, sb - 1, dst_b - 1) : 0;
    if (!ga || !gb) { *nkey = key; *val = 0.0; return; }
    *nkey = o_from_onr(h, onr);
    *prod = 4;
    *val = h->u / M * ((double)ga * (double)gb);
    return;
  }
  if (h->kind == O_REAL1D) {
    /* hopnextneighbour restated on the ONR, as in test/BitStringAddresses.jl:251-267. */
    int site = (chosen + 1) / 2;
    int i = o_find_occupied(onr, M, site);
    int j = (chosen % 2 == 1) ? (i + 1) % M : (i - 1 + M) % M;
    *prod = (long)onr[i] * (onr[j] + 1);
    onr[i] -= 1;
    onr[j] += 1;
    *nkey = o_from_onr(h, onr);
    *val = -h->t * sqrt((double)((onr[i] + 1) * onr[j]));
    return;
  }
  if (h->kind == O_REALSPACE) {
    int nb = 2 * h->ndim;
    int particle = (chosen - 1) / nb + 1, neigh = (chosen - 1) % nb + 1;
    int src = o_find_occupied(onr, M, particle);
    int dst = o_neighbor_site(h, src, neigh);
    if (dst < 0) { *nkey = key; *val = 0.0; return; }
    if (h->fermion) {
      int sgn = o_fermi_hop(onr, src, dst);
      if (!sgn) { *nkey = key; *val = 0.0; return; }
      *nkey = o_from_onr(h, onr);
      *val = -h->t * (double)sgn;
      *prod = 1;
      return;
    }
    int value = onr[src] * (onr[dst] + 1);   /* bose_excitation_value, fockaddress.jl:559-567 */
    *prod = value;
    onr[src] -= 1;
    onr[dst] += 1;
    *nkey = o_from_onr(h, onr);
    *val = -h->t * sqrt((double)value);
    return;
  }
  /* HubbardMom1D: momentum_transfer_excitation with fold=true, excitations.jl:26-80. */
  int map_mode[O_MAXM], map_occ[O_MAXM], s = 0;
  for (int i = 0; i < M; ++i) if (onr[i] > 0) { map_mode[s] = i + 1; map_occ[s] = onr[i]; ++s; }
  int dbl = chosen - s * (s - 1) * (M - 2);
  int p_idx, q_idx, mom_change;
  if (dbl > 0) {
    int which = (dbl - 1) / (M - 1) + 1;
    mom_change = (dbl - 1) % (M - 1) + 1;
    int idx = 0;
    for (int k = 0; k < s; ++k) {
      which -= map_occ[k] >= 2;
      if (which == 0) { idx = k; break; }
    }
    p_idx = q_idx = idx;
  } else {
    int pair = (chosen - 1) / (M - 2) + 1;
    mom_change = (chosen - 1) % (M - 2) + 1;
    int fst = (pair - 1) / (s - 1) + 1, snd = (pair - 1) % (s - 1) + 1;
    int f_hole, s_hole;
    if (snd < fst) { f_hole = snd; s_hole = fst; } else { f_hole = fst; s_hole = snd + 1; }
    p_idx = f_hole - 1;
    q_idx = s_hole - 1;
    if (mom_change >= map_mode[q_idx] - map_mode[p_idx]) mom_change += 1;
  }
  int src1 = map_mode[p_idx], src2 = map_mode[q_idx];
  int dst1 = ((src1 + mom_change - 1) % M + M) % M + 1;
  int dst2 = ((src2 - mom_change - 1) % M + M) % M + 1;
  /* a†_{dst1} a†_{dst2} a_{src2} a_{src1}: destroy then create, multiplying occupations. */
  long value = 1;
  value *= onr[src2 - 1]; onr[src2 - 1] -= 1;
  value *= onr[src1 - 1]; onr[src1 - 1] -= 1;
  value *= onr[dst2 - 1] + 1; onr[dst2 - 1] += 1;
  value *= onr[dst1 - 1] + 1; onr[dst1 - 1] += 1;
  if (value == 0) { *nkey = key; *val = 0.0; return; }
  *nkey = o_from_onr(h, onr);
  *prod = value;
  /* get_offdiagonal: ham.u/(2*M)*onproduct, HubbardMom1D.jl:189-194 */
  *val = h->u / (2 * M) * sqrt((double)value);
}

int o_num_offdiagonals(const o_model *h, uint64_t key) { return o_noff(h, key); }
void o_get_offdiagonal_p(const o_model *h, uint64_t key, int chosen, uint64_t *nkey,
                         double *val, long *prod) {
  okey nk;
  o_offdiag_k(h, key, chosen, &nk, val, prod);
  *nkey = o_lo(nk);
}
void o_get_offdiagonal(const o_model *h, uint64_t key, int chosen, uint64_t *nkey, double *val) {
  long prod;
  o_get_offdiagonal_p(h, key, chosen, nkey, val, &prod);
}
/* Two-word forms: keys as (lo, hi). */
int o_num_offdiagonals_w(const o_model *h, uint64_t lo, uint64_t hi) {
  return o_noff(h, o_key_of(lo, hi));
}
void o_get_offdiagonal_w(const o_model *h, uint64_t lo, uint64_t hi, int chosen, uint64_t *nkey2,
                         double *val) {
  okey nk;
  long prod;
  o_offdiag_k(h, o_key_of(lo, hi), chosen, &nk, val, &prod);
  nkey2[0] = o_lo(nk);
  nkey2[1] = o_hi(nk);
}

/* external_potential of one component (HubbardRealSpace.jl:90-97). */
static double o_potential(const int *onr, int M, const double *pot) {
  double pe = 0.0;
  for (int i = 0; i < M; ++i) if (onr[i]) pe += onr[i] * pot[i];
  return pe;
}

static double o_diag_k(const o_model *h, okey key);
double o_diagonal(const o_model *h, uint64_t key) { return o_diag_k(h, key); }
double o_diagonal_w(const o_model *h, uint64_t lo, uint64_t hi) { return o_diag_k(h, o_key_of(lo, hi)); }

static double o_diag_k(const o_model *h, okey key) {
  int onr[O_MAXC * O_MAXM];
  o_to_onr(h, key, onr);
  int M = h->M;
  if (h->ncomp == 2 && h->kind == O_MOM1D) {
    /* dot(kes, map_a) + dot(kes, map_b) + u/2M * 2 n_a n_b (HubbardMom1D.jl:182-187) */
    double ka = 0.0, kb = 0.0;
    long na = 0, nb = 0;
    for (int i = 0; i < M; ++i) if (onr[i]) { ka += h->kes[i] * 1; ++na; }
    for (int i = 0; i < M; ++i) if (onr[M + i]) { kb += h->kes[i] * 1; ++nb; }
    return ka + kb + h->u / (2 * M) * (double)(2 * na * nb);
  }
  if (h->ncomp >= 2) {
    /* local_interaction(CompositeFS, u) = _interactions(components, u) (HubbardRealSpace.jl:
     * 18-61), evaluated as the reference's recursion does:
     *   _interactions((a, as...)) = self + row + _interactions(as),  _interactions(()) = 0.0,
     *   row = _interaction_col(a, as) = li(a, b1) + (li(a, b2) + (... + 0)),
     * where self = u[s,s] * bose_hubbard_interaction / 2 for a BoseFS and the integer 0 for a
     * FermiFS, li(a, b) = u[s,j] * dot(occupations), and the closing 0 of _interaction_col is
     * an integer: integer 0 + double x is 0.0 + x.  Here the integer zeros are the flags
     * *_int.  Then the trap, pe = 0.0 + pot_1 + pot_2 + ... (:100-107); diagonal = int + pot
     * (:284-287).  The interaction term is 0.0 when u is all zero (h.u === nothing). */
    const int C = h->ncomp;
    int any_u = 0;
    for (int i = 0; i < C * (C + 1) / 2; ++i) any_u |= h->cu[i] != 0.0;
    double in = 0.0;
    if (any_u) {
      double rest = 0.0;
      for (int s2 = C - 1; s2 >= 0; --s2) {
        const int *os = onr + s2 * M;
        double row = 0.0;
        int row_int = 1;
        for (int j = C - 1; j > s2; --j) {
          long dot = 0;
          for (int i = 0; i < M; ++i) dot += (long)os[i] * onr[j * M + i];
          double li = o_cu(h, s2, j) * (double)dot;
          row = row_int ? li + 0.0 : li + row;
          row_int = 0;
        }
        double first;
        int first_int;
        if (h->cferm[s2]) {
          first = row_int ? 0.0 : 0.0 + row;
          first_int = row_int;
        } else {
          long bhi = 0;
          for (int i = 0; i < M; ++i) bhi += (long)os[i] * (os[i] - 1);
          double self = o_cu(h, s2, s2) * (double)bhi / 2;
          first = row_int ? self + 0.0 : self + row;
          first_int = 0;
        }
        rest = first_int ? 0.0 + rest : first + rest;
      }
      in = rest;
    }
    double pe = 0.0;
    if (h->pot) {
      for (int c = 0; c < C; ++c) pe += o_potential(onr + c * M, M, h->pot + c * M);
    }
    return in + pe;
  }
  if (h->kind == O_REAL1D) {
    long bhi = 0;
    for (int i = 0; i < M; ++i) bhi += (long)onr[i] * (onr[i] - 1);
    return h->u * (double)bhi / 2;                         /* HubbardReal1D.jl:55-57 */
  }
  if (h->kind == O_REALSPACE) {
    double in = 0.0;
    if (!h->fermion && h->u != 0.0) {
      long bhi = 0;
      for (int i = 0; i < M; ++i) bhi += (long)onr[i] * (onr[i] - 1);
      in = h->u * (double)bhi / 2;                         /* HubbardRealSpace.jl:18 */
    }
    double pe = 0.0;
    if (h->pot) for (int i = 0; i < M; ++i) if (onr[i]) pe += onr[i] * h->pot[i];
    return in + pe;                                        /* HubbardRealSpace.jl:284-293 */
  }
  double kin = 0.0;                                        /* fockaddress.jl:316-322 */
  long onp = 0;                                            /* excitations.jl:126-137 */
  int occ[O_MAXM], s = 0;
  for (int i = 0; i < M; ++i) if (onr[i]) { kin += h->kes[i] * onr[i]; occ[s++] = onr[i]; }
  for (int i = 0; i < s; ++i) {
    onp += (long)occ[i] * (occ[i] - 1);
    for (int j = 0; j < i; ++j) onp += 4L * occ[i] * occ[j];
  }
  return kin + h->u / (2 * M) * (double)onp;               /* HubbardMom1D.jl:163-177 */
}

/* ------------------------------------------------------------------------------------ */
/* FCIQMC step                                                                           */
/* ------------------------------------------------------------------------------------ */
enum { O_STYLE_INTEGER = 0, O_STYLE_DETERMINISTIC = 1, O_STYLE_DSS = 2 };
enum { O_OP_TRANSITION = 0, O_OP_HAMILTONIAN = 1 };

typedef struct {
  int style;            /* O_STYLE_* */
  int op;               /* O_OP_TRANSITION: T = 1 + dt (S - H); O_OP_HAMILTONIAN: H */
  double dt, shift;
  double boost;
  double proj_threshold;       /* on-the-fly projection threshold (0: none) */
  double compression;          /* ThresholdCompression threshold (0: no compression) */
  double rel_threshold, abs_threshold; /* DynamicSemistochastic thresholds */
  uint64_t seed;
  uint32_t step;
  uint32_t replica;
  int init_rule;               /* O_INIT_*: initiator rule of an InitiatorDVec (initiators.jl) */
  double init_threshold;       /* its threshold: initiators have |value| > threshold */
} o_params;

/* Initiator rules (initiators.jl:132-234) and the classes of a contribution
 * (_default_to_initiator_value, initiators.jl:142-157). */
enum { O_INIT_NONE = 0, O_INIT_INITIATOR = 1, O_INIT_SIMPLE = 2, O_INIT_COHERENT = 3 };
enum { O_CLS_SAFE = 0, O_CLS_UNSAFE = 1, O_CLS_INITIATOR = 2 };

typedef struct {
  double norm;          /* walkernumber after the step */
  int64_t len;
  int64_t len_before;   /* ThresholdCompression statistic */
  int64_t exact_steps, inexact_steps, spawn_attempts;
  double spawns;        /* sum of |deposited spawn| */
  int64_t clones, deaths, zombies;   /* IsStochasticInteger only */
} o_stats;

typedef struct { okey key; int cls; int kind; double v; int64_t iv; } o_contrib;

static uint64_t o_ordered_bits(double v) {
  uint64_t u;
  memcpy(&u, &v, 8);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
static int o_cmp_contrib_f(const void *a, const void *b) {
  const o_contrib *x = a, *y = b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  if (x->cls != y->cls) return x->cls < y->cls ? -1 : 1;
  if (x->kind != y->kind) return x->kind < y->kind ? -1 : 1;
  uint64_t ox = o_ordered_bits(x->v), oy = o_ordered_bits(y->v);
  return ox < oy ? -1 : ox > oy;
}
static int o_cmp_contrib_i(const void *a, const void *b) {
  const o_contrib *x = a, *y = b;
  if (x->key != y->key) return x->key < y->key ? -1 : 1;
  if (x->cls != y->cls) return x->cls < y->cls ? -1 : 1;
  if (x->kind != y->kind) return x->kind < y->kind ? -1 : 1;
  return x->iv < y->iv ? -1 : x->iv > y->iv;
}

typedef struct { o_contrib *c; int64_t n, cap; int err; } o_buf;
static void o_push(o_buf *b, okey key, int cls, int kind, double v, int64_t iv) {
  if (b->n == b->cap) {
    int64_t nc = b->cap ? 2 * b->cap : 1024;
    o_contrib *p = realloc(b->c, nc * sizeof(o_contrib));
    if (!p) { b->err = 1; return; }
    b->c = p; b->cap = nc;
  }
  b->c[b->n].key = key; b->c[b->n].cls = cls; b->c[b->n].kind = kind; b->c[b->n].v = v;
  b->c[b->n].iv = iv;
  b->n++;
}

/* Transition operator elements (fciqmc.jl:93-112). */
static double o_t_diag(const o_model *h, const o_params *p, okey key) {
  double d = o_diag_k(h, key);
  return p->op == O_OP_HAMILTONIAN ? d : 1 - p->dt * (d - p->shift);
}
static double o_t_off(const o_params *p, double hval) {
  return p->op == O_OP_HAMILTONIAN ? hval : -hval * p->dt;
}

/* Integer stochastic rounding (spawning.jl:33-45): sign(x) * floor(|x| + r), restated as
 * floor(|x|) + [r < frac(|x|)] with the comparison evaluated exactly. */
static int64_t o_round_int(double x, uint64_t u53) {
  double ax = fabs(x);
  double k = floor(ax);
  double f = ax - k;
  int64_t n = (int64_t)k + (o_bernoulli(u53, f) ? 1 : 0);
  return x < 0 ? -n : n;
}
/* Threshold projection for floats (spawning.jl:13-31). */
static double o_project(double x, double thresh, uint64_t u53) {
  double ax = fabs(x);
  if (ax < thresh) {
    double prob = (thresh == 1.0) ? ax : ax / thresh;
    if (o_bernoulli(u53, prob)) return x < 0 ? -thresh : thresh;
    return 0.0;
  }
  return x;
}

/* 1/n as used by the spawn-amplitude factor: (val * (1/n_att)) * n_off. */
static double o_recip(int64_t n) { return 1.0 / (double)n; }

/* Integer part of a non-negative double below 2^62. */
static int64_t o_floor_i(double x) { return (int64_t)floor(x); }

/* Unsigned 128-bit fixed point (2^-64 units) used for exact, order-independent norms. */
typedef unsigned __int128 o_u128;
static o_u128 o_fixed(double ax) {
  if (ax == 0.0) return 0;
  int e;
  double m = frexp(ax, &e);                /* ax = m * 2^e, m in [0.5, 1) */
  uint64_t mant = (uint64_t)ldexp(m, 53);  /* 53-bit integer, ax = mant * 2^(e-53) */
  int sh = e - 53 + 64;                    /* fixed = mant * 2^sh */
  if (sh >= 0) return sh >= 75 ? ~(o_u128)0 : ((o_u128)mant) << sh;
  if (-sh >= 64) return 0;
  return (o_u128)(mant >> (-sh));
}
static double o_fixed_to_double(o_u128 x) {
  return ldexp((double)x, -64);
}

/* x as a signed multiple of 2^-64, if it is one and |x| < 2^48 (so that up to 2^15
 * contributions cannot overflow the 128-bit sum). */
static int o_to_fixed(double x, __int128 *out) {
  if (x == 0.0) { *out = 0; return 1; }
  double ax = fabs(x);
  if (!(ax < 281474976710656.0)) return 0;             /* 2^48 */
  double scaled = ldexp(ax, 64);
  if (scaled != floor(scaled)) return 0;               /* bits below 2^-64 */
  /* scaled < 2^112: split into two 64-bit halves exactly */
  double hi = floor(ldexp(scaled, -64));
  double lo = scaled - ldexp(hi, 64);
  unsigned __int128 u = ((unsigned __int128)(uint64_t)hi << 64) | (uint64_t)lo;
  *out = x < 0 ? -(__int128)u : (__int128)u;
  return 1;
}
/* Nearest double (ties to even) of fx * 2^-64, computed on the integer. */
static double o_fixed_signed_to_double(__int128 fx) {
  if (fx == 0) return 0.0;
  int neg = fx < 0;
  unsigned __int128 u = neg ? (unsigned __int128)(-fx) : (unsigned __int128)fx;
  int top = 127;
  while (!((u >> top) & 1)) --top;
  double r;
  if (top <= 52) {
    r = ldexp((double)(uint64_t)u, -64);
  } else {
    int drop = top - 52;
    unsigned __int128 m = u >> drop;
    unsigned __int128 rem = u & ((((unsigned __int128)1) << drop) - 1);
    unsigned __int128 half = ((unsigned __int128)1) << (drop - 1);
    if (rem > half || (rem == half && (m & 1))) m += 1;
    r = ldexp((double)(uint64_t)m, drop - 64);     /* m <= 2^53: exact */
  }
  return neg ? -r : r;
}

/* Value of an address from its field sums by the initiator rule (from_initiator_value,
 * initiators.jl:138-140, 181-183, 208-214); without a rule every contribution is "safe". */
static void o_initiator_value(const o_params *p, const double f[3], const int64_t n[3],
                              double *s, int64_t *si) {
  const double fs = f[O_CLS_SAFE], fu = f[O_CLS_UNSAFE], fi = f[O_CLS_INITIATOR];
  const int64_t ns = n[O_CLS_SAFE], nu = n[O_CLS_UNSAFE], ni = n[O_CLS_INITIATOR];
  switch (p->init_rule) {
    case O_INIT_INITIATOR:      /* safe + initiator + !iszero(initiator) * unsafe */
      *s = fs + fi;
      if (fi != 0.0) *s = *s + fu;
      *si = ns + ni + (ni != 0 ? nu : 0);
      return;
    case O_INIT_SIMPLE:         /* safe + initiator */
      *s = fs + fi;
      *si = ns + ni;
      return;
    case O_INIT_COHERENT:       /* initiator + safe (+ unsafe if initiator or |unsafe| > threshold) */
      *s = fi + fs;
      if (fi != 0.0 || fabs(fu) > p->init_threshold) *s = *s + fu;
      *si = ni + ns;
      if (ni != 0 || fabs((double)nu) > p->init_threshold) *si += nu;
      return;
    default:
      *s = fs;
      *si = ns;
  }
}

/* Receiver of the contributions of one column: (target address, class, kind 0 = diagonal
 * term / 1 = spawn, float value, integer value). */
typedef void (*o_emit_fn)(void *ctx, okey key, int cls, int kind, double v, int64_t iv);

/* The contributions of one source walker (apply_column!, styles.jl:21-25, 101-105, 210-214):
 * its diagonal step and its spawns, handed to `emit`; the statistics go to *st and the spawn
 * magnitudes (float walkers) to *spawn_acc in exact fixed point. */
/* HubbardReal1D on the bit string, for the threaded step's comparator runs: the reference's
 * own bit-level algorithms on one chunk, hopnextneighbour (bosefs.jl:297-345) walking the
 * occupied modes with trailing_zeros/trailing_ones (occupied_modes, bitstring.jl:636-656) and
 * bose_hubbard_interaction (bosefs.jl:415-428).  Same keys and values as the ONR functions
 * (tests/test_oracle_threaded.py checks every basis state of several sizes). */
static inline int o_tz(uint64_t x) { return x ? __builtin_ctzll(x) : 64; }
static inline uint64_t o_shr(uint64_t x, int s) { return s >= 64 ? 0 : x >> s; }
static long o_bits_interaction(uint64_t chunk) {
  long acc = 0;
  while (chunk) {
    chunk = o_shr(chunk, o_tz(chunk));             /* proceed to the next occupied mode */
    const int n = o_tz(~chunk);                    /* bosons in it */
    chunk = o_shr(chunk, n);
    acc += (long)n * (n - 1);
  }
  return acc;
}
static int o_bits_noff(uint64_t a) { return 2 * __builtin_popcountll(a & ~(a << 1)); }
static void o_bits_hop(uint64_t a, int N, int M, int chosen, uint64_t *nk, long *prod) {
  const int B = N + M - 1;
  const uint64_t mask = B >= 64 ? ~0ull : ((1ull << B) - 1);
  const int site = (chosen + 1) >> 1;
  if (chosen & 1) {                                /* hop to the right */
    long next = 0, curr = 0;
    int offset = 0, sc = 0, reached_end = 0, i = 0, mode = 1, bit = 0;
    uint64_t x = a;
    while (x) {
      const int z = o_tz(x);
      x = o_shr(x, z); mode += z; bit += z;
      const int num = o_tz(~x);
      ++i;
      next = (long)num * (mode == sc + 1);
      reached_end = i == site + 1;
      if (reached_end) break;
      curr = num; offset = bit + num; sc = mode;
      x = o_shr(x, num); bit += num;
    }
    if (sc == M) {
      *nk = ((a << 1) | 1) & mask;
      *prod = curr * (o_tz(~a) + 1);
    } else {
      next *= reached_end;
      *nk = a ^ (3ull << (offset - 1));
      *prod = curr * (next + 1);
    }
    return;
  }
  if (site == 1 && (a & 1)) {                      /* leftmost site: rotate by one bit */
    const uint64_t na = (a >> 1) | (1ull << (B - 1));
    int lead = 0;
    for (int b = B - 1; b >= 0 && ((na >> b) & 1); --b) ++lead;
    *nk = na;
    *prod = (long)o_tz(~a) * lead;
    return;
  }
  long prev = 0, curr = 0;
  int offset = 0, sp = 0, i = 0, mode = 1, bit = 0;
  uint64_t x = a;
  while (x) {
    const int z = o_tz(x);
    x = o_shr(x, z); mode += z; bit += z;
    const int num = o_tz(~x);
    ++i;
    prev = curr * (mode == sp + 1);
    curr = num;
    offset = bit;
    if (i == site) break;
    sp = mode;
    x = o_shr(x, num); bit += num;
  }
  *nk = a ^ (3ull << (offset - 1));
  *prod = curr * (prev + 1);
}

/* Exported for the tests: key and value of offdiagonal `chosen` by the bit-level path. */
void o_real1d_bits_offdiag(const o_model *h, uint64_t key, int chosen, uint64_t *nkey,
                           double *val) {
  long prod;
  o_bits_hop(key, h->N, h->M, chosen, nkey, &prod);
  *val = -h->t * sqrt((double)prod);
}
double o_real1d_bits_diagonal(const o_model *h, uint64_t key) {
  return h->u * (double)o_bits_interaction(key) / 2;
}

static int o_use_bits(const o_model *h) {
  return h->kind == O_REAL1D && h->ncomp < 2 && h->N + h->M - 1 <= 64;
}
static int o_noff_f(const o_model *h, okey key, int fast) {
  return fast ? o_bits_noff(o_lo(key)) : o_noff(h, key);
}
static double o_t_diag_f(const o_model *h, const o_params *p, okey key, int fast) {
  if (!fast) return o_t_diag(h, p, key);
  const double d = h->u * (double)o_bits_interaction(o_lo(key)) / 2;   /* HubbardReal1D.jl:55-57 */
  return p->op == O_OP_HAMILTONIAN ? d : 1 - p->dt * (d - p->shift);
}
static void o_offdiag_f(const o_model *h, okey key, int chosen, okey *nkey, double *val,
                        long *prod, int fast) {
  if (!fast) { o_offdiag_k(h, key, chosen, nkey, val, prod); return; }
  uint64_t nk;
  o_bits_hop(o_lo(key), h->N, h->M, chosen, &nk, prod);
  *nkey = (okey)nk;
  *val = -h->t * sqrt((double)*prod);                /* HubbardReal1D.jl:59-62 */
}

static void o_apply_column(const o_model *h, const o_params *p, okey key, double sval,
                           int64_t sival, o_emit_fn emit, void *ctx, o_stats *st,
                           o_u128 *spawn_acc, int fast) {
  const int is_int = p->style == O_STYLE_INTEGER;
  double val = is_int ? (double)sival : sval;
  /* classes of this walker's contributions (_default_to_initiator_value,
   * initiators.jl:142-157): its diagonal term counts as "initiator" and its spawns as
   * "safe" when |value| > threshold, else as "safe" and "unsafe" */
  const int parent_init = fabs(val) > p->init_threshold;
  const int diag_cls = p->init_rule == O_INIT_NONE ? O_CLS_SAFE
                                                    : (parent_init ? O_CLS_INITIATOR : O_CLS_SAFE);
  const int spawn_cls = p->init_rule == O_INIT_NONE ? O_CLS_SAFE
                                                     : (parent_init ? O_CLS_SAFE : O_CLS_UNSAFE);
  /* ---- diagonal_step! (spawning.jl:73-77) ---- */
  double x = o_t_diag_f(h, p, key, fast) * val;
  if (is_int) {
    uint32_t r[4];
    o_draw_k(p->seed, O_PURPOSE_DIAG, p->replica, p->step, key, 0, r);
    int64_t res = o_round_int(x, o_u53(r));
    int64_t v = sival;
    if (res != 0) emit(ctx, key, diag_cls, 0, 0.0, res);
    /* clones_deaths_zombies, spawning.jl:79-93 */
    int sr = (res > 0) - (res < 0), sv = (v > 0) - (v < 0);
    if (res > v) st->clones += res - v;
    else if (sr != sv) { st->deaths += v < 0 ? -v : v; st->zombies += res < 0 ? -res : res; }
    else st->deaths += (res - v) < 0 ? v - res : res - v;
  } else {
    double res = x;
    if (p->proj_threshold > 0) {
      uint32_t r[4];
      o_draw_k(p->seed, O_PURPOSE_DIAG, p->replica, p->step, key, 0, r);
      res = o_project(x, p->proj_threshold, o_u53(r));
    }
    if (res != 0.0) emit(ctx, key, diag_cls, 0, res, 0);
  }
  /* ---- spawn! ---- */
  int noff = o_noff_f(h, key, fast);
  int exact = 0;
  if (p->style == O_STYLE_DETERMINISTIC) {
    exact = 1;                       /* apply_column! returns (1,), styles.jl:101-105 */
    st->exact_steps++;
  } else if (p->style == O_STYLE_DSS) {
    /* DynamicSemistochastic, spawning.jl:364-378 */
    double thresh = p->abs_threshold < (double)noff ? p->abs_threshold : (double)noff;
    double amount = p->boost * fabs(val) * p->rel_threshold;
    exact = amount >= thresh;
    if (exact) st->exact_steps++; else st->inexact_steps++;
  }
  /* IsStochasticInteger always samples (WithReplacement); a column without offdiagonals
   * has nothing to sample from. */
  if (noff == 0) return;
  if (exact) {
    /* Exact, spawning.jl:174-182: deposit val * mat_elem for every offdiagonal. */
    st->spawn_attempts += noff;
    for (int c = 1; c <= noff; ++c) {
      okey nk; double hv; long prod;
      o_offdiag_f(h, key, c, &nk, &hv, &prod, fast);
      double y = val * o_t_off(p, hv);
      if (p->proj_threshold > 0 && p->style == O_STYLE_DSS) {
        uint32_t r[4];
        o_draw_k(p->seed, O_PURPOSE_SPAWN, p->replica, p->step, key, (uint32_t)(c - 1), r);
        y = o_project(y, p->proj_threshold, o_u53(r));
      }
      if (y != 0.0) { emit(ctx, nk, spawn_cls, 1, y, 0); *spawn_acc += o_fixed(fabs(y)); }
    }
    return;
  }
  /* WithReplacement, spawning.jl:232-243.  The per-attempt amplitude is
   * mat_elem * magnitude / prob with magnitude = val / n_att and prob = 1 / n_off; this
   * restatement evaluates it as mat_elem * ((val * (1/n_att)) * n_off), which is the same
   * value up to rounding.  For integer walkers with boost 1, val / n_att = sign(val). */
  int64_t natt = o_floor_i(fabs(val) * p->boost);
  if (natt < 1) natt = 1;
  st->spawn_attempts += natt;
  double c;
  if (is_int && p->boost == 1.0) c = (val < 0 ? -1.0 : 1.0) * (double)noff;
  else c = (val * o_recip(natt)) * (double)noff;
  /* Float walkers without on-the-fly projection need only the offdiagonal index per
   * attempt: attempt j takes word j % 4 of Philox block j / 4.  Otherwise attempt j uses
   * its own block: word 0 for the index, words 1-2 for the rounding. */
  const int grouped = !is_int && p->proj_threshold == 0;
  for (int64_t j = 0; j < natt; ++j) {
    uint32_t r[4];
    uint32_t word;
    if (grouped) {
      o_draw_k(p->seed, O_PURPOSE_SPAWN, p->replica, p->step, key, (uint32_t)(j >> 2), r);
      word = r[j & 3];
    } else {
      o_draw_k(p->seed, O_PURPOSE_SPAWN, p->replica, p->step, key, (uint32_t)j, r);
      word = r[0];
    }
    int chosen = (int)(((uint64_t)word * (uint64_t)noff) >> 32) + 1;
    okey nk; double hv; long prod;
    o_offdiag_f(h, key, chosen, &nk, &hv, &prod, fast);
    double y = c * o_t_off(p, hv);
    if (is_int) {
      int64_t k = o_round_int(y, o_u53(r));
      if (k != 0) { emit(ctx, nk, spawn_cls, 1, 0.0, k); st->spawns += (double)(k < 0 ? -k : k); }
    } else {
      if (p->proj_threshold > 0) y = o_project(y, p->proj_threshold, o_u53(r));
      if (y != 0.0) { emit(ctx, nk, spawn_cls, 1, y, 0); *spawn_acc += o_fixed(fabs(y)); }
    }
  }
}

static void o_emit_buf(void *ctx, okey key, int cls, int kind, double v, int64_t iv) {
  o_push((o_buf *)ctx, key, cls, kind, v, iv);
}

/* One apply_operator! step (dictvectors.jl:112-140) from `src` into a sorted `dst`.
 * Values are doubles for the float styles and int64 (separate arrays) for
 * IsStochasticInteger.  Returns 0 on success, nonzero on allocation failure.  *dst arrays
 * are malloc'd. */
static int o_step_k(const o_model *h, const o_params *p,
                    const okey *skeys, const double *svals, const int64_t *sivals, int64_t n,
                    okey **okeys, double **ovals, int64_t **oivals, int64_t *on, o_stats *st) {
  memset(st, 0, sizeof(*st));
  o_buf b = {0};
  int is_int = p->style == O_STYLE_INTEGER;
  o_u128 spawn_acc = 0;
  for (int64_t e = 0; e < n; ++e)
    o_apply_column(h, p, skeys[e], is_int ? 0.0 : svals[e], is_int ? sivals[e] : 0, o_emit_buf,
                   &b, st, &spawn_acc, 0);
  if (b.err) { free(b.c); return 1; }
  if (!is_int) st->spawns = o_fixed_to_double(spawn_acc);
  /* ---- annihilation: sum the contributions per address ----
   * Rule (the GPU follows it exactly): if every contribution to an address is a multiple of
   * 2^-64 with magnitude below 2^48, the result is the exact sum rounded once to the nearest
   * double (ties to even); otherwise the contributions are added in canonical order, the
   * diagonal term first and then the spawns in increasing numerical order. */
  qsort(b.c, (size_t)b.n, sizeof(o_contrib), is_int ? o_cmp_contrib_i : o_cmp_contrib_f);
  okey *ok = malloc((size_t)(b.n ? b.n : 1) * sizeof(okey));
  double *ov = malloc((size_t)(b.n ? b.n : 1) * 8);
  int64_t *oi = malloc((size_t)(b.n ? b.n : 1) * 8);
  if (!ok || !ov || !oi) { free(b.c); free(ok); free(ov); free(oi); return 1; }
  int64_t m = 0;
  for (int64_t i = 0; i < b.n;) {
    const okey key = b.c[i].key;
    double fs[3] = {0.0, 0.0, 0.0};
    int64_t is[3] = {0, 0, 0};
    int64_t j = i;
    while (j < b.n && b.c[j].key == key) {       /* one field (class) at a time */
      const int cls = b.c[j].cls;
      double s = 0.0;
      int64_t si = 0;
      int first = 1, exact = 1;
      __int128 fx = 0;
      while (j < b.n && b.c[j].key == key && b.c[j].cls == cls) {
        if (is_int) si += b.c[j].iv;
        else {
          s = first ? b.c[j].v : s + b.c[j].v;
          first = 0;
          __int128 t;
          if (exact && o_to_fixed(b.c[j].v, &t)) fx += t; else exact = 0;
        }
        ++j;
      }
      if (!is_int && exact) s = o_fixed_signed_to_double(fx);
      fs[cls] = s;
      is[cls] = si;
    }
    double s;
    int64_t si;
    o_initiator_value(p, fs, is, &s, &si);
    if (is_int ? si != 0 : s != 0.0) { ok[m] = key; ov[m] = s; oi[m] = si; ++m; }
    i = j;
  }
  free(b.c);
  /* ---- compression (compression.jl:18-42) ---- */
  st->len_before = m;
  if (!is_int && p->compression > 0) {
    int64_t q = 0;
    for (int64_t i = 0; i < m; ++i) {
      double w = ov[i];
      double prob = (p->compression == 1.0) ? fabs(w) : fabs(w) / p->compression;
      if (prob < 1) {
        uint32_t r[4];
        o_draw_k(p->seed, O_PURPOSE_COMPRESS, p->replica, p->step, ok[i], 0, r);
        w = o_bernoulli(o_u53(r), prob) ? (w < 0 ? -p->compression : p->compression) : 0.0;
      }
      if (w != 0.0) { ok[q] = ok[i]; ov[q] = w; oi[q] = 0; ++q; }
    }
    m = q;
  }
  o_u128 acc = 0;
  for (int64_t i = 0; i < m; ++i) acc += o_fixed(fabs(is_int ? (double)oi[i] : ov[i]));
  st->norm = o_fixed_to_double(acc);
  st->len = m;
  *okeys = ok; *ovals = ov; *oivals = oi; *on = m;
  return 0;
}

void o_free(void *p) { free(p); }

/* One step with 64-bit addresses (single chunk). */
int o_step(const o_model *h, const o_params *p,
           const uint64_t *skeys, const double *svals, const int64_t *sivals, int64_t n,
           uint64_t **okeys, double **ovals, int64_t **oivals, int64_t *on, o_stats *st) {
  okey *sk = malloc((size_t)(n ? n : 1) * sizeof(okey));
  if (!sk) return 1;
  for (int64_t i = 0; i < n; ++i) sk[i] = skeys[i];
  okey *ok;
  int rc = o_step_k(h, p, sk, svals, sivals, n, &ok, ovals, oivals, on, st);
  free(sk);
  if (rc) return rc;
  uint64_t *out = malloc((size_t)(*on ? *on : 1) * 8);
  if (!out) { free(ok); free(*ovals); free(*oivals); return 1; }
  for (int64_t i = 0; i < *on; ++i) out[i] = o_lo(ok[i]);
  free(ok);
  *okeys = out;
  return 0;
}

/* One step with addresses of up to 128 bits as (lo, hi) word pairs (2n words in and out). */
int o_step_w(const o_model *h, const o_params *p,
             const uint64_t *skeys2, const double *svals, const int64_t *sivals, int64_t n,
             uint64_t **okeys2, double **ovals, int64_t **oivals, int64_t *on, o_stats *st) {
  okey *sk = malloc((size_t)(n ? n : 1) * sizeof(okey));
  if (!sk) return 1;
  for (int64_t i = 0; i < n; ++i) sk[i] = o_key_of(skeys2[2 * i], skeys2[2 * i + 1]);
  okey *ok;
  int rc = o_step_k(h, p, sk, svals, sivals, n, &ok, ovals, oivals, on, st);
  free(sk);
  if (rc) return rc;
  uint64_t *out = malloc((size_t)(*on ? 2 * *on : 2) * 8);
  if (!out) { free(ok); free(*ovals); free(*oivals); return 1; }
  for (int64_t i = 0; i < *on; ++i) { out[2 * i] = o_lo(ok[i]); out[2 * i + 1] = o_hi(ok[i]); }
  free(ok);
  *okeys2 = out;
  return 0;
}

/* ------------------------------------------------------------------------------------ */
/* Threaded step: the PDVec working-memory step (pdworkingmemory.jl:191-309) on all cores  */
/* ------------------------------------------------------------------------------------ */
/* The reference's PDVec splits the vector into segments by a hash of the address
 * (fastrange_hash, pdvec.jl:6-9) and steps it in three parallel phases:
 *   perform_spawns!    every thread applies the columns of its source segment and deposits
 *                      each contribution into its own dictionary for the target's segment
 *                      (pdworkingmemory.jl:191-217);
 *   collect_local!     per target segment, the threads' dictionaries are summed into one
 *                      (:228-235);
 *   move_and_compress! per segment, the sums become the new vector, compressed (:262-273).
 * This restatement keeps the phases: per-thread buffers of contributions tagged with their
 * target segment, then one thread per segment sums its contributions in an open-addressing
 * hash table and compresses.  Sums follow the summation rule of o_step_k (exact fixed point
 * when every contribution allows it, else the canonical order), so the result equals
 * o_step_k's for any thread count.  When the contributions of one step would exceed
 * `mem_budget` bytes, the segments are processed in passes and the columns re-applied in
 * each pass (their draws are counter-based, so every pass sees the same contributions).
 * Addresses of at most 64 bits, no initiator rule.  With `bits`, HubbardReal1D columns are
 * applied by the bit-level functions above (same results). */
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { uint64_t key; uint64_t vb; uint32_t row; uint32_t kind; } o_rec;   /* 24 B */
typedef struct { o_rec *r; int64_t n, cap; int err; } o_rbuf;
typedef struct { o_rbuf *buf; int pass, rows_per_pass, rows; int is_int; } o_mtctx;

static uint32_t o_row_of(uint64_t key, int rows) {       /* fastrange on a mixed hash */
  return (uint32_t)(((unsigned __int128)o_mix64(key) * (uint64_t)rows) >> 64);
}
static void o_emit_rec(void *vctx, okey key, int cls, int kind, double v, int64_t iv) {
  (void)cls;
  o_mtctx *c = (o_mtctx *)vctx;
  const uint64_t k = o_lo(key);
  const uint32_t row = o_row_of(k, c->rows);
  if ((int)(row / (uint32_t)c->rows_per_pass) != c->pass) return;
  o_rbuf *b = c->buf;
  if (b->n == b->cap) {
    int64_t nc = b->cap ? 2 * b->cap : 4096;
    o_rec *q = realloc(b->r, (size_t)nc * sizeof(o_rec));
    if (!q) { b->err = 1; return; }
    b->r = q; b->cap = nc;
  }
  uint64_t vb;
  if (c->is_int) vb = (uint64_t)iv; else memcpy(&vb, &v, 8);
  b->r[b->n].key = k; b->r[b->n].vb = vb; b->r[b->n].row = row; b->r[b->n].kind = (uint32_t)kind;
  b->n++;
}

/* o_to_fixed on the IEEE bits (the same answers; the threaded step's hot path): x as a signed
 * multiple of 2^-64 when it is one and |x| < 2^48. */
static int o_to_fixed_bits(double x, __int128 *out) {
  uint64_t b;
  memcpy(&b, &x, 8);
  const uint64_t ab = b & 0x7fffffffffffffffull;
  if (ab == 0) { *out = 0; return 1; }
  const int e = (int)(ab >> 52);
  if (e == 0 || e >= 1023 + 48) return 0;          /* subnormal, or |x| >= 2^48 (or inf/nan) */
  const uint64_t mant = (ab & ((1ull << 52) - 1)) | (1ull << 52);
  const int sh = e - 1075 + 64;                    /* |x| = mant * 2^(sh - 64) */
  unsigned __int128 u;
  if (sh >= 0) {
    u = (unsigned __int128)mant << sh;
  } else {
    if (-sh >= 53 || (mant & ((1ull << -sh) - 1))) return 0;   /* bits below 2^-64 */
    u = mant >> -sh;
  }
  *out = (b >> 63) ? -(__int128)u : (__int128)u;
  return 1;
}

/* Exported for the tests: whether the two conversions agree on x (1) or not (0). */
int o_to_fixed_agree(double x) {
  __int128 a = 0, b = 0;
  const int ra = o_to_fixed(x, &a), rb = o_to_fixed_bits(x, &b);
  return ra == rb && (!ra || a == b);
}

/* One slot of a segment's table: the address, the head of its contribution list, whether
 * every contribution so far is exact in fixed point, and their fixed-point (or integer) sum. */
typedef struct { uint64_t key; int64_t head; int used, exact; __int128 fx; } o_slot;
typedef struct { uint64_t ob; int kind; } o_ord;
static int o_cmp_ord(const void *a, const void *b) {
  const o_ord *x = a, *y = b;
  if (x->kind != y->kind) return x->kind < y->kind ? -1 : 1;
  return x->ob < y->ob ? -1 : x->ob > y->ob;
}

/* collect_local! + move_and_compress! of one segment: `rec` holds its m contributions.
 * Writes the surviving entries to (ok, ov, oi) and returns their number, or -1 when out of
 * memory; *len_before and *acc get the compression statistic and the exact norm. */
static int64_t o_reduce_segment(const o_params *p, const o_rec *rec, int64_t m, uint64_t *ok,
                                double *ov, int64_t *oi, int64_t *len_before, o_u128 *acc) {
  const int is_int = p->style == O_STYLE_INTEGER;
  int64_t T = 16;
  while (T < 2 * m) T <<= 1;
  o_slot *tab = calloc((size_t)T, sizeof(o_slot));
  int64_t *nxt = malloc((size_t)(m ? m : 1) * sizeof(int64_t));
  if (!tab || !nxt) { free(tab); free(nxt); return -1; }
  for (int64_t c = 0; c < m; ++c) {
    int64_t sl = (int64_t)((o_mix64(rec[c].key) * 0x9E3779B97F4A7C15ull) >> 20) & (T - 1);
    while (tab[sl].used && tab[sl].key != rec[c].key) sl = (sl + 1) & (T - 1);
    o_slot *s = &tab[sl];
    if (!s->used) { s->used = 1; s->key = rec[c].key; s->head = -1; s->exact = 1; s->fx = 0; }
    if (is_int) {
      s->fx += (int64_t)rec[c].vb;
    } else if (s->exact) {
      double v; memcpy(&v, &rec[c].vb, 8);
      __int128 t;
      if (o_to_fixed_bits(v, &t)) s->fx += t; else s->exact = 0;
    }
    nxt[c] = s->head;
    s->head = c;
  }
  int64_t q = 0, cap_ord = 0;
  o_ord *ord = NULL;
  for (int64_t i = 0; i < T; ++i) {
    const o_slot *s = &tab[i];
    if (!s->used) continue;
    double w = 0.0;
    int64_t wi = 0;
    if (is_int) {
      wi = (int64_t)s->fx;
      if (wi == 0) continue;
    } else {
      if (s->exact) {
        w = o_fixed_signed_to_double(s->fx);
      } else {
        /* canonical order: the diagonal term, then the spawns by increasing value */
        int64_t k = 0;
        for (int64_t c = s->head; c >= 0; c = nxt[c]) ++k;
        if (k > cap_ord) {
          o_ord *no = realloc(ord, (size_t)k * sizeof(o_ord));
          if (!no) { free(ord); free(tab); free(nxt); return -1; }
          ord = no; cap_ord = k;
        }
        k = 0;
        for (int64_t c = s->head; c >= 0; c = nxt[c]) {
          double v; memcpy(&v, &rec[c].vb, 8);
          ord[k].ob = o_ordered_bits(v); ord[k].kind = (int)rec[c].kind; ++k;
        }
        qsort(ord, (size_t)k, sizeof(o_ord), o_cmp_ord);
        for (int64_t j = 0; j < k; ++j) {
          const uint64_t o = ord[j].ob;
          const uint64_t u = (o >> 63) ? (o & 0x7fffffffffffffffull) : ~o;
          double v; memcpy(&v, &u, 8);
          w = j == 0 ? v : w + v;
        }
      }
      if (w == 0.0) continue;
    }
    ++*len_before;
    if (!is_int && p->compression > 0) {    /* compression.jl:18-42 */
      const double prob = (p->compression == 1.0) ? fabs(w) : fabs(w) / p->compression;
      if (prob < 1) {
        uint32_t r[4];
        o_draw_k(p->seed, O_PURPOSE_COMPRESS, p->replica, p->step, (okey)s->key, 0, r);
        w = o_bernoulli(o_u53(r), prob) ? (w < 0 ? -p->compression : p->compression) : 0.0;
      }
      if (w == 0.0) continue;
    }
    ok[q] = s->key; ov[q] = is_int ? 0.0 : w; oi[q] = is_int ? wi : 0;
    *acc += o_fixed(fabs(is_int ? (double)wi : w));
    ++q;
  }
  free(ord); free(tab); free(nxt);
  return q;
}

/* One step on `nthreads` threads (0: all available); same arguments and results as o_step
 * except that the output is not sorted.  Returns 0 on success, 1 when out of memory, 2 for
 * an unsupported model or rule. */
int o_step_mt(const o_model *h, const o_params *p, const uint64_t *skeys, const double *svals,
              const int64_t *sivals, int64_t n, int nthreads, int64_t mem_budget, int bits,
              uint64_t **okeys, double **ovals, int64_t **oivals, int64_t *on, o_stats *st) {
  memset(st, 0, sizeof(*st));
  if (p->init_rule != O_INIT_NONE) return 2;
  {
    int B = h->fermion ? h->M : h->N + h->M - 1;
    if (h->ncomp >= 2) {
      B = 0;
      for (int c = 0; c < h->ncomp; ++c) B += o_comp_bits(h, c);
    }
    if (B > 64) return 2;
  }
  int nt = 1;
#ifdef _OPENMP
  nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
#endif
  const int is_int = p->style == O_STYLE_INTEGER;
  const int fast = bits && o_use_bits(h);
  /* contributions of the step (an upper bound: the diagonal term and every unit) */
  int64_t total = 0;
#pragma omp parallel for num_threads(nt) reduction(+ : total) schedule(static)
  for (int64_t e = 0; e < n; ++e) {
    const double val = is_int ? (double)sivals[e] : svals[e];
    const int noff = o_noff_f(h, (okey)skeys[e], fast);
    int64_t units = noff;
    if (p->style == O_STYLE_INTEGER || (p->style == O_STYLE_DSS &&
        !(p->boost * fabs(val) * p->rel_threshold >=
          (p->abs_threshold < (double)noff ? p->abs_threshold : (double)noff)))) {
      int64_t natt = o_floor_i(fabs(val) * p->boost);
      units = noff == 0 ? 0 : (natt < 1 ? 1 : natt);
    }
    total += 1 + units;
  }
  const int64_t per_rec = 2 * (int64_t)sizeof(o_rec);   /* thread buffers + grouped copy */
  int passes = 1;
  if (mem_budget > 0 && total * per_rec > mem_budget)
    passes = (int)((total * per_rec + mem_budget - 1) / mem_budget);
  /* segments of about 16k contributions, so that each one's table stays in cache */
  int64_t per_pass = (total + passes - 1) / passes;
  int rows_per_pass = 8 * nt;
  if (per_pass / 16384 > rows_per_pass) rows_per_pass = (int)(per_pass / 16384 < 65536 ? per_pass / 16384 : 65536);
  const int rows = passes * rows_per_pass;
  o_rbuf *bufs = calloc((size_t)nt, sizeof(o_rbuf));
  o_stats *tst = calloc((size_t)nt, sizeof(o_stats));
  o_u128 *tacc = calloc((size_t)nt, sizeof(o_u128)), *tspawn = calloc((size_t)nt, sizeof(o_u128));
  int64_t *tlb = calloc((size_t)nt, sizeof(int64_t));
  /* per-segment outputs, concatenated at the end */
  uint64_t **sk = calloc((size_t)rows, sizeof(uint64_t *));
  double **sv = calloc((size_t)rows, sizeof(double *));
  int64_t **si = calloc((size_t)rows, sizeof(int64_t *));
  int64_t *sn = calloc((size_t)rows, sizeof(int64_t));
  int64_t *cnt = calloc((size_t)nt * rows_per_pass + 1, sizeof(int64_t));
  int err = !bufs || !tst || !tacc || !tspawn || !tlb || !sk || !sv || !si || !sn || !cnt;
  for (int pass = 0; pass < passes && !err; ++pass) {
    /* ---- perform_spawns!: each thread into its own buffer ---- */
#pragma omp parallel num_threads(nt)
    {
      int t = 0;
#ifdef _OPENMP
      t = omp_get_thread_num();
#endif
      o_mtctx ctx = {&bufs[t], pass, rows_per_pass, rows, is_int};
      bufs[t].n = 0;
      o_stats junk;
      o_u128 junk_acc = 0;
      o_stats *stp = pass == 0 ? &tst[t] : &junk;
      o_u128 *accp = pass == 0 ? &tspawn[t] : &junk_acc;
#pragma omp for schedule(dynamic, 1024)
      for (int64_t e = 0; e < n; ++e)
        o_apply_column(h, p, (okey)skeys[e], is_int ? 0.0 : svals[e], is_int ? sivals[e] : 0,
                       o_emit_rec, &ctx, stp, accp, fast);
    }
    for (int t = 0; t < nt; ++t) err |= bufs[t].err;
    if (err) break;
    /* ---- group by segment: counts per (thread, segment), then a stable scatter ---- */
    const int R = rows_per_pass;
    memset(cnt, 0, ((size_t)nt * R + 1) * sizeof(int64_t));
#pragma omp parallel for num_threads(nt) schedule(static, 1)
    for (int t = 0; t < nt; ++t)
      for (int64_t i = 0; i < bufs[t].n; ++i) cnt[(size_t)(bufs[t].r[i].row % R) * nt + t + 1]++;
    for (size_t i = 1; i <= (size_t)nt * R; ++i) cnt[i] += cnt[i - 1];
    const int64_t m_all = cnt[(size_t)nt * R];
    o_rec *grp = malloc((size_t)(m_all ? m_all : 1) * sizeof(o_rec));
    if (!grp) { err = 1; break; }
#pragma omp parallel for num_threads(nt) schedule(static, 1)
    for (int t = 0; t < nt; ++t) {
      int64_t *pos = malloc((size_t)R * sizeof(int64_t));
      if (!pos) { bufs[t].err = 1; continue; }
      for (int r = 0; r < R; ++r) pos[r] = cnt[(size_t)r * nt + t];
      for (int64_t i = 0; i < bufs[t].n; ++i) grp[pos[bufs[t].r[i].row % R]++] = bufs[t].r[i];
      free(pos);
    }
    for (int t = 0; t < nt; ++t) err |= bufs[t].err;
    /* ---- collect_local! + move_and_compress!, one segment per task ---- */
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1)
    for (int r = 0; r < R; ++r) {
      if (err) continue;
      int t = 0;
#ifdef _OPENMP
      t = omp_get_thread_num();
#endif
      const int64_t b0 = cnt[(size_t)r * nt], m = cnt[(size_t)(r + 1) * nt] - b0;
      const int g = pass * R + r;
      sk[g] = malloc((size_t)(m ? m : 1) * 8);
      sv[g] = malloc((size_t)(m ? m : 1) * 8);
      si[g] = malloc((size_t)(m ? m : 1) * 8);
      if (!sk[g] || !sv[g] || !si[g]) { err = 1; continue; }
      const int64_t q = o_reduce_segment(p, grp + b0, m, sk[g], sv[g], si[g], &tlb[t], &tacc[t]);
      if (q < 0) err = 1; else sn[g] = q;
    }
    free(grp);
  }
  int64_t tot = 0;
  for (int g = 0; g < rows && !err; ++g) tot += sn[g];
  uint64_t *ok = NULL; double *ov = NULL; int64_t *oi = NULL;
  if (!err) {
    ok = malloc((size_t)(tot ? tot : 1) * 8);
    ov = malloc((size_t)(tot ? tot : 1) * 8);
    oi = malloc((size_t)(tot ? tot : 1) * 8);
    if (!ok || !ov || !oi) err = 1;
  }
  if (!err) {
    int64_t o = 0;
    for (int g = 0; g < rows; ++g) {
      memcpy(ok + o, sk[g], (size_t)sn[g] * 8);
      memcpy(ov + o, sv[g], (size_t)sn[g] * 8);
      memcpy(oi + o, si[g], (size_t)sn[g] * 8);
      o += sn[g];
    }
    o_u128 acc = 0, sacc = 0;
    for (int t = 0; t < nt; ++t) {
      acc += tacc[t]; sacc += tspawn[t];
      st->len_before += tlb[t];
      st->exact_steps += tst[t].exact_steps; st->inexact_steps += tst[t].inexact_steps;
      st->spawn_attempts += tst[t].spawn_attempts; st->spawns += tst[t].spawns;
      st->clones += tst[t].clones; st->deaths += tst[t].deaths; st->zombies += tst[t].zombies;
    }
    if (!is_int) st->spawns = o_fixed_to_double(sacc);
    st->norm = o_fixed_to_double(acc);
    st->len = tot;
    *okeys = ok; *ovals = ov; *oivals = oi; *on = tot;
  } else {
    free(ok); free(ov); free(oi);
  }
  for (int t = 0; bufs && t < nt; ++t) free(bufs[t].r);
  for (int g = 0; g < rows; ++g) {
    if (sk) free(sk[g]);
    if (sv) free(sv[g]);
    if (si) free(si[g]);
  }
  free(bufs); free(tst); free(tacc); free(tspawn); free(tlb); free(sk); free(sv); free(si);
  free(sn); free(cnt);
  return err ? 1 : 0;
}

/* ------------------------------------------------------------------------------------ */
/* Matrix-free product on the full sorted basis (abstractdvec.jl:275-284 in pull form).  */
/* ------------------------------------------------------------------------------------ */
static int64_t o_bsearch(const uint64_t *keys, int64_t n, uint64_t k) {
  int64_t lo = 0, hi = n - 1;
  while (lo <= hi) {
    int64_t mid = lo + (hi - lo) / 2;
    if (keys[mid] == k) return mid;
    if (keys[mid] < k) lo = mid + 1; else hi = mid - 1;
  }
  return -1;
}

/* w = H v over the sorted basis `keys` (D entries).  H is real symmetric, so row i is
 * read from the offdiagonals of column i.  Terms are accumulated as d_i v_i followed by
 * fused multiply-adds in offdiagonal order. Returns number of missing targets (0). */
int64_t o_hv_basis(const o_model *h, const uint64_t *keys, int64_t D, const double *v, double *w) {
  int64_t missing = 0;
  /* rows are independent: the threads change nothing in any row's arithmetic */
#pragma omp parallel for reduction(+ : missing) schedule(dynamic, 4096)
  for (int64_t i = 0; i < D; ++i) {
    double acc = o_diagonal(h, keys[i]) * v[i];
    int noff = o_num_offdiagonals(h, keys[i]);
    for (int c = 1; c <= noff; ++c) {
      uint64_t nk; double hv;
      o_get_offdiagonal(h, keys[i], c, &nk, &hv);
      if (hv == 0.0) continue;
      int64_t j = o_bsearch(keys, D, nk);
      if (j < 0) { ++missing; continue; }
      acc = fma(hv, v[j], acc);
    }
    w[i] = acc;
  }
  return missing;
}

/* Adjoint of w = H(u, t) v for HubbardReal1D / one-component bosonic HubbardRealSpace
 * without trap.  H = D(u) + t K with the hopping part K_ij = -sqrt(prod_ij) symmetric, so
 *   gv = H^T gw = D gw + t (K gw),
 *   gu = <gw, dH/du v> = sum_i gw_i (I_i / 2) v_i      (I_i = sum_k n_k (n_k - 1)),
 *   gt = <gw, dH/dt v> = <gw, K v> = <v, K gw>,
 * and one pass over the rows with one gather of gw per nonzero gives all three: the hop sum
 * k_i = (K gw)_i of row i in offdiagonal order (fused multiply-adds from 0), then
 * gv_i = fma(t, k_i, d_i gw_i), gu += gw_i ((I_i / 2) v_i) and gt += v_i k_i (fused). */
int64_t o_hv_basis_adjoint(const o_model *h, const uint64_t *keys, int64_t D, const double *v,
                           const double *gw, double *gv, double *gu, double *gt) {
  int64_t missing = 0;
  /* the rows in parallel (kg_i and gv_i depend on row i alone), then the two sums in row
   * order on one thread: the same arithmetic as a single sequential pass */
  double *kgs = malloc((size_t)(D ? D : 1) * sizeof(double));
  long *bhis = malloc((size_t)(D ? D : 1) * sizeof(long));
  if (!kgs || !bhis) { free(kgs); free(bhis); return -1; }
#pragma omp parallel for reduction(+ : missing) schedule(dynamic, 4096)
  for (int64_t i = 0; i < D; ++i) {
    int onr[O_MAXC * O_MAXM];
    o_to_onr(h, keys[i], onr);
    long bhi = 0;
    for (int k = 0; k < h->M; ++k) bhi += (long)onr[k] * (onr[k] - 1);
    double kg = 0.0;
    int noff = o_num_offdiagonals(h, keys[i]);
    for (int c = 1; c <= noff; ++c) {
      uint64_t nk; double hv; long prod;
      o_get_offdiagonal_p(h, keys[i], c, &nk, &hv, &prod);
      if (hv == 0.0) continue;
      int64_t j = o_bsearch(keys, D, nk);
      if (j < 0) { ++missing; continue; }
      kg = fma(-sqrt((double)prod), gw[j], kg);   /* K_ij = dH_ij/dt = -sqrt(prod) */
    }
    gv[i] = fma(h->t, kg, o_diagonal(h, keys[i]) * gw[i]);
    kgs[i] = kg;
    bhis[i] = bhi;
  }
  double su = 0.0, st = 0.0;
  for (int64_t i = 0; i < D; ++i) {
    su = fma(gw[i], (double)bhis[i] / 2 * v[i], su);
    st = fma(v[i], kgs[i], st);
  }
  free(kgs); free(bhis);
  *gu = su;
  *gt = st;
  return missing;
}

/* Sparse matrix of H over a sorted basis in CSR form (for exact diagonalisation in the
 * tests).  Duplicate columns within a row are summed by the caller. */
int64_t o_count_nnz(const o_model *h, const uint64_t *keys, int64_t D) {
  int64_t nnz = 0;
  for (int64_t i = 0; i < D; ++i) nnz += 1 + o_num_offdiagonals(h, keys[i]);
  return nnz;
}
int o_build_coo(const o_model *h, const uint64_t *keys, int64_t D,
                int64_t *rows, int64_t *cols, double *vals, int64_t *nnz_out) {
  int64_t z = 0;
  for (int64_t i = 0; i < D; ++i) {
    rows[z] = i; cols[z] = i; vals[z] = o_diagonal(h, keys[i]); ++z;
    int noff = o_num_offdiagonals(h, keys[i]);
    for (int c = 1; c <= noff; ++c) {
      uint64_t nk; double hv;
      o_get_offdiagonal(h, keys[i], c, &nk, &hv);
      if (hv == 0.0) continue;
      int64_t j = o_bsearch(keys, D, nk);
      if (j < 0) return 1;
      rows[z] = j; cols[z] = i; vals[z] = hv; ++z;
    }
  }
  *nnz_out = z;
  return 0;
}

/* All B-bit words with exactly w ones, ascending (the sorted build_basis order,
 * basis_fock.jl:12-36): BoseFS{N,M} is B = N+M-1, w = N; FermiFS{N,M} is B = M, w = N. */
int64_t o_enumerate_fixed_weight(int B, int w, uint64_t *out, int64_t cap) {
  if (w == 0) { if (cap > 0) out[0] = 0; return 1; }
  if (w > B || B > 63) return -1;
  uint64_t x = ((uint64_t)1 << w) - 1, limit = (uint64_t)1 << B;
  int64_t n = 0;
  while (x < limit) {
    if (n < cap) out[n] = x;
    ++n;
    uint64_t c = x & (~x + 1), r = x + c;      /* Gosper's hack */
    x = (((r ^ x) >> 2) / c) | r;
  }
  return n;
}

/* Basis of the block connected to `start` by offdiagonals with nonzero elements
 * (build_basis(H, address), basis_breadth_first_search.jl), sorted ascending.
 * Returns the number of addresses found (may exceed cap: then out holds the first cap). */
static int o_cmp_u64(const void *a, const void *b) {
  uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
  return x < y ? -1 : x > y;
}
int64_t o_connected_basis(const o_model *h, uint64_t start, uint64_t *out, int64_t cap) {
  int64_t tcap = 1024;
  while (tcap < 4 * (cap > 0 ? cap : 1)) tcap <<= 1;
  uint64_t *tab = malloc((size_t)tcap * 8);
  uint64_t *queue = malloc((size_t)tcap * 8);
  if (!tab || !queue) { free(tab); free(queue); return -1; }
  const uint64_t EMPTY = ~0ull;
  for (int64_t i = 0; i < tcap; ++i) tab[i] = EMPTY;
  int64_t head = 0, tail = 0;
#define O_INSERT(k) do { \
    uint64_t _k = (k), _h = (_k * 0x9E3779B97F4A7C15ull) & (uint64_t)(tcap - 1); \
    while (tab[_h] != EMPTY && tab[_h] != _k) _h = (_h + 1) & (uint64_t)(tcap - 1); \
    if (tab[_h] == EMPTY) { \
      if (tail >= tcap / 2) { free(tab); free(queue); return -2; } \
      tab[_h] = _k; queue[tail++] = _k; } } while (0)
  O_INSERT(start);
  while (head < tail) {
    uint64_t k = queue[head++];
    int noff = o_num_offdiagonals(h, k);
    for (int c = 1; c <= noff; ++c) {
      uint64_t nk; double hv;
      o_get_offdiagonal(h, k, c, &nk, &hv);
      if (hv != 0.0) O_INSERT(nk);
    }
  }
#undef O_INSERT
  qsort(queue, (size_t)tail, 8, o_cmp_u64);
  for (int64_t i = 0; i < tail && i < cap; ++i) out[i] = queue[i];
  free(tab); free(queue);
  return tail;
}
