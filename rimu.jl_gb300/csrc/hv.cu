// hv.cu -- matrix-free w = H v on the full sorted basis, and its adjoint.
//
// The basis of BoseFS{N,M} (FermiFS{N,M}) is every B-bit word with exactly N set bits, in
// increasing order (build_basis, ExactDiagonalization/basis_fock.jl:12-36).  Row r is
// unranked with the combinatorial number system (colex rank = sum_i C(p_i, i) over the set
// bits p_1 < p_2 < ...), so no address is stored: the only HBM traffic is v, w and the
// gathers of v at neighbouring ranks.
//
// Pull form: H is real symmetric (LOStructure IsHermitian, HubbardReal1D.jl:44), so row r of
// H is read from the offdiagonals of column r, in the reference's offdiagonal order, with
// one fused multiply-add per nonzero:  w_r = d_r v_r, then w_r = fma(H_jr, v_j, w_r).
// For HubbardReal1D the rank of a hop target is updated from the row's rank by one binomial
// (a set bit moves by one position); periodic wrap-around hops are ranked in full.
#include <cuda_runtime.h>
#include "rimu_internal.h"

namespace rimu {

constexpr int HB = 256;
constexpr int MAXB = 64;

// Word operations of the H*v kernels on a W-bit address word.  Addresses of at most 32 bits
// (the full-basis workloads: HubbardReal1D M = N = 14 has 27) run on 32-bit words and 32-bit
// ranks, where a shift or a bit count is one instruction instead of two; wider addresses
// run on 64-bit words.  Both give the same ranks, products and therefore the same sums.
template <class W> struct HW;
template <> struct HW<uint32_t> {
  static constexpr int BITS = 32;
  __device__ static __forceinline__ int ctz(uint32_t x) { return x ? __ffs((int)x) - 1 : 32; }
  __device__ static __forceinline__ int popc(uint32_t x) { return __popc(x); }
  __device__ static __forceinline__ uint32_t shr(uint32_t x, int s) { return s >= 32 ? 0u : x >> s; }
  __device__ static __forceinline__ uint32_t low(int n) { return n >= 32 ? ~0u : ((1u << n) - 1u); }
};
template <> struct HW<uint64_t> {
  static constexpr int BITS = 64;
  __device__ static __forceinline__ int ctz(uint64_t x) { return ctz64(x); }
  __device__ static __forceinline__ int popc(uint64_t x) { return __popcll(x); }
  __device__ static __forceinline__ uint64_t shr(uint64_t x, int s) { return shr64(x, s); }
  __device__ static __forceinline__ uint64_t low(int n) { return lowmask(n); }
};

// Binomial table c[p * (w + 1) + i] = C(p, i), p in [0, B], i in [0, w], staged in shared
// memory as W words (every C(p, i) with p <= 32 fits 32 bits).
template <class W>
__device__ __forceinline__ W C(const W *tab, int w, int p, int i) {
  return tab[p * (w + 1) + i];
}

template <class W>
__device__ __forceinline__ W unrank(uint64_t r64, int B, int w, const W *tab) {
  W r = (W)r64, key = 0;
  int i = w;
  for (int p = B - 1; p >= 0 && i > 0; --p) {
    const W c = C(tab, w, p, i);
    if (c <= r) { key |= (W)1 << p; r -= c; --i; }
  }
  return key;
}

// The next larger word with the same number of set bits (Gosper's hack): row r + 1 of the
// basis from row r, since the basis is in increasing numeric order.
template <class W>
__device__ __forceinline__ W next_combination(W x) {
  const W c = x & (~x + 1);           // lowest set bit
  const W r = x + c;
  return r | (((x ^ r) >> 2) >> HW<W>::ctz(x));
}

// Rows per thread: a thread unranks the first row of its run and steps to the next ones.
constexpr int HV_ROWS = 4;

template <class W>
__device__ __forceinline__ W rank_of(W key, int w, const W *tab) {
  W r = 0;
  int i = 1;
  while (key) {
    const int p = HW<W>::ctz(key);
    r += C(tab, w, p, i);
    ++i;
    key &= key - 1;
  }
  return r;
}

// sum_i n_i (n_i - 1) of a BoseFS word (bose_hubbard_interaction, bosefs.jl:415-428): a run
// of n ones holds n - d windows of d + 1 ones, so sum_{d >= 1} popcount(windows of d + 1
// ones) = sum_i n_i (n_i - 1) / 2.
template <class W>
__device__ __forceinline__ int bose_interaction_hv(W key) {
  int acc = 0;
  W y = key & (key >> 1);
  while (y) { acc += HW<W>::popc(y); y &= y >> 1; }
  return 2 * acc;
}

// One HubbardReal1D row in the reference's offdiagonal order: acc = fma(coef[p_j], v_j, acc)
// from the given start, with coef = H's hopping elements -t sqrt(p) and start d v_row for
// H v, or coef = -sqrt(p) and start 0 for the hopping part alone (the adjoint).
// A rank outside the basis can only come from an inconsistent address: the gather is skipped
// and the row's result is NaN so that callers see it (real1d_row returns NaN; the generic
// rows below use RIMU_GATHER_GUARD).
#define RIMU_GATHER_GUARD(j) if ((j) >= (uint64_t)dim) { acc = __longlong_as_double(0x7ff8000000000000ll); continue; }

template <class W>
__device__ __forceinline__ double real1d_row(const DevModel &h, const W *tab, W row, W dim, W key,
                                             const double *coef, const double *__restrict__ v,
                                             double acc) {
  using O = HW<W>;
  const int B = h.nbits, M = h.M, w = h.N;
  W y = key;
  int mode = 1, bit = 0, prev_mode = 0, prev_occ = 0;
  while (y) {
    const int z = O::ctz(y);          // < BITS: y is not zero
    y >>= z; mode += z; bit += z;
    const int n = O::ctz(~y);         // run length, below BITS (M >= 2 leaves a zero)
    // right hop (odd chosen)
    {
      W j;
      int prod;
      if (mode == M) {
        const W nk = ((key << 1) | (W)1) & O::low(B);
        prod = n * (O::ctz(~key) + 1);
        j = rank_of(nk, w, tab);
      } else {
        const int q = bit + n - 1;
        const int next = O::ctz(~O::shr(key, bit + n + 1));
        prod = n * (next + 1);
        // ones in bits [0, q]: the bosons of modes 1..mode (bit - (mode - 1) before this one)
        const int idx = bit - mode + 1 + n;
        j = row + C(tab, w, q, idx - 1);
      }
      if (j >= dim) return __longlong_as_double(0x7ff8000000000000ll);
      acc = fma(coef[prod], v[j], acc);
    }
    // left hop (even chosen)
    {
      W j;
      int prod;
      if (mode == 1) {
        const W nk = (key >> 1) | ((W)1 << (B - 1));
        int lead = 0;                             // ones at the top of the B-bit word nk
        for (int b = B - 1; b >= 0 && ((nk >> b) & 1); --b) ++lead;
        prod = O::ctz(~key) * lead;
        j = rank_of(nk, w, tab);
      } else {
        const int po = (prev_mode == mode - 1) ? prev_occ : 0;
        prod = n * (po + 1);
        const int idx = bit - mode + 2;          // ones in bits [0, bit]
        j = row - C(tab, w, bit - 1, idx - 1);
      }
      if (j >= dim) return __longlong_as_double(0x7ff8000000000000ll);
      acc = fma(coef[prod], v[j], acc);
    }
    prev_mode = mode; prev_occ = n;
    y >>= n; bit += n;
  }
  return acc;
}

template <int KIND>
__device__ __forceinline__ double generic_row(const DevModel &h, const uint64_t *tab,
                                              uint64_t row, int64_t dim, uint64_t key,
                                              const double *v, double diag) {
  double acc = diag * v[row];
  int noff;
  MomMap m;
  if (KIND == MODEL_MOM1D) { mom_map(key, m); noff = num_offdiagonals_mom(h, m); }
  else noff = num_offdiagonals_real(h, key);
  for (int c = 1; c <= noff; ++c) {
    Offdiag od;
    if (KIND == MODEL_MOM1D) od = mom1d_offdiag(h, key, m, c);
    else od = realspace_offdiag(h, key, c);
    if (od.prod == 0) continue;
    double hv = h.hoff[od.prod];
    if (od.sign < 0) hv = -hv;
    uint64_t j = rank_of(od.key, h.N, tab);
    RIMU_GATHER_GUARD(j);
    acc = fma(hv, v[j], acc);
  }
  return acc;
}

// Hamiltonian diagonal per address for the generic path (same expressions as the step).
template <int KIND>
__device__ double hv_diag(const DevModel &h, uint64_t key) {
  if (KIND == MODEL_MOM1D) {
    uint64_t x = key;
    int mode = 1, s = 0;
    int occ[MAXB];
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
  double in = 0.0;
  if (!h.fermion && h.u != 0.0) in = h.u * (double)bose_interaction_hv(key) / 2;
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

// Binomial table into shared memory as W words.
template <class W>
__device__ __forceinline__ void load_binom(W *s_tab, const uint64_t *g_tab, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) s_tab[i] = (W)g_tab[i];
  __syncthreads();
}

template <int KIND, class W>
__global__ void __launch_bounds__(HB) k_hv(DevModel h, const uint64_t *binom, int ntab,
                                           const double *__restrict__ v, double *__restrict__ w,
                                           int64_t dim, const double *dtabH) {
  static_assert(KIND == MODEL_REAL1D || sizeof(W) == 8, "32-bit words: HubbardReal1D only");
  extern __shared__ __align__(16) unsigned char hv_smem[];
  W *s_tab = reinterpret_cast<W *>(hv_smem);
  load_binom(s_tab, binom, ntab);
  const int B = h.nbits, wt = h.N;
  for (int64_t row0 = (blockIdx.x * (int64_t)HB + threadIdx.x) * HV_ROWS; row0 < dim;
       row0 += (int64_t)gridDim.x * HB * HV_ROWS) {
    W key = unrank<W>((uint64_t)row0, B, wt, s_tab);
    for (int k = 0; k < HV_ROWS; ++k) {
      const int64_t row = row0 + k;
      if (row >= dim) break;
      if (k) key = next_combination(key);
      double acc;
      if constexpr (KIND == MODEL_REAL1D) {
        acc = real1d_row<W>(h, s_tab, (W)row, (W)dim, key, h.hoff, v,
                            dtabH[bose_interaction_hv(key)] * v[row]);
      } else {
        acc = generic_row<KIND>(h, s_tab, (uint64_t)row, dim, key, v, hv_diag<KIND>(h, key));
      }
      w[row] = acc;
    }
  }
}

// Adjoint of w = H(u, t) v with H = D(u) + t K, K the hopping part (K_ij = -sqrt p_ij,
// symmetric): per row the hop sum k_r = (K gw)_r, one gather of gw per nonzero, gives
//   gv_r = (H gw)_r = fma(t, k_r, d_r gw_r)
// and the per-block partial sums, written to partial[2 * blockIdx.x + {0, 1}], of
//   gu = sum_r gw_r ((I_r / 2) v_r)   (dH/du = sum_i n_i (n_i - 1) / 2)
//   gt = sum_r v_r k_r                (<gw, K v> = <v, K gw>; dH/dt = K).
template <int KIND, class W>
__global__ void __launch_bounds__(HB) k_hv_adjoint(DevModel h, const uint64_t *binom, int ntab,
                                                   const double *__restrict__ v,
                                                   const double *__restrict__ gw,
                                                   double *__restrict__ gv, int64_t dim,
                                                   const double *dtabH, const double *dhdt,
                                                   double *partial) {
  static_assert(KIND == MODEL_REAL1D || sizeof(W) == 8, "32-bit words: HubbardReal1D only");
  extern __shared__ __align__(16) unsigned char hv_smem[];
  W *s_tab = reinterpret_cast<W *>(hv_smem);
  __shared__ double s_red[2][HB / 32];
  load_binom(s_tab, binom, ntab);
  const int B = h.nbits, wt = h.N;
  double su = 0.0, st = 0.0;
  for (int64_t row0 = (blockIdx.x * (int64_t)HB + threadIdx.x) * HV_ROWS; row0 < dim;
       row0 += (int64_t)gridDim.x * HB * HV_ROWS) {
    W key = unrank<W>((uint64_t)row0, B, wt, s_tab);
    for (int kr = 0; kr < HV_ROWS; ++kr) {
      const int64_t row = row0 + kr;
      if (row >= dim) break;
      if (kr) key = next_combination(key);
      const int I = bose_interaction_hv(key);
      double kg;
      if constexpr (KIND == MODEL_REAL1D) {
        kg = real1d_row<W>(h, s_tab, (W)row, (W)dim, key, dhdt, gw, 0.0);
      } else {
        // bosonic one-component HubbardRealSpace without trap
        double acc = 0.0;
        int noff = num_offdiagonals_real(h, key);
        for (int c = 1; c <= noff; ++c) {
          Offdiag od = realspace_offdiag(h, key, c);
          if (od.prod == 0) continue;
          uint64_t j = rank_of(od.key, wt, s_tab);
          RIMU_GATHER_GUARD(j);
          acc = fma(dhdt[od.prod], gw[j], acc);
        }
        kg = acc;
      }
      const double g = gw[row], x = v[row];
      gv[row] = fma(h.t, kg, dtabH[I] * g);
      su = fma(g, (double)I / 2 * x, su);
      st = fma(x, kg, st);
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    su += __shfl_down_sync(0xffffffffu, su, o);
    st += __shfl_down_sync(0xffffffffu, st, o);
  }
  if ((threadIdx.x & 31) == 0) { s_red[0][threadIdx.x >> 5] = su; s_red[1][threadIdx.x >> 5] = st; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int i = 0; i < HB / 32; ++i) { a += s_red[0][i]; b += s_red[1][i]; }
    partial[2 * blockIdx.x] = a;
    partial[2 * blockIdx.x + 1] = b;
  }
}

// Fixed-order sum of the block partials (deterministic result for a given grid).
__global__ void k_reduce_partials(const double *partial, int nblocks, double *out2) {
  __shared__ double s[2][32];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < nblocks; i += 32) { a += partial[2 * i]; b += partial[2 * i + 1]; }
  s[0][threadIdx.x] = a;
  s[1][threadIdx.x] = b;
  __syncwarp();
  if (threadIdx.x == 0) {
    double x = 0.0, y = 0.0;
    for (int i = 0; i < 32; ++i) { x += s[0][i]; y += s[1][i]; }
    out2[0] = x;
    out2[1] = y;
  }
}

}  // namespace rimu

using namespace rimu;

int rimu_hv_grid(rimu_ctx *ctx, int64_t dim) {
  int64_t want = (dim + (int64_t)HB * HV_ROWS - 1) / ((int64_t)HB * HV_ROWS);
  int64_t cap = (int64_t)ctx->num_sms * 8;
  return (int)(want < cap ? (want < 1 ? 1 : want) : cap);
}

// HubbardReal1D addresses of at most 32 bits run on 32-bit words: every rank is below
// C(32, 16) < 2^32.
static bool narrow_words(const DevModel &h) { return h.kind == MODEL_REAL1D && h.nbits <= 32; }

int rimu_launch_hv(rimu_ctx *ctx, const DevModel &h, const uint64_t *binom, int ntab,
                   const double *v, double *w, int64_t dim, const double *dtabH) {
  int grid = rimu_hv_grid(ctx, dim);
  const size_t smem = (size_t)ntab * 8;
  if (narrow_words(h)) {
    k_hv<MODEL_REAL1D, uint32_t><<<grid, HB, (size_t)ntab * 4, ctx->stream>>>(h, binom, ntab, v, w, dim, dtabH);
    return rimu_cuda_check(cudaGetLastError(), "k_hv");
  }
  switch (h.kind) {
    case MODEL_REAL1D: k_hv<MODEL_REAL1D, uint64_t><<<grid, HB, smem, ctx->stream>>>(h, binom, ntab, v, w, dim, dtabH); break;
    case MODEL_REALSPACE: k_hv<MODEL_REALSPACE, uint64_t><<<grid, HB, smem, ctx->stream>>>(h, binom, ntab, v, w, dim, dtabH); break;
    default: k_hv<MODEL_MOM1D, uint64_t><<<grid, HB, smem, ctx->stream>>>(h, binom, ntab, v, w, dim, dtabH); break;
  }
  return rimu_cuda_check(cudaGetLastError(), "k_hv");
}

// The adjoint kernel and the fixed-order reduction of its block partials, on `st`.
static void launch_adjoint(const DevModel &h, const uint64_t *binom, int ntab, const double *v,
                           const double *gw, double *gv, int64_t dim, const double *dtabH,
                           const double *dhdt, double *partial, int grid, double *out2,
                           cudaStream_t st) {
  if (narrow_words(h))
    k_hv_adjoint<MODEL_REAL1D, uint32_t><<<grid, HB, (size_t)ntab * 4, st>>>(
        h, binom, ntab, v, gw, gv, dim, dtabH, dhdt, partial);
  else if (h.kind == MODEL_REAL1D)
    k_hv_adjoint<MODEL_REAL1D, uint64_t><<<grid, HB, (size_t)ntab * 8, st>>>(
        h, binom, ntab, v, gw, gv, dim, dtabH, dhdt, partial);
  else
    k_hv_adjoint<MODEL_REALSPACE, uint64_t><<<grid, HB, (size_t)ntab * 8, st>>>(
        h, binom, ntab, v, gw, gv, dim, dtabH, dhdt, partial);
  k_reduce_partials<<<1, 32, 0, st>>>(partial, grid, out2);
}

int rimu_launch_hv_adjoint(rimu_ctx *ctx, const DevModel &h, const uint64_t *binom, int ntab,
                           const double *v, const double *gw, double *gv, int64_t dim,
                           const double *dtabH, const double *dhdt, double *partial,
                           int grid, double *out2) {
  launch_adjoint(h, binom, ntab, v, gw, gv, dim, dtabH, dhdt, partial, grid, out2, ctx->stream);
  return rimu_cuda_check(cudaGetLastError(), "k_hv_adjoint");
}

// ---------------------------------------------------------------------------------------------
// Allocation-free adjoint.
//
// rimu_hv_basis_adjoint keeps its tables and its per-block partial sums in device memory that
// the library allocates.  Some callers cannot let a library allocate: applications whose device
// memory is owned by their own allocator or budget (an inference server that reserves the GPU's
// memory at start-up, a Julia/CUDA.jl program whose memory pool holds it), where a cudaMalloc
// either fails or takes memory the owner has promised elsewhere; and loops that cannot afford
// the device-wide synchronisation cudaMalloc and cudaFree may imply.  This entry point does the
// same computation with all of its scratch in one file-scope device array of fixed size, so
// that it calls no allocator at all.
//
// The array is global to the library: every GPU that loads the library holds it until the
// process exits, every call shares it, and it keeps the last call's contents.  Calls whose
// kernels overlap on the GPU (two streams, two host threads) race on it.
// ---------------------------------------------------------------------------------------------
namespace rimu {

constexpr int NOALLOC_MAX_BLOCKS = 2048;        // grid blocks (one pair of partial sums each)
constexpr int NOALLOC_MAX_BINOM = 64 * 64;      // (B + 1) * (N + 1) binomial coefficients
constexpr int NOALLOC_MAX_DIAG = 4096;          // N (N - 1) + 1 interaction entries
constexpr int NOALLOC_MAX_PROD = 4096;          // N (N + 1) + 1 occupation products

struct NoAllocScratch {
  double partial[2 * NOALLOC_MAX_BLOCKS];
  double out2[2];
  uint64_t binom[NOALLOC_MAX_BINOM];
  double dtabH[NOALLOC_MAX_DIAG];
  double hoff[NOALLOC_MAX_PROD];
  double dhdt[NOALLOC_MAX_PROD];
};

// About 160 KB per device.
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

}  // namespace rimu

namespace {
constexpr int kMaxDevices = 64;
rimu::NoAllocScratch *g_noalloc_ptr[kMaxDevices] = {nullptr};
int g_noalloc_sms[kMaxDevices] = {0};
// host staging of the tables (no heap): calls are not thread safe
uint64_t g_h_binom[rimu::NOALLOC_MAX_BINOM];
double g_h_diag[rimu::NOALLOC_MAX_DIAG];
double g_h_hoff[rimu::NOALLOC_MAX_PROD];
double g_h_dhdt[rimu::NOALLOC_MAX_PROD];
}  // namespace

extern "C" int rimu_hv_basis_adjoint_noalloc(const rimu_model_desc *d, const double *v,
                                             const double *gw, double *gv, double *gu,
                                             double *gt, int64_t dim, void *stream_handle) {
  using namespace rimu;
  if (!d || !v || !gw || !gv || !gu || !gt) {
    rimu_set_error("rimu_hv_basis_adjoint_noalloc: NULL argument");
    return RIMU_ERR_BADARG;
  }
  const bool realspace = d->kind == RIMU_MODEL_REALSPACE;
  if (d->n_components >= 2 || d->fermion ||
      !(d->kind == RIMU_MODEL_REAL1D || (realspace && !d->potential))) {
    rimu_set_error("rimu_hv_basis_adjoint_noalloc: needs HubbardReal1D or one-component bosonic HubbardRealSpace without trap");
    return RIMU_ERR_BADARG;
  }
  const int N = d->n_particles, M = d->n_modes, B = N + M - 1;
  if (N < 1 || M < 2 || B > 63) {
    rimu_set_error("rimu_hv_basis_adjoint_noalloc: need N >= 1, M >= 2 and N + M - 1 <= 63");
    return RIMU_ERR_BADARG;
  }
  const int nbinom = (B + 1) * (N + 1), ndiag = N * (N - 1) + 1, nprod = N * (N + 1) + 1;
  if (nbinom > NOALLOC_MAX_BINOM || ndiag > NOALLOC_MAX_DIAG || nprod > NOALLOC_MAX_PROD) {
    rimu_set_error("rimu_hv_basis_adjoint_noalloc: model exceeds the static scratch limits "
                   "((N+M)(N+1) <= 4096, N(N+1)+1 <= 4096)");
    return RIMU_ERR_BADARG;
  }
  int ndim = realspace ? d->ndim : 1;
  if (ndim < 1 || ndim > 3) {
    rimu_set_error("rimu_hv_basis_adjoint_noalloc: ndim must be 1..3");
    return RIMU_ERR_BADARG;
  }
  if (realspace) {
    // the checks of rimu_model_create: every extent at least 2, product n_modes
    long long prod = 1;
    for (int i = 0; i < ndim; ++i) {
      if (d->dims[i] < 2 || d->dims[i] > M) {
        rimu_set_error("rimu_hv_basis_adjoint_noalloc: all dimensions must be at least 2");
        return RIMU_ERR_BADARG;
      }
      prod *= d->dims[i];
    }
    if (prod != M) {
      rimu_set_error("rimu_hv_basis_adjoint_noalloc: geometry does not match n_modes");
      return RIMU_ERR_BADARG;
    }
  }
  // dimension C(B, N) must fit int64 and match dim
  unsigned __int128 D = 1;
  for (int i = 1; i <= N; ++i) {
    D = D * (unsigned)(B - N + i) / (unsigned)i;
    if (D > (unsigned __int128)INT64_MAX) {
      rimu_set_error("rimu_hv_basis_adjoint_noalloc: basis dimension does not fit int64");
      return RIMU_ERR_BADARG;
    }
  }
  if ((int64_t)D != dim) {
    rimu_set_error("rimu_hv_basis_adjoint_noalloc: dim does not match the basis dimension");
    return RIMU_ERR_BADARG;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return rimu_cuda_check(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) {
    rimu_set_error("rimu_hv_basis_adjoint_noalloc: device index out of range");
    return RIMU_ERR_BADARG;
  }
  // Set-up, once per device with that device current: the host-side symbol is only a
  // stand-in, the kernels need the device address of the array.
  if (!g_noalloc_ptr[dev]) {
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess) return rimu_cuda_check(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    e = cudaDeviceGetAttribute(&g_noalloc_sms[dev], cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return rimu_cuda_check(e, "cudaDeviceGetAttribute");
    g_noalloc_ptr[dev] = static_cast<NoAllocScratch *>(ptr);
  }
  NoAllocScratch *s = g_noalloc_ptr[dev];
  cudaStream_t st = (cudaStream_t)stream_handle;
  // tables: the same values as the handle-based entry point builds
  for (int p = 0; p <= B; ++p)
    for (int i = 0; i <= N; ++i) {
      unsigned __int128 c = 1;
      if (i > p) c = 0;
      else for (int k = 1; k <= i; ++k) c = c * (unsigned)(p - i + k) / (unsigned)k;
      g_h_binom[p * (N + 1) + i] = c > (unsigned __int128)UINT64_MAX ? ~0ull : (uint64_t)c;
    }
  for (int I = 0; I < ndiag; ++I) g_h_diag[I] = d->u * (double)I / 2;
  for (int p = 0; p < nprod; ++p) {
    double q = sqrt((double)p);
    g_h_hoff[p] = -d->t * q;
    g_h_dhdt[p] = -q;
  }
  struct { void *dst; const void *src; size_t n; } copies[] = {
      {s->binom, g_h_binom, nbinom * sizeof(uint64_t)},
      {s->dtabH, g_h_diag, ndiag * sizeof(double)},
      {s->hoff, g_h_hoff, nprod * sizeof(double)},
      {s->dhdt, g_h_dhdt, nprod * sizeof(double)}};
  for (auto &c : copies) {
    e = cudaMemcpyAsync(c.dst, c.src, c.n, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return rimu_cuda_check(e, "cudaMemcpyAsync (tables)");
  }
  DevModel h{};
  h.kind = d->kind; h.fermion = 0; h.N = N; h.M = M; h.nbits = B; h.u = d->u; h.t = d->t;
  h.ndim = ndim;
  for (int i = 0; i < 3; ++i) {
    h.dims[i] = realspace ? (i < ndim ? d->dims[i] : 1) : (i == 0 ? M : 1);
    h.periodic[i] = realspace ? (i < ndim ? d->periodic[i] : 1) : 1;
  }
  h.hoff = s->hoff;
  h.aoff = s->hoff;
  h.aoff_len = nprod;
  int64_t want = (dim + (int64_t)HB * HV_ROWS - 1) / ((int64_t)HB * HV_ROWS);
  int64_t cap = (int64_t)g_noalloc_sms[dev] * 8;
  if (cap > NOALLOC_MAX_BLOCKS) cap = NOALLOC_MAX_BLOCKS;
  int grid = (int)(want < cap ? (want < 1 ? 1 : want) : cap);
  launch_adjoint(h, s->binom, nbinom, v, gw, gv, dim, s->dtabH, s->dhdt, s->partial, grid,
                 s->out2, st);
  e = cudaGetLastError();
  if (e != cudaSuccess) return rimu_cuda_check(e, "k_hv_adjoint (no-alloc)");
  double out[2];
  e = cudaMemcpyAsync(out, s->out2, sizeof(out), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return rimu_cuda_check(e, "cudaMemcpyAsync (gu, gt)");
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return rimu_cuda_check(e, "cudaStreamSynchronize");
  *gu = out[0];
  *gt = out[1];
  return RIMU_OK;
}
