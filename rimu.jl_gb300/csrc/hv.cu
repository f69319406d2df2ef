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

struct Binom {
  const uint64_t *c;   // c[p * (w + 1) + i] = C(p, i), p in [0, B], i in [0, w]
  int w;
};

__device__ __forceinline__ uint64_t C(const uint64_t *tab, int w, int p, int i) {
  return tab[p * (w + 1) + i];
}

__device__ __forceinline__ uint64_t unrank(uint64_t r, int B, int w, const uint64_t *tab) {
  uint64_t key = 0;
  int i = w;
  for (int p = B - 1; p >= 0 && i > 0; --p) {
    uint64_t c = C(tab, w, p, i);
    if (c <= r) { key |= 1ull << p; r -= c; --i; }
  }
  return key;
}

__device__ __forceinline__ uint64_t rank_of(uint64_t key, int w, const uint64_t *tab) {
  uint64_t r = 0;
  int i = 1;
  while (key) {
    int p = ctz64(key);
    r += C(tab, w, p, i);
    ++i;
    key &= key - 1;
  }
  return r;
}

__device__ __forceinline__ int bose_interaction_hv(uint64_t key) {
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

// One HubbardReal1D row: w = d v + sum fma(H, v_j), optionally also k = sum fma(-sqrt p, x_j)
// for the hopping derivative (second vector x).
// A rank outside the basis can only come from an inconsistent address; the gather is
// skipped and the row marked NaN so that callers see it.
#define RIMU_GATHER_GUARD(j) if ((j) >= (uint64_t)dim) { acc = __longlong_as_double(0x7ff8000000000000ll); continue; }

template <bool ADJ>
__device__ __forceinline__ void real1d_row(const DevModel &h, const uint64_t *tab, uint64_t row,
                                           int64_t dim,
                                           uint64_t key, const double *__restrict__ v,
                                           const double *__restrict__ x, const double *dtabH,
                                           const double *dhdt, double &acc, double &kacc) {
  const int B = h.nbits, M = h.M, w = h.N;
  acc = dtabH[bose_interaction_hv(key)] * v[row];
  kacc = 0.0;
  uint64_t y = key;
  int mode = 1, bit = 0, prev_mode = 0, prev_occ = 0;
  while (y) {
    int z = ctz64(y);
    y = shr64(y, z); mode += z; bit += z;
    const int n = ctz64(~y);
    // right hop (odd chosen)
    {
      uint64_t j;
      int prod;
      if (mode == M) {
        uint64_t nk = ((key << 1) | 1ull) & lowmask(B);
        prod = n * (ctz64(~key) + 1);
        j = rank_of(nk, w, tab);
      } else {
        int q = bit + n - 1;
        int next = ctz64(~shr64(key, bit + n + 1));
        prod = n * (next + 1);
        int idx = popc64(key & lowmask(q + 1));
        j = row + C(tab, w, q, idx - 1);
      }
      if (j >= (uint64_t)dim) { acc = __longlong_as_double(0x7ff8000000000000ll); break; }
      acc = fma(h.hoff[prod], v[j], acc);
      if (ADJ) kacc = fma(dhdt[prod], x[j], kacc);
    }
    // left hop (even chosen)
    {
      uint64_t j;
      int prod;
      if (mode == 1) {
        uint64_t nk = (key >> 1) | (1ull << (B - 1));
        int lead = 0;
        for (int b = B - 1; b >= 0 && ((nk >> b) & 1); --b) ++lead;
        prod = ctz64(~key) * lead;
        j = rank_of(nk, w, tab);
      } else {
        int po = (prev_mode == mode - 1) ? prev_occ : 0;
        prod = n * (po + 1);
        int idx = popc64(key & lowmask(bit + 1));
        j = row - C(tab, w, bit - 1, idx - 1);
      }
      if (j >= (uint64_t)dim) { acc = __longlong_as_double(0x7ff8000000000000ll); break; }
      acc = fma(h.hoff[prod], v[j], acc);
      if (ADJ) kacc = fma(dhdt[prod], x[j], kacc);
    }
    prev_mode = mode; prev_occ = n;
    y = shr64(y, n); bit += n;
  }
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

__device__ __forceinline__ void load_binom(uint64_t *s_tab, const uint64_t *g_tab, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) s_tab[i] = g_tab[i];
  __syncthreads();
}

template <int KIND>
__global__ void __launch_bounds__(HB) k_hv(DevModel h, const uint64_t *binom, int ntab,
                                           const double *__restrict__ v, double *__restrict__ w,
                                           int64_t dim, const double *dtabH) {
  extern __shared__ uint64_t s_tab[];
  load_binom(s_tab, binom, ntab);
  const int B = h.nbits, wt = h.N;
  for (int64_t row = blockIdx.x * (int64_t)HB + threadIdx.x; row < dim;
       row += (int64_t)gridDim.x * HB) {
    uint64_t key = unrank((uint64_t)row, B, wt, s_tab);
    double acc;
    if (KIND == MODEL_REAL1D) {
      double k;
      real1d_row<false>(h, s_tab, (uint64_t)row, dim, key, v, nullptr, dtabH, nullptr, acc, k);
    } else {
      acc = generic_row<KIND>(h, s_tab, (uint64_t)row, dim, key, v, hv_diag<KIND>(h, key));
    }
    w[row] = acc;
  }
}

// Adjoint: gv = H gw (H symmetric), and per-block partial sums of
//   gu = sum_r gw_r * ((I_r / 2) * v_r)       (dH/du = sum_i n_i (n_i - 1) / 2)
//   gt = sum_r gw_r * (sum_j (-sqrt p_rj) v_j) (dH/dt = hopping part / t)
// written to partial[2 * blockIdx.x + {0, 1}].
template <int KIND>
__global__ void __launch_bounds__(HB) k_hv_adjoint(DevModel h, const uint64_t *binom, int ntab,
                                                   const double *__restrict__ v,
                                                   const double *__restrict__ gw,
                                                   double *__restrict__ gv, int64_t dim,
                                                   const double *dtabH, const double *dhdt,
                                                   double *partial) {
  extern __shared__ uint64_t s_tab[];
  __shared__ double s_red[2][HB / 32];
  load_binom(s_tab, binom, ntab);
  const int B = h.nbits, wt = h.N;
  double su = 0.0, st = 0.0;
  for (int64_t row = blockIdx.x * (int64_t)HB + threadIdx.x; row < dim;
       row += (int64_t)gridDim.x * HB) {
    uint64_t key = unrank((uint64_t)row, B, wt, s_tab);
    double acc, kv;
    if (KIND == MODEL_REAL1D) {
      real1d_row<true>(h, s_tab, (uint64_t)row, dim, key, gw, v, dtabH, dhdt, acc, kv);
    } else {
      // bosonic one-component HubbardRealSpace without trap
      acc = dtabH[bose_interaction_hv(key)] * gw[row];
      kv = 0.0;
      int noff = num_offdiagonals_real(h, key);
      for (int c = 1; c <= noff; ++c) {
        Offdiag od = realspace_offdiag(h, key, c);
        if (od.prod == 0) continue;
        uint64_t j = rank_of(od.key, wt, s_tab);
        RIMU_GATHER_GUARD(j);
        acc = fma(h.hoff[od.prod], gw[j], acc);
        kv = fma(dhdt[od.prod], v[j], kv);
      }
    }
    gv[row] = acc;
    const double g = gw[row];
    su += g * ((double)bose_interaction_hv(key) / 2 * v[row]);
    st += g * kv;
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
  int64_t want = (dim + HB - 1) / HB;
  int64_t cap = (int64_t)ctx->num_sms * 8;
  return (int)(want < cap ? (want < 1 ? 1 : want) : cap);
}

int rimu_launch_hv(rimu_ctx *ctx, const DevModel &h, const uint64_t *binom, int ntab,
                   const double *v, double *w, int64_t dim, const double *dtabH) {
  int grid = rimu_hv_grid(ctx, dim);
  size_t smem = (size_t)ntab * 8;
  switch (h.kind) {
    case MODEL_REAL1D: k_hv<MODEL_REAL1D><<<grid, HB, smem, ctx->stream>>>(h, binom, ntab, v, w, dim, dtabH); break;
    case MODEL_REALSPACE: k_hv<MODEL_REALSPACE><<<grid, HB, smem, ctx->stream>>>(h, binom, ntab, v, w, dim, dtabH); break;
    default: k_hv<MODEL_MOM1D><<<grid, HB, smem, ctx->stream>>>(h, binom, ntab, v, w, dim, dtabH); break;
  }
  return rimu_cuda_check(cudaGetLastError(), "k_hv");
}

int rimu_launch_hv_adjoint(rimu_ctx *ctx, const DevModel &h, const uint64_t *binom, int ntab,
                           const double *v, const double *gw, double *gv, int64_t dim,
                           const double *dtabH, const double *dhdt, double *partial,
                           int grid, double *out2) {
  size_t smem = (size_t)ntab * 8;
  if (h.kind == MODEL_REAL1D)
    k_hv_adjoint<MODEL_REAL1D><<<grid, HB, smem, ctx->stream>>>(h, binom, ntab, v, gw, gv, dim, dtabH, dhdt, partial);
  else
    k_hv_adjoint<MODEL_REALSPACE><<<grid, HB, smem, ctx->stream>>>(h, binom, ntab, v, gw, gv, dim, dtabH, dhdt, partial);
  k_reduce_partials<<<1, 32, 0, ctx->stream>>>(partial, grid, out2);
  return rimu_cuda_check(cudaGetLastError(), "k_hv_adjoint");
}
