// vecops.cu -- operations between two device walker lists: the dot product (inner,
// src/DictVectors/abstractdvec.jl:214-230) and a value-type conversion.
//
// Two lists may use different bucket counts (2^bits_a <= 2^bits_b); both bucket an address by
// the top bits of mix64, so bucket i of the coarser list covers buckets
// [i << (bits_b - bits_a), (i + 1) << (bits_b - bits_a)) of the finer one.  One CTA per coarse
// bucket loads that bucket into a shared-memory table (in chunks if it is larger than the table)
// and streams the matching fine buckets against it.  Products are accumulated per thread in a
// fixed order and reduced per CTA and over CTAs in a fixed order, so the result does not change
// from run to run.
#include <cuda_runtime.h>
#include <string>
#include <vector>
#include "rimu_internal.h"

using namespace rimu;

namespace {

constexpr int DOT_THREADS = 256;

// Table of the coarse bucket: 2048 slots for one-word addresses (32 KB of keys and values),
// 1024 for two-word ones (24 KB), half of them filled per chunk.
template <class K> struct DotSlots { static constexpr uint32_t n = KT<K>::BITS == 64 ? 2048 : 1024; };

__device__ __forceinline__ double value_of(uint64_t bits, int kind) {
  return kind == RIMU_VAL_I64 ? (double)(int64_t)bits : bitsd(bits);
}

__device__ __forceinline__ bool claim(uint64_t *slot, uint64_t key) {
  return atomicCAS((unsigned long long *)slot, (unsigned long long)EMPTY_KEY,
                   (unsigned long long)key) == EMPTY_KEY;
}
__device__ __forceinline__ bool claim(Key128 *slot, Key128 key) {
  return atomicCAS(slot, KT<Key128>::empty(), key) == KT<Key128>::empty();
}

template <class K>
__global__ void __launch_bounds__(DOT_THREADS) k_vec_dot(
    const RecT<K> *ra, const uint32_t *ca, int bits_a, uint32_t capv_a, int kind_a,
    const RecT<K> *rb, const uint32_t *cb, int bits_b, uint32_t capv_b, int kind_b,
    double *partials) {
  constexpr uint32_t SLOTS = DotSlots<K>::n, CHUNK = SLOTS / 2;
  constexpr int TBITS = SLOTS == 2048 ? 11 : 10;
  __shared__ K tkey[SLOTS];
  __shared__ double tval[SLOTS];
  __shared__ double red[DOT_THREADS];
  const int tid = threadIdx.x;
  const int nba = 1 << bits_a, sub = 1 << (bits_b - bits_a);
  const K EMPTY = KT<K>::empty();
  double acc = 0.0;
  for (int i = blockIdx.x; i < nba; i += gridDim.x) {
    const uint32_t na = ca[i] < capv_a ? ca[i] : capv_a;
    for (uint32_t c0 = 0; c0 < na; c0 += CHUNK) {
      const uint32_t c1 = c0 + CHUNK < na ? c0 + CHUNK : na;
      for (uint32_t s = tid; s < SLOTS; s += DOT_THREADS) tkey[s] = EMPTY;
      __syncthreads();
      for (uint32_t e = c0 + tid; e < c1; e += DOT_THREADS) {
        const RecT<K> rec = ra[(size_t)i * capv_a + e];
        uint32_t sl = (uint32_t)((kword(rec.key) * 0x9E3779B97F4A7C15ull) >> (64 - TBITS));
        for (uint32_t p = 0; p < SLOTS; ++p) {     // addresses of a list are distinct
          if (claim(&tkey[sl], rec.key)) { tval[sl] = value_of(rec.val, kind_a); break; }
          sl = (sl + 1) & (SLOTS - 1);
        }
      }
      __syncthreads();
      for (int j = i * sub; j < (i + 1) * sub; ++j) {
        const uint32_t nb = cb[j] < capv_b ? cb[j] : capv_b;
        for (uint32_t e = tid; e < nb; e += DOT_THREADS) {
          const RecT<K> rec = rb[(size_t)j * capv_b + e];
          uint32_t sl = (uint32_t)((kword(rec.key) * 0x9E3779B97F4A7C15ull) >> (64 - TBITS));
          for (uint32_t p = 0; p < SLOTS; ++p) {
            const K k = tkey[sl];
            if (k == rec.key) { acc += tval[sl] * value_of(rec.val, kind_b); break; }
            if (k == EMPTY) break;
            sl = (sl + 1) & (SLOTS - 1);
          }
        }
      }
      __syncthreads();
    }
  }
  red[tid] = acc;
  __syncthreads();
  for (int s = DOT_THREADS / 2; s > 0; s >>= 1) {
    if (tid < s) red[tid] += red[tid + s];
    __syncthreads();
  }
  if (tid == 0) partials[blockIdx.x] = red[0];
}

__global__ void k_sum_partials(const double *partials, int n, double *out) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += partials[i];
    *out = s;
  }
}

template <class K>
__global__ void k_convert_i64_f64(const RecT<K> *src, RecT<K> *dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
       i += (size_t)gridDim.x * blockDim.x) {
    const RecT<K> r = src[i];
    dst[i] = RecT<K>{r.key, dbits((double)(int64_t)r.val)};
  }
}

int fail_arg(const std::string &msg) {
  rimu_set_error(msg);
  return RIMU_ERR_BADARG;
}

// ---- scale! and add! (VectorInterface, src/DictVectors/abstractdvec.jl:121-188) ----------
// A value that becomes an exact zero is removed, as setindex! of a zero removes the key.
// Integer lists take integer factors; their products and sums wrap as Int64 arithmetic does.

__device__ __forceinline__ uint64_t scale_bits(uint64_t v, int kind, double a, long long ia) {
  return kind == RIMU_VAL_I64 ? (uint64_t)(long long)v * (uint64_t)ia : dbits(__dmul_rn(a, bitsd(v)));
}
__device__ __forceinline__ bool nonzero_bits(uint64_t v, int kind) {
  return kind == RIMU_VAL_I64 ? v != 0 : !is_zero_d(bitsd(v));
}

// scale!(v, alpha): one warp per bucket, the survivors compacted in place (a round's reads all
// happen before the ballot, and its writes land below the next round's reads).
template <class K>
__global__ void k_vec_scale(RecT<K> *recs, uint32_t *count, int nb, uint32_t capv, int kind,
                            double alpha, long long ialpha, unsigned long long *removed) {
  const int lane = threadIdx.x & 31, warps = blockDim.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  unsigned long long rm = 0;
  for (int b = blockIdx.x * warps + (threadIdx.x >> 5); b < nb; b += gridDim.x * warps) {
    const uint32_t n = count[b] < capv ? count[b] : capv;
    RecT<K> *rb = recs + (size_t)b * capv;
    uint32_t out = 0;
    for (uint32_t f0 = 0; f0 < n; f0 += 32) {
      const uint32_t f = f0 + (uint32_t)lane;
      RecT<K> rec{};
      bool keep = false;
      if (f < n) {
        rec = rb[f];
        rec.val = scale_bits(rec.val, kind, alpha, ialpha);
        keep = nonzero_bits(rec.val, kind);
        rm += keep ? 0 : 1;
      }
      const uint32_t m = __ballot_sync(0xffffffffu, keep);
      if (keep) rb[out + (uint32_t)__popc(m & lt)] = rec;
      out += (uint32_t)__popc(m);
      __syncwarp();
    }
    if (lane == 0) count[b] = out;
  }
  for (int o = 16; o > 0; o >>= 1) rm += __shfl_down_sync(0xffffffffu, rm, o);
  if (lane == 0 && rm) atomicAdd(removed, rm);
}

constexpr int AX_THREADS = 128;
constexpr uint32_t AX_MAXV = 1024;   // entries of v's bucket held in shared memory

// add!(w, v, alpha, beta) on two lists with the same buckets: out = beta*w + alpha*v per
// address (scale!(w, beta), then w[key] += alpha*val), into a third list.  One CTA per bucket:
// v's entries in shared memory, each of w's entries looks its address up there; then the
// addresses only v has.  flag bit 0: a bucket of v larger than AX_MAXV; bit 1: an output
// bucket over capacity.
template <class K>
__global__ void __launch_bounds__(AX_THREADS) k_vec_axpby(
    const RecT<K> *rw, const uint32_t *cw, uint32_t capw, const RecT<K> *rv,
    const uint32_t *cv, uint32_t capv, RecT<K> *ro, uint32_t *co, uint32_t capo, int nb, int kind,
    double alpha, double beta, long long ialpha, long long ibeta, int w_empty, unsigned int *flag,
    unsigned long long *total) {
  __shared__ K vkey[AX_MAXV];
  __shared__ uint64_t vval[AX_MAXV];
  __shared__ uint8_t vtaken[AX_MAXV];
  __shared__ uint32_t s_out;
  const int tid = threadIdx.x;
  unsigned long long tot = 0;
  for (int b = blockIdx.x; b < nb; b += gridDim.x) {
    const uint32_t nv = cv[b] < capv ? cv[b] : capv;
    const uint32_t nw = w_empty ? 0u : (cw[b] < capw ? cw[b] : capw);
    if (nv > AX_MAXV) {                 // the same for every thread of the CTA
      if (tid == 0) { atomicOr(flag, 1u); co[b] = 0; }
      continue;
    }
    for (uint32_t e = tid; e < nv; e += AX_THREADS) {
      const RecT<K> rec = rv[(size_t)b * capv + e];
      vkey[e] = rec.key;
      vval[e] = rec.val;
      vtaken[e] = 0;
    }
    if (tid == 0) s_out = 0;
    __syncthreads();
    RecT<K> *ob = ro + (size_t)b * capo;
    for (uint32_t e = tid; e < nw; e += AX_THREADS) {
      const RecT<K> rec = rw[(size_t)b * capw + e];
      int j = -1;
      for (uint32_t i = 0; i < nv; ++i)
        if (vkey[i] == rec.key) { j = (int)i; break; }
      uint64_t x;
      if (kind == RIMU_VAL_I64) {
        x = scale_bits(rec.val, kind, beta, ibeta);
        if (j >= 0) { vtaken[j] = 1; x += scale_bits(vval[j], kind, alpha, ialpha); }
      } else {
        double y = __dmul_rn(beta, bitsd(rec.val));
        if (j >= 0) { vtaken[j] = 1; y = __dadd_rn(y, __dmul_rn(alpha, bitsd(vval[j]))); }
        x = dbits(y);
      }
      if (nonzero_bits(x, kind)) {
        const uint32_t pos = atomicAdd(&s_out, 1u);
        if (pos < capo) ob[pos] = RecT<K>{rec.key, x};
      }
    }
    __syncthreads();
    for (uint32_t e = tid; e < nv; e += AX_THREADS) {
      if (vtaken[e]) continue;
      const uint64_t x = scale_bits(vval[e], kind, alpha, ialpha);   // zero + alpha*val
      if (nonzero_bits(x, kind)) {
        const uint32_t pos = atomicAdd(&s_out, 1u);
        if (pos < capo) ob[pos] = RecT<K>{vkey[e], x};
      }
    }
    __syncthreads();
    if (tid == 0) {
      const uint32_t o = s_out;
      co[b] = o < capo ? o : capo;
      if (o > capo) atomicOr(flag, 2u);
      tot += o < capo ? o : capo;
    }
    __syncthreads();
  }
  if (tid == 0 && tot) atomicAdd(total, tot);
}

}  // namespace

int rimu_launch_vec_scale(rimu_ctx *ctx, void *recs, uint32_t *count, int nb, uint32_t capv,
                          int kind, int kw, double alpha, long long ialpha,
                          unsigned long long *removed) {
  const int warps = 4;
  const int want = (nb + warps - 1) / warps, cap = ctx->num_sms * 16;
  const int grid = want < cap ? want : cap;
  if (kw == 2)
    k_vec_scale<Key128><<<grid, warps * 32, 0, ctx->stream>>>(static_cast<Rec2 *>(recs), count, nb,
                                                              capv, kind, alpha, ialpha, removed);
  else
    k_vec_scale<uint64_t><<<grid, warps * 32, 0, ctx->stream>>>(static_cast<Rec *>(recs), count, nb,
                                                                capv, kind, alpha, ialpha, removed);
  return rimu_cuda_check(cudaGetLastError(), "k_vec_scale");
}

int rimu_launch_vec_axpby(rimu_ctx *ctx, const void *rw, const uint32_t *cw, uint32_t capw,
                          const void *rv, const uint32_t *cv, uint32_t capv, void *ro, uint32_t *co,
                          uint32_t capo, int nb, int kind, int kw, double alpha, double beta,
                          long long ialpha, long long ibeta, int w_empty, unsigned int *flag,
                          unsigned long long *total) {
  const int cap = ctx->num_sms * 8;
  const int grid = nb < cap ? nb : cap;
  if (kw == 2)
    k_vec_axpby<Key128><<<grid, AX_THREADS, 0, ctx->stream>>>(
        static_cast<const Rec2 *>(rw), cw, capw, static_cast<const Rec2 *>(rv), cv, capv,
        static_cast<Rec2 *>(ro), co, capo, nb, kind, alpha, beta, ialpha, ibeta, w_empty, flag, total);
  else
    k_vec_axpby<uint64_t><<<grid, AX_THREADS, 0, ctx->stream>>>(
        static_cast<const Rec *>(rw), cw, capw, static_cast<const Rec *>(rv), cv, capv,
        static_cast<Rec *>(ro), co, capo, nb, kind, alpha, beta, ialpha, ibeta, w_empty, flag, total);
  return rimu_cuda_check(cudaGetLastError(), "k_vec_axpby");
}

extern "C" int rimu_vec_dot(rimu_vec *a, rimu_vec *b, double *out) {
  if (!a || !b || !out) return fail_arg("rimu_vec_dot: NULL argument");
  if (a->ctx != b->ctx) return fail_arg("rimu_vec_dot: vectors of different contexts");
  if (a->kw != b->kw) return fail_arg("rimu_vec_dot: vectors of different address widths");
  if (a->nb_bits > b->nb_bits) std::swap(a, b);
  rimu_ctx *ctx = a->ctx;
  const int nba = 1 << a->nb_bits;
  const int grid = nba < ctx->num_sms * 8 ? nba : ctx->num_sms * 8;
  double *partials = nullptr, *res = nullptr;
  int rc;
  if ((rc = dalloc(ctx, &partials, grid)) || (rc = dalloc(ctx, &res, 1))) return rc;
  if (a->kw == 2)
    k_vec_dot<Key128><<<grid, DOT_THREADS, 0, ctx->stream>>>(
        reinterpret_cast<const Rec2 *>(a->recs), a->count, a->nb_bits, a->capv, a->val_kind,
        reinterpret_cast<const Rec2 *>(b->recs), b->count, b->nb_bits, b->capv, b->val_kind, partials);
  else
    k_vec_dot<uint64_t><<<grid, DOT_THREADS, 0, ctx->stream>>>(
        a->recs, a->count, a->nb_bits, a->capv, a->val_kind,
        b->recs, b->count, b->nb_bits, b->capv, b->val_kind, partials);
  k_sum_partials<<<1, 32, 0, ctx->stream>>>(partials, grid, res);
  rc = rimu_cuda_check(cudaGetLastError(), "k_vec_dot");
  if (!rc) rc = d2h(ctx, out, res, 1);
  if (!rc) rc = rimu_cuda_check(cudaStreamSynchronize(ctx->stream), "rimu_vec_dot");
  dfree(ctx, partials);
  dfree(ctx, res);
  return rc;
}

extern "C" int rimu_vec_convert(rimu_vec *dst, const rimu_vec *src, int val_kind) {
  if (!dst || !src) return fail_arg("rimu_vec_convert: NULL argument");
  if (dst == src) return fail_arg("rimu_vec_convert: dst and src must differ");
  if (val_kind != RIMU_VAL_F64 && val_kind != RIMU_VAL_I64) return fail_arg("rimu_vec_convert: bad val_kind");
  if (src->val_kind != val_kind && val_kind != RIMU_VAL_F64)
    return fail_arg("rimu_vec_convert: only Int64 to Float64 converts");
  int rc;
  if ((rc = rimu_vec_copy(dst, src))) return rc;
  if (src->val_kind == val_kind) return RIMU_OK;
  rimu_ctx *ctx = dst->ctx;
  const size_t n = ((size_t)1 << dst->nb_bits) * dst->capv;
  if (dst->kw == 2)
    k_convert_i64_f64<Key128><<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(
        reinterpret_cast<Rec2 *>(dst->recs), reinterpret_cast<Rec2 *>(dst->recs), n);
  else
    k_convert_i64_f64<uint64_t><<<ctx->num_sms * 8, 256, 0, ctx->stream>>>(
        dst->recs, dst->recs, n);
  dst->val_kind = RIMU_VAL_F64;
  return rimu_cuda_check(cudaGetLastError(), "k_convert_i64_f64");
}
