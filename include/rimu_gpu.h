/*
 * rimu_gpu.h -- C ABI of librimu_gpu, the GB300 (sm_103a) implementation of the Rimu.jl
 * FCIQMC step and its matrix-free Hamiltonian application.
 *
 * Plain C types only: opaque handles, host pointers for host data, raw device pointers
 * (as const double * / double *) where a call works on device vectors.  Every call returns
 * a status code; rimu_last_error() gives the message of the last failure on the calling
 * thread.  Calls on one context are not thread safe; separate contexts are independent.
 *
 * Each entry point names the Rimu.jl interface it stands behind (file:line of the reference
 * Rimu.jl v0.14.0 sources).
 */
#ifndef RIMU_GPU_H
#define RIMU_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define RIMU_OK 0
#define RIMU_ERR_BADARG 1    /* invalid argument (ArgumentError in the reference)          */
#define RIMU_ERR_OOM 2       /* device or host allocation failed                            */
#define RIMU_ERR_OVERFLOW 3  /* a capacity could not be grown enough                        */
#define RIMU_ERR_TIMEOUT 4   /* a bounded device wait gave up                               */
#define RIMU_ERR_CUDA 5      /* a CUDA runtime call failed                                  */
#define RIMU_ERR_STATE 6     /* handle used in an invalid state                             */

/* Walker amplitude types: Float64 (IsDeterministic, IsDynamicSemistochastic) and Int64
 * (IsStochasticInteger), src/StochasticStyles/styles.jl:11-12,76-82,175-195. */
#define RIMU_VAL_F64 0
#define RIMU_VAL_I64 1

/* Hamiltonians: src/Hamiltonians/HubbardReal1D.jl:22, HubbardRealSpace.jl:163,
 * HubbardMom1D.jl:43. */
#define RIMU_MODEL_REAL1D 1
#define RIMU_MODEL_REALSPACE 2
#define RIMU_MODEL_MOM1D 3

/* Stochastic styles: IsStochasticInteger (styles.jl:11), IsDeterministic (styles.jl:76),
 * IsDynamicSemistochastic (styles.jl:175). */
#define RIMU_STYLE_INTEGER 0
#define RIMU_STYLE_DETERMINISTIC 1
#define RIMU_STYLE_DSS 2

/* Operator applied by rimu_apply_operator: the FirstOrderTransitionOperator
 * T = 1 + dt (S - H) (src/fciqmc.jl:78-112), or H itself (mul!, abstractdvec.jl:275-284). */
#define RIMU_OP_TRANSITION 0
#define RIMU_OP_HAMILTONIAN 1

typedef struct rimu_ctx rimu_ctx;
typedef struct rimu_model rimu_model;
typedef struct rimu_vec rimu_vec;
typedef struct rimu_wm rimu_wm;

/* Hamiltonian description.  Addresses are bit strings (BoseFS: n_particles + n_modes - 1
 * bits; FermiFS: n_modes bits) with the layout of src/BitStringAddresses/bitstring.jl:464-472
 * (bosons) and 713-723 (fermions).  Up to 64 bits an address is one uint64_t.  HubbardReal1D,
 * one-component HubbardRealSpace and HubbardMom1D (BoseFS, at most 64 modes) also take
 * addresses of 65-128 bits (the reference's two-chunk BitString, bitstring.jl:6-18): wherever
 * such an address crosses this interface it
 * is a pair of uint64_t, (lo, hi), bit k of the address being bit k of lo for k < 64 and bit
 * k - 64 of hi otherwise; key arrays then hold 2 words per address.  Walker lists for them
 * are created with rimu_vec_create_kw(..., key_words = 2, ...).
 *
 * Multi-component addresses (CompositeFS, multicomponent.jl:10-30, and its alias FermiFS2C,
 * :87-103): n_components = C in 2..RIMU_MAX_COMPONENTS, each component a BoseFS or FermiFS
 * with the same n_modes (at most 64), all in one key: component C in the low comp_bits(C)
 * bits, component C-1 above it, ..., component 1 in the highest bits, so that unsigned key
 * order is the reference's order of the component tuple (multicomponent.jl:79).  Each
 * component takes at most 64 bits; up to 64 bits in all the key is one word, up to 128 a
 * (lo, hi) pair as above.  Supported for HubbardRealSpace (CompositeFS of BoseFS/FermiFS
 * components, HubbardRealSpace.jl:18-61, 100-107, 344-391) and, with C = 2, HubbardMom1D
 * (FermiFS2C, HubbardMom1D.jl:141-205). */
#define RIMU_MAX_COMPONENTS 4
typedef struct {
  int kind;                 /* RIMU_MODEL_* */
  int fermion;              /* 1: FermiFS addresses (RIMU_MODEL_REALSPACE only) */
  int n_particles;          /* all components together */
  int n_modes;              /* per component */
  double u;                 /* interaction (HubbardRealSpace: u[1,1]) */
  double t;                 /* hopping */
  int ndim;                 /* HubbardRealSpace CubicGrid dimensions (1..3) */
  int dims[3];
  int periodic[3];          /* 1: PeriodicBoundaries, 0: HardwallBoundaries per dimension */
  const double *potential;  /* HubbardRealSpace trap energy per site (n_modes; with C
                               components C * n_modes, component 1's sites first: the
                               reference's h.potential matrix in column order) or NULL */
  const double *dispersion; /* HubbardMom1D kinetic energies h.kes (n_modes), required */
  int n_components;         /* 0 or 1: one component; C >= 2: C components */
  int comp_fermion[RIMU_MAX_COMPONENTS];    /* per component: 1 FermiFS, 0 BoseFS */
  int comp_particles[RIMU_MAX_COMPONENTS];  /* particles per component */
  double comp_t[RIMU_MAX_COMPONENTS];       /* HubbardRealSpace hopping t[c] */
  /* HubbardRealSpace interaction matrix u (symmetric C x C), its upper triangle row by row:
   * u[1,1], u[1,2], ..., u[1,C], u[2,2], ..., u[C,C] (for C = 2: u[1,1], u[1,2], u[2,2]) */
  double comp_u[RIMU_MAX_COMPONENTS * (RIMU_MAX_COMPONENTS + 1) / 2];
} rimu_model_desc;

/* Parameters of one projector step (apply_operator!, src/Interfaces/dictvectors.jl:112). */
typedef struct {
  int style;                     /* RIMU_STYLE_* */
  int op;                        /* RIMU_OP_* */
  double dt;                     /* time step dτ */
  double shift;                  /* shift S */
  double boost;                  /* apply_operator! boost (1.0) */
  double proj_threshold;         /* on-the-fly projection threshold (0: none) */
  double compression;            /* ThresholdCompression threshold after annihilation (0: none) */
  double rel_spawning_threshold; /* DynamicSemistochastic rel_threshold (1.0) */
  double abs_spawning_threshold; /* DynamicSemistochastic abs_threshold (Inf) */
  uint64_t seed;                 /* random stream seed */
  uint64_t step;                 /* step number (part of every random counter) */
  uint32_t replica;              /* replica id (part of every random key) */
  int initiator;                 /* RIMU_INIT_*: initiator rule of an InitiatorDVec */
  double initiator_threshold;    /* initiators are addresses with |value| > threshold */
} rimu_step_params;

/* Initiator rules (initiators.jl:132-234): NonInitiator, Initiator, SimpleInitiator,
 * CoherentInitiator.  With a rule, addresses must fit in 63 bits, or in 127 bits of two words
 * (a spawn's class travels in the top bit of its address's top word). */
enum { RIMU_INIT_NONE = 0, RIMU_INIT_INITIATOR = 1, RIMU_INIT_SIMPLE = 2, RIMU_INIT_COHERENT = 3 };

/* Step statistics (step_stats, styles.jl:14-19,94-96,203-208; compression.jl:16) plus the
 * walkernumber_and_length of the new vector (abstractdvec.jl:270) and the ProjectedEnergy
 * dot products of the working-memory projector (poststepstrategy.jl:110-121). */
typedef struct {
  double norm;
  int64_t len;
  int64_t len_before;
  int64_t exact_steps;
  int64_t inexact_steps;
  int64_t spawn_attempts;
  double spawns;
  int64_t clones;
  int64_t deaths;
  int64_t zombies;
  double vproj;
  double hproj;
  int64_t spawn_records;
  int32_t retries;
  int32_t nb_bits;
} rimu_step_stats;

/* Library and errors (plumbing of the C ABI, no counterpart in the reference, whose errors are
 * Julia exceptions such as the ArgumentError of pdvec.jl:814-818). */
int rimu_version(void);
int rimu_last_error(char *buf, size_t len);

/* Context: one device and one stream; stream NULL means the CUDA default stream.  All work
 * of the context is ordered on that stream.  No counterpart in the reference (its vectors live
 * in host memory). */
int rimu_ctx_create(int device, void *stream, rimu_ctx **out);
int rimu_ctx_destroy(rimu_ctx *ctx);
int rimu_ctx_synchronize(rimu_ctx *ctx);

/* Hamiltonian handle: stands behind the AbstractHamiltonian constructors
 * (HubbardReal1D.jl:26, HubbardRealSpace.jl:182, HubbardMom1D.jl:49). */
int rimu_model_create(rimu_ctx *ctx, const rimu_model_desc *desc, rimu_model **out);
int rimu_model_destroy(rimu_model *m);
/* diagonal_element (Interfaces/hamiltonians.jl:241) for n host addresses (2n words for a
 * model with addresses wider than 64 bits). */
int rimu_model_diagonal(rimu_model *m, const uint64_t *keys, int64_t n, double *out);
/* num_offdiagonals / offdiagonals (Interfaces/hamiltonians.jl:263,309): all offdiagonal
 * (address, element) pairs of one column, in the reference's order; illegal hard-wall moves
 * give (address, 0.0) as in HubbardRealSpace.jl:331-332. */
int rimu_model_num_offdiagonals(rimu_model *m, uint64_t key, int *out);
/* The same with the address as (lo, hi) and, for wide models, keys as 2 words each. */
int rimu_model_num_offdiagonals_w(rimu_model *m, const uint64_t *key2, int *out);
int rimu_model_offdiagonals_w(rimu_model *m, const uint64_t *key2, uint64_t *keys2, double *vals,
                              int cap, int *n);
int rimu_model_offdiagonals(rimu_model *m, uint64_t key, uint64_t *keys, double *vals, int cap,
                            int *n);

/* Device-resident walker list: stands behind DVec / PDVec (src/DictVectors/dvec.jl,
 * pdvec.jl) as an AbstractDVec (Interfaces/dictvectors.jl:40). */
int rimu_vec_create(rimu_ctx *ctx, int val_kind, int64_t capacity_hint, rimu_vec **out);
/* A walker list with key_words = 1 (addresses of at most 64 bits) or 2 (65-128 bits; its key
 * arrays in upload, download and lookup hold (lo, hi) pairs).  Two-word lists step with
 * rimu_apply_operator (without projectors), and take dot products and conversions with lists
 * of the same width; batched runs take one-word lists. */
int rimu_vec_create_kw(rimu_ctx *ctx, int val_kind, int key_words, int64_t capacity_hint,
                       rimu_vec **out);
int rimu_vec_key_words(const rimu_vec *v, int *key_words);
int rimu_vec_destroy(rimu_vec *v);
/* Replace the contents with n (address, value) pairs from host memory; addresses must be
 * distinct.  vals points to double (RIMU_VAL_F64) or int64_t (RIMU_VAL_I64). */
int rimu_vec_upload(rimu_vec *v, const uint64_t *keys, const void *vals, int64_t n);
/* Copy all pairs to host memory (any order); *n receives the length. */
int rimu_vec_download(rimu_vec *v, uint64_t *keys, void *vals, int64_t cap, int64_t *n);
int rimu_vec_length(rimu_vec *v, int64_t *len);
/* walkernumber_and_length (abstractdvec.jl:258-270; pdvec.jl:896-902). */
int rimu_vec_walkernumber_and_length(rimu_vec *v, double *norm, int64_t *len);
/* getindex for n host addresses (0 where absent): the dot products of dot(P, v). */
int rimu_vec_lookup(rimu_vec *v, const uint64_t *keys, int64_t n, void *vals);
int rimu_vec_copy(rimu_vec *dst, const rimu_vec *src);
int rimu_vec_empty(rimu_vec *v);
/* dot(v, w) = inner(v, w) (abstractdvec.jl:214-230) of two device lists of the same address
 * type, computed on the device; the summation order is fixed, so repeated calls agree. */
int rimu_vec_dot(rimu_vec *v, rimu_vec *w, double *out);
/* dst = src with values converted to val_kind (Int64 to Float64, exact below 2^53, or a plain
 * copy): the promotion of an integer vector before dot(w, H, v) with a Float64 operator. */
int rimu_vec_convert(rimu_vec *dst, const rimu_vec *src, int val_kind);
/* scale!(v, alpha) (VectorInterface, abstractdvec.jl:131-140): every value times alpha; alpha
 * = 0 empties v, alpha = 1 leaves it; values that become exact zeros are removed.  An Int64
 * list takes integer alpha only (its products wrap as Int64 arithmetic does). */
int rimu_vec_scale(rimu_vec *v, double alpha);
/* add!(w, v, alpha, beta) = axpby!(alpha, v, beta, w) (abstractdvec.jl:180-208): w becomes
 * beta*w + alpha*v address by address, computed as (beta*w_k) + (alpha*v_k) with one IEEE
 * rounding per operation, exact zeros removed; beta = 0 empties w first.  v may be w itself
 * (then w is scaled first, as the reference does) and may use another bucket count; an
 * Int64 v is added to a Float64 w as Float64 values; an Int64 w takes an Int64 v and integer
 * factors only. */
int rimu_vec_add(rimu_vec *w, const rimu_vec *v, double alpha, double beta);

/* Working memory: stands behind working_memory(v) (Interfaces/dictvectors.jl:87,
 * pdworkingmemory.jl:295). */
int rimu_wm_create(rimu_ctx *ctx, rimu_wm **out);
int rimu_wm_destroy(rimu_wm *wm);
/* ProjectedEnergy projector (poststepstrategy.jl:90-121): sorted distinct addresses with
 * projector values P and (H'P) values; each step reports vproj = <P|v'> and hproj = <H'P|v'>.
 * n = 0 removes the projector. */
int rimu_wm_set_projector(rimu_wm *wm, const uint64_t *keys, const double *pvals,
                          const double *hpvals, int n);
/* The same for models with addresses of 65-128 bits: keys2 holds n (lo, hi) pairs, sorted by
 * (hi, lo) and distinct.  A working memory steps two-word vectors only with such a projector
 * (or none), one-word vectors only with the plain form. */
int rimu_wm_set_projector_w(rimu_wm *wm, const uint64_t *keys2, const double *pvals,
                            const double *hpvals, int n);

/* Per-kernel timing of the steps run with this working memory (CUDA events on the context
 * stream; the reference times steps with its Timer post-step strategy and communicator
 * reports, poststepstrategy.jl:195, communicators.jl:580-603).  rimu_wm_set_timing resets
 * the accumulators.  rimu_wm_timing fills out7 with: milliseconds in the spawn, heavy-spawn
 * and annihilation kernels, the number of timed steps, the algorithmic bytes of the spawn
 * and annihilation kernels (16-byte records read and written), and the number of steps. */
int rimu_wm_set_timing(rimu_wm *wm, int enable);
int rimu_wm_timing(rimu_wm *wm, double *out7);

/* Launch shape of the step kernels (no counterpart in the reference, whose walker list is a
 * hash dictionary per thread, pdvec.jl:1-120).  keys_per_bucket: the bucket count is chosen
 * so that the expected number of contributions (source walkers plus spawns) per bucket lies
 * between keys_per_bucket / 2 and keys_per_bucket; 16..4096; by default 384 for addresses of
 * up to 64 bits without an initiator rule, else 1024.  Such buckets of at most 512
 * contributions are annihilated by one warp each, larger ones (and all buckets of other
 * steps) by one CTA each.  table_slots: slots of the shared-memory table of one annihilation
 * CTA, a power of two in 512..4096, or 0 to size it from the expected bucket load and the
 * model's largest column; buckets that do not fit are processed in several passes.  Results
 * do not depend on either value. */
int rimu_wm_set_launch_shape(rimu_wm *wm, int keys_per_bucket, int table_slots);

/* How the buckets that one warp annihilates group their spawns by address: RIMU_ANN_HASH (the
 * default) inserts them into a shared-memory hash table with a list per address; RIMU_ANN_SORT
 * sorts them by (address, value) with a bitonic network and takes the runs of equal addresses.
 * Both give the same results bit for bit (no counterpart in the reference, whose annihilation
 * is a dictionary insertion, dictvectors.jl:49-51); the choice only changes the speed. */
enum { RIMU_ANN_HASH = 0, RIMU_ANN_SORT = 1 };
int rimu_wm_set_annihilation(rimu_wm *wm, int mode);

/* One projector step target = T(source), with stats: apply_operator!(wm, target, source,
 * op, boost) of src/Interfaces/dictvectors.jl:112-140 and pdworkingmemory.jl:297-309,
 * including the compression of compression.jl:28-42.  source is not modified. */
int rimu_apply_operator(rimu_model *m, rimu_wm *wm, rimu_vec *target, const rimu_vec *source,
                        const rimu_step_params *params, rimu_step_stats *stats);

/* ---- Batched replicas ------------------------------------------------------------------
 * Many independent FCIQMC runs stepped together: the replicas of one Hamiltonian
 * (ProjectorMonteCarloProblem(H; n_replicas), which the reference steps one after another,
 * pmc_simulation.jl:288-290) or Hamiltonians that differ only in the interaction u (models whose
 * diagonal is tabulated: HubbardReal1D and one-component HubbardRealSpace without trap), each
 * with its own start vector, shift, target walker number, statistics and projector.  Replica r
 * uses random key (seed, r): its steps equal those of rimu_apply_operator with replica = r and the
 * same shifts.  One launch of each step kernel covers all replicas; the shift update
 * (DoubleLogUpdate, shiftstrategy.jl:174-181) runs on the device after every step, so that a
 * segment of steps is one graph replay without host round trips.  The batch works on its own
 * stream of the context's device. */
typedef struct rimu_batch rimu_batch;

typedef struct {
  int style;                     /* RIMU_STYLE_* */
  double dt;
  double boost;                  /* 1.0 */
  double proj_threshold, compression, rel_spawning_threshold, abs_spawning_threshold;
  uint64_t seed;
  int shift_update;              /* 0: shifts stay fixed; 1: DoubleLogUpdate */
  double zeta, xi;               /* DoubleLogUpdate damping (reference defaults 0.08, zeta^2/4) */
  int segment_steps;             /* steps per segment (rounded up to even; 0: 64) */
  int use_graph;                 /* replay each full segment as one captured CUDA graph */
  int autotune;                  /* time five launch shapes on the first steps with at least
                                    2^20 entries and keep the fastest: 2048 and 1024
                                    contributions per bucket (one CTA per bucket), 448 and 256
                                    (one warp per bucket, hashed), and 448 sorted */
} rimu_batch_params;

/* Per replica and step: the step statistics of rimu_step_stats and the shift after the update
 * (the value the reference reports for the step). */
typedef struct {
  double shift;
  double norm;
  double vproj;
  double hproj;
  double spawns;
  int64_t len;
  int64_t len_before;
  int64_t exact_steps;
  int64_t inexact_steps;
  int64_t spawn_attempts;
  int64_t spawn_records;
  int64_t clones;
  int64_t deaths;
  int64_t zombies;
} rimu_batch_stats;

int rimu_batch_create(rimu_ctx *ctx, int nrep, int val_kind, rimu_batch **out);
int rimu_batch_destroy(rimu_batch *b);
/* Model, start vector (host pairs), initial shift and target walker number of one replica;
 * only before the first run.  Batched runs take addresses of at most 64 bits. */
int rimu_batch_set_replica(rimu_batch *b, int replica, rimu_model *m, const uint64_t *keys,
                           const void *vals, int64_t n, double shift, double target_walkers);
/* ProjectedEnergy projector of one replica (as rimu_wm_set_projector). */
int rimu_batch_set_projector(rimu_batch *b, int replica, const uint64_t *keys,
                             const double *pvals, const double *hpvals, int n);
/* Launch shape (as rimu_wm_set_launch_shape); setting it turns the autotuner off. */
int rimu_batch_set_launch_shape(rimu_batch *b, int keys_per_bucket, int table_slots);
/* Annihilation of the warp-sized buckets (as rimu_wm_set_annihilation); setting it turns the
 * autotuner off. */
int rimu_batch_set_annihilation(rimu_batch *b, int mode);
/* nsteps steps with step numbers first_step+1 ... ; out receives nsteps * nrep records,
 * step-major. */
int rimu_batch_run(rimu_batch *b, const rimu_batch_params *p, uint64_t first_step, int nsteps,
                   rimu_batch_stats *out);
/* The walker list of one replica, as rimu_vec_download. */
int rimu_batch_download(rimu_batch *b, int replica, uint64_t *keys, void *vals, int64_t cap,
                        int64_t *n);
/* out8: keys per bucket in use, annihilation table slots, buckets, graph segments, eager
 * segments, re-run segments, milliseconds in the segments (CUDA events), steps run. */
int rimu_batch_info(rimu_batch *b, double *out8);
/* The annihilation mode in use (RIMU_ANN_*: the one set, or the autotuner's choice). */
int rimu_batch_annihilation(rimu_batch *b, int *mode);

/* Full sorted basis (build_basis, ExactDiagonalization/basis_fock.jl:33-36): all BoseFS
 * (FermiFS) addresses in increasing bit-string order. */
int rimu_basis_dimension(rimu_model *m, int64_t *dim);
int rimu_basis_keys(rimu_model *m, int64_t start, int64_t n, uint64_t *keys);

/* Matrix-free w = H v on the full sorted basis, v and w device arrays of length dim: the
 * mul!(w, H, v) behind KrylovKit's OperatorMultiplier (ext/KrylovKitExt.jl:23-46,
 * abstractdvec.jl:275-284).  Runs on the context stream. */
int rimu_hv_basis(rimu_model *m, const double *v, double *w, int64_t dim);
/* Adjoint of w = H(u, t) v for HubbardReal1D and bosonic one-component HubbardRealSpace
 * without trap: gv = H^T gw, gu = <gw, dH/du v>, gt = <gw, dH/dt v> (no counterpart in the
 * reference; the rrule a ChainRulesCore extension would register for mul!). */
int rimu_hv_basis_adjoint(rimu_model *m, const double *v, const double *gw, double *gv,
                          double *gu, double *gt, int64_t dim);

/* Allocation-free variant of rimu_hv_basis_adjoint.  No counterpart in the reference.  It is
 * for callers that cannot let a library allocate device memory: applications whose GPU memory
 * is owned by their own allocator or budget (a server that reserves the memory at start-up, a
 * Julia program whose CUDA.jl pool holds it), where cudaMalloc fails or takes memory promised
 * elsewhere, and loops that cannot afford the device-wide synchronisation that cudaMalloc and
 * cudaFree may imply.  It takes the plain model description instead of a handle (creating a
 * handle allocates) and runs on `stream` (NULL: the default stream); v, gw and gv are device
 * arrays of length dim, gu and gt host outputs.  It calls no cudaMalloc, cudaFree or other
 * allocating routine: its tables and partial sums live in one static device array of about
 * 160 KB that every GPU loading the library keeps until the process exits.  It waits for its
 * stream before returning, to hand gu and gt back on the host.
 * Limits: HubbardReal1D or bosonic one-component HubbardRealSpace without trap, with
 * N+M-1 <= 63 address bits, (N+M)(N+1) <= 4096 and N(N+1)+1 <= 4096; anything else returns
 * RIMU_ERR_BADARG.  The first call on a device does the set-up (it looks up the array's device
 * address with cudaGetSymbolAddress) and should come before any stream capture.  All calls
 * share the array and it keeps the last call's contents; calls whose kernels overlap on the
 * GPU race on it, so they must be ordered on one stream (the host-side table staging is not
 * thread safe either). */
int rimu_hv_basis_adjoint_noalloc(const rimu_model_desc *desc, const double *v, const double *gw,
                                  double *gv, double *gu, double *gt, int64_t dim, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* RIMU_GPU_H */
