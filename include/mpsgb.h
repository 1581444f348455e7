/*
 * mpsgb.h -- C ABI of libmpsgb.so, the GB300 (sm_103a) effective-Hamiltonian engine
 * that stands in for MPSKit.jl's derivative-operator hot path.
 *
 * Every entry point returns an int status (GB_OK = 0).  No C++ exception crosses the
 * ABI; the message of the last failure on the calling thread is gb_last_error().
 *
 * Host buffers passed to *_upload / *_download hold tensors exactly as TensorKit stores
 * a dense (Trivial-sector) TensorMap block: column-major, legs in TensorMap order
 * (codomain legs, then domain legs).  The library keeps its own device layouts and
 * converts at the boundary:
 *
 *   kind            reference leg order (host)    device layout (column-major)
 *   GB_KIND_MPS     A[l s; r]                     (l, s, r)
 *   GB_KIND_BOND    C[l; r]                       (l, r)
 *   GB_KIND_AC2     x[l s1; r s2]                 (l, s1, s2, r)
 *   GB_KIND_GL      GL[a w; a']                   (a, a', w)
 *   GB_KIND_GR      GR[b' w; b]                   (b', w, b)
 *   GB_KIND_MPO     W[wl s; s' wr] (dense over the (wl, s, s', wr)
 *                   channel sum space; channel 0 = "not started", last = "finished")
 *
 * References (MPSKit.jl v0.13.13, paths relative to the project root) are given for
 * each entry point: the reference interface the call replaces.
 */
#ifndef MPSGB_H
#define MPSGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status codes */
enum {
  GB_OK = 0,
  GB_ERR_ARG = 1,      /* invalid argument / shape mismatch                         */
  GB_ERR_OOM = 2,      /* device allocation failed                                  */
  GB_ERR_CUDA = 3,     /* CUDA runtime / library failure                            */
  GB_ERR_NOCONV = 4,   /* reserved: non-convergence is reported in info.converged   */
  GB_ERR_TIMEOUT = 5,  /* a bounded device wait gave up (kernel status word)        */
  GB_ERR_NAN = 6,      /* non-finite value detected in a result                     */
  GB_ERR_UNSUPPORTED = 7
};

enum { GB_F64 = 1, GB_C128 = 2 };

enum {
  GB_KIND_GENERIC = 0,
  GB_KIND_MPS = 1,
  GB_KIND_BOND = 2,
  GB_KIND_AC2 = 3,
  GB_KIND_GL = 4,
  GB_KIND_GR = 5,
  GB_KIND_MPO = 6
};

/* derivative-operator kinds */
enum { GB_HEFF_C = 0, GB_HEFF_AC = 1, GB_HEFF_AC2 = 2, GB_HEFF_AC_MPO = 3, GB_HEFF_AC2_MPO = 4 };

/* arithmetic of the bulk contractions */
enum {
  GB_PREC_FP64 = 0,    /* plain FP64 (CUDA-core FMA)                                 */
  GB_PREC_BF16X3 = 1,  /* split precision: hi/lo BF16 operands, 3 products
                          (hi*hi + hi*lo + lo*hi), FP32 accumulate in TMEM
                          (tcgen05), FP64 output                                      */
  GB_PREC_TF32X3 = 2   /* the same scheme with hi/lo TF32 operands (22 significant bits
                          against 16; tcgen05 kind::tf32 runs at half the BF16 rate)   */
};

typedef struct gb_ctx gb_ctx;
typedef struct gb_tensor gb_tensor;
typedef struct gb_heff gb_heff;
typedef struct gb_packed gb_packed;

/* KrylovKit ConvergenceInfo fields read by MPSKit (src/algorithms/groundstate/dmrg.jl:153,239,
 * src/algorithms/timestep/integrators.jl:27) */
typedef struct {
  int converged;
  int numops;
  int numiter;
  double normres;
} gb_krylov_info;

/* ---------------------------------------------------------------- library / context */
int gb_version(void);
const char* gb_last_error(void);

/* One context per device and per host task; holds the stream, library handles and the
 * launch counter.  (Replaces the per-sweep allocator/scheduler state of
 * src/utility/allocator.jl:29-41.) */
int gb_ctx_create(int device, uint32_t flags, gb_ctx** out);
int gb_ctx_destroy(gb_ctx* ctx);
int gb_ctx_synchronize(gb_ctx* ctx);
/* number of libmpsgb kernels launched through this context so far */
int gb_ctx_kernel_launches(gb_ctx* ctx, int64_t* out);
/* device status word written by bounded waits inside kernels (0 = clean); cleared on read */
int gb_ctx_device_status(gb_ctx* ctx, int32_t* out);
/* Bound (seconds, default 2) on every pipeline wait of the tensor-core kernels launched
 * through this context.  A wait that runs out records GB_ERR_TIMEOUT in the status word
 * (gb_ctx_device_status); the kernel then waits (with the default bound) for the copies
 * and MMAs it has already issued, releases its tensor memory and returns, so the context
 * stays usable.  No counterpart in the reference (it has no device code); it is the
 * failure-detection knob of this library, and tests shorten it to exercise that path. */
int gb_ctx_set_wait_bound(gb_ctx* ctx, double seconds);
/* arithmetic of the auxiliary state contractions of this context (gb_mps_ac2,
 * gb_mps_mul_front, gb_mps_mul_tail, gb_project_complement); GB_PREC_FP64 by default */
int gb_ctx_set_precision(gb_ctx* ctx, int precision);
/* Tracing of the tensor-core GEMM (the dominant kernel): between profile_begin and
 * profile_end every split-precision GEMM launch is bracketed by CUDA events on the
 * context's stream.  profile_end synchronises and returns the summed kernel time (ms),
 * the number of launches, their algorithmic flops (unsplit shapes) and the wall time of
 * the whole region measured by events on the same stream (ms).  (Replaces the
 * TimerOutputs tracing of src/algorithms/groundstate/dmrg.jl:289-292.) */
int gb_ctx_profile_begin(gb_ctx* ctx);
int gb_ctx_profile_end(gb_ctx* ctx, double* gemm_ms, int64_t* gemm_launches,
                       double* gemm_flops, double* region_ms);
/* The same region split by kernel family (valid after gb_ctx_profile_end): summed kernel
 * time (ms), launches and flops.  GB_PROF_PERSISTENT: the split GEMMs over dense-embedded
 * operands (flops of their full shapes); GB_PROF_GROUPED: the grouped sector-block GEMMs
 * (flops of their charge blocks, 2 sum_g M_g N_g K_g -- the work a blockwise library does). */
enum { GB_PROF_PERSISTENT = 0, GB_PROF_GROUPED = 1 };
int gb_ctx_profile_kernel(gb_ctx* ctx, int kernel, double* ms, int64_t* launches,
                          double* flops);

/* Launch trace of the context's stream: between trace_begin and trace_end every kernel the
 * library launches (and every traced library call) records an event tagged with its source
 * site; trace_end charges the time between consecutive events to the later site (its work
 * plus any idle gap before it -- host latency shows up there) and returns the number of
 * distinct sites and the traced span (ms).  gb_ctx_trace_site reads site i: its
 * "file.cu:line" name, ms and event count.  Work on auxiliary lane streams appears as time
 * of the next main-stream site.  (The per-section TimerOutputs of dmrg.jl:289-292 and
 * vumps.jl, at kernel granularity.) */
int gb_ctx_trace_begin(gb_ctx* ctx);
int gb_ctx_trace_end(gb_ctx* ctx, int64_t* n_sites, double* total_ms);
int gb_ctx_trace_site(gb_ctx* ctx, int64_t i, char* name, size_t name_len, double* ms,
                      int64_t* events);

/* Schedule of the split-precision tensor-core GEMM (the choice TensorOperations leaves to
 * its contraction backend, `backend::AbstractBackend` carried by every derivative operator,
 * src/algorithms/derivatives/mpo_derivatives.jl:10-16).  tile_n = output tile width along
 * N (128 or 256; 0 = chosen per GEMM shape). */
enum {
  GB_SCHED_PERSISTENT = 0,       /* one CTA per SM over a tile counter, accumulator double-
                                    buffered in TMEM; k-blocks whose packed A and B tiles
                                    are both zero are skipped (block-sparse operands stored
                                    densely with charge-sorted legs)                      */
  GB_SCHED_PERSISTENT_DENSE = 1, /* the same kernel over every k-block                    */
  GB_SCHED_TILE = 2,             /* one CTA per output tile, single accumulator          */
  GB_SCHED_GROUPED = 3           /* the default: operators whose U(1) sectors are known
                                    (gb_heff_set_sectors; real data, split precision) run
                                    every GEMM as one persistent launch over its charge
                                    blocks only -- operands packed block by block, tiles
                                    sized to each block, as TensorKit contracts a symmetric
                                    TensorMap blockwise; every other GEMM runs as
                                    GB_SCHED_PERSISTENT.  The schedule is read when an
                                    operator is built. */
};
int gb_ctx_set_gemm_schedule(gb_ctx* ctx, int schedule, int tile_n);
/* Work counters of the split-precision GEMMs (the flop accounting of the block-sparse
 * measurement; the reference's TimerOutputs sections, src/algorithms/groundstate/dmrg.jl:
 * 289-292, count time only).  tile_flops: flops the tensor pipe executes per split product,
 * summed over the k-blocks every output tile runs (accumulated while profiling or counting).
 * nonzero_flops: 2 x the number of nonzero scalar products sum_k nnz(A[:,k]) nnz(B[k,:]) of
 * every split GEMM while counting is on -- the block-sparse algorithmic count; counting adds
 * a pass over each packed operand, so keep it off inside timed regions. */
int gb_ctx_set_counting(gb_ctx* ctx, int on);
int gb_ctx_read_work(gb_ctx* ctx, double* tile_flops, double* nonzero_flops, int reset);

/* ---------------------------------------------------------------- tensors */
/* Storage of TensorMap blocks (TensorKit `TensorMap{T,S,N1,N2}` with Trivial sectors). */
int gb_tensor_create(gb_ctx* ctx, int kind, int dtype, int ndim, const int64_t* dims,
                     gb_tensor** out);
int gb_tensor_free(gb_tensor* t);
/* Tile-packed copy of a block-sparse tensor (e.g. a U(1) environment in its charge-sorted
 * dense embedding): only the 64 x 64 tiles of its matrix view (rows = first device
 * dimension) that hold a nonzero are kept.  gb_packed_unpack rebuilds the dense tensor
 * exactly into `out` (same kind, dtype and shape; zeros elsewhere).  Lets the environment
 * cache keep every GL/GR of a sweep resident (src/environments/finite_envs.jl:110-151).
 * gb_packed_info: tiles kept / total and the bytes held. */
int gb_tensor_pack(gb_ctx* ctx, const gb_tensor* t, gb_packed** out);
int gb_packed_unpack(gb_ctx* ctx, const gb_packed* p, gb_tensor* out);
int gb_packed_info(const gb_packed* p, int64_t* tiles_kept, int64_t* tiles_total,
                   size_t* bytes);
int gb_packed_free(gb_packed* p);
int gb_tensor_shape(const gb_tensor* t, int* kind, int* dtype, int* ndim, int64_t* dims);
int gb_tensor_upload(gb_tensor* t, const void* host, size_t bytes);
int gb_tensor_download(const gb_tensor* t, void* host, size_t bytes);

/* VectorInterface operations used by the Krylov solvers (KrylovKit over TensorMaps) */
int gb_tensor_copy(gb_tensor* dst, const gb_tensor* src);
/* t *= (re + i im); a zero factor writes zeros whatever t held (zerovector!) */
int gb_tensor_scale(gb_tensor* t, double re, double im);
int gb_tensor_axpy(gb_tensor* y, double re, double im, const gb_tensor* x);
int gb_tensor_dot(const gb_tensor* x, const gb_tensor* y, double* re, double* im);
int gb_tensor_norm(const gb_tensor* x, double* out);

/* ---------------------------------------------------------------- derivative operators */
/* Build and prepare an effective local operator.
 *   GB_HEFF_AC2: JordanMPO_AC2_Hamiltonian(GL, W1, W2, GR) + prepare_operator!!
 *                (src/algorithms/derivatives/hamiltonian_derivatives.jl:206-217, 272-468)
 *   GB_HEFF_AC : JordanMPO_AC_Hamiltonian(GL, W, GR) + prepare_operator!!
 *                (hamiltonian_derivatives.jl:44-157);  W2 must be NULL
 *   GB_HEFF_C  : MPO_C_Hamiltonian(GL, GR)  (src/algorithms/derivatives/mpo_derivatives.jl:37-45,
 *                92-98, 216-219);  W1 and W2 must be NULL
 *   GB_HEFF_AC_MPO / GB_HEFF_AC2_MPO : MPO_AC_Hamiltonian(GL, W, GR) / MPO_AC2_Hamiltonian(GL,
 *                W1, W2, GR) of an arbitrary MPO, no Jordan structure assumed
 *                (mpo_derivatives.jl:46-66, 100-107, 144-153): every channel pair is
 *                contracted; the operator then behaves as GB_HEFF_AC / GB_HEFF_AC2 (vector
 *                kinds, sectors, solvers) and gb_heff_terms reports "A" / "AA"
 * GL/GR must be GB_KIND_GL/GB_KIND_GR tensors, W* GB_KIND_MPO. */
int gb_heff_build(gb_ctx* ctx, int kind, const gb_tensor* GL, const gb_tensor* W1,
                  const gb_tensor* W2, const gb_tensor* GR, int precision, gb_heff** out);
int gb_heff_free(gb_heff* h);
/* comma-separated list of the terms left after prepare, e.g. "IC,BE" */
int gb_heff_terms(const gb_heff* h, char* buf, size_t len);
/* one text line per contraction step of the prepared operator (GEMM shapes; for a grouped
 * sector-block GEMM its groups, tiles and K-blocks), for tuning and diagnostics */
int gb_heff_describe(const gb_heff* h, char* buf, size_t len);
/* algorithmic flops of one application (unsplit shapes; 2 flops/real MAC, 8/complex MAC) */
int gb_heff_flops(const gb_heff* h, double* flops);
int gb_heff_set_precision(gb_heff* h, int precision);
/* U(1) sectors of the operator's vector space: x[l, s1, r, s2] (AC2) or x[l, s, r] (AC) is
 * allowed where q_left[l] + q_phys1[s1] (+ q_phys2[s2]) = q_right[r], with q_left sorted
 * ascending (the charge-sorted dense embedding).  The continuing-channel charges are read off
 * the left environment; the fused AA chain then computes only the charge-allowed entries of
 * its intermediate -- the others are exact zeros -- instead of the whole dense embedding.
 * Optional: results are unchanged.  (TensorKit's block structure of the same contraction,
 * src/algorithms/derivatives/hamiltonian_derivatives.jl:243-369.)  GB_ERR_ARG if the
 * environment does not conserve the given charges. */
int gb_heff_set_sectors(gb_heff* h, const int32_t* q_left, const int32_t* q_phys1,
                        const int32_t* q_phys2, const int32_t* q_right);
/* y = H(x)   (hamiltonian_derivatives.jl:472-500; mpo_derivatives.jl:85-98) */
int gb_heff_apply(gb_heff* h, const gb_tensor* x, gb_tensor* y);
/* fixedpoint(H, x0, :SR, Lanczos(krylovdim, maxiter, tol, eager)) run entirely on the
 * device (src/algorithms/fixedpoint.jl:15-18 -> KrylovKit.eigsolve).  x is overwritten with
 * the normalised Ritz vector. */
int gb_heff_eigsolve(gb_heff* h, gb_tensor* x, int krylovdim, int maxiter, double tol,
                     int eager, double* lambda, gb_krylov_info* info);
/* x <- exp(t H) x with t = t_re + i t_im  (src/algorithms/timestep/integrators.jl:44-53 ->
 * KrylovKit.exponentiate).  x must be GB_C128 unless t is real. */
int gb_heff_exponentiate(gb_heff* h, gb_tensor* x, double t_re, double t_im, int krylovdim,
                         int maxiter, double tol, gb_krylov_info* info);

/* ---------------------------------------------------------------- environments */
/* GL_out = GL * TransferMatrix(A, W, Abar)   (src/transfermatrix/transfer.jl:125-127) */
int gb_env_transfer_left(gb_ctx* ctx, const gb_tensor* GL, const gb_tensor* W,
                         const gb_tensor* A, const gb_tensor* Abar, int precision,
                         gb_tensor* GL_out);
/* GR_out = TransferMatrix(A, W, Abar) * GR   (src/transfermatrix/transfer.jl:128-130) */
int gb_env_transfer_right(gb_ctx* ctx, const gb_tensor* GR, const gb_tensor* W,
                          const gb_tensor* A, const gb_tensor* Abar, int precision,
                          gb_tensor* GR_out);
/* x - T(x) = b for one level of an infinite environment: KrylovKit
 * linsolve(T, b, x0, GMRES(krylovdim, maxiter, tol), 1, -1) as compute_leftenvs! /
 * compute_rightenvs! call it (src/environments/infinite_envs.jl:236, 252, 307, 322).
 * side 0: T(v) = transfer_left(v, W, A, A); side 1: transfer_right.  With lvec/rvec
 * (GB_KIND_BOND) every channel of T(v) is regularised as by gb_env_regularize (the
 * identity levels).  x holds x0 on entry and the solution on exit; info as in eigsolve.
 * Split-precision transfers stop when a restart no longer reduces the residual. */
int gb_env_linsolve(gb_ctx* ctx, int side, const gb_tensor* W, const gb_tensor* A, int precision,
                    const gb_tensor* lvec, const gb_tensor* rvec, const gb_tensor* b,
                    gb_tensor* x, int krylovdim, int maxiter, double tol, gb_krylov_info* info);
/* regularize!(v, lvec, rvec): v -= tr(lvec * v) * rvec on the channel slice `chan` of an
 * environment (src/transfermatrix/transfermatrix.jl:231-237) */
int gb_env_regularize(gb_ctx* ctx, gb_tensor* env, int64_t chan, const gb_tensor* lvec,
                      const gb_tensor* rvec);

/* Copy the channel slice [src_c0, src_c0 + nchan) of one environment into the slice
 * [dst_c0, dst_c0 + nchan) of another of the same kind and bond dimensions (the block
 * assignment GL[site][i] = ... of src/environments/infinite_envs.jl:230-260) */
int gb_env_channel_copy(gb_ctx* ctx, gb_tensor* dst, int64_t dst_c0, const gb_tensor* src,
                        int64_t src_c0, int64_t nchan);

/* ---------------------------------------------------------------- state manipulation */
/* AC2 = A * _transpose_tail(B)   (src/states/finitemps.jl:376-385) */
int gb_mps_ac2(gb_ctx* ctx, const gb_tensor* A, const gb_tensor* B, gb_tensor* AC2);
/* out = C * A   (mul_front, src/utility/utility.jl:11) */
int gb_mps_mul_front(gb_ctx* ctx, const gb_tensor* C, const gb_tensor* A, gb_tensor* out);
/* out = A * C   (mul_tail) */
int gb_mps_mul_tail(gb_ctx* ctx, const gb_tensor* A, const gb_tensor* C, gb_tensor* out);
/* out = C' (TensorKit `adjoint` of a bond tensor, used by regauge!, src/states/ortho.jl:178-184) */
int gb_tensor_adjoint(gb_ctx* ctx, const gb_tensor* C, gb_tensor* out);
/* Mixed transfer maps of a bond matrix, the operators whose dominant eigenvectors the
 * uniform gauge fixing accelerates with (flip(TransferMatrix(A, AL)) and
 * TransferMatrix(A, AR) in gauge_eigsolve_step!, src/states/ortho.jl:254-263, 315-324):
 * side 0: out = sum_s B[s]' X A[s];  side 1: out = sum_s A[s] X B[s]'. */
int gb_mps_transfer_bond(gb_ctx* ctx, int side, const gb_tensor* A, const gb_tensor* B,
                         const gb_tensor* X, gb_tensor* out);
/* Y <- (1 - X X') Y on the first two legs of Y (project_complement!, src/utility/utility.jl:22) */
int gb_project_complement(gb_ctx* ctx, gb_tensor* Y, const gb_tensor* X);
/* Y <- Y (1 - X' X) on the last two legs of Y, X an MPS tensor with orthonormal rows
 * (k x (s r)), e.g. a right-isometric AR: with gb_project_complement this gives
 * NL NL' Y NR' NR, the two-site update projected onto the complements of both sites
 * (left_null / right_null! of changebond!(::OptimalExpand),
 * src/algorithms/changebonds/optimalexpand.jl:122-135, 148-161) without forming the null
 * spaces: the right singular vectors of the projected Y are Vh * NR. */
int gb_project_complement_right(gb_ctx* ctx, gb_tensor* Y, const gb_tensor* X);
/* Krylov-basis helpers for host-driven Krylov loops over operators that have no device solver
 * of their own (the Arnoldi of uniform_leftorth!/uniform_rightorth!, src/states/ortho.jl:
 * 254-263, 315-324, which KrylovKit runs with the basis in memory): `basis` is a
 * GB_KIND_GENERIC tensor (n, kmax) whose column j holds a vector of n elements.
 *   gb_basis_set:           column j <- v
 *   gb_basis_orthogonalize: w <- w - sum_j <v_j, w> v_j over columns 0..k-1, classical
 *                           Gram-Schmidt in two passes; h[2j], h[2j+1] = the projection
 *                           (re, im) summed over both passes
 *   gb_basis_combine:       out <- sum_j coef[j] v_j (coef as re, im pairs) */
int gb_basis_set(gb_ctx* ctx, gb_tensor* basis, int64_t j, const gb_tensor* v);
int gb_basis_orthogonalize(gb_ctx* ctx, const gb_tensor* basis, int64_t k, gb_tensor* w,
                           double* h);
int gb_basis_combine(gb_ctx* ctx, const gb_tensor* basis, int64_t k, const double* coef,
                     gb_tensor* out);
/* contract_mpo_expval-style scalar <x|y> after a heff apply is gb_tensor_dot. */

/* ---------------------------------------------------------------- projections */
/* One application of a generic (non-Jordan) derivative operator between two different
 * states (C_projection / AC_projection / AC2_projection with below != above,
 * src/algorithms/derivatives/derivatives.jl:194-216, through MPO_C/AC_Hamiltonian,
 * mpo_derivatives.jl:37-55, 92-107): GL[bra l, w; ket l'] and GR[ket r', w; bra r] carry
 * different bra and ket bonds.
 *   W = NULL : y[l; r]    = GL[l w; l'] x[l'; r'] GR[r' w; r]              (GB_KIND_BOND)
 *   W        : y[l s; r]  = GL[l w; l'] x[l' s'; r'] W[w s; s' w'] GR[r' w'; r]  (GB_KIND_MPS)
 * The two-site form is the one-site form with the two physical legs fused: W1 W2 contracted
 * over their shared channel into one MPO tensor (wl, d1 d2, d1 d2, wr), x and y two-site
 * tensors relabelled (gb_tensor_reshape) as MPS tensors (Dl, d1 d2, Dr) -- their device orders
 * agree.  x holds the ket bonds, y (caller-created) the bra bonds. */
int gb_mpo_project(gb_ctx* ctx, const gb_tensor* GL, const gb_tensor* W, const gb_tensor* GR,
                   const gb_tensor* x, int precision, gb_tensor* y);

/* ---------------------------------------------------------------- bond expansion */
/* The DMRG3S perturbation MPO_AC_Hamiltonian(env, W, combiner) * AC
 * (src/algorithms/post_expand/dmrg3s.jl:133-192), the combiner fusing the bond with the MPO
 * channel (bond index fastest):
 *   side 0 (env = GL of the site): out[l s; (r w)]  = GL[l w'; l'] AC[l' s'; r] W[w' s; s' w],
 *                                  out dims (Dl_bra, d, Dr * wr)
 *   side 1 (env = GR of the site): out[(l w) s; r]  = W[w s; s' w'] AC[l s'; r'] GR[r' w'; r],
 *                                  out dims (Dl * wl, d, Dr_bra)
 * `out` is caller-created (GB_KIND_MPS); precision as for the transfers. */
int gb_mps_perturb(gb_ctx* ctx, int side, const gb_tensor* env, const gb_tensor* W,
                   const gb_tensor* AC, int precision, gb_tensor* out);
/* out = A (+) B along one virtual leg of MPS tensors (catdomain / catcodomain on the right
 * (leg 2) or left (leg 0) bond, dmrg3s.jl:148-156, optimalexpand.jl:138-142); B = NULL
 * appends zeros (zeros(T, Vpert <- domain(B)), dmrg3s.jl:153).  The other legs must agree;
 * out (caller-created) has the summed dimension. */
int gb_mps_cat(gb_ctx* ctx, const gb_tensor* A, const gb_tensor* B, int leg, gb_tensor* out);
/* out = A with its left (leg 0) or right (leg 2) bond index permuted: out[i] = A[perm[i]]
 * along that leg (perm: host array of the leg's length).  Used to keep a U(1) bond sorted by
 * charge after directions are appended to it (catdomain / catcodomain of charged spaces). */
int gb_mps_permute(gb_ctx* ctx, const gb_tensor* A, int leg, const int64_t* perm,
                   gb_tensor* out);
/* Relabel the kind and shape of an MPS, two-site, bond or generic tensor without moving
 * data: the new shape reads the same device storage in its own device order (MPS (l, s, r),
 * two-site (l, s1, s2, r), bond (l, r)).  E.g. an MPS tensor (l, s, r) is the two-site tensor
 * (Dl, d, Dr, 1) or (Dl, 1, Dr, d), whose truncated SVD is left_gauge / right_gauge with a
 * truncation (src/states/orthoview.jl:326-341).  The element count must not change. */
int gb_tensor_reshape(gb_tensor* t, int kind, int ndim, const int64_t* dims);

/* ---------------------------------------------------------------- gauge */
/* factorisation used by gb_svd_trunc */
enum {
  GB_SVD_GESVD = 0,   /* cuSOLVER QR-iteration SVD (default)                          */
  GB_SVD_GESVDP = 1,  /* cuSOLVER polar-decomposition SVD                             */
  GB_SVD_GRAM = 2     /* eigendecomposition of the Gram matrix of the smaller side
                         (FP64 syevd; per charge block for U(1)).  Its singular values
                         are rounding noise below ~1e-7 of the largest (of the block):
                         when a kept value or the first discarded one is that small, the
                         call falls back to the SVD (GB_SVD_GESVD) for that
                         factorisation.  The bond factor S it returns is triangular
                         (R Sigma or Sigma L, making AL and AR exact isometries), not
                         diagonal; the truncated state AL S AR is the same.           */
};
int gb_ctx_set_svd_method(gb_ctx* ctx, int method);
/* Gauge-step options: the Hermitian eigensolver of the Gram route (GB_EIG_SYEVD: cuSOLVER
 * divide and conquer through its 64-bit interface, the default; GB_EIG_SYEVJ: cuSOLVER cyclic
 * Jacobi at machine-accuracy tolerance; GB_EIG_SYEVD_DEVICE: divide and conquer through the
 * 32-bit interface, which takes no host workspace) and the number of host-thread lanes
 * (1..32, default 8) over which the per-sector factorisations of a U(1) tensor are spread. */
enum { GB_EIG_SYEVD = 0, GB_EIG_SYEVJ = 1, GB_EIG_SYEVD_DEVICE = 2 };
int gb_ctx_set_gauge(gb_ctx* ctx, int eig_method, int lanes);
/* Implementation switches that leave every result unchanged (for comparisons):
 *   GB_OPT_STAGED_MIX: the U(1) chain mix of the grouped schedule either stages the inputs
 *   of each charge's rows through shared memory or runs one warp per output row and column
 *   reading the intermediate directly; both sum in the same order.  0: direct, 2: staged,
 *   1 (default): staged when the mix has at least 4 entries per row (a long-range MPO's
 *   chain mix is close to a permutation, ~1 entry per row, where the direct form wins). */
enum { GB_OPT_STAGED_MIX = 0 };
int gb_ctx_set_option(gb_ctx* ctx, int option, int64_t value);
/* Truncated SVD of a two-site tensor, gauge2! (src/states/orthoview.jl:401-420) with
 * truncrank(maxdim) & trunctol(atol): AL[l s1; k], S (GB_KIND_BOND k x k: diagonal, or
 * triangular under GB_SVD_GRAM),
 * AR[k s2; r].  Returns the discarded-weight norm eps.  Outputs are newly created. */
int gb_svd_trunc(gb_ctx* ctx, const gb_tensor* AC2, int64_t maxdim, double atol,
                 int normalize, gb_tensor** AL, gb_tensor** S, gb_tensor** AR, double* eps);
/* Compact SVDs of `count` independent matrices at once (svd_compact, the factorisations of
 * GradientGrassmann's retraction and preconditioner, src/algorithms/grassmann.jl:93-122,
 * 243-255): M[i] an MPS tensor (Dl, d, Dr) read as (Dl d) x Dr, or a bond tensor; rows >=
 * columns.  Outputs created: U[i] (the input's kind, last leg of size Dr), Vh[i] (Dr x Dr
 * bond), and the singular values, descending, concatenated into the host array S (sum of
 * the Dr).  The factorisations run on the context's lanes (cuSOLVER gesvd). */
int gb_svd_batch(gb_ctx* ctx, int64_t count, const gb_tensor* const* M, gb_tensor** U,
                 gb_tensor** Vh, double* S);
/* left_gauge(AC) with Householder(positive = true): AC = AL * C
 * (src/states/orthoview.jl:322-326); outputs created. */
int gb_left_orth(gb_ctx* ctx, const gb_tensor* AC, gb_tensor** AL, gb_tensor** C);
/* right_gauge(AC): AC = C * AR (src/states/orthoview.jl:334-338); outputs created. */
int gb_right_orth(gb_ctx* ctx, const gb_tensor* AC, gb_tensor** C, gb_tensor** AR);

/* ---------------------------------------------------------------- U(1) symmetry */
/* U(1)-symmetric tensors are stored densely with every leg sorted by charge; entries
 * outside the charge-conserving blocks are exactly zero (for A[l s; r]: q_l + q_s = q_r;
 * for AC2[l s1; r s2]: q_l + q_s1 + q_s2 = q_r).  Contractions need no extra argument: the
 * split-precision GEMM skips zero tiles (GB_SCHED_PERSISTENT).  The factorisations below act
 * per charge block, as TensorKit's do on a symmetric TensorMap (MatrixAlgebraKit called on
 * each block), so that no rounding leaks between sectors.  Charges are host int32 arrays per
 * leg; q_k receives the charges of the new bond (ascending; capacity min of the two fused
 * dimensions) and k its dimension.  Inputs with weight outside their blocks are rejected. */
/* left_gauge(AC) (src/states/orthoview.jl:322-326) block by block: AC = AL * C */
int gb_u1_left_orth(gb_ctx* ctx, const gb_tensor* AC, const int32_t* q_l, const int32_t* q_s,
                    const int32_t* q_r, gb_tensor** AL, gb_tensor** C, int32_t* q_k,
                    int64_t* k);
/* right_gauge(AC) (src/states/orthoview.jl:334-338) block by block: AC = C * AR */
int gb_u1_right_orth(gb_ctx* ctx, const gb_tensor* AC, const int32_t* q_l, const int32_t* q_s,
                     const int32_t* q_r, gb_tensor** C, gb_tensor** AR, int32_t* q_k,
                     int64_t* k);
/* gauge2! with svd_trunc (src/states/orthoview.jl:401-420) on a symmetric two-site tensor:
 * per-block factorisation (method of gb_ctx_set_svd_method), truncation by truncrank(maxdim)
 * & trunctol(atol) over the singular values of all blocks together (ties broken by charge,
 * then by position).  Charges in reference leg order (l, s1, r, s2). */
int gb_u1_svd_trunc(gb_ctx* ctx, const gb_tensor* AC2, const int32_t* q_l, const int32_t* q_s1,
                    const int32_t* q_r, const int32_t* q_s2, int64_t maxdim, double atol,
                    int normalize, gb_tensor** AL, gb_tensor** S, gb_tensor** AR, int32_t* q_k,
                    int64_t* k, double* eps);

/* ---------------------------------------------------------------- allocation-free variant */
/* y = GL . x . GR (the bond operator of GB_HEFF_C) on caller-owned DEVICE buffers in the
 * device layouts above (GL (a, a', w), GR (b', w, b), x and y (l, r)), launched on
 * `stream` (a cudaStream_t; NULL = legacy default stream) of the current device.
 * No counterpart in the reference: it exists for callers that cannot allocate device
 * memory (an external Krylov solver whose arrays all come from its own pool, or launches
 * recorded into a CUDA graph).  It allocates nothing: the intermediate x . GR
 * (Dl*w*Dr elements) lives in a 64 MiB file-scope device array shared by all calls, so
 * larger problems are rejected with GB_ERR_ARG and calls that overlap on the GPU race.
 * The first call on a device looks up the array's address; make it before any stream
 * capture.  The address is cached for the life of the process and cudaDeviceReset unloads
 * the array: after a reset of a device, do not call this entry point on that device again
 * in the same process. */
int gb_c_apply_noalloc(const void* GL, const void* GR, const void* x, void* y, int64_t Dl,
                       int64_t Dr, int64_t w, int dtype, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MPSGB_H */
