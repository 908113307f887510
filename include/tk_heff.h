/*
 * tk_heff.h -- C ABI of the GB300 two-site H_eff library (libtk_heff.so).
 *
 * Every entry point takes plain pointers and sizes.  Host-side structures
 * (tk_qindex, tk_bst, tk_env) describe tensors in the reference's own
 * formats; device buffers are passed as raw device pointers and streams as
 * the `cudaStream_t` value cast to `void*` (NULL = legacy default stream).
 * Errors are reported as tk_status codes, never by aborting; the message of
 * the last failure on the calling thread is returned by tk_last_error().
 *
 * Reference interfaces replaced (paths inside kyungminlee/tensorkraft-design):
 *   build_heff_two_site        tk-dmrg/src/environments/mod.rs:491-602
 *   Environment (dense)        tk-dmrg/src/environments/mod.rs:24-103
 *   BlockSparseTensor          tk-symmetry/src/block_sparse.rs:21-159
 *   FlatBlockStorage           tk-symmetry/src/flat_storage.rs:14-167
 *   QIndex / PackedSectorKey   tk-symmetry/src/sector_key.rs:18-148
 *   LinAlgBackend::gemm        tk-linalg/src/traits.rs:114-121
 *   SparseLinAlgBackend        tk-linalg/src/traits.rs:190-205
 *   IterativeEigensolver       tk-dmrg/src/eigensolver/mod.rs:22-55
 *   LanczosSolver              tk-dmrg/src/eigensolver/mod.rs:58-164
 *   DavidsonSolver             tk-dmrg/src/eigensolver/mod.rs:299-601
 *   exp_krylov_f64             tk-dmrg/src/tdvp/mod.rs:197-396
 *   contract_left/right_environment  tk-dmrg/src/environments/mod.rs:221-483
 *   LinAlgError / DmrgError    tk-linalg/src/error.rs:5-39, tk-dmrg/src/error.rs:9-59
 */
#ifndef TK_HEFF_H
#define TK_HEFF_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  TK_ERR_CUDA carries the failing CUDA call and its message
 * in tk_last_error(), the same (op, detail) pair as LinAlgError::CudaError
 * (tk-linalg/src/error.rs:30-31). */
typedef int32_t tk_status;
#define TK_OK                   0
#define TK_ERR_INVALID_ARG      1
#define TK_ERR_SECTOR_MISMATCH  2
#define TK_ERR_OOM              3
#define TK_ERR_CUDA             4
#define TK_ERR_TIMEOUT          5
#define TK_ERR_CANCELLED        6
#define TK_ERR_UNSUPPORTED      7

/* Quantum-number kinds (tk-symmetry/src/builtins.rs:12-152).  TK_QN_U1U1 is
 * new: (N, 2Sz) with 8 bits per component, component 0 in the low byte. */
#define TK_QN_U1      1
#define TK_QN_Z2      2
#define TK_QN_U1Z2    3
#define TK_QN_U1WIDE  4
#define TK_QN_U1U1    5

/* LegDirection (tk-symmetry/src/quantum_number.rs:49-54). */
#define TK_LEG_INCOMING 0
#define TK_LEG_OUTGOING 1

/* Arithmetic of the sector GEMMs inside one matvec. */
#define TK_PREC_FP64    0  /* FP64 throughout */
#define TK_PREC_BF16X3  1  /* operands split into bf16 hi+lo, three products, fp32 accumulation */

typedef struct tk_ctx tk_ctx;
typedef struct tk_heff2_plan tk_heff2_plan;

/* QIndex: sectors sorted by quantum number, charges are `ncomp` int32 per
 * sector (ncomp = 2 for U1Z2 and U1U1, else 1). */
typedef struct {
    int32_t n_sectors;
    const int32_t* charges;
    const int64_t* dims;
} tk_qindex;

/* BlockSparseTensor in FlatBlockStorage form, host memory.  Keys ascending,
 * packed as PackedSectorKey (leg l at bits l*BIT_WIDTH); each block
 * row-major with the dims its key selects in `legs`. */
typedef struct {
    int32_t qn_kind;
    int32_t rank;
    const tk_qindex* legs;
    const int8_t* leg_dirs;
    const int32_t* flux;
    int64_t n_blocks;
    const uint64_t* keys;
    const int64_t* block_offsets;
    const double* data;
} tk_bst;

/* Environment: dense (bra, w, ket) row-major, host memory. */
typedef struct {
    tk_qindex bra;
    tk_qindex mpo;
    tk_qindex ket;
    const double* data;
} tk_env;

/* Library context bound to one CUDA device. */
tk_status tk_ctx_create(int32_t device, tk_ctx** out);
void tk_ctx_destroy(tk_ctx* ctx);
/* Message of the last failure on this thread ("" if none). */
const char* tk_last_error(void);
/* Library version, for the loader check. */
int32_t tk_version(void);

/*
 * Two-site H_eff plan: replaces build_heff_two_site
 * (tk-dmrg/src/environments/mod.rs:491-602).  Uploads the non-zero sector
 * slabs of L and R, fuses W_i*W_j, and flattens every sector GEMM of one
 * matvec into device task tables.  `psi_flux` selects the two-site sectors
 * with q(s_i)+q(s_j)+q(a_L)-q(a_R) == psi_flux; NULL keeps every sector
 * combination, which makes the plan equal to the reference's dense matrix
 * on every input.  The plan owns all device memory it uses.
 */
tk_status tk_heff2_plan_create(tk_ctx* ctx, const tk_env* env_l, const tk_env* env_r,
                               const tk_bst* w_i, const tk_bst* w_j,
                               const int32_t* psi_flux, int32_t precision,
                               tk_heff2_plan** out);
void tk_heff2_plan_destroy(tk_heff2_plan* plan);

/* Plan sizing without a GPU (no reference counterpart; for callers that
 * pre-size device memory before the Krylov loop, as the specified
 * SweepArena does, techspec/6_tech-spec_tk-dmrg.md:543-572): builds the
 * plan's host tables exactly as tk_heff2_plan_create does and reports the
 * block-layout length, the number of two-site blocks and the device bytes
 * the plan holds for its tables, operands and intermediates in `precision`
 * with its default FP64 schedule (eigensolver and host-call workspaces and
 * the grouped schedules' state, allocated on first use, are not included).
 * Calls no CUDA API; any output pointer may be NULL. */
tk_status tk_heff2_plan_footprint(const tk_env* env_l, const tk_env* env_r, const tk_bst* w_i,
                                  const tk_bst* w_j, const int32_t* psi_flux, int32_t precision,
                                  int64_t* block_dim, int64_t* n_blocks, int64_t* device_bytes);
/* Test hooks (no reference counterpart) for the TK_ERR_OOM paths: from the
 * next call on, the countdown-th host-allocation checkpoint of the plan-table
 * builders, or the countdown-th device allocation made for a plan, fails as
 * if memory were exhausted (counted from 1; 0 disarms).  The failing call
 * returns TK_ERR_OOM and releases what it had allocated. */
void tk_debug_fail_host_alloc(int32_t countdown);
void tk_debug_fail_device_alloc(int32_t countdown);

/* dense_dim = d_i*d_j*D_L*D_R (the closure's `dim`); block_dim = length of
 * the block-layout vector; n_blocks = two-site blocks. */
tk_status tk_heff2_dims(const tk_heff2_plan* plan, int64_t* dense_dim, int64_t* block_dim,
                        int64_t* n_blocks);
/* The two-site block layout: packed keys (ascending) and element offsets. */
tk_status tk_heff2_blocks(const tk_heff2_plan* plan, uint64_t* keys, int64_t* offsets);
/* Algorithmic FP64 flops and bytes of one matvec, from the sector tables. */
tk_status tk_heff2_cost(const tk_heff2_plan* plan, double* flops, double* bytes);
/* Kernel launches one tk_heff2_apply (or tk_heff2_apply_complex) issues in
 * the plan's current precision and schedule (no reference counterpart:
 * launch accounting for benchmarks). */
tk_status tk_heff2_launches(const tk_heff2_plan* plan, int32_t* per_apply);
/* How tk_heff2_apply_host_flat moves x and y (no reference counterpart).
 * The direct forms apply when the plan runs split precision and the buffer
 * is page-locked host memory mapped into the device address space
 * (cudaHostAlloc / cudaHostRegister); otherwise that buffer is staged.
 * TK_HOST_IO_STAGED: copy x into a device buffer, run, copy y back.
 * TK_HOST_IO_DIRECT: the kernels read psi from x and write y in host memory
 *   over the CPU-GPU link, overlapping the transfers with the GEMMs.
 * TK_HOST_IO_DIRECT_OUT: x is copied in; the stage-3 kernel writes y to host
 *   memory directly (every y element is written once).
 * TK_HOST_IO_AUTO (default): DIRECT_OUT (measured fastest on the Hubbard,
 *   Heisenberg and cylinder workloads; the in-GEMM psi split reads columns
 *   with a stride, which the link serves poorly under DIRECT).
 * Whenever x is copied and every stage-1 stack splits psi inside the GEMM
 * kernel, the copy runs in pieces on a second stream (two by default,
 * tk_heff2_set_psi_pieces) and the stage-1 tiles that read only the pieces
 * already copied start while the rest is in flight. */
#define TK_HOST_IO_STAGED     0
#define TK_HOST_IO_DIRECT     1
#define TK_HOST_IO_DIRECT_OUT 2
#define TK_HOST_IO_AUTO       3
tk_status tk_heff2_set_host_io(tk_heff2_plan* plan, int32_t mode);
/* Host-buffer split matvec: psi is copied in `pieces` pieces (1, 2, 4 or 8;
 * default 2) at block boundaries near equal shares, and the stage-1 tiles that
 * read only the pieces already on the device start while the rest is in
 * flight (when every stage-1 stack splits psi inside the GEMM kernel; else
 * one copy).  Results are the same bits for every setting. */
tk_status tk_heff2_set_psi_pieces(tk_heff2_plan* plan, int32_t pieces);
tk_status tk_heff2_set_precision(tk_heff2_plan* plan, int32_t precision);

/* Launch schedule of the FP64 sector GEMMs.  TK_SCHED_GROUPED: all
 * sector GEMMs of a stage in one grouped launch.  TK_SCHED_PER_BLOCK: one
 * launch per output block, the GPU analogue of the reference's one-task-at-a-
 * time block_gemm loop (tk-linalg/src/device/faer.rs:439-512), kept as the
 * baseline the grouped launch is measured against.  TK_SCHED_STACKED (the
 * default, built with the plan): the sector GEMMs regrouped
 * into operand stacks, one per ket sector of L and one per bra sector of R
 * (the split-precision path's grouping, in FP64), cut into pieces of at most
 * 32 x 64 outputs that step over the stack columns their rows hold, so that
 * nearly every FP64 FMA issued is one of the product's own (complex plans:
 * the same pieces with complex FMAs on planar operands; the default of
 * complex plans too).  Every schedule computes the same sums in FP64; they
 * differ only in the order of the additions. */
#define TK_SCHED_GROUPED   0
#define TK_SCHED_PER_BLOCK 1
#define TK_SCHED_STACKED   2
tk_status tk_heff2_set_schedule(tk_heff2_plan* plan, int32_t schedule);
tk_status tk_heff2_get_schedule(const tk_heff2_plan* plan, int32_t* schedule);

/* Cooperative cancellation (DMRGEngine::run_with_cancel_flag,
 * tk-dmrg/src/sweep/mod.rs:273-289, checks an AtomicBool before every step):
 * `flag` points to a host int32 (NULL detaches it) that tk_lanczos_lowest,
 * tk_davidson_lowest and tk_expm_krylov read before every restart, iteration
 * or eighth Krylov step.  Once it reads non-zero the call waits for its
 * stream, so that none of its work is left in flight, and returns
 * TK_ERR_CANCELLED; the eigenvector buffer then holds the last iterate.  The
 * flag is read with acquire ordering and may be set from any thread. */
tk_status tk_heff2_set_cancel_flag(tk_heff2_plan* plan, const int32_t* flag);
/* Test hook, no reference counterpart: writes `code` (non-zero) into the
 * device error word of a split-precision plan's tensor-core kernels, as a
 * bounded wait that ran out would.  The next call that reads the word back
 * (tk_heff2_apply_host_flat, the eigensolvers) returns TK_ERR_TIMEOUT and
 * clears it.  TK_ERR_UNSUPPORTED for an FP64 plan. */
tk_status tk_heff2_inject_error_word(tk_heff2_plan* plan, int32_t code);

/* Schedule of the split-precision kernels (no reference counterpart; the
 * plan-time choices of the specification's autotuner):
 *   tall_max_mtiles: stage-1 stacks (one per ket sector of L) of at most this
 *     many 128-row tiles split psi inside the GEMM kernel; taller stacks take
 *     a bf16 split copy of psi made once per matvec (default 3);
 *   fuse_max_ntiles: stage-3 stacks of at most this many 64-column tiles run
 *     the W_i W_j combine inside the stage-3 kernel instead of a separate
 *     combine launch (default 0: never);
 *   combine_warps: the form of the separate combine: one CTA per job (0,
 *     default), persistent warps that load their next job while storing the
 *     current one (1), one warp per job, consecutive lanes on consecutive
 *     elements (2), or one 64-thread CTA per job with eight elements per
 *     thread (3).  Every form writes the same T2 bits;
 *   stage1_persistent: the stage-1 stacks that split psi inside the GEMM run
 *     as one persistent, warp-specialised kernel (1: producer warps fill the
 *     psi operand and issue the TMA and MMAs of tile i + 1 while epilogue
 *     warps store tile i from the other of two TMEM accumulators) or as one
 *     CTA per tile (0, default).  Both compute the same T1 bits;
 *   stage1_narrow: the one-CTA-per-tile stage 1 takes the K of a stack in
 *     32-wide chunks through one 24 KB shared-memory stage, eight CTAs per SM
 *     (1), or in 64-wide chunks, four CTAs per SM (0, default); the same MMAs
 *     in the same order, so the same T1 bits.  Ignored with stage1_persistent.
 * tk_heff2_set_tc_options rebuilds the plan's split tables and operands;
 * FP64 matvecs are unaffected.  TK_ERR_UNSUPPORTED for complex plans. */
typedef struct {
    int32_t tall_max_mtiles;
    int32_t fuse_max_ntiles;
    int32_t combine_warps;
    int32_t stage1_persistent;
    int32_t stage1_narrow;
} tk_tc_options;
tk_status tk_heff2_set_tc_options(tk_heff2_plan* plan, const tk_tc_options* opts);
tk_status tk_heff2_get_tc_options(const tk_heff2_plan* plan, tk_tc_options* opts);

/* Autotuner (no reference counterpart; ARCHITECTURE.md's per-histogram
 * schedule choice): times `reps` split-precision matvecs of every distinct
 * candidate schedule on the plan's own sector tables (CUDA events on the
 * plan's stream, after two warm-up matvecs) and keeps the fastest.  The
 * choice is cached process-wide under the plan's sector-size histogram
 * class (quantum-number kind, physical and MPO dimensions, and for both bonds
 * the log2 buckets of the sector count, the largest sector and the total
 * dimension); with use_cache a plan of a known
 * class takes the cached choice without timing.  `out` receives the choice,
 * its time and up to 8 candidates with their times (ms per matvec). */
typedef struct {
    tk_tc_options chosen;
    float chosen_ms;
    int32_t from_cache;
    int32_t n_candidates;
    tk_tc_options candidates[8];
    float candidate_ms[8];
} tk_autotune_result;
tk_status tk_heff2_autotune(tk_heff2_plan* plan, int32_t reps, int32_t use_cache, tk_autotune_result* out);

/* Per-stage kernel timing for roofline reports (no reference counterpart;
 * observability in the spirit of DMRGStats, tk-dmrg/src/sweep/mod.rs:85-111):
 * runs `reps` complete matvecs y = H_eff x on `stream` -- the same launches
 * as tk_heff2_apply -- with a CUDA event before, between and after the
 * three stages, waits for each, and writes the mean milliseconds of stage 1
 * (L x psi GEMMs), stage 2 (W_i W_j combine) and stage 3 (x R GEMMs) to
 * ms[0..2], the algorithmic flops of each stage to flops[0..2] and its
 * compulsory global-memory bytes (operands read once, results written once,
 * in the precision the plan runs) to bytes[0..2]; flops/bytes may be NULL.
 * In split precision the W_i W_j combine of narrow stage-3 stacks runs inside
 * the stage-3 kernel; stage 2 then covers only the wide stacks' combine (0 ms
 * and 0 bytes when there are none) and stage 3 the rest, T1 reads included. */
tk_status tk_heff2_profile(tk_heff2_plan* plan, const double* x_dev, double* y_dev, void* stream,
                           int32_t reps, float* ms, double* flops, double* bytes);

/* y = H_eff x on device vectors in the block layout; stream-ordered. */
tk_status tk_heff2_apply(tk_heff2_plan* plan, const double* x_dev, double* y_dev, void* stream);
/* The closure `Fn(&[f64], &mut [f64])`: host vectors in the dense
 * (s_i, s_j, a_L, a_R) layout of length dense_dim; y fully overwritten.
 * Synchronous. */
tk_status tk_heff2_apply_host(tk_heff2_plan* plan, const double* x, double* y);
/* Same on host vectors in the block layout (FlatBlockStorage), synchronous.
 * With page-locked x and y the call runs as one CUDA graph (transfers per
 * tk_heff2_set_host_io, kernels, error-word read-back), instantiated on the
 * first call and reused while x, y and the plan settings stay the same. */
tk_status tk_heff2_apply_host_flat(tk_heff2_plan* plan, const double* x, double* y);
/* Dense <-> block layout conversion on the host. */
tk_status tk_heff2_dense_to_flat(const tk_heff2_plan* plan, const double* dense, double* flat);
tk_status tk_heff2_flat_to_dense(const tk_heff2_plan* plan, const double* flat, double* dense);

/*
 * Lanczos lowest eigenpair on the device: replaces
 * LanczosSolver::lowest_eigenpair (tk-dmrg/src/eigensolver/mod.rs:80-164).
 * Same start vector ((i*7+13)%97)/97-0.5 when x0 is NULL, full
 * re-orthogonalisation, Sturm bisection for the eigenvalue; the Ritz vector
 * is solved for (the reference leaves it unsolved) and the residual
 * ||H x - E x|| is computed with an FP64 matvec.  With a split-precision
 * plan, up to `refine` Jacobi-Davidson steps follow each Lanczos run: one
 * FP64 matvec each for an FP64 Rayleigh-Ritz step, with the correction
 * equation solved by split-precision conjugate gradients.  Vectors are in the
 * block layout on the device.
 */
typedef struct {
    int32_t krylov_dim;
    int32_t max_restarts;
    double tol;
    int32_t refine;
} tk_lanczos_cfg;

typedef struct {
    double eigenvalue;
    double residual_norm;
    int32_t converged;
    int32_t matvec_count;
    int32_t fp64_matvec_count;
    int32_t restarts;
} tk_eigen_result;

tk_status tk_lanczos_lowest(tk_heff2_plan* plan, const tk_lanczos_cfg* cfg, const double* x0_dev,
                            double* evec_dev, tk_eigen_result* out, void* stream);

/*
 * Davidson lowest eigenpair on the device: replaces
 * DavidsonSolver::lowest_eigenpair (tk-dmrg/src/eigensolver/mod.rs:325-517),
 * the sweep's default eigensolver (tk-dmrg/src/sweep/mod.rs:174-179).  Same
 * start vector as Lanczos when x0 is NULL; Rayleigh-Ritz on V^T H V each
 * iteration; stop when ||H y - theta y|| < tol; the correction is the
 * residual, divided by (theta - H_ii) where |theta - H_ii| > 1e-14 when
 * `diagonal` is given, orthogonalised against the search space, with the raw
 * residual as fallback when it collapses below 1e-14; at `max_subspace`
 * directions the space restarts from the Ritz vector (one matvec; the
 * reference's `restart_vectors` is unused there too).  Every matvec of the
 * search space is FP64.  With a split-precision plan and inner > 0 the
 * correction instead solves (I-yy^T)(H-theta)(I-yy^T) t = -r by at most
 * `inner` conjugate-gradient steps with split-precision matvecs
 * (Jacobi-Davidson), stopping once the CG residual has fallen by 1e-4;
 * inner = 0 keeps the reference's correction.  `restarts` is reported as 0.
 */
typedef struct {
    int32_t max_subspace;    /* DavidsonSolver::max_subspace (reference default 60), <= 256 */
    int32_t max_iter;        /* DavidsonSolver::max_iter (reference default 1000) */
    double tol;              /* DavidsonSolver::tol (reference default 1e-10) */
    const double* diagonal;  /* DavidsonSolver::diagonal: H_ii in the block layout (device) or NULL */
    int32_t inner;           /* split-precision plans: CG steps per correction (0: the residual) */
} tk_davidson_cfg;

tk_status tk_davidson_lowest(tk_heff2_plan* plan, const tk_davidson_cfg* cfg, const double* x0_dev,
                             double* evec_dev, tk_eigen_result* out, void* stream);

/*
 * Krylov matrix exponential out = exp(alpha H_eff) v on the device: replaces
 * exp_krylov_f64 (tk-dmrg/src/tdvp/mod.rs:197-270) and fills in the complex
 * case the reference leaves as a stub (exp_krylov<T>, :386-396) for the real
 * symmetric H_eff of a plan.  m = min(krylov_dim, dim) steps; a zero input
 * (norm < 1e-30) gives zeros; the Krylov space is cut at the first step whose
 * new norm is below `tol` (happy breakdown); exp(alpha T_m) e_1 comes from the
 * eigendecomposition of the projected tridiagonal matrix, exact for any
 * complex alpha (alpha = -dt for imaginary time, -i dt for real time).
 * v_im == NULL means a real input; out_im may be NULL only for a real input
 * and a real alpha.  Vectors are in the block layout on the device; a
 * complex input costs two matvecs per Krylov step.  Synchronous.
 */
typedef struct {
    int32_t krylov_dim;
    double tol;
} tk_expm_cfg;

typedef struct {
    int32_t krylov_used;    /* Krylov dimension after a breakdown cut */
    int32_t matvec_count;
    double input_norm;      /* ||v|| */
} tk_expm_result;

tk_status tk_expm_krylov(tk_heff2_plan* plan, const tk_expm_cfg* cfg, double alpha_re, double alpha_im,
                         const double* v_re, const double* v_im, double* out_re, double* out_im,
                         tk_expm_result* result, void* stream);

/*
 * LinAlgBackend::gemm (tk-linalg/src/traits.rs:114-121) on device memory:
 * C = alpha*op(A)*op(B) + beta*C with element strides as in MatRef/MatMut
 * (tk-core/src/matview.rs:12-33).  `is_conjugated` is a no-op for f64.
 */
typedef struct {
    const double* data;
    int64_t rows, cols, row_stride, col_stride;
    int32_t is_conjugated;
} tk_mat;

typedef struct {
    double* data;
    int64_t rows, cols, row_stride, col_stride;
} tk_mat_mut;

tk_status tk_gemm_f64(tk_ctx* ctx, double alpha, const tk_mat* a, const tk_mat* b, double beta,
                      tk_mat_mut* c, void* stream);

/*
 * No counterpart in the reference.  tk_gemm_f64 for callers that cannot
 * allocate device memory at call time (a sweep running out of a pre-sized
 * arena, a runtime that only hands over memory it manages, latency-bound
 * loops): same arguments and result, but the kernel's tile tables live in a
 * fixed 1 MiB device array inside the library instead of per-call
 * cudaMalloc'd buffers, so nothing is allocated or freed and the call does
 * not synchronise (stream-ordered on `stream`).  At most 65 520 64x64 output
 * tiles per call; larger calls return TK_ERR_INVALID_ARG.  The first call on
 * a device looks up the array's address (make it before any stream capture);
 * that address is cached for the process, so the entry point must not be
 * used again after cudaDeviceReset.  Calls share the array: calls on
 * different streams that overlap on the GPU race on it.
 */
tk_status tk_gemm_f64_noalloc(tk_ctx* ctx, double alpha, const tk_mat* a, const tk_mat* b,
                              double beta, tk_mat_mut* c, void* stream);

/*
 * SparseLinAlgBackend::block_gemm (tk-linalg/src/traits.rs:200-204,
 * tk-linalg/src/device/faer.rs:390-575) for rank-2 tensors: task per
 * compatible (key_a, key_b) pair, contributions to the same output key
 * summed, output keys ascending.  Host tensors in, host tensor out; `out`
 * arrays are allocated by the library and released by tk_bst_free.
 */
typedef struct {
    int32_t qn_kind;
    int32_t rank;
    tk_qindex legs[2];
    int8_t leg_dirs[2];
    int32_t flux[2];
    int64_t n_blocks;
    uint64_t* keys;
    int64_t* block_offsets;
    double* data;
    int64_t total;
    /* charges / dims of legs that the library made (fused legs of a
     * contraction); NULL when legs point into an input's QIndex */
    int32_t* owned_charges;
    int64_t* owned_dims;
} tk_bst_out;

/* Host tensors in, host tensor out (one copy in and one copy out through the
 * context's page-locked staging and device scratch; no device allocation once
 * the scratch has grown to the call's size).  Synchronous. */
tk_status tk_block_gemm_f64(tk_ctx* ctx, const tk_bst* a, const tk_bst* b, tk_bst_out* out);
/* The same on device buffers: a->data and b->data are device pointers in
 * the FlatBlockStorage layout.  Fills the output layout (keys, offsets,
 * total; out->data stays NULL) and, when c_dev is not NULL, computes C into
 * c_dev (out->total doubles) on `stream`, waiting for it before returning
 * (the tables live in the context's shared scratch).  Call once with
 * c_dev = NULL to size the output buffer. */
tk_status tk_block_gemm_f64_dev(tk_ctx* ctx, const tk_bst* a, const tk_bst* b, tk_bst_out* out, double* c_dev,
                                void* stream);
/* Releases the arrays of a tk_bst_out (keys, offsets, data, owned legs). */
void tk_bst_free(tk_bst_out* t);

/*
 * One pairwise step of the block-sparse contraction executor:
 * SparseContractionExecutor::execute_pairwise_sparse with reshape_for_gemm
 * (tk-contract/src/sparse.rs:124-265).  A's legs a_legs[0..n) and B's legs
 * b_legs[0..n) are contracted: each operand is permuted (free legs, then
 * contracted legs, each in ascending leg order; contracted first for B),
 * its free and its contracted legs are fused into one leg each
 * (BlockSparseTensor::fuse_legs, tk-symmetry/src/block_sparse.rs:444-611:
 * a fused leg is Incoming, sectors = distinct fused charges ascending,
 * combinations in Cartesian order inside a sector; a single leg stays as it
 * is), and the rank-2 operands are multiplied as by tk_block_gemm_f64.  The
 * result is the rank-2 tensor (fused free legs of A, fused free legs of B)
 * in FlatBlockStorage form; its fused legs are owned by `out` (released by
 * tk_bst_free).  Host tensors in and out, ranks 1 to 8; the permutation, the
 * fusion and the GEMM run on the device through the context's scratch.
 * An operand without a free or without a contracted leg is
 * TK_ERR_UNSUPPORTED.  Synchronous.
 */
tk_status tk_contract_pairwise_f64(tk_ctx* ctx, const tk_bst* a, const int32_t* a_legs, int32_t n_a,
                                   const tk_bst* b, const int32_t* b_legs, int32_t n_b, tk_bst_out* out);

/* All eigenpairs of `batch` symmetric n x n matrices (host memory, each
 * matrix n*n doubles back to back; symmetric, so row- and column-major
 * agree; the lower triangle is read): w_host[b*n + j] ascending eigenvalues
 * of matrix b, z_host[b*n*n + i + j*n] component i of its eigenvector j
 * (column-major).  One cuSOLVER batched call (syevBatched) on the device.
 * Serves the density-matrix truncation of a two-site split, one matrix per
 * bond charge padded to a common n (no reference counterpart; the reference
 * diagonalises sector by sector on the CPU, truncation/mod.rs:71-99 via
 * LinAlgBackend::svd_truncated). */
tk_status tk_eigh_batched_f64(tk_ctx* ctx, int64_t n, int64_t batch, const double* a_host, double* w_host,
                              double* z_host);
/*
 * The dense factorisations of LinAlgBackend (tk-linalg/src/traits.rs:63-148) on
 * device matrices (tk_mat strides, real f64), with the faer backend's result
 * conventions (tk-linalg/src/device/faer.rs:127-325).  Synchronous.
 *   tk_svd_truncated_f64: svd_truncated_gesdd -- singular values descending,
 *     rank = count of sigma >= cutoff * sigma_max up to max_rank, truncation
 *     error = sum of the discarded sigma^2; U (m x rank) and Vt (rank x n)
 *     row-major into device buffers of m*min(m,n) and min(m,n)*n doubles;
 *     the kept singular values into s_host (min(m,n) doubles).
 *   tk_eigh_lowest_f64: the k lowest eigenpairs of a symmetric matrix,
 *     eigenvalues ascending (host), eigenvectors as the columns of an (n x k)
 *     row-major device matrix; k > n is TK_ERR_INVALID_ARG (EighKTooLarge).
 *   tk_qr_f64: thin QR, Q (m x k) and R (k x n) row-major, k = min(m, n).
 */
tk_status tk_svd_truncated_f64(tk_ctx* ctx, const tk_mat* a, int64_t max_rank, double cutoff, double* u_dev,
                               double* s_host, double* vt_dev, int64_t* rank, double* truncation_error,
                               void* stream);
tk_status tk_eigh_lowest_f64(tk_ctx* ctx, const tk_mat* a, int64_t k, double* evals_host, double* evecs_dev,
                             void* stream);
tk_status tk_qr_f64(tk_ctx* ctx, const tk_mat* a, double* q_dev, double* r_dev, void* stream);

/*
 * The same three factorisations for complex (C64) matrices, the reference's
 * `LinAlgBackend<C64>` (traits.rs:63-148 for T = Complex<f64>; faer.rs conventions),
 * in the planar form the rest of this interface uses for complex data:
 * element (i, j) = re[i*row_stride + j*col_stride] + i * im[...], and
 * `is_conjugated` makes the matrix stand for its elementwise conjugate
 * (MatRef::is_conjugated).  Outputs are planar row-major device buffers of
 * the real versions' shapes:
 *   tk_svd_truncated_c64: A = U S V^H; U (m x rank), Vt = V^H (rank x n),
 *     singular values (real) descending, the same rank rule and truncation
 *     error as tk_svd_truncated_f64;
 *   tk_eigh_lowest_c64: a Hermitian matrix (lower triangle read), the k lowest
 *     eigenvalues (real, ascending) and eigenvectors as the columns of n x k;
 *   tk_qr_c64: thin QR with Q unitary-column (m x k) and R upper (k x n).
 */
typedef struct {
    const double* re;
    const double* im;
    int64_t rows, cols, row_stride, col_stride;
    int32_t is_conjugated;
} tk_cmat;
tk_status tk_svd_truncated_c64(tk_ctx* ctx, const tk_cmat* a, int64_t max_rank, double cutoff, double* u_re,
                               double* u_im, double* s_host, double* vt_re, double* vt_im, int64_t* rank,
                               double* truncation_error, void* stream);
tk_status tk_eigh_lowest_c64(tk_ctx* ctx, const tk_cmat* a, int64_t k, double* evals_host, double* evecs_re,
                             double* evecs_im, void* stream);
tk_status tk_qr_c64(tk_ctx* ctx, const tk_cmat* a, double* q_re, double* q_im, double* r_re, double* r_im,
                    void* stream);

/* SparseLinAlgBackend::spmv (tk-linalg/src/traits.rs:193-198): y = A x for
 * a rank-2 host tensor and host vectors (y fully overwritten). */
tk_status tk_spmv_f64(tk_ctx* ctx, const tk_bst* a, const double* x, double* y);

/*
 * Complex (planar) variants for real-time evolution: build_heff_two_site and
 * the environment contractions are generic over the scalar type in the
 * reference (T = C64 included); here complex environments and vectors are
 * stored as separate real and imaginary arrays in the same layouts, and each
 * complex sector GEMM runs as four real grouped GEMMs over the same tables.
 * FP64 only.  The MPO stays real.
 *   tk_heff2_plan_create_dev_complex: as tk_heff2_plan_create_dev with the
 *     imaginary parts of both environments (device, canonical layout).
 *   tk_heff2_apply_complex: y = H_eff x on planar device vectors.
 *   tk_env_grow_left/right_complex: the contractions with conj(A) on the bra.
 *   tk_heff2_two_site_product_complex: psi = A_i A_j.
 * tk_expm_krylov on a complex plan treats its input as complex (v_im may be
 * NULL for a zero imaginary part) and needs out_im.
 */
tk_status tk_heff2_plan_create_dev_complex(tk_ctx* ctx, const tk_env* env_l, const double* env_l_im,
                                           const tk_env* env_r, const double* env_r_im, const tk_bst* w_i,
                                           const tk_bst* w_j, const int32_t* psi_flux, tk_heff2_plan** out);
tk_status tk_heff2_apply_complex(tk_heff2_plan* plan, const double* x_re, const double* x_im, double* y_re,
                                 double* y_im, void* stream);
tk_status tk_env_grow_left_complex(tk_ctx* ctx, const tk_env* env_l, const double* env_l_im, const tk_bst* a,
                                   const double* a_im, const tk_bst* w, double* out_re, double* out_im, void* stream);
tk_status tk_env_grow_right_complex(tk_ctx* ctx, const tk_env* env_r, const double* env_r_im, const tk_bst* a,
                                    const double* a_im, const tk_bst* w, double* out_re, double* out_im, void* stream);
tk_status tk_heff2_two_site_product_complex(tk_heff2_plan* plan, const tk_bst* a_i, const double* a_i_im,
                                            const tk_bst* a_j, const double* a_j_im, double* psi_re, double* psi_im,
                                            void* stream);

/*
 * Self-check, no reference counterpart: the split-precision kernels convert
 * psi from fp64 to fp32 from the IEEE 754 bit layouts on the integer pipes
 * (the FP64 pipe of this GPU is narrow).  Compares that conversion with the
 * hardware one on n device doubles (where the result is a normal fp32) and
 * writes the number of mismatches to *mismatches.  Synchronous.
 */
tk_status tk_check_split_conversions(tk_ctx* ctx, const double* x_dev, int64_t n, uint64_t* mismatches);

/*
 * Device-resident environments for two-site sweeps.  The reference's
 * Environment (tk-dmrg/src/environments/mod.rs:24-103) is a dense
 * (bra, w, ket) array; a symmetric environment is non-zero only on sector
 * triples with q(bra) = q(ket) + q(w), and these calls keep exactly those
 * blocks: the canonical block layout lists every such triple, ascending by
 * packed rank-3 key (bra leg in the low bits), blocks back to back, each
 * row-major (a', w, a).  In the calls below a tk_env's `data` is a device
 * pointer to that layout.
 */
/* Block count, keys, offsets (nullable: counts only; otherwise *n_blocks is
 * the capacity on entry) and total length of the canonical layout. */
tk_status tk_env_layout(int32_t qn_kind, const tk_qindex* bra, const tk_qindex* mpo, const tk_qindex* ket,
                        int64_t* n_blocks, uint64_t* keys, int64_t* block_offsets, int64_t* total);
/* build_heff_two_site (environments/mod.rs:491-602) over device environments
 * in the canonical layout; otherwise as tk_heff2_plan_create.  The
 * environments are read once during the call. */
tk_status tk_heff2_plan_create_dev(tk_ctx* ctx, const tk_env* env_l, const tk_env* env_r, const tk_bst* w_i,
                                   const tk_bst* w_j, const int32_t* psi_flux, int32_t precision,
                                   tk_heff2_plan** out);
/* contract_left_environment (environments/mod.rs:221-355):
 *   L'[b', v, b] = sum conj(A[s', a', b']) L[a', w, a] W[s, s', w, v] A[s, a, b]
 * A: rank-3 MPS site tensor (s, a_L, a_R), blocks with q(s) + q(a_L) = q(a_R),
 * host keys/offsets and DEVICE data; W: rank-4 MPO site tensor, host data.
 * L lies on (A's left bond, W's left bond); out_dev receives the canonical
 * layout of (A's right bond, W's right bond, A's right bond), fully written.
 * Stream-ordered; no host synchronisation. */
tk_status tk_env_grow_left(tk_ctx* ctx, const tk_env* env_l, const tk_bst* a, const tk_bst* w, double* out_dev,
                           void* stream);
/* contract_right_environment (environments/mod.rs:357-483):
 *   R'[a', w, a] = sum conj(A[s', a', b']) R[b', v, b] W[s, s', w, v] A[s, a, b]
 * R lies on (A's right bond, W's right bond); out_dev receives the canonical
 * layout of (A's left bond, W's left bond, A's left bond). */
tk_status tk_env_grow_right(tk_ctx* ctx, const tk_env* env_r, const tk_bst* a, const tk_bst* w, double* out_dev,
                            void* stream);
/* Two-site start vector psi(s_i, s_j, a, b) = sum_c A_i(s_i, a, c) A_j(s_j, c, b)
 * in the plan's block layout (device data in, device vector out).  The
 * reference's sweep starts its eigensolver from no vector
 * (sweep/mod.rs:390-396); this is the usual two-site guess instead. */
tk_status tk_heff2_two_site_product(tk_heff2_plan* plan, const tk_bst* a_i, const tk_bst* a_j, double* psi_dev,
                                    void* stream);

/*
 * The two-site truncation's data path (no single reference counterpart: it
 * moves the data for truncate_svd, tk-dmrg/src/truncation/mod.rs:56-127,
 * applied to every bond charge of the two-site matrix
 * M[(s_i, a_L), (s_j, a_R)], which is block diagonal in
 * q = q(s_i) + q(a_L) = q(a_R) - q(s_j) for a flux-zero two-site vector).
 * Rows of M_q: (s_i state, a_L sector), states then sectors ascending;
 * columns (s_j state, a_R sector) likewise; charges ascending.
 *   tk_split_plan_create: from the two-site block layout (legs s_i, s_j, a_L,
 *     a_R; keys and offsets as tk_heff2_blocks returns them), host only.
 *   tk_split_charges: the charges (ncomp int32 each) and the rows / columns
 *     of each M_q; any array may be NULL.
 *   tk_split_gather: every M_q from the device vector psi_dev, packed charge
 *     after charge (row-major), copied to m_host (sum of rows x cols doubles;
 *     page-locked memory copies fastest).  Synchronous on `stream`.
 *   tk_split_set_kept: kept[i] states of charge i (0 .. min(rows, cols));
 *     returns the block counts and lengths of the new site tensors A_i
 *     (s_i, a_L, bond) and A_j (s_j, bond, a_R), bond = the charges with
 *     kept[i] > 0, ascending.
 *   tk_split_layout: their packed keys and block offsets (side 0: A_i, 1: A_j).
 *   tk_split_factors: u_host packs U_q (rows x kept, row-major) and v_host
 *     V_q (kept x cols, row-major) charge after charge (charges with kept 0
 *     take no space); they are scattered into the device buffers ai_dev and
 *     aj_dev (the caller scales them, e.g. A_i = U, A_j = S V^T / norm).
 *     Synchronous on `stream`.
 * The calls use the context's scratch and are not thread-safe per context.
 */
typedef struct tk_split_plan tk_split_plan;
tk_status tk_split_plan_create(tk_ctx* ctx, int32_t qn_kind, const tk_qindex* legs, int64_t n_blocks,
                               const uint64_t* keys, const int64_t* offsets, tk_split_plan** out);
void tk_split_plan_destroy(tk_split_plan* split);
tk_status tk_split_charges(const tk_split_plan* split, int32_t* n_charges, int32_t* charges, int64_t* rows,
                           int64_t* cols);
tk_status tk_split_gather(tk_split_plan* split, const double* psi_dev, double* m_host, void* stream);
tk_status tk_split_set_kept(tk_split_plan* split, const int64_t* kept, int64_t* n_blocks_i, int64_t* total_i,
                            int64_t* n_blocks_j, int64_t* total_j);
tk_status tk_split_layout(const tk_split_plan* split, int32_t side, uint64_t* keys, int64_t* offsets);
tk_status tk_split_factors(tk_split_plan* split, const double* u_host, const double* v_host, double* ai_dev,
                           double* aj_dev, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TK_HEFF_H */
