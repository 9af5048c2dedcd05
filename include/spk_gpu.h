/*
 * spk_gpu.h - C ABI of the GB300 (sm_103a) numeric engine for the Sparspak
 * LU SparseSolver.
 *
 * The host keeps ordering, elimination tree and symbolic factorisation (see
 * spk_host.h) and hands the resulting supernodal structure to this library,
 * which owns all numeric work on one GPU: value assembly (_inmatrix!), the
 * supernodal LU with in-block partial pivoting (_lufactor!), the triangular
 * solves (_lulsolve!/_luusolve!), a residual and iterative refinement.
 * There is no CPU fallback: without a usable CUDA device every call fails.
 *
 * Conventions
 *  - Structure arrays are int64 and use the reference's layout; index_base
 *    says whether their values are 1-based (the reference's) or 0-based.
 *  - Every function returns SPK_OK (0) or a negative SPK_E* code, never
 *    throws across the ABI, and leaves a message for spk_last_error().
 *  - A handle is used by one host thread at a time.  Work is issued on the
 *    handle's stream (spk_set_stream); functions that return results to the
 *    host synchronise that stream before returning.
 *  - `where` arguments: SPK_HOST for host memory, SPK_DEVICE for device
 *    memory of the handle's device.
 */
#ifndef SPK_GPU_H
#define SPK_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPK_OK 0
#define SPK_EARG (-1)      /* invalid argument                                    */
#define SPK_ECUDA (-2)     /* CUDA runtime error (no device, launch failure, ...)  */
#define SPK_ENOMEM (-3)    /* device or host allocation failed                     */
#define SPK_ESEQ (-4)      /* call out of sequence (e.g. solve before factor)      */
#define SPK_ESTRUCT (-5)   /* structure inconsistent, or A has an entry with no
                              slot in the factor ("No space for matrix element")   */
#define SPK_ESINGULAR (-6) /* a diagonal block had an exactly zero pivot           */
#define SPK_ENOCONV (-7)   /* refinement did not reach the requested tolerance     */
#define SPK_ETIMEOUT (-8)  /* a bounded device wait ran out (no progress within its
                              budget): the factors are invalid, the context stays
                              usable and the next spk_factor reassembles A       */

#define SPK_HOST 0
#define SPK_DEVICE 1

#define SPK_FP64 0         /* factor, solve and residual in double                */
#define SPK_FP32 1         /* factor and solve in float; residual and correction
                              in double (mixed form for spk_refine); the large
                              rank updates as 3xTF32 tensor-core products        */
#define SPK_SPD 16         /* flag, or-ed with a precision: the symmetric form for
                              symmetric positive definite A (the SPD solver's
                              Cholesky, src/SparseSpdMethod/SpkLDLtFactor.jl,
                              on the LU supernode partition): no interchanges
                              (POTRF-like diagonal blocks), only the lower part
                              of every rank update is formed (SYRK-like, half
                              the update flops) and the U side, U = D L^T, is
                              written from the L panels; solves as for LU.
                              Its own factor storage, beside the LU one.     */
#define SPK_BF16S 2        /* as SPK_FP32, but the large rank updates (Schur
                              complements and trailing updates) take BF16
                              operands with a power-of-two scale per block panel
                              and FP32 accumulation on the tensor cores; for
                              spk_refine, GMRES-IR when plain refinement
                              stagnates                                          */

typedef struct spk_handle spk_handle;

/*
 * Create a handle for one supernodal structure and copy it to the device.
 * Replaces the allocation of lnz/unz/ipiv at the end of _symbolicfactor!
 * (src/SparseMethod/SpkSparseBase.jl:236-248) and precomputes, once per
 * structure, what _lufactor! rebuilds on every call: the relative index
 * maps of _ldindx!/_igathr! (src/SparseSpdMethod/SpkSpdMMOps.jl:70-102) and
 * the order of supernode updates (the link lists of
 * src/SparseMethod/SpkLUFactor.jl:89-228), as an elimination-tree level
 * schedule.  Arrays: xsuper[nsuper+1], snode[n], xlindx[nsuper+1],
 * lindx[xlindx[nsuper+1]-1], xlnz[n+1], xunz[n+1] (reference meaning).
 * Supernodes may be at most 64 columns wide (with maxblocksize 30 the
 * reference's splitting rule yields pieces of up to 46 columns).
 */
int spk_create(int64_t n, int64_t nsuper, const int64_t* xsuper, const int64_t* snode,
               const int64_t* xlindx, const int64_t* lindx, const int64_t* xlnz,
               const int64_t* xunz, int index_base, spk_handle** out);

/* Issue all further work of this handle on `stream` (a cudaStream_t, or
 * NULL for the handle's own stream). */
int spk_set_stream(spk_handle* h, void* stream);

/*
 * Fix the sparsity pattern of A (CSC: colptr[ncols+1], rowval[nnz]) and the
 * permutation (rperm[new] = old, rinvp[old] = new; rows and columns are
 * permuted alike, as in the reference).  Builds the value -> factor-slot map
 * that _inmatrix! finds by linear search for every entry
 * (src/SparseCSCInterface/SparseCSCInterface.jl:101-169 and
 * src/SparseMethod/SpkSparseBase.jl:302-372), and the row-ordered copy of
 * the pattern used by the residual.  Fails with SPK_ESTRUCT, naming the
 * entry, when an entry of A has no slot in the factor.
 */
int spk_set_pattern(spk_handle* h, int64_t ncols, const int64_t* colptr, const int64_t* rowval,
                    const int64_t* rperm, const int64_t* rinvp, int index_base);

/*
 * Load the values of A (nzval[nnz], in the CSC order given to
 * spk_set_pattern) into the factor storage of the given precision: zero
 * the storage, then scatter-add each value into its slot.  Replaces the body
 * of _inmatrix!.  Also keeps an FP64 copy of A on the device for spk_refine.
 */
int spk_load_values(spk_handle* h, const double* nzval, int where, int precision);

/*
 * Numeric LU factorisation in place, in the given precision.  Replaces
 * _lufactor! (src/SparseMethod/SpkLUFactor.jl:60-255) as called by _factor!
 * (src/SparseMethod/SpkSparseBase.jl:378-391): the same supernode partition,
 * in-block partial pivoting with the first strict maximum as pivot
 * (src/Utilities/GenericBlasLapackFragments.jl:56-100) and the same pivots.
 * *first_singular (may be NULL) receives 0, or the 1-based index of the
 * first supernode whose diagonal block had an exactly zero pivot, in which
 * case the call returns SPK_ESINGULAR (the reference only reports the last
 * supernode's status, SpkLUFactor.jl:230-233).
 */
int spk_factor(spk_handle* h, int precision, int64_t* first_singular);

/*
 * Solve A X = B for nrhs right-hand sides stored column-major with leading
 * dimension ldb, in original (unpermuted) order, overwritten by X.  Uses the
 * factor of the given precision.  Replaces _triangularsolve!
 * (src/SparseMethod/SpkSparseBase.jl:400-416) = permute, _lulsolve!,
 * _luusolve! (src/SparseMethod/SpkLUFactor.jl:269-377), unpermute; the
 * reference solves one vector per call.
 */
int spk_solve(spk_handle* h, double* b, int64_t nrhs, int64_t ldb, int where, int precision);

/*
 * Solve A^T X = B with the same factors, arguments as spk_solve.  Replaces
 * the reference's transposed solve, which exists only as a commented-out
 * `transposetriangularsolve` (src/SparseSpdMethod/SpkSparseSpdSolver.jl:384):
 * U^T is applied in the forward order of the fronts and blocks, then L^T
 * (with the in-block interchanges transposed) in the backward order.
 */
int spk_solve_transpose(spk_handle* h, double* b, int64_t nrhs, int64_t ldb, int where, int precision);

/*
 * Iterative refinement: x := solve(b) with the factor of `precision`, then
 * repeat r = b - A x (FP64), x += solve(r) until max_j ||r_j||_2/||b_j||_2
 * <= tol or max_iter corrections were applied.  b and x are n x nrhs,
 * column-major, leading dimension ld, original order.  Reports the number
 * of corrections and the final relative residual.  Returns SPK_ENOCONV if
 * tol was not reached.  Modelled on the reference's commented-out
 * refinement (src/SparseSpdMethod/SpkSparseSpdSolver.jl:267-343).  When a
 * correction fails to halve the residual (as with SPK_BF16S factors of
 * ill-conditioned systems) it continues with GMRES-IR (spk_refine_ex,
 * SPK_SOLVER_AUTO).
 */
int spk_refine(spk_handle* h, const double* b, double* x, int64_t nrhs, int64_t ld, int where,
               int precision, double tol, int max_iter, int* iters, double* relres);

/*
 * Iterative refinement with a choice of solver for the correction equation
 * A d = r (no counterpart in the reference):
 *   SPK_SOLVER_IR     plain refinement, d = solve(r), as spk_refine;
 *   SPK_SOLVER_GMRES  GMRES-IR: restarted GMRES in FP64 on A d = r,
 *                     preconditioned on the right by the factor of
 *                     `precision` (one triangular solve per iteration);
 *   SPK_SOLVER_AUTO   plain refinement while each correction at least halves
 *                     the residual, then (a correction that made it worse is
 *                     taken back) GMRES-IR; spk_refine behaves like this.
 * max_iter bounds the preconditioned solves after the first (corrections
 * plus GMRES iterations), reported in *iters; *solver_used (may be NULL)
 * receives SPK_SOLVER_IR or SPK_SOLVER_GMRES.  Other arguments and results
 * as spk_refine.
 */
#define SPK_SOLVER_AUTO 0
#define SPK_SOLVER_IR 1
#define SPK_SOLVER_GMRES 2
int spk_refine_ex(spk_handle* h, const double* b, double* x, int64_t nrhs, int64_t ld, int where, int precision,
                  double tol, int max_iter, int solver, int* iters, double* relres, int* solver_used);

/*
 * Factorisation and refined solve in one call (the role of the reference's
 * solve!, which runs factor! and the triangular solve in turn,
 * src/SparseMethod/SpkSparseSolver.jl:237-256): spk_factor, then
 * spk_refine_ex, with the first solve's forward substitution of all but the
 * last two levels of the front tree run beside the factorisation of those
 * two levels (once its fronts are final).  Same arguments and results as
 * spk_refine_ex, plus *first_singular (may be NULL) as spk_factor.  At most
 * MAXRHS (16) right-hand sides take the overlapped path; more are factored
 * and refined one after the other.
 */
int spk_factor_refine(spk_handle* h, const double* b, double* x, int64_t nrhs, int64_t ld, int where, int precision,
                      double tol, int max_iter, int solver, int* iters, double* relres, int* solver_used,
                      int64_t* first_singular);

/* Iterative refinement of A^T x = b (spk_solve_transpose and the FP64
 * residual b - A^T x), arguments and results as spk_refine. */
int spk_refine_transpose(spk_handle* h, const double* b, double* x, int64_t nrhs, int64_t ld, int where,
                         int precision, double tol, int max_iter, int* iters, double* relres);

/*
 * Gradient with respect to A's stored entries: dA[k] = -sum_r lambda_r[i_k]
 * x_r[j_k] for the entries (i_k, j_k) of the pattern given to
 * spk_set_pattern, in its CSC order.  For a loss of x = A^{-1} b, lambda is
 * the adjoint A^{-T} dloss/dx (spk_solve_transpose / spk_refine_transpose).
 * lambda and x are n x nrhs, column-major, leading dimension ld, original
 * order.  The reference's only derivative path is forward-mode Dual numbers
 * through its generic Julia code (test/test_generic.jl:58-98).
 */
int spk_grad_pattern(spk_handle* h, const double* lambda, const double* x, int64_t nrhs, int64_t ld, int where,
                     double* dA);

/*
 * Relative residual max_j ||b_j - A x_j||_2 / ||b_j||_2 in FP64 for the
 * current A (the reference's analogue is computeresidual,
 * src/Problem/SpkProblem.jl:448-496).
 */
int spk_residual(spk_handle* h, const double* b, const double* x, int64_t nrhs, int64_t ld,
                 int where, double* relres);

/*
 * Allocation-free residual (no counterpart in the reference).  Same result
 * as spk_residual with device-resident b and x (n x nrhs, leading dimension
 * ld), for callers that cannot allocate device memory when they call the
 * library: applications that hand all device memory to their own pool or
 * run under a fixed memory budget (a cudaMalloc there fails or evicts
 * something else), and latency-critical loops that cannot afford the
 * device-wide synchronisation cudaMalloc/cudaFree may cause.  It calls no
 * cudaMalloc/cudaFree and no allocating library routine: its only work space
 * (two doubles per right-hand side) is a file-scope device array of the
 * library, held by every device that loads it until the process exits.
 * At most SPK_NOALLOC_MAX_RHS right-hand sides per call (SPK_EARG beyond).
 * Like spk_residual it waits for the handle's stream before it returns, so
 * it cannot be part of a stream capture: called while the handle's stream
 * is capturing it returns SPK_ESEQ and leaves the capture untouched.
 * The first call on a device looks up that array's device address (with the
 * device current) and keeps it for the life of the process, so make the
 * first call before any stream capture, and do not use it across a
 * cudaDeviceReset.  All calls share the array (it is cleared at the start of
 * each call): calls that overlap on the GPU, from any handle on the same
 * device, race.
 */
#define SPK_NOALLOC_MAX_RHS 64
int spk_residual_noalloc(spk_handle* h, const double* b, const double* x, int64_t nrhs, int64_t ld, double* relres);

/*
 * Copy the factor of the given precision back in the reference's layout:
 * lnz[xlnz[n+1]-1], unz[xunz[n+1]-1] and ipiv[n] (1-based, local to each
 * supernode's diagonal block), exactly as _SparseBase holds them after
 * factor! (src/SparseMethod/SpkSparseBase.jl:99-125).  Before spk_factor
 * (after spk_load_values) it returns the assembled A, with ipiv all zero, as
 * after inmatrix!.  Any pointer may be NULL.  With SPK_SPD: the Cholesky
 * factor C (A = C C^T) in lnz's lower part (each supernode's diagonal block
 * and the rows below it, the layout of the SPD solver's lnz,
 * src/SparseSpdMethod/SpkSparseSpdBase.jl:210-227), C^T in the upper part
 * of the diagonal blocks and in unz, ipiv the identity; SPK_ESINGULAR if a
 * pivot is not positive.
 */
int spk_get_factors(spk_handle* h, int precision, double* lnz, double* unz, int64_t* ipiv);

/* Statistics of the structure: fronts (merged chains of supernodes), levels of
 * the schedule, factor entries, and the LU flop count sum_j (c_j-1)+2(c_j-1)^2. */
int spk_stats(spk_handle* h, int64_t* nfronts, int64_t* nlevels, int64_t* factor_entries,
              double* lu_flops);

/* Kernel classes for launch accounting and event timing. */
#define SPK_K_ASSEMBLE 0   /* value scatter (_inmatrix!)                        */
#define SPK_K_GETRF 1      /* first diagonal block of each front                */
#define SPK_K_PANEL 2      /* panel triangular solves (_trsm!, _luswap!)         */
#define SPK_K_TRAIL 3      /* rank-w update inside a front, CUDA cores           */
#define SPK_K_SCHUR 4      /* front Schur complement + scatter-add (_gemm!, _assmb!),
                              CUDA cores                                         */
#define SPK_K_FWD 5        /* forward substitution (_lulsolve!)                 */
#define SPK_K_BWD 6        /* backward substitution (_luusolve!)                */
#define SPK_K_PERMUTE 7    /* right-hand side permutation                       */
#define SPK_K_RESIDUAL 8   /* r = b - A x                                       */
#define SPK_K_BLOCKINV 9   /* whole-block solve operators, after the factorisation */
#define SPK_K_TC_TRAIL 10  /* rank-w update inside a front, tensor cores (tcgen05) */
#define SPK_K_TC_SCHUR 11  /* front Schur complement + scatter-add, tensor cores  */
#define SPK_K_COUNT 12

/*
 * Launch accounting (no counterpart in the reference, whose only timing is
 * the tests' @time).  Every kernel launch of the handle is counted with its
 * algorithmic flops and bytes; spk_profile(h, mask) additionally brackets
 * each launch of the classes in `mask` (bit SPK_K_*) with CUDA events on the
 * handle's stream.  spk_profile_read returns, for one class since the last
 * spk_profile_reset: summed event time in ms (0 for untimed classes),
 * launches, algorithmic flops and algorithmic bytes.
 */
int spk_profile(spk_handle* h, unsigned mask);
int spk_profile_reset(spk_handle* h);
int spk_profile_read(spk_handle* h, int kind, double* ms, int64_t* launches, double* flops, double* bytes);

/*
 * Measured throughput of the current device (no counterpart in the
 * reference; the denominators of the CUDA-core kernels' roofline figures):
 * FP32 FMA, FP64 FMA and FP64 tensor-core (mma.sync m8n8k4 f64) rates in
 * TFLOP/s, each from one timed launch of several CTAs per SM running
 * independent chains.  Any pointer may be NULL.
 */
int spk_measure_peaks(double* fp32_tflops, double* fp64_tflops, double* dmma_tflops);

/*
 * Options of the factorisation (no counterpart in the reference).  Changing
 * one takes effect at the next spk_factor; the tensor-core thresholds also
 * discard the FP32 / BF16S factors (factor again after spk_load_values).
 *  SPK_OPT_LEAF_QUEUE    1: the bottom subtrees of small fronts (one block
 *                        of at most 32 columns, at most 32 rows below it,
 *                        every descendant alike) are factored by one
 *                        persistent launch: a work queue in level order with
 *                        a dependency counter per front and bounded waits;
 *                        0 (default): one launch per level and width class.
 *                        The reference's own work list is the `link` list of
 *                        _lufactor! (src/SparseMethod/SpkLUFactor.jl:89-228).
 *  SPK_OPT_WAIT_BUDGET   polls of a queue wait before it gives up and the
 *                        factorisation returns SPK_ETIMEOUT (default 2^20,
 *                        about a second at the longest).
 *  SPK_OPT_STALL_TEST    test hook: the queue position whose wait nothing
 *                        ends (-1, the default: none); with a small budget it
 *                        shows the timeout path without a GPU fault.
 *  SPK_OPT_TC_SCHUR_M    FP32 / BF16S: a front with at least this many rows
 *                        below its pivot columns takes the tensor-core rank
 *                        updates (default 96);
 *  SPK_OPT_TC_TRAIL_ROWS or one of several blocks with at least this many
 *                        rows below its first block (default 128).
 *  SPK_OPT_TC_WIDE       1 (default): the tensor-core Schur complements in
 *                        tiles of 128 x 256 (each staged L chunk serves two
 *                        products); 0: tiles of 128 x 128.
 *  SPK_OPT_LU_PIECES     1: blocks whose pieces (supernodes) are all at
 *                        most 32 columns wide are factored piece by piece
 *                        (a warp per piece's diagonal block, then the block's
 *                        triangular solves and update in parallel): the
 *                        reference's operation order (ggetrf!, trsm, gemm
 *                        per supernode), hence FP64 factors closer to its
 *                        rounding, but a slower chain on GB300 (the piece's
 *                        column steps are as long as the block form's);
 *                        0 (default): every wide block in column groups.
 *  SPK_OPT_SOLVE_CLUSTER_MINB  fronts of at least this many blocks (2..128,
 *                        default 4) are solved by one 16-CTA cluster each
 *                        (all block steps in one launch); smaller ones by a
 *                        launch per block step.  Keeps the factors.
 *  SPK_OPT_PANEL_SPLIT   1 (default): in the float forms, a block step
 *                        whose trailing update is all on the tensor cores
 *                        launches its panel in two parts: the lines the next
 *                        block's diagonal block is updated from (the first
 *                        128 rows below the block and columns right of it)
 *                        on the launch stream, the others beside them on the
 *                        look-ahead stream; 0: one panel launch.  The same
 *                        arithmetic either way.
 *  SPK_OPT_SCHUR_SPLIT   1 (default): in the float forms, the tiles of a
 *                        level's tensor-core Schur complements whose target
 *                        fronts (the owner of the smaller of row and column)
 *                        are factored two or more levels up run on a third
 *                        stream on SPK_OPT_SCHUR_FAR_SMS SMs, beside the
 *                        next level's factorisation, and are awaited two
 *                        levels on, before any of their targets is
 *                        factored; 0: all tiles before the next level.
 *                        Atomic scatter-adds either way (the sums come in
 *                        another order: FP32 rounding).
 *  SPK_OPT_SCHUR_FAR_SMS CTAs (one per SM) of those far tiles (0, the
 *                        default: seven eighths of the SMs; the launch
 *                        stream's kernels take SMs first as they free up).
 *  SPK_OPT_SOLVE_CHUNK   1 (default): a root front (no rows below it) of more
 *                        than 16 blocks is solved in chunks of at most 16
 *                        consecutive blocks, one cluster launch each, the
 *                        chunks linked by a product over all SMs (forward
 *                        the L rows below a chunk, backward the U rows
 *                        above it); 0: one cluster launch.  Keeps the
 *                        factors.
 */
#define SPK_OPT_LEAF_QUEUE 0
#define SPK_OPT_WAIT_BUDGET 1
#define SPK_OPT_STALL_TEST 2
#define SPK_OPT_TC_SCHUR_M 3
#define SPK_OPT_TC_TRAIL_ROWS 4
#define SPK_OPT_TC_WIDE 5
#define SPK_OPT_LU_PIECES 6
#define SPK_OPT_SOLVE_CLUSTER_MINB 7
#define SPK_OPT_PANEL_SPLIT 8
#define SPK_OPT_SCHUR_SPLIT 9
#define SPK_OPT_SCHUR_FAR_SMS 10
#define SPK_OPT_SOLVE_CHUNK 11
int spk_set_option(spk_handle* h, int option, int64_t value);
int spk_get_option(spk_handle* h, int option, int64_t* value);

/*
 * Tune the options above for the loaded A in the given precision (no
 * counterpart in the reference): times `reps` factorisations (median, CUDA
 * events, after one untimed) with the leaf queue off and on, then, for the
 * float forms, a set of tensor-core thresholds and the Schur tile width;
 * keeps the fastest, leaves A
 * assembled for spk_factor and returns the best factor time in *best_ms (may
 * be NULL).  Needs spk_load_values first.
 */
int spk_autotune(spk_handle* h, int precision, int reps, double* best_ms);

/* Text of the last error on this handle (never NULL); with h == NULL, the
 * reason the last spk_create on this thread failed. */
const char* spk_last_error(spk_handle* h);

/* Release the handle and its device memory. */
void spk_destroy(spk_handle* h);

#ifdef __cplusplus
}
#endif

#endif /* SPK_GPU_H */
