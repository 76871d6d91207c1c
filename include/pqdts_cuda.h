/*
 * pqdts_cuda.h -- C ABI of libpqdts_cuda.so, the GB300 (sm_103a) drop-in for
 * the two-metric projected truncated Newton solve of pc2/pqdts.
 *
 * Every entry point is extern "C" with plain pointers and fixed-width
 * scalars only, so it binds from Fortran (iso_c_binding, see
 * pqdts_gb300/fortran/pqdts_cuda_mod.f90), C/C++ and Python ctypes.
 *
 * Conventions
 *   - Return value: 0 on success, a negative PQDTS_E* code on failure; the
 *     message is available from pqdts_cuda_last_error().  No entry point
 *     aborts the process or falls back to a CPU implementation.
 *   - Host arrays are borrowed only for the duration of the call (copied).
 *   - X-shaped host arrays are (M, N) column-major, exactly the reference's
 *     X(M,N) (pqdts.f90:1540); P-shaped arrays are the reference's P(N,D)
 *     column-major, i.e. (D, N) row-major (pqdts.f90:1528).
 *   - Indices are 0-based; maxr = -1 marks the full-space representation.
 *   - A context owns its device memory and one CUDA stream; calls on one
 *     context must not overlap (single-threaded per context).
 */
#ifndef PQDTS_CUDA_H
#define PQDTS_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pqdts_ctx pqdts_ctx;

enum {
  PQDTS_OK = 0,
  PQDTS_E_ARG = -1,     /* invalid argument (sizes, indices, null pointer) */
  PQDTS_E_CUDA = -2,    /* CUDA runtime error (message has the details) */
  PQDTS_E_STATE = -3,   /* call out of order (e.g. no problem set) */
  PQDTS_E_IO = -4,      /* file could not be read or written */
  PQDTS_E_NOMEM = -5    /* device allocation failed */
};

enum { PQDTS_FP64 = 0, PQDTS_MIXED = 1 };

/* Context on CUDA device `device`.  Replaces the process-level set-up of
 * program pqdts (pqdts.f90:1222-1293). */
int pqdts_cuda_create(int32_t device, pqdts_ctx** ctx);
int pqdts_cuda_destroy(pqdts_ctx* ctx);
/* Copies the last error message (NUL-terminated, truncated to len). */
int pqdts_cuda_last_error(pqdts_ctx* ctx, char* buf, int64_t len);
/* Number of CUDA kernels this context has launched so far. */
int pqdts_cuda_kernel_launches(pqdts_ctx* ctx, int64_t* count);
/* Options of a context.  No counterpart in the reference (launch tuning of
 * this implementation; results of the FP64 path do not depend on them).
 *   "graphs"   1 (default): each chunk of CG iterations is replayed as one
 *              captured CUDA graph; 0: the same kernels launched one by one.
 *   "autotune" 1 (default): the banded products' launch schedule is timed on
 *              the problem at set-up (once per size bucket per process);
 *              0: heuristic shapes.  Takes effect at the next set_problem.
 *   "tensor_cores" -1 (default, auto) / 1: the mixed CG's Hessian products
 *              run on the tensor cores (tcgen05, split-BF16x3, FP32
 *              accumulation) on compute capability 10.x devices; 0: FP32
 *              CUDA-core tiles.  Takes effect at the next set_problem.
 *   "rows_kernels" -1 (default, autotuned) / 0 / 1: the FP64 banded products
 *              in their row-flattened form (every lane busy when N is not a
 *              multiple of 32; the same bits) where it applies.
 *   "timers"   1 (default): GPU time per reference timer region
 *              (pqdts_cuda_timer); 0: no events recorded.
 *   "tc_persistent" -1 (default, autotuned) / 0 / 1: the tensor-core kernel
 *              form (one CTA per output tile, or persistent with
 *              double-buffered accumulators); "tc_splits1" -1 (autotuned) or
 *              1..8: K segments of the tensor-core F.V product.
 *   "row_masks" 1 (default) / 0: the FP64 banded products visit, for
 *              each column of their operand, only its non-zero rows (the
 *              iterate, the CG direction and the residual are mostly exact
 *              zeros), and the mixed path's double-FP32 step check only the
 *              rows where a warp's 32 columns hold a non-zero; the FP64
 *              results are the same bits either way (a skipped term adds
 *              +-0 to a sum that is never -0); off when F holds a value
 *              that is not finite.
 *   "count_fmas" 0 (default) / 1: the zero-skipping FP64 products count
 *              the FMAs they execute (per output lane, including the zero
 *              fill of F's 32-row tiles), read back as "fmas.forward" and
 *              "fmas.transposed" (cumulative).
 *   "tc_screen" -1 (default) / 0: the mixed line search's probe products
 *              F.dX (its screen of step lengths, before the chosen step's
 *              double-FP32 check) as one tensor-core product over all
 *              probes' columns wherever the CG's products run on the tensor
 *              cores; 0: FP32 CUDA-core tiles.
 *   "df_products" -1 (default, auto) / 1: the mixed path's gradient F^T.R
 *              and its objective checks (residual F.X - P) in double-FP32
 *              (pairs of FP32 numbers, ~sqrt(K) * 2^-48 relative to the
 *              sum of the K terms' magnitudes) on the CUDA cores; 0: native
 *              FP64.  Takes
 *              effect at the next set_problem.  "df_rows" 0 (default,
 *              chosen by size) / 2 / 4 / 8: band rows per block of those
 *              products (each thread accumulates that many outputs).
 *   "internal_f" -1 (default) / 0 / 1: where the internal F of
 *              pqdts_cuda_set_problem_coo (nnzF < 0) is computed: -1 on the
 *              device for PQDTS_MIXED problems and on the host for PQDTS_FP64
 *              (the host's libm lgamma / exp / log, as the reference's, keep
 *              the FP64 drop-in bitwise); 0 host; 1 device (CUDA's lgamma /
 *              exp / log: values within ~1e-12 relative of the host's).
 *   "fp64_refine" 0 (default) / 1: when a mixed-precision solve runs its CG
 *              in FP64 (the final refinement, counted in stats[6]): 0 from
 *              the first stage-2 iteration whose FP32 Newton step gives no
 *              decrease; 1 for every stage-2 iteration.
 *   "tc_wait_ms" 2000 (default) / 1..60000: limit of each barrier wait in
 *              the tensor-core kernels; a wait that runs out makes the call
 *              fail with PQDTS_E_CUDA ("a barrier wait timed out"), the
 *              kernel having stored nothing and freed its tensor memory, and
 *              the context stays usable.
 *   "tc_wait_probe" 0 (default) / 1: test hook of that error path -- the
 *              kernels' copy producer first waits on a barrier that nothing
 *              arrives on, so the wait runs out before any copy or MMA.
 * Unknown names return PQDTS_E_ARG. */
int pqdts_cuda_set_option(pqdts_ctx* ctx, const char* name, int64_t value);
/* Reads an option above or a field of the schedule in use:
 * "sched.fwd_tile", "sched.trn_tile" (0 = 64x64, 1 = 64x32, 2 = 32x32 FP32
 * tiles of F.V and F^T.R), "sched.trn_splits" (K segments of F^T.R),
 * "sched.trans_threads", "sched.trans_cols" (FP64 F^T product block shape),
 * "sched.tuned" (1 = timed, 0 = heuristic), "sched.tc" (1 = tensor-core
 * Hessian products in use), "sched.tc_bn" (their N tile width),
 * "sched.fwd_rows", "sched.trans_rows" (row-flattened FP64 products in use),
 * "sched.tc_splits" (K segments of their F^T product), "sched.tc_splits1"
 * (of their F.V product), "sched.tc_persistent" (kernel form),
 * "sched.df_fwd", "sched.df_trans" (double-FP32 residual / gradient
 * products in use), "sched.tc_screen" (line-search probe products on the
 * tensor cores), "graphs.captured" (graphs held). */
int pqdts_cuda_get_option(pqdts_ctx* ctx, const char* name, int64_t* value);
/* verbose = 1 prints the reference's stdout lines (iter, newton-pcg, line
 * search, positivity constraints) exactly as rank 0 of pqdts_omp.x. */
int pqdts_cuda_set_verbose(pqdts_ctx* ctx, int32_t verbose);

/* Problem from the reference's per-row dense bands of F (Flocalrow0/1 +
 * Frows, pqdts.f90:77-83, 1357-1363): row d covers columns
 * band_lo[d]..band_hi[d] (band_lo[d] = -1: empty row) and its values are
 * consecutive in band_vals.  P_ND is (D, N) row-major.  precision:
 * PQDTS_FP64 or PQDTS_MIXED (FP32 / tensor-core Hessian products and CG
 * vectors; gradient and objective products in double-FP32, option
 * "df_products"; FP64 line-search decisions and projections). */
int pqdts_cuda_set_problem(pqdts_ctx* ctx, int64_t M, int64_t N, int64_t D, const int64_t* band_lo,
                           const int64_t* band_hi, const double* band_vals, const double* P_ND, double gamma,
                           int32_t precision);

/* Problem from the reference's input files' COO triplets
 * (read_sparse_from_python, pqdts.f90:1080-1107; band build 1318-1365; P
 * assembly 1527-1538).  nnzF < 0: F computed internally (1366-1466, needs
 * M == (D-1)^2).  nnzP < 0: random P from the documented seeded stream.
 * Duplicate entries overwrite in input order, as in the reference. */
int pqdts_cuda_set_problem_coo(pqdts_ctx* ctx, int64_t M, int64_t N, int64_t D, int64_t nnzF, const int32_t* F_row,
                               const int32_t* F_col, const double* F_val, int64_t nnzP, const int32_t* P_row,
                               const int32_t* P_col, const double* P_val, double gamma, int32_t precision);

/* Problem data inspection: band of F as built (band_lo/hi may be null). */
int pqdts_cuda_get_bands(pqdts_ctx* ctx, int64_t* band_lo, int64_t* band_hi, int64_t* nnz);

/* Current iterate X (M,N) column-major (pqdts.f90:1834-1838, 1874). */
int pqdts_cuda_set_x(pqdts_ctx* ctx, const double* X_colmajor);
int pqdts_cuda_get_x(pqdts_ctx* ctx, double* X_colmajor);
/* X = 1/N on the device, the reference's starting point (pqdts.f90:1834-1838). */
int pqdts_cuda_init_x(pqdts_ctx* ctx);

/* The context's CUDA stream (cudaStream_t) for event timing by the caller. */
int pqdts_cuda_get_stream(pqdts_ctx* ctx, void** stream);
/* Bytes this context has copied host->device and device->host so far. */
int pqdts_cuda_transfer_bytes(pqdts_ctx* ctx, int64_t* h2d, int64_t* d2h);

/* Space of the per-operation entry points below: fullspace = 1 is the
 * reference's tfullspace = .true.; otherwise maxr (M entries, 0-based) is
 * the max column of each row (pqdts.f90:97, 1970-1983). */
int pqdts_cuda_set_space(pqdts_ctx* ctx, int32_t fullspace, const int32_t* maxr);
int pqdts_cuda_get_maxr(pqdts_ctx* ctx, int32_t* maxr);

/* Per-operation entry points on the context's X (parity and benchmarking).
 * Like the reference, L, dL and conv_test rebuild X's max column first in
 * the reduced space, and conv_test switches to the full space.  On a
 * PQDTS_MIXED problem L, dL and conv_test use the mixed solver's products
 * (double-FP32 unless "df_products" is 0); redO, BF and Bdiag are FP64. */
int pqdts_cuda_L(pqdts_ctx* ctx, double* val);                     /* L, pqdts.f90:917-973 */
int pqdts_cuda_dL(pqdts_ctx* ctx, double* G_colmajor);             /* dL, pqdts.f90:975-1032 */
int pqdts_cuda_redO(pqdts_ctx* ctx, double* O_ND);                 /* redO local part, 707-736 */
int pqdts_cuda_BF(pqdts_ctx* ctx, const double* V_colmajor, double* HV_colmajor); /* BF, 246-342 (FP64) */
int pqdts_cuda_Bdiag(pqdts_ctx* ctx, double* BD_colmajor);         /* Bdiag, 208-244 */
/* pdot (589-614): sum(A*B) over the problem's M x N arrays.  FP64 problems
 * add in the reference's order (one chain per column over the rows, the
 * columns' results then added in ascending order), bit for bit. */
int pqdts_cuda_pdot(pqdts_ctx* ctx, const double* A_colmajor, const double* B_colmajor, double* out);
/* BF in the mixed-precision solver's arithmetic (FP32 values and
 * accumulation; PQDTS_MIXED problems only): the CG's Hessian product. */
int pqdts_cuda_BF32(pqdts_ctx* ctx, const double* V_colmajor, double* HV_colmajor);
int pqdts_cuda_doproj(pqdts_ctx* ctx);                              /* doproj, 1120-1140 */
int pqdts_cuda_doproj2(pqdts_ctx* ctx, double* xmin);              /* doproj2, 1142-1164 */
int pqdts_cuda_conv_test(pqdts_ctx* ctx, double* conv);            /* conv_test, 1034-1067 */

/* Euclidean projection of `rows` consecutive vectors of length len onto the
 * unit simplex (host buffers, y and x may alias).  rows = 1 is the drop-in
 * for simplexproj_condat_(y, x, &len) (condat_simplexproj.c:60, called at
 * pqdts.f90:1133). */
int pqdts_cuda_simplexproj(pqdts_ctx* ctx, const double* y, double* x, int64_t len, int64_t rows);

/* The reference's own symbol, with its exact signature (condat_simplexproj.c:60;
 * pqdts.f90:1133 calls it as simplexproj_Condat(x3, x2, n2) through an
 * implicit interface, which gfortran resolves to this name): x[0..len-1]
 * receives the projection of y onto the unit simplex, bitwise equal to the
 * reference's.  No context argument and no return value: each host thread
 * gets its own stream and device buffers on the current device (threads may
 * call it concurrently on private buffers, as the reference's OpenMP loop
 * does); x == y is allowed; on a CUDA failure a message goes to stderr and x
 * is filled with NaN.  Linking pqdts.f90 against libpqdts_cuda.so instead of
 * condat_simplexproj.c needs no source change. */
void simplexproj_condat_(double* y, double* x, int* plength);

/* The same projection for callers that cannot allocate device memory, e.g.
 * a host that owns all device memory through its own pool and forbids other
 * allocations after start-up.  No counterpart in the reference.  Needs no
 * context and allocates nothing: d_y and d_x (rows*len doubles each, may
 * alias) are the caller's device buffers, the kernel's scratch is a fixed
 * static device array of PQDTS_NOALLOC_SCRATCH doubles (8 MiB) that every
 * GPU loading this library holds until the process exits.  rows*len above
 * that capacity is rejected with PQDTS_E_ARG and a message on stderr.
 * Runs asynchronously on `stream` (a cudaStream_t; NULL = legacy default
 * stream) of the current device.  The first call on a device looks up the
 * scratch address on that device, and so does the first call after that
 * device's current CUDA context has changed (a cudaDeviceReset, or a
 * caller's own driver-API context); make that first call before any stream
 * capture.  All calls share the one scratch array (its contents are fully
 * rewritten before use, nothing needs clearing), so calls whose kernels can
 * overlap on the GPU -- different streams, different host threads -- race
 * and must be serialised by the caller. */
enum { PQDTS_NOALLOC_SCRATCH = 1 << 20 };
int pqdts_cuda_simplexproj_noalloc(const double* d_y, double* d_x, int64_t len, int64_t rows, void* stream);

/* Smoothing of a restart state (pqdts.f90:1877-1902, used when smo_fact > 0
 * with a starting point read from file): each row j > 100 (1-based) of X
 * (M, N column-major, host memory, in place) becomes the mean of rows
 * max(1, j-d)..min(M, j+d), d = nint(j / smo_fact), summed in ascending
 * order, then is divided by its sum; rows 1..100 are kept.  Needs no device
 * or context. */
int pqdts_cuda_smooth(int64_t M, int64_t N, double smo_fact, double* X_colmajor);

/* Solve statistics filled by the solve entry points (may be null):
 * [0] final L  [1] final conv  [2] ||der||  [3] outer iterations
 * [4] CG iterations  [5] line-search L evaluations  [6] FP64 refinement
 * iterations (mixed precision)  [7] solve seconds (the reference's `min`
 * timer, pqdts.f90:1922-2168). */
enum { PQDTS_NSTATS = 8 };

/* One stage `oiter` (1 = full space, 2 = reduced space) of mode 1
 * (projected gradient, 1934-1951) or mode 2 (two-metric projected truncated
 * Newton, 1953-2110) up to maxiiter iterations or conv < conv_thres, then the
 * stage-end conv_test (2139; output >= 3 prints its lambda lines). */
int pqdts_cuda_run_stage(pqdts_ctx* ctx, int32_t mode, int32_t oiter, int32_t maxiiter, double conv_thres,
                         int32_t output, double* stats);

/* The minimisation of program pqdts from the first objective (1908-1915)
 * through stages start_stage..2 (1927-2167).  stage_cb, when not null, runs
 * after each stage with the current X (M,N column-major) so the host can
 * write the stage files (2139-2166). */
typedef void (*pqdts_stage_cb)(void* user, int32_t oiter, const double* X_colmajor);
int pqdts_cuda_solve(pqdts_ctx* ctx, int32_t mode, int32_t maxiiter, double conv_thres, int32_t start_stage,
                     int32_t output, pqdts_stage_cb stage_cb, void* user, double* stats);

/* Optional extra stopping rule (not in the reference, off by default): end
 * the solve as soon as an outer iteration's objective L <= target (target
 * <= 0 disables it).  Used to time a solver to a given objective. */
int pqdts_cuda_set_objective_target(pqdts_ctx* ctx, double target);

/* Accumulated GPU time (CUDA events) of a named region of the reference's
 * timers ("L", "dL", "BF", "CG", "Lalpha_min", "doproj", "doproj2", "min"). */
int pqdts_cuda_timer(pqdts_ctx* ctx, const char* name, double* seconds, int64_t* count);

/* Batched solve of n_inst independent instances on one device (a gamma sweep
 * or resampled P matrices, no counterpart in the single-instance reference:
 * it replaces n_inst separate pqdts_omp.x runs).  Instance k uses
 * M[k], N[k], D[k], the bands band_lo/hi/vals + offsets, P + offset, gamma[k];
 * X holds sum_k M[k]*N[k] doubles (column-major per instance, in order),
 * starting points on entry and results on exit.  target_L (may be null):
 * per-instance objective targets as pqdts_cuda_set_objective_target.
 * stats: PQDTS_NSTATS per instance.  Host workers (the host's hardware
 * threads up to 16, or the environment variable PQDTS_BATCH_WORKERS; at
 * most one per task) each own a context and stream and take tasks in
 * order, so tasks overlap on the device; each context's CG chunks replay as
 * CUDA graphs and instances of one size bucket share one autotuned launch
 * schedule.  A task is one instance, or, when the environment variable
 * PQDTS_BATCH_GROUPS=1 turns the grouping on (PQDTS_MIXED, mode 2,
 * N <= 4096), a group of up to 4 instances with the same M, N, D and
 * identical F (bands and values: resampled P, gamma sweeps), solved in
 * lockstep: each member keeps its own line search and stages, and their
 * FP32 CG runs jointly -- every CG launch serves all members, the
 * tensor-core products taking the members' vectors as the columns of one
 * wider product.  Off by default: independent solves were faster on the
 * 64-instance batch (5.0 s against 6.4 s). */
int pqdts_cuda_solve_batch(int32_t device, int32_t n_inst, const int64_t* M, const int64_t* N, const int64_t* D,
                           const int64_t* band_lo, const int64_t* band_hi, const double* band_vals,
                           const int64_t* band_row_offset, const int64_t* band_val_offset, const double* P,
                           const int64_t* P_offset, const double* gamma, int32_t precision, int32_t mode,
                           int32_t maxiiter, double conv_thres, const double* target_L, double* X, double* stats);

/* The grouping pqdts_cuda_solve_batch uses for a mixed-precision mode-2
 * batch when PQDTS_BATCH_GROUPS=1 (same arguments as there): group_of[k] =
 * the group of instance k
 * (instances solved in lockstep with a joint CG) or -1 (solved alone).  Host
 * only, needs no device.  No counterpart in the reference. */
int pqdts_cuda_batch_groups(int32_t n_inst, const int64_t* M, const int64_t* N, const int64_t* D,
                            const int64_t* band_lo, const int64_t* band_hi, const double* band_vals,
                            const int64_t* band_row_offset, const int64_t* band_val_offset, int32_t* group_of);

#ifdef __cplusplus
}
#endif

#endif /* PQDTS_CUDA_H */
