/*
 * fhg: GB300 (sm_103a) solve phase of fhhos4 behind a C ABI.
 *
 * One context = one multigrid hierarchy resident on one GPU + its solver state.
 * Host pointers passed in are borrowed for the duration of the call only; the
 * context owns every device allocation. Calls on one context must not overlap
 * (one context per host thread / stream), matching the reference's
 * non-reentrant, main-thread solver API (src/Solver/Solver.h:6-43).
 *
 * Every function returns FHG_OK (0) or a negative FHG_ERR_* code; the message of
 * the last failure is available from fhg_last_error(). The reference reports
 * errors through Utils::FatalError (print + exit, src/Utils/Utils.h:258-264); the
 * C++ adapter shown in INTEGRATION.md maps a nonzero status to that call.
 *
 * Matrices are scalar CSR with 32-bit indices and columns ascending within a
 * row, i.e. exactly the arrays of the reference's row-major Eigen SparseMatrix
 * with SMALL_INDEX (src/Utils/Types.h:11-27): outerIndexPtr / innerIndexPtr /
 * valuePtr after makeCompressed().
 */
#ifndef FHG_H
#define FHG_H

#ifdef __cplusplus
extern "C" {
#endif

#define FHG_OK 0
#define FHG_ERR_INVALID_ARG (-1)
#define FHG_ERR_CUDA (-2)
#define FHG_ERR_NOT_READY (-3)
#define FHG_ERR_SINGULAR_BLOCK (-4)   /* a diagonal block has no inverse (FullPivLU, BlockGaussSeidel.h:55-72) */
#define FHG_ERR_NOT_SPD (-5)          /* coarsest factorisation failed (EigenSparseCholesky.h:27-33) */
#define FHG_ERR_DIVERGED (-6)         /* inf residual: "divergence of the solver" (IterativeSolver.h:237-238) */
#define FHG_ERR_NAN (-7)              /* NaN residual: "the residual is NaN." (IterativeSolver.h:239-240) */
#define FHG_ERR_TOO_LARGE (-8)        /* a size beyond what this build supports */
#define FHG_ERR_UNSUPPORTED (-9)

/* Smoother codes, as SmootherFactory::Create (src/Solver/Multigrid/SmootherFactory.h:37-100). */
#define FHG_SMOOTHER_BGS 0    /* "bgs": block Gauss-Seidel, forward (colour order) */
#define FHG_SMOOTHER_RBGS 1   /* "rbgs": block Gauss-Seidel, backward (reverse colour order) */
#define FHG_SMOOTHER_BJ 2     /* "bj": block Jacobi, relaxation omega */
#define FHG_SMOOTHER_BJ23 3   /* "bj23": block Jacobi, omega = 2/3 */
#define FHG_SMOOTHER_SBGS 4   /* "sbgs": symmetric block Gauss-Seidel (forward then backward) */
#define FHG_SMOOTHER_ABGS 5   /* "abgs": alternating block Gauss-Seidel, forward first */
#define FHG_SMOOTHER_RABGS 6  /* "rabgs": alternating block Gauss-Seidel, backward first */

/* Krylov codes: "fcg" = FlexibleConjugateGradient(1) (src/Solver/Krylov/FlexibleConjugateGradient.h:21-25),
 * "cg" = ConjugateGradient (src/Solver/Krylov/ConjugateGradient.h:6-104). */
#define FHG_KRYLOV_FCG 0
#define FHG_KRYLOV_CG 1

/* V-cycle precision: FP64 everywhere, or FP32 smoothers/transfers/operators inside the
 * FP64 Krylov iteration with an FP64 coarsest solve. */
#define FHG_PREC_FP64 0
#define FHG_PREC_FP32 1

typedef struct fhg_ctx fhg_ctx;

typedef struct {
    int krylov;                 /* FHG_KRYLOV_* */
    int pre_smoother;           /* FHG_SMOOTHER_* (reference default "bgs", ProgramArguments.h:67) */
    int post_smoother;          /* FHG_SMOOTHER_* (reference default "rbgs", ProgramArguments.h:68) */
    int pre_iterations;         /* Multigrid::PreSmoothingIterations */
    int post_iterations;        /* Multigrid::PostSmoothingIterations */
    double omega;               /* Multigrid::RelaxationParameter (used by "bj") */
    double tolerance;           /* IterativeSolver::Tolerance on ||r||/||b|| */
    int max_iterations;         /* IterativeSolver::MaxIterations */
    int vcycle_precision;       /* FHG_PREC_* */
    int colouring;              /* 1: greedy multicolour ordering (GPU-parallel GS); 0: keep the given order
                                   as colours of one block row each (sequential order, for small checks) */
    int use_graphs;             /* 1: capture one Krylov iteration in a CUDA graph */
    int autotune;               /* 1: pick lanes-per-block-row of every operator by timing at setup */
    int max_coarse_rows;        /* dense coarsest solve limit (0: default 8192) */
    int outer_split;            /* FP32 V-cycle only: 1 = the outer FCG operator product in double-FP32
                                   arithmetic (FP32 pairs, ~2^-47 relative per term, on the FP32 pipe);
                                   0 = native FP64. GB300's FP64 pipe is 56x slower than FP32. */
    int w_loops;                /* Multigrid::WLoops: 1 = V-cycle, 2 = W-cycle ("-cycle W,..", main.cpp:1179-1215) */
} fhg_options;

typedef struct {
    int iterations;             /* IterativeSolver::IterationCount */
    int status;                 /* FHG_OK or FHG_ERR_* */
    double normalized_residual; /* last ||r||/||b|| (recursive residual, IterationResult.h:121-139) */
    double solve_ms;            /* device time of the solve (CUDA events on the context stream) */
} fhg_solve_info;

/* Fill *opts with the reference defaults of "-s fcgmg -cycle V,1,1": FCG(1), bgs/rbgs, 1+1
 * smoothing steps, tol 1e-8 (ProgramArguments.h:92), 200 iterations, FP64. */
void fhg_default_options(fhg_options* opts);

/* Create a context on CUDA device `device`. */
int fhg_create(fhg_ctx** ctx, int device);
void fhg_destroy(fhg_ctx* ctx);
const char* fhg_last_error(const fhg_ctx* ctx);

/* Level l operator A_l (n x n, CSR) and, for l < nlevels-1, the prolongation P_l
 * (n_l x n_{l+1}, CSR) that LevelForHHO::SetupProlongation_H builds
 * (src/Solver/Multigrid/MultigridForHHO/LevelForHHO.h:182-213); R_l = P_l^T
 * (LevelForHHO.h:535-543). Replaces Level::Setup's operator/transfer setup
 * (src/Solver/Multigrid/Level.h:56-131). Copies the arrays. */
int fhg_set_level(fhg_ctx* ctx, int level, int block_size, int n,
                  const int* rowptr, const int* colidx, const double* vals);
int fhg_set_prolongation(fhg_ctx* ctx, int level, int n_fine, int n_coarse,
                         const int* rowptr, const int* colidx, const double* vals);

/* Multigrid::Setup + FlexibleConjugateGradient::Setup (src/Solver/Multigrid/Multigrid.h:88-313,
 * FlexibleConjugateGradient.h:32-37): block structure, colouring, pre-inverted diagonal
 * blocks (BlockGaussSeidel.h:55-72), coarsest factorisation (EigenSparseCholesky.h:19-34),
 * upload. nlevels = number of levels given with fhg_set_level. */
int fhg_setup(fhg_ctx* ctx, int nlevels, const fhg_options* opts);

/* IterativeSolver::Solve(b, "0") (src/Solver/IterativeSolver.h:55-73) through
 * FlexibleConjugateGradient::Solve (FlexibleConjugateGradient.h:47-171): b and x are HOST
 * arrays of length n_0; history (may be NULL) receives max_iterations+1 normalised
 * residuals, the values OnIterationEnd would see (IterativeSolver.h:224-227). */
int fhg_solve(fhg_ctx* ctx, const double* b, double* x, double* history, fhg_solve_info* info);

/* Same, with b and x DEVICE pointers on the context's device (inputs already resident). */
int fhg_solve_device(fhg_ctx* ctx, const double* b_dev, double* x_dev, double* history,
                     fhg_solve_info* info);

/* One operator of level `level`, host arrays in the caller's numbering. Ops: */
#define FHG_OP_SPMV 0         /* out = A in                        (Multigrid.h:478 product)        */
#define FHG_OP_RESIDUAL 1     /* out = aux - A in                  (Multigrid.h:478)                */
#define FHG_OP_RESTRICT 2     /* out = R in   (in: level l, out: level l+1)  (Level.h:139-143)     */
#define FHG_OP_PROLONG_ADD 3  /* out = aux + P in (in: level l+1, aux/out: level l) (Level.h:150-154, Multigrid.h:554) */
#define FHG_OP_GS_FORWARD 4   /* out = one forward block-GS sweep from x=in, rhs=aux (BlockGaussSeidel.h:86-90) */
#define FHG_OP_GS_BACKWARD 5  /* out = one backward sweep (BlockGaussSeidel.h:91-95)                */
#define FHG_OP_JACOBI 6       /* out = one block-Jacobi sweep, omega from the options (BlockJacobi.h:77-98) */
#define FHG_OP_SYM_SPMV 7     /* out = A.selfadjointView<Lower>() in (FlexibleConjugateGradient.h:124), level 0 */
#define FHG_OP_COARSE_SOLVE 8 /* out = A_coarsest^{-1} in          (Multigrid.h:445-452)            */
#define FHG_OP_VCYCLE 9       /* out = one V-cycle from zero on rhs in (Preconditioner.h:162-167), level 0 */
int fhg_apply(fhg_ctx* ctx, int level, int op, const double* in, const double* aux, double* out);

/* Device timing of one operator (same ops; vectors left in device memory) in FHG_PREC_FP64 or
 * FHG_PREC_FP32 (the V-cycle copies): average ms per application over `reps` back-to-back
 * applications after `warmup`, CUDA events on the context stream. A block-GS sweep is all of
 * its colour launches. */
int fhg_time_op(fhg_ctx* ctx, int level, int op, int precision, int warmup, int reps, double* avg_ms);

/* Change the cycle of a set-up context: smoothers (FHG_SMOOTHER_*), smoothing steps and WLoops,
 * the Multigrid fields PreSmootherCode/PostSmootherCode/Pre-/PostSmoothingIterations/WLoops
 * (src/Solver/Multigrid/Multigrid.h:19-26), without rebuilding the hierarchy. */
int fhg_set_cycle(fhg_ctx* ctx, int pre_smoother, int post_smoother, int pre_iterations, int post_iterations,
                  int w_loops);

/* Switch the V-cycle precision of a set-up context (FP32 needs a setup with FHG_PREC_FP32,
 * which keeps both copies). The outer Krylov iteration stays FP64. */
int fhg_set_vcycle_precision(fhg_ctx* ctx, int precision);

/* Sizes of level `level` after setup: block rows, stored blocks of A, colours, lanes per block row
 * of the A operator, stored blocks of P (0 on the coarsest). */
int fhg_level_info(const fhg_ctx* ctx, int level, int* n_block_rows, long long* n_blocks,
                   int* n_colours, int* lanes, long long* p_blocks);

/* The colour permutation of `level` after setup: perm[new_block_row] = given_block_row. */
int fhg_get_permutation(const fhg_ctx* ctx, int level, int* perm);

/* Number of kernels this library has launched in this process (graph replays included). */
long long fhg_kernel_launches(const fhg_ctx* ctx);

/* Residual 2-norm ||b - A x|| of a face-block system, computed without allocating any memory.
 * No counterpart in the reference: it exists for callers that cannot call cudaMalloc when they
 * check a solution (while capturing a stream into a CUDA graph, or when every byte of device
 * memory is owned by the caller's own pool or budget). The caller passes, in device memory it
 * owns: the operator in libfhg's block layout (rowptr[n_block_rows+1], block colidx, values
 * entry-major: entry r*bs+c of block p at vals[(r*bs+c)*ld + p], ld >= number of blocks), x, b
 * (n_block_rows*block_size doubles each) and norm_out (one double, written on `stream`; NULL =
 * the default stream). `lanes` (4, 8, 16, 32) is the number of lanes per block row.
 * The per-block partial sums live in a fixed array inside the library, FHG_NOALLOC_MAX_PARTIALS
 * doubles (1 MiB) on every GPU that loads it, held until the process exits; one partial sum per
 * 256/lanes block rows, so n_block_rows may be at most FHG_NOALLOC_MAX_PARTIALS*256/lanes
 * (4,194,304 block rows at 8 lanes): larger sizes return FHG_ERR_TOO_LARGE and launch nothing.
 * The first call on a device looks up the array's device address on that device (make it before
 * any stream capture). Calls share the array: two calls that overlap on the GPU race on it.
 * Makes the device current for the call and restores the caller's current device. */
#define FHG_NOALLOC_MAX_PARTIALS 131072
int fhg_residual_norm_noalloc(int device, int n_block_rows, int block_size, int lanes,
                              const int* rowptr, const int* colidx, const double* vals, long long ld,
                              const double* x, const double* b, double* norm_out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* FHG_H */
