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
 * C++ adapter include/fhg_reference_adapter.hpp maps a nonzero status to that call.
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
#define FHG_ERR_TOO_LARGE (-8)        /* a size beyond what the library supports */
#define FHG_ERR_UNSUPPORTED (-9)

/* Smoother codes, as SmootherFactory::Create (src/Solver/Multigrid/SmootherFactory.h:37-100). */
#define FHG_SMOOTHER_BGS 0    /* "bgs": block Gauss-Seidel, forward (colour order) */
#define FHG_SMOOTHER_RBGS 1   /* "rbgs": block Gauss-Seidel, backward (reverse colour order) */
#define FHG_SMOOTHER_BJ 2     /* "bj": block Jacobi, relaxation omega */
#define FHG_SMOOTHER_BJ23 3   /* "bj23": block Jacobi, omega = 2/3 */
#define FHG_SMOOTHER_SBGS 4   /* "sbgs": symmetric block Gauss-Seidel (forward then backward) */
#define FHG_SMOOTHER_ABGS 5   /* "abgs": alternating block Gauss-Seidel, forward first */
#define FHG_SMOOTHER_RABGS 6  /* "rabgs": alternating block Gauss-Seidel, backward first */
/* Block SOR: SmootherFactory builds BlockSOR (src/Solver/FixedPoint/BlockSOR.h:99-227) for the GS codes
 * and their aliases "bsor", "rbsor", "sbsor", "absor", "rabsor" whenever the relaxation parameter is
 * not 1; here the GS codes do the same with fhg_options.omega. The hybrid codes "hbgs" / "hrbgs"
 * (chunk-parallel sweeps whose result depends on the host thread schedule, BlockGaussSeidel.h:124-185)
 * map to FHG_SMOOTHER_BGS / FHG_SMOOTHER_RBGS, this library's parallel (multicolour) sweeps. */

/* Krylov codes: "fcg" = FlexibleConjugateGradient(1) (src/Solver/Krylov/FlexibleConjugateGradient.h:21-25),
 * "cg" = ConjugateGradient (src/Solver/Krylov/ConjugateGradient.h:6-104). */
#define FHG_KRYLOV_FCG 0
#define FHG_KRYLOV_CG 1

/* V-cycle precision: FP64 everywhere, or FP32 smoothers/transfers/operators inside the
 * FP64 Krylov iteration with an FP64 coarsest solve. */
#define FHG_CYCLE_K (-1)   /* fhg_options.w_loops / fhg_set_cycle: the K-cycle */

#define FHG_PREC_FP64 0
#define FHG_PREC_FP32 1
/* FP64-class V-cycle on the FP32 pipe: operators, inverted diagonal blocks and vectors as FP32
 * pairs hi + lo (about 48 significant bits, a few units of 2^-47 per multiply-add), the outer FCG
 * iteration in the same pair arithmetic with FP64 x and Krylov scalars, the reference's loop
 * otherwise unchanged. GB300's FP64 pipe runs at 1/56 of its FP32 rate; with the pair values in
 * the 8 bytes a double takes, the block products stay bound by HBM instead of the FP64 pipe. */
#define FHG_PREC_DF 2

/* Learned correction step of the FP32 V-cycle (no counterpart in the reference): off, on with
 * the fallback rule of fhg_set_learned, or on for every iteration. */
#define FHG_LEARNED_OFF 0
#define FHG_LEARNED_FALLBACK 1
#define FHG_LEARNED_ALWAYS 2
#define FHG_LEARNED_MMA_SYNC 16  /* or-ed into the mode: run the step with mma.sync tiles instead of
                                    tcgen05 tensor-memory accumulators (the two give the same result
                                    up to FP32 summation order) */
#define FHG_LEARNED_PARAMS 24848  /* FP32 parameters: W1 128x48, b1 128, W2 128x128, b2 128, W3 16x128, b3 16 */

/* fhg_options.gs_layout */
#define FHG_GS_AUTO 0
#define FHG_GS_ROW 1
#define FHG_GS_SLOT 2

typedef struct fhg_ctx fhg_ctx;

typedef struct {
    int krylov;                 /* FHG_KRYLOV_* */
    int pre_smoother;           /* FHG_SMOOTHER_* (reference default "bgs", ProgramArguments.h:67) */
    int post_smoother;          /* FHG_SMOOTHER_* (reference default "rbgs", ProgramArguments.h:68) */
    int pre_iterations;         /* Multigrid::PreSmoothingIterations */
    int post_iterations;        /* Multigrid::PostSmoothingIterations */
    double omega;               /* Multigrid::RelaxationParameter: "bj"'s relaxation and, when not 1, block SOR
                                   in place of every Gauss-Seidel code (SmootherFactory.h:37-100) */
    double tolerance;           /* IterativeSolver::Tolerance on ||r||/||b|| */
    int max_iterations;         /* IterativeSolver::MaxIterations */
    int vcycle_precision;       /* FHG_PREC_* */
    int colouring;              /* 1: greedy multicolour ordering (GPU-parallel GS); 0: keep the given order
                                   as colours of one block row each (sequential order, for small checks) */
    int use_graphs;             /* 1: capture one Krylov iteration in a CUDA graph */
    int autotune;               /* 1: pick the launch shape of every operator by timing at setup (lanes per block row,
                                   blocks per lane step, row- or slot-major padded views); with gs_layout auto the
                                   shapes are kept per operator structure in the process, so operators of the same
                                   sizes (problems of one mesh size and degree) are timed once */
    int max_coarse_rows;        /* dense coarsest solve limit (0: default 8192) */
    int outer_split;            /* FP32 V-cycle only: 1 = the outer FCG operator product in double-FP32
                                   arithmetic (FP32 pairs, ~2^-47 relative per term, on the FP32 pipe);
                                   0 = native FP64. GB300's FP64 pipe is 56x slower than FP32. */
    int w_loops;                /* Multigrid::WLoops: 1 = V-cycle, 2 = W-cycle ("-cycle W,..", main.cpp:1179-1215);
                                   FHG_CYCLE_K = K-cycle ("-cycle K,..", Multigrid.h:523-537,611-656: two FCG steps
                                   on every coarse level but the coarsest, the second only when the first reduced
                                   the residual by less than 0.25; decided on the host, so solves do not replay
                                   CUDA graphs) */
    int galerkin;               /* Multigrid::UseGalerkinOperator ("-g 1", main.cpp:1307): coarse operators
                                   A_{l+1} = P_l^T A_l P_l formed at setup (Level.h:133-137); operators given
                                   for levels >= 1 are then not needed and are replaced */
    int coarse_pre_iterations;  /* smoothing steps before the coarse correction on levels >= 1; -1 (the
                                   default): pre_iterations, as the reference (one count for every level).
                                   No counterpart in the reference. */
    int coarse_post_iterations; /* the same after it; -1: post_iterations */
    int gs_layout;              /* FP32 GS sweeps: FHG_GS_AUTO (the autotuner picks row- or slot-major padded
                                   rows; row-major without autotuning), FHG_GS_ROW, FHG_GS_SLOT. Same
                                   arithmetic, different storage order and launch shape; FHG_GS_SLOT also
                                   makes the products with A use the slot-major view of all of A, and
                                   the transfers of levels 0 and 1 their jagged views (rows sorted by
                                   block count, one thread per row); the autotuner compares those too. */
    int extra_precisions;       /* bit mask (1 << FHG_PREC_FP32, 1 << FHG_PREC_DF) of V-cycle precisions whose
                                   operator copies setup also builds, besides vcycle_precision's, so that
                                   fhg_set_vcycle_precision can switch to them (FP64 copies are always built) */
    int replace_residual;       /* 1: residual replacement in every precision: when the recursive residual meets the
                                   tolerance but the true one does not, r = b - A x and FCG continues (at most 8
                                   times); 0 (default): only with the FP32 V-cycle, the FP64 modes keep the
                                   reference's loop (IterativeSolver.h:224-247). The true residual that misses the
                                   tolerance in FP64 is evaluated again in compensated arithmetic. No counterpart
                                   in the reference. */
    int fused_coarse;           /* 1 (default): with GS / SOR smoothers and a V or W cycle in FP32 or DF, the cycle
                                   below some level (>= 1) runs as one thread-block-cluster launch (8 or 16 CTAs,
                                   phases separated by the cluster barrier) instead of one launch per colour and
                                   product. With autotune, setup (and fhg_set_cycle / fhg_set_coarse_smoothing)
                                   times one cycle below level 0 launch by launch and fused from every eligible
                                   level (every level below it at most 65,536 block rows and 24 colours, at most
                                   6 levels) and keeps the fastest, per precision and hierarchy structure;
                                   without, it fuses from the first level of at most 8,192 block rows with 8
                                   CTAs of 512 threads. Timing also tries CTAs of 1024 threads (twice the warps
                                   per SM, one row in flight per lane group). 2: as 1, but without autotuning
                                   the CTAs have 1024 threads. 0: launch by launch. Same arithmetic up to the
                                   summation order of a row. */
} fhg_options;

typedef struct {
    int iterations;             /* IterativeSolver::IterationCount */
    int status;                 /* FHG_OK or FHG_ERR_* */
    double normalized_residual; /* last ||r||/||b|| (recursive residual, IterationResult.h:121-139) */
    double solve_ms;            /* device time of the solve (CUDA events on the context stream) */
    int learned_iterations;     /* iterations whose V-cycle applied the learned correction */
    double true_relative_residual; /* FP64 ||b - A x|| / ||b|| of the returned x (-1 if the solve failed) */
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
 * (src/Solver/Multigrid/Level.h:56-131). Copies the arrays. block_size is the level's own
 * (BlockSizeForBlockSmoothers): it may drop from one level to the next only where P_l is the
 * natural injection between face degrees of the p-multigrid (P_LevelForHHO::SetupProlongation,
 * src/Solver/Multigrid/MultigridForHHO/P_MultigridForHHO.h:69-92: the same faces, a 1 at
 * (f * bs_l + i, f * bs_{l+1} + i) for i < bs_{l+1}); fhg_setup refuses any other change with
 * FHG_ERR_UNSUPPORTED. */
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
#define FHG_OP_VCYCLE_LEARNED 10 /* same with the learned correction (FP32; fhg_apply_internal, fhg_time_op) */
#define FHG_OP_LEARNED_STEP 11 /* out = in + learned correction of the residual aux - A in (FP32, level 0;
                                  fhg_apply_internal, fhg_time_op) */
int fhg_apply(fhg_ctx* ctx, int level, int op, const double* in, const double* aux, double* out);

/* Device timing of one operator (same ops; vectors left in device memory) in FHG_PREC_FP64,
 * FHG_PREC_FP32 or FHG_PREC_DF (the V-cycle copies): average ms per application over `reps` back-to-back
 * applications after `warmup`, CUDA events on the context stream. A block-GS sweep is all of
 * its colour launches. */
int fhg_time_op(fhg_ctx* ctx, int level, int op, int precision, int warmup, int reps, double* avg_ms);

/* Change the cycle of a set-up context: smoothers (FHG_SMOOTHER_*), smoothing steps and WLoops,
 * the Multigrid fields PreSmootherCode/PostSmootherCode/Pre-/PostSmoothingIterations/WLoops
 * (src/Solver/Multigrid/Multigrid.h:19-26), without rebuilding the hierarchy. */
int fhg_set_cycle(fhg_ctx* ctx, int pre_smoother, int post_smoother, int pre_iterations, int post_iterations,
                  int w_loops);

/* Smoothing steps on levels >= 1 (-1: those of level 0, the reference's behaviour); cycles already
 * captured in graphs are rebuilt. No counterpart in the reference. */
int fhg_set_coarse_smoothing(fhg_ctx* ctx, int pre_iterations, int post_iterations);

/* Switch the V-cycle precision of a set-up context (FP32 and DF need their copies: a setup in that
 * precision or with its bit in extra_precisions). The outer Krylov iteration keeps FP64 x and
 * scalars. */
int fhg_set_vcycle_precision(fhg_ctx* ctx, int precision);

/* Sizes of level `level` after setup: block rows, stored blocks of A, colours, lanes per block row
 * of the A operator, stored blocks of P (0 on the coarsest). */
int fhg_level_info(const fhg_ctx* ctx, int level, int* n_block_rows, long long* n_blocks,
                   int* n_colours, int* lanes, long long* p_blocks);

/* The coarse sub-cycle of V-cycle precision `precision` (FHG_PREC_FP32 or FHG_PREC_DF) as the context
 * runs it now: the first level of the one-launch sub-cycle (-1: launch by launch), the CTAs of its
 * cluster and the threads of each CTA. Any pointer may be NULL. No counterpart in the reference. */
int fhg_fused_coarse_info(const fhg_ctx* ctx, int precision, int* first_level, int* cluster_ctas,
                          int* cta_threads);

/* The colour permutation of `level` after setup: perm[new_block_row] = given_block_row. */
int fhg_get_permutation(const fhg_ctx* ctx, int level, int* perm);

/* Device memory the context holds after setup, in bytes (its own allocations). No counterpart in the
 * reference. */
long long fhg_device_bytes(const fhg_ctx* ctx);

/* Number of kernels this library has launched in this process (graph replays included). */
long long fhg_kernel_launches(const fhg_ctx* ctx);

/* Residual 2-norm ||b - A x|| of a face-block system, computed without allocating any memory.
 * No counterpart in the reference: it exists for callers that may not allocate device memory
 * when they check a solution - a process that reserved all of the GPU's memory for its own pool
 * or budget at start-up, an embedder that must not let a library grow its footprint, or a
 * latency-bound loop that cannot afford cudaMalloc's device-wide synchronisation. The caller
 * passes, in device memory it owns: the operator in libfhg's block layout (rowptr[n_block_rows+1],
 * block colidx, values entry-major: entry r*bs+c of block p at vals[(r*bs+c)*ld + p], ld >= number
 * of blocks), x, b (n_block_rows*block_size doubles each) and norm_out (one double, written on
 * `stream`; NULL = the default stream). `lanes` (4, 8, 16, 32) is the number of lanes per block row.
 * The per-block partial sums live in a fixed array inside the library, FHG_NOALLOC_MAX_PARTIALS
 * doubles (1 MiB) on every GPU that loads it, held until the process exits; one partial sum per
 * 256/lanes block rows, so n_block_rows may be at most FHG_NOALLOC_MAX_PARTIALS*256/lanes
 * (4,194,304 block rows at 8 lanes): larger sizes return FHG_ERR_TOO_LARGE and launch nothing.
 * The first call on a device (and the first after that device's context was replaced, e.g. by
 * cudaDeviceReset) looks up the array's device address in the current context (cudaGetSymbolAddress);
 * later calls reuse it. Calls share the array and leave their partial sums in it: two calls that
 * overlap on the GPU race on it. A CUDA error left pending by earlier work is returned as
 * FHG_ERR_CUDA before anything is launched and is not cleared. Makes the device current for the
 * call and restores the caller's current device. */
#define FHG_NOALLOC_MAX_PARTIALS 131072
int fhg_residual_norm_noalloc(int device, int n_block_rows, int block_size, int lanes,
                              const int* rowptr, const int* colidx, const double* vals, long long ld,
                              const double* x, const double* b, double* norm_out, void* stream);

/* ---- Learned correction step (no counterpart in the reference) --------------------------------
 * A per-face-patch network adds a correction at the end of the finest level's post-smoothing in
 * the FP32 V-cycle: x_i += s_i N(u_i), where u_i holds the block-Jacobi-scaled residual
 * D^-1 (b - A x) of face i and of its six most strongly coupled neighbours (divided by their RMS
 * s_i) and the diffusion tensors of the face's two elements; N is a 48-128-128-16 GELU MLP run
 * on BF16 tensor cores with FP32 accumulation. The Krylov method must be FCG (it absorbs the
 * variable preconditioner). */

/* Diffusion tensors of the two elements of every face block of level 0, in the caller's
 * numbering: tensors[12 u .. 12 u + 11] = element 1 then element 2, each (xx, yy, zz, xy, xz, yz)
 * ((xx, yy, xy, 0, 0, 0) in 2D). Call after fhg_set_level(0, ...), before or after setup. Faces
 * without tensors get zero features. */
int fhg_set_face_tensors(fhg_ctx* ctx, int n_blocks, const double* tensors);

/* Install a network (params: FHG_LEARNED_PARAMS floats, host; NULL keeps the installed one) and
 * select the mode. Needs a setup with FHG_PREC_FP32, two levels or more and block size 2..4;
 * call after every fhg_setup. FHG_LEARNED_FALLBACK: from the sixth iteration of a solve on,
 * when the geometric mean rho of the last four residual reductions falls behind the plain
 * method's per-iteration reduction rho_p (rho > rho_p; rho_p measured once per cycle configuration
 * on a seeded random right-hand side, before the first solve's timed region), the remaining
 * iterations use the plain V-cycle. */
int fhg_set_learned(fhg_ctx* ctx, const float* params, int n_params, int mode);

/* The plain method's calibrated per-iteration reduction (over its iterations 2 to 12). */
int fhg_learned_reference_rate(fhg_ctx* ctx, double* rho);

/* Network inputs for a level-0 residual r (FP32, DEVICE, the context's colour numbering):
 * features = n_block_rows x 48 BF16 values (uint16 bits), scale = n_block_rows FP32 (s_i). */
int fhg_learned_features(fhg_ctx* ctx, const float* r, void* features, float* scale);

/* fhg_apply on DEVICE vectors in the context's colour numbering (fhg_get_permutation), in
 * FHG_PREC_FP64 (double), FHG_PREC_FP32 (float, the V-cycle copies; FHG_OP_VCYCLE_LEARNED
 * applies the installed network) or FHG_PREC_DF (interleaved FP32 pairs hi, lo: 8 bytes per value).
 * Returns after the stream has finished. */
int fhg_apply_internal(fhg_ctx* ctx, int level, int op, int precision, const void* in, const void* aux, void* out);

/* Training of the network on the GPU (FP32 master weights, BF16 tensor-core forward and backward,
 * Adam). One step on one field: r = A e (FP32, DEVICE, colour numbering of `ctx`, which must
 * satisfy fhg_set_learned's conditions) for an error e with energy = e.A e > 0. The loss is the
 * relative energy error after the correction, |e - c|_A^2 / |e|_A^2, c the network's correction of
 * every face; *loss receives it before the update, grad (host, nullable) its gradient. update = 0
 * leaves the parameters unchanged. */
typedef struct fhg_net fhg_net;
int fhg_net_num_params(void);
int fhg_net_create(fhg_net** net, int device);
void fhg_net_destroy(fhg_net* net);
const char* fhg_net_last_error(const fhg_net* net);
int fhg_net_set_params(fhg_net* net, const float* params, int n_params);  /* also resets Adam */
int fhg_net_get_params(const fhg_net* net, float* params, int n_params);
int fhg_net_train_step(fhg_net* net, fhg_ctx* ctx, const float* r, double energy, float lr, float weight_decay,
                       int update, double* loss, float* grad);

/* ---- Batched solve (no counterpart in the reference) --------------------------------------------
 * Many independent systems, each a set-up FCG context (plain V-cycle, FP64 or FP32), solved by ONE
 * graph launch: per context a prelude, a WHILE conditional node whose body is one FCG iteration
 * followed by the stopping test evaluated on the device (||r||/||b|| < tolerance, NaN/inf or
 * max_iterations), and an epilogue (FP64 true residual, x out). Each context reads b from and writes
 * x to its own device buffers (fhg_io_buffers, the caller's numbering). The contexts are borrowed;
 * setting one up again makes the next solve rebuild the graph. The launch sequence of every system
 * is that of fhg_solve_device, so iteration counts and results are the same. */
typedef struct fhg_batch fhg_batch;
int fhg_io_buffers(fhg_ctx* ctx, double** b_dev, double** x_dev);
int fhg_io_upload(fhg_ctx* ctx, const double* b);   /* host b -> the context's device b */
int fhg_io_download(fhg_ctx* ctx, double* x);       /* the context's device x -> host x */
int fhg_batch_create(fhg_batch** batch, int device);
void fhg_batch_destroy(fhg_batch* batch);
const char* fhg_batch_last_error(const fhg_batch* batch);
int fhg_batch_add(fhg_batch* batch, fhg_ctx* ctx);
/* infos: one per added context, in order (solve_ms = the whole batch); elapsed_ms: device time of
 * the launch (CUDA events on the batch's stream). */
int fhg_batch_solve(fhg_batch* batch, fhg_solve_info* infos, double* elapsed_ms);

/* ---- Post-processing of a face solution ----------------------------------------------------------
 * Cell-unknown recovery x_T = A_TT^{-1} b_T - A_TT^{-1} A_TF x_F per element
 * (Diffusion_HHO::HybridCoeffsBySolvingCellUnknowns, src/Discretizations/HHO/Diffusion_HHO.h:855-882),
 * the k+1 reconstruction of [x_T; x_F] (ReconstructHigherOrderApproximationFromHybridCoeffs, :896-912)
 * and its relative L2 error against a closed-form solution (Diffusion_HHO::L2Error, :120-150), on the
 * GPU. The element tables are those of the finest level: per element its class, the unknown block of
 * each local face (-1: Dirichlet), its centroid (3 doubles) and A_TT^{-1} b_T (n_cell); per class
 * -A_TT^{-1} A_TF (n_cell x n_face_dofs, row-major), the reconstruction (n_recon x (n_cell +
 * n_face_dofs)), and at n_points cell quadrature points their weights, offsets from the centroid (3
 * doubles each) and reconstruction basis values (n_points x n_recon). A caller whose elements are not
 * grouped in classes passes one class per element. */
#define FHG_EXACT_NONE 0   /* no error evaluation: cell unknowns only */
#define FHG_EXACT_SINE 1   /* u = prod_d sin(pi x_d), the solution of the "sine" test case source */
typedef struct fhg_post fhg_post;
int fhg_post_create(fhg_post** post, int device, int dim, int n_elements, int n_classes, int n_cell,
                    int n_face_dofs, int n_recon, int n_points, const int* elem_class, const int* elem_faces,
                    const double* elem_centre, const double* cell_rhs, const double* solve_cells,
                    const double* recon, const double* weights, const double* offsets, const double* basis);
/* x_faces: device face solution in the given numbering (fhg_solve's x); x_cells: device output
 * (n_elements x n_cell) or null; rel_l2_error: host output with FHG_EXACT_SINE; elapsed_ms: device
 * time (CUDA events) or null. */
int fhg_post_run(fhg_post* post, const double* x_faces, double* x_cells, int exact, double* rel_l2_error,
                 double* elapsed_ms);
const char* fhg_post_last_error(const fhg_post* post);
void fhg_post_destroy(fhg_post* post);

/* ---- Static condensation and assembly of the finest face system -----------------------------------
 * A = A_FF - A_TF^T A_TT^{-1} A_TF and b = -A_TF^T A_TT^{-1} b_T assembled over the interior faces
 * (Diffusion_HHO::Assemble with static condensation, src/Discretizations/HHO/Diffusion_HHO.h:627-638),
 * on the GPU in FP64. Inputs: per class the local operator before condensation ((n_cell +
 * n_face_dofs)^2, row-major, cell unknowns first; one class per element when the elements are not
 * grouped), per element its class, its faces' unknown blocks (-1: Dirichlet) and b_T (n_cell), per
 * unknown face block its two elements with the face's local index in each, (e1, lf1, e2, lf2), in the
 * order their contributions are added. fhg_cond_run condenses and assembles on the device and
 * returns the number of stored entries; fhg_cond_result gives device pointers to the scalar CSR
 * (rows face block * face DOFs + a: rowptr, colidx, vals) and b, valid until the next run or destroy,
 * in the layout fhg_set_level takes. Every row is written by one thread in a fixed order (the result
 * is bitwise reproducible). No counterpart in the reference's API: it replaces the host assembly. */
typedef struct fhg_cond fhg_cond;
int fhg_cond_create(fhg_cond** cond, int device, int dim, int n_elements, int n_classes, int n_cell,
                    int n_face_dofs, int n_face_blocks, const int* elem_class, const int* elem_faces,
                    const int* face_elems, const double* local, const double* b_cell);
int fhg_cond_run(fhg_cond* cond, long long* n_entries, double* elapsed_ms);
int fhg_cond_result(fhg_cond* cond, int** rowptr, int** colidx, double** vals, double** b);
/* The same copied to host arrays (rows + 1, n_entries, n_entries, rows); null ones are skipped. */
int fhg_cond_download(fhg_cond* cond, int* rowptr, int* colidx, double* vals, double* b);
const char* fhg_cond_last_error(const fhg_cond* cond);
void fhg_cond_destroy(fhg_cond* cond);

#ifdef __cplusplus
}
#endif
#endif /* FHG_H */
