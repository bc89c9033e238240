/*
 * CPU restatement of the fhhos4 solve phase: the checker for the CUDA path.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py load this library. The product path never calls it.
 *
 * Every function names the reference code it restates (paths are relative to
 * the fhhos4 source tree). Matrices are row-major CSR with 32-bit indices, as
 * the reference's SparseMatrix with SMALL_INDEX (src/Utils/Types.h:11-27).
 */
#ifndef FCGMG_ORACLE_H
#define FCGMG_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int n_rows, n_cols;
    const int* rowptr;   /* n_rows + 1 */
    const int* colidx;   /* nnz, ascending within a row */
    const double* vals;  /* nnz */
} orc_csr;

enum { ORC_BGS_FORWARD = 0, ORC_BGS_BACKWARD = 1, ORC_BJ = 2, ORC_BGS_SYMMETRIC = 3,
       ORC_BGS_ALTERNATING_FORWARD_FIRST = 4, ORC_BGS_ALTERNATING_BACKWARD_FIRST = 5 };
enum { ORC_KRYLOV_FCG = 0, ORC_KRYLOV_CG = 1 };

typedef struct {
    int pre_smoother, post_smoother;   /* ORC_BGS_FORWARD / ORC_BGS_BACKWARD / ORC_BJ */
    double omega;                      /* block Jacobi relaxation (bj: 1, bj23: 2/3) */
    int pre_iterations, post_iterations;
    int krylov;                        /* ORC_KRYLOV_FCG (FCG(1)) or ORC_KRYLOV_CG */
    double tolerance;
    int max_iterations;
    int w_loops;                       /* Multigrid::WLoops: 1 V-cycle, 2 W-cycle; ORC_CYCLE_K: K-cycle */
    /* Smoothing steps on levels >= 1; -1: pre_iterations / post_iterations (the reference has one
     * count for every level). An extension of the restatement with no counterpart in the
     * reference, mirroring fhg_options.coarse_pre_iterations / coarse_post_iterations. */
    int coarse_pre_iterations, coarse_post_iterations;
    /* Relaxation parameter of the Gauss-Seidel codes: 1 = block Gauss-Seidel, otherwise block SOR
     * (SmootherFactory.h:37-100 turns bgs/rbgs/sbgs/abgs/rabgs and their bsor aliases into BlockSOR
     * when Multigrid::RelaxationParameter != 1; BlockSOR.h:199-227). */
    double sor_omega;
} orc_options;
#define ORC_CYCLE_K (-1)

/* y = A x, one sequential sum per row in column order (Eigen SparseDenseProduct.h:34-70). */
void orc_spmv(const orc_csr* A, const double* x, double* y);
/* r = b - A x (Multigrid.h:478). */
void orc_residual(const orc_csr* A, const double* b, const double* x, double* r);
/* y = A.selfadjointView<Lower>() x (FlexibleConjugateGradient.h:124; Eigen SparseSelfAdjointView.h:278-330). */
void orc_spmv_sym_lower(const orc_csr* A, const double* x, double* y);
/* Transpose (values and sorted column indices) into caller buffers sized n_cols+1 / nnz. */
void orc_transpose(const orc_csr* A, int* rowptr_t, int* colidx_t, double* vals_t);

/* One block Gauss-Seidel sweep in place (BlockGaussSeidel.h:75-123,193-223); orc_options.sor_omega
 * selects block SOR inside the multigrid cycle. */
void orc_block_gs(const orc_csr* A, int bs, const double* b, double* x, int backward);
/* One block Jacobi sweep in place (BlockJacobi.h:77-127). */
void orc_block_jacobi(const orc_csr* A, int bs, double omega, const double* b, double* x);

/* Greedy colouring of the block graph in block-row order; returns the colour count.
 * colour[i] = smallest colour absent from the already-coloured neighbours of block row i. */
int orc_greedy_colouring(const orc_csr* A, int bs, int* colour);
/* Block permutation grouping block rows by ascending colour, stable within a colour:
 * perm[new_block] = old_block. */
void orc_colour_permutation(int nb, const int* colour, int ncolours, int* perm);

/* FCG(1) or PCG preconditioned by one V-cycle from zero (FlexibleConjugateGradient.h:47-171,
 * ConjugateGradient.h:27-104, Multigrid.h:438-608). A[0..nlevels-1], P[0..nlevels-2]
 * (P[l]: level l rows, level l+1 columns), R = P^T. Writes x, the normalised residual
 * history (max_iterations+1 entries) and the iteration count. Returns 0, or
 * nonzero on a breakdown (NaN/inf residual, singular block). */
int orc_fcgmg_solve(int nlevels, int bs, const orc_csr* A, const orc_csr* P,
                    const double* b, double* x, const orc_options* opt,
                    double* history, int* iterations);
/* The same with a block size per level (bs[l]): the p-multigrid of P_MultigridForHHO, whose levels
 * differ in face degree (src/Solver/Multigrid/MultigridForHHO/P_MultigridForHHO.h), P[l] the natural
 * injection between them. */
int orc_fcgmg_solve_levels(int nlevels, const int* bs, const orc_csr* A, const orc_csr* P,
                           const double* b, double* x, const orc_options* opt,
                           double* history, int* iterations);

/* Wall seconds of the last orc_fcgmg_solve: setup (transposes, diagonal LU, coarse LDL^T)
 * and the Krylov iterations. */
void orc_last_timing(double* setup_s, double* iterations_s);
/* OpenMP threads of the row-parallel products (1 without OpenMP). */
void orc_set_threads(int n);
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
