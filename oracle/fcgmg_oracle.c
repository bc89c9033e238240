/*
 * CPU restatement of the fhhos4 solve phase: the checker for the CUDA path.
 *
 * TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and the CPU
 * baseline leg of bench.py; never by the product. Pinned against the reference
 * harness (oracle/ref_driver.cpp) through the golden fixtures in tests/golden/.
 *
 * Restated reference code (paths relative to the fhhos4 source tree):
 *   FCG(1)        src/Solver/Krylov/FlexibleConjugateGradient.h:47-171
 *   PCG           src/Solver/Krylov/ConjugateGradient.h:27-104
 *   V-cycle       src/Solver/Multigrid/Multigrid.h:438-608 (x = 0 on entry, one cycle
 *                 per preconditioner application, Preconditioner.h:100-118,162-167)
 *   block GS      src/Solver/FixedPoint/BlockGaussSeidel.h:55-123,193-223
 *   block Jacobi  src/Solver/FixedPoint/BlockJacobi.h:57-127
 *   transfers     src/Solver/Multigrid/Level.h:139-159, R = P^T (LevelForHHO.h:535-543)
 *   coarse solve  src/Solver/Direct/EigenSparseCholesky.h:19-41 (restated as a dense
 *                 LDL^T without reordering: same factorisation, different rounding)
 *   stopping      src/Solver/IterativeSolver.h:224-247, IterationResult.h:121-139
 * Eigen 3.3.5 arithmetic restated: row-major SpMV (SparseDenseProduct.h:34-70),
 * selfadjoint-lower SpMV (SparseSelfAdjointView.h:278-330), FullPivLU (full
 * pivoting LU with unit lower factor).
 */
#include "fcgmg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static double now_s(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return t.tv_sec + 1e-9 * t.tv_nsec;
}

void orc_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

int orc_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------- */
/* Sparse products                                                           */

/* Rows are independent: with OpenMP (the reference's Eigen built with -fopenmp parallelises
 * row-major SpMV the same way, SparseDenseProduct.h:39-58) each row keeps its sequential sum. */
void orc_spmv(const orc_csr* A, const double* x, double* y)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < A->n_rows; i++) {
        double t = 0.0;
        for (int p = A->rowptr[i]; p < A->rowptr[i + 1]; p++)
            t += A->vals[p] * x[A->colidx[p]];
        y[i] = t;
    }
}

void orc_residual(const orc_csr* A, const double* b, const double* x, double* r)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < A->n_rows; i++) {
        double t = 0.0;
        for (int p = A->rowptr[i]; p < A->rowptr[i + 1]; p++)
            t += A->vals[p] * x[A->colidx[p]];
        r[i] = b[i] - t;
    }
}

void orc_spmv_sym_lower(const orc_csr* A, const double* x, double* y)
{
    int n = A->n_rows;
    memset(y, 0, sizeof(double) * (size_t)n);
    for (int j = 0; j < n; j++) {
        int p = A->rowptr[j], e = A->rowptr[j + 1];
        double xj = x[j];
        double acc = 0.0;
        for (; p < e && A->colidx[p] < j; p++) {
            double a = A->vals[p];
            int i = A->colidx[p];
            acc += a * x[i];
            y[i] += a * xj;
        }
        y[j] += acc;
        if (p < e && A->colidx[p] == j)
            y[j] += A->vals[p] * xj;
    }
}

void orc_transpose(const orc_csr* A, int* rp, int* ci, double* va)
{
    int m = A->n_cols;
    memset(rp, 0, sizeof(int) * (size_t)(m + 1));
    int nnz = A->rowptr[A->n_rows];
    for (int p = 0; p < nnz; p++) rp[A->colidx[p] + 1]++;
    for (int j = 0; j < m; j++) rp[j + 1] += rp[j];
    int* fill = (int*)malloc(sizeof(int) * (size_t)(m > 0 ? m : 1));
    memcpy(fill, rp, sizeof(int) * (size_t)m);
    for (int i = 0; i < A->n_rows; i++)
        for (int p = A->rowptr[i]; p < A->rowptr[i + 1]; p++) {
            int q = fill[A->colidx[p]]++;
            ci[q] = i;
            va[q] = A->vals[p];
        }
    free(fill);
}

/* ------------------------------------------------------------------------- */
/* Full-pivoting LU of a bs x bs block (the FullPivLU of BlockGaussSeidel::Setup). */

typedef struct {
    int n;
    double* lu;  /* n*n row-major, unit lower + upper */
    int* rp;     /* row permutation: factored row k came from row rp[k] */
    int* cp;     /* column permutation: factored column k is column cp[k] */
} orc_lu;

static int lu_factor(double* a, int n, int* rp, int* cp)
{
    for (int k = 0; k < n; k++) { rp[k] = k; cp[k] = k; }
    for (int k = 0; k < n; k++) {
        int bi = k, bj = k;
        double best = -1.0;
        for (int j = k; j < n; j++)
            for (int i = k; i < n; i++) {
                double v = fabs(a[i * n + j]);
                if (v > best) { best = v; bi = i; bj = j; }
            }
        if (best == 0.0) return 1;
        if (bi != k) {
            for (int j = 0; j < n; j++) { double t = a[k * n + j]; a[k * n + j] = a[bi * n + j]; a[bi * n + j] = t; }
            int t = rp[k]; rp[k] = rp[bi]; rp[bi] = t;
        }
        if (bj != k) {
            for (int i = 0; i < n; i++) { double t = a[i * n + k]; a[i * n + k] = a[i * n + bj]; a[i * n + bj] = t; }
            int t = cp[k]; cp[k] = cp[bj]; cp[bj] = t;
        }
        double piv = a[k * n + k];
        for (int i = k + 1; i < n; i++) a[i * n + k] /= piv;
        for (int i = k + 1; i < n; i++)
            for (int j = k + 1; j < n; j++)
                a[i * n + j] -= a[i * n + k] * a[k * n + j];
    }
    return 0;
}

static void lu_solve(const double* a, int n, const int* rp, const int* cp, const double* b, double* x)
{
    double c[64];
    for (int k = 0; k < n; k++) c[k] = b[rp[k]];
    for (int i = 0; i < n; i++)
        for (int j = 0; j < i; j++) c[i] -= a[i * n + j] * c[j];
    for (int i = n - 1; i >= 0; i--) {
        for (int j = i + 1; j < n; j++) c[i] -= a[i * n + j] * c[j];
        c[i] /= a[i * n + i];
    }
    for (int k = 0; k < n; k++) x[cp[k]] = c[k];
}

/* Diagonal-block LU factors of every block row. */
typedef struct {
    int nb, bs;
    double* lu;
    int* rp;
    int* cp;
} orc_blockdiag;

static int blockdiag_setup(orc_blockdiag* D, const orc_csr* A, int bs)
{
    int nb = A->n_rows / bs;
    D->nb = nb; D->bs = bs;
    D->lu = (double*)calloc((size_t)nb * bs * bs, sizeof(double));
    D->rp = (int*)malloc(sizeof(int) * (size_t)nb * bs);
    D->cp = (int*)malloc(sizeof(int) * (size_t)nb * bs);
    for (int ib = 0; ib < nb; ib++) {
        double* a = D->lu + (size_t)ib * bs * bs;
        for (int k = 0; k < bs; k++) {
            int i = ib * bs + k;
            for (int p = A->rowptr[i]; p < A->rowptr[i + 1]; p++) {
                int j = A->colidx[p];
                if (j / bs == ib) a[k * bs + (j - ib * bs)] = A->vals[p];
            }
        }
        if (lu_factor(a, bs, D->rp + (size_t)ib * bs, D->cp + (size_t)ib * bs)) return 1;
    }
    return 0;
}

static void blockdiag_free(orc_blockdiag* D)
{
    free(D->lu); free(D->rp); free(D->cp);
}

/* One block row of block Gauss-Seidel (BlockGaussSeidel.h:193-223) or, for omega != 1, of block
 * SOR (BlockSOR.h:199-227: x_i = D_i^-1 (omega b_i + (1 - omega) D_i x_i - omega sum_{j != i} A_ij x_j),
 * the smoother SmootherFactory.h:37-100 builds for the GS codes when the relaxation parameter is
 * not 1). */
static void gs_row(const orc_csr* A, const orc_blockdiag* D, const double* b, double* x, int ib, double omega)
{
    int bs = D->bs;
    double t[64];
    for (int k = 0; k < bs; k++) {
        int i = ib * bs + k;
        if (omega == 1.0) {
            double v = b[i];
            for (int p = A->rowptr[i]; p < A->rowptr[i + 1]; p++) {
                int j = A->colidx[p];
                if (j / bs != ib) v -= A->vals[p] * x[j];
            }
            t[k] = v;
        } else {
            double v = omega * b[i];
            for (int p = A->rowptr[i]; p < A->rowptr[i + 1]; p++) {
                int j = A->colidx[p];
                if (j / bs == ib) v += (1 - omega) * A->vals[p] * x[j];
                else v += -omega * A->vals[p] * x[j];
            }
            t[k] = v;
        }
    }
    lu_solve(D->lu + (size_t)ib * bs * bs, bs, D->rp + (size_t)ib * bs, D->cp + (size_t)ib * bs, t, x + (size_t)ib * bs);
}

static void gs_sweep(const orc_csr* A, const orc_blockdiag* D, const double* b, double* x, int backward, double omega)
{
    int nb = D->nb;
    if (!backward)
        for (int ib = 0; ib < nb; ib++) gs_row(A, D, b, x, ib, omega);
    else
        for (int ib = nb - 1; ib >= 0; ib--) gs_row(A, D, b, x, ib, omega);
}

static void jacobi_sweep(const orc_csr* A, const orc_blockdiag* D, double omega, const double* b, double* x, double* xnew)
{
    int bs = D->bs, nb = D->nb;
    double t[64];
    for (int ib = 0; ib < nb; ib++) {
        for (int k = 0; k < bs; k++) {
            int i = ib * bs + k;
            double v = omega * b[i];
            for (int p = A->rowptr[i]; p < A->rowptr[i + 1]; p++) {
                int j = A->colidx[p];
                if (j / bs == ib) v += (1 - omega) * A->vals[p] * x[j];
                else v += -omega * A->vals[p] * x[j];
            }
            t[k] = v;
        }
        lu_solve(D->lu + (size_t)ib * bs * bs, bs, D->rp + (size_t)ib * bs, D->cp + (size_t)ib * bs, t, xnew + (size_t)ib * bs);
    }
    memcpy(x, xnew, sizeof(double) * (size_t)nb * bs);
}

void orc_block_gs(const orc_csr* A, int bs, const double* b, double* x, int backward)
{
    orc_blockdiag D;
    if (blockdiag_setup(&D, A, bs) == 0) gs_sweep(A, &D, b, x, backward, 1.0);
    blockdiag_free(&D);
}

void orc_block_jacobi(const orc_csr* A, int bs, double omega, const double* b, double* x)
{
    orc_blockdiag D;
    double* xn = (double*)malloc(sizeof(double) * (size_t)A->n_rows);
    if (blockdiag_setup(&D, A, bs) == 0) jacobi_sweep(A, &D, omega, b, x, xn);
    blockdiag_free(&D);
    free(xn);
}

/* ------------------------------------------------------------------------- */
/* Colouring                                                                 */

int orc_greedy_colouring(const orc_csr* A, int bs, int* colour)
{
    int nb = A->n_rows / bs;
    /* Column pattern (transpose) so that the block graph is symmetric. */
    int nnz = A->rowptr[A->n_rows];
    int* trp = (int*)calloc((size_t)A->n_cols + 1, sizeof(int));
    int* tci = (int*)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
    for (int p = 0; p < nnz; p++) trp[A->colidx[p] + 1]++;
    for (int j = 0; j < A->n_cols; j++) trp[j + 1] += trp[j];
    int* fill = (int*)malloc(sizeof(int) * (size_t)(A->n_cols > 0 ? A->n_cols : 1));
    memcpy(fill, trp, sizeof(int) * (size_t)A->n_cols);
    for (int i = 0; i < A->n_rows; i++)
        for (int p = A->rowptr[i]; p < A->rowptr[i + 1]; p++) tci[fill[A->colidx[p]]++] = i;
    free(fill);

    int maxc = 1;
    int* mark = (int*)malloc(sizeof(int) * (size_t)(nb + 1));
    for (int c = 0; c <= nb; c++) mark[c] = -1;
    for (int ib = 0; ib < nb; ib++) colour[ib] = -1;
    for (int ib = 0; ib < nb; ib++) {
        for (int k = 0; k < bs; k++) {
            int i = ib * bs + k;
            for (int p = A->rowptr[i]; p < A->rowptr[i + 1]; p++) {
                int jb = A->colidx[p] / bs;
                if (jb != ib && colour[jb] >= 0) mark[colour[jb]] = ib;
            }
            for (int p = trp[i]; p < trp[i + 1]; p++) {
                int jb = tci[p] / bs;
                if (jb != ib && colour[jb] >= 0) mark[colour[jb]] = ib;
            }
        }
        int c = 0;
        while (mark[c] == ib) c++;
        colour[ib] = c;
        if (c + 1 > maxc) maxc = c + 1;
    }
    free(mark); free(trp); free(tci);
    return nb > 0 ? maxc : 0;
}

void orc_colour_permutation(int nb, const int* colour, int ncolours, int* perm)
{
    int* start = (int*)calloc((size_t)ncolours + 1, sizeof(int));
    for (int i = 0; i < nb; i++) start[colour[i] + 1]++;
    for (int c = 0; c < ncolours; c++) start[c + 1] += start[c];
    for (int i = 0; i < nb; i++) perm[start[colour[i]]++] = i;
    free(start);
}

/* ------------------------------------------------------------------------- */
/* Dense LDL^T for the coarsest level                                        */

typedef struct { int n; double* L; double* d; } orc_ldlt;

static int ldlt_setup(orc_ldlt* F, const orc_csr* A)
{
    int n = A->n_rows;
    F->n = n;
    F->L = (double*)calloc((size_t)n * n, sizeof(double));
    F->d = (double*)calloc((size_t)n, sizeof(double));
    double* a = F->L;
    for (int i = 0; i < n; i++)
        for (int p = A->rowptr[i]; p < A->rowptr[i + 1]; p++) a[(size_t)i * n + A->colidx[p]] = A->vals[p];
    for (int j = 0; j < n; j++) {
        double dj = a[(size_t)j * n + j];
        for (int k = 0; k < j; k++) dj -= a[(size_t)j * n + k] * a[(size_t)j * n + k] * F->d[k];
        if (!(dj > 0.0)) return 1;
        F->d[j] = dj;
        for (int i = j + 1; i < n; i++) {
            double v = a[(size_t)i * n + j];
            for (int k = 0; k < j; k++) v -= a[(size_t)i * n + k] * a[(size_t)j * n + k] * F->d[k];
            a[(size_t)i * n + j] = v / dj;
        }
    }
    return 0;
}

static void ldlt_solve(const orc_ldlt* F, const double* b, double* x)
{
    int n = F->n;
    const double* L = F->L;
    for (int i = 0; i < n; i++) {
        double v = b[i];
        for (int k = 0; k < i; k++) v -= L[(size_t)i * n + k] * x[k];
        x[i] = v;
    }
    for (int i = 0; i < n; i++) x[i] /= F->d[i];
    for (int i = n - 1; i >= 0; i--) {
        double v = x[i];
        for (int k = i + 1; k < n; k++) v -= L[(size_t)k * n + i] * x[k];
        x[i] = v;
    }
}

/* ------------------------------------------------------------------------- */
/* V-cycle and Krylov drivers                                                */

typedef struct {
    int nlevels;
    const orc_csr* A;
    const orc_csr* P;
    orc_csr* R;
    orc_blockdiag* D;
    orc_ldlt coarse;
    const orc_options* opt;
    double** r;   /* per-level scratch */
    double** rc;
    double** ec;
    double** tmp;
    double** kc;  /* K-cycle: per-level c, A c, d, A d */
    double** kv;
    double** kd;
    double** kw;
} orc_mg;

/* One smoother application of `iters` iterations: BlockGaussSeidel::ExecuteOneIteration's
 * directions (BlockGaussSeidel.h:84-120): symmetric = forward then backward; alternating =
 * forward/backward by iteration parity (IterationCount restarts at 0 in every Solve). */
static void smooth(orc_mg* mg, int l, int code, int iters, const double* b, double* x)
{
    const double w = mg->opt->sor_omega;
    for (int s = 0; s < iters; s++) {
        switch (code) {
        case ORC_BJ: jacobi_sweep(&mg->A[l], &mg->D[l], mg->opt->omega, b, x, mg->tmp[l]); break;
        case ORC_BGS_FORWARD: gs_sweep(&mg->A[l], &mg->D[l], b, x, 0, w); break;
        case ORC_BGS_BACKWARD: gs_sweep(&mg->A[l], &mg->D[l], b, x, 1, w); break;
        case ORC_BGS_SYMMETRIC:
            gs_sweep(&mg->A[l], &mg->D[l], b, x, 0, w);
            gs_sweep(&mg->A[l], &mg->D[l], b, x, 1, w);
            break;
        case ORC_BGS_ALTERNATING_FORWARD_FIRST: gs_sweep(&mg->A[l], &mg->D[l], b, x, s % 2, w); break;
        default: gs_sweep(&mg->A[l], &mg->D[l], b, x, 1 - s % 2, w); break;
        }
    }
}

static void cycle(orc_mg* mg, int l, const double* b, double* x, int x_zero);

static double dot(const double* a, const double* b, int n)
{
    double s = 0.0;
    for (int i = 0; i < n; i++) s += a[i] * b[i];
    return s;
}

/* Multigrid::FCGForKCycle (Multigrid.h:611-656): x = the coarse correction on level m from two
 * FCG steps preconditioned by the cycle on level m, the second only when the first reduced ||r||
 * by less than t = 0.25. r is overwritten (r -= (alpha1 / rho1) A c). */
static void kcycle_fcg(orc_mg* mg, int m, double* r, double* x)
{
    const int n = mg->A[m].n_rows;
    double *c = mg->kc[m], *v = mg->kv[m], *d = mg->kd[m], *w = mg->kw[m];
    cycle(mg, m, r, c, 1);
    orc_spmv(&mg->A[m], c, v);
    const double rho1 = dot(c, v, n), alpha1 = dot(c, r, n);
    const double norm_old = sqrt(dot(r, r, n));
    for (int i = 0; i < n; i++) r[i] -= (alpha1 / rho1) * v[i];
    const double norm_new = sqrt(dot(r, r, n));
    if (norm_new <= 0.25 * norm_old) {
        for (int i = 0; i < n; i++) x[i] = (alpha1 / rho1) * c[i];
        return;
    }
    cycle(mg, m, r, d, 1);
    orc_spmv(&mg->A[m], d, w);
    const double gamma = dot(d, v, n), beta = dot(d, w, n), alpha2 = dot(d, r, n);
    const double rho2 = beta - gamma * gamma / rho1;
    const double a = alpha1 / rho1 - gamma * alpha2 / (rho1 * rho2), bb = alpha2 / rho2;
    for (int i = 0; i < n; i++) x[i] = a * c[i] + bb * d[i];
}

/* Multigrid::MultigridCycle (Multigrid.h:438-608) for V (WLoops 1), W (WLoops 2) and K: x is the
 * initial guess (zero when x_zero); the coarse correction loops WLoops times except directly
 * above the coarsest level, or (K) is kcycle_fcg on the coarser level unless that is the
 * coarsest. */
static void cycle(orc_mg* mg, int l, const double* b, double* x, int x_zero)
{
    int n = mg->A[l].n_rows;
    if (l == mg->nlevels - 1) {
        ldlt_solve(&mg->coarse, b, x);
        return;
    }
    if (x_zero) memset(x, 0, sizeof(double) * (size_t)n);
    const int npre = l > 0 && mg->opt->coarse_pre_iterations >= 0 ? mg->opt->coarse_pre_iterations
                                                                  : mg->opt->pre_iterations;
    const int npost = l > 0 && mg->opt->coarse_post_iterations >= 0 ? mg->opt->coarse_post_iterations
                                                                    : mg->opt->post_iterations;
    smooth(mg, l, mg->opt->pre_smoother, npre, b, x);
    orc_residual(&mg->A[l], b, x, mg->r[l]);
    orc_spmv(&mg->R[l], mg->r[l], mg->rc[l]);
    int nc = mg->A[l + 1].n_rows;
    memset(mg->ec[l], 0, sizeof(double) * (size_t)nc);
    if (mg->opt->w_loops == ORC_CYCLE_K && l + 1 < mg->nlevels - 1) {
        kcycle_fcg(mg, l + 1, mg->rc[l], mg->ec[l]);
    } else {
        const int loops = mg->opt->w_loops > 1 ? mg->opt->w_loops : 1;
        for (int w = 0; w < loops; w++) {
            cycle(mg, l + 1, mg->rc[l], mg->ec[l], w == 0);
            if (l + 1 == mg->nlevels - 1) break;
        }
    }
    orc_spmv(&mg->P[l], mg->ec[l], mg->r[l]);
    for (int i = 0; i < n; i++) x[i] += mg->r[l][i];
    smooth(mg, l, mg->opt->post_smoother, npost, b, x);
}

static void vcycle(orc_mg* mg, int l, const double* b, double* x) { cycle(mg, l, b, x, 1); }

static double g_setup_s = 0.0, g_iter_s = 0.0;

void orc_last_timing(double* setup_s, double* iterations_s)
{
    *setup_s = g_setup_s;
    *iterations_s = g_iter_s;
}

int orc_fcgmg_solve(int nlevels, int bs, const orc_csr* A, const orc_csr* P,
                    const double* b, double* x, const orc_options* opt,
                    double* history, int* iterations)
{
    int* bs_l = (int*)malloc(sizeof(int) * (size_t)(nlevels > 0 ? nlevels : 1));
    for (int l = 0; l < nlevels; l++) bs_l[l] = bs;
    int rc = orc_fcgmg_solve_levels(nlevels, bs_l, A, P, b, x, opt, history, iterations);
    free(bs_l);
    return rc;
}

int orc_fcgmg_solve_levels(int nlevels, const int* bs, const orc_csr* A, const orc_csr* P,
                           const double* b, double* x, const orc_options* opt,
                           double* history, int* iterations)
{
    const double t0 = now_s();
    orc_mg mg;
    memset(&mg, 0, sizeof(mg));
    mg.nlevels = nlevels; mg.A = A; mg.P = P; mg.opt = opt;
    int rc = 0;
    mg.R = (orc_csr*)calloc((size_t)(nlevels > 1 ? nlevels - 1 : 1), sizeof(orc_csr));
    mg.D = (orc_blockdiag*)calloc((size_t)nlevels, sizeof(orc_blockdiag));
    mg.r = (double**)calloc((size_t)nlevels, sizeof(double*));
    mg.rc = (double**)calloc((size_t)nlevels, sizeof(double*));
    mg.ec = (double**)calloc((size_t)nlevels, sizeof(double*));
    mg.tmp = (double**)calloc((size_t)nlevels, sizeof(double*));
    mg.kc = (double**)calloc((size_t)nlevels, sizeof(double*));
    mg.kv = (double**)calloc((size_t)nlevels, sizeof(double*));
    mg.kd = (double**)calloc((size_t)nlevels, sizeof(double*));
    mg.kw = (double**)calloc((size_t)nlevels, sizeof(double*));
    for (int l = 0; l < nlevels; l++) {
        const size_t nl = (size_t)A[l].n_rows;
        mg.kc[l] = (double*)malloc(sizeof(double) * nl);
        mg.kv[l] = (double*)malloc(sizeof(double) * nl);
        mg.kd[l] = (double*)malloc(sizeof(double) * nl);
        mg.kw[l] = (double*)malloc(sizeof(double) * nl);
    }
    for (int l = 0; l + 1 < nlevels; l++) {
        int nnz = P[l].rowptr[P[l].n_rows];
        int* rp = (int*)malloc(sizeof(int) * (size_t)(P[l].n_cols + 1));
        int* ci = (int*)malloc(sizeof(int) * (size_t)(nnz > 0 ? nnz : 1));
        double* va = (double*)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
        orc_transpose(&P[l], rp, ci, va);
        mg.R[l].n_rows = P[l].n_cols; mg.R[l].n_cols = P[l].n_rows;
        mg.R[l].rowptr = rp; mg.R[l].colidx = ci; mg.R[l].vals = va;
        if (blockdiag_setup(&mg.D[l], &A[l], bs[l])) rc = 2;
        mg.r[l] = (double*)malloc(sizeof(double) * (size_t)A[l].n_rows);
        mg.tmp[l] = (double*)malloc(sizeof(double) * (size_t)A[l].n_rows);
        mg.rc[l] = (double*)malloc(sizeof(double) * (size_t)A[l + 1].n_rows);
        mg.ec[l] = (double*)malloc(sizeof(double) * (size_t)A[l + 1].n_rows);
    }
    if (ldlt_setup(&mg.coarse, &A[nlevels - 1])) rc = 3;

    const double t1 = now_s();
    g_setup_s = t1 - t0;
    int n = A[0].n_rows;
    double* r = (double*)malloc(sizeof(double) * (size_t)n);
    double* z = (double*)malloc(sizeof(double) * (size_t)n);
    double* d = (double*)malloc(sizeof(double) * (size_t)n);
    double* Ad = (double*)malloc(sizeof(double) * (size_t)n);
    double* dp = (double*)malloc(sizeof(double) * (size_t)n);
    double* Adp = (double*)malloc(sizeof(double) * (size_t)n);
    int it = 0;
    if (rc == 0) {
        memset(x, 0, sizeof(double) * (size_t)n);
        memcpy(r, b, sizeof(double) * (size_t)n);
        double bnorm = sqrt(dot(b, b, n));
        double nr = 1.0;
        history[0] = nr;
        if (opt->krylov == ORC_KRYLOV_CG) {
            vcycle(&mg, 0, r, z);
            memcpy(d, z, sizeof(double) * (size_t)n);
            double rz = dot(r, z, n), beta = 0.0;
            while (!(it > 0 && (it >= opt->max_iterations || nr < opt->tolerance))) {
                if (it > 0)
                    for (int i = 0; i < n; i++) d[i] = z[i] + beta * d[i];
                orc_spmv(&A[0], d, Ad);
                double alpha = rz / dot(d, Ad, n);
                for (int i = 0; i < n; i++) x[i] += alpha * d[i];
                double old = rz;
                for (int i = 0; i < n; i++) r[i] -= alpha * Ad[i];
                vcycle(&mg, 0, r, z);
                rz = dot(r, z, n);
                beta = rz / old;
                it++;
                double rn = sqrt(dot(r, r, n));
                nr = bnorm > 0 ? rn / bnorm : rn;
                history[it] = nr;
                if (isnan(nr) || isinf(nr)) { rc = 4; break; }
            }
        } else {
            int have_prev = 0;
            double dAd_prev = 0.0;
            while (!(it > 0 && (it >= opt->max_iterations || nr < opt->tolerance))) {
                vcycle(&mg, 0, r, z);
                memcpy(d, z, sizeof(double) * (size_t)n);
                if (have_prev) {
                    double s = dot(z, Adp, n) / dAd_prev;
                    for (int i = 0; i < n; i++) d[i] -= s * dp[i];
                }
                orc_spmv_sym_lower(&A[0], d, Ad);
                double dAd = dot(d, Ad, n);
                double alpha = dot(r, d, n) / dAd;
                for (int i = 0; i < n; i++) x[i] += alpha * d[i];
                for (int i = 0; i < n; i++) r[i] -= alpha * Ad[i];
                memcpy(dp, d, sizeof(double) * (size_t)n);
                memcpy(Adp, Ad, sizeof(double) * (size_t)n);
                dAd_prev = dAd;
                have_prev = 1;
                it++;
                double rn = sqrt(dot(r, r, n));
                nr = bnorm > 0 ? rn / bnorm : rn;
                history[it] = nr;
                if (isnan(nr) || isinf(nr)) { rc = 4; break; }
            }
        }
    }
    *iterations = it;
    g_iter_s = now_s() - t1;

    free(r); free(z); free(d); free(Ad); free(dp); free(Adp);
    for (int l = 0; l + 1 < nlevels; l++) {
        free((void*)mg.R[l].rowptr); free((void*)mg.R[l].colidx); free((void*)mg.R[l].vals);
        blockdiag_free(&mg.D[l]);
        free(mg.r[l]); free(mg.tmp[l]); free(mg.rc[l]); free(mg.ec[l]);
    }
    free(mg.coarse.L); free(mg.coarse.d);
    for (int l = 0; l < nlevels; l++) { free(mg.kc[l]); free(mg.kv[l]); free(mg.kd[l]); free(mg.kw[l]); }
    free(mg.kc); free(mg.kv); free(mg.kd); free(mg.kw);
    free(mg.R); free(mg.D); free(mg.r); free(mg.rc); free(mg.ec); free(mg.tmp);
    return rc;
}
