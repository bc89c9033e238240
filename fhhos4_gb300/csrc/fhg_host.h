// Host-side algebra of libfhg's setup (no CUDA): scalar and block CSR containers, the conversion
// between them, the greedy colouring, block permutations, transposes and products, the
// symmetrised outer operator, the natural injection of the p-multigrid and its Galerkin operator,
// and the small and dense inverses. Plain C++, included by fhg_api.cu; it builds without the CUDA
// toolkit as well.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <utility>
#include <vector>

namespace fhg {
namespace host {

// ---------------------------------------------------------------------------
// Host containers

struct HostCsr {
    int n_rows = 0, n_cols = 0;
    std::vector<int> rowptr, colidx;
    std::vector<double> vals;
    bool set = false;
};

// Block values block-major, row-major inside a block (host form).
struct HostBsr {
    int nbr = 0, nbc = 0, bs = 0;
    std::vector<int> rowptr, colidx;
    std::vector<double> vals;
    long long nnzb() const { return (long long)colidx.size(); }
};

// Scalar CSR -> BSR with square bs x bs blocks (missing entries of a stored block are 0).
inline void csr_to_bsr(const HostCsr& A, int bs, HostBsr& B)
{
    B.bs = bs;
    B.nbr = A.n_rows / bs;
    B.nbc = A.n_cols / bs;
    B.rowptr.assign(B.nbr + 1, 0);
    std::vector<int> mark(B.nbc, -1);
    for (int I = 0; I < B.nbr; I++) {
        int cnt = 0;
        for (int k = 0; k < bs; k++) {
            const int i = I * bs + k;
            for (int p = A.rowptr[i]; p < A.rowptr[i + 1]; p++) {
                const int J = A.colidx[p] / bs;
                if (mark[J] != I) { mark[J] = I; cnt++; }
            }
        }
        B.rowptr[I + 1] = B.rowptr[I] + cnt;
    }
    B.colidx.assign(B.rowptr[B.nbr], 0);
    B.vals.assign((size_t)B.rowptr[B.nbr] * bs * bs, 0.0);
    std::fill(mark.begin(), mark.end(), -1);
    std::vector<int> slot(B.nbc, 0);
    std::vector<int> cols;
    for (int I = 0; I < B.nbr; I++) {
        cols.clear();
        for (int k = 0; k < bs; k++) {
            const int i = I * bs + k;
            for (int p = A.rowptr[i]; p < A.rowptr[i + 1]; p++) {
                const int J = A.colidx[p] / bs;
                if (mark[J] != I) { mark[J] = I; cols.push_back(J); }
            }
        }
        std::sort(cols.begin(), cols.end());
        const int base = B.rowptr[I];
        for (size_t q = 0; q < cols.size(); q++) {
            B.colidx[base + q] = cols[q];
            slot[cols[q]] = base + (int)q;
        }
        for (int k = 0; k < bs; k++) {
            const int i = I * bs + k;
            for (int p = A.rowptr[i]; p < A.rowptr[i + 1]; p++) {
                const int j = A.colidx[p], J = j / bs;
                B.vals[(size_t)slot[J] * bs * bs + k * bs + (j - J * bs)] = A.vals[p];
            }
        }
    }
}

// Greedy colouring of the symmetric block graph in block-row order: colour(I) is the
// smallest colour absent from the already-coloured neighbours of I (rows and columns of
// the stored pattern). Same algorithm as the oracle's orc_greedy_colouring.
inline int greedy_colouring(const HostBsr& B, std::vector<int>& colour)
{
    const int nb = B.nbr;
    // transpose pattern
    std::vector<int> trp(nb + 1, 0), tci(B.colidx.size());
    for (int J : B.colidx) trp[J + 1]++;
    for (int j = 0; j < nb; j++) trp[j + 1] += trp[j];
    std::vector<int> fill(trp.begin(), trp.end() - 1);
    for (int I = 0; I < nb; I++)
        for (int p = B.rowptr[I]; p < B.rowptr[I + 1]; p++) tci[fill[B.colidx[p]]++] = I;
    colour.assign(nb, -1);
    std::vector<int> mark(nb + 1, -1);
    int maxc = 0;
    for (int I = 0; I < nb; I++) {
        for (int p = B.rowptr[I]; p < B.rowptr[I + 1]; p++) {
            const int J = B.colidx[p];
            if (J != I && colour[J] >= 0) mark[colour[J]] = I;
        }
        for (int p = trp[I]; p < trp[I + 1]; p++) {
            const int J = tci[p];
            if (J != I && colour[J] >= 0) mark[colour[J]] = I;
        }
        int c = 0;
        while (mark[c] == I) c++;
        colour[I] = c;
        maxc = std::max(maxc, c + 1);
    }
    return maxc;
}

// B' with rows perm_r (new -> old) and columns renumbered by iperm_c (old -> new).
inline void permute_bsr(const HostBsr& B, const std::vector<int>& perm_r, const std::vector<int>& iperm_c, HostBsr& O)
{
    const int bs = B.bs, bb = bs * bs;
    O.bs = bs; O.nbr = B.nbr; O.nbc = B.nbc;
    O.rowptr.assign(O.nbr + 1, 0);
    for (int I = 0; I < O.nbr; I++) {
        const int src = perm_r[I];
        O.rowptr[I + 1] = O.rowptr[I] + (B.rowptr[src + 1] - B.rowptr[src]);
    }
    O.colidx.resize(B.colidx.size());
    O.vals.resize(B.vals.size());
    std::vector<std::pair<int, int>> row;
    for (int I = 0; I < O.nbr; I++) {
        const int src = perm_r[I];
        row.clear();
        for (int p = B.rowptr[src]; p < B.rowptr[src + 1]; p++) row.emplace_back(iperm_c[B.colidx[p]], p);
        std::sort(row.begin(), row.end());
        int q = O.rowptr[I];
        for (auto& e : row) {
            O.colidx[q] = e.first;
            std::memcpy(&O.vals[(size_t)q * bb], &B.vals[(size_t)e.second * bb], sizeof(double) * bb);
            q++;
        }
    }
}

inline void transpose_bsr(const HostBsr& B, HostBsr& T)
{
    const int bs = B.bs, bb = bs * bs;
    T.bs = bs; T.nbr = B.nbc; T.nbc = B.nbr;
    T.rowptr.assign(T.nbr + 1, 0);
    for (int J : B.colidx) T.rowptr[J + 1]++;
    for (int j = 0; j < T.nbr; j++) T.rowptr[j + 1] += T.rowptr[j];
    T.colidx.resize(B.colidx.size());
    T.vals.resize(B.vals.size());
    std::vector<int> fill(T.rowptr.begin(), T.rowptr.end() - 1);
    for (int I = 0; I < B.nbr; I++)
        for (int p = B.rowptr[I]; p < B.rowptr[I + 1]; p++) {
            const int q = fill[B.colidx[p]]++;
            T.colidx[q] = I;
            for (int r = 0; r < bs; r++)
                for (int c = 0; c < bs; c++) T.vals[(size_t)q * bb + c * bs + r] = B.vals[(size_t)p * bb + r * bs + c];
        }
}

// C = A B for block-sparse operators of one block size: row-parallel Gustavson (each thread owns
// a contiguous slice of block rows and a dense block-column marker); every row is summed in the
// same order whatever the thread count.
inline void bsr_multiply(const HostBsr& A, const HostBsr& B, HostBsr& C)
{
    const int bs = A.bs, bb = bs * bs;
    C.bs = bs;
    C.nbr = A.nbr;
    C.nbc = B.nbc;
    C.rowptr.assign(C.nbr + 1, 0);
    const int nt = std::max(1, std::min((int)std::thread::hardware_concurrency(), 64));
    const int chunk = (C.nbr + nt - 1) / nt;
    auto run = [&](auto body) {
        std::vector<std::thread> th;
        for (int t = 0; t < nt; t++) {
            const int r0 = t * chunk, r1 = std::min(C.nbr, r0 + chunk);
            if (r0 < r1) th.emplace_back(body, r0, r1);
        }
        for (auto& x : th) x.join();
    };
    run([&](int r0, int r1) {
        std::vector<int> mark(C.nbc, -1);
        for (int I = r0; I < r1; I++) {
            int cnt = 0;
            for (int p = A.rowptr[I]; p < A.rowptr[I + 1]; p++) {
                const int J = A.colidx[p];
                for (int q = B.rowptr[J]; q < B.rowptr[J + 1]; q++)
                    if (mark[B.colidx[q]] != I) { mark[B.colidx[q]] = I; cnt++; }
            }
            C.rowptr[I + 1] = cnt;
        }
    });
    for (int I = 0; I < C.nbr; I++) C.rowptr[I + 1] += C.rowptr[I];
    C.colidx.assign(C.rowptr[C.nbr], 0);
    C.vals.assign((size_t)C.rowptr[C.nbr] * bb, 0.0);
    run([&](int r0, int r1) {
        std::vector<int> mark(C.nbc, -1), slot(C.nbc, 0);
        std::vector<int> cols;
        for (int I = r0; I < r1; I++) {
            cols.clear();
            for (int p = A.rowptr[I]; p < A.rowptr[I + 1]; p++) {
                const int J = A.colidx[p];
                for (int q = B.rowptr[J]; q < B.rowptr[J + 1]; q++)
                    if (mark[B.colidx[q]] != I) { mark[B.colidx[q]] = I; cols.push_back(B.colidx[q]); }
            }
            std::sort(cols.begin(), cols.end());
            const int base = C.rowptr[I];
            for (size_t k = 0; k < cols.size(); k++) {
                C.colidx[base + k] = cols[k];
                slot[cols[k]] = base + (int)k;
            }
            for (int p = A.rowptr[I]; p < A.rowptr[I + 1]; p++) {
                const double* a = &A.vals[(size_t)p * bb];
                const int J = A.colidx[p];
                for (int q = B.rowptr[J]; q < B.rowptr[J + 1]; q++) {
                    const double* b = &B.vals[(size_t)q * bb];
                    double* c = &C.vals[(size_t)slot[B.colidx[q]] * bb];
                    for (int r = 0; r < bs; r++)
                        for (int m = 0; m < bs; m++) {
                            const double arm = a[r * bs + m];
                            for (int k = 0; k < bs; k++) c[r * bs + k] += arm * b[m * bs + k];
                        }
                }
            }
        }
    });
}

// Scalar CSR of a block operator: every entry of every stored block, columns ascending.
inline void bsr_to_csr(const HostBsr& B, HostCsr& A)
{
    const int bs = B.bs, bb = bs * bs;
    A.n_rows = B.nbr * bs;
    A.n_cols = B.nbc * bs;
    A.rowptr.assign(A.n_rows + 1, 0);
    for (int I = 0; I < B.nbr; I++)
        for (int r = 0; r < bs; r++)
            A.rowptr[I * bs + r + 1] = A.rowptr[I * bs + r] + (B.rowptr[I + 1] - B.rowptr[I]) * bs;
    A.colidx.resize(A.rowptr[A.n_rows]);
    A.vals.resize(A.rowptr[A.n_rows]);
    for (int I = 0; I < B.nbr; I++)
        for (int r = 0; r < bs; r++) {
            int o = A.rowptr[I * bs + r];
            for (int p = B.rowptr[I]; p < B.rowptr[I + 1]; p++)
                for (int c = 0; c < bs; c++) {
                    A.colidx[o] = B.colidx[p] * bs + c;
                    A.vals[o++] = B.vals[(size_t)p * bb + r * bs + c];
                }
        }
    A.set = true;
}

// tril(A) + tril(A,-1)^T: the operator A.selfadjointView<Eigen::Lower>() applies
// (src/Solver/Krylov/FlexibleConjugateGradient.h:124).
inline void symmetrise_lower(const HostCsr& A, HostCsr& S)
{
    const int n = A.n_rows;
    std::vector<int> urp(n + 1, 0);
    for (int i = 0; i < n; i++)
        for (int p = A.rowptr[i]; p < A.rowptr[i + 1]; p++)
            if (A.colidx[p] < i) urp[A.colidx[p] + 1]++;
    for (int i = 0; i < n; i++) urp[i + 1] += urp[i];
    std::vector<int> uci(urp[n]);
    std::vector<double> uva(urp[n]);
    std::vector<int> fill(urp.begin(), urp.end() - 1);
    for (int i = 0; i < n; i++)
        for (int p = A.rowptr[i]; p < A.rowptr[i + 1]; p++)
            if (A.colidx[p] < i) {
                const int q = fill[A.colidx[p]]++;
                uci[q] = i;
                uva[q] = A.vals[p];
            }
    S.n_rows = S.n_cols = n;
    S.rowptr.assign(n + 1, 0);
    S.colidx.clear(); S.vals.clear();
    S.colidx.reserve(A.colidx.size());
    S.vals.reserve(A.vals.size());
    for (int i = 0; i < n; i++) {
        for (int p = A.rowptr[i]; p < A.rowptr[i + 1] && A.colidx[p] <= i; p++) {
            S.colidx.push_back(A.colidx[p]);
            S.vals.push_back(A.vals[p]);
        }
        for (int q = urp[i]; q < urp[i + 1]; q++) {
            S.colidx.push_back(uci[q]);
            S.vals.push_back(uva[q]);
        }
        S.rowptr[i + 1] = (int)S.colidx.size();
    }
    S.set = true;
}

// Whether P (scalar CSR, nb * nh rows) is the natural injection of P_LevelForHHO::SetupProlongation
// (src/Solver/Multigrid/MultigridForHHO/P_MultigridForHHO.h:69-92) onto nl < nh unknowns per face:
// row f * nh + i holds the single entry 1 at column f * nl + i for i < nl, and rows with i >= nl are
// empty. nl is read from the column count.
inline bool natural_injection(const HostCsr& P, int nh, int nb, int* nl_out)
{
    if (nb <= 0 || P.n_rows != nb * nh || P.n_cols % nb) return false;
    const int nl = P.n_cols / nb;
    if (nl <= 0 || nl >= nh) return false;
    for (int f = 0; f < nb; f++)
        for (int i = 0; i < nh; i++) {
            const int r = f * nh + i;
            const int len = P.rowptr[r + 1] - P.rowptr[r];
            if (i >= nl ? len != 0
                        : (len != 1 || P.colidx[P.rowptr[r]] != f * nl + i || P.vals[P.rowptr[r]] != 1.0))
                return false;
        }
    *nl_out = nl;
    return true;
}

// P^T A P for the natural injection: the leading nl x nl part of every nh x nh block of A, the
// entries as they are (the Galerkin operator of a p-multigrid level, Level.h:133-137).
inline void inject_galerkin(const HostCsr& A, int nh, int nl, HostCsr& C)
{
    const int nb = A.n_rows / nh;
    C = HostCsr();
    C.n_rows = C.n_cols = nb * nl;
    C.rowptr.assign(1, 0);
    for (int f = 0; f < nb; f++)
        for (int i = 0; i < nl; i++) {
            const int r = f * nh + i;
            for (int p = A.rowptr[r]; p < A.rowptr[r + 1]; p++) {
                const int c = A.colidx[p];
                if (c % nh < nl) {
                    C.colidx.push_back(c / nh * nl + c % nh);
                    C.vals.push_back(A.vals[p]);
                }
            }
            C.rowptr.push_back((int)C.colidx.size());
        }
    C.set = true;
}

inline bool csr_equal(const HostCsr& A, const HostCsr& B)
{
    return A.rowptr == B.rowptr && A.colidx == B.colidx &&
           std::memcmp(A.vals.data(), B.vals.data(), sizeof(double) * A.vals.size()) == 0;
}

// Inverse of a bs x bs block by Gauss-Jordan elimination with full pivoting (FP64).
inline bool invert_block(const double* a_in, int n, double* inv)
{
    double a[64], b[64];
    int rp[8], cp[8];
    std::memcpy(a, a_in, sizeof(double) * n * n);
    for (int i = 0; i < n * n; i++) b[i] = 0.0;
    for (int i = 0; i < n; i++) b[i * n + i] = 1.0;
    (void)rp; (void)cp;
    int colperm[8];
    for (int i = 0; i < n; i++) colperm[i] = i;
    for (int k = 0; k < n; k++) {
        int bi = k, bj = k;
        double best = -1.0;
        for (int i = k; i < n; i++)
            for (int j = k; j < n; j++)
                if (std::fabs(a[i * n + j]) > best) { best = std::fabs(a[i * n + j]); bi = i; bj = j; }
        if (!(best > 0.0) || !std::isfinite(best)) return false;
        if (bi != k)
            for (int j = 0; j < n; j++) { std::swap(a[k * n + j], a[bi * n + j]); std::swap(b[k * n + j], b[bi * n + j]); }
        if (bj != k) {
            for (int i = 0; i < n; i++) std::swap(a[i * n + k], a[i * n + bj]);
            std::swap(colperm[k], colperm[bj]);
        }
        const double piv = a[k * n + k];
        for (int j = 0; j < n; j++) { a[k * n + j] /= piv; b[k * n + j] /= piv; }
        for (int i = 0; i < n; i++) {
            if (i == k) continue;
            const double f = a[i * n + k];
            if (f == 0.0) continue;
            for (int j = 0; j < n; j++) { a[i * n + j] -= f * a[k * n + j]; b[i * n + j] -= f * b[k * n + j]; }
        }
    }
    // a is now the column permutation Q^T of the identity: (A Q)^{-1} = b  =>  A^{-1} = Q b.
    for (int k = 0; k < n; k++)
        for (int j = 0; j < n; j++) inv[colperm[k] * n + j] = b[k * n + j];
    return true;
}

// Dense Cholesky A = L L^T in place (lower), then A^{-1} = L^{-T} L^{-1}; multithreaded over columns.
inline int dense_spd_inverse(std::vector<double>& a, int n, std::vector<double>& inv)
{
    const unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    for (int j = 0; j < n; j++) {
        double d = a[(size_t)j * n + j];
        for (int k = 0; k < j; k++) d -= a[(size_t)j * n + k] * a[(size_t)j * n + k];
        if (!(d > 0.0) || !std::isfinite(d)) return 1;
        const double ljj = std::sqrt(d);
        a[(size_t)j * n + j] = ljj;
        auto work = [&](int i0, int i1) {
            for (int i = i0; i < i1; i++) {
                double v = a[(size_t)i * n + j];
                const double* ai = &a[(size_t)i * n];
                const double* aj = &a[(size_t)j * n];
                for (int k = 0; k < j; k++) v -= ai[k] * aj[k];
                a[(size_t)i * n + j] = v / ljj;
            }
        };
        const int rows = n - j - 1;
        if (rows > 256 && nt > 1) {
            std::vector<std::thread> th;
            const int chunk = (rows + nt - 1) / nt;
            for (unsigned t = 0; t < nt; t++) {
                const int i0 = j + 1 + t * chunk, i1 = std::min(n, i0 + chunk);
                if (i0 < i1) th.emplace_back(work, i0, i1);
            }
            for (auto& t : th) t.join();
        } else {
            work(j + 1, n);
        }
    }
    inv.assign((size_t)n * n, 0.0);
    auto cols = [&](int c0, int c1) {
        std::vector<double> y(n);
        for (int c = c0; c < c1; c++) {
            for (int i = 0; i < n; i++) {
                double v = (i == c) ? 1.0 : 0.0;
                const double* ai = &a[(size_t)i * n];
                for (int k = c; k < i; k++) v -= ai[k] * y[k];
                y[i] = i < c ? 0.0 : v / ai[i];
            }
            for (int i = n - 1; i >= 0; i--) {
                double v = y[i];
                for (int k = i + 1; k < n; k++) v -= a[(size_t)k * n + i] * y[k];
                y[i] = v / a[(size_t)i * n + i];
            }
            for (int i = 0; i < n; i++) inv[(size_t)i * n + c] = y[i];
        }
    };
    if (n > 128 && nt > 1) {
        std::vector<std::thread> th;
        const int chunk = (n + nt - 1) / nt;
        for (unsigned t = 0; t < nt; t++) {
            const int c0 = t * chunk, c1 = std::min(n, c0 + chunk);
            if (c0 < c1) th.emplace_back(cols, c0, c1);
        }
        for (auto& t : th) t.join();
    } else {
        cols(0, n);
    }
    return 0;
}

}  // namespace host
}  // namespace fhg
