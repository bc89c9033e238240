// Host-side setup algebra of libfhg (fhhos4_gb300/csrc/fhg_host.h) behind a small C interface, so
// that CPU tests can compare it with the oracle and with scipy (TEST INFRASTRUCTURE: built by
// `make -C oracle hostcheck` into oracle/_build/libhostcheck.so; the product does not use it).
// Matrices are scalar CSR (n_rows + 1 row pointers, column indices, values); an output matrix is
// written only when its capacity `cap` holds it, and its size is returned either way.
#include "fhg_host.h"

using namespace fhg::host;

namespace {

HostCsr wrap(int n_rows, int n_cols, const int* rp, const int* ci, const double* v)
{
    HostCsr A;
    A.n_rows = n_rows;
    A.n_cols = n_cols;
    A.rowptr.assign(rp, rp + n_rows + 1);
    A.colidx.assign(ci, ci + rp[n_rows]);
    A.vals.assign(v, v + rp[n_rows]);
    A.set = true;
    return A;
}

// n_rows, n_cols and the entry count of C; C's arrays when they fit in cap entries.
long long unwrap(const HostCsr& C, int* n_rows, int* n_cols, int* rp, int* ci, double* v, long long cap)
{
    *n_rows = C.n_rows;
    *n_cols = C.n_cols;
    const long long nnz = (long long)C.colidx.size();
    if (nnz <= cap && rp && ci && v) {
        std::copy(C.rowptr.begin(), C.rowptr.end(), rp);
        std::copy(C.colidx.begin(), C.colidx.end(), ci);
        std::copy(C.vals.begin(), C.vals.end(), v);
    }
    return nnz;
}

}  // namespace

extern "C" {

// The greedy colouring setup uses on A's block graph; returns the colour count.
int hc_colouring(int n, const int* rp, const int* ci, const double* v, int bs, int* colour)
{
    HostBsr B;
    csr_to_bsr(wrap(n, n, rp, ci, v), bs, B);
    std::vector<int> c;
    const int nc = greedy_colouring(B, c);
    std::copy(c.begin(), c.end(), colour);
    return nc;
}

// The coarse block size when P (n_rows x n_cols) is the natural injection from block size nh, else 0.
int hc_natural_injection(int n_rows, int n_cols, const int* rp, const int* ci, const double* v, int nh)
{
    int nl = 0;
    return natural_injection(wrap(n_rows, n_cols, rp, ci, v), nh, n_rows / nh, &nl) ? nl : 0;
}

// P^T A P for the natural injection (the leading nl x nl part of every block of A).
long long hc_inject_galerkin(int n, const int* rp, const int* ci, const double* v, int nh, int nl, int* out_n,
                             int* out_rp, int* out_ci, double* out_v, long long cap)
{
    HostCsr C;
    inject_galerkin(wrap(n, n, rp, ci, v), nh, nl, C);
    int cols = 0;
    return unwrap(C, out_n, &cols, out_rp, out_ci, out_v, cap);
}

// R A P with R = P^T through the block products of a Galerkin setup (block size bs on both levels).
long long hc_galerkin(int n, const int* arp, const int* aci, const double* av, int nc, const int* prp,
                      const int* pci, const double* pv, int bs, int* out_n, int* out_rp, int* out_ci,
                      double* out_v, long long cap)
{
    HostBsr Ab, Pb, Rb, APb, Cb;
    csr_to_bsr(wrap(n, n, arp, aci, av), bs, Ab);
    csr_to_bsr(wrap(n, nc, prp, pci, pv), bs, Pb);
    transpose_bsr(Pb, Rb);
    bsr_multiply(Ab, Pb, APb);
    bsr_multiply(Rb, APb, Cb);
    HostCsr C;
    bsr_to_csr(Cb, C);
    int cols = 0;
    return unwrap(C, out_n, &cols, out_rp, out_ci, out_v, cap);
}

// tril(A) + tril(A, -1)^T, the outer operator of the Krylov iteration.
long long hc_symmetrise_lower(int n, const int* rp, const int* ci, const double* v, int* out_rp, int* out_ci,
                              double* out_v, long long cap)
{
    HostCsr S;
    symmetrise_lower(wrap(n, n, rp, ci, v), S);
    int rows = 0, cols = 0;
    return unwrap(S, &rows, &cols, out_rp, out_ci, out_v, cap);
}

// Inverse of an n x n block (full pivoting); 0 when singular.
int hc_invert_block(const double* a, int n, double* inv) { return invert_block(a, n, inv) ? 1 : 0; }

// Dense SPD inverse of the coarsest solve; nonzero when A is not positive definite.
int hc_dense_spd_inverse(const double* a, int n, double* inv)
{
    std::vector<double> w(a, a + (size_t)n * n), out;
    const int rc = dense_spd_inverse(w, n, out);
    if (rc == 0) std::copy(out.begin(), out.end(), inv);
    return rc;
}

}  // extern "C"
