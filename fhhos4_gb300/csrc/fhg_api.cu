// libfhg host side: the C ABI of include/fhg.h.
//
// Setup (host, once; the reference's Multigrid::Setup, src/Solver/Multigrid/Multigrid.h:88-313):
//   scalar CSR of every A_l, P_l  ->  face-block BSR  ->  greedy multicolouring of the block
//   graph  ->  colour-grouped numbering  ->  pre-inverted diagonal blocks, R = P^T,
//   symmetrised outer operator, dense inverse of the coarsest operator  ->  upload.
// Solve (device only): FCG(1) or PCG preconditioned by one V-cycle from zero, Krylov
// scalars on the device, one CUDA graph per iteration, one 8-byte read-back of the
// normalised residual per iteration for the stopping test.
#include "fhg.h"
#include "fhg_coarse.h"
#include "fhg_host.h"
#include "fhg_internal.h"

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
#include <vector>

using fhg::BsrView;
using fhg::dfl;
using namespace fhg::host;

namespace {

template <class T>
struct DevBsr {
    BsrView<T> v;
    T* vals = nullptr;
    int* rowptr = nullptr;   // row pointers (CSR), or the row permutation of a jagged view
    int* colidx = nullptr;
    int* jds_start = nullptr;  // slot offsets of a jagged view
    bool owns_index = true;
};

struct Level {
    int n = 0, nb = 0, bs = 0;
    HostCsr A_in, P_in;
    bool A_is_galerkin = false;    // A_in was computed as R A P by a setup with galerkin = 1
    int ncolours = 0;
    // Launch shape of the GS/Jacobi sweeps per value type (index FHG_PREC_FP64 / FP32 / DF):
    // lanes per block row (0: those of A), blocks per lane step, and whether the sweeps use the
    // slot-major view (setup: gs_layout or the autotuner).
    int gs_lanes[3] = {0, 0, 0};
    int gs_unroll[3] = {1, 1, 1};
    bool gs_slot[3] = {false, false, false};
    bool prod_slot[3] = {false, false, false};  // products with A use the slot-major view
    int outer_lanes = 0;           // level 0: lanes of the FP64 outer product (0: those of its view)
    bool outer_slot = true;        // level 0: the pair outer product on the slot-major view (Ahat2s)
    std::vector<int> colour_start;  // block-row offsets of every colour, ncolours + 1
    std::vector<int> perm;          // new block row -> given block row
    DevBsr<double> A, Ahat, P, R;
    bool ahat_is_a = true;
    DevBsr<float> A32, P32, R32;
    DevBsr<float> G32;          // FP32 GS operator: A's off-diagonal blocks in padded rows, when they fit
    DevBsr<float> A32p;         // FP32 A in padded rows (all blocks), when they fit
    DevBsr<float> G32s;         // the GS view slot-major per colour (one thread per row), when built
    DevBsr<float> A32s;         // FP32 A slot-major (all blocks, one thread per row), when built
    // FP32-pair copies (FHG_PREC_DF: FP64-class V-cycle on the FP32 pipe), same views as FP32
    DevBsr<dfl> A2, P2, R2, G2, A2p, G2s, A2s;
    // jagged (JDS) views of the transfers, levels 0 and 1 (the large ones), and whether the products
    // use them (per V-cycle precision, chosen by timing at setup)
    DevBsr<float> P32j, R32j;
    DevBsr<dfl> P2j, R2j;
    bool p_jds[3] = {false, false, false}, r_jds[3] = {false, false, false};
    dfl* dinv2 = nullptr;
    dfl *x2 = nullptr, *b2 = nullptr, *r2 = nullptr;
    dfl* kv2[4] = {nullptr, nullptr, nullptr, nullptr};
    DevBsr<dfl> Ahat2s;         // level 0: the outer operator as FP32 pairs, slot-major (when its rows allow)
    DevBsr<float> Ahat_hi;      // level 0, FP32 V-cycle: outer operator as an FP32 pair (hi part)
    float* ahat_lo = nullptr;   // (lo part, same layout)
    double* dinv = nullptr;
    float* dinv32 = nullptr;
    int* perm_d = nullptr;
    double *x = nullptr, *b = nullptr, *r = nullptr;
    float *x32 = nullptr, *b32 = nullptr, *r32 = nullptr;
    double* kv64[4] = {nullptr, nullptr, nullptr, nullptr};  // K-cycle c, A c, d, A d (levels 1..L-2)
    float* kv32[4] = {nullptr, nullptr, nullptr, nullptr};
    double* cinv = nullptr;  // coarsest only, n x n row-major
    long long p_blocks = 0;
    // The transfer to the next level is the natural injection between face degrees (a p-multigrid
    // level: same faces, the next level's block size smaller): no P / R operators, the map of block
    // rows (this level's order -> the next level's) instead.
    bool inject = false;
    int* inj_map = nullptr;
};

}  // namespace

// Iterations over which the learned step's residual reduction is compared with the plain method's.
constexpr int kFallbackWindow = 4;

struct fhg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    std::vector<Level> levels;
    int nlevels = 0;
    fhg_options opts{};
    bool ready = false;
    // Krylov state (level-0 numbering after permutation)
    double *kx = nullptr, *kr = nullptr, *kb = nullptr, *kz[2] = {nullptr, nullptr}, *kAd[2] = {nullptr, nullptr};
    double* kt = nullptr;        // b - A x of the returned x (the true residual)
    double* partials = nullptr;  // 8 * kReduceCtas
    double* scal = nullptr;      // [0]=bnorm [1]=dAdp [2]=nr [3]=rz [4]=beta
    double* hist_d = nullptr;
    int* counter_d = nullptr;
    int* loop_state = nullptr;   // device-loop state (fhg::kLoop*): replacements left, go on, compensated check
    double* nr_host = nullptr;   // pinned
    double* io = nullptr;        // user-numbered I/O scratch (2 * n0)
    // Double-FP32 outer iteration (FP32 V-cycle with the split outer operator): the low part of r,
    // whose high part is the V-cycle input b32; d and Ad live as FP32 pairs in kz[p] and kAd[p]
    // (hi: n floats, then lo); x stays FP64 in kx.
    float* rlo = nullptr;
    float* rhi = nullptr;        // the high part of r when the V-cycle is not FP32 (pair V-cycle)
    cudaGraphExec_t graph[2] = {nullptr, nullptr};
    long long graph_kernels[2] = {0, 0};
    int graphs_built = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<void*> allocations;
    std::vector<size_t> allocation_bytes;   // beside allocations, same order
    // Learned correction of the FP32 V-cycle on the finest level (built at setup when the
    // V-cycle is FP32 and bs <= 4; the network is installed with fhg_set_learned).
    int* nbr_d = nullptr;              // nb0 x 6 neighbour blocks by decreasing |A_ij|_F, -1 padded
    uint16_t* tfeat_d = nullptr;       // nb0 x 16 BF16 element-tensor features (colour numbering)
    std::vector<double> tensors_host;  // nb0 x 12 element tensors, caller's numbering
    float* lw = nullptr;               // D^-1 r scratch (n0)
    float* lparams = nullptr;          // FP32 parameters of the installed network
    uint16_t* lwts = nullptr;          // its BF16 weights
    float* lbias = nullptr;            // its FP32 biases
    int* lstatus = nullptr;            // set to 1 by a learned-step kernel whose bounded wait expired
    int learned_kernel = 0;            // fhg::kLearnedKernelTcgen05 or kLearnedKernelMmaSync
    int learned_mode = FHG_LEARNED_OFF;
    bool learned_now = false;          // the cycle being launched or captured applies the step
    double rho_plain = 0.0;            // calibrated per-iteration reduction of the plain method
    cudaGraphExec_t graph_l[2] = {nullptr, nullptr};
    long long graph_l_kernels[2] = {0, 0};
    int graphs_l_built = 0;
    bool device_loop = false;          // capturing for the device-side loop: no host read-back
    int fused_from[3] = {-1, -1, -1};  // per V-cycle precision: first level of the coarse sub-cycle run as
                                       // one cluster launch (-1: none), and the cluster's CTAs
    int fused_ctas[3] = {fhg::kClusterCtasPortable, fhg::kClusterCtasPortable, fhg::kClusterCtasPortable};
    int fused_threads[3] = {fhg::kFusedThreads, fhg::kFusedThreads, fhg::kFusedThreads};  // and its CTAs' threads
    long long epoch = 0;               // incremented by every setup (batched graphs hold its buffers)
};

// Many independent solves in one graph launch (fhg_batch_*): per problem a captured prelude, a
// WHILE conditional node whose body is one FCG iteration and the device-side stopping test, and a
// captured epilogue (FP64 true residual, x out).
struct fhg_batch {
    int device = 0;
    std::string err;
    std::vector<fhg_ctx*> probs;
    std::vector<long long> epochs;     // setup epoch of every context when the graph was built
    std::vector<long long> body_kernels;   // per problem: kernels of one loop iteration
    std::vector<long long> check_kernels;  // per problem: kernels of one true-residual check (IF body)
    long long fixed_kernels = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraphExec_t exec = nullptr;
};

// Training state of one network (fhg_net_*): FP32 master parameters, Adam moments and the
// activations of one field.
struct fhg_net {
    int device = 0;
    std::string err;
    float *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;
    uint16_t* wts = nullptr;
    float* bias = nullptr;
    int step = 0;
    long long rows_cap = 0;
    uint16_t *feat = nullptr, *h1 = nullptr, *h2 = nullptr, *dy = nullptr, *d2 = nullptr, *d1 = nullptr;
    float *a1 = nullptr, *a2 = nullptr, *y = nullptr, *dh = nullptr, *scale = nullptr, *c = nullptr, *q = nullptr;
    float *gparts = nullptr, *cparts = nullptr;
    double* lparts = nullptr;
    double* lparts_host = nullptr;
    std::vector<void*> fixed, scratch;
};

namespace {

int fail(fhg_ctx* c, int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define CK(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return fail(ctx, FHG_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));       \
    } while (0)

template <class T>
int dalloc(fhg_ctx* ctx, T** p, size_t count)
{
    void* q = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&q, count * sizeof(T));
    if (e != cudaSuccess)
        return fail(ctx, FHG_ERR_CUDA, "cudaMalloc(%zu bytes) failed: %s", count * sizeof(T), cudaGetErrorString(e));
    ctx->allocations.push_back(q);
    ctx->allocation_bytes.push_back(count * sizeof(T));
    *p = (T*)q;
    return FHG_OK;
}

// Free one allocation of the context (null: nothing).
void dfree(fhg_ctx* ctx, const void* q)
{
    if (!q) return;
    auto it = std::find(ctx->allocations.begin(), ctx->allocations.end(), q);
    if (it == ctx->allocations.end()) return;
    ctx->allocation_bytes.erase(ctx->allocation_bytes.begin() + (it - ctx->allocations.begin()));
    ctx->allocations.erase(it);
    cudaFree(const_cast<void*>(q));
}

template <class T>
int upload(fhg_ctx* ctx, T** p, const T* src, size_t count)
{
    int rc = dalloc(ctx, p, count);
    if (rc) return rc;
    if (count) CK(cudaMemcpy(*p, src, count * sizeof(T), cudaMemcpyHostToDevice));
    return FHG_OK;
}

int check_csr(fhg_ctx* ctx, const char* what, int n_rows, int n_cols, const int* rp, const int* ci)
{
    if (rp[0] != 0) return fail(ctx, FHG_ERR_INVALID_ARG, "%s: rowptr[0] != 0", what);
    for (int i = 0; i < n_rows; i++) {
        if (rp[i + 1] < rp[i]) return fail(ctx, FHG_ERR_INVALID_ARG, "%s: rowptr decreases at row %d", what, i);
        for (int p = rp[i]; p < rp[i + 1]; p++) {
            if (ci[p] < 0 || ci[p] >= n_cols)
                return fail(ctx, FHG_ERR_INVALID_ARG, "%s: column %d out of range in row %d", what, ci[p], i);
            if (p > rp[i] && ci[p] <= ci[p - 1])
                return fail(ctx, FHG_ERR_INVALID_ARG, "%s: columns not strictly ascending in row %d", what, i);
        }
    }
    return FHG_OK;
}

long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

int default_lanes(const HostBsr& B)
{
    const double avg = B.nbr ? (double)B.nnzb() / B.nbr : 1.0;
    if (avg <= 4.5) return 4;
    if (avg <= 9.0) return 8;
    if (avg <= 18.0) return 16;
    return 32;
}

template <class T>
int upload_bsr(fhg_ctx* ctx, const HostBsr& B, DevBsr<T>& D, const DevBsr<double>* share_index)
{
    const int bb = B.bs * B.bs;
    const long long nnzb = B.nnzb();
    const long long ld = round_up(std::max<long long>(nnzb, 1), 32);
    std::vector<T> soa((size_t)ld * bb, T(0));
    for (long long p = 0; p < nnzb; p++)
        for (int e = 0; e < bb; e++) soa[(size_t)e * ld + p] = (T)B.vals[(size_t)p * bb + e];
    int rc;
    if (share_index) {
        D.rowptr = share_index->rowptr;
        D.colidx = share_index->colidx;
        D.owns_index = false;
    } else {
        if ((rc = upload(ctx, &D.rowptr, B.rowptr.data(), B.rowptr.size()))) return rc;
        if ((rc = upload(ctx, &D.colidx, B.colidx.data(), B.colidx.size()))) return rc;
    }
    if ((rc = upload(ctx, &D.vals, soa.data(), soa.size()))) return rc;
    D.v.nbr = B.nbr; D.v.nbc = B.nbc; D.v.bs = B.bs; D.v.nnzb = nnzb; D.v.ld = ld;
    D.v.rowptr = D.rowptr; D.v.colidx = D.colidx; D.v.vals = D.vals;
    D.v.lanes = default_lanes(B);
    return FHG_OK;
}

// A block operator in padded rows (FP32, entry-major, column order kept; empty slots hold zero
// values and a column inside the operator: the row's own, skipped by a GS sweep as the diagonal,
// for the off-diagonal view; the row's last stored column (0 for an empty row) otherwise, which a
// product adds as an exact zero):
// W = the most blocks of a row, row i's blocks at i * W, so a kernel reads no row pointer before
// them. `offdiag`: only the off-diagonal blocks (the GS sweeps, which apply D^-1 instead). Built
// when W <= max_w and the padding adds at most half to the stored blocks (about 1% for the
// operators of a 64^3 tetrahedral mesh, more on small meshes whose faces near the boundary have
// fewer neighbours); otherwise D stays empty and the kernels use the CSR form.
template <class T>
int upload_padded(fhg_ctx* ctx, const HostBsr& B, DevBsr<T>& D, bool offdiag, int max_w)
{
    D = DevBsr<T>();
    int W = 0;
    long long kept = 0;
    for (int i = 0; i < B.nbr; i++) {
        int c = 0;
        for (int p = B.rowptr[i]; p < B.rowptr[i + 1]; p++) c += !(offdiag && B.colidx[p] == i);
        W = std::max(W, c);
        kept += c;
    }
    const long long slots = (long long)B.nbr * W;
    if (W == 0 || W > max_w || slots > kept + kept / 2 || slots > INT32_MAX) return FHG_OK;
    const int bb = B.bs * B.bs;
    const long long ld = round_up(slots, 32);
    std::vector<int> col((size_t)slots);
    std::vector<T> soa((size_t)ld * bb, T(0));
    for (int i = 0; i < B.nbr; i++) {
        long long q = (long long)i * W;
        int last = 0;
        for (int p = B.rowptr[i]; p < B.rowptr[i + 1]; p++) {
            if (offdiag && B.colidx[p] == i) continue;
            col[(size_t)q] = last = B.colidx[p];
            for (int e = 0; e < bb; e++) soa[(size_t)e * ld + q] = (T)B.vals[(size_t)p * bb + e];
            q++;
        }
        for (; q < (long long)(i + 1) * W; q++) col[(size_t)q] = offdiag ? i : last;
    }
    int rc;
    if ((rc = upload(ctx, &D.colidx, col.data(), col.size()))) return rc;
    if ((rc = upload(ctx, &D.vals, soa.data(), soa.size()))) return rc;
    D.v.nbr = B.nbr; D.v.nbc = B.nbc; D.v.bs = B.bs; D.v.nnzb = slots; D.v.ld = ld; D.v.ell = W;
    D.v.rowptr = nullptr; D.v.colidx = D.colidx; D.v.vals = D.vals;
    D.v.lanes = W <= 4 ? 4 : (W <= 8 ? 8 : 16);
    return FHG_OK;
}

// The off-diagonal GS view slot-major per colour: slot s of row i of colour [c0, c1) at
// c0 * W + s * (c1 - c0) + (i - c0) (W = the most off-diagonal blocks of a row, 4..8), so that a
// sweep with one thread per row reads each slot of 32 consecutive rows as 32 consecutive words.
// Empty slots hold the row's own column and zero values, as in upload_padded. Built only when W
// is in 4..8 and the padding adds at most half; otherwise D stays empty.
template <class T>
int upload_offdiag_slot_major(fhg_ctx* ctx, const HostBsr& B, const std::vector<int>& colour_start,
                              DevBsr<T>& D)
{
    D = DevBsr<T>();
    int W = 0;
    long long kept = 0;
    for (int i = 0; i < B.nbr; i++) {
        int c = 0;
        for (int p = B.rowptr[i]; p < B.rowptr[i + 1]; p++) c += B.colidx[p] != i;
        W = std::max(W, c);
        kept += c;
    }
    const long long slots = (long long)B.nbr * W;
    if (W < 4 || W > 8 || slots > kept + kept / 2 || slots > INT32_MAX) return FHG_OK;
    if (colour_start.empty() || colour_start.back() != B.nbr) return FHG_OK;
    const int bb = B.bs * B.bs;
    const long long ld = round_up(slots, 32);
    std::vector<int> col((size_t)slots);
    std::vector<T> soa((size_t)ld * bb, T(0));
    for (size_t c = 0; c + 1 < colour_start.size(); c++) {
        const long long c0 = colour_start[c], nrc = colour_start[c + 1] - c0;
        for (long long i = c0; i < c0 + nrc; i++) {
            int k = 0;
            for (int p = B.rowptr[i]; p < B.rowptr[i + 1]; p++) {
                if (B.colidx[p] == i) continue;
                const long long q = c0 * W + k * nrc + (i - c0);
                col[(size_t)q] = B.colidx[p];
                for (int e = 0; e < bb; e++) soa[(size_t)e * ld + q] = (T)B.vals[(size_t)p * bb + e];
                k++;
            }
            for (; k < W; k++) col[(size_t)(c0 * W + k * nrc + (i - c0))] = (int)i;
        }
    }
    int rc;
    if ((rc = upload(ctx, &D.colidx, col.data(), col.size()))) return rc;
    if ((rc = upload(ctx, &D.vals, soa.data(), soa.size()))) return rc;
    D.v.nbr = B.nbr; D.v.nbc = B.nbc; D.v.bs = B.bs; D.v.nnzb = slots; D.v.ld = ld; D.v.ell = W;
    D.v.slot_major = 1;
    D.v.rowptr = nullptr; D.v.colidx = D.colidx; D.v.vals = D.vals;
    D.v.lanes = 1;
    return FHG_OK;
}

// All of a block operator slot-major, for products (one thread per row): slot k of row i at
// k * nbr + i (W = the most blocks of a row, 5..8), columns ascending; empty slots hold zero values
// and the row's last stored column (an exact zero added). Built only when W is in 5..8 and the
// padding adds at most half; otherwise D stays empty.
template <class T>
int upload_slot_major_all(fhg_ctx* ctx, const HostBsr& B, DevBsr<T>& D)
{
    D = DevBsr<T>();
    int W = 0;
    for (int i = 0; i < B.nbr; i++) W = std::max(W, B.rowptr[i + 1] - B.rowptr[i]);
    const long long kept = B.nnzb();
    const long long slots = (long long)B.nbr * W;
    if (W < 5 || W > 8 || slots > kept + kept / 2 || slots > INT32_MAX) return FHG_OK;
    const int bb = B.bs * B.bs;
    const long long ld = round_up(slots, 32);
    std::vector<int> col((size_t)slots);
    std::vector<T> soa((size_t)ld * bb, T(0));
    for (int i = 0; i < B.nbr; i++) {
        int k = 0, last = i;
        for (int p = B.rowptr[i]; p < B.rowptr[i + 1]; p++, k++) {
            const long long q = (long long)k * B.nbr + i;
            col[(size_t)q] = last = B.colidx[p];
            for (int e = 0; e < bb; e++) soa[(size_t)e * ld + q] = (T)B.vals[(size_t)p * bb + e];
        }
        for (; k < W; k++) col[(size_t)((long long)k * B.nbr + i)] = last;
    }
    int rc;
    if ((rc = upload(ctx, &D.colidx, col.data(), col.size()))) return rc;
    if ((rc = upload(ctx, &D.vals, soa.data(), soa.size()))) return rc;
    D.v.nbr = B.nbr; D.v.nbc = B.nbc; D.v.bs = B.bs; D.v.nnzb = slots; D.v.ld = ld; D.v.ell = W;
    D.v.slot_major = 1;
    D.v.rowptr = nullptr; D.v.colidx = D.colidx; D.v.vals = D.vals;
    D.v.lanes = 1;
    return FHG_OK;
}

// Jagged (JDS) view of a transfer operator: rows stably sorted by decreasing block count, slot s of
// sorted row k at start[s] + k, values entry-major with no padding. Not built above 64 blocks a row.
template <class T>
int upload_jds(fhg_ctx* ctx, const HostBsr& B, DevBsr<T>& D)
{
    D = DevBsr<T>();
    const int nbr = B.nbr;
    int W = 0;
    for (int i = 0; i < nbr; i++) W = std::max(W, B.rowptr[i + 1] - B.rowptr[i]);
    if (nbr == 0 || W == 0 || W > 64) return FHG_OK;
    std::vector<int> perm(nbr);
    for (int i = 0; i < nbr; i++) perm[i] = i;
    std::stable_sort(perm.begin(), perm.end(), [&](int a, int b) {
        return B.rowptr[a + 1] - B.rowptr[a] > B.rowptr[b + 1] - B.rowptr[b];
    });
    std::vector<int> start(W + 1, 0);
    for (int sl = 0; sl < W; sl++) {
        int rows = 0;
        while (rows < nbr && B.rowptr[perm[rows] + 1] - B.rowptr[perm[rows]] > sl) rows++;
        start[sl + 1] = start[sl] + rows;
    }
    const long long nnzb = B.nnzb();
    const int bb = B.bs * B.bs;
    const long long ld = round_up(std::max<long long>(nnzb, 1), 32);
    std::vector<int> col((size_t)nnzb);
    std::vector<T> soa((size_t)ld * bb, T(0));
    for (int sl = 0; sl < W; sl++)
        for (int k = 0; k < start[sl + 1] - start[sl]; k++) {
            const long long p = B.rowptr[perm[k]] + sl;
            const long long q = start[sl] + k;
            col[(size_t)q] = B.colidx[(size_t)p];
            for (int e = 0; e < bb; e++) soa[(size_t)e * ld + q] = (T)B.vals[(size_t)p * bb + e];
        }
    int rc;
    int *dperm = nullptr, *dstart = nullptr;
    if ((rc = upload(ctx, &dperm, perm.data(), perm.size())) || (rc = upload(ctx, &dstart, start.data(), start.size())) ||
        (rc = upload(ctx, &D.colidx, col.data(), col.size())) || (rc = upload(ctx, &D.vals, soa.data(), soa.size())))
        return rc;
    D.rowptr = dperm;   // owned with the view (freed with it): the permutation and the slot offsets
    D.v.nbr = B.nbr; D.v.nbc = B.nbc; D.v.bs = B.bs; D.v.nnzb = nnzb; D.v.ld = ld;
    D.v.rowptr = nullptr; D.v.colidx = D.colidx; D.v.vals = D.vals;
    D.v.jds_perm = dperm; D.v.jds_start = dstart; D.v.jds_slots = W;
    D.v.lanes = 1;
    D.jds_start = dstart;
    return FHG_OK;
}

// Outer operator as an FP32 pair: hi = fl32(a), lo = fl32(a - hi), entry-major like upload_bsr.
int upload_bsr_split(fhg_ctx* ctx, const HostBsr& B, DevBsr<float>& D, float** lo_out, const DevBsr<double>& share_index)
{
    const int bb = B.bs * B.bs;
    const long long nnzb = B.nnzb();
    const long long ld = round_up(std::max<long long>(nnzb, 1), 32);
    std::vector<float> hi((size_t)ld * bb, 0.f), lo((size_t)ld * bb, 0.f);
    for (long long p = 0; p < nnzb; p++)
        for (int e = 0; e < bb; e++) {
            const double v = B.vals[(size_t)p * bb + e];
            const float h = (float)v;
            hi[(size_t)e * ld + p] = h;
            lo[(size_t)e * ld + p] = (float)(v - (double)h);
        }
    int rc;
    D.rowptr = share_index.rowptr;
    D.colidx = share_index.colidx;
    D.owns_index = false;
    if ((rc = upload(ctx, &D.vals, hi.data(), hi.size()))) return rc;
    if ((rc = upload(ctx, lo_out, lo.data(), lo.size()))) return rc;
    D.v.nbr = B.nbr; D.v.nbc = B.nbc; D.v.bs = B.bs; D.v.nnzb = nnzb; D.v.ld = ld;
    D.v.rowptr = D.rowptr; D.v.colidx = D.colidx; D.v.vals = D.vals;
    D.v.lanes = share_index.v.lanes;
    return FHG_OK;
}

bool supported_bs(int bs) { return bs == 2 || bs == 3 || bs == 4 || bs == 6; }

// ---------------------------------------------------------------------------
// Learned-step setup (host)

// For every block row of the (permuted) finest operator: its off-diagonal block columns by
// decreasing |A_ij|_F^2 rounded to FP32 (so that couplings equal up to rounding order tie), ties
// by smaller column, the first six, -1 padded.
void learned_neighbours(const HostBsr& B, std::vector<int>& nbr)
{
    const int K = fhg::learned::kNeighbours;
    const int bb = B.bs * B.bs;
    nbr.assign((size_t)B.nbr * K, -1);
    std::vector<std::pair<float, int>> row;
    for (int i = 0; i < B.nbr; i++) {
        row.clear();
        for (int p = B.rowptr[i]; p < B.rowptr[i + 1]; p++) {
            const int j = B.colidx[p];
            if (j == i) continue;
            double f = 0.0;
            for (int e = 0; e < bb; e++) f += B.vals[(size_t)p * bb + e] * B.vals[(size_t)p * bb + e];
            row.push_back({(float)f, j});
        }
        std::sort(row.begin(), row.end(), [](const std::pair<float, int>& a, const std::pair<float, int>& b) {
            return a.first != b.first ? a.first > b.first : a.second < b.second;
        });
        for (int k = 0; k < K && k < (int)row.size(); k++) nbr[(size_t)i * K + k] = row[k].second;
    }
}

// float -> bfloat16 bits, round to nearest even (finite inputs).
uint16_t to_bf16(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}

// Element-tensor features of every face in colour numbering: both tensors divided by the larger
// of their Frobenius norms; zeros when no tensors were given.
int upload_tensor_features(fhg_ctx* ctx)
{
    Level& L = ctx->levels[0];
    if (!ctx->tfeat_d) return FHG_OK;
    const int S = fhg::learned::kTensorSlots;
    std::vector<uint16_t> f((size_t)L.nb * S, 0);
    if (ctx->tensors_host.size() == (size_t)L.nb * 12) {
        for (int I = 0; I < L.nb; I++) {
            const double* t = &ctx->tensors_host[(size_t)L.perm[I] * 12];
            double nrm[2] = {0, 0};
            for (int side = 0; side < 2; side++) {
                const double* T = t + 6 * side;
                nrm[side] = std::sqrt(T[0] * T[0] + T[1] * T[1] + T[2] * T[2] +
                                      2 * (T[3] * T[3] + T[4] * T[4] + T[5] * T[5]));
            }
            const double tau = std::max(nrm[0], nrm[1]);
            if (!(tau > 0) || !std::isfinite(tau)) continue;
            for (int q = 0; q < 12; q++) f[(size_t)I * S + q] = to_bf16((float)(t[q] / tau));
        }
    }
    CK(cudaMemcpy(ctx->tfeat_d, f.data(), f.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
    return FHG_OK;
}

// ---------------------------------------------------------------------------
// Device operations

template <class T> struct LevelVecs;
template <> struct LevelVecs<double> {
    static constexpr int kPrec = FHG_PREC_FP64;
    static double* x(Level& L) { return L.x; }
    static double* b(Level& L) { return L.b; }
    static double* r(Level& L) { return L.r; }
    static const BsrView<double>& A(Level& L) { return L.A.v; }
    static const BsrView<double>& P(Level& L) { return L.P.v; }
    static const BsrView<double>& R(Level& L) { return L.R.v; }
    static const BsrView<double>& Pcsr(Level& L) { return L.P.v; }
    static const BsrView<double>& Rcsr(Level& L) { return L.R.v; }
    static const double* dinv(Level& L) { return L.dinv; }
    static double* k(Level& L, int i) { return L.kv64[i]; }
    static const BsrView<double>& gs(Level& L) { return L.A.v; }
    static const BsrView<double>& Acsr(Level& L) { return L.A.v; }
};
template <> struct LevelVecs<float> {
    static constexpr int kPrec = FHG_PREC_FP32;
    static float* x(Level& L) { return L.x32; }
    static float* b(Level& L) { return L.b32; }
    static float* r(Level& L) { return L.r32; }
    // products with A: the slot-major or the row-major padded view when setup built one
    static const BsrView<float>& A(Level& L)
    {
        if (L.prod_slot[kPrec] && L.A32s.vals) return L.A32s.v;
        return L.A32p.vals ? L.A32p.v : L.A32.v;
    }
    // transfers: the jagged view when setup kept it, else CSR (padded rows of P cost what the saved
    // row-pointer load gains: its rows hold 1 to 7 blocks)
    static const BsrView<float>& P(Level& L) { return L.p_jds[kPrec] && L.P32j.vals ? L.P32j.v : L.P32.v; }
    static const BsrView<float>& R(Level& L) { return L.r_jds[kPrec] && L.R32j.vals ? L.R32j.v : L.R32.v; }
    static const BsrView<float>& Pcsr(Level& L) { return L.P32.v; }
    static const BsrView<float>& Rcsr(Level& L) { return L.R32.v; }
    static const float* dinv(Level& L) { return L.dinv32; }
    static float* k(Level& L, int i) { return L.kv32[i]; }
    // GS sweeps: the slot-major or padded off-diagonal view when setup built one
    static const BsrView<float>& gs(Level& L)
    {
        if (L.gs_slot[kPrec] && L.G32s.vals) return L.G32s.v;
        return L.G32.vals ? L.G32.v : L.A32.v;
    }
    static const BsrView<float>& Acsr(Level& L) { return L.A32.v; }   // Jacobi: row pointers
};
// FP32 pairs: the FP32 V-cycle's views with 8-byte pair values (FP64-class arithmetic on the FP32 pipe).
template <> struct LevelVecs<dfl> {
    static constexpr int kPrec = FHG_PREC_DF;
    static dfl* x(Level& L) { return L.x2; }
    static dfl* b(Level& L) { return L.b2; }
    static dfl* r(Level& L) { return L.r2; }
    static const BsrView<dfl>& A(Level& L)
    {
        if (L.prod_slot[kPrec] && L.A2s.vals) return L.A2s.v;
        return L.A2p.vals ? L.A2p.v : L.A2.v;
    }
    static const BsrView<dfl>& P(Level& L) { return L.p_jds[kPrec] && L.P2j.vals ? L.P2j.v : L.P2.v; }
    static const BsrView<dfl>& R(Level& L) { return L.r_jds[kPrec] && L.R2j.vals ? L.R2j.v : L.R2.v; }
    static const BsrView<dfl>& Pcsr(Level& L) { return L.P2.v; }
    static const BsrView<dfl>& Rcsr(Level& L) { return L.R2.v; }
    static const dfl* dinv(Level& L) { return L.dinv2; }
    static dfl* k(Level& L, int i) { return L.kv2[i]; }
    static const BsrView<dfl>& gs(Level& L)
    {
        if (L.gs_slot[kPrec] && L.G2s.vals) return L.G2s.v;
        return L.G2.vals ? L.G2.v : L.A2.v;
    }
    static const BsrView<dfl>& Acsr(Level& L) { return L.A2.v; }
};

// `from_zero`: x holds zeros on entry (the pre-smoothing of a V-cycle), so the first GS sweep
// skips the blocks that multiply not-yet-updated entries.
template <class T>
void smooth(fhg_ctx* ctx, int l, int code, int iters, const T* b, T* x, bool from_zero = false)
{
    Level& L = ctx->levels[l];
    using V = LevelVecs<T>;
    cudaStream_t s = ctx->stream;
    constexpr int P = V::kPrec;
    BsrView<T> Ag = V::gs(L);   // GS sweeps (tuned shape)
    if (L.gs_lanes[P]) { Ag.lanes = L.gs_lanes[P]; Ag.unroll = L.gs_unroll[P]; }
    BsrView<T> A = V::Acsr(L);  // Jacobi (row pointers and the diagonal blocks)
    if (L.gs_lanes[P] && Ag.ell == 0) { A.lanes = L.gs_lanes[P]; A.unroll = L.gs_unroll[P]; }
    // Multigrid::RelaxationParameter: the GS codes become block SOR when it is not 1
    // (SmootherFactory.h:37-100, BlockSOR.h:199-227).
    const T w = T(ctx->opts.omega);
    auto forward = [&](bool zero) {
        for (int c = 0; c < L.ncolours; c++)
            fhg::launch_gs<T>(Ag, L.colour_start[c], L.colour_start[c + 1], V::dinv(L), L.nb, b, x, s, 0,
                              zero ? L.colour_start[c + 1] : 0x7fffffff, w);
    };
    auto backward = [&](bool zero) {
        for (int c = L.ncolours - 1; c >= 0; c--)
            fhg::launch_gs<T>(Ag, L.colour_start[c], L.colour_start[c + 1], V::dinv(L), L.nb, b, x, s,
                              zero ? L.colour_start[c] : 0, 0x7fffffff, w);
    };
    for (int it = 0; it < iters; it++) {
        const bool zero = from_zero && it == 0;
        // BlockGaussSeidel directions (src/Solver/FixedPoint/BlockGaussSeidel.h:84-120); the
        // alternating ones switch by iteration parity, IterationCount restarting at every smoothing.
        if (code == FHG_SMOOTHER_BGS) {
            forward(zero);
        } else if (code == FHG_SMOOTHER_RBGS) {
            backward(zero);
        } else if (code == FHG_SMOOTHER_SBGS) {
            forward(zero);
            backward(false);
        } else if (code == FHG_SMOOTHER_ABGS) {
            if (it % 2 == 0) forward(zero); else backward(false);
        } else if (code == FHG_SMOOTHER_RABGS) {
            if (it % 2 == 0) backward(zero); else forward(false);
        } else {
            const T omega = code == FHG_SMOOTHER_BJ23 ? T(2.0 / 3.0) : T(ctx->opts.omega);
            T* tmp = V::r(L);
            fhg::launch_jacobi<T>(A, V::dinv(L), L.nb, omega, b, x, tmp, s);
            cudaMemcpyAsync(x, tmp, sizeof(T) * (size_t)L.n, cudaMemcpyDeviceToDevice, s);
        }
    }
}

bool is_gs(int code) { return code != FHG_SMOOTHER_BJ && code != FHG_SMOOTHER_BJ23; }

// Learned correction at the end of the finest level's post-smoothing: w = D^-1 (b - A x) in one
// pass, then x += s N(w-patch, tensors) face by face (fhg_learned.cu).
void learned_step(fhg_ctx* ctx, const float* b, float* x)
{
    Level& L = ctx->levels[0];
    cudaStream_t s = ctx->stream;
    fhg::launch_residual_dinv(LevelVecs<float>::A(L), L.dinv32, L.nb, x, b, ctx->lw, s);
    fhg::launch_learned_apply(L.nb, L.bs, ctx->nbr_d, ctx->lw, ctx->tfeat_d, ctx->lwts, ctx->lbias, x, ctx->lstatus,
                              ctx->learned_kernel, s);
}

template <class T>
void mg_cycle(fhg_ctx* ctx, int l, const T* b, T* x, bool x_zero);

// Dot products a_q . b_q (q < nq) on the device, summed on the host in a fixed order (one
// read-back: the K-cycle's branch is decided on the host).
template <class T>
void host_dots(fhg_ctx* ctx, long long n, int nq, const T* a0, const T* b0, const T* a1, const T* b1, const T* a2,
               const T* b2, double* out)
{
    double* p = ctx->partials + (size_t)5 * fhg::kReduceCtas;  // parts 5-7: free inside a cycle
    fhg::launch_dots3<T>(n, nq, a0, b0, a1, b1, a2, b2, p, ctx->stream);
    std::vector<double> h((size_t)3 * fhg::kReduceCtas);
    cudaMemcpyAsync(h.data(), p, sizeof(double) * nq * fhg::kReduceCtas, cudaMemcpyDeviceToHost, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    for (int q = 0; q < nq; q++) {
        double t = 0.0;
        for (int i = 0; i < fhg::kReduceCtas; i++) t += h[(size_t)q * fhg::kReduceCtas + i];
        out[q] = t;
    }
}

// Multigrid::FCGForKCycle (src/Solver/Multigrid/Multigrid.h:611-656): x = the coarse correction
// on level m from two FCG steps preconditioned by the cycle on level m, the second only when the
// first reduced ||r|| by less than t = 0.25. r is overwritten (r -= (alpha1 / rho1) A c).
template <class T>
void kcycle_fcg(fhg_ctx* ctx, int m, T* r, T* x)
{
    Level& L = ctx->levels[m];
    using V = LevelVecs<T>;
    cudaStream_t s = ctx->stream;
    const long long n = L.n;
    T *c = V::k(L, 0), *v = V::k(L, 1), *d = V::k(L, 2), *w = V::k(L, 3);
    mg_cycle<T>(ctx, m, r, c, true);
    fhg::launch_spmv<T>(V::A(L), fhg::kSpmvAssign, c, nullptr, v, s);
    double q[3];
    host_dots<T>(ctx, n, 3, c, v, c, r, r, r, q);
    const double rho1 = q[0], alpha1 = q[1], norm_old = std::sqrt(q[2]);
    fhg::launch_axpy<T>(n, -(alpha1 / rho1), v, r, s);
    host_dots<T>(ctx, n, 1, r, r, (const T*)nullptr, (const T*)nullptr, (const T*)nullptr, (const T*)nullptr, q);
    const double norm_new = std::sqrt(q[0]);
    if (norm_new <= 0.25 * norm_old) {
        fhg::launch_lincomb<T>(n, alpha1 / rho1, c, 0.0, c, x, s);
        return;
    }
    mg_cycle<T>(ctx, m, r, d, true);
    fhg::launch_spmv<T>(V::A(L), fhg::kSpmvAssign, d, nullptr, w, s);
    host_dots<T>(ctx, n, 3, d, v, d, w, d, r, q);
    const double gamma = q[0], beta = q[1], alpha2 = q[2];
    const double rho2 = beta - gamma * gamma / rho1;
    fhg::launch_lincomb<T>(n, alpha1 / rho1 - gamma * alpha2 / (rho1 * rho2), c, alpha2 / rho2, d, x, s);
}

// Lanes of the fused kernel per block row of an operator: enough for the average row's blocks to be
// loaded together, a power of two from 4 to 16.
template <class T>
int fused_lanes(const BsrView<T>& B)
{
    const double avg = B.nbr ? (double)B.nnzb / B.nbr : 1.0;
    return avg <= 5.0 ? 4 : avg <= 12.0 ? 8 : 16;
}

// The coarse sub-cycle from level l down as one cluster launch (fhg_coarse.cu), when setup found the
// levels small enough and the cycle is one it covers: GS / SOR smoothers, V or W cycle, FP32 or pair
// values. Returns false when the caller must run the sub-cycle launch by launch.
template <class T>
bool fused_cycle(fhg_ctx* ctx, int l, const T* b, T* x, bool x_zero)
{
    if constexpr (std::is_same<T, double>::value) {
        return false;
    } else {
        using V = LevelVecs<T>;
        const fhg_options& o = ctx->opts;
        if (!o.fused_coarse || l != ctx->fused_from[V::kPrec] || l <= 0 || o.w_loops == FHG_CYCLE_K ||
            !is_gs(o.pre_smoother) || !is_gs(o.post_smoother))
            return false;
        Level& L0 = ctx->levels[l];
        if (b != V::b(L0) || x != V::x(L0)) return false;
        auto dir = [](int code) {
            switch (code) {
            case FHG_SMOOTHER_BGS: return fhg::kFusedForward;
            case FHG_SMOOTHER_RBGS: return fhg::kFusedBackward;
            case FHG_SMOOTHER_SBGS: return fhg::kFusedSymmetric;
            case FHG_SMOOTHER_ABGS: return fhg::kFusedAlternatingForward;
            default: return fhg::kFusedAlternatingBackward;
            }
        };
        fhg::FusedCycle<T> P;
        P.nlev = ctx->nlevels - l;
        P.pre = dir(o.pre_smoother);
        P.post = dir(o.post_smoother);
        P.npre = o.coarse_pre_iterations >= 0 ? o.coarse_pre_iterations : o.pre_iterations;
        P.npost = o.coarse_post_iterations >= 0 ? o.coarse_post_iterations : o.post_iterations;
        P.w_loops = o.w_loops > 1 ? o.w_loops : 1;
        P.x_zero = x_zero ? 1 : 0;
        P.omega = T(o.omega);
        for (int k = 0; k < P.nlev; k++) {
            Level& L = ctx->levels[l + k];
            fhg::FusedLevel<T>& F = P.lev[k];
            F.nb = L.nb;
            F.x = V::x(L);
            F.b = V::b(L);
            F.r = V::r(L);
            if (l + k == ctx->nlevels - 1) {
                P.n_coarse = L.n;
                P.cinv = L.cinv;
                continue;
            }
            F.ncol = L.ncolours;
            for (int c = 0; c <= L.ncolours; c++) F.colour_start[c] = L.colour_start[c];
            const BsrView<T>& A = V::Acsr(L);
            F.a_rowptr = A.rowptr; F.a_colidx = A.colidx; F.a_vals = A.vals; F.a_ld = A.ld;
            F.dinv = V::dinv(L);
            const BsrView<T>& Pv = V::Pcsr(L);
            F.p_rowptr = Pv.rowptr; F.p_colidx = Pv.colidx; F.p_vals = Pv.vals; F.p_ld = Pv.ld;
            const BsrView<T>& Rv = V::Rcsr(L);
            F.r_rowptr = Rv.rowptr; F.r_colidx = Rv.colidx; F.r_vals = Rv.vals; F.r_ld = Rv.ld;
            F.lanes = fused_lanes(A);
            F.t_lanes = fused_lanes(Rv);
            const BsrView<T>* G = nullptr;
            const BsrView<T>* Ap = nullptr;
            if constexpr (std::is_same<T, float>::value) {
                if (L.G32.vals) G = &L.G32.v;
                if (L.A32p.vals) Ap = &L.A32p.v;
            } else {
                if (L.G2.vals) G = &L.G2.v;
                if (L.A2p.vals) Ap = &L.A2p.v;
            }
            if (G && G->ell > 0 && G->ell <= F.lanes) {
                F.g_ell = G->ell; F.g_colidx = G->colidx; F.g_vals = G->vals; F.g_ld = G->ld;
            }
            if (Ap && Ap->ell > 0 && Ap->ell <= F.lanes) {
                F.ap_ell = Ap->ell; F.ap_colidx = Ap->colidx; F.ap_vals = Ap->vals; F.ap_ld = Ap->ld;
            }
        }
        if (fhg::launch_fused_cycle<T>(P, L0.bs, ctx->fused_ctas[V::kPrec], ctx->fused_threads[V::kPrec], ctx->stream) !=
            cudaSuccess)
            return false;
        fhg::g_kernel_launches++;
        return true;
    }
}

// First level (>= 1, above the coarsest) from which every level has at most max_rows block rows and
// at most kFusedMaxColours colours, within kFusedMaxLevels levels, all of one block size and joined by
// products with P (no natural injection); -1 when there is none.
int fused_first_level(const fhg_ctx* ctx, int max_rows)
{
    const int nlevels = ctx->nlevels;
    for (int l = 1; l + 1 < nlevels; l++) {
        bool ok = nlevels - l <= fhg::kFusedMaxLevels;
        for (int k = l; k < nlevels && ok; k++)
            ok = ctx->levels[k].nb <= max_rows && ctx->levels[k].bs == ctx->levels[l].bs &&
                 (k == nlevels - 1 || (ctx->levels[k].ncolours <= fhg::kFusedMaxColours && !ctx->levels[k].inject));
        if (ok) return l;
    }
    return -1;
}

// Timing-based choice of the coarse sub-cycle, kept per hierarchy structure and cycle in the process
// (the same sizes, colours, block counts, smoothers and counts give the same choice).
struct FusedKey {
    std::vector<long long> sig;
    bool operator<(const FusedKey& o) const { return sig < o.sig; }
};
struct FusedChoice {
    int from = -1, ctas = fhg::kClusterCtasPortable, threads = fhg::kFusedThreads;
};
std::mutex g_fused_mutex;
std::map<FusedKey, FusedChoice> g_fused_cache;

template <class T>
void mg_cycle(fhg_ctx* ctx, int l, const T* b, T* x, bool x_zero);

// Time one cycle below level 0 (from level 1, x = 0) for launch by launch and for every eligible first
// level of the fused sub-cycle with 8 and 16 CTAs of 512 and 1024 threads; keep the fastest (ties: the
// earlier candidate).
template <class T>
int choose_fused(fhg_ctx* ctx)
{
    using V = LevelVecs<T>;
    constexpr int PR = V::kPrec;
    const fhg_options& o = ctx->opts;
    const int nlevels = ctx->nlevels;
    const int first = fused_first_level(ctx, fhg::kFusedMaxRows);
    ctx->fused_from[PR] = -1;
    ctx->fused_ctas[PR] = fhg::kClusterCtasPortable;
    ctx->fused_threads[PR] = fhg::kFusedThreads;
    if (first < 0) return FHG_OK;
    const int bs = ctx->levels[first].bs;   // every candidate level's (fused_first_level)
    FusedKey key;
    key.sig = {PR, ctx->levels[0].bs, bs, nlevels, o.pre_smoother, o.post_smoother, o.pre_iterations, o.post_iterations,
               o.coarse_pre_iterations, o.coarse_post_iterations, o.w_loops, o.omega == 1.0 ? 1 : 0};
    for (int l = 1; l < nlevels; l++) {
        const Level& L = ctx->levels[l];
        key.sig.push_back(L.nb);
        key.sig.push_back(L.bs);
        key.sig.push_back(L.ncolours);
        key.sig.push_back(V::Acsr(const_cast<Level&>(L)).nnzb);
    }
    {
        std::lock_guard<std::mutex> lock(g_fused_mutex);
        auto it = g_fused_cache.find(key);
        if (it != g_fused_cache.end()) {
            ctx->fused_from[PR] = it->second.from;
            ctx->fused_ctas[PR] = it->second.ctas;
            ctx->fused_threads[PR] = it->second.threads;
            return FHG_OK;
        }
    }
    Level& L1 = ctx->levels[1];
    cudaStream_t s = ctx->stream;
    CK(cudaMemsetAsync(V::b(L1), 0, sizeof(T) * (size_t)L1.n, s));
    auto time_cycle = [&](double* ms) -> int {
        for (int w = 0; w < 2; w++) mg_cycle<T>(ctx, 1, V::b(L1), V::x(L1), true);
        const int reps = 5;
        CK(cudaEventRecord(ctx->ev0, s));
        for (int r = 0; r < reps; r++) mg_cycle<T>(ctx, 1, V::b(L1), V::x(L1), true);
        CK(cudaEventRecord(ctx->ev1, s));
        CK(cudaEventSynchronize(ctx->ev1));
        float t = 0;
        CK(cudaEventElapsedTime(&t, ctx->ev0, ctx->ev1));
        *ms = t / reps;
        return FHG_OK;
    };
    double best = 0.0;
    int rc = time_cycle(&best);
    if (rc) return rc;
    FusedChoice choice;
    for (int threads : {fhg::kFusedThreads, fhg::kFusedThreadsWide}) {
        for (int ctas : {fhg::kClusterCtasPortable, fhg::kClusterCtasLarge}) {
            if (fhg::fused_cycle_clusters<T>(bs, ctas, threads) < 1) continue;
            for (int l = first; l + 1 < nlevels; l++) {
                ctx->fused_from[PR] = l;
                ctx->fused_ctas[PR] = ctas;
                ctx->fused_threads[PR] = threads;
                double ms = 0.0;
                if ((rc = time_cycle(&ms))) break;
                if (ms < best) {
                    best = ms;
                    choice = {l, ctas, threads};
                }
            }
            if (rc) break;
        }
        if (rc) break;
    }
    ctx->fused_from[PR] = choice.from;
    ctx->fused_ctas[PR] = choice.ctas;
    ctx->fused_threads[PR] = choice.threads;
    if (rc) return rc;
    std::lock_guard<std::mutex> lock(g_fused_mutex);
    g_fused_cache[key] = choice;
    return FHG_OK;
}

// Views the launch choices do not use, freed once setup has made them (each precision keeps the GS
// view and the product view its sweeps and products run on, level 0 the outer operator's chosen
// pair view): at 64^3 the padded and slot-major copies each take about the size of the FP32 operator.
template <class T>
void release_bsr(fhg_ctx* ctx, DevBsr<T>& D)
{
    dfree(ctx, D.vals);
    if (D.owns_index) {
        dfree(ctx, D.rowptr);
        dfree(ctx, D.colidx);
        dfree(ctx, D.jds_start);
    }
    D = DevBsr<T>();
}

void release_unused_views(fhg_ctx* ctx)
{
    for (int l = 0; l + 1 < ctx->nlevels; l++) {
        Level& L = ctx->levels[l];
        // levels >= 1 keep their padded-row views: the one-launch coarse sub-cycle reads them
        const bool keep_padded = l > 0;
        if (L.G32s.vals && L.gs_slot[FHG_PREC_FP32]) { if (!keep_padded) release_bsr(ctx, L.G32); }
        else if (L.G32s.vals) release_bsr(ctx, L.G32s);
        if (L.A32s.vals && L.prod_slot[FHG_PREC_FP32]) { if (!keep_padded) release_bsr(ctx, L.A32p); }
        else if (L.A32s.vals) release_bsr(ctx, L.A32s);
        if (L.G2s.vals && L.gs_slot[FHG_PREC_DF]) { if (!keep_padded) release_bsr(ctx, L.G2); }
        else if (L.G2s.vals) release_bsr(ctx, L.G2s);
        if (L.A2s.vals && L.prod_slot[FHG_PREC_DF]) { if (!keep_padded) release_bsr(ctx, L.A2p); }
        else if (L.A2s.vals) release_bsr(ctx, L.A2s);
        if (L.P32j.vals && !L.p_jds[FHG_PREC_FP32]) release_bsr(ctx, L.P32j);
        if (L.R32j.vals && !L.r_jds[FHG_PREC_FP32]) release_bsr(ctx, L.R32j);
        if (L.P2j.vals && !L.p_jds[FHG_PREC_DF]) release_bsr(ctx, L.P2j);
        if (L.R2j.vals && !L.r_jds[FHG_PREC_DF]) release_bsr(ctx, L.R2j);
    }
    Level& L0 = ctx->levels[0];
    if (L0.Ahat2s.vals && L0.outer_slot && L0.ahat_lo) {
        dfree(ctx, L0.Ahat_hi.vals);
        dfree(ctx, L0.ahat_lo);
        L0.Ahat_hi = DevBsr<float>();
        L0.ahat_lo = nullptr;
    } else if (L0.Ahat2s.vals && !L0.outer_slot) {
        release_bsr(ctx, L0.Ahat2s);
    }
}

// Timing at setup (launch shapes, the coarse sub-cycle) runs one context at a time, so contexts set up
// on several host threads do their host work concurrently without disturbing each other's timings.
std::recursive_mutex g_timing_mutex;

// The coarse sub-cycle of every V-cycle precision the context holds: off, by timing (autotuning), or
// from the first level of at most kFusedDefaultRows block rows with 8 CTAs. Called at setup and when
// the cycle changes.
int refresh_fused(fhg_ctx* ctx)
{
    std::lock_guard<std::recursive_mutex> timing(g_timing_mutex);
    const fhg_options& o = ctx->opts;
    const bool fp32 = ctx->levels[0].A32.vals != nullptr, pair = ctx->levels[0].A2.vals != nullptr;
    for (int p = 0; p < 3; p++) {
        ctx->fused_from[p] = -1;
        ctx->fused_ctas[p] = fhg::kClusterCtasPortable;
        ctx->fused_threads[p] = fhg::kFusedThreads;
    }
    if (!o.fused_coarse || o.w_loops == FHG_CYCLE_K || !is_gs(o.pre_smoother) || !is_gs(o.post_smoother))
        return FHG_OK;
    int rc = FHG_OK;
    if (o.autotune) {
        if (fp32 && (rc = choose_fused<float>(ctx))) return rc;
        if (pair && (rc = choose_fused<dfl>(ctx))) return rc;
        return cudaStreamSynchronize(ctx->stream) == cudaSuccess ? FHG_OK
                                                                 : fail(ctx, FHG_ERR_CUDA, "coarse sub-cycle timing failed");
    }
    const int first = fused_first_level(ctx, fhg::kFusedDefaultRows);
    if (first < 0) return FHG_OK;
    const int bs = ctx->levels[first].bs;
    const int threads = o.fused_coarse == 2 ? fhg::kFusedThreadsWide : fhg::kFusedThreads;
    if (fp32 && fhg::fused_cycle_clusters<float>(bs, fhg::kClusterCtasPortable, threads) >= 1) {
        ctx->fused_from[FHG_PREC_FP32] = first;
        ctx->fused_threads[FHG_PREC_FP32] = threads;
    }
    if (pair && fhg::fused_cycle_clusters<dfl>(bs, fhg::kClusterCtasPortable, threads) >= 1) {
        ctx->fused_from[FHG_PREC_DF] = first;
        ctx->fused_threads[FHG_PREC_DF] = threads;
    }
    return FHG_OK;
}

// b_{l+1} = R_l r (Multigrid.h:494): the product with R_l, or the natural injection's restriction.
template <class T>
void restrict_to(fhg_ctx* ctx, int l, const T* r, T* bc)
{
    Level& L = ctx->levels[l];
    if (L.inject)
        fhg::launch_inject<T>(L.nb, L.bs, ctx->levels[l + 1].bs, L.inj_map, r, nullptr, bc, false, ctx->stream);
    else
        fhg::launch_spmv<T>(LevelVecs<T>::R(L), fhg::kSpmvAssign, r, nullptr, bc, ctx->stream);
}

// out = aux + P_l e (Multigrid.h:554), aux NULL reading as zero.
template <class T>
void prolong_add(fhg_ctx* ctx, int l, const T* e, const T* aux, T* out)
{
    Level& L = ctx->levels[l];
    if (L.inject)
        fhg::launch_inject<T>(L.nb, L.bs, ctx->levels[l + 1].bs, L.inj_map, e, aux, out, true, ctx->stream);
    else
        fhg::launch_spmv<T>(LevelVecs<T>::P(L), aux ? fhg::kSpmvAddTo : fhg::kSpmvAssign, e, aux, out, ctx->stream);
}

// One multigrid cycle on level l (src/Solver/Multigrid/Multigrid.h:438-608): V for w_loops = 1,
// W for 2 (the coarse correction repeated, except directly above the coarsest level), K for
// FHG_CYCLE_K (kcycle_fcg on the coarser level unless that is the coarsest). x is the initial
// guess, zero when x_zero.
template <class T>
void mg_cycle(fhg_ctx* ctx, int l, const T* b, T* x, bool x_zero)
{
    Level& L = ctx->levels[l];
    using V = LevelVecs<T>;
    cudaStream_t s = ctx->stream;
    if (l == ctx->nlevels - 1) {
        fhg::launch_coarse<T>(L.n, L.cinv, b, x, s);
        return;
    }
    if (fused_cycle<T>(ctx, l, b, x, x_zero)) return;
    Level& C = ctx->levels[l + 1];
    // Smoothing steps of this level: the coarse counts apply on levels >= 1 when set.
    const int npre = l > 0 && ctx->opts.coarse_pre_iterations >= 0 ? ctx->opts.coarse_pre_iterations
                                                                    : ctx->opts.pre_iterations;
    const int npost = l > 0 && ctx->opts.coarse_post_iterations >= 0 ? ctx->opts.coarse_post_iterations
                                                                      : ctx->opts.post_iterations;
    // A zero-start GS sweep writes every entry before any is read: no clearing needed then (block
    // SOR reads the old value of the entry it writes, so it starts from cleared x).
    const int pre = ctx->opts.pre_smoother;
    const bool gs_zero = x_zero && is_gs(pre) && npre > 0 && ctx->opts.omega == 1.0;
    if (x_zero && !gs_zero) cudaMemsetAsync(x, 0, sizeof(T) * (size_t)L.n, s);
    smooth<T>(ctx, l, pre, npre, b, x, gs_zero);
    fhg::launch_spmv<T>(V::A(L), fhg::kSpmvResidual, x, b, V::r(L), s);
    restrict_to<T>(ctx, l, V::r(L), V::b(C));
    if (ctx->opts.w_loops == FHG_CYCLE_K && l + 1 < ctx->nlevels - 1) {
        kcycle_fcg<T>(ctx, l + 1, V::b(C), V::x(C));
    } else {
        const int loops = ctx->opts.w_loops > 1 ? ctx->opts.w_loops : 1;
        for (int w = 0; w < loops; w++) {
            mg_cycle<T>(ctx, l + 1, V::b(C), V::x(C), w == 0);
            if (l + 1 == ctx->nlevels - 1) break;
        }
    }
    prolong_add<T>(ctx, l, V::x(C), x, x);
    smooth<T>(ctx, l, ctx->opts.post_smoother, npost, b, x);
    if constexpr (std::is_same<T, float>::value) {
        if (l == 0 && ctx->learned_now) learned_step(ctx, b, x);
    }
}

template <class T>
void vcycle(fhg_ctx* ctx, int l, const T* b, T* x) { mg_cycle<T>(ctx, l, b, x, true); }

// z = M r in the configured precision (level-0 numbering, FP64 in/out).
void precondition(fhg_ctx* ctx, const double* r, double* z)
{
    Level& L = ctx->levels[0];
    if (ctx->opts.vcycle_precision == FHG_PREC_FP32) {
        fhg::launch_convert<double, float>(L.n, r, L.b32, ctx->stream);
        vcycle<float>(ctx, 0, L.b32, L.x32);
        fhg::launch_convert<float, double>(L.n, L.x32, z, ctx->stream);
    } else if (ctx->opts.vcycle_precision == FHG_PREC_DF) {
        fhg::launch_convert<double, dfl>(L.n, r, L.b2, ctx->stream);
        vcycle<dfl>(ctx, 0, L.b2, L.x2);
        fhg::launch_convert<dfl, double>(L.n, L.x2, z, ctx->stream);
    } else {
        vcycle<double>(ctx, 0, r, z);
    }
}

double* part(fhg_ctx* ctx, int i) { return ctx->partials + (size_t)i * fhg::kReduceCtas; }

// Ad = Â d in pair arithmetic with the partials of d.Ad and r.d: on the slot-major pair view when
// setup built one and the autotuner kept it, else on the row-major split view.
void outer_product_df(fhg_ctx* ctx, const float* dh, const float* dl, const float* rh, const float* rl, float* Adh,
                      float* Adl, double* partials)
{
    Level& L0 = ctx->levels[0];
    if (L0.Ahat2s.vals && (L0.outer_slot || !L0.ahat_lo))
        fhg::launch_spmv_dots_df_slot(L0.Ahat2s.v, dh, dl, rh, rl, Adh, Adl, partials, ctx->stream);
    else
        fhg::launch_spmv_dots_df(L0.Ahat_hi.v, L0.ahat_lo, dh, dl, rh, rl, Adh, Adl, partials, ctx->stream);
}

// The outer iteration runs on FP32 pairs (double-FP32 outer product built at setup): with the FP32
// V-cycle, and with the pair V-cycle.
bool outer_df(const fhg_ctx* ctx)
{
    const int p = ctx->opts.vcycle_precision;
    return (p == FHG_PREC_FP32 || (p == FHG_PREC_DF && ctx->rhi)) && ctx->opts.krylov == FHG_KRYLOV_FCG &&
           (ctx->levels[0].ahat_lo || ctx->levels[0].Ahat2s.vals) && ctx->rlo;
}

// High part of the outer residual pair: the FP32 V-cycle reads it as its right-hand side.
float* outer_rh(fhg_ctx* ctx)
{
    return ctx->opts.vcycle_precision == FHG_PREC_DF ? ctx->rhi : ctx->levels[0].b32;
}

// The pair V-cycle's right-hand side (interleaved pairs of r), written with the outer residual.
dfl* outer_r2(fhg_ctx* ctx)
{
    return ctx->opts.vcycle_precision == FHG_PREC_DF ? ctx->levels[0].b2 : nullptr;
}

// FP32 pair views of an n-long FP64 buffer (hi: first n floats, lo: next n).
float* pair_hi(double* v) { return reinterpret_cast<float*>(v); }
float* pair_lo(double* v, long long n) { return reinterpret_cast<float*>(v) + n; }

// Start of a double-FP32 outer iteration: (rh, rlo) = r, and r as pairs for a pair V-cycle.
void outer_df_start(fhg_ctx* ctx, const double* r)
{
    fhg::launch_split_df(ctx->levels[0].n, r, outer_rh(ctx), ctx->rlo, ctx->stream, outer_r2(ctx));
}

// One FCG(1) iteration (src/Solver/Krylov/FlexibleConjugateGradient.h:80-162), parity p
// selects the ping-pong buffers (z/d, Ad) of this iteration.
void fcg_iteration(fhg_ctx* ctx, int p)
{
    const long long n = ctx->levels[0].n;
    cudaStream_t s = ctx->stream;
    double* z = ctx->kz[p];
    double* dp = ctx->kz[1 - p];
    double* Ad = ctx->kAd[p];
    double* Adp = ctx->kAd[1 - p];
    Level& L0 = ctx->levels[0];
    const bool fp32 = ctx->opts.vcycle_precision == FHG_PREC_FP32;
    if (outer_df(ctx)) {
        // FP32 pairs for r, d, Ad: z = M r (FP32 V-cycle on r_hi, or the pair V-cycle on r),
        // d = z - s dp, Ad = Â d, r -= alpha Ad with no FP64 instruction per element; x += alpha d in FP64.
        const bool pv = ctx->opts.vcycle_precision == FHG_PREC_DF;
        float* rh = outer_rh(ctx);
        const float* z32 = nullptr;
        const dfl* z2 = nullptr;
        if (pv) {
            vcycle<dfl>(ctx, 0, L0.b2, L0.x2);
            z2 = L0.x2;
        } else {
            vcycle<float>(ctx, 0, L0.b32, L0.x32);
            z32 = L0.x32;
        }
        float *dh = pair_hi(z), *dl = pair_lo(z, n), *Adh = pair_hi(Ad), *Adl = pair_lo(Ad, n);
        fhg::launch_dot_df(n, z32, pair_hi(Adp), pair_lo(Adp, n), part(ctx, 0), s, z2);
        fhg::launch_fcg_direction_df(n, z32, pair_hi(dp), pair_lo(dp, n), part(ctx, 0), ctx->scal + 1, dh, dl, s, z2);
        outer_product_df(ctx, dh, dl, rh, ctx->rlo, Adh, Adl, part(ctx, 1));
        fhg::launch_krylov_step_df(n, ctx->kx, rh, ctx->rlo, dh, dl, Adh, Adl, part(ctx, 2), part(ctx, 1),
                                   ctx->scal + 1, part(ctx, 3), s, outer_r2(ctx));
        fhg::launch_finalize_norm(part(ctx, 3), ctx->scal + 0, ctx->scal + 2, ctx->hist_d, ctx->counter_d,
                                  ctx->opts.max_iterations + 1, s);
        if (!ctx->device_loop) cudaMemcpyAsync(ctx->nr_host, ctx->scal + 2, sizeof(double), cudaMemcpyDeviceToHost, s);
        return;
    }
    if (fp32) {
        // V-cycle on the FP32 copy of r written by the previous step; z stays FP32 and is
        // widened inside the direction update.
        vcycle<float>(ctx, 0, L0.b32, L0.x32);
        fhg::launch_dot_mixed(n, L0.x32, Adp, part(ctx, 0), s);
        fhg::launch_fcg_direction_mixed(n, L0.x32, dp, part(ctx, 0), ctx->scal + 1, z, s);
    } else {
        precondition(ctx, ctx->kr, z);
        fhg::launch_dot(n, z, Adp, part(ctx, 0), s);
        fhg::launch_fcg_direction(n, z, dp, part(ctx, 0), ctx->scal + 1, z, s);
    }
    {
        BsrView<double> Ah = L0.ahat_is_a ? L0.A.v : L0.Ahat.v;
        if (L0.outer_lanes) Ah.lanes = L0.outer_lanes;
        fhg::launch_spmv_dots(Ah, z, ctx->kr, Ad, part(ctx, 1), s);
    }
    // parts 1 = d.Ad, 2 = r.d
    fhg::launch_krylov_step(n, ctx->kx, ctx->kr, z, Ad, part(ctx, 2), part(ctx, 1), ctx->scal + 1, part(ctx, 3), s,
                            fp32 ? L0.b32 : nullptr);
    fhg::launch_finalize_norm(part(ctx, 3), ctx->scal + 0, ctx->scal + 2, ctx->hist_d, ctx->counter_d,
                              ctx->opts.max_iterations + 1, s);
    if (!ctx->device_loop) cudaMemcpyAsync(ctx->nr_host, ctx->scal + 2, sizeof(double), cudaMemcpyDeviceToHost, s);
}

// One PCG iteration (src/Solver/Krylov/ConjugateGradient.h:58-96); z, d, Ad = kz[0], kz[1], kAd[0].
void cg_iteration(fhg_ctx* ctx)
{
    const long long n = ctx->levels[0].n;
    cudaStream_t s = ctx->stream;
    double* z = ctx->kz[0];
    double* d = ctx->kz[1];
    double* Ad = ctx->kAd[0];
    fhg::launch_cg_direction(n, z, ctx->scal + 4, d, s);
    fhg::launch_spmv_dots(ctx->levels[0].A.v, d, ctx->kr, Ad, part(ctx, 1), s);
    fhg::launch_cg_step(n, ctx->kx, ctx->kr, d, Ad, ctx->scal + 3, part(ctx, 1), part(ctx, 3), s);
    precondition(ctx, ctx->kr, z);
    fhg::launch_dot(n, ctx->kr, z, part(ctx, 0), s);
    fhg::launch_cg_beta(part(ctx, 0), ctx->scal + 3, ctx->scal + 4, s);
    fhg::launch_finalize_norm(part(ctx, 3), ctx->scal + 0, ctx->scal + 2, ctx->hist_d, ctx->counter_d,
                              ctx->opts.max_iterations + 1, s);
    cudaMemcpyAsync(ctx->nr_host, ctx->scal + 2, sizeof(double), cudaMemcpyDeviceToHost, s);
}

// One captured Krylov iteration per ping-pong parity; `learned`: the V-cycle of the captured
// iteration applies the learned correction (graph_l) or not (graph).
int build_graphs(fhg_ctx* ctx, bool learned = false)
{
    const int ngraphs = ctx->opts.krylov == FHG_KRYLOV_CG ? 1 : 2;
    cudaGraphExec_t* exec = learned ? ctx->graph_l : ctx->graph;
    long long* kernels = learned ? ctx->graph_l_kernels : ctx->graph_kernels;
    ctx->learned_now = learned;
    for (int g = 0; g < ngraphs; g++) {
        cudaGraph_t graph = nullptr;
        const long long before = fhg::g_kernel_launches.load();
        cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            if (ctx->opts.krylov == FHG_KRYLOV_CG) cg_iteration(ctx);
            else fcg_iteration(ctx, g);
            e = cudaStreamEndCapture(ctx->stream, &graph);
        }
        const long long after = fhg::g_kernel_launches.load();
        fhg::g_kernel_launches -= (after - before);  // captured, not executed
        kernels[g] = after - before;
        if (e == cudaSuccess) e = cudaGraphInstantiate(&exec[g], graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            ctx->learned_now = false;
            return fail(ctx, FHG_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        }
    }
    ctx->learned_now = false;
    if (learned) ctx->graphs_l_built = ngraphs;
    else ctx->graphs_built = ngraphs;
    return FHG_OK;
}

// Autotuning of the launch shape of one operator: lanes per block row G in {4, 8, 16, 32} and
// blocks per lane step U in {1, 2} (U = 2 for bs <= 3 only), timed with the launch that will
// run; the fastest pair is kept. `run(G, U)` launches the operator once.
template <class F>
int tune(fhg_ctx* ctx, int bs, int& lanes, int& unroll, F run, float* best_ms = nullptr)
{
    // Three rounds over all candidates, each candidate's time the minimum over the rounds: a
    // single timing per candidate let one slow measurement decide, and the chosen shapes then
    // changed from run to run.
    constexpr int kRounds = 3;
    float t[2][4];
    for (auto& row : t)
        for (float& v : row) v = 1e30f;
    for (int round = 0; round < kRounds; round++) {
        for (int U : {1, 2}) {
            if (U == 2 && bs > 3) continue;
            for (int gi = 0; gi < 4; gi++) {
                const int G = 4 << gi;
                for (int w = 0; w < 2; w++) run(G, U);
                CK(cudaEventRecord(ctx->ev0, ctx->stream));
                const int reps = 8;
                for (int r = 0; r < reps; r++) run(G, U);
                CK(cudaEventRecord(ctx->ev1, ctx->stream));
                CK(cudaEventSynchronize(ctx->ev1));
                float ms = 0;
                CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
                t[U - 1][gi] = std::min(t[U - 1][gi], ms);
            }
        }
    }
    float best = 1e30f;
    int bestG = lanes, bestU = unroll;
    for (int U : {1, 2})
        for (int gi = 0; gi < 4; gi++)
            if (t[U - 1][gi] < best) { best = t[U - 1][gi]; bestG = 4 << gi; bestU = U; }
    lanes = bestG;
    unroll = bestU;
    if (best_ms) *best_ms = best;
    return FHG_OK;
}

// Time `run` like one candidate of tune: minimum over three rounds of eight launches.
template <class F>
int time_candidate(fhg_ctx* ctx, F run, float* ms_out)
{
    float best = 1e30f;
    for (int round = 0; round < 3; round++) {
        for (int w = 0; w < 2; w++) run();
        CK(cudaEventRecord(ctx->ev0, ctx->stream));
        for (int r = 0; r < 8; r++) run();
        CK(cudaEventRecord(ctx->ev1, ctx->stream));
        CK(cudaEventSynchronize(ctx->ev1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        best = std::min(best, ms);
    }
    *ms_out = best;
    return FHG_OK;
}

// Launch shapes found by tune_level, per operator structure (value type, block size, block rows,
// stored blocks of A and P, colours, padded widths): operators of identical structure (problems of one
// mesh size and degree, whatever their coefficients) share the best shape, so a process that sets up
// many of them times each structure once.
struct TuneKey {
    int prec, bs, nb, ncol, gs_w, prod_w, p_nbr, r_nbr;
    long long nnzb, p_blocks;
    bool operator<(const TuneKey& o) const
    {
        return std::tie(prec, bs, nb, ncol, gs_w, prod_w, p_nbr, r_nbr, nnzb, p_blocks) <
               std::tie(o.prec, o.bs, o.nb, o.ncol, o.gs_w, o.prod_w, o.p_nbr, o.r_nbr, o.nnzb, o.p_blocks);
    }
};
struct TuneShapes {
    int a_lanes, a_unroll, gs_lanes, gs_unroll, p_lanes, p_unroll, r_lanes, r_unroll;
    bool prod_slot, gs_slot;
    bool p_jds = false, r_jds = false;
};
std::mutex g_tune_mutex;
std::map<TuneKey, TuneShapes> g_tune_cache;
struct OuterChoice {
    int lanes, df_lanes;
    bool slot;
};
std::map<std::vector<long long>, OuterChoice> g_outer_cache;   // the outer operator's, per structure

template <class T>
int tune_level_uncached(fhg_ctx* ctx, int l);

template <class T>
int tune_level(fhg_ctx* ctx, int l)
{
    using V = LevelVecs<T>;
    constexpr int PR = V::kPrec;
    Level& L = ctx->levels[l];
    const bool coarsest = l == ctx->nlevels - 1;
    if (ctx->opts.gs_layout != FHG_GS_AUTO) return tune_level_uncached<T>(ctx, l);
    // the key from the row-major views (what the uncached tuning starts from)
    const bool ps0 = L.prod_slot[PR], gs0 = L.gs_slot[PR];
    L.prod_slot[PR] = false;
    L.gs_slot[PR] = false;
    BsrView<T>& A = const_cast<BsrView<T>&>(V::A(L));
    TuneKey key{PR, L.bs, L.nb, L.ncolours, V::gs(L).ell, A.ell, coarsest ? 0 : V::Pcsr(L).nbr,
                coarsest ? 0 : V::Rcsr(L).nbr, A.nnzb, coarsest ? 0 : V::Pcsr(L).nnzb};
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) {
            const TuneShapes& t = it->second;
            A.lanes = t.a_lanes;
            A.unroll = t.a_unroll;
            L.prod_slot[PR] = t.prod_slot;
            L.gs_lanes[PR] = t.gs_lanes;
            L.gs_unroll[PR] = t.gs_unroll;
            L.gs_slot[PR] = t.gs_slot;
            if (!coarsest) {
                BsrView<T>& P = const_cast<BsrView<T>&>(V::Pcsr(L));
                BsrView<T>& R = const_cast<BsrView<T>&>(V::Rcsr(L));
                P.lanes = t.p_lanes; P.unroll = t.p_unroll;
                R.lanes = t.r_lanes; R.unroll = t.r_unroll;
                L.p_jds[PR] = t.p_jds;
                L.r_jds[PR] = t.r_jds;
            }
            return FHG_OK;
        }
    }
    L.prod_slot[PR] = ps0;
    L.gs_slot[PR] = gs0;
    int rc = tune_level_uncached<T>(ctx, l);
    if (rc) return rc;
    const bool ps = L.prod_slot[PR];
    L.prod_slot[PR] = false;
    const BsrView<T>& Ar = V::A(L);
    TuneShapes t{Ar.lanes, Ar.unroll, L.gs_lanes[PR], L.gs_unroll[PR], 0, 1, 0, 1, ps, L.gs_slot[PR]};
    L.prod_slot[PR] = ps;
    if (!coarsest) {
        t.p_lanes = V::Pcsr(L).lanes; t.p_unroll = V::Pcsr(L).unroll;
        t.r_lanes = V::Rcsr(L).lanes; t.r_unroll = V::Rcsr(L).unroll;
        t.p_jds = L.p_jds[PR];
        t.r_jds = L.r_jds[PR];
    }
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[key] = t;
    return FHG_OK;
}

template <class T>
int tune_level_uncached(fhg_ctx* ctx, int l)
{
    using V = LevelVecs<T>;
    Level& L = ctx->levels[l];
    cudaStream_t s = ctx->stream;
    const int bs = L.bs;
    CK(cudaMemsetAsync(V::x(L), 0, sizeof(T) * L.n, s));
    CK(cudaMemsetAsync(V::b(L), 0, sizeof(T) * L.n, s));
    // Products with A: the row-major view's launch shape, then (layout auto) the slot-major view
    // against it.
    const bool forced_prod_slot = L.prod_slot[V::kPrec];
    L.prod_slot[V::kPrec] = false;
    BsrView<T>& A = const_cast<BsrView<T>&>(V::A(L));
    float row_prod_ms = 0.f;
    int rc = tune(ctx, bs, A.lanes, A.unroll, [&](int G, int U) {
        BsrView<T> v = A; v.lanes = G; v.unroll = U;
        fhg::launch_spmv<T>(v, fhg::kSpmvResidual, V::x(L), V::b(L), V::r(L), s);
    }, &row_prod_ms);
    if (rc) return rc;
    L.prod_slot[V::kPrec] = forced_prod_slot;
    if constexpr (!std::is_same<T, double>::value) {
        const BsrView<T>* slot = nullptr;
        if constexpr (std::is_same<T, float>::value) slot = L.A32s.vals ? &L.A32s.v : nullptr;
        else slot = L.A2s.vals ? &L.A2s.v : nullptr;
        if (!forced_prod_slot && slot && ctx->opts.gs_layout == FHG_GS_AUTO) {
            float slot_ms = 0.f;
            rc = time_candidate(ctx, [&]() { fhg::launch_spmv<T>(*slot, fhg::kSpmvResidual, V::x(L), V::b(L), V::r(L), s); },
                                &slot_ms);
            if (rc) return rc;
            L.prod_slot[V::kPrec] = slot_ms < row_prod_ms;
        }
    }
    if (l < ctx->nlevels - 1) {
        Level& C = ctx->levels[l + 1];
        int g = A.lanes, gu = A.unroll;
        // the row-major sweep's launch shape first, then (gs_layout auto) the slot-major sweep
        // against it
        constexpr int PR = V::kPrec;
        const bool forced_slot = L.gs_slot[PR];
        L.gs_slot[PR] = false;
        float row_ms = 0.f;
        if (V::gs(L).ell > 0) { g = V::gs(L).lanes; gu = 1; }
        rc = tune(ctx, bs, g, gu, [&](int G, int U) {
            BsrView<T> v = V::gs(L); v.lanes = G; v.unroll = U;
            for (int c = 0; c < L.ncolours; c++)
                fhg::launch_gs<T>(v, L.colour_start[c], L.colour_start[c + 1], V::dinv(L), L.nb, V::b(L), V::x(L), s);
        }, &row_ms);
        if (rc) return rc;
        L.gs_lanes[PR] = g;
        L.gs_unroll[PR] = gu;
        L.gs_slot[PR] = forced_slot;
        if constexpr (!std::is_same<T, double>::value) {
            const BsrView<T>* slot = nullptr;
            if constexpr (std::is_same<T, float>::value) slot = L.G32s.vals ? &L.G32s.v : nullptr;
            else slot = L.G2s.vals ? &L.G2s.v : nullptr;
            if (!forced_slot && slot && ctx->opts.gs_layout == FHG_GS_AUTO) {
                float slot_ms = 0.f;
                rc = time_candidate(ctx, [&]() {
                    for (int c = 0; c < L.ncolours; c++)
                        fhg::launch_gs<T>(*slot, L.colour_start[c], L.colour_start[c + 1], V::dinv(L), L.nb,
                                          V::b(L), V::x(L), s);
                }, &slot_ms);
                if (rc) return rc;
                L.gs_slot[PR] = slot_ms < row_ms;
            }
        }
        if (L.inject) return FHG_OK;   // the natural injection has no launch shape
        BsrView<T>& P = const_cast<BsrView<T>&>(V::Pcsr(L));
        BsrView<T>& R = const_cast<BsrView<T>&>(V::Rcsr(L));
        const bool forced_jds = ctx->opts.gs_layout == FHG_GS_SLOT;   // the jagged views, not compared
        const bool pj0 = L.p_jds[V::kPrec], rj0 = L.r_jds[V::kPrec];
        L.p_jds[V::kPrec] = false;
        L.r_jds[V::kPrec] = false;
        CK(cudaMemsetAsync(V::x(C), 0, sizeof(T) * C.n, s));
        float p_ms = 0.f, r_ms = 0.f;
        if ((rc = tune(ctx, bs, P.lanes, P.unroll, [&](int G, int U) {
                 BsrView<T> v = P; v.lanes = G; v.unroll = U;
                 fhg::launch_spmv<T>(v, fhg::kSpmvAddTo, V::x(C), V::r(L), V::r(L), s);
             }, &p_ms)))
            return rc;
        if ((rc = tune(ctx, bs, R.lanes, R.unroll, [&](int G, int U) {
                 BsrView<T> v = R; v.lanes = G; v.unroll = U;
                 fhg::launch_spmv<T>(v, fhg::kSpmvAssign, V::r(L), nullptr, V::b(C), s);
             }, &r_ms)))
            return rc;
        // the jagged views against the best CSR shapes
        if (forced_jds) {
            L.p_jds[V::kPrec] = pj0;
            L.r_jds[V::kPrec] = rj0;
        } else if constexpr (!std::is_same<T, double>::value) {
            const BsrView<T>* pj = nullptr;
            const BsrView<T>* rj = nullptr;
            if constexpr (std::is_same<T, float>::value) {
                if (L.P32j.vals) pj = &L.P32j.v;
                if (L.R32j.vals) rj = &L.R32j.v;
            } else {
                if (L.P2j.vals) pj = &L.P2j.v;
                if (L.R2j.vals) rj = &L.R2j.v;
            }
            float ms = 0.f;
            if (pj) {
                if ((rc = time_candidate(ctx, [&]() { fhg::launch_spmv<T>(*pj, fhg::kSpmvAddTo, V::x(C), V::r(L), V::r(L), s); }, &ms)))
                    return rc;
                L.p_jds[V::kPrec] = ms < p_ms;
            }
            if (rj) {
                if ((rc = time_candidate(ctx, [&]() { fhg::launch_spmv<T>(*rj, fhg::kSpmvAssign, V::r(L), nullptr, V::b(C), s); }, &ms)))
                    return rc;
                L.r_jds[V::kPrec] = ms < r_ms;
            }
        }
    }
    return FHG_OK;
}

void free_graphs(fhg_ctx* ctx)
{
    for (int g = 0; g < 2; g++) {
        if (ctx->graph[g]) { cudaGraphExecDestroy(ctx->graph[g]); ctx->graph[g] = nullptr; }
        if (ctx->graph_l[g]) { cudaGraphExecDestroy(ctx->graph_l[g]); ctx->graph_l[g] = nullptr; }
    }
    ctx->graphs_built = 0;
    ctx->graphs_l_built = 0;
}

// Device-side state of a level (the given host operators stay): cleared with the allocations so
// that a later setup in another precision finds no pointer into freed memory.
void reset_device_state(Level& L)
{
    L.A = DevBsr<double>();
    L.Ahat = DevBsr<double>();
    L.P = DevBsr<double>();
    L.R = DevBsr<double>();
    L.A32 = DevBsr<float>();
    L.P32 = DevBsr<float>();
    L.R32 = DevBsr<float>();
    L.G32 = DevBsr<float>();
    L.A32p = DevBsr<float>();
    L.G32s = DevBsr<float>();
    L.A32s = DevBsr<float>();
    L.A2 = DevBsr<dfl>();
    L.P2 = DevBsr<dfl>();
    L.R2 = DevBsr<dfl>();
    L.G2 = DevBsr<dfl>();
    L.A2p = DevBsr<dfl>();
    L.G2s = DevBsr<dfl>();
    L.A2s = DevBsr<dfl>();
    L.P32j = DevBsr<float>();
    L.R32j = DevBsr<float>();
    L.P2j = DevBsr<dfl>();
    L.R2j = DevBsr<dfl>();
    for (int i = 0; i < 3; i++) { L.p_jds[i] = false; L.r_jds[i] = false; }
    L.dinv2 = nullptr;
    L.x2 = L.b2 = L.r2 = nullptr;
    for (int i = 0; i < 3; i++) { L.gs_slot[i] = false; L.prod_slot[i] = false; L.gs_lanes[i] = 0; L.gs_unroll[i] = 1; }
    L.Ahat_hi = DevBsr<float>();
    L.Ahat2s = DevBsr<dfl>();
    L.outer_slot = true;
    L.ahat_is_a = true;
    L.ahat_lo = nullptr;
    L.dinv = nullptr;
    L.dinv32 = nullptr;
    L.perm_d = nullptr;
    L.x = L.b = L.r = nullptr;
    L.x32 = L.b32 = L.r32 = nullptr;
    for (int i = 0; i < 4; i++) { L.kv64[i] = nullptr; L.kv32[i] = nullptr; L.kv2[i] = nullptr; }
    L.cinv = nullptr;
    L.outer_lanes = 0;
    L.inject = false;
    L.inj_map = nullptr;
}

void free_all(fhg_ctx* ctx)
{
    free_graphs(ctx);
    for (Level& L : ctx->levels) reset_device_state(L);
    ctx->nbr_d = nullptr; ctx->tfeat_d = nullptr; ctx->lw = nullptr; ctx->lstatus = nullptr;
    ctx->rlo = nullptr;
    ctx->rhi = nullptr;
    ctx->lparams = nullptr; ctx->lwts = nullptr; ctx->lbias = nullptr;
    ctx->learned_mode = FHG_LEARNED_OFF;
    ctx->learned_now = false;
    ctx->rho_plain = 0.0;
    for (void* p : ctx->allocations) cudaFree(p);
    ctx->allocations.clear();
    ctx->allocation_bytes.clear();
    if (ctx->nr_host) { cudaFreeHost(ctx->nr_host); ctx->nr_host = nullptr; }
    ctx->ready = false;
}

// A learned-step kernel whose bounded wait on the tensor cores expired leaves 1 in lstatus.
int check_learned_status(fhg_ctx* ctx)
{
    if (!ctx->lstatus) return FHG_OK;
    int st = 0;
    CK(cudaMemcpyAsync(&st, ctx->lstatus, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (st == 0) return FHG_OK;
    CK(cudaMemsetAsync(ctx->lstatus, 0, sizeof(int), ctx->stream));
    return fail(ctx, FHG_ERR_CUDA, "learned step: a wait on the tensor-core pipeline expired");
}

int run_solve(fhg_ctx* ctx, double* history, fhg_solve_info* info)
{
    Level& L0 = ctx->levels[0];
    const long long n = L0.n;
    cudaStream_t s = ctx->stream;
    const int maxit = ctx->opts.max_iterations;
    // x = 0, r = b, ||b||, first-iteration placeholders (dp = 0, Adp = 0, d.Ad_prev = 1).
    CK(cudaMemsetAsync(ctx->kx, 0, sizeof(double) * n, s));
    CK(cudaMemcpyAsync(ctx->kr, ctx->kb, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    for (int q = 0; q < 2; q++) {
        CK(cudaMemsetAsync(ctx->kz[q], 0, sizeof(double) * n, s));
        CK(cudaMemsetAsync(ctx->kAd[q], 0, sizeof(double) * n, s));
    }
    fhg::launch_dot(n, ctx->kb, ctx->kb, part(ctx, 0), s);
    fhg::launch_sqrt_sum(part(ctx, 0), ctx->scal + 0, s);
    const double init[4] = {1.0, 1.0, 0.0, 0.0};  // dAdp, nr, rz, beta
    CK(cudaMemcpyAsync(ctx->scal + 1, init, sizeof(init), cudaMemcpyHostToDevice, s));
    const int one = 1;
    CK(cudaMemcpyAsync(ctx->counter_d, &one, sizeof(int), cudaMemcpyHostToDevice, s));
    if (outer_df(ctx))
        outer_df_start(ctx, ctx->kr);  // r = b as an FP32 pair
    else if (ctx->opts.krylov == FHG_KRYLOV_FCG && ctx->opts.vcycle_precision == FHG_PREC_FP32)
        fhg::launch_convert<double, float>(n, ctx->kr, L0.b32, s);  // FP32 copy of r = b
    if (ctx->opts.krylov == FHG_KRYLOV_CG) {
        // z = M r; d = 0 so that the first direction is z; rz = r.z
        precondition(ctx, ctx->kr, ctx->kz[0]);
        fhg::launch_dot(n, ctx->kr, ctx->kz[0], part(ctx, 0), s);
        fhg::launch_sum(part(ctx, 0), ctx->scal + 3, s);
    }
    // The learned correction runs inside FP32 V-cycles of FCG (the flexible method absorbs the
    // variable preconditioner).
    bool learned = ctx->learned_mode != FHG_LEARNED_OFF && ctx->lwts && ctx->opts.krylov == FHG_KRYLOV_FCG &&
                   ctx->opts.vcycle_precision == FHG_PREC_FP32;
    // The K-cycle decides its second coarse FCG step on the host: no graph replay then.
    const bool graphs = ctx->opts.use_graphs && ctx->opts.w_loops != FHG_CYCLE_K;
    if (graphs && !ctx->graphs_built) {
        int rc = build_graphs(ctx, false);
        if (rc) return rc;
    }
    if (learned && graphs && !ctx->graphs_l_built) {
        int rc = build_graphs(ctx, true);
        if (rc) return rc;
    }
    std::vector<double> hist(maxit + 1, 0.0);
    hist[0] = 1.0;
    double nr = 1.0;
    int it = 0, learned_its = 0, replacements = 0;
    int status = FHG_OK;
    double true_rel = -1.0;
    const bool fp32 = ctx->opts.vcycle_precision == FHG_PREC_FP32;
    while (true) {
        while (!(it > 0 && (it >= maxit || nr < ctx->opts.tolerance))) {
            const int p = it & 1;
            if (graphs) {
                const int g = ctx->opts.krylov == FHG_KRYLOV_CG ? 0 : p;
                CK(cudaGraphLaunch(learned ? ctx->graph_l[g] : ctx->graph[g], s));
                fhg::g_kernel_launches += learned ? ctx->graph_l_kernels[g] : ctx->graph_kernels[g];
            } else if (ctx->opts.krylov == FHG_KRYLOV_CG) {
                cg_iteration(ctx);
            } else {
                ctx->learned_now = learned;
                fcg_iteration(ctx, p);
                ctx->learned_now = false;
            }
            CK(cudaStreamSynchronize(s));
            nr = *ctx->nr_host;
            it++;
            hist[it] = nr;
            if (learned) learned_its++;
            if (std::isinf(nr)) { status = fail(ctx, FHG_ERR_DIVERGED, "divergence of the solver"); break; }
            if (std::isnan(nr)) { status = fail(ctx, FHG_ERR_NAN, "the residual is NaN."); break; }
            // Fallback rule: from the sixth iteration on, when the per-iteration residual reduction
            // (the geometric mean over the last four iterations, which evens out FCG's irregular
            // first iterations and its alternation) falls behind the plain method's calibrated
            // per-iteration reduction, the remaining iterations use the plain V-cycle.
            if (learned && ctx->learned_mode == FHG_LEARNED_FALLBACK && it >= kFallbackWindow + 2 &&
                ctx->rho_plain > 0.0) {
                const double rho = std::pow(hist[it] / hist[it - kFallbackWindow], 1.0 / kFallbackWindow);
                if (!(rho <= ctx->rho_plain)) learned = false;
            }
        }
        if (learned_its > 0 && status == FHG_OK) status = check_learned_status(ctx);
        if (status != FHG_OK) break;
        // The FP64 true residual ||b - A x|| / ||b|| judges the solve (A the full level-0 operator).
        fhg::launch_spmv<double>(L0.A.v, fhg::kSpmvResidual, ctx->kx, ctx->kb, ctx->kt, s);
        fhg::launch_dot(n, ctx->kt, ctx->kt, part(ctx, 0), s);
        fhg::launch_sqrt_sum(part(ctx, 0), ctx->scal + 5, s);
        double h[6];
        CK(cudaMemcpyAsync(h, ctx->scal, sizeof(h), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        true_rel = h[0] > 0 ? h[5] / h[0] : h[5];
        if (!(true_rel < ctx->opts.tolerance) && std::isfinite(true_rel)) {
            // A plain FP64 evaluation of b - A x errs by up to u sum_j |a_ij x_j| per row, which at high
            // coefficient contrast exceeds the tolerance: evaluate it again in compensated arithmetic
            // (accurate to about one unit of each r_i) before judging the solve or replacing r.
            fhg::launch_residual_comp(L0.A.v, ctx->kx, ctx->kb, ctx->kt, part(ctx, 0), s);
            fhg::launch_sqrt_sum(part(ctx, 0), ctx->scal + 5, s);
            CK(cudaMemcpyAsync(h, ctx->scal, sizeof(h), cudaMemcpyDeviceToHost, s));
            CK(cudaStreamSynchronize(s));
            true_rel = h[0] > 0 ? h[5] / h[0] : h[5];
        }
        // FP32 V-cycle (and, with fhg_options.replace_residual, the FP64 ones): the recursive residual
        // of the outer iteration can drift from the true one (the outer product loses digits to
        // cancellation at high coefficient contrast). Residual replacement: r = b - A x and the
        // iteration continues (the direction recurrence is kept) until the true residual meets the
        // tolerance. Without the option the FP64 modes keep the reference's loop unchanged.
        const bool replace = fp32 || ctx->opts.replace_residual;
        if (replace && ctx->opts.krylov == FHG_KRYLOV_FCG && it < maxit && !(true_rel < ctx->opts.tolerance) &&
            replacements < 8) {
            replacements++;
            CK(cudaMemcpyAsync(ctx->kr, ctx->kt, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
            CK(cudaMemcpyAsync(ctx->scal + 2, &true_rel, sizeof(double), cudaMemcpyHostToDevice, s));
            // the V-cycle's right-hand side: the FP32 pair of r, or r in FP32 (the FP64 and pair
            // V-cycles without the split outer iteration read r itself)
            if (outer_df(ctx)) outer_df_start(ctx, ctx->kr);
            else if (fp32) fhg::launch_convert<double, float>(n, ctx->kr, L0.b32, s);
            CK(cudaStreamSynchronize(s));
            nr = true_rel;
            continue;
        }
        break;
    }
    if (history)
        for (int k = 0; k <= maxit; k++) history[k] = k <= it ? hist[k] : 0.0;
    if (info) {
        info->iterations = it;
        info->status = status;
        info->normalized_residual = nr;
        info->learned_iterations = learned_its;
        info->true_relative_residual = true_rel;
    }
    return status;
}

// Per-iteration reduction of the plain method (FCG with the plain V-cycle of the current
// options) on a seeded random right-hand side: the geometric mean over iterations 3..12.
int calibrate_plain(fhg_ctx* ctx)
{
    Level& L0 = ctx->levels[0];
    std::vector<double> b(L0.n);
    uint64_t st = 0x5DEECE66DULL;
    for (auto& v : b) {
        st += 0x9E3779B97F4A7C15ull;
        uint64_t z = st;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        v = (double)(z >> 11) * (2.0 / 9007199254740992.0) - 1.0;
    }
    CK(cudaMemcpyAsync(ctx->kb, b.data(), sizeof(double) * L0.n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    const fhg_options saved = ctx->opts;
    const int mode = ctx->learned_mode;
    const int K = std::min(12, std::max(4, saved.max_iterations));
    ctx->opts.tolerance = 0.0;
    ctx->opts.max_iterations = K;
    ctx->learned_mode = FHG_LEARNED_OFF;
    std::vector<double> hist(K + 1);
    fhg_solve_info info{};
    int rc = run_solve(ctx, hist.data(), &info);
    ctx->opts = saved;
    ctx->learned_mode = mode;
    if (rc) return rc;
    const int k1 = std::min(info.iterations, K);
    ctx->rho_plain = k1 >= 4 && hist[2] > 0 ? std::pow(hist[k1] / hist[2], 1.0 / (k1 - 2)) : 0.0;
    return FHG_OK;
}

}  // namespace

// ===========================================================================
// C ABI

extern "C" {

void fhg_default_options(fhg_options* o)
{
    std::memset(o, 0, sizeof(*o));
    o->krylov = FHG_KRYLOV_FCG;
    o->pre_smoother = FHG_SMOOTHER_BGS;
    o->post_smoother = FHG_SMOOTHER_RBGS;
    o->pre_iterations = 1;
    o->post_iterations = 1;
    o->omega = 1.0;
    o->tolerance = 1e-8;
    o->max_iterations = 200;
    o->vcycle_precision = FHG_PREC_FP64;
    o->colouring = 1;
    o->use_graphs = 1;
    o->autotune = 0;
    o->max_coarse_rows = 8192;
    o->outer_split = 1;
    o->w_loops = 1;
    o->galerkin = 0;
    o->coarse_pre_iterations = -1;
    o->coarse_post_iterations = -1;
    o->gs_layout = FHG_GS_AUTO;
    o->extra_precisions = 0;
    o->replace_residual = 0;
    o->fused_coarse = 1;
}

int fhg_create(fhg_ctx** out, int device)
{
    if (!out) return FHG_ERR_INVALID_ARG;
    *out = nullptr;
    fhg_ctx* ctx = new fhg_ctx();
    ctx->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&ctx->ev1);
    if (e != cudaSuccess) {
        ctx->err = std::string("CUDA initialisation failed: ") + cudaGetErrorString(e);
        *out = ctx;
        return FHG_ERR_CUDA;
    }
    fhg_default_options(&ctx->opts);
    *out = ctx;
    return FHG_OK;
}

void fhg_destroy(fhg_ctx* ctx)
{
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    free_all(ctx);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* fhg_last_error(const fhg_ctx* ctx)
{
    return ctx ? ctx->err.c_str() : "null context";
}

int fhg_set_level(fhg_ctx* ctx, int level, int block_size, int n, const int* rowptr, const int* colidx,
                  const double* vals)
{
    if (!ctx) return FHG_ERR_INVALID_ARG;
    if (level < 0 || level > 63) return fail(ctx, FHG_ERR_INVALID_ARG, "level %d out of range", level);
    if (!supported_bs(block_size))
        return fail(ctx, FHG_ERR_UNSUPPORTED, "block size %d not supported (2, 3, 4, 6)", block_size);
    if (n <= 0 || n % block_size) return fail(ctx, FHG_ERR_INVALID_ARG, "n=%d is not a positive multiple of %d", n, block_size);
    if (!rowptr || !colidx || (!vals && rowptr[n] > 0)) return fail(ctx, FHG_ERR_INVALID_ARG, "null CSR array");
    int rc = check_csr(ctx, "A", n, n, rowptr, colidx);
    if (rc) return rc;
    if ((int)ctx->levels.size() <= level) ctx->levels.resize(level + 1);
    Level& L = ctx->levels[level];
    L.n = n; L.bs = block_size; L.nb = n / block_size;
    L.A_in.n_rows = L.A_in.n_cols = n;
    L.A_in.rowptr.assign(rowptr, rowptr + n + 1);
    L.A_in.colidx.assign(colidx, colidx + rowptr[n]);
    L.A_in.vals.assign(vals, vals + rowptr[n]);
    L.A_in.set = true;
    L.A_is_galerkin = false;
    ctx->ready = false;
    return FHG_OK;
}

int fhg_set_prolongation(fhg_ctx* ctx, int level, int n_fine, int n_coarse, const int* rowptr, const int* colidx,
                         const double* vals)
{
    if (!ctx) return FHG_ERR_INVALID_ARG;
    if (level < 0 || level > 63) return fail(ctx, FHG_ERR_INVALID_ARG, "level %d out of range", level);
    if (n_fine <= 0 || n_coarse <= 0) return fail(ctx, FHG_ERR_INVALID_ARG, "bad prolongation shape");
    if (!rowptr || !colidx || (!vals && rowptr[n_fine] > 0)) return fail(ctx, FHG_ERR_INVALID_ARG, "null CSR array");
    int rc = check_csr(ctx, "P", n_fine, n_coarse, rowptr, colidx);
    if (rc) return rc;
    if ((int)ctx->levels.size() <= level) ctx->levels.resize(level + 1);
    Level& L = ctx->levels[level];
    L.P_in.n_rows = n_fine; L.P_in.n_cols = n_coarse;
    L.P_in.rowptr.assign(rowptr, rowptr + n_fine + 1);
    L.P_in.colidx.assign(colidx, colidx + rowptr[n_fine]);
    L.P_in.vals.assign(vals, vals + rowptr[n_fine]);
    L.P_in.set = true;
    ctx->ready = false;
    return FHG_OK;
}

int fhg_setup(fhg_ctx* ctx, int nlevels, const fhg_options* opts)
{
    if (!ctx) return FHG_ERR_INVALID_ARG;
    CK(cudaSetDevice(ctx->device));
    free_all(ctx);
    ctx->epoch++;
    if (opts) ctx->opts = *opts;
    fhg_options& o = ctx->opts;
    if (o.max_coarse_rows <= 0) o.max_coarse_rows = 8192;
    if (o.max_iterations < 0 || o.pre_iterations < 0 || o.post_iterations < 0 || o.coarse_pre_iterations < -1 ||
        o.coarse_post_iterations < -1)
        return fail(ctx, FHG_ERR_INVALID_ARG, "negative iteration count");
    if (o.gs_layout < FHG_GS_AUTO || o.gs_layout > FHG_GS_SLOT)
        return fail(ctx, FHG_ERR_INVALID_ARG, "unknown GS layout %d", o.gs_layout);
    if (o.pre_smoother < 0 || o.pre_smoother > 6 || o.post_smoother < 0 || o.post_smoother > 6)
        return fail(ctx, FHG_ERR_INVALID_ARG, "unknown smoother code");
    if (o.w_loops < 1 && o.w_loops != FHG_CYCLE_K) o.w_loops = 1;
    if (o.galerkin && nlevels > 0 && nlevels <= 64 && (int)ctx->levels.size() < nlevels) ctx->levels.resize(nlevels);
    if (nlevels <= 0 || nlevels > (int)ctx->levels.size())
        return fail(ctx, FHG_ERR_INVALID_ARG, "nlevels=%d but %zu levels were given", nlevels, ctx->levels.size());
    ctx->nlevels = nlevels;
    if (o.galerkin) {
        // Galerkin coarse operators A_{l+1} = R_l A_l P_l, R_l = P_l^T (Level::ComputeGalerkinOperator,
        // src/Solver/Multigrid/Level.h:133-137; "-g 1"), replacing any operator given for l >= 1.
        if (!ctx->levels[0].A_in.set) return fail(ctx, FHG_ERR_INVALID_ARG, "level 0 operator not set");
        for (int l = 0; l + 1 < nlevels; l++) {
            Level& L = ctx->levels[l];
            Level& C = ctx->levels[l + 1];
            const int bs = L.bs;
            if (!L.P_in.set) return fail(ctx, FHG_ERR_INVALID_ARG, "level %d prolongation not set", l);
            int nl = 0;
            if (natural_injection(L.P_in, bs, L.nb, &nl)) {
                inject_galerkin(L.A_in, bs, nl, C.A_in);
                C.n = L.nb * nl;
                C.bs = nl;
                C.nb = L.nb;
                C.A_is_galerkin = true;
                continue;
            }
            if (L.P_in.n_rows != L.n || L.P_in.n_cols % bs)
                return fail(ctx, FHG_ERR_INVALID_ARG, "level %d prolongation is %dx%d for %d rows", l, L.P_in.n_rows,
                            L.P_in.n_cols, L.n);
            HostBsr Ab, Pb, Rb, APb, Cb;
            csr_to_bsr(L.A_in, bs, Ab);
            csr_to_bsr(L.P_in, bs, Pb);
            transpose_bsr(Pb, Rb);
            bsr_multiply(Ab, Pb, APb);
            Ab = HostBsr();
            bsr_multiply(Rb, APb, Cb);
            bsr_to_csr(Cb, C.A_in);
            C.n = L.P_in.n_cols;
            C.bs = bs;
            C.nb = C.n / bs;
            C.A_is_galerkin = true;
        }
    } else {
        for (int l = 1; l < nlevels; l++)
            if (ctx->levels[l].A_is_galerkin)
                return fail(ctx, FHG_ERR_INVALID_ARG, "level %d holds a Galerkin operator from an earlier setup: set it again", l);
    }
    for (int l = 0; l < nlevels; l++) {
        Level& L = ctx->levels[l];
        if (!L.A_in.set) return fail(ctx, FHG_ERR_INVALID_ARG, "level %d operator not set", l);
        L.inject = false;
        if (l < nlevels - 1) {
            const Level& C = ctx->levels[l + 1];
            if (!L.P_in.set) return fail(ctx, FHG_ERR_INVALID_ARG, "level %d prolongation not set", l);
            if (L.P_in.n_rows != L.n || L.P_in.n_cols != C.n)
                return fail(ctx, FHG_ERR_INVALID_ARG, "level %d prolongation is %dx%d, expected %dx%d", l,
                            L.P_in.n_rows, L.P_in.n_cols, L.n, C.n);
            // A change of block size (p-coarsening) only through the natural injection.
            if (C.bs != L.bs) {
                int nl = 0;
                if (C.nb != L.nb || !natural_injection(L.P_in, L.bs, L.nb, &nl) || nl != C.bs)
                    return fail(ctx, FHG_ERR_UNSUPPORTED,
                                "level %d block size %d differs from level %d's %d and the prolongation is not the "
                                "natural injection between face degrees", l + 1, C.bs, l, L.bs);
                L.inject = true;
            }
        }
    }
    Level& LC = ctx->levels[nlevels - 1];
    if (LC.n > o.max_coarse_rows)
        return fail(ctx, FHG_ERR_TOO_LARGE, "coarsest level has %d rows, above the dense direct-solve limit %d", LC.n,
                    o.max_coarse_rows);
    if (o.vcycle_precision < FHG_PREC_FP64 || o.vcycle_precision > FHG_PREC_DF)
        return fail(ctx, FHG_ERR_INVALID_ARG, "unknown V-cycle precision %d", o.vcycle_precision);
    // Operator copies: FP64 always; FP32 and FP32 pairs for the V-cycle precision and the extra ones.
    const bool fp32 = o.vcycle_precision == FHG_PREC_FP32 || (o.extra_precisions & (1 << FHG_PREC_FP32));
    const bool pair = o.vcycle_precision == FHG_PREC_DF || (o.extra_precisions & (1 << FHG_PREC_DF));
    int rc;

    // Block structure, colouring and permutation of every level.
    std::vector<HostBsr> Ab(nlevels);
    for (int l = 0; l < nlevels; l++) {
        Level& L = ctx->levels[l];
        csr_to_bsr(L.A_in, L.bs, Ab[l]);
        L.perm.resize(L.nb);
        std::iota(L.perm.begin(), L.perm.end(), 0);
        if (l == nlevels - 1) {
            L.ncolours = 0;
            L.colour_start.assign(1, 0);
        } else if (o.colouring) {
            std::vector<int> colour;
            L.ncolours = greedy_colouring(Ab[l], colour);
            L.colour_start.assign(L.ncolours + 1, 0);
            for (int c : colour) L.colour_start[c + 1]++;
            for (int c = 0; c < L.ncolours; c++) L.colour_start[c + 1] += L.colour_start[c];
            std::vector<int> fill(L.colour_start.begin(), L.colour_start.end() - 1);
            for (int I = 0; I < L.nb; I++) L.perm[fill[colour[I]]++] = I;
        } else {
            // Given order, one block row per colour: the sequential sweep of the reference.
            L.ncolours = L.nb;
            L.colour_start.resize(L.nb + 1);
            std::iota(L.colour_start.begin(), L.colour_start.end(), 0);
        }
    }
    std::vector<std::vector<int>> iperm(nlevels);
    for (int l = 0; l < nlevels; l++) {
        Level& L = ctx->levels[l];
        iperm[l].resize(L.nb);
        for (int I = 0; I < L.nb; I++) iperm[l][L.perm[I]] = I;
    }

    for (int l = 0; l < nlevels; l++) {
        Level& L = ctx->levels[l];
        HostBsr Ap;
        permute_bsr(Ab[l], L.perm, iperm[l], Ap);
        Ab[l] = HostBsr();
        if ((rc = upload_bsr<double>(ctx, Ap, L.A, nullptr))) return rc;
        if (fp32 && (rc = upload_bsr<float>(ctx, Ap, L.A32, &L.A))) return rc;
        if (pair && (rc = upload_bsr<dfl>(ctx, Ap, L.A2, &L.A))) return rc;
        // slot-major views (GS sweeps and products): when forced, or for the autotuner to compare
        const bool want_slot = o.colouring && (o.gs_layout == FHG_GS_SLOT || (o.gs_layout == FHG_GS_AUTO && o.autotune));
        if (fp32 && l < nlevels - 1) {
            if (o.colouring && (rc = upload_padded(ctx, Ap, L.G32, true, 8))) return rc;
            if ((rc = upload_padded(ctx, Ap, L.A32p, false, 8))) return rc;
            if (want_slot && (rc = upload_offdiag_slot_major(ctx, Ap, L.colour_start, L.G32s))) return rc;
            if (want_slot && (rc = upload_slot_major_all(ctx, Ap, L.A32s))) return rc;
            L.gs_slot[FHG_PREC_FP32] = o.gs_layout == FHG_GS_SLOT && L.G32s.vals;
            L.prod_slot[FHG_PREC_FP32] = o.gs_layout == FHG_GS_SLOT && L.A32s.vals;
        }
        if (pair && l < nlevels - 1) {
            if (o.colouring && (rc = upload_padded(ctx, Ap, L.G2, true, 8))) return rc;
            if ((rc = upload_padded(ctx, Ap, L.A2p, false, 8))) return rc;
            if (want_slot && (rc = upload_offdiag_slot_major(ctx, Ap, L.colour_start, L.G2s))) return rc;
            if (want_slot && (rc = upload_slot_major_all(ctx, Ap, L.A2s))) return rc;
            L.gs_slot[FHG_PREC_DF] = o.gs_layout == FHG_GS_SLOT && L.G2s.vals;
            L.prod_slot[FHG_PREC_DF] = o.gs_layout == FHG_GS_SLOT && L.A2s.vals;
        }
        if ((rc = upload(ctx, &L.perm_d, L.perm.data(), L.perm.size()))) return rc;
        if (l < nlevels - 1) {
            // Pre-inverted diagonal blocks (FP64, rounded for the FP32 copy).
            const int bs = L.bs;
            const int bb = bs * bs;
            std::vector<double> inv((size_t)L.nb * bb);
            for (int I = 0; I < L.nb; I++) {
                int pd = -1;
                for (int p = Ap.rowptr[I]; p < Ap.rowptr[I + 1]; p++)
                    if (Ap.colidx[p] == I) { pd = p; break; }
                if (pd < 0 || !invert_block(&Ap.vals[(size_t)pd * bb], bs, &inv[(size_t)I * bb]))
                    return fail(ctx, FHG_ERR_SINGULAR_BLOCK, "level %d: diagonal block %d is singular", l, L.perm[I]);
            }
            std::vector<double> soa((size_t)L.nb * bb);
            for (int I = 0; I < L.nb; I++)
                for (int e = 0; e < bb; e++) soa[(size_t)e * L.nb + I] = inv[(size_t)I * bb + e];
            if ((rc = upload(ctx, &L.dinv, soa.data(), soa.size()))) return rc;
            if (fp32) {
                std::vector<float> s32(soa.begin(), soa.end());
                if ((rc = upload(ctx, &L.dinv32, s32.data(), s32.size()))) return rc;
            }
            if (pair) {
                std::vector<dfl> s2(soa.size());
                for (size_t q = 0; q < soa.size(); q++) s2[q] = dfl(soa[q]);
                if ((rc = upload(ctx, &L.dinv2, s2.data(), s2.size()))) return rc;
            }
            if (L.inject) {
                // The natural injection: block row i of this level is block row map[i] of the next.
                std::vector<int> map(L.nb);
                for (int I = 0; I < L.nb; I++) map[I] = iperm[l + 1][L.perm[I]];
                if ((rc = upload(ctx, &L.inj_map, map.data(), map.size()))) return rc;
                L.p_blocks = 0;
            } else {
                // Transfers: P' = Pi_l P Pi_{l+1}^T, R' = P'^T.
                HostBsr Pb, Pp, Rp;
                csr_to_bsr(L.P_in, bs, Pb);
                permute_bsr(Pb, L.perm, iperm[l + 1], Pp);
                Pb = HostBsr();
                transpose_bsr(Pp, Rp);
                L.p_blocks = Pp.nnzb();
                if ((rc = upload_bsr<double>(ctx, Pp, L.P, nullptr))) return rc;
                if ((rc = upload_bsr<double>(ctx, Rp, L.R, nullptr))) return rc;
                if (fp32) {
                    if ((rc = upload_bsr<float>(ctx, Pp, L.P32, &L.P))) return rc;
                    if ((rc = upload_bsr<float>(ctx, Rp, L.R32, &L.R))) return rc;
                }
                if (pair) {
                    if ((rc = upload_bsr<dfl>(ctx, Pp, L.P2, &L.P))) return rc;
                    if ((rc = upload_bsr<dfl>(ctx, Rp, L.R2, &L.R))) return rc;
                }
                // the jagged transfer views of the two largest levels: compared by the autotuner, or used
                // with FHG_GS_SLOT
                const bool want_jds = o.gs_layout == FHG_GS_SLOT || (o.gs_layout == FHG_GS_AUTO && o.autotune);
                if (want_jds && l <= 1) {
                    if (fp32 && ((rc = upload_jds(ctx, Pp, L.P32j)) || (rc = upload_jds(ctx, Rp, L.R32j)))) return rc;
                    if (pair && ((rc = upload_jds(ctx, Pp, L.P2j)) || (rc = upload_jds(ctx, Rp, L.R2j)))) return rc;
                    if (o.gs_layout == FHG_GS_SLOT)
                        for (int q : {FHG_PREC_FP32, FHG_PREC_DF}) {
                            L.p_jds[q] = true;
                            L.r_jds[q] = true;
                        }
                }
            }
        }
        if (l == 0 && fp32 && nlevels > 1 && fhg::learned_supports(L.bs)) {
            // Learned-step inputs: neighbour table, scratch and element-tensor features.
            std::vector<int> nbr;
            learned_neighbours(Ap, nbr);
            if ((rc = upload(ctx, &ctx->nbr_d, nbr.data(), nbr.size()))) return rc;
            if ((rc = dalloc(ctx, &ctx->lw, L.n))) return rc;
            if ((rc = dalloc(ctx, &ctx->lstatus, 1))) return rc;
            CK(cudaMemset(ctx->lstatus, 0, sizeof(int)));
            if ((rc = dalloc(ctx, &ctx->tfeat_d, (size_t)L.nb * fhg::learned::kTensorSlots))) return rc;
            if ((rc = upload_tensor_features(ctx))) return rc;
        }
        if (l == 0) {
            HostCsr S;
            symmetrise_lower(L.A_in, S);
            L.ahat_is_a = csr_equal(S, L.A_in);
            const bool split = (fp32 || pair) && o.outer_split;
            if (!L.ahat_is_a) {
                HostBsr Sb, Sp;
                csr_to_bsr(S, L.bs, Sb);
                permute_bsr(Sb, L.perm, iperm[0], Sp);
                if ((rc = upload_bsr<double>(ctx, Sp, L.Ahat, nullptr))) return rc;
                if (split && (rc = upload_bsr_split(ctx, Sp, L.Ahat_hi, &L.ahat_lo, L.Ahat))) return rc;
                if (split && (rc = upload_slot_major_all(ctx, Sp, L.Ahat2s))) return rc;
            } else if (split) {
                if ((rc = upload_bsr_split(ctx, Ap, L.Ahat_hi, &L.ahat_lo, L.A))) return rc;
                if ((rc = upload_slot_major_all(ctx, Ap, L.Ahat2s))) return rc;
            }
        }
        if (l == nlevels - 1) {
            std::vector<double> dense((size_t)L.n * L.n, 0.0), inv;
            for (int i = 0; i < L.n; i++)
                for (int p = L.A_in.rowptr[i]; p < L.A_in.rowptr[i + 1]; p++)
                    dense[(size_t)i * L.n + L.A_in.colidx[p]] = L.A_in.vals[p];
            if (dense_spd_inverse(dense, L.n, inv))
                return fail(ctx, FHG_ERR_NOT_SPD, "coarsest operator (%d rows) is not symmetric positive definite", L.n);
            if ((rc = upload(ctx, &L.cinv, inv.data(), inv.size()))) return rc;
        }
        // Vectors.
        if ((rc = dalloc(ctx, &L.x, L.n)) || (rc = dalloc(ctx, &L.b, L.n)) || (rc = dalloc(ctx, &L.r, L.n))) return rc;
        if (fp32 && ((rc = dalloc(ctx, &L.x32, L.n)) || (rc = dalloc(ctx, &L.b32, L.n)) || (rc = dalloc(ctx, &L.r32, L.n))))
            return rc;
        if (pair && ((rc = dalloc(ctx, &L.x2, L.n)) || (rc = dalloc(ctx, &L.b2, L.n)) || (rc = dalloc(ctx, &L.r2, L.n))))
            return rc;
        if (l > 0 && l < nlevels - 1)  // K-cycle vectors (the K-cycle runs FCG on levels 1..L-2)
            for (int i = 0; i < 4; i++) {
                if ((rc = dalloc(ctx, &L.kv64[i], L.n))) return rc;
                if (fp32 && (rc = dalloc(ctx, &L.kv32[i], L.n))) return rc;
                if (pair && (rc = dalloc(ctx, &L.kv2[i], L.n))) return rc;
            }
    }
    const long long n0 = ctx->levels[0].n;
    if ((rc = dalloc(ctx, &ctx->kx, n0)) || (rc = dalloc(ctx, &ctx->kr, n0)) || (rc = dalloc(ctx, &ctx->kb, n0)) ||
        (rc = dalloc(ctx, &ctx->kz[0], n0)) || (rc = dalloc(ctx, &ctx->kz[1], n0)) || (rc = dalloc(ctx, &ctx->kt, n0)) ||
        (rc = dalloc(ctx, &ctx->kAd[0], n0)) || (rc = dalloc(ctx, &ctx->kAd[1], n0)) ||
        (rc = dalloc(ctx, &ctx->partials, (size_t)8 * fhg::kReduceCtas)) || (rc = dalloc(ctx, &ctx->scal, 8)) ||
        (rc = dalloc(ctx, &ctx->hist_d, (size_t)o.max_iterations + 2)) || (rc = dalloc(ctx, &ctx->counter_d, 1)) ||
        (rc = dalloc(ctx, &ctx->loop_state, 4)) ||
        (rc = dalloc(ctx, &ctx->io, (size_t)2 * n0)))
        return rc;
    ctx->rlo = nullptr;
    ctx->rhi = nullptr;
    if ((fp32 || pair) && o.outer_split && (rc = dalloc(ctx, &ctx->rlo, n0))) return rc;
    // the high part of r: the FP32 V-cycle's right-hand side b32 itself; a buffer of its own otherwise
    if (pair && o.outer_split && (rc = dalloc(ctx, &ctx->rhi, n0))) return rc;
    CK(cudaMallocHost(&ctx->nr_host, sizeof(double)));
    std::unique_lock<std::recursive_mutex> timing(g_timing_mutex, std::defer_lock);
    if (o.autotune) timing.lock();
    if (o.autotune) {
        // Tune in the precision the V-cycle runs in (the FP64 copies keep the FP32 choices,
        // the same access pattern); the outer operators on their own launches.
        for (int l = 0; l < nlevels; l++) {
            Level& L = ctx->levels[l];
            if (fp32 && (rc = tune_level<float>(ctx, l))) return rc;
            if (pair && (rc = tune_level<dfl>(ctx, l))) return rc;
            if (!fp32 && !pair) {
                if ((rc = tune_level<double>(ctx, l))) return rc;
                continue;
            }
            // The FP64 copies take the shapes of the pair copies (same 8-byte values), else the FP32
            // ones: the row-major views' lanes (a slot-major view runs one thread per row).
            auto take = [&](const auto& A, const auto& P, const auto& R, int src) {
                L.A.v.lanes = A.lanes;
                L.A.v.unroll = A.unroll;
                L.gs_lanes[FHG_PREC_FP64] = L.gs_lanes[src];
                L.gs_unroll[FHG_PREC_FP64] = L.gs_unroll[src];
                if (l < nlevels - 1) {
                    L.P.v.lanes = P.lanes; L.P.v.unroll = P.unroll;
                    L.R.v.lanes = R.lanes; L.R.v.unroll = R.unroll;
                }
            };
            if (pair) take(L.A2p.vals ? L.A2p.v : L.A2.v, L.P2.v, L.R2.v, FHG_PREC_DF);
            else take(L.A32p.vals ? L.A32p.v : L.A32.v, L.P32.v, L.R32.v, FHG_PREC_FP32);
        }
        Level& L0 = ctx->levels[0];
        BsrView<double>& Ah = L0.ahat_is_a ? L0.A.v : L0.Ahat.v;
        // the outer operator's choices, kept per structure like the levels' shapes
        const std::vector<long long> okey = {L0.bs, L0.nb, (long long)Ah.nnzb, L0.ahat_is_a ? 1 : 0,
                                             L0.ahat_lo ? 1 : 0, L0.Ahat2s.vals ? 1 : 0, o.gs_layout};
        bool cached = false;
        if (o.gs_layout == FHG_GS_AUTO) {
            std::lock_guard<std::mutex> lock(g_tune_mutex);
            auto it = g_outer_cache.find(okey);
            if (it != g_outer_cache.end()) {
                L0.outer_lanes = it->second.lanes;
                if (L0.ahat_lo) L0.Ahat_hi.v.lanes = it->second.df_lanes;
                L0.outer_slot = it->second.slot;
                cached = true;
            }
        }
        if (!cached) {
            int g = Ah.lanes, gu = 1;
            CK(cudaMemsetAsync(ctx->kz[0], 0, sizeof(double) * L0.n, ctx->stream));
            if ((rc = tune(ctx, 9, g, gu, [&](int G, int) {
                     BsrView<double> v = Ah; v.lanes = G;
                     fhg::launch_spmv_dots(v, ctx->kz[0], ctx->kz[0], ctx->kAd[0], part(ctx, 5), ctx->stream);
                 })))
                return rc;
            L0.outer_lanes = g;
            if (L0.ahat_lo) {
                int gd = g, gdu = 1;
                const long long n = L0.n;
                float row_ms = 0.f;
                if ((rc = tune(ctx, 9, gd, gdu, [&](int G, int) {
                         BsrView<float> v = L0.Ahat_hi.v; v.lanes = G;
                         fhg::launch_spmv_dots_df(v, L0.ahat_lo, pair_hi(ctx->kz[0]), pair_lo(ctx->kz[0], n),
                                                  pair_hi(ctx->kz[0]), pair_lo(ctx->kz[0], n), pair_hi(ctx->kAd[0]),
                                                  pair_lo(ctx->kAd[0], n), part(ctx, 5), ctx->stream);
                     }, &row_ms)))
                    return rc;
                // the slot-major pair view against the best row-major shape
                if (L0.Ahat2s.vals) {
                    float slot_ms = 0.f;
                    if ((rc = time_candidate(ctx, [&]() {
                             fhg::launch_spmv_dots_df_slot(L0.Ahat2s.v, pair_hi(ctx->kz[0]), pair_lo(ctx->kz[0], n),
                                                           pair_hi(ctx->kz[0]), pair_lo(ctx->kz[0], n), pair_hi(ctx->kAd[0]),
                                                           pair_lo(ctx->kAd[0], n), part(ctx, 5), ctx->stream);
                         }, &slot_ms)))
                        return rc;
                    L0.outer_slot = slot_ms < row_ms;
                }
                L0.Ahat_hi.v.lanes = gd;
            }
            if (o.gs_layout == FHG_GS_AUTO) {
                std::lock_guard<std::mutex> lock(g_tune_mutex);
                g_outer_cache[okey] = OuterChoice{L0.outer_lanes, L0.ahat_lo ? L0.Ahat_hi.v.lanes : 0, L0.outer_slot};
            }
        }
    }
    // the coarse sub-cycle: one cluster launch or launch by launch (timed when autotuning)
    if ((rc = refresh_fused(ctx))) return rc;
    if (timing.owns_lock()) timing.unlock();
    release_unused_views(ctx);
    CK(cudaStreamSynchronize(ctx->stream));
    ctx->ready = true;
    return FHG_OK;
}

int fhg_solve_device(fhg_ctx* ctx, const double* b_dev, double* x_dev, double* history, fhg_solve_info* info)
{
    if (!ctx) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    CK(cudaSetDevice(ctx->device));
    Level& L0 = ctx->levels[0];
    if (ctx->learned_mode == FHG_LEARNED_FALLBACK && ctx->rho_plain == 0.0 &&
        ctx->opts.vcycle_precision == FHG_PREC_FP32 && ctx->opts.krylov == FHG_KRYLOV_FCG) {
        int rc0 = calibrate_plain(ctx);
        if (rc0) return rc0;
    }
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    // b' = Pi_0 b
    fhg::launch_permute<double>(L0.nb, L0.bs, L0.perm_d, b_dev, ctx->kb, true, ctx->stream);
    int rc = run_solve(ctx, history, info);
    // x = Pi_0^T x'
    fhg::launch_permute<double>(L0.nb, L0.bs, L0.perm_d, ctx->kx, x_dev, false, ctx->stream);
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    cudaError_t e = cudaEventSynchronize(ctx->ev1);
    if (rc == FHG_OK && e != cudaSuccess) return fail(ctx, FHG_ERR_CUDA, "solve: %s", cudaGetErrorString(e));
    float ms = 0;
    CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    if (info) info->solve_ms = ms;
    return rc;
}

int fhg_solve(fhg_ctx* ctx, const double* b, double* x, double* history, fhg_solve_info* info)
{
    if (!ctx) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    if (!b || !x) return fail(ctx, FHG_ERR_INVALID_ARG, "null vector");
    CK(cudaSetDevice(ctx->device));
    const long long n = ctx->levels[0].n;
    CK(cudaMemcpyAsync(ctx->io, b, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream));
    int rc = fhg_solve_device(ctx, ctx->io, ctx->io + n, history, info);
    cudaError_t e = cudaMemcpyAsync(x, ctx->io + n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (rc == FHG_OK && e != cudaSuccess) return fail(ctx, FHG_ERR_CUDA, "solve copy-out: %s", cudaGetErrorString(e));
    return rc;
}

extern "C++" {
template <class T>
static int apply_device_t(fhg_ctx* ctx, int level, int op, T* in, T* aux, T* out)
{
    // in/aux/out already in the permuted numbering on the device.
    using V = LevelVecs<T>;
    Level& L = ctx->levels[level];
    cudaStream_t s = ctx->stream;
    const bool coarsest = level == ctx->nlevels - 1;
    switch (op) {
    case FHG_OP_SPMV: fhg::launch_spmv<T>(V::A(L), fhg::kSpmvAssign, in, nullptr, out, s); break;
    case FHG_OP_RESIDUAL: fhg::launch_spmv<T>(V::A(L), fhg::kSpmvResidual, in, aux, out, s); break;
    case FHG_OP_RESTRICT:
        if (coarsest) return fail(ctx, FHG_ERR_INVALID_ARG, "no restriction on the coarsest level");
        restrict_to<T>(ctx, level, in, out);
        break;
    case FHG_OP_PROLONG_ADD:
        if (coarsest) return fail(ctx, FHG_ERR_INVALID_ARG, "no prolongation on the coarsest level");
        prolong_add<T>(ctx, level, in, aux, out);
        break;
    case FHG_OP_GS_FORWARD:
    case FHG_OP_GS_BACKWARD:
    case FHG_OP_JACOBI: {
        if (coarsest) return fail(ctx, FHG_ERR_INVALID_ARG, "no smoother on the coarsest level");
        if (out != in) CK(cudaMemcpyAsync(out, in, sizeof(T) * L.n, cudaMemcpyDeviceToDevice, s));
        const int code = op == FHG_OP_GS_FORWARD ? FHG_SMOOTHER_BGS
                         : op == FHG_OP_GS_BACKWARD ? FHG_SMOOTHER_RBGS
                                                    : (ctx->opts.pre_smoother == FHG_SMOOTHER_BJ23 ? FHG_SMOOTHER_BJ23 : FHG_SMOOTHER_BJ);
        smooth<T>(ctx, level, code, 1, aux, out);
        break;
    }
    case FHG_OP_COARSE_SOLVE:
        if (!coarsest) return fail(ctx, FHG_ERR_INVALID_ARG, "coarse solve on level %d (coarsest is %d)", level, ctx->nlevels - 1);
        fhg::launch_coarse<T>(L.n, L.cinv, in, out, s);
        break;
    default: return fail(ctx, FHG_ERR_INVALID_ARG, "op %d not available here", op);
    }
    return FHG_OK;
}

}  // extern "C++"

static int apply_device(fhg_ctx* ctx, int level, int op, double* in, double* aux, double* out)
{
    Level& L = ctx->levels[level];
    cudaStream_t s = ctx->stream;
    if (op == FHG_OP_SYM_SPMV) {
        if (level != 0) return fail(ctx, FHG_ERR_INVALID_ARG, "symmetric operator exists on level 0 only");
        BsrView<double> Ah = L.ahat_is_a ? L.A.v : L.Ahat.v;
        if (L.outer_lanes) Ah.lanes = L.outer_lanes;
        fhg::launch_spmv_dots(Ah, in, in, out, part(ctx, 4), s);
        return FHG_OK;
    }
    if (op == FHG_OP_VCYCLE) {
        if (level != 0) return fail(ctx, FHG_ERR_INVALID_ARG, "V-cycle starts on level 0");
        precondition(ctx, in, out);
        return FHG_OK;
    }
    if (op < 0 || op > FHG_OP_VCYCLE) return fail(ctx, FHG_ERR_INVALID_ARG, "unknown op %d", op);
    return apply_device_t<double>(ctx, level, op, in, aux, out);
}

static void op_levels(int level, int op, int* in_level, int* out_level)
{
    *in_level = level; *out_level = level;
    if (op == FHG_OP_RESTRICT) *out_level = level + 1;
    if (op == FHG_OP_PROLONG_ADD) *in_level = level + 1;
}

int fhg_apply(fhg_ctx* ctx, int level, int op, const double* in, const double* aux, double* out)
{
    if (!ctx) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    if (level < 0 || level >= ctx->nlevels) return fail(ctx, FHG_ERR_INVALID_ARG, "level %d out of range", level);
    CK(cudaSetDevice(ctx->device));
    int li, lo;
    op_levels(level, op, &li, &lo);
    if (lo >= ctx->nlevels || li >= ctx->nlevels) return fail(ctx, FHG_ERR_INVALID_ARG, "operator leaves the hierarchy");
    Level& Li = ctx->levels[li];
    Level& Lo = ctx->levels[lo];
    const bool need_aux = op == FHG_OP_RESIDUAL || op == FHG_OP_PROLONG_ADD || op == FHG_OP_GS_FORWARD ||
                          op == FHG_OP_GS_BACKWARD || op == FHG_OP_JACOBI;
    if (!in || !out || (need_aux && !aux)) return fail(ctx, FHG_ERR_INVALID_ARG, "null vector");
    const int aux_level = op == FHG_OP_PROLONG_ADD ? lo : li;
    Level& La = ctx->levels[aux_level];
    const size_t mx = (size_t)std::max(std::max(Li.n, Lo.n), La.n);
    double *t = nullptr;
    int rc = dalloc(ctx, &t, 6 * mx);
    if (rc) return rc;
    double *din = t, *daux = t + mx, *dout = t + 2 * mx, *pin = t + 3 * mx, *paux = t + 4 * mx, *pout = t + 5 * mx;
    cudaStream_t s = ctx->stream;
    CK(cudaMemcpyAsync(din, in, sizeof(double) * Li.n, cudaMemcpyHostToDevice, s));
    fhg::launch_permute<double>(Li.nb, Li.bs, Li.perm_d, din, pin, true, s);
    if (need_aux) {
        CK(cudaMemcpyAsync(daux, aux, sizeof(double) * La.n, cudaMemcpyHostToDevice, s));
        fhg::launch_permute<double>(La.nb, La.bs, La.perm_d, daux, paux, true, s);
    }
    if (op == FHG_OP_PROLONG_ADD) CK(cudaMemcpyAsync(pout, paux, sizeof(double) * Lo.n, cudaMemcpyDeviceToDevice, s));
    rc = apply_device(ctx, level, op, pin, paux, op == FHG_OP_PROLONG_ADD ? pout : pout);
    if (rc == FHG_OK) {
        fhg::launch_permute<double>(Lo.nb, Lo.bs, Lo.perm_d, pout, dout, false, s);
        cudaError_t e = cudaMemcpyAsync(out, dout, sizeof(double) * Lo.n, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) rc = fail(ctx, FHG_ERR_CUDA, "apply: %s", cudaGetErrorString(e));
    }
    cudaStreamSynchronize(s);
    dfree(ctx, t);
    return rc;
}

extern "C++" {
template <class T>
static int time_op_t(fhg_ctx* ctx, int level, int op, int warmup, int reps, double* avg_ms)
{
    int li, lo;
    op_levels(level, op, &li, &lo);
    if (lo >= ctx->nlevels || li >= ctx->nlevels) return fail(ctx, FHG_ERR_INVALID_ARG, "operator leaves the hierarchy");
    const size_t mx = (size_t)std::max(ctx->levels[li].n, ctx->levels[lo].n);
    T* t = nullptr;
    int rc = dalloc(ctx, &t, 3 * mx);
    if (rc) return rc;
    T *in = t, *aux = t + mx, *out = t + 2 * mx;
    cudaStream_t s = ctx->stream;
    CK(cudaMemsetAsync(out, 0, sizeof(T) * mx, s));
    // Inputs: the level's last V-cycle vectors (finite, representative values), converted.
    const int la = op == FHG_OP_PROLONG_ADD ? lo : li;
    if constexpr (std::is_same<T, double>::value) {
        CK(cudaMemcpyAsync(in, ctx->levels[li].x, sizeof(T) * ctx->levels[li].n, cudaMemcpyDeviceToDevice, s));
        CK(cudaMemcpyAsync(aux, ctx->levels[la].b, sizeof(T) * ctx->levels[la].n, cudaMemcpyDeviceToDevice, s));
    } else {
        fhg::launch_convert<double, T>(ctx->levels[li].n, ctx->levels[li].x, in, s);
        fhg::launch_convert<double, T>(ctx->levels[la].n, ctx->levels[la].b, aux, s);
    }
    auto one = [&]() -> int {
        if (op == FHG_OP_GS_FORWARD || op == FHG_OP_GS_BACKWARD) {
            if (level == ctx->nlevels - 1) return fail(ctx, FHG_ERR_INVALID_ARG, "no smoother on the coarsest level");
            smooth<T>(ctx, level, op == FHG_OP_GS_FORWARD ? FHG_SMOOTHER_BGS : FHG_SMOOTHER_RBGS, 1, aux, in);
            return FHG_OK;
        }
        if constexpr (std::is_same<T, float>::value) {
            if (op == FHG_OP_VCYCLE || op == FHG_OP_VCYCLE_LEARNED) {
                ctx->learned_now = op == FHG_OP_VCYCLE_LEARNED;
                vcycle<float>(ctx, 0, aux, out);
                ctx->learned_now = false;
                return FHG_OK;
            }
            if (op == FHG_OP_LEARNED_STEP) {
                learned_step(ctx, aux, out);
                return FHG_OK;
            }
        }
        if constexpr (std::is_same<T, dfl>::value) {
            if (op == FHG_OP_VCYCLE) {
                vcycle<dfl>(ctx, 0, aux, out);
                return FHG_OK;
            }
        }
        return apply_device_t<T>(ctx, level, op, in, aux, out);
    };
    for (int w = 0; w < warmup && rc == FHG_OK; w++) rc = one();
    if (rc == FHG_OK) {
        CK(cudaEventRecord(ctx->ev0, s));
        for (int r = 0; r < reps && rc == FHG_OK; r++) rc = one();
        CK(cudaEventRecord(ctx->ev1, s));
        CK(cudaEventSynchronize(ctx->ev1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        *avg_ms = ms / reps;
    }
    cudaStreamSynchronize(s);
    dfree(ctx, t);
    return rc;
}

}  // extern "C++"

int fhg_time_op(fhg_ctx* ctx, int level, int op, int precision, int warmup, int reps, double* avg_ms)
{
    if (!ctx || !avg_ms || reps <= 0) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    if (level < 0 || level >= ctx->nlevels) return fail(ctx, FHG_ERR_INVALID_ARG, "level %d out of range", level);
    CK(cudaSetDevice(ctx->device));
    if (op == FHG_OP_VCYCLE_LEARNED || op == FHG_OP_LEARNED_STEP || (op == FHG_OP_VCYCLE && precision == FHG_PREC_FP32)) {
        if (level != 0 || precision != FHG_PREC_FP32 || !ctx->levels[0].A32.vals)
            return fail(ctx, FHG_ERR_INVALID_ARG, "op %d is timed on level 0 in FP32 (FP32 setup)", op);
        if (op != FHG_OP_VCYCLE && !ctx->lwts) return fail(ctx, FHG_ERR_NOT_READY, "no network installed");
        int rc = time_op_t<float>(ctx, 0, op, warmup, reps, avg_ms);
        if (rc == FHG_OK && op != FHG_OP_VCYCLE) rc = check_learned_status(ctx);
        return rc;
    }
    if (op == FHG_OP_VCYCLE && precision == FHG_PREC_DF) {
        if (level != 0 || !ctx->levels[0].A2.vals)
            return fail(ctx, FHG_ERR_INVALID_ARG, "the pair V-cycle is timed on level 0 (pair copies built at setup)");
        return time_op_t<dfl>(ctx, 0, op, warmup, reps, avg_ms);
    }
    if (op == FHG_OP_SYM_SPMV || op == FHG_OP_VCYCLE) {
        Level& L0 = ctx->levels[0];
        // FP32 or DF: the outer operator in double-FP32 arithmetic (the one product both use)
        const bool split = op == FHG_OP_SYM_SPMV && (precision == FHG_PREC_FP32 || precision == FHG_PREC_DF);
        if (precision != FHG_PREC_FP64 && !split) return fail(ctx, FHG_ERR_INVALID_ARG, "op %d is timed in FP64 only", op);
        if (split && ((!L0.ahat_lo && !L0.Ahat2s.vals) || !ctx->rlo))
            return fail(ctx, FHG_ERR_NOT_READY, "the double-FP32 outer operator was not built at setup");
        const size_t n0 = L0.n;
        double* t = nullptr;
        int rc = dalloc(ctx, &t, 2 * n0);
        if (rc) return rc;
        CK(cudaMemcpyAsync(t, ctx->kr, sizeof(double) * n0, cudaMemcpyDeviceToDevice, ctx->stream));
        // double-FP32: d = r (FP32 pair in the first n0 doubles), Ad pair in the second
        float* dh = pair_hi(t);
        float* dl = pair_lo(t, (long long)n0);
        if (split) fhg::launch_split_df((long long)n0, ctx->kr, dh, dl, ctx->stream);
        auto one = [&]() -> int {
            if (split) {
                outer_product_df(ctx, dh, dl, dh, dl, pair_hi(t + n0), pair_lo(t + n0, (long long)n0), part(ctx, 4));
                return FHG_OK;
            }
            return apply_device(ctx, level, op, t, nullptr, t + n0);
        };
        for (int w = 0; w < warmup && rc == FHG_OK; w++) rc = one();
        CK(cudaEventRecord(ctx->ev0, ctx->stream));
        for (int r = 0; r < reps && rc == FHG_OK; r++) rc = one();
        CK(cudaEventRecord(ctx->ev1, ctx->stream));
        CK(cudaEventSynchronize(ctx->ev1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        *avg_ms = ms / reps;
        dfree(ctx, t);
        return rc;
    }
    if (precision == FHG_PREC_FP32) {
        if (!ctx->levels[0].A32.vals) return fail(ctx, FHG_ERR_NOT_READY, "FP32 operators were not built at setup");
        return time_op_t<float>(ctx, level, op, warmup, reps, avg_ms);
    }
    if (precision == FHG_PREC_DF) {
        if (!ctx->levels[0].A2.vals) return fail(ctx, FHG_ERR_NOT_READY, "pair operators were not built at setup");
        return time_op_t<dfl>(ctx, level, op, warmup, reps, avg_ms);
    }
    return time_op_t<double>(ctx, level, op, warmup, reps, avg_ms);
}

int fhg_set_cycle(fhg_ctx* ctx, int pre_smoother, int post_smoother, int pre_iterations, int post_iterations,
                  int w_loops)
{
    if (!ctx) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    if (pre_smoother < 0 || pre_smoother > 6 || post_smoother < 0 || post_smoother > 6)
        return fail(ctx, FHG_ERR_INVALID_ARG, "unknown smoother code");
    if (pre_iterations < 0 || post_iterations < 0 || (w_loops < 1 && w_loops != FHG_CYCLE_K))
        return fail(ctx, FHG_ERR_INVALID_ARG, "negative smoothing count or cycle loops < 1");
    free_graphs(ctx);
    ctx->epoch++;          // batched graphs that captured the old cycle are rebuilt
    ctx->rho_plain = 0.0;  // the plain method's reduction is measured again for the new cycle
    ctx->opts.pre_smoother = pre_smoother;
    ctx->opts.post_smoother = post_smoother;
    ctx->opts.pre_iterations = pre_iterations;
    ctx->opts.post_iterations = post_iterations;
    ctx->opts.w_loops = w_loops;
    return refresh_fused(ctx);
}

int fhg_set_coarse_smoothing(fhg_ctx* ctx, int pre_iterations, int post_iterations)
{
    if (!ctx) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    if (pre_iterations < -1 || post_iterations < -1) return fail(ctx, FHG_ERR_INVALID_ARG, "negative iteration count");
    if (ctx->opts.coarse_pre_iterations != pre_iterations || ctx->opts.coarse_post_iterations != post_iterations) {
        free_graphs(ctx);
        ctx->epoch++;
        ctx->rho_plain = 0.0;
        ctx->opts.coarse_pre_iterations = pre_iterations;
        ctx->opts.coarse_post_iterations = post_iterations;
        return refresh_fused(ctx);
    }
    return FHG_OK;
}

int fhg_set_vcycle_precision(fhg_ctx* ctx, int precision)
{
    if (!ctx) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    if (precision != FHG_PREC_FP64 && precision != FHG_PREC_FP32 && precision != FHG_PREC_DF)
        return fail(ctx, FHG_ERR_INVALID_ARG, "unknown precision");
    if (precision == FHG_PREC_FP32 && !ctx->levels[0].A32.vals)
        return fail(ctx, FHG_ERR_NOT_READY, "FP32 operators were not built: set up with FHG_PREC_FP32");
    if (precision == FHG_PREC_DF && !ctx->levels[0].A2.vals)
        return fail(ctx, FHG_ERR_NOT_READY, "pair operators were not built: set up with FHG_PREC_DF");
    if (ctx->opts.vcycle_precision != precision) {
        free_graphs(ctx);
        ctx->epoch++;
        ctx->rho_plain = 0.0;
        ctx->opts.vcycle_precision = precision;
    }
    return FHG_OK;
}

int fhg_level_info(const fhg_ctx* ctx, int level, int* n_block_rows, long long* n_blocks, int* n_colours, int* lanes,
                   long long* p_blocks)
{
    if (!ctx || !ctx->ready || level < 0 || level >= ctx->nlevels) return FHG_ERR_INVALID_ARG;
    const Level& L = ctx->levels[level];
    if (n_block_rows) *n_block_rows = L.nb;
    if (n_blocks) *n_blocks = L.A.v.nnzb;
    if (n_colours) *n_colours = L.ncolours;
    if (lanes) *lanes = L.A.v.lanes;
    if (p_blocks) *p_blocks = L.p_blocks;
    return FHG_OK;
}

long long fhg_device_bytes(const fhg_ctx* ctx)
{
    if (!ctx) return -1;
    long long total = 0;
    for (size_t b : ctx->allocation_bytes) total += (long long)b;
    return total;
}

int fhg_fused_coarse_info(const fhg_ctx* ctx, int precision, int* first_level, int* cluster_ctas,
                          int* cta_threads)
{
    if (!ctx || !ctx->ready || precision < 0 || precision > 2) return FHG_ERR_INVALID_ARG;
    if (first_level) *first_level = ctx->fused_from[precision];
    if (cluster_ctas) *cluster_ctas = ctx->fused_ctas[precision];
    if (cta_threads) *cta_threads = ctx->fused_threads[precision];
    return FHG_OK;
}

int fhg_get_permutation(const fhg_ctx* ctx, int level, int* perm)
{
    if (!ctx || !ctx->ready || level < 0 || level >= ctx->nlevels || !perm) return FHG_ERR_INVALID_ARG;
    const Level& L = ctx->levels[level];
    std::copy(L.perm.begin(), L.perm.end(), perm);
    return FHG_OK;
}

long long fhg_kernel_launches(const fhg_ctx* ctx)
{
    (void)ctx;
    return fhg::g_kernel_launches.load();
}

// ---------------------------------------------------------------------------
// Learned correction step and its training (no counterpart in the reference)

int fhg_set_face_tensors(fhg_ctx* ctx, int n_blocks, const double* tensors)
{
    if (!ctx) return FHG_ERR_INVALID_ARG;
    if (ctx->levels.empty() || !ctx->levels[0].A_in.set)
        return fail(ctx, FHG_ERR_NOT_READY, "the finest operator must be set before its face tensors");
    if (n_blocks != ctx->levels[0].nb || !tensors)
        return fail(ctx, FHG_ERR_INVALID_ARG, "%d face blocks given, level 0 has %d", n_blocks, ctx->levels[0].nb);
    ctx->tensors_host.assign(tensors, tensors + (size_t)n_blocks * 12);
    if (!ctx->ready) return FHG_OK;
    CK(cudaSetDevice(ctx->device));
    return upload_tensor_features(ctx);
}

int fhg_set_learned(fhg_ctx* ctx, const float* params, int n_params, int mode)
{
    using namespace fhg::learned;
    if (!ctx) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    const int kernel = (mode & FHG_LEARNED_MMA_SYNC) ? fhg::kLearnedKernelMmaSync : fhg::kLearnedKernelTcgen05;
    mode &= ~FHG_LEARNED_MMA_SYNC;
    if (mode < FHG_LEARNED_OFF || mode > FHG_LEARNED_ALWAYS) return fail(ctx, FHG_ERR_INVALID_ARG, "unknown mode %d", mode);
    CK(cudaSetDevice(ctx->device));
    if ((params || mode != FHG_LEARNED_OFF) && !ctx->nbr_d)
        return fail(ctx, FHG_ERR_UNSUPPORTED,
                    "the learned step needs a setup with the FP32 V-cycle, two levels or more and block size 2..4");
    Level& L0 = ctx->levels[0];
    cudaStream_t s = ctx->stream;
    int rc;
    if (kernel != ctx->learned_kernel) {
        ctx->learned_kernel = kernel;
        for (int g = 0; g < 2; g++)
            if (ctx->graph_l[g]) { cudaGraphExecDestroy(ctx->graph_l[g]); ctx->graph_l[g] = nullptr; }
        ctx->graphs_l_built = 0;
    }
    if (params) {
        if (n_params != kParams) return fail(ctx, FHG_ERR_INVALID_ARG, "%d parameters given, the network has %d", n_params, kParams);
        for (int i = 0; i < kParams; i++)
            if (!std::isfinite(params[i])) return fail(ctx, FHG_ERR_INVALID_ARG, "parameter %d is not finite", i);
        if (!ctx->lparams) {
            if ((rc = dalloc(ctx, &ctx->lparams, kParams)) || (rc = dalloc(ctx, &ctx->lwts, kWeights)) ||
                (rc = dalloc(ctx, &ctx->lbias, kBiases)))
                return rc;
        }
        CK(cudaMemcpyAsync(ctx->lparams, params, sizeof(float) * kParams, cudaMemcpyHostToDevice, s));
        fhg::launch_split_params(ctx->lparams, ctx->lwts, ctx->lbias, s);
        // First launch outside any capture: fixes the kernel's shared-memory limit and grid. With
        // w = 0 every scale is 0 and nothing is added to x.
        CK(cudaMemsetAsync(ctx->lw, 0, sizeof(float) * L0.n, s));
        if (fhg::launch_learned_apply(L0.nb, L0.bs, ctx->nbr_d, ctx->lw, ctx->tfeat_d, ctx->lwts, ctx->lbias, L0.x32,
                                      ctx->lstatus, ctx->learned_kernel, s))
            return fail(ctx, FHG_ERR_CUDA, "the learned-step kernel cannot run on this device");
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(s));
        if ((rc = check_learned_status(ctx))) return rc;
        for (int g = 0; g < 2; g++)
            if (ctx->graph_l[g]) { cudaGraphExecDestroy(ctx->graph_l[g]); ctx->graph_l[g] = nullptr; }
        ctx->graphs_l_built = 0;
    } else if (mode != FHG_LEARNED_OFF && !ctx->lwts) {
        return fail(ctx, FHG_ERR_NOT_READY, "no network installed");
    }
    ctx->learned_mode = mode;
    ctx->rho_plain = 0.0;
    ctx->epoch++;
    return FHG_OK;
}

int fhg_learned_reference_rate(fhg_ctx* ctx, double* rho)
{
    if (!ctx || !rho) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    CK(cudaSetDevice(ctx->device));
    if (ctx->rho_plain == 0.0) {
        int rc = calibrate_plain(ctx);
        if (rc) return rc;
    }
    *rho = ctx->rho_plain;
    return FHG_OK;
}

int fhg_learned_features(fhg_ctx* ctx, const float* r, void* features, float* scale)
{
    if (!ctx || !r || !features || !scale) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready || !ctx->nbr_d) return fail(ctx, FHG_ERR_NOT_READY, "no learned-step data (FP32 setup, bs 2..4)");
    CK(cudaSetDevice(ctx->device));
    Level& L = ctx->levels[0];
    fhg::launch_block_diag(L.nb, L.bs, L.dinv32, L.nb, r, ctx->lw, ctx->stream);
    fhg::launch_features(L.nb, L.nb, L.bs, ctx->nbr_d, ctx->lw, ctx->tfeat_d, features, scale, ctx->stream);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
    return FHG_OK;
}

int fhg_apply_internal(fhg_ctx* ctx, int level, int op, int precision, const void* in, const void* aux, void* out)
{
    if (!ctx) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    if (level < 0 || level >= ctx->nlevels) return fail(ctx, FHG_ERR_INVALID_ARG, "level %d out of range", level);
    if (!in || !out) return fail(ctx, FHG_ERR_INVALID_ARG, "null vector");
    CK(cudaSetDevice(ctx->device));
    int rc = FHG_OK;
    if (precision == FHG_PREC_FP64) {
        if (op == FHG_OP_VCYCLE_LEARNED) return fail(ctx, FHG_ERR_INVALID_ARG, "the learned step runs in the FP32 V-cycle");
        if (op == FHG_OP_VCYCLE && ctx->opts.vcycle_precision != FHG_PREC_FP64)
            return fail(ctx, FHG_ERR_INVALID_ARG, "FP64 V-cycle requested while the context runs FP32");
        rc = apply_device(ctx, level, op, (double*)in, (double*)aux, (double*)out);
    } else if (precision == FHG_PREC_FP32) {
        if (!ctx->levels[0].A32.vals) return fail(ctx, FHG_ERR_NOT_READY, "FP32 operators were not built at setup");
        if (op == FHG_OP_VCYCLE || op == FHG_OP_VCYCLE_LEARNED) {
            if (level != 0) return fail(ctx, FHG_ERR_INVALID_ARG, "V-cycle starts on level 0");
            if (op == FHG_OP_VCYCLE_LEARNED && !ctx->lwts) return fail(ctx, FHG_ERR_NOT_READY, "no network installed");
            ctx->learned_now = op == FHG_OP_VCYCLE_LEARNED;
            vcycle<float>(ctx, 0, (const float*)in, (float*)out);
            ctx->learned_now = false;
            if (op == FHG_OP_VCYCLE_LEARNED && (rc = check_learned_status(ctx))) return rc;
        } else if (op == FHG_OP_LEARNED_STEP) {
            if (level != 0 || !ctx->lwts || !aux) return fail(ctx, FHG_ERR_INVALID_ARG, "learned step: level 0, installed network, aux = b");
            if (out != in) CK(cudaMemcpyAsync(out, in, sizeof(float) * ctx->levels[0].n, cudaMemcpyDeviceToDevice, ctx->stream));
            learned_step(ctx, (const float*)aux, (float*)out);
            if ((rc = check_learned_status(ctx))) return rc;
        } else if (op == FHG_OP_SYM_SPMV) {
            return fail(ctx, FHG_ERR_INVALID_ARG, "the outer operator is FP64");
        } else {
            rc = apply_device_t<float>(ctx, level, op, (float*)in, (float*)aux, (float*)out);
        }
    } else if (precision == FHG_PREC_DF) {
        if (!ctx->levels[0].A2.vals) return fail(ctx, FHG_ERR_NOT_READY, "pair operators were not built at setup");
        if (op == FHG_OP_VCYCLE) {
            if (level != 0) return fail(ctx, FHG_ERR_INVALID_ARG, "V-cycle starts on level 0");
            vcycle<dfl>(ctx, 0, (const dfl*)in, (dfl*)out);
        } else if (op == FHG_OP_SYM_SPMV || op == FHG_OP_VCYCLE_LEARNED || op == FHG_OP_LEARNED_STEP) {
            return fail(ctx, FHG_ERR_INVALID_ARG, "op %d has no pair form", op);
        } else {
            rc = apply_device_t<dfl>(ctx, level, op, (dfl*)in, (dfl*)aux, (dfl*)out);
        }
    } else {
        return fail(ctx, FHG_ERR_INVALID_ARG, "unknown precision %d", precision);
    }
    if (rc) return rc;
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(ctx->stream));
    return FHG_OK;
}

}  // extern "C"

namespace {

int net_fail(fhg_net* net, int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (net) net->err = buf;
    return code;
}

#define NCK(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return net_fail(net, FHG_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));    \
    } while (0)

template <class T>
int net_alloc(fhg_net* net, T** p, size_t count, bool scratch)
{
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess)
        return net_fail(net, FHG_ERR_CUDA, "cudaMalloc(%zu bytes) failed: %s", count * sizeof(T), cudaGetErrorString(e));
    (scratch ? net->scratch : net->fixed).push_back(q);
    *p = (T*)q;
    return FHG_OK;
}

// Activation buffers for `rows` (a multiple of 64) faces.
int net_reserve(fhg_net* net, long long rows)
{
    using namespace fhg::learned;
    if (rows <= net->rows_cap) return FHG_OK;
    for (void* p : net->scratch) cudaFree(p);
    net->scratch.clear();
    net->rows_cap = 0;
    const size_t R = (size_t)rows;
    int rc;
    if ((rc = net_alloc(net, &net->feat, R * kIn, true)) || (rc = net_alloc(net, &net->h1, R * kHid, true)) ||
        (rc = net_alloc(net, &net->h2, R * kHid, true)) || (rc = net_alloc(net, &net->dy, R * kOut, true)) ||
        (rc = net_alloc(net, &net->d2, R * kHid, true)) || (rc = net_alloc(net, &net->d1, R * kHid, true)) ||
        (rc = net_alloc(net, &net->a1, R * kHid, true)) || (rc = net_alloc(net, &net->a2, R * kHid, true)) ||
        (rc = net_alloc(net, &net->y, R * kOut, true)) || (rc = net_alloc(net, &net->dh, R * kHid, true)) ||
        (rc = net_alloc(net, &net->scale, R, true)) || (rc = net_alloc(net, &net->c, R * kMaxLearnedBs, true)) ||
        (rc = net_alloc(net, &net->q, R * kMaxLearnedBs, true)))
        return rc;
    net->rows_cap = rows;
    return FHG_OK;
}

}  // namespace

extern "C" {

int fhg_net_num_params(void) { return fhg::learned::kParams; }

int fhg_net_create(fhg_net** out, int device)
{
    using namespace fhg::learned;
    if (!out) return FHG_ERR_INVALID_ARG;
    fhg_net* net = new fhg_net();
    *out = net;
    net->device = device;
    NCK(cudaSetDevice(device));
    int rc;
    if ((rc = net_alloc(net, &net->params, kParams, false)) || (rc = net_alloc(net, &net->grad, kParams, false)) ||
        (rc = net_alloc(net, &net->m, kParams, false)) || (rc = net_alloc(net, &net->v, kParams, false)) ||
        (rc = net_alloc(net, &net->wts, kWeights, false)) || (rc = net_alloc(net, &net->bias, kBiases, false)) ||
        (rc = net_alloc(net, &net->gparts, (size_t)64 * kHid * kHid, false)) ||
        (rc = net_alloc(net, &net->cparts, (size_t)kColsumChunks * kHid, false)) ||
        (rc = net_alloc(net, &net->lparts, (size_t)fhg::kReduceCtas, false)))
        return rc;
    NCK(cudaMallocHost(&net->lparts_host, sizeof(double) * fhg::kReduceCtas));
    NCK(cudaMemset(net->params, 0, sizeof(float) * kParams));
    NCK(cudaMemset(net->m, 0, sizeof(float) * kParams));
    NCK(cudaMemset(net->v, 0, sizeof(float) * kParams));
    fhg::launch_split_params(net->params, net->wts, net->bias, 0);
    NCK(cudaDeviceSynchronize());
    return FHG_OK;
}

void fhg_net_destroy(fhg_net* net)
{
    if (!net) return;
    cudaSetDevice(net->device);
    for (void* p : net->scratch) cudaFree(p);
    for (void* p : net->fixed) cudaFree(p);
    if (net->lparts_host) cudaFreeHost(net->lparts_host);
    delete net;
}

const char* fhg_net_last_error(const fhg_net* net) { return net ? net->err.c_str() : "null network"; }

int fhg_net_set_params(fhg_net* net, const float* params, int n_params)
{
    using namespace fhg::learned;
    if (!net || !params) return FHG_ERR_INVALID_ARG;
    if (n_params != kParams) return net_fail(net, FHG_ERR_INVALID_ARG, "%d parameters given, the network has %d", n_params, kParams);
    NCK(cudaSetDevice(net->device));
    NCK(cudaMemcpy(net->params, params, sizeof(float) * kParams, cudaMemcpyHostToDevice));
    NCK(cudaMemset(net->m, 0, sizeof(float) * kParams));
    NCK(cudaMemset(net->v, 0, sizeof(float) * kParams));
    net->step = 0;
    fhg::launch_split_params(net->params, net->wts, net->bias, 0);
    NCK(cudaDeviceSynchronize());
    return FHG_OK;
}

int fhg_net_get_params(const fhg_net* net, float* params, int n_params)
{
    using namespace fhg::learned;
    if (!net || !params || n_params != kParams) return FHG_ERR_INVALID_ARG;
    if (cudaSetDevice(net->device) != cudaSuccess) return FHG_ERR_CUDA;
    if (cudaMemcpy(params, net->params, sizeof(float) * kParams, cudaMemcpyDeviceToHost) != cudaSuccess) return FHG_ERR_CUDA;
    return FHG_OK;
}

int fhg_net_train_step(fhg_net* net, fhg_ctx* ctx, const float* r, double energy, float lr, float weight_decay,
                       int update, double* loss, float* grad)
{
    using namespace fhg::learned;
    if (!net || !ctx || !r) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready || !ctx->nbr_d)
        return net_fail(net, FHG_ERR_NOT_READY, "the context has no learned-step data (FP32 setup, bs 2..4)");
    if (net->device != ctx->device) return net_fail(net, FHG_ERR_INVALID_ARG, "network and context on different devices");
    if (!(energy > 0) || !std::isfinite(energy)) return net_fail(net, FHG_ERR_INVALID_ARG, "the energy e.Ae must be positive");
    NCK(cudaSetDevice(ctx->device));
    Level& L = ctx->levels[0];
    const int nb = L.nb, bs = L.bs;
    const long long R = ((long long)nb + 63) / 64 * 64;
    int rc = net_reserve(net, R);
    if (rc) return rc;
    cudaStream_t s = ctx->stream;
    const uint16_t* W1 = net->wts;
    const uint16_t* W2 = W1 + kHid * kIn;
    const uint16_t* W3 = W2 + kHid * kHid;
    const float* b1 = net->bias;
    const float* b2 = b1 + kHid;
    const float* b3 = b2 + kHid;
    const int M = (int)R;
    // Forward over every face of the field, the correction, and q = A c.
    fhg::launch_block_diag(nb, bs, L.dinv32, nb, r, ctx->lw, s);
    fhg::launch_features(nb, M, bs, ctx->nbr_d, ctx->lw, ctx->tfeat_d, net->feat, net->scale, s);
    fhg::launch_gemm(kGemmFwdHid, M, kIn, net->feat, kIn, W1, kIn, net->a1, nullptr, 1, 0, s);
    fhg::launch_bias_gelu(R, net->a1, b1, net->h1, s);
    fhg::launch_gemm(kGemmFwdHid, M, kHid, net->h1, kHid, W2, kHid, net->a2, nullptr, 1, 0, s);
    fhg::launch_bias_gelu(R, net->a2, b2, net->h2, s);
    fhg::launch_gemm(kGemmFwdOut, M, kHid, net->h2, kHid, W3, kHid, net->y, nullptr, 1, 0, s);
    fhg::launch_correction(nb, bs, net->y, b3, net->scale, net->c, s);
    fhg::launch_spmv<float>(L.A32.v, fhg::kSpmvAssign, net->c, nullptr, net->q, s);
    fhg::launch_energy_grad(nb, M, bs, r, net->q, net->c, net->scale, 1.0 / energy, net->dy, net->lparts, s);
    // Backward (weight gradients reduced over the faces in fixed-order K splits).
    float* g = net->grad;
    const int ns = (int)std::max(1LL, std::min(64LL, R / 512));
    fhg::launch_colsum(R, kOut, net->dy, net->cparts, g + kOffB3, s);
    fhg::launch_gemm(kGemmGradHid, kOut, M, net->dy, kOut, net->h2, kHid, g + kOffW3, net->gparts, ns, 0, s);
    fhg::launch_gemm(kGemmBwdData, M, kOut, net->dy, kOut, W3, kHid, net->dh, nullptr, 1, 0, s);
    fhg::launch_gelu_back(R * kHid, net->dh, net->a2, net->d2, s);
    fhg::launch_colsum(R, kHid, net->d2, net->cparts, g + kOffB2, s);
    fhg::launch_gemm(kGemmGradHid, kHid, M, net->d2, kHid, net->h1, kHid, g + kOffW2, net->gparts, ns, 0, s);
    fhg::launch_gemm(kGemmBwdData, M, kHid, net->d2, kHid, W2, kHid, net->dh, nullptr, 1, 0, s);
    fhg::launch_gelu_back(R * kHid, net->dh, net->a1, net->d1, s);
    fhg::launch_colsum(R, kHid, net->d1, net->cparts, g + kOffB1, s);
    fhg::launch_gemm(kGemmGradIn, kHid, M, net->d1, kHid, net->feat, kIn, g + kOffW1, net->gparts, ns, 0, s);
    NCK(cudaMemcpyAsync(net->lparts_host, net->lparts, sizeof(double) * fhg::kReduceCtas, cudaMemcpyDeviceToHost, s));
    if (grad) NCK(cudaMemcpyAsync(grad, g, sizeof(float) * kParams, cudaMemcpyDeviceToHost, s));
    if (update) {
        net->step++;
        fhg::launch_adam(kParams, net->params, g, net->m, net->v, lr, 0.9f, 0.999f, 1e-8f, net->step, weight_decay, s);
        fhg::launch_split_params(net->params, net->wts, net->bias, s);
    }
    NCK(cudaGetLastError());
    NCK(cudaStreamSynchronize(s));
    if (loss) {
        double t = 0.0;
        for (int i = 0; i < fhg::kReduceCtas; i++) t += net->lparts_host[i];
        *loss = 1.0 + t / energy;
    }
    return FHG_OK;
}

// ---------------------------------------------------------------------------
// Batched solve (no counterpart in the reference)

int fhg_io_buffers(fhg_ctx* ctx, double** b_dev, double** x_dev)
{
    if (!ctx || !b_dev || !x_dev) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    *b_dev = ctx->io;
    *x_dev = ctx->io + ctx->levels[0].n;
    return FHG_OK;
}

int fhg_io_upload(fhg_ctx* ctx, const double* b)
{
    if (!ctx || !b) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    CK(cudaSetDevice(ctx->device));
    CK(cudaMemcpyAsync(ctx->io, b, sizeof(double) * ctx->levels[0].n, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return FHG_OK;
}

int fhg_io_download(fhg_ctx* ctx, double* x)
{
    if (!ctx || !x) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return fail(ctx, FHG_ERR_NOT_READY, "fhg_setup has not completed");
    CK(cudaSetDevice(ctx->device));
    const long long n = ctx->levels[0].n;
    CK(cudaMemcpyAsync(x, ctx->io + n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return FHG_OK;
}

}  // extern "C"

namespace {

int batch_fail(fhg_batch* b, int code, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (b) b->err = buf;
    return code;
}

#define BCK(call)                                                                                  \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return batch_fail(batch, FHG_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

// Start of a solve on the device (run_solve's prelude): b' = Pi b, x = 0, r = b, direction
// placeholders, ||b||, scalars and counter.
void batch_prelude(fhg_ctx* ctx)
{
    Level& L0 = ctx->levels[0];
    const long long n = L0.n;
    cudaStream_t s = ctx->stream;
    fhg::launch_permute<double>(L0.nb, L0.bs, L0.perm_d, ctx->io, ctx->kb, true, s);
    cudaMemsetAsync(ctx->kx, 0, sizeof(double) * n, s);
    cudaMemcpyAsync(ctx->kr, ctx->kb, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
    for (int q = 0; q < 2; q++) {
        cudaMemsetAsync(ctx->kz[q], 0, sizeof(double) * n, s);
        cudaMemsetAsync(ctx->kAd[q], 0, sizeof(double) * n, s);
    }
    fhg::launch_dot(n, ctx->kb, ctx->kb, part(ctx, 0), s);
    fhg::launch_sqrt_sum(part(ctx, 0), ctx->scal + 0, s);
    // residual replacement in the device loop as in run_solve: with the FP32 V-cycle, or when asked
    const bool replace = ctx->opts.krylov == FHG_KRYLOV_FCG &&
                         (ctx->opts.vcycle_precision == FHG_PREC_FP32 || ctx->opts.replace_residual);
    fhg::launch_init_solve(ctx->scal, ctx->counter_d, s, ctx->loop_state, replace ? 8 : 0);
    if (outer_df(ctx)) outer_df_start(ctx, ctx->kr);
    else if (ctx->opts.vcycle_precision == FHG_PREC_FP32) fhg::launch_convert<double, float>(n, ctx->kr, L0.b32, s);
}

// The true residual t = b - A x on the device: FP64, and again in compensated arithmetic when the FP64
// one misses the tolerance (run_solve's rule); scal[5] = ||t||. replace = 1 (inside the device loop):
// r = t and go on while replacements are left, when the true residual misses the tolerance.
void device_true_residual(fhg_ctx* ctx, int replace)
{
    Level& L0 = ctx->levels[0];
    const long long n = L0.n;
    cudaStream_t s = ctx->stream;
    const double tol = ctx->opts.tolerance;
    fhg::launch_spmv<double>(L0.A.v, fhg::kSpmvResidual, ctx->kx, ctx->kb, ctx->kt, s);
    fhg::launch_dot(n, ctx->kt, ctx->kt, part(ctx, 0), s);
    fhg::launch_check_fp64(part(ctx, 0), ctx->scal, tol, ctx->loop_state, s);
    fhg::launch_residual_comp(L0.A.v, ctx->kx, ctx->kb, ctx->kt, part(ctx, 1), s, ctx->loop_state + fhg::kLoopNeedComp);
    fhg::launch_check_comp(part(ctx, 1), ctx->scal, tol, ctx->loop_state, replace, s);
    if (replace) {
        const bool df = outer_df(ctx);
        fhg::launch_replace_apply(n, ctx->loop_state, ctx->kt, ctx->kr, df ? outer_rh(ctx) : nullptr,
                                  df ? ctx->rlo : nullptr, df ? outer_r2(ctx) : nullptr,
                                  !df && ctx->opts.vcycle_precision == FHG_PREC_FP32 ? L0.b32 : nullptr, s);
    }
}

// End of a solve: the true residual into scal[5] (||b - A x||), x = Pi^T x'.
void batch_epilogue(fhg_ctx* ctx)
{
    Level& L0 = ctx->levels[0];
    const long long n = L0.n;
    device_true_residual(ctx, 0);
    fhg::launch_permute<double>(L0.nb, L0.bs, L0.perm_d, ctx->kx, ctx->io + n, false, ctx->stream);
}

// Capture `fn(ctx)` on the context's stream into `g` (a new graph when g is null, else the given
// body graph).
template <class F>
cudaError_t capture(fhg_ctx* ctx, cudaGraph_t* g, bool into, F fn)
{
    cudaError_t e = into ? cudaStreamBeginCaptureToGraph(ctx->stream, *g, nullptr, nullptr, 0,
                                                         cudaStreamCaptureModeThreadLocal)
                         : cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return e;
    fn(ctx);
    cudaGraph_t out = nullptr;
    e = cudaStreamEndCapture(ctx->stream, &out);
    if (e == cudaSuccess && !into) *g = out;
    return e;
}

int batch_build(fhg_batch* batch)
{
    cudaGraph_t top = nullptr;
    BCK(cudaGraphCreate(&top, 0));
    batch->body_kernels.assign(batch->probs.size(), 0);
    batch->check_kernels.assign(batch->probs.size(), 0);
    batch->fixed_kernels = 0;
    int rc = FHG_OK;
    for (size_t i = 0; i < batch->probs.size() && rc == FHG_OK; i++) {
        fhg_ctx* ctx = batch->probs[i];
        cudaError_t e = cudaSuccess;
        const long long k0 = fhg::g_kernel_launches.load();
        cudaGraph_t pre = nullptr, post = nullptr;
        cudaGraphNode_t npre = nullptr, nwhile = nullptr, npost = nullptr;
        e = capture(ctx, &pre, false, batch_prelude);
        if (e == cudaSuccess) e = cudaGraphAddChildGraphNode(&npre, top, nullptr, 0, pre);
        const long long k1 = fhg::g_kernel_launches.load();
        long long kc0 = 0, kc1 = 0;
        cudaGraphConditionalHandle h = 0;
        if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, top, 1, cudaGraphCondAssignDefault);
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        if (e == cudaSuccess) e = cudaGraphAddNode(&nwhile, top, &npre, nullptr, 1, &cp);
        if (e == cudaSuccess) {
            // Body: one FCG iteration, the stopping test, an IF node that checks the true residual once
            // the recursive one meets the tolerance (replacing r when it misses), then the WHILE
            // condition.
            cudaGraph_t body = cp.conditional.phGraph_out[0];
            cudaGraph_t check_body = nullptr;
            ctx->device_loop = true;
            const double tol = ctx->opts.tolerance;
            const int maxit = ctx->opts.max_iterations;
            cudaGraphConditionalHandle hc = 0;
            e = cudaGraphConditionalHandleCreate(&hc, body, 0, cudaGraphCondAssignDefault);
            if (e == cudaSuccess)
                e = capture(ctx, &body, true, [&](fhg_ctx* c) {
                    fcg_iteration(c, 0);
                    const long long n = c->levels[0].n;
                    fhg::launch_copy2(n, c->kz[0], c->kz[1], c->kAd[0], c->kAd[1], c->stream);
                    fhg::launch_loop_decide(c->scal + 2, c->counter_d, tol, maxit, c->loop_state, hc, c->stream);
                    // the IF node, appended to the graph being captured
                    cudaStreamCaptureStatus st;
                    cudaGraph_t g = nullptr;
                    const cudaGraphNode_t* deps = nullptr;
                    const cudaGraphEdgeData* edges = nullptr;   // queried (a query without them can be lossy),
                    size_t nd = 0;                              // then the IF node gets default full edges
                    cudaError_t ce = cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, &deps, &edges, &nd);
                    std::vector<cudaGraphNode_t> dv;
                    if (ce == cudaSuccess) dv.assign(deps, deps + nd);
                    cudaGraphNodeParams ip = {};
                    ip.type = cudaGraphNodeTypeConditional;
                    ip.conditional.handle = hc;
                    ip.conditional.type = cudaGraphCondTypeIf;
                    ip.conditional.size = 1;
                    cudaGraphNode_t nif = nullptr;
                    if (ce == cudaSuccess) ce = cudaGraphAddNode(&nif, g, dv.data(), nullptr, dv.size(), &ip);
                    if (ce == cudaSuccess)
                        ce = cudaStreamUpdateCaptureDependencies(c->stream, &nif, nullptr, 1,
                                                                 cudaStreamSetCaptureDependencies);
                    if (ce == cudaSuccess) check_body = ip.conditional.phGraph_out[0];
                    fhg::launch_loop_finish(c->loop_state, h, c->stream);
                });
            if (e == cudaSuccess && !check_body) e = cudaErrorStreamCaptureInvalidated;
            kc0 = fhg::g_kernel_launches.load();
            if (e == cudaSuccess) e = capture(ctx, &check_body, true, [&](fhg_ctx* c) { device_true_residual(c, 1); });
            kc1 = fhg::g_kernel_launches.load();
            ctx->device_loop = false;
        }
        const long long k2 = fhg::g_kernel_launches.load();
        if (e == cudaSuccess) e = capture(ctx, &post, false, batch_epilogue);
        if (e == cudaSuccess) e = cudaGraphAddChildGraphNode(&npost, top, &nwhile, 1, post);
        const long long k3 = fhg::g_kernel_launches.load();
        fhg::g_kernel_launches -= (k3 - k0);  // captured, not executed
        batch->fixed_kernels += (k1 - k0) + (k3 - k2);
        batch->body_kernels[i] = (k2 - k1) - (kc1 - kc0);
        batch->check_kernels[i] = kc1 - kc0;
        if (pre) cudaGraphDestroy(pre);
        if (post) cudaGraphDestroy(post);
        if (e != cudaSuccess) rc = batch_fail(batch, FHG_ERR_CUDA, "problem %zu: graph construction: %s", i, cudaGetErrorString(e));
    }
    if (rc == FHG_OK) {
        cudaError_t e = cudaGraphInstantiate(&batch->exec, top, 0);
        if (e != cudaSuccess) rc = batch_fail(batch, FHG_ERR_CUDA, "graph instantiation: %s", cudaGetErrorString(e));
    }
    cudaGraphDestroy(top);
    return rc;
}

}  // namespace

extern "C" {

int fhg_batch_create(fhg_batch** out, int device)
{
    if (!out) return FHG_ERR_INVALID_ARG;
    fhg_batch* batch = new fhg_batch();
    *out = batch;
    batch->device = device;
    BCK(cudaSetDevice(device));
    BCK(cudaStreamCreateWithFlags(&batch->stream, cudaStreamNonBlocking));
    BCK(cudaEventCreate(&batch->ev0));
    BCK(cudaEventCreate(&batch->ev1));
    return FHG_OK;
}

void fhg_batch_destroy(fhg_batch* batch)
{
    if (!batch) return;
    cudaSetDevice(batch->device);
    if (batch->exec) cudaGraphExecDestroy(batch->exec);
    if (batch->ev0) cudaEventDestroy(batch->ev0);
    if (batch->ev1) cudaEventDestroy(batch->ev1);
    if (batch->stream) cudaStreamDestroy(batch->stream);
    delete batch;
}

const char* fhg_batch_last_error(const fhg_batch* batch) { return batch ? batch->err.c_str() : "null batch"; }

int fhg_batch_add(fhg_batch* batch, fhg_ctx* ctx)
{
    if (!batch || !ctx) return FHG_ERR_INVALID_ARG;
    if (!ctx->ready) return batch_fail(batch, FHG_ERR_NOT_READY, "the context has not been set up");
    if (ctx->device != batch->device) return batch_fail(batch, FHG_ERR_INVALID_ARG, "context on device %d, batch on %d", ctx->device, batch->device);
    if (ctx->opts.krylov != FHG_KRYLOV_FCG) return batch_fail(batch, FHG_ERR_UNSUPPORTED, "the batched solve runs FCG");
    if (ctx->opts.w_loops == FHG_CYCLE_K)
        return batch_fail(batch, FHG_ERR_UNSUPPORTED, "the K-cycle decides on the host: not in a batched solve");
    if (ctx->learned_mode != FHG_LEARNED_OFF) return batch_fail(batch, FHG_ERR_UNSUPPORTED, "the batched solve runs the plain V-cycle");
    for (fhg_ctx* c : batch->probs)
        if (c == ctx) return batch_fail(batch, FHG_ERR_INVALID_ARG, "context added twice");
    if (batch->exec) {
        cudaGraphExecDestroy(batch->exec);
        batch->exec = nullptr;
    }
    batch->probs.push_back(ctx);
    return FHG_OK;
}

int fhg_batch_solve(fhg_batch* batch, fhg_solve_info* infos, double* elapsed_ms)
{
    if (!batch) return FHG_ERR_INVALID_ARG;
    if (batch->probs.empty()) return batch_fail(batch, FHG_ERR_INVALID_ARG, "empty batch");
    BCK(cudaSetDevice(batch->device));
    bool stale = !batch->exec || batch->epochs.size() != batch->probs.size();
    for (size_t i = 0; i < batch->probs.size(); i++) {
        fhg_ctx* c = batch->probs[i];
        if (!c->ready) return batch_fail(batch, FHG_ERR_NOT_READY, "a context of the batch is not set up");
        if (!stale && batch->epochs[i] != c->epoch) stale = true;  // set up again since the graph was built
        BCK(cudaStreamSynchronize(c->stream));
    }
    if (stale) {
        if (batch->exec) {
            cudaGraphExecDestroy(batch->exec);
            batch->exec = nullptr;
        }
        int rc = batch_build(batch);
        if (rc) return rc;
        batch->epochs.clear();
        for (fhg_ctx* c : batch->probs) batch->epochs.push_back(c->epoch);
    }
    BCK(cudaEventRecord(batch->ev0, batch->stream));
    BCK(cudaGraphLaunch(batch->exec, batch->stream));
    BCK(cudaEventRecord(batch->ev1, batch->stream));
    BCK(cudaEventSynchronize(batch->ev1));
    float ms = 0;
    BCK(cudaEventElapsedTime(&ms, batch->ev0, batch->ev1));
    if (elapsed_ms) *elapsed_ms = ms;
    int status = FHG_OK;
    long long kernels = batch->fixed_kernels;
    for (size_t i = 0; i < batch->probs.size(); i++) {
        fhg_ctx* c = batch->probs[i];
        double sc[6];
        int counter = 0;
        int state[4] = {0, 0, 0, 0};
        BCK(cudaMemcpy(sc, c->scal, sizeof(sc), cudaMemcpyDeviceToHost));
        BCK(cudaMemcpy(&counter, c->counter_d, sizeof(int), cudaMemcpyDeviceToHost));
        BCK(cudaMemcpy(state, c->loop_state, sizeof(state), cudaMemcpyDeviceToHost));
        const int its = counter - 1;
        kernels += (long long)its * batch->body_kernels[i];
        // true-residual checks that ran: one per replacement, plus the last one when replacement is on
        const bool replace = c->opts.krylov == FHG_KRYLOV_FCG &&
                             (c->opts.vcycle_precision == FHG_PREC_FP32 || c->opts.replace_residual);
        if (replace) kernels += (long long)(8 - state[fhg::kLoopReplaceLeft] + 1) * batch->check_kernels[i];
        int st = FHG_OK;
        if (std::isinf(sc[2])) st = FHG_ERR_DIVERGED;
        else if (std::isnan(sc[2])) st = FHG_ERR_NAN;
        if (st != FHG_OK && status == FHG_OK) status = st;
        if (infos) {
            infos[i].iterations = its;
            infos[i].status = st;
            infos[i].normalized_residual = sc[2];
            infos[i].solve_ms = ms;
            infos[i].learned_iterations = 0;
            infos[i].true_relative_residual = st == FHG_OK ? (sc[0] > 0 ? sc[5] / sc[0] : sc[5]) : -1.0;
        }
    }
    fhg::g_kernel_launches += kernels;
    if (status != FHG_OK) batch_fail(batch, status, "a problem of the batch diverged or produced NaN");
    return status;
}

}  // extern "C"
