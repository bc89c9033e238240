// Internal declarations shared by the host side (fhg_api.cu) and the kernels
// (fhg_kernels.cu) of libfhg.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "fhg_pair.h"

namespace fhg {

// Device block-sparse-row operator. Block values are stored entry-major
// ("structure of arrays"): entry e = r*bs + c of stored block p lives at
// vals[e * ld + p], ld = nnzb rounded up to a multiple of 32, so that the lanes of a
// warp walking consecutive blocks read consecutive addresses for every entry.
template <class T>
struct BsrView {
    int nbr = 0;          // block rows
    int nbc = 0;          // block columns
    int bs = 0;           // block size (square blocks)
    int lanes = 8;        // lanes per block row (power of two, 4..32)
    int unroll = 1;       // blocks per lane step in the row walk (1 or 2; 2 only for bs <= 3)
    long long nnzb = 0;   // stored blocks
    long long ld = 0;     // leading dimension of vals
    int ell = 0;          // > 0: padded rows of `ell` slots, slot s of row i at i * ell + s, empty
                          // slots with zero values and an in-range column, rowptr unused (accepted
                          // by launch_spmv, launch_gs and launch_residual_dinv; Jacobi needs rowptr)
    int slot_major = 0;   // with ell > 0 (GS views only): slot s of row i of a colour [c0, c1) at
                          // c0 * ell + s * (c1 - c0) + (i - c0), swept one thread per row
    const int* rowptr = nullptr;
    const int* colidx = nullptr;
    const T* vals = nullptr;
    // Jagged view (JDS, the transfer operators): rows sorted by decreasing block count, row
    // jds_perm[k] in sorted place k, its slot s at jds_start[s] + k (jds_start[s + 1] - jds_start[s]
    // rows have more than s blocks); no padding, rowptr unused; products only (assign, add-to).
    const int* jds_perm = nullptr;
    const int* jds_start = nullptr;
    int jds_slots = 0;
};

// Fixed number of CTAs of the reduction kernels: the partial-sum arrays they write
// have exactly this many entries per quantity, and every consumer reduces them in the
// same fixed order, so the Krylov scalars are bitwise reproducible run to run.
constexpr int kReduceCtas = 608;   // 4 x 152 SMs
constexpr int kReduceThreads = 256;

// Process-wide count of kernels launched by this library.
extern std::atomic<long long> g_kernel_launches;

enum SpmvMode { kSpmvAssign = 0, kSpmvResidual = 1, kSpmvAddTo = 2 };

template <class T>
void launch_spmv(const BsrView<T>& A, int mode, const T* x, const T* aux, T* y, cudaStream_t s);
// col_lo/col_hi: block columns outside [col_lo, col_hi) are skipped (zero-start sweeps).
// A may be a padded (ell > 0) view of the off-diagonal blocks. omega != 1: block SOR,
// x_i <- omega D_i^-1 (b_i - sum_{j != i} A_ij x_j) + (1 - omega) x_i.
template <class T>
void launch_gs(const BsrView<T>& A, int row0, int row1, const T* dinv, long long dld,
               const T* b, T* x, cudaStream_t s, int col_lo = 0, int col_hi = 0x7fffffff, T omega = T(1));
template <class T>
void launch_jacobi(const BsrView<T>& A, const T* dinv, long long dld, T omega, const T* b,
                   const T* xold, T* xnew, cudaStream_t s);
// Ad = A d with per-CTA partials of d.Ad (partials[0..kReduceCtas)) and r.d
// (partials[kReduceCtas..2*kReduceCtas)).
void launch_spmv_dots(const BsrView<double>& A, const double* d, const double* r, double* Ad,
                      double* partials, cudaStream_t s);
// x = Cinv b, Cinv dense n x n row-major FP64; b, x in T.
template <class T>
void launch_coarse(int n, const double* cinv, const T* b, T* x, cudaStream_t s);
// r = b - A x in compensated (Dot2) FP64 summation, accurate to about one unit of r_i; partials of r.r.
// A must be the CSR form (rowptr). enable (optional, device): the kernel returns at once if *enable == 0.
void launch_residual_comp(const BsrView<double>& A, const double* x, const double* b, double* r, double* partials,
                          cudaStream_t s, const int* enable = nullptr);
// partials[0..kReduceCtas) of sum a_i b_i.
void launch_dot(long long n, const double* a, const double* b, double* partials, cudaStream_t s);
// FCG(1) direction: s = sum(partials_zadp) / *dadp; d = z - s * dp (d may alias z).
void launch_fcg_direction(long long n, const double* z, const double* dp, const double* partials_zadp,
                          const double* dadp, double* d, cudaStream_t s);
// FCG/CG step: alpha = num / den with num, den reduced from partials (num_off, den_off offsets);
// x += alpha d; r -= alpha Ad; partials_rr = per-CTA sum r_i^2; *den_out = den (if not null).
// r32 (optional): FP32 copy of the updated r, the next V-cycle's right-hand side.
void launch_krylov_step(long long n, double* x, double* r, const double* d, const double* Ad,
                        const double* partials_num, const double* partials_den, double* den_out,
                        double* partials_rr, cudaStream_t s, float* r32 = nullptr);
// FP32 preconditioned residual z into the FP64 FCG: partials of z.Adp; d = z - s dp.
void launch_dot_mixed(long long n, const float* a, const double* b, double* partials, cudaStream_t s);
// (dhi, dlo optional: FP32 pair of d for the double-FP32 outer product)
void launch_fcg_direction_mixed(long long n, const float* z, const double* dp, const double* partials_zadp,
                                const double* dadp, double* d, cudaStream_t s, float* dhi = nullptr,
                                float* dlo = nullptr);
// Double-FP32 outer iteration (FP32 pairs hi + lo for r, d, Ad; FP64 x and Krylov scalars).
// Ad = Â d (Â = hi + lo), partials as launch_spmv_dots (d.Ad, then r.d).
void launch_spmv_dots_df(const BsrView<float>& Ahi, const float* vlo, const float* dhi, const float* dlo,
                         const float* rhi, const float* rlo, float* Adhi, float* Adlo, double* partials,
                         cudaStream_t s);
// The same on the slot-major pair view of Â (ell = 5..8 slots; bs 2, 3, 4, 6).
void launch_spmv_dots_df_slot(const BsrView<dfl>& A, const float* dhi, const float* dlo, const float* rhi,
                              const float* rlo, float* Adhi, float* Adlo, double* partials, cudaStream_t s);
// partials of z.Adp (z FP32, or z2 non-null: the pair V-cycle's output as interleaved pairs).
void launch_dot_df(long long n, const float* z, const float* ah, const float* al, double* partials, cudaStream_t s,
                   const dfl* z2 = nullptr);
// d = z - s dp, s = sum(partials_zadp) / *dadp (z as in launch_dot_df).
void launch_fcg_direction_df(long long n, const float* z, const float* dph, const float* dpl,
                             const double* partials_zadp, const double* dadp, float* dh, float* dl, cudaStream_t s,
                             const dfl* z2 = nullptr);
// As launch_krylov_step with r, d, Ad as pairs; rh doubles as the next V-cycle's FP32 right-hand side,
// r2 (optional) receives r as interleaved pairs, the pair V-cycle's right-hand side.
void launch_krylov_step_df(long long n, double* x, float* rh, float* rl, const float* dh, const float* dl,
                           const float* Adh, const float* Adl, const double* partials_num,
                           const double* partials_den, double* den_out, double* partials_rr, cudaStream_t s,
                           dfl* r2 = nullptr);
// v -> (h, l) and, optionally, v2 interleaved.
void launch_split_df(long long n, const double* v, float* h, float* l, cudaStream_t s, dfl* v2 = nullptr);
// ||r|| / ||b||: reduces partials_rr, divides by *bnorm, writes *nr_out and hist[*counter],
// then ++*counter.
void launch_finalize_norm(const double* partials_rr, const double* bnorm, double* nr_out,
                          double* hist, int* counter, int hist_len, cudaStream_t s);
// *out = sqrt(sum partials).
void launch_sqrt_sum(const double* partials, double* out, cudaStream_t s);
// *out = sum partials.
void launch_sum(const double* partials, double* out, cudaStream_t s);
// CG direction: d = z + (*beta) d.
void launch_cg_direction(long long n, const double* z, const double* beta, double* d, cudaStream_t s);
// CG: rz_new = sum(partials); *beta = rz_new / *rz; *rz = rz_new.
void launch_cg_beta(const double* partials, double* rz, double* beta, cudaStream_t s);
// CG step numerator from a device scalar: alpha = *num / sum(partials_den).
void launch_cg_step(long long n, double* x, double* r, const double* d, const double* Ad,
                    const double* num, const double* partials_den, double* partials_rr, cudaStream_t s);

template <class Tin, class Tout>
void launch_convert(long long n, const Tin* in, Tout* out, cudaStream_t s);
// K-cycle: partials[q * kReduceCtas ..] of a_q . b_q for q < nq (FP64 accumulation); y += alpha x;
// out = a c + b d.
template <class T>
void launch_dots3(long long n, int nq, const T* a0, const T* b0, const T* a1, const T* b1, const T* a2, const T* b2,
                  double* partials, cudaStream_t s);
template <class T>
void launch_axpy(long long n, double alpha, const T* x, T* y, cudaStream_t s);
template <class T>
void launch_lincomb(long long n, double a, const T* c, double b, const T* d, T* out, cudaStream_t s);
// Device-side solve loop: b0 = a0 and b1 = a1; solve scalars, iteration counter and loop state at
// their start values.
void launch_copy2(long long n, const double* a0, double* b0, const double* a1, double* b1, cudaStream_t s);
// Device-loop state per context (int[4]): replacements left, go on, compensated check needed.
constexpr int kLoopReplaceLeft = 0, kLoopGo = 1, kLoopNeedComp = 2;
void launch_init_solve(double* scal, int* counter, cudaStream_t s, int* state = nullptr, int replacements = 0);
// After an iteration of the device loop: state[kLoopGo] and the IF condition `check` (true-residual check).
void launch_loop_decide(const double* nr, const int* counter, double tol, int maxit, int* state,
                        cudaGraphConditionalHandle check, cudaStream_t s);
// True-residual checks (partials of r.r): FP64, then compensated when state[kLoopNeedComp].
void launch_check_fp64(const double* partials, double* scal, double tol, int* state, cudaStream_t s);
void launch_check_comp(const double* partials, double* scal, double tol, int* state, int replace, cudaStream_t s);
void launch_replace_apply(long long n, const int* state, const double* t, double* r, float* rh, float* rl, dfl* r2,
                          float* b32, cudaStream_t s);
// The WHILE node's condition from state[kLoopGo].
void launch_loop_finish(const int* state, cudaGraphConditionalHandle loop, cudaStream_t s);
// gather: out[b*bs+c] = in[perm[b]*bs+c]; scatter: out[perm[b]*bs+c] = in[b*bs+c].
template <class T>
void launch_permute(int nb, int bs, const int* perm, const T* in, T* out, bool gather, cudaStream_t s);
// The natural injection between face degrees (nh fine, nl coarse unknowns per face, fine block i ->
// coarse block map[i]): prolong: out = aux + P in (aux may be NULL or out); else out = P^T in.
template <class T>
void launch_inject(int nb, int nh, int nl, const int* map, const T* in, const T* aux, T* out, bool prolong,
                   cudaStream_t s);

// ---------------------------------------------------------------------------
// Learned correction step (fhg_learned.cu)

namespace learned {
constexpr int kIn = 48;            // network input per face
constexpr int kHid = 128;          // two hidden layers
constexpr int kOut = 16;           // output rows (the first bs are the correction)
constexpr int kResidualSlots = 32; // input [0, 32): scaled residual of the face and 6 neighbours (7 bs used)
constexpr int kTensorSlots = 16;   // input [32, 48): two element tensors (2 x 6) and 4 zeros
constexpr int kNeighbours = 6;
constexpr int kMaxLearnedBs = 4;
// FP32 master parameter layout: W1 [128][48], b1, W2 [128][128], b2, W3 [16][128], b3.
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kHid * kIn;
constexpr int kOffW2 = kOffB1 + kHid;
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;
constexpr int kOffB3 = kOffW3 + kOut * kHid;
constexpr int kParams = kOffB3 + kOut;
constexpr int kWeights = kHid * kIn + kHid * kHid + kOut * kHid;  // BF16 copy: W1, W2, W3
constexpr int kBiases = 2 * kHid + kOut;                           // FP32: b1, b2, b3
constexpr int kColsumChunks = 256;
enum GemmKind { kGemmFwdHid = 0, kGemmFwdOut = 1, kGemmBwdData = 2, kGemmGradHid = 3, kGemmGradIn = 4 };
}  // namespace learned

bool learned_supports(int bs);
// w = D^-1 (b - A x) in one pass (FP32; lanes >= bs, i.e. the learned step's block sizes).
void launch_residual_dinv(const BsrView<float>& A, const float* dinv, long long dld, const float* x, const float* b,
                          float* w, cudaStream_t s);
// w = D^-1 r on the level's blocks (FP32).
void launch_block_diag(int nb, int bs, const float* dinv, long long dld, const float* r, float* w, cudaStream_t s);
// Training features: feat (rows x 48 BF16, rows >= nb zero), scale (rows).
void launch_features(int nb, int rows, int bs, const int* nbr, const float* w, const void* tfeat, void* feat,
                     float* scale, cudaStream_t s);
// x += s y for every face (fused gather + 3-layer MLP). kernel: kLearnedKernelTcgen05 (tensor
// memory accumulators; a bounded wait that expires sets *status = 1) or kLearnedKernelMmaSync.
// Returns non-zero if the kernel cannot run.
constexpr int kLearnedKernelTcgen05 = 0;
constexpr int kLearnedKernelMmaSync = 1;
int launch_learned_apply(int nb, int bs, const int* nbr, const float* w, const void* tfeat, const void* wts,
                         const float* bias, float* x, int* status, int kernel, cudaStream_t s);
void launch_gemm(int kind, int M, int K, const void* A, int lda, const void* B, int ldb, float* C, float* parts,
                 int nsplit, int accumulate, cudaStream_t s);
void launch_bias_gelu(long long rows, float* a, const float* bias, void* h, cudaStream_t s);
void launch_gelu_back(long long count, const float* dh, const float* a, void* delta, cudaStream_t s);
void launch_correction(int nb, int bs, const float* y, const float* b3, const float* scale, float* c, cudaStream_t s);
// dy (rows x 16 BF16) = dL/dy of the energy loss; partials[kReduceCtas] of (c.q - 2 c.r).
void launch_energy_grad(int nb, int rows, int bs, const float* r, const float* q, const float* c, const float* scale,
                        double inv_energy, void* dy, double* partials, cudaStream_t s);
// out[ncol] = column sums of a BF16 rows x ncol matrix (parts: kColsumChunks * ncol floats).
void launch_colsum(long long rows, int ncol, const void* m, float* parts, float* out, cudaStream_t s);
void launch_adam(int n, float* p, const float* grad, float* m, float* v, float lr, float beta1, float beta2, float eps,
                 int step, float weight_decay, cudaStream_t s);
void launch_split_params(const float* p, void* wts, float* bias, cudaStream_t s);

}  // namespace fhg
