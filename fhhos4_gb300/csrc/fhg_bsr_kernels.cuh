#pragma once
// Block-sparse kernels of the fhhos4 solve phase for GB300 (sm_103a), templated on the value type
// (double, float, or the FP32 pair dfl) and instantiated by fhg_kernels.cu (float, double) and
// fhg_kernels_pair.cu (pairs).
//
// Every kernel is memory-bound: block-sparse products over face-block operators
// (bs = face DOFs: 2/3/4/6), colour sweeps of block Gauss-Seidel, and the FCG vector
// updates. The design targets HBM bandwidth:
//   * block values entry-major (vals[e*ld + p]) so a warp reading consecutive blocks
//     issues fully coalesced 8-byte (FP64) or 4-byte (FP32) loads per entry;
//   * a group of G lanes (G = 4..32, chosen per operator) per block row, partial sums
//     reduced with warp shuffles;
//   * reductions write fixed-size per-CTA partial arrays that every consumer reduces
//     in the same order (bitwise reproducible Krylov scalars, no atomics);
//   * Krylov scalars never leave the device: consumers read them from device memory,
//     so one whole iteration can be replayed as a CUDA graph.
#include "fhg_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <type_traits>
#include <utility>

namespace fhg {

namespace {


constexpr int kThreads = 256;

// Programmatic dependent launch: every kernel of this file is launched with programmatic stream
// serialization, so the next kernel's CTAs are scheduled while its predecessor drains instead of
// after it, and begins with pdl_wait() (griddepcontrol.wait), which returns once the predecessor
// grid has completed and its memory writes are visible. No global access precedes the wait, so
// the order of every read and write is that of plain stream order; only launch latency overlaps.
// Kernels launched without the attribute pass the wait at once. FHG_PDL=0 in the environment
// launches without it.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

bool pdl_enabled()
{
    static const bool on = [] {
        const char* e = std::getenv("FHG_PDL");
        return !(e && e[0] == '0');
    }();
    return on;
}

template <class... KArgs, class... Args>
void pdl_launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

template <int G, class T>
__device__ __forceinline__ T group_sum(T v)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
    return v;
}

// A pair's group sum: both parts shuffled, the partner's pair added with TwoSum.
template <int G>
__device__ __forceinline__ dfl group_sum(dfl v)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, v.h, o, G);
        const float ol = __shfl_xor_sync(0xffffffffu, v.l, o, G);
        df_add(v.h, v.l, oh, ol);
    }
    return v;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the CTA; result valid in every thread. `sh` holds >= 33 doubles.
__device__ __forceinline__ double block_sum(double v, double* sh)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    v = warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        double t = lane < nw ? sh[lane] : 0.0;
        t = warp_sum(t);
        if (lane == 0) sh[32] = t;
    }
    __syncthreads();
    return sh[32];
}

// Fixed-order reduction of a kReduceCtas-long partial array by one CTA.
__device__ __forceinline__ double reduce_partials(const double* __restrict__ p, double* sh)
{
    double v = 0.0;
    for (int i = threadIdx.x; i < kReduceCtas; i += blockDim.x) v += p[i];
    return block_sum(v, sh);
}

// Element loop of the fixed-grid vector kernels: thread t of CTA c visits
// i = c * kReduceThreads + t, then i + S, i + 2 S, ... (S = kReduceCtas * kReduceThreads) in that
// order, so every per-thread sum is taken in one fixed order. Four elements go per step with all
// their loads issued before the first use: one element per thread per step leaves too few bytes
// in flight for HBM (a quarter of what the copy rate needs at 152 x 4 CTAs of 256 threads).
// `load(i)` returns the element's inputs, `use(i, v)` computes and stores.
constexpr long long kRedStride = (long long)kReduceCtas * kReduceThreads;
constexpr int kRedUnroll = 4;

template <class Load, class Use>
__device__ __forceinline__ void for_each_element(long long n, Load load, Use use)
{
    long long i = (long long)blockIdx.x * kReduceThreads + threadIdx.x;
    for (; i + (kRedUnroll - 1) * kRedStride < n; i += kRedUnroll * kRedStride) {
        decltype(load(i)) v[kRedUnroll];
#pragma unroll
        for (int u = 0; u < kRedUnroll; u++) v[u] = load(i + u * kRedStride);
#pragma unroll
        for (int u = 0; u < kRedUnroll; u++) use(i + u * kRedStride, v[u]);
    }
    for (; i < n; i += kRedStride) use(i, load(i));
}

template <class A, class B>
struct Pair2 {
    A a;
    B b;
};

template <class T>
struct Quad4 {
    T a, b, c, d;
};

// ---------------------------------------------------------------------------
// Row accumulation: acc[r] += sum over this lane's blocks of (A_block x_col)[r].
// `sel(col)` returns 0 (skip the block), 1 (use it) or 2 (stop: columns are sorted, nothing
// after it is used). With U = 2 (bs <= 3) each lane walks two blocks per step so that the loads
// of both (column index, bs^2 values, bs entries of x) are in flight together, at the cost of
// registers (fewer resident warps); U is chosen per operator by the autotuner. The
// accumulation order is block by block either way.
template <class T, int BS, int G, int U, class Sel>
__device__ __forceinline__ void accumulate_row(int p0, int p1, int lane, const int* __restrict__ colidx,
                                               const T* __restrict__ vals, long long ld, const T* x, T* acc,
                                               Sel sel)
{
    if constexpr (U == 2 && BS <= 3) {
        for (int p = p0 + lane; p < p1; p += 2 * G) {
            const int q = p + G;
            const int ca = colidx[p];
            const int cb = q < p1 ? colidx[q] : -1;
            const int ua = sel(ca);
            if (ua == 2) break;
            const int ub = cb >= 0 ? sel(cb) : 0;
            T va[BS * BS], vb[BS * BS], xa[BS], xb[BS];
            if (ua == 1) {
#pragma unroll
                for (int e = 0; e < BS * BS; e++) va[e] = vals[(long long)e * ld + p];
#pragma unroll
                for (int c = 0; c < BS; c++) xa[c] = x[(long long)ca * BS + c];
            }
            if (ub == 1) {
#pragma unroll
                for (int e = 0; e < BS * BS; e++) vb[e] = vals[(long long)e * ld + q];
#pragma unroll
                for (int c = 0; c < BS; c++) xb[c] = x[(long long)cb * BS + c];
            }
            if (ua == 1) {
#pragma unroll
                for (int r = 0; r < BS; r++)
#pragma unroll
                    for (int c = 0; c < BS; c++) acc[r] = fma(va[r * BS + c], xa[c], acc[r]);
            }
            if (ub == 1) {
#pragma unroll
                for (int r = 0; r < BS; r++)
#pragma unroll
                    for (int c = 0; c < BS; c++) acc[r] = fma(vb[r * BS + c], xb[c], acc[r]);
            }
            if (ub == 2) break;
        }
    } else {
        for (int p = p0 + lane; p < p1; p += G) {
            const int col = colidx[p];
            const int u = sel(col);
            if (u == 2) break;
            if (u == 0) continue;
            T xv[BS];
#pragma unroll
            for (int c = 0; c < BS; c++) xv[c] = x[(long long)col * BS + c];
#pragma unroll
            for (int r = 0; r < BS; r++)
#pragma unroll
                for (int c = 0; c < BS; c++) acc[r] = fma(vals[(long long)(r * BS + c) * ld + p], xv[c], acc[r]);
        }
    }
}

struct UseAll {
    __device__ __forceinline__ int operator()(int) const { return 1; }
};

// First and one-past-last stored position of a block row: padded views (ell > 0) put row i at
// i * ell, with no row-pointer load ahead of the row walk. Their empty slots hold zero values and
// a column inside the operator (the row's own in the off-diagonal GS view, where the sweep skips
// it as the diagonal; a stored column of the row otherwise, where a product adds an exact zero).
__device__ __forceinline__ void row_range(int row, int ell, const int* __restrict__ rowptr, int& p0, int& p1)
{
    if (ell > 0) {
        p0 = row * ell;
        p1 = p0 + ell;
    } else {
        p0 = rowptr[row];
        p1 = rowptr[row + 1];
    }
}

// ---------------------------------------------------------------------------
// y = A x  |  y = aux - A x  |  y = aux + A x      (aux may alias y)
template <class T, int BS, int G, int U, int MODE>
__global__ void __launch_bounds__(kThreads) k_bsr_spmv(int nbr, const int* __restrict__ rowptr,
                                                       const int* __restrict__ colidx,
                                                       const T* __restrict__ vals, long long ld,
                                                       const T* __restrict__ x, const T* aux, T* y, int ell)
{
    pdl_wait();
    const int lane = threadIdx.x & (G - 1);
    const int row = (int)(((long long)blockIdx.x * kThreads + threadIdx.x) / G);
    T acc[BS];
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = T(0);
    // Lane r < BS writes output r of the row (G >= BS here: G is at least 4 and bs at most 3 on
    // this path, or lanes loop over outputs below when bs > G). The added vector is loaded
    // before the row walk so that its latency overlaps it.
    T av = T(0);
    if (MODE != kSpmvAssign && G >= BS && row < nbr && lane < BS) av = aux[(long long)row * BS + lane];
    if (row < nbr) {
        int p0, p1;
        row_range(row, ell, rowptr, p0, p1);
        accumulate_row<T, BS, G, U>(p0, p1, lane, colidx, vals, ld, x, acc, UseAll());
    }
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = group_sum<G>(acc[r]);
    if (row < nbr) {
#pragma unroll
        for (int r = 0; r < BS; r++) {
            if (lane == r % G) {
                const long long i = (long long)row * BS + r;
                const T a = (G >= BS) ? av : ((MODE == kSpmvAssign) ? T(0) : aux[i]);
                if (MODE == kSpmvAssign) y[i] = fin(acc[r]);
                else if (MODE == kSpmvResidual) y[i] = a - acc[r];
                else y[i] = a + acc[r];
            }
        }
    }
}

// y = M x | y = y + M x on the jagged view (rows sorted by decreasing block count, slot s of sorted
// row k at start[s] + k): one thread per row, every slot's load of a warp is 32 consecutive blocks with
// no padding, the sorted order ends a row's walk at its own length. The output row is scattered by
// the permutation (the vectors of one level stay in L2). The row's blocks are summed in column order.
constexpr int kMaxJdsSlots = 64;

template <class T, int BS, int MODE>
__global__ void __launch_bounds__(kThreads) k_bsr_spmv_jds(int nbr, int nslots, const int* __restrict__ perm,
                                                           const int* __restrict__ start,
                                                           const int* __restrict__ colidx,
                                                           const T* __restrict__ vals, long long ld,
                                                           const T* __restrict__ x, const T* aux, T* y)
{
    // Slots go in groups of kJdsGroup with every load of a group issued before its sums (predicated on
    // the row's length, the sorted order making the valid slots a prefix), so that a row's loads are in
    // flight together instead of one slot's after the other's.
    constexpr int kBlockBytes = BS * BS * (int)sizeof(T);
    constexpr int kJdsGroup = kBlockBytes <= 36 ? 4 : kBlockBytes <= 72 ? 2 : 1;   // registers: ~144 values
    pdl_wait();
    __shared__ int sh_start[kMaxJdsSlots + kJdsGroup + 1];
    for (int i = threadIdx.x; i <= nslots + kJdsGroup; i += blockDim.x) sh_start[i] = start[i < nslots ? i : nslots];
    __syncthreads();
    const int k = (int)(blockIdx.x * kThreads + threadIdx.x);
    if (k >= nbr) return;
    const long long row = perm[k];
    T av[BS];
    if (MODE != kSpmvAssign)
#pragma unroll
        for (int r = 0; r < BS; r++) av[r] = aux[row * BS + r];
    T acc[BS];
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = T(0);
    for (int s0 = 0; s0 < nslots; s0 += kJdsGroup) {
        if (sh_start[s0] + k >= sh_start[s0 + 1]) break;   // the row has no slot s0
        int col[kJdsGroup];
        bool ok[kJdsGroup];
#pragma unroll
        for (int g = 0; g < kJdsGroup; g++) {
            const int p = sh_start[s0 + g] + k;
            ok[g] = s0 + g < nslots && p < sh_start[s0 + g + 1];
            col[g] = ok[g] ? colidx[p] : 0;
        }
        T xv[kJdsGroup][BS], av2[kJdsGroup][BS * BS];
#pragma unroll
        for (int g = 0; g < kJdsGroup; g++) {
            const long long p = (long long)sh_start[s0 + g] + k;
#pragma unroll
            for (int c = 0; c < BS; c++) xv[g][c] = ok[g] ? x[(long long)col[g] * BS + c] : T(0);
#pragma unroll
            for (int e = 0; e < BS * BS; e++) av2[g][e] = ok[g] ? vals[(long long)e * ld + p] : T(0);
        }
#pragma unroll
        for (int g = 0; g < kJdsGroup; g++) {
            if (!ok[g]) continue;
#pragma unroll
            for (int r = 0; r < BS; r++)
#pragma unroll
                for (int c = 0; c < BS; c++) acc[r] = fma(av2[g][r * BS + c], xv[g][c], acc[r]);
        }
    }
#pragma unroll
    for (int r = 0; r < BS; r++) {
        if (MODE == kSpmvAssign) y[row * BS + r] = fin(acc[r]);
        else y[row * BS + r] = av[r] + acc[r];
    }
}

// w = D^-1 (b - A x) (block-Jacobi-scaled residual, the learned step's input): the residual of a
// row is reduced over the row's lanes, then lane r < BS applies row r of the row's D^-1.
template <class T, int BS, int G, int U>
__global__ void __launch_bounds__(kThreads) k_bsr_residual_dinv(int nbr, const int* __restrict__ rowptr,
                                                                const int* __restrict__ colidx,
                                                                const T* __restrict__ vals, long long ld,
                                                                const T* __restrict__ dinv, long long dld,
                                                                const T* __restrict__ x, const T* __restrict__ b,
                                                                T* __restrict__ w, int ell)
{
    pdl_wait();
    const int lane = threadIdx.x & (G - 1);
    const int row = (int)(((long long)blockIdx.x * kThreads + threadIdx.x) / G);
    T acc[BS];
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = T(0);
    T bv[BS], dv[BS];
    if (row < nbr) {
#pragma unroll
        for (int c = 0; c < BS; c++) bv[c] = b[(long long)row * BS + c];
        if (lane < BS)
#pragma unroll
            for (int c = 0; c < BS; c++) dv[c] = dinv[(long long)(lane * BS + c) * dld + row];
        int p0, p1;
        row_range(row, ell, rowptr, p0, p1);
        accumulate_row<T, BS, G, U>(p0, p1, lane, colidx, vals, ld, x, acc, UseAll());
    }
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = group_sum<G>(acc[r]);
    if (row < nbr && lane < BS) {
        T v = T(0);
#pragma unroll
        for (int c = 0; c < BS; c++) v += dv[c] * (bv[c] - acc[c]);
        w[(long long)row * BS + lane] = v;
    }
}

// One colour of block Gauss-Seidel: rows [row0, row1) are mutually uncoupled.
// x_i <- D_i^{-1} (b_i - sum_{j != i} A_ij x_j)
// Columns outside [col_lo, col_hi) are skipped: in a sweep that starts from x = 0 they hold
// zeros not yet overwritten (later colours of a forward sweep, earlier ones of a backward
// sweep), so skipping them changes no bit of the result and saves their loads. Block columns
// are sorted, so the skipped ones form a head and a tail of each row. The empty slots at the end
// of a padded (ell) row hold the row's own column and are skipped as the diagonal is; a stop on a
// column >= col_hi happens at a real block before them.
template <class T, int BS, int G, int U>
__global__ void __launch_bounds__(kThreads) k_bsr_gs(int row0, int row1, const int* __restrict__ rowptr,
                                                     const int* __restrict__ colidx,
                                                     const T* __restrict__ vals, long long ld,
                                                     const T* __restrict__ dinv, long long dld,
                                                     const T* __restrict__ b, T* x, int col_lo, int col_hi,
                                                     int ell, T omega)
{
    pdl_wait();
    const int lane = threadIdx.x & (G - 1);
    const int row = row0 + (int)(((long long)blockIdx.x * kThreads + threadIdx.x) / G);
    T acc[BS];
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = T(0);
    // b_i and the D_i^-1 row this lane applies (lane r < BS owns output r when G >= BS), loaded
    // before the row walk so that their latency overlaps it instead of following it.
    T bv[BS], dv[BS];
    if (G >= BS && row < row1) {
#pragma unroll
        for (int c = 0; c < BS; c++) bv[c] = b[(long long)row * BS + c];
        if (lane < BS)
#pragma unroll
            for (int c = 0; c < BS; c++) dv[c] = dinv[(long long)(lane * BS + c) * dld + row];
    }
    if (row < row1) {
        auto sel = [row, col_lo, col_hi](int col) -> int {
            if (col >= col_hi) return 2;
            return (col == row || col < col_lo) ? 0 : 1;
        };
        int p0, p1;
        row_range(row, ell, rowptr, p0, p1);
        accumulate_row<T, BS, G, U>(p0, p1, lane, colidx, vals, ld, x, acc, sel);
    }
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = group_sum<G>(acc[r]);
    if (row < row1) {
        if (G >= BS) {
            if (lane < BS) {
                T v = T(0);
#pragma unroll
                for (int c = 0; c < BS; c++) v = fma(dv[c], bv[c] - acc[c], v);
                const long long i = (long long)row * BS + lane;
                // block SOR: x_i <- omega D_i^-1 (b_i - sum_{j != i} A_ij x_j) + (1 - omega) x_i
                if (omega != T(1)) v = fma(omega, v, (T(1) - omega) * x[i]);
                x[i] = fin(v);
            }
        } else {
            T t[BS];
#pragma unroll
            for (int c = 0; c < BS; c++) t[c] = b[(long long)row * BS + c] - acc[c];
#pragma unroll
            for (int r = 0; r < BS; r++) {
                if (lane == r % G) {
                    T v = T(0);
#pragma unroll
                    for (int c = 0; c < BS; c++) v = fma(dinv[(long long)(r * BS + c) * dld + row], t[c], v);
                    const long long i = (long long)row * BS + r;
                    if (omega != T(1)) v = fma(omega, v, (T(1) - omega) * x[i]);
                    x[i] = fin(v);
                }
            }
        }
    }
}

// One colour of block GS on a slot-major padded view (slot_major, ell = W): one thread per block
// row. Slot s of row i of the colour [row0, row1) lives at row0 * W + s * (row1 - row0) + (i - row0),
// so a warp's loads of one slot are 32 consecutive words. The W column indices, then the used
// slots' values and x entries are loaded before the sums, so all of a row's loads are in flight
// together; no lane reduction follows. The column rules are those of k_bsr_gs (empty slots hold
// the row's own column). ZERO: a zero-start sweep, whose skipped blocks are not loaded; other
// sweeps load every slot and drop the diagonal ones by a select.
template <class T, int BS, int W, bool ZERO>
__global__ void __launch_bounds__(kThreads, 2) k_bsr_gs_slot(int row0, int row1, const int* __restrict__ colidx,
                                                            const T* __restrict__ vals, long long ld,
                                                            const T* __restrict__ dinv, long long dld,
                                                            const T* __restrict__ b, T* x, int col_lo, int col_hi,
                                                            T omega)
{
    pdl_wait();
    const int row = row0 + (int)(blockIdx.x * kThreads + threadIdx.x);
    if (row >= row1) return;
    const long long nrc = row1 - row0;
    const long long base = (long long)row0 * W + (row - row0);
    int col[W];
#pragma unroll
    for (int s = 0; s < W; s++) col[s] = colidx[base + s * nrc];
    T bv[BS], dv[BS * BS];
#pragma unroll
    for (int c = 0; c < BS; c++) bv[c] = b[(long long)row * BS + c];
#pragma unroll
    for (int e = 0; e < BS * BS; e++) dv[e] = dinv[(long long)e * dld + row];
    T acc[BS];
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = T(0);
#pragma unroll
    for (int s = 0; s < W; s++) {
        const int j = col[s];
        const bool use = j != row && (!ZERO || (j >= col_lo && j < col_hi));
        if (ZERO && !use) continue;
        const long long p = base + s * nrc;
        T xv[BS];
#pragma unroll
        for (int c = 0; c < BS; c++) xv[c] = x[(long long)j * BS + c];
#pragma unroll
        for (int r = 0; r < BS; r++)
#pragma unroll
            for (int c = 0; c < BS; c++) {
                const T a = vals[(long long)(r * BS + c) * ld + p];
                acc[r] = fma(use ? a : T(0), xv[c], acc[r]);
            }
    }
#pragma unroll
    for (int r = 0; r < BS; r++) {
        T v = T(0);
#pragma unroll
        for (int c = 0; c < BS; c++) v = fma(dv[r * BS + c], bv[c] - acc[c], v);
        const long long i = (long long)row * BS + r;
        if (omega != T(1)) v = fma(omega, v, (T(1) - omega) * x[i]);   // block SOR
        x[i] = fin(v);
    }
}

// y = A x | y = aux - A x on a slot-major padded view of all of A (slot_major, ell = W, one "colour"
// of every row): slot s of row i at s * nbr + i, one thread per block row. The W column indices,
// then every slot's values and x entries, are loaded before the sums, so all of a row's loads are in
// flight together and a warp's load of one slot is 32 consecutive values; no lane reduction follows.
// Empty slots hold zero values and a column of the row (an exact zero added). The summation order
// is block by block in column order, as in the row-major kernels.
template <class T, int BS, int W, int MODE>
__global__ void __launch_bounds__(kThreads, 2) k_bsr_spmv_slot(int nbr, const int* __restrict__ colidx,
                                                              const T* __restrict__ vals, long long ld,
                                                              const T* __restrict__ x, const T* aux, T* y)
{
    pdl_wait();
    const int row = (int)(blockIdx.x * kThreads + threadIdx.x);
    if (row >= nbr) return;
    int col[W];
#pragma unroll
    for (int k = 0; k < W; k++) col[k] = colidx[(long long)k * nbr + row];
    T av[BS];
    if (MODE != kSpmvAssign)
#pragma unroll
        for (int r = 0; r < BS; r++) av[r] = aux[(long long)row * BS + r];
    T acc[BS];
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = T(0);
#pragma unroll
    for (int k = 0; k < W; k++) {
        const long long p = (long long)k * nbr + row;
        T xv[BS];
#pragma unroll
        for (int c = 0; c < BS; c++) xv[c] = x[(long long)col[k] * BS + c];
#pragma unroll
        for (int r = 0; r < BS; r++)
#pragma unroll
            for (int c = 0; c < BS; c++) acc[r] = fma(vals[(long long)(r * BS + c) * ld + p], xv[c], acc[r]);
    }
#pragma unroll
    for (int r = 0; r < BS; r++) {
        const long long i = (long long)row * BS + r;
        if (MODE == kSpmvAssign) y[i] = fin(acc[r]);
        else if (MODE == kSpmvResidual) y[i] = av[r] - acc[r];
        else y[i] = av[r] + acc[r];
    }
}

// w = D^-1 (b - A x) on the slot-major view of all of A (the learned step's input), one thread per row.
template <class T, int BS, int W>
__global__ void __launch_bounds__(kThreads, 2) k_bsr_residual_dinv_slot(int nbr, const int* __restrict__ colidx,
                                                                       const T* __restrict__ vals, long long ld,
                                                                       const T* __restrict__ dinv, long long dld,
                                                                       const T* __restrict__ x,
                                                                       const T* __restrict__ b, T* __restrict__ w)
{
    pdl_wait();
    const int row = (int)(blockIdx.x * kThreads + threadIdx.x);
    if (row >= nbr) return;
    int col[W];
#pragma unroll
    for (int k = 0; k < W; k++) col[k] = colidx[(long long)k * nbr + row];
    T bv[BS], dv[BS * BS];
#pragma unroll
    for (int c = 0; c < BS; c++) bv[c] = b[(long long)row * BS + c];
#pragma unroll
    for (int e = 0; e < BS * BS; e++) dv[e] = dinv[(long long)e * dld + row];
    T acc[BS];
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = T(0);
#pragma unroll
    for (int k = 0; k < W; k++) {
        const long long p = (long long)k * nbr + row;
        T xv[BS];
#pragma unroll
        for (int c = 0; c < BS; c++) xv[c] = x[(long long)col[k] * BS + c];
#pragma unroll
        for (int r = 0; r < BS; r++)
#pragma unroll
            for (int c = 0; c < BS; c++) acc[r] = fma(vals[(long long)(r * BS + c) * ld + p], xv[c], acc[r]);
    }
#pragma unroll
    for (int r = 0; r < BS; r++) {
        T v = T(0);
#pragma unroll
        for (int c = 0; c < BS; c++) v = fma(dv[r * BS + c], bv[c] - acc[c], v);
        w[(long long)row * BS + r] = fin(v);
    }
}

// Block Jacobi: xnew_i = D_i^{-1} (omega b_i + (1-omega) D_i xold_i - omega sum_{j!=i} A_ij xold_j)
template <class T, int BS, int G>
__global__ void __launch_bounds__(kThreads) k_bsr_jacobi(int nbr, const int* __restrict__ rowptr,
                                                         const int* __restrict__ colidx,
                                                         const T* __restrict__ vals, long long ld,
                                                         const T* __restrict__ dinv, long long dld, T omega,
                                                         const T* __restrict__ b, const T* __restrict__ xold,
                                                         T* __restrict__ xnew)
{
    pdl_wait();
    const int lane = threadIdx.x & (G - 1);
    const int row = (int)(((long long)blockIdx.x * kThreads + threadIdx.x) / G);
    T off[BS], dia[BS];
#pragma unroll
    for (int r = 0; r < BS; r++) { off[r] = T(0); dia[r] = T(0); }
    if (row < nbr) {
        const int p1 = rowptr[row + 1];
        for (int p = rowptr[row] + lane; p < p1; p += G) {
            const int col = colidx[p];
            T xv[BS];
#pragma unroll
            for (int c = 0; c < BS; c++) xv[c] = xold[(long long)col * BS + c];
            if (col == row) {
#pragma unroll
                for (int r = 0; r < BS; r++)
#pragma unroll
                    for (int c = 0; c < BS; c++) dia[r] = fma(vals[(long long)(r * BS + c) * ld + p], xv[c], dia[r]);
            } else {
#pragma unroll
                for (int r = 0; r < BS; r++)
#pragma unroll
                    for (int c = 0; c < BS; c++) off[r] = fma(vals[(long long)(r * BS + c) * ld + p], xv[c], off[r]);
            }
        }
    }
#pragma unroll
    for (int r = 0; r < BS; r++) { off[r] = group_sum<G>(off[r]); dia[r] = group_sum<G>(dia[r]); }
    if (row < nbr) {
        T t[BS];
#pragma unroll
        for (int c = 0; c < BS; c++)
            t[c] = omega * b[(long long)row * BS + c] + (T(1) - omega) * dia[c] - omega * off[c];
#pragma unroll
        for (int r = 0; r < BS; r++) {
            if (lane == r % G) {
                T v = T(0);
#pragma unroll
                for (int c = 0; c < BS; c++) v = fma(dinv[(long long)(r * BS + c) * dld + row], t[c], v);
                xnew[(long long)row * BS + r] = fin(v);
            }
        }
    }
}

// x = Cinv b, one warp per row, FP64 accumulation.
template <class T>
__global__ void __launch_bounds__(kThreads) k_coarse(int n, const double* __restrict__ cinv,
                                                     const T* __restrict__ b, T* __restrict__ x)
{
    pdl_wait();
    const int lane = threadIdx.x & 31;
    const int row = (blockIdx.x * kThreads + threadIdx.x) >> 5;
    if (row >= n) return;  // whole warps exit together
    const double* a = cinv + (long long)row * n;
    double acc = 0.0;
    for (int j = lane; j < n; j += 32) acc = fma(a[j], (double)b[j], acc);
    acc = warp_sum(acc);
    if (lane == 0) x[row] = (T)acc;
}

// Up to three dot products in one pass (K-cycle): partials[q * kReduceCtas + cta] of a_q . b_q,
// FP64 accumulation whatever T.
template <class T>
__global__ void __launch_bounds__(kReduceThreads) k_dots3(long long n, int nq, const T* __restrict__ a0,
                                                          const T* __restrict__ b0, const T* __restrict__ a1,
                                                          const T* __restrict__ b1, const T* __restrict__ a2,
                                                          const T* __restrict__ b2, double* __restrict__ partials)
{
    pdl_wait();
    __shared__ double sh[33];
    double v0 = 0.0, v1 = 0.0, v2 = 0.0;
    struct E {
        T a0, b0, a1, b1, a2, b2;
    };
    for_each_element(
        n,
        [&](long long i) {
            E e{a0[i], b0[i], T(0), T(0), T(0), T(0)};
            if (nq > 1) { e.a1 = a1[i]; e.b1 = b1[i]; }
            if (nq > 2) { e.a2 = a2[i]; e.b2 = b2[i]; }
            return e;
        },
        [&](long long, const E& e) {
            v0 = fma((double)e.a0, (double)e.b0, v0);
            if (nq > 1) v1 = fma((double)e.a1, (double)e.b1, v1);
            if (nq > 2) v2 = fma((double)e.a2, (double)e.b2, v2);
        });
    v0 = block_sum(v0, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = v0;
    if (nq > 1) {
        v1 = block_sum(v1, sh);
        if (threadIdx.x == 0) partials[kReduceCtas + blockIdx.x] = v1;
    }
    if (nq > 2) {
        v2 = block_sum(v2, sh);
        if (threadIdx.x == 0) partials[2 * kReduceCtas + blockIdx.x] = v2;
    }
}

// y += alpha x; out = a c + b d (K-cycle updates, coefficients from the host).
template <class T>
__global__ void k_axpy(long long n, double alpha, const T* __restrict__ x, T* __restrict__ y)
{
    pdl_wait();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        y[i] = y[i] + (T)alpha * x[i];
}

template <class T>
__global__ void k_lincomb(long long n, double a, const T* __restrict__ c, double b, const T* __restrict__ d,
                          T* __restrict__ out)
{
    pdl_wait();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = (T)a * c[i] + (T)b * d[i];
}

template <class Tin, class Tout>
__global__ void __launch_bounds__(kThreads) k_convert(long long n, const Tin* __restrict__ in, Tout* __restrict__ out)
{
    pdl_wait();
    const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (i < n) out[i] = (Tout)in[i];
}

template <class T>
__global__ void __launch_bounds__(kThreads) k_permute(int nb, int bs, const int* __restrict__ perm,
                                                      const T* __restrict__ in, T* __restrict__ out, int gather)
{
    pdl_wait();
    const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (i >= (long long)nb * bs) return;
    const int blk = (int)(i / bs), c = (int)(i - (long long)blk * bs);
    const long long o = (long long)perm[blk] * bs + c;
    if (gather) out[i] = in[o];
    else out[o] = in[i];
}

// The natural injection between two face degrees on the same faces (P_LevelForHHO::SetupProlongation,
// src/Solver/Multigrid/MultigridForHHO/P_MultigridForHHO.h:69-92): fine face block i (nh unknowns)
// is coarse block map[i] (nl < nh unknowns, the first nl functions of the hierarchical face basis).
// Restriction by P^T: out[map[i] * nl + q] = in[i * nh + q] for q < nl.
template <class T>
__global__ void __launch_bounds__(kThreads) k_inject_restrict(int nb, int nh, int nl, const int* __restrict__ map,
                                                              const T* __restrict__ in, T* __restrict__ out)
{
    pdl_wait();
    const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (i >= (long long)nb * nl) return;
    const int blk = (int)(i / nl), q = (int)(i - (long long)blk * nl);
    out[(long long)map[blk] * nl + q] = in[(long long)blk * nh + q];
}

// Prolongation by P: out[i * nh + q] = aux[i * nh + q] + (q < nl ? in[map[i] * nl + q] : 0), aux NULL
// reading as zero; out may be aux. The one entry of P is 1, so this is the product's arithmetic.
template <class T>
__global__ void __launch_bounds__(kThreads) k_inject_prolong(int nb, int nh, int nl, const int* __restrict__ map,
                                                             const T* __restrict__ in, const T* aux, T* out)
{
    pdl_wait();
    const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (i >= (long long)nb * nh) return;
    const int blk = (int)(i / nh), q = (int)(i - (long long)blk * nh);
    if (q < nl) {
        const T e = in[(long long)map[blk] * nl + q];
        out[i] = aux ? aux[i] + e : e;
    } else {
        out[i] = aux ? aux[i] : T(0);
    }
}

inline unsigned grid_for(long long work, int per_cta)
{
    long long g = (work + per_cta - 1) / per_cta;
    return (unsigned)(g > 0 ? g : 1);
}

}  // namespace

#define FHG_DISPATCH_BS_G(BSV, GV, ...)                                              \
    switch (BSV) {                                                                    \
    case 2: FHG_DISPATCH_G(2, GV, __VA_ARGS__); break;                                       \
    case 3: FHG_DISPATCH_G(3, GV, __VA_ARGS__); break;                                       \
    case 4: FHG_DISPATCH_G(4, GV, __VA_ARGS__); break;                                       \
    case 6: FHG_DISPATCH_G(6, GV, __VA_ARGS__); break;                                       \
    default: break;                                                                   \
    }
#define FHG_DISPATCH_G(BS_, GV, ...)                                                 \
    switch (GV) {                                                                     \
    case 4: { constexpr int BS = BS_, G = 4; __VA_ARGS__; } break;                          \
    case 8: { constexpr int BS = BS_, G = 8; __VA_ARGS__; } break;                          \
    case 16: { constexpr int BS = BS_, G = 16; __VA_ARGS__; } break;                        \
    default: { constexpr int BS = BS_, G = 32; __VA_ARGS__; } break;                        \
    }

template <class T, int BS, int G, int U>
void spmv_u(const BsrView<T>& A, unsigned grid, int mode, const T* x, const T* aux, T* y, cudaStream_t s)
{
    if (mode == kSpmvAssign)
        pdl_launch(k_bsr_spmv<T, BS, G, U, kSpmvAssign>, grid, kThreads, 0, s, A.nbr, A.rowptr, A.colidx, A.vals, A.ld, x, aux, y,
                   A.ell);
    else if (mode == kSpmvResidual)
        pdl_launch(k_bsr_spmv<T, BS, G, U, kSpmvResidual>, grid, kThreads, 0, s, A.nbr, A.rowptr, A.colidx, A.vals, A.ld, x, aux, y,
                   A.ell);
    else
        pdl_launch(k_bsr_spmv<T, BS, G, U, kSpmvAddTo>, grid, kThreads, 0, s, A.nbr, A.rowptr, A.colidx, A.vals, A.ld, x, aux, y,
                   A.ell);
}

// Slot-major products: dispatch on the block size and the slot count W (5..8).
template <class T, int BS, int W>
void spmv_slot_shape(const BsrView<T>& A, unsigned grid, int mode, const T* x, const T* aux, T* y, cudaStream_t s)
{
    if (mode == kSpmvAssign)
        pdl_launch(k_bsr_spmv_slot<T, BS, W, kSpmvAssign>, grid, kThreads, 0, s, A.nbr, A.colidx, A.vals, A.ld, x,
                   aux, y);
    else if (mode == kSpmvResidual)
        pdl_launch(k_bsr_spmv_slot<T, BS, W, kSpmvResidual>, grid, kThreads, 0, s, A.nbr, A.colidx, A.vals, A.ld, x,
                   aux, y);
    else
        pdl_launch(k_bsr_spmv_slot<T, BS, W, kSpmvAddTo>, grid, kThreads, 0, s, A.nbr, A.colidx, A.vals, A.ld, x,
                   aux, y);
}

template <class T, int BS>
void spmv_slot_w(const BsrView<T>& A, unsigned grid, int mode, const T* x, const T* aux, T* y, cudaStream_t s)
{
    switch (A.ell) {
    case 5: spmv_slot_shape<T, BS, 5>(A, grid, mode, x, aux, y, s); break;
    case 6: spmv_slot_shape<T, BS, 6>(A, grid, mode, x, aux, y, s); break;
    case 7: spmv_slot_shape<T, BS, 7>(A, grid, mode, x, aux, y, s); break;
    case 8: spmv_slot_shape<T, BS, 8>(A, grid, mode, x, aux, y, s); break;
    default: break;   // setup builds slot-major product views for W in 5..8 only
    }
}

template <class T>
void launch_spmv(const BsrView<T>& A, int mode, const T* x, const T* aux, T* y, cudaStream_t s)
{
    if (A.nbr == 0) return;
    if (A.jds_perm) {
        // jagged views exist only for the transfers (assign, add-to) with at most kMaxJdsSlots blocks
        // a row (setup builds no other); they have no row pointers to fall back on
        if ((mode != kSpmvAssign && mode != kSpmvAddTo) || A.jds_slots > kMaxJdsSlots) return;
        const unsigned grid = grid_for(A.nbr, kThreads);
#define FHG_JDS_LAUNCH(BSV)                                                                                     \
        if (mode == kSpmvAssign)                                                                                 \
            pdl_launch(k_bsr_spmv_jds<T, BSV, kSpmvAssign>, grid, kThreads, 0, s, A.nbr, A.jds_slots, A.jds_perm, \
                       A.jds_start, A.colidx, A.vals, A.ld, x, aux, y);                                          \
        else                                                                                                     \
            pdl_launch(k_bsr_spmv_jds<T, BSV, kSpmvAddTo>, grid, kThreads, 0, s, A.nbr, A.jds_slots, A.jds_perm,  \
                       A.jds_start, A.colidx, A.vals, A.ld, x, aux, y);
        switch (A.bs) {
        case 2: FHG_JDS_LAUNCH(2) break;
        case 3: FHG_JDS_LAUNCH(3) break;
        case 4: FHG_JDS_LAUNCH(4) break;
        case 6: FHG_JDS_LAUNCH(6) break;
        default: break;
        }
#undef FHG_JDS_LAUNCH
        g_kernel_launches++;
        return;
    }
    if constexpr (!std::is_same<T, double>::value) {
        if (A.slot_major) {   // FP32 and pair product views (no FP64 slot-major view is built)
            const unsigned grid = grid_for(A.nbr, kThreads);
            switch (A.bs) {
            case 2: spmv_slot_w<T, 2>(A, grid, mode, x, aux, y, s); break;
            case 3: spmv_slot_w<T, 3>(A, grid, mode, x, aux, y, s); break;
            case 4: spmv_slot_w<T, 4>(A, grid, mode, x, aux, y, s); break;
            case 6: spmv_slot_w<T, 6>(A, grid, mode, x, aux, y, s); break;
            default: break;
            }
            g_kernel_launches++;
            return;
        }
    }
    // (the grid follows the dispatched lane count G, so every row is covered whatever A.lanes says)
    FHG_DISPATCH_BS_G(A.bs, A.lanes, {
        const unsigned grid = grid_for((long long)A.nbr * G, kThreads);
        if (A.unroll == 2) spmv_u<T, BS, G, 2>(A, grid, mode, x, aux, y, s);
        else spmv_u<T, BS, G, 1>(A, grid, mode, x, aux, y, s);
    });
    g_kernel_launches++;
}

// Slot-major sweeps: dispatch on the block size and the slot count W (4..8).
template <class T, int BS, int W>
void gs_slot_shape(const BsrView<T>& A, unsigned grid, int row0, int row1, const T* dinv, long long dld,
                   const T* b, T* x, cudaStream_t s, int col_lo, int col_hi, T omega)
{
    if (col_lo > 0 || col_hi < 0x7fffffff)
        pdl_launch(k_bsr_gs_slot<T, BS, W, true>, grid, kThreads, 0, s, row0, row1, A.colidx, A.vals, A.ld, dinv,
                   dld, b, x, col_lo, col_hi, omega);
    else
        pdl_launch(k_bsr_gs_slot<T, BS, W, false>, grid, kThreads, 0, s, row0, row1, A.colidx, A.vals, A.ld, dinv,
                   dld, b, x, col_lo, col_hi, omega);
}

template <class T, int BS>
void gs_slot_w(const BsrView<T>& A, unsigned grid, int row0, int row1, const T* dinv, long long dld,
               const T* b, T* x, cudaStream_t s, int col_lo, int col_hi, T omega)
{
    switch (A.ell) {
    case 4: gs_slot_shape<T, BS, 4>(A, grid, row0, row1, dinv, dld, b, x, s, col_lo, col_hi, omega); break;
    case 5: gs_slot_shape<T, BS, 5>(A, grid, row0, row1, dinv, dld, b, x, s, col_lo, col_hi, omega); break;
    case 6: gs_slot_shape<T, BS, 6>(A, grid, row0, row1, dinv, dld, b, x, s, col_lo, col_hi, omega); break;
    case 7: gs_slot_shape<T, BS, 7>(A, grid, row0, row1, dinv, dld, b, x, s, col_lo, col_hi, omega); break;
    case 8: gs_slot_shape<T, BS, 8>(A, grid, row0, row1, dinv, dld, b, x, s, col_lo, col_hi, omega); break;
    default: break;   // setup builds slot-major views for W in 4..8 only
    }
}

template <class T>
void launch_gs_slot(const BsrView<T>& A, int row0, int row1, const T* dinv, long long dld, const T* b,
                    T* x, cudaStream_t s, int col_lo, int col_hi, T omega)
{
    const unsigned grid = grid_for((long long)(row1 - row0), kThreads);
    switch (A.bs) {
    case 2: gs_slot_w<T, 2>(A, grid, row0, row1, dinv, dld, b, x, s, col_lo, col_hi, omega); break;
    case 3: gs_slot_w<T, 3>(A, grid, row0, row1, dinv, dld, b, x, s, col_lo, col_hi, omega); break;
    case 4: gs_slot_w<T, 4>(A, grid, row0, row1, dinv, dld, b, x, s, col_lo, col_hi, omega); break;
    case 6: gs_slot_w<T, 6>(A, grid, row0, row1, dinv, dld, b, x, s, col_lo, col_hi, omega); break;
    default: break;
    }
}

template <class T>
void launch_gs(const BsrView<T>& A, int row0, int row1, const T* dinv, long long dld, const T* b, T* x, cudaStream_t s,
               int col_lo, int col_hi, T omega)
{
    if (row1 <= row0) return;
    if constexpr (!std::is_same<T, double>::value) {
        if (A.slot_major) {   // FP32 and pair views (setup builds no FP64 slot-major view)
            launch_gs_slot<T>(A, row0, row1, dinv, dld, b, x, s, col_lo, col_hi, omega);
            g_kernel_launches++;
            return;
        }
    }
    FHG_DISPATCH_BS_G(A.bs, A.lanes, {
        const unsigned grid = grid_for((long long)(row1 - row0) * G, kThreads);
        if (A.unroll == 2)
            pdl_launch(k_bsr_gs<T, BS, G, 2>, grid, kThreads, 0, s, row0, row1, A.rowptr, A.colidx, A.vals, A.ld, dinv,
                       dld, b, x, col_lo, col_hi, A.ell, omega);
        else
            pdl_launch(k_bsr_gs<T, BS, G, 1>, grid, kThreads, 0, s, row0, row1, A.rowptr, A.colidx, A.vals, A.ld, dinv,
                       dld, b, x, col_lo, col_hi, A.ell, omega);
    });
    g_kernel_launches++;
}

template <class T>
void launch_jacobi(const BsrView<T>& A, const T* dinv, long long dld, T omega, const T* b, const T* xold, T* xnew,
                   cudaStream_t s)
{
    if (A.nbr == 0 || A.ell > 0) return;   // the Jacobi row walk needs the row pointers (callers pass A)
    FHG_DISPATCH_BS_G(A.bs, A.lanes, {
        const unsigned grid = grid_for((long long)A.nbr * G, kThreads);
        pdl_launch(k_bsr_jacobi<T, BS, G>, grid, kThreads, 0, s, A.nbr, A.rowptr, A.colidx, A.vals, A.ld, dinv, dld, omega, b,
                                                         xold, xnew);
    });
    g_kernel_launches++;
}

template <class T>
void launch_coarse(int n, const double* cinv, const T* b, T* x, cudaStream_t s)
{
    pdl_launch(k_coarse<T>, grid_for((long long)n * 32, kThreads), kThreads, 0, s, n, cinv, b, x);
    g_kernel_launches++;
}

template <class T>
void launch_dots3(long long n, int nq, const T* a0, const T* b0, const T* a1, const T* b1, const T* a2, const T* b2,
                  double* partials, cudaStream_t s)
{
    pdl_launch(k_dots3<T>, kReduceCtas, kReduceThreads, 0, s, n, nq, a0, b0, a1 ? a1 : a0, b1 ? b1 : b0, a2 ? a2 : a0,
                                                      b2 ? b2 : b0, partials);
    g_kernel_launches++;
}

template <class T>
void launch_axpy(long long n, double alpha, const T* x, T* y, cudaStream_t s)
{
    const long long blocks = std::min<long long>((n + 255) / 256, 4 * 152);
    pdl_launch(k_axpy<T>, (unsigned)std::max<long long>(blocks, 1), 256, 0, s, n, alpha, x, y);
    g_kernel_launches++;
}

template <class T>
void launch_lincomb(long long n, double a, const T* c, double b, const T* d, T* out, cudaStream_t s)
{
    const long long blocks = std::min<long long>((n + 255) / 256, 4 * 152);
    pdl_launch(k_lincomb<T>, (unsigned)std::max<long long>(blocks, 1), 256, 0, s, n, a, c, b, d, out);
    g_kernel_launches++;
}

template <class Tin, class Tout>
void launch_convert(long long n, const Tin* in, Tout* out, cudaStream_t s)
{
    if (n == 0) return;
    pdl_launch(k_convert<Tin, Tout>, grid_for(n, kThreads), kThreads, 0, s, n, in, out);
    g_kernel_launches++;
}

template <class T>
void launch_permute(int nb, int bs, const int* perm, const T* in, T* out, bool gather, cudaStream_t s)
{
    if (nb == 0) return;
    pdl_launch(k_permute<T>, grid_for((long long)nb * bs, kThreads), kThreads, 0, s, nb, bs, perm, in, out, gather ? 1 : 0);
    g_kernel_launches++;
}

template <class T>
void launch_inject(int nb, int nh, int nl, const int* map, const T* in, const T* aux, T* out, bool prolong,
                   cudaStream_t s)
{
    if (nb == 0) return;
    if (prolong)
        pdl_launch(k_inject_prolong<T>, grid_for((long long)nb * nh, kThreads), kThreads, 0, s, nb, nh, nl, map, in,
                   aux, out);
    else
        pdl_launch(k_inject_restrict<T>, grid_for((long long)nb * nl, kThreads), kThreads, 0, s, nb, nh, nl, map, in,
                   out);
    g_kernel_launches++;
}

}  // namespace fhg
