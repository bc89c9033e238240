// The coarse part of a multigrid cycle in one kernel launch.
//
// Below some level the operators are small (tens of thousands of block rows or fewer) and a cycle
// there is a long chain of short phases: every colour of every smoothing sweep, the residual, the
// restriction, the coarsest solve, the prolongation. Launched one kernel per phase, each costs a
// launch slot of a few microseconds while its work takes a fraction of that. Here one thread-block
// cluster (8 or 16 CTAs, co-scheduled by the hardware) runs the whole sub-cycle: every phase
// spreads its rows over all threads of the cluster, and phases are separated by the hardware
// cluster barrier (barrier.cluster with release/acquire semantics at cluster scope, which orders the
// global-memory writes of one phase before the reads of the next across the cluster's CTAs). The
// barrier cannot wait forever: all CTAs of a cluster are resident together and every thread takes
// the same path through the cycle.
//
// A block row is walked by a group of `lanes` threads (block p of the row by lane p mod lanes,
// partial sums added by shuffles), and each group keeps up to four rows in flight (all their loads
// issued before the sums), so that loads overlap: one thread per row waits for them one after another,
// and a phase of a few rows per thread is a chain of memory round trips. The cycle runs as a loop over levels with a
// count of coarse corrections per level (no device recursion, so the stack is fixed at compile time).
//
// The arithmetic is the multigrid cycle of Multigrid::MultigridCycle (src/Solver/Multigrid/
// Multigrid.h:438-608) on the levels it covers: block Gauss-Seidel / SOR sweeps in colour order
// (BlockGaussSeidel.h:84-120, BlockSOR.h:199-227), r = b - A x (Multigrid.h:478), R r (Level.h:139-143),
// the coarse correction (V, or W with WLoops: repeated on the same right-hand side, except directly
// above the coarsest level), the coarsest dense solve, x += P e (Level.h:150-154, Multigrid.h:554).
// The FP32 and pair (dfl) value types are instantiated.
#include "fhg_coarse.h"

#include <mutex>
#include <type_traits>

namespace fhg {

namespace {

// Every thread of the cluster arrives (release) and waits (acquire); the non-aligned form does not
// require the threads of a warp to arrive together.
__device__ __forceinline__ void cluster_sync()
{
    asm volatile("barrier.cluster.arrive.release;\n"
                 "barrier.cluster.wait.acquire;\n" ::: "memory");
}

__device__ __forceinline__ void pdl_wait_coarse() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

// Sum over the g lanes of a group (g a power of two <= 32; every lane of the warp calls it).
__device__ __forceinline__ float lanes_sum(float v, int g)
{
    for (int o = g >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, g);
    return v;
}

__device__ __forceinline__ dfl lanes_sum(dfl v, int g)
{
    for (int o = g >> 1; o > 0; o >>= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, v.h, o, g);
        const float ol = __shfl_xor_sync(0xffffffffu, v.l, o, g);
        df_add(v.h, v.l, oh, ol);
    }
    return v;
}

__device__ __forceinline__ double lanes_sum(double v, int g)
{
    for (int o = g >> 1; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, g);
    return v;
}

template <class T>
struct Ctx {
    const FusedCycle<T>& P;
    long long t, nthr;   // thread index within the cluster, threads of the cluster
};

// Rows [r0, r1) of a phase, `g` lanes per row: calls f(i, valid, lane) in passes that every thread
// of the cluster takes the same number of times (the shuffles of a group need all lanes of the warp).
template <class T, class F>
__device__ __forceinline__ void row_passes(const Ctx<T>& C, long long r0, long long r1, int g, F f)
{
    const long long gid = C.t / g, ngroups = C.nthr / g;
    const int lane = (int)(C.t % g);
    const long long passes = (r1 - r0 + ngroups - 1) / ngroups;
    for (long long ps = 0; ps < passes; ps++) {
        const long long i = r0 + ps * ngroups + gid;
        f(i, i < r1, lane);
    }
}

// Rows [r0, r1) of a phase with `g` lanes per row and R rows per group in flight: in each pass a group
// takes R rows, loads the row bounds of all R, then each step loads one block of every row (column
// index, the x entries it names, the values) before any sum, so the loads of R rows overlap instead of
// following one another. A row is summed block by block in each lane's order (blocks lane, lane + g,
// ...), then over the lanes by shuffles. emit(i, lane, acc) runs for every valid row after the sums.
template <class T, int BS, int R, class Emit>
__device__ __forceinline__ void rows_multi(const Ctx<T>& C, long long r0, long long r1, int g, int ell,
                                           const int* __restrict__ rowptr, const int* __restrict__ colidx,
                                           const T* __restrict__ vals, long long ld, const T* x, bool skip_diag,
                                           Emit emit)
{
    const long long gid = C.t / g, ngroups = C.nthr / g;
    const int lane = (int)(C.t % g);
    const long long span = ngroups * R;
    const long long passes = (r1 - r0 + span - 1) / span;
    for (long long ps = 0; ps < passes; ps++) {
        int i[R];   // rows and columns fit in 32 bits (at most kFusedMaxRows block rows)
        int p0[R], p1[R];
#pragma unroll
        for (int q = 0; q < R; q++) {
            const long long iq = r0 + ps * span + (long long)q * ngroups + gid;
            i[q] = (int)iq;
            const bool v = iq < r1;
            if (ell > 0) {   // padded rows: no row-pointer round trip
                p0[q] = v ? i[q] * ell : 0;
                p1[q] = v ? p0[q] + ell : 0;
            } else {
                p0[q] = v ? rowptr[i[q]] : 0;
                p1[q] = v ? rowptr[i[q] + 1] : 0;
            }
        }
        T acc[R][BS];
#pragma unroll
        for (int q = 0; q < R; q++)
#pragma unroll
            for (int r = 0; r < BS; r++) acc[q][r] = T(0);
        for (int base = lane;; base += g) {
            bool ok[R], any = false;
            int col[R];
#pragma unroll
            for (int q = 0; q < R; q++) {
                ok[q] = p0[q] + base < p1[q];
                any |= ok[q];
                col[q] = ok[q] ? colidx[p0[q] + base] : 0;
            }
            if (!any) break;   // per lane; no shuffle inside the loop
            T xv[R][BS], av[R][BS * BS];
#pragma unroll
            for (int q = 0; q < R; q++) {
#pragma unroll
                for (int c = 0; c < BS; c++) xv[q][c] = ok[q] ? x[(long long)col[q] * BS + c] : T(0);
#pragma unroll
                for (int e = 0; e < BS * BS; e++) av[q][e] = ok[q] ? vals[(long long)e * ld + p0[q] + base] : T(0);
            }
#pragma unroll
            for (int q = 0; q < R; q++) {
                if (!ok[q] || (skip_diag && col[q] == i[q])) continue;
#pragma unroll
                for (int r = 0; r < BS; r++)
#pragma unroll
                    for (int c = 0; c < BS; c++) acc[q][r] = fma(av[q][r * BS + c], xv[q][c], acc[q][r]);
            }
        }
#pragma unroll
        for (int q = 0; q < R; q++)
#pragma unroll
            for (int r = 0; r < BS; r++) acc[q][r] = lanes_sum(acc[q][r], g);
#pragma unroll
        for (int q = 0; q < R; q++)
            if (i[q] < r1) emit((long long)i[q], lane, acc[q]);
    }
}

// Rows in flight per lane group, by the bytes of a block: what fits in 128 registers (512-thread
// CTAs) without spills; one row with 64 registers (1024-thread CTAs).
template <class T, int BS, int THREADS>
constexpr int kRowsInFlight = THREADS > kFusedThreads ? 1
                              : BS * BS * (int)sizeof(T) <= 16 ? 4 : BS * BS * (int)sizeof(T) <= 36 ? 3
                              : BS * BS * (int)sizeof(T) <= 72 ? 2 : 1;

// One colour [c0, c1) of a block GS / SOR sweep on level L: x_i <- D_i^-1 (b_i - sum_{j != i} A_ij x_j),
// relaxed by omega; output r of a row written by lane r (lanes loop when BS > lanes).
template <class T, int BS, int TH>
__device__ void gs_colour(const Ctx<T>& C, const FusedLevel<T>& L, int c0, int c1)
{
    const T w = C.P.omega;
    const bool pad = L.g_ell > 0;
    rows_multi<T, BS, kRowsInFlight<T, BS, TH>>(C, c0, c1, L.lanes, L.g_ell, L.a_rowptr, pad ? L.g_colidx : L.a_colidx,
                                            pad ? L.g_vals : L.a_vals, pad ? L.g_ld : L.a_ld, L.x, true,
                                            [&](long long i, int lane, const T* acc) {
        for (int r = lane; r < BS; r += L.lanes) {
            T v = T(0);
#pragma unroll
            for (int c = 0; c < BS; c++) v = fma(L.dinv[(long long)(r * BS + c) * L.nb + i], L.b[i * BS + c] - acc[c], v);
            if (w != T(1)) v = fma(w, v, (T(1) - w) * L.x[i * BS + r]);
            L.x[i * BS + r] = fin(v);
        }
    });
    cluster_sync();
}

template <class T, int BS, int TH>
__device__ void sweep(const Ctx<T>& C, const FusedLevel<T>& L, bool backward)
{
    if (!backward)
        for (int c = 0; c < L.ncol; c++) gs_colour<T, BS, TH>(C, L, L.colour_start[c], L.colour_start[c + 1]);
    else
        for (int c = L.ncol - 1; c >= 0; c--) gs_colour<T, BS, TH>(C, L, L.colour_start[c], L.colour_start[c + 1]);
}

// The smoother directions of BlockGaussSeidel::ExecuteOneIteration (alternating ones by iteration parity).
template <class T, int BS, int TH>
__device__ void smooth(const Ctx<T>& C, const FusedLevel<T>& L, int code, int iters)
{
    for (int it = 0; it < iters; it++) {
        if (code == kFusedForward) sweep<T, BS, TH>(C, L, false);
        else if (code == kFusedBackward) sweep<T, BS, TH>(C, L, true);
        else if (code == kFusedSymmetric) { sweep<T, BS, TH>(C, L, false); sweep<T, BS, TH>(C, L, true); }
        else if (code == kFusedAlternatingForward) sweep<T, BS, TH>(C, L, it % 2 != 0);
        else sweep<T, BS, TH>(C, L, it % 2 == 0);
    }
}

// L.r = L.b - A x (all blocks, the diagonal included).
template <class T, int BS, int TH>
__device__ void residual(const Ctx<T>& C, const FusedLevel<T>& L)
{
    const bool pad = L.ap_ell > 0;
    rows_multi<T, BS, kRowsInFlight<T, BS, TH>>(C, 0, L.nb, L.lanes, L.ap_ell, L.a_rowptr, pad ? L.ap_colidx : L.a_colidx,
                                            pad ? L.ap_vals : L.a_vals, pad ? L.ap_ld : L.a_ld, L.x, false,
                                            [&](long long i, int lane, const T* acc) {
        for (int r = lane; r < BS; r += L.lanes) L.r[i * BS + r] = L.b[i * BS + r] - acc[r];
    });
    cluster_sync();
}

// out (rows of M) = M in, or out += M in: the transfers as block products over CSR operators.
template <class T, int BS, int TH>
__device__ void product(const Ctx<T>& C, int rows, int g, const int* rowptr, const int* colidx, const T* vals,
                        long long ld, const T* in, T* out, bool add)
{
    rows_multi<T, BS, kRowsInFlight<T, BS, TH>>(C, 0, rows, g, 0, rowptr, colidx, vals, ld, in, false,
                                            [&](long long i, int lane, const T* acc) {
        for (int r = lane; r < BS; r += g) out[i * BS + r] = add ? out[i * BS + r] + acc[r] : fin(acc[r]);
    });
    cluster_sync();
}

template <class T>
__device__ void zero(const Ctx<T>& C, T* x, long long n)
{
    for (long long i = C.t; i < n; i += C.nthr) x[i] = T(0);
    cluster_sync();
}

// The coarsest level: x = C^{-1} b, C^{-1} dense FP64 row-major, FP64 accumulation; 8 lanes a row.
template <class T>
__device__ void coarse_solve(const Ctx<T>& C, const FusedLevel<T>& L)
{
    const long long n = C.P.n_coarse;
    row_passes(C, 0, n, 8, [&](long long i, bool valid, int lane) {
        double acc = 0.0;
        if (valid) {
            const double* a = C.P.cinv + i * n;
            for (long long j = lane; j < n; j += 8) acc = fma(a[j], (double)L.b[j], acc);
        }
        acc = lanes_sum(acc, 8);
        if (valid && lane == 0) L.x[i] = T(acc);
    });
    cluster_sync();
}

// The cycle from lev[0] down: descend (zero x on a fresh level, pre-smooth, residual, restrict) to the
// coarsest, solve there, then ascend (prolongate, post-smooth) until a level still owes a coarse
// correction (W-cycle), from which the next descent starts with the coarser level's x kept.
template <class T, int BS, int TH>
__device__ void run_cycle(const Ctx<T>& C)
{
    const FusedCycle<T>& P = C.P;
    const int last = P.nlev - 1;
    int done[kFusedMaxLevels];   // coarse corrections completed on each level of the current descent
    int l = 0;
    bool xz = P.x_zero != 0;
    while (true) {
        for (; l < last; l++) {
            const FusedLevel<T>& L = P.lev[l];
            const FusedLevel<T>& N = P.lev[l + 1];
            if (xz) zero(C, L.x, (long long)L.nb * BS);
            smooth<T, BS, TH>(C, L, P.pre, P.npre);
            residual<T, BS, TH>(C, L);
            product<T, BS, TH>(C, N.nb, L.t_lanes, L.r_rowptr, L.r_colidx, L.r_vals, L.r_ld, L.r, N.b, false);
            done[l] = 0;
            xz = true;
        }
        coarse_solve(C, P.lev[last]);
        bool again = false;
        while (l > 0) {
            l--;
            done[l]++;
            const int loops = (l + 1 == last || P.w_loops < 1) ? 1 : P.w_loops;
            if (done[l] < loops) {
                again = true;
                break;
            }
            const FusedLevel<T>& L = P.lev[l];
            const FusedLevel<T>& N = P.lev[l + 1];
            product<T, BS, TH>(C, L.nb, L.lanes, L.p_rowptr, L.p_colidx, L.p_vals, L.p_ld, N.x, L.x, true);
            smooth<T, BS, TH>(C, L, P.post, P.npost);
        }
        if (!again) return;
        l++;          // the next coarse correction of level l - 1 starts on level l
        xz = false;   // from the x the previous one left
    }
}

template <class T, int BS, int TH>
__global__ void __launch_bounds__(TH, 1) k_fused_cycle(const __grid_constant__ FusedCycle<T> P)
{
    pdl_wait_coarse();
    const Ctx<T> C{P, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x};
    run_cycle<T, BS, TH>(C);
}

template <class T, int TH>
void* kernel_for_th(int bs)
{
    switch (bs) {
    case 2: return (void*)k_fused_cycle<T, 2, TH>;
    case 3: return (void*)k_fused_cycle<T, 3, TH>;
    case 4: return (void*)k_fused_cycle<T, 4, TH>;
    case 6: return (void*)k_fused_cycle<T, 6, TH>;
    default: return nullptr;
    }
}

template <class T>
void* kernel_for(int bs, int threads)
{
    if (threads == kFusedThreads) return kernel_for_th<T, kFusedThreads>(bs);
    if (threads == kFusedThreadsWide) return kernel_for_th<T, kFusedThreadsWide>(bs);
    return nullptr;
}

void fused_config(cudaLaunchConfig_t& cfg, cudaLaunchAttribute* attr, int ctas, int threads, cudaStream_t s)
{
    cfg = {};
    cfg.gridDim = dim3(ctas);
    cfg.blockDim = dim3(threads);
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = ctas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
}

// Clusters above the portable size need the kernel's opt-in attribute, set once per kernel.
std::mutex g_fused_attr_mutex;

cudaError_t allow_large_clusters(const void* k)
{
    std::lock_guard<std::mutex> lock(g_fused_attr_mutex);
    return cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
}

}  // namespace

template <class T>
int fused_cycle_clusters(int bs, int ctas, int threads)
{
    const void* k = kernel_for<T>(bs, threads);
    if (!k || (ctas != kClusterCtasPortable && ctas != kClusterCtasLarge)) return 0;
    if (ctas > kClusterCtasPortable && allow_large_clusters(k) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[2];
    fused_config(cfg, attr, ctas, threads, nullptr);
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

template <class T>
cudaError_t launch_fused_cycle(const FusedCycle<T>& P, int bs, int ctas, int threads, cudaStream_t s)
{
    const void* k = kernel_for<T>(bs, threads);
    if (!k) return cudaErrorInvalidValue;
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[2];
    fused_config(cfg, attr, ctas, threads, s);
    void* args[] = {const_cast<FusedCycle<T>*>(&P)};
    return cudaLaunchKernelExC(&cfg, k, args);
}

template cudaError_t launch_fused_cycle<float>(const FusedCycle<float>&, int, int, int, cudaStream_t);
template cudaError_t launch_fused_cycle<dfl>(const FusedCycle<dfl>&, int, int, int, cudaStream_t);
template int fused_cycle_clusters<float>(int, int, int);
template int fused_cycle_clusters<dfl>(int, int, int);

}  // namespace fhg
