// The coarse part of a multigrid cycle in one kernel launch.
//
// Below some level the operators are small (tens of thousands of block rows or fewer) and a cycle
// there is a long chain of short phases: every colour of every smoothing sweep, the residual, the
// restriction, the coarsest solve, the prolongation. Launched one kernel per phase, each costs a
// launch slot of a few microseconds while its work takes a fraction of that. Here one thread-block
// cluster (kClusterCtas CTAs, co-scheduled by the hardware) runs the whole sub-cycle: every phase
// spreads its rows over all threads of the cluster, and phases are separated by the hardware
// cluster barrier (barrier.cluster with release/acquire semantics at cluster scope, which orders the
// global-memory writes of one phase before the reads of the next across the cluster's CTAs). The
// barrier cannot wait forever: all CTAs of a cluster are resident together and every thread takes
// the same path through the cycle.
//
// The arithmetic is the multigrid cycle of Multigrid::MultigridCycle (src/Solver/Multigrid/
// Multigrid.h:438-608) on the levels it covers: block Gauss-Seidel / SOR sweeps in colour order
// (BlockGaussSeidel.h:84-120, BlockSOR.h:199-227), r = b - A x (Multigrid.h:478), R r (Level.h:139-143),
// recursion (V, or W with WLoops), the coarsest dense solve, x += P e (Level.h:150-154, Multigrid.h:554).
// Each row is summed block by block in column order by one thread; the FP32 and pair (dfl) value
// types are instantiated.
#include "fhg_coarse.h"

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

template <class T>
struct Ctx {
    const FusedCycle<T>& P;
    long long t, nthr;   // thread index within the cluster, threads of the cluster
};

// One colour [c0, c1) of a block GS / SOR sweep on level L.
template <class T, int BS>
__device__ void gs_colour(const Ctx<T>& C, const FusedLevel<T>& L, int c0, int c1)
{
    const T w = C.P.omega;
    for (long long i = c0 + C.t; i < c1; i += C.nthr) {
        T acc[BS];
#pragma unroll
        for (int r = 0; r < BS; r++) acc[r] = T(0);
        const int p1 = L.a_rowptr[i + 1];
        for (int p = L.a_rowptr[i]; p < p1; p++) {
            const long long j = L.a_colidx[p];
            if (j == i) continue;
            T xv[BS];
#pragma unroll
            for (int c = 0; c < BS; c++) xv[c] = L.x[j * BS + c];
#pragma unroll
            for (int r = 0; r < BS; r++)
#pragma unroll
                for (int c = 0; c < BS; c++) acc[r] = fma(L.a_vals[(long long)(r * BS + c) * L.a_ld + p], xv[c], acc[r]);
        }
        T t[BS];
#pragma unroll
        for (int c = 0; c < BS; c++) t[c] = L.b[i * BS + c] - acc[c];
#pragma unroll
        for (int r = 0; r < BS; r++) {
            T v = T(0);
#pragma unroll
            for (int c = 0; c < BS; c++) v = fma(L.dinv[(long long)(r * BS + c) * L.nb + i], t[c], v);
            if (w != T(1)) v = fma(w, v, (T(1) - w) * L.x[i * BS + r]);
            L.x[i * BS + r] = fin(v);
        }
    }
    cluster_sync();
}

template <class T, int BS>
__device__ void sweep(const Ctx<T>& C, const FusedLevel<T>& L, bool backward)
{
    if (!backward)
        for (int c = 0; c < L.ncol; c++) gs_colour<T, BS>(C, L, L.colour_start[c], L.colour_start[c + 1]);
    else
        for (int c = L.ncol - 1; c >= 0; c--) gs_colour<T, BS>(C, L, L.colour_start[c], L.colour_start[c + 1]);
}

// The smoother directions of BlockGaussSeidel::ExecuteOneIteration (alternating ones by iteration parity).
template <class T, int BS>
__device__ void smooth(const Ctx<T>& C, const FusedLevel<T>& L, int code, int iters)
{
    for (int it = 0; it < iters; it++) {
        if (code == kFusedForward) sweep<T, BS>(C, L, false);
        else if (code == kFusedBackward) sweep<T, BS>(C, L, true);
        else if (code == kFusedSymmetric) { sweep<T, BS>(C, L, false); sweep<T, BS>(C, L, true); }
        else if (code == kFusedAlternatingForward) sweep<T, BS>(C, L, it % 2 != 0);
        else sweep<T, BS>(C, L, it % 2 == 0);
    }
}

// L.r = L.b - A x (all blocks, the diagonal included).
template <class T, int BS>
__device__ void residual(const Ctx<T>& C, const FusedLevel<T>& L)
{
    for (long long i = C.t; i < L.nb; i += C.nthr) {
        T acc[BS];
#pragma unroll
        for (int r = 0; r < BS; r++) acc[r] = T(0);
        const int p1 = L.a_rowptr[i + 1];
        for (int p = L.a_rowptr[i]; p < p1; p++) {
            const long long j = L.a_colidx[p];
            T xv[BS];
#pragma unroll
            for (int c = 0; c < BS; c++) xv[c] = L.x[j * BS + c];
#pragma unroll
            for (int r = 0; r < BS; r++)
#pragma unroll
                for (int c = 0; c < BS; c++) acc[r] = fma(L.a_vals[(long long)(r * BS + c) * L.a_ld + p], xv[c], acc[r]);
        }
#pragma unroll
        for (int r = 0; r < BS; r++) L.r[i * BS + r] = L.b[i * BS + r] - acc[r];
    }
    cluster_sync();
}

// out (rows of M) = M in, or out += M in: the transfers as block products over CSR operators.
template <class T, int BS>
__device__ void product(const Ctx<T>& C, int rows, const int* rowptr, const int* colidx, const T* vals, long long ld,
                        const T* in, T* out, bool add)
{
    for (long long i = C.t; i < rows; i += C.nthr) {
        T acc[BS];
#pragma unroll
        for (int r = 0; r < BS; r++) acc[r] = T(0);
        const int p1 = rowptr[i + 1];
        for (int p = rowptr[i]; p < p1; p++) {
            const long long j = colidx[p];
            T xv[BS];
#pragma unroll
            for (int c = 0; c < BS; c++) xv[c] = in[j * BS + c];
#pragma unroll
            for (int r = 0; r < BS; r++)
#pragma unroll
                for (int c = 0; c < BS; c++) acc[r] = fma(vals[(long long)(r * BS + c) * ld + p], xv[c], acc[r]);
        }
#pragma unroll
        for (int r = 0; r < BS; r++) out[i * BS + r] = add ? out[i * BS + r] + acc[r] : fin(acc[r]);
    }
    cluster_sync();
}

template <class T>
__device__ void zero(const Ctx<T>& C, T* x, long long n)
{
    for (long long i = C.t; i < n; i += C.nthr) x[i] = T(0);
    cluster_sync();
}

// The coarsest level: x = C^{-1} b, C^{-1} dense FP64 row-major, FP64 accumulation.
template <class T>
__device__ void coarse_solve(const Ctx<T>& C, const FusedLevel<T>& L)
{
    const long long n = C.P.n_coarse;
    for (long long i = C.t; i < n; i += C.nthr) {
        const double* a = C.P.cinv + i * n;
        double acc = 0.0;
        for (long long j = 0; j < n; j++) acc = fma(a[j], (double)L.b[j], acc);
        L.x[i] = T(acc);
    }
    cluster_sync();
}

template <class T, int BS>
__device__ void cycle(const Ctx<T>& C, int l, bool x_zero)
{
    const FusedLevel<T>& L = C.P.lev[l];
    if (l == C.P.nlev - 1) {
        coarse_solve(C, L);
        return;
    }
    const FusedLevel<T>& N = C.P.lev[l + 1];
    if (x_zero) zero(C, L.x, (long long)L.nb * BS);
    smooth<T, BS>(C, L, C.P.pre, C.P.npre);
    residual<T, BS>(C, L);
    product<T, BS>(C, N.nb, L.r_rowptr, L.r_colidx, L.r_vals, L.r_ld, L.r, N.b, false);
    const int loops = C.P.w_loops > 1 ? C.P.w_loops : 1;
    for (int w = 0; w < loops; w++) {
        cycle<T, BS>(C, l + 1, w == 0);
        if (l + 1 == C.P.nlev - 1) break;
    }
    product<T, BS>(C, L.nb, L.p_rowptr, L.p_colidx, L.p_vals, L.p_ld, N.x, L.x, true);
    smooth<T, BS>(C, L, C.P.post, C.P.npost);
}

template <class T, int BS>
__global__ void __launch_bounds__(kFusedThreads) k_fused_cycle(const __grid_constant__ FusedCycle<T> P)
{
    pdl_wait_coarse();
    const Ctx<T> C{P, (long long)blockIdx.x * blockDim.x + threadIdx.x, (long long)gridDim.x * blockDim.x};
    cycle<T, BS>(C, 0, P.x_zero != 0);
}

}  // namespace

namespace {

template <class T>
void fused_config(cudaLaunchConfig_t& cfg, cudaLaunchAttribute* attr, cudaStream_t s)
{
    cfg = {};
    cfg.gridDim = dim3(kClusterCtas);
    cfg.blockDim = dim3(kFusedThreads);
    cfg.stream = s;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kClusterCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
}

template <class T, int BS>
int clusters_of()
{
    cudaLaunchConfig_t cfg;
    cudaLaunchAttribute attr[2];
    fused_config<T>(cfg, attr, nullptr);
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_fused_cycle<T, BS>, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

}  // namespace

template <class T>
int fused_cycle_clusters(int bs)
{
    switch (bs) {
    case 2: return clusters_of<T, 2>();
    case 3: return clusters_of<T, 3>();
    case 4: return clusters_of<T, 4>();
    case 6: return clusters_of<T, 6>();
    default: return 0;
    }
}

template <class T>
cudaError_t launch_fused_cycle(const FusedCycle<T>& P, int bs, cudaStream_t s)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kClusterCtas);
    cfg.blockDim = dim3(kFusedThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kClusterCtas;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    switch (bs) {
    case 2: return cudaLaunchKernelEx(&cfg, k_fused_cycle<T, 2>, P);
    case 3: return cudaLaunchKernelEx(&cfg, k_fused_cycle<T, 3>, P);
    case 4: return cudaLaunchKernelEx(&cfg, k_fused_cycle<T, 4>, P);
    case 6: return cudaLaunchKernelEx(&cfg, k_fused_cycle<T, 6>, P);
    default: return cudaErrorInvalidValue;
    }
}

template cudaError_t launch_fused_cycle<float>(const FusedCycle<float>&, int, cudaStream_t);
template cudaError_t launch_fused_cycle<dfl>(const FusedCycle<dfl>&, int, cudaStream_t);
template int fused_cycle_clusters<float>(int);
template int fused_cycle_clusters<dfl>(int);

}  // namespace fhg
