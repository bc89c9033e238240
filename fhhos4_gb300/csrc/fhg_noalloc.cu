// fhg_residual_norm_noalloc: the residual 2-norm ||b - A x|| of a face-block system, computed
// without allocating anything.
//
// Who needs it: callers that may not allocate device memory when they check a solution - a
// serving process that reserved all of the GPU's memory for its own pool or budget at start-up,
// an embedder that must not let a library grow its footprint after start-up, and latency-bound
// loops that cannot afford cudaMalloc's device-wide synchronisation. They pass the operator, x,
// b and a one-double output buffer, all in memory they own; the per-block partial sums this
// reduction needs live in a fixed array compiled into the library instead of a temporary
// allocation.
//
// The scratch array `g_residual_partials` below (FHG_NOALLOC_MAX_PARTIALS doubles, 1 MiB) is a
// file-scope __device__ array: every GPU that loads the library holds it until the process
// exits. Host code cannot pass its name to a kernel (the name is a host-side stand-in, not a
// device address), so the first call on each device (and the first call after that device's
// context was replaced, e.g. by cudaDeviceReset) looks its device address up with
// cudaGetSymbolAddress while that device is current and caches it with the context's id; later
// calls make no runtime lookup. All calls share the array: a call overwrites the
// partial sums it uses (nothing accumulates across calls, so nothing needs clearing), and two
// calls that overlap on the GPU - on different streams, or from different host threads at once -
// race on it and must be serialised by the caller.
#include "fhg.h"

#include <cuda_runtime.h>

#include <mutex>

namespace {

constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_residual_partials[FHG_NOALLOC_MAX_PARTIALS];

template <int G>
__device__ __forceinline__ double group_sum(double v)
{
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
    return v;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Residual rows of the block-sparse residual kernel, reduced to one partial sum of r_i^2 per
// CTA instead of being stored (same block layout and lane mapping as the library's SpMV).
template <int BS, int G>
__global__ void __launch_bounds__(kThreads) k_residual_norm_partials(int nbr, const int* __restrict__ rowptr,
                                                                     const int* __restrict__ colidx,
                                                                     const double* __restrict__ vals, long long ld,
                                                                     const double* __restrict__ x,
                                                                     const double* __restrict__ b,
                                                                     double* __restrict__ partials)
{
    __shared__ double sh[kThreads / 32];
    const int lane = threadIdx.x & (G - 1);
    const int row = (int)(((long long)blockIdx.x * kThreads + threadIdx.x) / G);
    double acc[BS];
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = 0.0;
    if (row < nbr) {
        const int p1 = rowptr[row + 1];
        for (int p = rowptr[row] + lane; p < p1; p += G) {
            const int col = colidx[p];
            double xv[BS];
#pragma unroll
            for (int c = 0; c < BS; c++) xv[c] = x[(long long)col * BS + c];
#pragma unroll
            for (int r = 0; r < BS; r++)
#pragma unroll
                for (int c = 0; c < BS; c++) acc[r] = fma(vals[(long long)(r * BS + c) * ld + p], xv[c], acc[r]);
        }
    }
#pragma unroll
    for (int r = 0; r < BS; r++) acc[r] = group_sum<G>(acc[r]);
    double sq = 0.0;
    if (row < nbr && lane == 0) {
#pragma unroll
        for (int r = 0; r < BS; r++) {
            const double ri = b[(long long)row * BS + r] - acc[r];
            sq = fma(ri, ri, sq);
        }
    }
    sq = warp_sum(sq);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; w++) t += sh[w];
        partials[blockIdx.x] = t;
    }
}

// out = sqrt(sum of the n partial sums), summed in a fixed order by one CTA.
__global__ void __launch_bounds__(kThreads) k_residual_norm_finalize(const double* __restrict__ partials, int n,
                                                                     double* __restrict__ out)
{
    __shared__ double sh[kThreads / 32];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += kThreads) v += partials[i];
    v = warp_sum(v);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; w++) t += sh[w];
        *out = sqrt(t);
    }
}

std::mutex g_setup_mutex;
double* g_partials_ptr[kMaxDevices] = {nullptr};
unsigned long long g_partials_ctx[kMaxDevices] = {0};

// Id of the current context (0 when none or when the driver cannot say), through the driver entry
// points the runtime hands out, so that the library needs no link against libcuda.
unsigned long long current_context_id()
{
    using GetCurrent = int (*)(void**);
    using GetId = int (*)(void*, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        looked_up = true;
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (GetCurrent)f;
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (GetId)f;
    }
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

// Device address of the scratch array on `device` (must be current): looked up on the first call
// on a device and again whenever the device's current context differs from the one it was looked
// up in (a context id of 0, unknown, always looks it up).
int scratch_address(int device, double** ptr)
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    const unsigned long long ctx = current_context_id();
    if (!g_partials_ptr[device] || ctx == 0 || ctx != g_partials_ctx[device]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_residual_partials) != cudaSuccess || !p) {
            g_partials_ptr[device] = nullptr;
            return FHG_ERR_CUDA;
        }
        g_partials_ptr[device] = (double*)p;
        g_partials_ctx[device] = current_context_id();
    }
    *ptr = g_partials_ptr[device];
    return FHG_OK;
}

template <int BS>
void launch(int lanes, unsigned grid, cudaStream_t s, int nbr, const int* rowptr, const int* colidx,
            const double* vals, long long ld, const double* x, const double* b, double* partials)
{
    switch (lanes) {
    case 4: k_residual_norm_partials<BS, 4><<<grid, kThreads, 0, s>>>(nbr, rowptr, colidx, vals, ld, x, b, partials); break;
    case 8: k_residual_norm_partials<BS, 8><<<grid, kThreads, 0, s>>>(nbr, rowptr, colidx, vals, ld, x, b, partials); break;
    case 16: k_residual_norm_partials<BS, 16><<<grid, kThreads, 0, s>>>(nbr, rowptr, colidx, vals, ld, x, b, partials); break;
    default: k_residual_norm_partials<BS, 32><<<grid, kThreads, 0, s>>>(nbr, rowptr, colidx, vals, ld, x, b, partials); break;
    }
}

}  // namespace

extern "C" int fhg_residual_norm_noalloc(int device, int n_block_rows, int block_size, int lanes,
                                         const int* rowptr, const int* colidx, const double* vals, long long ld,
                                         const double* x, const double* b, double* norm_out, void* stream)
{
    if (device < 0 || device >= kMaxDevices || n_block_rows <= 0 || !rowptr || !colidx || !vals || !x || !b ||
        !norm_out)
        return FHG_ERR_INVALID_ARG;
    if (block_size != 2 && block_size != 3 && block_size != 4 && block_size != 6) return FHG_ERR_UNSUPPORTED;
    if (lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32) return FHG_ERR_INVALID_ARG;
    const long long ctas = ((long long)n_block_rows * lanes + kThreads - 1) / kThreads;
    if (ctas > FHG_NOALLOC_MAX_PARTIALS) return FHG_ERR_TOO_LARGE;  // more partial sums than the scratch holds
    int previous = 0;
    if (cudaGetDevice(&previous) != cudaSuccess) return FHG_ERR_CUDA;
    if (previous != device && cudaSetDevice(device) != cudaSuccess) return FHG_ERR_CUDA;
    // An error left pending by the caller's earlier work is reported, not cleared, and nothing is
    // launched; after the launches, cudaGetLastError sees this call's own launch errors only.
    int rc = cudaPeekAtLastError() == cudaSuccess ? FHG_OK : FHG_ERR_CUDA;
    double* partials = nullptr;
    if (rc == FHG_OK) rc = scratch_address(device, &partials);
    if (rc == FHG_OK) {
        cudaStream_t s = (cudaStream_t)stream;
        const unsigned grid = (unsigned)ctas;
        switch (block_size) {
        case 2: launch<2>(lanes, grid, s, n_block_rows, rowptr, colidx, vals, ld, x, b, partials); break;
        case 3: launch<3>(lanes, grid, s, n_block_rows, rowptr, colidx, vals, ld, x, b, partials); break;
        case 4: launch<4>(lanes, grid, s, n_block_rows, rowptr, colidx, vals, ld, x, b, partials); break;
        default: launch<6>(lanes, grid, s, n_block_rows, rowptr, colidx, vals, ld, x, b, partials); break;
        }
        k_residual_norm_finalize<<<1, kThreads, 0, s>>>(partials, (int)ctas, norm_out);
        if (cudaGetLastError() != cudaSuccess) rc = FHG_ERR_CUDA;
    }
    if (previous != device) cudaSetDevice(previous);
    return rc;
}
