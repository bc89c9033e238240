// The coarse part of a multigrid cycle in one thread-block-cluster launch (fhg_coarse.cu).
#pragma once

#include <cuda_runtime.h>

#include "fhg_pair.h"

namespace fhg {

constexpr int kClusterCtasPortable = 8;   // CTAs of the one cluster: the portable maximum, or
constexpr int kClusterCtasLarge = 16;     // the non-portable one where the device runs it
constexpr int kFusedThreads = 512;        // threads per CTA (128 registers, up to four rows in flight)
constexpr int kFusedThreadsWide = 1024;   // or twice the warps per SM (64 registers, one row in flight)
constexpr int kFusedMaxLevels = 6;        // levels of a fused sub-cycle, the coarsest included
constexpr int kFusedMaxColours = 24;
constexpr int kFusedMaxRows = 65536;      // block rows of the largest level a fused sub-cycle takes
constexpr int kFusedDefaultRows = 8192;   // the same without timing at setup (autotuning off)

// Smoother directions of a fused sub-cycle (the GS codes; Jacobi is not fused).
enum { kFusedForward = 0, kFusedBackward = 1, kFusedSymmetric = 2, kFusedAlternatingForward = 3,
       kFusedAlternatingBackward = 4 };

// One level of the sub-cycle in the launch parameters: A in CSR form (all blocks, entry-major values,
// leading dimension a_ld), D^-1 entry-major (leading dimension nb), the colour offsets, P (this
// level's rows, the next level's columns) and R = P^T (the next level's rows), and the level's x, b
// and residual vectors. `lanes` threads (4, 8 or 16) walk one block row of A, `t_lanes` one row of R.
// On the coarsest level only x and b are used.
template <class T>
struct FusedLevel {
    int nb = 0, ncol = 0, lanes = 8, t_lanes = 8;
    int colour_start[kFusedMaxColours + 1] = {};
    const int* a_rowptr = nullptr;
    const int* a_colidx = nullptr;
    const T* a_vals = nullptr;
    long long a_ld = 0;
    // padded-row views when setup built them (row i's `ell` slots at i * ell, no row pointers): the
    // off-diagonal blocks for the sweeps (empty slots: the row's own column) and all of A for the
    // residual (empty slots: zero blocks)
    int g_ell = 0, ap_ell = 0;
    const int* g_colidx = nullptr;
    const T* g_vals = nullptr;
    long long g_ld = 0;
    const int* ap_colidx = nullptr;
    const T* ap_vals = nullptr;
    long long ap_ld = 0;
    const T* dinv = nullptr;
    const int* p_rowptr = nullptr;
    const int* p_colidx = nullptr;
    const T* p_vals = nullptr;
    long long p_ld = 0;
    const int* r_rowptr = nullptr;
    const int* r_colidx = nullptr;
    const T* r_vals = nullptr;
    long long r_ld = 0;
    T* x = nullptr;
    T* b = nullptr;
    T* r = nullptr;
};

template <class T>
struct FusedCycle {
    int nlev = 0;                 // levels, the coarsest included (lev[nlev - 1])
    int n_coarse = 0;             // unknowns of the coarsest level
    const double* cinv = nullptr; // its dense FP64 inverse, row-major
    int pre = 0, post = 1, npre = 1, npost = 1, w_loops = 1;
    int x_zero = 1;               // x of the first level starts at zero
    T omega = T(1);               // relaxation of the GS sweeps (block SOR when not 1)
    FusedLevel<T> lev[kFusedMaxLevels];
};

// One cluster of `ctas` CTAs (kClusterCtasPortable or kClusterCtasLarge) of `threads` threads
// (kFusedThreads or kFusedThreadsWide).
template <class T>
cudaError_t launch_fused_cycle(const FusedCycle<T>& P, int bs, int ctas, int threads, cudaStream_t s);
// Clusters of `ctas` CTAs of `threads` threads of the fused kernel that fit on the current device at
// once (0: it cannot run here).
template <class T>
int fused_cycle_clusters(int bs, int ctas, int threads);

}  // namespace fhg
