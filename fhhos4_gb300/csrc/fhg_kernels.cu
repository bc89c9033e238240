// CUDA kernels of the fhhos4 solve phase for GB300 (sm_103a): the Krylov kernels (FP64 and
// double-FP32), the fused outer products with their dot products, and the device-side solve loop;
// the block-sparse kernels shared with the pair instantiations are in fhg_bsr_kernels.cuh.
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
#include "fhg_bsr_kernels.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <type_traits>
#include <utility>

namespace fhg {

std::atomic<long long> g_kernel_launches{0};

namespace {

// Ad = A d, with per-CTA partials of d.Ad and r.d (fixed grid, grid-stride over block rows).
template <int BS, int G>
__global__ void __launch_bounds__(kReduceThreads) k_bsr_spmv_dots(int nbr, const int* __restrict__ rowptr,
                                                                  const int* __restrict__ colidx,
                                                                  const double* __restrict__ vals, long long ld,
                                                                  const double* __restrict__ d,
                                                                  const double* __restrict__ rvec,
                                                                  double* __restrict__ Ad,
                                                                  double* __restrict__ partials)
{
    pdl_wait();
    __shared__ double sh[33];
    const int lane = threadIdx.x & (G - 1);
    // Loop bounds are uniform per warp (every lane runs the same shuffle rounds).
    constexpr int kGroupsPerWarp = 32 / G;
    const long long warp_id = ((long long)blockIdx.x * kReduceThreads + threadIdx.x) >> 5;
    const long long warp_stride = (long long)kReduceCtas * kReduceThreads / 32 * kGroupsPerWarp;
    const int group_in_warp = (threadIdx.x & 31) / G;
    double dad = 0.0, rd = 0.0;
    for (long long row0 = warp_id * kGroupsPerWarp; row0 < nbr; row0 += warp_stride) {
        const int row = (int)(row0 + group_in_warp);
        double acc[BS];
#pragma unroll
        for (int r = 0; r < BS; r++) acc[r] = 0.0;
        const bool active = row < nbr;
        if (active) accumulate_row<double, BS, G, 2>(rowptr[row], rowptr[row + 1], lane, colidx, vals, ld, d, acc, UseAll());
#pragma unroll
        for (int r = 0; r < BS; r++) acc[r] = group_sum<G>(acc[r]);
        if (active) {
#pragma unroll
            for (int r = 0; r < BS; r++) {
                if (lane == r % G) {
                    const long long i = (long long)row * BS + r;
                    Ad[i] = acc[r];
                    const double di = d[i];
                    dad = fma(di, acc[r], dad);
                    rd = fma(rvec[i], di, rd);
                }
            }
        }
    }
    const double s1 = block_sum(dad, sh);
    const double s2 = block_sum(rd, sh);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = s1;
        partials[kReduceCtas + blockIdx.x] = s2;
    }
}


// ---------------------------------------------------------------------------
// Ad = Â d in double-FP32 ("double-single") arithmetic on the FP32 pipe, with per-CTA partials
// of d.Ad and r.d. Â = a_hi + a_lo, d = d_hi + d_lo, r = r_hi + r_lo and the result Ad are FP32
// pairs (the lo parts the FP32-rounded remainders); every product a_hi*d_hi is split exactly with
// an FMA, the cross terms a_hi*d_lo + a_lo*d_hi are added in FP32, a_lo*d_lo (2^-48 relative) is
// dropped, and the running sum is a (hi, lo) FP32 pair kept exact with TwoSum. Relative accuracy
// of every term ~2^-47: the result carries FP64-class accuracy (a few units in 1e-14) with no
// FP64 instruction per element (GB300's FP64 pipe is 56x slower than FP32); the dot products are
// summed per thread as pairs too and only the per-thread sums are widened to FP64.
template <int BS, int G>
__global__ void __launch_bounds__(kReduceThreads) k_bsr_spmv_dots_df(int nbr, const int* __restrict__ rowptr,
                                                                     const int* __restrict__ colidx,
                                                                     const float* __restrict__ vhi,
                                                                     const float* __restrict__ vlo, long long ld,
                                                                     const float* __restrict__ dhi,
                                                                     const float* __restrict__ dlo,
                                                                     const float* __restrict__ rhi,
                                                                     const float* __restrict__ rlo,
                                                                     float* __restrict__ Adhi, float* __restrict__ Adlo,
                                                                     double* __restrict__ partials)
{
    pdl_wait();
    __shared__ double sh_red[33];
    const int lane = threadIdx.x & (G - 1);
    constexpr int kGroupsPerWarp = 32 / G;
    const long long warp_id = ((long long)blockIdx.x * kReduceThreads + threadIdx.x) >> 5;
    const long long warp_stride = (long long)kReduceCtas * kReduceThreads / 32 * kGroupsPerWarp;
    const int group_in_warp = (threadIdx.x & 31) / G;
    float dad_h = 0.f, dad_l = 0.f, rd_h = 0.f, rd_l = 0.f;
    for (long long row0 = warp_id * kGroupsPerWarp; row0 < nbr; row0 += warp_stride) {
        const int row = (int)(row0 + group_in_warp);
        float hi[BS], lo[BS];
#pragma unroll
        for (int r = 0; r < BS; r++) { hi[r] = 0.f; lo[r] = 0.f; }
        float dvh = 0.f, dvl = 0.f, rvh = 0.f, rvl = 0.f;
        if (row < nbr) {
            if (lane < BS) {
                const long long i = (long long)row * BS + lane;
                dvh = dhi[i];
                dvl = dlo[i];
                rvh = rhi[i];
                rvl = rlo[i];
            }
            const int p1 = rowptr[row + 1];
            for (int p = rowptr[row] + lane; p < p1; p += G) {
                const int col = colidx[p];
                float ahv[BS * BS], alv[BS * BS], xh[BS], xl[BS];
#pragma unroll
                for (int e = 0; e < BS * BS; e++) {
                    ahv[e] = vhi[(long long)e * ld + p];
                    alv[e] = vlo[(long long)e * ld + p];
                }
#pragma unroll
                for (int c = 0; c < BS; c++) { xh[c] = dhi[(long long)col * BS + c]; xl[c] = dlo[(long long)col * BS + c]; }
#pragma unroll
                for (int r = 0; r < BS; r++)
#pragma unroll
                    for (int c = 0; c < BS; c++) {
                        float ph, pl;
                        df_mul(ahv[r * BS + c], alv[r * BS + c], xh[c], xl[c], ph, pl);
                        df_add(hi[r], lo[r], ph, pl);
                    }
            }
        }
#pragma unroll
        for (int r = 0; r < BS; r++) {
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, hi[r], o, G);
                const float ol = __shfl_xor_sync(0xffffffffu, lo[r], o, G);
                df_add(hi[r], lo[r], oh, ol);
            }
        }
        if (row < nbr) {
#pragma unroll
            for (int r = 0; r < BS; r++) {
                if (lane == r) {   // G >= BS: launch_spmv_dots_df rejects smaller G
                    const long long i = (long long)row * BS + r;
                    float ah, al, ph, pl;
                    df_norm(hi[r], lo[r], ah, al);
                    Adhi[i] = ah;
                    Adlo[i] = al;
                    df_mul(dvh, dvl, ah, al, ph, pl);
                    df_add(dad_h, dad_l, ph, pl);
                    df_mul(rvh, rvl, dvh, dvl, ph, pl);
                    df_add(rd_h, rd_l, ph, pl);
                }
            }
        }
    }
    const double s1 = block_sum((double)dad_h + (double)dad_l, sh_red);
    const double s2 = block_sum((double)rd_h + (double)rd_l, sh_red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = s1;
        partials[kReduceCtas + blockIdx.x] = s2;
    }
}

// The same on the slot-major pair view of Â (slot s of row i at s * nbr + i; values as interleaved
// FP32 pairs, one 8-byte load each; empty slots hold zero pairs and a column of the row): one thread
// per block row over the fixed grid, the row's column indices and then its slots' values and d
// entries loaded ahead of the sums, no row pointers and no lane reduction. The row's terms are
// summed block by block in column order with the same pair arithmetic per term.
template <int BS, int W>
__global__ void __launch_bounds__(kReduceThreads, 2) k_bsr_spmv_dots_df_slot(int nbr, const int* __restrict__ colidx,
                                                                          const dfl* __restrict__ vals, long long ld,
                                                                          const float* __restrict__ dhi,
                                                                          const float* __restrict__ dlo,
                                                                          const float* __restrict__ rhi,
                                                                          const float* __restrict__ rlo,
                                                                          float* __restrict__ Adhi,
                                                                          float* __restrict__ Adlo,
                                                                          double* __restrict__ partials)
{
    pdl_wait();
    __shared__ double sh_red[33];
    float dad_h = 0.f, dad_l = 0.f, rd_h = 0.f, rd_l = 0.f;
    const long long stride = (long long)kReduceCtas * kReduceThreads;
    for (long long row = (long long)blockIdx.x * kReduceThreads + threadIdx.x; row < nbr; row += stride) {
        int col[W];
#pragma unroll
        for (int k = 0; k < W; k++) col[k] = colidx[(long long)k * nbr + row];
        float hi[BS], lo[BS];
#pragma unroll
        for (int r = 0; r < BS; r++) { hi[r] = 0.f; lo[r] = 0.f; }
#pragma unroll
        for (int k = 0; k < W; k++) {
            const long long p = (long long)k * nbr + row;
            float xh[BS], xl[BS];
#pragma unroll
            for (int c = 0; c < BS; c++) {
                xh[c] = dhi[(long long)col[k] * BS + c];
                xl[c] = dlo[(long long)col[k] * BS + c];
            }
#pragma unroll
            for (int r = 0; r < BS; r++)
#pragma unroll
                for (int c = 0; c < BS; c++) {
                    const dfl a = vals[(long long)(r * BS + c) * ld + p];
                    float ph, pl;
                    df_mul(a.h, a.l, xh[c], xl[c], ph, pl);
                    df_add(hi[r], lo[r], ph, pl);
                }
        }
#pragma unroll
        for (int r = 0; r < BS; r++) {
            const long long i = row * BS + r;
            float ah, al, ph, pl;
            df_norm(hi[r], lo[r], ah, al);
            Adhi[i] = ah;
            Adlo[i] = al;
            const float dvh = dhi[i], dvl = dlo[i];
            df_mul(dvh, dvl, ah, al, ph, pl);
            df_add(dad_h, dad_l, ph, pl);
            df_mul(rhi[i], rlo[i], dvh, dvl, ph, pl);
            df_add(rd_h, rd_l, ph, pl);
        }
    }
    const double s1 = block_sum((double)dad_h + (double)dad_l, sh_red);
    const double s2 = block_sum((double)rd_h + (double)rd_l, sh_red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = s1;
        partials[kReduceCtas + blockIdx.x] = s2;
    }
}

// r = b - A x with compensated summation (Ogita, Rump and Oishi 2005, "Accurate sum and dot
// product", Dot2): every product split exactly by an FMA (TwoProduct), the running sum kept exact by
// TwoSum, the rounding errors summed apart and added once, so r_i carries an error of about one unit
// of FP64 in r_i itself whatever the cancellation between b_i and the products (which bounds a plain
// FP64 evaluation at u sum_j |a_ij x_j|). One thread per block row over a fixed grid; per-CTA
// partials of sum r_i^2. FP64 pipe work of about ten operations per term: used only when the plain
// FP64 true residual misses the tolerance. `enable` (optional, the device loop): run only if *enable.
template <int BS>
__global__ void __launch_bounds__(kReduceThreads) k_bsr_residual_comp(int nbr, const int* __restrict__ rowptr,
                                                                      const int* __restrict__ colidx,
                                                                      const double* __restrict__ vals, long long ld,
                                                                      const double* __restrict__ x,
                                                                      const double* __restrict__ b,
                                                                      double* __restrict__ r,
                                                                      double* __restrict__ partials,
                                                                      const int* __restrict__ enable)
{
    pdl_wait();
    if (enable && *enable == 0) return;
    __shared__ double sh[33];
    double rr = 0.0;
    for (long long row = (long long)blockIdx.x * kReduceThreads + threadIdx.x; row < nbr; row += kRedStride) {
        double sum[BS], err[BS];
#pragma unroll
        for (int k = 0; k < BS; k++) { sum[k] = b[row * BS + k]; err[k] = 0.0; }
        for (int p = rowptr[row]; p < rowptr[row + 1]; p++) {
            const long long col = colidx[p];
            double xv[BS];
#pragma unroll
            for (int c = 0; c < BS; c++) xv[c] = x[col * BS + c];
#pragma unroll
            for (int k = 0; k < BS; k++)
#pragma unroll
                for (int c = 0; c < BS; c++) {
                    const double a = vals[(long long)(k * BS + c) * ld + p];
                    const double pr = a * xv[c];
                    const double q = fma(a, xv[c], -pr);        // a x = pr + q exactly
                    const double t = sum[k] - pr;                // TwoSum(sum, -pr)
                    const double z = t - sum[k];
                    const double e = (sum[k] - (t - z)) + (-pr - z);
                    sum[k] = t;
                    err[k] += e - q;
                }
        }
#pragma unroll
        for (int k = 0; k < BS; k++) {
            const double v = sum[k] + err[k];
            r[row * BS + k] = v;
            rr = fma(v, v, rr);
        }
    }
    rr = block_sum(rr, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = rr;
}

__global__ void __launch_bounds__(kReduceThreads) k_dot(long long n, const double* __restrict__ a,
                                                        const double* __restrict__ b, double* __restrict__ partials)
{
    pdl_wait();
    __shared__ double sh[33];
    double v = 0.0;
    for_each_element(n, [&](long long i) { return Pair2<double, double>{a[i], b[i]}; },
                     [&](long long, const Pair2<double, double>& e) { v = fma(e.a, e.b, v); });
    v = block_sum(v, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
}

__global__ void __launch_bounds__(kReduceThreads) k_dot_mixed(long long n, const float* __restrict__ a,
                                                              const double* __restrict__ b, double* __restrict__ partials)
{
    pdl_wait();
    __shared__ double sh[33];
    double v = 0.0;
    for_each_element(n, [&](long long i) { return Pair2<float, double>{a[i], b[i]}; },
                     [&](long long, const Pair2<float, double>& e) { v = fma((double)e.a, e.b, v); });
    v = block_sum(v, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
}

__global__ void __launch_bounds__(kReduceThreads) k_fcg_direction_mixed(long long n, const float* __restrict__ z,
                                                                        const double* __restrict__ dp,
                                                                        const double* __restrict__ partials,
                                                                        const double* __restrict__ dadp, double* __restrict__ d,
                                                                        float* __restrict__ dhi, float* __restrict__ dlo)
{
    pdl_wait();
    __shared__ double sh[33];
    const double s = reduce_partials(partials, sh) / *dadp;
    for_each_element(n, [&](long long i) { return Pair2<float, double>{z[i], dp[i]}; },
                     [&](long long i, const Pair2<float, double>& e) {
                         const double v = (double)e.a - s * e.b;
                         d[i] = v;
                         if (dhi) {
                             const float h = (float)v;
                             dhi[i] = h;
                             dlo[i] = (float)(v - (double)h);
                         }
                     });
}

__global__ void __launch_bounds__(kReduceThreads) k_fcg_direction(long long n, const double* z, const double* __restrict__ dp,
                                                                  const double* __restrict__ partials,
                                                                  const double* __restrict__ dadp, double* d)
{
    pdl_wait();
    __shared__ double sh[33];
    const double s = reduce_partials(partials, sh) / *dadp;
    for_each_element(n, [&](long long i) { return Pair2<double, double>{z[i], dp[i]}; },
                     [&](long long i, const Pair2<double, double>& e) { d[i] = e.a - s * e.b; });
}

__global__ void __launch_bounds__(kReduceThreads) k_krylov_step(long long n, double* __restrict__ x, double* __restrict__ r,
                                                                const double* __restrict__ d, const double* __restrict__ Ad,
                                                                const double* __restrict__ pnum, const double* __restrict__ pden,
                                                                double* __restrict__ den_out, double* __restrict__ prr,
                                                                float* __restrict__ r32)
{
    pdl_wait();
    __shared__ double sh[33];
    const double num = reduce_partials(pnum, sh);
    const double den = reduce_partials(pden, sh);
    const double alpha = num / den;
    if (blockIdx.x == 0 && threadIdx.x == 0 && den_out) *den_out = den;
    double rr = 0.0;
    for_each_element(n, [&](long long i) { return Quad4<double>{x[i], d[i], r[i], Ad[i]}; },
                     [&](long long i, const Quad4<double>& e) {
                         x[i] = e.a + alpha * e.b;
                         const double ri = e.c - alpha * e.d;
                         r[i] = ri;
                         if (r32) r32[i] = (float)ri;
                         rr = fma(ri, ri, rr);
                     });
    rr = block_sum(rr, sh);
    if (threadIdx.x == 0) prr[blockIdx.x] = rr;
}

// Double-FP32 outer iteration: r, d and Ad are FP32 pairs (hi, lo), so that the direction update
// and the dot products run no FP64 instruction per element; the Krylov scalars stay FP64 and are
// split into pairs once per thread. x stays FP64: its rounding sets the floor of the true residual
// ||b - A x|| (about kappa times the unit roundoff of x), which a pair (2^-48) would raise 32-fold.
// partials of z.Adp with z the FP32 V-cycle output.
// z is the FP32 V-cycle output, or (z2 non-null) the pair V-cycle's output as interleaved pairs.
__global__ void __launch_bounds__(kReduceThreads) k_dot_df(long long n, const float* __restrict__ z,
                                                           const dfl* __restrict__ z2,
                                                           const float* __restrict__ ah, const float* __restrict__ al,
                                                           double* __restrict__ partials)
{
    pdl_wait();
    __shared__ double sh[33];
    float vh = 0.f, vl = 0.f;
    struct E {
        float zh, zl, h, l;
    };
    for_each_element(n,
                     [&](long long i) {
                         if (z2) {
                             const dfl p = z2[i];
                             return E{p.h, p.l, ah[i], al[i]};
                         }
                         return E{z[i], 0.f, ah[i], al[i]};
                     },
                     [&](long long, const E& e) {
                         float ph, pl;
                         df_mul(e.zh, e.zl, e.h, e.l, ph, pl);
                         df_add(vh, vl, ph, pl);
                     });
    const double v = block_sum((double)vh + (double)vl, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = v;
}

// d = z - s dp, s = sum(partials_zadp) / *dadp.
__global__ void __launch_bounds__(kReduceThreads) k_fcg_direction_df(long long n, const float* __restrict__ z,
                                                                     const dfl* __restrict__ z2,
                                                                     const float* __restrict__ dph,
                                                                     const float* __restrict__ dpl,
                                                                     const double* __restrict__ partials,
                                                                     const double* __restrict__ dadp,
                                                                     float* __restrict__ dh, float* __restrict__ dl)
{
    pdl_wait();
    __shared__ double sh[33];
    float sh_, sl_;
    df_split(reduce_partials(partials, sh) / *dadp, sh_, sl_);
    struct E {
        float zh, zl, h, l;
    };
    for_each_element(n,
                     [&](long long i) {
                         if (z2) {
                             const dfl p = z2[i];
                             return E{p.h, p.l, dph[i], dpl[i]};
                         }
                         return E{z[i], 0.f, dph[i], dpl[i]};
                     },
                     [&](long long i, const E& e) {
                         float ph, pl, h, l;
                         df_mul(sh_, sl_, e.h, e.l, ph, pl);
                         df_sum(e.zh, e.zl, -ph, -pl, h, l);
                         dh[i] = h;
                         dl[i] = l;
                     });
}

// alpha = num / den; x += alpha d (FP64); r -= alpha Ad (rh is the next V-cycle's FP32 right-hand
// side); partials_rr of r.r; *den_out = den.
__global__ void __launch_bounds__(kReduceThreads) k_krylov_step_df(long long n, double* __restrict__ x,
                                                                   float* __restrict__ rh,
                                                                   float* __restrict__ rl, const float* __restrict__ dh,
                                                                   const float* __restrict__ dl,
                                                                   const float* __restrict__ Adh,
                                                                   const float* __restrict__ Adl,
                                                                   const double* __restrict__ pnum,
                                                                   const double* __restrict__ pden,
                                                                   double* __restrict__ den_out, double* __restrict__ prr,
                                                                   dfl* __restrict__ r2)
{
    pdl_wait();
    __shared__ double sh[33];
    const double num = reduce_partials(pnum, sh);
    const double den = reduce_partials(pden, sh);
    if (blockIdx.x == 0 && threadIdx.x == 0 && den_out) *den_out = den;
    const double alpha = num / den;
    float ah, al;
    df_split(alpha, ah, al);
    float rrh = 0.f, rrl = 0.f;
    struct E {
        double x;
        float rh, rl, dh, dl, ah, al;
    };
    for_each_element(n, [&](long long i) { return E{x[i], rh[i], rl[i], dh[i], dl[i], Adh[i], Adl[i]}; },
                     [&](long long i, const E& e) {
                         float ph, pl, h, l;
                         x[i] = fma(alpha, (double)e.dh + (double)e.dl, e.x);
                         df_mul(ah, al, e.ah, e.al, ph, pl);
                         df_sum(e.rh, e.rl, -ph, -pl, h, l);
                         rh[i] = h;
                         rl[i] = l;
                         if (r2) r2[i] = dfl(h, l);   // the pair V-cycle's right-hand side
                         df_mul(h, l, h, l, ph, pl);
                         df_add(rrh, rrl, ph, pl);
                     });
    const double rr = block_sum((double)rrh + (double)rrl, sh);
    if (threadIdx.x == 0) prr[blockIdx.x] = rr;
}

// FP64 -> FP32 pair (the start of the double-FP32 iteration and residual replacement).
__global__ void __launch_bounds__(kThreads) k_split_df(long long n, const double* __restrict__ v, float* __restrict__ h,
                                                      float* __restrict__ l, dfl* __restrict__ v2)
{
    pdl_wait();
    const long long i = (long long)blockIdx.x * kThreads + threadIdx.x;
    if (i < n) {
        float hi, lo;
        df_split(v[i], hi, lo);
        h[i] = hi;
        l[i] = lo;
        if (v2) v2[i] = dfl(hi, lo);
    }
}


__global__ void __launch_bounds__(kReduceThreads) k_cg_step(long long n, double* __restrict__ x, double* __restrict__ r,
                                                            const double* __restrict__ d, const double* __restrict__ Ad,
                                                            const double* __restrict__ num, const double* __restrict__ pden,
                                                            double* __restrict__ prr)
{
    pdl_wait();
    __shared__ double sh[33];
    const double den = reduce_partials(pden, sh);
    const double alpha = *num / den;
    double rr = 0.0;
    for_each_element(n, [&](long long i) { return Quad4<double>{x[i], d[i], r[i], Ad[i]}; },
                     [&](long long i, const Quad4<double>& e) {
                         x[i] = e.a + alpha * e.b;
                         const double ri = e.c - alpha * e.d;
                         r[i] = ri;
                         rr = fma(ri, ri, rr);
                     });
    rr = block_sum(rr, sh);
    if (threadIdx.x == 0) prr[blockIdx.x] = rr;
}

__global__ void __launch_bounds__(kReduceThreads) k_cg_direction(long long n, const double* __restrict__ z,
                                                                 const double* __restrict__ beta, double* __restrict__ d)
{
    pdl_wait();
    const double bt = *beta;
    for_each_element(n, [&](long long i) { return Pair2<double, double>{z[i], d[i]}; },
                     [&](long long i, const Pair2<double, double>& e) { d[i] = e.a + bt * e.b; });
}

__global__ void __launch_bounds__(kReduceThreads) k_finalize_norm(const double* __restrict__ prr, const double* __restrict__ bnorm,
                                                                  double* nr_out, double* hist, int* counter, int hist_len)
{
    pdl_wait();
    __shared__ double sh[33];
    const double rn = sqrt(reduce_partials(prr, sh));
    if (threadIdx.x == 0) {
        const double bn = *bnorm;
        const double nr = bn > 0.0 ? rn / bn : rn;
        *nr_out = nr;
        const int k = *counter;
        if (k < hist_len) hist[k] = nr;
        *counter = k + 1;
    }
}

__global__ void __launch_bounds__(kReduceThreads) k_sqrt_sum(const double* __restrict__ p, double* out)
{
    pdl_wait();
    __shared__ double sh[33];
    const double v = reduce_partials(p, sh);
    if (threadIdx.x == 0) *out = sqrt(v);
}

__global__ void __launch_bounds__(kReduceThreads) k_sum(const double* __restrict__ p, double* out)
{
    pdl_wait();
    __shared__ double sh[33];
    const double v = reduce_partials(p, sh);
    if (threadIdx.x == 0) *out = v;
}

__global__ void __launch_bounds__(kReduceThreads) k_cg_beta(const double* __restrict__ p, double* rz, double* beta)
{
    pdl_wait();
    __shared__ double sh[33];
    const double v = reduce_partials(p, sh);
    if (threadIdx.x == 0) {
        *beta = v / *rz;
        *rz = v;
    }
}

}  // namespace

// The scaled residual needs G >= bs (lane r applies row r of D^-1); inside a template the other
// shapes are discarded rather than instantiated.
template <int BS, int G>
void residual_dinv_shape(const BsrView<float>& A, unsigned grid, const float* dinv, long long dld, const float* x,
                         const float* b, float* w, cudaStream_t s)
{
    if constexpr (G >= BS) {
        if (A.unroll == 2)
            pdl_launch(k_bsr_residual_dinv<float, BS, G, 2>, grid, kThreads, 0, s, A.nbr, A.rowptr, A.colidx, A.vals,
                       A.ld, dinv, dld, x, b, w, A.ell);
        else
            pdl_launch(k_bsr_residual_dinv<float, BS, G, 1>, grid, kThreads, 0, s, A.nbr, A.rowptr, A.colidx, A.vals,
                       A.ld, dinv, dld, x, b, w, A.ell);
    }
}

template <int BS>
void residual_dinv_slot(const BsrView<float>& A, const float* dinv, long long dld, const float* x, const float* b,
                        float* w, cudaStream_t s)
{
    const unsigned grid = grid_for(A.nbr, kThreads);
    switch (A.ell) {
    case 5: pdl_launch(k_bsr_residual_dinv_slot<float, BS, 5>, grid, kThreads, 0, s, A.nbr, A.colidx, A.vals, A.ld,
                       dinv, dld, x, b, w); break;
    case 6: pdl_launch(k_bsr_residual_dinv_slot<float, BS, 6>, grid, kThreads, 0, s, A.nbr, A.colidx, A.vals, A.ld,
                       dinv, dld, x, b, w); break;
    case 7: pdl_launch(k_bsr_residual_dinv_slot<float, BS, 7>, grid, kThreads, 0, s, A.nbr, A.colidx, A.vals, A.ld,
                       dinv, dld, x, b, w); break;
    case 8: pdl_launch(k_bsr_residual_dinv_slot<float, BS, 8>, grid, kThreads, 0, s, A.nbr, A.colidx, A.vals, A.ld,
                       dinv, dld, x, b, w); break;
    default: break;
    }
}

void launch_residual_dinv(const BsrView<float>& A, const float* dinv, long long dld, const float* x, const float* b,
                          float* w, cudaStream_t s)
{
    if (A.nbr == 0) return;
    if (A.slot_major) {   // block sizes of the learned step (2..4)
        if (A.bs == 2) residual_dinv_slot<2>(A, dinv, dld, x, b, w, s);
        else if (A.bs == 3) residual_dinv_slot<3>(A, dinv, dld, x, b, w, s);
        else if (A.bs == 4) residual_dinv_slot<4>(A, dinv, dld, x, b, w, s);
        g_kernel_launches++;
        return;
    }
    FHG_DISPATCH_BS_G(A.bs, A.lanes, {
        const unsigned grid = grid_for((long long)A.nbr * G, kThreads);
        residual_dinv_shape<BS, G>(A, grid, dinv, dld, x, b, w, s);
    });
    g_kernel_launches++;
}

void launch_spmv_dots(const BsrView<double>& A, const double* d, const double* r, double* Ad, double* partials,
                      cudaStream_t s)
{
    FHG_DISPATCH_BS_G(A.bs, A.lanes, {
        pdl_launch(k_bsr_spmv_dots<BS, G>, kReduceCtas, kReduceThreads, 0, s, A.nbr, A.rowptr, A.colidx, A.vals, A.ld, d, r,
                                                                      Ad, partials);
    });
    g_kernel_launches++;
}

void launch_residual_comp(const BsrView<double>& A, const double* x, const double* b, double* r, double* partials,
                          cudaStream_t s, const int* enable)
{
    switch (A.bs) {
    case 2: pdl_launch(k_bsr_residual_comp<2>, kReduceCtas, kReduceThreads, 0, s, A.nbr, A.rowptr, A.colidx, A.vals,
                       A.ld, x, b, r, partials, enable); break;
    case 3: pdl_launch(k_bsr_residual_comp<3>, kReduceCtas, kReduceThreads, 0, s, A.nbr, A.rowptr, A.colidx, A.vals,
                       A.ld, x, b, r, partials, enable); break;
    case 4: pdl_launch(k_bsr_residual_comp<4>, kReduceCtas, kReduceThreads, 0, s, A.nbr, A.rowptr, A.colidx, A.vals,
                       A.ld, x, b, r, partials, enable); break;
    default: pdl_launch(k_bsr_residual_comp<6>, kReduceCtas, kReduceThreads, 0, s, A.nbr, A.rowptr, A.colidx, A.vals,
                        A.ld, x, b, r, partials, enable); break;
    }
    g_kernel_launches++;
}

void launch_dot(long long n, const double* a, const double* b, double* partials, cudaStream_t s)
{
    pdl_launch(k_dot, kReduceCtas, kReduceThreads, 0, s, n, a, b, partials);
    g_kernel_launches++;
}

template void launch_dots3<double>(long long, int, const double*, const double*, const double*, const double*,
                                   const double*, const double*, double*, cudaStream_t);
template void launch_dots3<float>(long long, int, const float*, const float*, const float*, const float*, const float*,
                                  const float*, double*, cudaStream_t);
template void launch_axpy<double>(long long, double, const double*, double*, cudaStream_t);
template void launch_axpy<float>(long long, double, const float*, float*, cudaStream_t);
template void launch_lincomb<double>(long long, double, const double*, double, const double*, double*, cudaStream_t);
template void launch_lincomb<float>(long long, double, const float*, double, const float*, float*, cudaStream_t);

void launch_fcg_direction(long long n, const double* z, const double* dp, const double* partials_zadp,
                          const double* dadp, double* d, cudaStream_t s)
{
    pdl_launch(k_fcg_direction, kReduceCtas, kReduceThreads, 0, s, n, z, dp, partials_zadp, dadp, d);
    g_kernel_launches++;
}

void launch_krylov_step(long long n, double* x, double* r, const double* d, const double* Ad,
                        const double* partials_num, const double* partials_den, double* den_out,
                        double* partials_rr, cudaStream_t s, float* r32)
{
    pdl_launch(k_krylov_step, kReduceCtas, kReduceThreads, 0, s, n, x, r, d, Ad, partials_num, partials_den, den_out,
                                                         partials_rr, r32);
    g_kernel_launches++;
}

void launch_dot_mixed(long long n, const float* a, const double* b, double* partials, cudaStream_t s)
{
    pdl_launch(k_dot_mixed, kReduceCtas, kReduceThreads, 0, s, n, a, b, partials);
    g_kernel_launches++;
}

void launch_fcg_direction_mixed(long long n, const float* z, const double* dp, const double* partials_zadp,
                                const double* dadp, double* d, cudaStream_t s, float* dhi, float* dlo)
{
    pdl_launch(k_fcg_direction_mixed, kReduceCtas, kReduceThreads, 0, s, n, z, dp, partials_zadp, dadp, d, dhi, dlo);
    g_kernel_launches++;
}

void launch_spmv_dots_df(const BsrView<float>& Ahi, const float* vlo, const float* dhi, const float* dlo,
                         const float* rhi, const float* rlo, float* Adhi, float* Adlo, double* partials,
                         cudaStream_t s)
{
    // lane r writes output r: needs G >= bs (always true for G >= 4 and bs <= 4; bs = 6 uses 8)
    const int lanes = Ahi.lanes < Ahi.bs ? 8 : Ahi.lanes;
    FHG_DISPATCH_BS_G(Ahi.bs, lanes, {
        pdl_launch(k_bsr_spmv_dots_df<BS, G>, kReduceCtas, kReduceThreads, 0, s, Ahi.nbr, Ahi.rowptr, Ahi.colidx, Ahi.vals, vlo,
                                                                         Ahi.ld, dhi, dlo, rhi, rlo, Adhi, Adlo,
                                                                         partials);
    });
    g_kernel_launches++;
}

void launch_spmv_dots_df_slot(const BsrView<dfl>& A, const float* dhi, const float* dlo, const float* rhi,
                              const float* rlo, float* Adhi, float* Adlo, double* partials, cudaStream_t s)
{
#define FHG_OUTER_SLOT(BSV, WV)                                                                              \
    if (A.bs == BSV && A.ell == WV) {                                                                       \
        pdl_launch(k_bsr_spmv_dots_df_slot<BSV, WV>, kReduceCtas, kReduceThreads, 0, s, A.nbr, A.colidx, A.vals, A.ld, \
                   dhi, dlo, rhi, rlo, Adhi, Adlo, partials);                                              \
        g_kernel_launches++;                                                                               \
        return;                                                                                            \
    }
#define FHG_OUTER_SLOT_W(BSV) FHG_OUTER_SLOT(BSV, 5) FHG_OUTER_SLOT(BSV, 6) FHG_OUTER_SLOT(BSV, 7) FHG_OUTER_SLOT(BSV, 8)
    FHG_OUTER_SLOT_W(2)
    FHG_OUTER_SLOT_W(3)
    FHG_OUTER_SLOT_W(4)
    FHG_OUTER_SLOT_W(6)
#undef FHG_OUTER_SLOT_W
#undef FHG_OUTER_SLOT
}

void launch_dot_df(long long n, const float* z, const float* ah, const float* al, double* partials, cudaStream_t s,
                   const dfl* z2)
{
    pdl_launch(k_dot_df, kReduceCtas, kReduceThreads, 0, s, n, z, z2, ah, al, partials);
    g_kernel_launches++;
}

void launch_fcg_direction_df(long long n, const float* z, const float* dph, const float* dpl,
                             const double* partials_zadp, const double* dadp, float* dh, float* dl, cudaStream_t s,
                             const dfl* z2)
{
    pdl_launch(k_fcg_direction_df, kReduceCtas, kReduceThreads, 0, s, n, z, z2, dph, dpl, partials_zadp, dadp, dh, dl);
    g_kernel_launches++;
}

void launch_krylov_step_df(long long n, double* x, float* rh, float* rl, const float* dh, const float* dl,
                           const float* Adh, const float* Adl, const double* partials_num,
                           const double* partials_den, double* den_out, double* partials_rr, cudaStream_t s,
                           dfl* r2)
{
    pdl_launch(k_krylov_step_df, kReduceCtas, kReduceThreads, 0, s, n, x, rh, rl, dh, dl, Adh, Adl, partials_num,
                                                            partials_den, den_out, partials_rr, r2);
    g_kernel_launches++;
}

void launch_split_df(long long n, const double* v, float* h, float* l, cudaStream_t s, dfl* v2)
{
    pdl_launch(k_split_df, grid_for(n, kThreads), kThreads, 0, s, n, v, h, l, v2);
    g_kernel_launches++;
}


void launch_cg_step(long long n, double* x, double* r, const double* d, const double* Ad, const double* num,
                    const double* partials_den, double* partials_rr, cudaStream_t s)
{
    pdl_launch(k_cg_step, kReduceCtas, kReduceThreads, 0, s, n, x, r, d, Ad, num, partials_den, partials_rr);
    g_kernel_launches++;
}

void launch_cg_direction(long long n, const double* z, const double* beta, double* d, cudaStream_t s)
{
    pdl_launch(k_cg_direction, kReduceCtas, kReduceThreads, 0, s, n, z, beta, d);
    g_kernel_launches++;
}

void launch_cg_beta(const double* partials, double* rz, double* beta, cudaStream_t s)
{
    pdl_launch(k_cg_beta, 1, kReduceThreads, 0, s, partials, rz, beta);
    g_kernel_launches++;
}

void launch_finalize_norm(const double* partials_rr, const double* bnorm, double* nr_out, double* hist, int* counter,
                          int hist_len, cudaStream_t s)
{
    pdl_launch(k_finalize_norm, 1, kReduceThreads, 0, s, partials_rr, bnorm, nr_out, hist, counter, hist_len);
    g_kernel_launches++;
}

void launch_sqrt_sum(const double* partials, double* out, cudaStream_t s)
{
    pdl_launch(k_sqrt_sum, 1, kReduceThreads, 0, s, partials, out);
    g_kernel_launches++;
}

void launch_sum(const double* partials, double* out, cudaStream_t s)
{
    pdl_launch(k_sum, 1, kReduceThreads, 0, s, partials, out);
    g_kernel_launches++;
}

template void launch_spmv<double>(const BsrView<double>&, int, const double*, const double*, double*, cudaStream_t);
template void launch_convert<double, dfl>(long long, const double*, dfl*, cudaStream_t);
template void launch_spmv<float>(const BsrView<float>&, int, const float*, const float*, float*, cudaStream_t);
template void launch_gs<double>(const BsrView<double>&, int, int, const double*, long long, const double*, double*,
                                cudaStream_t, int, int, double);
template void launch_gs<float>(const BsrView<float>&, int, int, const float*, long long, const float*, float*,
                               cudaStream_t, int, int, float);
template void launch_jacobi<double>(const BsrView<double>&, const double*, long long, double, const double*,
                                    const double*, double*, cudaStream_t);
template void launch_jacobi<float>(const BsrView<float>&, const float*, long long, float, const float*, const float*,
                                   float*, cudaStream_t);
template void launch_coarse<double>(int, const double*, const double*, double*, cudaStream_t);
template void launch_coarse<float>(int, const double*, const float*, float*, cudaStream_t);
template void launch_convert<double, float>(long long, const double*, float*, cudaStream_t);
template void launch_convert<float, double>(long long, const float*, double*, cudaStream_t);
template void launch_permute<double>(int, int, const int*, const double*, double*, bool, cudaStream_t);
template void launch_permute<float>(int, int, const int*, const float*, float*, bool, cudaStream_t);
template void launch_inject<double>(int, int, int, const int*, const double*, const double*, double*, bool, cudaStream_t);
template void launch_inject<float>(int, int, int, const int*, const float*, const float*, float*, bool, cudaStream_t);


// ---------------------------------------------------------------------------
// Device-side solve loop (batched solve): the stopping test runs on the device and drives the
// WHILE node of the graph.

namespace {

__global__ void k_copy2(long long n, const double* __restrict__ a0, double* __restrict__ b0,
                        const double* __restrict__ a1, double* __restrict__ b1)
{
    pdl_wait();
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        b0[i] = a0[i];
        b1[i] = a1[i];
    }
}

__global__ void k_init_solve(double* scal, int* counter, int* state, int replacements)
{
    pdl_wait();
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        scal[1] = 1.0;  // d.Ad of the (absent) previous direction
        scal[2] = 1.0;  // ||r|| / ||b||
        scal[3] = 0.0;
        scal[4] = 0.0;
        *counter = 1;
        if (state) {
            state[kLoopReplaceLeft] = replacements;
            state[kLoopGo] = 1;
            state[kLoopNeedComp] = 0;
        }
    }
}

// After an iteration of the device loop (IterativeSolver's stopping test, IterativeSolver.h:224-247):
// go on while iterations < maxit and ||r||/||b|| >= tol, finite; once the recursive residual meets
// tol and replacements are left, set the IF node's condition so that the true residual is checked
// (k_check_* decide then whether to stop or to replace r and go on).
__global__ void k_loop_decide(const double* nr, const int* counter, double tol, int maxit, int* state,
                              cudaGraphConditionalHandle check)
{
    pdl_wait();
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double v = *nr;
        const int it = *counter - 1;
        int go = 0, chk = 0;
        if (isfinite(v) && it < maxit) {
            if (!(v < tol)) go = 1;
            else if (state[kLoopReplaceLeft] > 0) chk = 1;
        }
        state[kLoopGo] = go;
        state[kLoopNeedComp] = 0;
        cudaGraphSetConditional(check, chk ? 1u : 0u);
    }
}

// True residual from the FP64 evaluation (partials of r.r): it meets tol (stop), or it is evaluated
// again in compensated arithmetic (state[kLoopNeedComp] = 1). scal[5] receives ||b - A x||.
__global__ void __launch_bounds__(kReduceThreads) k_check_fp64(const double* __restrict__ p, double* scal, double tol,
                                                               int* state)
{
    pdl_wait();
    __shared__ double sh[33];
    const double rn = sqrt(reduce_partials(p, sh));
    if (threadIdx.x == 0) {
        scal[5] = rn;
        const double bn = scal[0];
        const double tr = bn > 0.0 ? rn / bn : rn;
        state[kLoopGo] = 0;
        state[kLoopNeedComp] = (tr < tol) ? 0 : 1;
    }
}

// After the compensated evaluation (when it ran): stop if the true residual meets tol, else replace
// r (k_replace_apply) and go on while replacements are left. replace = 0: the epilogue's check only.
__global__ void __launch_bounds__(kReduceThreads) k_check_comp(const double* __restrict__ p, double* scal, double tol,
                                                               int* state, int replace)
{
    pdl_wait();
    if (state[kLoopNeedComp] == 0) return;
    __shared__ double sh[33];
    const double rn = sqrt(reduce_partials(p, sh));
    if (threadIdx.x == 0) {
        scal[5] = rn;
        const double bn = scal[0];
        const double tr = bn > 0.0 ? rn / bn : rn;
        if (replace && !(tr < tol) && isfinite(tr) && state[kLoopReplaceLeft] > 0) {
            state[kLoopReplaceLeft]--;
            state[kLoopGo] = 1;
            scal[2] = tr;
        } else {
            state[kLoopGo] = 0;
        }
    }
}

// Residual replacement when state[kLoopGo]: r = t (the true residual) and the V-cycle's right-hand
// side from it (FP32 pair (rh, rl) and optionally interleaved pairs r2, or FP32 b32).
__global__ void __launch_bounds__(kReduceThreads) k_replace_apply(long long n, const int* __restrict__ state,
                                                                  const double* __restrict__ t, double* __restrict__ r,
                                                                  float* __restrict__ rh, float* __restrict__ rl,
                                                                  dfl* __restrict__ r2, float* __restrict__ b32)
{
    pdl_wait();
    if (state[kLoopGo] == 0) return;
    for (long long i = (long long)blockIdx.x * kReduceThreads + threadIdx.x; i < n; i += kRedStride) {
        const double v = t[i];
        r[i] = v;
        if (rh) {
            float h, l;
            df_split(v, h, l);
            rh[i] = h;
            rl[i] = l;
            if (r2) r2[i] = dfl(h, l);
        } else if (b32) {
            b32[i] = (float)v;
        }
    }
}

__global__ void k_loop_finish(const int* state, cudaGraphConditionalHandle loop)
{
    pdl_wait();
    if (threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(loop, state[kLoopGo] ? 1u : 0u);
}

}  // namespace

void launch_copy2(long long n, const double* a0, double* b0, const double* a1, double* b1, cudaStream_t s)
{
    const long long blocks = std::min<long long>((n + 255) / 256, 4 * 152);
    pdl_launch(k_copy2, (unsigned)std::max<long long>(blocks, 1), 256, 0, s, n, a0, b0, a1, b1);
    g_kernel_launches++;
}

void launch_init_solve(double* scal, int* counter, cudaStream_t s, int* state, int replacements)
{
    pdl_launch(k_init_solve, 1, 32, 0, s, scal, counter, state, replacements);
    g_kernel_launches++;
}

void launch_loop_decide(const double* nr, const int* counter, double tol, int maxit, int* state,
                        cudaGraphConditionalHandle check, cudaStream_t s)
{
    pdl_launch(k_loop_decide, 1, 32, 0, s, nr, counter, tol, maxit, state, check);
    g_kernel_launches++;
}

void launch_check_fp64(const double* partials, double* scal, double tol, int* state, cudaStream_t s)
{
    pdl_launch(k_check_fp64, 1, kReduceThreads, 0, s, partials, scal, tol, state);
    g_kernel_launches++;
}

void launch_check_comp(const double* partials, double* scal, double tol, int* state, int replace, cudaStream_t s)
{
    pdl_launch(k_check_comp, 1, kReduceThreads, 0, s, partials, scal, tol, state, replace);
    g_kernel_launches++;
}

void launch_replace_apply(long long n, const int* state, const double* t, double* r, float* rh, float* rl, dfl* r2,
                          float* b32, cudaStream_t s)
{
    pdl_launch(k_replace_apply, kReduceCtas, kReduceThreads, 0, s, n, state, t, r, rh, rl, r2, b32);
    g_kernel_launches++;
}

// Launched without programmatic serialization: it follows a conditional node, not a kernel.
void launch_loop_finish(const int* state, cudaGraphConditionalHandle loop, cudaStream_t s)
{
    k_loop_finish<<<1, 32, 0, s>>>(state, loop);
    g_kernel_launches++;
}

}  // namespace fhg
