// Learned correction step of the FP32 V-cycle: a per-face-patch MLP, its BF16 tensor-core
// inference and training kernels (FP32 accumulation), and the energy-norm loss.
//
// The network sees, for every face block i of the finest level, the block-Jacobi-scaled
// residual w = D^-1 (b - A x) on the face and on its (up to) six neighbours in the operator,
// ordered by decreasing coupling strength |A_ij|_F, plus the diffusion tensors of the face's
// two elements:
//
//   input  u_i (48)  = [ w_i / s_i, w_j1 / s_i, ..., w_j6 / s_i  (7 bs, zero padded to 32),
//                        T_1 / tau_i, T_2 / tau_i  (2 x 6: xx yy zz xy xz yz), 0 0 0 0 ]
//   s_i             = sqrt(mean of the squares of the 7 bs residual slots)
//   h1 = gelu(W1 u + b1)    (128)
//   h2 = gelu(W2 h1 + b2)   (128)
//   y  = W3 h2 + b3         (16, entries >= bs unused)
//   x_i += s_i y_i[0..bs)
//
// so the correction is positively homogeneous in the residual (a residual scaled by a > 0
// gets a correction scaled by a), which keeps it meaningful across the twelve orders of
// magnitude of a solve. gelu is the tanh form of Hendrycks & Gimpel (2016),
// 0.5 a (1 + tanh(sqrt(2/pi) (a + 0.044715 a^3))), evaluated in packed BF16 arithmetic with the
// hardware bf16x2 tanh (its result is the BF16 operand of the next layer); the backward pass uses
// the FP32 derivative of the same formula.
//
// Tensor cores: mma.sync.m16n8k16 BF16 x BF16 -> FP32 with ldmatrix fragment loads. The
// inference kernel keeps a 16-face tile in registers through all three layers (the FP32
// accumulator fragment of one layer is exactly the BF16 A fragment of the next), with the
// weights staged once per CTA in shared memory; the training kernels are tiled GEMMs.
#include "fhg_internal.h"

#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

namespace fhg {
namespace {

using bf16 = __nv_bfloat16;
using namespace learned;

// ---------------------------------------------------------------------------
// Fragment helpers (m16n8k16, row.col, BF16 in, FP32 accumulate)

__device__ __forceinline__ unsigned smem_u32(const void* p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const bf16* p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], const bf16* p)
{
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(smem_u32(p)));
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};\n"
                 : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ float tanh_fast(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

constexpr float kGeluC0 = 0.7978845608028654f;  // sqrt(2/pi)
constexpr float kGeluC1 = 0.044715f;

// tanh(x (c0 + c0 c1 x^2)) of two BF16 values in packed BF16 arithmetic: x^2, one FMA with the
// BF16-rounded constants c0 c1 and c0, one multiply, then the bf16x2 hardware tanh (one
// multi-function op per two values).
__device__ __forceinline__ __nv_bfloat162 gelu_tanh_bf16x2(__nv_bfloat162 x)
{
    const __nv_bfloat162 c0 = __float2bfloat162_rn(kGeluC0);
    const __nv_bfloat162 c01 = __float2bfloat162_rn(kGeluC0 * kGeluC1);
    const __nv_bfloat162 q = __hfma2(__hmul2(x, x), c01, c0);
    const __nv_bfloat162 u = __hmul2(x, q);
    uint32_t ui = *reinterpret_cast<const uint32_t*>(&u), ti;
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(ti) : "r"(ui));
    return *reinterpret_cast<const __nv_bfloat162*>(&ti);
}

// gelu of two values in packed BF16 arithmetic, the activation the network uses: the inputs are
// rounded to BF16, t = gelu_tanh_bf16x2(x), h = x / 2 (exact), gelu = h t + h in one bf16x2 FMA.
// Returns the packed result (the next layer's BF16 operand).
__device__ __forceinline__ uint32_t gelu_bf16x2(float a0, float a1)
{
    const __nv_bfloat162 x = __floats2bfloat162_rn(a0, a1);
    const __nv_bfloat162 t = gelu_tanh_bf16x2(x);
    const __nv_bfloat162 h = __hmul2(x, __float2bfloat162_rn(0.5f));
    const __nv_bfloat162 g = __hfma2(h, t, h);
    return *reinterpret_cast<const uint32_t*>(&g);
}

// 2 gelu of two values, x t + x in one bf16x2 FMA: bit for bit twice gelu_bf16x2 (scaling by 2
// commutes with round-to-nearest away from the subnormal range), one multiply fewer. A layer fed
// with it uses weights scaled by 1/2, again exactly, so its accumulators are unchanged.
__device__ __forceinline__ uint32_t gelu2_bf16x2(float a0, float a1)
{
    const __nv_bfloat162 x = __floats2bfloat162_rn(a0, a1);
    const __nv_bfloat162 g = __hfma2(x, gelu_tanh_bf16x2(x), x);
    return *reinterpret_cast<const uint32_t*>(&g);
}

__device__ __forceinline__ float gelu_grad(float a)
{
    const float a2 = a * a;
    const float t = tanh_fast(kGeluC0 * fmaf(kGeluC1 * a, a2, a));
    return 0.5f * (1.0f + t) + 0.5f * a * (1.0f - t * t) * kGeluC0 * fmaf(3.0f * kGeluC1, a2, 1.0f);
}

// ---------------------------------------------------------------------------
// Input features of one face (shared by inference and training so that both see the same
// bits). Writes the 32 residual slots of the input row as BF16 and returns s_i.

template <int BS>
__device__ __forceinline__ float face_inputs(int f, const int* __restrict__ nbr, const float* __restrict__ w,
                                             bf16* row)
{
    static_assert(7 * BS <= kResidualSlots, "7 bs residual slots must fit");
    float v[7 * BS];
#pragma unroll
    for (int c = 0; c < BS; c++) v[c] = w[(long long)f * BS + c];
#pragma unroll
    for (int j = 0; j < kNeighbours; j++) {
        const int g = nbr[(long long)f * kNeighbours + j];
#pragma unroll
        for (int c = 0; c < BS; c++) v[(j + 1) * BS + c] = g >= 0 ? w[(long long)g * BS + c] : 0.0f;
    }
    float ss = 0.0f;
#pragma unroll
    for (int q = 0; q < 7 * BS; q++) ss = fmaf(v[q], v[q], ss);
    const float s = sqrtf(ss * (1.0f / (7 * BS)));
    const float inv = s > 0.0f ? 1.0f / s : 0.0f;
    uint32_t packed[kResidualSlots / 2];
#pragma unroll
    for (int q = 0; q < kResidualSlots / 2; q++) {
        const float lo = 2 * q < 7 * BS ? v[2 * q] * inv : 0.0f;
        const float hi = 2 * q + 1 < 7 * BS ? v[2 * q + 1] * inv : 0.0f;
        packed[q] = pack_bf16(lo, hi);
    }
    uint4* dst = reinterpret_cast<uint4*>(row);
#pragma unroll
    for (int q = 0; q < kResidualSlots / 8; q++)
        dst[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
    return s;
}

// Features of every face (training path): feat[f] = input row (48 BF16), scale[f] = s_f.
// Rows in [nb, rows) are zero (padding of the GEMM tiles).
template <int BS>
__global__ void __launch_bounds__(256) k_features(int nb, int rows, const int* __restrict__ nbr,
                                                  const float* __restrict__ w, const bf16* __restrict__ tfeat,
                                                  bf16* __restrict__ feat, float* __restrict__ scale)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= rows) return;
    bf16* row = feat + (long long)f * kIn;
    uint4* dst = reinterpret_cast<uint4*>(row);
    if (f >= nb) {
#pragma unroll
        for (int q = 0; q < kIn / 8; q++) dst[q] = make_uint4(0, 0, 0, 0);
        scale[f] = 0.0f;
        return;
    }
    scale[f] = face_inputs<BS>(f, nbr, w, row);
    const uint4* src = reinterpret_cast<const uint4*>(tfeat + (long long)f * kTensorSlots);
    dst[kResidualSlots / 8] = src[0];
    dst[kResidualSlots / 8 + 1] = src[1];
}

// ---------------------------------------------------------------------------
// Fused inference: x_i += s_i y_i for every face, one warp per 16-face tile.

constexpr int kApplyWarps = 8;
constexpr int kLd1 = kIn + 8;    // padded shared-memory row of W1 and of the input tile (BF16)
constexpr int kLd2 = kHid + 8;   // padded row of W2 and W3
constexpr size_t kApplySmem =
    sizeof(bf16) * ((size_t)kHid * kLd1 + (size_t)kHid * kLd2 + (size_t)kOut * kLd2 + (size_t)kApplyWarps * 16 * kLd1) +
    sizeof(float) * (kHid + kHid + kOut);

template <int BS>
__global__ void __launch_bounds__(kApplyWarps * 32, 2)
    k_learned_apply(int nb, const int* __restrict__ nbr, const float* __restrict__ w, const bf16* __restrict__ tfeat,
                    const bf16* __restrict__ wts, const float* __restrict__ bias, float* __restrict__ x)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    bf16* sW1 = reinterpret_cast<bf16*>(smem_raw);
    bf16* sW2 = sW1 + kHid * kLd1;
    bf16* sW3 = sW2 + kHid * kLd2;
    bf16* sX = sW3 + kOut * kLd2;
    float* sB = reinterpret_cast<float*>(sX + kApplyWarps * 16 * kLd1);
    // Stage the weights (global layout: W1 [128][48], W2 [128][128], W3 [16][128], row-major).
    const bf16* gW1 = wts;
    const bf16* gW2 = gW1 + kHid * kIn;
    const bf16* gW3 = gW2 + kHid * kHid;
    for (int v = threadIdx.x; v < kHid * kIn / 8; v += blockDim.x) {
        const int r = v / (kIn / 8), c = (v % (kIn / 8)) * 8;
        *reinterpret_cast<uint4*>(sW1 + r * kLd1 + c) = *reinterpret_cast<const uint4*>(gW1 + r * kIn + c);
    }
    for (int v = threadIdx.x; v < kHid * kHid / 8; v += blockDim.x) {
        const int r = v / (kHid / 8), c = (v % (kHid / 8)) * 8;
        *reinterpret_cast<uint4*>(sW2 + r * kLd2 + c) = *reinterpret_cast<const uint4*>(gW2 + r * kHid + c);
    }
    for (int v = threadIdx.x; v < kOut * kHid / 8; v += blockDim.x) {
        const int r = v / (kHid / 8), c = (v % (kHid / 8)) * 8;
        *reinterpret_cast<uint4*>(sW3 + r * kLd2 + c) = *reinterpret_cast<const uint4*>(gW3 + r * kHid + c);
    }
    for (int v = threadIdx.x; v < 2 * kHid + kOut; v += blockDim.x) sB[v] = bias[v];
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = lane >> 2, t = lane & 3, q = lane >> 3, r8 = lane & 7;
    bf16* tile = sX + warp * 16 * kLd1;
    const int ntiles = (nb + 15) / 16;
    for (int tI = blockIdx.x * kApplyWarps + warp; tI < ntiles; tI += gridDim.x * kApplyWarps) {
        const int f0 = tI * 16;
        // Gather: lanes 0-15 build the residual slots of face f0+lane, lanes 16-31 copy its tensors.
        float s = 0.0f;
        {
            const int row = lane & 15;
            const int f = f0 + row;
            bf16* dst = tile + row * kLd1;
            if (lane < 16) {
                if (f < nb) {
                    s = face_inputs<BS>(f, nbr, w, dst);
                } else {
#pragma unroll
                    for (int c = 0; c < kResidualSlots / 8; c++) reinterpret_cast<uint4*>(dst)[c] = make_uint4(0, 0, 0, 0);
                }
            } else {
                uint4 a = make_uint4(0, 0, 0, 0), b = a;
                if (f < nb) {
                    const uint4* src = reinterpret_cast<const uint4*>(tfeat + (long long)f * kTensorSlots);
                    a = src[0];
                    b = src[1];
                }
                reinterpret_cast<uint4*>(dst + kResidualSlots)[0] = a;
                reinterpret_cast<uint4*>(dst + kResidualSlots)[1] = b;
            }
        }
        __syncwarp();
        const float s_lo = __shfl_sync(0xffffffffu, s, g);
        const float s_hi = __shfl_sync(0xffffffffu, s, g + 8);

        float acc[kHid / 8][4];
#pragma unroll
        for (int j = 0; j < kHid / 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
        // Layer 1: [16 x 48] x W1^T
#pragma unroll
        for (int ks = 0; ks < kIn / 16; ks++) {
            uint32_t a[4];
            ldsm_x4(a, tile + (r8 + (q & 1) * 8) * kLd1 + ks * 16 + (q >> 1) * 8);
#pragma unroll
            for (int j = 0; j < kHid / 8; j += 2) {
                uint32_t b[4];
                ldsm_x4(b, sW1 + (8 * j + r8 + (q >> 1) * 8) * kLd1 + ks * 16 + (q & 1) * 8);
                mma16816(acc[j], a, b[0], b[1]);
                mma16816(acc[j + 1], a, b[2], b[3]);
            }
        }
        uint32_t h[kHid / 16][4];
#pragma unroll
        for (int kk = 0; kk < kHid / 16; kk++) {
#pragma unroll
            for (int half = 0; half < 2; half++) {
                const int j = 2 * kk + half;
                const float b0 = sB[8 * j + 2 * t], b1 = sB[8 * j + 2 * t + 1];
                h[kk][2 * half] = gelu_bf16x2(acc[j][0] + b0, acc[j][1] + b1);
                h[kk][2 * half + 1] = gelu_bf16x2(acc[j][2] + b0, acc[j][3] + b1);
            }
        }
        // Layer 2: [16 x 128] x W2^T
#pragma unroll
        for (int j = 0; j < kHid / 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
        for (int kk = 0; kk < kHid / 16; kk++) {
#pragma unroll
            for (int j = 0; j < kHid / 8; j += 2) {
                uint32_t b[4];
                ldsm_x4(b, sW2 + (8 * j + r8 + (q >> 1) * 8) * kLd2 + kk * 16 + (q & 1) * 8);
                mma16816(acc[j], h[kk], b[0], b[1]);
                mma16816(acc[j + 1], h[kk], b[2], b[3]);
            }
        }
#pragma unroll
        for (int kk = 0; kk < kHid / 16; kk++) {
#pragma unroll
            for (int half = 0; half < 2; half++) {
                const int j = 2 * kk + half;
                const float b0 = sB[kHid + 8 * j + 2 * t], b1 = sB[kHid + 8 * j + 2 * t + 1];
                h[kk][2 * half] = gelu_bf16x2(acc[j][0] + b0, acc[j][1] + b1);
                h[kk][2 * half + 1] = gelu_bf16x2(acc[j][2] + b0, acc[j][3] + b1);
            }
        }
        // Layer 3: [16 x 128] x W3^T -> 16 outputs
        float y[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
        for (int kk = 0; kk < kHid / 16; kk++) {
            uint32_t b[4];
            ldsm_x4(b, sW3 + (r8 + (q >> 1) * 8) * kLd2 + kk * 16 + (q & 1) * 8);
            mma16816(y[0], h[kk], b[0], b[1]);
            mma16816(y[1], h[kk], b[2], b[3]);
        }
#pragma unroll
        for (int j = 0; j < 2; j++) {
#pragma unroll
            for (int e = 0; e < 2; e++) {
                const int col = 8 * j + 2 * t + e;
                if (col < BS) {
                    const float bo = sB[2 * kHid + col];
                    const int fa = f0 + g, fb = f0 + g + 8;
                    const float ca = s_lo * (y[j][e] + bo), cb = s_hi * (y[j][2 + e] + bo);
                    // A non-finite network output adds nothing (the step is then the plain cycle's).
                    if (fa < nb && isfinite(ca)) x[(long long)fa * BS + col] += ca;
                    if (fb < nb && isfinite(cb)) x[(long long)fb * BS + col] += cb;
                }
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Fused inference on the 5th-generation tensor cores: one persistent CTA per SM with four
// independent tile pipelines, one per warpgroup (slot), each on its own tiles of 128 faces. In a
// slot, thread t gathers the residual patch and the tensor features of face t (the next tile's are
// loaded while the current tile's layers run), one thread issues tcgen05.mma (BF16 x BF16 -> FP32,
// M = 128 faces, N = 128 or 16, K = 16 per instruction) with the accumulator in the slot's 128 TMEM
// columns (TMEM lane t = face t), and the warpgroup reads it back with tcgen05.ld, applies gelu
// and writes the BF16 A operand of the next layer. The biases of the hidden layers ride in the
// MMAs: b1 as three BF16 parts (hi + mid + lo = the FP32 bias) in the input columns 44..46 of W1,
// which face constant-1 inputs (those tensor-feature slots are zero in the network's input), and
// b2 the same way in an extra K = 16 chunk of layer 2 against a constant tile of ones. The
// epilogue writes 2 gelu (gelu2_bf16x2) and W2, W3 are staged halved, both exact, so the
// epilogue is one conversion, four bf16x2 ops and a tanh per two values. The slots share the weights in
// shared memory and synchronise only within the warpgroup (named barriers, one mbarrier each), so
// the MMA waits, gathers and epilogues of four tiles overlap on every SM. Operands live in shared
// memory in the canonical K-major layout without swizzle: 8-row x 16-byte core matrices, element
// (row r, k) at byte
//   (r / 8) * SBO + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2,
// i.e. LBO = 128 bytes between core matrices along K and SBO = (K / 8) * 128 bytes between 8-row
// groups; a slot's input tile (K = 48) occupies the first bytes of its hidden tile (K = 128), which
// is written only after the layer-1 MMA has read the inputs. Every wait on an MMA-completion
// mbarrier is bounded (about a second of SM clocks): on expiry the slot records the failure and
// stops, and the CTA frees its TMEM and returns.

constexpr int kTcSlots = 4;
constexpr int kTcRows = 128;                       // faces per tile (TMEM lanes)
constexpr int kTcThreads = kTcRows * kTcSlots;     // one warpgroup per slot
constexpr uint32_t kTmemCols = 128 * kTcSlots;     // per slot: layer accumulators (the output reuses 16)
constexpr int kTcSW1 = 0;                          // W1: 128 x 48
constexpr int kTcSW2 = kTcSW1 + kHid * kIn * 2;    // W2: 128 x 128
constexpr int kTcSW3 = kTcSW2 + kHid * kHid * 2;   // W3: 16 x 128
constexpr int kTcSBias = kTcSW3 + kOut * kHid * 2; // b1, b2, b3 (FP32; the output layer reads b3)
constexpr int kTcSOnes = ((kTcSBias + (2 * kHid + kOut) * 4 + 1023) / 1024) * 1024;  // 128 x 16: ones in K 0..2
constexpr int kTcSB2 = kTcSOnes + kTcRows * 16 * 2;  // 128 x 16: b2 as hi, mid, lo BF16 in K 0..2
constexpr int kTcSlot0 = kTcSB2 + kHid * 16 * 2;
constexpr int kTcSlotBytes = kTcRows * kHid * 2;   // hidden tile (the input tile aliases its start)
constexpr int kTcSScale = kTcSlot0 + kTcSlots * kTcSlotBytes;  // s of every slot's faces
constexpr int kTcSMisc = kTcSScale + kTcSlots * kTcRows * 4;   // mbarriers (8 each), TMEM base (4)
constexpr size_t kTcSmem = kTcSMisc + 8 * kTcSlots + 16 + 1024;  // + alignment slack for a 1024-byte base
constexpr long long kTcWaitCycles = 2000000000LL;
static_assert(kTcSmem <= 232448, "one CTA per SM must fit in shared memory");

__device__ __forceinline__ uint32_t core_off(int row, int kchunk, int sbo)
{
    return (uint32_t)((row >> 3) * sbo + kchunk * 128 + (row & 7) * 16);
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N.
__host__ __device__ constexpr uint32_t mma_idesc(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                 :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" :: "r"(mbar)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// Bounded wait for the mbarrier phase with parity `parity`; false on expiry.
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity)
{
    const long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                     "selp.u32 %0, 1, 0, p;\n\t}\n"
                     : "=r"(done) : "r"(mbar), "r"(parity) : "memory");
        if (done) return true;
        if (clock64() - t0 > kTcWaitCycles) return false;
    }
}

// 32 consecutive FP32 accumulator columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                   "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                   "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                 "[%16];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                   "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// 2 gelu of the 128 accumulator columns (bias included) of this thread's lane into its row of the
// hidden tile.
__device__ __forceinline__ void tc_hidden_epilogue(uint32_t taddr, unsigned char* sH, int row)
{
#pragma unroll 1
    for (int q = 0; q < kHid / 32; q++) {
        float v[32];
        tmem_ld32(taddr + q * 32, v);
#pragma unroll
        for (int c = 0; c < 4; c++) {
            uint32_t w[4];
#pragma unroll
            for (int e = 0; e < 4; e++) w[e] = gelu2_bf16x2(v[c * 8 + 2 * e], v[c * 8 + 2 * e + 1]);
            *reinterpret_cast<uint4*>(sH + core_off(row, q * 4 + c, kHid * 16)) = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}

// Eight BF16 weights scaled by 1/2 (exact).
__device__ __forceinline__ uint4 halve_bf16x8(uint4 v)
{
    const __nv_bfloat162 h = __float2bfloat162_rn(0.5f);
    uint32_t* w = reinterpret_cast<uint32_t*>(&v);
#pragma unroll
    for (int i = 0; i < 4; i++) {
        __nv_bfloat162 x = *reinterpret_cast<__nv_bfloat162*>(&w[i]);
        x = __hmul2(x, h);
        w[i] = *reinterpret_cast<uint32_t*>(&x);
    }
    return v;
}

// An FP32 bias as three BF16 parts hi + mid + lo (each remainder is exact in FP32), packed as
// {hi, mid} and {lo, 0}.
__device__ __forceinline__ uint2 bias_parts(float b)
{
    const float hi = __bfloat162float(__float2bfloat16_rn(b));
    const float r1 = b - hi;
    const float mid = __bfloat162float(__float2bfloat16_rn(r1));
    const float lo = r1 - mid;
    return make_uint2(pack_bf16(hi, mid), pack_bf16(lo, 0.0f));
}

// Named barrier of one slot's 128 threads.
__device__ __forceinline__ void slot_sync(int slot)
{
    asm volatile("bar.sync %0, %1;\n" :: "r"(1 + slot), "r"(kTcRows) : "memory");
}

// Named barrier returning the AND of `pred` over the slot's threads.
__device__ __forceinline__ bool slot_and(int slot, bool pred)
{
    uint32_t r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
                 "bar.red.and.pred q, %2, %3, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
                 : "=r"(r) : "r"(pred ? 1u : 0u), "r"(1 + slot), "r"(kTcRows) : "memory");
    return r != 0;
}

// Neighbour blocks of face f (-1 where none; all -1 past the last face).
__device__ __forceinline__ void load_neighbours(int f, int nb, const int* __restrict__ nbr, int (&g)[kNeighbours])
{
#pragma unroll
    for (int j = 0; j < kNeighbours; j++) g[j] = f < nb ? nbr[(long long)f * kNeighbours + j] : -1;
}

// Residual patch of face f from its neighbour list: own block then the six neighbours (zero where
// none or past the last face).
template <int BS>
__device__ __forceinline__ void load_patch(int f, int nb, const int (&g)[kNeighbours], const float* __restrict__ w,
                                           float (&v)[7 * BS])
{
#pragma unroll
    for (int c = 0; c < BS; c++) v[c] = f < nb ? w[(long long)f * BS + c] : 0.0f;
#pragma unroll
    for (int j = 0; j < kNeighbours; j++)
#pragma unroll
        for (int c = 0; c < BS; c++) v[(j + 1) * BS + c] = g[j] >= 0 ? w[(long long)g[j] * BS + c] : 0.0f;
}

// Scaled BF16 residual slots of a patch into a row of the canonical input tile; returns s.
template <int BS>
__device__ __forceinline__ float store_patch(const float (&v)[7 * BS], unsigned char* sA, int row)
{
    float ss = 0.0f;
#pragma unroll
    for (int q = 0; q < 7 * BS; q++) ss = fmaf(v[q], v[q], ss);
    const float s = sqrtf(ss * (1.0f / (7 * BS)));
    const float inv = s > 0.0f ? 1.0f / s : 0.0f;
#pragma unroll
    for (int c = 0; c < kResidualSlots / 8; c++) {
        uint32_t p4[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int q = c * 8 + 2 * e;
            p4[e] = pack_bf16(q < 7 * BS ? v[q] * inv : 0.0f, q + 1 < 7 * BS ? v[q + 1] * inv : 0.0f);
        }
        *reinterpret_cast<uint4*>(sA + core_off(row, c, kIn * 16)) = make_uint4(p4[0], p4[1], p4[2], p4[3]);
    }
    return s;
}

template <int BS>
__global__ void __launch_bounds__(kTcThreads, 1)
    k_learned_apply_tc(int nb, const int* __restrict__ nbr, const float* __restrict__ w, const bf16* __restrict__ tfeat,
                       const bf16* __restrict__ wts, const float* __restrict__ bias, float* __restrict__ x,
                       int* __restrict__ status)
{
    extern __shared__ unsigned char smem_dyn[];
    unsigned char* sm = reinterpret_cast<unsigned char*>(((uintptr_t)smem_dyn + 1023) & ~(uintptr_t)1023);
    float* sBias = reinterpret_cast<float*>(sm + kTcSBias);
    uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(sm + kTcSMisc + 8 * kTcSlots);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int slot = tid / kTcRows;           // warpgroup = tile pipeline
    const int row = tid % kTcRows;            // face of the tile / TMEM lane
    const uint32_t s_base = smem_u32(sm);
    const uint32_t mbar = smem_u32(sm + kTcSMisc + 8 * slot);
    unsigned char* sSlot = sm + kTcSlot0 + slot * kTcSlotBytes;
    const uint32_t sSlot_a = s_base + kTcSlot0 + slot * kTcSlotBytes;
    float* sScale = reinterpret_cast<float*>(sm + kTcSScale) + slot * kTcRows;

    // Weights into the canonical layout, biases, barriers, TMEM (whole CTA).
    const bf16* gW1 = wts;
    const bf16* gW2 = gW1 + kHid * kIn;
    const bf16* gW3 = gW2 + kHid * kHid;
    static_assert(kIn == 48 && kResidualSlots + kTensorSlots == kIn, "bias columns 44..46 of W1");
    for (int v = tid; v < kHid * kIn / 8; v += kTcThreads) {
        const int r = v / (kIn / 8), c = v % (kIn / 8);
        uint4 w8 = *reinterpret_cast<const uint4*>(gW1 + r * kIn + 8 * c);
        if (c == kIn / 8 - 1) {   // columns 40..47: 44..46 carry b1 (their inputs are 1), 47 is 0
            const uint2 bp = bias_parts(bias[r]);
            w8.z = bp.x;
            w8.w = bp.y;
        }
        *reinterpret_cast<uint4*>(sm + kTcSW1 + core_off(r, c, kIn * 16)) = w8;
    }
    for (int v = tid; v < kHid * kHid / 8; v += kTcThreads) {
        const int r = v / (kHid / 8), c = v % (kHid / 8);
        *reinterpret_cast<uint4*>(sm + kTcSW2 + core_off(r, c, kHid * 16)) =
            halve_bf16x8(*reinterpret_cast<const uint4*>(gW2 + r * kHid + 8 * c));
    }
    for (int v = tid; v < kOut * kHid / 8; v += kTcThreads) {
        const int r = v / (kHid / 8), c = v % (kHid / 8);
        *reinterpret_cast<uint4*>(sm + kTcSW3 + core_off(r, c, kHid * 16)) =
            halve_bf16x8(*reinterpret_cast<const uint4*>(gW3 + r * kHid + 8 * c));
    }
    for (int v = tid; v < 2 * kHid + kOut; v += kTcThreads) sBias[v] = bias[v];
    // Layer 2's bias chunk (K = 16): A = ones in K 0..2 for every face, B = b2 parts per unit.
    for (int v = tid; v < 2 * kTcRows; v += kTcThreads) {
        const int r = v >> 1, c = v & 1;
        const uint2 bp = c == 0 ? bias_parts(bias[kHid + r]) : make_uint2(0, 0);
        *reinterpret_cast<uint4*>(sm + kTcSOnes + core_off(r, c, 16 * 16)) =
            c == 0 ? make_uint4(0x3F803F80u, 0x00003F80u, 0, 0) : make_uint4(0, 0, 0, 0);
        *reinterpret_cast<uint4*>(sm + kTcSB2 + core_off(r, c, 16 * 16)) = make_uint4(bp.x, bp.y, 0, 0);
    }
    if (row == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" :: "r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n"
                     :: "r"(smem_u32(tmem_holder)), "r"(kTmemCols) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_holder + (uint32_t)(slot * 128);           // the slot's columns
    const uint32_t t_lane = tmem + ((uint32_t)((warp & 3) * 32) << 16);    // this warp's 32 lanes

    const uint32_t idesc_h = mma_idesc(kTcRows, kHid);
    const uint32_t idesc_o = mma_idesc(kTcRows, kOut);
    const int ntiles = (nb + kTcRows - 1) / kTcRows;
    const int stride = gridDim.x * kTcSlots;
    uint32_t phase = 0;
    bool ok = true;
    // Two-stage prefetch: neighbour lists two tiles ahead, patch values and tensor features one
    // tile ahead, so that no dependent load waits inside a tile.
    float v[7 * BS];
    int g[kNeighbours];
    uint4 ta, tb;
    auto load_tensors = [&](int f) {
        ta = make_uint4(0, 0, 0, 0);
        tb = ta;
        if (f < nb) {
            const uint4* src = reinterpret_cast<const uint4*>(tfeat + (long long)f * kTensorSlots);
            ta = src[0];
            tb = src[1];
        }
    };
    int tile = blockIdx.x * kTcSlots + slot;
    load_neighbours(tile * kTcRows + row, nb, nbr, g);
    load_patch<BS>(tile * kTcRows + row, nb, g, w, v);
    load_tensors(tile * kTcRows + row);
    load_neighbours((tile + stride) * kTcRows + row, nb, nbr, g);
    for (; tile < ntiles && ok; tile += stride) {
        const int f = tile * kTcRows + row;
        // x entries this tile updates, loaded now so that the update at the end does not wait
        float xo[BS];
#pragma unroll
        for (int c = 0; c < BS; c++) xo[c] = f < nb ? x[(long long)f * BS + c] : 0.0f;
        // 1. inputs of face f into row `row` of the slot's input tile; input slots 44..46 (tensor
        // slots 12..14, zero in every feature row) are set to 1 for the bias columns of W1
        sScale[row] = f < nb ? store_patch<BS>(v, sSlot, row) : 0.0f;
        tb.z = 0x3F803F80u;
        tb.w = 0x00003F80u;
        *reinterpret_cast<uint4*>(sSlot + core_off(row, kResidualSlots / 8, kIn * 16)) = ta;
        *reinterpret_cast<uint4*>(sSlot + core_off(row, kResidualSlots / 8 + 1, kIn * 16)) = tb;
        fence_async_smem();
        tc_fence_before();
        slot_sync(slot);
        // 2. layer 1; meanwhile the next tile's inputs are loaded
        if (row == 0) {
            tc_fence_after();
#pragma unroll
            for (int k = 0; k < kIn / 16; k++)
                tc_mma(tmem, smem_desc(sSlot_a + k * 256, 128, kIn * 16), smem_desc(s_base + kTcSW1 + k * 256, 128, kIn * 16),
                       idesc_h, k > 0);
            tc_commit(mbar);
        }
        load_patch<BS>((tile + stride) * kTcRows + row, nb, g, w, v);
        load_tensors((tile + stride) * kTcRows + row);
        load_neighbours((tile + 2 * stride) * kTcRows + row, nb, nbr, g);
        ok = slot_and(slot, mbar_wait(mbar, phase));   // the slot leaves together if a wait expired
        phase ^= 1;
        if (!ok) break;
        tc_fence_after();
        tc_hidden_epilogue(t_lane, sSlot, row);
        fence_async_smem();
        tc_fence_before();
        slot_sync(slot);
        // 3. layer 2
        if (row == 0) {
            tc_fence_after();
#pragma unroll
            for (int k = 0; k < kHid / 16; k++)
                tc_mma(tmem, smem_desc(sSlot_a + k * 256, 128, kHid * 16), smem_desc(s_base + kTcSW2 + k * 256, 128, kHid * 16),
                       idesc_h, k > 0);
            tc_mma(tmem, smem_desc(s_base + kTcSOnes, 128, 16 * 16), smem_desc(s_base + kTcSB2, 128, 16 * 16), idesc_h, 1);
            tc_commit(mbar);
        }
        ok = slot_and(slot, mbar_wait(mbar, phase));
        phase ^= 1;
        if (!ok) break;
        tc_fence_after();
        tc_hidden_epilogue(t_lane, sSlot, row);
        fence_async_smem();
        tc_fence_before();
        slot_sync(slot);
        // 4. layer 3 into the slot's first 16 columns
        if (row == 0) {
            tc_fence_after();
#pragma unroll
            for (int k = 0; k < kHid / 16; k++)
                tc_mma(tmem, smem_desc(sSlot_a + k * 256, 128, kHid * 16), smem_desc(s_base + kTcSW3 + k * 256, 128, kHid * 16),
                       idesc_o, k > 0);
            tc_commit(mbar);
        }
        ok = slot_and(slot, mbar_wait(mbar, phase));
        phase ^= 1;
        if (!ok) break;
        tc_fence_after();
        float y[16];
        tmem_ld16(t_lane, y);
        if (f < nb) {
            const float sc = sScale[row];
#pragma unroll
            for (int c = 0; c < BS; c++) {
                const float cv = sc * (y[c] + sBias[2 * kHid + c]);
                if (isfinite(cv)) x[(long long)f * BS + c] = xo[c] + cv;
            }
        }
        tc_fence_before();
        slot_sync(slot);
    }
    if (!ok && row == 0 && status) atomicExch(status, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" :: "r"(*tmem_holder), "r"(kTmemCols)
                     : "memory");
}

// ---------------------------------------------------------------------------
// Training GEMM: C (+split) = sum_{k in chunk} A(m, k) B(k, n), 64 x BN tile per CTA (4 warps of
// 16 rows), K staged 32 at a time. A(m, k) = A[m*lda + k] (AM = false) or A[k*lda + m]
// (AM = true); B(k, n) = B[n*ldb + k] (BNM = false) or B[k*ldb + n] (BNM = true). N == BN.
// M, lda, ldb and the chunk bounds are multiples of 8. Split y writes C + y * M * BN.

template <int BN, bool AM, bool BNM>
__global__ void __launch_bounds__(128) k_gemm(int M, int K, int k_chunk, const bf16* __restrict__ A, int lda,
                                              const bf16* __restrict__ B, int ldb, float* __restrict__ C)
{
    constexpr int BK = 32;
    constexpr int LA = AM ? 64 + 8 : BK + 8;
    constexpr int LB = BNM ? BN + 8 : BK + 8;
    __shared__ __align__(16) bf16 sA[AM ? BK * LA : 64 * LA];
    __shared__ __align__(16) bf16 sB[BNM ? BK * LB : BN * LB];
    const int m0 = blockIdx.x * 64;
    const int kb = blockIdx.y * k_chunk;
    const int ke = min(K, kb + k_chunk);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int q = lane >> 3, r8 = lane & 7;
    float acc[BN / 8][4];
#pragma unroll
    for (int j = 0; j < BN / 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    const uint4 zero = make_uint4(0, 0, 0, 0);
    for (int k0 = kb; k0 < ke; k0 += BK) {
        if (!AM) {
            for (int v = threadIdx.x; v < 64 * (BK / 8); v += blockDim.x) {
                const int r = v / (BK / 8), c = (v % (BK / 8)) * 8;
                const int m = m0 + r, k = k0 + c;
                *reinterpret_cast<uint4*>(sA + r * LA + c) =
                    (m < M && k < ke) ? *reinterpret_cast<const uint4*>(A + (long long)m * lda + k) : zero;
            }
        } else {
            for (int v = threadIdx.x; v < BK * 8; v += blockDim.x) {
                const int r = v / 8, c = (v % 8) * 8;
                const int k = k0 + r, m = m0 + c;
                *reinterpret_cast<uint4*>(sA + r * LA + c) =
                    (k < ke && m < M) ? *reinterpret_cast<const uint4*>(A + (long long)k * lda + m) : zero;
            }
        }
        if (!BNM) {
            for (int v = threadIdx.x; v < BN * (BK / 8); v += blockDim.x) {
                const int r = v / (BK / 8), c = (v % (BK / 8)) * 8;
                const int k = k0 + c;
                *reinterpret_cast<uint4*>(sB + r * LB + c) =
                    k < ke ? *reinterpret_cast<const uint4*>(B + (long long)r * ldb + k) : zero;
            }
        } else {
            for (int v = threadIdx.x; v < BK * (BN / 8); v += blockDim.x) {
                const int r = v / (BN / 8), c = (v % (BN / 8)) * 8;
                const int k = k0 + r;
                *reinterpret_cast<uint4*>(sB + r * LB + c) =
                    k < ke ? *reinterpret_cast<const uint4*>(B + (long long)k * ldb + c) : zero;
            }
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < BK; ks += 16) {
            uint32_t a[4];
            if (!AM) ldsm_x4(a, sA + (16 * warp + r8 + (q & 1) * 8) * LA + ks + (q >> 1) * 8);
            else ldsm_x4_t(a, sA + (ks + r8 + (q >> 1) * 8) * LA + 16 * warp + (q & 1) * 8);
#pragma unroll
            for (int j = 0; j < BN / 8; j += 2) {
                uint32_t b[4];
                if (!BNM) ldsm_x4(b, sB + (8 * j + r8 + (q >> 1) * 8) * LB + ks + (q & 1) * 8);
                else ldsm_x4_t(b, sB + (ks + r8 + (q & 1) * 8) * LB + 8 * j + (q >> 1) * 8);
                mma16816(acc[j], a, b[0], b[1]);
                mma16816(acc[j + 1], a, b[2], b[3]);
            }
        }
        __syncthreads();
    }
    float* Cp = C + (long long)blockIdx.y * M * BN;
    const int g = lane >> 2, t = lane & 3;
    const int ma = m0 + 16 * warp + g, mb = ma + 8;
#pragma unroll
    for (int j = 0; j < BN / 8; j++) {
        const int n = 8 * j + 2 * t;
        if (ma < M) { Cp[(long long)ma * BN + n] = acc[j][0]; Cp[(long long)ma * BN + n + 1] = acc[j][1]; }
        if (mb < M) { Cp[(long long)mb * BN + n] = acc[j][2]; Cp[(long long)mb * BN + n + 1] = acc[j][3]; }
    }
}

// out[i] (+)= sum_s parts[s * count + i], fixed order.
__global__ void k_sum_splits(int nsplit, long long count, const float* __restrict__ parts, float* __restrict__ out,
                             int accumulate)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float v = 0.0f;
    for (int s = 0; s < nsplit; s++) v += parts[(long long)s * count + i];
    out[i] = accumulate ? out[i] + v : v;
}

// a += bias (per column, 128 columns); h = gelu(a) as the inference kernels compute it (pairs
// of columns in bf16x2). a keeps the pre-activation.
__global__ void k_bias_gelu(long long rows, float* __restrict__ a, const float* __restrict__ bias, bf16* __restrict__ h)
{
    const long long i = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (i >= rows * kHid) return;
    const float v0 = a[i] + bias[i % kHid], v1 = a[i + 1] + bias[(i + 1) % kHid];
    a[i] = v0;
    a[i + 1] = v1;
    *reinterpret_cast<uint32_t*>(h + i) = gelu_bf16x2(v0, v1);
}

// delta = bf16(dh * gelu'(a)).
__global__ void k_gelu_back(long long count, const float* __restrict__ dh, const float* __restrict__ a,
                            bf16* __restrict__ delta)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    delta[i] = __float2bfloat16_rn(dh[i] * gelu_grad(a[i]));
}

// Correction c_f = s_f (y_f + b3)[0..bs) into the level-0 vector layout.
template <int BS>
__global__ void k_correction(int nb, const float* __restrict__ y, const float* __restrict__ b3,
                             const float* __restrict__ scale, float* __restrict__ c)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nb) return;
#pragma unroll
    for (int k = 0; k < BS; k++) c[(long long)f * BS + k] = scale[f] * (y[(long long)f * kOut + k] + b3[k]);
}

// Energy loss L = |e - c|_A^2 / E with E = e^T A e = e^T r, r = A e, q = A c:
//   L = 1 + (c.q - 2 c.r) / E,   dL/dc = -2 (r - q) / E,   dL/dy_f = s_f dL/dc_f.
// dy rows >= nb (GEMM padding) are zero. partials[cta] = sum (c.q - 2 c.r) of the CTA.
template <int BS>
__global__ void __launch_bounds__(256) k_energy_grad(int nb, int rows, const float* __restrict__ r,
                                                     const float* __restrict__ q, const float* __restrict__ c,
                                                     const float* __restrict__ scale, double inv_energy,
                                                     bf16* __restrict__ dy, double* __restrict__ partials)
{
    __shared__ double sh[256 / 32];
    double acc = 0.0;
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < rows; f += gridDim.x * blockDim.x) {
        uint32_t packed[kOut / 2];
        float gv[kOut];
#pragma unroll
        for (int k = 0; k < kOut; k++) gv[k] = 0.0f;
        if (f < nb) {
#pragma unroll
            for (int k = 0; k < BS; k++) {
                const long long i = (long long)f * BS + k;
                const float ri = r[i], qi = q[i], ci = c[i];
                acc += (double)ci * qi - 2.0 * (double)ci * ri;
                gv[k] = (float)(scale[f] * (-2.0 * ((double)ri - qi) * inv_energy));
            }
        }
#pragma unroll
        for (int k = 0; k < kOut / 2; k++) packed[k] = pack_bf16(gv[2 * k], gv[2 * k + 1]);
        uint4* dst = reinterpret_cast<uint4*>(dy + (long long)f * kOut);
        dst[0] = make_uint4(packed[0], packed[1], packed[2], packed[3]);
        dst[1] = make_uint4(packed[4], packed[5], packed[6], packed[7]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int wI = 0; wI < 256 / 32; wI++) t += sh[wI];
        partials[blockIdx.x] = t;
    }
}

// Column sums of a BF16 [rows x ncol] matrix into parts[chunk][ncol] (fixed row chunks).
__global__ void k_colsum(long long rows, int ncol, long long chunk, const bf16* __restrict__ m,
                         float* __restrict__ parts)
{
    const int col = threadIdx.x;
    if (col >= ncol) return;
    const long long r0 = (long long)blockIdx.x * chunk, r1 = min(rows, r0 + chunk);
    float v = 0.0f;
    for (long long r = r0; r < r1; r++) v += __bfloat162float(m[r * ncol + col]);
    parts[(long long)blockIdx.x * ncol + col] = v;
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters, then the BF16 weight copy.
__global__ void k_adam(int n, float* __restrict__ p, const float* __restrict__ grad, float* __restrict__ m,
                       float* __restrict__ v, float lr, float beta1, float beta2, float eps, float c1, float c2,
                       float weight_decay)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gI = grad[i];
    const float mi = beta1 * m[i] + (1.0f - beta1) * gI;
    const float vi = beta2 * v[i] + (1.0f - beta2) * gI * gI;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * ((mi / c1) / (sqrtf(vi / c2) + eps) + weight_decay * p[i]);
}

// Master parameters -> BF16 weights (W1, W2, W3 contiguous) and FP32 biases (b1, b2, b3).
__global__ void k_split_params(const float* __restrict__ p, bf16* __restrict__ wts, float* __restrict__ bias)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kHid * kIn) wts[i] = __float2bfloat16_rn(p[kOffW1 + i]);
    if (i < kHid * kHid) wts[kHid * kIn + i] = __float2bfloat16_rn(p[kOffW2 + i]);
    if (i < kOut * kHid) wts[kHid * kIn + kHid * kHid + i] = __float2bfloat16_rn(p[kOffW3 + i]);
    if (i < kHid) { bias[i] = p[kOffB1 + i]; bias[kHid + i] = p[kOffB2 + i]; }
    if (i < kOut) bias[2 * kHid + i] = p[kOffB3 + i];
}

// w = D^-1 r (block diagonal, D^-1 entry-major: entry (r, c) of block i at dinv[(r*BS + c)*dld + i]).
template <int BS>
__global__ void k_block_diag(int nb, const float* __restrict__ dinv, long long dld, const float* __restrict__ r,
                             float* __restrict__ w)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nb) return;
    float t[BS];
#pragma unroll
    for (int c = 0; c < BS; c++) t[c] = r[(long long)i * BS + c];
#pragma unroll
    for (int rr = 0; rr < BS; rr++) {
        float v = 0.0f;
#pragma unroll
        for (int c = 0; c < BS; c++) v = fmaf(dinv[(long long)(rr * BS + c) * dld + i], t[c], v);
        w[(long long)i * BS + rr] = v;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers

#define FHG_LEARNED_BS(BSV, ...)                                                                   \
    switch (BSV) {                                                                                 \
    case 2: { constexpr int BS = 2; __VA_ARGS__; } break;                                          \
    case 3: { constexpr int BS = 3; __VA_ARGS__; } break;                                          \
    case 4: { constexpr int BS = 4; __VA_ARGS__; } break;                                          \
    default: break;                                                                                \
    }

bool learned_supports(int bs) { return bs >= 2 && bs <= kMaxLearnedBs; }

void launch_block_diag(int nb, int bs, const float* dinv, long long dld, const float* r, float* w, cudaStream_t s)
{
    const int grid = (nb + 255) / 256;
    FHG_LEARNED_BS(bs, k_block_diag<BS><<<grid, 256, 0, s>>>(nb, dinv, dld, r, w));
    g_kernel_launches++;
}

void launch_features(int nb, int rows, int bs, const int* nbr, const float* w, const void* tfeat, void* feat,
                     float* scale, cudaStream_t s)
{
    const int grid = (rows + 255) / 256;
    FHG_LEARNED_BS(bs, k_features<BS><<<grid, 256, 0, s>>>(nb, rows, nbr, w, (const bf16*)tfeat, (bf16*)feat, scale));
    g_kernel_launches++;
}

int launch_learned_apply(int nb, int bs, const int* nbr, const float* w, const void* tfeat, const void* wts,
                         const float* bias, float* x, int* status, int kernel, cudaStream_t s)
{
    // Persistent grids: as many CTAs as fit on the device at once, computed once per kernel, block
    // size and device (the shared-memory attribute is set with it). Contexts on several host threads
    // may launch at once: the table and the attribute calls are under one lock.
    static int grid_of[2][kMaxLearnedBs + 1][16] = {};
    static std::mutex grid_mutex;
    int dev = 0;
    if (!learned_supports(bs) || cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 16) return -1;
    const int kk = kernel == kLearnedKernelMmaSync ? 1 : 0;
    std::unique_lock<std::mutex> grid_lock(grid_mutex);
    if (grid_of[kk][bs][dev] == 0) {
        // tcgen05: one CTA per SM (all 512 TMEM columns, four tile pipelines, 181 KB of shared
        // memory); mma.sync: two CTAs per SM (registers <= 128 per thread, 2 x 70 KB of shared
        // memory). The shared-memory limit and carveout are set once here.
        cudaError_t e = cudaErrorInvalidValue;
        int sms = 0;
        if (kk == 1) {
            FHG_LEARNED_BS(bs, {
                e = cudaFuncSetAttribute(k_learned_apply<BS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kApplySmem);
                if (e == cudaSuccess)
                    e = cudaFuncSetAttribute(k_learned_apply<BS>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             (int)cudaSharedmemCarveoutMaxShared);
            });
        } else {
            FHG_LEARNED_BS(bs, {
                e = cudaFuncSetAttribute(k_learned_apply_tc<BS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
                if (e == cudaSuccess)
                    e = cudaFuncSetAttribute(k_learned_apply_tc<BS>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                             (int)cudaSharedmemCarveoutMaxShared);
            });
        }
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess || sms < 1) return -1;
        grid_of[kk][bs][dev] = (kk == 1 ? 2 : 1) * sms;
    }
    const int grid_max = grid_of[kk][bs][dev];
    grid_lock.unlock();
    if (kk == 1) {
        const int tiles = (nb + 15) / 16;
        const int grid = std::min(grid_max, (tiles + kApplyWarps - 1) / kApplyWarps);
        if (grid < 1) return 0;
        FHG_LEARNED_BS(bs, k_learned_apply<BS><<<grid, kApplyWarps * 32, kApplySmem, s>>>(
                               nb, nbr, w, (const bf16*)tfeat, (const bf16*)wts, bias, x));
    } else {
        const int tiles = (nb + kTcRows - 1) / kTcRows;
        const int grid = std::min(grid_max, (tiles + kTcSlots - 1) / kTcSlots);
        if (grid < 1) return 0;
        FHG_LEARNED_BS(bs, k_learned_apply_tc<BS><<<grid, kTcThreads, kTcSmem, s>>>(
                               nb, nbr, w, (const bf16*)tfeat, (const bf16*)wts, bias, x, status));
    }
    g_kernel_launches++;
    return 0;
}

// C = A B over K (see k_gemm); nsplit > 1 splits K into chunks written to `parts`
// (nsplit * M * N floats) and summed into C in a fixed order.
void launch_gemm(int kind, int M, int K, const void* A, int lda, const void* B, int ldb, float* C, float* parts,
                 int nsplit, int accumulate, cudaStream_t s)
{
    const bf16* a = (const bf16*)A;
    const bf16* b = (const bf16*)B;
    int chunk = K;
    if (nsplit > 1) chunk = ((K + nsplit - 1) / nsplit + 31) / 32 * 32;
    if (chunk < 32) chunk = 32;
    const int splits = (K + chunk - 1) / chunk;
    float* out = splits > 1 || accumulate ? parts : C;
    dim3 grid((M + 63) / 64, splits);
    int N = 0;
    switch (kind) {
    case kGemmFwdHid: k_gemm<kHid, false, false><<<grid, 128, 0, s>>>(M, K, chunk, a, lda, b, ldb, out); N = kHid; break;
    case kGemmFwdOut: k_gemm<kOut, false, false><<<grid, 128, 0, s>>>(M, K, chunk, a, lda, b, ldb, out); N = kOut; break;
    case kGemmBwdData: k_gemm<kHid, false, true><<<grid, 128, 0, s>>>(M, K, chunk, a, lda, b, ldb, out); N = kHid; break;
    case kGemmGradHid: k_gemm<kHid, true, true><<<grid, 128, 0, s>>>(M, K, chunk, a, lda, b, ldb, out); N = kHid; break;
    case kGemmGradIn: k_gemm<kIn, true, true><<<grid, 128, 0, s>>>(M, K, chunk, a, lda, b, ldb, out); N = kIn; break;
    default: return;
    }
    g_kernel_launches++;
    if (out == parts) {
        const long long count = (long long)M * N;
        k_sum_splits<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(splits, count, parts, C, accumulate);
        g_kernel_launches++;
    }
}

void launch_bias_gelu(long long rows, float* a, const float* bias, void* h, cudaStream_t s)
{
    const long long n = rows * kHid / 2;
    k_bias_gelu<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(rows, a, bias, (bf16*)h);
    g_kernel_launches++;
}

void launch_gelu_back(long long count, const float* dh, const float* a, void* delta, cudaStream_t s)
{
    k_gelu_back<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(count, dh, a, (bf16*)delta);
    g_kernel_launches++;
}

void launch_correction(int nb, int bs, const float* y, const float* b3, const float* scale, float* c, cudaStream_t s)
{
    FHG_LEARNED_BS(bs, k_correction<BS><<<(nb + 255) / 256, 256, 0, s>>>(nb, y, b3, scale, c));
    g_kernel_launches++;
}

void launch_energy_grad(int nb, int rows, int bs, const float* r, const float* q, const float* c, const float* scale,
                        double inv_energy, void* dy, double* partials, cudaStream_t s)
{
    FHG_LEARNED_BS(bs, k_energy_grad<BS><<<kReduceCtas, 256, 0, s>>>(nb, rows, r, q, c, scale, inv_energy, (bf16*)dy,
                                                                     partials));
    g_kernel_launches++;
}

void launch_colsum(long long rows, int ncol, const void* m, float* parts, float* out, cudaStream_t s)
{
    const long long chunk = (rows + kColsumChunks - 1) / kColsumChunks;
    k_colsum<<<kColsumChunks, 128, 0, s>>>(rows, ncol, chunk > 0 ? chunk : 1, (const bf16*)m, parts);
    k_sum_splits<<<(ncol + 255) / 256, 256, 0, s>>>(kColsumChunks, ncol, parts, out, 0);
    g_kernel_launches += 2;
}

void launch_adam(int n, float* p, const float* grad, float* m, float* v, float lr, float beta1, float beta2, float eps,
                 int step, float weight_decay, cudaStream_t s)
{
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    k_adam<<<(n + 255) / 256, 256, 0, s>>>(n, p, grad, m, v, lr, beta1, beta2, eps, c1, c2, weight_decay);
    g_kernel_launches++;
}

void launch_split_params(const float* p, void* wts, float* bias, cudaStream_t s)
{
    k_split_params<<<(kHid * kHid + 255) / 256, 256, 0, s>>>(p, (bf16*)wts, bias);
    g_kernel_launches++;
}

}  // namespace fhg
