// FP32 pairs ("double-FP32"): a value v held as hi + lo with hi = fl32(v) and lo = fl32(v - hi),
// about 48 significant bits, computed on the FP32 pipe. GB300's FP64 pipe runs at 1/56 of its FP32
// rate, so block products whose FP64 multiply-adds would outrun HBM are computed this way instead:
// the value pair occupies the 8 bytes a double does, and every multiply-add is split exactly with
// an FMA (Dekker 1971, "A floating-point technique for extending the available precision";
// Knuth, TAOCP vol. 2, 4.2.2, TwoSum), for a relative error of a few units of 2^-47 per term.
#pragma once

#include <cuda_runtime.h>

namespace fhg {

// The math library's fma overloads stay visible next to the pair's.
using ::fma;

// (sh, sl) += (ph, pl): TwoSum of the high parts, low parts and the rounding error added; the
// result is left unnormalised (a running sum's low part absorbs the errors of many terms).
__host__ __device__ __forceinline__ void df_add(float& sh, float& sl, float ph, float pl)
{
    const float s = sh + ph;
    const float bv = s - sh;
    const float err = (sh - (s - bv)) + (ph - bv);
    sl = sl + (err + pl);
    sh = s;
}

// Product of two pairs (a_lo * b_lo, 2^-48 relative, dropped): ph + pl, ph = fl(a_hi b_hi) and its
// FMA-exact error carrying the cross terms.
__device__ __forceinline__ void df_mul(float ah, float al, float bh, float bl, float& ph, float& pl)
{
    ph = ah * bh;
    pl = fmaf(ah, bh, -ph) + fmaf(ah, bl, al * bh);
}

// The normalised pair of s + e: hi = fl(s + e) (the FP32 value nearest the pair), lo the rest.
__host__ __device__ __forceinline__ void df_norm(float s, float e, float& h, float& l)
{
    h = s + e;
    l = e - (h - s);
}

// (xh, xl) + (ph, pl), normalised.
__host__ __device__ __forceinline__ void df_sum(float xh, float xl, float ph, float pl, float& h, float& l)
{
    df_add(xh, xl, ph, pl);
    df_norm(xh, xl, h, l);
}

// An FP64 value as an FP32 pair (exact to 2^-48 relative).
__host__ __device__ __forceinline__ void df_split(double v, float& h, float& l)
{
    h = (float)v;
    l = (float)(v - (double)h);
}

// A pair as a value type, so that the block kernels written for float and double run on pairs
// unchanged: + - * give normalised results, fma(a, b, c) = c + a b leaves the running sum
// unnormalised (fin() normalises it before it is stored). 8-byte aligned: one 64-bit load per pair.
struct alignas(8) dfl {
    float h, l;
    dfl() = default;
    __host__ __device__ constexpr dfl(float hi, float lo) : h(hi), l(lo) {}
    __host__ __device__ explicit dfl(int v) : h((float)v), l(0.f) {}
    __host__ __device__ explicit dfl(float v) : h(v), l(0.f) {}
    __host__ __device__ explicit dfl(double v) { df_split(v, h, l); }
    __host__ __device__ explicit operator double() const { return (double)h + (double)l; }
    __host__ __device__ explicit operator float() const { return h + l; }
};

__device__ __forceinline__ dfl operator+(dfl a, dfl b)
{
    dfl r;
    df_sum(a.h, a.l, b.h, b.l, r.h, r.l);
    return r;
}
__device__ __forceinline__ dfl operator-(dfl a) { return dfl(-a.h, -a.l); }
__device__ __forceinline__ dfl operator-(dfl a, dfl b) { return a + (-b); }
__device__ __forceinline__ dfl operator*(dfl a, dfl b)
{
    float ph, pl;
    df_mul(a.h, a.l, b.h, b.l, ph, pl);
    dfl r;
    df_norm(ph, pl, r.h, r.l);
    return r;
}
__device__ __forceinline__ dfl& operator+=(dfl& a, dfl b)
{
    df_add(a.h, a.l, b.h, b.l);
    return a;
}
__device__ __forceinline__ dfl fma(dfl a, dfl b, dfl c)
{
    float ph, pl;
    df_mul(a.h, a.l, b.h, b.l, ph, pl);
    df_add(c.h, c.l, ph, pl);
    return c;
}
__host__ __device__ __forceinline__ bool operator!=(dfl a, dfl b) { return a.h != b.h || a.l != b.l; }
__host__ __device__ __forceinline__ bool operator==(dfl a, dfl b) { return a.h == b.h && a.l == b.l; }

// Value to store: pairs normalised, float and double unchanged.
template <class T>
__device__ __forceinline__ T fin(T v) { return v; }
template <>
__device__ __forceinline__ dfl fin<dfl>(dfl v)
{
    dfl r;
    df_norm(v.h, v.l, r.h, r.l);
    return r;
}

}  // namespace fhg
