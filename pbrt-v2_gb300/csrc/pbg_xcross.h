// pbg_xcross.h -- pbrt's Cross() component in FP32 arithmetic.
//
// pbrt-v2's Cross (core/geometry.h:481-488) forms each component as
//     (float)((double)a * b - (double)c * d)
// i.e. two exact products, one subtraction rounded to double, then rounded to
// float.  FP64 runs at a small fraction of the FP32 rate on this part (and the
// exact test runs warp-divergent), so xcross_f32() reproduces that value with
// error-free FP32 transformations and proves it is right, or reports that it
// cannot (ok = false) and the caller evaluates the FP64 form instead.
//
// Method (u = 2^-24):
//   ph = fl(ab), pl = fma(a, b, -ph)      ab = ph + pl exactly   (TwoProduct)
//   qh = fl(cd), ql = fma(c, d, -qh)      cd = qh + ql exactly
//   (s, e1) = TwoSum(ph, -qh), (t, e2) = TwoSum(pl, -ql)   x = s + e1 + t + e2
//   r1 = fl(e1 + e2), r2 = fl(t + r1), (hi, lo) = TwoSum(s, r2)
//   then x = hi + lo - delta with |delta| <= u(|r1| + |r2|), and the double
//   rounding moves x by at most 2^-53|x| <= 2^-52|hi|.  With B the sum of
//   those two bounds, if |lo| + B is below half the gap from hi to its
//   neighbouring floats (a quarter of ulp(hi) when hi is a power of two),
//   both x and fl64(x) round to hi, so (float)fl64(x) == hi.
// The products must stay clear of overflow and of the subnormal range for
// TwoProduct to be exact (|ab|, |cd| in [2^-90, 2^100) or exactly zero);
// otherwise, at exact float midpoints, and under deep cancellation
// (|hi| < 2^-67 or B too large) the result is not proven: ok = false.
// An exact zero product makes x = -cd or ab exactly, which the double
// subtraction does not round; the float subtraction gives the same value and
// the same sign of zero.
#pragma once
#include <math.h>

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define PBG_XHD __host__ __device__ __forceinline__
#else
#define PBG_XHD inline
#endif

namespace pbg {

PBG_XHD float xc_add(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}

PBG_XHD float xc_sub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}

PBG_XHD float xc_mul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}

PBG_XHD float xc_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

PBG_XHD uint32_t xc_bits(float x) {
#if defined(__CUDA_ARCH__)
    return __float_as_uint(x);
#else
    uint32_t b;
    std::memcpy(&b, &x, 4);
    return b;
#endif
}

PBG_XHD float xc_float(uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __uint_as_float(b);
#else
    float x;
    std::memcpy(&x, &b, 4);
    return x;
#endif
}

// Knuth's TwoSum: s + e == a + b exactly (no overflow).
PBG_XHD void xc_two_sum(float a, float b, float& s, float& e) {
    s = xc_add(a, b);
    const float bb = xc_sub(s, a);
    e = xc_add(xc_sub(a, xc_sub(s, bb)), xc_sub(b, bb));
}

// (float)((double)a * b - (double)c * d) when provable; ok is cleared
// otherwise (it is never set, so one flag can cover several calls).
PBG_XHD float xcross_f32(float a, float b, float c, float d, bool& ok) {
    const float ph = xc_mul(a, b), qh = xc_mul(c, d);
    const float aph = fabsf(ph), aqh = fabsf(qh);
    if (!(aph < 0x1p100f) || !(aqh < 0x1p100f) ||  // also NaN and inf
        (aph < 0x1p-90f && a != 0.f && b != 0.f) || (aqh < 0x1p-90f && c != 0.f && d != 0.f)) {
        ok = false;
        return 0.f;
    }
    if (ph == 0.f || qh == 0.f) return xc_sub(ph, qh);
    const float pl = xc_fma(a, b, -ph), ql = xc_fma(c, d, -qh);
    float s, e1, t, e2;
    xc_two_sum(ph, -qh, s, e1);
    xc_two_sum(pl, -ql, t, e2);
    const float r1 = xc_add(e1, e2);
    const float r2 = xc_add(t, r1);
    float hi, lo;
    xc_two_sum(s, r2, hi, lo);
    const uint32_t hb = xc_bits(hi);
    const uint32_t ex = (hb >> 23) & 0xffu;
    if (ex < 60u) {  // |hi| < 2^-67, including hi == 0
        ok = false;
        return 0.f;
    }
    const float ulp = xc_float((ex - 23u) << 23);
    const float gap = xc_mul(ulp, (hb & 0x7fffffu) == 0u ? 0.25f : 0.5f);
    // B, doubled to absorb its own rounding
    const float bound = xc_fma(0x1p-23f, xc_add(fabsf(r1), fabsf(r2)),
                              xc_mul(0x1p-51f, fabsf(hi)));
    if (!(xc_add(fabsf(lo), bound) < gap)) {
        ok = false;
        return 0.f;
    }
    return hi;
}

}  // namespace pbg
