// pbg_exact.cuh -- the ray/triangle test every accelerator shares.
//
// Results must equal pbrt-v2's CPU test, Triangle::Intersect / IntersectP
// (shapes/trianglemesh.cpp:119-156, :203-240), bit for bit.  That test mixes
// precisions: Cross() multiplies and subtracts in double and rounds each
// component to float (core/geometry.h:481-488); Dot() is float
// (core/geometry.h:469-472); invDivisor = 1.f / divisor.  FP64 is a small
// fraction of FP32 throughput on this part, so the test is split in two:
//
//   pbg_filter()  FP32 with FMA and no division.  It rejects a pair only when
//                 the exact test certainly rejects it, using error bounds on
//                 every quantity it compares (derivation below).
//   pbg_exact()   pbrt's arithmetic restated with correctly rounded
//                 intrinsics (__fmul_rn/__fadd_rn for Dot, __frcp_rn for
//                 1.f/divisor), run only on the pairs the filter keeps.  Each
//                 Cross component comes from xcross_f32() (pbg_xcross.h:
//                 FP32 error-free transformations with a proof of the
//                 double-then-float rounding) or, when that proof fails
//                 (rare), from __dmul_rn/__dsub_rn in FP64.
//
// Error bound used by the filter (u = 2^-24):
//   a Cross component ab - cd: pbrt's value is within 1.01u(|ab|+|cd|) of the
//   exact real, the FMA form fma(a,b,-(c*d)) within 2.01u(|ab|+|cd|), so they
//   differ by at most 3.02u(|ab|+|cd|).  Summed over a Dot with a third vector
//   x, with both Dots' own rounding (gamma_3 each), every numerator / divisor
//   the test compares differs from pbrt's by at most 9.1u * K, where K is the
//   product of the three vectors' L1 norms (K bounds sum|x_i|(|ab|+|cd|)).
//   The filter uses 32u*K + 2^-100 (the constant covers underflow) and a
//   further 32u relative margin at every threshold for the final rounding of
//   b = n * fl(1/div) and of b1 + b2.  A NaN or infinite bound never rejects.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "pbg_xcross.h"

namespace pbg {

// One triangle as the kernels read it: 48 bytes, three 16-byte words.
//   a = (p1.xyz, |e1|_1), b = (e1.xyz, |e2|_1), c = (e2.xyz, original index)
// with e1 = p2 - p1 and e2 = p3 - p1 rounded exactly as pbrt rounds them.
struct __align__(16) TriRec {
    float4 a, b, c;
};

#ifdef __CUDACC__
constexpr float kFilterC = 0x1p-19f;     // 32u
constexpr float kFilterR = 0x1p-19f;     // threshold rounding margin
constexpr float kFilterTiny = 0x1p-100f; // underflow guard

__device__ __forceinline__ float xcross(float a, float b, float c, float d) {
    // (a*b) - (c*d) evaluated in double, rounded once to float
    return __double2float_rn(__dsub_rn(__dmul_rn((double)a, (double)b),
                                       __dmul_rn((double)c, (double)d)));
}

__device__ __forceinline__ float xdot(float ax, float ay, float az, float bx, float by, float bz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// pbrt's test with its own rounding.  e1/e2 as stored (already pbrt-rounded).
static __device__ __noinline__ bool pbg_exact(float p1x, float p1y, float p1z, float e1x, float e1y,
                                       float e1z, float e2x, float e2y, float e2z, float ox,
                                       float oy, float oz, float dx, float dy, float dz, float mint,
                                       float maxt, float* t_out, float* b1_out, float* b2_out) {
    bool ok = true;
    float s1x = xcross_f32(dy, e2z, dz, e2y, ok);
    float s1y = xcross_f32(dz, e2x, dx, e2z, ok);
    float s1z = xcross_f32(dx, e2y, dy, e2x, ok);
    if (!ok) {
        s1x = xcross(dy, e2z, dz, e2y);
        s1y = xcross(dz, e2x, dx, e2z);
        s1z = xcross(dx, e2y, dy, e2x);
    }
    float divisor = xdot(s1x, s1y, s1z, e1x, e1y, e1z);
    if (divisor == 0.f) return false;
    float inv = __frcp_rn(divisor);
    float vx = __fsub_rn(ox, p1x), vy = __fsub_rn(oy, p1y), vz = __fsub_rn(oz, p1z);
    float b1 = __fmul_rn(xdot(vx, vy, vz, s1x, s1y, s1z), inv);
    if (b1 < 0.f || b1 > 1.f) return false;
    ok = true;
    float s2x = xcross_f32(vy, e1z, vz, e1y, ok);
    float s2y = xcross_f32(vz, e1x, vx, e1z, ok);
    float s2z = xcross_f32(vx, e1y, vy, e1x, ok);
    if (!ok) {
        s2x = xcross(vy, e1z, vz, e1y);
        s2y = xcross(vz, e1x, vx, e1z);
        s2z = xcross(vx, e1y, vy, e1x);
    }
    float b2 = __fmul_rn(xdot(dx, dy, dz, s2x, s2y, s2z), inv);
    if (b2 < 0.f || __fadd_rn(b1, b2) > 1.f) return false;
    float t = __fmul_rn(xdot(e2x, e2y, e2z, s2x, s2y, s2z), inv);
    if (t < mint || t > maxt) return false;
    *t_out = t;
    *b1_out = b1;
    *b2_out = b2;
    return true;
}

__device__ __forceinline__ bool pbg_exact_rec(const TriRec& tr, float4 o, float4 d, float maxt,
                                              float* t, float* b1, float* b2) {
    return pbg_exact(tr.a.x, tr.a.y, tr.a.z, tr.b.x, tr.b.y, tr.b.z, tr.c.x, tr.c.y, tr.c.z, o.x,
                     o.y, o.z, d.x, d.y, d.z, o.w, maxt, t, b1, b2);
}

__device__ __forceinline__ float flip_sign(float v, float s) {
    return __uint_as_float(__float_as_uint(v) ^ (__float_as_uint(s) & 0x80000000u));
}

// Conservative FP32 filter.  o.w = mint, maxt = current upper bound (the
// best exact t so far, which the exact test accepts when equal).  nd = |d|_1.
// Returns false only when pbg_exact() would return false for the same maxt.
// stage2 (counting kernels only): incremented when the test goes past the
// first barycentric check.
__device__ __forceinline__ bool pbg_filter(const TriRec& tr, float4 o, float4 d, float nd,
                                           float maxt, uint32_t* stage2 = nullptr) {
    const float e1x = tr.b.x, e1y = tr.b.y, e1z = tr.b.z;
    const float e2x = tr.c.x, e2y = tr.c.y, e2z = tr.c.z;
    const float ne1 = tr.a.w, ne2 = tr.b.w;
    float s1x = fmaf(d.y, e2z, -(d.z * e2y));
    float s1y = fmaf(d.z, e2x, -(d.x * e2z));
    float s1z = fmaf(d.x, e2y, -(d.y * e2x));
    float div = fmaf(s1x, e1x, fmaf(s1y, e1y, s1z * e1z));
    float vx = __fsub_rn(o.x, tr.a.x), vy = __fsub_rn(o.y, tr.a.y), vz = __fsub_rn(o.z, tr.a.z);
    float n1 = fmaf(vx, s1x, fmaf(vy, s1y, vz * s1z));
    float nv = fabsf(vx) + fabsf(vy) + fabsf(vz);
    float ck = kFilterC * nd * ne2;           // 32u |d| |e2|
    float ediv = fmaf(ck, ne1, kFilterTiny);  // bound on |div_f - div_ref|
    float e1b = fmaf(ck, nv, kFilterTiny);    // bound on |n1_f - n1_ref|
    float D = fabsf(div);
    if (!(D > ediv)) return true;  // sign of the divisor (or zero) uncertain
    float a1 = flip_sign(n1, div);
    float top = fmaf(D, 1.f + kFilterR, ediv);
    if (a1 < -e1b || a1 > top + e1b) return false;
    if (stage2) ++*stage2;
    float s2x = fmaf(vy, e1z, -(vz * e1y));
    float s2y = fmaf(vz, e1x, -(vx * e1z));
    float s2z = fmaf(vx, e1y, -(vy * e1x));
    float n2 = fmaf(d.x, s2x, fmaf(d.y, s2y, d.z * s2z));
    float nt = fmaf(e2x, s2x, fmaf(e2y, s2y, e2z * s2z));
    float cv = kFilterC * nv * ne1;  // 32u |v| |e1|
    float e2b = fmaf(cv, nd, kFilterTiny);
    float etb = fmaf(cv, ne2, kFilterTiny);
    float a2 = flip_sign(n2, div);
    float at = flip_sign(nt, div);
    if (a2 < -e2b) return false;
    if (a1 + a2 > top + e1b + e2b + kFilterR * (fabsf(a1) + fabsf(a2))) return false;
    float slack = fmaf(D, kFilterR, ediv);
    if (at > fmaf(maxt, D, fmaf(fabsf(maxt), slack, etb))) return false;
    if (at < fmaf(o.w, D, -fmaf(fabsf(o.w), slack, etb))) return false;
    return true;
}

// Orderable key for a nearest hit: larger key = nearer hit; equal t -> larger
// triangle index, which is the answer of pbrt's in-order loop (equal t is
// accepted again, so the last index wins).  0 = no hit.
__device__ __forceinline__ unsigned long long hit_key(float t, int32_t prim) {
    uint32_t b = __float_as_uint(t);
    uint32_t ord = (b & 0x80000000u) ? ~b : (b | 0x80000000u);  // ascending in t
    return ((unsigned long long)(~ord) << 32) | (uint32_t)prim;
}

__device__ __forceinline__ float key_t(unsigned long long k) {
    uint32_t ord = ~(uint32_t)(k >> 32);
    uint32_t b = (ord & 0x80000000u) ? (ord & 0x7fffffffu) : ~ord;
    return __uint_as_float(b);
}

__device__ __forceinline__ int32_t key_prim(unsigned long long k) { return (int32_t)(uint32_t)k; }
#endif  // __CUDACC__

}  // namespace pbg
