// pbg_dg.cuh -- device arithmetic in pbrt's rounding (no contraction), and
// the DifferentialGeometry of a triangle hit.
//
//   Cross        core/geometry.h:481-488  (double products, one rounding)
//   Dot          core/geometry.h:469-472  ((x*x + y*y) + z*z in float)
//   Normalize    core/geometry.h:511      (v * (1/|v|), |v| = sqrtf)
//   Transform    core/transform.h:184-212 (point: divide by w unless w == 1)
//   dg of a hit  shapes/trianglemesh.cpp:158-190, core/diffgeom.cpp:32-47
#pragma once
#include <cstdint>

#include "pbg_exact.cuh"

namespace pbg {

#ifdef __CUDACC__
struct V3 {
    float x, y, z;
};

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) {
    return V3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
__device__ __forceinline__ V3 vadd(V3 a, V3 b) {
    return V3{__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)};
}
__device__ __forceinline__ V3 vmul(V3 a, float s) {
    return V3{__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)};
}
__device__ __forceinline__ V3 vneg(V3 a) { return V3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float vdot(V3 a, V3 b) { return xdot(a.x, a.y, a.z, b.x, b.y, b.z); }
__device__ __forceinline__ V3 vcross(V3 a, V3 b) {
    return V3{xcross(a.y, b.z, a.z, b.y), xcross(a.z, b.x, a.x, b.z), xcross(a.x, b.y, a.y, b.x)};
}
__device__ __forceinline__ float vlen(V3 a) { return __fsqrt_rn(vdot(a, a)); }
__device__ __forceinline__ V3 vnormalize(V3 a) { return vmul(a, __frcp_rn(vlen(a))); }

// Row-major 4x4 applied to a point / a vector (core/transform.h:184-212).
__device__ __forceinline__ V3 xform_point(const float* m, V3 p) {
    const float xp = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], p.x), __fmul_rn(m[1], p.y)), __fmul_rn(m[2], p.z)), m[3]);
    const float yp = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[4], p.x), __fmul_rn(m[5], p.y)), __fmul_rn(m[6], p.z)), m[7]);
    const float zp = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[8], p.x), __fmul_rn(m[9], p.y)), __fmul_rn(m[10], p.z)), m[11]);
    const float wp = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[12], p.x), __fmul_rn(m[13], p.y)), __fmul_rn(m[14], p.z)), m[15]);
    if (wp == 1.f) return V3{xp, yp, zp};
    const float inv = __frcp_rn(wp);
    return V3{__fmul_rn(inv, xp), __fmul_rn(inv, yp), __fmul_rn(inv, zp)};
}

__device__ __forceinline__ V3 xform_vector(const float* m, V3 v) {
    return V3{__fadd_rn(__fadd_rn(__fmul_rn(m[0], v.x), __fmul_rn(m[1], v.y)), __fmul_rn(m[2], v.z)),
              __fadd_rn(__fadd_rn(__fmul_rn(m[4], v.x), __fmul_rn(m[5], v.y)), __fmul_rn(m[6], v.z)),
              __fadd_rn(__fadd_rn(__fmul_rn(m[8], v.x), __fmul_rn(m[9], v.y)), __fmul_rn(m[10], v.z))};
}

struct HitDG {
    V3 p, dpdu, dpdv, nn;
    float u, v;
};

// DifferentialGeometry of the hit on triangle v[9] (uv6 may be NULL for
// pbrt's default (0,0),(1,0),(1,1)); p = o + d*t.
__device__ __forceinline__ HitDG hit_dg(const float* v, const float* uv6, V3 o, V3 d, float t,
                                        float b1, float b2) {
    float u[3][2];
    if (uv6) {
        u[0][0] = uv6[0]; u[0][1] = uv6[1]; u[1][0] = uv6[2]; u[1][1] = uv6[3]; u[2][0] = uv6[4]; u[2][1] = uv6[5];
    } else {
        u[0][0] = 0.f; u[0][1] = 0.f; u[1][0] = 1.f; u[1][1] = 0.f; u[2][0] = 1.f; u[2][1] = 1.f;
    }
    const float du1 = __fsub_rn(u[0][0], u[2][0]), du2 = __fsub_rn(u[1][0], u[2][0]);
    const float dv1 = __fsub_rn(u[0][1], u[2][1]), dv2 = __fsub_rn(u[1][1], u[2][1]);
    const V3 p1 = v3(v[0], v[1], v[2]), p2 = v3(v[3], v[4], v[5]), p3 = v3(v[6], v[7], v[8]);
    const V3 dp1 = vsub(p1, p3), dp2 = vsub(p2, p3);
    HitDG g;
    const float det = __fsub_rn(__fmul_rn(du1, dv2), __fmul_rn(dv1, du2));
    if (det == 0.f) {
        const V3 e1 = vsub(p2, p1), e2 = vsub(p3, p1);
        const V3 v1 = vnormalize(vcross(e2, e1));
        if (fabsf(v1.x) > fabsf(v1.y)) {
            const float il = __frcp_rn(__fsqrt_rn(__fadd_rn(__fmul_rn(v1.x, v1.x), __fmul_rn(v1.z, v1.z))));
            g.dpdu = v3(__fmul_rn(-v1.z, il), 0.f, __fmul_rn(v1.x, il));
        } else {
            const float il = __frcp_rn(__fsqrt_rn(__fadd_rn(__fmul_rn(v1.y, v1.y), __fmul_rn(v1.z, v1.z))));
            g.dpdu = v3(0.f, __fmul_rn(v1.z, il), __fmul_rn(-v1.y, il));
        }
        g.dpdv = vcross(v1, g.dpdu);
    } else {
        const float invdet = __frcp_rn(det);
        g.dpdu = vmul(vsub(vmul(dp1, dv2), vmul(dp2, dv1)), invdet);
        g.dpdv = vmul(vadd(vmul(dp1, -du2), vmul(dp2, du1)), invdet);
    }
    const float b0 = __fsub_rn(__fsub_rn(1.f, b1), b2);
    g.u = __fadd_rn(__fadd_rn(__fmul_rn(b0, u[0][0]), __fmul_rn(b1, u[1][0])), __fmul_rn(b2, u[2][0]));
    g.v = __fadd_rn(__fadd_rn(__fmul_rn(b0, u[0][1]), __fmul_rn(b1, u[1][1])), __fmul_rn(b2, u[2][1]));
    g.p = vadd(o, vmul(d, t));
    g.nn = vnormalize(vcross(g.dpdu, g.dpdv));
    return g;
}
#endif  // __CUDACC__

}  // namespace pbg
