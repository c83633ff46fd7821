// Checks xcross_f32() (pbrt-v2_gb300/csrc/pbg_xcross.h) against pbrt's
// Cross() component (float)((double)a * b - (double)c * d), bit for bit, on
// seeded random and adversarial inputs.  Prints "cases proven fallbacks
// mismatches"; exit status 1 on any mismatch among proven results.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "../../pbrt-v2_gb300/csrc/pbg_xcross.h"

static uint64_t state = 0x9e3779b97f4a7c15ull;
static uint64_t next_u64() {  // splitmix64
    uint64_t z = (state += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
static float from_bits(uint32_t b) {
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}
static uint32_t to_bits(float f) {
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}
static float rnd_float(int emin, int emax) {  // random sign, exponent, mantissa
    uint64_t r = next_u64();
    int e = emin + (int)(r % (uint64_t)(emax - emin + 1));
    uint32_t m = (uint32_t)(r >> 20) & 0x7fffffu;
    uint32_t s = (uint32_t)(r >> 63) << 31;
    return from_bits(s | ((uint32_t)(e + 127) << 23) | m);
}
static float few_bits(int bits, int emin, int emax) {  // mantissa with few set bits
    uint64_t r = next_u64();
    int e = emin + (int)(r % (uint64_t)(emax - emin + 1));
    uint32_t m = ((uint32_t)(r >> 20) & ((1u << bits) - 1u)) << (23 - bits);
    uint32_t s = (uint32_t)(r >> 63) << 31;
    return from_bits(s | ((uint32_t)(e + 127) << 23) | m);
}
static float unit() { return (float)((next_u64() >> 40) * 0x1p-24); }

int main(int argc, char** argv) {
    long n = argc > 1 ? atol(argv[1]) : 10000000;
    long proven = 0, fallback = 0, bad = 0;
    const float specials[] = {0.f, -0.f, 1.f, -1.f, 0.5f, 3.f, 1e-30f, -1e-30f, 1e-45f, 1e38f,
                              INFINITY, -INFINITY, NAN, 0x1p-90f, 0x1p100f, 0x1.fffffep-1f};
    for (long i = 0; i < n; ++i) {
        float a, b, c, d;
        switch (i % 8) {
            case 0:  // generic magnitudes
                a = rnd_float(-30, 30), b = rnd_float(-30, 30), c = rnd_float(-30, 30),
                d = rnd_float(-30, 30);
                break;
            case 1: {  // near cancellation: cd close to ab
                a = rnd_float(-8, 8), b = rnd_float(-8, 8);
                c = from_bits(to_bits(a) + (uint32_t)(next_u64() % 5) - 2u);
                d = from_bits(to_bits(b) + (uint32_t)(next_u64() % 5) - 2u);
                break;
            }
            case 2:  // few mantissa bits: exact products, float midpoints
                a = few_bits(6, -4, 4), b = few_bits(6, -4, 4), c = few_bits(6, -4, 4),
                d = few_bits(6, -4, 4);
                break;
            case 3:  // very different magnitudes: the double rounding matters
                a = rnd_float(-2, 2), b = rnd_float(-2, 2), c = rnd_float(-40, -20),
                d = rnd_float(-10, 0);
                break;
            case 4: {  // unit directions against scene-sized edges
                a = unit() * 2.f - 1.f, b = (unit() - 0.5f) * 0.125f, c = unit() * 2.f - 1.f,
                d = (unit() - 0.5f) * 0.125f;
                break;
            }
            case 5:  // specials mixed in
                a = specials[next_u64() % 16], b = rnd_float(-10, 10),
                c = (next_u64() & 1) ? specials[next_u64() % 16] : rnd_float(-10, 10),
                d = rnd_float(-10, 10);
                break;
            case 6:  // tiny and huge
                a = rnd_float(-70, -40), b = rnd_float(-70, -20), c = rnd_float(40, 60),
                d = rnd_float(30, 50);
                break;
            default: {  // products exactly at float midpoints, off by one double ulp
                a = few_bits(12, -3, 3), b = few_bits(12, -3, 3);
                c = rnd_float(-40, -30), d = rnd_float(-20, -10);
                break;
            }
        }
        bool ok = true;
        float got = pbg::xcross_f32(a, b, c, d, ok);
        float want = (float)((double)a * (double)b - (double)c * (double)d);
        if (!ok) {
            ++fallback;
            continue;
        }
        ++proven;
        if (to_bits(got) != to_bits(want)) {
            if (bad < 10)
                printf("MISMATCH a=%a b=%a c=%a d=%a got=%a want=%a\n", a, b, c, d, got, want);
            ++bad;
        }
    }
    printf("%ld %ld %ld %ld\n", n, proven, fallback, bad);
    return bad ? 1 : 0;
}
