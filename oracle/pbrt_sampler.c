/*
 * pbrt_sampler.c -- restatement of the random numbers one breadth-first
 * render task draws, for feeding the GPU renderer the reference's own sample
 * stream.  TEST INFRASTRUCTURE ONLY (loaded by tests/).
 *
 *   RNG             core/rng.cpp: the Mersenne Twister MT19937 (Matsumoto and
 *                   Nishimura, 1998; the published init_genrand seeding and
 *                   tempering), RandomUInt = one tempered 32-bit output,
 *                   RandomFloat = (RandomUInt & 0xffffff) / 2^24
 *   task            renderers/breadth-first.cpp:18-48: RNG rng(taskNum);
 *                   GetMoreSamples per pixel until the task's sample count
 *   sampler         samplers/stratified.cpp:60-105 GetMoreSamples: image and
 *                   lens samples by StratifiedSample2D, time by
 *                   StratifiedSample1D, lens and time shuffled, then for each
 *                   sample every 1-D and 2-D integrator array drawn by
 *                   LatinHypercube (core/montecarlo.cpp:140-179,
 *                   core/montecarlo.h:167-173)
 * The integrator then draws from the same RNG; orc_pbrt_task_samples returns
 * that continuation too.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define MT_N 624
#define MT_M 397

typedef struct {
    uint32_t mt[MT_N];
    int mti;
} orc_rng;

static void rng_seed(orc_rng* r, uint32_t seed) {
    r->mt[0] = seed;
    for (int i = 1; i < MT_N; ++i) r->mt[i] = 1812433253u * (r->mt[i - 1] ^ (r->mt[i - 1] >> 30)) + (uint32_t)i;
    r->mti = MT_N;
}

static uint32_t rng_uint(orc_rng* r) {
    if (r->mti >= MT_N) {
        for (int k = 0; k < MT_N; ++k) {
            const uint32_t y = (r->mt[k] & 0x80000000u) | (r->mt[(k + 1) % MT_N] & 0x7fffffffu);
            r->mt[k] = r->mt[(k + MT_M) % MT_N] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        r->mti = 0;
    }
    uint32_t y = r->mt[r->mti++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

static float rng_float(orc_rng* r) { return (float)(rng_uint(r) & 0xffffffu) / 16777216.f; }

static const float kOneMinusEps = 0x1.fffffep-1f;

static float fmin1(float v) { return v < kOneMinusEps ? v : kOneMinusEps; }

static void strat2d(float* s, int nx, int ny, orc_rng* r, int jitter) {
    const float dx = 1.f / (float)nx, dy = 1.f / (float)ny;
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            const float jx = jitter ? rng_float(r) : 0.5f;
            const float jy = jitter ? rng_float(r) : 0.5f;
            *s++ = fmin1(((float)x + jx) * dx);
            *s++ = fmin1(((float)y + jy) * dy);
        }
}

static void strat1d(float* s, int n, orc_rng* r, int jitter) {
    const float inv = 1.f / (float)n;
    for (int i = 0; i < n; ++i) {
        const float d = jitter ? rng_float(r) : 0.5f;
        *s++ = fmin1(((float)i + d) * inv);
    }
}

static void shuffle(float* s, uint32_t count, uint32_t dims, orc_rng* r) {
    for (uint32_t i = 0; i < count; ++i) {
        const uint32_t other = i + (rng_uint(r) % (count - i));
        for (uint32_t j = 0; j < dims; ++j) {
            const float t = s[dims * i + j];
            s[dims * i + j] = s[dims * other + j];
            s[dims * other + j] = t;
        }
    }
}

static void latin(float* s, uint32_t n, uint32_t dims, orc_rng* r) {
    const float delta = 1.f / (float)n;
    for (uint32_t i = 0; i < n; ++i)
        for (uint32_t j = 0; j < dims; ++j) s[dims * i + j] = fmin1(((float)i + rng_float(r)) * delta);
    for (uint32_t i = 0; i < dims; ++i)
        for (uint32_t j = 0; j < n; ++j) {
            const uint32_t other = j + (rng_uint(r) % (n - j));
            const float t = s[dims * j + i];
            s[dims * j + i] = s[dims * other + i];
            s[dims * other + i] = t;
        }
}

/* One task's samples.  The sampler covers pixels [x0, x1) x [y0, y1)
 * (the film's sample extent), spx x spy samples per pixel.  n1d[k1] /
 * n2d[k2]: sizes of the integrators' 1-D and 2-D arrays in request order.
 * Outputs per sample: image_xy[2], oned[sum n1d] (arrays concatenated),
 * twod[2 * sum n2d]; then rng_out[nrng] = the RNG's next RandomFloat draws.
 * Returns the number of samples produced (at most count). */
int64_t orc_pbrt_task_samples(uint32_t task, int x0, int x1, int y0, int y1, int spx, int spy, int jitter,
                              const int* n1d, int k1, const int* n2d, int k2, int64_t count, float* image_xy,
                              float* oned, float* twod, int64_t nrng, float* rng_out) {
    orc_rng r;
    rng_seed(&r, task);
    const int ns = spx * spy;
    int t1 = 0, t2 = 0;
    for (int k = 0; k < k1; ++k) t1 += n1d[k];
    for (int k = 0; k < k2; ++k) t2 += n2d[k];
    float* img = (float*)malloc(sizeof(float) * 2 * ns);
    float* lens = (float*)malloc(sizeof(float) * 2 * ns);
    float* tim = (float*)malloc(sizeof(float) * ns);
    int64_t got = 0;
    int xp = x0, yp = y0;
    while (got < count && yp < y1) {
        strat2d(img, spx, spy, &r, jitter);
        strat2d(lens, spx, spy, &r, jitter);
        strat1d(tim, ns, &r, jitter);
        for (int o = 0; o < 2 * ns; o += 2) {
            img[o] += (float)xp;
            img[o + 1] += (float)yp;
        }
        shuffle(lens, (uint32_t)ns, 2, &r);
        shuffle(tim, (uint32_t)ns, 1, &r);
        for (int i = 0; i < ns && got < count; ++i, ++got) {
            image_xy[2 * got] = img[2 * i];
            image_xy[2 * got + 1] = img[2 * i + 1];
            float* o1 = oned + got * t1;
            for (int k = 0; k < k1; ++k) {
                latin(o1, (uint32_t)n1d[k], 1, &r);
                o1 += n1d[k];
            }
            float* o2 = twod + got * 2 * t2;
            for (int k = 0; k < k2; ++k) {
                latin(o2, (uint32_t)n2d[k], 2, &r);
                o2 += 2 * n2d[k];
            }
        }
        if (++xp == x1) {
            xp = x0;
            ++yp;
        }
    }
    for (int64_t k = 0; k < nrng; ++k) rng_out[k] = rng_float(&r);
    free(img);
    free(lens);
    free(tim);
    return got;
}
