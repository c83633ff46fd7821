// pbg_count.cuh -- traversal work counters for the counting kernel variants
// (profiling level 2): per-thread tallies, added to global counters once per
// thread when its traversal ends.
#pragma once
#include <cstdint>

namespace pbg {

struct WorkCount {
    // filt2: filter tests that passed the first barycentric check and went
    // on to the second edge function and t (the Moller-Trumbore stages 2-3)
    uint32_t node = 0, leaf = 0, filt = 0, exact = 0, hit = 0, filt2 = 0;

    __device__ __forceinline__ void flush(unsigned long long* wc) {
        const uint32_t v[6] = {node, leaf, filt, exact, hit, filt2};
#pragma unroll
        for (int k = 0; k < 6; ++k)
            if (v[k]) atomicAdd(&wc[k], (unsigned long long)v[k]);
    }
};

}  // namespace pbg
