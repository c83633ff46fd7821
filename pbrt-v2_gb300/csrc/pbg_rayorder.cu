// pbg_rayorder.cu -- placeholder ordering (identity) until the ray-hierarchy
// sort lands.
#include "pbg_internal.h"

namespace pbg {

int ray_order(pbg_scene* s, const float4* o, const float4* d, int64_t n, const int32_t** perm,
              cudaStream_t st) {
    (void)s; (void)o; (void)d; (void)n; (void)st;
    *perm = nullptr;
    return PBG_OK;
}

int rh_nearest(pbg_scene*, const float4*, const float4*, const uint8_t*, int64_t, int32_t*,
               float*, float*, float*, cudaStream_t) {
    set_last_error("rayhierarchy traversal not built yet");
    return PBG_ERR_UNSUPPORTED;
}

int rh_occluded(pbg_scene*, const float4*, const float4*, const uint8_t*, int64_t, uint8_t*,
                cudaStream_t) {
    set_last_error("rayhierarchy traversal not built yet");
    return PBG_ERR_UNSUPPORTED;
}

}  // namespace pbg
