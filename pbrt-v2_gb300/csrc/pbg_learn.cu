// pbg_learn.cu -- learned traversal ordering for Accelerator "ray-bvh".
//
// No counterpart in the reference.  A small MLP scores, for each ray, which
// of the K = 256 top clusters of the scene's BVH holds its first hit; the
// traversal then walks the predicted cluster first (any-hit rays often stop
// there; nearest-hit rays enter the full walk with a tight t_max) and the
// full exact walk still follows, so results never change.
//
//   features   105 per ray, padded to 112: o, d, clamped 1/d, and a 16-band
//              sin/cos encoding of the origin normalised to the scene box
//              (bands at pi * 2^(b/2), b = 0..15)
//   network    112 -> 64 -> 64 -> 256, ReLU, BF16 weights, FP32 accumulation
//   inference  one fused kernel: three tcgen05 GEMMs per 128-ray tile, weights
//              resident in shared memory, activations bounced through TMEM
//              and shared memory, arg-max written per ray
//   training   softmax cross-entropy against the cluster of the ray's first
//              hit (records from earlier batches), plain minibatch SGD with
//              momentum; every GEMM of the forward and backward pass is the
//              tcgen05 GEMM of pbg_mlp.cu, with small CUDA-core kernels for
//              bias, ReLU, softmax, transposes and the update.
#include <algorithm>
#include <cmath>
#include <vector>

#include "pbg_internal.h"
#include "pbg_learn.h"
#include "pbg_tc.cuh"

namespace pbg {

int tc_gemm(const uint16_t* A, const uint16_t* B, float* C, int M, int N, int K, int accumulate,
            int* status, cudaStream_t st, float* work);
size_t tc_gemm_work_floats(int M, int N, int K);

// ------------------------------------------------------------ features

// The features of one ray in order, passed to emit(value) one at a time
// (fully unrolled, so a caller can pack them as they come).
template <class Emit>
__device__ __forceinline__ void for_each_feature(float4 o, float4 d, const float* lo, const float* inv_ext,
                                                 Emit&& emit) {
    const float len = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
    const float il = len > 0.f ? 1.f / len : 0.f;
    const float dx = d.x * il, dy = d.y * il, dz = d.z * il;
    const float u[3] = {(o.x - lo[0]) * inv_ext[0], (o.y - lo[1]) * inv_ext[1], (o.z - lo[2]) * inv_ext[2]};
    // normalised origin, direction, clamped reciprocal direction
    emit(u[0] * 2.f - 1.f);
    emit(u[1] * 2.f - 1.f);
    emit(u[2] * 2.f - 1.f);
    emit(dx);
    emit(dy);
    emit(dz);
    emit(fminf(fmaxf(dx != 0.f ? 1.f / dx : 16.f, -16.f), 16.f) * 0.0625f);
    emit(fminf(fmaxf(dy != 0.f ? 1.f / dy : 16.f, -16.f), 16.f) * 0.0625f);
    emit(fminf(fmaxf(dz != 0.f ? 1.f / dz : 16.f, -16.f), 16.f) * 0.0625f);
#pragma unroll
    for (int b = 0; b < 16; ++b) {
        const float w = 3.14159265358979f * exp2f(0.5f * (float)b);
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            float sn, cs;
            __sincosf(w * u[a], &sn, &cs);
            emit(sn);
            emit(cs);
        }
    }
#pragma unroll
    for (int k = 9 + 96; k < kFeat; ++k) emit(0.f);
}

__device__ __forceinline__ void ray_features(float4 o, float4 d, const float* lo, const float* inv_ext,
                                             float* f /* kFeat */) {
    int k = 0;
    for_each_feature(o, d, lo, inv_ext, [&](float v) { f[k++] = v; });
}

// X [n_pad x 112] bf16 rows; rows >= n are zero.
__global__ void features_kernel(const float4* __restrict__ ro, const float4* __restrict__ rd,
                                const int32_t* __restrict__ idx, int64_t n, int64_t n_pad,
                                LearnBox box, uint16_t* __restrict__ X) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_pad) return;
    float f[kFeat];
    if (i < n) {
        const int64_t r = idx ? (int64_t)idx[i] : i;
        ray_features(ro[r], rd[r], box.lo, box.inv_ext, f);
    } else {
        for (int k = 0; k < kFeat; ++k) f[k] = 0.f;
    }
    uint16_t* row = X + i * kFeat;
#pragma unroll
    for (int k = 0; k < kFeat; ++k) row[k] = f2bf(f[k]);
}

// ------------------------------------------------------- training step

// H = relu(Z + b) as bf16 (row-major [rows x cols]); Z fp32 in place kept.
__global__ void bias_relu_kernel(float* __restrict__ Z, const float* __restrict__ b, int64_t rows,
                                 int cols, int relu, uint16_t* __restrict__ H) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols) return;
    const int c = (int)(i % cols);
    float v = Z[i] + b[c];
    if (relu) v = fmaxf(v, 0.f);
    Z[i] = v;
    if (H) H[i] = f2bf(v);
}

// dZ = (softmax(Z) - onehot(label)) / B for valid rows; loss and accuracy
// accumulated in acc[0..1].  One warp per row of 256 logits.
__global__ void softmax_grad_kernel(const float* __restrict__ Z, const int32_t* __restrict__ label,
                                    int64_t rows, int64_t valid_rows, float scale,
                                    float* __restrict__ dZ, uint16_t* __restrict__ dZb,
                                    float* __restrict__ acc) {
    const int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (r >= rows) return;
    const float* z = Z + r * kClusters;
    float v[8];
    float mx = -INFINITY;
    int am = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = z[lane + 32 * k];
        if (v[k] > mx) {
            mx = v[k];
            am = lane + 32 * k;
        }
    }
    for (int off = 16; off; off >>= 1) {
        const float om = __shfl_xor_sync(0xffffffffu, mx, off);
        const int oa = __shfl_xor_sync(0xffffffffu, am, off);
        if (om > mx || (om == mx && oa < am)) {
            mx = om;
            am = oa;
        }
    }
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        v[k] = __expf(v[k] - mx);
        s += v[k];
    }
    for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    const bool ok = r < valid_rows;
    const int y = ok ? label[r] : -1;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
        const int c = lane + 32 * k;
        float g = ok ? (v[k] / s - (c == y ? 1.f : 0.f)) * scale : 0.f;
        dZ[r * kClusters + c] = g;
        dZb[r * kClusters + c] = f2bf(g);
        if (ok && c == y && lane == (y & 31)) {
            atomicAdd(&acc[0], -__logf(fmaxf(v[k] / s, 1e-30f)));
            if (am == y) atomicAdd(&acc[1], 1.f);
        }
    }
}

// T[cols_pad x rows] = M[rows x cols]^T (bf16), rows beyond `cols` zero.
__global__ void transpose_bf16_kernel(const uint16_t* __restrict__ M, int64_t rows, int cols,
                                      int cols_pad, uint16_t* __restrict__ T) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * cols_pad) return;
    const int c = (int)(i / rows);
    const int64_t r = i % rows;
    T[i] = c < cols ? M[r * cols + c] : (uint16_t)0;
}

// dH (fp32) -> dZ = dH * (Zact > 0), kept in place (for the bias sums) and
// as bf16 (for the next GEMMs)
__global__ void relu_grad_kernel(float* __restrict__ dH, const float* __restrict__ Zact, int64_t n,
                                 uint16_t* __restrict__ dZ) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float v = Zact[i] > 0.f ? dH[i] : 0.f;
    dH[i] = v;
    dZ[i] = f2bf(v);
}

// column sums of dZ [rows x cols] into db
__global__ void colsum_kernel(const float* __restrict__ dZ, int64_t rows, int cols, float* __restrict__ db) {
    const int c = blockIdx.x;
    float s = 0.f;
    for (int64_t r = threadIdx.x; r < rows; r += blockDim.x) s += dZ[r * cols + c];
    for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    __shared__ float ws[32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
        db[c] = t;
    }
}

// SGD with momentum on FP32 master weights; refreshes the BF16 copies in
// both orientations (out x in for the forward GEMMs, in x out for dH).
__global__ void sgd_kernel(float* __restrict__ W, float* __restrict__ V, const float* __restrict__ G,
                           int out, int in, int in_pad, float lr, float mom,
                           uint16_t* __restrict__ Wb, uint16_t* __restrict__ WbT, int out_padT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= out * in_pad) return;
    const int o = i / in_pad, k = i % in_pad;
    if (k >= in) {
        Wb[i] = 0;
        return;
    }
    const float g = G[(size_t)o * in_pad + k];
    float v = mom * V[i] + g;
    V[i] = v;
    const float w = W[i] - lr * v;
    W[i] = w;
    const uint16_t h = f2bf(w);
    Wb[i] = h;
    if (WbT) WbT[(size_t)k * out_padT + o] = h;
}

__global__ void sgd_bias_kernel(float* __restrict__ b, float* __restrict__ v, const float* __restrict__ g,
                                int n, float lr, float mom) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float vv = mom * v[i] + g[i];
    v[i] = vv;
    b[i] -= lr * vv;
}

// ------------------------------------------------------------ inference

constexpr int kInferThreads = 128;
constexpr size_t kSmW1 = (size_t)kHidden * kFeat * 2, kSmW2 = (size_t)kHidden * kHidden * 2,
                 kSmW3 = (size_t)kClusters * kHidden * 2, kSmX = 128ull * kFeat * 2,
                 kSmH = 128ull * kHidden * 2;
// H2 reuses the X tile (X is dead once layer 1's MMA has completed), and the
// three layers share 256 TMEM columns (layer 1 at 0, layer 2 at 64, layer 3
// at 0 after both have been read), so two CTAs fit on an SM.
constexpr size_t kInferSmem = kSmW1 + kSmW2 + kSmW3 + kSmX + kSmH + (kHidden * 2 + kClusters) * 4 + 64;
constexpr uint32_t kInferTmemCols = 256;

// Row-major [rows x K] bf16 from global into the core-matrix layout.
__device__ __forceinline__ void stage_rows(uint8_t* dst, const uint16_t* src, int rows, int K) {
    const int kb = K >> 3;
    for (int idx = threadIdx.x; idx < rows * kb; idx += blockDim.x) {
        const int r = idx / kb, g = idx % kb;
        *(uint4*)(dst + core_offset(r, g * 8, K)) = *(const uint4*)(src + (size_t)r * K + g * 8);
    }
}

// Eight values as bf16 into a row's group of a core-matrix tile.
__device__ __forceinline__ void store_group(uint8_t* dst, int r, int g, int cols, const float* v) {
    uint4 w;
    w.x = (uint32_t)f2bf(v[0]) | ((uint32_t)f2bf(v[1]) << 16);
    w.y = (uint32_t)f2bf(v[2]) | ((uint32_t)f2bf(v[3]) << 16);
    w.z = (uint32_t)f2bf(v[4]) | ((uint32_t)f2bf(v[5]) << 16);
    w.w = (uint32_t)f2bf(v[6]) | ((uint32_t)f2bf(v[7]) << 16);
    *(uint4*)(dst + core_offset(r, g, cols)) = w;
}

// A ray's features straight into its row of the X tile, eight at a time.
__device__ __forceinline__ void store_features(uint8_t* dst, int r, float4 o, float4 d, const float* lo,
                                               const float* inv_ext) {
    float buf[8];
    int n = 0, g = 0;
    for_each_feature(o, d, lo, inv_ext, [&](float v) {
        buf[n++] = v;
        if (n == 8) {
            store_group(dst, r, g, kFeat, buf);
            g += 8;
            n = 0;
        }
    });
}

// Bias + ReLU of 64 hidden values read 16 at a time from TMEM (columns
// col..col+63 of this warp's lanes), packed into the row of a bf16 tile.
__device__ __forceinline__ void store_hidden(uint8_t* dst, int r, uint32_t taddr, const float* bias) {
#pragma unroll
    for (int c = 0; c < kHidden; c += 16) {
        float z[16];
        tmem_ld16(taddr + (uint32_t)c, z);
#pragma unroll
        for (int j = 0; j < 16; ++j) z[j] = fmaxf(z[j] + bias[c + j], 0.f);
        store_group(dst, r, c, kHidden, z);
        store_group(dst, r, c + 8, kHidden, z + 8);
    }
}

// Issues one layer: D (TMEM columns dcol..) = A[128 x K] * B[N x K]^T.
__device__ __forceinline__ void issue_layer(uint32_t tbase, uint32_t dcol, const uint8_t* a, const uint8_t* b,
                                            int N, int K, uint64_t* bar) {
    const uint32_t sbo = (uint32_t)(K >> 3) * 128u;
    for (int ks = 0; ks < (K >> 4); ++ks)
        tc_mma(tbase + dcol, smem_desc(a + ks * 256, 128u, sbo), smem_desc(b + ks * 256, 128u, sbo),
               idesc_bf16(128, N), ks > 0 ? 1u : 0u);
    tc_commit(bar);
}

// Fused three-layer forward over 128-ray tiles; pred[i] = arg-max cluster.
__global__ void __launch_bounds__(kInferThreads)
    mlp_infer_kernel(const float4* __restrict__ ro, const float4* __restrict__ rd, int64_t n, LearnBox box,
                     const uint16_t* __restrict__ W1b, const uint16_t* __restrict__ W2b,
                     const uint16_t* __restrict__ W3b, const float* __restrict__ b1,
                     const float* __restrict__ b2, const float* __restrict__ b3, float margin,
                     uint16_t* __restrict__ pred, int* status) {
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t* sW1 = smem;
    uint8_t* sW2 = sW1 + kSmW1;
    uint8_t* sW3 = sW2 + kSmW2;
    uint8_t* sX = sW3 + kSmW3;
    uint8_t* sH1 = sX + kSmX;
    uint8_t* sH2 = sX;
    float* sb1 = (float*)(sH1 + kSmH);
    float* sb2 = sb1 + kHidden;
    float* sb3 = sb2 + kHidden;
    uint64_t* bar = (uint64_t*)(sb3 + kClusters);
    uint32_t* tslot = (uint32_t*)(bar + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) tmem_alloc(tslot, kInferTmemCols);
    stage_rows(sW1, W1b, kHidden, kFeat);
    stage_rows(sW2, W2b, kHidden, kHidden);
    stage_rows(sW3, W3b, kClusters, kHidden);
    for (int k = threadIdx.x; k < kHidden; k += blockDim.x) {
        sb1[k] = b1[k];
        sb2[k] = b2[k];
    }
    for (int k = threadIdx.x; k < kClusters; k += blockDim.x) sb3[k] = b3[k];
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_fence_init();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tbase = *tslot;
    const uint32_t lane_addr = (uint32_t)(warp * 32) << 16;
    const int r = threadIdx.x;
    uint32_t phase = 0;
    bool ok = true;
    for (int64_t tile = blockIdx.x; tile * 128 < n && ok; tile += gridDim.x) {
        const int64_t ray = tile * 128 + r;
        if (ray < n) {
            store_features(sX, r, ro[ray], rd[ray], box.lo, box.inv_ext);
        } else {
            const float zero[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            for (int g = 0; g < kFeat; g += 8) store_group(sX, r, g, kFeat, zero);
        }
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        // layer 1 -> TMEM columns 0..63
        if (threadIdx.x == 0) issue_layer(tbase, 0, sX, sW1, kHidden, kFeat, bar);
        ok = mbar_wait_bounded(bar, phase, status);
        phase ^= 1u;
        tc_fence_after();
        if (!ok) break;
        store_hidden(sH1, r, tbase + lane_addr, sb1);
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        // layer 2 -> columns 64..127
        if (threadIdx.x == 0) issue_layer(tbase, 64, sH1, sW2, kHidden, kHidden, bar);
        ok = mbar_wait_bounded(bar, phase, status);
        phase ^= 1u;
        tc_fence_after();
        if (!ok) break;
        store_hidden(sH2, r, tbase + lane_addr + 64u, sb2);
        fence_proxy_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        // layer 3 -> columns 0..255
        if (threadIdx.x == 0) issue_layer(tbase, 0, sH2, sW3, kClusters, kHidden, bar);
        ok = mbar_wait_bounded(bar, phase, status);
        phase ^= 1u;
        tc_fence_after();
        if (!ok) break;
        float best = -INFINITY, second = -INFINITY;
        int arg = 0;
        for (int c0 = 0; c0 < kClusters; c0 += 16) {
            float z[16];
            tmem_ld16(tbase + lane_addr + (uint32_t)c0, z);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float v = z[j] + sb3[c0 + j];
                if (v > best) {
                    second = best;
                    best = v;
                    arg = c0 + j;
                } else if (v > second) {
                    second = v;
                }
            }
        }
        if (ray < n) pred[ray] = (margin < 0.f || best - second >= margin) ? (uint16_t)arg : kNoCluster;
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }
    if (!ok && threadIdx.x == 0) mbar_wait_bounded(bar, phase ^ 1u, status);
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_free(tbase, kInferTmemCols);
    (void)lane;
}

// ---------------------------------------------------------- host logic

static int upload_params(Learner* L, const std::vector<float>& w1, const std::vector<float>& b1,
                         const std::vector<float>& w2, const std::vector<float>& b2,
                         const std::vector<float>& w3, const std::vector<float>& b3, cudaStream_t st);

// Child references of the BVH cut into up to kClusters subtrees: starting
// from the root's two children, the largest inner subtree is split until
// there are kClusters (or only leaves remain).  record_cluster[pos] = the
// cluster of every record in the tree; records outside it get kClusters.
static void build_clusters(const std::vector<BvhNode>& nodes, int64_t nrec, std::vector<int32_t>* refs,
                           std::vector<uint16_t>* rec_cluster) {
    std::vector<int64_t> count(nodes.size(), 0);
    for (int64_t i = (int64_t)nodes.size() - 1; i >= 0; --i) {  // children have larger indices
        const BvhNode& nd = nodes[(size_t)i];
        int64_t c = 0;
        c += nd.n3.x >= 0 ? count[(size_t)nd.n3.x] : nd.n3.z;
        c += nd.n3.y >= 0 ? count[(size_t)nd.n3.y] : nd.n3.w;
        count[(size_t)i] = c;
    }
    auto size_of = [&](int32_t ref, int32_t leafcnt) { return ref >= 0 ? count[(size_t)ref] : (int64_t)leafcnt; };
    struct Ref { int32_t ref, cnt; };
    std::vector<Ref> fr;
    if (!nodes.empty()) {
        fr.push_back({nodes[0].n3.x, nodes[0].n3.z});
        fr.push_back({nodes[0].n3.y, nodes[0].n3.w});
    }
    while ((int)fr.size() < kClusters) {
        int best = -1;
        int64_t bs = -1;
        for (int k = 0; k < (int)fr.size(); ++k)
            if (fr[k].ref >= 0 && size_of(fr[k].ref, 0) > bs) {
                bs = size_of(fr[k].ref, 0);
                best = k;
            }
        if (best < 0) break;
        const BvhNode& nd = nodes[(size_t)fr[best].ref];
        fr[best] = {nd.n3.x, nd.n3.z};
        fr.push_back({nd.n3.y, nd.n3.w});
    }
    refs->clear();
    rec_cluster->assign((size_t)nrec, (uint16_t)kClusters);
    // unused cluster slots (small trees) hold INT32_MIN: the walk ignores them
    refs->reserve(2 * kClusters);
    for (int k = 0; k < (int)fr.size(); ++k) {
        refs->push_back(fr[k].ref);
        refs->push_back(fr[k].cnt);
        std::vector<int32_t> st;
        if (fr[k].ref < 0) {
            for (int32_t j = 0; j < fr[k].cnt; ++j) (*rec_cluster)[(size_t)(~fr[k].ref + j)] = (uint16_t)k;
            continue;
        }
        st.push_back(fr[k].ref);
        while (!st.empty()) {
            const BvhNode& nd = nodes[(size_t)st.back()];
            st.pop_back();
            const int32_t c[2] = {nd.n3.x, nd.n3.y}, cn[2] = {nd.n3.z, nd.n3.w};
            for (int s = 0; s < 2; ++s) {
                if (c[s] >= 0) st.push_back(c[s]);
                else for (int32_t j = 0; j < cn[s]; ++j) (*rec_cluster)[(size_t)(~c[s] + j)] = (uint16_t)k;
            }
        }
    }
}

void learn_free(Learner* L) {
    if (!L) return;
    DeviceBuffer* all[] = {&L->cluster_ref, &L->record_cluster, &L->W1, &L->W2, &L->W3, &L->V1, &L->V2,
                           &L->V3, &L->b1, &L->b2, &L->b3, &L->vb1, &L->vb2, &L->vb3, &L->W1b, &L->W2b,
                           &L->W3b, &L->W2Tb, &L->W3Tb, &L->recX, &L->recY, &L->X, &L->XT, &L->Z1,
                           &L->Z2, &L->Z3, &L->H1, &L->H2, &L->H1T, &L->H2T, &L->dZ3, &L->dZ3b,
                           &L->dZ3T, &L->dH2, &L->dZ2b, &L->dZ2T, &L->dH1, &L->dZ1b, &L->dZ1T, &L->G1,
                           &L->G2, &L->G3, &L->gb1, &L->gb2, &L->gb3, &L->acc, &L->feat, &L->pred,
                           &L->gemm_work, &L->occ_prim};
    for (DeviceBuffer* b : all) release(*b);
    for (cudaEvent_t e : L->infer_ev) cudaEventDestroy(e);
    for (cudaEvent_t e : L->infer_pool) cudaEventDestroy(e);
    delete L;
}

int ensure_clusters(pbg_scene* s) {
    if (s->accel != PBG_ACCEL_RAYBVH) {
        set_last_error("cluster hints need Accelerator \"ray-bvh\"");
        return PBG_ERR_UNSUPPORTED;
    }
    if (!s->learn) s->learn = new Learner();
    Learner* L = s->learn;
    if (L->clusters_built) return PBG_OK;
    if (s->host_nodes.empty() && s->bvh_nodes > 0) {  // a tree built on the device: the cut is made on the host
        s->host_nodes.resize((size_t)s->bvh_nodes);
        PBG_CUDA(cudaMemcpy(s->host_nodes.data(), s->bvh.ptr, s->host_nodes.size() * sizeof(BvhNode),
                            cudaMemcpyDeviceToHost));
    }
    std::vector<int32_t> refs;
    std::vector<uint16_t> rc16;
    build_clusters(s->host_nodes, s->ntri, &refs, &rc16);
    L->nclusters = (int)(refs.size() / 2);
    while (refs.size() < 2 * (size_t)kClusters) {
        refs.push_back(INT32_MIN);
        refs.push_back(0);
    }
    int rc;
    if ((rc = ensure(L->cluster_ref, refs.size() * 4 + 8)) || (rc = ensure(L->record_cluster, rc16.size() * 2 + 8)))
        return rc;
    if (!refs.empty()) PBG_CUDA(cudaMemcpy(L->cluster_ref.ptr, refs.data(), refs.size() * 4, cudaMemcpyHostToDevice));
    if (!rc16.empty()) PBG_CUDA(cudaMemcpy(L->record_cluster.ptr, rc16.data(), rc16.size() * 2, cudaMemcpyHostToDevice));
    L->clusters_built = true;
    return PBG_OK;
}

__global__ void clusters_of_kernel(const int32_t* __restrict__ prim, int64_t n, const int32_t* __restrict__ pos,
                                   const uint16_t* __restrict__ rec_cluster, uint16_t* __restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t p = prim[i];
    const uint16_t c = p >= 0 ? rec_cluster[pos[p]] : (uint16_t)kNoCluster;
    out[i] = c < kClusters ? c : kNoCluster;
}

int clusters_of(pbg_scene* s, const int32_t* prim, int64_t n, uint16_t* out, cudaStream_t st) {
    int rc = ensure_clusters(s);
    if (rc || n <= 0) return rc;
    clusters_of_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
        prim, n, (const int32_t*)s->tri_pos.ptr, (const uint16_t*)s->learn->record_cluster.ptr, out);
    PBG_CUDA(cudaGetLastError());
    s->counters.kernel_launches += 1;
    return PBG_OK;
}

int learn_init(pbg_scene* s, const pbg_learn_params* p) {
    if (s->accel != PBG_ACCEL_RAYBVH) {
        set_last_error("learned ordering needs Accelerator \"ray-bvh\"");
        return PBG_ERR_UNSUPPORTED;
    }
    Learner* L = s->learn ? s->learn : new Learner();
    s->learn = L;
    if (p) {
        if (p->batch > 0) L->batch = (p->batch + 127) / 128 * 128;
        if (p->steps_per_train > 0) L->steps_per_train = p->steps_per_train;
        if (p->lr > 0.f) L->lr = p->lr;
        if (p->margin != 0.f) L->margin = p->margin;
        if (p->momentum > 0.f) L->momentum = p->momentum;
        if (p->records > 0 && !L->W1.ptr) L->capacity = p->records;  // the ring is sized once
        if (p->seed) L->seed = p->seed;
    }
    if (p && p->queries > 0) L->queries = p->queries & 3;
    if (L->W1.ptr) {  // initialised before: keep the weights and records
        L->enabled = true;
        return PBG_OK;
    }
    if (L->capacity < L->batch) L->capacity = L->batch;
    for (int a = 0; a < 3; ++a) {
        L->box.lo[a] = s->scene_lo[a];
        const float e = s->scene_hi[a] - s->scene_lo[a];
        L->box.inv_ext[a] = e > 0.f ? 1.f / e : 1.f;
    }
    cudaStream_t st = s->stream;
    int rc;
    if ((rc = ensure_clusters(s))) return rc;
    // He-style initialisation from a seeded generator
    uint64_t z = L->seed * 0x9E3779B97F4A7C15ull + 12345;
    auto u01 = [&]() {
        z ^= z >> 12; z ^= z << 25; z ^= z >> 27;
        return (double)((z * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
    };
    auto normal = [&]() { return std::sqrt(-2.0 * std::log(u01() + 1e-300)) * std::cos(6.283185307179586 * u01()); };
    std::vector<float> w1((size_t)kHidden * kFeat, 0.f), w2((size_t)kHidden * kHidden), w3((size_t)kClusters * kHidden);
    std::vector<float> b1(kHidden, 0.f), b2(kHidden, 0.f), b3(kClusters, 0.f);
    for (int o = 0; o < kHidden; ++o)
        for (int k = 0; k < 105; ++k) w1[(size_t)o * kFeat + k] = (float)(normal() * std::sqrt(2.0 / 105));
    for (auto& w : w2) w = (float)(normal() * std::sqrt(2.0 / kHidden));
    for (auto& w : w3) w = (float)(normal() * std::sqrt(1.0 / kHidden));
    if ((rc = upload_params(L, w1, b1, w2, b2, w3, b3, st))) return rc;
    L->enabled = true;
    L->count = L->head = 0;
    if ((rc = ensure(L->acc, 64))) return rc;
    PBG_CUDA(cudaMemset(L->acc.ptr, 0, 64));  // loss, accuracy, batch count, running record total
    L->trained_steps = 0;
    return PBG_OK;
}

// Uploads FP32 parameters, zeroes momentum, refreshes the BF16 copies.
__global__ void to_bf16_kernel(const float* __restrict__ W, int out, int in, uint16_t* __restrict__ Wb,
                               uint16_t* __restrict__ WbT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= out * in) return;
    const int o = i / in, k = i % in;
    const uint16_t h = f2bf(W[i]);
    Wb[i] = h;
    if (WbT) WbT[(size_t)k * out + o] = h;
}

static int upload_params(Learner* L, const std::vector<float>& w1, const std::vector<float>& b1,
                         const std::vector<float>& w2, const std::vector<float>& b2,
                         const std::vector<float>& w3, const std::vector<float>& b3, cudaStream_t st) {
    int rc;
    const size_t n1 = (size_t)kHidden * kFeat, n2 = (size_t)kHidden * kHidden, n3 = (size_t)kClusters * kHidden;
    if ((rc = ensure(L->W1, n1 * 4)) || (rc = ensure(L->W2, n2 * 4)) || (rc = ensure(L->W3, n3 * 4)) ||
        (rc = ensure(L->V1, n1 * 4)) || (rc = ensure(L->V2, n2 * 4)) || (rc = ensure(L->V3, n3 * 4)) ||
        (rc = ensure(L->b1, kHidden * 4)) || (rc = ensure(L->b2, kHidden * 4)) || (rc = ensure(L->b3, kClusters * 4)) ||
        (rc = ensure(L->vb1, kHidden * 4)) || (rc = ensure(L->vb2, kHidden * 4)) || (rc = ensure(L->vb3, kClusters * 4)) ||
        (rc = ensure(L->W1b, n1 * 2)) || (rc = ensure(L->W2b, n2 * 2)) || (rc = ensure(L->W3b, n3 * 2)) ||
        (rc = ensure(L->W2Tb, n2 * 2)) || (rc = ensure(L->W3Tb, n3 * 2)))
        return rc;
    PBG_CUDA(cudaMemcpyAsync(L->W1.ptr, w1.data(), n1 * 4, cudaMemcpyHostToDevice, st));
    PBG_CUDA(cudaMemcpyAsync(L->W2.ptr, w2.data(), n2 * 4, cudaMemcpyHostToDevice, st));
    PBG_CUDA(cudaMemcpyAsync(L->W3.ptr, w3.data(), n3 * 4, cudaMemcpyHostToDevice, st));
    PBG_CUDA(cudaMemcpyAsync(L->b1.ptr, b1.data(), kHidden * 4, cudaMemcpyHostToDevice, st));
    PBG_CUDA(cudaMemcpyAsync(L->b2.ptr, b2.data(), kHidden * 4, cudaMemcpyHostToDevice, st));
    PBG_CUDA(cudaMemcpyAsync(L->b3.ptr, b3.data(), kClusters * 4, cudaMemcpyHostToDevice, st));
    DeviceBuffer* zero[] = {&L->V1, &L->V2, &L->V3, &L->vb1, &L->vb2, &L->vb3};
    for (DeviceBuffer* b : zero) PBG_CUDA(cudaMemsetAsync(b->ptr, 0, b->bytes, st));
    to_bf16_kernel<<<(unsigned)((n1 + 255) / 256), 256, 0, st>>>((const float*)L->W1.ptr, kHidden, kFeat,
                                                                  (uint16_t*)L->W1b.ptr, nullptr);
    to_bf16_kernel<<<(unsigned)((n2 + 255) / 256), 256, 0, st>>>((const float*)L->W2.ptr, kHidden, kHidden,
                                                                  (uint16_t*)L->W2b.ptr, (uint16_t*)L->W2Tb.ptr);
    to_bf16_kernel<<<(unsigned)((n3 + 255) / 256), 256, 0, st>>>((const float*)L->W3.ptr, kClusters, kHidden,
                                                                  (uint16_t*)L->W3b.ptr, (uint16_t*)L->W3Tb.ptr);
    PBG_CUDA(cudaGetLastError());
    PBG_CUDA(cudaStreamSynchronize(st));
    return PBG_OK;
}

// Adds the inference launches' event-pair times to infer_ms and returns the
// events to the pool: all of them (wait_all, when the statistics are read),
// else only the pairs already complete.
static void harvest_infer_events(Learner* L, bool wait_all) {
    size_t k = 0;
    for (; k + 1 < L->infer_ev.size(); k += 2) {
        if (wait_all) {
            if (cudaEventSynchronize(L->infer_ev[k + 1]) != cudaSuccess) break;
        } else if (cudaEventQuery(L->infer_ev[k + 1]) != cudaSuccess) {
            cudaGetLastError();  // cudaErrorNotReady is not an error here
            break;
        }
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, L->infer_ev[k], L->infer_ev[k + 1]) == cudaSuccess) L->infer_ms += ms;
        L->infer_pool.push_back(L->infer_ev[k]);
        L->infer_pool.push_back(L->infer_ev[k + 1]);
    }
    L->infer_ev.erase(L->infer_ev.begin(), L->infer_ev.begin() + (std::ptrdiff_t)k);
}

int learn_predict(pbg_scene* s, const float4* o, const float4* d, int64_t n, const uint16_t** pred,
                  const int32_t** cluster_ref, cudaStream_t st) {
    Learner* L = s->learn;
    *pred = nullptr;
    if (!L || !L->enabled || L->trained_steps == 0 || n <= 0) return PBG_OK;
    int rc = ensure(L->pred, (size_t)n * 2);
    if (rc) return rc;
    // a per-device setting (cheap, idempotent): set on every call so that each
    // device the library launches on has it
    PBG_CUDA(cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem));
    int sms = 152;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
    const int64_t tiles = (n + 127) / 128;
    const unsigned grid = (unsigned)std::min<int64_t>(tiles, 2 * (int64_t)sms);  // two CTAs per SM
    if (L->infer_ev.size() >= 256) harvest_infer_events(L, false);  // keep the list short
    cudaEvent_t ev[2];
    for (cudaEvent_t& e : ev) {
        if (!L->infer_pool.empty()) {
            e = L->infer_pool.back();
            L->infer_pool.pop_back();
        } else {
            PBG_CUDA(cudaEventCreate(&e));
        }
    }
    PBG_CUDA(cudaEventRecord(ev[0], st));
    prof_begin(s, st);
    mlp_infer_kernel<<<grid, kInferThreads, kInferSmem, st>>>(
        o, d, n, L->box, (const uint16_t*)L->W1b.ptr, (const uint16_t*)L->W2b.ptr, (const uint16_t*)L->W3b.ptr,
        (const float*)L->b1.ptr, (const float*)L->b2.ptr, (const float*)L->b3.ptr, L->margin,
        (uint16_t*)L->pred.ptr, (int*)s->err.ptr);
    prof_end(s, st, kStageOther, 1);
    PBG_CUDA(cudaGetLastError());
    PBG_CUDA(cudaEventRecord(ev[1], st));
    L->infer_ev.push_back(ev[0]);
    L->infer_ev.push_back(ev[1]);
    *pred = (const uint16_t*)L->pred.ptr;
    *cluster_ref = (const int32_t*)L->cluster_ref.ptr;
    return PBG_OK;
}

// Appends up to `take` records: rays that hit, their features and the
// cluster of the record they hit.  Picks every stride-th hit.
__global__ void collect_kernel(const float4* __restrict__ ro, const float4* __restrict__ rd,
                               const int32_t* __restrict__ prim, const int32_t* __restrict__ pos,
                               const uint16_t* __restrict__ rec_cluster, int64_t n, int64_t stride,
                               LearnBox box, uint16_t* __restrict__ recX, int32_t* __restrict__ recY,
                               int64_t cap, const unsigned long long* __restrict__ total,
                               unsigned int* __restrict__ taken, int64_t take) {
    const int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * stride;
    if (i >= n) return;
    const int32_t p = prim[i];
    if (p < 0) return;
    const uint16_t c = rec_cluster[pos[p]];
    if (c >= kClusters) return;
    const unsigned int k = atomicAdd(taken, 1u);
    if ((int64_t)k >= take) return;
    const int64_t slot = (int64_t)((*total + k) % (unsigned long long)cap);
    float f[kFeat];
    ray_features(ro[i], rd[i], box.lo, box.inv_ext, f);
    uint16_t* row = recX + slot * kFeat;
    for (int j = 0; j < kFeat; ++j) row[j] = f2bf(f[j]);
    recY[slot] = c;
}

// The ring's running total advances by this batch's records (stream order:
// the next batch's collect_kernel sees the new total).
__global__ void collect_advance_kernel(unsigned long long* total, const unsigned int* taken, int64_t take) {
    *total += (unsigned long long)min((int64_t)*taken, take);
}

// Records are written and counted on the device; the host reads the count
// only when it trains (learn_train), so collecting never stalls the stream.
int learn_collect(pbg_scene* s, const float4* o, const float4* d, const int32_t* prim, int64_t n,
                  cudaStream_t st) {
    Learner* L = s->learn;
    if (!L || !L->enabled || n <= 0) return PBG_OK;
    int rc;
    if ((rc = ensure(L->recX, (size_t)L->capacity * kFeat * 2)) || (rc = ensure(L->recY, (size_t)L->capacity * 4)) ||
        (rc = ensure(L->acc, 64)))
        return rc;
    const int64_t take = std::min<int64_t>(L->capacity / 4, n);
    const int64_t stride = std::max<int64_t>(1, n / std::max<int64_t>(take, 1));
    PBG_CUDA(cudaMemsetAsync((uint8_t*)L->acc.ptr + 32, 0, 4, st));
    const int64_t threads = (n + stride - 1) / stride;
    collect_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(
        o, d, prim, (const int32_t*)s->tri_pos.ptr, (const uint16_t*)L->record_cluster.ptr, n, stride, L->box,
        (uint16_t*)L->recX.ptr, (int32_t*)L->recY.ptr, L->capacity,
        (const unsigned long long*)((uint8_t*)L->acc.ptr + 40), (unsigned int*)((uint8_t*)L->acc.ptr + 32), take);
    PBG_CUDA(cudaGetLastError());
    collect_advance_kernel<<<1, 1, 0, st>>>((unsigned long long*)((uint8_t*)L->acc.ptr + 40),
                                            (const unsigned int*)((uint8_t*)L->acc.ptr + 32), take);
    PBG_CUDA(cudaGetLastError());
    s->counters.kernel_launches += 2;
    return PBG_OK;
}

// Records collected so far (a synchronising read of the device total).
static int records_available(Learner* L, cudaStream_t st) {
    unsigned long long total = 0;
    if (L->acc.ptr) {
        PBG_CUDA(cudaMemcpyAsync(&total, (uint8_t*)L->acc.ptr + 40, 8, cudaMemcpyDeviceToHost, st));
        PBG_CUDA(cudaStreamSynchronize(st));
    }
    L->count = (int64_t)std::min<unsigned long long>((unsigned long long)L->capacity, total);
    return PBG_OK;
}

// One forward + backward pass on B rows of X (bf16 [B x 112]) with labels
// Y; gradients into G1/G2/G3, gb1/gb2/gb3 (FP32); loss / correct in acc.
// tc_gemm with its launches counted: the GEMM, and the split-K reduction
// when a work buffer spreads K over slices.
static int gemm(pbg_scene* s, const uint16_t* A, const uint16_t* B, float* C, int M, int N, int K, int acc,
                int* status, cudaStream_t st, float* work) {
    const int rc = tc_gemm(A, B, C, M, N, K, acc, status, st, work);
    if (rc == PBG_OK)
        s->counters.kernel_launches += 1 + (work && tc_gemm_work_floats(M, N, K) > (size_t)M * (size_t)N ? 1 : 0);
    return rc;
}

static int forward_backward(pbg_scene* s, Learner* L, const uint16_t* X, const int32_t* Y, int B,
                            cudaStream_t st) {
    int* status = (int*)s->err.ptr;
    int rc;
    const size_t b = (size_t)B;
    if ((rc = ensure(L->XT, b * kFeat * 2)) || (rc = ensure(L->Z1, b * kHidden * 4)) ||
        (rc = ensure(L->Z2, b * kHidden * 4)) || (rc = ensure(L->Z3, b * kClusters * 4)) ||
        (rc = ensure(L->H1, b * kHidden * 2)) || (rc = ensure(L->H2, b * kHidden * 2)) ||
        (rc = ensure(L->H1T, b * kHidden * 2)) || (rc = ensure(L->H2T, b * kHidden * 2)) ||
        (rc = ensure(L->dZ3, b * kClusters * 4)) || (rc = ensure(L->dZ3b, b * kClusters * 2)) ||
        (rc = ensure(L->dZ3T, b * kClusters * 2)) || (rc = ensure(L->dH2, b * kHidden * 4)) ||
        (rc = ensure(L->dZ2b, b * kHidden * 2)) || (rc = ensure(L->dZ2T, b * 128 * 2)) ||
        (rc = ensure(L->dH1, b * kHidden * 4)) || (rc = ensure(L->dZ1b, b * kHidden * 2)) ||
        (rc = ensure(L->dZ1T, b * 128 * 2)) || (rc = ensure(L->G1, 128 * kFeat * 4)) ||
        (rc = ensure(L->G2, 128 * kHidden * 4)) || (rc = ensure(L->G3, kClusters * kHidden * 4)) ||
        (rc = ensure(L->gb1, kHidden * 4)) || (rc = ensure(L->gb2, kHidden * 4)) ||
        (rc = ensure(L->gb3, kClusters * 4)) || (rc = ensure(L->acc, 64)))
        return rc;
    {  // split-K workspace of the weight gradients (K = the batch)
        const size_t wf = std::max({tc_gemm_work_floats(kClusters, kHidden, B),
                                    tc_gemm_work_floats(128, kHidden, B), tc_gemm_work_floats(128, kFeat, B)});
        if ((rc = ensure(L->gemm_work, wf * 4))) return rc;
    }
    auto blocks = [](size_t n) { return (unsigned)((n + 255) / 256); };
    // forward
    if ((rc = gemm(s, X, (const uint16_t*)L->W1b.ptr, (float*)L->Z1.ptr, B, kHidden, kFeat, 0, status, st, nullptr))) return rc;
    bias_relu_kernel<<<blocks(b * kHidden), 256, 0, st>>>((float*)L->Z1.ptr, (const float*)L->b1.ptr, B, kHidden, 1,
                                                           (uint16_t*)L->H1.ptr);
    if ((rc = gemm(s, (const uint16_t*)L->H1.ptr, (const uint16_t*)L->W2b.ptr, (float*)L->Z2.ptr, B, kHidden,
                      kHidden, 0, status, st, nullptr))) return rc;
    bias_relu_kernel<<<blocks(b * kHidden), 256, 0, st>>>((float*)L->Z2.ptr, (const float*)L->b2.ptr, B, kHidden, 1,
                                                           (uint16_t*)L->H2.ptr);
    if ((rc = gemm(s, (const uint16_t*)L->H2.ptr, (const uint16_t*)L->W3b.ptr, (float*)L->Z3.ptr, B, kClusters,
                      kHidden, 0, status, st, nullptr))) return rc;
    bias_relu_kernel<<<blocks(b * kClusters), 256, 0, st>>>((float*)L->Z3.ptr, (const float*)L->b3.ptr, B,
                                                             kClusters, 0, nullptr);
    PBG_CUDA(cudaMemsetAsync(L->acc.ptr, 0, 8, st));
    softmax_grad_kernel<<<(unsigned)((b * 32 + 255) / 256), 256, 0, st>>>(
        (const float*)L->Z3.ptr, Y, B, B, 1.f / (float)B, (float*)L->dZ3.ptr, (uint16_t*)L->dZ3b.ptr,
        (float*)L->acc.ptr);
    // backward: dW3 = dZ3^T H2
    transpose_bf16_kernel<<<blocks(b * kClusters), 256, 0, st>>>((const uint16_t*)L->dZ3b.ptr, B, kClusters,
                                                                  kClusters, (uint16_t*)L->dZ3T.ptr);
    transpose_bf16_kernel<<<blocks(b * kHidden), 256, 0, st>>>((const uint16_t*)L->H2.ptr, B, kHidden, kHidden,
                                                                (uint16_t*)L->H2T.ptr);
    if ((rc = gemm(s, (const uint16_t*)L->dZ3T.ptr, (const uint16_t*)L->H2T.ptr, (float*)L->G3.ptr, kClusters,
                      kHidden, B, 0, status, st, (float*)L->gemm_work.ptr))) return rc;
    colsum_kernel<<<kClusters, 256, 0, st>>>((const float*)L->dZ3.ptr, B, kClusters, (float*)L->gb3.ptr);
    // dH2 = dZ3 W3 ; dZ2 = dH2 * relu'
    if ((rc = gemm(s, (const uint16_t*)L->dZ3b.ptr, (const uint16_t*)L->W3Tb.ptr, (float*)L->dH2.ptr, B, kHidden,
                      kClusters, 0, status, st, nullptr))) return rc;
    relu_grad_kernel<<<blocks(b * kHidden), 256, 0, st>>>((float*)L->dH2.ptr, (const float*)L->Z2.ptr, b * kHidden,
                                                           (uint16_t*)L->dZ2b.ptr);
    colsum_kernel<<<kHidden, 256, 0, st>>>((const float*)L->dH2.ptr, B, kHidden, (float*)L->gb2.ptr);
    // dW2 = dZ2^T H1 (rows padded to 128)
    transpose_bf16_kernel<<<blocks(b * 128), 256, 0, st>>>((const uint16_t*)L->dZ2b.ptr, B, kHidden, 128,
                                                            (uint16_t*)L->dZ2T.ptr);
    transpose_bf16_kernel<<<blocks(b * kHidden), 256, 0, st>>>((const uint16_t*)L->H1.ptr, B, kHidden, kHidden,
                                                                (uint16_t*)L->H1T.ptr);
    if ((rc = gemm(s, (const uint16_t*)L->dZ2T.ptr, (const uint16_t*)L->H1T.ptr, (float*)L->G2.ptr, 128, kHidden,
                      B, 0, status, st, (float*)L->gemm_work.ptr))) return rc;
    // dH1 = dZ2 W2 ; dZ1 = dH1 * relu'
    if ((rc = gemm(s, (const uint16_t*)L->dZ2b.ptr, (const uint16_t*)L->W2Tb.ptr, (float*)L->dH1.ptr, B, kHidden,
                      kHidden, 0, status, st, nullptr))) return rc;
    relu_grad_kernel<<<blocks(b * kHidden), 256, 0, st>>>((float*)L->dH1.ptr, (const float*)L->Z1.ptr, b * kHidden,
                                                           (uint16_t*)L->dZ1b.ptr);
    colsum_kernel<<<kHidden, 256, 0, st>>>((const float*)L->dH1.ptr, B, kHidden, (float*)L->gb1.ptr);
    // dW1 = dZ1^T X (rows padded to 128)
    transpose_bf16_kernel<<<blocks(b * 128), 256, 0, st>>>((const uint16_t*)L->dZ1b.ptr, B, kHidden, 128,
                                                            (uint16_t*)L->dZ1T.ptr);
    transpose_bf16_kernel<<<blocks(b * kFeat), 256, 0, st>>>(X, B, kFeat, kFeat, (uint16_t*)L->XT.ptr);
    if ((rc = gemm(s, (const uint16_t*)L->dZ1T.ptr, (const uint16_t*)L->XT.ptr, (float*)L->G1.ptr, 128, kFeat, B,
                      0, status, st, (float*)L->gemm_work.ptr))) return rc;
    PBG_CUDA(cudaGetLastError());
    s->counters.kernel_launches += 15;  // bias/ReLU 3, softmax 1, transposes 6, column sums 3, ReLU grads 2
    return PBG_OK;
}

static int sgd_update(Learner* L, cudaStream_t st) {
    const float lr = L->lr, m = L->momentum;
    auto blocks = [](size_t n) { return (unsigned)((n + 255) / 256); };
    sgd_kernel<<<blocks(kHidden * kFeat), 256, 0, st>>>((float*)L->W1.ptr, (float*)L->V1.ptr, (const float*)L->G1.ptr,
                                                         kHidden, 105, kFeat, lr, m, (uint16_t*)L->W1b.ptr, nullptr, 0);
    sgd_kernel<<<blocks(kHidden * kHidden), 256, 0, st>>>((float*)L->W2.ptr, (float*)L->V2.ptr,
                                                           (const float*)L->G2.ptr, kHidden, kHidden, kHidden, lr, m,
                                                           (uint16_t*)L->W2b.ptr, (uint16_t*)L->W2Tb.ptr, kHidden);
    sgd_kernel<<<blocks(kClusters * kHidden), 256, 0, st>>>((float*)L->W3.ptr, (float*)L->V3.ptr,
                                                             (const float*)L->G3.ptr, kClusters, kHidden, kHidden, lr,
                                                             m, (uint16_t*)L->W3b.ptr, (uint16_t*)L->W3Tb.ptr,
                                                             kClusters);
    sgd_bias_kernel<<<1, kHidden, 0, st>>>((float*)L->b1.ptr, (float*)L->vb1.ptr, (const float*)L->gb1.ptr, kHidden, lr, m);
    sgd_bias_kernel<<<1, kHidden, 0, st>>>((float*)L->b2.ptr, (float*)L->vb2.ptr, (const float*)L->gb2.ptr, kHidden, lr, m);
    sgd_bias_kernel<<<1, kClusters, 0, st>>>((float*)L->b3.ptr, (float*)L->vb3.ptr, (const float*)L->gb3.ptr, kClusters, lr, m);
    PBG_CUDA(cudaGetLastError());
    return PBG_OK;
}

int learn_train(pbg_scene* s, int steps, cudaStream_t st) {
    Learner* L = s->learn;
    if (!L || !L->enabled) return PBG_OK;
    if (steps <= 0) steps = L->steps_per_train;
    int rc0 = records_available(L, st);
    if (rc0) return rc0;
    if (L->count < L->batch) return PBG_OK;  // not enough records yet
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    const int64_t nb = L->count / L->batch;
    int rc = PBG_OK;
    for (int k = 0; k < steps && rc == PBG_OK; ++k) {
        const int64_t start = ((int64_t)(L->trained_steps % (uint64_t)nb)) * L->batch;
        const uint16_t* X = (const uint16_t*)L->recX.ptr + start * kFeat;
        const int32_t* Y = (const int32_t*)L->recY.ptr + start;
        rc = forward_backward(s, L, X, Y, L->batch, st);
        if (rc == PBG_OK) rc = sgd_update(L, st);
        if (rc == PBG_OK) s->counters.kernel_launches += 6;
        ++L->trained_steps;
    }
    cudaEventRecord(e1, st);
    float acc[2] = {0.f, 0.f};
    cudaMemcpyAsync(acc, L->acc.ptr, 8, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    L->train_ms += ms;
    L->last_loss = acc[0] / (float)L->batch;
    L->last_acc = acc[1] / (float)L->batch;
    if (rc) return rc;
    return check_device_status(s, st);
}

}  // namespace pbg

using namespace pbg;

extern "C" {

int pbg_learn_enable(pbg_scene* s, int32_t on, const pbg_learn_params* p) {
    if (!s) return PBG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->device);
    if (!on) {
        if (s->learn) s->learn->enabled = false;
        return PBG_OK;
    }
    return learn_init(s, p);
}

int pbg_learn_train(pbg_scene* s, int32_t steps) {
    if (!s) return PBG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->device);
    return learn_train(s, steps, s->stream);
}

int pbg_learn_get_stats(pbg_scene* s, pbg_learn_stats* out) {
    if (!s || !out) return PBG_ERR_INVALID_ARGUMENT;
    Learner* L = s->learn;
    memset(out, 0, sizeof(*out));
    if (!L) return PBG_OK;
    cudaSetDevice(s->device);
    int rc = records_available(L, s->stream);
    if (rc) return rc;
    out->trained_steps = L->trained_steps;
    out->records = (uint64_t)L->count;
    out->last_loss = L->last_loss;
    out->last_accuracy = L->last_acc;
    harvest_infer_events(L, true);
    out->infer_ms = L->infer_ms;
    out->train_ms = L->train_ms;
    return PBG_OK;
}

int pbg_learn_params_io(pbg_scene* s, float* params, int32_t get) {
    if (!s || !params || !s->learn) return PBG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->device);
    Learner* L = s->learn;
    const size_t n1 = (size_t)kHidden * kFeat, n2 = (size_t)kHidden * kHidden, n3 = (size_t)kClusters * kHidden;
    float* p = params;
    if (get) {
        PBG_CUDA(cudaMemcpy(p, L->W1.ptr, n1 * 4, cudaMemcpyDeviceToHost)); p += n1;
        PBG_CUDA(cudaMemcpy(p, L->b1.ptr, kHidden * 4, cudaMemcpyDeviceToHost)); p += kHidden;
        PBG_CUDA(cudaMemcpy(p, L->W2.ptr, n2 * 4, cudaMemcpyDeviceToHost)); p += n2;
        PBG_CUDA(cudaMemcpy(p, L->b2.ptr, kHidden * 4, cudaMemcpyDeviceToHost)); p += kHidden;
        PBG_CUDA(cudaMemcpy(p, L->W3.ptr, n3 * 4, cudaMemcpyDeviceToHost)); p += n3;
        PBG_CUDA(cudaMemcpy(p, L->b3.ptr, kClusters * 4, cudaMemcpyDeviceToHost));
        return PBG_OK;
    }
    std::vector<float> w1(p, p + n1); p += n1;
    std::vector<float> b1(p, p + kHidden); p += kHidden;
    std::vector<float> w2(p, p + n2); p += n2;
    std::vector<float> b2(p, p + kHidden); p += kHidden;
    std::vector<float> w3(p, p + n3); p += n3;
    std::vector<float> b3(p, p + kClusters);
    return upload_params(L, w1, b1, w2, b2, w3, b3, s->stream);
}

int pbg_learn_gradients(pbg_scene* s, const float* x, const int32_t* labels, int32_t B, float* grads,
                        float* loss) {
    if (!s || !x || !labels || !grads || B <= 0 || B % 128 || !s->learn) return PBG_ERR_INVALID_ARGUMENT;
    cudaSetDevice(s->device);
    Learner* L = s->learn;
    cudaStream_t st = s->stream;
    std::vector<uint16_t> xb((size_t)B * kFeat);
    for (size_t i = 0; i < xb.size(); ++i) {
        uint32_t u;
        memcpy(&u, &x[i], 4);
        u += 0x7FFFu + ((u >> 16) & 1u);
        xb[i] = (uint16_t)(u >> 16);
    }
    int rc;
    if ((rc = ensure(L->X, xb.size() * 2)) || (rc = ensure(L->feat, (size_t)B * 4))) return rc;
    PBG_CUDA(cudaMemcpyAsync(L->X.ptr, xb.data(), xb.size() * 2, cudaMemcpyHostToDevice, st));
    PBG_CUDA(cudaMemcpyAsync(L->feat.ptr, labels, (size_t)B * 4, cudaMemcpyHostToDevice, st));
    if ((rc = forward_backward(s, L, (const uint16_t*)L->X.ptr, (const int32_t*)L->feat.ptr, B, st))) return rc;
    const size_t n1 = (size_t)kHidden * kFeat, n2 = (size_t)kHidden * kHidden, n3 = (size_t)kClusters * kHidden;
    float* g = grads;
    PBG_CUDA(cudaMemcpyAsync(g, L->G1.ptr, n1 * 4, cudaMemcpyDeviceToHost, st)); g += n1;  // first 64 rows
    PBG_CUDA(cudaMemcpyAsync(g, L->gb1.ptr, kHidden * 4, cudaMemcpyDeviceToHost, st)); g += kHidden;
    PBG_CUDA(cudaMemcpyAsync(g, L->G2.ptr, n2 * 4, cudaMemcpyDeviceToHost, st)); g += n2;
    PBG_CUDA(cudaMemcpyAsync(g, L->gb2.ptr, kHidden * 4, cudaMemcpyDeviceToHost, st)); g += kHidden;
    PBG_CUDA(cudaMemcpyAsync(g, L->G3.ptr, n3 * 4, cudaMemcpyDeviceToHost, st)); g += n3;
    PBG_CUDA(cudaMemcpyAsync(g, L->gb3.ptr, kClusters * 4, cudaMemcpyDeviceToHost, st));
    float acc[2];
    PBG_CUDA(cudaMemcpyAsync(acc, L->acc.ptr, 8, cudaMemcpyDeviceToHost, st));
    PBG_CUDA(cudaStreamSynchronize(st));
    if (loss) *loss = acc[0] / (float)B;
    return check_device_status(s, st);
}

}  // extern "C"
