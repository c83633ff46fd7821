// pbg_learn.h -- state of the learned traversal ordering (see pbg_learn.cu).
#pragma once
#include <cstdint>
#include <vector>

#include "pbg_internal.h"

namespace pbg {

constexpr int kFeat = 112;      // 105 features padded to a multiple of 16
constexpr int kHidden = 64;
constexpr int kClusters = 256;

struct LearnBox {
    float lo[3], inv_ext[3];
};

// Device buffers of one learner.  W*: FP32 master weights [out x in_pad],
// V*: momentum, Wb*: BF16 [out x in_pad] (forward), WTb*: BF16 [in x out]
// (backward dH), b*: biases.
struct Learner {
    bool enabled = false;
    int batch = 8192;
    int steps_per_train = 8;
    float lr = 0.05f, momentum = 0.9f;
    float margin = 1.0f;  // logit lead of the top cluster needed to use it
    int64_t capacity = 1 << 18;  // training records kept (ring)
    int64_t count = 0, head = 0;
    uint64_t trained_steps = 0;
    uint64_t seed = 1;
    LearnBox box{};
    int queries = 3;  // 1: nearest-hit batches, 2: any-hit batches, 3: both
    // clusters of the BVH: child references and per-record cluster ids (built
    // once, also for caller-supplied hints without a trained network)
    DeviceBuffer cluster_ref, record_cluster;
    int nclusters = 0;
    bool clusters_built = false;
    DeviceBuffer occ_prim;  // any-hit batches: the occluder each walk found
    // parameters
    DeviceBuffer W1, W2, W3, V1, V2, V3, b1, b2, b3, vb1, vb2, vb3, W1b, W2b, W3b, W2Tb, W3Tb;
    // training scratch
    DeviceBuffer recX, recY, X, XT, Z1, Z2, Z3, H1, H2, H1T, H2T, dZ3, dZ3b, dZ3T, dH2, dZ2b, dZ2T,
        dH1, dZ1b, dZ1T, G1, G2, G3, gb1, gb2, gb3, acc, gemm_work;
    // per-batch inference scratch
    DeviceBuffer feat, pred;
    float last_loss = 0.f, last_acc = 0.f;
    double infer_ms = 0.0, train_ms = 0.0;
    // event pairs around inference launches, summed into infer_ms when the
    // statistics are read (no synchronisation on the launch path)
    std::vector<cudaEvent_t> infer_ev, infer_pool;
};

int learn_init(pbg_scene* s, const pbg_learn_params* p);
// The cluster tables (kClusters subtrees of the BVH) without a network.
int ensure_clusters(pbg_scene* s);
// out[i] = the cluster of triangle prim[i] (kNoCluster for -1 or a triangle
// outside the clusters).  Device arrays.
int clusters_of(pbg_scene* s, const int32_t* prim, int64_t n, uint16_t* out, cudaStream_t st);
void learn_free(Learner* L);
// Predicted cluster per ray for the batch (NULL when the learner is off or
// untrained; kNoCluster for a ray whose prediction is not confident);
// *cluster_ref receives the device table of cluster references.
constexpr uint16_t kNoCluster = 0xffffu;
int learn_predict(pbg_scene* s, const float4* o, const float4* d, int64_t n, const uint16_t** pred,
                  const int32_t** cluster_ref, cudaStream_t st);
// Appends training records (features + the cluster of prim[i]) from a
// finished batch: first hits of nearest-hit rays, occluders of any-hit rays.
int learn_collect(pbg_scene* s, const float4* o, const float4* d, const int32_t* prim, int64_t n,
                  cudaStream_t st);
int learn_train(pbg_scene* s, int steps, cudaStream_t st);

}  // namespace pbg
