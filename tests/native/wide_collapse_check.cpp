// CPU check of the eight-wide collapse (collapse_wide, exported by the
// library): for a scene read from argv[1] (float[9*n] triangles) it builds
// the two-wide tree on the host cores, collapses it, and checks that
//   * the record map is a permutation of the triangle records,
//   * every node's children fit the format (inner children contiguous and
//     in range, leaf masks inside the node's 32 records),
//   * every record that a ray reaches through the two-wide tree (its slab
//     test, maxt = inf) it also reaches through the wide tree, for seeded
//     rays (axis-parallel and negative-zero directions included).
// Prints "ok <wide nodes> <binary nodes> <wide visits per ray> <binary
// visits per ray>" and exits 0, or the first failure and exits 1.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "pbg_wide.cuh"

using namespace pbg;

namespace {

float safe_inv(float d) {
    const float r = 1.f / d;
    return std::isfinite(r) ? r : std::copysign(1e30f, d);
}

struct Ray {
    float ox, oy, oz, ix, iy, iz;
};

// the walks' slab test (min/max form), maxt = inf, mint = 0
bool slab(const Ray& r, float lx, float hx, float ly, float hy, float lz, float hz) {
    const float tx0 = (lx - r.ox) * r.ix, tx1 = (hx - r.ox) * r.ix;
    const float ty0 = (ly - r.oy) * r.iy, ty1 = (hy - r.oy) * r.iy;
    const float tz0 = (lz - r.oz) * r.iz, tz1 = (hz - r.oz) * r.iz;
    const float tn = std::fmax(std::fmax(std::fmin(tx0, tx1), std::fmin(ty0, ty1)), std::fmax(std::fmin(tz0, tz1), 0.f));
    const float tf = std::fmin(std::fmin(std::fmax(tx0, tx1), std::fmax(ty0, ty1)), std::fmin(std::fmax(tz0, tz1), INFINITY));
    return tn <= std::fma(std::fabs(tf), 2.f * 3.f * 0x1p-24f / (1.f - 3.f * 0x1p-24f), tf);
}

long reach_binary(const std::vector<BvhNode>& nodes, const Ray& r, std::vector<char>& mark) {
    long visits = 0;
    std::vector<int> st{0};
    while (!st.empty()) {
        const BvhNode& b = nodes[(size_t)st.back()];
        st.pop_back();
        ++visits;
        for (int c = 0; c < 2; ++c) {
            const float4 bx = c ? b.n1 : b.n0;
            const float lz = c ? b.n2.z : b.n2.x, hz = c ? b.n2.w : b.n2.y;
            const int ref = c ? b.n3.y : b.n3.x, cnt = c ? b.n3.w : b.n3.z;
            if ((ref < 0 && cnt == 0) || !slab(r, bx.x, bx.y, bx.z, bx.w, lz, hz)) continue;
            if (ref >= 0) st.push_back(ref);
            else
                for (int k = 0; k < cnt; ++k) mark[(size_t)(~ref + k)] = 1;
        }
    }
    return visits;
}

long reach_wide(const std::vector<WideNode>& wn, const std::vector<int32_t>& src, const Ray& r,
                std::vector<char>& mark) {
    long visits = 0;
    std::vector<int> st{0};
    while (!st.empty()) {
        const WideNode& w = wn[(size_t)st.back()];
        st.pop_back();
        ++visits;
        const float* pl = reinterpret_cast<const float*>(w.plane);
        const uint32_t* tm = reinterpret_cast<const uint32_t*>(w.tris);
        const uint32_t imask = (uint32_t)w.refs.x >> 24;
        const int base = w.refs.x & 0xffffff;
        int rank = 0;
        for (int k = 0; k < 8; ++k) {
            const bool hit = slab(r, pl[k], pl[8 + k], pl[16 + k], pl[24 + k], pl[32 + k], pl[40 + k]);
            if (imask >> k & 1) {
                if (hit) st.push_back(base + rank);
                ++rank;
            } else if (hit) {
                for (int q = 0; q < 32; ++q)
                    if (tm[k] >> q & 1) mark[(size_t)src[(size_t)(w.refs.y + q)]] = 1;
            }
        }
    }
    return visits;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 2;
    std::vector<float> t;
    float buf[9];
    while (fread(buf, sizeof(float), 9, f) == 9) t.insert(t.end(), buf, buf + 9);
    fclose(f);
    const int64_t n = (int64_t)(t.size() / 9);
    const int rays = atoi(argv[2]);
    HostBvh hb;
    build_bvh(t.data(), n, 4, &hb);
    std::vector<WideNode> wn;
    std::vector<int32_t> src;
    if (!collapse_wide(hb.nodes, hb.unculled, n, kWideAbsorb, kWideTriCost, &wn, &src)) {
        printf("collapse refused the tree\n");
        return 1;
    }
    std::vector<int> seen((size_t)n, 0);
    for (int32_t x : src) {
        if (x < 0 || x >= n) {
            printf("record map out of range: %d\n", x);
            return 1;
        }
        seen[(size_t)x]++;
    }
    for (int64_t i = 0; i < n; ++i)
        if (seen[(size_t)i] != 1) {
            printf("record %ld mapped %d times\n", (long)i, seen[(size_t)i]);
            return 1;
        }
    for (size_t i = 0; i < wn.size(); ++i) {
        const uint32_t imask = (uint32_t)wn[i].refs.x >> 24;
        const int64_t base = wn[i].refs.x & 0xffffff;
        if (imask && (base <= (int64_t)i || base + __builtin_popcount(imask) > (int64_t)wn.size())) {
            printf("node %zu: inner children out of range\n", i);
            return 1;
        }
        const uint32_t* tm = reinterpret_cast<const uint32_t*>(wn[i].tris);
        for (int k = 0; k < 8; ++k)
            if (tm[k] && (imask >> k & 1)) {
                printf("node %zu slot %d: inner and leaf\n", i, k);
                return 1;
            }
    }
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = 0; i < t.size(); ++i) {
        lo[i % 3] = std::fmin(lo[i % 3], t[i]);
        hi[i % 3] = std::fmax(hi[i % 3], t[i]);
    }
    std::mt19937 g(7);
    std::uniform_real_distribution<float> u(0.f, 1.f);
    std::normal_distribution<float> nd;
    std::vector<char> mb((size_t)n), mw((size_t)n);
    long vb = 0, vw = 0;
    for (int i = 0; i < rays; ++i) {
        float o[3], d[3];
        for (int a = 0; a < 3; ++a) {
            o[a] = lo[a] + (hi[a] - lo[a]) * u(g);
            d[a] = nd(g);
        }
        if (i % 7 == 0) d[i % 3] = 0.f;
        if (i % 11 == 0) d[(i + 1) % 3] = -0.f;
        const Ray r{o[0], o[1], o[2], safe_inv(d[0]), safe_inv(d[1]), safe_inv(d[2])};
        std::fill(mb.begin(), mb.end(), 0);
        std::fill(mw.begin(), mw.end(), 0);
        vb += reach_binary(hb.nodes, r, mb);
        vw += reach_wide(wn, src, r, mw);
        for (int64_t k = 0; k < n; ++k)
            if (mb[(size_t)k] && !mw[(size_t)k]) {
                printf("ray %d reaches record %ld through the two-wide tree only\n", i, (long)k);
                return 1;
            }
    }
    printf("ok %zu %zu %.2f %.2f\n", wn.size(), hb.nodes.size(), (double)vw / rays, (double)vb / rays);
    return 0;
}
