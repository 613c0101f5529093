// cluster.cpp - spatial clusters of emitters for the learned candidate proposal.
//
// Seeded k-means over light centres (no reference counterpart). Initial centres are k
// distinct lights drawn by a seeded hash; Lloyd iterations assign every light to the
// nearest centre (ties to the lower cluster index) and move centres to member means;
// an emptied cluster is re-seeded at the light farthest from its centre. Deterministic:
// assignments are independent per light and the means are summed in light order.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "world.hpp"

namespace vxr {

namespace {
inline uint64_t mixc(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
void light_centre(const vxr_light& l, double c[3]) {
    const uint32_t y = l.position / (1024u * 1024u), z = (l.position / 1024u) % 1024u, x = l.position % 1024u;
    c[0] = x + 0.5 * l.size;
    c[1] = y + 0.5 * l.size;
    c[2] = z + 0.5 * l.size;
}
}  // namespace

int cluster_lights(World& w, uint32_t k, uint32_t seed, uint32_t iters) {
    const uint32_t n = (uint32_t)w.lights.size();
    w.lightCluster.assign(n, 0u);
    w.clusterCount = 0;
    if (n == 0 || k == 0) return VXR_OK;
    k = std::min(k, n);
    std::vector<double> P((size_t)n * 3);
    for (uint32_t i = 0; i < n; i++) light_centre(w.lights[i], &P[3 * (size_t)i]);
    // seeded distinct initial centres
    std::vector<double> C((size_t)k * 3);
    std::vector<uint8_t> taken(n, 0);
    uint64_t s = mixc(0xC1u + seed);
    for (uint32_t c = 0; c < k; c++) {
        uint32_t pick;
        do {
            s = mixc(s);
            pick = (uint32_t)(s % n);
        } while (taken[pick]);
        taken[pick] = 1;
        for (int a = 0; a < 3; a++) C[3 * (size_t)c + a] = P[3 * (size_t)pick + a];
    }
    std::vector<uint32_t>& asg = w.lightCluster;
    std::vector<double> sum((size_t)k * 3);
    std::vector<uint32_t> cnt(k);
    for (uint32_t it = 0; it <= iters; it++) {
#pragma omp parallel for schedule(static)
        for (long long i = 0; i < (long long)n; i++) {
            const double* p = &P[3 * (size_t)i];
            double best = 1e300;
            uint32_t bc = 0;
            for (uint32_t c = 0; c < k; c++) {
                const double* q = &C[3 * (size_t)c];
                const double d = (p[0] - q[0]) * (p[0] - q[0]) + (p[1] - q[1]) * (p[1] - q[1]) + (p[2] - q[2]) * (p[2] - q[2]);
                if (d < best) { best = d; bc = c; }
            }
            asg[i] = bc;
        }
        if (it == iters) break;
        std::fill(sum.begin(), sum.end(), 0.0);
        std::fill(cnt.begin(), cnt.end(), 0u);
        for (uint32_t i = 0; i < n; i++) {
            const uint32_t c = asg[i];
            cnt[c]++;
            for (int a = 0; a < 3; a++) sum[3 * (size_t)c + a] += P[3 * (size_t)i + a];
        }
        for (uint32_t c = 0; c < k; c++) {
            if (cnt[c]) {
                for (int a = 0; a < 3; a++) C[3 * (size_t)c + a] = sum[3 * (size_t)c + a] / cnt[c];
            } else {
                // re-seed at the light farthest from its centre
                double far = -1.0;
                uint32_t fi = 0;
                for (uint32_t i = 0; i < n; i++) {
                    const double* p = &P[3 * (size_t)i];
                    const double* q = &C[3 * (size_t)asg[i]];
                    const double d = (p[0] - q[0]) * (p[0] - q[0]) + (p[1] - q[1]) * (p[1] - q[1]) + (p[2] - q[2]) * (p[2] - q[2]);
                    if (d > far) { far = d; fi = i; }
                }
                for (int a = 0; a < 3; a++) C[3 * (size_t)c + a] = P[3 * (size_t)fi + a];
                asg[fi] = c;
            }
        }
    }
    w.clusterCount = k;
    w.clusterVersion++;
    return VXR_OK;
}

}  // namespace vxr
