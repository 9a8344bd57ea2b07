// oracle_lbvh.cpp -- CPU restatement of the reference LBVH (test infrastructure).
//
// Follows crates/ppf-cts-solver/src/cpp/lbvh/lbvh.cu:
//   centroids          lbvh.cu:120-167
//   scene bounds       lbvh.cu:170-246
//   Morton codes       lbvh.cu:253-279
//   stable sort        kernels/radix_sort.cu:126-159 (LSD, stable)
//   Karras topology    lbvh.cu:289-385
//   leaf boxes         lbvh.cu:623-731
//   level-wise merge   lbvh.cu:778-857 (here: children before parents, which
//                      is the order the per-level launches establish)
// Built with -ffp-contract=off so every float operation rounds separately, the
// same arithmetic the GPU kernels perform.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

unsigned expand_bits(unsigned v) {
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

int clz32(unsigned x) { return x == 0 ? 32 : __builtin_clz(x); }

int lcp(const std::vector<unsigned> &k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    if (k[i] == k[j]) return 32 + clz32((unsigned)(i ^ j));
    return clz32(k[i] ^ k[j]);
}

void centroid(int kind, const float *x, const unsigned *prims, unsigned i,
              float c[3]) {
    if (kind == 3) {
        const unsigned *f = prims + 3 * i;
        for (int d = 0; d < 3; ++d)
            c[d] = (x[3 * f[0] + d] + x[3 * f[1] + d] + x[3 * f[2] + d]) / 3.0f;
    } else if (kind == 2) {
        const unsigned *e = prims + 2 * i;
        for (int d = 0; d < 3; ++d)
            c[d] = (x[3 * e[0] + d] + x[3 * e[1] + d]) / 2.0f;
    } else {
        unsigned v = prims ? prims[i] : i;
        for (int d = 0; d < 3; ++d) c[d] = x[3 * v + d];
    }
}

} // namespace

extern "C" void oracle_stable_sort(unsigned *keys, unsigned *vals, unsigned n,
                                   int key_bits) {
    unsigned mask = key_bits >= 32 ? 0xffffffffu : ((1u << key_bits) - 1u);
    std::vector<std::pair<unsigned, unsigned>> kv(n);
    for (unsigned i = 0; i < n; ++i) kv[i] = {keys[i], vals[i]};
    std::stable_sort(kv.begin(), kv.end(),
                     [mask](const std::pair<unsigned, unsigned> &a,
                            const std::pair<unsigned, unsigned> &b) {
                         return (a.first & mask) < (b.first & mask);
                     });
    for (unsigned i = 0; i < n; ++i) {
        keys[i] = kv[i].first;
        vals[i] = kv[i].second;
    }
}

extern "C" unsigned oracle_lbvh_build(int kind, const float *x0, const float *x1,
                                      unsigned n_verts, const unsigned *prims,
                                      unsigned n, const float *margin,
                                      float extrapolate, unsigned *out_node,
                                      float *out_box, unsigned *out_keys) {
    (void)n_verts;
    if (n == 0) return 0;
    const unsigned nn = 2 * n - 1;
    std::vector<unsigned> node(2 * nn, 0u);
    std::vector<unsigned> keys(n), vals(n);
    unsigned root = 0;
    if (n == 1) {
        node[0] = 1u;
        node[1] = 0u;
        keys[0] = 0u;
    } else {
        // centroids of x1 (the tree is ordered by the END of the sweep)
        std::vector<float> c(3 * n);
        float lo[3] = {INFINITY, INFINITY, INFINITY};
        float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (unsigned i = 0; i < n; ++i) {
            centroid(kind, x1, prims, i, &c[3 * i]);
            for (int d = 0; d < 3; ++d) {
                lo[d] = std::fmin(lo[d], c[3 * i + d]);
                hi[d] = std::fmax(hi[d], c[3 * i + d]);
            }
        }
        for (unsigned i = 0; i < n; ++i) {
            unsigned q[3];
            for (int d = 0; d < 3; ++d) {
                float ext = hi[d] - lo[d];
                float scale = ext > 1e-10f ? 1023.0f / ext : 0.0f;
                float t = (c[3 * i + d] - lo[d]) * scale;
                q[d] = (unsigned)std::fmin(1023.0f, std::fmax(0.0f, t));
            }
            keys[i] = expand_bits(q[0]) | (expand_bits(q[1]) << 1) |
                      (expand_bits(q[2]) << 2);
            vals[i] = i;
        }
        oracle_stable_sort(keys.data(), vals.data(), n, 32);
        for (unsigned i = 0; i < n; ++i) {
            node[2 * i] = vals[i] + 1u;
            node[2 * i + 1] = 0u;
        }
        const int N = (int)n;
        for (int i = 0; i + 1 < N; ++i) {
            int d = lcp(keys, N, i, i + 1) > lcp(keys, N, i, i - 1) ? 1 : -1;
            int dmin = lcp(keys, N, i, i - d);
            int lmax = 2;
            while (lcp(keys, N, i, i + lmax * d) > dmin) lmax *= 2;
            int l = 0;
            for (int t = lmax / 2; t >= 1; t /= 2)
                if (lcp(keys, N, i, i + (l + t) * d) > dmin) l += t;
            int j = i + l * d;
            int left = std::min(i, j), right = std::max(i, j);
            int dn = lcp(keys, N, left, right);
            int s = 0, t = right - left;
            do {
                t = (t + 1) / 2;
                if (lcp(keys, N, left, left + s + t) > dn) s += t;
            } while (t > 1);
            int split = left + s;
            unsigned lc = left == split ? (unsigned)left : n + (unsigned)split;
            unsigned rc =
                split + 1 == right ? (unsigned)right : n + (unsigned)split + 1u;
            node[2 * (n + i)] = lc + 1u;
            node[2 * (n + i) + 1] = rc + 1u;
        }
        root = n;
    }
    // boxes: leaves, then internal nodes children-first (post-order walk)
    std::vector<float> box(8 * (size_t)nn, 0.0f);
    for (unsigned leaf = 0; leaf < n; ++leaf) {
        unsigned prim = node[2 * leaf] - 1u;
        unsigned v[3];
        int nv = kind;
        if (kind == 3) {
            for (int k = 0; k < 3; ++k) v[k] = prims[3 * prim + k];
        } else if (kind == 2) {
            for (int k = 0; k < 2; ++k) v[k] = prims[2 * prim + k];
        } else {
            v[0] = prims ? prims[prim] : prim;
            nv = 1;
        }
        float mg = margin[prim];
        float *b = &box[8 * (size_t)leaf];
        for (int d = 0; d < 3; ++d) {
            float a0 = INFINITY, b0 = -INFINITY, a1 = INFINITY, b1 = -INFINITY;
            for (int k = 0; k < nv; ++k) {
                float y0 = x0[3 * v[k] + d], y1 = x1[3 * v[k] + d];
                float z = std::fma(extrapolate, y1 - y0, y0);
                a0 = std::fmin(a0, y0);
                b0 = std::fmax(b0, y0);
                a1 = std::fmin(a1, z);
                b1 = std::fmax(b1, z);
            }
            b[d] = std::fmin(a0, a1) - mg;
            b[4 + d] = std::fmax(b0, b1) + mg;
        }
        b[3] = 1.0f;
        b[7] = 0.0f;
    }
    if (n > 1) {
        // iterative post-order from the root
        std::vector<std::pair<unsigned, int>> stack;
        stack.push_back({root, 0});
        while (!stack.empty()) {
            auto &top = stack.back();
            unsigned id = top.first;
            if (node[2 * id + 1] == 0u) {
                stack.pop_back();
                continue;
            }
            if (top.second == 0) {
                top.second = 1;
                stack.push_back({node[2 * id] - 1u, 0});
                continue;
            }
            if (top.second == 1) {
                top.second = 2;
                stack.push_back({node[2 * id + 1] - 1u, 0});
                continue;
            }
            stack.pop_back();
            const float *L = &box[8 * (size_t)(node[2 * id] - 1u)];
            const float *R = &box[8 * (size_t)(node[2 * id + 1] - 1u)];
            float *o = &box[8 * (size_t)id];
            bool la = L[3] != 0.0f, ra = R[3] != 0.0f;
            if (la && ra) {
                for (int d = 0; d < 3; ++d) {
                    o[d] = L[d] < R[d] ? L[d] : R[d];
                    o[4 + d] = L[4 + d] > R[4 + d] ? L[4 + d] : R[4 + d];
                }
                o[3] = 1.0f;
                o[7] = 0.0f;
            } else if (la) {
                std::memcpy(o, L, 8 * sizeof(float));
            } else if (ra) {
                std::memcpy(o, R, 8 * sizeof(float));
            } else {
                std::memcpy(o, L, 8 * sizeof(float));
                o[3] = 0.0f;
            }
        }
    }
    if (out_node) std::memcpy(out_node, node.data(), 2 * nn * sizeof(unsigned));
    if (out_box) std::memcpy(out_box, box.data(), 8 * (size_t)nn * sizeof(float));
    if (out_keys) std::memcpy(out_keys, keys.data(), n * sizeof(unsigned));
    return root;
}
