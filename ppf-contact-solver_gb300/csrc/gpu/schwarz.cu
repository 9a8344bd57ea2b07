// schwarz.cu -- aggregation and per-aggregate factors of the additive-Schwarz
// preconditioner (schwarz.cuh).
#include <algorithm>
#include <array>
#include <cmath>
#include <numeric>

#include "fatal.cuh"
#include "schwarz.cuh"

namespace ppf {
namespace gpu {

namespace {

constexpr unsigned kUnset = 0xFFFFFFFFu;
constexpr unsigned kFactorThreads = 64;
constexpr unsigned kCoarseFactorThreads = 256;

__host__ __device__ __forceinline__ unsigned tri_size(unsigned d) { return d * (d + 1u) / 2u; }

__device__ __forceinline__ float frob_slot(const float *v, size_t stride) {
    float s = 0.0f;
#pragma unroll
    for (int e = 0; e < 9; ++e) {
        const float x = v[e * stride];
        s += x * x;
    }
    return sqrtf(s);
}

// Frobenius norm of every (slot, lane) block of a SELL part.
__global__ void k_sell_weights(unsigned elems, const float *val, float *w) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= elems) return;
    const unsigned s = t / kSliceRows, lane = t % kSliceRows;
    w[t] = frob_slot(val + (size_t)s * 9 * kSliceRows + lane, kSliceRows);
}
__global__ void k_ovf_weights(unsigned entries, const float *val, float *w) {
    const unsigned e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= entries) return;
    w[e] = frob_slot(val + 9 * (size_t)e, 1);
}

template <class T> std::vector<T> to_host(const T *d, size_t n) {
    std::vector<T> h(n);
    if (n) PPF_CUDA(cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost));
    return h;
}

// Every stored block of row i of the operator: f(j, v, stride) with column j
// and entry (r, c) of the block at v[(3 c + r) stride] (fixed slots, contact
// slots, then overflow entries; the fixed part holds the diagonal).
template <class F>
__device__ __forceinline__ void walk_row(const PcgOperator &A, unsigned i, F &&f) {
    {
        const unsigned sl = i / kSliceRows, ln = i % kSliceRows;
        for (unsigned s = A.fixed.slice_off[sl]; s < A.fixed.slice_off[sl + 1]; ++s)
            f(__ldg(A.fixed.col + (size_t)s * kSliceRows + ln),
              A.fixed.val + (size_t)s * 9 * kSliceRows + ln, (size_t)kSliceRows);
    }
    const unsigned q = __ldg(A.contact.index + i);
    if (q == kUnset) return;
    const unsigned sl = q / kSliceRows, ln = q % kSliceRows;
    const SellMatrix &C = A.contact.sell;
    for (unsigned s = C.slice_off[sl]; s < C.slice_off[sl + 1]; ++s)
        f(__ldg(C.col + (size_t)s * kSliceRows + ln), C.val + (size_t)s * 9 * kSliceRows + ln,
          (size_t)kSliceRows);
    const unsigned k = __ldg(A.ovf.index + i);
    if (k != kUnset) {
        const uint2 rg = A.ovf.range[k];
        for (unsigned e = rg.x; e < rg.x + rg.y; ++e)
            f(__ldg(A.ovf.col + e), A.ovf.val + 9 * (size_t)e, (size_t)1);
    }
}

// Floors the diagonal of the d x d matrix L (row-major, shared), factors it
// L L^T in place and writes G = L^{-1} as a packed lower triangle to out; G
// is d x d shared scratch. Called by the whole block.
__device__ void factor_store(float *L, float *G, unsigned d, float *out, unsigned *status) {
    const unsigned tid = threadIdx.x, nt = blockDim.x;
    __shared__ float s_floor;
    // absolute diagonal floor (schwarz.cu:234-246): 1e-6 of the mean
    // diagonal plus 1e-8, added to the diagonal and kept as the pivot clamp
    if (tid == 0) {
        float tr = 0.0f;
        for (unsigned k = 0; k < d; ++k) tr += L[k * d + k];
        const float fl = 1e-6f * (tr / (float)d) + 1e-8f;
        for (unsigned k = 0; k < d; ++k) L[k * d + k] += fl;
        s_floor = fl;
    }
    __syncthreads();
    // Cholesky by columns: pivot, then the rows below it in parallel
    for (unsigned j = 0; j < d; ++j) {
        if (tid == 0) {
            float s = L[j * d + j];
            for (unsigned k = 0; k < j; ++k) s -= L[j * d + k] * L[j * d + k];
            if (!(s > s_floor)) {
                if (!(s == s)) atomicOr(status, STATUS_PRECOND_NONSPD);
                s = s_floor;
            }
            L[j * d + j] = sqrtf(s);
        }
        __syncthreads();
        const float inv = 1.0f / L[j * d + j];
        for (unsigned i = j + 1 + tid; i < d; i += nt) {
            float s = L[i * d + j];
            for (unsigned k = 0; k < j; ++k) s -= L[i * d + k] * L[j * d + k];
            L[i * d + j] = s * inv;
        }
        __syncthreads();
    }
    // G = L^{-1}, one column per thread (columns are independent)
    for (unsigned c = tid; c < d; c += nt) {
        G[c * d + c] = 1.0f / L[c * d + c];
        for (unsigned i = c + 1; i < d; ++i) {
            float s = 0.0f;
            for (unsigned k = c; k < i; ++k) s += L[i * d + k] * G[k * d + c];
            G[i * d + c] = -s / L[i * d + i];
        }
    }
    __syncthreads();
    for (unsigned e = tid; e < d * d; e += nt) {
        const unsigned i = e / d, j = e % d;
        if (j <= i) out[tri_size(i) + j] = G[e];
    }
}

// One block per aggregate: gather A_loc from the operator rows of its
// members (thread a owns rows 3a..3a+2, so the sums are in slot order),
// then floor, factor and store G = L^{-1}.
__global__ void k_schwarz_factor(PcgOperator A, const unsigned *agg, const unsigned *loc,
                                 unsigned *status) {
    extern __shared__ float sm[];
    const SchwarzView &S = A.schwarz;
    const unsigned g = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    const unsigned base = S.agg_off[g], m = S.agg_off[g + 1] - base, d = 3u * m;
    float *L = sm;            // d x d, row-major
    float *G = sm + d * d;    // d x d, row-major (lower triangle used)
    for (unsigned e = tid; e < 2u * d * d; e += nt) sm[e] = 0.0f;
    __syncthreads();
    for (unsigned a = tid; a < m; a += nt)
        walk_row(A, S.members[base + a], [&](unsigned j, const float *v, size_t stride) {
            if (__ldg(agg + j) != g) return;
            const unsigned b = __ldg(loc + j);
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int r = 0; r < 3; ++r)
                    L[(3 * a + r) * d + 3 * b + c] += __ldg(v + (3 * c + r) * stride);
        });
    __syncthreads();
    factor_store(L, G, d, const_cast<float *>(S.ainv) + S.ainv_off[g], status);
}

// One block per coarse domain: its Galerkin block, entry (a, b) the sum of
// A(i, j) over the vertices i of node a and j of node b (schwarz.cu:1225-1327
// and the gather of 1043-1145 in one pass), one thread per member vertex
// adding with shared atomics; then floor, factor and store.
__global__ void k_schwarz_coarse_factor(PcgOperator A, const unsigned *agg, const unsigned *dom,
                                        const unsigned *dom_loc, unsigned *status) {
    extern __shared__ float sm[];
    __shared__ unsigned s_start[kSchwarzMaxMembers + 1], s_node[kSchwarzMaxMembers];
    const SchwarzView &S = A.schwarz;
    const unsigned D = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    const unsigned base = S.dom_off[D], m = S.dom_off[D + 1] - base, d = 3u * m;
    float *L = sm, *G = sm + d * d;
    for (unsigned e = tid; e < 2u * d * d; e += nt) sm[e] = 0.0f;
    if (tid == 0) {
        s_start[0] = 0;
        for (unsigned a = 0; a < m; ++a) {
            const unsigned node = S.dom_members[base + a];
            s_node[a] = node;
            s_start[a + 1] = s_start[a] + S.agg_off[node + 1] - S.agg_off[node];
        }
    }
    __syncthreads();
    for (unsigned t = tid; t < s_start[m]; t += nt) {
        unsigned a = 0;
        while (s_start[a + 1] <= t) ++a;
        const unsigned i = S.members[S.agg_off[s_node[a]] + t - s_start[a]];
        walk_row(A, i, [&](unsigned j, const float *v, size_t stride) {
            const unsigned h = __ldg(agg + j);
            if (__ldg(dom + h) != D) return;
            const unsigned b = __ldg(dom_loc + h);
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
                for (int r = 0; r < 3; ++r)
                    atomicAdd(&L[(3 * a + r) * d + 3 * b + c], __ldg(v + (3 * c + r) * stride));
        });
    }
    __syncthreads();
    factor_store(L, G, d, const_cast<float *>(S.ainv1) + S.ainv1_off[D], status);
}

// The 9 values of every (slot, lane) block of a SELL part, contiguous.
__global__ void k_sell_blocks(unsigned elems, const float *val, float *out) {
    const unsigned t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= elems) return;
    const unsigned s = t / kSliceRows, lane = t % kSliceRows;
#pragma unroll
    for (int e = 0; e < 9; ++e) out[9 * (size_t)t + e] = val[((size_t)s * 9 + e) * kSliceRows + lane];
}

} // namespace

unsigned schwarz_aggregate(unsigned n, const std::vector<unsigned> &off,
                           const std::vector<unsigned> &col, const std::vector<float> &wgt,
                           unsigned kmax, std::vector<unsigned> &agg) {
    agg.assign(n, kUnset);
    // seeds in order of decreasing summed coupling (ties: lower index first)
    std::vector<double> incw(n, 0.0);
    for (unsigned i = 0; i < n; ++i)
        for (unsigned k = off[i]; k < off[i + 1]; ++k)
            if (col[k] != i) incw[i] += wgt[k];
    std::vector<unsigned> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(),
                     [&](unsigned a, unsigned b) { return incw[a] > incw[b]; });
    std::vector<float> gain(n, 0.0f);
    std::vector<unsigned> touched;
    unsigned nid = 0;
    auto absorb = [&](unsigned v) {
        for (unsigned k = off[v]; k < off[v + 1]; ++k) {
            const unsigned u = col[k];
            if (u == v || agg[u] != kUnset) continue;
            if (gain[u] == 0.0f) touched.push_back(u);
            gain[u] += wgt[k];
        }
    };
    for (unsigned seed : order) {
        if (agg[seed] != kUnset) continue;
        agg[seed] = nid;
        unsigned size = 1;
        touched.clear();
        absorb(seed);
        // grow by the unset neighbour most strongly coupled to the aggregate
        while (size < kmax) {
            float best = 0.0f;
            unsigned bv = kUnset;
            for (unsigned v : touched)
                if (agg[v] == kUnset && gain[v] > best) {
                    best = gain[v];
                    bv = v;
                }
            if (bv == kUnset) break;
            agg[bv] = nid;
            ++size;
            absorb(bv);
        }
        for (unsigned v : touched) gain[v] = 0.0f;
        ++nid;
    }
    return nid;
}

unsigned schwarz_coarsen(unsigned n, const std::vector<unsigned> &off,
                         const std::vector<unsigned> &col, const float *blk,
                         const std::vector<unsigned> &agg, unsigned n_agg, unsigned kmax,
                         std::vector<unsigned> &dom) {
    // Galerkin blocks of distinct aggregate pairs, in order of first sight
    std::vector<std::vector<std::pair<unsigned, unsigned>>> crow(n_agg); // (h, sum index)
    std::vector<std::array<float, 9>> sums;
    for (unsigned i = 0; i < n; ++i) {
        const unsigned g = agg[i];
        for (unsigned k = off[i]; k < off[i + 1]; ++k) {
            const unsigned h = agg[col[k]];
            if (h == g) continue;
            unsigned idx = kUnset;
            for (const auto &e : crow[g])
                if (e.first == h) {
                    idx = e.second;
                    break;
                }
            if (idx == kUnset) {
                idx = (unsigned)sums.size();
                sums.push_back({});
                crow[g].push_back({h, idx});
            }
            for (int e = 0; e < 9; ++e) sums[idx][e] += blk[9 * (size_t)k + e];
        }
    }
    std::vector<unsigned> coff(n_agg + 1, 0u), ccol;
    std::vector<float> cw;
    for (unsigned g = 0; g < n_agg; ++g) {
        std::sort(crow[g].begin(), crow[g].end());
        for (const auto &e : crow[g]) {
            float w = 0.0f;
            for (int q = 0; q < 9; ++q) w += sums[e.second][q] * sums[e.second][q];
            ccol.push_back(e.first);
            cw.push_back(std::sqrt(w));
        }
        coff[g + 1] = (unsigned)ccol.size();
    }
    return schwarz_aggregate(n_agg, coff, ccol, cw, kmax, dom);
}

namespace {

// Groups items 0..n-1 by their group id: offsets, members in ascending item
// order, each item's position in its group; returns the largest group.
unsigned group_members(const std::vector<unsigned> &grp, unsigned n_grp,
                       std::vector<unsigned> &goff, std::vector<unsigned> &mem,
                       std::vector<unsigned> &loc) {
    const unsigned n = (unsigned)grp.size();
    goff.assign(n_grp + 1, 0u);
    mem.assign(n, 0u);
    loc.assign(n, 0u);
    for (unsigned i = 0; i < n; ++i) goff[grp[i] + 1]++;
    unsigned max_m = 0;
    for (unsigned g = 0; g < n_grp; ++g) {
        max_m = std::max(max_m, goff[g + 1]);
        goff[g + 1] += goff[g];
    }
    std::vector<unsigned> cur(goff.begin(), goff.end() - 1);
    for (unsigned i = 0; i < n; ++i) {
        loc[i] = cur[grp[i]] - goff[grp[i]];
        mem[cur[grp[i]]++] = i;
    }
    return max_m;
}

// Float offsets of packed factors of 3 m x 3 m blocks, each starting on a
// 16-byte boundary (they are staged with 16-byte loads).
std::vector<unsigned> factor_offsets(const std::vector<unsigned> &goff) {
    const unsigned n_grp = (unsigned)goff.size() - 1;
    std::vector<unsigned> out(n_grp + 1, 0u);
    for (unsigned g = 0; g < n_grp; ++g)
        out[g + 1] = out[g] + ((tri_size(3u * (goff[g + 1] - goff[g])) + 3u) & ~3u);
    return out;
}

} // namespace

void schwarz_setup(const PcgOperator &A, SchwarzLayout &S, unsigned levels, cudaStream_t q) {
    const unsigned n = A.n;
    const bool coarse = levels >= 2;
    // weights (Frobenius norms) and, for the coarse level, the values of
    // every stored block, read back with the pattern
    auto readback = [&](unsigned elems, const float *val, bool sell, std::vector<float> &blk) {
        DevBuf<float> w;
        w.reserve(elems + 1);
        DevBuf<float> b;
        if (coarse) b.reserve(9 * (size_t)elems + 1);
        if (elems) {
            if (sell) {
                k_sell_weights<<<div_up(elems, 256u), 256, 0, q>>>(elems, val, w.data());
                if (coarse)
                    k_sell_blocks<<<div_up(elems, 256u), 256, 0, q>>>(elems, val, b.data());
            } else {
                k_ovf_weights<<<div_up(elems, 256u), 256, 0, q>>>(elems, val, w.data());
            }
            PPF_LAUNCH_CHECK();
        }
        PPF_CUDA(cudaStreamSynchronize(q));
        std::vector<float> h = to_host(w.data(), elems);
        if (coarse) blk = sell ? to_host(b.data(), 9 * (size_t)elems) : to_host(val, 9 * (size_t)elems);
        return h;
    };
    struct Entry {
        unsigned col;
        float w;
        const float *blk;
        bool operator<(const Entry &o) const { return col < o.col; }
    };
    std::vector<std::vector<Entry>> rows(n);
    std::vector<std::vector<float>> keep; // block values the entries point into
    keep.reserve(3);
    auto add_sell = [&](const SellMatrix &M, unsigned n_rows, const unsigned *perm_d) {
        if (!M.n_slices) return;
        std::vector<unsigned> so = to_host(M.slice_off, M.n_slices + 1);
        const unsigned elems = so[M.n_slices] * kSliceRows;
        std::vector<unsigned> c = to_host(M.col, elems);
        keep.emplace_back();
        std::vector<float> w = readback(elems, M.val, true, keep.back());
        const float *bv = keep.back().data();
        std::vector<unsigned> perm;
        if (perm_d) perm = to_host(perm_d, n_rows);
        for (unsigned sl = 0; sl < M.n_slices; ++sl)
            for (unsigned l = 0; l < kSliceRows; ++l) {
                const unsigned t = sl * kSliceRows + l;
                if (t >= n_rows) break;
                const unsigned i = perm_d ? perm[t] : t;
                for (unsigned s = so[sl]; s < so[sl + 1]; ++s) {
                    const size_t e = (size_t)s * kSliceRows + l;
                    if (c[e] != i) rows[i].push_back({c[e], w[e], coarse ? bv + 9 * e : nullptr});
                }
            }
    };
    PPF_CUDA(cudaStreamSynchronize(q));
    add_sell(A.fixed, n, nullptr);
    add_sell(A.contact.sell, A.contact.rows, A.contact.perm);
    if (A.ovf.count) {
        std::vector<unsigned> orow = to_host(A.ovf.row, A.ovf.count);
        std::vector<uint2> orange = to_host(A.ovf.range, A.ovf.count);
        const unsigned entries = orange.back().x + orange.back().y;
        std::vector<unsigned> oc = to_host(A.ovf.col, entries);
        keep.emplace_back();
        std::vector<float> ow = readback(entries, A.ovf.val, false, keep.back());
        const float *bv = keep.back().data();
        for (unsigned k = 0; k < A.ovf.count; ++k)
            for (unsigned e = orange[k].x; e < orange[k].x + orange[k].y; ++e)
                if (oc[e] != orow[k])
                    rows[orow[k]].push_back({oc[e], ow[e], coarse ? bv + 9 * (size_t)e : nullptr});
    }
    std::vector<unsigned> off(n + 1, 0u), col;
    std::vector<float> wgt, blk;
    for (unsigned i = 0; i < n; ++i) {
        std::stable_sort(rows[i].begin(), rows[i].end());
        for (auto &e : rows[i]) {
            col.push_back(e.col);
            wgt.push_back(e.w);
            if (coarse) blk.insert(blk.end(), e.blk, e.blk + 9);
        }
        off[i + 1] = (unsigned)col.size();
    }
    std::vector<unsigned> agg;
    const unsigned n_agg = schwarz_aggregate(n, off, col, wgt, kSchwarzKmax, agg);
    std::vector<unsigned> agg_off, members, loc;
    const unsigned max_m = group_members(agg, n_agg, agg_off, members, loc);
    const std::vector<unsigned> ainv_off = factor_offsets(agg_off);
    auto up = [&](DevBuf<unsigned> &d, const std::vector<unsigned> &h) {
        d.reserve(h.size() + 1);
        PPF_CUDA(cudaMemcpy(d.data(), h.data(), h.size() * 4, cudaMemcpyHostToDevice));
    };
    up(S.agg, agg);
    up(S.loc, loc);
    up(S.agg_off, agg_off);
    up(S.members, members);
    up(S.ainv_off, ainv_off);
    S.ainv.reserve((size_t)ainv_off[n_agg] + 1);
    S.n = n;
    S.n_agg = n_agg;
    S.max_members = max_m;
    S.levels = 1;
    S.n_dom = 0;
    S.max_dom_members = 0;
    if (coarse && n_agg > 0) {
        std::vector<unsigned> dom;
        const unsigned n_dom =
            schwarz_coarsen(n, off, col, blk.data(), agg, n_agg, kSchwarzKmax, dom);
        std::vector<unsigned> dom_off, dom_members, dom_loc;
        S.max_dom_members = group_members(dom, n_dom, dom_off, dom_members, dom_loc);
        const std::vector<unsigned> ainv1_off = factor_offsets(dom_off);
        up(S.dom, dom);
        up(S.dom_loc, dom_loc);
        up(S.dom_off, dom_off);
        up(S.dom_members, dom_members);
        up(S.ainv1_off, ainv1_off);
        S.ainv1.reserve((size_t)ainv1_off[n_dom] + 1);
        S.rc.reserve(n_agg);
        S.n_dom = n_dom;
        S.levels = 2;
    }
    S.levels_req = levels;
    S.ready = true;
}

void launch_schwarz_factor(const PcgOperator &A, SchwarzLayout &S, unsigned *d_status,
                           cudaStream_t q) {
    if (!S.n_agg) return;
    PcgOperator op = A;
    op.schwarz = S.view();
    {
        const unsigned dmax = 3u * S.max_members;
        const size_t smem = 2u * (size_t)dmax * dmax * sizeof(float);
        k_schwarz_factor<<<S.n_agg, kFactorThreads, smem, q>>>(op, S.agg.data(), S.loc.data(),
                                                               d_status);
        PPF_LAUNCH_CHECK();
    }
    if (S.n_dom) {
        const unsigned dmax = 3u * S.max_dom_members;
        const size_t smem = 2u * (size_t)dmax * dmax * sizeof(float);
        k_schwarz_coarse_factor<<<S.n_dom, kCoarseFactorThreads, smem, q>>>(
            op, S.agg.data(), S.dom.data(), S.dom_loc.data(), d_status);
        PPF_LAUNCH_CHECK();
    }
}

} // namespace gpu
} // namespace ppf
