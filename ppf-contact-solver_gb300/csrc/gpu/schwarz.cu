// schwarz.cu -- aggregation and per-aggregate factors of the additive-Schwarz
// preconditioner (schwarz.cuh).
#include <algorithm>
#include <numeric>

#include "fatal.cuh"
#include "schwarz.cuh"

namespace ppf {
namespace gpu {

namespace {

constexpr unsigned kUnset = 0xFFFFFFFFu;
constexpr unsigned kFactorThreads = 64;

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

// Adds the block of one stored slot to rows 3a..3a+2 of the aggregate's
// dense matrix (row-major, leading dimension d) when its column is a member.
__device__ __forceinline__ void add_slot(float *L, unsigned d, unsigned a, unsigned j,
                                         unsigned g, const unsigned *agg, const unsigned *loc,
                                         const float *v, size_t stride) {
    if (__ldg(agg + j) != g) return;
    const unsigned b = __ldg(loc + j);
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r)
            L[(3 * a + r) * d + 3 * b + c] += __ldg(v + (3 * c + r) * stride);
}

// One block per aggregate: gather A_loc from the operator (fixed slots,
// contact slots, overflow entries of each member row; the fixed part holds
// the diagonal), floor its diagonal, factor it and store G = L^{-1}.
__global__ void k_schwarz_factor(PcgOperator A, const unsigned *agg, const unsigned *loc,
                                 unsigned *status) {
    extern __shared__ float sm[];
    const SchwarzView &S = A.schwarz;
    const unsigned g = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
    const unsigned base = S.agg_off[g], m = S.agg_off[g + 1] - base, d = 3u * m;
    float *L = sm;            // d x d, row-major
    float *G = sm + d * d;    // d x d, row-major (lower triangle used)
    __shared__ float s_floor;
    for (unsigned e = tid; e < 2u * d * d; e += nt) sm[e] = 0.0f;
    __syncthreads();
    for (unsigned a = tid; a < m; a += nt) {
        const unsigned i = S.members[base + a];
        {
            const unsigned sl = i / kSliceRows, ln = i % kSliceRows;
            for (unsigned s = A.fixed.slice_off[sl]; s < A.fixed.slice_off[sl + 1]; ++s)
                add_slot(L, d, a, __ldg(A.fixed.col + (size_t)s * kSliceRows + ln), g, agg, loc,
                         A.fixed.val + (size_t)s * 9 * kSliceRows + ln, kSliceRows);
        }
        const unsigned q = __ldg(A.contact.index + i);
        if (q != kUnset) {
            const unsigned sl = q / kSliceRows, ln = q % kSliceRows;
            const SellMatrix &C = A.contact.sell;
            for (unsigned s = C.slice_off[sl]; s < C.slice_off[sl + 1]; ++s)
                add_slot(L, d, a, __ldg(C.col + (size_t)s * kSliceRows + ln), g, agg, loc,
                         C.val + (size_t)s * 9 * kSliceRows + ln, kSliceRows);
            const unsigned k = __ldg(A.ovf.index + i);
            if (k != kUnset) {
                const uint2 rg = A.ovf.range[k];
                for (unsigned e = rg.x; e < rg.x + rg.y; ++e)
                    add_slot(L, d, a, __ldg(A.ovf.col + e), g, agg, loc,
                             A.ovf.val + 9 * (size_t)e, 1);
            }
        }
    }
    __syncthreads();
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
    float *out = const_cast<float *>(S.ainv) + S.ainv_off[g];
    for (unsigned e = tid; e < d * d; e += nt) {
        const unsigned i = e / d, j = e % d;
        if (j <= i) out[tri_size(i) + j] = G[e];
    }
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

void schwarz_setup(const PcgOperator &A, SchwarzLayout &S, cudaStream_t q) {
    const unsigned n = A.n;
    // weights of every stored block, read back with the pattern
    auto weights = [&](unsigned elems, const float *val, bool sell) {
        DevBuf<float> w;
        w.reserve(elems + 1);
        if (elems) {
            if (sell)
                k_sell_weights<<<div_up(elems, 256u), 256, 0, q>>>(elems, val, w.data());
            else
                k_ovf_weights<<<div_up(elems, 256u), 256, 0, q>>>(elems, val, w.data());
            PPF_LAUNCH_CHECK();
        }
        PPF_CUDA(cudaStreamSynchronize(q));
        std::vector<float> h = to_host(w.data(), elems);
        w.release();
        return h;
    };
    std::vector<std::vector<std::pair<unsigned, float>>> rows(n);
    auto add_sell = [&](const SellMatrix &M, unsigned n_rows, const unsigned *perm_d) {
        if (!M.n_slices) return;
        std::vector<unsigned> so = to_host(M.slice_off, M.n_slices + 1);
        const unsigned elems = so[M.n_slices] * kSliceRows;
        std::vector<unsigned> c = to_host(M.col, elems);
        std::vector<float> w = weights(elems, M.val, true);
        std::vector<unsigned> perm;
        if (perm_d) perm = to_host(perm_d, n_rows);
        for (unsigned sl = 0; sl < M.n_slices; ++sl)
            for (unsigned l = 0; l < kSliceRows; ++l) {
                const unsigned t = sl * kSliceRows + l;
                if (t >= n_rows) break;
                const unsigned i = perm_d ? perm[t] : t;
                for (unsigned s = so[sl]; s < so[sl + 1]; ++s) {
                    const size_t e = (size_t)s * kSliceRows + l;
                    if (c[e] != i) rows[i].push_back({c[e], w[e]});
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
        std::vector<float> ow = weights(entries, A.ovf.val, false);
        for (unsigned k = 0; k < A.ovf.count; ++k)
            for (unsigned e = orange[k].x; e < orange[k].x + orange[k].y; ++e)
                if (oc[e] != orow[k]) rows[orow[k]].push_back({oc[e], ow[e]});
    }
    std::vector<unsigned> off(n + 1, 0u), col;
    std::vector<float> wgt;
    for (unsigned i = 0; i < n; ++i) {
        std::sort(rows[i].begin(), rows[i].end());
        for (auto &e : rows[i]) {
            col.push_back(e.first);
            wgt.push_back(e.second);
        }
        off[i + 1] = (unsigned)col.size();
    }
    std::vector<unsigned> agg;
    const unsigned n_agg = schwarz_aggregate(n, off, col, wgt, kSchwarzKmax, agg);
    // members by aggregate in ascending vertex order, positions, factor offsets
    std::vector<unsigned> agg_off(n_agg + 1, 0u), members(n), loc(n), ainv_off(n_agg + 1, 0u);
    for (unsigned i = 0; i < n; ++i) agg_off[agg[i] + 1]++;
    unsigned max_m = 0;
    for (unsigned g = 0; g < n_agg; ++g) {
        max_m = std::max(max_m, agg_off[g + 1]);
        // each factor starts on a 16-byte boundary (staged with 16-byte loads)
        ainv_off[g + 1] = ainv_off[g] + ((tri_size(3u * agg_off[g + 1]) + 3u) & ~3u);
        agg_off[g + 1] += agg_off[g];
    }
    std::vector<unsigned> cur(agg_off.begin(), agg_off.end() - 1);
    for (unsigned i = 0; i < n; ++i) {
        loc[i] = cur[agg[i]] - agg_off[agg[i]];
        members[cur[agg[i]]++] = i;
    }
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
    S.ready = true;
}

void launch_schwarz_factor(const PcgOperator &A, SchwarzLayout &S, unsigned *d_status,
                           cudaStream_t q) {
    if (!S.n_agg) return;
    const unsigned dmax = 3u * S.max_members;
    const size_t smem = 2u * (size_t)dmax * dmax * sizeof(float);
    PcgOperator op = A;
    op.schwarz = S.view();
    k_schwarz_factor<<<S.n_agg, kFactorThreads, smem, q>>>(op, S.agg.data(), S.loc.data(),
                                                           d_status);
    PPF_LAUNCH_CHECK();
}

} // namespace gpu
} // namespace ppf
