// CCH potential on the device: p(v) = min(0, min_u dist(u, v)) read off a
// customized metric (cpp/cch.cpp:631-655, python/cch.py:734-755), the
// virtual-source distances Johnson's algorithm gets from Bellman-Ford.
//
// The reference sweeps every vertex upward in rank order (pushing p(x) +
// up(x, y) to the heads of x's row), then downward in reverse rank order
// (p(x) = min(p(x), p(y) + dn(x, y)) over the row). Here both sweeps go by
// supernode level, so a whole level runs at once:
//
// upward (levels from the bottom): a vertex's lower neighbours lie in its own
// supernode or in descendant supernodes, which pushed their candidates into
// p with atomicMin when their level ran. Inside a supernode the rows i < j
// form a triangular (min,+) solve, done 32 rows at a time: the 32x32 diagonal
// block by shuffles, the rest of the chunk's columns as a (min,+) product.
// The boundary columns (ancestors) are pushed at the end.
//
// downward (levels from the top): the boundary values are final, so every
// row first takes its (min,+) product with them; then the rows are solved
// from the bottom, 32 at a time, against the rows below them.
//
// Small supernodes take one warp each, large ones a CTA of 256 threads.

#include <algorithm>

#include "common.cuh"
#include "customize.h"
#include "supernodal.h"
#include "topology.h"

namespace nwcch {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ int64_t warp_min64(int64_t v) {
    for (int o = 16; o > 0; o >>= 1) v = min(v, (int64_t)__shfl_xor_sync(FULL, (long long)v, o));
    return v;
}

// arc of supernode row i (vertex s0+i), column j (j > i): first[s0+i] + (j-i-1)
__device__ __forceinline__ int64_t arc_at(const DevTopo& D, int32_t s0, int32_t i, int32_t j) {
    return D.first[s0 + i] + (j - i - 1);
}

// ---------------------------------------------------------------- upward

// Rows [i0, i0+rows) of a supernode: the diagonal block, by one warp.
// Lane j's column of the diagonal block [i0, i0+rows): w(i0+r, i0+j) for
// r < j, loaded up front so that the solve below is shuffles only.
template <class T>
__device__ __forceinline__ void diag_weights(const DevTopo& D, int32_t s0, int32_t i0, int rows, const T* W,
                                             T (&u)[31]) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int r = 0; r < 31; r++)
        u[r] = (r < lane && lane < rows) ? W[arc_at(D, s0, i0 + r, i0 + lane)] : Lim<T>::INF;
}

template <class T>
__device__ void up_diagonal(const DevTopo& D, int32_t s0, int32_t i0, int rows, const T* __restrict__ up,
                            int64_t* p, int& e) {
    const int lane = threadIdx.x & 31;
    int64_t pj = lane < rows ? p[s0 + i0 + lane] : 0;
    T u[31];
    diag_weights<T>(D, s0, i0, rows, up, u);
#pragma unroll
    for (int r = 0; r < 31; r++) {
        const int64_t pr = __shfl_sync(FULL, (long long)pj, r);
        const int64_t c = label_plus(pr, u[r], e);  // INF unless r < lane < rows
        if (c < pj) pj = c;
    }
    if (lane < rows) p[s0 + i0 + lane] = pj;
}

// Column j of the supernode against rows [i0, i1): min over the rows.
template <class T>
__device__ __forceinline__ int64_t up_column(const DevTopo& D, int32_t s0, int32_t i0, int32_t i1, int32_t j,
                                             const T* __restrict__ up, const int64_t* p, int& e) {
    int64_t acc = INF64;
#pragma unroll 8
    for (int32_t i = i0; i < i1; i++) acc = min(acc, label_plus(p[s0 + i], up[arc_at(D, s0, i, j)], e));
    return acc;
}

template <class T>
__global__ void __launch_bounds__(128) k_pot_up_warp(DevTopo D, SnDev S, const int32_t* __restrict__ sns,
                                                     int64_t count, const T* __restrict__ up, int64_t* p, int* err) {
    const int lane = threadIdx.x & 31;
    const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    int e = 0;
    for (int64_t it = w; it < count; it += nw) {
        const int32_t sn = sns[it];
        const int32_t s0 = S.s0[sn], k = S.k[sn], b = S.b[sn];
        // k <= 32: one diagonal block holds every internal row
        up_diagonal<T>(D, s0, 0, k, up, p, e);
        __syncwarp();
        const int64_t brow = D.first[s0 + k - 1];  // the last row lists the boundary
        for (int32_t q = lane; q < b; q += 32) {
            const int64_t acc = up_column<T>(D, s0, 0, k, k + q, up, p, e);
            if (acc < 0) atomicMin(reinterpret_cast<long long*>(p + D.head[brow + q]), (long long)acc);
        }
        __syncwarp();
    }
    if (e) atomicOr(err, e);
}

template <class T>
__global__ void __launch_bounds__(256) k_pot_up_cta(DevTopo D, SnDev S, const int32_t* __restrict__ sns,
                                                    int64_t count, const T* __restrict__ up, int64_t* p, int* err) {
    const int warp = threadIdx.x >> 5;
    int e = 0;
    for (int64_t it = blockIdx.x; it < count; it += gridDim.x) {
        const int32_t sn = sns[it];
        const int32_t s0 = S.s0[sn], k = S.k[sn], b = S.b[sn];
        for (int32_t i0 = 0; i0 < k; i0 += 32) {
            const int rows = min(32, k - i0);
            if (warp == 0) up_diagonal<T>(D, s0, i0, rows, up, p, e);
            __syncthreads();
            for (int32_t j = i0 + rows + threadIdx.x; j < k; j += blockDim.x) {
                const int64_t acc = up_column<T>(D, s0, i0, i0 + rows, j, up, p, e);
                if (acc < p[s0 + j]) p[s0 + j] = acc;
            }
            __syncthreads();
        }
        (void)b;  // the boundary push is k_pot_up_bnd's, spread over many CTAs
    }
    if (e) atomicOr(err, e);
}

// Upward boundary push of the CTA-swept supernodes: a CTA per (supernode,
// 256 boundary columns), a thread per column, the minimum over every row of
// the (final) supernode pushed into the ancestor.
template <class T>
__global__ void __launch_bounds__(256) k_pot_up_bnd(DevTopo D, SnDev S, const int32_t* __restrict__ items,
                                                    int64_t count, const T* __restrict__ up, int64_t* p, int* err) {
    int e = 0;
    for (int64_t it = blockIdx.x; it < count; it += gridDim.x) {
        const int32_t sn = items[2 * it], tile = items[2 * it + 1];
        const int32_t s0 = S.s0[sn], k = S.k[sn], b = S.b[sn];
        const int32_t q = tile * 256 + threadIdx.x;
        if (q < b) {
            const int64_t acc = up_column<T>(D, s0, 0, k, k + q, up, p, e);
            if (acc < 0) atomicMin(reinterpret_cast<long long*>(p + D.head[D.first[s0 + k - 1] + q]), (long long)acc);
        }
    }
    if (e) atomicOr(err, e);
}

// ---------------------------------------------------------------- downward

// Row i against columns [j0, j1) (vertices final): min over the columns, by
// one warp; column j's vertex value comes from `val`.
template <class T, class V>
__device__ __forceinline__ int64_t down_row(const DevTopo& D, int32_t s0, int32_t i, int32_t j0, int32_t j1,
                                            const T* __restrict__ dn, V val, int& e) {
    const int lane = threadIdx.x & 31;
    int64_t acc = INF64;
    for (int32_t j = j0 + lane; j < j1; j += 32) acc = min(acc, label_plus(val(j), dn[arc_at(D, s0, i, j)], e));
    return warp_min64(acc);
}

// Rows [i0, i0+rows), bottom-up, against each other: the diagonal block.
template <class T>
__device__ void down_diagonal(const DevTopo& D, int32_t s0, int32_t i0, int rows, const T* __restrict__ dn,
                              int64_t* p, int& e) {
    // push form: when row j is final (every row below it has pushed), rows
    // r < j take p(j) + dn(r, j); lane r holds dn(r, j) for j > r in
    // registers, so each step is one shuffle and one min
    const int lane = threadIdx.x & 31;
    int64_t mine = lane < rows ? p[s0 + i0 + lane] : INF64;
    T u[32];
#pragma unroll
    for (int j = 0; j < 32; j++)
        u[j] = (lane < j && j < rows) ? dn[arc_at(D, s0, i0 + lane, i0 + j)] : Lim<T>::INF;
#pragma unroll
    for (int jj = 0; jj < 31; jj++) {
        const int j = 31 - jj;  // bottom-up; constant indices keep u in registers
        const int64_t pj = __shfl_sync(FULL, (long long)mine, j);
        const int64_t c = label_plus(pj, u[j], e);  // INF unless lane < j < rows
        if (c < mine) mine = c;
    }
    if (lane < rows) p[s0 + i0 + lane] = mine;
}

template <class T>
__global__ void __launch_bounds__(128) k_pot_down_warp(DevTopo D, SnDev S, const int32_t* __restrict__ sns,
                                                       int64_t count, const T* __restrict__ dn, int64_t* p,
                                                       int* err) {
    const int lane = threadIdx.x & 31;
    const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    int e = 0;
    for (int64_t it = w; it < count; it += nw) {
        const int32_t sn = sns[it];
        const int32_t s0 = S.s0[sn], k = S.k[sn], b = S.b[sn];
        const int32_t* B = D.head + D.first[s0 + k - 1];
        auto bval = [&](int32_t j) { return p[B[j - k]]; };
        for (int32_t i = 0; i < k; i++) {
            const int64_t c = down_row<T>(D, s0, i, k, k + b, dn, bval, e);
            if (lane == 0 && c < p[s0 + i]) p[s0 + i] = c;
        }
        __syncwarp();
        down_diagonal<T>(D, s0, 0, k, dn, p, e);
        __syncwarp();
    }
    if (e) atomicOr(err, e);
}

template <class T>
__global__ void __launch_bounds__(256) k_pot_down_cta(DevTopo D, SnDev S, const int32_t* __restrict__ sns,
                                                      int64_t count, const T* __restrict__ dn, int64_t* p, int* err) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    int e = 0;
    for (int64_t it = blockIdx.x; it < count; it += gridDim.x) {
        const int32_t sn = sns[it];
        const int32_t s0 = S.s0[sn], k = S.k[sn];
        // the boundary product came first (k_pot_down_bnd); here the rows
        // are solved against each other, bottom-up
        auto ival = [&](int32_t j) { return p[s0 + j]; };
        for (int32_t i1 = k; i1 > 0; i1 -= 32) {
            const int32_t i0 = max(0, i1 - 32);
            // the chunk's rows against the final rows [i1, k)
            for (int32_t i = i0 + warp; i < i1; i += nwarps) {
                const int64_t c = down_row<T>(D, s0, i, i1, k, dn, ival, e);
                if (lane == 0 && c < p[s0 + i]) p[s0 + i] = c;
            }
            __syncthreads();
            if (warp == 0) down_diagonal<T>(D, s0, i0, i1 - i0, dn, p, e);
            __syncthreads();
        }
    }
    if (e) atomicOr(err, e);
}

// Downward boundary product of the CTA-swept supernodes: a CTA per
// (supernode, 32 rows), each warp 4 rows at once (the boundary values, final,
// loaded once per 4 rows), p(row) = min(p(row), min_q p(B[q]) + dn(row, q)).
template <class T>
__global__ void __launch_bounds__(256) k_pot_down_bnd(DevTopo D, SnDev S, const int32_t* __restrict__ items,
                                                      int64_t count, const T* __restrict__ dn, int64_t* p, int* err) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int e = 0;
    for (int64_t it = blockIdx.x; it < count; it += gridDim.x) {
        const int32_t sn = items[2 * it], tile = items[2 * it + 1];
        const int32_t s0 = S.s0[sn], k = S.k[sn], b = S.b[sn];
        const int32_t* B = D.head + D.first[s0 + k - 1];
        const int32_t r0 = tile * 32 + warp * 4;
        int64_t acc[4] = {INF64, INF64, INF64, INF64};
        int64_t base[4];
#pragma unroll
        for (int u = 0; u < 4; u++) base[u] = r0 + u < k ? D.first[s0 + r0 + u] + (k - (r0 + u) - 1) : 0;
        for (int32_t q = lane; q < b; q += 32) {
            const int64_t pb = p[B[q]];
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (r0 + u < k) acc[u] = min(acc[u], label_plus(pb, dn[base[u] + q], e));
        }
#pragma unroll
        for (int u = 0; u < 4; u++) {
            const int64_t c = warp_min64(acc[u]);
            if (lane == 0 && r0 + u < k && c < p[s0 + r0 + u]) p[s0 + r0 + u] = c;
        }
    }
    if (e) atomicOr(err, e);
}

// Single-vertex supernodes (k = 1, most of a road-like graph): a thread per
// vertex. Upward: its value is final (its lower neighbours are in earlier
// levels), push it along its row. Downward: its heads are final, pull.
template <class T>
__global__ void __launch_bounds__(256) k_pot_up_single(DevTopo D, SnDev S, const int32_t* __restrict__ sns,
                                                       int64_t count, const T* __restrict__ up, int64_t* p, int* err) {
    int e = 0;
    for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < count;
         it += (int64_t)gridDim.x * blockDim.x) {
        const int32_t x = S.s0[sns[it]];
        const int64_t px = p[x];
        for (int64_t a = D.first[x]; a < D.first[x + 1]; a++) {
            const int64_t c = label_plus(px, up[a], e);
            if (c < 0) atomicMin(reinterpret_cast<long long*>(p + D.head[a]), (long long)c);
        }
    }
    if (e) atomicOr(err, e);
}

template <class T>
__global__ void __launch_bounds__(256) k_pot_down_single(DevTopo D, SnDev S, const int32_t* __restrict__ sns,
                                                         int64_t count, const T* __restrict__ dn, int64_t* p,
                                                         int* err) {
    int e = 0;
    for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < count;
         it += (int64_t)gridDim.x * blockDim.x) {
        const int32_t x = S.s0[sns[it]];
        int64_t best = p[x];
        for (int64_t a = D.first[x]; a < D.first[x + 1]; a++) best = min(best, label_plus(p[D.head[a]], dn[a], e));
        p[x] = best;
    }
    if (e) atomicOr(err, e);
}

int thread_grid(int64_t count) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((count + 255) / 256, (int64_t)device_sms() * 16));
}

int warp_grid(int64_t count) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((count + 3) / 4, (int64_t)device_sms() * 64));
}

}  // namespace

template <class T>
int potential_launches(nwcch_topology* t, SnPlan* P, const T* up, const T* dn, int64_t* p, int* err, cudaStream_t s) {
    const DevTopo& D = t->d;
    NWCCH_CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(int64_t) * std::max<int64_t>(1, D.n), s));
    const int32_t L = P->levels;
    for (int32_t l = 0; l < L; l++) {
        const int64_t off = P->sn_level_off[l], big = P->sn_level_big[l], single = P->sn_level_single[l];
        const int64_t cnt = P->sn_level_off[l + 1] - off;
        const int32_t* o = P->d_sn_order + off;
        if (big) {
            k_pot_up_cta<T><<<(unsigned)std::min<int64_t>(big, (int64_t)t->sms * 8), 256, 0, s>>>(D, P->dev, o, big, up, p, err);
            const int64_t bo = P->pot_bu_off[l], bn = P->pot_bu_off[l + 1] - bo;
            if (bn)
                k_pot_up_bnd<T><<<(unsigned)std::min<int64_t>(bn, (int64_t)t->sms * 16), 256, 0, s>>>(D, P->dev, P->d_pot_bu + 2 * bo,
                                                                                        bn, up, p, err);
        }
        if (single > big)
            k_pot_up_warp<T><<<warp_grid(single - big), 128, 0, s>>>(D, P->dev, o + big, single - big, up, p, err);
        if (cnt > single)
            k_pot_up_single<T><<<thread_grid(cnt - single), 256, 0, s>>>(D, P->dev, o + single, cnt - single, up, p,
                                                                         err);
    }
    for (int32_t l = L - 1; l >= 0; l--) {
        const int64_t off = P->sn_level_off[l], big = P->sn_level_big[l], single = P->sn_level_single[l];
        const int64_t cnt = P->sn_level_off[l + 1] - off;
        const int32_t* o = P->d_sn_order + off;
        if (big) {
            const int64_t bo = P->pot_bd_off[l], bn = P->pot_bd_off[l + 1] - bo;
            if (bn)
                k_pot_down_bnd<T><<<(unsigned)std::min<int64_t>(bn, (int64_t)t->sms * 16), 256, 0, s>>>(
                    D, P->dev, P->d_pot_bd + 2 * bo, bn, dn, p, err);
            k_pot_down_cta<T><<<(unsigned)std::min<int64_t>(big, (int64_t)t->sms * 8), 256, 0, s>>>(D, P->dev, o, big, dn, p, err);
        }
        if (single > big)
            k_pot_down_warp<T><<<warp_grid(single - big), 128, 0, s>>>(D, P->dev, o + big, single - big, dn, p, err);
        if (cnt > single)
            k_pot_down_single<T><<<thread_grid(cnt - single), 256, 0, s>>>(D, P->dev, o + single, cnt - single, dn, p,
                                                                           err);
    }
    NWCCH_CUDA_TRY(cudaGetLastError());
    return NWCCH_OK;
}

// The sweeps' launches (4 per supernode level) replay as one CUDA graph per
// (up, dn, p) binding.
template <class T>
int potential(nwcch_topology* t, const T* up, const T* dn, int64_t* p, cudaStream_t s) {
    auto* P = static_cast<SnPlan*>(t->sn_plan);
    if (!P) return NWCCH_ERR_TOPOLOGY;
    int* err = stream_slot(t, s).err;
    SnGraph key{SN_GRAPH_POTENTIAL, (int)sizeof(T), 1, err, p, up, dn, nullptr, 0};
    return launch_cached(P, key, s, [&](cudaStream_t cs) { return potential_launches<T>(t, P, up, dn, p, err, cs); });
}

}  // namespace nwcch

using namespace nwcch;

extern "C" int nwcch_potential_async(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev, int64_t* p_dev,
                                     void* stream) {
    if (!t || !p_dev || (t->d.m_plus > 0 && (!up_dev || !dn_dev))) return NWCCH_ERR_ARG;
    return potential<int32_t>(t, up_dev, dn_dev, p_dev, (cudaStream_t)stream);
}

extern "C" int nwcch_potential(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev, int64_t* p_dev,
                               void* stream) {
    const int rc = nwcch_potential_async(t, up_dev, dn_dev, p_dev, stream);
    if (rc) return rc;
    return consume_error(t, (cudaStream_t)stream);
}

extern "C" int nwcch_potential_i64(nwcch_topology* t, const int64_t* up_dev, const int64_t* dn_dev, int64_t* p_dev,
                                   void* stream) {
    if (!t || !p_dev || (t->d.m_plus > 0 && (!up_dev || !dn_dev))) return NWCCH_ERR_ARG;
    const int rc = potential<int64_t>(t, up_dev, dn_dev, p_dev, (cudaStream_t)stream);
    if (rc) return rc;
    return consume_error(t, (cudaStream_t)stream);
}
