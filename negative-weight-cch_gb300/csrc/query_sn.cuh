// Device routines of the supernodal elimination-tree query, shared by the
// per-query kernels (query_sn.cu) and the batched pipeline (query_top.cu).
#pragma once

#include "common.cuh"
#include "supernodal.h"
#include "topology.h"

namespace nwcch {

constexpr unsigned FULL = 0xffffffffu;

// Label arithmetic. Int32 storage: labels are int64 with "no path" as the
// sentinel BIG = 2^61; an arc weight INF32 maps to BIG as well, so a + w is a
// plain add (|label| <= depth * 2^31 < 2^52; BIG + BIG = 2^62 still fits) and
// any sum >= 2^60 means "no path". Int64 storage keeps the saturating sum.
template <class T>
struct QArith;
template <>
struct QArith<int32_t> {
    static constexpr int64_t BIG = (int64_t)1 << 61;
    static constexpr int64_t NOPATH = (int64_t)1 << 60;
    __device__ static int64_t w(int32_t x) { return x == INF32 ? BIG : (int64_t)x; }
    __device__ static int64_t add(int64_t a, int64_t b, int&) { return a + b; }
    __device__ static int64_t norm(int64_t x) { return x >= NOPATH ? BIG : x; }
    __device__ static bool none(int64_t x) { return x >= NOPATH; }
    __device__ static int64_t out(int64_t x) { return x >= NOPATH ? INF64 : x; }
};
template <>
struct QArith<int64_t> {
    static constexpr int64_t BIG = INF64;
    __device__ static int64_t w(int64_t x) { return x; }
    __device__ static int64_t add(int64_t a, int64_t b, int& e) {
        if (a == INF64 || b == INF64) return INF64;
        int64_t s;
        splus(a, b, s, e);
        return s;
    }
    __device__ static int64_t norm(int64_t x) { return x; }
    __device__ static bool none(int64_t x) { return x == INF64; }
    __device__ static int64_t out(int64_t x) { return x; }
};

// A chunk of fewer than `dense_rows` rows (small supernodes, the chain
// entering a supernode near its end) goes row by row instead: each row's
// label is final when its turn comes, and the warp pushes it along the row,
// 4 x 32 entries in flight at a time. Rows of consecutive ranks are
// consecutive in the CSR, so row r+1 starts where row r ends.
template <class T, bool RECORD, bool MEET>
__device__ __forceinline__ void rows_q(const DevTopo& D, const T* __restrict__ W, int32_t s0, int32_t k,
                                       int32_t cols, int i0, int c0, int64_t rowb, int32_t pos0, int32_t dstart,
                                       int32_t dx, int64_t* L, int32_t* chain, const int64_t* F,
                                       const int32_t* chain_s, int32_t ds, int64_t& best, int& e) {
    using Q = QArith<T>;
    const int lane = threadIdx.x & 31;
    for (int r = c0; r < k; r++) {
        const int len = cols - r - 1;
        const int p = pos0 + (r - i0);
        __syncwarp();
        const int64_t lab = Q::norm(L[p]);
        if (lane == 0) {
            L[p] = lab;
            if (RECORD) chain[p] = s0 + r;
            if (MEET && !Q::none(lab)) {
                const int32_t dv = dx - (r - i0);
                if (dv <= ds && chain_s[ds - dv] == s0 + r) {
                    const int64_t fv = F[ds - dv];
                    if (!Q::none(fv)) best = min(best, Q::add(lab, fv, e));
                }
            }
        }
        if (!Q::none(lab)) {
            for (int e0 = 0; e0 < len; e0 += 128) {
                int64_t wv[4];
                int32_t pj[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int j = e0 + 32 * u + lane;
                    pj[u] = -1;
                    wv[u] = Q::BIG;
                    if (j < len) {
                        const int c = r + 1 + j;
                        wv[u] = Q::w(W[rowb + j]);
                        pj[u] = c < k ? pos0 + (c - i0) : dstart - D.hdep[rowb + j];
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    if (pj[u] >= 0) {
                        const int64_t cand = Q::add(lab, wv[u], e);
                        if (!Q::none(cand) && cand < L[pj[u]]) L[pj[u]] = cand;
                    }
                }
            }
        }
        rowb += len;
    }
    __syncwarp();
}

template <class T, bool RECORD, bool MEET>
__device__ void sn_sweep(const DevTopo& D, const SnDev& S, const T* __restrict__ W, int32_t start, int32_t dstart,
                         int64_t* L, int32_t* chain, const int64_t* F, const int32_t* chain_s, int32_t ds,
                         int64_t& best, int& e, int dense_rows) {
    using Q = QArith<T>;
    const int lane = threadIdx.x & 31;
    int32_t x = start;
    while (x >= 0) {
        const int32_t sn = S.sn_id[x];
        const int32_t s0 = S.s0[sn], k = S.k[sn], cols = k + S.b[sn];
        const int i0 = x - s0;
        const int32_t dx = D.depth[x];
        const int32_t pos0 = dstart - dx;
        int64_t base = D.first[x];  // row base of the chunk's first row
        for (int c0 = i0; c0 < k; c0 += 32) {
            const int n = min(32, k - c0);
            if (n < dense_rows) {
                rows_q<T, RECORD, MEET>(D, W, s0, k, cols, i0, c0, base, pos0, dstart, dx, L, chain, F, chain_s, ds,
                                        best, e);
                break;
            }
            const int64_t step = cols - c0 - 1;  // length of row c0
            // row base of chunk row r: rows shrink by one entry per vertex
            auto rb = [&](int r) -> int64_t { return base + (int64_t)r * step - (int64_t)r * (r - 1) / 2; };
            const int p = pos0 + (c0 - i0) + lane;
            int64_t lab = lane < n ? L[p] : Q::BIG;
            if (RECORD && lane < n) chain[p] = s0 + c0 + lane;
            // the chunk's own 32x32 triangle, by shuffles
            {
                int64_t u[31];
#pragma unroll
                for (int r = 0; r < 31; r++)
                    u[r] = (r < lane && lane < n) ? Q::w(W[rb(r) + (lane - r - 1)]) : Q::BIG;
#pragma unroll
                for (int r = 0; r < 31; r++) {
                    const int64_t fr = Q::norm(__shfl_sync(FULL, lab, r));
                    lab = min(lab, Q::add(fr, u[r], e));
                }
            }
            lab = Q::norm(lab);
            if (lane < n) L[p] = lab;
            if (MEET && lane < n && !Q::none(lab)) {
                const int32_t v = s0 + c0 + lane;
                const int32_t dv = dx - (c0 - i0) - lane;
                if (dv <= ds && chain_s[ds - dv] == v) {
                    const int64_t fv = F[ds - dv];
                    if (!Q::none(fv)) best = min(best, Q::add(lab, fv, e));
                }
            }
            // the chunk's rows beyond its own vertices: later segment
            // vertices (j < k) and the boundary (j >= k); row r's label comes
            // by shuffle and its offset incrementally, so few registers stay
            // live and the 32 loads of a column group are in flight at once
            const T* Wb = W + base - c0 - 1;
            for (int jb = c0 + n; jb < cols; jb += 32) {
                const int j = jb + lane;
                const bool ok = j < cols;
                int64_t acc = Q::BIG;
                int64_t ro = 0;  // rb(r) - base - r
#pragma unroll
                for (int r = 0; r < 32; r++) {
                    const int64_t fr = __shfl_sync(FULL, lab, r);
                    if (ok && r < n) acc = min(acc, Q::add(fr, Q::w(Wb[ro + j]), e));
                    ro += step - 1 - r;
                }
                if (ok && !Q::none(acc)) {
                    const int32_t pj = j < k ? pos0 + (j - i0) : dstart - D.hdep[base + (j - c0 - 1)];
                    if (acc < L[pj]) L[pj] = acc;
                }
            }
            __syncwarp();
            base = rb(32);
        }
        x = D.parent[s0 + k - 1];
    }
}

// ---------------------------------------------------------------------------
// 32-bit labels. When every finite customized value satisfies
// |w| <= 2^28 / (depth + 2), every label and every candidate sum is the
// weight of a path of at most depth+1 arcs, hence within +-2^28; arc weights
// enter as min(w, CINF) (INF32 -> CINF = 2^30-1), a candidate involving no
// path is >= CINF - 2^28 > THR = 2^29 + 1, labels are normalised to CINF
// above THR before they are reused, and a + w then never overflows int32.
// The (min,+) step is the DPX add-min instruction.
struct Q32 {
    static constexpr int32_t CINF = (1 << 30) - 1;
    static constexpr int32_t THR = (1 << 29) + 1;
    __device__ static int32_t w(int32_t x) { return min(x, CINF); }
    __device__ static int32_t norm(int32_t x) { return x > THR ? CINF : x; }
    __device__ static bool none(int32_t x) { return x > THR; }
};

// Largest |finite value| of a metric, for choosing 32- or 64-bit labels
// (defined in query_sn.cu).
__global__ void k_maxabs(const int32_t* __restrict__ up, const int32_t* __restrict__ dn, int64_t count,
                         unsigned int* __restrict__ out);

__device__ __forceinline__ bool small_labels(const DevTopo& D, const unsigned int* maxabs) {
    return (int64_t)*maxabs * (int64_t)(D.max_depth + 2) <= ((int64_t)1 << 28);
}

// Barrier of the threads that share one query: the warp, or the whole CTA
// when WARPS warps work on one query.
template <int WARPS>
__device__ __forceinline__ void qsync() {
    if (WARPS == 1) __syncwarp();
    else __syncthreads();
}

// The row-by-row form of a thin chunk (see rows_q). With WARPS > 1 the
// warps split each row's entries; the label of a row is read by all of them
// after the barrier that ends the previous row.
template <bool RECORD, bool MEET, int WARPS>
__device__ __forceinline__ void rows32(const DevTopo& D, const int32_t* __restrict__ W, int32_t s0, int32_t k,
                                       int32_t cols, int i0, int c0, int64_t rowb, int32_t pos0, int32_t dstart,
                                       int32_t dx, int32_t* L, int32_t* chain, const int32_t* F,
                                       const int32_t* chain_s, int32_t ds, int32_t& best) {
    const int lane = threadIdx.x & 31, wq = WARPS == 1 ? 0 : (threadIdx.x >> 5);
    for (int r = c0; r < k; r++) {
        const int len = cols - r - 1;
        const int p = pos0 + (r - i0);
        qsync<WARPS>();
        const int32_t lab = Q32::norm(L[p]);
        if (wq == 0 && lane == 0) {
            if (RECORD) chain[p] = s0 + r;
            if (MEET && !Q32::none(lab)) {
                const int32_t dv = dx - (r - i0);
                if (dv <= ds && chain_s[ds - dv] == s0 + r) {
                    const int32_t fv = F[ds - dv];
                    if (!Q32::none(fv)) best = min(best, lab + fv);
                }
            }
        }
        if (!Q32::none(lab)) {
            for (int e0 = 128 * wq; e0 < len; e0 += 128 * WARPS) {
                int32_t wv[4], pj[4];
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const int j = e0 + 32 * u + lane;
                    pj[u] = -1;
                    wv[u] = Q32::CINF;
                    if (j < len) {
                        const int c = r + 1 + j;
                        wv[u] = Q32::w(W[rowb + j]);
                        pj[u] = c < k ? pos0 + (c - i0) : dstart - D.hdep[rowb + j];
                    }
                }
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    if (pj[u] >= 0) {
                        const int32_t cand = lab + wv[u];
                        if (!Q32::none(cand) && cand < L[pj[u]]) L[pj[u]] = cand;
                    }
                }
            }
        }
        rowb += len;
    }
    qsync<WARPS>();
}

// One sweep of a 32-bit query. WARPS = 1: one warp per query. WARPS > 1:
// a CTA per query, the warps solving each chunk's 32x32 triangle redundantly
// (no extra barrier; warp 0 alone writes labels and meets) and splitting the
// chunk's column groups and the rows' entries between them.
//
// STOP: the sweep ends at the first vertex whose supernode is marked in
// `stop_at` (stop_at[sn] >= 0) and returns that vertex (-1 when the chain
// ran to its root): the batched pipeline sweeps the chain's lower part here
// and its top supernodes as (min,+) products over many chains at once.
template <bool RECORD, bool MEET, int WARPS, bool REGS = false, bool STOP = false>
__device__ int32_t sn_sweep32(const DevTopo& D, const SnDev& S, const int32_t* __restrict__ W, int32_t start,
                              int32_t dstart, int32_t* L, int32_t* chain, const int32_t* F, const int32_t* chain_s,
                              int32_t ds, int32_t& best, int dense_rows, const int32_t* stop_at = nullptr) {
    const int lane = threadIdx.x & 31, wq = WARPS == 1 ? 0 : (threadIdx.x >> 5);
    int32_t x = start;
    while (x >= 0) {
        const int32_t sn = S.sn_id[x];
        if (STOP && stop_at[sn] >= 0) return x;
        const int32_t s0 = S.s0[sn], k = S.k[sn], cols = k + S.b[sn];
        const int i0 = x - s0;
        const int32_t dx = D.depth[x];
        const int32_t pos0 = dstart - dx;
        int64_t base = D.first[x];
        for (int c0 = i0; c0 < k; c0 += 32) {
            const int n = min(32, k - c0);
            if (n < dense_rows) {
                rows32<RECORD, MEET, WARPS>(D, W, s0, k, cols, i0, c0, base, pos0, dstart, dx, L, chain, F, chain_s,
                                            ds, best);
                break;
            }
            const int64_t step = cols - c0 - 1;
            auto rb = [&](int r) -> int64_t { return base + (int64_t)r * step - (int64_t)r * (r - 1) / 2; };
            const int p = pos0 + (c0 - i0) + lane;
            int32_t lab = lane < n ? L[p] : Q32::CINF;
            if (RECORD && wq == 0 && lane < n) chain[p] = s0 + c0 + lane;
            {
                int32_t u[31];
#pragma unroll
                for (int r = 0; r < 31; r++)
                    u[r] = (r < lane && lane < n) ? Q32::w(W[rb(r) + (lane - r - 1)]) : Q32::CINF;
#pragma unroll
                for (int r = 0; r < 31; r++) lab = __viaddmin_s32(Q32::norm(__shfl_sync(FULL, lab, r)), u[r], lab);
            }
            lab = Q32::norm(lab);
            if (WARPS > 1) qsync<WARPS>();  // every warp has read the chunk's labels
            if (wq == 0 && lane < n) L[p] = lab;
            if (MEET && wq == 0 && lane < n && !Q32::none(lab)) {
                const int32_t v = s0 + c0 + lane;
                const int32_t dv = dx - (c0 - i0) - lane;
                if (dv <= ds && chain_s[ds - dv] == v) {
                    const int32_t fv = F[ds - dv];
                    if (!Q32::none(fv)) best = min(best, lab + fv);
                }
            }
            // row r's label by shuffle, its offset (rb(r) - base - r,
            // int32: a supernode's trapezoid is far below 2^31 arcs)
            // incrementally, so few registers stay live across the 32 loads
            const int32_t* Wb = W + base - c0 - 1;
            const int32_t st = (int32_t)step - 1;
            if (REGS) {
                // the chunk's labels and row offsets held in registers across
                // the column groups: fewer instructions per arc, more registers
                int32_t fr[32], ro[32];
                int32_t o = 0;
#pragma unroll
                for (int r = 0; r < 32; r++) {
                    fr[r] = __shfl_sync(FULL, lab, r);
                    ro[r] = o;
                    o += st - r;
                }
                for (int jb = c0 + n + 32 * wq; jb < cols; jb += 32 * WARPS) {
                    const int j = jb + lane;
                    const bool ok = j < cols;
                    int32_t acc = Q32::CINF;
#pragma unroll
                    for (int r = 0; r < 32; r++)
                        if (ok && r < n) acc = __viaddmin_s32(fr[r], Q32::w(Wb[ro[r] + j]), acc);
                    if (ok && !Q32::none(acc)) {
                        const int32_t pj = j < k ? pos0 + (j - i0) : dstart - D.hdep[base + (j - c0 - 1)];
                        if (acc < L[pj]) L[pj] = acc;
                    }
                }
            } else {
                for (int jb = c0 + n + 32 * wq; jb < cols; jb += 32 * WARPS) {
                    const int j = jb + lane;
                    const bool ok = j < cols;
                    int32_t acc = Q32::CINF;
                    int32_t ro = 0;
#pragma unroll
                    for (int r = 0; r < 32; r++) {
                        const int32_t fr = __shfl_sync(FULL, lab, r);
                        if (ok && r < n) acc = __viaddmin_s32(fr, Q32::w(Wb[ro + j]), acc);
                        ro += st - r;
                    }
                    if (ok && !Q32::none(acc)) {
                        const int32_t pj = j < k ? pos0 + (j - i0) : dstart - D.hdep[base + (j - c0 - 1)];
                        if (acc < L[pj]) L[pj] = acc;
                    }
                }
            }
            qsync<WARPS>();
            base = rb(32);
        }
        x = D.parent[s0 + k - 1];
    }
    return -1;
}

}  // namespace nwcch
