// Supernodal elimination-tree query: one warp per (s, t) pair, labels in
// shared memory, the chain walked supernode segment by segment.
//
// Same sweeps as the reference query (python/cch_nb.py:577-615): forward
// labels along the ancestors of s with up weights, backward labels along the
// ancestors of t with dn weights, minimum of their sum over shared ancestors.
// Along the chain, the vertices of one supernode are consecutive ranks whose
// rows are nested (row of s0+i = ranks s0+i+1.. then the boundary B), so a
// segment is a dense (min,+) triangular solve: 32 chain vertices at a time,
// lane l owns vertex c0+l; the 32x32 diagonal part is solved with shuffles
// (lane r's label is final when step r broadcasts it), the rest of the
// chunk's rows (later segment vertices and B) is a (min,+) product folded
// into the label array. Only one parent pointer is followed per segment.
// Labels are indexed by chain position: depth(start) - depth(v).

#include <algorithm>
#include <cstdlib>

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

// Largest |finite value| of a metric, for choosing 32- or 64-bit labels.
__global__ void k_maxabs(const int32_t* __restrict__ up, const int32_t* __restrict__ dn, int64_t count,
                         unsigned int* __restrict__ out) {
    unsigned int mx = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t u = up[i], d = dn[i];
        if (u != INF32) mx = max(mx, (unsigned int)(u < 0 ? -(int64_t)u : u));
        if (d != INF32) mx = max(mx, (unsigned int)(d < 0 ? -(int64_t)d : d));
    }
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(FULL, mx, o));
    if ((threadIdx.x & 31) == 0 && mx) atomicMax(out, mx);
}

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
template <bool RECORD, bool MEET, int WARPS, bool REGS = false>
__device__ void sn_sweep32(const DevTopo& D, const SnDev& S, const int32_t* __restrict__ W, int32_t start,
                           int32_t dstart, int32_t* L, int32_t* chain, const int32_t* F, const int32_t* chain_s,
                           int32_t ds, int32_t& best, int dense_rows) {
    const int lane = threadIdx.x & 31, wq = WARPS == 1 ? 0 : (threadIdx.x >> 5);
    int32_t x = start;
    while (x >= 0) {
        const int32_t sn = S.sn_id[x];
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
}

// Labels live in shared memory, or - for trees so deep that shared memory
// would leave only a few warps per SM - in a global scratch (`gscratch`,
// 12 * (depth + 1) + 16 bytes per warp, L1/L2-resident while in use).
template <int MINB, bool REGS>
__global__ void __launch_bounds__(512, MINB) k_query_sn32(DevTopo D, SnDev S, const int32_t* __restrict__ up, const int32_t* __restrict__ dn,
                             const int32_t* __restrict__ s_rank, const int32_t* __restrict__ t_rank, int64_t nq,
                             int64_t* __restrict__ dist, const unsigned int* __restrict__ maxabs,
                             unsigned char* __restrict__ gscratch, int* __restrict__ err, int dense_rows) {
    if (!small_labels(D, maxabs)) return;  // the 64-bit kernel answers this batch
    extern __shared__ __align__(16) unsigned char smraw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t Dp = D.max_depth + 1;
    const int64_t per_warp = ((12 * Dp + 16) + 15) & ~15LL;
    const int64_t warp = blockIdx.x * (int64_t)(blockDim.x >> 5) + wib;
    unsigned char* mine = gscratch ? gscratch + warp * per_warp : smraw + wib * per_warp;
    int32_t* F = reinterpret_cast<int32_t*>(mine);
    int32_t* R = F + Dp;
    int32_t* chain = R + Dp;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    int e = 0;
    for (int64_t q = warp; q < nq; q += nwarps) {
        const int32_t s = s_rank[q], t = t_rank[q];
        if (s < 0 || s >= D.n || t < 0 || t >= D.n) {
            if (lane == 0) dist[q] = INF64;
            e |= ERR_ARG;
            continue;
        }
        const int32_t ds = D.depth[s], dt = D.depth[t];
        for (int i = lane; i <= ds; i += 32) F[i] = Q32::CINF;
        for (int i = lane; i <= dt; i += 32) R[i] = Q32::CINF;
        __syncwarp();
        if (lane == 0) {
            F[0] = 0;
            R[0] = 0;
        }
        __syncwarp();
        int32_t best = Q32::CINF;
        sn_sweep32<true, false, 1, REGS>(D, S, up, s, ds, F, chain, nullptr, nullptr, 0, best, dense_rows);
        __syncwarp();
        sn_sweep32<false, true, 1, REGS>(D, S, dn, t, dt, R, nullptr, F, chain, ds, best, dense_rows);
        for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(FULL, best, o));
        if (lane == 0) dist[q] = Q32::none(best) ? INF64 : (int64_t)best;
        __syncwarp();
    }
    if (e) atomicOr(err, e);
}

// Few queries: a CTA of WARPS warps per (s, t) pair, labels in shared memory,
// so that a small batch (the serving loop at low load, one query per call)
// is not left to one warp per query.
template <int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_query_sn32_cta(DevTopo D, SnDev S, const int32_t* __restrict__ up,
                                                               const int32_t* __restrict__ dn,
                                                               const int32_t* __restrict__ s_rank,
                                                               const int32_t* __restrict__ t_rank, int64_t nq,
                                                               int64_t* __restrict__ dist,
                                                               const unsigned int* __restrict__ maxabs,
                                                               int* __restrict__ err, int dense_rows) {
    if (!small_labels(D, maxabs)) return;  // the 64-bit kernel answers this batch
    extern __shared__ __align__(16) unsigned char smraw[];
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    const int64_t Dp = D.max_depth + 1;
    int32_t* F = reinterpret_cast<int32_t*>(smraw);
    int32_t* R = F + Dp;
    int32_t* chain = R + Dp;
    int e = 0;
    for (int64_t q = blockIdx.x; q < nq; q += gridDim.x) {
        const int32_t s = s_rank[q], t = t_rank[q];
        if (s < 0 || s >= D.n || t < 0 || t >= D.n) {
            if (threadIdx.x == 0) dist[q] = INF64;
            e |= ERR_ARG;
            continue;
        }
        const int32_t ds = D.depth[s], dt = D.depth[t];
        for (int i = threadIdx.x; i <= ds; i += blockDim.x) F[i] = Q32::CINF;
        for (int i = threadIdx.x; i <= dt; i += blockDim.x) R[i] = Q32::CINF;
        __syncthreads();
        if (threadIdx.x == 0) {
            F[0] = 0;
            R[0] = 0;
        }
        __syncthreads();
        int32_t best = Q32::CINF;
        sn_sweep32<true, false, WARPS>(D, S, up, s, ds, F, chain, nullptr, nullptr, 0, best, dense_rows);
        __syncthreads();
        sn_sweep32<false, true, WARPS>(D, S, dn, t, dt, R, nullptr, F, chain, ds, best, dense_rows);
        if (wq == 0) {
            for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(FULL, best, o));
            if (lane == 0) dist[q] = Q32::none(best) ? INF64 : (int64_t)best;
        }
        __syncthreads();
    }
    if (e) atomicOr(err, e);
}

template <class T>
__global__ void k_query_sn(DevTopo D, SnDev S, const T* __restrict__ up, const T* __restrict__ dn,
                           const int32_t* __restrict__ s_rank, const int32_t* __restrict__ t_rank, int64_t nq,
                           int64_t* __restrict__ dist, const unsigned int* __restrict__ maxabs,
                           int* __restrict__ err, int dense_rows) {
    if (sizeof(T) == 4 && small_labels(D, maxabs)) return;  // answered by k_query_sn32
    extern __shared__ __align__(16) unsigned char smraw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t Dp = D.max_depth + 1;
    const int64_t per_warp = 16 * Dp + 4 * Dp + 16;
    unsigned char* mine = smraw + wib * ((per_warp + 15) & ~15LL);
    int64_t* F = reinterpret_cast<int64_t*>(mine);
    int64_t* R = F + Dp;
    int32_t* chain = reinterpret_cast<int32_t*>(R + Dp);
    const int64_t warp = blockIdx.x * (int64_t)(blockDim.x >> 5) + wib;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    int e = 0;
    for (int64_t q = warp; q < nq; q += nwarps) {
        const int32_t s = s_rank[q], t = t_rank[q];
        if (s < 0 || s >= D.n || t < 0 || t >= D.n) {
            if (lane == 0) dist[q] = INF64;
            e |= ERR_ARG;
            continue;
        }
        const int32_t ds = D.depth[s], dt = D.depth[t];
        using Q = QArith<T>;
        for (int i = lane; i <= ds; i += 32) F[i] = Q::BIG;
        for (int i = lane; i <= dt; i += 32) R[i] = Q::BIG;
        __syncwarp();
        if (lane == 0) {
            F[0] = 0;
            R[0] = 0;
        }
        __syncwarp();
        int64_t best = Q::BIG;
        sn_sweep<T, true, false>(D, S, up, s, ds, F, chain, nullptr, nullptr, 0, best, e, dense_rows);
        __syncwarp();
        sn_sweep<T, false, true>(D, S, dn, t, dt, R, nullptr, F, chain, ds, best, e, dense_rows);
        for (int o = 16; o > 0; o >>= 1) best = min(best, (int64_t)__shfl_xor_sync(FULL, best, o));
        if (lane == 0) dist[q] = Q::out(best);
        __syncwarp();
    }
    if (e) atomicOr(err, e);
}

static unsigned grid_for_queries(int64_t count) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((count + 255) / 256, (int64_t)device_sms() * 8));
}

// Shared-memory budget per block and warps (queries in flight) per block,
// for `bytes_per_pos` bytes of per-warp state per chain position.
static bool sn_query_shape(const nwcch_topology* t, int64_t bytes_per_pos, int* warps, size_t* smem) {
    const int64_t Dp = t->d.max_depth + 1;
    const int64_t per_warp = ((bytes_per_pos * Dp + 16) + 15) & ~15LL;
    const int64_t budget = 200 * 1024;
    if (per_warp > budget) return false;
    *warps = (int)std::max<int64_t>(1, std::min<int64_t>(16, budget / per_warp));
    *smem = (size_t)(*warps * per_warp);
    return true;
}

template <class K>
static int launch_shape(K kernel, int warps, size_t smem, int64_t nq, int64_t* blocks) {
    NWCCH_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, sms = 0, per_sm = 0;
    NWCCH_CUDA_TRY(cudaGetDevice(&dev));
    NWCCH_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    NWCCH_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 32 * warps, smem));
    const int64_t want = (nq + warps - 1) / warps;
    *blocks = std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * std::max(1, per_sm)));
    return NWCCH_OK;
}

template <class T>
int query_sn_async(nwcch_topology* t, const T* up, const T* dn, const int32_t* s_rank, const int32_t* t_rank,
                   int64_t nq, int64_t* dist, cudaStream_t s, bool allow_alloc, bool* used) {
    int w64 = 0;
    size_t smem64 = 0;
    *used = false;
    if (!t->sn_plan || !sn_query_shape(t, 20, &w64, &smem64)) return NWCCH_OK;
    const SnDev& S = static_cast<SnPlan*>(t->sn_plan)->dev;
    const StreamSlot slot = stream_slot(t, s);
    unsigned int* maxabs = reinterpret_cast<unsigned int*>(slot.counters + 3);
    int* err = slot.err;
    if (sizeof(T) == 4) {
        // 32-bit labels when the metric's values allow them (decided on the
        // device: each kernel returns at once when the batch is not its own)
        NWCCH_CUDA_TRY(cudaMemsetAsync(maxabs, 0, sizeof(unsigned int), s));
        k_maxabs<<<grid_for_queries(t->d.m_plus), 256, 0, s>>>(reinterpret_cast<const int32_t*>(up),
                                                               reinterpret_cast<const int32_t*>(dn), t->d.m_plus,
                                                               maxabs);
        const int64_t Dp = t->d.max_depth + 1;
        const int64_t per_warp = ((12 * Dp + 16) + 15) & ~15LL;
        const auto* u32 = reinterpret_cast<const int32_t*>(up);
        const auto* d32 = reinterpret_cast<const int32_t*>(dn);
        const bool force_global = getenv("NWCCH_QUERY_GLOBAL_LABELS") != nullptr;  // for tests
        // register cap: MINB = 2 holds 64 registers (two 512-thread blocks
        // per SM) at the price of a few spills; MINB = 1 leaves the compiler free
        // 3: chunk labels and row offsets in registers (the most registers)
        auto kern = t->tune.query_occupancy == 3   ? k_query_sn32<1, true>
                    : t->tune.query_occupancy == 2 ? k_query_sn32<2, false>
                                                   : k_query_sn32<1, false>;
        const size_t cta_smem = (size_t)(((12 * Dp + 16) + 15) & ~15LL);
        if (nq <= t->tune.query_cta_max && cta_smem <= 200 * 1024) {
            // few queries: a CTA per query, 16 warps when there are at most
            // as many queries as SMs, else 8
            int64_t blocks = 0;
            const int rows = t->tune.query_cta_dense_rows;
            if (nq <= t->tune.query_cta_wide_max) {
                int rc = launch_shape(k_query_sn32_cta<16>, 16, cta_smem, nq * 16, &blocks);
                if (rc) return rc;
                k_query_sn32_cta<16><<<(unsigned)blocks, 512, cta_smem, s>>>(t->d, S, u32, d32, s_rank, t_rank, nq,
                                                                            dist, maxabs, err, rows);
            } else {
                int rc = launch_shape(k_query_sn32_cta<8>, 8, cta_smem, nq * 8, &blocks);  // one query per CTA
                if (rc) return rc;
                k_query_sn32_cta<8><<<(unsigned)blocks, 256, cta_smem, s>>>(t->d, S, u32, d32, s_rank, t_rank, nq,
                                                                           dist, maxabs, err, rows);
            }
        } else if (allow_alloc && (force_global || per_warp > t->tune.query_smem_labels_max)) {
            // deep tree: labels in global scratch, occupancy set by registers
            int64_t blocks = 0;
            int rc = launch_shape(kern, 4, 0, nq, &blocks);
            if (rc) return rc;
            void* scratch = nullptr;
            NWCCH_CUDA_TRY(cudaMallocAsync(&scratch, (size_t)(blocks * 4 * per_warp), s));
            kern<<<(unsigned)blocks, 128, 0, s>>>(t->d, S, u32, d32, s_rank, t_rank, nq, dist, maxabs,
                                                          static_cast<unsigned char*>(scratch), err,
                                                          t->tune.query_dense_rows);
            const cudaError_t launch = cudaGetLastError();
            NWCCH_CUDA_TRY(cudaFreeAsync(scratch, s));
            NWCCH_CUDA_TRY(launch);
        } else {
            int w32 = 0;
            size_t smem32 = 0;
            if (sn_query_shape(t, 12, &w32, &smem32)) {
                int64_t blocks = 0;
                int rc = launch_shape(kern, w32, smem32, nq, &blocks);
                if (rc) return rc;
                kern<<<(unsigned)blocks, 32 * w32, smem32, s>>>(t->d, S, u32, d32, s_rank, t_rank, nq, dist,
                                                                        maxabs, nullptr, err,
                                                                        t->tune.query_dense_rows);
            }
        }
    }
    int64_t blocks = 0;
    int rc = launch_shape(k_query_sn<T>, w64, smem64, nq, &blocks);
    if (rc) return rc;
    k_query_sn<T><<<(unsigned)blocks, 32 * w64, smem64, s>>>(t->d, S, up, dn, s_rank, t_rank, nq, dist, maxabs,
                                                             err, t->tune.query_dense_rows);
    NWCCH_CUDA_TRY(cudaGetLastError());
    *used = true;
    return NWCCH_OK;
}

template int query_sn_async<int32_t>(nwcch_topology*, const int32_t*, const int32_t*, const int32_t*,
                                     const int32_t*, int64_t, int64_t*, cudaStream_t, bool, bool*);
template int query_sn_async<int64_t>(nwcch_topology*, const int64_t*, const int64_t*, const int32_t*,
                                     const int32_t*, int64_t, int64_t*, cudaStream_t, bool, bool*);

}  // namespace nwcch
