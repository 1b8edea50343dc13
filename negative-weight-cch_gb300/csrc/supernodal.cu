// Supernodal customization.
//
// The lower-triangle recurrence of python/cch_nb.py:529-563 is regrouped by
// supernodes (maximal rank runs with nested rows, see supernodal.h). Every
// lower triangle (x; y, z) has its lowest vertex x in exactly one supernode S;
// it is either
//   internal - y in S as well: the (min,+) elimination of S's own dense
//              trapezoid, row by row;
//   outgoing - y, z in the boundary B of S: the (min,+) product
//              Dn(S, B)^T (x) U(S, B), scattered (atomic minimum) into the
//              arcs (y, z) of S's ancestors.
// Supernodes of one level of the supernode tree are independent; a level's
// internal work precedes its outgoing work, and all supernodes below it are
// done first. Integer minima are order independent, so the result equals the
// reference's serial loop bit for bit.
//
// Kernels per level:
//   k_sn_int_small  warp per supernode with k <= 32: row i pushes its pairs;
//   k_sn_panel      big supernodes, one 32-row panel: every CTA factors the
//                   panel's 32x32 diagonal triangle in shared memory, then
//                   each thread runs the panel recurrence down one column in
//                   registers (columns are independent given that triangle);
//   k_sn_tile       (min,+) tile product, for the trailing update of a panel
//                   (plain min into the supernode's own arcs) and for the
//                   outgoing block (atomic min into ancestor arcs).

#include <algorithm>
#include <atomic>
#include <new>
#include <thread>
#include <vector>

#include "common.cuh"
#include "customize.h"
#include "supernodal.h"
#include "topology.h"

namespace nwcch {

constexpr int SN_P = 32;          // panel height
constexpr int SN_SMALL_K = 32;    // supernodes up to this width use the warp kernel
constexpr int PANEL_THREADS = 128;

// ------------------------------------------------------------------ plan

namespace {

template <class X>
int upload_vec(SnPlan* p, const std::vector<X>& v, X** out) {
    void* d = nullptr;
    const size_t bytes = std::max<size_t>(1, v.size()) * sizeof(X);
    if (cudaMalloc(&d, bytes) != cudaSuccess) return NWCCH_ERR_NOMEM;
    p->allocations.push_back(d);
    p->bytes += bytes;
    if (!v.empty() && cudaMemcpy(d, v.data(), v.size() * sizeof(X), cudaMemcpyHostToDevice) != cudaSuccess)
        return NWCCH_ERR_CUDA;
    *out = static_cast<X*>(d);
    return NWCCH_OK;
}

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace

void free_supernodal_plan(SnPlan* p) {
    if (!p) return;
    for (void* a : p->allocations) cudaFree(a);
    delete p;
}

SnPlan* build_supernodal_plan(int64_t n, const int64_t* first, const int32_t* head, const int32_t* parent, int* rc) {
    *rc = NWCCH_OK;
    auto* P = new (std::nothrow) SnPlan();
    if (!P) {
        *rc = NWCCH_ERR_NOMEM;
        return nullptr;
    }
    // supernodes: x joins x+1 when x+1 is its parent and the rows are nested
    std::vector<int32_t> s0v, kv, bv, sid(n);
    for (int64_t x = 0; x < n; x++) {
        const bool joins_prev = x > 0 && parent[x - 1] == x &&
                                (first[x] - first[x - 1]) == (first[x + 1] - first[x]) + 1;
        if (!joins_prev) {
            s0v.push_back((int32_t)x);
            kv.push_back(0);
        }
        kv.back()++;
        sid[x] = (int32_t)s0v.size() - 1;
    }
    const int64_t ns = (int64_t)s0v.size();
    bv.resize(ns);
    std::vector<int32_t> lvl(ns, 0);
    int32_t L = 0;
    for (int64_t s = 0; s < ns; s++) {
        const int64_t last = s0v[s] + kv[s] - 1;
        bv[s] = (int32_t)(first[last + 1] - first[last]);
        const int32_t p = parent[last];
        if (p >= 0) lvl[sid[p]] = std::max(lvl[sid[p]], lvl[s] + 1);
        L = std::max(L, lvl[s] + 1);
    }
    P->nsn = ns;
    P->levels = L;
    // arc ids of (B[p], B[q]) for every supernode, found by merging B's tail
    // into the row of B[p] (chordality puts it there)
    std::vector<int64_t> rel_off(ns + 1, 0);
    for (int64_t s = 0; s < ns; s++) rel_off[s + 1] = rel_off[s] + (int64_t)bv[s] * (bv[s] - 1) / 2;
    std::vector<int32_t> rel(rel_off[ns]);
    {
        std::atomic<int> bad{0};
        const int nth = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> ts;
        for (int th = 0; th < nth; th++)
            ts.emplace_back([&, th] {
                for (int64_t s = th; s < ns; s += nth) {
                    const int32_t b = bv[s];
                    if (b < 2) continue;
                    const int64_t last = s0v[s] + kv[s] - 1;
                    const int32_t* B = head + first[last];
                    int64_t o = rel_off[s];
                    for (int32_t p = 0; p + 1 < b; p++) {
                        const int32_t y = B[p];
                        int64_t pos = first[y];
                        const int64_t end = first[y + 1];
                        for (int32_t q = p + 1; q < b; q++) {
                            while (pos < end && head[pos] < B[q]) pos++;
                            if (pos >= end || head[pos] != B[q]) {
                                bad = 1;
                                return;
                            }
                            rel[o++] = (int32_t)pos;
                        }
                    }
                }
            });
        for (auto& t : ts) t.join();
        if (bad) {
            *rc = NWCCH_ERR_TOPOLOGY;
            delete P;
            return nullptr;
        }
    }
    P->rel_entries = rel_off[ns];
    // work items per level
    std::vector<std::vector<int32_t>> small(L), big(L), out_small(L), out_big(L);
    for (int64_t s = 0; s < ns; s++) {
        const int32_t l = lvl[s];
        if (kv[s] >= 2 && kv[s] <= SN_SMALL_K) small[l].push_back((int32_t)s);
        if (kv[s] > SN_SMALL_K) big[l].push_back((int32_t)s);
        const int32_t b = bv[s];
        if (b >= 2) {
            if (b > 32) {
                const int64_t nt = ceil_div(b, 64);
                for (int64_t tp = 0; tp < nt; tp++)
                    for (int64_t tq = tp; tq < nt; tq++) {
                        out_big[l].push_back((int32_t)s);
                        out_big[l].push_back((int32_t)tp);
                        out_big[l].push_back((int32_t)tq);
                    }
            } else {
                const int64_t nt = ceil_div(b, 16);
                for (int64_t tp = 0; tp < nt; tp++)
                    for (int64_t tq = tp; tq < nt; tq++) {
                        out_small[l].push_back((int32_t)s);
                        out_small[l].push_back((int32_t)tp);
                        out_small[l].push_back((int32_t)tq);
                    }
            }
        }
    }
    std::vector<int32_t> items;
    auto add = [&](int kind, int level, int panel, const std::vector<int32_t>& v) {
        if (v.empty()) return;
        SnLaunch la{kind, level, panel, (int64_t)items.size() / 3, (int64_t)v.size() / 3};
        items.insert(items.end(), v.begin(), v.end());
        P->launches.push_back(la);
    };
    for (int32_t l = 0; l < L; l++) {
        std::vector<int32_t> v;
        for (int32_t s : small[l]) v.insert(v.end(), {s, 0, 0});
        add(SN_INT_SMALL, l, 0, v);
        int32_t maxp = 0;
        for (int32_t s : big[l]) maxp = std::max<int32_t>(maxp, (int32_t)ceil_div(kv[s], SN_P));
        for (int32_t pi = 0; pi < maxp; pi++) {
            std::vector<int32_t> pv, tv;
            for (int32_t s : big[l]) {
                const int64_t k = kv[s], b = bv[s];
                const int64_t i0 = (int64_t)pi * SN_P;
                if (i0 >= k) continue;
                const int64_t pn = std::min<int64_t>(SN_P, k - i0);
                const int64_t ncols = (k + b) - (i0 + pn);
                const int64_t ct = std::max<int64_t>(1, ceil_div(ncols, PANEL_THREADS));
                for (int64_t c = 0; c < ct; c++) pv.insert(pv.end(), {s, (int32_t)c, 0});
                const int64_t nrows = k - i0 - pn;
                if (nrows > 0) {
                    const int64_t tr_n = ceil_div(nrows, 64), tc_n = ceil_div(ncols, 64);
                    for (int64_t tr = 0; tr < tr_n; tr++)
                        for (int64_t tc = tr; tc < tc_n; tc++) tv.insert(tv.end(), {s, (int32_t)tr, (int32_t)tc});
                }
            }
            add(SN_PANEL, l, pi, pv);
            add(SN_TRAIL, l, pi, tv);
        }
        add(SN_OUT_SMALL, l, 0, out_small[l]);
        add(SN_OUT_BIG, l, 0, out_big[l]);
    }
    P->items = (int64_t)items.size() / 3;
    int32_t *d_s0, *d_k, *d_b, *d_rel;
    int64_t* d_rel_off;
    if ((*rc = upload_vec(P, s0v, &d_s0)) || (*rc = upload_vec(P, kv, &d_k)) || (*rc = upload_vec(P, bv, &d_b)) ||
        (*rc = upload_vec(P, rel_off, &d_rel_off)) || (*rc = upload_vec(P, rel, &d_rel)) ||
        (*rc = upload_vec(P, items, &P->d_items))) {
        free_supernodal_plan(P);
        return nullptr;
    }
    P->dev = SnDev{d_s0, d_k, d_b, d_rel_off, d_rel};
    return P;
}

// ------------------------------------------------------------------ kernels

// Extended accumulator of a (min,+) product over storage T: int32 storage
// accumulates in int64 with "no path" as a large sentinel (no branch per
// term); int64 storage uses the saturating sum.
template <class T>
struct Acc;
template <>
struct Acc<int32_t> {
    using V = int64_t;
    static constexpr int64_t BIG = (int64_t)1 << 61;    // any sum >= 2^60 is "no path"
    __device__ static V load(int32_t x) { return x == INF32 ? BIG : (int64_t)x; }
    __device__ static V init() { return BIG; }
    __device__ static void relax(V& acc, V a, V b, int&) { acc = min(acc, a + b); }
    // fold into the stored value; returns the new stored value
    __device__ static int32_t fold(int32_t cur, V acc, int& err) {
        if (acc >= ((int64_t)1 << 60)) return cur;
        int32_t c;
        if (acc > Lim<int32_t>::HI) {
            c = Lim<int32_t>::HI;
            err |= ERR_RANGE;
        } else if (acc < Lim<int32_t>::LO) {
            c = Lim<int32_t>::LO;
            err |= ERR_RANGE;
        } else {
            c = (int32_t)acc;
        }
        return min(cur, c);
    }
    __device__ static bool finite(V acc) { return acc < ((int64_t)1 << 60); }
};
template <>
struct Acc<int64_t> {
    using V = int64_t;
    __device__ static V load(int64_t x) { return x; }
    __device__ static V init() { return INF64; }
    __device__ static void relax(V& acc, V a, V b, int& err) {
        int64_t s;
        if (splus(a, b, s, err)) acc = min(acc, s);
    }
    __device__ static int64_t fold(int64_t cur, V acc, int&) { return min(cur, acc); }
    __device__ static bool finite(V acc) { return acc != INF64; }
};

__device__ __forceinline__ void atomic_min_t(int32_t* p, int32_t v) { atomicMin(p, v); }
__device__ __forceinline__ void atomic_min_t(int64_t* p, int64_t v) {
    atomicMin(reinterpret_cast<long long*>(p), (long long)v);
}

// Internal triangles of a supernode with k <= 32, one warp each: for row i
// (final once rows < i are done), every pair (r, j), i < r < j, relaxes
// arc (r, j) by (i -> r -> ... ) i.e. y = s0+r, z = column j.
template <class T>
__global__ void __launch_bounds__(128) k_sn_int_small(DevTopo D, SnDev S, const int32_t* __restrict__ items,
                                                      int64_t count, T* __restrict__ up, T* __restrict__ dn,
                                                      int* __restrict__ err) {
    const int lane = threadIdx.x & 31;
    const int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    int e = 0;
    for (int64_t it = w; it < count; it += nw) {
        const int32_t s = items[3 * it];
        const int32_t s0 = S.s0[s], k = S.k[s], cols = k + S.b[s];
        for (int i = 0; i + 1 < k; i++) {
            const int64_t bi = D.first[s0 + i];
            for (int r = i + 1; r < k; r++) {
                const T d_ir = dn[bi + r - i - 1], u_ir = up[bi + r - i - 1];
                const int64_t br = D.first[s0 + r];
                for (int j = r + 1 + lane; j < cols; j += 32) {
                    const T u_ij = up[bi + j - i - 1], d_ij = dn[bi + j - i - 1];
                    const int64_t a = br + j - r - 1;
                    T c;
                    if (splus(d_ir, u_ij, c, e) && c < up[a]) up[a] = c;  // y -> x -> z
                    if (splus(d_ij, u_ir, c, e) && c < dn[a]) dn[a] = c;  // z -> x -> y
                }
            }
            __syncwarp();
        }
    }
    if (e) atomicOr(err, e);
}

// One 32-row panel [i0, i0+pn) of a big supernode. Every CTA loads and
// factors the panel's diagonal triangle (arcs among the panel's own vertices)
// in shared memory; CTA 0 writes it back. Each thread then owns one column j
// beyond the panel and runs the panel recurrence down it in registers.
template <class T>
__global__ void __launch_bounds__(PANEL_THREADS) k_sn_panel(DevTopo D, SnDev S, const int32_t* __restrict__ items,
                                                            int panel, T* __restrict__ up, T* __restrict__ dn,
                                                            int* __restrict__ err) {
    __shared__ T Ud[SN_P][SN_P + 1], Dd[SN_P][SN_P + 1];
    __shared__ int64_t rowb[SN_P];
    const int32_t s = items[3 * blockIdx.x], ct = items[3 * blockIdx.x + 1];
    const int32_t s0 = S.s0[s], k = S.k[s], cols = k + S.b[s];
    const int i0 = panel * SN_P;
    const int pn = min(SN_P, k - i0);
    const int tid = threadIdx.x;
    int e = 0;
    if (tid < pn) rowb[tid] = D.first[s0 + i0 + tid];
    __syncthreads();
    for (int t = tid; t < pn * pn; t += blockDim.x) {
        const int a = t / pn, c = t % pn;
        if (a < c) {
            Ud[a][c] = up[rowb[a] + c - a - 1];
            Dd[a][c] = dn[rowb[a] + c - a - 1];
        }
    }
    __syncthreads();
    for (int a = 0; a + 2 < pn; a++) {
        for (int t = tid; t < pn * pn; t += blockDim.x) {
            const int r = t / pn, c = t % pn;
            if (a < r && r < c) {
                T v;
                if (splus(Dd[a][r], Ud[a][c], v, e) && v < Ud[r][c]) Ud[r][c] = v;
                if (splus(Dd[a][c], Ud[a][r], v, e) && v < Dd[r][c]) Dd[r][c] = v;
            }
        }
        __syncthreads();
    }
    if (ct == 0) {
        for (int t = tid; t < pn * pn; t += blockDim.x) {
            const int a = t / pn, c = t % pn;
            if (a < c) {
                up[rowb[a] + c - a - 1] = Ud[a][c];
                dn[rowb[a] + c - a - 1] = Dd[a][c];
            }
        }
    }
    const int j = i0 + pn + ct * PANEL_THREADS + tid;
    if (j < cols) {
        T cu[SN_P], cd[SN_P];
#pragma unroll
        for (int a = 0; a < SN_P; a++)
            if (a < pn) {
                const int64_t idx = rowb[a] + (j - (i0 + a)) - 1;
                cu[a] = up[idx];
                cd[a] = dn[idx];
            }
#pragma unroll
        for (int a = 0; a < SN_P; a++) {
#pragma unroll
            for (int r = a + 1; r < SN_P; r++) {
                if (r < pn) {
                    T v;
                    if (splus(Dd[a][r], cu[a], v, e) && v < cu[r]) cu[r] = v;
                    if (splus(cd[a], Ud[a][r], v, e) && v < cd[r]) cd[r] = v;
                }
            }
        }
#pragma unroll
        for (int a = 1; a < SN_P; a++)
            if (a < pn) {
                const int64_t idx = rowb[a] + (j - (i0 + a)) - 1;
                up[idx] = cu[a];
                dn[idx] = cd[a];
            }
    }
    if (e) atomicOr(err, e);
}

// (min,+) tile product over the rows [ibeg, iend) of a supernode:
//   U(x, y) <- min_i Dn(i, ycol) + U(i, xcol)   (arc y -> z through x = s0+i)
//   Dn(x, y) <- min_i Dn(i, xcol) + U(i, ycol)
// for the tile's "row" columns A (the y of the output arc) and "column"
// columns B (the z). OUT = false: trailing update of panel `panel`, rows are
// the supernode's own vertices after the panel; outputs folded into its own
// arcs. OUT = true: rows and columns are boundary entries, inner rows are the
// whole supernode, outputs atomically folded into the ancestors' arcs.
template <class T, int TILE, int MT, bool OUT>
__global__ void __launch_bounds__((TILE / MT) * (TILE / MT))
    k_sn_tile(DevTopo D, SnDev S, const int32_t* __restrict__ items, int panel, T* __restrict__ up,
              T* __restrict__ dn, int* __restrict__ err) {
    using A = Acc<T>;
    using V = typename A::V;
    constexpr int TH = TILE / MT;        // threads per tile edge
    constexpr int NT = TH * TH;
    constexpr int CH = sizeof(T) == 4 ? 32 : 16;  // inner rows staged per round
    __shared__ T Ad[CH][TILE], Au[CH][TILE], Bu[CH][TILE], Bd[CH][TILE];
    __shared__ int64_t rowb[CH];
    const int32_t s = items[3 * blockIdx.x], tr = items[3 * blockIdx.x + 1], tc = items[3 * blockIdx.x + 2];
    const int32_t s0 = S.s0[s], k = S.k[s], b = S.b[s], cols = k + b;
    int ibeg, iend, abase, bbase, alim;
    if (OUT) {
        ibeg = 0;
        iend = k;
        abase = k + tr * TILE;
        bbase = k + tc * TILE;
        alim = cols;
    } else {
        ibeg = panel * SN_P;
        iend = min(k, ibeg + SN_P);
        abase = iend + tr * TILE;
        bbase = iend + tc * TILE;
        alim = k;
    }
    const int tid = threadIdx.x, ty = tid / TH, tx = tid % TH;
    int e = 0;
    V accU[MT][MT], accD[MT][MT];
#pragma unroll
    for (int ii = 0; ii < MT; ii++)
#pragma unroll
        for (int jj = 0; jj < MT; jj++) {
            accU[ii][jj] = A::init();
            accD[ii][jj] = A::init();
        }
    for (int i0 = ibeg; i0 < iend; i0 += CH) {
        const int nch = min(CH, iend - i0);
        if (tid < CH) rowb[tid] = tid < nch ? D.first[s0 + i0 + tid] : 0;
        __syncthreads();
        for (int t = tid; t < CH * TILE; t += NT) {
            const int a = t / TILE, c = t % TILE;
            const int ac = abase + c, bc = bbase + c;
            const bool okr = a < nch;
            const int64_t rb = rowb[a] - (i0 + a) - 1;
            Ad[a][c] = (okr && ac < alim) ? dn[rb + ac] : Lim<T>::INF;
            Au[a][c] = (okr && ac < alim) ? up[rb + ac] : Lim<T>::INF;
            Bu[a][c] = (okr && bc < cols) ? up[rb + bc] : Lim<T>::INF;
            Bd[a][c] = (okr && bc < cols) ? dn[rb + bc] : Lim<T>::INF;
        }
        __syncthreads();
        for (int a = 0; a < nch; a++) {
            V ad[MT], au[MT], bu[MT], bd[MT];
#pragma unroll
            for (int ii = 0; ii < MT; ii++) {
                ad[ii] = A::load(Ad[a][ty + TH * ii]);
                au[ii] = A::load(Au[a][ty + TH * ii]);
                bu[ii] = A::load(Bu[a][tx + TH * ii]);
                bd[ii] = A::load(Bd[a][tx + TH * ii]);
            }
#pragma unroll
            for (int ii = 0; ii < MT; ii++)
#pragma unroll
                for (int jj = 0; jj < MT; jj++) {
                    A::relax(accU[ii][jj], ad[ii], bu[jj], e);
                    A::relax(accD[ii][jj], bd[jj], au[ii], e);
                }
        }
        __syncthreads();
    }
#pragma unroll
    for (int ii = 0; ii < MT; ii++)
#pragma unroll
        for (int jj = 0; jj < MT; jj++) {
            const int rr = abase + ty + TH * ii, cc = bbase + tx + TH * jj;  // columns of the trapezoid
            if (cc <= rr || cc >= cols || rr >= alim) continue;
            if (OUT) {
                const int p = rr - k, q = cc - k;
                const int64_t a = S.rel[S.rel_off[s] + (int64_t)p * (2 * b - p - 1) / 2 + (q - p - 1)];
                if (A::finite(accU[ii][jj])) atomic_min_t(&up[a], A::fold(Lim<T>::INF, accU[ii][jj], e));
                if (A::finite(accD[ii][jj])) atomic_min_t(&dn[a], A::fold(Lim<T>::INF, accD[ii][jj], e));
            } else {
                const int64_t a = D.first[s0 + rr] + (cc - rr - 1);
                up[a] = A::fold(up[a], accU[ii][jj], e);
                dn[a] = A::fold(dn[a], accD[ii][jj], e);
            }
        }
    if (e) atomicOr(err, e);
}

template <class T>
int run_supernodal(nwcch_topology* t, SnPlan* P, const int32_t* w, T* up, T* dn, cudaStream_t s) {
    int rc = base_init<T>(t, w, up, dn, s);
    if (rc) return rc;
    const DevTopo& D = t->d;
    for (const SnLaunch& la : P->launches) {
        const int32_t* it = P->d_items + 3 * la.off;
        switch (la.kind) {
            case SN_INT_SMALL: {
                const int64_t blocks = std::min<int64_t>(ceil_div(la.count, 4), 152 * 64);
                k_sn_int_small<T><<<(unsigned)blocks, 128, 0, s>>>(D, P->dev, it, la.count, up, dn, t->err);
                break;
            }
            case SN_PANEL:
                k_sn_panel<T><<<(unsigned)la.count, PANEL_THREADS, 0, s>>>(D, P->dev, it, la.panel, up, dn, t->err);
                break;
            case SN_TRAIL:
                k_sn_tile<T, 64, 4, false><<<(unsigned)la.count, 256, 0, s>>>(D, P->dev, it, la.panel, up, dn, t->err);
                break;
            case SN_OUT_BIG:
                k_sn_tile<T, 64, 4, true><<<(unsigned)la.count, 256, 0, s>>>(D, P->dev, it, 0, up, dn, t->err);
                break;
            case SN_OUT_SMALL:
                k_sn_tile<T, 16, 2, true><<<(unsigned)la.count, 64, 0, s>>>(D, P->dev, it, 0, up, dn, t->err);
                break;
        }
    }
    return cudaGetLastError() == cudaSuccess ? NWCCH_OK : NWCCH_ERR_CUDA;
}

template int run_supernodal<int32_t>(nwcch_topology*, SnPlan*, const int32_t*, int32_t*, int32_t*, cudaStream_t);
template int run_supernodal<int64_t>(nwcch_topology*, SnPlan*, const int32_t*, int64_t*, int64_t*, cudaStream_t);

}  // namespace nwcch
