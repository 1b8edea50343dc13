// Kernels of the supernodal customization (included by supernodal.cu).
//
// Arithmetic policies. Exact<T> relaxes with the saturating sum of common.cuh
// (the reference semantics, storage int32 or int64). FastI32 is the int32
// path on the DPX min-plus instruction: operands are stored "compact" (no
// path = CINF = 2^30-1, finite values within +-2^28), so a + b never
// overflows int32, finite sums stay within +-2^29 and sums involving no-path
// are >= 2^30-1-2^28 > 2^29. A block takes the fast path only if every value
// it reads is within +-2^28 and (for recurrences that feed results back as
// operands) every value it would write is too; otherwise it recomputes with
// Exact from the unchanged inputs. Within those bounds both paths are the
// same integer arithmetic, so the result does not depend on the path.
#pragma once

#include <type_traits>

#include "common.cuh"

namespace nwcch {

struct FastI32 {
    using V = int32_t;
    static constexpr int32_t CINF = (1 << 30) - 1;
    static constexpr int32_t THR = 1 << 29;    // above: no path
    static constexpr int32_t RANGE = 1 << 28;  // finite operands stay within +-RANGE
    __device__ static V from(int32_t x) { return x == INF32 ? CINF : x; }
    __device__ static bool in(int32_t x) { return x == INF32 || (x >= -RANGE && x <= RANGE); }
    __device__ static V clean(V x) { return x > THR ? CINF : x; }
    __device__ static V inf() { return CINF; }
    __device__ static void relax(V& c, V a, V b, int&) { c = __viaddmin_s32(a, b, c); }
    __device__ static bool out_ok(V x) { return x > THR || (x >= -RANGE && x <= RANGE); }
    __device__ static bool finite(V x) { return x <= THR; }
    __device__ static int32_t to(V x) { return x > THR ? INF32 : x; }
};

template <class T>
struct Exact {
    using V = T;
    __device__ static V from(T x) { return x; }
    __device__ static V clean(V x) { return x; }
    __device__ static V inf() { return Lim<T>::INF; }
    __device__ static void relax(V& c, V a, V b, int& e) {
        V s;
        if (splus(a, b, s, e) && s < c) c = s;
    }
    __device__ static bool out_ok(V) { return true; }
    __device__ static bool finite(V x) { return x != Lim<T>::INF; }
    __device__ static T to(V x) { return x; }
};

// Loads of customized values. LdPlain: the arcs a kernel reads were written
// by earlier launches. LdL2: they may have been written by other CTAs of the
// same (persistent) launch before a grid barrier, so the load bypasses L1
// (which is not kept coherent between SMs) and reads L2.
struct LdPlain {
    template <class T>
    __device__ static T ld(const T* p) { return *p; }
};
struct LdL2 {
    template <class T>
    __device__ static T ld(const T* p) {
        if constexpr (sizeof(T) == 4) return (T)__ldcg(reinterpret_cast<const int*>(p));
        else return (T)__ldcg(reinterpret_cast<const long long*>(p));
    }
};

__device__ __forceinline__ void atomic_min_t(int32_t* p, int32_t v) { atomicMin(p, v); }
__device__ __forceinline__ void atomic_min_t(int64_t* p, int64_t v) {
    atomicMin(reinterpret_cast<long long*>(p), (long long)v);
}

// First arc of row r of a supernode's trapezoid (rows shrink by one entry a
// vertex): the closed form of first[s0 + r].
__device__ __forceinline__ int64_t sn_row_base(int64_t base, int32_t cols, int32_t r) {
    return base + (int64_t)r * (cols - 1) - (int64_t)r * (r - 1) / 2;
}

// ------------------------------------------------------------------ panel

// Shared state of one panel block: the panel's diagonal triangle (arcs among
// its own <= 32 vertices) and CT columns of its rows.
template <class V, int CT>
struct PanelSmem {
    V Ud[SN_P][SN_P + 1], Dd[SN_P][SN_P + 1];
    V cU[SN_P][CT], cD[SN_P][CT];
    int64_t rowb[SN_P];
};

// Factor the diagonal triangle, then run the panel recurrence down this
// thread's column. Rows a < r of the panel: for every column c beyond r,
//   U(r, c) <- Dn(a, r) + U(a, c),   Dn(r, c) <- Dn(a, c) + U(a, r).
// The panel recurrence down one column (this thread's) in registers, for a
// panel of at most NP rows: rows at or past pn are neither read nor relaxed.
template <class P, class V, int CT, int NP>
__device__ __forceinline__ void panel_column(PanelSmem<V, CT>& sm, int pn, int& e) {
    const int tid = threadIdx.x;
    V cu[NP], cd[NP];
#pragma unroll
    for (int r = 0; r < NP; r++) {
        cu[r] = r < pn ? sm.cU[r][tid] : P::inf();
        cd[r] = r < pn ? sm.cD[r][tid] : P::inf();
    }
#pragma unroll
    for (int a = 0; a + 1 < NP; a++) {
        if (a + 1 < pn) {
            const V ua = P::clean(cu[a]), da = P::clean(cd[a]);
#pragma unroll
            for (int r = a + 1; r < NP; r++) {
                if (r < pn) {
                    P::relax(cu[r], sm.Dd[a][r], ua, e);
                    P::relax(cd[r], da, sm.Ud[a][r], e);
                }
            }
        }
    }
#pragma unroll
    for (int r = 0; r < NP; r++) {
        if (r < pn) {
            sm.cU[r][tid] = cu[r];
            sm.cD[r][tid] = cd[r];
        }
    }
}

template <class P, class V, int CT>
__device__ void panel_compute(PanelSmem<V, CT>& sm, int pn, bool hasj, int& e) {
    constexpr int RS = CT / 32;  // row stride of the diagonal mapping
    const int tid = threadIdx.x;
    const int c = tid & 31, r0 = tid >> 5;
    // Diagonal triangle, right-looking: step a relaxes every pair a < r < c.
    // Row a + 1 receives its last update in step a and becomes the operand row
    // of step a + 1, so it is stored clean right then (row 0 is clean input).
    for (int a = 0; a + 2 < pn; a++) {
        if (c < pn && c > a + 1) {
            const V uac = sm.Ud[a][c], dac = sm.Dd[a][c];
            int r = a + 1 + ((r0 - a - 1) % RS + RS) % RS;
            for (; r < c; r += RS) {
                V u = sm.Ud[r][c], d = sm.Dd[r][c];
                P::relax(u, sm.Dd[a][r], uac, e);
                P::relax(d, dac, sm.Ud[a][r], e);
                if (r == a + 1) {
                    u = P::clean(u);
                    d = P::clean(d);
                }
                sm.Ud[r][c] = u;
                sm.Dd[r][c] = d;
            }
        }
        __syncthreads();
    }
    // the last row may not have been touched: clean every entry once
    for (int t = tid; t < SN_P * SN_P; t += CT) {
        const int rr = t >> 5, cc = t & 31;
        if (rr < cc && cc < pn) {
            sm.Ud[rr][cc] = P::clean(sm.Ud[rr][cc]);
            sm.Dd[rr][cc] = P::clean(sm.Dd[rr][cc]);
        }
    }
    __syncthreads();
    if (!hasj) return;
    if constexpr (std::is_same<P, FastI32>::value) {
        // the fast path: the thread's column lives in registers (fully
        // unrolled for a bound of 8, 16 or 32 rows, the smallest that holds
        // the panel; constant indices), the diagonal is read by broadcast.
        // The exact path (rare) keeps the column in shared memory, which
        // keeps the kernel's code small.
        if (pn <= 8) panel_column<P, V, CT, 8>(sm, pn, e);
        else if (pn <= 16) panel_column<P, V, CT, 16>(sm, pn, e);
        else panel_column<P, V, CT, SN_P>(sm, pn, e);
    } else {
        for (int a = 0; a + 1 < pn; a++) {
            const V cu = P::clean(sm.cU[a][tid]), cd = P::clean(sm.cD[a][tid]);
#pragma unroll 4
            for (int r = a + 1; r < pn; r++) {
                P::relax(sm.cU[r][tid], sm.Dd[a][r], cu, e);
                P::relax(sm.cD[r][tid], cd, sm.Ud[a][r], e);
            }
        }
    }
}

// Loads the diagonal triangle and the thread's column (converted by P).
// Returns true if some value is outside the fast range (FastI32 only).
template <class P, class T, class V, int CT, class LD = LdPlain>
__device__ bool panel_load(PanelSmem<V, CT>& sm, const T* __restrict__ up, const T* __restrict__ dn, int pn,
                           int i0, int j, bool hasj) {
    // every load of a group is issued before its values are used, so the
    // group's global latencies overlap instead of adding up
    const int tid = threadIdx.x;
    bool bad = false;
    constexpr int DI = SN_P * SN_P / CT;  // diagonal entries per thread
    T du[DI], dd[DI];
#pragma unroll
    for (int q = 0; q < DI; q++) {
        const int t = tid + q * CT, a = t >> 5, c = t & 31;
        du[q] = Lim<T>::INF;
        dd[q] = Lim<T>::INF;
        if (a < c && c < pn) {
            du[q] = LD::ld(up + sm.rowb[a] + c - a - 1);
            dd[q] = LD::ld(dn + sm.rowb[a] + c - a - 1);
        }
    }
    // the diagonal's loads and (for 32-bit values) all of the column's are
    // in flight together: one round trip to memory for the whole panel
    auto put_diag = [&]() {
#pragma unroll
        for (int q = 0; q < DI; q++) {
            const int t = tid + q * CT, a = t >> 5, c = t & 31;
            if (a < c && c < pn) {
                if constexpr (std::is_same<P, FastI32>::value) bad |= !P::in(du[q]) || !P::in(dd[q]);
                sm.Ud[a][c] = P::from(du[q]);
                sm.Dd[a][c] = P::from(dd[q]);
            }
        }
    };
    if (!hasj) put_diag();
    if (hasj) {
        constexpr int G = sizeof(T) == 4 ? SN_P : 8;  // column loads in flight per group
#pragma unroll
        for (int a0 = 0; a0 < SN_P; a0 += G) {
            T cu[G], cd[G];
#pragma unroll
            for (int q = 0; q < G; q++) {
                const int a = a0 + q;
                cu[q] = Lim<T>::INF;
                cd[q] = Lim<T>::INF;
                if (a < pn) {
                    const int64_t idx = sm.rowb[a] + (j - (i0 + a)) - 1;
                    cu[q] = LD::ld(up + idx);
                    cd[q] = LD::ld(dn + idx);
                }
            }
            if (a0 == 0) put_diag();
#pragma unroll
            for (int q = 0; q < G; q++) {
                const int a = a0 + q;
                if (a < pn) {
                    if constexpr (std::is_same<P, FastI32>::value) bad |= !P::in(cu[q]) || !P::in(cd[q]);
                    sm.cU[a][tid] = P::from(cu[q]);
                    sm.cD[a][tid] = P::from(cd[q]);
                }
            }
        }
    }
    return bad;
}

template <class P, class T, class V, int CT>
__device__ void panel_store(PanelSmem<V, CT>& sm, T* __restrict__ up, T* __restrict__ dn, int pn, int i0, int j,
                            bool hasj, bool diag) {
    const int tid = threadIdx.x;
    if (diag)
        for (int t = tid; t < SN_P * SN_P; t += CT) {
            const int a = t >> 5, c = t & 31;
            if (a < c && c < pn) {
                up[sm.rowb[a] + c - a - 1] = P::to(sm.Ud[a][c]);
                dn[sm.rowb[a] + c - a - 1] = P::to(sm.Dd[a][c]);
            }
        }
    if (hasj)
        for (int a = 1; a < pn; a++) {
            const int64_t idx = sm.rowb[a] + (j - (i0 + a)) - 1;
            up[idx] = P::to(sm.cU[a][tid]);
            dn[idx] = P::to(sm.cD[a][tid]);
        }
}

template <class P, class V, int CT>
__device__ bool panel_outputs_ok(const PanelSmem<V, CT>& sm, int pn, bool hasj) {
    const int tid = threadIdx.x;
    bool ok = true;
    for (int t = tid; t < SN_P * SN_P; t += CT) {
        const int a = t >> 5, c = t & 31;
        if (a < c && c < pn) ok &= P::out_ok(sm.Ud[a][c]) && P::out_ok(sm.Dd[a][c]);
    }
    if (hasj)
        for (int a = 0; a < pn; a++) ok &= P::out_ok(sm.cU[a][tid]) && P::out_ok(sm.cD[a][tid]);
    return ok;
}

// One 32-row panel [i0, i0+pn) of a supernode with k >= 2, CT columns per
// block (the item's 128-column tile in 128/CT passes). Block ct == 0 also
// writes the diagonal triangle.
template <class T, int CT>
__global__ void __launch_bounds__(CT) k_sn_panel(DevTopo D, SnDev S, const int32_t* __restrict__ items, int panel,
                                                 T* __restrict__ up, T* __restrict__ dn, int* __restrict__ err) {
    using E = Exact<T>;
    __shared__ PanelSmem<T, CT> sm;
    pdl_wait();
    pdl_launch_dependents();
    up += blockIdx.y * D.m_plus;  // metric blockIdx.y of a metric-major batch
    dn += blockIdx.y * D.m_plus;
    const int32_t s = items[3 * blockIdx.x], ct = items[3 * blockIdx.x + 1];
    const QsNode nd = S.node[s];
    const int32_t k = nd.k, cols = k + nd.b;
    const int i0 = panel * SN_P;
    const int pn = min(SN_P, k - i0);
    const int tid = threadIdx.x;
    int e = 0;
    if (tid < pn) sm.rowb[tid] = sn_row_base(nd.base, cols, i0 + tid);
    __syncthreads();
    for (int pass = 0; pass < 128 / CT; pass++) {
        const int j = i0 + pn + ct * 128 + pass * CT + tid;
        const bool hasj = j < cols;
        const bool diag = ct == 0 && pass == 0;
        bool done = false;
        if constexpr (sizeof(T) == 4) {
            auto& fs = reinterpret_cast<PanelSmem<int32_t, CT>&>(sm);
            const bool bad = panel_load<FastI32, T, int32_t, CT>(fs, up, dn, pn, i0, j, hasj);
            if (!__syncthreads_or(bad)) {
                panel_compute<FastI32, int32_t, CT>(fs, pn, hasj, e);
                const bool ok = panel_outputs_ok<FastI32, int32_t, CT>(fs, pn, hasj);
                if (!__syncthreads_or(!ok)) {
                    panel_store<FastI32, T, int32_t, CT>(fs, up, dn, pn, i0, j, hasj, diag);
                    done = true;
                }
            }
        }
        if (!done) {
            __syncthreads();
            panel_load<E, T, T, CT>(sm, up, dn, pn, i0, j, hasj);
            __syncthreads();
            panel_compute<E, T, CT>(sm, pn, hasj, e);
            panel_store<E, T, T, CT>(sm, up, dn, pn, i0, j, hasj, diag);
        }
        __syncthreads();
    }
    if (e) atomicOr(err, e);
}

// ------------------------------------------------------------------ tiles

// (min,+) tile product over inner rows [ibeg, iend) of a supernode:
//   U(y, z)  <- min_i Dn(i, y) + U(i, z)     (arc y -> z through x = s0+i)
//   Dn(y, z) <- min_i Dn(i, z) + U(i, y)
// for the tile's output rows y (columns abase.. of the trapezoid) and output
// columns z (bbase..). OUT = false: trailing update of `panel`, y ranges over
// the supernode's own later vertices, outputs folded into its own arcs.
// OUT = true: y and z are boundary entries, the inner rows are the whole
// supernode, outputs atomically folded into the ancestors' arcs.
template <class T, int TILE, int MT, bool OUT>
struct TileCtx {
    int32_t s, s0, k, b, cols;
    int ibeg, iend, abase, bbase, alim;
    int64_t base;  // first arc of the trapezoid
};

// The tile of work item `it` (a triple: supernode, row tile, column tile).
template <class T, int TILE, int MT, bool OUT>
__device__ __forceinline__ TileCtx<T, TILE, MT, OUT> tile_ctx(const SnDev& S, const int32_t* it, int panel) {
    TileCtx<T, TILE, MT, OUT> c;
    c.s = it[0];
    const int tr = it[1], tc = it[2];
    const QsNode nd = S.node[c.s];
    c.s0 = nd.s0;
    c.k = nd.k;
    c.b = nd.b;
    c.base = nd.base;
    c.cols = c.k + c.b;
    if (OUT) {
        c.ibeg = 0;
        c.iend = c.k;
        c.abase = c.k + tr * TILE;
        c.bbase = c.k + tc * TILE;
        c.alim = c.cols;
    } else {
        c.ibeg = panel * SN_P;
        c.iend = min(c.k, c.ibeg + SN_P);
        c.abase = c.iend + tr * TILE;
        c.bbase = c.iend + tc * TILE;
        c.alim = c.k;
    }
    return c;
}

template <class V, int TILE, int CH>
struct TileSmem {
    V Ad[CH][TILE], Au[CH][TILE], Bu[CH][TILE], Bd[CH][TILE];
    int64_t rowb[CH];
};

// Runs the product with policy P; returns false (fast policy only) as soon as
// an operand leaves the fast range, leaving the accumulators meaningless.
template <class P, class T, int TILE, int MT, int CH, bool OUT, class LD = LdPlain>
__device__ bool tile_product(const DevTopo& D, const TileCtx<T, TILE, MT, OUT>& c,
                             TileSmem<typename P::V, TILE, CH>& sm, const T* __restrict__ up,
                             const T* __restrict__ dn, typename P::V (&accU)[MT][MT], typename P::V (&accD)[MT][MT],
                             int& e) {
    using V = typename P::V;
    constexpr int TH = TILE / MT;
    constexpr int NT = TH * TH;
    constexpr bool FAST = std::is_same<P, FastI32>::value;
    const int tid = threadIdx.x, ty = tid / TH, tx = tid % TH;
#pragma unroll
    for (int ii = 0; ii < MT; ii++)
#pragma unroll
        for (int jj = 0; jj < MT; jj++) {
            accU[ii][jj] = P::inf();
            accD[ii][jj] = P::inf();
        }
    for (int i0 = c.ibeg; i0 < c.iend; i0 += CH) {
        const int nch = min(CH, c.iend - i0);
        __syncthreads();
        if (tid < CH) sm.rowb[tid] = tid < nch ? sn_row_base(c.base, c.cols, i0 + tid) : 0;
        __syncthreads();
        bool bad = false;
        // all of a thread's loads are issued before any is used (their
        // global latencies overlap), then converted into shared memory
        constexpr int NL = CH * TILE / NT;
        static_assert(CH * TILE % NT == 0, "tile loads split evenly");
        T ad[NL], au[NL], bu[NL], bd[NL];
#pragma unroll
        for (int q = 0; q < NL; q++) {
            const int t = tid + q * NT, a = t / TILE, cc = t % TILE;
            const int ac = c.abase + cc, bc = c.bbase + cc;
            const bool okr = a < nch;
            const int64_t rb = sm.rowb[a] - (i0 + a) - 1;
            ad[q] = (okr && ac < c.alim) ? LD::ld(dn + rb + ac) : Lim<T>::INF;
            au[q] = (okr && ac < c.alim) ? LD::ld(up + rb + ac) : Lim<T>::INF;
            bu[q] = (okr && bc < c.cols) ? LD::ld(up + rb + bc) : Lim<T>::INF;
            bd[q] = (okr && bc < c.cols) ? LD::ld(dn + rb + bc) : Lim<T>::INF;
        }
#pragma unroll
        for (int q = 0; q < NL; q++) {
            const int t = tid + q * NT, a = t / TILE, cc = t % TILE;
            if constexpr (FAST)
                bad |= !FastI32::in(ad[q]) || !FastI32::in(au[q]) || !FastI32::in(bu[q]) || !FastI32::in(bd[q]);
            sm.Ad[a][cc] = P::from(ad[q]);
            sm.Au[a][cc] = P::from(au[q]);
            sm.Bu[a][cc] = P::from(bu[q]);
            sm.Bd[a][cc] = P::from(bd[q]);
        }
        if constexpr (FAST) {
            if (__syncthreads_or(bad)) return false;
        } else {
            __syncthreads();
        }
        for (int a = 0; a < nch; a++) {
            V ad[MT], au[MT], bu[MT], bd[MT];
#pragma unroll
            for (int ii = 0; ii < MT; ii++) {
                ad[ii] = sm.Ad[a][ty + TH * ii];
                au[ii] = sm.Au[a][ty + TH * ii];
                bu[ii] = sm.Bu[a][tx + TH * ii];
                bd[ii] = sm.Bd[a][tx + TH * ii];
            }
#pragma unroll
            for (int ii = 0; ii < MT; ii++)
#pragma unroll
                for (int jj = 0; jj < MT; jj++) {
                    P::relax(accU[ii][jj], ad[ii], bu[jj], e);
                    P::relax(accD[ii][jj], bd[jj], au[ii], e);
                }
        }
    }
    return true;
}

template <class P, class T, int TILE, int MT, bool OUT, class LD = LdPlain>
__device__ void tile_store(const DevTopo& D, const SnDev& S, const TileCtx<T, TILE, MT, OUT>& c, T* __restrict__ up,
                           T* __restrict__ dn, const typename P::V (&accU)[MT][MT],
                           const typename P::V (&accD)[MT][MT]) {
    constexpr int TH = TILE / MT;
    const int tid = threadIdx.x, ty = tid / TH, tx = tid % TH;
#pragma unroll
    for (int ii = 0; ii < MT; ii++)
#pragma unroll
        for (int jj = 0; jj < MT; jj++) {
            const int rr = c.abase + ty + TH * ii, cc = c.bbase + tx + TH * jj;  // trapezoid columns
            if (cc <= rr || cc >= c.cols || rr >= c.alim) continue;
            const bool fu = P::finite(accU[ii][jj]), fd = P::finite(accD[ii][jj]);
            if (!fu && !fd) continue;
            int64_t a;
            if (OUT) {
                const int p = rr - c.k, q = cc - c.k;
                a = S.rel[S.rel_off[c.s] + (int64_t)p * (2 * c.b - p - 1) / 2 + (q - p - 1)];
                if (fu) atomic_min_t(&up[a], (T)P::to(accU[ii][jj]));
                if (fd) atomic_min_t(&dn[a], (T)P::to(accD[ii][jj]));
            } else {
                a = sn_row_base(c.base, c.cols, rr) + (cc - rr - 1);
                if (fu) up[a] = min(LD::ld(up + a), (T)P::to(accU[ii][jj]));
                if (fd) dn[a] = min(LD::ld(dn + a), (T)P::to(accD[ii][jj]));
            }
        }
}

// What a tile's store needs that does not depend on its product, loaded
// before the product so that those loads overlap it: the ancestor arc of
// every output pair (OUT), or the current values of every output arc.
template <class T, int MT, bool OUT>
struct TilePre {
    int32_t a[MT][MT];                        // OUT: arc ids (-1: no output)
    T u[OUT ? 1 : MT][OUT ? 1 : MT], d[OUT ? 1 : MT][OUT ? 1 : MT];  // !OUT: current values
};

template <class T, int TILE, int MT, bool OUT>
__device__ __forceinline__ void tile_prefetch(const SnDev& S, const TileCtx<T, TILE, MT, OUT>& c,
                                              const T* __restrict__ up, const T* __restrict__ dn,
                                              TilePre<T, MT, OUT>& pre) {
    constexpr int TH = TILE / MT;
    const int tid = threadIdx.x, ty = tid / TH, tx = tid % TH;
    const int64_t roff = OUT ? S.rel_off[c.s] : 0;
#pragma unroll
    for (int ii = 0; ii < MT; ii++)
#pragma unroll
        for (int jj = 0; jj < MT; jj++) {
            const int rr = c.abase + ty + TH * ii, cc = c.bbase + tx + TH * jj;
            const bool valid = !(cc <= rr || cc >= c.cols || rr >= c.alim);
            if constexpr (OUT) {
                const int p = rr - c.k, q = cc - c.k;
                pre.a[ii][jj] = valid ? S.rel[roff + (int64_t)p * (2 * c.b - p - 1) / 2 + (q - p - 1)] : -1;
            } else {
                pre.a[ii][jj] = valid ? 1 : -1;
                if (valid) {
                    const int64_t a = sn_row_base(c.base, c.cols, rr) + (cc - rr - 1);
                    pre.u[ii][jj] = up[a];
                    pre.d[ii][jj] = dn[a];
                }
            }
        }
}

template <class P, class T, int TILE, int MT, bool OUT>
__device__ void tile_store_pre(const TileCtx<T, TILE, MT, OUT>& c, T* __restrict__ up, T* __restrict__ dn,
                               const typename P::V (&accU)[MT][MT], const typename P::V (&accD)[MT][MT],
                               const TilePre<T, MT, OUT>& pre) {
    constexpr int TH = TILE / MT;
    const int tid = threadIdx.x, ty = tid / TH, tx = tid % TH;
#pragma unroll
    for (int ii = 0; ii < MT; ii++)
#pragma unroll
        for (int jj = 0; jj < MT; jj++) {
            if (pre.a[ii][jj] < 0) continue;
            const bool fu = P::finite(accU[ii][jj]), fd = P::finite(accD[ii][jj]);
            if (!fu && !fd) continue;
            if constexpr (OUT) {
                const int32_t a = pre.a[ii][jj];
                if (fu) atomic_min_t(&up[a], (T)P::to(accU[ii][jj]));
                if (fd) atomic_min_t(&dn[a], (T)P::to(accD[ii][jj]));
            } else {
                const int rr = c.abase + ty + TH * ii, cc = c.bbase + tx + TH * jj;
                const int64_t a = sn_row_base(c.base, c.cols, rr) + (cc - rr - 1);
                const T nu = (T)P::to(accU[ii][jj]), nv = (T)P::to(accD[ii][jj]);
                if (fu && nu < pre.u[ii][jj]) up[a] = nu;
                if (fd && nv < pre.d[ii][jj]) dn[a] = nv;
            }
        }
}

template <class T, int TILE, int MT, bool OUT>
__global__ void __launch_bounds__((TILE / MT) * (TILE / MT))
    k_sn_tile(DevTopo D, SnDev S, const int32_t* __restrict__ items, int panel, T* __restrict__ up,
              T* __restrict__ dn, int* __restrict__ err) {
    constexpr int CH = sizeof(T) == 4 ? 32 : 16;
    using E = Exact<T>;
    __shared__ TileSmem<T, TILE, CH> sm;
    pdl_wait();
    pdl_launch_dependents();
    up += blockIdx.y * D.m_plus;  // metric blockIdx.y of a metric-major batch
    dn += blockIdx.y * D.m_plus;
    const auto c = tile_ctx<T, TILE, MT, OUT>(S, items + 3 * blockIdx.x, panel);
    TilePre<T, MT, OUT> pre;
    tile_prefetch<T, TILE, MT, OUT>(S, c, up, dn, pre);
    int e = 0;
    bool done = false;
    if constexpr (sizeof(T) == 4) {
        auto& fs = reinterpret_cast<TileSmem<int32_t, TILE, CH>&>(sm);
        int32_t accU[MT][MT], accD[MT][MT];
        if (tile_product<FastI32, T, TILE, MT, CH, OUT>(D, c, fs, up, dn, accU, accD, e)) {
            tile_store_pre<FastI32, T, TILE, MT, OUT>(c, up, dn, accU, accD, pre);
            done = true;
        }
    }
    if (!done) {
        T accU[MT][MT], accD[MT][MT];
        tile_product<E, T, TILE, MT, CH, OUT>(D, c, sm, up, dn, accU, accD, e);
        tile_store_pre<E, T, TILE, MT, OUT>(c, up, dn, accU, accD, pre);
    }
    if (e) atomicOr(err, e);
}

// ------------------------------------------------------------------ small supernodes

// One warp customizes a whole small supernode (k <= 32 rows, trapezoid of at
// most SN_WARP_CAP arcs): the trapezoid's rows are consecutive in the CSR, so
// it is staged into shared memory with coalesced loads; the pivots run in
// order (pivot i relaxes every later row j against row i: the triangles
// (s0+i; s0+j, column l)); then every boundary pair (B[p], B[q]) takes the
// minimum over the k rows and is scattered into the ancestors' arcs by
// atomicMin through `rel`; the trapezoid is written back. Small supernodes
// are most of a road-like graph, where a CTA per panel or 16x16 tile would
// leave nearly all of its threads idle.
template <class T, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_sn_warp(DevTopo D, SnDev S, const int32_t* __restrict__ items,
                                                        int64_t count, T* __restrict__ up, T* __restrict__ dn,
                                                        int* __restrict__ err) {
    __shared__ T su[WARPS][SN_WARP_CAP];
    __shared__ T sd[WARPS][SN_WARP_CAP];
    pdl_wait();
    pdl_launch_dependents();
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    up += blockIdx.y * D.m_plus;
    dn += blockIdx.y * D.m_plus;
    T* U = su[wib];
    T* Dn = sd[wib];
    int e = 0;
    for (int64_t it = (int64_t)blockIdx.x * WARPS + wib; it < count; it += (int64_t)gridDim.x * WARPS) {
        const int32_t sn = items[3 * it];
        const QsNode nd = S.node[sn];
        const int32_t k = nd.k, b = nd.b;
        const int32_t width = k + b;
        const int64_t base = nd.base;
        const int32_t total = (int32_t)sn_trapezoid(k, b);
        // staged 4 loads deep per array, so their latencies overlap
        for (int x0 = 0; x0 < total; x0 += 128) {
            T vu[4], vd[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int x = x0 + 32 * q + lane;
                vu[q] = x < total ? up[base + x] : Lim<T>::INF;
                vd[q] = x < total ? dn[base + x] : Lim<T>::INF;
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int x = x0 + 32 * q + lane;
                if (x < total) {
                    U[x] = vu[q];
                    Dn[x] = vd[q];
                }
            }
        }
        __syncwarp();
        auto ro = [&](int i) { return i * (width - 1) - i * (i - 1) / 2; };  // row i's first arc
        for (int i = 0; i + 1 < k; i++) {
            const int ri = ro(i);
            for (int j = i + 1; j < k; j++) {
                const T dij = Dn[ri + (j - i - 1)], uij = U[ri + (j - i - 1)];
                const int rj = ro(j);
                for (int l = j + 1 + lane; l < width; l += 32) {
                    const T uil = U[ri + (l - i - 1)], dil = Dn[ri + (l - i - 1)];
                    const int ejl = rj + (l - j - 1);
                    T v;
                    if (splus(dij, uil, v, e) && v < U[ejl]) U[ejl] = v;
                    if (splus(dil, uij, v, e) && v < Dn[ejl]) Dn[ejl] = v;
                }
            }
            __syncwarp();
        }
        const int32_t* rel = S.rel + S.rel_off[sn];
        for (int p = 0; p + 1 < b; p++) {
            const int prow = p * (2 * b - p - 1) / 2 - p - 1;  // + q: pair (p, q)
            for (int q = p + 1 + lane; q < b; q += 32) {
                T cu = Lim<T>::INF, cd = Lim<T>::INF;
                for (int i = 0; i < k; i++) {
                    const int ri = ro(i) - i - 1 + k;
                    T v;
                    if (splus(Dn[ri + p], U[ri + q], v, e) && v < cu) cu = v;
                    if (splus(Dn[ri + q], U[ri + p], v, e) && v < cd) cd = v;
                }
                const int32_t a = rel[prow + q];
                if (cu != Lim<T>::INF) atomic_min_t(&up[a], cu);
                if (cd != Lim<T>::INF) atomic_min_t(&dn[a], cd);
            }
        }
        for (int x = lane; x < total; x += 32) {
            up[base + x] = U[x];
            dn[base + x] = Dn[x];
        }
        __syncwarp();
    }
    if (e) atomicOr(err, e);
}


// ------------------------------------------------------------------ tiny supernodes

// One thread customizes a whole tiny supernode (trapezoid of at most
// SN_THREAD_CAP arcs): the same steps as k_sn_warp (stage the trapezoid,
// pivots in order, every boundary pair's minimum scattered into the
// ancestors' arcs, write back), with the thread's arcs interleaved in shared
// memory (arc x of thread t at [x][t], so that the threads of a warp never
// hit the same bank). The bottom levels of a road-like graph hold millions of
// supernodes of 2 to 20 arcs, where a warp per supernode leaves most lanes
// idle.
template <class T, int TT, int CAP>
__global__ void __launch_bounds__(TT) k_sn_thread(DevTopo D, SnDev S, const int32_t* __restrict__ items,
                                                  int64_t count, T* __restrict__ up, T* __restrict__ dn,
                                                  int* __restrict__ err) {
    __shared__ T su[CAP][TT];  // CAP: the plan's trapezoid cap (16 or 32 arcs)
    __shared__ T sd[CAP][TT];
    pdl_wait();
    pdl_launch_dependents();
    const int tid = threadIdx.x;
    up += blockIdx.y * D.m_plus;
    dn += blockIdx.y * D.m_plus;
    int e = 0;
    for (int64_t it = (int64_t)blockIdx.x * TT + tid; it < count; it += (int64_t)gridDim.x * TT) {
        const int32_t sn = items[3 * it];
        const QsNode nd = S.node[sn];
        const int32_t k = nd.k, b = nd.b;
        const int32_t width = k + b;
        const int64_t base = nd.base;
        const int32_t total = (int32_t)sn_trapezoid(k, b);
        if (total > CAP) {  // the plan never hands out such a supernode
            e |= ERR_CAPACITY;
            continue;
        }
        for (int x = 0; x < total; x++) {
            su[x][tid] = up[base + x];
            sd[x][tid] = dn[base + x];
        }
        auto ro = [&](int i) { return i * (width - 1) - i * (i - 1) / 2; };  // row i's first arc
        for (int i = 0; i + 1 < k; i++) {
            const int ri = ro(i);
            for (int j = i + 1; j < k; j++) {
                const T dij = sd[ri + (j - i - 1)][tid], uij = su[ri + (j - i - 1)][tid];
                const int rj = ro(j);
                for (int l = j + 1; l < width; l++) {
                    const T uil = su[ri + (l - i - 1)][tid], dil = sd[ri + (l - i - 1)][tid];
                    const int ejl = rj + (l - j - 1);
                    T v;
                    if (splus(dij, uil, v, e) && v < su[ejl][tid]) su[ejl][tid] = v;
                    if (splus(dil, uij, v, e) && v < sd[ejl][tid]) sd[ejl][tid] = v;
                }
            }
        }
        const int32_t* rel = S.rel + S.rel_off[sn];
        for (int p = 0; p + 1 < b; p++) {
            const int prow = p * (2 * b - p - 1) / 2 - p - 1;  // + q: pair (p, q)
            for (int q = p + 1; q < b; q++) {
                T cu = Lim<T>::INF, cd = Lim<T>::INF;
                for (int i = 0; i < k; i++) {
                    const int ri = ro(i) - i - 1 + k;
                    T v;
                    if (splus(sd[ri + p][tid], su[ri + q][tid], v, e) && v < cu) cu = v;
                    if (splus(sd[ri + q][tid], su[ri + p][tid], v, e) && v < cd) cd = v;
                }
                const int32_t a = rel[prow + q];
                if (cu != Lim<T>::INF) atomic_min_t(&up[a], cu);
                if (cd != Lim<T>::INF) atomic_min_t(&dn[a], cd);
            }
        }
        for (int x = 0; x < total; x++) {
            up[base + x] = su[x][tid];
            dn[base + x] = sd[x][tid];
        }
    }
    if (e) atomicOr(err, e);
}

// ------------------------------------------------------------------ top chain

// Near the root of the supernode tree a level holds one or a few supernodes,
// and one launch per panel, trailing update and outgoing product leaves most
// of the GPU idle while each launch waits for the previous one. k_sn_chain
// runs all of those levels in one cooperative launch: every phase (the items
// of one former launch) is spread over the CTAs, and a grid barrier separates
// consecutive phases. Values written before a barrier are read back through
// L2 (LdL2). int32 storage; the phases and items come from the plan.

// Barrier of all CTAs of the chain launch (co-resident: cooperative launch).
// bar[0] counts arrivals, bar[1] is the generation. A wait that runs past
// spin_limit iterations records ERR_TIMEOUT and returns false; the kernel then
// stops. `extra` (a test hook, normally 0) makes the barrier wait for that
// many arrivals more than the grid has, so that its wait runs out.
__device__ __forceinline__ bool chain_barrier(unsigned int* bar, long long spin_limit, int extra, int* err) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* gen = bar + 1;
        const unsigned int g = *gen;
        __threadfence();
        ok = 1;
        if (atomicAdd(bar, 1u) == gridDim.x + extra - 1) {
            atomicExch(bar, 0u);
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            long long spins = 0;
            while (*gen == g) {
                __nanosleep(32);
                if (++spins > spin_limit) {
                    atomicOr(err, ERR_TIMEOUT);
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok;
}

// One panel item of the chain: rows [i0, i0 + pn) of supernode it[0], the
// CT columns of column tile it[1].
template <int CT>
__device__ void chain_panel(const DevTopo& D, const SnDev& S, const int32_t* it, int panel, int32_t* up,
                            int32_t* dn, int& e, PanelSmem<int32_t, CT>& sm) {
    const int32_t s = it[0], ct = it[1];
    const QsNode nd = S.node[s];
    const int32_t k = nd.k, cols = k + nd.b;
    const int i0 = panel * SN_P;
    const int pn = min(SN_P, k - i0);
    const int tid = threadIdx.x;
    if (tid < pn) sm.rowb[tid] = sn_row_base(nd.base, cols, i0 + tid);
    __syncthreads();
    const int j = i0 + pn + ct * CT + tid;
    const bool hasj = j < cols;
    const bool diag = ct == 0;
    bool done = false;
    const bool bad = panel_load<FastI32, int32_t, int32_t, CT, LdL2>(sm, up, dn, pn, i0, j, hasj);
    if (!__syncthreads_or(bad)) {
        panel_compute<FastI32, int32_t, CT>(sm, pn, hasj, e);
        const bool ok = panel_outputs_ok<FastI32, int32_t, CT>(sm, pn, hasj);
        if (!__syncthreads_or(!ok)) {
            panel_store<FastI32, int32_t, int32_t, CT>(sm, up, dn, pn, i0, j, hasj, diag);
            done = true;
        }
    }
    if (!done) {
        using E = Exact<int32_t>;
        __syncthreads();
        panel_load<E, int32_t, int32_t, CT, LdL2>(sm, up, dn, pn, i0, j, hasj);
        __syncthreads();
        panel_compute<E, int32_t, CT>(sm, pn, hasj, e);
        panel_store<E, int32_t, int32_t, CT>(sm, up, dn, pn, i0, j, hasj, diag);
    }
    __syncthreads();
}

// One 64 x 64 tile item of the chain (trailing update, or outgoing product).
template <bool OUT>
__device__ void chain_tile(const DevTopo& D, const SnDev& S, const int32_t* it, int panel, int32_t* up,
                           int32_t* dn, int& e, TileSmem<int32_t, 64, 32>& sm) {
    const auto c = tile_ctx<int32_t, 64, 4, OUT>(S, it, panel);
    int32_t accU[4][4], accD[4][4];
    if (tile_product<FastI32, int32_t, 64, 4, 32, OUT, LdL2>(D, c, sm, up, dn, accU, accD, e)) {
        tile_store<FastI32, int32_t, 64, 4, OUT, LdL2>(D, S, c, up, dn, accU, accD);
    } else {
        using E = Exact<int32_t>;
        tile_product<E, int32_t, 64, 4, 32, OUT, LdL2>(D, c, sm, up, dn, accU, accD, e);
        tile_store<E, int32_t, 64, 4, OUT, LdL2>(D, S, c, up, dn, accU, accD);
    }
}

// Shared memory of a chain CTA: the larger of a panel's and a tile's.
constexpr size_t chain_smem_bytes() {
    return sizeof(PanelSmem<int32_t, CHAIN_THREADS>) > sizeof(TileSmem<int32_t, 64, 32>)
               ? sizeof(PanelSmem<int32_t, CHAIN_THREADS>)
               : sizeof(TileSmem<int32_t, 64, 32>);
}

// The chain's phases in order; metric m of a metric-major batch is item
// (w / count) of phase-wide index w. Grid: one CTA per SM, co-resident.
__global__ void __launch_bounds__(CHAIN_THREADS, 1)
    k_sn_chain(DevTopo D, SnDev S, const int32_t* __restrict__ items, const ChainPhase* __restrict__ phases,
               int32_t nphases, int32_t* up, int32_t* dn, int* __restrict__ err, unsigned int* bar,
               long long spin_limit, int32_t barrier_extra, int32_t metrics) {
    extern __shared__ __align__(16) unsigned char chain_smem[];
    auto& psm = *reinterpret_cast<PanelSmem<int32_t, CHAIN_THREADS>*>(chain_smem);
    auto& tsm = *reinterpret_cast<TileSmem<int32_t, 64, 32>*>(chain_smem);
    int e = 0;
    for (int32_t p = 0; p < nphases; p++) {
        const ChainPhase ph = phases[p];
        const int64_t total = ph.count * metrics;
        for (int64_t w = blockIdx.x; w < total; w += gridDim.x) {
            const int64_t m = w / ph.count, i = w - m * ph.count;
            int32_t* upm = up + m * D.m_plus;
            int32_t* dnm = dn + m * D.m_plus;
            const int32_t* it = items + 3 * (ph.off + i);
            if (ph.kind == SN_PANEL) chain_panel<CHAIN_THREADS>(D, S, it, ph.panel, upm, dnm, e, psm);
            else if (ph.kind == SN_TRAIL) chain_tile<false>(D, S, it, ph.panel, upm, dnm, e, tsm);
            else chain_tile<true>(D, S, it, 0, upm, dnm, e, tsm);
        }
        if (p + 1 < nphases && !chain_barrier(bar, spin_limit, barrier_extra, err)) break;
    }
    if (e) atomicOr(err, e);
}

}  // namespace nwcch
