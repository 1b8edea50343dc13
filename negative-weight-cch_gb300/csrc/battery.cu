// Battery-constrained CCH profiles on the device (python/cch_nb_battery.py).
//
// A piece (in, cost, out) is the state-of-charge function
// f(b) = min(out, b - cost) for b >= in (python/cch_battery.py:1-40); a
// profile is the list of pieces of one shortcut direction d = 2*arc +
// (0 up, 1 down) that survive merging its candidates in turn.
//
// Customization, pull form. The reference pushes every lower triangle
// (x; y, z) into the arc (y, z) for x ascending (python/cch_nb_battery.py:
// 84-182); merged one at a time with a tolerance in the dominance test, the
// order of the candidates decides which of two near-equal pieces survives.
// Here the arcs are taken level by level (the level of an arc's lower
// endpoint y; every lower triangle of (y, z) has x in a lower level, so its
// sources are final), one warp per arc (y, z), which merges that arc's
// candidates in the reference's order: its original arcs in input order,
// then its lower triangles by ascending x, each triangle's pieces in the
// reference's (source piece, target piece) order. The profiles are then the
// reference's, piece for piece.
//
// A profile of up to 32 pieces lives in registers, piece l in lane l: one
// merge is a ballot over the pieces that dominate the candidate, a ballot
// over the pieces it dominates, a shuffle compaction and an append. Longer
// profiles continue in the warp's global buffer. The lower triangles of
// (y, z) are the x of y's downward list whose rows hold z: 32 are tested at
// a time (binary search of z in x's row), and the lanes compose the
// candidates of single-piece sources (most of them) before the merges run in
// order. Finished profiles are appended to a pool at atomic offsets; counts
// and offsets index it. A pool or buffer that overflows is flagged, grown
// by the host, and the customization runs again.
//
// Queries (python/cch_nb_battery.py:296-343): one warp per (s, t, b0). The
// upward pass over s's ancestors in increasing rank pushes each label through
// the up profiles of the vertex's arcs (lanes over arcs; the heads of a row
// are distinct); the downward pass over t's ancestors in decreasing rank
// takes the warp maximum of the down profiles applied to the labels above.
// Labels are indexed by depth. Maxima do not depend on the order, so the
// answers equal the reference's exactly on the same profiles.

#include <algorithm>
#include <cmath>
#include <new>
#include <vector>

#include "common.cuh"
#include "topology.h"

namespace nwcch {

namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr double EPS = 1e-9;
constexpr int BAT_POOL_OVERFLOW = 1;
constexpr int BAT_WORK_OVERFLOW = 2;
constexpr int LEVEL_WARPS = 4;
constexpr int LEVEL_BLOCKS = 152 * 8;  // resident blocks of the level kernel; one buffer slot per warp
constexpr int QUERY_WARPS = 4;

struct Piece {
    double i, c, o;
};

struct BatStatus {
    unsigned long long pool_used;
    int flags;
    int largest;
};

struct BatPlan {
    int32_t* arcs = nullptr;   // [m+] arcs by level of their tail, then tail rank
    int32_t* dtail = nullptr;  // [m+] tail of darc[p] (the x of y's downward list)
};

// python/cch_nb_battery.py:16-44: f(b) >= g(b) on [0, M] (with tolerance),
// tested where the difference can be extreme: g's feasibility start, M and
// either breakpoint.
__device__ __forceinline__ bool dominates(const Piece& f, const Piece& g, double M) {
    if (f.i > g.i + EPS) return false;
    const double lo = g.i - EPS, hi = M + EPS;
    const double bs[4] = {g.i, M, f.o + f.c, g.o + g.c};
#pragma unroll
    for (int t = 0; t < 4; t++) {
        const double b = bs[t];
        if (lo <= b && b <= hi) {
            if (b < f.i - EPS) return false;
            double vf = b - f.c;
            if (f.o < vf) vf = f.o;
            double vg = b - g.c;
            if (g.o < vg) vg = g.o;
            if (vf < vg - EPS) return false;
        }
    }
    return true;
}

// python/cch_nb_battery.py:159-173: f then g.
__device__ __forceinline__ bool compose(const Piece& f, const Piece& g, double M, Piece& h) {
    if (f.o < g.i - EPS) return false;
    const double hi = f.i > g.i + f.c ? f.i : g.i + f.c;
    if (hi > M + EPS) return false;
    const double hc = f.c + g.c;
    double ho = g.o;
    if (f.o - g.c < ho) ho = f.o - g.c;
    if (M - hc < ho) ho = M - hc;
    h.i = hi;
    h.c = hc;
    h.o = ho;
    return true;
}

// Position of the n-th (0-based) set bit of m; n < popc(m).
__device__ __forceinline__ int nth_set_bit(unsigned m, int n) {
    int pos = 0;
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        const unsigned low = m & ((1u << s) - 1u);
        const int c = __popc(low);
        if (n >= c) {
            n -= c;
            m >>= s;
            pos += s;
        } else {
            m = low;
        }
    }
    return pos;
}

__device__ __forceinline__ Piece shfl_piece(const Piece& p, int src) {
    return Piece{__shfl_sync(FULL, p.i, src), __shfl_sync(FULL, p.c, src), __shfl_sync(FULL, p.o, src)};
}

// The profile being built: in registers (lane l holds piece l) while it has
// at most 32 pieces, else in buf. n and glob are warp-uniform.
struct Work {
    Piece r;
    int n;
    bool glob;
    Piece* buf;
};

struct BatArgs {
    const double* w;
    double M;
    const int32_t* arcs;
    const int32_t* dtail;
    int32_t* cnt;
    int64_t* pos;
    Piece* pool;
    int64_t pool_cap;
    Piece* gbuf;  // 2 * gcap pieces per warp slot
    int32_t gcap;
    BatStatus* status;
    unsigned long long* next;  // per level: arcs handed out
};

// python/cch_nb_battery.py:186-254: one candidate into the profile.
__device__ void merge(Work& W, const Piece& h, double M, int32_t gcap, int lane, int& flags) {
    if (!W.glob) {
        const bool live = lane < W.n;
        if (__any_sync(FULL, live && dominates(W.r, h, M))) return;
        const bool keep = live && !dominates(h, W.r, M);
        const unsigned km = __ballot_sync(FULL, keep);
        const int k = __popc(km);
        Piece g = shfl_piece(W.r, lane < k ? nth_set_bit(km, lane) : lane);
        if (k < 32) {
            if (lane == k) g = h;
            W.r = g;
            W.n = k + 1;
        } else {  // 33 pieces: continue in the global buffer (gcap >= 64)
            W.buf[lane] = g;
            if (lane == 0) W.buf[32] = h;
            W.n = 33;
            W.glob = true;
            __syncwarp();
        }
        return;
    }
    for (int b = 0; b < W.n; b += 32) {
        const bool live = b + lane < W.n;
        Piece g{0.0, 0.0, 0.0};
        if (live) g = W.buf[b + lane];
        if (__any_sync(FULL, live && dominates(g, h, M))) return;
    }
    int k = 0;
    for (int b = 0; b < W.n; b += 32) {
        const bool live = b + lane < W.n;
        Piece g{0.0, 0.0, 0.0};
        if (live) g = W.buf[b + lane];
        const bool keep = live && !dominates(h, g, M);
        const unsigned km = __ballot_sync(FULL, keep);
        // writes land at or below every position this round has read
        if (keep) W.buf[k + __popc(km & ((1u << lane) - 1u))] = g;
        k += __popc(km);
    }
    if (k + 1 > gcap) {
        flags |= BAT_WORK_OVERFLOW;
        W.n = k;
        __syncwarp();
        return;
    }
    if (lane == 0) W.buf[k] = h;
    W.n = k + 1;
    __syncwarp();
    if (W.n <= 32) {
        W.r = lane < W.n ? W.buf[lane] : Piece{0.0, 0.0, 0.0};
        W.glob = false;
    }
}

// The candidates of one lower triangle side with general source profiles:
// f pieces (direction df) then g pieces (dg), f-major as the reference.
__device__ void merge_triangle(Work& W, const BatArgs& A, int64_t df, int64_t dg, int lane, int& flags) {
    const int32_t na = A.cnt[df], nb = A.cnt[dg];
    if (na == 0 || nb == 0) return;
    const int64_t fa = A.pos[df], ga = A.pos[dg];
    const int64_t tot = (int64_t)na * nb;
    for (int64_t qb = 0; qb < tot; qb += 32) {
        const int64_t q = qb + lane;
        Piece h{0.0, 0.0, 0.0};
        bool ok = false;
        if (q < tot) ok = compose(A.pool[fa + q / nb], A.pool[ga + q % nb], A.M, h);
        unsigned vm = __ballot_sync(FULL, ok);
        while (vm) {
            const int src = __ffs(vm) - 1;
            vm &= vm - 1;
            merge(W, shfl_piece(h, src), A.M, A.gcap, lane, flags);
        }
    }
}

__device__ void finish(const Work& W, const BatArgs& A, int64_t d, int lane, int& flags, int& seen) {
    const int n = W.n;
    unsigned long long p = 0;
    if (lane == 0 && n > 0) p = atomicAdd(&A.status->pool_used, (unsigned long long)n);
    p = __shfl_sync(FULL, p, 0);
    if (n > 0 && (int64_t)(p + n) > A.pool_cap) {
        flags |= BAT_POOL_OVERFLOW;
        if (lane == 0) {
            A.cnt[d] = 0;
            A.pos[d] = 0;
        }
        return;
    }
    if (!W.glob) {
        if (lane < n) A.pool[p + lane] = W.r;
    } else {
        for (int t = lane; t < n; t += 32) A.pool[p + t] = W.buf[t];
    }
    if (lane == 0) {
        A.cnt[d] = n;
        A.pos[d] = (int64_t)p;
        if (n > seen) seen = max(n, atomicMax(&A.status->largest, n));
    }
}

__device__ __forceinline__ int side_kind(int32_t nf, int32_t ng) {
    return (nf == 0 || ng == 0) ? 0 : (nf == 1 && ng == 1) ? 1 : 2;
}

__device__ void customize_arc(const DevTopo& D, const BatArgs& A, int32_t j, Piece* gb, int lane, int& flags,
                              int& seen) {
    const double M = A.M;
    const int32_t y = D.tail[j], z = D.head[j];
    Work U{Piece{0.0, 0.0, 0.0}, 0, false, gb};
    Work V{Piece{0.0, 0.0, 0.0}, 0, false, gb + A.gcap};
    // python/cch_nb_battery.py:67-82: the original arcs onto j, input order
    for (int64_t e = D.aeoff[j]; e < D.aeoff[j + 1]; e++) {
        const int32_t k = D.aeidx[e];
        const double c = A.w[k];
        Piece h;
        if (c >= 0) {
            if (c > M) continue;
            h = Piece{c, c, M - c};
        } else {
            h = Piece{0.0, c, M};
        }
        if (D.e_up[k]) merge(U, h, M, A.gcap, lane, flags);
        else merge(V, h, M, A.gcap, lane, flags);
    }
    // lower triangles (x; y, z), x ascending:
    //   up(y,z)   <- down(x,y) then up(x,z)
    //   down(y,z) <- down(x,z) then up(x,y)
    const int64_t p1 = D.doff[y + 1];
    for (int64_t pb = D.doff[y]; pb < p1; pb += 32) {
        const int64_t p = pb + lane;
        int64_t i = -1, kk = -1;
        if (p < p1) {
            i = D.darc[p];
            const int32_t x = A.dtail[p];
            const int64_t end = D.first[x + 1];
            int64_t lo = i + 1, hi = end;
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (D.head[mid] < z) lo = mid + 1;
                else hi = mid;
            }
            if (lo < end && D.head[lo] == z) kk = lo;
        }
        unsigned hits = __ballot_sync(FULL, kk >= 0);
        if (!hits) continue;
        int ku = 0, kd = 0;
        bool oku = false, okd = false;
        Piece hu{0.0, 0.0, 0.0}, hd{0.0, 0.0, 0.0};
        if (kk >= 0) {
            ku = side_kind(A.cnt[2 * i + 1], A.cnt[2 * kk]);
            kd = side_kind(A.cnt[2 * kk + 1], A.cnt[2 * i]);
            if (ku == 1) oku = compose(A.pool[A.pos[2 * i + 1]], A.pool[A.pos[2 * kk]], M, hu);
            if (kd == 1) okd = compose(A.pool[A.pos[2 * kk + 1]], A.pool[A.pos[2 * i]], M, hd);
        }
        while (hits) {
            const int src = __ffs(hits) - 1;
            hits &= hits - 1;
            const int su = __shfl_sync(FULL, ku, src), sd = __shfl_sync(FULL, kd, src);
            const int64_t si = __shfl_sync(FULL, i, src), sk = __shfl_sync(FULL, kk, src);
            if (su == 1) {
                if (__shfl_sync(FULL, (int)oku, src)) merge(U, shfl_piece(hu, src), M, A.gcap, lane, flags);
            } else if (su == 2) {
                merge_triangle(U, A, 2 * si + 1, 2 * sk, lane, flags);
            }
            if (sd == 1) {
                if (__shfl_sync(FULL, (int)okd, src)) merge(V, shfl_piece(hd, src), M, A.gcap, lane, flags);
            } else if (sd == 2) {
                merge_triangle(V, A, 2 * sk + 1, 2 * si, lane, flags);
            }
        }
    }
    finish(U, A, 2 * (int64_t)j, lane, flags, seen);
    finish(V, A, 2 * (int64_t)j + 1, lane, flags, seen);
}

__global__ void __launch_bounds__(32 * LEVEL_WARPS) k_bat_level(DevTopo D, BatArgs A, int64_t a0, int64_t a1,
                                                                 int32_t level) {
    const int lane = threadIdx.x & 31;
    const int64_t slot = (int64_t)blockIdx.x * LEVEL_WARPS + (threadIdx.x >> 5);
    Piece* gb = A.gbuf + slot * 2 * (int64_t)A.gcap;
    int flags = 0, seen = 0;
    for (;;) {
        unsigned long long idx = 0;
        if (lane == 0) idx = atomicAdd(&A.next[level], 1ull);
        idx = __shfl_sync(FULL, idx, 0);
        const int64_t e = a0 + (int64_t)idx;
        if (e >= a1) break;
        customize_arc(D, A, A.arcs[e], gb, lane, flags, seen);
    }
    flags = (int)__reduce_or_sync(FULL, (unsigned)flags);
    if (flags && lane == 0) atomicOr(&A.status->flags, flags);
}

__global__ void k_dtail(const int32_t* __restrict__ darc, const int32_t* __restrict__ tail, int64_t m_plus,
                        int32_t* __restrict__ dtail) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < m_plus; p += (int64_t)gridDim.x * blockDim.x)
        dtail[p] = tail[darc[p]];
}

struct BatDev {
    const int32_t* cnt;
    const int64_t* pos;
    const Piece* pool;
};

// python/cch_nb_battery.py:272-293
__device__ __forceinline__ double eval_profile(const BatDev& B, int64_t d, double b) {
    double best = -INFINITY;
    const int32_t n = B.cnt[d];
    const Piece* p = B.pool + B.pos[d];
    for (int32_t t = 0; t < n; t++) {
        const Piece f = p[t];
        if (b >= f.i - EPS) {
            double v = b - f.c;
            if (f.o < v) v = f.o;
            if (v > best) best = v;
        }
    }
    return best;
}

__global__ void __launch_bounds__(32 * QUERY_WARPS)
    k_bat_query(DevTopo D, BatDev B, const int32_t* __restrict__ s_rank, const int32_t* __restrict__ t_rank,
                const double* __restrict__ b0, int64_t nq, double* __restrict__ out, unsigned char* scratch,
                int64_t per_warp, int* err) {
    const int lane = threadIdx.x & 31;
    const int64_t gw = (int64_t)blockIdx.x * QUERY_WARPS + (threadIdx.x >> 5);
    const int64_t nw = (int64_t)gridDim.x * QUERY_WARPS;
    const int64_t Dp = D.max_depth + 1;
    double* soc = reinterpret_cast<double*>(scratch + gw * per_warp);
    double* dsoc = soc + Dp;
    int32_t* cs = reinterpret_cast<int32_t*>(dsoc + Dp);
    int32_t* ct = cs + Dp;
    int e = 0;
    for (int64_t q = gw; q < nq; q += nw) {
        const int32_t s = s_rank[q], t = t_rank[q];
        if (s < 0 || s >= D.n || t < 0 || t >= D.n) {
            if (lane == 0) out[q] = -INFINITY;
            e |= ERR_ARG;
            continue;
        }
        const int32_t ds = D.depth[s], dt = D.depth[t];
        for (int32_t d = lane; d <= ds; d += 32) soc[d] = -INFINITY;
        __syncwarp();
        if (lane == 0) soc[ds] = b0[q];
        __syncwarp();
        int32_t d = ds;
        for (int32_t x = s; x >= 0; x = D.parent[x], d--) {
            if (lane == 0) cs[d] = x;
            const double bx = soc[d];
            if (bx > -INFINITY) {
                const int64_t a1 = D.first[x + 1];
                for (int64_t a = D.first[x] + lane; a < a1; a += 32) {
                    const double v = eval_profile(B, 2 * a, bx);
                    const int32_t hd = D.hdep[a];
                    if (v > soc[hd]) soc[hd] = v;
                }
            }
            __syncwarp();
        }
        d = dt;
        for (int32_t x = t; x >= 0; x = D.parent[x], d--)
            if (lane == 0) ct[d] = x;
        __syncwarp();
        for (d = 0; d <= dt; d++) {
            const int32_t x = ct[d];
            double best = (d <= ds && cs[d] == x) ? soc[d] : -INFINITY;
            const int64_t a1 = D.first[x + 1];
            for (int64_t a = D.first[x] + lane; a < a1; a += 32) {
                const double by = dsoc[D.hdep[a]];
                if (by > -INFINITY) {
                    const double v = eval_profile(B, 2 * a + 1, by);
                    if (v > best) best = v;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) best = fmax(best, __shfl_xor_sync(FULL, best, o));
            if (lane == 0) dsoc[d] = best;
            __syncwarp();
        }
        if (lane == 0) out[q] = dsoc[dt];
        __syncwarp();
    }
    if (e && lane == 0) atomicOr(err, e);
}

void free_battery_plan(nwcch_topology* t) {
    auto* P = static_cast<BatPlan*>(t->battery_plan);
    if (!P) return;
    cudaFree(P->arcs);
    cudaFree(P->dtail);
    delete P;
    t->battery_plan = nullptr;
}

int get_plan(nwcch_topology* t, BatPlan** out) {
    std::lock_guard<std::mutex> lock(t->mu);
    if (t->battery_plan) {
        *out = static_cast<BatPlan*>(t->battery_plan);
        return NWCCH_OK;
    }
    const int64_t n = t->d.n, mp = t->d.m_plus;
    std::vector<int64_t> first(n + 1);
    std::vector<int32_t> verts(n);
    NWCCH_CUDA_TRY(cudaMemcpy(first.data(), t->d.first, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost));
    if (n) NWCCH_CUDA_TRY(cudaMemcpy(verts.data(), t->level_verts, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    std::vector<int32_t> arcs;
    arcs.reserve(mp);
    for (int64_t p = 0; p < n; p++)
        for (int64_t a = first[verts[p]]; a < first[verts[p] + 1]; a++) arcs.push_back((int32_t)a);
    if ((int64_t)arcs.size() != mp) return NWCCH_ERR_TOPOLOGY;
    auto* P = new (std::nothrow) BatPlan();
    if (!P) return NWCCH_ERR_NOMEM;
    const size_t bytes = sizeof(int32_t) * std::max<int64_t>(1, mp);
    if (cudaMalloc(&P->arcs, bytes) != cudaSuccess || cudaMalloc(&P->dtail, bytes) != cudaSuccess) {
        cudaFree(P->arcs);
        delete P;
        return NWCCH_ERR_NOMEM;
    }
    if (mp) {
        if (cudaMemcpy(P->arcs, arcs.data(), sizeof(int32_t) * mp, cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaFree(P->arcs);
            cudaFree(P->dtail);
            delete P;
            return NWCCH_ERR_CUDA;
        }
        k_dtail<<<152 * 4, 256>>>(t->d.darc, t->d.tail, mp, P->dtail);
        if (cudaDeviceSynchronize() != cudaSuccess) {
            cudaFree(P->arcs);
            cudaFree(P->dtail);
            delete P;
            return NWCCH_ERR_CUDA;
        }
    }
    t->battery_plan = P;
    t->free_battery_plan = free_battery_plan;
    *out = P;
    return NWCCH_OK;
}

}  // namespace

}  // namespace nwcch

using namespace nwcch;

struct nwcch_battery {
    nwcch_topology* topo = nullptr;
    double M = 0.0;
    int64_t nd = 0;
    int32_t* cnt = nullptr;
    int64_t* pos = nullptr;
    Piece* pool = nullptr;
    int64_t pool_cap = 0;
    BatStatus* status = nullptr;
    int64_t pieces = 0;
    int32_t largest = 0;
};

extern "C" void nwcch_battery_free(nwcch_battery* b) {
    if (!b) return;
    cudaFree(b->cnt);
    cudaFree(b->pos);
    cudaFree(b->pool);
    cudaFree(b->status);
    delete b;
}

namespace {

int run_levels(nwcch_topology* t, nwcch_battery* b, const BatPlan* P, const double* w, Piece* gbuf, int32_t gcap,
               unsigned long long* next, cudaStream_t s, BatStatus* host) {
    NWCCH_CUDA_TRY(cudaMemsetAsync(next, 0, sizeof(unsigned long long) * std::max<int32_t>(1, t->levels), s));
    NWCCH_CUDA_TRY(cudaMemsetAsync(b->status, 0, sizeof(BatStatus), s));
    BatArgs A{w, b->M, P->arcs, P->dtail, b->cnt, b->pos, b->pool, b->pool_cap, gbuf, gcap, b->status, next};
    for (int32_t l = 0; l < t->levels; l++) {
        const int64_t a0 = t->level_arc_off[l], a1 = t->level_arc_off[l + 1];
        if (a1 == a0) continue;
        const int64_t blocks = std::min<int64_t>((a1 - a0 + LEVEL_WARPS - 1) / LEVEL_WARPS, LEVEL_BLOCKS);
        k_bat_level<<<(unsigned)blocks, 32 * LEVEL_WARPS, 0, s>>>(t->d, A, a0, a1, l);
    }
    NWCCH_CUDA_TRY(cudaGetLastError());
    NWCCH_CUDA_TRY(cudaMemcpyAsync(host, b->status, sizeof(BatStatus), cudaMemcpyDeviceToHost, s));
    NWCCH_CUDA_TRY(cudaStreamSynchronize(s));
    return NWCCH_OK;
}

}  // namespace

extern "C" int nwcch_battery_customize(nwcch_topology* t, const double* w_dev, double capacity, void* stream,
                                       nwcch_battery** out) {
    if (!t || !out || !std::isfinite(capacity) || capacity < 0 || (t->d.m > 0 && !w_dev)) return NWCCH_ERR_ARG;
    *out = nullptr;
    const cudaStream_t s = (cudaStream_t)stream;
    BatPlan* P = nullptr;
    int rc = get_plan(t, &P);
    if (rc) return rc;
    auto* b = new (std::nothrow) nwcch_battery();
    if (!b) return NWCCH_ERR_NOMEM;
    b->topo = t;
    b->M = capacity;
    b->nd = 2 * t->d.m_plus;
    const size_t nd1 = (size_t)std::max<int64_t>(1, b->nd);
    b->pool_cap = t->tune.battery_pool > 0 ? t->tune.battery_pool : b->nd + b->nd / 2 + 1024;
    if (cudaMalloc(&b->cnt, nd1 * sizeof(int32_t)) != cudaSuccess ||
        cudaMalloc(&b->pos, nd1 * sizeof(int64_t)) != cudaSuccess ||
        cudaMalloc(&b->pool, (size_t)b->pool_cap * sizeof(Piece)) != cudaSuccess ||
        cudaMalloc(&b->status, sizeof(BatStatus)) != cudaSuccess) {
        nwcch_battery_free(b);
        return NWCCH_ERR_NOMEM;
    }
    int32_t gcap = std::max<int32_t>(64, t->tune.battery_buffer);
    const int64_t slots = (int64_t)LEVEL_BLOCKS * LEVEL_WARPS;
    void* gbuf = nullptr;
    void* next = nullptr;
    BatStatus host{};
    rc = NWCCH_OK;
    if (cudaMallocAsync(&next, sizeof(unsigned long long) * std::max<int32_t>(1, t->levels), s) != cudaSuccess ||
        cudaMallocAsync(&gbuf, (size_t)slots * 2 * gcap * sizeof(Piece), s) != cudaSuccess)
        rc = NWCCH_ERR_NOMEM;
    for (int attempt = 0; rc == NWCCH_OK; attempt++) {
        rc = run_levels(t, b, P, w_dev, static_cast<Piece*>(gbuf), gcap, static_cast<unsigned long long*>(next), s,
                        &host);
        if (rc || host.flags == 0) break;
        if (attempt >= 12) {
            rc = NWCCH_ERR_CAPACITY;
            break;
        }
        if (host.flags & BAT_POOL_OVERFLOW) {
            const int64_t used = (int64_t)host.pool_used;
            b->pool_cap = std::max<int64_t>(2 * b->pool_cap, used + used / 4);
            cudaFree(b->pool);
            b->pool = nullptr;
            if (cudaMalloc(&b->pool, (size_t)b->pool_cap * sizeof(Piece)) != cudaSuccess) rc = NWCCH_ERR_NOMEM;
        }
        if (rc == NWCCH_OK && (host.flags & BAT_WORK_OVERFLOW)) {
            if (gcap >= (1 << 22)) {
                rc = NWCCH_ERR_CAPACITY;
                break;
            }
            gcap *= 4;
            cudaFreeAsync(gbuf, s);
            gbuf = nullptr;
            if (cudaMallocAsync(&gbuf, (size_t)slots * 2 * gcap * sizeof(Piece), s) != cudaSuccess)
                rc = NWCCH_ERR_NOMEM;
        }
    }
    if (gbuf) cudaFreeAsync(gbuf, s);
    if (next) cudaFreeAsync(next, s);
    if (rc == NWCCH_OK && cudaStreamSynchronize(s) != cudaSuccess) rc = NWCCH_ERR_CUDA;
    if (rc) {
        nwcch_battery_free(b);
        return rc;
    }
    b->pieces = (int64_t)host.pool_used;
    b->largest = host.largest;
    *out = b;
    return NWCCH_OK;
}

extern "C" int nwcch_battery_info(const nwcch_battery* b, int64_t* pieces, int32_t* largest) {
    if (!b) return NWCCH_ERR_ARG;
    if (pieces) *pieces = b->pieces;
    if (largest) *largest = b->largest;
    return NWCCH_OK;
}

extern "C" int nwcch_battery_export(const nwcch_battery* b, int32_t* cnt, int64_t* off, double* pieces) {
    if (!b || !cnt || !off) return NWCCH_ERR_ARG;
    std::vector<int64_t> pos(b->nd);
    if (b->nd) {
        NWCCH_CUDA_TRY(cudaMemcpy(cnt, b->cnt, sizeof(int32_t) * b->nd, cudaMemcpyDeviceToHost));
        NWCCH_CUDA_TRY(cudaMemcpy(pos.data(), b->pos, sizeof(int64_t) * b->nd, cudaMemcpyDeviceToHost));
    }
    int64_t acc = 0;
    for (int64_t d = 0; d < b->nd; d++) {
        off[d] = acc;
        acc += cnt[d];
    }
    off[b->nd] = acc;
    if (acc != b->pieces) return NWCCH_ERR_TOPOLOGY;
    if (pieces && acc) {
        std::vector<Piece> pool(b->pieces);
        NWCCH_CUDA_TRY(cudaMemcpy(pool.data(), b->pool, sizeof(Piece) * b->pieces, cudaMemcpyDeviceToHost));
        for (int64_t d = 0; d < b->nd; d++)
            for (int32_t k = 0; k < cnt[d]; k++) {
                const Piece& p = pool[pos[d] + k];
                double* o = pieces + 3 * (off[d] + k);
                o[0] = p.i;
                o[1] = p.c;
                o[2] = p.o;
            }
    }
    return NWCCH_OK;
}

extern "C" int nwcch_battery_query(nwcch_topology* t, const nwcch_battery* b, const int32_t* s_rank_dev,
                                   const int32_t* t_rank_dev, const double* b0_dev, int64_t nq, double* out_dev,
                                   void* stream) {
    if (!t || !b || b->topo != t || nq < 0 || (nq > 0 && (!s_rank_dev || !t_rank_dev || !b0_dev || !out_dev)))
        return NWCCH_ERR_ARG;
    if (nq == 0) return NWCCH_OK;
    const cudaStream_t s = (cudaStream_t)stream;
    const int64_t Dp = t->d.max_depth + 1;
    const int64_t per_warp = (24 * Dp + 64 + 255) & ~255LL;
    const int64_t warps = std::max<int64_t>(1, std::min<int64_t>(nq, 152 * 16));
    const int64_t blocks = (warps + QUERY_WARPS - 1) / QUERY_WARPS;
    void* scratch = nullptr;
    NWCCH_CUDA_TRY(cudaMallocAsync(&scratch, (size_t)(blocks * QUERY_WARPS * per_warp), s));
    k_bat_query<<<(unsigned)blocks, 32 * QUERY_WARPS, 0, s>>>(t->d, BatDev{b->cnt, b->pos, b->pool}, s_rank_dev,
                                                             t_rank_dev, b0_dev, nq, out_dev,
                                                             static_cast<unsigned char*>(scratch), per_warp,
                                                             stream_slot(t, s).err);
    const cudaError_t launch = cudaGetLastError();
    NWCCH_CUDA_TRY(cudaFreeAsync(scratch, s));
    NWCCH_CUDA_TRY(launch);
    return consume_error(t, s);
}
