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
// Float64 on GB300 runs at a small fraction of the integer rate, and the
// dominance test is most of the work (about 46 float64 operations as
// written). Here every comparison and minimum runs on order keys of the
// doubles (an integer order equal to IEEE order, -0 = +0), so the branches
// taken are the reference's; the values a test reads that depend on one
// piece only are computed once per piece, with the reference's own
// expressions (Rich); and the four subtractions left per test are skipped
// when integer bounds already decide the outcome. Only additions and
// subtractions produce doubles, each the reference's operation on the same
// operands.
//
// A profile of up to 32 pieces lives in the warp's shared memory, piece l
// at slot l; longer profiles continue in the warp's global buffer. The lower
// triangles of (y, z) are the x of y's downward list whose rows hold z: 32
// are tested at a time (binary search of z in x's row) and kept for the
// second direction; the lanes compose the candidates (single-piece sources,
// most of them, directly; longer ones 32 at a time) into shared memory, and
// each batch is merged as if one at a time (merge_staged). Finished profiles
// are appended to a pool at atomic offsets; counts and offsets index it. A
// pool or buffer that overflows is flagged, grown by the host, and the
// customization runs again; the grown sizes are kept for the topology's
// next customization.
//
// Queries (python/cch_nb_battery.py:296-343): one warp per (s, t, b0), or a
// CTA of 8 warps for small batches. The upward pass over s's ancestors in
// increasing rank pushes each label through the up profiles of the vertex's
// arcs (threads over arcs; the heads of a row are distinct; profiles longer
// than 8 pieces evaluated by a whole warp); the downward pass over t's
// ancestors in decreasing rank takes the maximum of the down profiles
// applied to the labels above. Labels are indexed by depth. Maxima (on order
// keys) do not depend on the order, so the answers equal the reference's
// exactly on the same profiles.

#include <algorithm>
#include <cmath>
#include <cstring>
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
constexpr int LEVEL_BLOCKS_PER_SM = 4;  // blocks of the level kernel per SM; one buffer slot per warp
constexpr int QUERY_WARPS = 4;

// A stored piece, with in - EPS for the queries' feasibility test.
struct Piece {
    double i, c, o, ime;
};

struct BatStatus {
    unsigned long long pool_used;
    int flags;
    int largest;
};

struct BatPlan {
    int32_t* arcs = nullptr;   // [m+] arcs by level of their tail, then tail rank
    int32_t* dtail = nullptr;  // [m+] tail of darc[p] (the x of y's downward list)
    int64_t max_down = 0;      // longest downward list
};

// Integer order key of a double: key(a) < key(b) iff a < b for non-NaN
// values, with -0 and +0 equal as in IEEE comparisons.
__device__ __forceinline__ long long dkey(double x) {
    const long long u = __double_as_longlong(x);
    return u < 0 ? -(u & 0x7fffffffffffffffLL) : u;
}

// "v = x; if a < v: v = a", the reference's minimum.
__device__ __forceinline__ double min_ref(double a, double x) { return dkey(a) < dkey(x) ? a : x; }

// A piece with what the dominance tests read, for capacity M. Flags: the
// tests' "lo <= b <= hi" and "b < in - EPS" outcomes that depend on the piece
// alone (python/cch_nb_battery.py:16-44, b in {in, M, out + cost}).
enum : int { R0 = 1, R1 = 2, R2 = 4, R3 = 8, MLT = 16, OCLT = 32 };

struct Rich {
    double i, c, o, oc;                                            // in, cost, out, out + cost
    long long ki, kipe, kime, ko, koc, kv0m, kvMm, kom, kv3m, kvM, kv3;
    int fl;
};

struct Cap {
    double M;
    long long kM, kMpe;  // keys of M and of M + EPS (the tests' hi)
};

__device__ __forceinline__ Rich derive(double i, double c, double o, const Cap& K) {
    Rich r;
    r.i = i;
    r.c = c;
    r.o = o;
    r.oc = o + c;
    r.ki = dkey(i);
    r.kipe = dkey(i + EPS);
    r.kime = dkey(i - EPS);
    r.ko = dkey(o);
    r.koc = dkey(r.oc);
    r.kv0m = dkey(min_ref(o, i - c) - EPS);       // b = in:        min(out, b - cost) - EPS
    const double vM = min_ref(o, K.M - c);        // b = M
    r.kvM = dkey(vM);
    r.kvMm = dkey(vM - EPS);
    r.kom = dkey(o - EPS);
    const double v3 = min_ref(o, r.oc - c);       // b = out + cost
    r.kv3 = dkey(v3);
    r.kv3m = dkey(v3 - EPS);
    int fl = 0;
    if (r.ki <= K.kMpe) fl |= R0;                 // in <= M + EPS
    if (r.kime <= K.kM) fl |= R1;                 // in - EPS <= M
    if (r.koc <= K.kMpe) fl |= R2;                // out + cost <= M + EPS
    if (r.kime <= r.koc && r.koc <= K.kMpe) fl |= R3;
    if (K.kM < r.kime) fl |= MLT;                 // M < in - EPS
    if (r.koc < r.kime) fl |= OCLT;               // out + cost < in - EPS
    r.fl = fl;
    return r;
}

// python/cch_nb_battery.py:16-44: f(b) >= g(b) on [0, M] (with tolerance),
// tested where the difference can be extreme: g's feasibility start, M and
// either breakpoint. The result is the conjunction of the reference's
// checks, so their order does not matter.
__device__ __forceinline__ bool dominates(const Rich& F, const Rich& G) {
    if (F.ki > G.kipe) return false;  // f.in > g.in + EPS
    if (G.fl & R0) {                  // b = g.in
        if (G.ki < F.kime) return false;
        if (F.ko < G.kv0m) return false;
        if (dkey(G.i - F.c) < G.kv0m) return false;
    }
    if ((G.fl & R1) && ((F.fl & MLT) || F.kvM < G.kvMm)) return false;  // b = M
    if ((F.fl & R2) && G.kime <= F.koc) {                                 // b = f.out + f.cost
        if (F.fl & OCLT) return false;
        if (F.kv3 < G.kom) {  // else vf >= g.out - EPS >= vg - EPS
            const double y = F.oc - G.c;
            const double vg = G.ko < dkey(y) ? G.o : y;
            if (F.kv3 < dkey(vg - EPS)) return false;
        }
    }
    if (G.fl & R3) {  // b = g.out + g.cost
        if (G.koc < F.kime) return false;
        if (F.ko < G.kv3m) return false;
        if (dkey(G.oc - F.c) < G.kv3m) return false;
    }
    return true;
}

// python/cch_nb_battery.py:159-173: f then g.
__device__ __forceinline__ bool compose(const Piece& f, const Piece& g, const Cap& K, Rich& h) {
    if (dkey(f.o) < dkey(g.ime)) return false;  // f.out < g.in - EPS
    const double s = g.i + f.c;
    const double hi = dkey(f.i) > dkey(s) ? f.i : s;
    if (dkey(hi) > K.kMpe) return false;
    const double hc = f.c + g.c;
    double ho = g.o;
    const double x = f.o - g.c;
    if (dkey(x) < dkey(ho)) ho = x;
    const double y = K.M - hc;
    if (dkey(y) < dkey(ho)) ho = y;
    h = derive(hi, hc, ho, K);
    return true;
}

// Up to 32 pieces of a profile in shared memory, one per lane, field by
// field (conflict-free: lane l reads word l of each field).
struct RichSet {
    double i[32], c[32], o[32], oc[32];
    long long ki[32], kipe[32], kime[32], ko[32], koc[32], kv0m[32], kvMm[32], kom[32], kv3m[32], kvM[32], kv3[32];
    int fl[32];
};

__device__ __forceinline__ Rich load_rich(const RichSet& S, int l) {
    return Rich{S.i[l],    S.c[l],    S.o[l],    S.oc[l],   S.ki[l],   S.kipe[l], S.kime[l], S.ko[l],
                S.koc[l],  S.kv0m[l], S.kvMm[l], S.kom[l],  S.kv3m[l], S.kvM[l],  S.kv3[l],  S.fl[l]};
}

__device__ __forceinline__ void store_rich(RichSet& S, int l, const Rich& r) {
    S.i[l] = r.i;
    S.c[l] = r.c;
    S.o[l] = r.o;
    S.oc[l] = r.oc;
    S.ki[l] = r.ki;
    S.kipe[l] = r.kipe;
    S.kime[l] = r.kime;
    S.ko[l] = r.ko;
    S.koc[l] = r.koc;
    S.kv0m[l] = r.kv0m;
    S.kvMm[l] = r.kvMm;
    S.kom[l] = r.kom;
    S.kv3m[l] = r.kv3m;
    S.kvM[l] = r.kvM;
    S.kv3[l] = r.kv3;
    S.fl[l] = r.fl;
}

// The profile being built: in the warp's shared RichSet (piece l at slot l)
// while it has at most 32 pieces, else in buf. n and glob are warp-uniform.
struct Work {
    RichSet* set;
    int n;
    bool glob;
    Rich* buf;
};

struct BatArgs {
    const double* w;
    Cap K;
    const int32_t* arcs;
    const int32_t* dtail;
    int32_t* cnt;
    int64_t* pos;
    Piece* pool;
    int64_t pool_cap;
    Rich* gbuf;  // gcap pieces per warp slot
    int2* tri;   // max_down lower triangles per warp slot
    int64_t max_down;
    int32_t gcap;
    BatStatus* status;
    unsigned long long* next;  // per level: arcs handed out
};

// python/cch_nb_battery.py:186-254: one candidate into the profile.
__device__ __noinline__ void merge(Work& W, const Rich& h, int32_t gcap, int lane, int& flags) {
    if (!W.glob) {
        const bool live = lane < W.n;
        Rich g;
        if (live) g = load_rich(*W.set, lane);
        if (__any_sync(FULL, live && dominates(g, h))) return;
        const bool keep = live && !dominates(h, g);
        const unsigned km = __ballot_sync(FULL, keep);
        const int k = __popc(km);
        if (k < 32) {
            if (km != (1u << k) - 1u) {
                __syncwarp();
                if (keep) store_rich(*W.set, __popc(km & ((1u << lane) - 1u)), g);
            }
            __syncwarp();
            if (lane == 0) store_rich(*W.set, k, h);
            W.n = k + 1;
            __syncwarp();
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
        if (__any_sync(FULL, live && dominates(W.buf[b + lane], h))) return;
    }
    int k = 0;
    for (int b = 0; b < W.n; b += 32) {
        const bool live = b + lane < W.n;
        Rich g;
        bool keep = false;
        if (live) {
            g = W.buf[b + lane];
            keep = !dominates(h, g);
        }
        const unsigned km = __ballot_sync(FULL, keep);
        // writes land at or below every position this chunk has read
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
        if (lane < W.n) store_rich(*W.set, lane, W.buf[lane]);
        W.glob = false;
        __syncwarp();
    }
}

// Merges the candidates staged in S (bits of vm, ascending lane order), with
// the outcome of merging them one at a time. In the shared-memory form the
// lanes first test their own candidates, in parallel, against the profile P0
// the batch starts from, newest piece first (most candidates are dominated
// by the newest piece). Then, in order: a candidate whose dominator is still
// present is dropped at the cost of a bit test; any other is tested exactly
// against the pieces present at its turn (P0's survivors and the batch's
// inserted candidates, held by their lanes), and if it is kept it removes
// what it dominates. The result is P0's survivors, then the inserted
// survivors, each in order: the one-at-a-time merge's profile.
__device__ __forceinline__ Rich piece_at(const Work& W, int k) {
    return W.glob ? W.buf[k] : load_rich(*W.set, k);
}

__device__ __noinline__ void merge_staged(Work& W, Rich* S, unsigned vm, const Cap& K, int32_t gcap, int lane,
                                          int& flags) {
    if (!vm) return;
    const int n = W.n;
    if (n > 32 * 32) {  // beyond the removal bitmap: one at a time
        while (vm) {
            const int src = __ffs(vm) - 1;
            vm &= vm - 1;
            merge(W, S[src], gcap, lane, flags);
        }
        return;
    }
    const bool mine = (vm >> lane) & 1u;
    Rich h{};
    int gj = -1;
    if (mine) {
        h = S[lane];
        for (int k = n - 1; k >= 0; k--)
            if (dominates(piece_at(W, k), h)) {
                gj = k;
                break;
            }
    }
    const int chunks = (n + 31) >> 5;
    unsigned remw = 0;  // lane c: P0 pieces 32c..32c+31 removed
    int nrem = 0;
    unsigned ins = 0;   // inserted candidates still present (bit = lane)
    unsigned todo = vm;
    while (todo) {
        const int j = __ffs(todo) - 1;
        todo &= todo - 1;
        const int g = __shfl_sync(FULL, gj, j);
        if (g >= 0 && !((__shfl_sync(FULL, remw, g >> 5) >> (g & 31)) & 1u)) continue;  // dominator present
        const Rich& hj = S[j];
        bool d = ((ins >> lane) & 1u) && dominates(h, hj);
        if (g >= 0) {
            for (int c = 0; c < chunks; c++) {
                const int k = 32 * c + lane;
                const unsigned rw = __shfl_sync(FULL, remw, c);
                if (k < n && !((rw >> lane) & 1u) && dominates(piece_at(W, k), hj)) d = true;
                if (__any_sync(FULL, d)) break;
            }
        }
        if (__any_sync(FULL, d)) continue;
        for (int c = 0; c < chunks; c++) {
            const int k = 32 * c + lane;
            const unsigned rw = __shfl_sync(FULL, remw, c);
            const bool rp = k < n && !((rw >> lane) & 1u) && dominates(hj, piece_at(W, k));
            const unsigned mk = __ballot_sync(FULL, rp);
            nrem += __popc(mk);
            if (lane == c) remw |= mk;
        }
        const bool ri = ((ins >> lane) & 1u) && dominates(hj, h);
        ins = (ins & ~__ballot_sync(FULL, ri)) | (1u << j);
    }
    if (!ins && !nrem) return;  // every candidate dropped
    const int np = n - nrem, total = np + __popc(ins);
    const unsigned lt = (1u << lane) - 1u;
    if (total > gcap) {
        flags |= BAT_WORK_OVERFLOW;
        return;
    }
    if (!W.glob && total <= 32) {
        const unsigned keepP = (n == 32 ? FULL : ((1u << n) - 1u)) & ~__shfl_sync(FULL, remw, 0);
        Rich g{};
        const bool kp = (keepP >> lane) & 1u;
        if (kp) g = load_rich(*W.set, lane);
        __syncwarp();
        if (kp) store_rich(*W.set, __popc(keepP & lt), g);
        if ((ins >> lane) & 1u) store_rich(*W.set, np + __popc(ins & lt), h);
        W.n = total;
        __syncwarp();
        return;
    }
    // the global buffer: P0's survivors (compacted in place when P0 is
    // there already: writes land at or below every position read), then the
    // inserted candidates
    int k0 = 0;
    for (int c = 0; c < chunks; c++) {
        const int k = 32 * c + lane;
        const unsigned rw = __shfl_sync(FULL, remw, c);
        const bool keep = k < n && !((rw >> lane) & 1u);
        Rich g{};
        if (keep) g = piece_at(W, k);
        const unsigned km = __ballot_sync(FULL, keep);
        __syncwarp();
        if (keep) W.buf[k0 + __popc(km & lt)] = g;
        k0 += __popc(km);
    }
    if ((ins >> lane) & 1u) W.buf[np + __popc(ins & lt)] = h;
    W.n = total;
    W.glob = true;
    __syncwarp();
    if (total <= 32) {
        if (lane < total) store_rich(*W.set, lane, W.buf[lane]);
        W.glob = false;
        __syncwarp();
    }
}

// The candidates of one lower triangle side with general source profiles:
// f pieces (direction df) then g pieces (dg), f-major as the reference.
__device__ __noinline__ void merge_triangle(Work& W, const BatArgs& A, int64_t df, int64_t dg, Rich* S, int lane, int& flags) {
    const int32_t na = A.cnt[df], nb = A.cnt[dg];
    if (na == 0 || nb == 0) return;
    const int64_t fa = A.pos[df], ga = A.pos[dg];
    const int32_t tot = na * nb;
    for (int32_t qb = 0; qb < tot; qb += 32) {
        const int32_t q = qb + lane;
        bool ok = false;
        if (q < tot) {
            Rich h;
            ok = compose(A.pool[fa + q / nb], A.pool[ga + q % nb], A.K, h);
            if (ok) S[lane] = h;
        }
        const unsigned vm = __ballot_sync(FULL, ok);
        __syncwarp();
        merge_staged(W, S, vm, A.K, A.gcap, lane, flags);
        __syncwarp();
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
        if (lane < n) {
            const double i = W.set->i[lane];
            A.pool[p + lane] = Piece{i, W.set->c[lane], W.set->o[lane], i - EPS};
        }
    } else {
        for (int t = lane; t < n; t += 32) {
            const Rich& r = W.buf[t];
            A.pool[p + t] = Piece{r.i, r.c, r.o, r.i - EPS};
        }
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

// Shared memory of one warp: the single-piece candidates of up to 32
// triangles and a chunk of a general triangle's.
struct WarpStage {
    Rich s1[32], sg[32];
    RichSet prof;
};

// One chunk of lower triangles, each lane one triangle side (sources df, dg;
// df < 0: none), in order: the candidates of single-piece sources are
// composed by their lanes and merged as a batch; a general triangle's are
// merged 32 at a time where it falls in the order.
__device__ void merge_chunk(Work& W, const BatArgs& A, WarpStage& st, int64_t df, int64_t dg, int lane,
                            int& flags) {
    int kind = 0;
    bool ok = false;
    if (df >= 0) {
        kind = side_kind(A.cnt[df], A.cnt[dg]);
        Rich h;
        if (kind == 1 && compose(A.pool[A.pos[df]], A.pool[A.pos[dg]], A.K, h)) {
            st.s1[lane] = h;
            ok = true;
        }
    }
    const unsigned m1 = __ballot_sync(FULL, ok);
    unsigned mg = __ballot_sync(FULL, kind == 2);
    __syncwarp();
    unsigned done = 0;  // lanes below the next general triangle are merged
    while (mg) {
        const int src = __ffs(mg) - 1;
        mg &= mg - 1;
        const unsigned below = (1u << src) - 1u;
        merge_staged(W, st.s1, m1 & below & ~done, A.K, A.gcap, lane, flags);
        done = below | (1u << src);
        const int64_t sf = __shfl_sync(FULL, df, src), sg = __shfl_sync(FULL, dg, src);
        merge_triangle(W, A, sf, sg, st.sg, lane, flags);
    }
    merge_staged(W, st.s1, m1 & ~done, A.K, A.gcap, lane, flags);
}

__device__ void merge_base(Work& W, const DevTopo& D, const BatArgs& A, int32_t j, int side, int lane, int& flags) {
    // python/cch_nb_battery.py:67-82: the original arcs onto j, input order
    const double M = A.K.M;
    for (int64_t e = D.aeoff[j]; e < D.aeoff[j + 1]; e++) {
        const int32_t k = D.aeidx[e];
        if ((D.e_up[k] != 0) != (side == 0)) continue;
        const double c = A.w[k];
        Rich h;
        if (c >= 0) {
            if (c > M) continue;
            h = derive(c, c, M - c, A.K);
        } else {
            h = derive(0.0, c, M, A.K);
        }
        merge(W, h, A.gcap, lane, flags);
    }
}

// The two profiles of arc j = (y, z), one after the other (one profile live
// at a time), over its lower triangles (x; y, z), x ascending:
//   up(y,z)   <- down(x,y) then up(x,z)
//   down(y,z) <- down(x,z) then up(x,y)
// The up pass finds the triangles (binary search of z in the rows of y's
// downward list) and keeps them in the warp's list tri; the down pass reads
// them back.
__device__ void customize_arc(const DevTopo& D, const BatArgs& A, int32_t j, Rich* gb, int2* tri, WarpStage& st,
                              int lane, int& flags, int& seen) {
    const int32_t y = D.tail[j], z = D.head[j];
    const unsigned lt = (1u << lane) - 1u;
    Work W{&st.prof, 0, false, gb};
    merge_base(W, D, A, j, 0, lane, flags);
    const int64_t p1 = D.doff[y + 1];
    int ntri = 0;
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
        const unsigned hm = __ballot_sync(FULL, kk >= 0);
        if (!hm) continue;
        if (kk >= 0) tri[ntri + __popc(hm & lt)] = make_int2((int)i, (int)kk);
        ntri += __popc(hm);
        merge_chunk(W, A, st, kk >= 0 ? 2 * i + 1 : -1, 2 * kk, lane, flags);
    }
    finish(W, A, 2 * (int64_t)j, lane, flags, seen);
    __syncwarp();
    W = Work{&st.prof, 0, false, gb};
    merge_base(W, D, A, j, 1, lane, flags);
    for (int c = 0; c < ntri; c += 32) {
        int64_t df = -1, dg = -1;
        if (c + lane < ntri) {
            const int2 t = tri[c + lane];
            df = 2 * (int64_t)t.y + 1;
            dg = 2 * (int64_t)t.x;
        }
        merge_chunk(W, A, st, df, dg, lane, flags);
    }
    finish(W, A, 2 * (int64_t)j + 1, lane, flags, seen);
}

__global__ void __launch_bounds__(32 * LEVEL_WARPS) k_bat_level(DevTopo D, BatArgs A, int64_t a0, int64_t a1,
                                                                 int32_t level) {
    extern __shared__ __align__(16) unsigned char bat_smem[];
    WarpStage* stages = reinterpret_cast<WarpStage*>(bat_smem);
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t slot = (int64_t)blockIdx.x * LEVEL_WARPS + wib;
    Rich* gb = A.gbuf + slot * (int64_t)A.gcap;
    int flags = 0, seen = 0;
    for (;;) {
        unsigned long long idx = 0;
        if (lane == 0) idx = atomicAdd(&A.next[level], 1ull);
        idx = __shfl_sync(FULL, idx, 0);
        const int64_t e = a0 + (int64_t)idx;
        if (e >= a1) break;
        customize_arc(D, A, A.arcs[e], gb, A.tri + slot * A.max_down, stages[wib], lane, flags, seen);
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

// python/cch_nb_battery.py:272-293, comparisons on order keys: the best
// value over pieces [t0, n) step dt of direction d at charge b.
__device__ __forceinline__ double eval_pieces(const BatDev& B, int64_t d, double b, int t0, int dt, long long& kbest) {
    double best = -INFINITY;
    kbest = dkey(-INFINITY);
    const long long kb = dkey(b);
    const int32_t n = B.cnt[d];
    const Piece* p = B.pool + B.pos[d];
    for (int32_t t = t0; t < n; t += dt) {
        const Piece f = p[t];
        if (kb >= dkey(f.ime)) {
            double v = b - f.c;
            if (dkey(f.o) < dkey(v)) v = f.o;
            const long long kv = dkey(v);
            if (kv > kbest) {
                best = v;
                kbest = kv;
            }
        }
    }
    return best;
}

// Warp maximum of (key, value) pairs; every lane gets it.
__device__ __forceinline__ double warp_max(double v, long long k) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const long long ko = __shfl_xor_sync(FULL, k, o);
        const double vo = __shfl_xor_sync(FULL, v, o);
        if (ko > k) {
            k = ko;
            v = vo;
        }
    }
    return v;
}

constexpr int32_t QUERY_WIDE = 8;  // profiles longer than this are evaluated by the whole warp
constexpr int QUERY_CTA_WARPS = 8;      // the single-query form: a CTA of 8 warps per query
constexpr int64_t QUERY_CTA_MAX = 304;  // batches up to this size use it

// The same query with a CTA per (s, t, b0), for small batches (latency):
// the 256 threads split each vertex's arcs, each warp evaluates the long
// profiles among its own 32 arcs, and the downward maximum is reduced
// across the warps through shared memory.
__global__ void __launch_bounds__(32 * QUERY_CTA_WARPS)
    k_bat_query_cta(DevTopo D, BatDev B, const int32_t* __restrict__ s_rank, const int32_t* __restrict__ t_rank,
                    const double* __restrict__ b0, int64_t nq, double* __restrict__ out, unsigned char* scratch,
                    int64_t per_cta, int* err) {
    __shared__ double red_v[QUERY_CTA_WARPS];
    __shared__ long long red_k[QUERY_CTA_WARPS];
    constexpr int NT = 32 * QUERY_CTA_WARPS;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, tid = threadIdx.x;
    const int64_t Dp = D.max_depth + 1;
    double* soc = reinterpret_cast<double*>(scratch + blockIdx.x * per_cta);
    double* dsoc = soc + Dp;
    int32_t* cs = reinterpret_cast<int32_t*>(dsoc + Dp);
    int32_t* ct = cs + Dp;
    const long long kneg = dkey(-INFINITY);
    int e = 0;
    for (int64_t q = blockIdx.x; q < nq; q += gridDim.x) {
        const int32_t s = s_rank[q], t = t_rank[q];
        if (s < 0 || s >= D.n || t < 0 || t >= D.n) {
            if (tid == 0) out[q] = -INFINITY;
            e |= ERR_ARG;
            continue;
        }
        const int32_t ds = D.depth[s], dt = D.depth[t];
        for (int32_t d = tid; d <= ds; d += NT) soc[d] = -INFINITY;
        __syncthreads();
        if (tid == 0) soc[ds] = b0[q];
        __syncthreads();
        int32_t d = ds;
        for (int32_t x = s; x >= 0; x = D.parent[x], d--) {
            if (tid == 0) cs[d] = x;
            const double bx = soc[d];
            if (dkey(bx) > kneg) {
                const int64_t a1 = D.first[x + 1];
                for (int64_t ab = D.first[x] + 32 * wib; ab < a1; ab += NT) {
                    const int64_t a = ab + lane;
                    const int32_t n = a < a1 ? B.cnt[2 * a] : 0;
                    const bool wide = n > QUERY_WIDE;
                    if (a < a1 && !wide && n > 0) {
                        long long kv;
                        const double v = eval_pieces(B, 2 * a, bx, 0, 1, kv);
                        const int32_t hd = D.hdep[a];
                        if (kv > dkey(soc[hd])) soc[hd] = v;
                    }
                    unsigned wm = __ballot_sync(FULL, wide);
                    while (wm) {
                        const int src = __ffs(wm) - 1;
                        wm &= wm - 1;
                        const int64_t aa = ab + src;
                        long long kv;
                        const double v = warp_max(eval_pieces(B, 2 * aa, bx, lane, 32, kv), kv);
                        if (lane == 0) {
                            const int32_t hd = D.hdep[aa];
                            if (dkey(v) > dkey(soc[hd])) soc[hd] = v;
                        }
                    }
                }
            }
            __syncthreads();
        }
        d = dt;
        for (int32_t x = t; x >= 0; x = D.parent[x], d--)
            if (tid == 0) ct[d] = x;
        __syncthreads();
        for (d = 0; d <= dt; d++) {
            const int32_t x = ct[d];
            double best = -INFINITY;
            long long kb = kneg;
            if (tid == 0 && d <= ds && cs[d] == x) {
                best = soc[d];
                kb = dkey(best);
            }
            const int64_t a1 = D.first[x + 1];
            for (int64_t ab = D.first[x] + 32 * wib; ab < a1; ab += NT) {
                const int64_t a = ab + lane;
                double by = -INFINITY;
                int32_t n = 0;
                if (a < a1) {
                    by = dsoc[D.hdep[a]];
                    if (dkey(by) > kneg) n = B.cnt[2 * a + 1];
                }
                const bool wide = n > QUERY_WIDE;
                if (n > 0 && !wide) {
                    long long kv;
                    const double v = eval_pieces(B, 2 * a + 1, by, 0, 1, kv);
                    if (kv > kb) {
                        best = v;
                        kb = kv;
                    }
                }
                unsigned wm = __ballot_sync(FULL, wide);
                while (wm) {
                    const int src = __ffs(wm) - 1;
                    wm &= wm - 1;
                    const double bys = __shfl_sync(FULL, by, src);
                    long long kv;
                    const double v = warp_max(eval_pieces(B, 2 * (ab + src) + 1, bys, lane, 32, kv), kv);
                    const long long kw = dkey(v);
                    if (lane == 0 && kw > kb) {
                        best = v;
                        kb = kw;
                    }
                }
            }
            best = warp_max(best, kb);
            if (lane == 0) {
                red_v[wib] = best;
                red_k[wib] = dkey(best);
            }
            __syncthreads();
            if (tid == 0) {
                double bv = red_v[0];
                long long bk = red_k[0];
                for (int w2 = 1; w2 < QUERY_CTA_WARPS; w2++)
                    if (red_k[w2] > bk) {
                        bk = red_k[w2];
                        bv = red_v[w2];
                    }
                dsoc[d] = bv;
            }
            __syncthreads();
        }
        if (tid == 0) out[q] = dsoc[dt];
        __syncthreads();
    }
    if (e && tid == 0) atomicOr(err, e);
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
    const long long kneg = dkey(-INFINITY);
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
        // upward: s's ancestors in increasing rank; lanes over arcs, long
        // profiles by the whole warp
        int32_t d = ds;
        for (int32_t x = s; x >= 0; x = D.parent[x], d--) {
            if (lane == 0) cs[d] = x;
            const double bx = soc[d];
            if (dkey(bx) > kneg) {
                const int64_t a1 = D.first[x + 1];
                for (int64_t ab = D.first[x]; ab < a1; ab += 32) {
                    const int64_t a = ab + lane;
                    const int32_t n = a < a1 ? B.cnt[2 * a] : 0;
                    const bool wide = n > QUERY_WIDE;
                    if (a < a1 && !wide && n > 0) {
                        long long kv;
                        const double v = eval_pieces(B, 2 * a, bx, 0, 1, kv);
                        const int32_t hd = D.hdep[a];
                        if (kv > dkey(soc[hd])) soc[hd] = v;
                    }
                    unsigned wm = __ballot_sync(FULL, wide);
                    while (wm) {
                        const int src = __ffs(wm) - 1;
                        wm &= wm - 1;
                        const int64_t aa = ab + src;
                        long long kv;
                        const double v = warp_max(eval_pieces(B, 2 * aa, bx, lane, 32, kv), kv);
                        if (lane == 0) {
                            const int32_t hd = D.hdep[aa];
                            if (dkey(v) > dkey(soc[hd])) soc[hd] = v;
                        }
                    }
                }
            }
            __syncwarp();
        }
        d = dt;
        for (int32_t x = t; x >= 0; x = D.parent[x], d--)
            if (lane == 0) ct[d] = x;
        __syncwarp();
        // downward: t's ancestors in decreasing rank
        for (d = 0; d <= dt; d++) {
            const int32_t x = ct[d];
            double best = (d <= ds && cs[d] == x) ? soc[d] : -INFINITY;
            long long kb = dkey(best);
            const int64_t a1 = D.first[x + 1];
            for (int64_t ab = D.first[x]; ab < a1; ab += 32) {
                const int64_t a = ab + lane;
                double by = -INFINITY;
                int32_t n = 0;
                if (a < a1) {
                    by = dsoc[D.hdep[a]];
                    if (dkey(by) > kneg) n = B.cnt[2 * a + 1];
                }
                const bool wide = n > QUERY_WIDE;
                if (n > 0 && !wide) {
                    long long kv;
                    const double v = eval_pieces(B, 2 * a + 1, by, 0, 1, kv);
                    if (kv > kb) {
                        best = v;
                        kb = kv;
                    }
                }
                unsigned wm = __ballot_sync(FULL, wide);
                while (wm) {
                    const int src = __ffs(wm) - 1;
                    wm &= wm - 1;
                    const double bys = __shfl_sync(FULL, by, src);
                    long long kv;
                    const double v = warp_max(eval_pieces(B, 2 * (ab + src) + 1, bys, lane, 32, kv), kv);
                    const long long kw = dkey(v);
                    if (lane == 0 && kw > kb) {
                        best = v;
                        kb = kw;
                    }
                }
            }
            best = warp_max(best, kb);
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
    std::vector<int64_t> first(n + 1), doff(n + 1);
    std::vector<int32_t> verts(n);
    NWCCH_CUDA_TRY(cudaMemcpy(first.data(), t->d.first, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost));
    NWCCH_CUDA_TRY(cudaMemcpy(doff.data(), t->d.doff, sizeof(int64_t) * (n + 1), cudaMemcpyDeviceToHost));
    int64_t max_down = 0;
    for (int64_t v = 0; v < n; v++) max_down = std::max(max_down, doff[v + 1] - doff[v]);
    if (n) NWCCH_CUDA_TRY(cudaMemcpy(verts.data(), t->level_verts, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    // within a level, the arcs of the tails with the longest downward lists
    // (the most lower triangles to search) first: the warps fetch arcs in
    // this order, so the longest candidate streams start early instead of
    // finishing the level alone
    for (int32_t l = 0; l < t->levels; l++)
        std::stable_sort(verts.begin() + t->level_off[l], verts.begin() + t->level_off[l + 1],
                         [&](int32_t a, int32_t b) { return doff[a + 1] - doff[a] > doff[b + 1] - doff[b]; });
    std::vector<int32_t> arcs;
    arcs.reserve(mp);
    for (int64_t p = 0; p < n; p++)
        for (int64_t a = first[verts[p]]; a < first[verts[p] + 1]; a++) arcs.push_back((int32_t)a);
    if ((int64_t)arcs.size() != mp) return NWCCH_ERR_TOPOLOGY;
    auto* P = new (std::nothrow) BatPlan();
    if (!P) return NWCCH_ERR_NOMEM;
    P->max_down = max_down;
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
        k_dtail<<<t->sms * 4, 256>>>(t->d.darc, t->d.tail, mp, P->dtail);
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

// dkey on the host (same integer order of doubles).
long long host_key(double x) {
    long long u;
    std::memcpy(&u, &x, sizeof(u));
    return u < 0 ? -(u & 0x7fffffffffffffffLL) : u;
}

int run_levels(nwcch_topology* t, nwcch_battery* b, const BatPlan* P, const double* w, Rich* gbuf, int32_t gcap,
               int2* tri, unsigned long long* next, cudaStream_t s, BatStatus* host) {
    NWCCH_CUDA_TRY(cudaMemsetAsync(next, 0, sizeof(unsigned long long) * std::max<int32_t>(1, t->levels), s));
    NWCCH_CUDA_TRY(cudaMemsetAsync(b->status, 0, sizeof(BatStatus), s));
    const double Mpe = b->M + EPS;  // the tests' hi, as the reference computes it
    Cap K{b->M, host_key(b->M), host_key(Mpe)};
    BatArgs A{w,    K,     P->arcs, P->dtail,    b->cnt,    b->pos,   b->pool,
              b->pool_cap, gbuf, tri, P->max_down, gcap, b->status, next};
    const size_t smem = sizeof(WarpStage) * LEVEL_WARPS;
    NWCCH_CUDA_TRY(allow_dynamic_smem((const void*)k_bat_level, smem));
    for (int32_t l = 0; l < t->levels; l++) {
        const int64_t a0 = t->level_arc_off[l], a1 = t->level_arc_off[l + 1];
        if (a1 == a0) continue;
        const int64_t blocks = std::min<int64_t>((a1 - a0 + LEVEL_WARPS - 1) / LEVEL_WARPS,
                                               (int64_t)LEVEL_BLOCKS_PER_SM * t->sms);
        k_bat_level<<<(unsigned)blocks, 32 * LEVEL_WARPS, smem, s>>>(t->d, A, a0, a1, l);
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
    int32_t gcap = 64;
    {
        // the sizes learned by earlier customizations of this handle (which
        // may run concurrently on other streams)
        std::lock_guard<std::mutex> lock(t->mu);
        b->pool_cap = t->tune.battery_pool > 0 ? t->tune.battery_pool
                                               : std::max<int64_t>(b->nd + b->nd / 2 + 1024, t->battery_pool_hint);
        gcap = std::max<int32_t>(64, t->tune.battery_buffer);
    }
    if (cudaMalloc(&b->cnt, nd1 * sizeof(int32_t)) != cudaSuccess ||
        cudaMalloc(&b->pos, nd1 * sizeof(int64_t)) != cudaSuccess ||
        cudaMalloc(&b->pool, (size_t)b->pool_cap * sizeof(Piece)) != cudaSuccess ||
        cudaMalloc(&b->status, sizeof(BatStatus)) != cudaSuccess) {
        nwcch_battery_free(b);
        return NWCCH_ERR_NOMEM;
    }
    const int64_t slots = (int64_t)LEVEL_BLOCKS_PER_SM * t->sms * LEVEL_WARPS;
    void* gbuf = nullptr;
    void* next = nullptr;
    void* tri = nullptr;
    BatStatus host{};
    rc = NWCCH_OK;
    if (scratch_alloc(&next, sizeof(unsigned long long) * std::max<int32_t>(1, t->levels), s) != cudaSuccess ||
        scratch_alloc(&tri, (size_t)slots * std::max<int64_t>(1, P->max_down) * sizeof(int2), s) != cudaSuccess ||
        scratch_alloc(&gbuf, (size_t)slots * gcap * sizeof(Rich), s) != cudaSuccess)
        rc = NWCCH_ERR_NOMEM;
    for (int attempt = 0; rc == NWCCH_OK; attempt++) {
        rc = run_levels(t, b, P, w_dev, static_cast<Rich*>(gbuf), gcap, static_cast<int2*>(tri),
                        static_cast<unsigned long long*>(next), s, &host);
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
            if (scratch_alloc(&gbuf, (size_t)slots * gcap * sizeof(Rich), s) != cudaSuccess)
                rc = NWCCH_ERR_NOMEM;
        }
    }
    if (gbuf) cudaFreeAsync(gbuf, s);
    if (tri) cudaFreeAsync(tri, s);
    if (next) cudaFreeAsync(next, s);
    if (rc == NWCCH_OK && cudaStreamSynchronize(s) != cudaSuccess) rc = NWCCH_ERR_CUDA;
    if (rc) {
        nwcch_battery_free(b);
        return rc;
    }
    b->pieces = (int64_t)host.pool_used;
    b->largest = host.largest;
    // the next customization of this topology starts with buffers that fit
    // (an overflow costs a whole rerun)
    {
        std::lock_guard<std::mutex> lock(t->mu);
        t->tune.battery_buffer = std::max<int32_t>(t->tune.battery_buffer, gcap);
        t->battery_pool_hint = std::max<int64_t>(t->battery_pool_hint, b->pieces + b->pieces / 8);
    }
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
    const int64_t per_query = (24 * Dp + 64 + 255) & ~255LL;  // labels and chains of one query in flight
    const BatDev B{b->cnt, b->pos, b->pool};
    int* err = stream_slot(t, s).err;
    void* scratch = nullptr;
    if (nq <= QUERY_CTA_MAX) {
        NWCCH_CUDA_TRY(scratch_alloc(&scratch, (size_t)(nq * per_query), s));
        k_bat_query_cta<<<(unsigned)nq, 32 * QUERY_CTA_WARPS, 0, s>>>(
            t->d, B, s_rank_dev, t_rank_dev, b0_dev, nq, out_dev, static_cast<unsigned char*>(scratch), per_query, err);
    } else {
        const int64_t warps = std::min<int64_t>(nq, (int64_t)t->sms * 16);
        const int64_t blocks = (warps + QUERY_WARPS - 1) / QUERY_WARPS;
        NWCCH_CUDA_TRY(scratch_alloc(&scratch, (size_t)(blocks * QUERY_WARPS * per_query), s));
        k_bat_query<<<(unsigned)blocks, 32 * QUERY_WARPS, 0, s>>>(
            t->d, B, s_rank_dev, t_rank_dev, b0_dev, nq, out_dev, static_cast<unsigned char*>(scratch), per_query, err);
    }
    const cudaError_t launch = cudaGetLastError();
    NWCCH_CUDA_TRY(cudaFreeAsync(scratch, s));
    NWCCH_CUDA_TRY(launch);
    return consume_error(t, s);
}
