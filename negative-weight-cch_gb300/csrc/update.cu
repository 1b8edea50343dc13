// Partial re-customization after original-arc weight changes.
//
// Follows CCH.update_edges (python/cch.py:349-402, Theorem 4 of the
// reference's technical note): the arcs the changed original arcs map to are
// queued; a queued arc c = (y,z) is re-evaluated from its base value (minimum
// over the original arcs mapped onto it) and its lower triangles, and if its
// (up, dn) pair changed, every arc that has c as a lower side is queued. The
// reference pops a heap keyed by the tail rank; here the queue is bucketed by
// the tail's level instead: the lower sides of an arc have tails of strictly
// lower level, so evaluating one level at a time, lowest first, sees the same
// final lower values and queues the same set of arcs.
//
// A change first sweeps in one CTA: its levels end at a block barrier, which
// is what most single-arc changes need (a few hundred arcs over some dozens
// of levels). When that sweep has evaluated `update_small_arcs` arcs or run
// `update_small_ns`, it hands its pending levels to one cooperative launch
// over the whole grid: its blocks are co-resident, and a level ends with a
// grid barrier whose spin is bounded (on timeout the kernel records
// ERR_TIMEOUT and every block returns; the host then resets the workspace
// and reports NWCCH_ERR_TIMEOUT). The kernel cleans its workspace (queued
// flags, bucket counts, pending bits) before it exits.
//
// The level sweep pays a barrier per level and a row search per lower
// triangle, so a change that spreads through the top separators costs more
// than customizing from scratch. The grid sweep therefore runs under a
// budget (about a quarter of a full customization's time, or the tuned
// value): past it, the sweep stops before its next arc, inside a level if
// need be, and the update is finished densely with the same results and
// statistics: the whole metric is re-customized into scratch by the
// supernodal kernels, the arcs whose values differ are the changed ones, and
// an arc above the stop counts as evaluated if it was queued before the stop
// or one of its lower triangles has a changed side (the set the sweep would
// have queued). Lower triangles are found through the supernode layout: a
// triangle inside a supernode through its trapezoid columns, one below it
// through the boundary pairs of a descendant supernode. A level left part
// way is counted once, whole, when it starts (the one-CTA sweep hands it over
// whole; the dense count starts at the level above it).

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "common.cuh"
#include "customize.h"
#include "supernodal.h"
#include "topology.h"

namespace nwcch {

struct UpdateWorkspace {
    uint8_t* queued = nullptr;        // [m+]  arc already queued in this update
    int32_t* bucket = nullptr;        // [m+]  queued arcs, grouped by tail level
    int32_t* bcount = nullptr;        // [L]   arcs queued per level
    uint32_t* pending = nullptr;      // [(L+31)/32] levels with queued arcs
    int32_t* done_levels = nullptr;   // [L]   levels processed, for the cleanup
    int32_t* changed = nullptr;       // [m+]  changed arcs, in processing order
    int64_t* edge_idx = nullptr;      // [cap] staged changes
    int32_t* new_w = nullptr;         // [cap]
    int64_t cap = 0;
    uint8_t* chg = nullptr;           // [m+]  arc changed in this update
    uint8_t* dq = nullptr;            // [m+]  dense finish: a lower triangle has a changed side
    uint8_t* acol = nullptr;          // [n]   dense finish: per supernode row, a changed arc above it
    void* up2 = nullptr;              // [m+]  dense finish: full re-customization (8-byte slots)
    void* dn2 = nullptr;
    // [0] evaluated [1] changed [2] changed with up+dn<0 [3] levels done
    // [5] barrier arrivals [6] barrier generation [7] stop level + 1
    // [8], [9] stop requests by level parity [10] hand-over level + 1 of a
    // one-CTA sweep [11], [12] part-way stop requests by level parity
    // [13] the stop or hand-over level was left part way
    unsigned long long* stats = nullptr;
    int blocks32 = 0, blocks64 = 0;
    int2* tiles = nullptr;            // dense finish: (supernode, 32-column tile) work items,
    int64_t ntiles = 0;               // those of the warp form (small supernodes) first
    int64_t nsmall = 0;
    int32_t* tsn = nullptr;           // dense finish: supernodes of at most 32 columns (a thread each)
    int64_t ntsn = 0;
    const void* tiles_plan = nullptr; // the supernodal plan the tiles were made for
};

template <class T>
struct UpdateArgs {
    DevTopo D;
    int32_t* w;
    T* up;
    T* dn;
    const int64_t* level_arc_off;
    int32_t levels;
    int64_t k;
    UpdateWorkspace ws;
    int* err;
    long long budget_ns;  // sweep time before the dense finish (0: dense from the start)
    int64_t max_arcs;     // evaluated arcs before the dense finish
    long long spin_limit; // spins of one barrier wait before ERR_TIMEOUT
    int barrier_extra;    // test hook: arrivals a barrier waits for beyond the grid (0)
    int64_t small_arcs;   // one-CTA sweep: evaluated arcs before it hands over to the grid sweep
    long long small_ns;   // one-CTA sweep: time before it hands over (changes that climb
                          // thousands of elimination levels go faster with the whole grid)
    int32_t resume_level; // >= 0: continue a handed-over sweep at this level (steps 1-2 done)
    int32_t resume_counted;  // the resumed level's arcs are already in the evaluated count
};

static constexpr int kStatWords = 16;

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ int32_t ldcg(const int32_t* p) { return __ldcg(p); }
__device__ __forceinline__ int64_t ldcg(const int64_t* p) {
    return (int64_t)__ldcg(reinterpret_cast<const long long*>(p));
}

template <class T>
static __device__ __forceinline__ void enqueue(const UpdateArgs<T>& A, int32_t c) {
    // byte flags, claimed with an atomic on the containing 32-bit word
    unsigned int* word = reinterpret_cast<unsigned int*>(A.ws.queued + (c & ~3));
    const unsigned int bit = 1u << (8 * (c & 3));
    if (atomicOr(word, bit) & bit) return;
    const int32_t L = A.D.vlevel[A.D.tail[c]];
    const int32_t pos = atomicAdd(&A.ws.bcount[L], 1);
    if (pos >= A.level_arc_off[L + 1] - A.level_arc_off[L]) {  // more arcs than the level has: cannot happen
        atomicOr(A.err, ERR_TOPOLOGY);
        return;
    }
    A.ws.bucket[A.level_arc_off[L] + pos] = c;
    atomicOr(&A.ws.pending[L >> 5], 1u << (L & 31));
}

// Bounded grid barrier. Returns false if it timed out (ERR_TIMEOUT recorded).
// A one-CTA sweep (gridDim 1) only needs the block's barrier.
template <class T>
static __device__ bool grid_sync(const UpdateArgs<T>& A) {
    if (gridDim.x == 1) {
        __syncthreads();
        return true;
    }
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long* count = A.ws.stats + 5;
        volatile unsigned long long* gen = A.ws.stats + 6;
        const unsigned long long g = *gen;
        __threadfence();
        ok = 1;
        if (atomicAdd(count, 1ull) == (unsigned long long)gridDim.x + A.barrier_extra - 1) {
            *count = 0;
            __threadfence();
            atomicAdd((unsigned long long*)gen, 1ull);
        } else {
            long long spins = 0;
            while (*gen == g) {
                __nanosleep(100);
                if (++spins > A.spin_limit) {
                    atomicOr(A.err, ERR_TIMEOUT);
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

static __device__ __forceinline__ int64_t find_in_row(const DevTopo& D, int64_t lo, int64_t hi, int32_t z) {
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (D.head[mid] < z) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// The pending levels from `from` up join the cleanup list of a stopped sweep.
template <class T>
static __device__ void list_pending_from(const UpdateArgs<T>& A, int32_t from) {
    unsigned long long d = A.ws.stats[3];
    for (int32_t wi = from >> 5; wi < ((A.levels + 31) >> 5); wi++) {
        uint32_t bits = __ldcg(A.ws.pending + wi);
        if (wi == (from >> 5)) bits &= ~((1u << (from & 31)) - 1u);
        while (bits && d < (unsigned long long)A.levels) {
            A.ws.done_levels[d++] = wi * 32 + __ffs(bits) - 1;
            bits &= bits - 1;
        }
    }
    A.ws.stats[3] = d;
}

template <class T>
__global__ void __launch_bounds__(256) k_update(UpdateArgs<T> A) {
    const DevTopo& D = A.D;
    const int lane = threadIdx.x & 31;
    const int64_t gtid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t gthreads = (int64_t)gridDim.x * blockDim.x;
    const int64_t gwarp = gtid >> 5, gwarps = gthreads >> 5;
    int e = 0;
    unsigned long long t_start = 0;
    const bool small = gridDim.x == 1;  // the one-CTA sweep of a small update
    // a level may be left part way when the sweep runs out of time: the top
    // separators' levels hold arcs whose lower triangles number in the
    // thousands each, and one such level outlasts the whole budget
    const long long limit = small ? A.small_ns : A.budget_ns;
    __shared__ unsigned long long t_block;
    if (threadIdx.x == 0) t_block = globaltimer_ns();
    if (gtid == 0) {
        t_start = globaltimer_ns();
        if (A.budget_ns <= 0) A.ws.stats[8] = 1;  // dense from the first level
    }
    if (A.resume_level < 0) {
        // 1. new weights (python/cch.py:357-360)
        for (int64_t j = gtid; j < A.k; j += gthreads) A.w[A.ws.edge_idx[j]] = A.ws.new_w[j];
        if (!grid_sync(A)) return;
        // 2. queue the arcs the changed original arcs map to
        for (int64_t j = gtid; j < A.k; j += gthreads) {
            const int64_t c = D.e_arc[A.ws.edge_idx[j]];
            if (c >= 0) enqueue(A, (int32_t)c);
        }
        if (!grid_sync(A)) return;
    }
    // 3. levels, lowest first (python/cch.py:376-401)
    __shared__ int32_t next_level;
    int32_t L = A.resume_level < 0 ? -1 : A.resume_level - 1;
    bool stopped = false;
    // a stop request for iteration i is written during iteration i-1 into
    // word 8 + (i & 1), so no block reads a word while it is being written
    for (int iter = 0;; iter++) {
        if (threadIdx.x < 32) {
            int32_t found = -1;
            const int32_t words = (A.levels + 31) >> 5;
            for (int32_t w0 = (L + 1) >> 5; w0 < words && found < 0; w0 += 32) {
                const int32_t wi = w0 + lane;
                uint32_t bits = wi < words ? __ldcg(A.ws.pending + wi) : 0u;
                if (wi == ((L + 1) >> 5)) bits &= ~((1u << ((L + 1) & 31)) - 1u);
                const unsigned m = __ballot_sync(0xffffffffu, bits != 0);
                if (m) {
                    const int src = __ffs(m) - 1;
                    const uint32_t b = __shfl_sync(0xffffffffu, bits, src);
                    found = (w0 + src) * 32 + __ffs(b) - 1;
                }
            }
            if (lane == 0) next_level = found;
        }
        __syncthreads();
        L = next_level;
        if (L < 0) break;
        if (small && __ldcg(A.ws.stats + 8 + (iter & 1))) {
            // the one-CTA sweep has grown: the grid sweep continues at L
            if (gtid == 0) A.ws.stats[10] = (unsigned long long)L + 1;
            if (e) atomicOr(A.err, e);
            return;
        }
        if (__ldcg(A.ws.stats + 8 + (iter & 1))) {
            stopped = true;
            if (gtid == 0) {
                A.ws.stats[7] = (unsigned long long)L + 1;
                list_pending_from(A, L);
            }
            break;
        }
        const int64_t base = A.level_arc_off[L];
        const int32_t cnt = (int32_t)min((int64_t)__ldcg(A.ws.bcount + L), A.level_arc_off[L + 1] - base);
        // a level handed over part way by the one-CTA sweep is evaluated
        // again whole (its evaluated arcs keep their values: their lower
        // sides are final) but is counted and listed once
        if (gtid == 0 && !(iter == 0 && A.resume_counted && L == A.resume_level)) {
            const unsigned long long d = atomicAdd(A.ws.stats + 3, 1ull);
            if (d < (unsigned long long)A.levels) A.ws.done_levels[d] = L;  // (a level is done once)
            atomicAdd(A.ws.stats + 0, (unsigned long long)cnt);
        }
        for (int64_t i = gwarp; i < cnt; i += gwarps) {
            // out of time: the warp stops before its next arc (an arc once
            // started is finished, with its changes queued)
            // (word 11 + (iter & 1): a word read after this level's barrier
            // is never written by a block already in the next level)
            int out = 0;
            if (lane == 0)
                out = __ldcg(A.ws.stats + 11 + (iter & 1)) != 0 || (long long)(globaltimer_ns() - t_block) > limit;
            if (__shfl_sync(0xffffffffu, out, 0)) {
                if (lane == 0) A.ws.stats[11 + (iter & 1)] = 1;
                break;
            }
            const int32_t c = __ldcg(A.ws.bucket + base + i);
            const int32_t y = D.tail[c], z = D.head[c];
            T nu = Lim<T>::INF, nd = Lim<T>::INF;
            for (int64_t j = D.aeoff[c] + lane; j < D.aeoff[c + 1]; j += 32) {
                const int32_t k = D.aeidx[j];
                const T wk = (T)__ldcg(A.w + k);
                if (D.e_up[k]) nu = min(nu, wk);
                else nd = min(nd, wk);
            }
            // lower triangles (x; y, z): x below y whose row holds z
            for (int64_t j = D.doff[y] + lane; j < D.doff[y + 1]; j += 32) {
                const int32_t a = D.darc[j];
                const int64_t rend = D.first[D.tail[a] + 1];
                const int64_t b = find_in_row(D, a + 1, rend, z);
                if (b >= rend || D.head[b] != z) continue;
                T v;
                if (splus(ldcg(A.dn + a), ldcg(A.up + b), v, e)) nu = min(nu, v);
                if (splus(ldcg(A.dn + b), ldcg(A.up + a), v, e)) nd = min(nd, v);
            }
            for (int o = 16; o > 0; o >>= 1) {
                nu = min(nu, (T)__shfl_xor_sync(0xffffffffu, nu, o));
                nd = min(nd, (T)__shfl_xor_sync(0xffffffffu, nd, o));
            }
            const T ou = ldcg(A.up + c), od = ldcg(A.dn + c);
            if (nu == ou && nd == od) continue;
            if (lane == 0) {
                A.up[c] = nu;
                A.dn[c] = nd;
                A.ws.chg[c] = 1;
                const unsigned long long p = atomicAdd(A.ws.stats + 1, 1ull);
                if (p < (unsigned long long)D.m_plus) A.ws.changed[p] = c;  // (an arc changes once)
                if (negative_pair(nu, nd)) atomicAdd(A.ws.stats + 2, 1ull);
            }
            // every triangle (y; v, z) or (y; z, v) of row y has c as a lower side
            for (int64_t kk = D.first[y] + lane; kk < D.first[y + 1]; kk += 32) {
                if (kk == c) continue;
                const int32_t v = D.head[kk];
                const int32_t lo = min(v, z), hi = max(v, z);
                const int64_t r = find_in_row(D, D.first[lo], D.first[lo + 1], hi);
                if (r >= D.first[lo + 1] || D.head[r] != hi) {
                    e |= ERR_TOPOLOGY;
                    continue;
                }
                enqueue(A, (int32_t)r);
            }
        }
        if (gtid == 0 && (small ? ((long long)A.ws.stats[0] > A.small_arcs ||
                                   (long long)(globaltimer_ns() - t_start) > A.small_ns)
                                : ((long long)(globaltimer_ns() - t_start) > A.budget_ns ||
                                   (long long)A.ws.stats[0] > A.max_arcs))) {
            A.ws.stats[8 + ((iter + 1) & 1)] = 1;
        }
        if (!grid_sync(A)) return;
        if (__ldcg(A.ws.stats + 11 + (iter & 1))) {
            // level L was left part way (its arcs are all in the evaluated
            // count and L in the cleanup list): the one-CTA sweep hands it
            // over whole, the grid sweep stops for the dense finish, which
            // counts from level L + 1 (stats[13])
            if (gtid == 0) {
                A.ws.stats[13] = 1;
                if (small) A.ws.stats[10] = (unsigned long long)L + 1;
                else {
                    A.ws.stats[7] = (unsigned long long)L + 1;
                    list_pending_from(A, L + 1);
                }
            }
            if (small) {
                if (e) atomicOr(A.err, e);
                return;
            }
            stopped = true;
            break;
        }
    }
    if (stopped) {  // the host finishes densely and cleans the workspace
        if (e) atomicOr(A.err, e);
        return;
    }
    // 4. clean the workspace for the next call
    const int64_t nchanged = min((int64_t)__ldcg(A.ws.stats + 1), D.m_plus);
    for (int64_t j = gtid; j < nchanged; j += gthreads) A.ws.chg[__ldcg(A.ws.changed + j)] = 0;
    const int32_t nd_levels = (int32_t)min((int64_t)__ldcg(A.ws.stats + 3), (int64_t)A.levels);
    for (int32_t li = 0; li < nd_levels; li++) {
        const int32_t l = __ldcg(A.ws.done_levels + li);
        const int64_t base = A.level_arc_off[l];
        const int32_t cnt = (int32_t)min((int64_t)__ldcg(A.ws.bcount + l), A.level_arc_off[l + 1] - base);
        for (int64_t i = gtid; i < cnt; i += gthreads) A.ws.queued[__ldcg(A.ws.bucket + base + i)] = 0;
    }
    if (!grid_sync(A)) return;
    for (int32_t li = gtid; li < nd_levels; li += gthreads) {
        const int32_t l = A.ws.done_levels[li];
        A.ws.bcount[l] = 0;
        A.ws.pending[l >> 5] = 0;
    }
    if (e) atomicOr(A.err, e);
}

// ---------------------------------------------------------------- dense finish

// Arcs whose full re-customization differs are changed: new values written,
// appended to the changed list, flagged, negative pairs counted.
template <class T>
__global__ void __launch_bounds__(256) k_dense_diff(int64_t m_plus, T* __restrict__ up, T* __restrict__ dn,
                                                    const T* __restrict__ up2, const T* __restrict__ dn2,
                                                    uint8_t* __restrict__ chg, int32_t* __restrict__ changed,
                                                    unsigned long long* __restrict__ stats) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t base = warp * 32; base < m_plus; base += nwarps * 32) {
        const int64_t c = base + lane;
        T nu = 0, nd = 0;
        bool d = false;
        if (c < m_plus) {
            nu = up2[c];
            nd = dn2[c];
            d = nu != up[c] || nd != dn[c];
        }
        const unsigned mask = __ballot_sync(0xffffffffu, d);
        if (!mask) continue;
        const unsigned neg = __ballot_sync(0xffffffffu, d && negative_pair(nu, nd));
        unsigned long long p0 = 0;
        if (lane == 0) {
            p0 = atomicAdd(stats + 1, (unsigned long long)__popc(mask));
            if (neg) atomicAdd(stats + 2, (unsigned long long)__popc(neg));
        }
        p0 = __shfl_sync(0xffffffffu, p0, 0);
        if (d) {
            up[c] = nu;
            dn[c] = nd;
            chg[c] = 1;
            const unsigned long long pos = p0 + __popc(mask & ((1u << lane) - 1u));
            if (pos < (unsigned long long)m_plus) changed[pos] = (int32_t)c;
        }
    }
}

// dq[a] = 1 for every arc a with a lower triangle that has a changed side.
// Supernode S (rows s0..s0+k-1, columns j of row i for i < j < k+b; column j
// is vertex s0+j below k and boundary vertex B[j-k] from k on):
//  - the triangles below target (p, j) inside S are (i; p, j) for i < p: the
//    target is marked if a side (i, p) or (i, j) changed, a column flag
//    above row p in column p or in column j;
//  - every row of S holds all of B, so S is the bottom of a triangle below
//    every boundary pair (B[p], B[q]): marked if column k+p or k+q of S
//    has a changed arc. Every lower triangle is one of the two kinds.
// Two passes over (supernode, 32-column tile) blocks: a lane per column, the
// block's 8 warps each over an eighth of the rows (coalesced across the
// tile), combined through shared memory: the column flags first (acol[s0 + j]
// inside, bflag at the column's last-row arc on the boundary), then the
// marks, each warp starting from the OR of the row segments above its own.
constexpr int kMarkWarps = 8;

// Supernodes of at most 32 columns (k + b <= 32: nearly all of a road-like
// graph's, one to a few rows each) take a thread each, both passes at once.
// Their arcs are one contiguous range (row p follows row p - 1), walked in
// order with a bit per column: bit j of `above` = an arc above the current
// row in column j changed. Target (p, j) is marked when bit j (a side (i, j),
// i < p) or bit p (a side (i, p)) is set, as in k_dense_mark; after the last
// row the bits of the boundary columns decide the boundary pairs.
__global__ void __launch_bounds__(256)
    k_dense_thread(DevTopo D, SnDev S, const int32_t* __restrict__ items, int64_t nitems,
                   const uint8_t* __restrict__ chg, uint8_t* __restrict__ dq) {
    for (int64_t it = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; it < nitems;
         it += (int64_t)gridDim.x * blockDim.x) {
        const int32_t sn = items[it];
        const int32_t s0 = S.s0[sn], k = S.k[sn], b = S.b[sn];
        const int32_t cols = k + b;  // <= 32 (host-checked)
        int64_t a = D.first[s0];
        uint32_t above = 0;
        for (int32_t p = 0; p < k; p++) {
            uint32_t row = 0;
            for (int32_t j = p + 1; j < cols; j++, a++) {
                if (((above >> j) | (above >> p)) & 1u) dq[a] = 1;
                if (chg[a]) row |= 1u << j;
            }
            above |= row;
        }
        if (b > 1) {  // (then k <= 30)
            const uint32_t B = above >> k;
            if (!B) continue;
            const int64_t ro = S.rel_off[sn];
            for (int32_t q = 1; q < b; q++)
                for (int32_t p = 0; p < q; p++)
                    if (((B >> p) | (B >> q)) & 1u) dq[S.rel[ro + (int64_t)p * (2 * b - p - 1) / 2 + (q - p - 1)]] = 1;
        }
    }
}

// Supernodes of at most kWarpTileRows rows and kWarpTileBoundary boundary
// columns (at the bottom of road-like graphs: tens of millions of them, one
// to a few rows each) take a warp per tile instead: a lane per column walks
// the rows, and its boundary pairs, in order, with no block barrier. Longer
// boundaries keep the block's 8 warps on their pairs.
constexpr int kWarpTileRows = 32;
constexpr int kWarpTileBoundary = 256;

__global__ void __launch_bounds__(256, 4)
    k_dense_cols_warp(DevTopo D, SnDev S, const int2* __restrict__ tiles, int64_t ntiles,
                      const uint8_t* __restrict__ chg, uint8_t* __restrict__ acol, uint8_t* __restrict__ bflag) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t it = warp; it < ntiles; it += nwarps) {
        const int2 tl = tiles[it];
        const int32_t s0 = S.s0[tl.x], k = S.k[tl.x], b = S.b[tl.x];
        const int32_t j = tl.y * 32 + lane;
        if (j >= k + b) continue;
        const int32_t rows = min(j, k);
        uint8_t r = 0;
        for (int32_t p = 0; p < rows; p++) r |= chg[D.first[s0 + p] + (j - p - 1)];
        if (j < k) acol[s0 + j] = r;
        else bflag[D.first[s0 + k - 1] + (j - k)] = r;
    }
}

__global__ void __launch_bounds__(256, 4)
    k_dense_mark_warp(DevTopo D, SnDev S, const int2* __restrict__ tiles, int64_t ntiles,
                      const uint8_t* __restrict__ chg, uint8_t* __restrict__ dq, const uint8_t* __restrict__ acol,
                      const uint8_t* __restrict__ bflag) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t it = warp; it < ntiles; it += nwarps) {
        const int2 tl = tiles[it];
        const int32_t s0 = S.s0[tl.x], k = S.k[tl.x], b = S.b[tl.x];
        const int32_t j = tl.y * 32 + lane;
        if (j >= k + b) continue;
        const int32_t rows = min(j, k);
        uint8_t r = 0;
        for (int32_t p = 0; p < rows; p++) {
            const int64_t a = D.first[s0 + p] + (j - p - 1);
            if (r || (p > 0 && acol[s0 + p])) dq[a] = 1;
            r |= chg[a];
        }
        if (j >= k) {  // boundary pairs (B[p], B[q]), q = j - k, as in k_dense_mark
            const int32_t q = j - k;
            const int64_t last = D.first[s0 + k - 1];
            const uint8_t aq = bflag[last + q];
            const int64_t ro = S.rel_off[tl.x];
            for (int32_t p = 0; p < q; p++)
                if (aq | bflag[last + p]) dq[S.rel[ro + (int64_t)p * (2 * b - p - 1) / 2 + (q - p - 1)]] = 1;
        }
    }
}

__global__ void __launch_bounds__(32 * kMarkWarps)
    k_dense_cols(DevTopo D, SnDev S, const int2* __restrict__ tiles, int64_t ntiles, const uint8_t* __restrict__ chg,
                 uint8_t* __restrict__ acol, uint8_t* __restrict__ bflag) {
    __shared__ uint8_t seg[kMarkWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int64_t it = blockIdx.x; it < ntiles; it += gridDim.x) {
        const int2 tl = tiles[it];
        const int32_t s0 = S.s0[tl.x], k = S.k[tl.x], b = S.b[tl.x];
        const int32_t j = tl.y * 32 + lane;
        const int32_t rows = j < k + b ? min(j, k) : 0;
        const int32_t per = (k + kMarkWarps - 1) / kMarkWarps, p0 = w * per, p1 = min(rows, p0 + per);
        uint8_t r = 0;
        for (int32_t p = p0; p < p1; p++) r |= chg[D.first[s0 + p] + (j - p - 1)];
        seg[w][lane] = r;
        __syncthreads();
        if (w == 0 && j < k + b) {
            uint8_t t = 0;
#pragma unroll
            for (int i = 0; i < kMarkWarps; i++) t |= seg[i][lane];
            if (j < k) acol[s0 + j] = t;
            else bflag[D.first[s0 + k - 1] + (j - k)] = t;
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(32 * kMarkWarps)
    k_dense_mark(DevTopo D, SnDev S, const int2* __restrict__ tiles, int64_t ntiles, const uint8_t* __restrict__ chg,
                 uint8_t* __restrict__ dq, const uint8_t* __restrict__ acol, const uint8_t* __restrict__ bflag) {
    __shared__ uint8_t seg[kMarkWarps][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int64_t it = blockIdx.x; it < ntiles; it += gridDim.x) {
        const int2 tl = tiles[it];
        const int32_t s0 = S.s0[tl.x], k = S.k[tl.x], b = S.b[tl.x];
        const int32_t j = tl.y * 32 + lane;
        const int32_t rows = j < k + b ? min(j, k) : 0;
        const int32_t per = (k + kMarkWarps - 1) / kMarkWarps, p0 = w * per, p1 = min(rows, p0 + per);
        uint8_t r = 0;
        for (int32_t p = p0; p < p1; p++) r |= chg[D.first[s0 + p] + (j - p - 1)];
        seg[w][lane] = r;
        __syncthreads();
        r = 0;
        for (int i = 0; i < w; i++) r |= seg[i][lane];
        for (int32_t p = p0; p < p1; p++) {
            const int64_t a = D.first[s0 + p] + (j - p - 1);
            if (r || (p > 0 && acol[s0 + p])) dq[a] = 1;
            r |= chg[a];
        }
        if (j >= k && j < k + b) {
            // boundary pairs (B[p], B[q]) with q = j - k: marked if either
            // column of S has a changed arc
            const int32_t q = j - k;
            const int64_t last = D.first[s0 + k - 1];
            const uint8_t aq = bflag[last + q];
            const int64_t ro = S.rel_off[tl.x];
            for (int32_t p = w; p < q; p += kMarkWarps)
                if (aq | bflag[last + p]) dq[S.rel[ro + (int64_t)p * (2 * b - p - 1) / 2 + (q - p - 1)]] = 1;
        }
        __syncthreads();
    }
}

// Arcs of level >= L queued by the sweep before it stopped or marked above.
__global__ void __launch_bounds__(256) k_dense_count(DevTopo D, int32_t L, const uint8_t* __restrict__ queued,
                                                     const uint8_t* __restrict__ dq,
                                                     unsigned long long* __restrict__ stats) {
    unsigned long long c = 0;
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < D.m_plus;
         a += (int64_t)gridDim.x * blockDim.x)
        if ((queued[a] | dq[a]) && D.vlevel[D.tail[a]] >= L) c++;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(stats + 0, c);
}

// The workspace cleanup of the sweep, for a stopped sweep.
__global__ void __launch_bounds__(256) k_update_clean(UpdateWorkspace ws, const int64_t* __restrict__ level_arc_off,
                                                      int64_t m_plus, int32_t levels) {
    const int64_t nchanged = min((int64_t)ws.stats[1], m_plus);
    const int32_t nd_levels = (int32_t)min((int64_t)ws.stats[3], (int64_t)levels);
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < nchanged;
         j += (int64_t)gridDim.x * blockDim.x)
        ws.chg[ws.changed[j]] = 0;
    for (int32_t li = blockIdx.x; li < nd_levels; li += gridDim.x) {
        const int32_t l = ws.done_levels[li];
        const int64_t base = level_arc_off[l];
        const int32_t cnt = (int32_t)min((int64_t)ws.bcount[l], level_arc_off[l + 1] - base);
        for (int32_t i = threadIdx.x; i < cnt; i += blockDim.x) ws.queued[ws.bucket[base + i]] = 0;
        __syncthreads();
        if (threadIdx.x == 0) {
            ws.bcount[l] = 0;
            ws.pending[l >> 5] = 0;
        }
    }
}

static void free_workspace(UpdateWorkspace* ws) {
    if (!ws) return;
    cudaFree(ws->tiles);
    cudaFree(ws->tsn);
    cudaFree(ws->chg);
    cudaFree(ws->dq);
    cudaFree(ws->acol);
    cudaFree(ws->up2);
    cudaFree(ws->dn2);
    cudaFree(ws->queued);
    cudaFree(ws->bucket);
    cudaFree(ws->bcount);
    cudaFree(ws->pending);
    cudaFree(ws->done_levels);
    cudaFree(ws->changed);
    cudaFree(ws->edge_idx);
    cudaFree(ws->new_w);
    cudaFree(ws->stats);
    delete ws;
}

namespace {

struct Plans {
    UpdateWorkspace* update = nullptr;
};

void free_plans(nwcch_topology* t) {
    auto* p = static_cast<Plans*>(t->plans);
    if (!p) return;
    free_workspace(p->update);
    delete p;
    t->plans = nullptr;
}

int cooperative_blocks(const void* kernel, int* out) {
    int per_sm = 0, sms = 0, dev = 0;
    NWCCH_CUDA_TRY(cudaGetDevice(&dev));
    NWCCH_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    NWCCH_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0));
    if (per_sm < 1) return NWCCH_ERR_CUDA;
    *out = sms * std::min(per_sm, 4);
    return NWCCH_OK;
}

int get_workspace(nwcch_topology* t, int64_t k, UpdateWorkspace** out) {
    if (!t->plans) {
        t->plans = new (std::nothrow) Plans();
        if (!t->plans) return NWCCH_ERR_NOMEM;
        t->free_plans = free_plans;
    }
    auto* p = static_cast<Plans*>(t->plans);
    const int64_t mp = t->d.m_plus, L = t->levels;
    if (!p->update) {
        auto* ws = new (std::nothrow) UpdateWorkspace();
        if (!ws) return NWCCH_ERR_NOMEM;
        const size_t qbytes = (size_t)((mp + 3) & ~3LL) + 4;
        bool ok = cudaMalloc(&ws->queued, qbytes) == cudaSuccess &&
                  cudaMalloc(&ws->bucket, std::max<int64_t>(1, mp) * 4) == cudaSuccess &&
                  cudaMalloc(&ws->bcount, L * 4) == cudaSuccess &&
                  cudaMalloc(&ws->pending, ((L + 31) / 32) * 4) == cudaSuccess &&
                  cudaMalloc(&ws->done_levels, L * 4) == cudaSuccess &&
                  cudaMalloc(&ws->changed, std::max<int64_t>(1, mp) * 4) == cudaSuccess &&
                  cudaMalloc(&ws->chg, qbytes) == cudaSuccess && cudaMalloc(&ws->dq, qbytes) == cudaSuccess &&
                  cudaMalloc(&ws->acol, std::max<int64_t>(1, t->d.n)) == cudaSuccess &&
                  cudaMalloc(&ws->stats, kStatWords * sizeof(unsigned long long)) == cudaSuccess;
        if (ok)
            ok = cudaMemset(ws->queued, 0, qbytes) == cudaSuccess && cudaMemset(ws->bcount, 0, L * 4) == cudaSuccess &&
                 cudaMemset(ws->pending, 0, ((L + 31) / 32) * 4) == cudaSuccess &&
                 cudaMemset(ws->chg, 0, qbytes) == cudaSuccess && cudaMemset(ws->dq, 0, qbytes) == cudaSuccess &&
                 cudaMemset(ws->stats, 0, kStatWords * sizeof(unsigned long long)) == cudaSuccess &&
                 setup_copies_done() == cudaSuccess;
        if (ok) ok = cooperative_blocks((const void*)k_update<int32_t>, &ws->blocks32) == NWCCH_OK &&
                     cooperative_blocks((const void*)k_update<int64_t>, &ws->blocks64) == NWCCH_OK;
        if (!ok) {
            free_workspace(ws);
            return NWCCH_ERR_NOMEM;
        }
        p->update = ws;
    }
    UpdateWorkspace* ws = p->update;
    if (ws->cap < k) {
        cudaFree(ws->edge_idx);
        cudaFree(ws->new_w);
        ws->edge_idx = nullptr;
        ws->new_w = nullptr;
        const int64_t cap = std::max<int64_t>(k, 1024);
        if (cudaMalloc(&ws->edge_idx, cap * 8) != cudaSuccess || cudaMalloc(&ws->new_w, cap * 4) != cudaSuccess) {
            ws->cap = 0;
            return NWCCH_ERR_NOMEM;
        }
        ws->cap = cap;
    }
    *out = ws;
    return NWCCH_OK;
}

}  // namespace

// Every per-arc and per-level flag of the workspace back to zero (after a
// sweep that could not clean up after itself).
static int reset_workspace(nwcch_topology* t, UpdateWorkspace* ws, cudaStream_t s) {
    const int64_t mp = t->d.m_plus, L = t->levels;
    const size_t qbytes = (size_t)((mp + 3) & ~3LL) + 4;
    NWCCH_CUDA_TRY(cudaMemsetAsync(ws->queued, 0, qbytes, s));
    NWCCH_CUDA_TRY(cudaMemsetAsync(ws->chg, 0, qbytes, s));
    NWCCH_CUDA_TRY(cudaMemsetAsync(ws->dq, 0, qbytes, s));
    NWCCH_CUDA_TRY(cudaMemsetAsync(ws->bcount, 0, L * 4, s));
    NWCCH_CUDA_TRY(cudaMemsetAsync(ws->pending, 0, ((L + 31) / 32) * 4, s));
    NWCCH_CUDA_TRY(cudaMemsetAsync(ws->stats, 0, kStatWords * sizeof(unsigned long long), s));
    NWCCH_CUDA_TRY(cudaStreamSynchronize(s));
    return NWCCH_OK;
}

// Time the level sweep may take before the update is finished densely: about
// a quarter of a full customization (which runs near 4e11 triangles/s on a
// GB300), at least 0.2 ms; the autotuner measures a better one per
// topology. NWCCH_UPDATE_MODE=dense or =incremental forces one form.
long long sweep_budget_ns(const nwcch_topology* t) {
    const char* mode = getenv("NWCCH_UPDATE_MODE");
    if (mode && !strcmp(mode, "dense")) return 0;
    if (mode && !strcmp(mode, "incremental")) return LLONG_MAX;
    if (t->tune.update_budget_ns > 0) return t->tune.update_budget_ns;
    return std::max<long long>(200000, (long long)(t->triangles / 1600));
}

template <class T>
int finish_dense(nwcch_topology* t, UpdateWorkspace* ws, const int32_t* w_dev, T* up_dev, T* dn_dev, int32_t L,
                 cudaStream_t s) {
    auto* P = static_cast<SnPlan*>(t->sn_plan);
    const int64_t mp = t->d.m_plus;
    if (!P) return NWCCH_ERR_TOPOLOGY;
    if (!ws->up2) {
        if (cudaMalloc(&ws->up2, std::max<int64_t>(1, mp) * 8) != cudaSuccess) return NWCCH_ERR_NOMEM;
        if (cudaMalloc(&ws->dn2, std::max<int64_t>(1, mp) * 8) != cudaSuccess) {
            cudaFree(ws->up2);
            ws->up2 = nullptr;
            return NWCCH_ERR_NOMEM;
        }
    }
    T* up2 = static_cast<T*>(ws->up2);
    T* dn2 = static_cast<T*>(ws->dn2);
    int rc = launch_supernodal<T>(t, P, w_dev, up2, dn2, s);
    if (rc) return rc;
    k_dense_diff<T><<<grid_for(mp, 256), 256, 0, s>>>(mp, up_dev, dn_dev, up2, dn2, ws->chg, ws->changed, ws->stats);
    // up2 is free after the diff: its first m+ bytes hold the boundary
    // column flags
    uint8_t* bflag = static_cast<uint8_t*>(ws->up2);
    if (ws->tiles_plan != P) {  // work items of this plan: supernodes, (supernode, 32-column tile) pairs
        cudaFree(ws->tiles);
        cudaFree(ws->tsn);
        ws->tiles = nullptr;
        ws->tsn = nullptr;
        ws->tiles_plan = nullptr;
        std::vector<int32_t> kk(P->nsn), bb(P->nsn);
        NWCCH_CUDA_TRY(cudaMemcpy(kk.data(), P->dev.k, sizeof(int32_t) * P->nsn, cudaMemcpyDeviceToHost));
        NWCCH_CUDA_TRY(cudaMemcpy(bb.data(), P->dev.b, sizeof(int32_t) * P->nsn, cudaMemcpyDeviceToHost));
        std::vector<int2> tl;
        std::vector<int32_t> th;
        for (int64_t sn = 0; sn < P->nsn; sn++)
            if (kk[sn] + bb[sn] <= 32) th.push_back((int32_t)sn);
        for (int pass = 0; pass < 2; pass++) {  // small supernodes first
            for (int64_t sn = 0; sn < P->nsn; sn++)
                if (kk[sn] + bb[sn] > 32 && (kk[sn] <= kWarpTileRows && bb[sn] <= kWarpTileBoundary) == (pass == 0))
                    for (int32_t c = 0; c * 32 < kk[sn] + bb[sn]; c++) tl.push_back(make_int2((int)sn, c));
            if (pass == 0) ws->nsmall = (int64_t)tl.size();
        }
        if (cudaMalloc(&ws->tsn, sizeof(int32_t) * std::max<size_t>(1, th.size())) != cudaSuccess)
            return NWCCH_ERR_NOMEM;
        if (!th.empty())
            NWCCH_CUDA_TRY(cudaMemcpy(ws->tsn, th.data(), sizeof(int32_t) * th.size(), cudaMemcpyHostToDevice));
        ws->ntsn = (int64_t)th.size();
        if (cudaMalloc(&ws->tiles, sizeof(int2) * std::max<size_t>(1, tl.size())) != cudaSuccess)
            return NWCCH_ERR_NOMEM;
        if (!tl.empty())
            NWCCH_CUDA_TRY(cudaMemcpy(ws->tiles, tl.data(), sizeof(int2) * tl.size(), cudaMemcpyHostToDevice));
        NWCCH_CUDA_TRY(setup_copies_done());
        ws->ntiles = (int64_t)tl.size();
        ws->tiles_plan = P;
    }
    // the column flags of every supernode before any mark reads them
    const int64_t nbig = ws->ntiles - ws->nsmall;
    const int2* big = ws->tiles + ws->nsmall;
    const unsigned wgrid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((ws->nsmall + 7) / 8, (int64_t)t->sms * 8));
    const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>(nbig, (int64_t)t->sms * 8));
    if (ws->ntsn)
        k_dense_thread<<<(unsigned)std::min<int64_t>((ws->ntsn + 255) / 256, (int64_t)t->sms * 16), 256, 0, s>>>(
            t->d, P->dev, ws->tsn, ws->ntsn, ws->chg, ws->dq);
    if (ws->nsmall)
        k_dense_cols_warp<<<wgrid, 256, 0, s>>>(t->d, P->dev, ws->tiles, ws->nsmall, ws->chg, ws->acol, bflag);
    if (nbig) k_dense_cols<<<grid, 32 * kMarkWarps, 0, s>>>(t->d, P->dev, big, nbig, ws->chg, ws->acol, bflag);
    if (ws->nsmall)
        k_dense_mark_warp<<<wgrid, 256, 0, s>>>(t->d, P->dev, ws->tiles, ws->nsmall, ws->chg, ws->dq, ws->acol,
                                                bflag);
    if (nbig)
        k_dense_mark<<<grid, 32 * kMarkWarps, 0, s>>>(t->d, P->dev, big, nbig, ws->chg, ws->dq, ws->acol, bflag);
    k_dense_count<<<grid_for(mp, 256), 256, 0, s>>>(t->d, L, ws->queued, ws->dq, ws->stats);
    k_update_clean<<<t->sms * 4, 256, 0, s>>>(*ws, t->d_level_arc_off, mp, t->levels);
    NWCCH_CUDA_TRY(cudaGetLastError());
    NWCCH_CUDA_TRY(cudaMemsetAsync(ws->dq, 0, (size_t)mp, s));
    return NWCCH_OK;
}

template <class T>
int update(nwcch_topology* t, int32_t* w_dev, T* up_dev, T* dn_dev, const int64_t* edge_idx, const int32_t* new_w,
           int64_t k, int64_t* stats, int32_t* changed_dev, cudaStream_t s) {
    // the last write to an original arc wins, as in the reference's loop
    std::vector<int64_t> idx;
    std::vector<int32_t> val;
    {
        std::vector<int64_t> order(k);
        for (int64_t j = 0; j < k; j++) {
            if (edge_idx[j] < 0 || edge_idx[j] >= t->d.m || new_w[j] == INF32) return NWCCH_ERR_ARG;
            order[j] = j;
        }
        std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return edge_idx[a] < edge_idx[b]; });
        for (int64_t j = 0; j < k; j++) {
            const int64_t o = order[j];
            if (j + 1 < k && edge_idx[order[j + 1]] == edge_idx[o]) continue;
            idx.push_back(edge_idx[o]);
            val.push_back(new_w[o]);
        }
    }
    const int64_t kk = (int64_t)idx.size();
    std::lock_guard<std::mutex> lock(t->mu);
    UpdateWorkspace* ws = nullptr;
    int rc = get_workspace(t, kk, &ws);
    if (rc) return rc;
    if (kk) {
        NWCCH_CUDA_TRY(cudaMemcpyAsync(ws->edge_idx, idx.data(), kk * 8, cudaMemcpyHostToDevice, s));
        NWCCH_CUDA_TRY(cudaMemcpyAsync(ws->new_w, val.data(), kk * 4, cudaMemcpyHostToDevice, s));
    }
    NWCCH_CUDA_TRY(cudaMemsetAsync(ws->stats, 0, kStatWords * sizeof(unsigned long long), s));
    UpdateArgs<T> A;
    A.D = t->d;
    A.w = w_dev;
    A.up = up_dev;
    A.dn = dn_dev;
    A.level_arc_off = t->d_level_arc_off;
    A.levels = t->levels;
    A.k = kk;
    A.ws = *ws;
    A.err = stream_slot(t, s).err;
    // large updates touch most of the top separators: finish densely at once
    A.budget_ns = (t->tune.update_dense_min > 0 && kk >= t->tune.update_dense_min) ? 0 : sweep_budget_ns(t);
    A.max_arcs = std::max<int64_t>(4096, t->d.m_plus / 8);
    A.spin_limit = t->tune.update_spin_limit;
    A.barrier_extra = t->tune.test_barrier_extra;
    A.small_arcs = t->tune.update_small_arcs;
    A.small_ns = t->tune.update_small_ns;
    A.resume_level = -1;
    A.resume_counted = 0;
    void* args[] = {&A};
    const int blocks = sizeof(T) == 4 ? ws->blocks32 : ws->blocks64;
    unsigned long long h[kStatWords];
    int herr = 0;
    bool grid_sweep = true;
    if (A.budget_ns > 0 && A.small_arcs > 0) {
        // a small change first sweeps in one CTA, with block barriers; if it
        // grows past small_arcs evaluated arcs it hands its pending levels
        // to the grid sweep (stats[10] = the level to resume at, plus one)
        k_update<T><<<1, 256, 0, s>>>(A);
        NWCCH_CUDA_TRY(cudaGetLastError());
        NWCCH_CUDA_TRY(cudaMemcpyAsync(h, ws->stats, sizeof(h), cudaMemcpyDeviceToHost, s));
        NWCCH_CUDA_TRY(cudaStreamSynchronize(s));
        grid_sweep = h[10] != 0;
        if (grid_sweep) {
            A.resume_level = (int32_t)(h[10] - 1);
            A.resume_counted = h[13] != 0;
            // the stop requests, the hand-over words and the part-way flags
            // (words 8-13) back to zero; the counts stay
            NWCCH_CUDA_TRY(cudaMemsetAsync(ws->stats + 8, 0, 6 * sizeof(unsigned long long), s));
        }
    }
    if (grid_sweep)
        NWCCH_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_update<T>, dim3(blocks), dim3(256), args, 0, s));
    NWCCH_CUDA_TRY(cudaMemcpyAsync(h, ws->stats, sizeof(h), cudaMemcpyDeviceToHost, s));
    NWCCH_CUDA_TRY(cudaMemcpyAsync(&herr, A.err, sizeof(int), cudaMemcpyDeviceToHost, s));
    NWCCH_CUDA_TRY(cudaStreamSynchronize(s));
    if (herr & ERR_TIMEOUT) {
        // a barrier wait ran out: the blocks left without the sweep's
        // cleanup, so the queued flags, bucket counts, pending bits and
        // change flags are reset here; w holds the new weights and up/dn are
        // partly updated (the caller customizes again)
        rc = reset_workspace(t, ws, s);
        const int rc2 = consume_error(t, s);
        return rc ? rc : rc2;
    }
    if (h[7]) {  // the sweep stopped at level h[7] - 1: finish densely
        // (from the level above when that level was left part way: its arcs
        // are counted already)
        rc = finish_dense<T>(t, ws, w_dev, up_dev, dn_dev, (int32_t)(h[7] - 1) + (h[13] ? 1 : 0), s);
        if (rc) return rc;
        NWCCH_CUDA_TRY(cudaMemcpyAsync(h, ws->stats, sizeof(h), cudaMemcpyDeviceToHost, s));
        NWCCH_CUDA_TRY(cudaStreamSynchronize(s));
    }
    if (h[1] > (unsigned long long)t->d.m_plus) return NWCCH_ERR_TOPOLOGY;  // an arc changed twice: inconsistent state
    if (changed_dev && h[1])
        NWCCH_CUDA_TRY(cudaMemcpyAsync(changed_dev, ws->changed, h[1] * 4, cudaMemcpyDeviceToDevice, s));
    rc = consume_error(t, s);
    stats[0] = (int64_t)h[0];
    stats[1] = (int64_t)h[1];
    stats[2] = (int64_t)h[2];
    return rc;
}

}  // namespace nwcch

using namespace nwcch;

extern "C" int nwcch_update(nwcch_topology* t, int32_t* w_dev, int32_t* up_dev, int32_t* dn_dev,
                            const int64_t* edge_idx, const int32_t* new_w, int64_t k, int64_t* stats,
                            int32_t* changed_dev, void* stream) {
    if (!t || (t->d.m > 0 && !w_dev) || (t->d.m_plus > 0 && (!up_dev || !dn_dev)) || k < 0 || (k > 0 && (!edge_idx || !new_w)) || !stats)
        return NWCCH_ERR_ARG;
    return update<int32_t>(t, w_dev, up_dev, dn_dev, edge_idx, new_w, k, stats, changed_dev, (cudaStream_t)stream);
}

extern "C" int nwcch_update_i64(nwcch_topology* t, int32_t* w_dev, int64_t* up_dev, int64_t* dn_dev,
                                const int64_t* edge_idx, const int32_t* new_w, int64_t k, int64_t* stats,
                                int32_t* changed_dev, void* stream) {
    if (!t || (t->d.m > 0 && !w_dev) || (t->d.m_plus > 0 && (!up_dev || !dn_dev)) || k < 0 || (k > 0 && (!edge_idx || !new_w)) || !stats)
        return NWCCH_ERR_ARG;
    return update<int64_t>(t, w_dev, up_dev, dn_dev, edge_idx, new_w, k, stats, changed_dev, (cudaStream_t)stream);
}
