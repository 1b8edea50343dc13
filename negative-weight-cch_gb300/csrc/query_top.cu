// Batched elimination-tree queries: the top of the tree as (min,+) products
// over many chains at once.
//
// A query sweeps the ancestor chain of s with up weights and that of t with
// dn weights (python/cch_nb.py:577-615). On road-like graphs nearly all of a
// chain's arcs lie in the few large supernodes near the root (the top
// separators), and every chain of a batch crosses them: per query the same
// trapezoids are read again. Here a batch is swept in three phases:
//
//  1. k_qlow, a warp per chain: the chain's lower part, supernode by
//     supernode as in the per-query kernel, up to the first vertex whose
//     supernode belongs to the top set (supernodes whose elimination subtree
//     holds at least tau vertices; the set is closed upwards). The chain's
//     labels, indexed by elimination-tree depth, go to a global row; the
//     chain is bucketed by its entry supernode (numbered in depth-first order
//     of the top tree, so that the chains crossing a top supernode S - those
//     entering at S or below it - form one contiguous run of buckets).
//  2. k_qtop, once per level of the top set, bottom up: a CTA takes a tile of
//     up to 32 chains crossing one supernode S (k rows, b boundary columns),
//     loads their labels of S's rows and boundary into shared memory and
//     solves the (min,+) triangular system of S for all of them: per 32-row
//     block a shuffle solve of the diagonal triangle (a warp per chain), then
//     the block's product with the columns to the right, where every weight
//     read from L2 serves the whole tile. Rows below a chain's entry row
//     (which are not its ancestors) hold "no path". A chain crosses one
//     supernode per level, so the tiles of a level write disjoint labels.
//  3. k_qmeet, a warp per query: the depth of the lowest common ancestor of s
//     and t (found during the lower sweep, or in the top tree by binary
//     lifting and a search of the supernode's rows by preorder intervals),
//     then the minimum of forward + backward labels over the depths up to it:
//     below that depth both chains hold the same vertices.
//
// Every label and sum is the 32-bit DPX form of the per-query kernel (values
// within +-2^28 when max|w| * (depth + 2) <= 2^28); batches outside that
// bound fall through to the 64-bit kernel, as there. Results equal the
// per-query kernels' exactly: the (min,+) relaxations are the same, in
// another order, and integer minima do not depend on order.

#include <algorithm>
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>
#include <vector>

#include "query_sn.cuh"

namespace nwcch {

namespace {

constexpr int QT_THREADS = 256;           // threads of a top-supernode CTA
constexpr int QT_MAX_CT = 32;             // chains in one tile
constexpr int64_t QT_SMEM = 100 * 1024;   // label tile per CTA (two CTAs an SM) ...
constexpr int64_t QT_SMEM_MAX = 200 * 1024;  // ... or one, for the widest supernodes
constexpr int64_t QL_SMEM = 200 * 1024;   // lower-sweep labels per block
constexpr int64_t QT_LABEL_BYTES = (int64_t)4 << 30;  // label rows of one pass over a batch

struct TopDev {
    const int32_t* top_dfs;  // [nsn] depth-first index of a top supernode, -1 below the top
    const int32_t* dfs_sn;   // [ntop] supernode of each depth-first index
    const int32_t* dfs_end;  // [ntop] end of its subtree's depth-first range
    const int32_t* lift;     // [J][ntop] 2^j-th ancestor in the top tree (-1 past a root)
    const int32_t* tin;      // [n] preorder index in the elimination tree
    const int32_t* tout;     // [n] tin + subtree size
    int32_t ntop;
    int32_t J;
};

struct TopPlan {
    std::vector<int64_t> lvl_off;     // [levels + 1] into the level order
    std::vector<int32_t> lvl_ct;      // chains per tile of each level (32, 16 or 8)
    std::vector<int32_t> lvl_rows;    // most rows (k) of a supernode of the level
    int32_t* d_lvl_dfs = nullptr;     // [ntop] depth-first index of each entry in level order
    int32_t* d_ent_ct = nullptr;      // [ntop] chains per tile of each entry (level order)
    TopDev dev{};
    std::vector<void*> allocations;
    bool usable = true;  // false: a top supernode is too wide for one label tile
};

struct QueryPlans {
    std::mutex mu;
    std::map<int32_t, std::unique_ptr<TopPlan>> top;  // by log2 of the subtree threshold
    int32_t* tin = nullptr;
    int32_t* tout = nullptr;
};

void free_top_plan(TopPlan* p) {
    if (!p) return;
    for (void* a : p->allocations) cudaFree(a);
    p->allocations.clear();
}

void free_query_plans(nwcch_topology* t) {
    auto* Q = static_cast<QueryPlans*>(t->query_plans);
    if (!Q) return;
    for (auto& kv : Q->top) free_top_plan(kv.second.get());
    cudaFree(Q->tin);
    cudaFree(Q->tout);
    delete Q;
    t->query_plans = nullptr;
}

template <class V>
int upload(std::vector<void*>& owner, const std::vector<V>& v, V** out) {
    *out = nullptr;
    void* p = nullptr;
    if (cudaMalloc(&p, sizeof(V) * std::max<size_t>(1, v.size())) != cudaSuccess) return NWCCH_ERR_NOMEM;
    owner.push_back(p);
    if (!v.empty()) NWCCH_CUDA_TRY(cudaMemcpy(p, v.data(), sizeof(V) * v.size(), cudaMemcpyHostToDevice));
    *out = static_cast<V*>(p);
    return NWCCH_OK;
}

// Builds (once per threshold) the top set of supernodes whose elimination
// subtree holds at least 2^log2_tau vertices, its depth-first numbering,
// binary-lifting table and level order; and, once per topology, the preorder
// intervals of the elimination tree. Caller holds Q->mu.
int build_top_plan(nwcch_topology* t, QueryPlans* Q, int32_t log2_tau, TopPlan** out) {
    *out = nullptr;
    auto* P = static_cast<SnPlan*>(t->sn_plan);
    const int64_t n = t->d.n, nsn = P->nsn;
    std::vector<int32_t> parent(n), s0(nsn), kk(nsn), bb(nsn), order(nsn);
    NWCCH_CUDA_TRY(cudaMemcpy(parent.data(), t->d.parent, sizeof(int32_t) * n, cudaMemcpyDeviceToHost));
    NWCCH_CUDA_TRY(cudaMemcpy(s0.data(), P->dev.s0, sizeof(int32_t) * nsn, cudaMemcpyDeviceToHost));
    NWCCH_CUDA_TRY(cudaMemcpy(kk.data(), P->dev.k, sizeof(int32_t) * nsn, cudaMemcpyDeviceToHost));
    NWCCH_CUDA_TRY(cudaMemcpy(bb.data(), P->dev.b, sizeof(int32_t) * nsn, cudaMemcpyDeviceToHost));
    NWCCH_CUDA_TRY(cudaMemcpy(order.data(), P->d_sn_order, sizeof(int32_t) * nsn, cudaMemcpyDeviceToHost));
    std::vector<int32_t> slvl(nsn, 0), sid(n);
    for (int32_t l = 0; l < P->levels; l++)
        for (int64_t i = P->sn_level_off[l]; i < P->sn_level_off[l + 1]; i++) slvl[order[i]] = l;
    for (int64_t s = 0; s < nsn; s++)
        for (int32_t i = 0; i < kk[s]; i++) sid[s0[s] + i] = (int32_t)s;
    // subtree sizes (parents have higher ranks than their children)
    std::vector<int32_t> sub(n, 1);
    for (int64_t x = 0; x < n; x++)
        if (parent[x] >= 0) sub[parent[x]] += sub[x];
    if (!Q->tin) {
        // preorder of the elimination tree: [tin[v], tin[v] + sub[v]) is v's subtree
        std::vector<int64_t> coff(n + 1, 0);
        for (int64_t x = 0; x < n; x++)
            if (parent[x] >= 0) coff[parent[x] + 1]++;
        for (int64_t v = 0; v < n; v++) coff[v + 1] += coff[v];
        std::vector<int32_t> kids(std::max<int64_t>(1, coff[n]));
        {
            std::vector<int64_t> fill(coff.begin(), coff.end() - 1);
            for (int64_t x = 0; x < n; x++)
                if (parent[x] >= 0) kids[fill[parent[x]]++] = (int32_t)x;
        }
        std::vector<int32_t> tin(n), tout(n), stack;
        int32_t clock = 0;
        for (int64_t r = 0; r < n; r++) {
            if (parent[r] >= 0) continue;
            stack.push_back((int32_t)r);
            while (!stack.empty()) {
                const int32_t v = stack.back();
                stack.pop_back();
                tin[v] = clock++;
                tout[v] = tin[v] + sub[v];
                for (int64_t a = coff[v]; a < coff[v + 1]; a++) stack.push_back(kids[a]);
            }
        }
        std::vector<void*> own;
        int rc = upload(own, tin, &Q->tin);
        if (!rc) rc = upload(own, tout, &Q->tout);
        if (rc) {
            for (void* p : own) cudaFree(p);
            Q->tin = Q->tout = nullptr;
            return rc;
        }
    }
    auto plan = std::make_unique<TopPlan>();
    TopPlan* T = plan.get();
    const int64_t tau = (int64_t)1 << log2_tau;
    // top supernodes and their tree (closed upwards: an ancestor's subtree
    // holds the descendant's)
    std::vector<int32_t> tops, tpar;
    std::vector<int32_t> top_local(nsn, -1);
    for (int64_t s = 0; s < nsn; s++) {
        const int32_t topv = s0[s] + kk[s] - 1;
        if (sub[topv] >= tau) {
            top_local[s] = (int32_t)tops.size();
            tops.push_back((int32_t)s);
        }
    }
    const int32_t ntop = (int32_t)tops.size();
    tpar.assign(ntop, -1);
    for (int32_t i = 0; i < ntop; i++) {
        const int32_t s = tops[i];
        const int32_t p = parent[s0[s] + kk[s] - 1];
        if (p >= 0) {
            tpar[i] = top_local[sid[p]];
            if (tpar[i] < 0) return NWCCH_ERR_TOPOLOGY;  // not closed upwards: cannot happen
        }
    }
    // depth-first numbering of the top tree
    std::vector<int64_t> toff(ntop + 1, 0);
    for (int32_t i = 0; i < ntop; i++)
        if (tpar[i] >= 0) toff[tpar[i] + 1]++;
    for (int32_t i = 0; i < ntop; i++) toff[i + 1] += toff[i];
    std::vector<int32_t> tkids(std::max<int64_t>(1, toff[ntop]));
    {
        std::vector<int64_t> fill(toff.begin(), toff.end() - 1);
        for (int32_t i = 0; i < ntop; i++)
            if (tpar[i] >= 0) tkids[fill[tpar[i]]++] = i;
    }
    std::vector<int32_t> dfs(ntop, -1), dfs_sn(ntop), dfs_end(ntop), tsub(ntop, 1);
    for (int32_t i = 0; i < ntop; i++)  // children before parents: supernodes ascend in rank
        if (tpar[i] >= 0) tsub[tpar[i]] += tsub[i];
    {
        int32_t clock = 0;
        std::vector<int32_t> stack;
        for (int32_t r = 0; r < ntop; r++) {
            if (tpar[r] >= 0) continue;
            stack.push_back(r);
            while (!stack.empty()) {
                const int32_t v = stack.back();
                stack.pop_back();
                dfs[v] = clock++;
                for (int64_t a = toff[v]; a < toff[v + 1]; a++) stack.push_back(tkids[a]);
            }
        }
    }
    std::vector<int32_t> top_dfs(nsn, -1);
    for (int32_t i = 0; i < ntop; i++) {
        top_dfs[tops[i]] = dfs[i];
        dfs_sn[dfs[i]] = tops[i];
        dfs_end[dfs[i]] = dfs[i] + tsub[i];
    }
    int32_t J = 1;
    while (((int64_t)1 << J) < std::max<int32_t>(ntop, 1)) J++;
    std::vector<int32_t> lift((size_t)J * std::max<int32_t>(ntop, 1), -1);
    for (int32_t i = 0; i < ntop; i++) lift[dfs[i]] = tpar[i] >= 0 ? dfs[tpar[i]] : -1;
    for (int32_t j = 1; j < J; j++)
        for (int32_t d = 0; d < ntop; d++) {
            const int32_t h = lift[(size_t)(j - 1) * ntop + d];
            lift[(size_t)j * ntop + d] = h >= 0 ? lift[(size_t)(j - 1) * ntop + h] : -1;
        }
    // level order: by supernode level, then depth-first index
    std::vector<int32_t> ent(ntop);
    for (int32_t i = 0; i < ntop; i++) ent[i] = dfs[i];
    std::sort(ent.begin(), ent.end(), [&](int32_t a, int32_t b) {
        const int32_t la = slvl[dfs_sn[a]], lb = slvl[dfs_sn[b]];
        return la != lb ? la < lb : a < b;
    });
    // chains per tile: the most of 32, 16, 8 whose rows fit the shared
    // memory budget ((ct + 4) x 4 bytes a row)
    std::vector<int32_t> ent_ct(ntop);
    for (int32_t i = 0; i < ntop;) {
        int32_t j = i, rows = 0;
        const int32_t l = slvl[dfs_sn[ent[i]]];
        while (j < ntop && slvl[dfs_sn[ent[j]]] == l) {
            rows = std::max(rows, kk[dfs_sn[ent[j]]]);
            j++;
        }
        int32_t ct = 0;
        for (int32_t c : {32, 16, 8})
            if (ct == 0 && (int64_t)(c + 4) * 4 * rows <= QT_SMEM) ct = c;
        if (ct == 0 && (int64_t)(8 + 4) * 4 * rows <= QT_SMEM_MAX) ct = 8;
        if (ct == 0) {
            T->usable = false;
            ct = 8;
        }
        T->lvl_off.push_back(i);
        T->lvl_ct.push_back(ct);
        T->lvl_rows.push_back(rows);
        for (int32_t e = i; e < j; e++) ent_ct[e] = ct;
        i = j;
    }
    T->lvl_off.push_back(ntop);
    int32_t *d_top_dfs, *d_dfs_sn, *d_dfs_end, *d_lift;
    int rc = upload(T->allocations, top_dfs, &d_top_dfs);
    if (!rc) rc = upload(T->allocations, dfs_sn, &d_dfs_sn);
    if (!rc) rc = upload(T->allocations, dfs_end, &d_dfs_end);
    if (!rc) rc = upload(T->allocations, lift, &d_lift);
    if (!rc) rc = upload(T->allocations, ent, &T->d_lvl_dfs);
    if (!rc) rc = upload(T->allocations, ent_ct, &T->d_ent_ct);
    if (rc) {
        free_top_plan(T);
        return rc;
    }
    T->dev = TopDev{d_top_dfs, d_dfs_sn, d_dfs_end, d_lift, Q->tin, Q->tout, ntop, J};
    if (setup_copies_done() != cudaSuccess) {  // the uploads above, before any stream reads them
        free_top_plan(T);
        return NWCCH_ERR_CUDA;
    }
    *out = T;
    Q->top[log2_tau] = std::move(plan);
    return NWCCH_OK;
}

// ---------------------------------------------------------------- device

__device__ __forceinline__ bool is_anc(const TopDev& T, int32_t a, int32_t tx) {
    return T.tin[a] <= tx && tx < T.tout[a];
}

// Lowest row of supernode (s0, k) that is an ancestor of (or is) the vertex
// with preorder index tx; the rows that are form a suffix (each row's
// vertex is the parent of the previous), and the top row must be one.
__device__ __forceinline__ int32_t lowest_anc_row(const TopDev& T, int32_t s0, int32_t k, int32_t tx) {
    int32_t lo = 0, hi = k - 1;
    while (lo < hi) {
        const int32_t mid = (lo + hi) >> 1;
        if (is_anc(T, s0 + mid, tx)) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// Depth of the lowest common ancestor of s and t if it lies on s's chain
// before vertex `stop` (the chain's first top vertex, or -1); -1 otherwise.
__device__ int32_t lower_lca(const DevTopo& D, const SnDev& S, const TopDev& T, int32_t s, int32_t t, int32_t stop) {
    const int32_t tt = T.tin[t];
    int32_t x = s;
    while (x >= 0 && x != stop) {
        const int32_t sn = S.sn_id[x];
        const int32_t s0 = S.s0[sn], k = S.k[sn], top = s0 + k - 1;
        if (is_anc(T, top, tt)) {
            int32_t lo = x - s0, hi = k - 1;
            while (lo < hi) {
                const int32_t mid = (lo + hi) >> 1;
                if (is_anc(T, s0 + mid, tt)) hi = mid;
                else lo = mid + 1;
            }
            return D.depth[s0 + lo];
        }
        x = D.parent[top];
    }
    return -1;
}

// Depth of the lowest common ancestor of two top vertices (-1: none).
__device__ int32_t top_lca_depth(const DevTopo& D, const SnDev& S, const TopDev& T, int32_t xs, int32_t xt) {
    int32_t a = T.top_dfs[S.sn_id[xs]];
    const int32_t b = T.top_dfs[S.sn_id[xt]];
    if (a < 0 || b < 0) return -1;
    auto holds = [&](int32_t u, int32_t v) { return u <= v && v < T.dfs_end[u]; };
    if (holds(b, a)) {
        a = b;
    } else if (!holds(a, b)) {
        for (int j = T.J - 1; j >= 0; j--) {
            const int32_t h = T.lift[(int64_t)j * T.ntop + a];
            if (h >= 0 && !holds(h, b)) a = h;
        }
        a = T.lift[a];
        if (a < 0) return -1;  // different trees of the forest
    }
    const int32_t sn = T.dfs_sn[a];
    const int32_t s0 = S.s0[sn], k = S.k[sn];
    const int32_t i = max(lowest_anc_row(T, s0, k, T.tin[xs]), lowest_anc_row(T, s0, k, T.tin[xt]));
    return D.depth[s0 + i];
}

// Phase 1: a warp per chain (chains [0, nq) from s with up weights, [nq,
// 2 nq) from t with dn weights).
__global__ void __launch_bounds__(256) k_qlow(DevTopo D, SnDev S, TopDev T, const int32_t* __restrict__ up,
                                              const int32_t* __restrict__ dn, const int32_t* __restrict__ s_rank,
                                              const int32_t* __restrict__ t_rank, int64_t nq, int32_t* __restrict__ Lg,
                                              int64_t Dp, int32_t* __restrict__ xin, int32_t* __restrict__ key,
                                              int32_t* __restrict__ hist, int32_t* __restrict__ lca,
                                              const unsigned int* __restrict__ maxabs, int* __restrict__ err,
                                              int dense_rows) {
    if (!small_labels(D, maxabs)) return;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t per_warp = (4 * Dp + 15) & ~15LL;
    int32_t* F = reinterpret_cast<int32_t*>(smraw + wib * per_warp);
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int32_t nb = T.ntop + 1;  // buckets per direction: top entries, then "no top"
    int e = 0;
    for (int64_t c = blockIdx.x * (int64_t)(blockDim.x >> 5) + wib; c < 2 * nq; c += nwarps) {
        const int dir = c >= nq ? 1 : 0;
        const int64_t q = dir ? c - nq : c;
        const int32_t s = dir ? t_rank[q] : s_rank[q];
        const int32_t other = dir ? s_rank[q] : t_rank[q];
        if (s < 0 || s >= D.n || other < 0 || other >= D.n) {
            if (lane == 0) {
                xin[c] = -1;
                key[c] = T.ntop;
                atomicAdd(&hist[dir * nb + T.ntop], 1);
                if (!dir) lca[q] = -2;
            }
            e |= ERR_ARG;
            continue;
        }
        const int32_t ds = D.depth[s];
        for (int i = lane; i <= ds; i += 32) F[i] = Q32::CINF;
        __syncwarp();
        if (lane == 0) F[0] = 0;
        __syncwarp();
        int32_t unused = Q32::CINF;
        const int32_t x = sn_sweep32<false, false, 1, false, true>(D, S, dir ? dn : up, s, ds, F, nullptr, nullptr,
                                                                   nullptr, 0, unused, dense_rows, T.top_dfs);
        __syncwarp();
        int32_t* Lc = Lg + c * Dp;
        for (int i = lane; i <= ds; i += 32) Lc[ds - i] = Q32::norm(F[i]);  // by depth
        if (lane == 0) {
            const int32_t b = x >= 0 ? T.top_dfs[S.sn_id[x]] : T.ntop;
            xin[c] = x;
            key[c] = b;
            atomicAdd(&hist[dir * nb + b], 1);
            if (!dir) lca[q] = lower_lca(D, S, T, s, other, x);
        }
        __syncwarp();
    }
    if (e) atomicOr(err, e);
}

// Exclusive scan of count(i), i < len, by one block into out[0..len]
// (out[len] = total).
template <class V, class F>
__device__ void block_scan(int64_t len, F count, V* out) {
    __shared__ V warp_sum[32];
    __shared__ V carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < len; base += blockDim.x) {
        const int64_t i = base + threadIdx.x;
        const V v = i < len ? count(i) : (V)0;
        V x = v;
        for (int o = 1; o < 32; o <<= 1) {
            const V y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_sum[w] = x;
        __syncthreads();
        if (w == 0) {
            V ws = lane < nw ? warp_sum[lane] : (V)0;
            for (int o = 1; o < 32; o <<= 1) {
                const V y = __shfl_up_sync(0xffffffffu, ws, o);
                if (lane >= o) ws += y;
            }
            if (lane < nw) warp_sum[lane] = ws;
        }
        __syncthreads();
        const V before = carry + (w > 0 ? warp_sum[w - 1] : (V)0) + x - v;
        if (i < len) out[i] = before;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = before + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) out[len] = carry;
    __syncthreads();
}

// Phase 1b (one block): bucket offsets per direction, and the tiles of every
// (top supernode, direction) entry in level order.
__global__ void __launch_bounds__(1024) k_qscan(TopDev T, const int32_t* __restrict__ hist,
                                                int32_t* __restrict__ boff, int32_t* __restrict__ fill,
                                                const int32_t* __restrict__ lvl_dfs, const int32_t* __restrict__ ent_ct,
                                                int64_t* __restrict__ tile_off) {
    const int32_t nb = T.ntop + 1;
    for (int dir = 0; dir < 2; dir++) {
        const int32_t* h = hist + dir * nb;
        block_scan<int32_t>(nb, [&](int64_t i) { return h[i]; }, boff + dir * (nb + 1));
    }
    for (int32_t i = threadIdx.x; i < 2 * nb; i += blockDim.x) fill[i] = 0;
    __syncthreads();
    block_scan<int64_t>(2 * (int64_t)T.ntop, [&](int64_t e) -> int64_t {
        const int dir = (int)(e & 1);
        const int32_t d = lvl_dfs[e >> 1];
        const int32_t* bo = boff + dir * (nb + 1);
        const int64_t len = bo[T.dfs_end[d]] - bo[d];
        const int64_t ct = ent_ct[e >> 1];
        return (len + ct - 1) / ct;
    }, tile_off);
}

// Phase 1c: the chains of every bucket, contiguous (order within a bucket is
// arbitrary).
__global__ void k_qscatter(DevTopo D, int64_t nq, int32_t nb, const int32_t* __restrict__ key,
                           const int32_t* __restrict__ boff, int32_t* __restrict__ fill, int32_t* __restrict__ order,
                           const unsigned int* __restrict__ maxabs, int* __restrict__ err) {
    if (!small_labels(D, maxabs)) return;  // the 64-bit kernel answers this batch
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < 2 * nq; c += (int64_t)gridDim.x * blockDim.x) {
        const int dir = c >= nq ? 1 : 0;
        const int32_t b = key[c];
        if (b < 0 || b >= nb) {  // cannot happen: every chain is bucketed
            atomicOr(err, ERR_TOPOLOGY);
            continue;
        }
        const int32_t pos = atomicAdd(&fill[dir * nb + b], 1);
        const int64_t o = (int64_t)boff[dir * (nb + 1) + b] + pos;
        if (o < 0 || o >= nq) {  // more chains than the histogram counted: cannot happen
            atomicOr(err, ERR_TOPOLOGY);
            continue;
        }
        order[dir * nq + o] = (int32_t)c;
    }
}

// Phase 2: the top supernodes of one level, a tile of up to CT chains per
// CTA. The tile's labels of S's rows live in shared memory row by row, the
// tile's chains side by side (Ls[r * CTP + q], CTP = CT + 4 so that 16-byte
// loads of different rows by the lanes of a warp hit different banks), and
// one broadcast 16-byte load feeds four chains:
//  (a) per 32-row block, the diagonal triangle: a warp per chain, four
//      chains at a time, by shuffles;
//  (b) the block's rows times the later rows' columns: a thread per column
//      holding the block's 32 weights and the tile's CT accumulators in
//      registers;
//  (c) after the last block, the boundary columns: a thread per column, each
//      row's weight read once and applied to the whole tile, the
//      accumulators starting from and returning to the chains' global rows
//      (boundary labels are outputs only, so they need no shared memory).
template <int CT>
__global__ void __launch_bounds__(QT_THREADS, 2) k_qtop(DevTopo D, SnDev S, TopDev T, const int32_t* __restrict__ up,
                                                     const int32_t* __restrict__ dn,
                                                     const int32_t* __restrict__ lvl_dfs, int64_t e_lo, int64_t e_hi,
                                                     const int64_t* __restrict__ tile_off,
                                                     const int32_t* __restrict__ boff,
                                                     const int32_t* __restrict__ order,
                                                     const int32_t* __restrict__ xin, int32_t* __restrict__ Lg,
                                                     int64_t Dp, int64_t nq, const unsigned int* __restrict__ maxabs,
                                                     int* __restrict__ err) {
    static_assert(CT % 4 == 0 && CT <= QT_MAX_CT, "tile of 4k chains");
    constexpr int CTP = CT + 4;
    if (!small_labels(D, maxabs)) return;
    extern __shared__ __align__(16) int32_t Ls[];  // (k - r_lo) x CTP labels
    __shared__ int32_t s_chain[CT], s_i0[CT];
    __shared__ int32_t s_imin;
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    const int32_t nb1 = T.ntop + 2;
    const int64_t t_lo = tile_off[e_lo], t_hi = tile_off[e_hi];
    int e_bits = 0;
    for (int64_t gt = t_lo + blockIdx.x; gt < t_hi; gt += gridDim.x) {
        int64_t lo = e_lo, hi = e_hi - 1;  // the entry holding tile gt
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (tile_off[mid] <= gt) lo = mid;
            else hi = mid - 1;
        }
        const int dir = (int)(lo & 1);
        const int32_t d = lvl_dfs[lo >> 1];
        const int32_t sn = T.dfs_sn[d];
        const int32_t s0 = S.s0[sn], k = S.k[sn], b = S.b[sn], cols = k + b;
        const int32_t c_hi = boff[dir * nb1 + T.dfs_end[d]];
        const int32_t first_c = boff[dir * nb1 + d] + (int32_t)(gt - tile_off[lo]) * CT;
        const int nct = min(CT, c_hi - first_c);
        const int32_t* __restrict__ W = dir ? dn : up;
        const int32_t d0 = D.depth[s0];
        const int64_t base0 = D.first[s0];
        if (threadIdx.x == 0) s_imin = k;
        __syncthreads();
        // the tile's chains, checked before any label row is addressed
        // through them (a tile with an inconsistent entry is skipped and
        // reported; this cannot happen)
        bool bad = nct < 1 || first_c < 0 || (int64_t)first_c + nct > nq || d0 < k - 1 || d0 >= Dp;
        if (threadIdx.x < CT) {
            int32_t c = -1, i0 = k;
            if (threadIdx.x < nct && !bad) {
                c = order[dir * nq + first_c + threadIdx.x];
                const int32_t x = (c >= 0 && c < 2 * nq) ? xin[c] : -1;
                if (x < 0 || x >= D.n) {
                    bad = true;
                } else {
                    const int32_t tx = T.tin[x];
                    i0 = lowest_anc_row(T, s0, k, tx);
                    if (!is_anc(T, s0 + i0, tx)) bad = true;  // the chain does not cross S
                }
                atomicMin(&s_imin, i0);
            }
            s_chain[threadIdx.x] = c;
            s_i0[threadIdx.x] = i0;
        }
        if (__syncthreads_or(bad)) {
            e_bits |= ERR_TOPOLOGY;
            continue;
        }
        const int32_t r_lo = s_imin & ~31, nr = k - r_lo;
        // rows r_lo.. of the tile's chains (no path below a chain's entry row,
        // and in the columns of absent chains)
        for (int idx = threadIdx.x; idx < CT * nr; idx += QT_THREADS) {
            const int q = idx / nr, rr = idx - q * nr, r = r_lo + rr;
            int32_t v = Q32::CINF;
            if (q < nct && r >= s_i0[q]) v = Lg[(int64_t)s_chain[q] * Dp + (d0 - r)];
            Ls[rr * CTP + q] = v;
        }
        __syncthreads();
        // row r's arcs start at first[s0 + r] = base0 + r (cols - 1) - r (r - 1) / 2
        auto rowb = [&](int32_t r) -> int64_t { return base0 + (int64_t)r * (cols - 1) - (int64_t)r * (r - 1) / 2; };
        for (int32_t c0 = r_lo; c0 < k; c0 += 32) {
            const int n = min(32, k - c0);
            const int32_t cr = c0 - r_lo;
            // (a) the 32 x 32 diagonal triangle
            if (wq < nct) {
                int32_t u[31];
#pragma unroll
                for (int r = 0; r < 31; r++)
                    u[r] = (r < lane && lane < n) ? Q32::w(W[rowb(c0 + r) + (lane - r - 1)]) : Q32::CINF;
                int32_t lab[4];
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    const int q = wq + 8 * m;
                    lab[m] = (q < nct && lane < n) ? Ls[(cr + lane) * CTP + q] : Q32::CINF;
                }
#pragma unroll
                for (int r = 0; r < 31; r++) {
#pragma unroll
                    for (int m = 0; m < 4; m++)
                        lab[m] = __viaddmin_s32(Q32::norm(__shfl_sync(FULL, lab[m], r)), u[r], lab[m]);
                }
#pragma unroll
                for (int m = 0; m < 4; m++) {
                    const int q = wq + 8 * m;
                    if (q < nct && lane < n) Ls[(cr + lane) * CTP + q] = Q32::norm(lab[m]);
                }
            }
            __syncthreads();
            // (b) the block's rows times the later rows' columns
            for (int32_t j = c0 + n + threadIdx.x; j < k; j += QT_THREADS) {
                int32_t acc[CT];
                int4* mine = reinterpret_cast<int4*>(Ls + (j - r_lo) * CTP);
#pragma unroll
                for (int q4 = 0; q4 < CT / 4; q4++) {
                    const int4 v = mine[q4];
                    acc[4 * q4] = v.x;
                    acc[4 * q4 + 1] = v.y;
                    acc[4 * q4 + 2] = v.z;
                    acc[4 * q4 + 3] = v.w;
                }
#pragma unroll 1
                for (int g = 0; g < n; g += 8) {  // 8 rows' weights at a time
                    int32_t wv[8];
#pragma unroll
                    for (int u = 0; u < 8; u++)
                        wv[u] = g + u < n ? Q32::w(W[rowb(c0 + g + u) + (j - c0 - g - u - 1)]) : Q32::CINF;
#pragma unroll
                    for (int u = 0; u < 8; u++) {
                        if (g + u < n) {
                            const int4* row = reinterpret_cast<const int4*>(Ls + (cr + g + u) * CTP);
#pragma unroll
                            for (int q4 = 0; q4 < CT / 4; q4++) {
                                const int4 l = row[q4];
                                acc[4 * q4] = __viaddmin_s32(l.x, wv[u], acc[4 * q4]);
                                acc[4 * q4 + 1] = __viaddmin_s32(l.y, wv[u], acc[4 * q4 + 1]);
                                acc[4 * q4 + 2] = __viaddmin_s32(l.z, wv[u], acc[4 * q4 + 2]);
                                acc[4 * q4 + 3] = __viaddmin_s32(l.w, wv[u], acc[4 * q4 + 3]);
                            }
                        }
                    }
                }
#pragma unroll
                for (int q4 = 0; q4 < CT / 4; q4++)
                    mine[q4] = make_int4(acc[4 * q4], acc[4 * q4 + 1], acc[4 * q4 + 2], acc[4 * q4 + 3]);
            }
            __syncthreads();
        }
        // (c) the boundary columns, from every row of the tile
        const int64_t bbase = rowb(k - 1);
        for (int32_t jb = threadIdx.x; jb < b; jb += QT_THREADS) {
            const int32_t j = k + jb;
            const int32_t hd = D.hdep[bbase + jb];
            if (hd < 0 || hd >= Dp) {  // a head deeper than the tree: cannot happen
                e_bits |= ERR_TOPOLOGY;
                continue;
            }
            int32_t acc[CT];
#pragma unroll
            for (int q = 0; q < CT; q++) acc[q] = q < nct ? Lg[(int64_t)s_chain[q] * Dp + hd] : Q32::CINF;
#pragma unroll 1
            for (int32_t r0 = r_lo; r0 < k; r0 += 8) {
                int32_t wv[8];
#pragma unroll
                for (int u = 0; u < 8; u++)
                    wv[u] = r0 + u < k ? Q32::w(W[rowb(r0 + u) + (j - r0 - u - 1)]) : Q32::CINF;
#pragma unroll
                for (int u = 0; u < 8; u++) {
                    if (r0 + u < k) {
                        const int4* row = reinterpret_cast<const int4*>(Ls + (r0 + u - r_lo) * CTP);
#pragma unroll
                        for (int q4 = 0; q4 < CT / 4; q4++) {
                            const int4 l = row[q4];
                            acc[4 * q4] = __viaddmin_s32(l.x, wv[u], acc[4 * q4]);
                            acc[4 * q4 + 1] = __viaddmin_s32(l.y, wv[u], acc[4 * q4 + 1]);
                            acc[4 * q4 + 2] = __viaddmin_s32(l.z, wv[u], acc[4 * q4 + 2]);
                            acc[4 * q4 + 3] = __viaddmin_s32(l.w, wv[u], acc[4 * q4 + 3]);
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < CT; q++)
                if (q < nct) Lg[(int64_t)s_chain[q] * Dp + hd] = Q32::norm(acc[q]);
        }
        // the rows back to the chains' global rows
        for (int idx = threadIdx.x; idx < nct * nr; idx += QT_THREADS) {
            const int q = idx / nr, rr = idx - q * nr, r = r_lo + rr;
            if (r >= s_i0[q]) Lg[(int64_t)s_chain[q] * Dp + (d0 - r)] = Q32::norm(Ls[rr * CTP + q]);
        }
        __syncthreads();
    }
    if (e_bits) atomicOr(err, e_bits);
}

// Phase 3: a warp per query, the meet over the common ancestors.
__global__ void __launch_bounds__(256) k_qmeet(DevTopo D, SnDev S, TopDev T, int64_t nq,
                                               const int32_t* __restrict__ xin, const int32_t* __restrict__ lca,
                                               const int32_t* __restrict__ Lg, int64_t Dp, int64_t* __restrict__ dist,
                                               const unsigned int* __restrict__ maxabs) {
    if (!small_labels(D, maxabs)) return;
    const int lane = threadIdx.x & 31;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t q = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; q < nq; q += nwarps) {
        int32_t dl = -1;
        if (lane == 0) {
            dl = lca[q];
            if (dl == -1) {
                const int32_t xs = xin[q], xt = xin[nq + q];
                if (xs >= 0 && xt >= 0 && xs < D.n && xt < D.n) dl = top_lca_depth(D, S, T, xs, xt);
            }
        }
        dl = min(__shfl_sync(FULL, dl, 0), (int32_t)(Dp - 1));
        const int32_t* F = Lg + q * Dp;
        const int32_t* R = Lg + (nq + q) * Dp;
        int32_t best = Q32::CINF;
        for (int32_t d = lane; d <= dl; d += 32) {
            const int32_t f = F[d], r = R[d];
            if (!Q32::none(f) && !Q32::none(r)) best = min(best, f + r);
        }
        for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(FULL, best, o));
        if (lane == 0) dist[q] = Q32::none(best) ? INF64 : (int64_t)best;
    }
}

// The plan of a threshold, built on first use; with lookup_only (a stream
// being captured, where the build's copies are not allowed) *out stays null
// when it is not built yet.
int get_top_plan(nwcch_topology* t, int32_t log2_tau, bool lookup_only, TopPlan** out) {
    *out = nullptr;
    std::lock_guard<std::mutex> lock(t->mu);
    if (!t->query_plans) {
        t->query_plans = new (std::nothrow) QueryPlans();
        if (!t->query_plans) return NWCCH_ERR_NOMEM;
        t->free_query_plans = free_query_plans;
    }
    auto* Q = static_cast<QueryPlans*>(t->query_plans);
    std::lock_guard<std::mutex> qlock(Q->mu);
    auto it = Q->top.find(log2_tau);
    if (it != Q->top.end()) {
        *out = it->second.get();
        return NWCCH_OK;
    }
    if (lookup_only) return NWCCH_OK;
    return build_top_plan(t, Q, log2_tau, out);
}

template <class K>
int occupancy_grid(K kernel, int threads, size_t smem, int64_t want, int sms, int64_t* blocks) {
    int per_sm = 0;
    NWCCH_CUDA_TRY(allow_dynamic_smem((const void*)kernel, smem));
    NWCCH_CUDA_TRY(blocks_per_sm((const void*)kernel, threads, smem, &per_sm));
    if (per_sm < 1) return NWCCH_ERR_CAPACITY;
    *blocks = std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sms * per_sm));
    return NWCCH_OK;
}

}  // namespace

// Enqueues the three-phase pipeline for a batch of int32-stored queries on
// stream s. *used = false (nothing enqueued) when the batch is not its case:
// the top path is switched off, the tree is too deep for the lower sweep's
// shared-memory labels, or a top supernode is too wide for a label tile.
int query_top_async(nwcch_topology* t, const int32_t* up, const int32_t* dn, const int32_t* s_rank,
                    const int32_t* t_rank, int64_t nq, int64_t* dist, const unsigned int* maxabs, int* err,
                    cudaStream_t s, bool* used, int64_t* launches) {
    *used = false;
    *launches = 0;
    const int64_t min_chains = t->tune.query_top_chains;
    if (min_chains <= 0 || !t->sn_plan || nq < 1) return NWCCH_OK;
    const int64_t Dp = t->d.max_depth + 1;
    const int64_t per_warp = (4 * Dp + 15) & ~15LL;
    const int warps = (int)std::min<int64_t>(8, QL_SMEM / per_warp);
    if (warps < 1) return NWCCH_OK;
    // a pass holds the label rows of at most `chunk` queries
    int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(nq, QT_LABEL_BYTES / (8 * Dp)));
    if (const char* cap = getenv("NWCCH_QUERY_TOP_PASS_QUERIES"))  // tests: several passes per batch
        chunk = std::max<int64_t>(1, std::min<int64_t>(chunk, atoll(cap)));
    // top set: supernodes that an expected min_chains chains of a pass cross
    const int64_t tau = std::max<int64_t>(2, (min_chains * t->d.n) / (2 * chunk));
    int32_t log2_tau = 1;
    while (((int64_t)1 << (log2_tau + 1)) <= tau) log2_tau++;
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    NWCCH_CUDA_TRY(cudaStreamIsCapturing(s, &capture));
    TopPlan* T = nullptr;
    int rc = get_top_plan(t, log2_tau, capture != cudaStreamCaptureStatusNone, &T);
    if (rc) return rc;
    if (!T || !T->usable) return NWCCH_OK;
    const auto* P = static_cast<SnPlan*>(t->sn_plan);
    const TopDev& TD = T->dev;
    const int32_t ntop = TD.ntop, nb = ntop + 1;
    const int sms = t->sms;
    // scratch of one pass: the regions in carving order, each rounded up to
    // 16 bytes; the allocation is the sum of exactly these sizes
    enum { R_LG, R_TILE_OFF, R_XIN, R_KEY, R_ORDER, R_LCA, R_HIST, R_FILL, R_BOFF, R_COUNT };
    size_t region[R_COUNT];
    region[R_LG] = (size_t)(2 * chunk * Dp) * 4;
    region[R_TILE_OFF] = (size_t)(2 * (int64_t)ntop + 1) * 8;
    region[R_XIN] = region[R_KEY] = region[R_ORDER] = (size_t)(2 * chunk) * 4;
    region[R_LCA] = (size_t)chunk * 4;
    region[R_HIST] = region[R_FILL] = (size_t)(2 * nb) * 4;
    region[R_BOFF] = (size_t)(2 * (nb + 1)) * 4;
    auto round16 = [](size_t bytes) { return (bytes + 15) & ~(size_t)15; };
    size_t total = 0;
    for (size_t r : region) total += round16(r);
    void* scratch = nullptr;
    NWCCH_CUDA_TRY(scratch_alloc(&scratch, total, s));
    char* p = static_cast<char*>(scratch);
    auto take = [&](int r) {
        char* at = p;
        p += round16(region[r]);
        return at;
    };
    int32_t* Lg = reinterpret_cast<int32_t*>(take(R_LG));
    int64_t* tile_off = reinterpret_cast<int64_t*>(take(R_TILE_OFF));
    int32_t* xin = reinterpret_cast<int32_t*>(take(R_XIN));
    int32_t* key = reinterpret_cast<int32_t*>(take(R_KEY));
    int32_t* order = reinterpret_cast<int32_t*>(take(R_ORDER));
    int32_t* lca = reinterpret_cast<int32_t*>(take(R_LCA));
    int32_t* hist = reinterpret_cast<int32_t*>(take(R_HIST));
    int32_t* fill = reinterpret_cast<int32_t*>(take(R_FILL));
    int32_t* boff = reinterpret_cast<int32_t*>(take(R_BOFF));
    const int dense_rows = t->tune.query_dense_rows;
    for (int64_t q0 = 0; q0 < nq && rc == NWCCH_OK; q0 += chunk) {
        const int64_t m = std::min(chunk, nq - q0);
        int64_t blocks = 0;
        if (cudaMemsetAsync(hist, 0, (size_t)(2 * nb) * 4, s) != cudaSuccess) {
            rc = NWCCH_ERR_CUDA;
            break;
        }
        const size_t lsmem = (size_t)warps * per_warp;
        if ((rc = occupancy_grid(k_qlow, 32 * warps, lsmem, (2 * m + warps - 1) / warps, sms, &blocks))) break;
        k_qlow<<<(unsigned)blocks, 32 * warps, lsmem, s>>>(t->d, P->dev, TD, up, dn, s_rank + q0, t_rank + q0, m, Lg,
                                                          Dp, xin, key, hist, lca, maxabs, err, dense_rows);
        k_qscan<<<1, 1024, 0, s>>>(TD, hist, boff, fill, T->d_lvl_dfs, T->d_ent_ct, tile_off);
        k_qscatter<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((2 * m + 255) / 256, (int64_t)sms * 8)), 256, 0,
                     s>>>(t->d, m, nb, key, boff, fill, order, maxabs, err);
        for (size_t l = 0; l + 1 < T->lvl_off.size(); l++) {
            const int ct = T->lvl_ct[l];
            const size_t tsmem = (size_t)(ct + 4) * 4 * std::max<int32_t>(1, T->lvl_rows[l]);
            const int64_t e0 = 2 * T->lvl_off[l], e1 = 2 * T->lvl_off[l + 1];
            if (ct == 32) {
                if ((rc = occupancy_grid(k_qtop<32>, QT_THREADS, tsmem, (int64_t)sms * 64, sms, &blocks))) break;
                k_qtop<32><<<(unsigned)blocks, QT_THREADS, tsmem, s>>>(t->d, P->dev, TD, up, dn, T->d_lvl_dfs, e0, e1,
                                                                       tile_off, boff, order, xin, Lg, Dp, m, maxabs,
                                                                       err);
            } else if (ct == 16) {
                if ((rc = occupancy_grid(k_qtop<16>, QT_THREADS, tsmem, (int64_t)sms * 64, sms, &blocks))) break;
                k_qtop<16><<<(unsigned)blocks, QT_THREADS, tsmem, s>>>(t->d, P->dev, TD, up, dn, T->d_lvl_dfs, e0, e1,
                                                                       tile_off, boff, order, xin, Lg, Dp, m, maxabs,
                                                                       err);
            } else {
                if ((rc = occupancy_grid(k_qtop<8>, QT_THREADS, tsmem, (int64_t)sms * 64, sms, &blocks))) break;
                k_qtop<8><<<(unsigned)blocks, QT_THREADS, tsmem, s>>>(t->d, P->dev, TD, up, dn, T->d_lvl_dfs, e0, e1,
                                                                      tile_off, boff, order, xin, Lg, Dp, m, maxabs,
                                                                      err);
            }
        }
        if (rc) break;
        *launches += 4 + (int64_t)(T->lvl_off.size() - 1);  // k_qlow, k_qscan, k_qscatter, k_qtop per level, k_qmeet
        k_qmeet<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((m + 7) / 8, (int64_t)sms * 16)), 256, 0, s>>>(
            t->d, P->dev, TD, m, xin, lca, Lg, Dp, dist + q0, maxabs);
        if (cudaGetLastError() != cudaSuccess) rc = NWCCH_ERR_CUDA;
    }
    const cudaError_t fe = cudaFreeAsync(scratch, s);
    if (rc) return rc;
    NWCCH_CUDA_TRY(fe);
    *used = true;
    return NWCCH_OK;
}

}  // namespace nwcch
