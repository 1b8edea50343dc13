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
// One cooperative launch runs the whole update: its blocks are co-resident,
// and a level ends with a grid barrier whose spin is bounded (on timeout the
// kernel records ERR_TIMEOUT and every block returns). The kernel cleans its
// workspace (queued flags, bucket counts, pending bits) before it exits.

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "common.cuh"
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
    // [0] evaluated [1] changed [2] changed with up+dn<0 [3] levels done
    // [5] barrier arrivals [6] barrier generation
    unsigned long long* stats = nullptr;
    int blocks32 = 0, blocks64 = 0;
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
};

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
    A.ws.bucket[A.level_arc_off[L] + pos] = c;
    atomicOr(&A.ws.pending[L >> 5], 1u << (L & 31));
}

// Bounded grid barrier. Returns false if it timed out (ERR_TIMEOUT recorded).
template <class T>
static __device__ bool grid_sync(const UpdateArgs<T>& A) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long* count = A.ws.stats + 5;
        volatile unsigned long long* gen = A.ws.stats + 6;
        const unsigned long long g = *gen;
        __threadfence();
        ok = 1;
        if (atomicAdd(count, 1ull) == (unsigned long long)gridDim.x - 1) {
            *count = 0;
            __threadfence();
            atomicAdd((unsigned long long*)gen, 1ull);
        } else {
            long long spins = 0;
            while (*gen == g) {
                __nanosleep(100);
                if (++spins > (1ll << 24)) {  // a few seconds
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

template <class T>
__global__ void __launch_bounds__(256) k_update(UpdateArgs<T> A) {
    const DevTopo& D = A.D;
    const int lane = threadIdx.x & 31;
    const int64_t gtid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t gthreads = (int64_t)gridDim.x * blockDim.x;
    const int64_t gwarp = gtid >> 5, gwarps = gthreads >> 5;
    int e = 0;
    // 1. new weights (python/cch.py:357-360)
    for (int64_t j = gtid; j < A.k; j += gthreads) A.w[A.ws.edge_idx[j]] = A.ws.new_w[j];
    if (!grid_sync(A)) return;
    // 2. queue the arcs the changed original arcs map to
    for (int64_t j = gtid; j < A.k; j += gthreads) {
        const int64_t c = D.e_arc[A.ws.edge_idx[j]];
        if (c >= 0) enqueue(A, (int32_t)c);
    }
    if (!grid_sync(A)) return;
    // 3. levels, lowest first (python/cch.py:376-401)
    __shared__ int32_t next_level;
    int32_t L = -1;
    while (true) {
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
        const int64_t base = A.level_arc_off[L];
        const int32_t cnt = __ldcg(A.ws.bcount + L);
        if (gtid == 0) {
            const unsigned long long d = atomicAdd(A.ws.stats + 3, 1ull);
            A.ws.done_levels[d] = L;
            atomicAdd(A.ws.stats + 0, (unsigned long long)cnt);
        }
        for (int64_t i = gwarp; i < cnt; i += gwarps) {
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
                const unsigned long long p = atomicAdd(A.ws.stats + 1, 1ull);
                A.ws.changed[p] = c;
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
        if (!grid_sync(A)) return;
    }
    // 4. clean the workspace for the next call
    const int32_t nd_levels = (int32_t)__ldcg(A.ws.stats + 3);
    for (int32_t li = 0; li < nd_levels; li++) {
        const int32_t l = __ldcg(A.ws.done_levels + li);
        const int64_t base = A.level_arc_off[l];
        const int32_t cnt = __ldcg(A.ws.bcount + l);
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

static void free_workspace(UpdateWorkspace* ws) {
    if (!ws) return;
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
                  cudaMalloc(&ws->stats, 8 * sizeof(unsigned long long)) == cudaSuccess;
        if (ok)
            ok = cudaMemset(ws->queued, 0, qbytes) == cudaSuccess && cudaMemset(ws->bcount, 0, L * 4) == cudaSuccess &&
                 cudaMemset(ws->pending, 0, ((L + 31) / 32) * 4) == cudaSuccess &&
                 cudaMemset(ws->stats, 0, 8 * sizeof(unsigned long long)) == cudaSuccess;
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
    NWCCH_CUDA_TRY(cudaMemsetAsync(ws->stats, 0, 8 * sizeof(unsigned long long), s));
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
    void* args[] = {&A};
    const int blocks = sizeof(T) == 4 ? ws->blocks32 : ws->blocks64;
    NWCCH_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_update<T>, dim3(blocks), dim3(256), args, 0, s));
    unsigned long long h[8];
    NWCCH_CUDA_TRY(cudaMemcpyAsync(h, ws->stats, sizeof(h), cudaMemcpyDeviceToHost, s));
    NWCCH_CUDA_TRY(cudaStreamSynchronize(s));
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
    if (!t || !w_dev || !up_dev || !dn_dev || k < 0 || (k > 0 && (!edge_idx || !new_w)) || !stats)
        return NWCCH_ERR_ARG;
    return update<int32_t>(t, w_dev, up_dev, dn_dev, edge_idx, new_w, k, stats, changed_dev, (cudaStream_t)stream);
}

extern "C" int nwcch_update_i64(nwcch_topology* t, int32_t* w_dev, int64_t* up_dev, int64_t* dn_dev,
                                const int64_t* edge_idx, const int32_t* new_w, int64_t k, int64_t* stats,
                                int32_t* changed_dev, void* stream) {
    if (!t || !w_dev || !up_dev || !dn_dev || k < 0 || (k > 0 && (!edge_idx || !new_w)) || !stats)
        return NWCCH_ERR_ARG;
    return update<int64_t>(t, w_dev, up_dev, dn_dev, edge_idx, new_w, k, stats, changed_dev, (cudaStream_t)stream);
}
