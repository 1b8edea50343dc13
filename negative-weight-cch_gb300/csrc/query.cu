// Plain elimination-tree query: one warp per (s, t) pair.
//
// The reference (python/cch_nb.py:577-615 = cpp/cch.cpp:549-575) relaxes the
// upward arcs of every ancestor of s in increasing rank (forward labels with
// up weights), then of every ancestor of t (backward labels with dn weights),
// and takes min(df + dr) over the ancestors the two chains share. Arcs out of
// an ancestor only reach ancestors, so labels are indexed by elimination-tree
// depth along one chain: the label of ancestor v of s lives at
// depth(s) - depth(v). Lanes relax the arcs of one row in parallel (distinct
// heads, no conflicts); the warp walks the chain in order.

#include <algorithm>
#include <mutex>

#include "common.cuh"
#include "supernodal.h"
#include "topology.h"

namespace nwcch {

template <class T>
__global__ void __launch_bounds__(128) k_query_plain(DevTopo D, const T* __restrict__ up, const T* __restrict__ dn,
                                                     const int32_t* __restrict__ s_rank,
                                                     const int32_t* __restrict__ t_rank, int64_t nq,
                                                     int64_t* __restrict__ dist, int64_t* __restrict__ scratch,
                                                     int* __restrict__ err) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t Dp = D.max_depth + 1;
    int64_t* F = scratch + warp * (2 * Dp + (Dp + 1) / 2 + 1);
    int64_t* R = F + Dp;
    int32_t* chain = reinterpret_cast<int32_t*>(R + Dp);
    int e = 0;
    for (int64_t q = warp; q < nq; q += nwarps) {
        const int32_t s = s_rank[q], t = t_rank[q];
        if (s < 0 || s >= D.n || t < 0 || t >= D.n) {
            if (lane == 0) dist[q] = INF64;
            e |= ERR_ARG;
            continue;
        }
        const int32_t ds = D.depth[s], dt = D.depth[t];
        for (int i = lane; i <= ds; i += 32) F[i] = INF64;
        for (int i = lane; i <= dt; i += 32) R[i] = INF64;
        __syncwarp();
        if (lane == 0) {
            F[0] = 0;
            R[0] = 0;
        }
        __syncwarp();
        int i = 0;
        for (int32_t x = s; x >= 0; x = D.parent[x], i++) {
            if (lane == 0) chain[i] = x;
            const int64_t fx = F[i];
            if (fx != INF64) {
                for (int64_t a = D.first[x] + lane; a < D.first[x + 1]; a += 32) {
                    const int64_t c = label_plus(fx, up[a], e);
                    int64_t* slot = &F[ds - D.hdep[a]];
                    if (c < *slot) *slot = c;
                }
            }
            __syncwarp();
        }
        int64_t best = INF64;
        i = 0;
        for (int32_t x = t; x >= 0; x = D.parent[x], i++) {
            const int64_t rx = R[i];
            if (rx != INF64) {
                const int32_t dx = dt - i;  // depth of x
                if (dx <= ds && chain[ds - dx] == x) {
                    const int64_t fx = F[ds - dx];
                    if (fx != INF64) {
                        int64_t v;
                        splus(rx, fx, v, e);
                        best = min(best, v);
                    }
                }
                for (int64_t a = D.first[x] + lane; a < D.first[x + 1]; a += 32) {
                    const int64_t c = label_plus(rx, dn[a], e);
                    int64_t* slot = &R[dt - D.hdep[a]];
                    if (c < *slot) *slot = c;
                }
            }
            __syncwarp();
        }
        if (lane == 0) dist[q] = best;
        __syncwarp();
    }
    if (e) atomicOr(err, e);
}

template <class T>
int query_plain(nwcch_topology* t, const T* up, const T* dn, const int32_t* s_rank, const int32_t* t_rank, int64_t nq,
                int64_t* dist, cudaStream_t s) {
    const int64_t Dp = t->d.max_depth + 1;
    const int64_t per_warp = 2 * Dp + (Dp + 1) / 2 + 1;  // int64 words: F, R, chain (int32)
    const int64_t warps = std::min<int64_t>(nq, (int64_t)t->sms * 32);
    const int block = 128;
    const int64_t blocks = (warps * 32 + block - 1) / block;
    void* scratch = nullptr;
    NWCCH_CUDA_TRY(scratch_alloc(&scratch, (size_t)(blocks * (block / 32)) * per_warp * sizeof(int64_t), s));
    k_query_plain<T><<<(unsigned)blocks, block, 0, s>>>(t->d, up, dn, s_rank, t_rank, nq, dist, (int64_t*)scratch,
                                                       stream_slot(t, s).err);
    const cudaError_t launch = cudaGetLastError();
    NWCCH_CUDA_TRY(cudaFreeAsync(scratch, s));
    NWCCH_CUDA_TRY(launch);
    return consume_error(t, s);
}

}  // namespace nwcch

using namespace nwcch;

extern "C" int nwcch_query_batch(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                                 const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq,
                                 int64_t* dist_dev, void* stream) {
    if (!t || nq < 0 || (nq > 0 && ((t->d.m_plus > 0 && (!up_dev || !dn_dev)) || !s_rank_dev || !t_rank_dev || !dist_dev)))
        return NWCCH_ERR_ARG;
    if (nq == 0) return NWCCH_OK;
    bool used = false;
    const int rc = query_sn_async<int32_t>(t, up_dev, dn_dev, s_rank_dev, t_rank_dev, nq, dist_dev,
                                           (cudaStream_t)stream, true, &used);
    if (rc) return rc;
    if (used) return consume_error(t, (cudaStream_t)stream);
    return query_plain<int32_t>(t, up_dev, dn_dev, s_rank_dev, t_rank_dev, nq, dist_dev, (cudaStream_t)stream);
}

extern "C" int nwcch_query_batch_async(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                                       const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq,
                                       int64_t* dist_dev, void* stream) {
    if (!t || nq < 0 || (nq > 0 && ((t->d.m_plus > 0 && (!up_dev || !dn_dev)) || !s_rank_dev || !t_rank_dev || !dist_dev)))
        return NWCCH_ERR_ARG;
    if (nq == 0) return NWCCH_OK;
    bool used = false;
    const int rc = query_sn_async<int32_t>(t, up_dev, dn_dev, s_rank_dev, t_rank_dev, nq, dist_dev,
                                           (cudaStream_t)stream, false, &used);
    if (rc || used) return rc;
    return NWCCH_ERR_CAPACITY;  // elimination tree too deep for the shared-memory labels
}

extern "C" int nwcch_query_batch_plain(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                                       const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq,
                                       int64_t* dist_dev, void* stream) {
    if (!t || nq < 0 || (nq > 0 && ((t->d.m_plus > 0 && (!up_dev || !dn_dev)) || !s_rank_dev || !t_rank_dev || !dist_dev)))
        return NWCCH_ERR_ARG;
    if (nq == 0) return NWCCH_OK;
    return query_plain<int32_t>(t, up_dev, dn_dev, s_rank_dev, t_rank_dev, nq, dist_dev, (cudaStream_t)stream);
}

extern "C" int nwcch_query_batch_i64(nwcch_topology* t, const int64_t* up_dev, const int64_t* dn_dev,
                                     const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq,
                                     int64_t* dist_dev, void* stream) {
    if (!t || nq < 0 || (nq > 0 && ((t->d.m_plus > 0 && (!up_dev || !dn_dev)) || !s_rank_dev || !t_rank_dev || !dist_dev)))
        return NWCCH_ERR_ARG;
    if (nq == 0) return NWCCH_OK;
    bool used = false;
    const int rc = query_sn_async<int64_t>(t, up_dev, dn_dev, s_rank_dev, t_rank_dev, nq, dist_dev,
                                           (cudaStream_t)stream, true, &used);
    if (rc) return rc;
    if (used) return consume_error(t, (cudaStream_t)stream);
    return query_plain<int64_t>(t, up_dev, dn_dev, s_rank_dev, t_rank_dev, nq, dist_dev, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// Allocation-free query entry point.
//
// nwcch_query_batch takes its per-warp label scratch from a stream-ordered allocation.
// Some callers cannot allocate at all: a serving loop whose admission control
// has already handed every byte of device memory to resident metrics, an
// embedding application whose own allocator owns the device and forbids
// direct CUDA allocations, or a latency-critical path that must not risk an
// allocator call stalling behind other work. nwcch_query_batch_noalloc serves
// them: the same query kernel, with its scratch in the fixed array below,
// which every GPU that loads this library holds until the process exits.

namespace nwcch {

// 32 MiB of label scratch, shared by every call on a device.
constexpr int64_t kStaticQueryWords = (int64_t)4 << 20;
static __device__ __align__(256) int64_t g_query_scratch[kStaticQueryWords];

namespace {
std::mutex g_scratch_mu;
int64_t* g_scratch_addr[256];  // device address of g_query_scratch, per device
}  // namespace

// The host cannot name a __device__ array directly (its host-side symbol is
// only a stand-in), so its device address is looked up once per device, with
// that device current, and cached. The cache belongs to the device's primary
// context: after cudaDeviceReset the process must not call this entry point
// again on that device (the cached address would be stale).
static int static_query_scratch(int64_t** out) {
    int dev = 0;
    NWCCH_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) return NWCCH_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_query_scratch) != cudaSuccess || !p) {
            cudaGetLastError();  // a failed lookup must not surface as a later launch's error
            return NWCCH_ERR_CUDA;
        }
        g_scratch_addr[dev] = static_cast<int64_t*>(p);
    }
    *out = g_scratch_addr[dev];
    return NWCCH_OK;
}

}  // namespace nwcch

extern "C" int nwcch_query_batch_noalloc(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                                         const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq,
                                         int64_t* dist_dev, void* stream) {
    if (!t || nq < 0 || (nq > 0 && ((t->d.m_plus > 0 && (!up_dev || !dn_dev)) || !s_rank_dev || !t_rank_dev || !dist_dev)))
        return NWCCH_ERR_ARG;
    if (nq == 0) return NWCCH_OK;
    const int64_t Dp = t->d.max_depth + 1;
    const int64_t per_warp = 2 * Dp + (Dp + 1) / 2 + 1;  // int64 words: F, R, chain
    const int block = 128, warps_per_block = block / 32;
    // whole blocks of warps must fit in the fixed scratch
    const int64_t max_blocks = kStaticQueryWords / (per_warp * warps_per_block);
    if (max_blocks < 1) return NWCCH_ERR_CAPACITY;  // elimination tree too deep for the fixed scratch
    int64_t* scratch = nullptr;
    const int rc = static_query_scratch(&scratch);
    if (rc) return rc;
    const int64_t want_blocks = (std::min<int64_t>(nq, (int64_t)t->sms * 32) + warps_per_block - 1) / warps_per_block;
    const int64_t blocks = std::min(want_blocks, max_blocks);
    cudaStream_t s = (cudaStream_t)stream;
    // no state in the scratch survives between queries: every label and chain
    // slot a query reads it writes first, so nothing needs clearing
    k_query_plain<int32_t><<<(unsigned)blocks, block, 0, s>>>(t->d, up_dev, dn_dev, s_rank_dev, t_rank_dev, nq,
                                                             dist_dev, scratch, stream_slot(t, s).err);
    NWCCH_CUDA_TRY(cudaGetLastError());
    return consume_error(t, s);
}
