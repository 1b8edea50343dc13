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

#include "query_sn.cuh"

namespace nwcch {

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

// wide != nullptr: only the queries flagged there (the rest is answered);
// otherwise every query, unless int32 values fit 32-bit labels.
template <class T>
__global__ void k_query_sn(DevTopo D, SnDev S, const T* __restrict__ up, const T* __restrict__ dn,
                           const int32_t* __restrict__ s_rank, const int32_t* __restrict__ t_rank, int64_t nq,
                           int64_t* __restrict__ dist, const unsigned int* __restrict__ maxabs,
                           int* __restrict__ err, int dense_rows, const int32_t* __restrict__ wide) {
    if (sizeof(T) == 4 && !wide && small_labels(D, maxabs)) return;  // answered by k_query_sn32
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
        if (wide && !wide[q]) continue;
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
    NWCCH_CUDA_TRY(allow_dynamic_smem((const void*)kernel, smem));
    int per_sm = 0;
    const int sms = device_sms();
    NWCCH_CUDA_TRY(blocks_per_sm((const void*)kernel, 32 * warps, smem, &per_sm));
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
    int64_t launches = 0;
    if (sizeof(T) == 4 && nq <= t->tune.query_stream_max) {
        // few queries: a CTA per chain, the chains streamed by bulk copies
        // (its 64-bit fallback flagged per query, no pass over the metric)
        bool stream_used = false;
        const int rc = query_stream_async(t, reinterpret_cast<const int32_t*>(up), reinterpret_cast<const int32_t*>(dn),
                                          s_rank, t_rank, nq, dist, err, s, &stream_used, &launches);
        if (rc) return rc;
        if (stream_used) {
            t->last_query_launches = launches;
            *used = true;
            return NWCCH_OK;
        }
    }
    if (sizeof(T) == 4) {
        // 32-bit labels when the metric's values allow them (decided on the
        // device: each kernel returns at once when the batch is not its own)
        NWCCH_CUDA_TRY(cudaMemsetAsync(maxabs, 0, sizeof(unsigned int), s));
        launches++;
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
        bool top_used = false;
        if (nq > t->tune.query_cta_max) {
            // large batch: the top of the tree as (min,+) products over
            // chains (stream-ordered scratch, also when enqueued only)
            int64_t top_launches = 0;
            const int rc = query_top_async(t, u32, d32, s_rank, t_rank, nq, dist, maxabs, err, s, &top_used,
                                           &top_launches);
            if (rc) return rc;
            launches += top_launches;
        }
        if (top_used) {
            // answered (or left to the 64-bit kernel below)
        } else if (nq <= t->tune.query_cta_max && cta_smem <= 200 * 1024) {
            // few queries: a CTA per query, 16 warps when there are at most
            // as many queries as SMs, else 8
            int64_t blocks = 0;
            const int rows = t->tune.query_cta_dense_rows;
            if (nq <= t->tune.query_cta_wide_max) {
                int rc = launch_shape(k_query_sn32_cta<16>, 16, cta_smem, nq * 16, &blocks);
                if (rc) return rc;
                launches++;
                k_query_sn32_cta<16><<<(unsigned)blocks, 512, cta_smem, s>>>(t->d, S, u32, d32, s_rank, t_rank, nq,
                                                                            dist, maxabs, err, rows);
            } else {
                int rc = launch_shape(k_query_sn32_cta<8>, 8, cta_smem, nq * 8, &blocks);  // one query per CTA
                if (rc) return rc;
                launches++;
                k_query_sn32_cta<8><<<(unsigned)blocks, 256, cta_smem, s>>>(t->d, S, u32, d32, s_rank, t_rank, nq,
                                                                           dist, maxabs, err, rows);
            }
        } else if (allow_alloc && (force_global || per_warp > t->tune.query_smem_labels_max)) {
            // deep tree: labels in global scratch, occupancy set by registers
            int64_t blocks = 0;
            int rc = launch_shape(kern, 4, 0, nq, &blocks);
            if (rc) return rc;
            void* scratch = nullptr;
            NWCCH_CUDA_TRY(scratch_alloc(&scratch, (size_t)(blocks * 4 * per_warp), s));
            launches++;
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
                launches++;
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
                                                             err, t->tune.query_dense_rows, nullptr);
    NWCCH_CUDA_TRY(cudaGetLastError());
    t->last_query_launches = launches + 1;
    *used = true;
    return NWCCH_OK;
}

int query_sn64_flagged(nwcch_topology* t, const int32_t* up, const int32_t* dn, const int32_t* s_rank,
                       const int32_t* t_rank, int64_t nq, int64_t* dist, const int32_t* wide, int* err,
                       cudaStream_t s) {
    int w64 = 0;
    size_t smem64 = 0;
    if (!t->sn_plan || !sn_query_shape(t, 20, &w64, &smem64)) return NWCCH_ERR_CAPACITY;
    const SnDev& S = static_cast<SnPlan*>(t->sn_plan)->dev;
    int64_t blocks = 0;
    int rc = launch_shape(k_query_sn<int32_t>, w64, smem64, nq, &blocks);
    if (rc) return rc;
    k_query_sn<int32_t><<<(unsigned)blocks, 32 * w64, smem64, s>>>(t->d, S, up, dn, s_rank, t_rank, nq, dist,
                                                                   nullptr, err, t->tune.query_dense_rows, wide);
    NWCCH_CUDA_TRY(cudaGetLastError());
    return NWCCH_OK;
}

template int query_sn_async<int32_t>(nwcch_topology*, const int32_t*, const int32_t*, const int32_t*,
                                     const int32_t*, int64_t, int64_t*, cudaStream_t, bool, bool*);
template int query_sn_async<int64_t>(nwcch_topology*, const int64_t*, const int64_t*, const int32_t*,
                                     const int32_t*, int64_t, int64_t*, cudaStream_t, bool, bool*);

}  // namespace nwcch
