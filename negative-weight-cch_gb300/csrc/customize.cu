// Plain per-metric customization and the negative-cycle scan.
//
// Customization computes, for every shortcut arc (y,z) of the upward graph,
//   up(y,z) = min(base_up(y,z), min_{x in N-(y) & N-(z)} dn(x,y) + up(x,z))
//   dn(y,z) = min(base_dn(y,z), min_{x in N-(y) & N-(z)} dn(x,z) + up(x,y))
// i.e. the lower-triangle (min,+) recurrence of python/cch_nb.py:529-563
// (= cpp/cch.cpp:437-463), evaluated in pull form: the arcs of one row y are
// owned by one thread block, which gathers every lower triangle (x; y, z) from
// the rows of its lower neighbours x. Rows of one level depend only on rows of
// lower levels (level = 1 + max level below, cpp/cch.cpp:468-480), so a level
// is one launch and needs no atomics outside shared memory. Integer minima are
// order independent, so the result equals the serial reference bit for bit.
//
// Storage T is int32 (fast) or int64 (exact for any conservative metric of a
// graph with n * max|w| < 2^62).

#include <algorithm>

#include "common.cuh"
#include "customize.h"
#include "supernodal.h"
#include "topology.h"

namespace nwcch {

// Base values gathered per shortcut arc: the minimum over the original arcs
// mapped onto it, by direction (their list is grouped by shortcut arc, so
// the arcs' values are written once, coalesced, with no fill and no atomics;
// an arc with none gets INF).
template <class T>
__global__ void __launch_bounds__(256) k_base_gather(DevTopo D, const int32_t* __restrict__ w, T* __restrict__ up,
                                                      T* __restrict__ dn, int* __restrict__ err) {
    pdl_wait();
    pdl_launch_dependents();
    w += blockIdx.y * D.m;  // metric blockIdx.y of a metric-major batch
    up += blockIdx.y * D.m_plus;
    dn += blockIdx.y * D.m_plus;
    int bad = 0;
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < D.m_plus;
         c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j0 = D.aeoff[c], j1 = D.aeoff[c + 1];
        T nu = Lim<T>::INF, nd = Lim<T>::INF;
        for (int64_t j = j0; j < j1; j++) {
            const int32_t x = D.aedir[j];
            const int32_t wk = w[x & 0x7fffffff];
            if (wk == INF32) {
                bad |= ERR_ARG;
                continue;
            }
            if (x < 0) nu = min(nu, (T)wk);
            else nd = min(nd, (T)wk);
        }
        up[c] = nu;
        dn[c] = nd;
    }
    if (bad) atomicOr(err, bad);
}

template <class T>
__device__ __forceinline__ void smin(T* p, T v);
template <>
__device__ __forceinline__ void smin<int32_t>(int32_t* p, int32_t v) {
    atomicMin(p, v);
}
template <>
__device__ __forceinline__ void smin<int64_t>(int64_t* p, int64_t v) {
    atomicMin(reinterpret_cast<long long*>(p), (long long)v);
}

// One block per row y of a level. Shared memory: the row's heads and its two
// accumulators. Warps take the downward arcs (x,y); lanes walk the part of
// row x above y, which chordality places inside row y.
template <class T>
__global__ void __launch_bounds__(128) k_pull_rows(DevTopo D, const int32_t* __restrict__ verts,
                                                   T* __restrict__ up, T* __restrict__ dn, int* __restrict__ err) {
    extern __shared__ __align__(16) unsigned char smraw[];
    const int32_t y = verts[blockIdx.x];
    const int64_t b = D.first[y];
    const int32_t d = (int32_t)(D.first[y + 1] - b);
    if (d == 0) return;
    T* au = reinterpret_cast<T*>(smraw);
    T* ad = au + d;
    int32_t* rowz = reinterpret_cast<int32_t*>(ad + d);
    for (int p = threadIdx.x; p < d; p += blockDim.x) {
        rowz[p] = D.head[b + p];
        au[p] = up[b + p];
        ad[p] = dn[b + p];
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    int e = 0;
    for (int64_t j = D.doff[y] + warp; j < D.doff[y + 1]; j += nwarps) {
        const int32_t a = D.darc[j];
        const int64_t rend = D.first[D.tail[a] + 1];
        const T dyx = dn[a], uxy = up[a];
        for (int64_t kk = a + 1 + lane; kk < rend; kk += 32) {
            const int32_t z = D.head[kk];
            int lo = 0, hi = d;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (rowz[mid] < z) lo = mid + 1;
                else hi = mid;
            }
            if (lo >= d || rowz[lo] != z) {
                e |= ERR_TOPOLOGY;
                continue;
            }
            T c;
            if (splus(dyx, up[kk], c, e)) smin(&au[lo], c);  // y -> x -> z
            if (splus(dn[kk], uxy, c, e)) smin(&ad[lo], c);  // z -> x -> y
        }
    }
    __syncthreads();
    for (int p = threadIdx.x; p < d; p += blockDim.x) {
        up[b + p] = au[p];
        dn[b + p] = ad[p];
    }
    if (e) atomicOr(err, e);
}

template <class T>
__global__ void k_negcycle(const T* __restrict__ up, const T* __restrict__ dn, int64_t count,
                           unsigned long long* __restrict__ out) {
    up += blockIdx.y * count;  // metric blockIdx.y of a metric-major batch
    dn += blockIdx.y * count;
    out += blockIdx.y;
    unsigned long long c = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count;
         i += (int64_t)gridDim.x * blockDim.x)
        c += negative_pair(up[i], dn[i]) ? 1ull : 0ull;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

__global__ void k_negloops(const int32_t* __restrict__ loops, int64_t nloops, const int32_t* __restrict__ w,
                           unsigned long long* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nloops;
         i += (int64_t)gridDim.x * blockDim.x)
        if (w[loops[i]] < 0) atomicAdd(out, 1ull);
}

int grid_for(int64_t count, int block) {
    const int64_t g = (count + block - 1) / block;
    return (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)device_sms() * 32));
}

template <class T>
int base_init(nwcch_topology* t, const int32_t* w, T* up, T* dn, cudaStream_t s, int* err, int metrics) {
    const DevTopo& D = t->d;
    NWCCH_CUDA_TRY(launch_pdl(t->tune.pdl != 0, k_base_gather<T>, dim3(grid_for(D.m_plus, 256), metrics), dim3(256),
                              0, s, D, w, up, dn, err));
    return cudaGetLastError() == cudaSuccess ? NWCCH_OK : NWCCH_ERR_CUDA;
}

template <class T>
int customize_plain(nwcch_topology* t, const int32_t* w, T* up, T* dn, cudaStream_t s) {
    int* err = stream_slot(t, s).err;
    int rc = base_init<T>(t, w, up, dn, s, err);
    if (rc) return rc;
    const int max_smem = 227 * 1024;
    NWCCH_CUDA_TRY(allow_dynamic_smem((const void*)k_pull_rows<T>, (size_t)max_smem));
    for (int32_t l = 1; l < t->levels; l++) {
        if (t->level_tri[l] == 0) continue;
        const int64_t v0 = t->level_off[l], nv = t->level_off[l + 1] - v0;
        const size_t smem = (2 * sizeof(T) + sizeof(int32_t)) * (size_t)t->level_maxdeg[l];
        if (smem > (size_t)max_smem) return NWCCH_ERR_CAPACITY;
        k_pull_rows<T><<<(unsigned)nv, 128, smem, s>>>(t->d, t->level_verts + v0, up, dn, err);
    }
    return cudaGetLastError() == cudaSuccess ? NWCCH_OK : NWCCH_ERR_CUDA;
}

template <class T>
int negative_cycle_arcs(nwcch_topology* t, const T* up, const T* dn, int64_t* count, cudaStream_t s) {
    unsigned long long* c = stream_slot(t, s).counters;
    NWCCH_CUDA_TRY(cudaMemsetAsync(c, 0, sizeof(unsigned long long), s));
    k_negcycle<T><<<grid_for(t->d.m_plus, 256), 256, 0, s>>>(up, dn, t->d.m_plus, c);
    NWCCH_CUDA_TRY(cudaGetLastError());
    unsigned long long h = 0;
    NWCCH_CUDA_TRY(cudaMemcpyAsync(&h, c, sizeof(h), cudaMemcpyDeviceToHost, s));
    NWCCH_CUDA_TRY(cudaStreamSynchronize(s));
    *count = (int64_t)h;
    return NWCCH_OK;
}

template int base_init<int32_t>(nwcch_topology*, const int32_t*, int32_t*, int32_t*, cudaStream_t, int*, int);
template int base_init<int64_t>(nwcch_topology*, const int32_t*, int64_t*, int64_t*, cudaStream_t, int*, int);

}  // namespace nwcch

using namespace nwcch;

extern "C" int nwcch_customize_async(nwcch_topology* t, const int32_t* w_dev, int32_t* up_dev,
                                     int32_t* dn_dev, void* stream) {
    if (!t || (t->d.m_plus > 0 && (!up_dev || !dn_dev)) || (t->d.m > 0 && !w_dev)) return NWCCH_ERR_ARG;
    return launch_supernodal<int32_t>(t, static_cast<SnPlan*>(t->sn_plan), w_dev, up_dev, dn_dev,
                                      (cudaStream_t)stream);
}

extern "C" int nwcch_customize_i64_async(nwcch_topology* t, const int32_t* w_dev, int64_t* up_dev,
                                         int64_t* dn_dev, void* stream) {
    if (!t || (t->d.m_plus > 0 && (!up_dev || !dn_dev)) || (t->d.m > 0 && !w_dev)) return NWCCH_ERR_ARG;
    return launch_supernodal<int64_t>(t, static_cast<SnPlan*>(t->sn_plan), w_dev, up_dev, dn_dev,
                                      (cudaStream_t)stream);
}

extern "C" int nwcch_customize_plain_async(nwcch_topology* t, const int32_t* w_dev, int32_t* up_dev,
                                           int32_t* dn_dev, void* stream) {
    if (!t || (t->d.m_plus > 0 && (!up_dev || !dn_dev)) || (t->d.m > 0 && !w_dev)) return NWCCH_ERR_ARG;
    return customize_plain<int32_t>(t, w_dev, up_dev, dn_dev, (cudaStream_t)stream);
}

extern "C" int nwcch_customize_plain(nwcch_topology* t, const int32_t* w_dev, int32_t* up_dev, int32_t* dn_dev,
                                     void* stream) {
    const int rc = nwcch_customize_plain_async(t, w_dev, up_dev, dn_dev, stream);
    if (rc) return rc;
    return consume_error(t, (cudaStream_t)stream);
}

extern "C" int nwcch_check(nwcch_topology* t, void* stream) {
    if (!t) return NWCCH_ERR_ARG;
    return consume_error(t, (cudaStream_t)stream);
}

extern "C" int nwcch_customize(nwcch_topology* t, const int32_t* w_dev, int32_t* up_dev, int32_t* dn_dev,
                               void* stream) {
    const int rc = nwcch_customize_async(t, w_dev, up_dev, dn_dev, stream);
    if (rc) return rc;
    return consume_error(t, (cudaStream_t)stream);
}

extern "C" int nwcch_customize_i64(nwcch_topology* t, const int32_t* w_dev, int64_t* up_dev, int64_t* dn_dev,
                                   void* stream) {
    const int rc = nwcch_customize_i64_async(t, w_dev, up_dev, dn_dev, stream);
    if (rc) return rc;
    return consume_error(t, (cudaStream_t)stream);
}

extern "C" int nwcch_negative_cycle_arcs(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                                         int64_t* count, void* stream) {
    if (!t || (t->d.m_plus > 0 && (!up_dev || !dn_dev)) || !count) return NWCCH_ERR_ARG;
    return negative_cycle_arcs<int32_t>(t, up_dev, dn_dev, count, (cudaStream_t)stream);
}

extern "C" int nwcch_negative_cycle_arcs_i64(nwcch_topology* t, const int64_t* up_dev, const int64_t* dn_dev,
                                             int64_t* count, void* stream) {
    if (!t || (t->d.m_plus > 0 && (!up_dev || !dn_dev)) || !count) return NWCCH_ERR_ARG;
    return negative_cycle_arcs<int64_t>(t, up_dev, dn_dev, count, (cudaStream_t)stream);
}

extern "C" int nwcch_customize_batch_async(nwcch_topology* t, int64_t metrics, const int32_t* w_dev,
                                           int32_t* up_dev, int32_t* dn_dev, void* stream) {
    if (!t || metrics < 1 || metrics > 65535 || (t->d.m_plus > 0 && (!up_dev || !dn_dev)) || (t->d.m > 0 && !w_dev)) return NWCCH_ERR_ARG;
    return launch_supernodal<int32_t>(t, static_cast<SnPlan*>(t->sn_plan), w_dev, up_dev, dn_dev,
                                      (cudaStream_t)stream, (int)metrics);
}

extern "C" int nwcch_customize_batch(nwcch_topology* t, int64_t metrics, const int32_t* w_dev, int32_t* up_dev,
                                     int32_t* dn_dev, void* stream) {
    const int rc = nwcch_customize_batch_async(t, metrics, w_dev, up_dev, dn_dev, stream);
    if (rc) return rc;
    return consume_error(t, (cudaStream_t)stream);
}

extern "C" int nwcch_negative_cycle_arcs_batch_async(nwcch_topology* t, int64_t metrics, const int32_t* up_dev,
                                                     const int32_t* dn_dev, int64_t* counts_dev, void* stream) {
    if (!t || metrics < 1 || metrics > 65535 || (t->d.m_plus > 0 && (!up_dev || !dn_dev)) || !counts_dev) return NWCCH_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    NWCCH_CUDA_TRY(cudaMemsetAsync(counts_dev, 0, sizeof(int64_t) * metrics, s));
    k_negcycle<int32_t><<<dim3(grid_for(t->d.m_plus, 256), (unsigned)metrics), 256, 0, s>>>(
        up_dev, dn_dev, t->d.m_plus, reinterpret_cast<unsigned long long*>(counts_dev));
    NWCCH_CUDA_TRY(cudaGetLastError());
    return NWCCH_OK;
}

extern "C" int nwcch_negative_cycle_arcs_async(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                                               int64_t* count_dev, void* stream) {
    if (!t || (t->d.m_plus > 0 && (!up_dev || !dn_dev)) || !count_dev) return NWCCH_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    NWCCH_CUDA_TRY(cudaMemsetAsync(count_dev, 0, sizeof(int64_t), s));
    k_negcycle<int32_t><<<grid_for(t->d.m_plus, 256), 256, 0, s>>>(
        up_dev, dn_dev, t->d.m_plus, reinterpret_cast<unsigned long long*>(count_dev));
    NWCCH_CUDA_TRY(cudaGetLastError());
    return NWCCH_OK;
}

extern "C" int nwcch_negative_loops(nwcch_topology* t, const int32_t* w_dev, int64_t* count, void* stream) {
    if (!t || !count || (t->nloops > 0 && !w_dev)) return NWCCH_ERR_ARG;
    *count = 0;
    if (t->nloops == 0) return NWCCH_OK;
    cudaStream_t s = (cudaStream_t)stream;
    unsigned long long* c = stream_slot(t, s).counters + 1;
    NWCCH_CUDA_TRY(cudaMemsetAsync(c, 0, sizeof(unsigned long long), s));
    k_negloops<<<grid_for(t->nloops, 256), 256, 0, s>>>(t->loops, t->nloops, w_dev, c);
    NWCCH_CUDA_TRY(cudaGetLastError());
    unsigned long long h = 0;
    NWCCH_CUDA_TRY(cudaMemcpyAsync(&h, c, sizeof(h), cudaMemcpyDeviceToHost, s));
    NWCCH_CUDA_TRY(cudaStreamSynchronize(s));
    *count = (int64_t)h;
    return NWCCH_OK;
}
