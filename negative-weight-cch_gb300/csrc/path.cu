// Shortest paths of ET queries, unpacked through the lower triangles that
// realise each shortcut (python/cch.py:406-507), on the device.
//
// One warp per (s, t) pair. Both sweeps walk the ancestor chain one vertex at
// a time, labels indexed by chain position, and keep the first arc (in the
// reference's sweep order: chain vertex ascending, then row order) that
// reaches each label's value: rows are processed in order and the heads of
// one row are distinct, so a plain strict-less update reproduces it. The
// peak is the lowest common ancestor reaching the minimum (a lexicographic
// warp minimum of (value, chain position)). The legs down from the peak are
// followed serially, then each leg is unpacked with an explicit stack: a
// shortcut (v, w) splits at its lowest lower-triangle vertex x whose sides
// add up to its value (32 candidates of the downward list at a time, the
// first by ballot), and is an original arc when there is none. Pass 0 counts
// each path's vertices, pass 1 writes them at the offsets the host computed.

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "topology.h"

namespace nwcch {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ int64_t find_arc(const DevTopo& D, int32_t lo, int32_t hi) {
    int64_t a = D.first[lo], b = D.first[lo + 1];
    const int64_t end = b;
    while (a < b) {
        const int64_t mid = (a + b) >> 1;
        if (D.head[mid] < hi) a = mid + 1;
        else b = mid;
    }
    return (a < end && D.head[a] == hi) ? a : -1;
}

// Per-warp scratch layout (bytes), Dp = depth + 1 chain positions.
struct PathScratch {
    int64_t* F;
    int64_t* R;
    int32_t* PF;
    int32_t* PR;
    int32_t* CS;
    int32_t* CT;
    int32_t* legs;   // pairs, 2 * Dp of them
    int32_t* stack;  // pairs, levels + 2 of them
};

__host__ __device__ inline int64_t path_scratch_bytes(int64_t Dp, int64_t levels) {
    return 16 * Dp + 16 * Dp + 16 * Dp + 8 * (levels + 2) + 64;
}

__device__ inline PathScratch carve(unsigned char* p, int64_t Dp) {
    PathScratch s;
    s.F = reinterpret_cast<int64_t*>(p);
    s.R = s.F + Dp;
    s.PF = reinterpret_cast<int32_t*>(s.R + Dp);
    s.PR = s.PF + Dp;
    s.CS = s.PR + Dp;
    s.CT = s.CS + Dp;
    s.legs = s.CT + Dp;
    s.stack = s.legs + 4 * Dp;
    return s;
}

// One sweep up the chain of `start` (depth dstart): labels L, first
// reaching arcs P, chain vertices C, all by chain position.
template <class T>
__device__ void sweep(const DevTopo& D, const T* __restrict__ W, int32_t start, int32_t dstart, int64_t* L,
                      int32_t* P, int32_t* C, int& e) {
    const int lane = threadIdx.x & 31;
    for (int32_t i = lane; i <= dstart; i += 32) {
        L[i] = INF64;
        P[i] = -1;
    }
    __syncwarp();
    if (lane == 0) L[0] = 0;
    __syncwarp();
    int32_t p = 0;
    for (int32_t x = start; x >= 0; x = D.parent[x], p++) {
        if (lane == 0) C[p] = x;
        const int64_t lx = L[p];
        if (lx != INF64) {
            for (int64_t a = D.first[x] + lane; a < D.first[x + 1]; a += 32) {
                const int64_t c = label_plus(lx, W[a], e);
                const int32_t q = dstart - D.hdep[a];
                if (c < L[q]) {
                    L[q] = c;
                    P[q] = (int32_t)a;
                }
            }
        }
        __syncwarp();
    }
}

template <class T, int PASS>
__global__ void __launch_bounds__(128) k_query_path(DevTopo D, const T* __restrict__ up, const T* __restrict__ dn,
                                                    const int32_t* __restrict__ s_rank,
                                                    const int32_t* __restrict__ t_rank, int64_t nq,
                                                    int64_t* __restrict__ dist, int64_t* __restrict__ off,
                                                    int32_t* __restrict__ path, unsigned char* __restrict__ scratch,
                                                    int64_t per_warp, int32_t stack_cap, int* __restrict__ err) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t Dp = D.max_depth + 1;
    PathScratch S = carve(scratch + warp * per_warp, Dp);
    int e = 0;
    for (int64_t q = warp; q < nq; q += nwarps) {
        const int32_t s = s_rank[q], t = t_rank[q];
        if (s < 0 || s >= D.n || t < 0 || t >= D.n) {
            if (lane == 0) {
                if (PASS == 0) {
                    dist[q] = INF64;
                    off[q + 1] = 0;
                }
            }
            e |= ERR_ARG;
            continue;
        }
        const int32_t ds = D.depth[s], dt = D.depth[t];
        sweep<T>(D, up, s, ds, S.F, S.PF, S.CS, e);
        sweep<T>(D, dn, t, dt, S.R, S.PR, S.CT, e);
        // the peak: (value, chain position) lexicographic minimum
        int64_t bv = INF64;
        int32_t bp = 0x7fffffff;
        for (int32_t p = lane; p <= ds; p += 32) {
            const int32_t x = S.CS[p];
            const int32_t dx = ds - p;
            if (dx <= dt && S.CT[dt - dx] == x) {
                const int64_t fv = S.F[p], rv = S.R[dt - dx];
                if (fv != INF64 && rv != INF64) {
                    int64_t v;
                    splus(fv, rv, v, e);
                    if (v < bv || (v == bv && p < bp)) {
                        bv = v;
                        bp = p;
                    }
                }
            }
        }
        for (int o = 16; o > 0; o >>= 1) {
            const int64_t ov = __shfl_xor_sync(FULL, bv, o);
            const int32_t op = __shfl_xor_sync(FULL, bp, o);
            if (ov < bv || (ov == bv && op < bp)) {
                bv = ov;
                bp = op;
            }
        }
        int64_t len = 0;
        const int64_t base = PASS == 1 ? off[q] : 0;
        if (bv != INF64) {
            // legs: s -> peak (reversed walk down the forward labels), then
            // peak -> t; lane 0 only
            // every step moves to a deeper chain vertex, so a walk has at
            // most depth + 1 steps; a missing arc (impossible for a finite
            // label) stops it with ERR_TOPOLOGY
            int32_t nlegs = 0;
            if (lane == 0) {
                const int32_t peak = S.CS[bp];
                int32_t cnt = 0;
                for (int32_t x = peak; x != s && cnt <= ds; cnt++) {
                    const int32_t a = S.PF[ds - D.depth[x]];
                    if (a < 0) {
                        e |= ERR_TOPOLOGY;
                        break;
                    }
                    x = D.tail[a];
                }
                int32_t i = cnt;
                for (int32_t x = peak; x != s && i > 0;) {
                    const int32_t a = S.PF[ds - D.depth[x]];
                    if (a < 0) break;
                    const int32_t v = D.tail[a];
                    --i;
                    S.legs[2 * i] = v;
                    S.legs[2 * i + 1] = x;
                    x = v;
                }
                nlegs = cnt;
                for (int32_t x = peak; x != t && nlegs < cnt + dt + 1;) {
                    const int32_t a = S.PR[dt - D.depth[x]];
                    if (a < 0) {
                        e |= ERR_TOPOLOGY;
                        break;
                    }
                    const int32_t v = D.tail[a];
                    S.legs[2 * nlegs] = x;
                    S.legs[2 * nlegs + 1] = v;
                    nlegs++;
                    x = v;
                }
            }
            nlegs = __shfl_sync(FULL, nlegs, 0);
            __syncwarp();
            if (lane == 0 && PASS == 1) path[base] = nlegs ? S.legs[0] : s;
            len = 1;
            for (int32_t l = 0; l < nlegs; l++) {
                int32_t sp = 0;
                if (lane == 0) {
                    S.stack[0] = S.legs[2 * l];
                    S.stack[1] = S.legs[2 * l + 1];
                }
                sp = 1;
                __syncwarp();
                while (sp > 0) {
                    sp--;
                    const int32_t v = S.stack[2 * sp], w = S.stack[2 * sp + 1];
                    __syncwarp();
                    const int32_t lo = min(v, w), hi = max(v, w);
                    const int64_t a = find_arc(D, lo, hi);
                    if (a < 0) {  // cannot happen on a chordal topology
                        e |= ERR_TOPOLOGY;
                        break;
                    }
                    const T cost = v < w ? up[a] : dn[a];
                    int32_t mid = -1;
                    for (int64_t j0 = D.doff[lo]; j0 < D.doff[lo + 1] && mid < 0; j0 += 32) {
                        const int64_t j = j0 + lane;
                        bool hit = false;
                        int32_t x = -1;
                        if (j < D.doff[lo + 1]) {
                            const int32_t xl = D.darc[j];
                            x = D.tail[xl];
                            const int64_t xh = find_arc(D, x, hi);
                            if (xh >= 0) {
                                const int64_t av = v == lo ? xl : xh, aw = w == lo ? xl : xh;
                                const T c1 = dn[av], c2 = up[aw];
                                if (c1 != Lim<T>::INF && c2 != Lim<T>::INF && cost != Lim<T>::INF) {
                                    int64_t c;
                                    int ee = 0;
                                    splus((int64_t)c1, (int64_t)c2, c, ee);
                                    hit = !ee && c == (int64_t)cost;
                                }
                            }
                        }
                        const unsigned m = __ballot_sync(FULL, hit);
                        if (m) mid = __shfl_sync(FULL, x, __ffs(m) - 1);
                    }
                    if (mid < 0) {
                        if (lane == 0 && PASS == 1) path[base + len] = w;
                        len++;
                    } else {
                        if (sp + 2 > stack_cap) {  // deeper than the level count: not chordal
                            e |= ERR_TOPOLOGY;
                            break;
                        }
                        if (lane == 0) {
                            S.stack[2 * sp] = mid;
                            S.stack[2 * sp + 1] = w;
                            S.stack[2 * sp + 2] = v;
                            S.stack[2 * sp + 3] = mid;
                        }
                        sp += 2;
                        __syncwarp();
                    }
                }
            }
        }
        if (lane == 0 && PASS == 0) {
            dist[q] = bv;
            off[q + 1] = len;
        }
        __syncwarp();
    }
    if (e) atomicOr(err, e);
}

}  // namespace

template <class T>
int query_paths(nwcch_topology* t, const T* up, const T* dn, const int32_t* s_rank, const int32_t* t_rank,
                int64_t nq, int64_t* dist, int64_t* off, int32_t* path, int64_t cap, int64_t* needed,
                cudaStream_t s) {
    const int64_t Dp = t->d.max_depth + 1;
    const int64_t per_warp = (path_scratch_bytes(Dp, t->levels) + 255) & ~255LL;
    const int64_t warps = std::max<int64_t>(1, std::min<int64_t>(nq, (int64_t)t->sms * 16));
    const int64_t blocks = (warps + 3) / 4;
    void* scratch = nullptr;
    NWCCH_CUDA_TRY(scratch_alloc(&scratch, (size_t)(blocks * 4 * per_warp), s));
    int* err = stream_slot(t, s).err;
    auto* sc = static_cast<unsigned char*>(scratch);
    NWCCH_CUDA_TRY(cudaMemsetAsync(off, 0, sizeof(int64_t), s));
    const int32_t stack_cap = t->levels + 2;
    k_query_path<T, 0><<<(unsigned)blocks, 128, 0, s>>>(t->d, up, dn, s_rank, t_rank, nq, dist, off, path, sc,
                                                       per_warp, stack_cap, err);
    cudaError_t launch = cudaGetLastError();
    if (launch != cudaSuccess) {
        cudaFreeAsync(scratch, s);
        return NWCCH_ERR_CUDA;
    }
    // path lengths -> offsets (host scan; paths are an interactive call)
    std::vector<int64_t> h(nq + 1);
    NWCCH_CUDA_TRY(cudaMemcpyAsync(h.data(), off, sizeof(int64_t) * (nq + 1), cudaMemcpyDeviceToHost, s));
    NWCCH_CUDA_TRY(cudaStreamSynchronize(s));
    for (int64_t i = 0; i < nq; i++) h[i + 1] += h[i];
    *needed = h[nq];
    if (h[nq] > cap) {
        NWCCH_CUDA_TRY(cudaMemcpyAsync(off, h.data(), sizeof(int64_t) * (nq + 1), cudaMemcpyHostToDevice, s));
        NWCCH_CUDA_TRY(cudaFreeAsync(scratch, s));
        NWCCH_CUDA_TRY(cudaStreamSynchronize(s));
        return NWCCH_ERR_CAPACITY;
    }
    NWCCH_CUDA_TRY(cudaMemcpyAsync(off, h.data(), sizeof(int64_t) * (nq + 1), cudaMemcpyHostToDevice, s));
    if (h[nq] > 0) {
        k_query_path<T, 1><<<(unsigned)blocks, 128, 0, s>>>(t->d, up, dn, s_rank, t_rank, nq, dist, off, path, sc,
                                                           per_warp, stack_cap, err);
        launch = cudaGetLastError();
    }
    NWCCH_CUDA_TRY(cudaFreeAsync(scratch, s));
    NWCCH_CUDA_TRY(launch);
    return consume_error(t, s);
}

}  // namespace nwcch

using namespace nwcch;

extern "C" int nwcch_query_paths(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                                 const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq, int64_t* dist_dev,
                                 int64_t* off_dev, int32_t* path_dev, int64_t cap, int64_t* needed, void* stream) {
    if (!t || nq < 0 || !off_dev || !needed || cap < 0 || (cap > 0 && !path_dev) ||
        (nq > 0 && ((t->d.m_plus > 0 && (!up_dev || !dn_dev)) || !s_rank_dev || !t_rank_dev || !dist_dev)))
        return NWCCH_ERR_ARG;
    *needed = 0;
    if (nq == 0) return cudaMemsetAsync(off_dev, 0, sizeof(int64_t), (cudaStream_t)stream) == cudaSuccess
                            ? NWCCH_OK : NWCCH_ERR_CUDA;
    return query_paths<int32_t>(t, up_dev, dn_dev, s_rank_dev, t_rank_dev, nq, dist_dev, off_dev, path_dev, cap,
                                needed, (cudaStream_t)stream);
}

extern "C" int nwcch_query_paths_i64(nwcch_topology* t, const int64_t* up_dev, const int64_t* dn_dev,
                                     const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq,
                                     int64_t* dist_dev, int64_t* off_dev, int32_t* path_dev, int64_t cap,
                                     int64_t* needed, void* stream) {
    if (!t || nq < 0 || !off_dev || !needed || cap < 0 || (cap > 0 && !path_dev) ||
        (nq > 0 && ((t->d.m_plus > 0 && (!up_dev || !dn_dev)) || !s_rank_dev || !t_rank_dev || !dist_dev)))
        return NWCCH_ERR_ARG;
    *needed = 0;
    if (nq == 0) return cudaMemsetAsync(off_dev, 0, sizeof(int64_t), (cudaStream_t)stream) == cudaSuccess
                            ? NWCCH_OK : NWCCH_ERR_CUDA;
    return query_paths<int64_t>(t, up_dev, dn_dev, s_rank_dev, t_rank_dev, nq, dist_dev, off_dev, path_dev, cap,
                                needed, (cudaStream_t)stream);
}
