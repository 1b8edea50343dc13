// The weight-independent arrays of a topology, derived on the device from
// the uploaded upward CSR (first, head), elimination tree (parent) and arc
// map (e_arc): the device half of the reference's preprocessing between
// symbolic() and customize() (python/cch_nb.py:431-515), which the host used
// to loop over.
//
//  - validation: rows strictly increasing above their vertex, parent = lowest
//    head, arc map in range;
//  - tail of every arc (one thread per row);
//  - elimination-tree depth by pointer jumping (log2 n rounds);
//  - level = elimination-tree height (1 + the highest level of a lower
//    neighbour: every lower neighbour of y lies in the subtree of one of y's
//    children, so the longest lower path is the longest child path), swept
//    up from the leaves, the last child to finish continuing to its parent;
//  - downward lists (arcs grouped by head, ascending tail) and the original
//    arcs of every shortcut arc (ascending arc id), by stable radix sorts;
//  - vertices by level, and per level the arcs, longest row and pull
//    triangles.
// Every array equals the one the host loops produced (tests compare them
// through nwcch_topology_export).

#include <cub/cub.cuh>

#include <algorithm>
#include <vector>

#include "common.cuh"
#include "topology.h"
#include "topology_build.h"

namespace nwcch {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__global__ void k_validate(int64_t n, int64_t mp, const int64_t* __restrict__ first, const int32_t* __restrict__ head,
                           const int32_t* __restrict__ parent, int* __restrict__ bad) {
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a0 = first[x], a1 = first[x + 1];
        if (a0 < 0 || a1 < a0 || a1 > mp) {
            *bad = 1;
            continue;
        }
        int64_t prev = x;
        for (int64_t a = a0; a < a1; a++) {
            const int32_t h = head[a];
            if (h <= prev || h >= n) {
                *bad = 1;
                break;
            }
            prev = h;
        }
        const int32_t p = a1 > a0 ? head[a0] : -1;
        if (parent[x] != p) *bad = 1;
    }
}

__global__ void k_validate_arcs(int64_t m, int64_t mp, const int64_t* __restrict__ e_arc, int* __restrict__ bad) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x)
        if (e_arc[k] < -1 || e_arc[k] >= mp) *bad = 1;
}

// tail of every arc; triangles (sum of d(d-1)/2) and the longest row
__global__ void k_rows(int64_t n, const int64_t* __restrict__ first, int32_t* __restrict__ tail,
                       unsigned long long* __restrict__ tri, int* __restrict__ maxdeg) {
    unsigned long long t = 0;
    int md = 0;
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a0 = first[x], a1 = first[x + 1], d = a1 - a0;
        for (int64_t a = a0; a < a1; a++) tail[a] = (int32_t)x;
        t += (unsigned long long)(d * (d - 1) / 2);
        md = max(md, (int)d);
    }
    for (int o = 16; o > 0; o >>= 1) {
        t += __shfl_xor_sync(FULL, t, o);
        md = max(md, __shfl_xor_sync(FULL, md, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (t) atomicAdd(tri, t);
        atomicMax(maxdeg, md);
    }
}

__global__ void k_jump_init(int64_t n, const int32_t* __restrict__ parent, int32_t* __restrict__ anc,
                            int32_t* __restrict__ dist, int32_t* __restrict__ nchild) {
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const int32_t p = parent[x];
        anc[x] = p;
        dist[x] = p >= 0 ? 1 : 0;
        if (p >= 0) atomicAdd(&nchild[p], 1);
    }
}

// one pointer-jumping round: dist += dist of the ancestor, ancestor doubled
__global__ void k_jump(int64_t n, const int32_t* __restrict__ anc_in, const int32_t* __restrict__ dist_in,
                       int32_t* __restrict__ anc_out, int32_t* __restrict__ dist_out) {
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const int32_t a = anc_in[x];
        if (a >= 0) {
            dist_out[x] = dist_in[x] + dist_in[a];
            anc_out[x] = anc_in[a];
        } else {
            dist_out[x] = dist_in[x];
            anc_out[x] = -1;
        }
    }
}

// heights from the leaves up: the child that finishes last continues with its
// parent (no thread waits for another)
__global__ void k_heights(int64_t n, const int32_t* __restrict__ parent, const int32_t* __restrict__ nchild,
                          int32_t* __restrict__ rem, int32_t* __restrict__ height) {
    for (int64_t v = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; v < n; v += (int64_t)gridDim.x * blockDim.x) {
        if (nchild[v] != 0) continue;
        int32_t x = (int32_t)v, h = 0;
        while (true) {
            const int32_t p = parent[x];
            if (p < 0) break;
            atomicMax(&height[p], h + 1);
            __threadfence();
            if (atomicSub(&rem[p], 1) != 1) break;
            x = p;
            h = atomicAdd(&height[p], 0);  // every child's maximum is in
        }
    }
}

__global__ void k_gather(int64_t count, const int32_t* __restrict__ idx, const int32_t* __restrict__ src,
                         int32_t* __restrict__ dst) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        dst[i] = src[idx[i]];
}

__global__ void k_iota(int64_t count, int32_t* __restrict__ out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (int32_t)i;
}

// sort key of an original arc: its shortcut arc, self-loops (-1) last
__global__ void k_arc_keys(int64_t m, int64_t mp, const int64_t* __restrict__ e_arc, int32_t* __restrict__ key,
                           int64_t* __restrict__ count) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < m; k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t a = e_arc[k];
        key[k] = a >= 0 ? (int32_t)a : (int32_t)mp;
        if (a >= 0) atomicAdd(reinterpret_cast<unsigned long long*>(&count[a]), 1ull);
    }
}

__global__ void k_count(int64_t count, const int32_t* __restrict__ key, int64_t* __restrict__ hist) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(reinterpret_cast<unsigned long long*>(&hist[key[i]]), 1ull);
}

__global__ void k_maxval(int64_t count, const int32_t* __restrict__ v, int* __restrict__ out) {
    int mx = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < count; i += (int64_t)gridDim.x * blockDim.x)
        mx = max(mx, v[i]);
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(FULL, mx, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, mx);
}

// per level: arcs (rows of the level's vertices), longest row
__global__ void k_level_rows(int64_t n, const int64_t* __restrict__ first, const int32_t* __restrict__ lvl,
                             unsigned long long* __restrict__ arcs, int* __restrict__ maxdeg) {
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const int32_t l = lvl[x];
        const int d = (int)(first[x + 1] - first[x]);
        // lanes of one level add once (levels of consecutive ranks repeat)
        const unsigned peers = __match_any_sync(__activemask(), l);
        const unsigned sum = __reduce_add_sync(peers, (unsigned)d);
        const int mx = (int)__reduce_max_sync(peers, (unsigned)d);
        if ((int)(threadIdx.x & 31) == __ffs(peers) - 1) {
            if (sum) atomicAdd(&arcs[l], (unsigned long long)sum);
            atomicMax(&maxdeg[l], mx);
        }
    }
}

// per level: pull triangles (arc (x, y) has first[x+1] - a - 1 of them, on
// y's level)
__global__ void k_level_tri(int64_t mp, const int64_t* __restrict__ first, const int32_t* __restrict__ tail,
                            const int32_t* __restrict__ head, const int32_t* __restrict__ lvl,
                            unsigned long long* __restrict__ tri) {
    for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < mp; a += (int64_t)gridDim.x * blockDim.x) {
        const int32_t l = lvl[head[a]];
        const unsigned c = (unsigned)(first[tail[a] + 1] - a - 1);
        const unsigned peers = __match_any_sync(__activemask(), l);
        const unsigned sum = __reduce_add_sync(peers, c);
        if ((int)(threadIdx.x & 31) == __ffs(peers) - 1 && sum) atomicAdd(&tri[l], (unsigned long long)sum);
    }
}

unsigned grid(int64_t count) {
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>((count + 255) / 256, (int64_t)device_sms() * 32));
}

int bits_for(int64_t v) {
    int b = 1;
    while (b < 62 && ((int64_t)1 << b) <= v) b++;
    return b;
}

// Scratch allocations of one derivation, freed on every exit path.
struct Scratch {
    std::vector<void*> ptrs;
    ~Scratch() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class V>
    V* get(int64_t count) {
        void* p = nullptr;
        if (cudaMalloc(&p, sizeof(V) * (size_t)std::max<int64_t>(1, count)) != cudaSuccess) return nullptr;
        ptrs.push_back(p);
        return static_cast<V*>(p);
    }
};

// Stable sort of (key, value) int32 pairs by the low `bits` bits of key.
int sort_pairs(Scratch& S, const int32_t* keys_in, int32_t* keys_out, const int32_t* vals_in, int32_t* vals_out,
               int64_t count, int bits) {
    if (count == 0) return NWCCH_OK;
    size_t bytes = 0;
    NWCCH_CUDA_TRY(cub::DeviceRadixSort::SortPairs(nullptr, bytes, keys_in, keys_out, vals_in, vals_out, count, 0,
                                                   bits));
    void* tmp = S.get<char>((int64_t)bytes);
    if (!tmp) return NWCCH_ERR_NOMEM;
    NWCCH_CUDA_TRY(cub::DeviceRadixSort::SortPairs(tmp, bytes, keys_in, keys_out, vals_in, vals_out, count, 0, bits));
    return NWCCH_OK;
}

// Exclusive prefix sums of count[0..len) into out[0..len] (out[len] = total).
int exclusive_scan(Scratch& S, const int64_t* count, int64_t* out, int64_t len) {
    NWCCH_CUDA_TRY(cudaMemset(out, 0, sizeof(int64_t)));
    if (len == 0) return NWCCH_OK;
    size_t bytes = 0;
    NWCCH_CUDA_TRY(cub::DeviceScan::InclusiveSum(nullptr, bytes, count, out + 1, len));
    void* tmp = S.get<char>((int64_t)bytes);
    if (!tmp) return NWCCH_ERR_NOMEM;
    NWCCH_CUDA_TRY(cub::DeviceScan::InclusiveSum(tmp, bytes, count, out + 1, len));
    return NWCCH_OK;
}

}  // namespace

int derive_topology(int64_t n, int64_t mp, int64_t m, const int64_t* first, const int32_t* head,
                    const int32_t* parent, const int64_t* e_arc, DerivedTopology* out) {
    Scratch S;
    int* flags = S.get<int>(4);  // bad, max degree, max depth, max level
    unsigned long long* tri = S.get<unsigned long long>(1);
    if (!flags || !tri) return NWCCH_ERR_NOMEM;
    NWCCH_CUDA_TRY(cudaMemset(flags, 0, 4 * sizeof(int)));
    NWCCH_CUDA_TRY(cudaMemset(tri, 0, sizeof(unsigned long long)));
    k_validate<<<grid(n), 256>>>(n, mp, first, head, parent, flags);
    k_validate_arcs<<<grid(m), 256>>>(m, mp, e_arc, flags);
    NWCCH_CUDA_TRY(cudaGetLastError());
    int bad = 0;
    NWCCH_CUDA_TRY(cudaMemcpy(&bad, flags, sizeof(int), cudaMemcpyDeviceToHost));
    if (bad) return NWCCH_ERR_TOPOLOGY;

    // tails, triangles, longest row
    k_rows<<<grid(n), 256>>>(n, first, out->tail, tri, flags + 1);
    // depths by pointer jumping, child counts
    int32_t *anc0 = S.get<int32_t>(n), *anc1 = S.get<int32_t>(n), *dist1 = S.get<int32_t>(n);
    int32_t *nchild = S.get<int32_t>(n), *rem = S.get<int32_t>(n);
    if (!anc0 || !anc1 || !dist1 || !nchild || !rem) return NWCCH_ERR_NOMEM;
    NWCCH_CUDA_TRY(cudaMemset(nchild, 0, sizeof(int32_t) * n));
    k_jump_init<<<grid(n), 256>>>(n, parent, anc0, out->depth, nchild);
    int32_t *ai = anc0, *di = out->depth, *ao = anc1, *dO = dist1;
    for (int r = 0; r < bits_for(n); r++) {
        k_jump<<<grid(n), 256>>>(n, ai, di, ao, dO);
        std::swap(ai, ao);
        std::swap(di, dO);
    }
    if (di != out->depth) NWCCH_CUDA_TRY(cudaMemcpy(out->depth, di, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice));
    k_maxval<<<grid(n), 256>>>(n, out->depth, flags + 2);
    k_gather<<<grid(mp), 256>>>(mp, head, out->depth, out->hdep);
    // levels (heights)
    NWCCH_CUDA_TRY(cudaMemcpy(rem, nchild, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice));
    NWCCH_CUDA_TRY(cudaMemset(out->vlevel, 0, sizeof(int32_t) * n));
    k_heights<<<grid(n), 256>>>(n, parent, nchild, rem, out->vlevel);
    k_maxval<<<grid(n), 256>>>(n, out->vlevel, flags + 3);
    NWCCH_CUDA_TRY(cudaGetLastError());

    // downward lists: arcs by head, stable (ascending arc id = ascending tail)
    int32_t* iota = S.get<int32_t>(std::max(std::max(mp, m), n));
    int32_t* keys = S.get<int32_t>(std::max(std::max(mp, m), n));
    int64_t* hist = S.get<int64_t>(std::max(n, mp) + 1);
    if (!iota || !keys || !hist) return NWCCH_ERR_NOMEM;
    k_iota<<<grid(std::max(std::max(mp, m), n)), 256>>>(std::max(std::max(mp, m), n), iota);
    int rc = sort_pairs(S, head, keys, iota, out->darc, mp, bits_for(n));
    if (rc) return rc;
    NWCCH_CUDA_TRY(cudaMemset(hist, 0, sizeof(int64_t) * (n + 1)));
    k_count<<<grid(mp), 256>>>(mp, head, hist);
    if ((rc = exclusive_scan(S, hist, out->doff, n))) return rc;

    // original arcs of every shortcut arc (ascending id), self-loops after them
    int32_t* sorted_k = S.get<int32_t>(m);
    if (!sorted_k) return NWCCH_ERR_NOMEM;
    NWCCH_CUDA_TRY(cudaMemset(hist, 0, sizeof(int64_t) * (mp + 1)));
    k_arc_keys<<<grid(m), 256>>>(m, mp, e_arc, keys, hist);
    int32_t* keys2 = S.get<int32_t>(m);
    if (!keys2) return NWCCH_ERR_NOMEM;
    if ((rc = sort_pairs(S, keys, keys2, iota, sorted_k, m, bits_for(mp)))) return rc;
    if ((rc = exclusive_scan(S, hist, out->aeoff, mp))) return rc;
    int64_t mapped = 0;
    NWCCH_CUDA_TRY(cudaMemcpy(&mapped, out->aeoff + mp, sizeof(int64_t), cudaMemcpyDeviceToHost));
    out->nloops = m - mapped;
    out->aeidx_sorted = sorted_k;  // [0, mapped): aeidx; [mapped, m): self-loops
    S.ptrs.erase(std::find(S.ptrs.begin(), S.ptrs.end(), (void*)sorted_k));  // handed to the caller

    // scalars
    int h[4] = {0, 0, 0, 0};
    unsigned long long htri = 0;
    NWCCH_CUDA_TRY(cudaMemcpy(h, flags, sizeof(h), cudaMemcpyDeviceToHost));
    NWCCH_CUDA_TRY(cudaMemcpy(&htri, tri, sizeof(htri), cudaMemcpyDeviceToHost));
    out->max_deg = h[1];
    out->max_depth = h[2];
    out->levels = n > 0 ? h[3] + 1 : 0;
    out->triangles = (int64_t)htri;
    const int64_t L = out->levels;

    // vertices by level (stable: ascending rank), and the level tables
    if ((rc = sort_pairs(S, out->vlevel, keys, iota, out->level_verts, n, bits_for(L)))) return rc;
    unsigned long long* larcs = S.get<unsigned long long>(L);
    unsigned long long* ltri = S.get<unsigned long long>(L);
    int* lmax = S.get<int>(L);
    if (!larcs || !ltri || !lmax) return NWCCH_ERR_NOMEM;
    NWCCH_CUDA_TRY(cudaMemset(hist, 0, sizeof(int64_t) * (L + 1)));
    NWCCH_CUDA_TRY(cudaMemset(larcs, 0, sizeof(unsigned long long) * L));
    NWCCH_CUDA_TRY(cudaMemset(ltri, 0, sizeof(unsigned long long) * L));
    NWCCH_CUDA_TRY(cudaMemset(lmax, 0, sizeof(int) * L));
    k_count<<<grid(n), 256>>>(n, out->vlevel, hist);
    k_level_rows<<<grid(n), 256>>>(n, first, out->vlevel, larcs, lmax);
    k_level_tri<<<grid(mp), 256>>>(mp, first, out->tail, head, out->vlevel, ltri);
    NWCCH_CUDA_TRY(cudaGetLastError());
    std::vector<int64_t> cnt(L);
    std::vector<unsigned long long> a(L), t(L);
    out->level_maxdeg.assign(L, 0);
    if (L) {
        NWCCH_CUDA_TRY(cudaMemcpy(cnt.data(), hist, sizeof(int64_t) * L, cudaMemcpyDeviceToHost));
        NWCCH_CUDA_TRY(cudaMemcpy(a.data(), larcs, sizeof(unsigned long long) * L, cudaMemcpyDeviceToHost));
        NWCCH_CUDA_TRY(cudaMemcpy(t.data(), ltri, sizeof(unsigned long long) * L, cudaMemcpyDeviceToHost));
        NWCCH_CUDA_TRY(cudaMemcpy(out->level_maxdeg.data(), lmax, sizeof(int) * L, cudaMemcpyDeviceToHost));
    }
    out->level_off.assign(L + 1, 0);
    out->level_arc_off.assign(L + 1, 0);
    out->level_tri.assign(L, 0);
    for (int64_t l = 0; l < L; l++) {
        out->level_off[l + 1] = out->level_off[l] + cnt[l];
        out->level_arc_off[l + 1] = out->level_arc_off[l] + (int64_t)a[l];
        out->level_tri[l] = (int64_t)t[l];
    }
    NWCCH_CUDA_TRY(cudaDeviceSynchronize());
    return NWCCH_OK;
}

}  // namespace nwcch
