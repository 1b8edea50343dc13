// Topology handle: uploads the upward CSR produced by the host-side
// preprocessing once, validates it and derives the structures the kernels
// need (tails, levels, elimination-tree depths, downward lists, arc ->
// original-arc index) on the device (topology_build.cu). Customization, scans, updates and queries for any
// number of metrics then run against this resident copy.

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "common.cuh"
#include "supernodal.h"
#include "topology.h"
#include "topology_build.h"

namespace nwcch {

namespace {

template <class T>
int alloc(nwcch_topology* t, int64_t count, T** dst) {
    void* p = nullptr;
    const size_t bytes = (size_t)std::max<int64_t>(1, count) * sizeof(T);
    if (cudaMalloc(&p, bytes) != cudaSuccess) return NWCCH_ERR_NOMEM;
    t->allocations.push_back(p);
    t->device_bytes += bytes;
    *dst = static_cast<T*>(p);
    return NWCCH_OK;
}

template <class T>
int upload(nwcch_topology* t, const T* src, size_t count, T** dst) {
    void* p = nullptr;
    const size_t bytes = std::max<size_t>(1, count) * sizeof(T);
    if (cudaMalloc(&p, bytes) != cudaSuccess) return NWCCH_ERR_NOMEM;
    t->allocations.push_back(p);
    t->device_bytes += bytes;
    if (count && cudaMemcpy(p, src, count * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
        return NWCCH_ERR_CUDA;
    *dst = static_cast<T*>(p);
    return NWCCH_OK;
}

void release(nwcch_topology* t) {
    if (t->free_plans) t->free_plans(t);
    if (t->free_battery_plan) t->free_battery_plan(t);
    if (t->free_query_plans) t->free_query_plans(t);
    free_supernodal_plan(static_cast<SnPlan*>(t->sn_plan));
    t->sn_plan = nullptr;
    for (void* p : t->allocations) cudaFree(p);
    t->allocations.clear();
}

}  // namespace

// aedir[j] = aeidx[j] with the sign bit set when the original arc goes up.
__global__ void k_arc_dir(int64_t count, const int32_t* __restrict__ aeidx, const int8_t* __restrict__ e_up,
                          int32_t* __restrict__ dir) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count; j += (int64_t)gridDim.x * blockDim.x) {
        const int32_t k = aeidx[j];
        dir[j] = e_up[k] ? (int32_t)((uint32_t)k | 0x80000000u) : k;
    }
}

// Allocates and zeroes one more block of kStreamSlots slots (caller holds
// t->slot_mu).
static int add_slot_block(nwcch_topology* t) {
    void* p = nullptr;
    const size_t bytes = (size_t)kStreamSlots * kSlotBytes;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return NWCCH_ERR_NOMEM;
    if (cudaMemset(p, 0, bytes) != cudaSuccess || setup_copies_done() != cudaSuccess) {
        cudaFree(p);
        return NWCCH_ERR_CUDA;
    }
    t->allocations.push_back(p);
    t->device_bytes += bytes;
    char* base = static_cast<char*>(p);
    for (int i = 0; i < kStreamSlots; i++) {
        StreamSlot slot;
        slot.err = reinterpret_cast<int*>(base + (size_t)i * kSlotBytes);
        slot.counters = slot_counters_of(slot.err);
        t->slots.push_back(slot);
    }
    return NWCCH_OK;
}

StreamSlot stream_slot(nwcch_topology* t, cudaStream_t stream) {
    std::lock_guard<std::mutex> lock(t->slot_mu);
    const size_t used = t->slot_stream.size();
    for (size_t i = 0; i < used; i++)
        if (t->slot_stream[i] == stream) return t->slots[i];
    if (used < t->slots.size() || add_slot_block(t) == NWCCH_OK) {
        t->slot_stream.push_back(stream);
        return t->slots[used];
    }
    return t->slots.back();
}

int consume_error(nwcch_topology* t, cudaStream_t stream) {
    const StreamSlot slot = stream_slot(t, stream);
    int h = 0;
    NWCCH_CUDA_TRY(cudaMemcpyAsync(&h, slot.err, sizeof(int), cudaMemcpyDeviceToHost, stream));
    NWCCH_CUDA_TRY(cudaStreamSynchronize(stream));
    if (h) NWCCH_CUDA_TRY(cudaMemsetAsync(slot.err, 0, sizeof(int), stream));
    if (h & ERR_TIMEOUT) return NWCCH_ERR_TIMEOUT;
    if (h & ERR_CAPACITY) return NWCCH_ERR_CAPACITY;
    if (h & ERR_TOPOLOGY) return NWCCH_ERR_TOPOLOGY;
    if (h & ERR_ARG) return NWCCH_ERR_ARG;
    if (h & ERR_RANGE) return NWCCH_SATURATED;
    return NWCCH_OK;
}

}  // namespace nwcch

using namespace nwcch;

extern "C" int nwcch_topology_create(int64_t n, const int64_t* first, const int32_t* head,
                                     const int32_t* parent, int64_t m, const int64_t* e_arc,
                                     const int8_t* e_up, nwcch_topology** out) {
    if (!out || n < 1 || n > INT32_MAX || !first || !parent || m < 0 || (m > 0 && (!e_arc || !e_up)))
        return NWCCH_ERR_ARG;
    *out = nullptr;
    const int64_t mp = first[n];
    if (first[0] != 0 || mp < 0 || mp >= INT32_MAX || (mp > 0 && !head) || m >= INT32_MAX)
        return NWCCH_ERR_TOPOLOGY;
    // row offsets ascend (the device checks every row: heads strictly
    // increasing above the tail, parent = lowest head, arc map in range)
    for (int64_t x = 0; x < n; x++)
        if (first[x + 1] < first[x]) return NWCCH_ERR_TOPOLOGY;

    int dev = 0, sms = 0;
    NWCCH_CUDA_TRY(cudaGetDevice(&dev));
    NWCCH_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    auto* t = new (std::nothrow) nwcch_topology();
    if (!t) return NWCCH_ERR_NOMEM;
    t->sms = std::max(1, sms);
    t->tune.query_cta_max = 8 * (int64_t)t->sms;
    t->tune.query_cta_wide_max = t->sms;
    int rc = NWCCH_OK;
    do {
        DevTopo& d = t->d;
        d.n = n;
        d.m_plus = mp;
        d.m = m;
        int64_t* p64;
        int32_t* p32;
        int8_t* p8;
        // the inputs, then everything derived from them on the device
        if ((rc = upload(t, first, n + 1, &p64))) break;
        d.first = p64;
        if ((rc = upload(t, head, mp, &p32))) break;
        d.head = p32;
        if ((rc = upload(t, parent, n, &p32))) break;
        d.parent = p32;
        if ((rc = upload(t, e_arc, m, &p64))) break;
        d.e_arc = p64;
        if ((rc = upload(t, e_up, m, &p8))) break;
        d.e_up = p8;
        DerivedTopology D;
        if ((rc = alloc(t, mp, &D.tail)) || (rc = alloc(t, n, &D.depth)) || (rc = alloc(t, mp, &D.hdep)) ||
            (rc = alloc(t, n + 1, &D.doff)) || (rc = alloc(t, mp, &D.darc)) || (rc = alloc(t, n, &D.vlevel)) ||
            (rc = alloc(t, mp + 1, &D.aeoff)) || (rc = alloc(t, n, &D.level_verts)))
            break;
        rc = derive_topology(n, mp, m, d.first, d.head, d.parent, d.e_arc, &D);
        if (D.aeidx_sorted) {
            t->allocations.push_back(D.aeidx_sorted);
            t->device_bytes += (size_t)std::max<int64_t>(1, m) * sizeof(int32_t);
        }
        if (rc) break;
        d.tail = D.tail;
        d.depth = D.depth;
        d.hdep = D.hdep;
        d.doff = D.doff;
        d.darc = D.darc;
        d.vlevel = D.vlevel;
        d.aeoff = D.aeoff;
        d.aeidx = D.aeidx_sorted;
        {
            // the base values' gather: each mapped original arc with its direction
            const int64_t mapped = m - D.nloops;
            int32_t* dir = nullptr;
            if ((rc = alloc(t, std::max<int64_t>(1, mapped), &dir))) break;
            if (mapped > 0) {
                k_arc_dir<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>((mapped + 255) / 256, 4096)), 256>>>(
                    mapped, D.aeidx_sorted, d.e_up, dir);
                if (cudaGetLastError() != cudaSuccess) {
                    rc = NWCCH_ERR_CUDA;
                    break;
                }
            }
            d.aedir = dir;
        }
        d.max_depth = D.max_depth;
        t->loops = D.aeidx_sorted + (m - D.nloops);
        t->nloops = D.nloops;
        t->level_verts = D.level_verts;
        t->triangles = D.triangles;
        t->max_deg = D.max_deg;
        t->levels = D.levels;
        t->level_off = std::move(D.level_off);
        t->level_arc_off = std::move(D.level_arc_off);
        t->level_tri = std::move(D.level_tri);
        t->level_maxdeg = std::move(D.level_maxdeg);
        if ((rc = upload(t, t->level_arc_off.data(), t->level_arc_off.size(), &p64))) break;
        t->d_level_arc_off = p64;
        // the supernodal plan, from the caller's host arrays (validated above)
        t->sn_plan = build_supernodal_plan(n, first, head, parent, SnPlanParams{}, &rc);
        if (rc) break;
        t->device_bytes += static_cast<SnPlan*>(t->sn_plan)->bytes;
        // per-stream slots (layout in topology.h)
        if ((rc = add_slot_block(t))) break;
        if (setup_copies_done() != cudaSuccess) rc = NWCCH_ERR_CUDA;
    } while (false);
    if (rc != NWCCH_OK) {
        release(t);
        delete t;
        return rc;
    }
    *out = t;
    return NWCCH_OK;
}

extern "C" int nwcch_topology_destroy(nwcch_topology* t) {
    if (!t) return NWCCH_ERR_ARG;
    cudaDeviceSynchronize();
    release(t);
    delete t;
    return NWCCH_OK;
}

namespace {

// Rebuilds the supernodal plan with new schedule parameters from the device
// copy of the topology. Every call on the handle must have completed (the
// old plan's arrays and captured graphs may be in use until then).
int replan(nwcch_topology* t, const SnPlanParams& prm) {
    NWCCH_CUDA_TRY(cudaDeviceSynchronize());
    const int64_t n = t->d.n, mp = t->d.m_plus;
    std::vector<int64_t> first(n + 1);
    std::vector<int32_t> head(std::max<int64_t>(1, mp)), parent(std::max<int64_t>(1, n));
    NWCCH_CUDA_TRY(cudaMemcpy(first.data(), t->d.first, (n + 1) * 8, cudaMemcpyDeviceToHost));
    if (mp) NWCCH_CUDA_TRY(cudaMemcpy(head.data(), t->d.head, mp * 4, cudaMemcpyDeviceToHost));
    if (n) NWCCH_CUDA_TRY(cudaMemcpy(parent.data(), t->d.parent, n * 4, cudaMemcpyDeviceToHost));
    int rc = NWCCH_OK;
    SnPlan* P = build_supernodal_plan(n, first.data(), head.data(), parent.data(), prm, &rc);
    if (!P) return rc ? rc : NWCCH_ERR_NOMEM;
    if (t->free_query_plans) t->free_query_plans(t);  // built over the old plan's supernodes
    auto* old = static_cast<SnPlan*>(t->sn_plan);
    if (old) t->device_bytes -= old->bytes;
    free_supernodal_plan(old);
    t->sn_plan = P;
    t->device_bytes += P->bytes;
    return NWCCH_OK;
}

}  // namespace

extern "C" int nwcch_tune_set(nwcch_topology* t, int key, int64_t value) {
    if (!t) return NWCCH_ERR_ARG;
    switch (key) {
        case NWCCH_TUNE_SN_WARP_CAP:
        case NWCCH_TUNE_SN_WARP_MIN_COUNT:
        case NWCCH_TUNE_SN_CHAIN_MAX_ITEMS:
        case NWCCH_TUNE_SN_THREAD_CAP: {
            if (value < 0 || !t->sn_plan) return NWCCH_ERR_ARG;
            SnPlanParams prm = static_cast<SnPlan*>(t->sn_plan)->params;
            if (key == NWCCH_TUNE_SN_WARP_CAP) prm.warp_cap = (int32_t)std::min<int64_t>(value, SN_WARP_CAP);
            else if (key == NWCCH_TUNE_SN_WARP_MIN_COUNT) prm.warp_min_count = value;
            else if (key == NWCCH_TUNE_SN_THREAD_CAP) prm.thread_cap = (int32_t)std::min<int64_t>(value, SN_THREAD_CAP);
            else prm.chain_max_items = value;
            return replan(t, prm);
        }
        case NWCCH_TUNE_QUERY_DENSE_ROWS:
            if (value < 1 || value > 33) return NWCCH_ERR_ARG;
            t->tune.query_dense_rows = (int32_t)value;
            return NWCCH_OK;
        case NWCCH_TUNE_QUERY_SMEM_LABELS_MAX:
            if (value < 0) return NWCCH_ERR_ARG;
            t->tune.query_smem_labels_max = value;
            return NWCCH_OK;
        case NWCCH_TUNE_UPDATE_BUDGET_NS:
            if (value < 0) return NWCCH_ERR_ARG;
            t->tune.update_budget_ns = value;
            return NWCCH_OK;
        case NWCCH_TUNE_QUERY_OCCUPANCY:
            if (value < 1 || value > 3) return NWCCH_ERR_ARG;
            t->tune.query_occupancy = (int32_t)value;
            return NWCCH_OK;
        case NWCCH_TUNE_QUERY_CTA_MAX:
            if (value < 0) return NWCCH_ERR_ARG;
            t->tune.query_cta_max = value;
            return NWCCH_OK;
        case NWCCH_TUNE_PDL:
            if (value < 0 || value > 1) return NWCCH_ERR_ARG;
            t->tune.pdl = (int32_t)value;
            return NWCCH_OK;
        case NWCCH_TUNE_QUERY_CTA_WIDE_MAX:
            if (value < 0) return NWCCH_ERR_ARG;
            t->tune.query_cta_wide_max = value;
            return NWCCH_OK;
        case NWCCH_TUNE_QUERY_CTA_DENSE_ROWS:
            if (value < 1 || value > 33) return NWCCH_ERR_ARG;
            t->tune.query_cta_dense_rows = (int32_t)value;
            return NWCCH_OK;
        case NWCCH_TUNE_UPDATE_DENSE_MIN:
            if (value < 0) return NWCCH_ERR_ARG;
            t->tune.update_dense_min = value;
            return NWCCH_OK;
        case NWCCH_TUNE_UPDATE_SPIN_LIMIT:
            if (value < 1) return NWCCH_ERR_ARG;
            t->tune.update_spin_limit = value;
            return NWCCH_OK;
        case NWCCH_TUNE_QUERY_TOP_CHAINS:
            if (value < 0) return NWCCH_ERR_ARG;
            t->tune.query_top_chains = value;
            return NWCCH_OK;
        case NWCCH_TUNE_QUERY_STREAM_MAX:
            if (value < 0) return NWCCH_ERR_ARG;
            t->tune.query_stream_max = value;
            return NWCCH_OK;
        case NWCCH_TUNE_UPDATE_SMALL_ARCS:
            if (value < 0) return NWCCH_ERR_ARG;
            t->tune.update_small_arcs = value;
            return NWCCH_OK;
        case NWCCH_TUNE_UPDATE_SMALL_NS:
            if (value < 1) return NWCCH_ERR_ARG;
            t->tune.update_small_ns = value;
            return NWCCH_OK;
        case NWCCH_TUNE_QUERY_STREAM_RING_KB:
            if (value < 0 || value > 227) return NWCCH_ERR_ARG;
            t->tune.query_stream_ring_kb = value;
            return NWCCH_OK;
        case NWCCH_TUNE_TEST_BARRIER_EXTRA:
            if (value < 0 || value > 1024) return NWCCH_ERR_ARG;
            t->tune.test_barrier_extra = (int32_t)value;
            return NWCCH_OK;
        case NWCCH_TUNE_BATTERY_POOL:
            if (value < 0) return NWCCH_ERR_ARG;
            {
                std::lock_guard<std::mutex> lock(t->mu);  // read by battery customizations
                t->tune.battery_pool = value;
            }
            return NWCCH_OK;
        case NWCCH_TUNE_BATTERY_BUFFER:
            if (value < 64 || value > (1 << 22)) return NWCCH_ERR_ARG;
            {
                std::lock_guard<std::mutex> lock(t->mu);
                t->tune.battery_buffer = (int32_t)value;
            }
            return NWCCH_OK;
        default:
            return NWCCH_ERR_ARG;
    }
}

extern "C" int nwcch_tune_get(const nwcch_topology* t, int key, int64_t* value) {
    if (!t || !value) return NWCCH_ERR_ARG;
    switch (key) {
        case NWCCH_TUNE_QUERY_DENSE_ROWS: *value = t->tune.query_dense_rows; return NWCCH_OK;
        case NWCCH_TUNE_QUERY_SMEM_LABELS_MAX: *value = t->tune.query_smem_labels_max; return NWCCH_OK;
        case NWCCH_TUNE_UPDATE_BUDGET_NS: *value = t->tune.update_budget_ns; return NWCCH_OK;
        case NWCCH_TUNE_QUERY_OCCUPANCY: *value = t->tune.query_occupancy; return NWCCH_OK;
        case NWCCH_TUNE_QUERY_CTA_MAX: *value = t->tune.query_cta_max; return NWCCH_OK;
        case NWCCH_TUNE_PDL: *value = t->tune.pdl; return NWCCH_OK;
        case NWCCH_TUNE_QUERY_CTA_WIDE_MAX: *value = t->tune.query_cta_wide_max; return NWCCH_OK;
        case NWCCH_TUNE_QUERY_CTA_DENSE_ROWS: *value = t->tune.query_cta_dense_rows; return NWCCH_OK;
        case NWCCH_TUNE_UPDATE_DENSE_MIN: *value = t->tune.update_dense_min; return NWCCH_OK;
        case NWCCH_TUNE_UPDATE_SPIN_LIMIT: *value = t->tune.update_spin_limit; return NWCCH_OK;
        case NWCCH_TUNE_TEST_BARRIER_EXTRA: *value = t->tune.test_barrier_extra; return NWCCH_OK;
        case NWCCH_TUNE_QUERY_TOP_CHAINS: *value = t->tune.query_top_chains; return NWCCH_OK;
        case NWCCH_TUNE_QUERY_STREAM_MAX: *value = t->tune.query_stream_max; return NWCCH_OK;
        case NWCCH_TUNE_UPDATE_SMALL_ARCS: *value = t->tune.update_small_arcs; return NWCCH_OK;
        case NWCCH_TUNE_UPDATE_SMALL_NS: *value = t->tune.update_small_ns; return NWCCH_OK;
        case NWCCH_TUNE_QUERY_STREAM_RING_KB: *value = t->tune.query_stream_ring_kb; return NWCCH_OK;
        case NWCCH_TUNE_BATTERY_POOL: *value = t->tune.battery_pool; return NWCCH_OK;
        case NWCCH_TUNE_BATTERY_BUFFER: *value = t->tune.battery_buffer; return NWCCH_OK;
        case NWCCH_TUNE_SN_WARP_CAP:
        case NWCCH_TUNE_SN_WARP_MIN_COUNT:
        case NWCCH_TUNE_SN_CHAIN_MAX_ITEMS:
        case NWCCH_TUNE_SN_THREAD_CAP: {
            if (!t->sn_plan) return NWCCH_ERR_ARG;
            const SnPlanParams& prm = static_cast<const SnPlan*>(t->sn_plan)->params;
            *value = key == NWCCH_TUNE_SN_WARP_CAP          ? prm.warp_cap
                     : key == NWCCH_TUNE_SN_WARP_MIN_COUNT ? prm.warp_min_count
                     : key == NWCCH_TUNE_SN_THREAD_CAP     ? prm.thread_cap
                                                           : prm.chain_max_items;
            return NWCCH_OK;
        }
        default: return NWCCH_ERR_ARG;
    }
}

extern "C" int nwcch_topology_info(const nwcch_topology* t, int64_t* info, int64_t len) {
    if (!t || !info || len < 8) return NWCCH_ERR_ARG;
    info[0] = t->d.n;
    info[1] = t->d.m_plus;
    info[2] = t->d.m;
    info[3] = t->triangles;
    info[4] = t->levels;
    info[5] = t->d.max_depth;
    info[6] = t->max_deg;
    info[7] = (int64_t)t->device_bytes;
    if (len >= 12) {
        const auto* p = static_cast<const SnPlan*>(t->sn_plan);
        info[8] = p ? p->nsn : 0;
        info[9] = p ? p->levels : 0;
        info[10] = p ? (int64_t)p->launches.size() : 0;
        info[11] = p ? p->rel_entries : 0;
    }
    if (len >= 15) {
        const auto* p = static_cast<const SnPlan*>(t->sn_plan);
        info[12] = p ? p->chain_level : 0;      // lowest level of the persistent launch (= levels: none)
        info[13] = p ? p->nchain_phases : 0;    // its phases
        info[14] = p ? (int64_t)p->chain_from : 0;  // launches before it (int32 storage)
    }
    if (len >= 16) info[15] = t->last_query_launches.load();  // kernels of the latest batched-query call
    return NWCCH_OK;
}

extern "C" int nwcch_topology_export(const nwcch_topology* t, int which, void* dst, int64_t count) {
    if (!t || !dst || count < 0) return NWCCH_ERR_ARG;
    const DevTopo& d = t->d;
    const int64_t mp = d.m_plus, n = d.n;
    const void* src = nullptr;
    int64_t len = 0;
    size_t elem = 4;
    const void* host = nullptr;
    switch (which) {
        case NWCCH_ARRAY_TAIL: src = d.tail; len = mp; break;
        case NWCCH_ARRAY_DEPTH: src = d.depth; len = n; break;
        case NWCCH_ARRAY_HDEP: src = d.hdep; len = mp; break;
        case NWCCH_ARRAY_DOFF: src = d.doff; len = n + 1; elem = 8; break;
        case NWCCH_ARRAY_DARC: src = d.darc; len = mp; break;
        case NWCCH_ARRAY_LEVEL: src = d.vlevel; len = n; break;
        case NWCCH_ARRAY_AEOFF: src = d.aeoff; len = mp + 1; elem = 8; break;
        case NWCCH_ARRAY_AEIDX: src = d.aeidx; len = d.m - t->nloops; break;
        case NWCCH_ARRAY_LEVEL_VERTS: src = t->level_verts; len = n; break;
        case NWCCH_ARRAY_LOOPS: src = t->loops; len = t->nloops; break;
        case NWCCH_ARRAY_LEVEL_OFF: host = t->level_off.data(); len = (int64_t)t->level_off.size(); elem = 8; break;
        case NWCCH_ARRAY_LEVEL_ARCS:
            host = t->level_arc_off.data(); len = (int64_t)t->level_arc_off.size(); elem = 8; break;
        case NWCCH_ARRAY_LEVEL_TRI: host = t->level_tri.data(); len = (int64_t)t->level_tri.size(); elem = 8; break;
        case NWCCH_ARRAY_LEVEL_MAXDEG: host = t->level_maxdeg.data(); len = (int64_t)t->level_maxdeg.size(); break;
        default: return NWCCH_ERR_ARG;
    }
    if (count != len) return NWCCH_ERR_ARG;
    if (len == 0) return NWCCH_OK;
    if (host) {
        std::memcpy(dst, host, (size_t)len * elem);
        return NWCCH_OK;
    }
    NWCCH_CUDA_TRY(cudaMemcpy(dst, src, (size_t)len * elem, cudaMemcpyDeviceToHost));
    return NWCCH_OK;
}
