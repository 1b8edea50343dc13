// Topology handle: validates the upward CSR produced by the host-side
// preprocessing, derives the structures the kernels need (tails, levels,
// elimination-tree depths, downward lists, arc -> original-arc index) and
// uploads everything once. Customization, scans, updates and queries for any
// number of metrics then run against this resident copy.

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "common.cuh"
#include "supernodal.h"
#include "topology.h"

namespace nwcch {

namespace {

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

StreamSlot stream_slot(nwcch_topology* t, cudaStream_t stream) {
    std::lock_guard<std::mutex> lock(t->slot_mu);
    const size_t used = t->slot_stream.size();
    for (size_t i = 0; i < used; i++)
        if (t->slot_stream[i] == stream) return t->slots[i];
    if (used < t->slots.size()) {
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
    // rows: strictly increasing heads above the tail; parent = lowest head
    for (int64_t x = 0; x < n; x++) {
        if (first[x + 1] < first[x]) return NWCCH_ERR_TOPOLOGY;
        int64_t prev = x;
        for (int64_t a = first[x]; a < first[x + 1]; a++) {
            if (head[a] <= prev || head[a] >= n) return NWCCH_ERR_TOPOLOGY;
            prev = head[a];
        }
        const int32_t p = first[x + 1] > first[x] ? head[first[x]] : -1;
        if (parent[x] != p) return NWCCH_ERR_TOPOLOGY;
    }
    for (int64_t k = 0; k < m; k++)
        if (e_arc[k] < -1 || e_arc[k] >= mp) return NWCCH_ERR_TOPOLOGY;

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
        std::vector<int32_t> tail(mp), depth(n, 0), hdep(mp), lvl(n, 0);
        int64_t tri = 0;
        int32_t maxdeg = 0;
        for (int64_t x = 0; x < n; x++) {
            const int64_t d = first[x + 1] - first[x];
            tri += d * (d - 1) / 2;
            maxdeg = std::max<int32_t>(maxdeg, (int32_t)d);
            for (int64_t a = first[x]; a < first[x + 1]; a++) {
                tail[a] = (int32_t)x;
                lvl[head[a]] = std::max(lvl[head[a]], lvl[x] + 1);
            }
        }
        int32_t maxd = 0;
        for (int64_t x = n - 1; x >= 0; x--)
            if (parent[x] >= 0) {
                depth[x] = depth[parent[x]] + 1;
                maxd = std::max(maxd, depth[x]);
            }
        for (int64_t a = 0; a < mp; a++) hdep[a] = depth[head[a]];
        // downward lists, ascending in the tail (arc ids grow with the tail)
        std::vector<int64_t> doff(n + 1, 0);
        for (int64_t a = 0; a < mp; a++) doff[head[a] + 1]++;
        for (int64_t v = 0; v < n; v++) doff[v + 1] += doff[v];
        std::vector<int32_t> darc(mp);
        {
            std::vector<int64_t> fill(doff.begin(), doff.end() - 1);
            for (int64_t a = 0; a < mp; a++) darc[fill[head[a]]++] = (int32_t)a;
        }
        // levels: vertices bucketed by level, stable in rank
        int32_t L = 0;
        for (int64_t x = 0; x < n; x++) L = std::max(L, lvl[x] + 1);
        t->levels = L;
        t->level_off.assign(L + 1, 0);
        for (int64_t x = 0; x < n; x++) t->level_off[lvl[x] + 1]++;
        for (int32_t l = 0; l < L; l++) t->level_off[l + 1] += t->level_off[l];
        std::vector<int32_t> lverts(n);
        t->level_maxdeg.assign(L, 0);
        t->level_tri.assign(L, 0);
        t->level_arc_off.assign(L + 1, 0);
        {
            std::vector<int64_t> fill(t->level_off.begin(), t->level_off.end() - 1);
            for (int64_t x = 0; x < n; x++) {
                const int32_t l = lvl[x];
                lverts[fill[l]++] = (int32_t)x;
                t->level_maxdeg[l] = std::max<int32_t>(t->level_maxdeg[l], (int32_t)(first[x + 1] - first[x]));
                t->level_arc_off[l + 1] += first[x + 1] - first[x];
            }
        }
        for (int32_t l = 0; l < L; l++) t->level_arc_off[l + 1] += t->level_arc_off[l];
        for (int64_t a = 0; a < mp; a++) {
            const int64_t x = tail[a];
            t->level_tri[lvl[head[a]]] += first[x + 1] - a - 1;  // pull work lands on the head's level
        }
        // original arcs mapped onto each shortcut arc, and the self-loops
        std::vector<int64_t> aeoff(mp + 1, 0);
        std::vector<int32_t> loops;
        for (int64_t k = 0; k < m; k++) {
            if (e_arc[k] >= 0) aeoff[e_arc[k] + 1]++;
            else loops.push_back((int32_t)k);
        }
        for (int64_t a = 0; a < mp; a++) aeoff[a + 1] += aeoff[a];
        std::vector<int32_t> aeidx(aeoff[mp]);
        {
            std::vector<int64_t> fill(aeoff.begin(), aeoff.end() - 1);
            for (int64_t k = 0; k < m; k++)
                if (e_arc[k] >= 0) aeidx[fill[e_arc[k]]++] = (int32_t)k;
        }
        t->sn_plan = build_supernodal_plan(n, first, head, parent, SnPlanParams{}, &rc);
        if (rc) break;
        t->device_bytes += static_cast<SnPlan*>(t->sn_plan)->bytes;
        t->triangles = tri;
        t->max_deg = maxdeg;
        t->nloops = (int64_t)loops.size();
        DevTopo& d = t->d;
        d.n = n;
        d.m_plus = mp;
        d.m = m;
        d.max_depth = maxd;
        int64_t* p64;
        int32_t* p32;
        int8_t* p8;
        if ((rc = upload(t, first, n + 1, &p64))) break;
        d.first = p64;
        if ((rc = upload(t, head, mp, &p32))) break;
        d.head = p32;
        if ((rc = upload(t, parent, n, &p32))) break;
        d.parent = p32;
        if ((rc = upload(t, depth.data(), n, &p32))) break;
        d.depth = p32;
        if ((rc = upload(t, hdep.data(), mp, &p32))) break;
        d.hdep = p32;
        if ((rc = upload(t, tail.data(), mp, &p32))) break;
        d.tail = p32;
        if ((rc = upload(t, doff.data(), n + 1, &p64))) break;
        d.doff = p64;
        if ((rc = upload(t, darc.data(), mp, &p32))) break;
        d.darc = p32;
        if ((rc = upload(t, lvl.data(), n, &p32))) break;
        d.vlevel = p32;
        if ((rc = upload(t, e_arc, m, &p64))) break;
        d.e_arc = p64;
        if ((rc = upload(t, e_up, m, &p8))) break;
        d.e_up = p8;
        if ((rc = upload(t, aeoff.data(), mp + 1, &p64))) break;
        d.aeoff = p64;
        if ((rc = upload(t, aeidx.data(), aeidx.size(), &p32))) break;
        d.aeidx = p32;
        if ((rc = upload(t, loops.data(), loops.size(), &p32))) break;
        t->loops = p32;
        if ((rc = upload(t, lverts.data(), n, &p32))) break;
        t->level_verts = p32;
        if ((rc = upload(t, t->level_arc_off.data(), t->level_arc_off.size(), &p64))) break;
        t->d_level_arc_off = p64;
        // per-stream slots: 256 bytes each, the error word first and the
        // 16 counters from byte 128
        const std::vector<int64_t> zeros((size_t)kStreamSlots * 32, 0);
        if ((rc = upload(t, zeros.data(), zeros.size(), &p64))) break;
        for (int i = 0; i < kStreamSlots; i++) {
            StreamSlot slot;
            slot.err = reinterpret_cast<int*>(p64 + 32 * i);
            slot.counters = reinterpret_cast<unsigned long long*>(p64 + 32 * i + 16);
            t->slots.push_back(slot);
        }
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
        case NWCCH_TUNE_SN_WARP_MIN_COUNT: {
            if (value < 0 || !t->sn_plan) return NWCCH_ERR_ARG;
            SnPlanParams prm = static_cast<SnPlan*>(t->sn_plan)->params;
            if (key == NWCCH_TUNE_SN_WARP_CAP) prm.warp_cap = (int32_t)std::min<int64_t>(value, SN_WARP_CAP);
            else prm.warp_min_count = value;
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
        case NWCCH_TUNE_BATTERY_POOL: *value = t->tune.battery_pool; return NWCCH_OK;
        case NWCCH_TUNE_BATTERY_BUFFER: *value = t->tune.battery_buffer; return NWCCH_OK;
        case NWCCH_TUNE_SN_WARP_CAP:
        case NWCCH_TUNE_SN_WARP_MIN_COUNT: {
            if (!t->sn_plan) return NWCCH_ERR_ARG;
            const SnPlanParams& prm = static_cast<const SnPlan*>(t->sn_plan)->params;
            *value = key == NWCCH_TUNE_SN_WARP_CAP ? prm.warp_cap : prm.warp_min_count;
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
    return NWCCH_OK;
}
