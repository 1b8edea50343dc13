// Supernodal customization.
//
// The lower-triangle recurrence of python/cch_nb.py:529-563 is regrouped by
// supernodes (maximal rank runs with nested rows, see supernodal.h). Every
// lower triangle (x; y, z) has its lowest vertex x in exactly one supernode S;
// it is either
//   internal - y in S as well: the (min,+) elimination of S's own dense
//              trapezoid, row by row;
//   outgoing - y, z in the boundary B of S: the (min,+) product
//              Dn(S, B)^T (x) U(S, B), scattered (atomic minimum) into the
//              arcs (y, z) of S's ancestors.
// Supernodes of one level of the supernode tree are independent; a level's
// internal work precedes its outgoing work, and all supernodes below it are
// done first. Integer minima are order independent, so the result equals the
// reference's serial loop bit for bit.
//
// Kernels per level:
//   k_sn_warp       small supernodes (k <= 32, b <= 64, trapezoid within a
//                   tuned cap, in levels with many of them): one warp does
//                   the whole supernode, internal and outgoing, from shared
//                   memory;
//   k_sn_panel      other supernodes, one 32-row panel: every CTA factors the
//                   panel's 32x32 diagonal triangle in shared memory, then
//                   each thread runs the panel recurrence down one column in
//                   registers (columns are independent given that triangle);
//   k_sn_tile       (min,+) tile product, for the trailing update of a panel
//                   (plain min into the supernode's own arcs) and for the
//                   outgoing block (atomic min into ancestor arcs).

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <new>
#include <thread>
#include <vector>

#include "common.cuh"
#include "customize.h"
#include "supernodal.h"
#include "topology.h"

namespace nwcch {

constexpr int SN_P = 32;          // panel height
constexpr int SN_SMALL_K = 1;     // every supernode with k >= 2 runs the panel kernel
constexpr int PANEL_THREADS = 128;

// ------------------------------------------------------------------ plan

namespace {

template <class X>
int upload_vec(SnPlan* p, const std::vector<X>& v, X** out) {
    void* d = nullptr;
    const size_t bytes = std::max<size_t>(1, v.size()) * sizeof(X);
    if (cudaMalloc(&d, bytes) != cudaSuccess) return NWCCH_ERR_NOMEM;
    p->allocations.push_back(d);
    p->bytes += bytes;
    if (!v.empty() && cudaMemcpy(d, v.data(), v.size() * sizeof(X), cudaMemcpyHostToDevice) != cudaSuccess)
        return NWCCH_ERR_CUDA;
    *out = static_cast<X*>(d);
    return NWCCH_OK;
}

int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace

void free_supernodal_plan(SnPlan* p) {
    if (!p) return;
    for (auto& g : p->graphs) cudaGraphExecDestroy(g.exec);
    for (void* a : p->allocations) cudaFree(a);
    delete p;
}

SnPlan* build_supernodal_plan(int64_t n, const int64_t* first, const int32_t* head, const int32_t* parent,
                              const SnPlanParams& prm, int* rc) {
    *rc = NWCCH_OK;
    auto* P = new (std::nothrow) SnPlan();
    if (!P) {
        *rc = NWCCH_ERR_NOMEM;
        return nullptr;
    }
    // supernodes: x joins x+1 when x+1 is its parent and the rows are nested
    std::vector<int32_t> s0v, kv, bv, sid(n);
    for (int64_t x = 0; x < n; x++) {
        const bool joins_prev = x > 0 && parent[x - 1] == x &&
                                (first[x] - first[x - 1]) == (first[x + 1] - first[x]) + 1;
        if (!joins_prev) {
            s0v.push_back((int32_t)x);
            kv.push_back(0);
        }
        kv.back()++;
        sid[x] = (int32_t)s0v.size() - 1;
    }
    const int64_t ns = (int64_t)s0v.size();
    bv.resize(ns);
    std::vector<int32_t> lvl(ns, 0);
    int32_t L = 0;
    for (int64_t s = 0; s < ns; s++) {
        const int64_t last = s0v[s] + kv[s] - 1;
        bv[s] = (int32_t)(first[last + 1] - first[last]);
        const int32_t p = parent[last];
        if (p >= 0) lvl[sid[p]] = std::max(lvl[sid[p]], lvl[s] + 1);
        L = std::max(L, lvl[s] + 1);
    }
    P->nsn = ns;
    P->levels = L;
    for (int64_t s = 0; s < ns; s++) P->max_b = std::max(P->max_b, bv[s]);
    // arc ids of (B[p], B[q]) for every supernode, found by merging B's tail
    // into the row of B[p] (chordality puts it there)
    std::vector<int64_t> rel_off(ns + 1, 0);
    for (int64_t s = 0; s < ns; s++) rel_off[s + 1] = rel_off[s] + (int64_t)bv[s] * (bv[s] - 1) / 2;
    std::vector<int32_t> rel(rel_off[ns]);
    {
        std::atomic<int> bad{0};
        const int nth = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> ts;
        for (int th = 0; th < nth; th++)
            ts.emplace_back([&, th] {
                for (int64_t s = th; s < ns; s += nth) {
                    const int32_t b = bv[s];
                    if (b < 2) continue;
                    const int64_t last = s0v[s] + kv[s] - 1;
                    const int32_t* B = head + first[last];
                    int64_t o = rel_off[s];
                    for (int32_t p = 0; p + 1 < b; p++) {
                        const int32_t y = B[p];
                        int64_t pos = first[y];
                        const int64_t end = first[y + 1];
                        for (int32_t q = p + 1; q < b; q++) {
                            while (pos < end && head[pos] < B[q]) pos++;
                            if (pos >= end || head[pos] != B[q]) {
                                bad = 1;
                                return;
                            }
                            rel[o++] = (int32_t)pos;
                        }
                    }
                }
            });
        for (auto& t : ts) t.join();
        if (bad) {
            *rc = NWCCH_ERR_TOPOLOGY;
            delete P;
            return nullptr;
        }
    }
    P->rel_entries = rel_off[ns];
    // the chain walk of the streaming query kernel
    std::vector<QsNode> qnodes(ns);
    for (int64_t s = 0; s < ns; s++) {
        const int32_t pv = parent[s0v[s] + kv[s] - 1];
        const int32_t nx = pv >= 0 ? sid[pv] : -1;
        qnodes[s] = QsNode{s0v[s], kv[s], bv[s], nx, nx >= 0 ? pv - s0v[nx] : 0, 0, first[s0v[s]]};
    }
    // work items per level
    P->params = prm;
    const int64_t cap = std::min<int64_t>(prm.warp_cap, SN_WARP_CAP);
    auto warp_ok = [&](int64_t s) { return kv[s] <= 32 && bv[s] <= 64 && sn_trapezoid(kv[s], bv[s]) <= cap; };
    std::vector<int64_t> warp_count(L, 0);
    for (int64_t s = 0; s < ns; s++)
        if (warp_ok(s)) warp_count[lvl[s]]++;
    const int64_t tcap = std::min<int64_t>(prm.thread_cap, SN_THREAD_CAP);
    std::vector<std::vector<int32_t>> small(L), big(L), out_small(L), out_big(L), warp(L), thread(L);
    for (int64_t s = 0; s < ns; s++) {
        const int32_t l = lvl[s];
        if (kv[s] == 1 && bv[s] < 2) continue;  // no triangle has its lowest vertex here
        if (warp_ok(s) && warp_count[l] >= prm.warp_min_count) {
            if (sn_trapezoid(kv[s], bv[s]) <= tcap) thread[l].insert(thread[l].end(), {(int32_t)s, 0, 0});
            else warp[l].insert(warp[l].end(), {(int32_t)s, 0, 0});
            continue;
        }
        if (kv[s] >= 2 && kv[s] <= SN_SMALL_K) small[l].push_back((int32_t)s);
        if (kv[s] > SN_SMALL_K) big[l].push_back((int32_t)s);
        const int32_t b = bv[s];
        if (b >= 2) {
            if (b > 32) {
                const int64_t nt = ceil_div(b, 64);
                for (int64_t tp = 0; tp < nt; tp++)
                    for (int64_t tq = tp; tq < nt; tq++) {
                        out_big[l].push_back((int32_t)s);
                        out_big[l].push_back((int32_t)tp);
                        out_big[l].push_back((int32_t)tq);
                    }
            } else {
                const int64_t nt = ceil_div(b, 16);
                for (int64_t tp = 0; tp < nt; tp++)
                    for (int64_t tq = tp; tq < nt; tq++) {
                        out_small[l].push_back((int32_t)s);
                        out_small[l].push_back((int32_t)tp);
                        out_small[l].push_back((int32_t)tq);
                    }
            }
        }
    }
    std::vector<int32_t> items;
    auto add = [&](int kind, int level, int panel, const std::vector<int32_t>& v) {
        if (v.empty()) return;
        SnLaunch la{kind, level, panel, (int64_t)items.size() / 3, (int64_t)v.size() / 3};
        items.insert(items.end(), v.begin(), v.end());
        P->launches.push_back(la);
    };
    for (int32_t l = 0; l < L; l++) {
        add(SN_THREAD, l, 0, thread[l]);
        add(SN_WARP, l, 0, warp[l]);
        std::vector<int32_t> v;
        for (int32_t s : small[l]) v.insert(v.end(), {s, 0, 0});
        add(SN_INT_SMALL, l, 0, v);
        int32_t maxp = 0;
        for (int32_t s : big[l]) maxp = std::max<int32_t>(maxp, (int32_t)ceil_div(kv[s], SN_P));
        for (int32_t pi = 0; pi < maxp; pi++) {
            std::vector<int32_t> pv, tv;
            for (int32_t s : big[l]) {
                const int64_t k = kv[s], b = bv[s];
                const int64_t i0 = (int64_t)pi * SN_P;
                if (i0 >= k) continue;
                const int64_t pn = std::min<int64_t>(SN_P, k - i0);
                const int64_t ncols = (k + b) - (i0 + pn);
                const int64_t ct = std::max<int64_t>(1, ceil_div(ncols, PANEL_THREADS));
                for (int64_t c = 0; c < ct; c++) pv.insert(pv.end(), {s, (int32_t)c, 0});
                const int64_t nrows = k - i0 - pn;
                if (nrows > 0) {
                    const int64_t tr_n = ceil_div(nrows, 64), tc_n = ceil_div(ncols, 64);
                    for (int64_t tr = 0; tr < tr_n; tr++)
                        for (int64_t tc = tr; tc < tc_n; tc++) tv.insert(tv.end(), {s, (int32_t)tr, (int32_t)tc});
                }
            }
            add(SN_PANEL, l, pi, pv);
            add(SN_TRAIL, l, pi, tv);
        }
        add(SN_OUT_SMALL, l, 0, out_small[l]);
        add(SN_OUT_BIG, l, 0, out_big[l]);
    }
    P->items = (int64_t)items.size() / 3;
    // the persistent top: from the lowest level such that it and every level
    // above it have no warp-kernel launch and no launch of more than
    // chain_max_items items, the levels run as phases of k_sn_chain (int32
    // storage): panels in CHAIN_THREADS-column items, trailing and outgoing
    // products in 64 x 64 tiles
    P->chain_level = L;
    if (prm.chain_max_items > 0) {
        std::vector<char> level_ok(L, 1);
        for (const SnLaunch& la : P->launches)
            if (la.kind == SN_WARP || la.kind == SN_THREAD || la.kind == SN_INT_SMALL || la.count > prm.chain_max_items)
                level_ok[la.level] = 0;
        while (P->chain_level > 0 && level_ok[P->chain_level - 1]) P->chain_level--;
    }
    P->chain_from = P->launches.size();
    for (size_t i = 0; i < P->launches.size(); i++)
        if (P->launches[i].level >= P->chain_level) {
            P->chain_from = i;
            break;
        }
    std::vector<int32_t> citems;
    std::vector<ChainPhase> phases;
    if (P->chain_from < P->launches.size()) {
        std::vector<std::vector<int32_t>> at(L - P->chain_level);  // supernodes of each chain level
        for (int64_t s = 0; s < ns; s++)
            if (lvl[s] >= P->chain_level) at[lvl[s] - P->chain_level].push_back((int32_t)s);
        auto phase = [&](int kind, int panel, const std::vector<int32_t>& v) {
            if (v.empty()) return;
            phases.push_back(ChainPhase{kind, panel, (int64_t)citems.size() / 3, (int64_t)v.size() / 3});
            citems.insert(citems.end(), v.begin(), v.end());
        };
        for (int32_t l = P->chain_level; l < L; l++) {
            const auto& ss = at[l - P->chain_level];
            int32_t maxp = 0;
            for (int32_t s : ss)
                if (kv[s] > SN_SMALL_K) maxp = std::max<int32_t>(maxp, (int32_t)ceil_div(kv[s], SN_P));
            for (int32_t pi = 0; pi < maxp; pi++) {
                std::vector<int32_t> pv, tv;
                for (int32_t s : ss) {
                    const int64_t k = kv[s], b = bv[s];
                    const int64_t i0 = (int64_t)pi * SN_P;
                    if (k <= SN_SMALL_K || i0 >= k) continue;
                    const int64_t pn = std::min<int64_t>(SN_P, k - i0);
                    const int64_t ncols = (k + b) - (i0 + pn);
                    const int64_t ct = std::max<int64_t>(1, ceil_div(ncols, CHAIN_THREADS));
                    for (int64_t c = 0; c < ct; c++) pv.insert(pv.end(), {s, (int32_t)c, 0});
                    const int64_t nrows = k - i0 - pn;
                    if (nrows > 0) {
                        const int64_t tr_n = ceil_div(nrows, 64), tc_n = ceil_div(ncols, 64);
                        for (int64_t tr = 0; tr < tr_n; tr++)
                            for (int64_t tc = tr; tc < tc_n; tc++) tv.insert(tv.end(), {s, (int32_t)tr, (int32_t)tc});
                    }
                }
                phase(SN_PANEL, pi, pv);
                phase(SN_TRAIL, pi, tv);
            }
            std::vector<int32_t> ov;
            for (int32_t s : ss) {
                if (bv[s] < 2) continue;
                const int64_t nt = ceil_div(bv[s], 64);
                for (int64_t tp = 0; tp < nt; tp++)
                    for (int64_t tq = tp; tq < nt; tq++) ov.insert(ov.end(), {s, (int32_t)tp, (int32_t)tq});
            }
            phase(SN_OUT_BIG, 0, ov);
        }
        P->nchain_phases = (int32_t)phases.size();
    }
    // supernodes by level: whole-CTA ones, then warp ones, then single
    // vertices (k = 1), which a thread each sweeps
    std::vector<int32_t> order;
    order.reserve(ns);
    P->sn_level_off.assign(L + 1, 0);
    P->sn_level_big.assign(L, 0);
    P->sn_level_single.assign(L, 0);
    {
        std::vector<std::vector<int32_t>> by_level(L);
        for (int64_t s = 0; s < ns; s++) by_level[lvl[s]].push_back((int32_t)s);
        for (int32_t l = 0; l < L; l++) {
            P->sn_level_off[l] = (int64_t)order.size();
            for (int32_t s : by_level[l])
                if (sn_sweep_big(kv[s], bv[s])) order.push_back(s);
            P->sn_level_big[l] = (int64_t)order.size() - P->sn_level_off[l];
            for (int32_t s : by_level[l])
                if (!sn_sweep_big(kv[s], bv[s]) && kv[s] > 1) order.push_back(s);
            P->sn_level_single[l] = (int64_t)order.size() - P->sn_level_off[l];
            for (int32_t s : by_level[l])
                if (!sn_sweep_big(kv[s], bv[s]) && kv[s] == 1) order.push_back(s);
        }
        P->sn_level_off[L] = (int64_t)order.size();
    }
    std::vector<int32_t> pot_bu, pot_bd;
    P->pot_bu_off.assign(L + 1, 0);
    P->pot_bd_off.assign(L + 1, 0);
    for (int32_t l = 0; l < L; l++) {
        P->pot_bu_off[l] = (int64_t)pot_bu.size() / 2;
        P->pot_bd_off[l] = (int64_t)pot_bd.size() / 2;
        for (int64_t i = P->sn_level_off[l]; i < P->sn_level_off[l] + P->sn_level_big[l]; i++) {
            const int32_t s = order[i];
            for (int64_t tile = 0; tile < ceil_div(bv[s], 256); tile++) pot_bu.insert(pot_bu.end(), {s, (int32_t)tile});
            for (int64_t tile = 0; tile < ceil_div(kv[s], 32); tile++) pot_bd.insert(pot_bd.end(), {s, (int32_t)tile});
        }
    }
    P->pot_bu_off[L] = (int64_t)pot_bu.size() / 2;
    P->pot_bd_off[L] = (int64_t)pot_bd.size() / 2;
    int32_t *d_s0, *d_k, *d_b, *d_rel, *d_sid;
    int64_t* d_rel_off;
    if ((*rc = upload_vec(P, s0v, &d_s0)) || (*rc = upload_vec(P, kv, &d_k)) || (*rc = upload_vec(P, bv, &d_b)) ||
        (*rc = upload_vec(P, rel_off, &d_rel_off)) || (*rc = upload_vec(P, rel, &d_rel)) ||
        (*rc = upload_vec(P, items, &P->d_items)) || (*rc = upload_vec(P, sid, &d_sid)) ||
        (*rc = upload_vec(P, order, &P->d_sn_order)) || (*rc = upload_vec(P, pot_bu, &P->d_pot_bu)) ||
        (*rc = upload_vec(P, pot_bd, &P->d_pot_bd)) || (*rc = upload_vec(P, citems, &P->d_chain_items)) ||
        (*rc = upload_vec(P, phases, &P->d_chain_phases)) || (*rc = upload_vec(P, qnodes, &P->d_qnodes))) {
        free_supernodal_plan(P);
        return nullptr;
    }
    P->dev = SnDev{P->d_qnodes, d_s0, d_k, d_b, d_rel_off, d_rel, d_sid};
    if (setup_copies_done() != cudaSuccess) {
        *rc = NWCCH_ERR_CUDA;
        free_supernodal_plan(P);
        return nullptr;
    }
    return P;
}


}  // namespace nwcch

#include "sn_kernels.cuh"

namespace nwcch {

// CTAs of the plan's persistent launch: one per SM if one fits (0: it cannot
// run, and its levels are launched one kernel at a time). Sized once per plan.
static int chain_grid(SnPlan* P) {
    std::lock_guard<std::mutex> lock(P->chain_mu);
    if (P->chain_grid >= 0) return P->chain_grid;
    P->chain_grid = 0;
    int dev = 0, coop = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop ||
        allow_dynamic_smem((const void*)k_sn_chain, chain_smem_bytes()) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sn_chain, CHAIN_THREADS, chain_smem_bytes()) !=
            cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    if (per_sm >= 1) P->chain_grid = device_sms();
    return P->chain_grid;
}

template <class T>
int run_supernodal(nwcch_topology* t, SnPlan* P, const int32_t* w, T* up, T* dn, cudaStream_t s, int* err,
                   int metrics) {
    int rc = base_init<T>(t, w, up, dn, s, err, metrics);
    if (rc) return rc;
    const DevTopo& D = t->d;
    constexpr int CT = sizeof(T) == 4 ? 128 : 32;
    const bool pdl = t->tune.pdl != 0;
    const bool chain = sizeof(T) == 4 && P->nchain_phases > 0 && chain_grid(P) > 0;
    const size_t end = chain ? P->chain_from : P->launches.size();
    for (size_t li = 0; li < end; li++) {
        const SnLaunch& la = P->launches[li];
        const int32_t* it = P->d_items + 3 * la.off;
        const dim3 grid((unsigned)la.count, metrics);
        cudaError_t e = cudaSuccess;
        switch (la.kind) {
            case SN_PANEL:
                e = launch_pdl(pdl, k_sn_panel<T, CT>, grid, dim3(CT), 0, s, D, P->dev, it, la.panel, up, dn, err);
                break;
            case SN_TRAIL:
                e = launch_pdl(pdl, k_sn_tile<T, 64, 4, false>, grid, dim3(256), 0, s, D, P->dev, it, la.panel, up, dn,
                               err);
                break;
            case SN_OUT_BIG:
                e = launch_pdl(pdl, k_sn_tile<T, 64, 4, true>, grid, dim3(256), 0, s, D, P->dev, it, 0, up, dn, err);
                break;
            case SN_OUT_SMALL:
                e = launch_pdl(pdl, k_sn_tile<T, 16, 2, true>, grid, dim3(64), 0, s, D, P->dev, it, 0, up, dn, err);
                break;
            case SN_THREAD: {
                constexpr int TT = sizeof(T) == 4 ? 128 : 64;  // 16 or 32 KB of staged arcs a block
                const int64_t blocks = std::min<int64_t>((la.count + TT - 1) / TT, (int64_t)device_sms() * 16);
                if (P->params.thread_cap <= 16)
                    e = launch_pdl(pdl, k_sn_thread<T, TT, 16>, dim3((unsigned)blocks, metrics), dim3(TT), 0, s, D,
                                   P->dev, it, la.count, up, dn, err);
                else
                    e = launch_pdl(pdl, k_sn_thread<T, TT, SN_THREAD_CAP>, dim3((unsigned)blocks, metrics), dim3(TT), 0,
                                   s, D, P->dev, it, la.count, up, dn, err);
                break;
            }
            case SN_WARP: {
                constexpr int WARPS = sizeof(T) == 4 ? 8 : 4;
                const int64_t blocks = std::min<int64_t>((la.count + WARPS - 1) / WARPS, (int64_t)device_sms() * 64);
                e = launch_pdl(pdl, k_sn_warp<T, WARPS>, dim3((unsigned)blocks, metrics), dim3(32 * WARPS), 0, s, D,
                               P->dev, it, la.count, up, dn, err);
                break;
            }
            default:
                return NWCCH_ERR_TOPOLOGY;
        }
        if (e != cudaSuccess) return NWCCH_ERR_CUDA;
    }
    if constexpr (sizeof(T) == 4) {
        if (chain) {
            // the barrier words start at zero; the launch is cooperative, so
            // its CTAs are co-resident and the barrier can complete
            unsigned int* bar = reinterpret_cast<unsigned int*>(slot_counters_of(err) + 8);
            NWCCH_CUDA_TRY(cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned int), s));
            cudaLaunchConfig_t cfg = {};
            cfg.gridDim = dim3((unsigned)P->chain_grid);
            cfg.blockDim = dim3(CHAIN_THREADS);
            cfg.dynamicSmemBytes = chain_smem_bytes();
            cfg.stream = s;
            cudaLaunchAttribute attr[1];
            attr[0].id = cudaLaunchAttributeCooperative;
            attr[0].val.cooperative = 1;
            cfg.attrs = attr;
            cfg.numAttrs = 1;
            NWCCH_CUDA_TRY(cudaLaunchKernelEx(&cfg, k_sn_chain, D, P->dev, (const int32_t*)P->d_chain_items,
                                              (const ChainPhase*)P->d_chain_phases, P->nchain_phases,
                                              reinterpret_cast<int32_t*>(up), reinterpret_cast<int32_t*>(dn), err,
                                              bar, (long long)t->tune.update_spin_limit,
                                              (int32_t)t->tune.test_barrier_extra, (int32_t)metrics));
        }
    }
    return cudaGetLastError() == cudaSuccess ? NWCCH_OK : NWCCH_ERR_CUDA;
}

int launch_cached(SnPlan* P, const SnGraph& key, cudaStream_t s, const std::function<int(cudaStream_t)>& enqueue) {
    static const bool no_graph = getenv("NWCCH_NO_GRAPH") != nullptr;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    NWCCH_CUDA_TRY(cudaStreamIsCapturing(s, &cap));
    if (no_graph || cap != cudaStreamCaptureStatusNone) return enqueue(s);
    std::lock_guard<std::mutex> lock(P->graph_mu);
    SnGraph* hit = nullptr;
    for (auto& g : P->graphs)
        if (g.kind == key.kind && g.storage == key.storage && g.metrics == key.metrics && g.err == key.err &&
            g.w == key.w && g.up == key.up && g.dn == key.dn && g.spin == key.spin && g.extra == key.extra)
            hit = &g;
    if (!hit) {
        cudaStream_t cs;
        NWCCH_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaGraph_t graph = nullptr;
        int rc = NWCCH_OK;
        if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = NWCCH_ERR_CUDA;
        if (!rc) rc = enqueue(cs);
        if (cudaStreamEndCapture(cs, &graph) != cudaSuccess && !rc) rc = NWCCH_ERR_CUDA;
        cudaGraphExec_t exec = nullptr;
        if (!rc && cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) rc = NWCCH_ERR_CUDA;
        if (graph) cudaGraphDestroy(graph);
        cudaStreamDestroy(cs);
        if (rc) return rc;
        if (P->graphs.size() >= 16) {
            auto old = std::min_element(P->graphs.begin(), P->graphs.end(),
                                        [](const SnGraph& a, const SnGraph& b) { return a.last_use < b.last_use; });
            cudaGraphExecDestroy(old->exec);
            P->graphs.erase(old);
        }
        SnGraph g = key;
        g.exec = exec;
        P->graphs.push_back(g);
        hit = &P->graphs.back();
    }
    hit->last_use = ++P->graph_clock;
    NWCCH_CUDA_TRY(cudaGraphLaunch(hit->exec, s));
    return NWCCH_OK;
}

template <class T>
int launch_supernodal(nwcch_topology* t, SnPlan* P, const int32_t* w, T* up, T* dn, cudaStream_t s, int metrics) {
    int* err = stream_slot(t, s).err;
    if (sizeof(T) == 4 && P->nchain_phases > 0) chain_grid(P);  // sized before any capture starts
    // the launch form (programmatic dependent launches or not) is part of the key
    SnGraph key{SN_GRAPH_CUSTOMIZE, (int)sizeof(T), metrics * 2 + (t->tune.pdl != 0), err, w, up, dn, nullptr, 0};
    key.spin = t->tune.update_spin_limit;  // the persistent launch's wait bound and test hook are baked in
    key.extra = t->tune.test_barrier_extra;
    return launch_cached(P, key, s, [&](cudaStream_t cs) { return run_supernodal<T>(t, P, w, up, dn, cs, err, metrics); });
}

template int launch_supernodal<int32_t>(nwcch_topology*, SnPlan*, const int32_t*, int32_t*, int32_t*, cudaStream_t, int);
template int launch_supernodal<int64_t>(nwcch_topology*, SnPlan*, const int32_t*, int64_t*, int64_t*, cudaStream_t, int);
template int run_supernodal<int32_t>(nwcch_topology*, SnPlan*, const int32_t*, int32_t*, int32_t*, cudaStream_t, int*,
                                     int);
template int run_supernodal<int64_t>(nwcch_topology*, SnPlan*, const int32_t*, int64_t*, int64_t*, cudaStream_t, int*,
                                     int);

}  // namespace nwcch
