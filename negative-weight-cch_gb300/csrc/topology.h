// Device-resident topology handle of libnwcch (internal layout).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <vector>

#include "nwcch.h"

namespace nwcch {

// Read-only views passed to kernels by value.
struct DevTopo {
    int64_t n, m_plus, m;
    int32_t max_depth;
    const int64_t* first;   // [n+1] upward CSR offsets (rank space)
    const int32_t* head;    // [m+]  upper endpoint of every arc, sorted per row
    const int32_t* parent;  // [n]   elimination-tree parent (-1 = root)
    const int32_t* depth;   // [n]   elimination-tree depth (root 0)
    const int32_t* hdep;    // [m+]  depth of head[a]
    const int32_t* tail;    // [m+]  lower endpoint of every arc
    const int64_t* doff;    // [n+1] downward lists: arcs (x,y) grouped by y ...
    const int32_t* darc;    // [m+]  ... ascending in x
    const int32_t* vlevel;  // [n]   level: 1 + max level of the lower neighbours
    const int64_t* e_arc;   // [m]   shortcut arc of every original arc (-1 = self-loop)
    const int8_t* e_up;     // [m]   1 if the original arc goes up in rank
    const int64_t* aeoff;   // [m+ + 1] original arcs mapped onto each shortcut arc ...
    const int32_t* aeidx;   // [...]     ... as original arc ids
    const int32_t* aedir;   // [...]     the same ids with the arc's direction in the sign bit (set: up)
};

// Schedules that depend on the graph and are picked by measurement
// (nwcch_tune_set; python nwcch.tune).
struct Tuning {
    int32_t query_dense_rows = 16;          // query chunks with fewer rows go row by row
    int64_t query_smem_labels_max = 8192;   // per-warp query labels above this go to global scratch
    int32_t query_occupancy = 1;            // 2: 32-bit query kernel capped at 64 registers
    int64_t query_cta_max = 0;              // batches up to this many queries: a CTA per query (8 per SM)
    int64_t query_cta_wide_max = 0;         // ... of 16 warps up to this many (one per SM), else of 8
    int64_t query_stream_max = 64;          // batches up to this many queries: the streaming kernel (a CTA a chain)
    int64_t query_stream_ring_kb = 0;       // its data ring (KB; 0: as large as fits, at most 192)
    int64_t update_small_arcs = 8192;       // updates sweep in one CTA until they evaluate this many arcs (0: never)
    int64_t update_small_ns = 300000;       // ... or until they have run this long (ns)
    int32_t query_cta_dense_rows = 1;       // the CTA form's row-by-row threshold
    int32_t pdl = 0;                        // customization kernels as programmatic dependent launches
    int64_t update_budget_ns = 0;           // level-sweep budget of an update (0: from the triangle count)
    int64_t update_dense_min = 0;           // updates of at least this many arcs skip the sweep (0: never)
    int64_t update_spin_limit = 1 << 24;    // spins (about 100 ns each) of one update barrier wait
    int32_t test_barrier_extra = 0;         // test hook: barrier waits for this many extra blocks
    int64_t query_top_chains = 64;          // batched queries: top supernodes = those crossed by about this
                                            // many chains of a batch (0: per-query kernels only)
    int64_t battery_pool = 0;               // initial battery piece pool (0: 1.5 pieces a direction)
    int32_t battery_buffer = 512;           // initial per-warp buffer of a long battery profile (pieces)
};

// Device words private to the calls enqueued on one stream: the error word
// and 16 scratch counters (scan results, query range flags). Calls on
// different streams of one handle never share them, so they may overlap.
struct StreamSlot {
    int* err = nullptr;
    unsigned long long* counters = nullptr;
};

// Layout of a slot (256 bytes): the error word at byte 0, the counters from
// byte 128. Counters: [0] and [1] scan results, [3] the query range flag,
// [8] the two 32-bit words (arrivals, generation) of the persistent
// customization launch's grid barrier.
constexpr int kSlotBytes = 256;
constexpr int kSlotCounterOffset = 128;
inline unsigned long long* slot_counters_of(int* err) {
    return reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(err) + kSlotCounterOffset);
}

}  // namespace nwcch

struct nwcch_topology {
    nwcch::DevTopo d{};
    int32_t sms = 0;                          // SMs of the device the handle was created on
    int64_t triangles = 0;
    int32_t levels = 0;
    int32_t max_deg = 0;
    int64_t nloops = 0;
    int32_t* loops = nullptr;                 // device: original arcs that are self-loops
    std::vector<int64_t> level_off;           // [levels+1] into level_verts
    std::vector<int32_t> level_maxdeg;        // longest row of each level
    std::vector<int64_t> level_tri;           // pull triangles of each level
    int32_t* level_verts = nullptr;           // device: vertices sorted by (level, rank)
    std::vector<int64_t> level_arc_off;       // [levels+1]: arcs bucketed by tail level
    int64_t* d_level_arc_off = nullptr;       // device copy
    nwcch::Tuning tune;                       // measured schedules (defaults until tuned)
    std::mutex slot_mu;                       // guards the stream slot table
    std::vector<cudaStream_t> slot_stream;    // stream bound to each slot in use
    std::vector<nwcch::StreamSlot> slots;     // device words, preallocated at create
    std::vector<void*> allocations;           // every cudaMalloc of this handle
    size_t device_bytes = 0;
    void* sn_plan = nullptr;                  // nwcch::SnPlan (supernodal customization)
    std::mutex mu;                            // serialises lazily built plans
    std::atomic<int64_t> last_query_launches{0};  // kernels the latest batched-query call enqueued
    void* plans = nullptr;                    // owned by the modules that build plans
    void (*free_plans)(nwcch_topology*) = nullptr;
    void* query_plans = nullptr;              // query_top.cu: top-supernode plans of batched queries
    void (*free_query_plans)(nwcch_topology*) = nullptr;
    void* battery_plan = nullptr;             // battery.cu: arcs in level order
    int64_t battery_pool_hint = 0;            // pieces of the largest battery customization so far (+1/8)
    void (*free_battery_plan)(nwcch_topology*) = nullptr;
};

namespace nwcch {

// Slots preallocated per handle (one per stream that enqueues work on it).
constexpr int kStreamSlots = 64;

// The slot of `stream` (bound on first use). Slots come in blocks of
// kStreamSlots; when every slot is bound, another block is allocated, so no
// two streams ever share one (their counters are scratch of in-flight work).
// Only if that allocation fails do the further streams share the last slot.
StreamSlot stream_slot(nwcch_topology* t, cudaStream_t stream);

// Reads and clears the error word of `stream`'s slot (synchronizes `stream`).
int consume_error(nwcch_topology* t, cudaStream_t stream);

}  // namespace nwcch
