// Supernodal customization plan (internal).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <mutex>
#include <vector>

struct nwcch_topology;

namespace nwcch {

// A supernode is a maximal run of ranks [s0, s0+k) in which every vertex's
// upper row is the next vertex plus the row of that next vertex (rows nested).
// Its arcs form a dense trapezoid: row i (vertex s0+i) holds the columns
// j in (i, k + b): ranks s0+i+1..s0+k-1 and then the boundary B (the row of
// the last vertex, b entries), at index first[s0+i] + (j - i - 1).
// A supernode in one 32-byte load: first vertex, rows, boundary size, next
// supernode on its elimination-tree path (-1 at a root) and the entry row
// there, first arc of its trapezoid (the customization kernels and the
// streaming query kernel read it instead of chasing s0/k/b and first[]).
struct QsNode {
    int32_t s0, k, b, next;
    int32_t next_row, pad;
    int64_t base;
};

struct SnDev {
    const QsNode* node;      // [nsn]
    const int32_t* s0;       // [nsn]
    const int32_t* k;        // [nsn]
    const int32_t* b;        // [nsn]
    const int64_t* rel_off;  // [nsn] start of the supernode's outgoing arc ids
    const int32_t* rel;      // arc id of (B[p], B[q]) for p < q, packed upper triangle
    const int32_t* sn_id;    // [n] supernode of every vertex
};

enum SnKind : int {
    SN_INT_SMALL = 0,  // warp per supernode: vertex-sequential internal triangles
    SN_PANEL = 1,      // CTA per (supernode, column tile): one 32-row panel
    SN_TRAIL = 2,      // CTA per (supernode, row tile, column tile): trailing update
    SN_OUT_BIG = 3,    // CTA per 64x64 tile of the outgoing boundary x boundary block
    SN_OUT_SMALL = 4,  // CTA per 16x16 tile of the same
    SN_WARP = 5,       // warp per small supernode: the whole supernode in shared memory
    SN_THREAD = 6,     // thread per tiny supernode: the whole supernode in shared memory
};

// A supernode whose trapezoid holds at most this many arcs (and k <= 32,
// b <= 64) is customized by one warp from shared memory in one launch.
constexpr int SN_WARP_CAP = 512;
// A supernode whose trapezoid holds at most this many arcs may be customized
// by one thread (levels with many of them: most of a road-like graph).
constexpr int SN_THREAD_CAP = 32;
__host__ __device__ inline int64_t sn_trapezoid(int64_t k, int64_t b) { return k * (k + b - 1) - k * (k - 1) / 2; }

struct SnLaunch {
    int kind;
    int level;
    int panel;
    int64_t off;    // first item (int32 triples) in the plan's item array
    int64_t count;  // items
};

enum SnGraphKind : int { SN_GRAPH_CUSTOMIZE = 0, SN_GRAPH_POTENTIAL = 1 };

// A captured launch sequence for one binding: (kind, storage, metrics, error
// word, w or the output, up, dn).
struct SnGraph {
    int kind;
    int storage;
    int metrics;
    int* err;
    const void* w;
    const void* up;
    const void* dn;
    cudaGraphExec_t exec;
    uint64_t last_use;
    long long spin = 0;  // device wait bound and test hook of the persistent launch
    int extra = 0;
};

// Schedule choices of a plan (measured per topology; results never depend
// on them): a supernode with k <= 32, b <= 64 and a trapezoid of at most
// warp_cap arcs takes the warp kernel when its level holds at least
// warp_min_count such supernodes (a throughput form: near the top of the
// tree a lone supernode finishes sooner on the panel and tile kernels).
struct SnPlanParams {
    int32_t warp_cap = SN_WARP_CAP;
    int64_t warp_min_count = 1024;
    // supernodes of such levels whose trapezoid holds at most thread_cap
    // (<= SN_THREAD_CAP) arcs take the thread kernel instead (0: none)
    int32_t thread_cap = 16;
    // levels near the root whose launches each hold at most this many items
    // (and no warp-kernel launch) run as one persistent launch, k_sn_chain
    // (int32 storage); 0: every level launches its kernels. Off by default:
    // on the 24M road-like graph the launches are faster (one CTA per SM runs
    // a phase's items in rounds, where separate launches keep several tiles
    // per SM in flight); the autotuner tries both.
    int64_t chain_max_items = 0;
};

// One phase of the persistent top-of-tree launch (the items of one former
// launch; consecutive phases are separated by a grid barrier).
struct ChainPhase {
    int32_t kind;   // SN_PANEL, SN_TRAIL or SN_OUT_BIG
    int32_t panel;  // panel index (SN_PANEL, SN_TRAIL)
    int64_t off;    // first item (int32 triples) in the chain's item array
    int64_t count;  // items
};

constexpr int CHAIN_THREADS = 256;  // threads of a chain CTA = panel columns of a chain panel item

struct SnPlan {
    SnPlanParams params;
    std::vector<SnGraph> graphs;  // up to 16, least recently used dropped first
    uint64_t graph_clock = 0;
    std::mutex graph_mu;
    int64_t nsn = 0;
    int32_t levels = 0;
    int64_t items = 0;
    int64_t rel_entries = 0;
    int32_t max_b = 0;            // longest boundary of any supernode
    // supernodes grouped by level (the vertex sweeps of the potential):
    // level l is sn_order[sn_level_off[l] .. sn_level_off[l+1]): entries
    // [0, sn_level_big[l]) take a whole CTA each, [sn_level_big[l],
    // sn_level_single[l]) a warp each, the rest (single vertices) a thread
    std::vector<int64_t> sn_level_off;
    std::vector<int64_t> sn_level_big;
    std::vector<int64_t> sn_level_single;
    // the potential's boundary products of those CTA-swept supernodes, as
    // (supernode, tile) pairs by level: upward 256 boundary columns a tile,
    // downward 32 rows a tile
    std::vector<int64_t> pot_bu_off, pot_bd_off;  // [levels+1], in pairs
    int32_t* d_pot_bu = nullptr;
    int32_t* d_pot_bd = nullptr;
    int32_t* d_sn_order = nullptr;
    std::vector<SnLaunch> launches;
    // the persistent top of the plan: launches[chain_from..] (levels >=
    // chain_level) as phases of k_sn_chain for int32 storage; the other
    // storage runs them as launches
    size_t chain_from = 0;
    int32_t chain_level = 0;
    int32_t nchain_phases = 0;
    int32_t* d_chain_items = nullptr;
    ChainPhase* d_chain_phases = nullptr;
    int chain_grid = -1;  // CTAs of the chain launch (-1: not sized yet, 0: cannot run)
    // chain walk of the streaming query kernel (one descriptor a supernode)
    struct QsNode* d_qnodes = nullptr;
    std::mutex chain_mu;
    SnDev dev{};
    int32_t* d_items = nullptr;
    std::vector<void*> allocations;
    size_t bytes = 0;
};

// Builds the plan from the host copy of a topology; nullptr on failure.
SnPlan* build_supernodal_plan(int64_t n, const int64_t* first, const int32_t* head, const int32_t* parent,
                              const SnPlanParams& prm, int* rc);
void free_supernodal_plan(SnPlan* p);

// Enqueues a full customization on stream s (base values + every launch) of
// `metrics` metrics stored metric-major (w: metrics x m, up/dn: metrics x m+);
// every launch gets the metric as its second grid dimension. Range errors go
// to the device word err.
template <class T>
int run_supernodal(nwcch_topology* t, SnPlan* P, const int32_t* w, T* up, T* dn, cudaStream_t s, int* err,
                   int metrics = 1);

// A supernode swept by a whole CTA rather than one warp.
inline bool sn_sweep_big(int64_t k, int64_t b) { return k > 32 || k * (k + b) > 32 * 1024; }

// Enqueues the supernodal query kernel (labels in shared memory); sets *used
// to false, enqueuing nothing, when the elimination tree is too deep for it.
template <class T>
int query_sn_async(nwcch_topology* t, const T* up, const T* dn, const int32_t* s_rank, const int32_t* t_rank,
                   int64_t nq, int64_t* dist, cudaStream_t s, bool allow_alloc, bool* used);

// Enqueues the batched query pipeline of query_top.cu (int32 storage; counts
// its kernel launches in *launches): the
// lower part of every chain per warp, the top supernodes as (min,+) products
// over tiles of chains, the meet per query. Its kernels return at once when
// the metric needs 64-bit labels (maxabs, on the device). *used = false when
// the batch is not its case (nothing enqueued).
int query_top_async(nwcch_topology* t, const int32_t* up, const int32_t* dn, const int32_t* s_rank,
                    const int32_t* t_rank, int64_t nq, int64_t* dist, const unsigned int* maxabs, int* err,
                    cudaStream_t s, bool* used, int64_t* launches);

// Enqueues the streaming query kernel of query_stream.cu for a batch of at
// most tune.query_stream_max int32-stored queries (a CTA per chain; counts
// its launches in *launches). *used = false when the batch or the topology is
// not its case (nothing enqueued).
int query_stream_async(nwcch_topology* t, const int32_t* up, const int32_t* dn, const int32_t* s_rank,
                       const int32_t* t_rank, int64_t nq, int64_t* dist, int* err, cudaStream_t s, bool* used,
                       int64_t* launches);

// Enqueues the 64-bit supernodal query kernel for the queries of a batch
// flagged in `wide` (int32 storage): the answers of the streaming kernel's
// queries that met a weight beyond the 32-bit label bound.
int query_sn64_flagged(nwcch_topology* t, const int32_t* up, const int32_t* dn, const int32_t* s_rank,
                       const int32_t* t_rank, int64_t nq, int64_t* dist, const int32_t* wide, int* err,
                       cudaStream_t s);

// The same through a CUDA graph captured once per (w, up, dn) binding and
// error word (the slot of stream s) and replayed afterwards; when s is itself
// being captured the launches are simply enqueued into the caller's capture.
template <class T>
int launch_supernodal(nwcch_topology* t, SnPlan* P, const int32_t* w, T* up, T* dn, cudaStream_t s,
                      int metrics = 1);

// Enqueues `enqueue`'s launches on s as a CUDA graph captured once per key
// (16 kept per plan, least recently used dropped first); enqueues them
// directly when s is being captured or NWCCH_NO_GRAPH is set.
int launch_cached(SnPlan* P, const SnGraph& key, cudaStream_t s, const std::function<int(cudaStream_t)>& enqueue);

}  // namespace nwcch
