/*
 * nwcch.h - C ABI of libnwcch, a GB300 (sm_103a) implementation of the
 * metric-dependent hot path of Customizable Contraction Hierarchies with
 * negative arc weights: triangle (min,+) customization, the negative-cycle
 * scan, partial re-customization and elimination-tree queries.
 *
 * Reference interface: python/cch_nb.py and python/cch.py of
 * AaravG/negative-weight-cch; each entry point names the reference function
 * (file:line) it replaces.
 *
 * Conventions
 *   - Every function returns int: NWCCH_OK (0), NWCCH_SATURATED (1, see
 *     below) or a negative NWCCH_ERR_* code.
 *   - Vertices of the contracted graph are ranks (0 = eliminated first), as in
 *     the reference (the upward CSR `first`/`head` is in rank space).
 *   - Original arc weights are int32 (NWCCH_INF32 is not a valid weight).
 *     Customized weights are stored as int32 (entry points without suffix)
 *     or int64 (suffix _i64), with INT_MAX of the type meaning "no path".
 *     An INF operand is tested before every addition. A finite sum outside
 *     the storage range [INT_MIN+1, INT_MAX-1] is clamped to it and the call
 *     returns NWCCH_SATURATED: every output is written, but clamped values
 *     are not exact. Without a negative cycle, no customized value exceeds
 *     n * max|w| in magnitude, so int64 storage saturates only on graphs
 *     with a negative cycle. Query distances are int64 with NWCCH_INF64.
 *   - Pointers named *_dev are device pointers (cudaMalloc / torch CUDA
 *     tensors); all others are host pointers. `stream` is a cudaStream_t
 *     (NULL = legacy default stream).
 *   - A topology handle is immutable after creation (but for its tuned
 *     schedules, nwcch_tune_set) and may be shared by calls on different
 *     streams; each stream gets its own error word.
 */
#ifndef NWCCH_H
#define NWCCH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NWCCH_OK 0
#define NWCCH_SATURATED 1       /* completed; some finite values were clamped to the storage range */
#define NWCCH_ERR_ARG (-1)      /* invalid argument (null pointer, bad size, id or weight out of range) */
#define NWCCH_ERR_NOMEM (-2)    /* host or device allocation failed */
#define NWCCH_ERR_CUDA (-3)     /* a CUDA runtime call failed */
#define NWCCH_ERR_TOPOLOGY (-4) /* arrays do not form a valid chordal upward CSR / arc map */
#define NWCCH_ERR_TIMEOUT (-6)  /* a bounded device-side wait gave up */
#define NWCCH_ERR_CAPACITY (-7) /* a fixed-size buffer is too small for the request */

#define NWCCH_INF32 ((int32_t)0x7fffffff)
#define NWCCH_INF64 ((int64_t)0x7fffffffffffffffLL)

/* ------------------------------------------------------------------------
 * Host-side, weight-independent preprocessing (stays on the host).
 * Buffers returned through T** are malloc'ed; free them with nwcch_host_free.
 * ---------------------------------------------------------------------- */

void nwcch_host_free(void* p);

/* Symmetric, de-duplicated neighbour lists without self-loops.
 * Replaces cch_nb.undirected_csr (python/cch_nb.py:22-71).
 * noff: int64[n+1] (caller-allocated); *nbr: int32[*slots] (library-allocated). */
int nwcch_undirected_csr(int64_t n, const int64_t* off, const int32_t* tgt, int64_t* noff,
                         int32_t** nbr, int64_t* slots);

/* Nested-dissection order by inertial-flow bisection, cells of <= leaf
 * vertices ordered by degree; rank[v] = position of v (0 = lowest).
 * threads <= 0 uses every hardware thread.
 * Replaces cch_nb.nested_dissection (python/cch_nb.py:336-426). */
int nwcch_nested_dissection(int64_t n, const int64_t* noff, const int32_t* nbr, const double* x,
                            const double* y, int64_t leaf, int threads, int32_t* rank);

/* Chordal completion in rank space: first int64[n+1] and parent int32[n]
 * (-1 = root) caller-allocated, *head int32[*m_plus] library-allocated,
 * sorted per row. Replaces cch_nb.symbolic (python/cch_nb.py:431-481). */
int nwcch_symbolic(int64_t n, const int64_t* noff, const int32_t* nbr, const int32_t* rank,
                   int64_t* first, int32_t* parent, int32_t** head, int64_t* m_plus);

/* Shortcut arc (-1 for a self-loop) and direction (1 = upward) of every
 * original arc. Replaces cch_nb.edge_arcs (python/cch_nb.py:496-514). */
int nwcch_edge_arcs(int64_t n, const int64_t* off, const int32_t* tgt, const int32_t* rank,
                    const int64_t* first, const int32_t* head, int64_t* e_arc, int8_t* e_up);

/* The same mapping computed on the device from device arrays (off_dev
 * int64[n+1], tgt_dev int32[m], rank_dev int32[n], first_dev int64[n+1],
 * head_dev int32[m+]) into e_arc_dev int64[m], e_up_dev int8[m].
 * NWCCH_ERR_TOPOLOGY if an arc has no shortcut (the order's chordal graph
 * does not hold it). Synchronous. */
int nwcch_edge_arcs_device(int64_t n, const int64_t* off_dev, const int32_t* tgt_dev, const int32_t* rank_dev,
                           const int64_t* first_dev, const int32_t* head_dev, int64_t* e_arc_dev, int8_t* e_up_dev,
                           void* stream);

/* Unique undirected edges (u < v, sorted) of a triangle list int64[ntri*3];
 * a helper of the synthetic graph generators (no reference counterpart). */
int nwcch_triangle_edges(int64_t n, int64_t ntri, const int64_t* tri, int64_t** eu, int64_t** ev,
                         int64_t* nedges);

/* Minimum spanning forest (Kruskal, ties by edge id) of m weighted edges:
 * mask[i] = 1 if edge i is in it. A helper of the synthetic road-like graph
 * generator (no reference counterpart). */
int nwcch_emst_mask(int64_t n, int64_t m, const int64_t* eu, const int64_t* ev, const double* length,
                    uint8_t* mask);

/* ------------------------------------------------------------------------
 * Device-resident topology. The reference passes first/head/parent/e_arc/
 * e_up to every call (python/cch_nb.py:529, 577) and derives what customize
 * and query need from them in Python (cch_nb.py:431-515); here they are
 * uploaded once, validated and extended on the device (tails, levels,
 * elimination-tree depths, downward lists, original arcs per shortcut arc).
 * ---------------------------------------------------------------------- */

typedef struct nwcch_topology nwcch_topology;

/* first int64[n+1], head int32[m+], parent int32[n], e_arc int64[m],
 * e_up int8[m] (host arrays, as produced by the functions above). */
int nwcch_topology_create(int64_t n, const int64_t* first, const int32_t* head,
                          const int32_t* parent, int64_t m, const int64_t* e_arc,
                          const int8_t* e_up, nwcch_topology** out);
int nwcch_topology_destroy(nwcch_topology* t);

/* info[0..7] = n, m+, m, lower triangles, levels, elimination-tree depth,
 * longest row, device bytes held by the handle; with len >= 12 also
 * info[8..11] = supernodes, supernode-tree levels, kernel launches of one
 * supernodal customization (after the two base-value launches), outgoing
 * arc ids stored. */
int nwcch_topology_info(const nwcch_topology* t, int64_t* info, int64_t len);

/* Copies one derived array of the handle into host memory `dst` of `count`
 * elements (count must equal the array's length): what the device built
 * from first/head/parent/e_arc, for inspection and tests (no counterpart in
 * the reference, whose arrays are Python locals). */
#define NWCCH_ARRAY_TAIL 0          /* int32[m+]: lower endpoint of every arc */
#define NWCCH_ARRAY_DEPTH 1         /* int32[n]: elimination-tree depth (root 0) */
#define NWCCH_ARRAY_HDEP 2          /* int32[m+]: depth of every arc's head */
#define NWCCH_ARRAY_DOFF 3          /* int64[n+1]: downward lists, arcs grouped by head ... */
#define NWCCH_ARRAY_DARC 4          /* int32[m+]:  ... ascending in the tail */
#define NWCCH_ARRAY_LEVEL 5         /* int32[n]: 1 + max level of the lower neighbours (0: none) */
#define NWCCH_ARRAY_AEOFF 6         /* int64[m+ + 1]: original arcs of every shortcut arc ... */
#define NWCCH_ARRAY_AEIDX 7         /* int32[aeoff[m+]]: ... ascending arc id */
#define NWCCH_ARRAY_LEVEL_VERTS 8   /* int32[n]: vertices by (level, rank) */
#define NWCCH_ARRAY_LOOPS 9         /* int32[self-loops]: original arcs with e_arc = -1 */
#define NWCCH_ARRAY_LEVEL_OFF 10    /* int64[levels+1]: into LEVEL_VERTS */
#define NWCCH_ARRAY_LEVEL_ARCS 11   /* int64[levels+1]: arcs whose tail is on each level, prefix sums */
#define NWCCH_ARRAY_LEVEL_TRI 12    /* int64[levels]: pull triangles landing on each level */
#define NWCCH_ARRAY_LEVEL_MAXDEG 13 /* int32[levels]: longest row of each level */
int nwcch_topology_export(const nwcch_topology* t, int which, void* dst, int64_t count);

/* Reads and clears the error word of `stream`'s calls on `t` (synchronizes
 * `stream`). Each stream that enqueues work on a handle gets its own error
 * word and scratch counters (64 per handle), so calls on different streams
 * may overlap. */
int nwcch_check(nwcch_topology* t, void* stream);

/* Schedules picked by measurement (no counterpart in the reference: the
 * autotuner of this library, python nwcch.tune, sets them per topology).
 * Results never depend on them. */
#define NWCCH_TUNE_QUERY_DENSE_ROWS 1      /* query chunks with fewer rows go row by row (1..33) */
#define NWCCH_TUNE_QUERY_SMEM_LABELS_MAX 2 /* per-warp query label bytes kept in shared memory */
#define NWCCH_TUNE_UPDATE_BUDGET_NS 3      /* update level-sweep budget before the dense finish (0: estimate) */
#define NWCCH_TUNE_QUERY_OCCUPANCY 4       /* 32-bit query kernel: 1 light, 2 light capped at 64 registers,
                                              3 chunk labels and row offsets held in registers */
#define NWCCH_TUNE_QUERY_CTA_MAX 5         /* batches of at most this many queries run a CTA per query */
/* Customization schedule: supernodes with k <= 32, b <= 64 and a trapezoid of
 * at most SN_WARP_CAP (<= 512) arcs are customized by one warp each, in
 * levels holding at least SN_WARP_MIN_COUNT of them. Setting either rebuilds
 * the plan (synchronizes the device; no other call on the handle meanwhile). */
#define NWCCH_TUNE_SN_WARP_CAP 6
#define NWCCH_TUNE_SN_WARP_MIN_COUNT 7
/* 1: the customization's kernels are programmatic dependent launches (each
 * may start while the previous drains, then waits for it on the device). */
#define NWCCH_TUNE_PDL 8
/* The CTA-per-query form: 16 warps a query for batches of at most
 * QUERY_CTA_WIDE_MAX queries (else 8); its own row-by-row threshold. */
#define NWCCH_TUNE_QUERY_CTA_WIDE_MAX 9
#define NWCCH_TUNE_QUERY_CTA_DENSE_ROWS 10
/* Battery customization: initial piece pool (0: 1.5 pieces a direction) and
 * initial per-warp buffer of profiles longer than 32 pieces (64..2^22
 * pieces); both grow, and the customization reruns, when outgrown. */
#define NWCCH_TUNE_BATTERY_POOL 11
#define NWCCH_TUNE_BATTERY_BUFFER 12
/* Updates of at least this many (distinct) arcs skip the level sweep and
 * finish densely at once (0: never; the sweep budget decides). */
#define NWCCH_TUNE_UPDATE_DENSE_MIN 13
/* Failure detection of the update's bounded grid barrier: the spin limit of
 * one wait (iterations of about 100 ns; default 2^24, a few seconds), and a
 * test hook that makes every barrier wait for this many blocks more than the
 * launch has (default 0), so that the wait runs out: the call then returns
 * NWCCH_ERR_TIMEOUT with w updated and up/dn partly re-customized (customize
 * again before use), and the handle's update workspace is reset so that the
 * next update is exact. */
#define NWCCH_TUNE_UPDATE_SPIN_LIMIT 14
#define NWCCH_TUNE_TEST_BARRIER_EXTRA 15
/* Batched queries (more than QUERY_CTA_MAX of them, int32 storage): the
 * supernodes crossed by about this many chains of the batch or more (the top
 * of the elimination tree) are swept as (min,+) products over tiles of up to
 * 32 chains, the rest of each chain per warp; 0 sweeps every chain per warp.
 * Default 64. */
#define NWCCH_TUNE_QUERY_TOP_CHAINS 16
/* Customization schedule near the root (int32 storage): the levels from
 * which every level has no warp-kernel launch and no launch of more than
 * this many items run as one persistent cooperative launch, one phase per
 * former launch with a bounded grid barrier between phases (a wait past the
 * NWCCH_TUNE_UPDATE_SPIN_LIMIT reports NWCCH_ERR_TIMEOUT); 0: every level
 * launches its own kernels. Default 0. Setting it rebuilds the plan, as
 * NWCCH_TUNE_SN_WARP_CAP does. */
#define NWCCH_TUNE_SN_CHAIN_MAX_ITEMS 17
/* Customization schedule at the bottom: in the levels where supernodes take
 * the warp kernel, those whose trapezoid holds at most this many arcs
 * (<= 32) take a kernel with one thread per supernode instead (0: none).
 * Default 16. Setting it rebuilds the plan. */
#define NWCCH_TUNE_SN_THREAD_CAP 18
/* Batches of at most this many queries (int32 storage) run the streaming
 * query kernel: a CTA per chain, the chain's rows streamed into shared
 * memory by bulk asynchronous copies, both chains of a query at once. Used
 * when the topology fits its shared memory (labels, boundary positions and
 * the copy ring; rows of at most 12,280 arcs). 0: off. Default 64. */
#define NWCCH_TUNE_QUERY_STREAM_MAX 19
/* Partial updates: the level sweep first runs in one CTA (block barriers, no
 * grid barrier per level) until it has evaluated this many arcs; then it
 * hands its pending levels to the sweep over the whole grid. Counts and
 * values are the same either way. 0: the grid sweep from the start.
 * Default 8192. */
#define NWCCH_TUNE_UPDATE_SMALL_ARCS 20
/* ... or until it has run this many nanoseconds (>= 1; default 300,000). A
 * sweep out of time stops before its next arc, inside a level if need be;
 * the level is finished by the grid sweep (or the dense finish, for the grid
 * sweep's own budget, NWCCH_TUNE_UPDATE_BUDGET_NS), counted once. */
#define NWCCH_TUNE_UPDATE_SMALL_NS 21
/* The streaming query kernel's shared-memory data ring, in KB (0: as large as
 * the labels leave, at most 192; default 0). Smaller rings hold fewer rows
 * per copied item; a topology whose longest row does not fit a third of the
 * ring goes to the other query forms. */
#define NWCCH_TUNE_QUERY_STREAM_RING_KB 22
int nwcch_tune_set(nwcch_topology* t, int key, int64_t value);
int nwcch_tune_get(const nwcch_topology* t, int key, int64_t* value);

/* ------------------------------------------------------------------------
 * Customization. Replaces cch_nb.customize (python/cch_nb.py:529-563) and
 * CCH::customize (cpp/cch.cpp:437-463): base values are the minimum over
 * parallel original arcs (self-loops skipped), then every lower triangle is
 * relaxed. w_dev int32[m]; up_dev, dn_dev int32[m+] receive the customized
 * weights. nwcch_customize synchronizes and reports NWCCH_SATURATED;
 * the _async form only enqueues (status surfaces at nwcch_check).
 * ---------------------------------------------------------------------- */
int nwcch_customize(nwcch_topology* t, const int32_t* w_dev, int32_t* up_dev, int32_t* dn_dev,
                    void* stream);
int nwcch_customize_async(nwcch_topology* t, const int32_t* w_dev, int32_t* up_dev,
                          int32_t* dn_dev, void* stream);
/* The same with int64 storage (python/cch_nb.py:529-563). */
int nwcch_customize_i64(nwcch_topology* t, const int32_t* w_dev, int64_t* up_dev, int64_t* dn_dev,
                        void* stream);
int nwcch_customize_i64_async(nwcch_topology* t, const int32_t* w_dev, int64_t* up_dev,
                              int64_t* dn_dev, void* stream);
/* Batched customization of `metrics` metrics over one topology (vehicle or
 * battery variants), in one launch sequence whose kernels take the metric
 * as a grid dimension: w_dev is metrics x m (metric-major), up_dev/dn_dev
 * metrics x m+. Same per-metric results as nwcch_customize
 * (python/cch_nb.py:529-563 applied to every metric). 1 <= metrics <= 65535. */
int nwcch_customize_batch(nwcch_topology* t, int64_t metrics, const int32_t* w_dev, int32_t* up_dev,
                          int32_t* dn_dev, void* stream);
int nwcch_customize_batch_async(nwcch_topology* t, int64_t metrics, const int32_t* w_dev, int32_t* up_dev,
                                int32_t* dn_dev, void* stream);
/* Negative-cycle counts of a batch: counts_dev[k] = arcs of metric k with
 * up + dn < 0 (python/cch_nb.py:566-572), enqueue only. */
int nwcch_negative_cycle_arcs_batch_async(nwcch_topology* t, int64_t metrics, const int32_t* up_dev,
                                          const int32_t* dn_dev, int64_t* counts_dev, void* stream);
/* The plain form of the same computation: one launch per elimination level,
 * a block per row pulling its lower triangles (the level structure of
 * CCH::levels / customize_parallel, cpp/cch.cpp:465-529). Same results; kept
 * as the per-metric baseline the supernodal path is measured against. */
int nwcch_customize_plain(nwcch_topology* t, const int32_t* w_dev, int32_t* up_dev, int32_t* dn_dev,
                          void* stream);
int nwcch_customize_plain_async(nwcch_topology* t, const int32_t* w_dev, int32_t* up_dev,
                                int32_t* dn_dev, void* stream);

/* Number of arcs with up + dn < 0 (Theorem 3: nonzero iff a negative cycle).
 * Replaces cch_nb.negative_cycle_arcs (python/cch_nb.py:566-572) and
 * CCH::negative_cycle_arcs (cpp/cch.cpp:531-536). Synchronous. */
int nwcch_negative_cycle_arcs(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                              int64_t* count, void* stream);
/* int64 storage (python/cch_nb.py:566-572). */
int nwcch_negative_cycle_arcs_i64(nwcch_topology* t, const int64_t* up_dev, const int64_t* dn_dev,
                                  int64_t* count, void* stream);
/* Enqueue-only form (int32 storage): the count lands in count_dev (one
 * int64 of device memory) in stream order (python/cch_nb.py:566-572). */
int nwcch_negative_cycle_arcs_async(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                                    int64_t* count_dev, void* stream);

/* Number of self-loop original arcs with a negative weight (loops never
 * enter the contracted graph). Replaces CCH._negative_loop
 * (python/cch.py:659-660). Synchronous. */
int nwcch_negative_loops(nwcch_topology* t, const int32_t* w_dev, int64_t* count, void* stream);

/* ------------------------------------------------------------------------
 * Partial re-customization. Replaces CCH.update_edges (python/cch.py:349-402)
 * together with the bookkeeping of CCH.update_created_negative_cycle
 * (python/cch.py:666-671). edge_idx/new_w are HOST arrays of k changes
 * (original arc ids, CSR order; the last write to an arc wins). w_dev is
 * updated in place, up_dev/dn_dev re-customized in place.
 * stats[0] = arcs re-evaluated, stats[1] = arcs changed, stats[2] = changed
 * arcs with up + dn < 0. changed_dev (nullable, capacity m+) receives the
 * changed arcs. Calls on one topology are serialized; synchronous.
 * ---------------------------------------------------------------------- */
int nwcch_update(nwcch_topology* t, int32_t* w_dev, int32_t* up_dev, int32_t* dn_dev,
                 const int64_t* edge_idx, const int32_t* new_w, int64_t k, int64_t* stats,
                 int32_t* changed_dev, void* stream);
/* int64 storage (python/cch.py:349-402). */
int nwcch_update_i64(nwcch_topology* t, int32_t* w_dev, int64_t* up_dev, int64_t* dn_dev,
                     const int64_t* edge_idx, const int32_t* new_w, int64_t k, int64_t* stats,
                     int32_t* changed_dev, void* stream);

/* ------------------------------------------------------------------------
 * Elimination-tree queries. Replaces cch_nb.query (python/cch_nb.py:577-615)
 * and Query::run (cpp/cch.cpp:549-575), batched: dist_dev[i] = distance from
 * rank s_rank_dev[i] to rank t_rank_dev[i] (NWCCH_INF64 if unreachable).
 * The caller-owned scratch df/dr/mark of the reference is not needed.
 * Synchronous. Batches of more than NWCCH_TUNE_QUERY_CTA_MAX queries sweep
 * the top of the elimination tree as (min,+) products over tiles of chains
 * (stream-ordered scratch of 8 bytes per query and depth level, in passes of
 * at most 4 GB); smaller batches take a CTA per query.
 * ---------------------------------------------------------------------- */
int nwcch_query_batch(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                      const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq,
                      int64_t* dist_dev, void* stream);
/* int64 storage (python/cch_nb.py:577-615). */
int nwcch_query_batch_i64(nwcch_topology* t, const int64_t* up_dev, const int64_t* dn_dev,
                          const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq,
                          int64_t* dist_dev, void* stream);
/* Enqueue-only batch (python/cch_nb.py:577-615), for CUDA-graph capture and
 * pipelines: no synchronization (argument errors in the rank arrays surface
 * at nwcch_check); large batches take the (min,+) product form with
 * stream-ordered scratch (cudaMallocAsync, which a capture records), once a
 * call outside any capture has built its plan; otherwise labels in shared
 * memory and no allocation. Returns
 * NWCCH_ERR_CAPACITY when the elimination tree is too deep for shared-memory
 * labels (about 10,000 levels); nwcch_query_batch then falls back to the
 * plain kernel. */
int nwcch_query_batch_async(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                            const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq,
                            int64_t* dist_dev, void* stream);
/* The plain per-query form (one warp per query, one ancestor at a time,
 * labels in global scratch): the same sweeps as Query::run
 * (cpp/cch.cpp:549-575), kept as the baseline of the batched form. */
int nwcch_query_batch_plain(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                            const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq,
                            int64_t* dist_dev, void* stream);

/* Allocation-free form of nwcch_query_batch (int32 storage); it has no
 * counterpart in the reference. For callers that must not allocate device
 * memory: a serving loop that has already given all device memory to
 * resident metrics, an application whose own allocator owns the device, or a
 * latency-critical path that cannot risk an allocator call. Instead of
 * cudaMallocAsync it uses a fixed 32 MiB label scratch compiled into the
 * library (held by every GPU that loads it until the process exits); it
 * calls no allocation routine. Limit: the per-warp scratch is
 * 8 * (2.5 * (depth + 1) + 1) bytes and whole blocks of 4 warps must fit, so
 * an elimination tree deeper than about 419,000 returns NWCCH_ERR_CAPACITY;
 * deeper trees just run fewer queries at a time. The first call on a device
 * looks up the scratch's device address (make it before any stream capture;
 * the address is cached for the process, so do not call this entry point on
 * a device again after cudaDeviceReset).
 * All calls on a device share the scratch: calls that overlap on the GPU
 * (other streams, other threads) race and must be serialized by the caller.
 * Synchronous; same results as nwcch_query_batch. */
int nwcch_query_batch_noalloc(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                              const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq,
                              int64_t* dist_dev, void* stream);

/* ------------------------------------------------------------------------
 * Shortest paths. Replaces CCH.query_path (python/cch.py:406-507): the
 * distance and the vertices of a shortest s-t path (ranks, s first, t last),
 * each shortcut unpacked through its lowest lower-triangle vertex whose two
 * sides add up to it, with the reference's choices among equal-length paths.
 * off_dev int64[nq+1] receives the offsets of every query's vertices in
 * path_dev (capacity cap; an unreachable pair gets none); *needed = the total.
 * If cap < *needed, NWCCH_ERR_CAPACITY with off_dev and *needed filled and
 * nothing written to path_dev. Synchronous.
 * ---------------------------------------------------------------------- */
int nwcch_query_paths(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev,
                      const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq, int64_t* dist_dev,
                      int64_t* off_dev, int32_t* path_dev, int64_t cap, int64_t* needed, void* stream);
int nwcch_query_paths_i64(nwcch_topology* t, const int64_t* up_dev, const int64_t* dn_dev,
                          const int32_t* s_rank_dev, const int32_t* t_rank_dev, int64_t nq, int64_t* dist_dev,
                          int64_t* off_dev, int32_t* path_dev, int64_t cap, int64_t* needed, void* stream);

/* ------------------------------------------------------------------------
 * CCH potential
 * ---------------------------------------------------------------------- */

/* p(v) = min(0, min_u dist(u, v)), the virtual-source distances of
 * Johnson's algorithm, read off a customized metric by an upward and a
 * downward sweep. Replaces cch_potential (cpp/cch.cpp:631-655) and
 * CCH.potential (python/cch.py:734-755). p_dev: int64[n] in RANK space (the
 * reference returns p[rank[v]] per vertex v). Meaningful for metrics without
 * a negative cycle; NWCCH_SATURATED if a sum left the int64 range. */
int nwcch_potential(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev, int64_t* p_dev,
                    void* stream);
int nwcch_potential_async(nwcch_topology* t, const int32_t* up_dev, const int32_t* dn_dev, int64_t* p_dev,
                          void* stream);
int nwcch_potential_i64(nwcch_topology* t, const int64_t* up_dev, const int64_t* dn_dev, int64_t* p_dev,
                        void* stream);

/* ------------------------------------------------------------------------
 * Battery-constrained profiles (float64)
 *
 * An arc of energy c maps a state of charge b to b - c when c >= 0 (and
 * b >= c), to min(M, b - c) when c < 0; every path induces a piece
 * (in, cost, out): f(b) = min(out, b - cost) for b >= in. A shortcut
 * direction d = 2*arc + (0 up, 1 down) holds a profile, the pieces left after
 * merging its candidates in the reference's order (the original arcs in input
 * order, then its lower triangles by ascending lowest vertex): a candidate
 * that a kept piece dominates is dropped, otherwise the pieces it dominates
 * are removed, order kept, and it is appended. Same float64 operations as
 * the reference, so the profiles are its profiles piece for piece.
 * ---------------------------------------------------------------------- */
typedef struct nwcch_battery nwcch_battery;

/* Replaces battery_customize (python/cch_nb_battery.py:48-183): w_dev
 * float64[m] arc energies (original arc order), battery capacity M > 0.
 * Synchronous on `stream`; device buffers grow and the customization reruns
 * if a profile outgrows them. *out is freed with nwcch_battery_free. */
int nwcch_battery_customize(nwcch_topology* t, const double* w_dev, double capacity, void* stream,
                            nwcch_battery** out);
/* Total pieces and the largest profile. */
int nwcch_battery_info(const nwcch_battery* b, int64_t* pieces, int32_t* largest);
/* Canonical HOST copy: cnt int32[2m+], off int64[2m+ + 1] (direction
 * order), pieces float64[total][3] as (in, cost, out); pieces may be NULL
 * (counts and offsets only). */
int nwcch_battery_export(const nwcch_battery* b, int32_t* cnt, int64_t* off, double* pieces);
/* Replaces battery_query (python/cch_nb_battery.py:296-343) for a batch:
 * best charge at t leaving s with charge b0 (-inf if infeasible); a CTA per
 * query for batches of up to 304, else a warp per query. s/t int32 rank
 * ids, b0_dev/out_dev float64[nq]. Synchronous (reads the error word). */
int nwcch_battery_query(nwcch_topology* t, const nwcch_battery* b, const int32_t* s_rank_dev,
                        const int32_t* t_rank_dev, const double* b0_dev, int64_t nq, double* out_dev,
                        void* stream);
void nwcch_battery_free(nwcch_battery* b);

#ifdef __cplusplus
}
#endif

#endif /* NWCCH_H */
