/*
 * CPU oracle for the metric-dependent CCH hot path - TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference algorithms (AaravG/negative-weight-
 * cch), each function citing the reference lines it follows, in exact integer
 * arithmetic: int32 arc weights, int64 customized values and distances, and
 * ORC_INF = INT64_MAX for "no path" (an INF operand is tested before every
 * addition). On integer weights the reference's float64 values are exact
 * integers (below 2^53), so equality with this oracle is bit-exact parity.
 *
 * Only tests, the smoke check and the benchmark's CPU-baseline / reference
 * legs may load this library; the product never does.
 *
 * Pinning: tests/test_oracle.py checks every function against golden vectors
 * produced by the reference's own code (tests/golden/make_golden.py).
 */
#ifndef NWCCH_ORACLE_H
#define NWCCH_ORACLE_H

#include <stdint.h>

#define ORC_INF INT64_MAX

/* python/cch_nb.py:529-563 (= cpp/cch.cpp:437-463): base values from the
 * original arcs, then lower triangles (x; y, z) for x ascending. */
void orc_customize(int64_t n, const int64_t* first, const int32_t* head, int64_t m, const int64_t* e_arc,
                   const int8_t* e_up, const int32_t* w, int64_t* up, int64_t* dn);

/* cpp/cch.cpp:468-529: vertices bucketed by level, each level in parallel
 * with OpenMP (threads <= 0: all) and an atomic minimum. Same result as
 * orc_customize. Returns the number of levels. */
int64_t orc_customize_parallel(int64_t n, const int64_t* first, const int32_t* head, int64_t m,
                               const int64_t* e_arc, const int8_t* e_up, const int32_t* w, int64_t* up,
                               int64_t* dn, int threads);

/* python/cch_nb.py:566-572: arcs with up + dn < 0. */
int64_t orc_negative_cycle_arcs(int64_t m_plus, const int64_t* up, const int64_t* dn);

/* python/cch_nb.py:577-615: elimination-tree query with caller scratch
 * df/dr (int64[n]) and mark (int64[n]); q is a fresh query id. */
int64_t orc_query(int64_t s_rank, int64_t t_rank, const int64_t* first, const int32_t* head,
                  const int64_t* parent, const int64_t* up, const int64_t* dn, int64_t* df, int64_t* dr,
                  int64_t* mark, int64_t q);

/* Batch of orc_query over rank pairs; threads <= 0 uses all cores. */
void orc_query_batch(int64_t n, const int64_t* first, const int32_t* head, const int64_t* parent,
                     const int64_t* up, const int64_t* dn, int64_t nq, const int64_t* s_rank,
                     const int64_t* t_rank, int64_t* out, int threads);

/* python/cch.py:349-402: partial re-customization. w (current weights, int32[m])
 * is updated in place by the k changes (last write wins), up/dn re-customized
 * in place. stats[0] = arcs evaluated, stats[1] = arcs changed,
 * stats[2] = changed arcs with up + dn < 0 (python/cch.py:666-671).
 * changed (nullable, capacity m+) receives the changed arcs in pop order. */
void orc_update(int64_t n, const int64_t* first, const int32_t* head, int64_t m, const int64_t* e_arc,
                const int8_t* e_up, int32_t* w, int64_t* up, int64_t* dn, int64_t k, const int64_t* edge_idx,
                const int32_t* new_w, int64_t* stats, int64_t* changed);

/* The same update split as the reference splits it: the update index
 * (python/cch.py:289-347) built once per topology, then any number of
 * updates on it (python/cch.py:349-402). The index keeps the topology's
 * pointers, which must outlive it. */
typedef struct OrcUpdateIndex OrcUpdateIndex;
OrcUpdateIndex* orc_update_index(int64_t n, const int64_t* first, const int32_t* head, int64_t m,
                                 const int64_t* e_arc, const int8_t* e_up);
void orc_update_indexed(OrcUpdateIndex* X, int32_t* w, int64_t* up, int64_t* dn, int64_t k,
                        const int64_t* edge_idx, const int32_t* new_w, int64_t* stats, int64_t* changed);
void orc_update_index_free(OrcUpdateIndex* X);

/* python/search.py:8-29 (queue-based Bellman-Ford) on the original graph,
 * single source, original vertex ids. Returns 1 if a negative cycle is
 * reachable from s (a vertex relaxed n times), else 0; dist int64[n]. */
int orc_bellman_ford(int64_t n, const int64_t* off, const int32_t* tgt, const int32_t* w, int64_t s,
                     int64_t* dist);

/* Negative-cycle test of the whole graph (python/preprocess.py:13-59 role:
 * virtual source with 0-arcs to every vertex). Returns 1 if a negative cycle
 * exists. */
int orc_has_negative_cycle(int64_t n, const int64_t* off, const int32_t* tgt, const int32_t* w);

/* cpp/cch.cpp:631-655 (= python/cch.py:734-755): the potential
 * p(v) = min(0, min_u dist(u, v)) read off a customized CCH, rank space:
 * an upward pass in increasing rank, then a downward pass in decreasing rank.
 * p int64[n]. */
void orc_potential(int64_t n, const int64_t* first, const int32_t* head, const int64_t* up, const int64_t* dn,
                   int64_t* p);

/* The same potential by Bellman-Ford from a virtual source with 0-arcs to
 * every vertex (the role of cpp/cch.cpp:608-629 johnson_potential), original
 * vertex ids. Returns 1 if a negative cycle exists (p then undefined). */
int orc_virtual_source_potential(int64_t n, const int64_t* off, const int32_t* tgt, const int32_t* w,
                                 int64_t* p);

/* python/cch.py:406-507: distance and shortest path (ranks, s first) with the
 * reference's choices among equal paths: the first arc (in sweep order) that
 * reaches a label's value, the lowest common ancestor reaching the minimum,
 * and each shortcut unpacked through its lowest lower-triangle vertex whose
 * two sides add up to it. tail int32[m+]: lower endpoint of every arc;
 * doff int64[n+1] / darc int32[m+]: arcs (x, y) grouped by y, ascending x.
 * Writes *dist (ORC_INF if unreachable); returns the path length (0 if
 * unreachable), or -(length) if cap is too small (nothing written then). */
int64_t orc_query_path(int64_t n, const int64_t* first, const int32_t* head, const int64_t* parent,
                       const int32_t* tail, const int64_t* doff, const int32_t* darc, const int64_t* up,
                       const int64_t* dn, int64_t s, int64_t t, int64_t* dist, int64_t* path, int64_t cap);

/* ---- battery-constrained profiles (oracle_battery.c), float64 ----------
 * python/cch_nb_battery.py:48-183: the customization, x ascending, into
 * per-direction profiles (d = 2*arc + (0 up, 1 down)). Returns an opaque
 * handle (NULL on allocation failure). w float64[m], battery capacity M. */
void* orc_battery_customize(int64_t n, const int64_t* first, const int32_t* head, int64_t m, const int64_t* e_arc,
                            const int8_t* e_up, const double* w, double M);
/* Total pieces of all profiles. */
int64_t orc_battery_pieces(const void* handle);
/* Canonical layout: cnt int32[2m+], off int64[2m+ + 1] (direction order),
 * pieces float64[total][3] as (in, cost, out). */
void orc_battery_export(const void* handle, int32_t* cnt, int64_t* off, double* pieces);
void orc_battery_free(void* handle);

/* python/cch_nb_battery.py:296-343: best charge at t leaving s with b0
 * (-inf if infeasible); scratch soc/dsoc float64[n], mark int64[n], q a fresh
 * query id. */
double orc_battery_query(int64_t s_rank, int64_t t_rank, double b0, const int64_t* first, const int32_t* head,
                         const int64_t* parent, const int32_t* cnt, const int64_t* off, const double* pieces,
                         double* soc, double* dsoc, int64_t* mark, int64_t q);
void orc_battery_query_batch(int64_t n, const int64_t* first, const int32_t* head, const int64_t* parent,
                             const int32_t* cnt, const int64_t* off, const double* pieces, int64_t nq,
                             const int64_t* s_rank, const int64_t* t_rank, const double* b0, double* out,
                             int threads);

/* python/cch_nb_battery.py:316-351: max charge at every vertex from s by
 * label correcting on the original graph (original ids); soc float64[n]. */
void orc_battery_label_correcting(int64_t n, const int64_t* off, const int32_t* tgt, const double* w, double M,
                                  int64_t s, double b0, double* soc);

#endif
