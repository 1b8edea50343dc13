/*
 * CPU oracle for the metric-dependent CCH hot path - TEST INFRASTRUCTURE ONLY.
 * See oracle.h for the contract; every function cites the reference lines
 * (AaravG/negative-weight-cch) it restates.
 */
#include "oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* a + b with "no path" absorbing: the INF test comes before the addition
 * (the saturated-infinity pitfall of python/test_techniques.py:216-220). */
static inline int add_ok(int64_t a, int64_t b, int64_t* out) {
    if (a == ORC_INF || b == ORC_INF) return 0;
    *out = a + b;
    return 1;
}

static void base_values(int64_t m_plus, int64_t m, const int64_t* e_arc, const int8_t* e_up, const int32_t* w,
                        int64_t* up, int64_t* dn) {
    /* python/cch_nb.py:531-542 */
    for (int64_t a = 0; a < m_plus; a++) {
        up[a] = ORC_INF;
        dn[a] = ORC_INF;
    }
    for (int64_t k = 0; k < m; k++) {
        const int64_t a = e_arc[k];
        if (a < 0) continue;
        int64_t* slot = e_up[k] ? &up[a] : &dn[a];
        if ((int64_t)w[k] < *slot) *slot = w[k];
    }
}

void orc_customize(int64_t n, const int64_t* first, const int32_t* head, int64_t m, const int64_t* e_arc,
                   const int8_t* e_up, const int32_t* w, int64_t* up, int64_t* dn) {
    base_values(first[n], m, e_arc, e_up, w, up, dn);
    /* python/cch_nb.py:544-562: lower triangles, lowest vertex first; the arc
     * (y, z) is found by a merge pointer j over row y */
    for (int64_t x = 0; x < n; x++) {
        const int64_t s = first[x], e = first[x + 1];
        for (int64_t i = s; i < e; i++) {
            const int64_t y = head[i];
            int64_t j = first[y];
            const int64_t je = first[y + 1];
            const int64_t d_yx = dn[i], u_xy = up[i];
            for (int64_t kk = i + 1; kk < e; kk++) {
                const int32_t z = head[kk];
                while (j < je && head[j] < z) j++;
                int64_t v;
                if (add_ok(d_yx, up[kk], &v) && v < up[j]) up[j] = v; /* y -> x -> z */
                if (add_ok(dn[kk], u_xy, &v) && v < dn[j]) dn[j] = v; /* z -> x -> y */
            }
        }
    }
}

static inline void atomic_min64(int64_t* slot, int64_t v) {
    /* cpp/cch.cpp:482-493 (compare-and-swap minimum) */
    int64_t cur = __atomic_load_n(slot, __ATOMIC_RELAXED);
    while (v < cur) {
        if (__atomic_compare_exchange_n(slot, &cur, v, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) return;
    }
}

int64_t orc_customize_parallel(int64_t n, const int64_t* first, const int32_t* head, int64_t m,
                               const int64_t* e_arc, const int8_t* e_up, const int32_t* w, int64_t* up,
                               int64_t* dn, int threads) {
    /* cpp/cch.cpp:468-480: level = one more than the highest lower neighbour */
    int32_t* lvl = (int32_t*)calloc((size_t)n, sizeof(int32_t));
    int32_t maxl = 0;
    for (int64_t x = 0; x < n; x++)
        for (int64_t a = first[x]; a < first[x + 1]; a++) {
            const int64_t y = head[a];
            if (lvl[x] + 1 > lvl[y]) lvl[y] = lvl[x] + 1;
            if (lvl[y] > maxl) maxl = lvl[y];
        }
    const int64_t L = (int64_t)maxl + 1;
    int64_t* boff = (int64_t*)calloc((size_t)L + 1, sizeof(int64_t));
    int32_t* bverts = (int32_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int32_t));
    for (int64_t x = 0; x < n; x++) boff[lvl[x] + 1]++;
    for (int64_t l = 0; l < L; l++) boff[l + 1] += boff[l];
    int64_t* fill = (int64_t*)malloc((size_t)L * sizeof(int64_t));
    memcpy(fill, boff, (size_t)L * sizeof(int64_t));
    for (int64_t x = 0; x < n; x++) bverts[fill[lvl[x]]++] = (int32_t)x;
    free(fill);
    base_values(first[n], m, e_arc, e_up, w, up, dn);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    /* cpp/cch.cpp:506-528: each level's vertices in parallel (wide levels
     * only), pushing their triangles with an atomic minimum */
    for (int64_t l = 0; l < L; l++) {
        const int64_t b0 = boff[l], cnt = boff[l + 1] - b0;
        const int par = cnt >= 512;
#pragma omp parallel for schedule(dynamic, 64) if (par)
        for (int64_t bi = 0; bi < cnt; bi++) {
            const int64_t x = bverts[b0 + bi];
            const int64_t s = first[x], e = first[x + 1];
            for (int64_t i = s; i < e; i++) {
                const int64_t y = head[i];
                int64_t j = first[y];
                const int64_t je = first[y + 1];
                const int64_t d_yx = dn[i], u_xy = up[i];
                for (int64_t kk = i + 1; kk < e; kk++) {
                    const int32_t z = head[kk];
                    while (j < je && head[j] < z) j++;
                    int64_t v;
                    if (add_ok(d_yx, up[kk], &v)) atomic_min64(&up[j], v);
                    if (add_ok(dn[kk], u_xy, &v)) atomic_min64(&dn[j], v);
                }
            }
        }
    }
    free(lvl);
    free(boff);
    free(bverts);
    return L;
}

int64_t orc_negative_cycle_arcs(int64_t m_plus, const int64_t* up, const int64_t* dn) {
    /* python/cch_nb.py:566-572 (< -1e-6 is < 0 on integers; INF never sums below 0) */
    int64_t c = 0;
    for (int64_t a = 0; a < m_plus; a++) {
        int64_t v;
        if (add_ok(up[a], dn[a], &v) && v < 0) c++;
    }
    return c;
}

int64_t orc_query(int64_t s_rank, int64_t t_rank, const int64_t* first, const int32_t* head,
                  const int64_t* parent, const int64_t* up, const int64_t* dn, int64_t* df, int64_t* dr,
                  int64_t* mark, int64_t q) {
    /* python/cch_nb.py:577-615 */
    for (int64_t x = s_rank; x >= 0; x = parent[x]) {
        df[x] = ORC_INF;
        mark[x] = q;
    }
    for (int64_t x = t_rank; x >= 0; x = parent[x]) dr[x] = ORC_INF;
    df[s_rank] = 0;
    dr[t_rank] = 0;
    for (int64_t x = s_rank; x >= 0; x = parent[x]) {
        const int64_t dx = df[x];
        if (dx == ORC_INF) continue;
        for (int64_t a = first[x]; a < first[x + 1]; a++) {
            int64_t v;
            const int64_t y = head[a];
            if (add_ok(dx, up[a], &v) && v < df[y]) df[y] = v;
        }
    }
    int64_t best = ORC_INF;
    for (int64_t x = t_rank; x >= 0; x = parent[x]) {
        const int64_t dx = dr[x];
        if (dx == ORC_INF) continue;
        int64_t v;
        if (mark[x] == q && add_ok(dx, df[x], &v) && v < best) best = v;
        for (int64_t a = first[x]; a < first[x + 1]; a++) {
            const int64_t y = head[a];
            if (add_ok(dx, dn[a], &v) && v < dr[y]) dr[y] = v;
        }
    }
    return best;
}

void orc_query_batch(int64_t n, const int64_t* first, const int32_t* head, const int64_t* parent,
                     const int64_t* up, const int64_t* dn, int64_t nq, const int64_t* s_rank,
                     const int64_t* t_rank, int64_t* out, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
#pragma omp parallel
    {
        int64_t* df = (int64_t*)malloc((size_t)n * sizeof(int64_t));
        int64_t* dr = (int64_t*)malloc((size_t)n * sizeof(int64_t));
        int64_t* mark = (int64_t*)calloc((size_t)n, sizeof(int64_t));
#pragma omp for schedule(dynamic, 16)
        for (int64_t i = 0; i < nq; i++)
            out[i] = orc_query(s_rank[i], t_rank[i], first, head, parent, up, dn, df, dr, mark, i + 1);
        free(df);
        free(dr);
        free(mark);
    }
}

/* ------------------------------------------------------------ update */

typedef struct {
    int64_t* key; /* (tail << 32) | arc */
    int64_t size, cap;
} Heap;

static void heap_push(Heap* h, int64_t k) {
    if (h->size == h->cap) {
        h->cap = h->cap ? 2 * h->cap : 1024;
        h->key = (int64_t*)realloc(h->key, (size_t)h->cap * sizeof(int64_t));
    }
    int64_t i = h->size++;
    while (i > 0) {
        const int64_t p = (i - 1) / 2;
        if (h->key[p] <= k) break;
        h->key[i] = h->key[p];
        i = p;
    }
    h->key[i] = k;
}

static int64_t heap_pop(Heap* h) {
    const int64_t top = h->key[0];
    const int64_t last = h->key[--h->size];
    int64_t i = 0;
    while (1) {
        int64_t c = 2 * i + 1;
        if (c >= h->size) break;
        if (c + 1 < h->size && h->key[c + 1] < h->key[c]) c++;
        if (h->key[c] >= last) break;
        h->key[i] = h->key[c];
        i = c;
    }
    if (h->size) h->key[i] = last;
    return top;
}

static int64_t find_arc(const int64_t* first, const int32_t* head, int64_t lo, int64_t hi_excl, int32_t z) {
    int64_t a = lo, b = hi_excl;
    while (a < b) {
        const int64_t mid = (a + b) / 2;
        if (head[mid] < z) a = mid + 1;
        else b = mid;
    }
    (void)first;
    return (a < hi_excl && head[a] == z) ? a : -1;
}

/* python/cch.py:289-347 build_update_index, built once per topology as the
 * reference does (lazily, on the first update_edges): tails, original arcs
 * per arc, and (in place of the stored triangle lists) downward lists. The
 * queued set of one update is an epoch stamp per arc, so no call clears it. */
struct OrcUpdateIndex {
    int64_t n, m, mp;
    const int64_t* first;
    const int32_t* head;
    const int64_t* e_arc;
    const int8_t* e_up;
    int32_t* tail;
    int64_t *aeoff, *aeidx, *doff, *darc;
    uint32_t* stamp;
    uint32_t epoch;
};

OrcUpdateIndex* orc_update_index(int64_t n, const int64_t* first, const int32_t* head, int64_t m,
                                 const int64_t* e_arc, const int8_t* e_up) {
    OrcUpdateIndex* X = (OrcUpdateIndex*)calloc(1, sizeof(OrcUpdateIndex));
    const int64_t mp = first[n];
    X->n = n;
    X->m = m;
    X->mp = mp;
    X->first = first;
    X->head = head;
    X->e_arc = e_arc;
    X->e_up = e_up;
    X->tail = (int32_t*)malloc((size_t)(mp > 0 ? mp : 1) * sizeof(int32_t));
    for (int64_t x = 0; x < n; x++)
        for (int64_t a = first[x]; a < first[x + 1]; a++) X->tail[a] = (int32_t)x;
    X->aeoff = (int64_t*)calloc((size_t)mp + 1, sizeof(int64_t));
    for (int64_t j = 0; j < m; j++)
        if (e_arc[j] >= 0) X->aeoff[e_arc[j] + 1]++;
    for (int64_t a = 0; a < mp; a++) X->aeoff[a + 1] += X->aeoff[a];
    X->aeidx = (int64_t*)malloc((size_t)(X->aeoff[mp] > 0 ? X->aeoff[mp] : 1) * sizeof(int64_t));
    int64_t* fill = (int64_t*)malloc((size_t)(mp > 0 ? mp : 1) * sizeof(int64_t));
    memcpy(fill, X->aeoff, (size_t)mp * sizeof(int64_t));
    for (int64_t j = 0; j < m; j++)
        if (e_arc[j] >= 0) X->aeidx[fill[e_arc[j]]++] = j;
    free(fill);
    X->doff = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
    for (int64_t a = 0; a < mp; a++) X->doff[head[a] + 1]++;
    for (int64_t v = 0; v < n; v++) X->doff[v + 1] += X->doff[v];
    X->darc = (int64_t*)malloc((size_t)(mp > 0 ? mp : 1) * sizeof(int64_t));
    int64_t* dfill = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    memcpy(dfill, X->doff, (size_t)n * sizeof(int64_t));
    for (int64_t a = 0; a < mp; a++) X->darc[dfill[head[a]]++] = a;
    free(dfill);
    X->stamp = (uint32_t*)calloc((size_t)mp + 1, sizeof(uint32_t));
    X->epoch = 0;
    return X;
}

void orc_update_index_free(OrcUpdateIndex* X) {
    if (!X) return;
    free(X->tail);
    free(X->aeoff);
    free(X->aeidx);
    free(X->doff);
    free(X->darc);
    free(X->stamp);
    free(X);
}

void orc_update_indexed(OrcUpdateIndex* X, int32_t* w, int64_t* up, int64_t* dn, int64_t k,
                        const int64_t* edge_idx, const int32_t* new_w, int64_t* stats, int64_t* changed) {
    const int64_t* first = X->first;
    const int32_t* head = X->head;
    const int64_t* e_arc = X->e_arc;
    const int8_t* e_up = X->e_up;
    const int32_t* tail = X->tail;
    if (++X->epoch == 0) { /* stamps wrapped: start over */
        memset(X->stamp, 0, (size_t)(X->mp + 1) * sizeof(uint32_t));
        X->epoch = 1;
    }
    const uint32_t ep = X->epoch;
    uint32_t* queued = X->stamp;
    /* python/cch.py:357-371: new weights; touched arcs */
    Heap h = {0, 0, 0};
    for (int64_t j = 0; j < k; j++) w[edge_idx[j]] = new_w[j];
    for (int64_t j = 0; j < k; j++) {
        const int64_t a = e_arc[edge_idx[j]];
        if (a >= 0 && queued[a] != ep) {
            queued[a] = ep;
            heap_push(&h, ((int64_t)tail[a] << 32) | a);
        }
    }
    /* python/cch.py:376-401: pop lowest tail first, recompute from the base
     * value and the lower triangles, queue the upper arcs on a change */
    int64_t evaluated = 0, nchanged = 0, neg = 0;
    while (h.size) {
        const int64_t c = heap_pop(&h) & 0xffffffffLL;
        evaluated++;
        int64_t nu = ORC_INF, nd = ORC_INF;
        for (int64_t j = X->aeoff[c]; j < X->aeoff[c + 1]; j++) {
            const int64_t e = X->aeidx[j];
            if (e_up[e]) {
                if ((int64_t)w[e] < nu) nu = w[e];
            } else if ((int64_t)w[e] < nd) {
                nd = w[e];
            }
        }
        const int64_t y = tail[c];
        const int32_t z = head[c];
        for (int64_t j = X->doff[y]; j < X->doff[y + 1]; j++) {
            const int64_t a = X->darc[j];
            const int64_t b = find_arc(first, head, a + 1, first[tail[a] + 1], z);
            if (b < 0) continue;
            int64_t v;
            if (add_ok(dn[a], up[b], &v) && v < nu) nu = v;
            if (add_ok(dn[b], up[a], &v) && v < nd) nd = v;
        }
        if (nu == up[c] && nd == dn[c]) continue;
        up[c] = nu;
        dn[c] = nd;
        if (changed) changed[nchanged] = c;
        nchanged++;
        {
            int64_t v;
            if (add_ok(nu, nd, &v) && v < 0) neg++;
        }
        for (int64_t kk = first[y]; kk < first[y + 1]; kk++) {
            if (kk == c) continue;
            const int32_t v = head[kk];
            const int32_t lo = v < z ? v : z, hi = v < z ? z : v;
            const int64_t c2 = find_arc(first, head, first[lo], first[lo + 1], hi);
            if (c2 >= 0 && queued[c2] != ep) {
                queued[c2] = ep;
                heap_push(&h, ((int64_t)lo << 32) | c2);
            }
        }
    }
    stats[0] = evaluated;
    stats[1] = nchanged;
    stats[2] = neg;
    free(h.key);
}

void orc_update(int64_t n, const int64_t* first, const int32_t* head, int64_t m, const int64_t* e_arc,
                const int8_t* e_up, int32_t* w, int64_t* up, int64_t* dn, int64_t k, const int64_t* edge_idx,
                const int32_t* new_w, int64_t* stats, int64_t* changed) {
    OrcUpdateIndex* X = orc_update_index(n, first, head, m, e_arc, e_up);
    orc_update_indexed(X, w, up, dn, k, edge_idx, new_w, stats, changed);
    orc_update_index_free(X);
}

/* ------------------------------------------------------------ Bellman-Ford */

static int spfa(int64_t n, const int64_t* off, const int32_t* tgt, const int32_t* w, int64_t* dist,
                unsigned char* inq, int64_t* queue, int64_t* count, int64_t nsrc, const int64_t* src) {
    /* python/search.py:8-29, queue-based; a vertex entering the queue n
     * times proves a negative cycle */
    const int64_t cap = n + 1;
    int64_t qh = 0, qt = 0, size = 0;
    for (int64_t i = 0; i < nsrc; i++) {
        queue[qt] = src[i];
        qt = (qt + 1) % cap;
        size++;
        inq[src[i]] = 1;
    }
    while (size > 0) {
        const int64_t u = queue[qh];
        qh = (qh + 1) % cap;
        size--;
        inq[u] = 0;
        const int64_t du = dist[u];
        for (int64_t k = off[u]; k < off[u + 1]; k++) {
            const int64_t v = tgt[k];
            const int64_t nd = du + (int64_t)w[k];
            if (nd < dist[v]) {
                dist[v] = nd;
                if (!inq[v]) {
                    if (++count[v] >= n + 1) return 1;
                    inq[v] = 1;
                    queue[qt] = v;
                    qt = (qt + 1) % cap;
                    size++;
                }
            }
        }
    }
    return 0;
}

int orc_bellman_ford(int64_t n, const int64_t* off, const int32_t* tgt, const int32_t* w, int64_t s,
                     int64_t* dist) {
    unsigned char* inq = (unsigned char*)calloc((size_t)n, 1);
    int64_t* queue = (int64_t*)malloc((size_t)(n + 1) * sizeof(int64_t));
    int64_t* count = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    for (int64_t v = 0; v < n; v++) dist[v] = ORC_INF;
    dist[s] = 0;
    /* INF never relaxes: only finite labels enter the queue */
    const int r = spfa(n, off, tgt, w, dist, inq, queue, count, 1, &s);
    free(inq);
    free(queue);
    free(count);
    return r;
}

void orc_potential(int64_t n, const int64_t* first, const int32_t* head, const int64_t* up, const int64_t* dn,
                   int64_t* p) {
    /* cpp/cch.cpp:636-644: upward pass, increasing rank */
    for (int64_t x = 0; x < n; x++) p[x] = 0;
    for (int64_t x = 0; x < n; x++) {
        const int64_t px = p[x];
        for (int64_t a = first[x]; a < first[x + 1]; a++) {
            int64_t v;
            if (add_ok(px, up[a], &v) && v < p[head[a]]) p[head[a]] = v;
        }
    }
    /* cpp/cch.cpp:645-652: downward pass, decreasing rank */
    for (int64_t x = n - 1; x >= 0; x--) {
        int64_t best = p[x];
        for (int64_t a = first[x]; a < first[x + 1]; a++) {
            int64_t v;
            if (add_ok(p[head[a]], dn[a], &v) && v < best) best = v;
        }
        p[x] = best;
    }
}

int orc_virtual_source_potential(int64_t n, const int64_t* off, const int32_t* tgt, const int32_t* w,
                                 int64_t* p) {
    unsigned char* inq = (unsigned char*)calloc((size_t)n, 1);
    int64_t* queue = (int64_t*)malloc((size_t)(n + 1) * sizeof(int64_t));
    int64_t* count = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    int64_t* src = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    for (int64_t v = 0; v < n; v++) {
        src[v] = v;
        p[v] = 0;
    }
    int r = 0;
    for (int64_t u = 0; u < n && !r; u++)
        for (int64_t k = off[u]; k < off[u + 1]; k++)
            if (tgt[k] == u && w[k] < 0) r = 1;
    if (!r) r = spfa(n, off, tgt, w, p, inq, queue, count, n, src);
    free(inq);
    free(queue);
    free(count);
    free(src);
    return r;
}

static int64_t arc_of(const int64_t* first, const int32_t* head, int64_t lo, int64_t hi) {
    int64_t a = first[lo], b = first[lo + 1];
    while (a < b) {
        const int64_t mid = (a + b) / 2;
        if (head[mid] < hi) a = mid + 1;
        else b = mid;
    }
    return (a < first[lo + 1] && head[a] == hi) ? a : -1;
}

int64_t orc_query_path(int64_t n, const int64_t* first, const int32_t* head, const int64_t* parent,
                       const int32_t* tail, const int64_t* doff, const int32_t* darc, const int64_t* up,
                       const int64_t* dn, int64_t s, int64_t t, int64_t* dist, int64_t* path, int64_t cap) {
    int64_t* df = (int64_t*)malloc((size_t)n * sizeof(int64_t));
    int64_t* dr = (int64_t*)malloc((size_t)n * sizeof(int64_t));
    int64_t* pf = (int64_t*)malloc((size_t)n * sizeof(int64_t));
    int64_t* pr = (int64_t*)malloc((size_t)n * sizeof(int64_t));
    unsigned char* anc = (unsigned char*)calloc((size_t)n, 1);
    int64_t* legs = (int64_t*)malloc((size_t)(4 * n + 4) * sizeof(int64_t));
    int64_t* stack = (int64_t*)malloc((size_t)(4 * n + 4) * sizeof(int64_t));
    int64_t len = 0, nlegs = 0;
    for (int64_t v = 0; v < n; v++) {
        df[v] = dr[v] = ORC_INF;
        pf[v] = pr[v] = -1;
    }
    /* python/cch.py:413-440: sweeps recording the first arc reaching each label */
    df[s] = 0;
    dr[t] = 0;
    for (int64_t x = s; x >= 0; x = parent[x])
        if (df[x] != ORC_INF)
            for (int64_t a = first[x]; a < first[x + 1]; a++) {
                int64_t v;
                if (add_ok(df[x], up[a], &v) && v < df[head[a]]) {
                    df[head[a]] = v;
                    pf[head[a]] = a;
                }
            }
    for (int64_t x = t; x >= 0; x = parent[x])
        if (dr[x] != ORC_INF)
            for (int64_t a = first[x]; a < first[x + 1]; a++) {
                int64_t v;
                if (add_ok(dr[x], dn[a], &v) && v < dr[head[a]]) {
                    dr[head[a]] = v;
                    pr[head[a]] = a;
                }
            }
    /* :441-452: the lowest common ancestor reaching the minimum */
    for (int64_t x = t; x >= 0; x = parent[x]) anc[x] = 1;
    int64_t best = ORC_INF, peak = -1;
    for (int64_t x = s; x >= 0; x = parent[x]) {
        int64_t v;
        if (anc[x] && add_ok(df[x], dr[x], &v) && v < best) {
            best = v;
            peak = x;
        }
    }
    *dist = best;
    if (peak >= 0) {
        /* :455-467: the shortcut legs, s -> peak, then peak -> t */
        for (int64_t x = peak; x != s;) {
            const int64_t v = tail[pf[x]];
            legs[2 * nlegs] = v;
            legs[2 * nlegs + 1] = x;
            nlegs++;
            x = v;
        }
        for (int64_t i = 0, j = nlegs - 1; i < j; i++, j--) {
            const int64_t a0 = legs[2 * i], a1 = legs[2 * i + 1];
            legs[2 * i] = legs[2 * j];
            legs[2 * i + 1] = legs[2 * j + 1];
            legs[2 * j] = a0;
            legs[2 * j + 1] = a1;
        }
        for (int64_t x = peak; x != t;) {
            const int64_t v = tail[pr[x]];
            legs[2 * nlegs] = x;
            legs[2 * nlegs + 1] = v;
            nlegs++;
            x = v;
        }
        /* :468-470, 482-501: unpack every leg */
#define PUSH_VERTEX(v) do { if (len < cap) path[len] = (v); len++; } while (0)
        PUSH_VERTEX(nlegs ? legs[0] : s);
        for (int64_t l = 0; l < nlegs; l++) {
            int64_t sp = 0;
            stack[sp++] = legs[2 * l];
            stack[sp++] = legs[2 * l + 1];
            while (sp > 0) {
                const int64_t w = stack[--sp], v = stack[--sp];
                const int64_t lo = v < w ? v : w, hi = v < w ? w : v;
                const int64_t a = arc_of(first, head, lo, hi);
                const int64_t cost = v < w ? up[a] : dn[a];
                int64_t mid = -1;
                for (int64_t j = doff[lo]; j < doff[lo + 1] && mid < 0; j++) {
                    const int64_t xl = darc[j], x = tail[xl];
                    const int64_t xh = arc_of(first, head, x, hi);
                    if (xh < 0) continue;
                    const int64_t av = v == lo ? xl : xh, aw = w == lo ? xl : xh;
                    int64_t c;
                    if (add_ok(dn[av], up[aw], &c) && c == cost) mid = x;
                }
                if (mid < 0) {
                    PUSH_VERTEX(w);
                } else {
                    stack[sp++] = mid;
                    stack[sp++] = w;
                    stack[sp++] = v;
                    stack[sp++] = mid;
                }
            }
        }
#undef PUSH_VERTEX
    }
    free(df);
    free(dr);
    free(pf);
    free(pr);
    free(anc);
    free(legs);
    free(stack);
    return len > cap ? -len : len;
}

int orc_has_negative_cycle(int64_t n, const int64_t* off, const int32_t* tgt, const int32_t* w) {
    int64_t* dist = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    unsigned char* inq = (unsigned char*)calloc((size_t)n, 1);
    int64_t* queue = (int64_t*)malloc((size_t)(n + 1) * sizeof(int64_t));
    int64_t* count = (int64_t*)calloc((size_t)n, sizeof(int64_t));
    int64_t* src = (int64_t*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int64_t));
    for (int64_t v = 0; v < n; v++) src[v] = v;
    /* self-loops with negative weight are negative cycles too */
    int r = 0;
    for (int64_t u = 0; u < n && !r; u++)
        for (int64_t k = off[u]; k < off[u + 1]; k++)
            if (tgt[k] == u && w[k] < 0) r = 1;
    if (!r) r = spfa(n, off, tgt, w, dist, inq, queue, count, n, src);
    free(dist);
    free(inq);
    free(queue);
    free(count);
    free(src);
    return r;
}
