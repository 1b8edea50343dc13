/*
 * CPU oracle for battery-constrained CCH profiles - TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of python/cch_nb_battery.py (AaravG/negative-weight-
 * cch), the Numba battery customization and query, in the same float64
 * operations and the same order, so that its profiles are the reference's
 * piece for piece:
 *
 *   * a piece is (in, cost, out): f(b) = min(out, b - cost) for b >= in,
 *     infeasible below in (python/cch_battery.py:1-40);
 *   * a shortcut direction d = 2*arc + (0 up, 1 down) holds a profile, the
 *     pieces left after merging every candidate in turn: a candidate that an
 *     existing piece dominates is dropped, otherwise the pieces it dominates
 *     are removed (order kept) and it is appended.
 *
 * Only tests and the benchmark's CPU legs load this library.
 */
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "oracle.h"

#define BAT_EPS 1e-9
#define BAT_NEG (-__builtin_inf())

typedef struct {
    double i, c, o;
} Piece;

typedef struct {
    int32_t n, cap;
    Piece* p;
} Prof;

typedef struct {
    int64_t nd, total;
    Prof* prof;
} BatteryProfiles;

/* python/cch_nb_battery.py:16-44: does f dominate g on [0, M]? The
 * difference of two such functions is extreme at g's feasibility start, at M
 * or at either function's breakpoint. */
static int dominates(const Piece* f, const Piece* g, double M) {
    if (f->i > g->i + BAT_EPS) return 0;
    const double lo = g->i - BAT_EPS, hi = M + BAT_EPS;
    const double bs[4] = {g->i, M, f->o + f->c, g->o + g->c};
    for (int t = 0; t < 4; t++) {
        const double b = bs[t];
        if (lo <= b && b <= hi) {
            if (b < f->i - BAT_EPS) return 0;
            double vf = b - f->c;
            if (f->o < vf) vf = f->o;
            double vg = b - g->c;
            if (g->o < vg) vg = g->o;
            if (vf < vg - BAT_EPS) return 0;
        }
    }
    return 1;
}

/* python/cch_nb_battery.py:159-173: f then g; 0 if infeasible. */
static int compose(const Piece* f, const Piece* g, double M, Piece* h) {
    if (f->o < g->i - BAT_EPS) return 0;
    const double hi = f->i > g->i + f->c ? f->i : g->i + f->c;
    if (hi > M + BAT_EPS) return 0;
    const double hc = f->c + g->c;
    double ho = g->o;
    if (f->o - g->c < ho) ho = f->o - g->c;
    if (M - hc < ho) ho = M - hc;
    h->i = hi;
    h->c = hc;
    h->o = ho;
    return 1;
}

/* python/cch_nb_battery.py:186-254 (storage aside): the merge of one
 * candidate. Returns 0 on allocation failure. */
static int merge(Prof* P, const Piece* h, double M) {
    for (int32_t t = 0; t < P->n; t++)
        if (dominates(&P->p[t], h, M)) return 1;
    int32_t k = 0;
    for (int32_t t = 0; t < P->n; t++)
        if (!dominates(h, &P->p[t], M)) P->p[k++] = P->p[t];
    if (k == P->cap) {
        const int32_t cap = P->cap ? 2 * P->cap : 1;
        Piece* q = (Piece*)realloc(P->p, (size_t)cap * sizeof(Piece));
        if (!q) return 0;
        P->p = q;
        P->cap = cap;
    }
    P->p[k] = *h;
    P->n = k + 1;
    return 1;
}

void orc_battery_free(void* handle) {
    BatteryProfiles* B = (BatteryProfiles*)handle;
    if (!B) return;
    for (int64_t d = 0; d < B->nd; d++) free(B->prof[d].p);
    free(B->prof);
    free(B);
}

void* orc_battery_customize(int64_t n, const int64_t* first, const int32_t* head, int64_t m, const int64_t* e_arc,
                            const int8_t* e_up, const double* w, double M) {
    const int64_t m_plus = first[n];
    BatteryProfiles* B = (BatteryProfiles*)calloc(1, sizeof(BatteryProfiles));
    if (!B) return NULL;
    B->nd = 2 * m_plus;
    B->prof = (Prof*)calloc((size_t)(B->nd > 0 ? B->nd : 1), sizeof(Prof));
    if (!B->prof) {
        free(B);
        return NULL;
    }
    int ok = 1;
    /* python/cch_nb_battery.py:67-82: the original arcs, in input order */
    for (int64_t k = 0; k < m && ok; k++) {
        const int64_t a = e_arc[k];
        if (a < 0) continue;
        const double c = w[k];
        Piece h;
        if (c >= 0) {
            if (c > M) continue;
            h.i = c;
            h.c = c;
            h.o = M - c;
        } else {
            h.i = 0.0;
            h.c = c;
            h.o = M;
        }
        ok = merge(&B->prof[2 * a + (e_up[k] ? 0 : 1)], &h, M);
    }
    /* python/cch_nb_battery.py:84-182: lower triangles (x; y, z), x ascending:
     * y -> x -> z = down(x,y) then up(x,z) into up(y,z), and
     * z -> x -> y = down(x,z) then up(x,y) into down(y,z). */
    Piece* sa = NULL;
    Piece* sb = NULL;
    int32_t sa_cap = 0, sb_cap = 0;
    for (int64_t x = 0; x < n && ok; x++) {
        const int64_t s = first[x], e = first[x + 1];
        for (int64_t i = s; i < e && ok; i++) {
            const int32_t y = head[i];
            int64_t j = first[y];
            const int64_t je = first[y + 1];
            for (int64_t kk = i + 1; kk < e && ok; kk++) {
                const int32_t z = head[kk];
                while (j < je && head[j] < z) j++;
                for (int side = 0; side < 2 && ok; side++) {
                    const int64_t da = side == 0 ? 2 * i + 1 : 2 * kk + 1;
                    const int64_t db = side == 0 ? 2 * kk : 2 * i;
                    const int64_t dt = side == 0 ? 2 * j : 2 * j + 1;
                    const Prof* A = &B->prof[da];
                    const Prof* Bp = &B->prof[db];
                    if (A->n == 0 || Bp->n == 0) continue;
                    /* sources are copied: the target may be reallocated */
                    if (A->n > sa_cap) {
                        free(sa);
                        sa_cap = 2 * A->n;
                        sa = (Piece*)malloc((size_t)sa_cap * sizeof(Piece));
                    }
                    if (Bp->n > sb_cap) {
                        free(sb);
                        sb_cap = 2 * Bp->n;
                        sb = (Piece*)malloc((size_t)sb_cap * sizeof(Piece));
                    }
                    if (!sa || !sb) {
                        ok = 0;
                        break;
                    }
                    const int32_t na = A->n, nb = Bp->n;
                    memcpy(sa, A->p, (size_t)na * sizeof(Piece));
                    memcpy(sb, Bp->p, (size_t)nb * sizeof(Piece));
                    for (int32_t ta = 0; ta < na && ok; ta++)
                        for (int32_t tb = 0; tb < nb && ok; tb++) {
                            Piece h;
                            if (compose(&sa[ta], &sb[tb], M, &h)) ok = merge(&B->prof[dt], &h, M);
                        }
                }
            }
        }
    }
    free(sa);
    free(sb);
    if (!ok) {
        orc_battery_free(B);
        return NULL;
    }
    int64_t total = 0;
    for (int64_t d = 0; d < B->nd; d++) total += B->prof[d].n;
    B->total = total;
    return B;
}

int64_t orc_battery_pieces(const void* handle) { return ((const BatteryProfiles*)handle)->total; }

void orc_battery_export(const void* handle, int32_t* cnt, int64_t* off, double* pieces) {
    const BatteryProfiles* B = (const BatteryProfiles*)handle;
    int64_t pos = 0;
    for (int64_t d = 0; d < B->nd; d++) {
        const Prof* P = &B->prof[d];
        cnt[d] = P->n;
        off[d] = pos;
        for (int32_t t = 0; t < P->n; t++) {
            pieces[3 * (pos + t)] = P->p[t].i;
            pieces[3 * (pos + t) + 1] = P->p[t].c;
            pieces[3 * (pos + t) + 2] = P->p[t].o;
        }
        pos += P->n;
    }
    off[B->nd] = pos;
}

/* python/cch_nb_battery.py:272-293: the profile's value at charge b. */
static double eval_profile(const int32_t* cnt, const int64_t* off, const double* pieces, int64_t d, double b) {
    double best = BAT_NEG;
    const double* p = pieces + 3 * off[d];
    for (int32_t t = 0; t < cnt[d]; t++, p += 3) {
        if (b >= p[0] - BAT_EPS) {
            double v = b - p[1];
            if (p[2] < v) v = p[2];
            if (v > best) best = v;
        }
    }
    return best;
}

double orc_battery_query(int64_t s_rank, int64_t t_rank, double b0, const int64_t* first, const int32_t* head,
                         const int64_t* parent, const int32_t* cnt, const int64_t* off, const double* pieces,
                         double* soc, double* dsoc, int64_t* mark, int64_t q) {
    /* python/cch_nb_battery.py:296-343 */
    for (int64_t x = s_rank; x >= 0; x = parent[x]) {
        soc[x] = BAT_NEG;
        mark[x] = q;
    }
    int64_t L = 0;
    for (int64_t x = t_rank; x >= 0; x = parent[x]) {
        dsoc[x] = BAT_NEG;
        L++;
    }
    soc[s_rank] = b0;
    for (int64_t x = s_rank; x >= 0; x = parent[x]) {
        const double bx = soc[x];
        if (bx > BAT_NEG)
            for (int64_t a = first[x]; a < first[x + 1]; a++) {
                const double v = eval_profile(cnt, off, pieces, 2 * a, bx);
                if (v > soc[head[a]]) soc[head[a]] = v;
            }
    }
    int64_t* chain = (int64_t*)malloc((size_t)(L > 0 ? L : 1) * sizeof(int64_t));
    if (!chain) return BAT_NEG;
    L = 0;
    for (int64_t x = t_rank; x >= 0; x = parent[x]) chain[L++] = x;
    for (int64_t idx = L - 1; idx >= 0; idx--) {
        const int64_t x = chain[idx];
        double best = mark[x] == q ? soc[x] : BAT_NEG;
        for (int64_t a = first[x]; a < first[x + 1]; a++) {
            const double by = dsoc[head[a]];
            if (by > BAT_NEG) {
                const double v = eval_profile(cnt, off, pieces, 2 * a + 1, by);
                if (v > best) best = v;
            }
        }
        dsoc[x] = best;
    }
    free(chain);
    return dsoc[t_rank];
}

void orc_battery_query_batch(int64_t n, const int64_t* first, const int32_t* head, const int64_t* parent,
                             const int32_t* cnt, const int64_t* off, const double* pieces, int64_t nq,
                             const int64_t* s_rank, const int64_t* t_rank, const double* b0, double* out,
                             int threads) {
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_max_threads();
#pragma omp parallel num_threads(threads)
#endif
    {
        double* soc = (double*)malloc((size_t)n * sizeof(double));
        double* dsoc = (double*)malloc((size_t)n * sizeof(double));
        int64_t* mark = (int64_t*)calloc((size_t)n, sizeof(int64_t));
        if (soc && dsoc && mark) {
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
            for (int64_t i = 0; i < nq; i++)
                out[i] = orc_battery_query(s_rank[i], t_rank[i], b0[i], first, head, parent, cnt, off, pieces, soc,
                                           dsoc, mark, i + 1);
        }
        free(soc);
        free(dsoc);
        free(mark);
    }
}

void orc_battery_label_correcting(int64_t n, const int64_t* off, const int32_t* tgt, const double* w, double M,
                                  int64_t s, double b0, double* soc) {
    /* python/cch_nb_battery.py:316-351: FIFO label correcting on the
     * original graph; exact when no cycle gains charge. */
    for (int64_t v = 0; v < n; v++) soc[v] = BAT_NEG;
    const int64_t cap = n + 1;
    int64_t* q = (int64_t*)malloc((size_t)cap * sizeof(int64_t));
    char* inq = (char*)calloc((size_t)(n > 0 ? n : 1), 1);
    if (!q || !inq) {
        free(q);
        free(inq);
        return;
    }
    int64_t qh = 0, qt = 1, size = 1;
    q[0] = s;
    soc[s] = b0;
    inq[s] = 1;
    while (size > 0) {
        const int64_t u = q[qh];
        qh = (qh + 1) % cap;
        size--;
        inq[u] = 0;
        const double bu = soc[u];
        for (int64_t k = off[u]; k < off[u + 1]; k++) {
            const double c = w[k];
            double nb;
            if (c >= 0) {
                if (bu < c - BAT_EPS) continue;
                nb = bu - c;
            } else {
                nb = bu - c;
                if (nb > M) nb = M;
            }
            const int64_t v = tgt[k];
            if (nb > soc[v] + BAT_EPS) {
                soc[v] = nb;
                if (!inq[v]) {
                    inq[v] = 1;
                    q[qt] = v;
                    qt = (qt + 1) % cap;
                    size++;
                }
            }
        }
    }
    free(q);
    free(inq);
}
