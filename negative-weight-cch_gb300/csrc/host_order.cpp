// Weight-independent preprocessing that stays on the host: undirected graph,
// nested-dissection order, symbolic contraction (chordal completion in rank
// space) and the mapping of original arcs onto shortcut arcs.
//
// Mirrors the roles of python/cch_nb.py undirected_csr (cch_nb.py:22-71),
// nested_dissection (cch_nb.py:336-426), symbolic (cch_nb.py:431-481) and
// edge_arcs (cch_nb.py:496-514) of the reference. The ordering is a fresh
// implementation of inertial-flow bisection (Schild & Sommer, "On Balanced
// Separators in Road Networks", SEA 2015): project the vertices of a cell on
// a direction, take the first and last quarter as source and sink sets, and
// cut the cell with a minimum vertex cut (Dinic max-flow on the node-split
// graph). Cells are independent, so they are processed by a thread pool; the
// result does not depend on the schedule.
//
// Symbolic contraction produces the unique fill graph of the order, so for the
// same order it returns exactly the reference's first/head/parent.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <condition_variable>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "host_internal.h"

namespace nwcch_host {

using std::vector;

// ---------------------------------------------------------------- undirected

void undirected_csr(int64_t n, const int64_t* off, const int32_t* tgt, vector<int64_t>& noff,
                    vector<int32_t>& nbr) {
    vector<int64_t> deg(n + 1, 0);
    for (int64_t u = 0; u < n; u++)
        for (int64_t k = off[u]; k < off[u + 1]; k++) {
            const int64_t v = tgt[k];
            if (v != u) {
                deg[u + 1]++;
                deg[v + 1]++;
            }
        }
    for (int64_t i = 0; i < n; i++) deg[i + 1] += deg[i];
    vector<int32_t> tmp(deg[n]);
    vector<int64_t> fill(deg.begin(), deg.end() - 1);
    for (int64_t u = 0; u < n; u++)
        for (int64_t k = off[u]; k < off[u + 1]; k++) {
            const int64_t v = tgt[k];
            if (v != u) {
                tmp[fill[u]++] = (int32_t)v;
                tmp[fill[v]++] = (int32_t)u;
            }
        }
    noff.assign(n + 1, 0);
    nbr.clear();
    nbr.reserve(deg[n]);
    for (int64_t u = 0; u < n; u++) {
        int32_t* b = tmp.data() + deg[u];
        int32_t* e = tmp.data() + deg[u + 1];
        std::sort(b, e);
        int32_t prev = -1;
        for (int32_t* p = b; p < e; p++)
            if (*p != prev) {
                nbr.push_back(*p);
                prev = *p;
            }
        noff[u + 1] = (int64_t)nbr.size();
    }
}

// ---------------------------------------------------------------- ordering

namespace {

// A cell of the dissection: its vertices and the rank range [lo, lo+size) it
// owns in the final order.
struct Cell {
    vector<int32_t> verts;
    int64_t lo;
};

// Local (cell-restricted) undirected graph: vertices 0..m-1, CSR adjacency,
// and for every slot the id of its undirected edge plus the orientation.
struct LocalGraph {
    int32_t m = 0;
    vector<int64_t> off;
    vector<int32_t> adj;
    vector<int64_t> eid;   // undirected edge id of each slot
    vector<int8_t> fwd;    // 1 if the slot goes from lower to higher local id
    int64_t edges = 0;
};

enum Role : int8_t { NORMAL = 0, SOURCE = 1, SINK = 2 };

struct CutResult {
    bool ok = false;
    vector<int32_t> sep, a, b;  // local ids
};

// Minimum vertex cut between the sources and sinks of `role` on the node-split
// graph of `g` (unit capacity on normal vertices, unbounded on sources/sinks
// and on edges). Node 2v is the in-copy of v, 2v+1 its out-copy.
class VertexCut {
  public:
    VertexCut(const LocalGraph& g, const vector<int8_t>& role) : g_(g), role_(role) {
        const int32_t m = g.m;
        through_.assign(m, 0);
        flow_.assign(g.edges, 0);
        level_.assign(2 * (size_t)m, 0);
        seen_.assign(2 * (size_t)m, 0);
        ptr_.assign(2 * (size_t)m, 0);
        // only sources with a non-source neighbour can start a path
        for (int32_t v = 0; v < m; v++) {
            if (role[v] != SOURCE) continue;
            for (int64_t j = g.off[v]; j < g.off[v + 1]; j++)
                if (role[g.adj[j]] != SOURCE) {
                    frontier_.push_back(v);
                    break;
                }
        }
    }

    CutResult run() {
        while (bfs()) blocking_flow();
        return extract();
    }

  private:
    const LocalGraph& g_;
    const vector<int8_t>& role_;
    vector<int8_t> through_;   // unit flow through a normal vertex (in -> out)
    vector<int8_t> flow_;      // flow on an undirected edge, + from lower to higher id
    vector<int32_t> level_;    // BFS depth, valid where seen_ == phase_
    vector<int32_t> seen_;
    int32_t phase_ = 0;
    vector<int64_t> ptr_;
    vector<int64_t> queue_;
    vector<int32_t> frontier_;

    // Sources are the super-source: always reached, at depth 0.
    bool reached(int64_t x) const { return role_[x >> 1] == SOURCE || seen_[x] == phase_; }
    int32_t depth(int64_t x) const { return role_[x >> 1] == SOURCE ? 0 : level_[x]; }
    void reach(int64_t x, int32_t d) {
        seen_[x] = phase_;
        level_[x] = d;
        queue_.push_back(x);
    }

    // flow on the slot j (from its owner vertex towards adj[j])
    int flow_on(int64_t j) const { return g_.fwd[j] ? flow_[g_.eid[j]] : -flow_[g_.eid[j]]; }
    void push_on(int64_t j, int d) {
        if (g_.fwd[j]) flow_[g_.eid[j]] += (int8_t)d;
        else flow_[g_.eid[j]] -= (int8_t)d;
    }

    // Residual arc number `a` out of node x: a == 0 is the internal arc, a >= 1
    // the (a-1)-th adjacency slot. Returns the head node, or -1 if saturated.
    int64_t arc_head(int64_t x, int64_t a) const {
        const int32_t v = (int32_t)(x >> 1);
        const bool out = x & 1;
        if (a == 0) {
            if (role_[v] != NORMAL) return out ? 2 * (int64_t)v : 2 * (int64_t)v + 1;
            if (out) return through_[v] ? 2 * (int64_t)v : -1;
            return through_[v] ? -1 : 2 * (int64_t)v + 1;
        }
        const int64_t j = g_.off[v] + a - 1;
        const int32_t u = g_.adj[j];
        if (out) return 2 * (int64_t)u;                    // out(v) -> in(u), unbounded
        return flow_on(j) < 0 ? 2 * (int64_t)u + 1 : -1;   // in(v) -> out(u) undoes u->v flow
    }

    int64_t degree(int64_t x) const {
        const int32_t v = (int32_t)(x >> 1);
        return g_.off[v + 1] - g_.off[v];
    }

    // Level graph from the sources; true if a sink was reached.
    bool bfs() {
        phase_++;
        queue_.clear();
        for (int32_t v : frontier_) {
            queue_.push_back(2 * (int64_t)v);
            queue_.push_back(2 * (int64_t)v + 1);
        }
        bool hit = false;
        for (size_t qh = 0; qh < queue_.size(); qh++) {
            const int64_t x = queue_[qh];
            if (role_[x >> 1] == SINK) {
                hit = true;
                continue;
            }
            const int32_t dx = depth(x);
            const int64_t deg = degree(x);
            for (int64_t a = 0; a <= deg; a++) {
                const int64_t y = arc_head(x, a);
                if (y >= 0 && !reached(y)) reach(y, dx + 1);
            }
        }
        return hit;
    }

    void blocking_flow() {
        for (int64_t x : queue_) ptr_[x] = 0;
        vector<int64_t> path;
        for (int32_t s : frontier_) {
            const int64_t start = 2 * (int64_t)s + 1;
            ptr_[start] = 0;
            while (true) {
                path.assign(1, start);
                bool found = false;
                while (!path.empty()) {
                    const int64_t x = path.back();
                    if (role_[x >> 1] == SINK) {
                        found = true;
                        break;
                    }
                    const int64_t deg = degree(x);
                    const int32_t want = depth(x) + 1;
                    bool advanced = false;
                    for (; ptr_[x] <= deg; ptr_[x]++) {
                        const int64_t y = arc_head(x, ptr_[x]);
                        if (y >= 0 && role_[y >> 1] != SOURCE && seen_[y] == phase_ && level_[y] == want) {
                            path.push_back(y);
                            advanced = true;
                            break;
                        }
                    }
                    if (!advanced) {
                        if (role_[x >> 1] != SOURCE) level_[x] = -2;  // dead end for this phase
                        path.pop_back();
                        if (!path.empty()) ptr_[path.back()]++;
                    }
                }
                if (!found) break;
                // augment one unit along the path
                for (size_t i = 0; i + 1 < path.size(); i++) {
                    const int64_t x = path[i];
                    const int32_t v = (int32_t)(x >> 1);
                    const int64_t a = ptr_[x];
                    if (a == 0) {
                        if (role_[v] == NORMAL) through_[v] = (x & 1) ? 0 : 1;
                    } else {
                        // out(v) -> in(u) sends a unit v->u; in(v) -> out(u)
                        // cancels a unit u->v: both raise the v->u flow by one
                        push_on(g_.off[v] + a - 1, +1);
                    }
                }
            }
        }
    }

    CutResult extract() {
        // residual reachability from the sources
        phase_++;
        queue_.clear();
        for (int32_t v : frontier_) {
            queue_.push_back(2 * (int64_t)v);
            queue_.push_back(2 * (int64_t)v + 1);
        }
        for (size_t qh = 0; qh < queue_.size(); qh++) {
            const int64_t x = queue_[qh];
            const int64_t deg = degree(x);
            for (int64_t a = 0; a <= deg; a++) {
                const int64_t y = arc_head(x, a);
                if (y >= 0 && !reached(y)) reach(y, 0);
            }
        }
        CutResult r;
        for (int32_t v = 0; v < g_.m; v++) {
            const bool rin = reached(2 * (int64_t)v), rout = reached(2 * (int64_t)v + 1);
            if (rin && !rout) r.sep.push_back(v);
            else if (rout) r.a.push_back(v);
            else r.b.push_back(v);
        }
        r.ok = !r.a.empty() && !r.b.empty();
        return r;
    }
};

class Dissector {
  public:
    Dissector(int64_t n, const int64_t* noff, const int32_t* nbr, const double* x, const double* y,
              int64_t leaf, int threads)
        : n_(n), noff_(noff), nbr_(nbr), x_(x), y_(y), leaf_(std::max<int64_t>(leaf, 1)),
          threads_(threads > 0 ? threads : (int)std::max(1u, std::thread::hardware_concurrency())),
          owner_(new std::atomic<int64_t>[n]), local_(n, 0), order_(n, -1) {
        for (int64_t i = 0; i < n; i++) owner_[i].store(-1, std::memory_order_relaxed);
    }

    void run(vector<int32_t>& rank) {
        Cell root;
        root.verts.resize(n_);
        std::iota(root.verts.begin(), root.verts.end(), 0);
        root.lo = 0;
        push(std::move(root));
        vector<std::thread> pool;
        for (int t = 0; t < threads_; t++) pool.emplace_back([this] { worker(); });
        for (auto& th : pool) th.join();
        rank.assign(n_, -1);
        for (int64_t i = 0; i < n_; i++) rank[order_[i]] = (int32_t)i;
    }

  private:
    int64_t n_;
    const int64_t* noff_;
    const int32_t* nbr_;
    const double *x_, *y_;
    int64_t leaf_;
    int64_t band_min_ = env_int("NWCCH_ND_BAND_MIN", 20000);
    int64_t band_div_ = env_int("NWCCH_ND_BAND_DIV", 100);
    // the middle-half band is also tried on cells up to this size (smaller
    // on huge graphs, where the narrow band alone keeps the order fast)
    int64_t wide_max_ = env_int("NWCCH_ND_WIDE_MAX", n_ <= 2000000 ? 300000 : 60000);
    bool verbose_ = env_int("NWCCH_ND_VERBOSE", 0) != 0;

    static int64_t env_int(const char* name, int64_t dflt) {
        const char* v = getenv(name);
        return v ? atoll(v) : dflt;
    }
    int threads_;
    std::unique_ptr<std::atomic<int64_t>[]> owner_;  // cell stamp currently holding a vertex
    vector<int32_t> local_;               // local id inside that cell
    vector<int32_t> order_;               // vertex at each final position

    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<Cell> work_;
    int64_t busy_ = 0;
    std::atomic<int64_t> stamp_{0};

    void push(Cell&& c) {
        std::lock_guard<std::mutex> lk(mu_);
        // large cells first: they gate the critical path
        if (!work_.empty() && c.verts.size() >= work_.front().verts.size()) work_.push_front(std::move(c));
        else work_.push_back(std::move(c));
        cv_.notify_one();
    }

    void worker() {
        while (true) {
            Cell c;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [this] { return !work_.empty() || busy_ == 0; });
                if (work_.empty()) {
                    cv_.notify_all();
                    return;
                }
                c = std::move(work_.front());
                work_.pop_front();
                busy_++;
            }
            process(std::move(c));
            {
                std::lock_guard<std::mutex> lk(mu_);
                busy_--;
                if (busy_ == 0 && work_.empty()) cv_.notify_all();
            }
        }
    }

    double key(int32_t v, int dir) const {
        switch (dir) {
            case 0: return x_[v];
            case 1: return y_[v];
            case 2: return x_[v] + y_[v];
            default: return x_[v] - y_[v];
        }
    }

    void build_local(const Cell& c, int64_t stamp, LocalGraph& g) {
        const int32_t m = (int32_t)c.verts.size();
        for (int32_t i = 0; i < m; i++) {
            owner_[c.verts[i]].store(stamp, std::memory_order_relaxed);
            local_[c.verts[i]] = i;
        }
        g.m = m;
        g.off.assign(m + 1, 0);
        g.adj.clear();
        for (int32_t i = 0; i < m; i++) {
            const int32_t v = c.verts[i];
            for (int64_t k = noff_[v]; k < noff_[v + 1]; k++) {
                const int32_t u = nbr_[k];
                if (owner_[u].load(std::memory_order_relaxed) == stamp) g.adj.push_back(local_[u]);
            }
            g.off[i + 1] = (int64_t)g.adj.size();
        }
        // local lists are not sorted (local ids follow the cell order): sort them
        for (int32_t i = 0; i < m; i++) std::sort(g.adj.begin() + g.off[i], g.adj.begin() + g.off[i + 1]);
        g.eid.assign(g.adj.size(), -1);
        g.fwd.assign(g.adj.size(), 0);
        int64_t e = 0;
        for (int32_t v = 0; v < m; v++)
            for (int64_t j = g.off[v]; j < g.off[v + 1]; j++) {
                const int32_t u = g.adj[j];
                if (u > v) {
                    g.eid[j] = e++;
                    g.fwd[j] = 1;
                } else {
                    const auto b = g.adj.begin() + g.off[u], en = g.adj.begin() + g.off[u + 1];
                    const auto it = std::lower_bound(b, en, v);
                    g.eid[j] = g.eid[it - g.adj.begin()];
                    g.fwd[j] = 0;
                }
            }
        g.edges = e;
    }

    // Band of the projection's middle in which a cut is searched: inertial
    // flow's middle half (sources and sinks the first and last quarter), or a
    // narrow band (m / band_div_, at least band_min_ vertices) that bounds the
    // flow work on big cells and forces balanced halves.
    int64_t narrow_band(int64_t m) const {
        if (m <= band_min_ * 2) return m / 2;
        return std::max<int64_t>(band_min_, m / std::max<int64_t>(2, band_div_));
    }

    CutResult flow_cut(const Cell& c, const LocalGraph& g, int dir, int64_t band) const {
        const int32_t m = g.m;
        const int32_t k = std::max<int32_t>(1, (int32_t)((m - band) / 2));
        // only the k lowest and k highest projections matter: two selections
        // instead of a sort (ties broken by local id, so the result is fixed)
        vector<double> kv(m);
        for (int32_t i = 0; i < m; i++) kv[i] = key(c.verts[i], dir);
        const auto less = [&](int32_t a, int32_t b) { return kv[a] < kv[b] || (kv[a] == kv[b] && a < b); };
        vector<int32_t> perm(m);
        std::iota(perm.begin(), perm.end(), 0);
        std::nth_element(perm.begin(), perm.begin() + k, perm.end(), less);
        std::nth_element(perm.begin() + k, perm.end() - k, perm.end(), less);
        vector<int8_t> role(m, NORMAL);
        for (int32_t i = 0; i < k; i++) {
            role[perm[i]] = SOURCE;
            role[perm[m - 1 - i]] = SINK;
        }
        // a source adjacent to a sink makes the cut unbounded
        for (int32_t v = 0; v < m; v++)
            if (role[v] == SOURCE)
                for (int64_t j = g.off[v]; j < g.off[v + 1]; j++)
                    if (role[g.adj[j]] == SINK) return CutResult{};
        VertexCut vc(g, role);
        return vc.run();
    }

    // Median split along the wider extent; separator = side-A vertices with a
    // side-B neighbour.
    CutResult geometric_cut(const Cell& c, const LocalGraph& g) const {
        const int32_t m = g.m;
        double x0 = 1e300, x1 = -1e300, y0 = 1e300, y1 = -1e300;
        for (int32_t v : c.verts) {
            x0 = std::min(x0, x_[v]);
            x1 = std::max(x1, x_[v]);
            y0 = std::min(y0, y_[v]);
            y1 = std::max(y1, y_[v]);
        }
        const int dir = (x1 - x0) >= (y1 - y0) ? 0 : 1;
        vector<int32_t> perm(m);
        std::iota(perm.begin(), perm.end(), 0);
        std::stable_sort(perm.begin(), perm.end(), [&](int32_t a, int32_t b) {
            return key(c.verts[a], dir) < key(c.verts[b], dir);
        });
        vector<int8_t> side(m, 0);
        for (int32_t i = m / 2; i < m; i++) side[perm[i]] = 1;
        CutResult r;
        for (int32_t v = 0; v < m; v++) {
            if (side[v]) {
                r.b.push_back(v);
                continue;
            }
            bool boundary = false;
            for (int64_t j = g.off[v]; j < g.off[v + 1] && !boundary; j++) boundary = side[g.adj[j]];
            (boundary ? r.sep : r.a).push_back(v);
        }
        r.ok = true;
        return r;
    }

    void process(Cell c) {
        const int64_t m = (int64_t)c.verts.size();
        if (m == 0) return;
        if (m <= leaf_) {
            // small cell: cheap minimum-degree flavour, by global degree
            std::stable_sort(c.verts.begin(), c.verts.end(), [&](int32_t a, int32_t b) {
                return noff_[a + 1] - noff_[a] < noff_[b + 1] - noff_[b];
            });
            for (int64_t i = 0; i < m; i++) order_[c.lo + i] = c.verts[i];
            return;
        }
        const int64_t stamp = ++stamp_;
        const auto t_start = std::chrono::steady_clock::now();
        LocalGraph g;
        build_local(c, stamp, g);
        CutResult best;
        int64_t best_sep = -1, best_bal = 0;
        // candidates: 4 directions x (narrow band, and the middle half on
        // cells small enough for it)
        vector<std::pair<int, int64_t>> cand;
        for (int d = 0; d < 4; d++) cand.push_back({d, narrow_band(m)});
        if (m <= wide_max_ && narrow_band(m) != m / 2)
            for (int d = 0; d < 4; d++) cand.push_back({d, m / 2});
        vector<CutResult> cuts(cand.size());
        if (m >= 20000 && threads_ > 1) {
            vector<std::thread> ts;
            for (size_t i = 0; i < cand.size(); i++)
                ts.emplace_back([&, i] { cuts[i] = flow_cut(c, g, cand[i].first, cand[i].second); });
            for (auto& t : ts) t.join();
        } else {
            for (size_t i = 0; i < cand.size(); i++) cuts[i] = flow_cut(c, g, cand[i].first, cand[i].second);
        }
        if (verbose_ && m >= 100000) {
            const double secs =
                std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
            fprintf(stderr, "[nd] cell %lld: %.2fs, %zu candidates\n", (long long)m, secs, cand.size());
        }
        // smallest separator per vertex of the smaller half (ties: smaller
        // separator, then better balance)
        double best_ratio = 0;
        for (size_t i = 0; i < cuts.size(); i++) {
            if (!cuts[i].ok) continue;
            const int64_t ns = (int64_t)cuts[i].sep.size();
            const int64_t na = (int64_t)cuts[i].a.size(), nb = (int64_t)cuts[i].b.size();
            const int64_t bal = std::llabs(na - nb);
            const double ratio = (double)ns / (double)(std::min(na, nb) + 1);
            if (best_sep < 0 || ratio < best_ratio || (ratio == best_ratio && (ns < best_sep || (ns == best_sep && bal < best_bal)))) {
                best_ratio = ratio;
                best_sep = ns;
                best_bal = bal;
                best = std::move(cuts[i]);
            }
        }
        if (best_sep < 0) best = geometric_cut(c, g);
        // A gets the lowest ranks of the cell, then B, the separator the highest
        const int64_t na = (int64_t)best.a.size(), nb = (int64_t)best.b.size();
        int64_t p = c.lo + na + nb;
        for (int32_t v : best.sep) order_[p++] = c.verts[v];
        Cell ca, cb;
        ca.lo = c.lo;
        cb.lo = c.lo + na;
        ca.verts.reserve(na);
        cb.verts.reserve(nb);
        for (int32_t v : best.a) ca.verts.push_back(c.verts[v]);
        for (int32_t v : best.b) cb.verts.push_back(c.verts[v]);
        c.verts.clear();
        c.verts.shrink_to_fit();
        push(std::move(ca));
        push(std::move(cb));
    }
};

}  // namespace

void nested_dissection(int64_t n, const int64_t* noff, const int32_t* nbr, const double* x,
                       const double* y, int64_t leaf, int threads, vector<int32_t>& rank) {
    Dissector d(n, noff, nbr, x, y, leaf, threads);
    d.run(rank);
}

// ---------------------------------------------------------------- symbolic

void symbolic(int64_t n, const int64_t* noff, const int32_t* nbr, const int32_t* rank,
              vector<int64_t>& first, vector<int32_t>& head, vector<int32_t>& parent) {
    vector<int32_t> inv(n);
    for (int64_t v = 0; v < n; v++) inv[rank[v]] = (int32_t)v;
    parent.assign(n, -1);
    first.assign(n + 1, 0);
    head.clear();
    head.reserve((size_t)(3 * n));
    // children of each vertex, as singly linked lists built while sweeping
    vector<int32_t> kid_first(n, -1), kid_next(n, -1);
    vector<int32_t> seen(n, -1);
    vector<int32_t> row;
    for (int64_t x = 0; x < n; x++) {
        row.clear();
        const int32_t v = inv[x];
        for (int64_t k = noff[v]; k < noff[v + 1]; k++) {
            const int32_t r = rank[nbr[k]];
            if (r > x && seen[r] != x) {
                seen[r] = (int32_t)x;
                row.push_back(r);
            }
        }
        // a child's upper neighbours (other than x) become x's neighbours
        for (int32_t c = kid_first[x]; c >= 0; c = kid_next[c])
            for (int64_t a = first[c]; a < first[c + 1]; a++) {
                const int32_t r = head[a];
                if (r != x && seen[r] != x) {
                    seen[r] = (int32_t)x;
                    row.push_back(r);
                }
            }
        std::sort(row.begin(), row.end());
        head.insert(head.end(), row.begin(), row.end());
        first[x + 1] = (int64_t)head.size();
        if (!row.empty()) {
            const int32_t p = row[0];
            parent[x] = p;
            kid_next[x] = kid_first[p];
            kid_first[p] = (int32_t)x;
        }
    }
}

// ---------------------------------------------------------------- arc mapping

static int64_t locate(const int64_t* first, const int32_t* head, int64_t lo, int32_t hi) {
    const int32_t* b = head + first[lo];
    const int32_t* e = head + first[lo + 1];
    const int32_t* it = std::lower_bound(b, e, hi);
    if (it == e || *it != hi) return -1;
    return it - head;
}

int edge_arcs(int64_t n, const int64_t* off, const int32_t* tgt, const int32_t* rank,
              const int64_t* first, const int32_t* head, int64_t* e_arc, int8_t* e_up) {
    for (int64_t u = 0; u < n; u++) {
        const int32_t ru = rank[u];
        for (int64_t k = off[u]; k < off[u + 1]; k++) {
            const int32_t rv = rank[tgt[k]];
            if (ru == rv) {
                e_arc[k] = -1;
                e_up[k] = 0;
                continue;
            }
            const bool up = ru < rv;
            const int64_t a = up ? locate(first, head, ru, rv) : locate(first, head, rv, ru);
            if (a < 0) return -1;  // the topology does not belong to this graph/order
            e_arc[k] = a;
            e_up[k] = up ? 1 : 0;
        }
    }
    return 0;
}

}  // namespace nwcch_host
