// Test-only harness around the reference C++ implementation (cpp/cch.cpp of
// AaravG/negative-weight-cch).
//
// This file contains no reference code. The Makefile in this directory compiles
// it with -DREF_CCH_CPP="<path of cpp/cch.cpp in the reference checkout>", and
// the #include below pulls the reference translation unit in unmodified, with
// its main() renamed so that the harness can be built as a shared library.
// The library lands in oracle/_ref/ (git-ignored) and is used only by the
// golden-fixture generator and the CPU tests, never by the product.
//
// Every entry point is extern "C" with plain pointers so that ctypes can bind
// it. The handle owns one reference Graph and one reference CCH.

#define main cch_reference_main
#include REF_CCH_CPP
#undef main

#include <cstdlib>

namespace {

struct RefHandle {
    Graph g;
    CCH c;
    vector<vector<i32>> buckets;
};

}  // namespace

extern "C" {

// Builds the reference Graph from a directed CSR (off int64[n+1], tgt int32[m])
// and coordinates (used by the reference nested dissection only).
void* ref_create(int64_t n, const int64_t* off, const int32_t* tgt, const double* x,
                 const double* y) {
    auto* h = new RefHandle();
    h->g.n = n;
    h->g.m = off[n];
    h->g.off.assign(off, off + n + 1);
    h->g.tgt.assign(tgt, tgt + off[n]);
    h->g.x.assign(x, x + n);
    h->g.y.assign(y, y + n);
    h->g.build_undirected();
    return h;
}

void ref_destroy(void* p) { delete static_cast<RefHandle*>(p); }

// Reference nested dissection (inertial flow, cch.cpp nested_dissection).
void ref_order(void* p, int64_t leaf, int32_t* rank_out) {
    auto* h = static_cast<RefHandle*>(p);
    h->c.rank = nested_dissection(h->g, leaf);
    std::copy(h->c.rank.begin(), h->c.rank.end(), rank_out);
}

void ref_set_order(void* p, const int32_t* rank) {
    auto* h = static_cast<RefHandle*>(p);
    h->c.rank.assign(rank, rank + h->g.n);
}

// Reference symbolic contraction + arc mapping; returns m+ (shortcut arcs).
int64_t ref_symbolic(void* p, int64_t* depth, int64_t* triangles) {
    auto* h = static_cast<RefHandle*>(p);
    h->c.symbolic(h->g);
    h->c.map_arcs(h->g);
    *depth = h->c.depth;
    *triangles = h->c.triangles;
    return (int64_t)h->c.head.size();
}

void ref_topology(void* p, int64_t* first, int32_t* head, int32_t* parent, int64_t* e_arc,
                  int8_t* e_up) {
    auto* h = static_cast<RefHandle*>(p);
    const CCH& c = h->c;
    std::copy(c.first.begin(), c.first.end(), first);
    std::copy(c.head.begin(), c.head.end(), head);
    std::copy(c.parent.begin(), c.parent.end(), parent);
    std::copy(c.e_arc.begin(), c.e_arc.end(), e_arc);
    std::copy(c.e_up.begin(), c.e_up.end(), e_up);
}

// Reference serial customization (CCH::customize). Returns seconds taken.
double ref_customize(void* p, const double* w, double* up, double* dn) {
    auto* h = static_cast<RefHandle*>(p);
    vector<double> ww(w, w + h->g.m), u, d;
    const double t0 = now();
    h->c.customize(ww, u, d);
    const double t = now() - t0;
    std::copy(u.begin(), u.end(), up);
    std::copy(d.begin(), d.end(), dn);
    return t;
}

// Reference level-parallel customization (CCH::levels + customize_parallel).
double ref_customize_parallel(void* p, const double* w, double* up, double* dn, int threads) {
    auto* h = static_cast<RefHandle*>(p);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    if (h->buckets.empty()) h->c.levels(h->buckets);
    vector<double> ww(w, w + h->g.m), u, d;
    const double t0 = now();
    h->c.customize_parallel(ww, u, d, h->buckets);
    const double t = now() - t0;
    std::copy(u.begin(), u.end(), up);
    std::copy(d.begin(), d.end(), dn);
    return t;
}

int64_t ref_levels(void* p) {
    auto* h = static_cast<RefHandle*>(p);
    if (h->buckets.empty()) h->c.levels(h->buckets);
    return (int64_t)h->buckets.size();
}

int64_t ref_negative_cycle_arcs(void* p, const double* up, const double* dn) {
    auto* h = static_cast<RefHandle*>(p);
    const size_t m = h->c.head.size();
    vector<double> u(up, up + m), d(dn, dn + m);
    return h->c.negative_cycle_arcs(u, d);
}

// Reference elimination-tree query (Query::run) on original vertex ids.
double ref_query_batch(void* p, const double* up, const double* dn, int64_t nq, const int64_t* s,
                       const int64_t* t, double* out) {
    auto* h = static_cast<RefHandle*>(p);
    const size_t m = h->c.head.size();
    vector<double> u(up, up + m), d(dn, dn + m);
    Query q(h->c);
    const double t0 = now();
    for (int64_t i = 0; i < nq; i++) out[i] = q.run(s[i], t[i], u, d);
    return now() - t0;
}

// Reference Johnson potential (FIFO Bellman-Ford) and Dijkstra on reduced
// weights: the large-graph ground truth used by the reference driver.
void ref_johnson_potential(void* p, const double* w, double* pot) {
    auto* h = static_cast<RefHandle*>(p);
    vector<double> ww(w, w + h->g.m);
    i64 pops = 0;
    auto pv = johnson_potential(h->g, ww, pops);
    std::copy(pv.begin(), pv.end(), pot);
}

// Reference CCH potential (two sweeps over the customized CCH), original ids.
void ref_cch_potential(void* p, const double* up, const double* dn, double* pot) {
    auto* h = static_cast<RefHandle*>(p);
    const size_t m = h->c.head.size();
    vector<double> u(up, up + m), d(dn, dn + m);
    auto pv = cch_potential(h->c, u, d);
    std::copy(pv.begin(), pv.end(), pot);
}

void ref_dijkstra_batch(void* p, const double* w, const double* pot, int64_t nq, const int64_t* s,
                        const int64_t* t, double* out) {
    auto* h = static_cast<RefHandle*>(p);
    vector<double> ww(w, w + h->g.m), pv(pot, pot + h->g.n), dist(h->g.n);
    vector<char> done(h->g.n);
    for (int64_t i = 0; i < nq; i++) {
        i64 scanned = 0;
        out[i] = dijkstra_potential(h->g, ww, pv, s[i], t[i], dist, done, scanned);
    }
}

}  // extern "C"
