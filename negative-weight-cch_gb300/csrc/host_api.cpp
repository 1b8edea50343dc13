// C-ABI entry points of the host-side (weight-independent) preprocessing.
// Variable-size outputs are returned in malloc'ed buffers that the caller
// releases with nwcch_host_free().

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <thread>
#include <vector>

#include "host_internal.h"
#include "nwcch.h"

namespace {

template <class T>
T* export_vector(const std::vector<T>& v) {
    T* p = static_cast<T*>(std::malloc(std::max<size_t>(1, v.size()) * sizeof(T)));
    if (p && !v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(T));
    return p;
}

}  // namespace

extern "C" {

void nwcch_host_free(void* p) { std::free(p); }

int nwcch_undirected_csr(int64_t n, const int64_t* off, const int32_t* tgt, int64_t* noff,
                         int32_t** nbr, int64_t* slots) {
    if (n < 0 || !off || (!tgt && off[n] > 0) || !noff || !nbr || !slots) return NWCCH_ERR_ARG;
    for (int64_t k = 0; k < off[n]; k++)
        if (tgt[k] < 0 || tgt[k] >= n) return NWCCH_ERR_ARG;
    std::vector<int64_t> o;
    std::vector<int32_t> b;
    nwcch_host::undirected_csr(n, off, tgt, o, b);
    std::memcpy(noff, o.data(), (n + 1) * sizeof(int64_t));
    *nbr = export_vector(b);
    *slots = (int64_t)b.size();
    return *nbr ? NWCCH_OK : NWCCH_ERR_NOMEM;
}

int nwcch_nested_dissection(int64_t n, const int64_t* noff, const int32_t* nbr, const double* x,
                            const double* y, int64_t leaf, int threads, int32_t* rank) {
    if (n < 0 || n > INT32_MAX || !noff || !x || !y || !rank) return NWCCH_ERR_ARG;
    std::vector<int32_t> r;
    nwcch_host::nested_dissection(n, noff, nbr, x, y, leaf, threads, r);
    std::copy(r.begin(), r.end(), rank);
    return NWCCH_OK;
}

int nwcch_symbolic(int64_t n, const int64_t* noff, const int32_t* nbr, const int32_t* rank,
                   int64_t* first, int32_t* parent, int32_t** head, int64_t* m_plus) {
    if (n < 0 || n > INT32_MAX || !noff || !rank || !first || !parent || !head || !m_plus)
        return NWCCH_ERR_ARG;
    {
        std::vector<char> seen(n, 0);
        for (int64_t v = 0; v < n; v++) {
            if (rank[v] < 0 || rank[v] >= n || seen[rank[v]]) return NWCCH_ERR_ARG;
            seen[rank[v]] = 1;
        }
    }
    std::vector<int64_t> f;
    std::vector<int32_t> h, p;
    nwcch_host::symbolic(n, noff, nbr, rank, f, h, p);
    std::memcpy(first, f.data(), (n + 1) * sizeof(int64_t));
    std::memcpy(parent, p.data(), n * sizeof(int32_t));
    *head = export_vector(h);
    *m_plus = (int64_t)h.size();
    return *head ? NWCCH_OK : NWCCH_ERR_NOMEM;
}

int nwcch_edge_arcs(int64_t n, const int64_t* off, const int32_t* tgt, const int32_t* rank,
                    const int64_t* first, const int32_t* head, int64_t* e_arc, int8_t* e_up) {
    if (n < 0 || !off || !rank || !first || !e_arc || !e_up) return NWCCH_ERR_ARG;
    return nwcch_host::edge_arcs(n, off, tgt, rank, first, head, e_arc, e_up) == 0 ? NWCCH_OK
                                                                                    : NWCCH_ERR_TOPOLOGY;
}

int nwcch_triangle_edges(int64_t n, int64_t ntri, const int64_t* tri, int64_t** eu, int64_t** ev,
                         int64_t* nedges) {
    if (n < 0 || ntri < 0 || (!tri && ntri > 0) || !eu || !ev || !nedges) return NWCCH_ERR_ARG;
    // counting sort of the 3 edges of every triangle by lower endpoint
    std::vector<int64_t> cnt(n + 1, 0);
    for (int64_t t = 0; t < ntri; t++)
        for (int k = 0; k < 3; k++) {
            const int64_t a = tri[3 * t + k], b = tri[3 * t + (k + 1) % 3];
            if (a < 0 || a >= n || b < 0 || b >= n || a == b) return NWCCH_ERR_ARG;
            cnt[std::min(a, b) + 1]++;
        }
    for (int64_t i = 0; i < n; i++) cnt[i + 1] += cnt[i];
    std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1), hi(cnt[n]);
    for (int64_t t = 0; t < ntri; t++)
        for (int k = 0; k < 3; k++) {
            const int64_t a = tri[3 * t + k], b = tri[3 * t + (k + 1) % 3];
            hi[pos[std::min(a, b)]++] = std::max(a, b);
        }
    const int nth = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<int64_t> uniq(n + 1, 0);
    {
        std::vector<std::thread> ts;
        for (int th = 0; th < nth; th++)
            ts.emplace_back([&, th] {
                for (int64_t u = th; u < n; u += nth) {
                    auto b = hi.begin() + cnt[u], e = hi.begin() + cnt[u + 1];
                    std::sort(b, e);
                    uniq[u + 1] = std::unique(b, e) - b;
                }
            });
        for (auto& t : ts) t.join();
    }
    for (int64_t i = 0; i < n; i++) uniq[i + 1] += uniq[i];
    const int64_t m = uniq[n];
    *eu = static_cast<int64_t*>(std::malloc(std::max<int64_t>(1, m) * sizeof(int64_t)));
    *ev = static_cast<int64_t*>(std::malloc(std::max<int64_t>(1, m) * sizeof(int64_t)));
    if (!*eu || !*ev) return NWCCH_ERR_NOMEM;
    for (int64_t u = 0; u < n; u++)
        for (int64_t j = 0; j < uniq[u + 1] - uniq[u]; j++) {
            (*eu)[uniq[u] + j] = u;
            (*ev)[uniq[u] + j] = hi[cnt[u] + j];
        }
    *nedges = m;
    return NWCCH_OK;
}

int nwcch_emst_mask(int64_t n, int64_t m, const int64_t* eu, const int64_t* ev, const double* length,
                    uint8_t* mask) {
    if (n < 0 || m < 0 || (m > 0 && (!eu || !ev || !length || !mask))) return NWCCH_ERR_ARG;
    // Kruskal: edges by (length, id), union-find with path halving
    std::vector<int64_t> order(m);
    for (int64_t i = 0; i < m; i++) {
        if (eu[i] < 0 || eu[i] >= n || ev[i] < 0 || ev[i] >= n) return NWCCH_ERR_ARG;
        order[i] = i;
    }
    const auto less = [&](int64_t a, int64_t b) {
        return length[a] < length[b] || (length[a] == length[b] && a < b);
    };
    const int nth = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    {
        // sort nth chunks in parallel, then merge pairwise
        std::vector<int64_t> bounds(nth + 1);
        for (int t = 0; t <= nth; t++) bounds[t] = m * t / nth;
        std::vector<std::thread> ts;
        for (int t = 0; t < nth; t++)
            ts.emplace_back([&, t] { std::sort(order.begin() + bounds[t], order.begin() + bounds[t + 1], less); });
        for (auto& th : ts) th.join();
        for (int width = 1; width < nth; width *= 2) {
            std::vector<std::thread> ms;
            for (int t = 0; t + width < nth; t += 2 * width) {
                const int64_t lo = bounds[t], mid = bounds[t + width], hi = bounds[std::min(nth, t + 2 * width)];
                ms.emplace_back([&, lo, mid, hi] {
                    std::inplace_merge(order.begin() + lo, order.begin() + mid, order.begin() + hi, less);
                });
            }
            for (auto& th : ms) th.join();
        }
    }
    std::vector<int64_t> up(n);
    for (int64_t v = 0; v < n; v++) up[v] = v;
    auto find = [&](int64_t v) {
        while (up[v] != v) {
            up[v] = up[up[v]];
            v = up[v];
        }
        return v;
    };
    std::memset(mask, 0, (size_t)m);
    for (int64_t i : order) {
        const int64_t a = find(eu[i]), b = find(ev[i]);
        if (a == b) continue;
        up[a] = b;
        mask[i] = 1;
    }
    return NWCCH_OK;
}

}  // extern "C"
