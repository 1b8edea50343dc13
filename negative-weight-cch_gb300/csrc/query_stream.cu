// Few elimination-tree queries at low latency: a CTA per chain, the chain's
// rows streamed into shared memory by bulk asynchronous copies.
//
// A query's cost is its two ancestor chains (python/cch_nb.py:577-615): the
// forward sweep over the ancestors of s with up weights and the backward
// sweep over those of t with dn weights. On a road-like graph a chain holds
// millions of arcs, read in chain order, and every step of the sweep waits
// for the previous one; a kernel that loads each chunk's weights when it
// needs them spends the query waiting on global memory. Here the two chains
// of a query run on two CTAs at once, and in each CTA
//  - a producer warp walks the chain (supernode descriptors: first vertex,
//    rows, boundary size, next supernode and its entry row) and streams it
//    into a ring of shared-memory slots with cp.async.bulk, one slot per
//    item: a supernode's boundary depths (the heads' depths of its last row,
//    which give the label positions of its boundary columns), then its rows
//    from the entry row in chunks of up to 32 rows (the rows of a supernode
//    are consecutive in the CSR, so a chunk is one contiguous range);
//  - eight consumer warps take the items in order: per chunk, warp 0 solves
//    the chunk's triangle by shuffles (row r's label is final when step r
//    broadcasts it), then every consumer thread takes columns to the right
//    and folds min over the chunk's rows of label + weight into the label
//    array. Slots are handed back through mbarriers.
// Labels are indexed by chain position (depth(start) - depth(v)), 32-bit DPX
// arithmetic as in query_sn.cuh (batches whose values need 64-bit labels
// leave at once and the 64-bit kernel answers them). At the end each CTA
// writes its labels and chain vertices by depth to global scratch; the CTA
// that finishes second takes the minimum of forward + backward labels over
// the depths where both chains hold the same vertex (the common ancestors).
// Every wait is bounded: a wait that runs out records ERR_TIMEOUT, the CTA
// waits (bounded again) for its copies in flight and returns.

#include <algorithm>
#include <cstdint>

#include "query_sn.cuh"

namespace nwcch {

namespace {

constexpr int QS_CONSUMERS = 256;                   // consumer threads (8 warps)
constexpr int QS_THREADS = QS_CONSUMERS + 32;       // + the producer warp
constexpr int QS_ITEMS = 32;                        // items in flight at most (descriptor ring)
constexpr int QS_RING_MAX_WORDS = 49152;            // data ring: at most 192 KB, as much as the labels leave
                                                    // (one item: at most a third of the ring)
constexpr long long QS_SPIN = 1 << 22;              // polls of one bounded wait (~0.2-1 s)

enum QsItem : int { QS_ROWS = 0, QS_BOUNDARY = 1, QS_END = 2 };

struct QsHeader {
    int32_t type;
    int32_t s0, k, cols;  // supernode: first vertex, rows, rows + boundary
    int32_t i0, pos;      // entry row, chain position of the entry row's vertex
    int32_t c0, n;        // QS_ROWS: rows [c0, c0 + n)
    int32_t off;          // first word of the item in the data ring
    int32_t b;            // QS_BOUNDARY: boundary size
};

// ---- mbarrier and bulk-copy primitives (PTX, shared::cta barriers)

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t* bar, unsigned parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}
// Bounded wait for the phase of `parity` to complete; false if it ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity) {
    for (long long i = 0; i < QS_SPIN; i++) {
        if (mbar_test(bar, parity)) return true;
        if (i > 64) __nanosleep(64);
    }
    return false;
}
// Global -> shared bulk copy completing on `bar` (addresses and size
// multiples of 16 bytes).
__device__ __forceinline__ void bulk_copy(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ int volatile_read(const int& x) { return *reinterpret_cast<const volatile int*>(&x); }

// Consumer-warp barrier (named barrier 1; the producer warp does not take part).
__device__ __forceinline__ void consumers_sync() { asm volatile("bar.sync 1, %0;" ::"n"(QS_CONSUMERS) : "memory"); }

// The 16-byte groups covering words [a0, a1) of array A (`len` words,
// 16-byte aligned base): [*w0, *w1). The groups wholly inside the array go
// by one bulk copy (*bulk_bytes from A + *w0); a last partial group is
// written into dst by plain loads here, before the caller's arrive
// publishes it.
__device__ void stage_range(const int32_t* A, int64_t len, int64_t a0, int64_t a1, int32_t* dst, int64_t* w0,
                            int64_t* w1, unsigned* bulk_bytes) {
    *w0 = a0 & ~3LL;
    *w1 = (a1 + 3) & ~3LL;
    const int64_t wb = std::min<int64_t>(*w1, len & ~3LL);
    *bulk_bytes = wb > *w0 ? (unsigned)((wb - *w0) * 4) : 0u;
    for (int64_t w = std::max(wb, *w0); w < *w1; w++) dst[w - *w0] = w < len ? A[w] : INF32;
}

}  // namespace

// Both chains of every query of the batch (CTA 2q: s with up weights, CTA
// 2q+1: t with dn weights). `thr`: the largest |weight| for which 32-bit
// labels are exact on this tree (2^28 / (depth + 2)); a chain that meets a
// larger finite weight marks its query in `wide` and leaves its answer to
// the 64-bit kernel.
__global__ void __launch_bounds__(QS_THREADS, 1)
    k_qstream(DevTopo D, const QsNode* __restrict__ nodes, const int32_t* __restrict__ sn_id,
              const int32_t* __restrict__ up, const int32_t* __restrict__ dn, const int32_t* __restrict__ s_rank,
              const int32_t* __restrict__ t_rank, int64_t nq, int64_t* __restrict__ dist, int32_t thr,
              int32_t* __restrict__ scratch, int32_t* __restrict__ wide, int* __restrict__ err, int32_t ring_words,
              int32_t item_words) {
    extern __shared__ __align__(128) unsigned char qs_smem[];
    const int64_t Dp = D.max_depth + 1;
    int32_t* ring = reinterpret_cast<int32_t*>(qs_smem);  // [ring_words] data ring
    int32_t* L = ring + ring_words;                        // [Dp] labels by chain position
    int32_t* bpos = L + ((Dp + 3) & ~3LL);                 // boundary positions of the current supernode
    __shared__ __align__(8) uint64_t full[QS_ITEMS], empty[QS_ITEMS];
    __shared__ QsHeader hdr[QS_ITEMS];
    __shared__ int32_t clab[32];
    __shared__ int abort_flag, second, wide_any;
    __shared__ int go[2];  // by item parity: read after an item's barrier, written before the next one's
    __shared__ int32_t red[QS_THREADS / 32];

    const int64_t c = blockIdx.x;  // chain: query c >> 1, direction c & 1
    const int64_t q = c >> 1;
    const int dir = (int)(c & 1);
    if (q >= nq) return;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int32_t s = dir ? t_rank[q] : s_rank[q];
    const int32_t other = dir ? s_rank[q] : t_rank[q];
    if (s < 0 || s >= D.n || other < 0 || other >= D.n) {  // uniform over the CTA
        if (tid == 0) {
            if (dir == 0) dist[q] = INF64;
            atomicOr(err, ERR_ARG);
        }
        return;
    }
    const int32_t* __restrict__ W = dir ? dn : up;
    const int32_t ds = D.depth[s];
    int32_t* Lg = scratch + q * (4 * Dp + 4);  // [2][Dp] labels by depth, [2][Dp] vertices by depth, counter
    int32_t* Vg = Lg + 2 * Dp;
    int* counter = reinterpret_cast<int*>(Lg + 4 * Dp);
    if (tid == 0) {
        for (int i = 0; i < QS_ITEMS; i++) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        abort_flag = 0;
        wide_any = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    for (int64_t i = tid; i <= ds; i += QS_THREADS) L[i] = Q32::CINF;
    __syncthreads();
    if (tid == 0) L[0] = 0;
    __syncthreads();
    int e = 0;

    if (warp == QS_CONSUMERS / 32) {
        // ------------------------------------------------ producer (one lane)
        if (lane == 0) {
            int64_t g = 0;                 // items issued
            int64_t rel = 0;               // items known to be released by the consumers
            int64_t head = 0, tail = 0;    // data ring: words handed out / words free again (monotonic)
            int64_t item_end[QS_ITEMS] = {};  // head after each item in flight
            bool ok = true;
            // waits until item `r` is released; its words are free again
            auto release_one = [&]() -> bool {
                if (!mbar_wait(&empty[rel % QS_ITEMS], (unsigned)((rel / QS_ITEMS) & 1))) return false;
                tail = item_end[rel % QS_ITEMS];
                rel++;
                return true;
            };
            // a descriptor and `words` (a multiple of 4) contiguous words of the ring
            auto take = [&](int64_t words, int& slot, int32_t*& dst, int32_t& off) -> bool {
                while (g - rel >= QS_ITEMS)
                    if (!release_one()) return false;
                int64_t pos = head % ring_words;
                if (pos + words > ring_words) {  // no wrap inside an item: skip to the ring's start
                    head += ring_words - pos;
                    pos = 0;
                }
                while (head + words - tail > ring_words)
                    if (!release_one()) return false;
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                slot = (int)(g % QS_ITEMS);
                dst = ring + pos;
                off = (int32_t)pos;
                head += words;
                item_end[slot] = head;
                return true;
            };
            auto issue = [&](int slot, const QsHeader& h, const int32_t* src, unsigned bytes, int32_t* dst) {
                hdr[slot] = h;
                mbar_arrive_tx(&full[slot], bytes);
                if (bytes) bulk_copy(dst, src, bytes, &full[slot]);
                g++;
            };
            int32_t sn = sn_id[s];
            QsNode d = nodes[sn];
            int32_t i0 = s - d.s0;
            int32_t pos = 0;
            while (ok && sn >= 0) {
                const QsNode nd = d.next >= 0 ? nodes[d.next] : d;  // next descriptor, loaded early
                const int32_t k = d.k, b = d.b, cols = k + b;
                if (b > 0) {  // boundary depths: the heads of the last row
                    const int64_t lastb = d.base + (int64_t)(k - 1) * (cols - 1) - (int64_t)(k - 1) * (k - 2) / 2;
                    const int64_t words = ((lastb + b + 3) & ~3LL) - (lastb & ~3LL);
                    int slot;
                    int32_t* dst;
                    int32_t off;
                    if (volatile_read(abort_flag) || !(ok = take(words, slot, dst, off))) break;
                    int64_t w0, w1;
                    unsigned bytes;
                    stage_range(D.hdep, D.m_plus, lastb, lastb + b, dst, &w0, &w1, &bytes);
                    issue(slot, QsHeader{QS_BOUNDARY, d.s0, k, cols, i0, pos, 0, 0, off + (int32_t)(lastb - w0), b},
                          D.hdep + w0, bytes, dst);
                }
                for (int32_t c0 = i0; c0 < k && ok;) {
                    // rows of the chunk: up to 32, as many as fit an item
                    int32_t n = min(32, k - c0);
                    auto words = [&](int32_t nn) {
                        return (int64_t)nn * (cols - c0 - 1) - (int64_t)nn * (nn - 1) / 2;
                    };
                    while (n > 1 && words(n) + 8 > item_words) n--;
                    if (words(n) + 8 > item_words) {  // a row longer than an item: the host excludes this
                        e |= ERR_CAPACITY;
                        ok = false;
                        break;
                    }
                    const int64_t a0 = d.base + (int64_t)c0 * (cols - 1) - (int64_t)c0 * (c0 - 1) / 2;
                    const int64_t a1 = a0 + words(n);
                    int slot;
                    int32_t* dst;
                    int32_t off;
                    if (volatile_read(abort_flag) || !(ok = take(((a1 + 3) & ~3LL) - (a0 & ~3LL), slot, dst, off)))
                        break;
                    int64_t w0, w1;
                    unsigned bytes;
                    stage_range(W, D.m_plus, a0, a1, dst, &w0, &w1, &bytes);
                    issue(slot, QsHeader{QS_ROWS, d.s0, k, cols, i0, pos, c0, n, off + (int32_t)(a0 - w0), b}, W + w0,
                          bytes, dst);
                    c0 += n;
                }
                pos += k - i0;
                i0 = d.next_row;
                sn = d.next;
                d = nd;
            }
            if (ok && !volatile_read(abort_flag)) {
                int slot;
                int32_t* dst;
                int32_t off;
                if ((ok = take(0, slot, dst, off))) issue(slot, QsHeader{QS_END, 0, 0, 0, 0, 0, 0, 0, 0, 0}, nullptr, 0, dst);
            }
            if (!ok || volatile_read(abort_flag)) {
                // stop the consumers, then wait (bounded) for the copies still
                // in flight: every item issued and not yet released
                e |= ERR_TIMEOUT;
                atomicExch(&abort_flag, 1);
                for (int64_t r = rel; r < g; r++) mbar_wait(&full[r % QS_ITEMS], (unsigned)((r / QS_ITEMS) & 1));
            }
        }
    } else {
        // ------------------------------------------------ consumers
        int32_t hi = INT32_MIN, lo = INT32_MAX;  // extreme finite weights this thread read
        for (int64_t g = 0;; g++) {
            const int slot = (int)(g % QS_ITEMS);
            const unsigned parity = (unsigned)((g / QS_ITEMS) & 1);
            if (tid == 0) {
                bool ready = false;
                for (long long i = 0; i < QS_SPIN && !ready; i++) {
                    ready = mbar_test(&full[slot], parity);
                    if (!ready && volatile_read(abort_flag)) break;
                    if (!ready && i > 64) __nanosleep(64);
                }
                if (!ready) {
                    e |= ERR_TIMEOUT;
                    atomicExch(&abort_flag, 1);
                }
                go[g & 1] = ready ? 1 : 0;  // one decision for all consumers
            }
            consumers_sync();
            // every consumer is done with item g - 1 (this barrier is its
            // end): its slot goes back to the producer
            if (g > 0 && tid == 0) mbar_arrive(&empty[(g - 1) % QS_ITEMS]);
            if (!go[g & 1]) break;
            if (tid != 0 && !mbar_test(&full[slot], parity)) mbar_wait(&full[slot], parity);  // acquire per thread
            const QsHeader h = hdr[slot];
            if (h.type == QS_END) break;
            const int32_t* sl = ring + h.off;
            if (h.type == QS_BOUNDARY) {
                for (int p = tid; p < h.b; p += QS_CONSUMERS) bpos[p] = ds - sl[p];
            } else {
                const int32_t cols = h.cols, c0 = h.c0, n = h.n, k = h.k;
                const int32_t pos_c0 = h.pos + (c0 - h.i0);
                auto rowoff = [&](int r) { return r * (cols - c0 - 1) - r * (r - 1) / 2; };
                if (warp == 0) {
                    // the chunk's triangle: lane r owns row c0 + r; its
                    // column of weights is read before the solve, so each
                    // step is a shuffle and an add-min
                    int32_t u[31];
#pragma unroll
                    for (int rr = 0; rr < 31; rr++) {
                        u[rr] = Q32::CINF;
                        if (rr < lane && lane < n) {
                            const int32_t raw = sl[rowoff(rr) + (lane - rr - 1)];
                            hi = max(hi, raw == INF32 ? INT32_MIN : raw);
                            lo = min(lo, raw);
                            u[rr] = Q32::w(raw);
                        }
                    }
                    int32_t lab = lane < n ? L[pos_c0 + lane] : Q32::CINF;
#pragma unroll
                    for (int rr = 0; rr < 31; rr++)
                        if (rr + 1 < n) lab = __viaddmin_s32(Q32::norm(__shfl_sync(FULL, lab, rr)), u[rr], lab);
                    lab = Q32::norm(lab);
                    if (lane < n) {
                        L[pos_c0 + lane] = lab;
                        clab[lane] = lab;
                        Vg[dir * Dp + (ds - (pos_c0 + lane))] = h.s0 + c0 + lane;
                    }
                }
                consumers_sync();
                // the chunk's rows times the columns to their right
                for (int32_t j = c0 + n + tid; j < cols; j += QS_CONSUMERS) {
                    int32_t acc = Q32::CINF;
                    int32_t o = j - c0 - 1;  // row r's entry for column j: rowoff(r) + (j - c0 - r - 1)
                    for (int r = 0; r < n; r++) {
                        const int32_t raw = sl[o];
                        o += cols - c0 - 2 - r;
                        hi = max(hi, raw == INF32 ? INT32_MIN : raw);
                        lo = min(lo, raw);
                        acc = __viaddmin_s32(clab[r], Q32::w(raw), acc);
                    }
                    if (!Q32::none(acc)) {
                        const int32_t pj = j < k ? h.pos + (j - h.i0) : bpos[j - k];
                        if (acc < L[pj]) L[pj] = acc;
                    }
                }
            }
        }
        if (hi > thr || lo < -thr) atomicOr(&wide_any, 1);
    }
    __syncthreads();
    if (volatile_read(abort_flag)) {
        if (tid == 0) {
            e |= ERR_TIMEOUT;
            dist[q] = INF64;
        }
        if (e) atomicOr(err, e);
        return;
    }
    // labels by depth to global; the second CTA of the query takes the meet
    for (int64_t i = tid; i <= ds; i += QS_THREADS) Lg[dir * Dp + (ds - i)] = L[i];
    if (tid == 0 && wide_any) atomicOr(wide + q, 1);
    __threadfence();
    __syncthreads();
    if (tid == 0) second = atomicAdd(counter, 1) == 1;
    __syncthreads();
    if (second) {
        __threadfence();
        if (__ldcg(wide + q)) {  // a weight beyond the 32-bit bound: the 64-bit kernel answers
            if (e) atomicOr(err, e);
            return;
        }
        const int32_t dt = D.depth[other];
        const int32_t dm = min(ds, dt);
        const int32_t* Lo = Lg + (1 - dir) * Dp;
        const int32_t* Vo = Vg + (1 - dir) * Dp;
        const int32_t* Vm = Vg + dir * Dp;
        int32_t best = Q32::CINF;
        for (int32_t d = tid; d <= dm; d += QS_THREADS) {
            if (__ldcg(Vm + d) != __ldcg(Vo + d)) continue;  // not a common ancestor
            const int32_t a = L[ds - d], o = __ldcg(Lo + d);
            if (!Q32::none(a) && !Q32::none(o)) best = min(best, a + o);
        }
        for (int o = 16; o > 0; o >>= 1) best = min(best, __shfl_xor_sync(FULL, best, o));
        if (lane == 0) red[warp] = best;
        __syncthreads();
        if (tid == 0) {
            for (int w = 0; w < QS_THREADS / 32; w++) best = min(best, red[w]);
            dist[q] = Q32::none(best) ? INF64 : (int64_t)best;
        }
    }
    if (e) atomicOr(err, e);
}

// Host: a batch of at most tune.query_stream_max int32-stored queries when
// the topology fits the kernel's shared memory (labels and boundary
// positions beside the data ring) and no row is longer than an item. *used =
// false otherwise (nothing enqueued). The queries that met a weight beyond
// the 32-bit label bound are answered by the 64-bit kernel right after.
int query_stream_async(nwcch_topology* t, const int32_t* up, const int32_t* dn, const int32_t* s_rank,
                       const int32_t* t_rank, int64_t nq, int64_t* dist, int* err, cudaStream_t s, bool* used,
                       int64_t* launches) {
    *used = false;
    *launches = 0;
    auto* P = static_cast<SnPlan*>(t->sn_plan);
    if (!P || !P->d_qnodes || nq < 1 || nq > t->tune.query_stream_max) return NWCCH_OK;
    if (((uintptr_t)up | (uintptr_t)dn | (uintptr_t)t->d.hdep) & 15) return NWCCH_OK;  // bulk copies: 16-byte bases
    const int64_t Dp = t->d.max_depth + 1;
    // the data ring takes what the labels and boundary positions leave of
    // the CTA's shared memory (4 KB kept for the static part), at most 192 KB
    // or the tuned size; an item holds at most a third of it
    const int64_t fixed = ((Dp + 3) & ~3LL) * 4 + (int64_t)P->max_b * 4;
    int64_t ring_words = t->tune.query_stream_ring_kb > 0 ? t->tune.query_stream_ring_kb * 256 : QS_RING_MAX_WORDS;
    ring_words = std::min<int64_t>(ring_words, (227 * 1024 - 4096 - fixed) / 4);
    ring_words = ring_words / 12 * 12;
    const int64_t item_words = ring_words / 3;  // a multiple of 4
    if (item_words < 16 || (int64_t)t->max_deg + 8 > item_words || (int64_t)P->max_b + 8 > item_words)
        return NWCCH_OK;
    const size_t smem = (size_t)(ring_words * 4 + fixed);
    NWCCH_CUDA_TRY(allow_dynamic_smem((const void*)k_qstream, smem));
    // scratch: per query labels and vertices by depth and a counter, then a
    // flag per query
    const size_t per_query = (size_t)(4 * Dp + 4) * 4;
    const size_t bytes = per_query * nq + (size_t)nq * 4;
    void* scratch = nullptr;
    NWCCH_CUDA_TRY(scratch_alloc(&scratch, bytes, s));
    int32_t* wide = reinterpret_cast<int32_t*>(static_cast<char*>(scratch) + per_query * nq);
    const int32_t thr = (int32_t)(((int64_t)1 << 28) / (Dp + 1));  // |w| * (depth + 2) <= 2^28
    int rc = NWCCH_OK;
    if (cudaMemsetAsync(scratch, 0, bytes, s) != cudaSuccess) rc = NWCCH_ERR_CUDA;  // counters and flags at zero
    if (!rc) {
        k_qstream<<<(unsigned)(2 * nq), QS_THREADS, smem, s>>>(t->d, P->d_qnodes, P->dev.sn_id, up, dn, s_rank,
                                                                t_rank, nq, dist, thr, static_cast<int32_t*>(scratch),
                                                                wide, err, (int32_t)ring_words, (int32_t)item_words);
        if (cudaGetLastError() != cudaSuccess) rc = NWCCH_ERR_CUDA;
    }
    if (!rc) rc = query_sn64_flagged(t, up, dn, s_rank, t_rank, nq, dist, wide, err, s);
    const cudaError_t fe = cudaFreeAsync(scratch, s);
    if (rc) return rc;
    NWCCH_CUDA_TRY(fe);
    *launches = 2;
    *used = true;
    return NWCCH_OK;
}

}  // namespace nwcch
