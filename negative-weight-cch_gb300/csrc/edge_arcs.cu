// Original arcs -> shortcut arcs on the device (python/cch_nb.py:496-514):
// for the arc u -> v with ranks ru != rv, the shortcut (min, max) found by
// binary search in the row of the lower rank, upward if ru < rv; a self-loop
// (ru == rv) maps to -1. One thread per original vertex walks its arcs.

#include <algorithm>

#include "common.cuh"

namespace nwcch {

namespace {

__global__ void __launch_bounds__(256) k_edge_arcs(int64_t n, const int64_t* __restrict__ off,
                                                   const int32_t* __restrict__ tgt, const int32_t* __restrict__ rank,
                                                   const int64_t* __restrict__ first, const int32_t* __restrict__ head,
                                                   int64_t* __restrict__ e_arc, int8_t* __restrict__ e_up,
                                                   int* __restrict__ bad) {
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < n; u += (int64_t)gridDim.x * blockDim.x) {
        const int32_t ru = rank[u];
        for (int64_t k = off[u]; k < off[u + 1]; k++) {
            const int32_t v = tgt[k];
            if (v < 0 || v >= n) {
                atomicOr(bad, ERR_ARG);
                e_arc[k] = -1;
                e_up[k] = 0;
                continue;
            }
            const int32_t rv = rank[v];
            if (ru == rv) {
                e_arc[k] = -1;
                e_up[k] = 0;
                continue;
            }
            const int32_t lo = min(ru, rv), hi = max(ru, rv);
            int64_t a = first[lo], b = first[lo + 1];
            const int64_t end = b;
            while (a < b) {
                const int64_t mid = (a + b) >> 1;
                if (head[mid] < hi) a = mid + 1;
                else b = mid;
            }
            if (a >= end || head[a] != hi) {
                atomicOr(bad, ERR_TOPOLOGY);  // not chordal for this order
                a = -1;
            }
            e_arc[k] = a;
            e_up[k] = ru < rv ? 1 : 0;
        }
    }
}

}  // namespace

}  // namespace nwcch

using namespace nwcch;

extern "C" int nwcch_edge_arcs_device(int64_t n, const int64_t* off_dev, const int32_t* tgt_dev,
                                      const int32_t* rank_dev, const int64_t* first_dev, const int32_t* head_dev,
                                      int64_t* e_arc_dev, int8_t* e_up_dev, void* stream) {
    if (n < 0 || (n > 0 && (!off_dev || !tgt_dev || !rank_dev || !first_dev || !head_dev || !e_arc_dev || !e_up_dev)))
        return NWCCH_ERR_ARG;
    if (n == 0) return NWCCH_OK;
    cudaStream_t s = (cudaStream_t)stream;
    int* bad = nullptr;
    NWCCH_CUDA_TRY(scratch_alloc(&bad, sizeof(int), s));
    NWCCH_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), s));
    const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)device_sms() * 32));
    k_edge_arcs<<<blocks, 256, 0, s>>>(n, off_dev, tgt_dev, rank_dev, first_dev, head_dev, e_arc_dev, e_up_dev, bad);
    const cudaError_t launch = cudaGetLastError();
    int h = 0;
    const cudaError_t copy = cudaMemcpyAsync(&h, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(bad, s);
    NWCCH_CUDA_TRY(launch);
    NWCCH_CUDA_TRY(copy);
    NWCCH_CUDA_TRY(cudaStreamSynchronize(s));
    if (h & ERR_ARG) return NWCCH_ERR_ARG;
    if (h & ERR_TOPOLOGY) return NWCCH_ERR_TOPOLOGY;
    return NWCCH_OK;
}
