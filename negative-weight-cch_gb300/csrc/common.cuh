// Shared device-side definitions of libnwcch.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <mutex>
#include <tuple>
#include <utility>

#include "nwcch.h"

namespace nwcch {

constexpr int32_t INF32 = NWCCH_INF32;
constexpr int64_t INF64 = NWCCH_INF64;

// Bits of the per-topology device error word.
enum ErrBits : int {
    ERR_RANGE = 1,     // a finite (min,+) value was clamped to the storage range
    ERR_TIMEOUT = 2,   // a bounded spin-wait gave up
    ERR_CAPACITY = 4,  // a fixed-size buffer overflowed
    ERR_TOPOLOGY = 8,  // an arc that chordality guarantees was not found
    ERR_ARG = 16,      // an input value is invalid (weight equal to INF, id out of range)
};

// Storage of customized weights: INF is "no path", finite values live in
// [LO, HI]. Sums leaving that range are clamped (saturated) and flagged.
template <class T>
struct Lim;
template <>
struct Lim<int32_t> {
    static constexpr int32_t INF = INT32_MAX;
    static constexpr int32_t HI = INT32_MAX - 1;
    static constexpr int32_t LO = INT32_MIN + 1;
};
template <>
struct Lim<int64_t> {
    static constexpr int64_t INF = INT64_MAX;
    static constexpr int64_t HI = INT64_MAX - 1;
    static constexpr int64_t LO = INT64_MIN + 1;
};

// Candidate a + b of a (min,+) relaxation. Returns false when either side is
// INF (no path): the INF test comes before the addition, so INF plus a
// negative weight never looks finite.
__device__ __forceinline__ bool splus(int32_t a, int32_t b, int32_t& out, int& err) {
    if (a == Lim<int32_t>::INF || b == Lim<int32_t>::INF) return false;
    const int64_t s = (int64_t)a + (int64_t)b;
    if (s > Lim<int32_t>::HI) {
        out = Lim<int32_t>::HI;
        err |= ERR_RANGE;
    } else if (s < Lim<int32_t>::LO) {
        out = Lim<int32_t>::LO;
        err |= ERR_RANGE;
    } else {
        out = (int32_t)s;
    }
    return true;
}

__device__ __forceinline__ bool splus(int64_t a, int64_t b, int64_t& out, int& err) {
    if (a == Lim<int64_t>::INF || b == Lim<int64_t>::INF) return false;
    if (b > 0 && a > Lim<int64_t>::HI - b) {
        out = Lim<int64_t>::HI;
        err |= ERR_RANGE;
    } else if (b < 0 && a < Lim<int64_t>::LO - b) {
        out = Lim<int64_t>::LO;
        err |= ERR_RANGE;
    } else {
        out = a + b;
    }
    return true;
}

// Query labels are int64 whatever the storage; the result keeps INF64.
template <class T>
__device__ __forceinline__ int64_t label_plus(int64_t d, T w, int& err) {
    if (d == INF64 || w == Lim<T>::INF) return INF64;
    int64_t out;
    splus(d, (int64_t)w, out, err);
    return out;
}

// Sign of up + dn without overflow (the negative-cycle test).
template <class T>
__device__ __forceinline__ bool negative_pair(T u, T v) {
    if (u == Lim<T>::INF || v == Lim<T>::INF) return false;
    int64_t s;
    int e = 0;
    splus((int64_t)u, (int64_t)v, s, e);
    return s < 0;
}

// Programmatic dependent launch. A kernel of the customization sequence may
// be launched before the previous one has finished (its CTAs then occupy
// free SM slots instead of waiting for the launch); pdl_wait() blocks until
// the previous grid has completed and its memory is visible, so it comes
// before any global access. pdl_launch_dependents() lets the next grid's CTAs
// be scheduled once every CTA of this grid has started. Without the launch
// attribute both are no-ops.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" :::); }

// Launches `kernel` on s, allowed to start before the previous kernel on s
// has finished when `pdl` (the kernel must begin with pdl_wait()).
template <class... KArgs, class... Args>
cudaError_t launch_pdl(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// SMs of the current device, cached per device: grids are sized in multiples
// of it (1 if the device cannot be queried; the launch then reports the error).
inline int device_sms() {
    static int cache[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (dev >= 0 && dev < 64 && cache[dev] > 0) return cache[dev];
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) return 1;
    if (dev >= 0 && dev < 64) cache[dev] = sms;
    return sms;
}

// Raises the dynamic shared memory limit of `kernel` on the current device to
// at least `bytes`; never lowers it. The limit is a property of the function,
// shared by every host thread: if one thread could lower it between another
// thread's setting and launch, that launch would be refused. Growing it only
// keeps every concurrent launch valid (a launch's occupancy follows the
// shared memory it requests, not this limit).
inline cudaError_t allow_dynamic_smem(const void* kernel, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<const void*, int>, size_t> granted;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    size_t& g = granted[{kernel, dev}];
    if (bytes <= g) return cudaSuccess;
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) g = bytes;
    return e;
}

// Blocks per SM of `kernel` at `threads` threads and `smem` bytes of dynamic
// shared memory, asked once per (kernel, shape, device) and kept: the query
// paths size every launch by it, and a call of a latency-bound path should
// not wait on the occupancy calculator.
inline cudaError_t blocks_per_sm(const void* kernel, int threads, size_t smem, int* out) {
    static std::mutex mu;
    static std::map<std::tuple<const void*, int, size_t, int>, int> known;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_tuple(kernel, threads, smem, dev);
    auto it = known.find(key);
    if (it != known.end()) {
        *out = it->second;
        return cudaSuccess;
    }
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, kernel, threads, smem);
    if (e == cudaSuccess) known[key] = *out;
    return e;
}

// Stream-ordered scratch of the query paths, from a memory pool of this
// library (one per device) that keeps up to kScratchKeep bytes of freed
// memory for the next calls instead of returning it to the driver at every
// synchronization: a small query batch then allocates without mapping pages.
constexpr uint64_t kScratchKeep = (uint64_t)512 << 20;
inline cudaError_t scratch_alloc(void** p, size_t bytes, cudaStream_t s) {
    static std::mutex mu;
    static std::map<int, cudaMemPool_t> pools;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    cudaMemPool_t pool = nullptr;
    {
        std::lock_guard<std::mutex> lock(mu);
        auto it = pools.find(dev);
        if (it != pools.end()) {
            pool = it->second;
        } else {
            cudaMemPoolProps props = {};
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            if ((e = cudaMemPoolCreate(&pool, &props)) != cudaSuccess) return e;
            uint64_t keep = kScratchKeep;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            pools[dev] = pool;
        }
    }
    return cudaMallocFromPoolAsync(p, bytes, pool, s);
}
template <class T>
inline cudaError_t scratch_alloc(T** p, size_t bytes, cudaStream_t s) {
    void* v = nullptr;
    const cudaError_t e = scratch_alloc(&v, bytes, s);
    *p = static_cast<T*>(v);
    return e;
}

// Set-up copies and fills issued with the host-synchronous calls (cudaMemcpy
// from pageable memory, cudaMemset) run on the legacy default stream and may
// still be in flight when the call returns: a pageable upload returns once its
// data is staged, a fill returns at once. Work that a caller enqueues on a
// non-blocking stream is not ordered after them, so every builder of device
// arrays waits for them before the arrays can be used on any stream.
inline cudaError_t setup_copies_done() { return cudaStreamSynchronize(cudaStreamLegacy); }

#define NWCCH_CUDA_TRY(expr)                            \
    do {                                                \
        cudaError_t _e = (expr);                        \
        if (_e != cudaSuccess) return NWCCH_ERR_CUDA;   \
    } while (0)

}  // namespace nwcch
