// Internal entry points shared between the customization sources.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

struct nwcch_topology;

namespace nwcch {

int grid_for(int64_t count, int block);

// Fills up/dn with INF and scatters the minimum original weight of every arc,
// for `metrics` metrics stored metric-major (w: metrics x m, up/dn:
// metrics x m+); range errors go to the device word err.
template <class T>
int base_init(nwcch_topology* t, const int32_t* w, T* up, T* dn, cudaStream_t s, int* err, int metrics = 1);

}  // namespace nwcch
