// Device derivation of a topology's weight-independent arrays (internal).
#pragma once

#include <stdint.h>

#include <vector>

namespace nwcch {

struct DerivedTopology {
    // device outputs, allocated by the caller
    int32_t* tail = nullptr;         // [m+]
    int32_t* depth = nullptr;        // [n]
    int32_t* hdep = nullptr;         // [m+]
    int64_t* doff = nullptr;         // [n+1]
    int32_t* darc = nullptr;         // [m+]
    int32_t* vlevel = nullptr;       // [n]
    int64_t* aeoff = nullptr;        // [m+ + 1]
    int32_t* level_verts = nullptr;  // [n]
    // set by derive_topology
    int32_t* aeidx_sorted = nullptr;  // device [m], owned by the caller: aeidx, then the self-loops
    int64_t nloops = 0;
    int32_t max_deg = 0, max_depth = 0, levels = 0;
    int64_t triangles = 0;
    std::vector<int64_t> level_off, level_arc_off, level_tri;
    std::vector<int32_t> level_maxdeg;
};

// Validates the device copies of (first, head, parent, e_arc) and derives the
// rest on the device (NWCCH_ERR_TOPOLOGY when the input is not a valid
// contracted graph). Synchronous.
int derive_topology(int64_t n, int64_t mp, int64_t m, const int64_t* first, const int32_t* head,
                    const int32_t* parent, const int64_t* e_arc, DerivedTopology* out);

}  // namespace nwcch
