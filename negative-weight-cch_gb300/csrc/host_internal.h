// Internal declarations shared by the host-side C++ sources of libnwcch.
#pragma once

#include <cstdint>
#include <vector>

namespace nwcch_host {

void undirected_csr(int64_t n, const int64_t* off, const int32_t* tgt, std::vector<int64_t>& noff,
                    std::vector<int32_t>& nbr);

void nested_dissection(int64_t n, const int64_t* noff, const int32_t* nbr, const double* x,
                       const double* y, int64_t leaf, int threads, std::vector<int32_t>& rank);

void symbolic(int64_t n, const int64_t* noff, const int32_t* nbr, const int32_t* rank,
              std::vector<int64_t>& first, std::vector<int32_t>& head,
              std::vector<int32_t>& parent);

int edge_arcs(int64_t n, const int64_t* off, const int32_t* tgt, const int32_t* rank,
              const int64_t* first, const int32_t* head, int64_t* e_arc, int8_t* e_up);

}  // namespace nwcch_host
