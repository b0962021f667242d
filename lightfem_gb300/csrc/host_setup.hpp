// Host-side setup of the solve path (host_setup.cpp).
#pragma once

#include <cstdint>
#include <vector>

namespace lfgpu {

struct HostPattern {
    long long n = 0, nnz = 0;
    std::vector<int64_t> rowptr;
    std::vector<int> col;
    std::vector<int> map;  // 64 per element, row-major 8x8
};

// en: 4 node indices per element.
HostPattern build_pattern(long long n_nodes, long long n_elem, const int* en);
int greedy_colors(long long n_nodes, long long n_elem, const int* en, std::vector<int>& colors);
void rcm_order(long long n_nodes, const long long* ids, long long n_elem, const long long* elem_ids, long long* order);
// Subdomain of every node for the subdomain block-Jacobi preconditioner: chunks of
// `per` consecutive nodes, or recursive coordinate bisection of xy (node index
// order).  Returns the subdomain count.
long long subdomain_split(long long n_nodes, const double* xy, long long per, bool rcb, std::vector<uint32_t>& owner);

}  // namespace lfgpu
