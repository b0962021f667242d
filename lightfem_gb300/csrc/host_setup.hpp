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

// Level schedule of one IC(0) triangular sweep on a structurally symmetric CSR
// pattern (diag[r]: position of row r's diagonal).  Forward: row r depends on the
// columns left of its diagonal, in ascending column order; backward: row c on the
// columns right of its diagonal, in descending column order.  A row's level is one
// more than the deepest level it depends on.  Rows are listed level by level
// (forward: ascending row within a level; backward: descending).
struct SweepSchedule {
    int levels = 0;
    int max_width = 0;             // rows of the widest level
    long long max_distance = 0;    // largest (position of a row) - (position of a row it depends on)
    std::vector<int> level_begin;  // 2 per level + 2: first position, first entry; then the totals
    std::vector<int> desc;         // 4 per position: row, first entry, end entry, output index
    std::vector<int> dep;          // per entry: position of the row it depends on
    std::vector<int> position;     // per row: its position
};
// out_index(row) fills desc[4p + 3]; entries are numbered in schedule order.
void sweep_schedule(int n, const int* rowptr, const int* col, const int* diag, bool forward, SweepSchedule& s);

}  // namespace lfgpu
