// The host element colouring (lightfem_gb300/csrc/host_setup.cpp) on a mesh read
// from a file: the first fit from per-node colour masks (greedy_colors) and the
// walk over node -> element lists it falls back to (greedy_colors_by_lists), both
// written out for the test to compare with each other and with the oracle.
//
//   colors_check <mesh file> <out file>
//   mesh file: int64 n_nodes, int64 n_elements, int32 element_nodes[4 * n_elements]
//   out file:  int32 colours (masks)[n_elements], int32 colours (lists)[n_elements]
#include "../../lightfem_gb300/csrc/host_setup.cpp"

#include <cstdio>
#include <vector>

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* in = std::fopen(argv[1], "rb");
    if (!in) return 2;
    long long head[2] = {0, 0};
    if (std::fread(head, sizeof(long long), 2, in) != 2) return 2;
    std::vector<int> en(static_cast<size_t>(4 * head[1]));
    if (std::fread(en.data(), sizeof(int), en.size(), in) != en.size()) return 2;
    std::fclose(in);
    std::vector<int> by_masks, by_lists;
    lfgpu::greedy_colors(head[0], head[1], en.data(), by_masks);
    lfgpu::greedy_colors_by_lists(head[0], head[1], en.data(), by_lists);
    FILE* out = std::fopen(argv[2], "wb");
    if (!out) return 2;
    std::fwrite(by_masks.data(), sizeof(int), by_masks.size(), out);
    std::fwrite(by_lists.data(), sizeof(int), by_lists.size(), out);
    std::fclose(out);
    return 0;
}
