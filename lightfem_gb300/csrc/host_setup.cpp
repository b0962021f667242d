// Host-side setup of the solve path: CSR pattern + element->value map, greedy
// element colouring and reverse Cuthill-McKee ordering.  These produce exactly
// what the reference produces (the pattern and map bit-for-bit), from flat arrays
// and without hash containers.
//
//   build_pattern   build_csr_assembly_pattern + CsrMatrix::value_index,
//                   src/sparse.cpp:15-74
//   greedy_colors   element_colors, src/solver.cpp:100-133
//   rcm_order       reverse_cuthill_mckee, src/reordering.cpp:11-62
//   subdomain_split split_by_chunks / split_by_coordinates, src/precond.cpp:19-105
//   sweep_schedule  level schedule of IncompleteCholesky0::apply's two sweeps,
//                   src/precond.cpp:386-412 (no counterpart: the reference sweeps
//                   serially)
//
// A Q4 element couples both DOFs of each of its nodes, so rows 2i and 2i+1 share
// one column list {2j, 2j+1 : j in S(i)} where S(i) is the set of nodes sharing an
// element with node i (i included).  The pattern is therefore built per node: the
// sorted set S(i), then the two rows.  A node in no element keeps only its two
// diagonal entries, as the reference's pattern does.
#include "host_setup.hpp"

#include <algorithm>
#include <numeric>
#include <queue>
#include <stdexcept>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace lfgpu {

namespace {

// node -> elements touching it, in element order
void node_elements(long long n_nodes, long long n_elem, const int* en, std::vector<long long>& ptr,
                   std::vector<int>& list) {
    ptr.assign(static_cast<size_t>(n_nodes) + 1, 0);
    for (long long e = 0; e < n_elem; ++e)
        for (int a = 0; a < 4; ++a) ++ptr[static_cast<size_t>(en[4 * e + a]) + 1];
    for (long long i = 0; i < n_nodes; ++i) ptr[i + 1] += ptr[i];
    list.resize(static_cast<size_t>(ptr[n_nodes]));
    std::vector<long long> fill(ptr.begin(), ptr.end() - 1);
    for (long long e = 0; e < n_elem; ++e)
        for (int a = 0; a < 4; ++a) list[static_cast<size_t>(fill[en[4 * e + a]]++)] = static_cast<int>(e);
}

}  // namespace

HostPattern build_pattern(long long n_nodes, long long n_elem, const int* en) {
    HostPattern p;
    std::vector<long long> nptr;
    std::vector<int> nlist;
    node_elements(n_nodes, n_elem, en, nptr, nlist);

    // S(i) for every node.
    std::vector<long long> sptr(static_cast<size_t>(n_nodes) + 1, 0);
    std::vector<std::vector<int>> sets(static_cast<size_t>(n_nodes));
#pragma omp parallel for schedule(dynamic, 4096)
    for (long long i = 0; i < n_nodes; ++i) {
        std::vector<int>& s = sets[static_cast<size_t>(i)];
        for (long long k = nptr[i]; k < nptr[i + 1]; ++k) {
            const int e = nlist[static_cast<size_t>(k)];
            for (int a = 0; a < 4; ++a) s.push_back(en[4 * static_cast<long long>(e) + a]);
        }
        std::sort(s.begin(), s.end());
        s.erase(std::unique(s.begin(), s.end()), s.end());
    }
    const long long n = 2 * n_nodes;
    p.n = n;
    p.rowptr.assign(static_cast<size_t>(n) + 1, 0);
    for (long long i = 0; i < n_nodes; ++i) {
        const long long len = sets[i].empty() ? 1 : 2 * static_cast<long long>(sets[i].size());
        p.rowptr[2 * i + 1] = p.rowptr[2 * i] + len;
        p.rowptr[2 * i + 2] = p.rowptr[2 * i + 1] + len;
    }
    p.nnz = p.rowptr[n];
    if (p.nnz >= (1LL << 31)) throw std::length_error("pattern exceeds 2^31 nonzeros");
    p.col.resize(static_cast<size_t>(p.nnz));
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n_nodes; ++i) {
        const std::vector<int>& s = sets[static_cast<size_t>(i)];
        for (int half = 0; half < 2; ++half) {
            int* out = p.col.data() + p.rowptr[2 * i + half];
            if (s.empty()) {
                out[0] = static_cast<int>(2 * i + half);
                continue;
            }
            for (size_t k = 0; k < s.size(); ++k) {
                out[2 * k] = 2 * s[k];
                out[2 * k + 1] = 2 * s[k] + 1;
            }
        }
    }
    p.map.resize(static_cast<size_t>(n_elem) * 64);
#pragma omp parallel for schedule(static)
    for (long long e = 0; e < n_elem; ++e) {
        const int* nd = en + 4 * e;
        for (int a = 0; a < 4; ++a) {
            const std::vector<int>& s = sets[static_cast<size_t>(nd[a])];
            for (int b = 0; b < 4; ++b) {
                const int pos = static_cast<int>(std::lower_bound(s.begin(), s.end(), nd[b]) - s.begin());
                for (int i = 0; i < 2; ++i) {
                    const long long row = 2LL * nd[a] + i;
                    const long long base = p.rowptr[row] + 2LL * pos;
                    p.map[static_cast<size_t>(e) * 64 + (2 * a + i) * 8 + 2 * b] = static_cast<int>(base);
                    p.map[static_cast<size_t>(e) * 64 + (2 * a + i) * 8 + 2 * b + 1] = static_cast<int>(base + 1);
                }
            }
        }
    }
    return p;
}

// The stamp walk over node -> element lists, for any number of colours.
static int greedy_colors_by_lists(long long n_nodes, long long n_elem, const int* en, std::vector<int>& colors) {
    std::vector<long long> nptr;
    std::vector<int> nlist;
    node_elements(n_nodes, n_elem, en, nptr, nlist);
    colors.assign(static_cast<size_t>(n_elem), -1);
    std::vector<long long> stamp(static_cast<size_t>(n_elem) + 1, -1);
    int top = -1;
    for (long long e = 0; e < n_elem; ++e) {
        for (int a = 0; a < 4; ++a) {
            const int nd = en[4 * e + a];
            for (long long k = nptr[nd]; k < nptr[nd + 1]; ++k) {
                const int o = colors[static_cast<size_t>(nlist[static_cast<size_t>(k)])];
                if (o >= 0) stamp[static_cast<size_t>(o)] = e;
            }
        }
        int c = 0;
        while (stamp[static_cast<size_t>(c)] == e) ++c;
        colors[static_cast<size_t>(e)] = c;
        top = std::max(top, c);
    }
    return top + 1;
}

// The colours taken around element e are those of the earlier elements that share
// one of its nodes.  Each node keeps a bit mask of the colours of the elements
// coloured so far that touch it, so e takes the lowest colour missing from the
// union of its four nodes' masks: the same first fit as the stamp walk, without
// the node -> element lists (about 10x faster on a 1000x1000 mesh).  A mesh that
// would need a 65th colour is coloured again by the stamp walk.
int greedy_colors(long long n_nodes, long long n_elem, const int* en, std::vector<int>& colors) {
    colors.assign(static_cast<size_t>(n_elem), -1);
    std::vector<unsigned long long> used(static_cast<size_t>(n_nodes), 0ull);
    int top = -1;
    for (long long e = 0; e < n_elem; ++e) {
        const int* nd = en + 4 * e;
        const unsigned long long taken = used[static_cast<size_t>(nd[0])] | used[static_cast<size_t>(nd[1])] |
                                         used[static_cast<size_t>(nd[2])] | used[static_cast<size_t>(nd[3])];
        if (taken == ~0ull) return greedy_colors_by_lists(n_nodes, n_elem, en, colors);
        const int c = __builtin_ctzll(~taken);
        const unsigned long long bit = 1ull << c;
        for (int a = 0; a < 4; ++a) used[static_cast<size_t>(nd[a])] |= bit;
        colors[static_cast<size_t>(e)] = c;
        top = std::max(top, c);
    }
    return top + 1;
}

void rcm_order(long long n_nodes, const long long* ids, long long n_elem, const long long* elem_ids,
               long long* order) {
    // Work on node indices in ascending-ID order; ties in degree break by ID,
    // which is the index order here.
    std::vector<long long> sorted(ids, ids + n_nodes);
    std::sort(sorted.begin(), sorted.end());
    auto index_of = [&](long long id) {
        const auto it = std::lower_bound(sorted.begin(), sorted.end(), id);
        if (it == sorted.end() || *it != id) throw std::invalid_argument("element references an unknown node ID");
        return static_cast<int>(it - sorted.begin());
    };
    std::vector<int> en(static_cast<size_t>(n_elem) * 4);
    for (long long k = 0; k < 4 * n_elem; ++k) en[static_cast<size_t>(k)] = index_of(elem_ids[k]);
    std::vector<long long> nptr;
    std::vector<int> nlist;
    node_elements(n_nodes, n_elem, en.data(), nptr, nlist);
    std::vector<std::vector<int>> adj(static_cast<size_t>(n_nodes));
#pragma omp parallel for schedule(dynamic, 4096)
    for (long long i = 0; i < n_nodes; ++i) {
        std::vector<int>& s = adj[static_cast<size_t>(i)];
        for (long long k = nptr[i]; k < nptr[i + 1]; ++k) {
            const int e = nlist[static_cast<size_t>(k)];
            for (int a = 0; a < 4; ++a) {
                const int j = en[4 * static_cast<size_t>(e) + a];
                if (j != i) s.push_back(j);
            }
        }
        std::sort(s.begin(), s.end());
        s.erase(std::unique(s.begin(), s.end()), s.end());
    }
    auto before = [&](int a, int b) {
        const size_t da = adj[static_cast<size_t>(a)].size(), db = adj[static_cast<size_t>(b)].size();
        return da != db ? da < db : a < b;
    };
#pragma omp parallel for schedule(dynamic, 4096)
    for (long long i = 0; i < n_nodes; ++i) std::sort(adj[i].begin(), adj[i].end(), before);
    std::vector<int> seeds(static_cast<size_t>(n_nodes));
    std::iota(seeds.begin(), seeds.end(), 0);
    std::stable_sort(seeds.begin(), seeds.end(), before);
    std::vector<char> seen(static_cast<size_t>(n_nodes), 0);
    std::vector<int> out;
    out.reserve(static_cast<size_t>(n_nodes));
    std::vector<int> fifo(static_cast<size_t>(n_nodes));
    for (const int s : seeds) {
        if (seen[static_cast<size_t>(s)]) continue;
        seen[static_cast<size_t>(s)] = 1;
        size_t head = 0, tail = 0;
        fifo[tail++] = s;
        while (head < tail) {
            const int cur = fifo[head++];
            out.push_back(cur);
            for (const int v : adj[static_cast<size_t>(cur)])
                if (!seen[static_cast<size_t>(v)]) {
                    seen[static_cast<size_t>(v)] = 1;
                    fifo[tail++] = v;
                }
        }
    }
    for (long long k = 0; k < n_nodes; ++k) order[k] = sorted[static_cast<size_t>(out[static_cast<size_t>(n_nodes - 1 - k)])];
}

long long subdomain_split(long long n_nodes, const double* xy, long long per, bool rcb, std::vector<uint32_t>& owner) {
    const size_t nodes = static_cast<size_t>(std::max(0LL, n_nodes));
    const size_t target = static_cast<size_t>(std::max(1LL, per));
    owner.assign(nodes, 0);
    if (nodes == 0) return 0;
    if (!rcb) {
        for (size_t k = 0; k < nodes; ++k) owner[k] = static_cast<uint32_t>(k / target);
        return static_cast<long long>((nodes + target - 1) / target);
    }
    // Recursive bisection: the largest remaining range of the node permutation is
    // cut at its median across the longer side of its bounding box until the
    // wanted count is reached; ranges are numbered in the heap's storage order.
    // The heap operations and the median selection are the standard library's,
    // on size_t node indices, so ties between equal coordinates fall the same way
    // as in the reference.
    const size_t wanted = (nodes + target - 1) / target;
    std::vector<size_t> perm(nodes);
    std::iota(perm.begin(), perm.end(), size_t{0});
    struct Span {
        size_t first, last;  // [first, last) of perm
    };
    auto shorter = [](const Span& a, const Span& b) { return a.last - a.first < b.last - b.first; };
    std::vector<Span> spans{Span{0, nodes}};
    for (size_t have = 1; have < wanted; ++have) {
        std::pop_heap(spans.begin(), spans.end(), shorter);
        const Span cut = spans.back();
        spans.pop_back();
        if (cut.last - cut.first < 2) {  // only single nodes are left
            spans.push_back(cut);
            std::push_heap(spans.begin(), spans.end(), shorter);
            break;
        }
        double lo_x = xy[2 * perm[cut.first]], hi_x = lo_x;
        double lo_y = xy[2 * perm[cut.first] + 1], hi_y = lo_y;
        for (size_t k = cut.first + 1; k < cut.last; ++k) {
            const double px = xy[2 * perm[k]], py = xy[2 * perm[k] + 1];
            lo_x = std::min(lo_x, px);
            hi_x = std::max(hi_x, px);
            lo_y = std::min(lo_y, py);
            hi_y = std::max(hi_y, py);
        }
        const int axis = (hi_x - lo_x) >= (hi_y - lo_y) ? 0 : 1;
        const size_t half = cut.first + (cut.last - cut.first) / 2;
        std::nth_element(perm.begin() + static_cast<std::ptrdiff_t>(cut.first),
                         perm.begin() + static_cast<std::ptrdiff_t>(half),
                         perm.begin() + static_cast<std::ptrdiff_t>(cut.last),
                         [&](size_t a, size_t b) { return xy[2 * a + axis] < xy[2 * b + axis]; });
        spans.push_back(Span{cut.first, half});
        std::push_heap(spans.begin(), spans.end(), shorter);
        spans.push_back(Span{half, cut.last});
        std::push_heap(spans.begin(), spans.end(), shorter);
    }
    for (size_t s = 0; s < spans.size(); ++s)
        for (size_t k = spans[s].first; k < spans[s].last; ++k) owner[perm[k]] = static_cast<uint32_t>(s);
    return static_cast<long long>(spans.size());
}

void sweep_schedule(int n, const int* rowptr, const int* col, const int* diag, bool forward, SweepSchedule& s) {
    if (n < 0) throw std::invalid_argument("sweep_schedule: negative size");
    // Level of every row: forward rows ascending (dependencies are smaller rows),
    // backward rows descending (dependencies are larger rows).
    std::vector<int> level(static_cast<size_t>(n), 0);
    int levels = 0;
    auto visit = [&](int r) {
        int lv = 0;
        const int b = forward ? rowptr[r] : diag[r] + 1;
        const int e = forward ? diag[r] : rowptr[r + 1];
        for (int k = b; k < e; ++k) lv = std::max(lv, level[static_cast<size_t>(col[k])] + 1);
        level[static_cast<size_t>(r)] = lv;
        levels = std::max(levels, lv + 1);
    };
    if (forward) {
        for (int r = 0; r < n; ++r) visit(r);
    } else {
        for (int r = n - 1; r >= 0; --r) visit(r);
    }
    s.levels = levels;
    // Positions: counting sort by level, rows ascending (forward) or descending
    // (backward) within a level.
    std::vector<int> count(static_cast<size_t>(levels) + 1, 0);
    for (int r = 0; r < n; ++r) ++count[static_cast<size_t>(level[static_cast<size_t>(r)]) + 1];
    s.max_width = 0;
    for (int l = 0; l < levels; ++l) s.max_width = std::max(s.max_width, count[static_cast<size_t>(l) + 1]);
    for (int l = 0; l < levels; ++l) count[static_cast<size_t>(l) + 1] += count[static_cast<size_t>(l)];
    std::vector<int> fill(count.begin(), count.end() - 1);
    std::vector<int> order(static_cast<size_t>(n));
    s.position.assign(static_cast<size_t>(n), 0);
    for (int i = 0; i < n; ++i) {
        const int r = forward ? i : n - 1 - i;
        const int p = fill[static_cast<size_t>(level[static_cast<size_t>(r)])]++;
        order[static_cast<size_t>(p)] = r;
        s.position[static_cast<size_t>(r)] = p;
    }
    // Entries in schedule order; each row's entries in the reference's order.
    s.desc.assign(4 * static_cast<size_t>(n), 0);
    long long entries = 0;
    for (int r = 0; r < n; ++r) entries += forward ? diag[r] - rowptr[r] : rowptr[r + 1] - diag[r] - 1;
    if (entries > 2147483647LL) throw std::invalid_argument("sweep_schedule: too many entries");
    s.dep.assign(static_cast<size_t>(entries), 0);
    s.level_begin.assign(2 * (static_cast<size_t>(levels) + 1), 0);
    int j = 0;
    int l = 0;
    s.max_distance = 0;
    for (int p = 0; p < n; ++p) {
        const int r = order[static_cast<size_t>(p)];
        while (l < levels && count[static_cast<size_t>(l)] == p) {  // first position of level l
            s.level_begin[2 * static_cast<size_t>(l)] = p;
            s.level_begin[2 * static_cast<size_t>(l) + 1] = j;
            ++l;
        }
        const int jb = j;
        if (forward) {
            for (int k = rowptr[r]; k < diag[r]; ++k) s.dep[static_cast<size_t>(j++)] = s.position[static_cast<size_t>(col[k])];
        } else {
            for (int k = rowptr[r + 1] - 1; k > diag[r]; --k)
                s.dep[static_cast<size_t>(j++)] = s.position[static_cast<size_t>(col[k])];
        }
        for (int t = jb; t < j; ++t)
            s.max_distance = std::max<long long>(s.max_distance, p - s.dep[static_cast<size_t>(t)]);
        s.desc[4 * static_cast<size_t>(p)] = r;
        s.desc[4 * static_cast<size_t>(p) + 1] = jb;
        s.desc[4 * static_cast<size_t>(p) + 2] = j;
        s.desc[4 * static_cast<size_t>(p) + 3] = r;
    }
    s.level_begin[2 * static_cast<size_t>(levels)] = n;
    s.level_begin[2 * static_cast<size_t>(levels) + 1] = j;
}

}  // namespace lfgpu
