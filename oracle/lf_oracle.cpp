// lf_oracle — CPU restatement of the LightFEM solve path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the lightfem_gb300 package links, loads or
// calls this library; it is the checker for the GPU path (tests/, the smoke check)
// and the timed CPU baseline of bench.py.  It is pinned against golden vectors that
// the reference's own sources produce (tests/golden, made by ref_dump.cpp).
//
// Every function restates one reference function, cited by file:line, keeping the
// order of floating-point operations wherever the result is compared bit-for-bit
// or where iteration counts depend on it (PCG level-1 loops, Dirichlet, IC0).
// Storage mirrors the reference too: CSR keeps size_t offsets and columns
// (16 bytes per nonzero with the value) and the SpMV is row-parallel OpenMP with a
// static schedule, so the CPU baseline moves the same bytes the reference moves.
// Built with -ffp-contract=off: no fused multiply-add on either host architecture.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <numeric>
#include <queue>
#include <stdexcept>
#include <vector>

#include <omp.h>

namespace {

using std::size_t;
using i64 = long long;

double now_ms() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// ---------------------------------------------------------------- element kernels
// constitutive_matrix, src/element.cpp:16-32.
void constitutive(double e, double nu, int plane_strain, double d[9]) {
    if (!plane_strain) {
        const double f = e / (1.0 - nu * nu);
        const double v[9] = {f, f * nu, 0.0, f * nu, f, 0.0, 0.0, 0.0, f * (1.0 - nu) * 0.5};
        std::memcpy(d, v, sizeof v);
    } else {
        const double f = e / ((1.0 + nu) * (1.0 - 2.0 * nu));
        const double v[9] = {f * (1.0 - nu), f * nu, 0.0, f * nu, f * (1.0 - nu), 0.0,
                             0.0, 0.0, f * (1.0 - 2.0 * nu) * 0.5};
        std::memcpy(d, v, sizeof v);
    }
}

// q4_kinematics, src/element.cpp:34-73.  Returns false for a non-positive Jacobian.
bool kinematics(const double xy[8], double xi, double eta, double b[24], double* det_out) {
    const double dxi[4] = {-0.25 * (1.0 - eta), +0.25 * (1.0 - eta), +0.25 * (1.0 + eta), -0.25 * (1.0 + eta)};
    const double deta[4] = {-0.25 * (1.0 - xi), -0.25 * (1.0 + xi), +0.25 * (1.0 + xi), +0.25 * (1.0 - xi)};
    double j00 = 0.0, j01 = 0.0, j10 = 0.0, j11 = 0.0;  // dx/dxi, dx/deta, dy/dxi, dy/deta
    for (int i = 0; i < 4; ++i) {
        j00 += dxi[i] * xy[2 * i];
        j01 += deta[i] * xy[2 * i];
        j10 += dxi[i] * xy[2 * i + 1];
        j11 += deta[i] * xy[2 * i + 1];
    }
    const double det = j00 * j11 - j01 * j10;
    if (!(det > 1.0e-14) || !std::isfinite(det)) return false;
    const double i00 = j11 / det, i01 = -j01 / det, i10 = -j10 / det, i11 = j00 / det;
    for (int i = 0; i < 4; ++i) {
        const double nx = i00 * dxi[i] + i10 * deta[i];
        const double ny = i01 * dxi[i] + i11 * deta[i];
        b[2 * i] = nx;
        b[2 * i + 1] = 0.0;
        b[8 + 2 * i] = 0.0;
        b[8 + 2 * i + 1] = ny;
        b[16 + 2 * i] = ny;
        b[16 + 2 * i + 1] = nx;
    }
    *det_out = det;
    return true;
}

constexpr double kGauss = 0.57735026918962576451;
const double kPoints[4][2] = {{-kGauss, -kGauss}, {kGauss, -kGauss}, {kGauss, kGauss}, {-kGauss, kGauss}};

// q4_stiffness, src/element.cpp:130-161.
bool q4_stiffness(const double xy[8], double e, double nu, double t, int plane_strain, double k[64]) {
    double d[9];
    constitutive(e, nu, plane_strain, d);
    std::fill(k, k + 64, 0.0);
    for (const auto& p : kPoints) {
        double b[24], det;
        if (!kinematics(xy, p[0], p[1], b, &det)) return false;
        double db[24] = {};
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 8; ++c)
                for (int s = 0; s < 3; ++s) db[8 * r + c] += d[3 * r + s] * b[8 * s + c];
        const double w = det * t;
        for (int r = 0; r < 8; ++r)
            for (int c = 0; c < 8; ++c) {
                double acc = 0.0;
                for (int s = 0; s < 3; ++s) acc += b[8 * s + r] * db[8 * s + c];
                k[8 * r + c] += acc * w;
            }
    }
    return true;
}

// q4_body_force, src/element.cpp:163-180.
bool q4_body_force(const double xy[8], double t, double bx, double by, double out[8]) {
    std::fill(out, out + 8, 0.0);
    for (const auto& p : kPoints) {
        double b[24], det;
        if (!kinematics(xy, p[0], p[1], b, &det)) return false;
        const double xi = p[0], eta = p[1];
        const double n[4] = {0.25 * (1.0 - xi) * (1.0 - eta), 0.25 * (1.0 + xi) * (1.0 - eta),
                             0.25 * (1.0 + xi) * (1.0 + eta), 0.25 * (1.0 - xi) * (1.0 + eta)};
        const double w = det * t;
        for (int a = 0; a < 4; ++a) {
            out[2 * a] += n[a] * bx * w;
            out[2 * a + 1] += n[a] * by * w;
        }
    }
    return true;
}

// q4_edge_traction / q4_edge_pressure, src/element.cpp:182-210 (edge_nodes :102-110).
bool q4_edge_load(const double xy[8], double t, int edge, int pressure, double a, double bval, double out[8]) {
    std::fill(out, out + 8, 0.0);
    if (edge < 1 || edge > 4) return false;
    const int first = edge - 1, second = edge % 4;
    const double dx = xy[2 * second] - xy[2 * first];
    const double dy = xy[2 * second + 1] - xy[2 * first + 1];
    const double len = std::hypot(dx, dy);
    if (!(len > 1.0e-14)) return false;
    double tx = a, ty = bval;
    if (pressure) {
        tx = -a * dy / len;
        ty = a * dx / len;
    }
    const double w = 0.5 * len * t;
    out[2 * first] = w * tx;
    out[2 * first + 1] = w * ty;
    out[2 * second] = w * tx;
    out[2 * second + 1] = w * ty;
    return true;
}

// ---------------------------------------------------------------- sparse storage
struct Csr {
    size_t n = 0;
    std::vector<size_t> ptr{0};
    std::vector<size_t> col;
    std::vector<double> val;

    size_t index_of(size_t r, size_t c) const {
        const auto b = col.begin() + static_cast<std::ptrdiff_t>(ptr[r]);
        const auto e = col.begin() + static_cast<std::ptrdiff_t>(ptr[r + 1]);
        const auto it = std::lower_bound(b, e, c);
        if (it == e || *it != c) throw std::logic_error("entry absent from pattern");
        return static_cast<size_t>(it - col.begin());
    }

    // CsrMatrix::multiply_into, src/sparse.cpp:104-120.
    void spmv(const double* x, double* y) const {
#pragma omp parallel for schedule(static)
        for (long long ri = 0; ri < static_cast<long long>(n); ++ri) {
            const size_t r = static_cast<size_t>(ri);
            double s = 0.0;
            for (size_t k = ptr[r]; k < ptr[r + 1]; ++k) s += val[k] * x[col[k]];
            y[r] = s;
        }
    }
};

// BsrMatrix, src/sparse.cpp:128-204.
struct Bsr {
    size_t n = 0;
    std::vector<size_t> ptr{0};
    std::vector<uint32_t> col;
    std::vector<double> val;

    static Bsr from_csr(const Csr& a) {
        if (a.n % 2 != 0) throw std::invalid_argument("odd dimension");
        Bsr b;
        b.n = a.n;
        const size_t none = std::numeric_limits<size_t>::max();
        for (size_t br = 0; br < a.n / 2; ++br) {
            size_t p0 = a.ptr[2 * br], p1 = a.ptr[2 * br + 1];
            const size_t e0 = a.ptr[2 * br + 1], e1 = a.ptr[2 * br + 2];
            while (p0 < e0 || p1 < e1) {
                const size_t c0 = p0 < e0 ? a.col[p0] : none;
                const size_t c1 = p1 < e1 ? a.col[p1] : none;
                const size_t bc = std::min(c0, c1) / 2;
                b.col.push_back(static_cast<uint32_t>(bc));
                double blk[4] = {0.0, 0.0, 0.0, 0.0};
                for (; p0 < e0 && a.col[p0] / 2 == bc; ++p0) blk[a.col[p0] - 2 * bc] = a.val[p0];
                for (; p1 < e1 && a.col[p1] / 2 == bc; ++p1) blk[2 + a.col[p1] - 2 * bc] = a.val[p1];
                b.val.insert(b.val.end(), blk, blk + 4);
            }
            b.ptr.push_back(b.col.size());
        }
        return b;
    }

    void spmv(const double* x, double* y) const {
        const long long rows = static_cast<long long>(n / 2);
#pragma omp parallel for schedule(static)
        for (long long bri = 0; bri < rows; ++bri) {
            const size_t br = static_cast<size_t>(bri);
            double s0 = 0.0, s1 = 0.0;
            for (size_t k = ptr[br]; k < ptr[br + 1]; ++k) {
                const size_t c = 2 * static_cast<size_t>(col[k]);
                const double* blk = &val[4 * k];
                const double x0 = x[c], x1 = x[c + 1];
                s0 += blk[0] * x0 + blk[1] * x1;
                s1 += blk[2] * x0 + blk[3] * x1;
            }
            y[2 * br] = s0;
            y[2 * br + 1] = s1;
        }
    }
};

// ---------------------------------------------------------------- preconditioners
struct Precond {
    virtual ~Precond() = default;
    virtual void apply(const double* in, double* out) const = 0;
    mutable double apply_ms = 0.0;
};

// JacobiPreconditioner + inverse_diagonal_of, src/solver.cpp:497-509, 656-669.
struct Jacobi : Precond {
    std::vector<double> inv;
    explicit Jacobi(const Csr& a) : inv(a.n) {
        for (size_t i = 0; i < a.n; ++i) {
            const double d = a.val[a.index_of(i, i)];
            if (!std::isfinite(d)) throw std::runtime_error("Jacobi preconditioner encountered a non-finite diagonal");
            inv[i] = std::abs(d) > 1.0e-30 ? 1.0 / d : 1.0;
        }
    }
    void apply(const double* in, double* out) const override {
        for (size_t i = 0; i < inv.size(); ++i) out[i] = inv[i] * in[i];
    }
};

// split_by_chunks / split_by_coordinates, src/precond.cpp:19-105.
std::vector<uint32_t> chunk_split(size_t nodes, size_t per, size_t* count) {
    const size_t size = std::max<size_t>(1, per);
    std::vector<uint32_t> owner(nodes);
    for (size_t k = 0; k < nodes; ++k) owner[k] = static_cast<uint32_t>(k / size);
    *count = nodes == 0 ? 0 : (nodes + size - 1) / size;
    return owner;
}

std::vector<uint32_t> rcb_split(const std::vector<double>& x, const std::vector<double>& y, size_t per, size_t* count) {
    const size_t nodes = std::min(x.size(), y.size());
    std::vector<uint32_t> owner(nodes, 0);
    *count = 0;
    if (nodes == 0) return owner;
    const size_t target = std::max<size_t>(1, per);
    const size_t wanted = (nodes + target - 1) / target;
    std::vector<size_t> order(nodes);
    std::iota(order.begin(), order.end(), size_t{0});
    struct Piece { size_t lo, hi; };
    const auto smaller = [](const Piece& a, const Piece& b) { return (a.hi - a.lo) < (b.hi - b.lo); };
    std::vector<Piece> heap{{0, nodes}};
    for (size_t pieces = 1; pieces < wanted; ++pieces) {
        std::pop_heap(heap.begin(), heap.end(), smaller);
        const Piece p = heap.back();
        heap.pop_back();
        const size_t len = p.hi - p.lo;
        if (len < 2) {
            heap.push_back(p);
            std::push_heap(heap.begin(), heap.end(), smaller);
            break;
        }
        double x0 = x[order[p.lo]], x1 = x0, y0 = y[order[p.lo]], y1 = y0;
        for (size_t i = p.lo + 1; i < p.hi; ++i) {
            x0 = std::min(x0, x[order[i]]);
            x1 = std::max(x1, x[order[i]]);
            y0 = std::min(y0, y[order[i]]);
            y1 = std::max(y1, y[order[i]]);
        }
        const bool along_x = (x1 - x0) >= (y1 - y0);
        const size_t mid = p.lo + len / 2;
        std::nth_element(order.begin() + static_cast<std::ptrdiff_t>(p.lo), order.begin() + static_cast<std::ptrdiff_t>(mid),
                         order.begin() + static_cast<std::ptrdiff_t>(p.hi),
                         [&](size_t a, size_t b) { return along_x ? x[a] < x[b] : y[a] < y[b]; });
        heap.push_back({p.lo, mid});
        std::push_heap(heap.begin(), heap.end(), smaller);
        heap.push_back({mid, p.hi});
        std::push_heap(heap.begin(), heap.end(), smaller);
    }
    uint32_t next = 0;
    for (const Piece& p : heap) {
        for (size_t i = p.lo; i < p.hi; ++i) owner[order[i]] = next;
        ++next;
    }
    *count = next;
    return owner;
}

// SubdomainBlockJacobi, src/precond.cpp:107-291: dense packed Cholesky per
// subdomain with reciprocal pivots; a failed block becomes the identity.
struct BlockJacobi : Precond {
    size_t n = 0, count = 0, largest = 0;
    std::vector<size_t> begin;
    std::vector<uint32_t> dofs;
    std::vector<size_t> fbegin;
    std::vector<double> factor;
    double capture = 0.0;
    size_t degenerate = 0;

    BlockJacobi(const Csr& a, const std::vector<uint32_t>& owner, size_t subdomains) : n(a.n), count(subdomains) {
        size_t inside = 0;
        for (size_t r = 0; r < n; ++r)
            for (size_t k = a.ptr[r]; k < a.ptr[r + 1]; ++k) inside += owner[a.col[k]] == owner[r];
        capture = a.val.empty() || count == 0 ? 0.0 : static_cast<double>(inside) / static_cast<double>(a.val.size());
        if (count == 0) return;
        std::vector<size_t> sizes(count, 0);
        for (const uint32_t o : owner) ++sizes[o];
        begin.assign(count + 1, 0);
        for (size_t s = 0; s < count; ++s) begin[s + 1] = begin[s] + sizes[s];
        dofs.resize(begin.back());
        std::vector<size_t> cursor(begin.begin(), begin.end() - 1);
        for (size_t d = 0; d < n; ++d) dofs[cursor[owner[d]]++] = static_cast<uint32_t>(d);
        std::vector<size_t> slot(n, 0);
        for (size_t s = 0; s < count; ++s)
            for (size_t i = begin[s]; i < begin[s + 1]; ++i) slot[dofs[i]] = i;
        fbegin.assign(count + 1, 0);
        for (size_t s = 0; s < count; ++s) {
            fbegin[s + 1] = fbegin[s] + sizes[s] * (sizes[s] + 1) / 2;
            largest = std::max(largest, sizes[s]);
        }
        factor.assign(fbegin.back(), 0.0);
        std::vector<char> bad(count, 0);
#pragma omp parallel for schedule(dynamic, 8)
        for (long long si = 0; si < static_cast<long long>(count); ++si) {
            const size_t s = static_cast<size_t>(si);
            const size_t b0 = begin[s], m = begin[s + 1] - b0;
            if (m == 0) continue;
            std::vector<double> dense(m * m, 0.0);
            for (size_t i = 0; i < m; ++i) {
                const size_t d = dofs[b0 + i];
                for (size_t k = a.ptr[d]; k < a.ptr[d + 1]; ++k) {
                    if (owner[a.col[k]] != s) continue;
                    dense[i * m + (slot[a.col[k]] - b0)] = a.val[k];
                }
            }
            bool ok = true;
            for (size_t i = 0; i < m && ok; ++i)
                for (size_t j = 0; j <= i; ++j) {
                    double sum = dense[i * m + j];
                    for (size_t k = 0; k < j; ++k) sum -= dense[i * m + k] * dense[j * m + k];
                    if (i == j) {
                        if (!(sum > 0.0) || !std::isfinite(sum)) {
                            ok = false;
                            break;
                        }
                        dense[i * m + i] = std::sqrt(sum);
                    } else {
                        dense[i * m + j] = sum / dense[j * m + j];
                    }
                }
            if (!ok) {
                bad[s] = 1;
                for (size_t i = 0; i < m; ++i)
                    for (size_t j = 0; j <= i; ++j) dense[i * m + j] = i == j ? 1.0 : 0.0;
            }
            double* f = &factor[fbegin[s]];
            for (size_t i = 0; i < m; ++i) {
                for (size_t j = 0; j <= i; ++j) f[i * (i + 1) / 2 + j] = dense[i * m + j];
                f[i * (i + 1) / 2 + i] = 1.0 / f[i * (i + 1) / 2 + i];
            }
        }
        for (const char b : bad) degenerate += b;
    }

    void apply(const double* in, double* out) const override {
#pragma omp parallel
        {
            std::vector<double> w(largest);
#pragma omp for schedule(dynamic, 8)
            for (long long si = 0; si < static_cast<long long>(count); ++si) {
                const size_t s = static_cast<size_t>(si);
                const size_t b0 = begin[s], m = begin[s + 1] - b0;
                if (m == 0) continue;
                const double* f = &factor[fbegin[s]];
                for (size_t i = 0; i < m; ++i) w[i] = in[dofs[b0 + i]];
                size_t base = 0;
                for (size_t i = 0; i < m; ++i) {
                    double sum = w[i];
                    for (size_t k = 0; k < i; ++k) sum -= f[base + k] * w[k];
                    w[i] = sum * f[base + i];
                    base += i + 1;
                }
                const size_t last = (m - 1) * m / 2;
                for (size_t i = m; i-- > 0;) {
                    double sum = w[i];
                    size_t start = last;
                    for (size_t k = m - 1; k > i; --k) {
                        sum -= f[start + i] * w[k];
                        start -= k;
                    }
                    w[i] = sum * f[i * (i + 1) / 2 + i];
                }
                for (size_t i = 0; i < m; ++i) out[dofs[b0 + i]] = w[i];
            }
        }
    }
};

// IncompleteCholesky0, src/precond.cpp:298-412.
struct Ic0 : Precond {
    size_t n = 0;
    std::vector<size_t> ptr{0};
    std::vector<uint32_t> col;
    std::vector<double> val, inv;
    size_t breakdowns = 0;

    explicit Ic0(const Csr& a) : n(a.n), inv(a.n, 1.0) {
        std::vector<size_t> diag(n, 0);
        for (size_t r = 0; r < n; ++r) {
            bool found = false;
            for (size_t k = a.ptr[r]; k < a.ptr[r + 1]; ++k) {
                if (a.col[k] > r) break;
                col.push_back(static_cast<uint32_t>(a.col[k]));
                val.push_back(a.val[k]);
                if (a.col[k] == r) {
                    diag[r] = val.size() - 1;
                    found = true;
                }
            }
            if (!found) {
                col.push_back(static_cast<uint32_t>(r));
                val.push_back(1.0);
                diag[r] = val.size() - 1;
            }
            ptr.push_back(val.size());
        }
        double scale = 0.0;
        for (size_t r = 0; r < n; ++r) scale = std::max(scale, std::abs(val[diag[r]]));
        const double floor_value = std::max(1.0e-30, 1.0e-14 * scale);
        for (size_t r = 0; r < n; ++r) {
            const size_t b = ptr[r], dg = diag[r];
            for (size_t k = b; k < dg; ++k) {
                const size_t c = col[k];
                double sum = val[k];
                size_t p = b, q = ptr[c];
                const size_t qend = diag[c];
                while (p < k && q < qend) {
                    if (col[p] < col[q]) {
                        ++p;
                    } else if (col[p] > col[q]) {
                        ++q;
                    } else {
                        sum -= val[p] * val[q];
                        ++p;
                        ++q;
                    }
                }
                val[k] = sum * inv[c];
            }
            double sum = val[dg];
            for (size_t k = b; k < dg; ++k) sum -= val[k] * val[k];
            if (!(sum > 0.0) || !std::isfinite(sum)) {
                ++breakdowns;
                sum = floor_value;
            }
            const double pivot = std::sqrt(sum);
            val[dg] = pivot;
            inv[r] = 1.0 / pivot;
        }
    }

    void apply(const double* in, double* out) const override {
        std::copy(in, in + n, out);
        for (size_t r = 0; r < n; ++r) {
            double sum = out[r];
            for (size_t k = ptr[r]; k + 1 < ptr[r + 1]; ++k) sum -= val[k] * out[col[k]];
            out[r] = sum * inv[r];
        }
        for (size_t r = n; r-- > 0;) {
            out[r] *= inv[r];
            const double v = out[r];
            for (size_t k = ptr[r]; k + 1 < ptr[r + 1]; ++k) out[col[k]] -= val[k] * v;
        }
    }
};

// ---------------------------------------------------------------- PCG
struct Report {
    double converged, iterations, initial_residual, final_residual, solve_ms, matvec_ms, matvec_calls,
        precond_apply_ms, status;
};

// pcg_solve<Matrix, Preconditioner>, src/solver.cpp:532-627.  status: 0 ok/maxit,
// 1 non-positive initial rho, 2 non-positive curvature, 3 non-positive rho.
// ``iteration_cap`` > 0 stops early without a convergence decision (bounded CPU-baseline samples).
template <typename M>
Report pcg(const M& a, const Precond& m, const double* b, double tol, size_t maxit, double* x, size_t iteration_cap) {
    const size_t n = a.n;
    Report rep{};
    const double t0 = now_ms();
    double mv_ms = 0.0;
    size_t mv = 0;
    std::vector<double> r(b, b + n), z(n, 0.0), p(n, 0.0), q(n, 0.0);
    std::fill(x, x + n, 0.0);
    auto finish = [&]() {
        rep.solve_ms = now_ms() - t0;
        rep.matvec_ms = mv_ms;
        rep.matvec_calls = static_cast<double>(mv);
        rep.precond_apply_ms = m.apply_ms;
        return rep;
    };
    auto precondition = [&]() {
        const double s = now_ms();
        m.apply(r.data(), z.data());
        m.apply_ms += now_ms() - s;
    };
    precondition();
    double rr = 0.0, rho = 0.0;
    for (size_t i = 0; i < n; ++i) {
        const double v = r[i];
        rr += v * v;
        p[i] = z[i];
        rho += v * z[i];
    }
    rep.initial_residual = std::sqrt(std::max(0.0, rr));
    const double target = tol * std::max(1.0, rep.initial_residual);
    if (rep.initial_residual <= target) {
        rep.converged = 1;
        rep.final_residual = rep.initial_residual;
        return finish();
    }
    if (!(rho > 0.0) || !std::isfinite(rho)) {
        rep.status = 1;
        return finish();
    }
    for (size_t it = 1; it <= maxit; ++it) {
        const double s = now_ms();
        a.spmv(p.data(), q.data());
        mv_ms += now_ms() - s;
        ++mv;
        double curv = 0.0;
        for (size_t i = 0; i < n; ++i) curv += p[i] * q[i];
        if (!(curv > 0.0) || !std::isfinite(curv)) {
            rep.status = 2;
            return finish();
        }
        const double alpha = rho / curv;
        rr = 0.0;
        for (size_t i = 0; i < n; ++i) {
            x[i] += alpha * p[i];
            const double v = r[i] - alpha * q[i];
            r[i] = v;
            rr += v * v;
        }
        rep.iterations = static_cast<double>(it);
        rep.final_residual = std::sqrt(std::max(0.0, rr));
        if (rep.final_residual <= target) {
            rep.converged = 1;
            return finish();
        }
        if (iteration_cap != 0 && it >= iteration_cap) return finish();
        precondition();
        double next = 0.0;
        for (size_t i = 0; i < n; ++i) next += r[i] * z[i];
        if (!(next > 0.0) || !std::isfinite(next)) {
            rep.status = 3;
            return finish();
        }
        const double beta = next / rho;
        for (size_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
        rho = next;
    }
    rep.final_residual = std::sqrt(std::max(0.0, rr));
    return finish();
}

Csr make_csr(i64 n, const i64* ptr, const i64* col, const double* val) {
    Csr a;
    a.n = static_cast<size_t>(n);
    a.ptr.assign(ptr, ptr + n + 1);
    a.col.assign(col, col + ptr[n]);
    a.val.assign(val, val + ptr[n]);
    return a;
}

struct Pattern {
    std::vector<i64> ptr, col, map;
};

}  // namespace

extern "C" {

int lfo_num_threads() { return omp_get_max_threads(); }
void lfo_set_threads(int t) {
    if (t > 0) omp_set_num_threads(t);
}

int lfo_q4_stiffness(const double* xy, double e, double nu, double t, int plane_strain, double* k) {
    return q4_stiffness(xy, e, nu, t, plane_strain, k) ? 0 : -1;
}

// build_csr_assembly_pattern + CsrMatrix::value_index, src/sparse.cpp:15-74.  The
// per-row column set is gathered by sort + unique instead of a hash set; the
// resulting pattern (diagonal always present, columns ascending) is the same.
void* lfo_pattern_build(i64 n, i64 n_elem, i64 per, const i64* dofs) {
    auto* p = new Pattern;
    std::vector<std::vector<i64>> rows(static_cast<size_t>(n));
    for (i64 r = 0; r < n; ++r) rows[r].push_back(r);
    for (i64 e = 0; e < n_elem; ++e)
        for (i64 a = 0; a < per; ++a)
            for (i64 b = 0; b < per; ++b) rows[dofs[e * per + a]].push_back(dofs[e * per + b]);
    p->ptr.assign(static_cast<size_t>(n) + 1, 0);
    for (i64 r = 0; r < n; ++r) {
        auto& v = rows[r];
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        p->ptr[r + 1] = p->ptr[r] + static_cast<i64>(v.size());
    }
    p->col.reserve(static_cast<size_t>(p->ptr[n]));
    for (auto& v : rows) p->col.insert(p->col.end(), v.begin(), v.end());
    p->map.resize(static_cast<size_t>(n_elem * per * per));
    for (i64 e = 0; e < n_elem; ++e)
        for (i64 a = 0; a < per; ++a) {
            const i64 r = dofs[e * per + a];
            for (i64 b = 0; b < per; ++b) {
                const i64 c = dofs[e * per + b];
                const auto lo = p->col.begin() + p->ptr[r], hi = p->col.begin() + p->ptr[r + 1];
                p->map[e * per * per + a * per + b] = std::lower_bound(lo, hi, c) - p->col.begin();
            }
        }
    return p;
}
i64 lfo_pattern_nnz(void* h) { return static_cast<Pattern*>(h)->ptr.back(); }
void lfo_pattern_copy(void* h, i64* ptr, i64* col, i64* map) {
    auto* p = static_cast<Pattern*>(h);
    std::copy(p->ptr.begin(), p->ptr.end(), ptr);
    std::copy(p->col.begin(), p->col.end(), col);
    std::copy(p->map.begin(), p->map.end(), map);
}
void lfo_pattern_free(void* h) { delete static_cast<Pattern*>(h); }

// element_colors, src/solver.cpp:100-133: greedy first fit in element order over
// elements that share a node.
i64 lfo_element_colors(i64 n_nodes, i64 n_elem, const i64* nodes, i64* colors) {
    std::vector<std::vector<i64>> touching(static_cast<size_t>(n_nodes));
    for (i64 e = 0; e < n_elem; ++e)
        for (int a = 0; a < 4; ++a) touching[nodes[4 * e + a]].push_back(e);
    std::vector<i64> stamp(static_cast<size_t>(n_elem) + 1, 0);
    i64 top = -1;
    for (i64 e = 0; e < n_elem; ++e) colors[e] = -1;
    for (i64 e = 0; e < n_elem; ++e) {
        for (int a = 0; a < 4; ++a)
            for (const i64 o : touching[nodes[4 * e + a]])
                if (colors[o] >= 0) stamp[colors[o]] = e + 1;
        i64 c = 0;
        while (stamp[c] == e + 1) ++c;
        colors[e] = c;
        top = std::max(top, c);
    }
    return top + 1;
}

// Element stiffness + scatter through the map in the given element order (serial
// strategy: natural order; colouring: colour groups in turn), src/solver.cpp:135-179
// with the per-element matrices of src/solver.cpp:244-270.  Returns -1 - e for a
// non-positive Jacobian in element e.
// With colour groups (color_ptr[n_colors + 1] offsets into `order`, elements of one
// colour sharing no node) each colour's scatter is a parallel loop, as
// coloring_assembly runs it (src/solver.cpp:163-179); every value still receives
// its terms in colour order, so the result equals the serial scatter bit for bit.
i64 lfo_assemble(const double* xy, i64 n_elem, const i64* nodes, const double* young, const double* poisson,
                 const double* thick, int plane_strain, const i64* map, const i64* order, double* values,
                 const i64* color_ptr, i64 n_colors) {
    std::vector<double> ke(static_cast<size_t>(n_elem) * 64);
    i64 bad = 0;
#pragma omp parallel for schedule(static)
    for (i64 e = 0; e < n_elem; ++e) {
        double c[8];
        for (int a = 0; a < 4; ++a) {
            c[2 * a] = xy[2 * nodes[4 * e + a]];
            c[2 * a + 1] = xy[2 * nodes[4 * e + a] + 1];
        }
        if (!q4_stiffness(c, young[e], poisson[e], thick[e], plane_strain, &ke[static_cast<size_t>(e) * 64])) {
#pragma omp critical
            bad = bad == 0 ? -1 - e : bad;
        }
    }
    if (bad != 0) return bad;
    if (order && color_ptr && n_colors > 0) {
        for (i64 c = 0; c < n_colors; ++c) {
#pragma omp parallel for schedule(static)
            for (i64 k = color_ptr[c]; k < color_ptr[c + 1]; ++k) {
                const i64 e = order[k];
                for (int j = 0; j < 64; ++j) values[map[e * 64 + j]] += ke[static_cast<size_t>(e) * 64 + j];
            }
        }
        return 0;
    }
    for (i64 k = 0; k < n_elem; ++k) {
        const i64 e = order ? order[k] : k;
        for (int j = 0; j < 64; ++j) values[map[e * 64 + j]] += ke[static_cast<size_t>(e) * 64 + j];
    }
    return 0;
}

// Load vector of src/solver.cpp:303-332: nodal loads (already summed in f by the
// caller), then body forces, then edge loads, each in record order.
int lfo_element_loads(const double* xy, const i64* nodes, const double* thick, i64 n_body, const i64* body_elem,
                      const double* bx, const double* by, i64 n_edge, const i64* edge_elem, const i64* edge_side,
                      const i64* edge_kind, const double* ea, const double* eb, double* f) {
    auto coords = [&](i64 e, double c[8]) {
        for (int a = 0; a < 4; ++a) {
            c[2 * a] = xy[2 * nodes[4 * e + a]];
            c[2 * a + 1] = xy[2 * nodes[4 * e + a] + 1];
        }
    };
    for (i64 k = 0; k < n_body; ++k) {
        double c[8], out[8];
        const i64 e = body_elem[k];
        coords(e, c);
        if (!q4_body_force(c, thick[e], bx[k], by[k], out)) return -1;
        for (int a = 0; a < 4; ++a) {
            f[2 * nodes[4 * e + a]] += out[2 * a];
            f[2 * nodes[4 * e + a] + 1] += out[2 * a + 1];
        }
    }
    for (i64 k = 0; k < n_edge; ++k) {
        double c[8], out[8];
        const i64 e = edge_elem[k];
        coords(e, c);
        if (!q4_edge_load(c, thick[e], static_cast<int>(edge_side[k]), static_cast<int>(edge_kind[k]), ea[k], eb[k], out))
            return -2;
        for (int a = 0; a < 4; ++a) {
            f[2 * nodes[4 * e + a]] += out[2 * a];
            f[2 * nodes[4 * e + a] + 1] += out[2 * a + 1];
        }
    }
    return 0;
}

// apply_dirichlet (O(nnz) path), src/solver.cpp:355-413, then the zero-pivot sweep of
// src/solver.cpp:920-940.  Returns 0, or -1 - dof for a loaded zero pivot.
i64 lfo_apply_dirichlet(i64 n, const i64* ptr, const i64* col, double* val, double* f, i64 n_c, const i64* c_dofs,
                        const double* c_vals) {
    if (n_c > 0) {
        std::vector<char> fixed(static_cast<size_t>(n), 0);
        std::vector<double> pres(static_cast<size_t>(n), 0.0);
        for (i64 k = 0; k < n_c; ++k) {
            fixed[c_dofs[k]] = 1;
            pres[c_dofs[k]] = c_vals[k];
        }
        for (i64 r = 0; r < n; ++r) {
            if (fixed[r]) {
                for (i64 k = ptr[r]; k < ptr[r + 1]; ++k) val[k] = 0.0;
                for (i64 k = ptr[r]; k < ptr[r + 1]; ++k)
                    if (col[k] == r) val[k] = 1.0;
                f[r] = pres[r];
                continue;
            }
            for (i64 k = ptr[r]; k < ptr[r + 1]; ++k) {
                if (!fixed[col[k]] || val[k] == 0.0) continue;
                f[r] -= val[k] * pres[col[k]];
                val[k] = 0.0;
            }
        }
    }
    double scale = 0.0;
    for (i64 i = 0; i < n; ++i) scale = std::max(scale, std::abs(f[i]));
    if (scale <= 0.0) scale = 1.0;
    for (i64 r = 0; r < n; ++r) {
        i64 dk = -1;
        for (i64 k = ptr[r]; k < ptr[r + 1]; ++k)
            if (col[k] == r) dk = k;
        if (std::abs(val[dk]) > 1.0e-30) continue;
        if (std::abs(f[r]) > 1.0e-12 * scale) return -1 - r;
        val[dk] = 1.0;
        f[r] = 0.0;
    }
    return 0;
}

void lfo_spmv_csr(i64 n, const i64* ptr, const i64* col, const double* val, const double* x, double* y) {
    make_csr(n, ptr, col, val).spmv(x, y);
}

// BsrMatrix::from_csr; outputs sized by lfo_bsr_count first.
i64 lfo_bsr_count(i64 n, const i64* ptr, const i64* col, const double* val) {
    return static_cast<i64>(Bsr::from_csr(make_csr(n, ptr, col, val)).col.size());
}
void lfo_bsr_convert(i64 n, const i64* ptr, const i64* col, const double* val, i64* bptr, i64* bcol, double* bval) {
    const Bsr b = Bsr::from_csr(make_csr(n, ptr, col, val));
    std::copy(b.ptr.begin(), b.ptr.end(), bptr);
    std::copy(b.col.begin(), b.col.end(), bcol);
    std::copy(b.val.begin(), b.val.end(), bval);
}

// The node split of the block preconditioner (split: 0 chunk, 1 rcb; xy in node
// index order); returns the subdomain count.
i64 lfo_subdomain_split(i64 nodes, const double* xy, i64 nodes_per, int split, uint32_t* owner) {
    size_t count = 0;
    std::vector<uint32_t> o;
    if (split == 0) {
        o = chunk_split(static_cast<size_t>(nodes), static_cast<size_t>(nodes_per), &count);
    } else {
        std::vector<double> x(static_cast<size_t>(nodes)), y(static_cast<size_t>(nodes));
        for (i64 k = 0; k < nodes; ++k) {
            x[static_cast<size_t>(k)] = xy[2 * k];
            y[static_cast<size_t>(k)] = xy[2 * k + 1];
        }
        o = rcb_split(x, y, static_cast<size_t>(nodes_per), &count);
    }
    std::copy(o.begin(), o.end(), owner);
    return static_cast<i64>(count);
}

// One preconditioner application z = M^-1 r.  precond: 0 jacobi, 1 block, 2 ic0.
// split: 0 chunk, 1 rcb (node coordinates in xy, node index order).
int lfo_precond_apply(i64 n, const i64* ptr, const i64* col, const double* val, int precond, int split, i64 nodes_per,
                      const double* xy, const double* r, double* z, double* stats) {
    const Csr a = make_csr(n, ptr, col, val);
    if (precond == 0) {
        Jacobi(a).apply(r, z);
    } else if (precond == 1) {
        size_t count = 0;
        const size_t nn = a.n / 2;
        std::vector<uint32_t> node_owner;
        if (split == 0) {
            node_owner = chunk_split(nn, static_cast<size_t>(nodes_per), &count);
        } else {
            std::vector<double> x(nn), y(nn);
            for (size_t k = 0; k < nn; ++k) {
                x[k] = xy[2 * k];
                y[k] = xy[2 * k + 1];
            }
            node_owner = rcb_split(x, y, static_cast<size_t>(nodes_per), &count);
        }
        std::vector<uint32_t> owner(a.n);
        for (size_t k = 0; k < nn; ++k) owner[2 * k] = owner[2 * k + 1] = node_owner[k];
        BlockJacobi bj(a, owner, count);
        bj.apply(r, z);
        if (stats) {
            stats[0] = static_cast<double>(count);
            stats[1] = bj.capture;
            stats[2] = static_cast<double>(bj.degenerate);
        }
    } else {
        Ic0 ic(a);
        ic.apply(r, z);
        if (stats) stats[0] = static_cast<double>(ic.breakdowns);
    }
    return 0;
}

// solve_iterative + pcg_solve, src/solver.cpp:675-747 and :532-627.
// storage: 0 csr, 1 bsr.  report[9] = Report fields; stats[3] as above.
int lfo_pcg(i64 n, const i64* ptr, const i64* col, const double* val, const double* b, double tol, i64 maxit,
            int storage, int precond, int split, i64 nodes_per, const double* xy, double* x, double* report,
            double* stats, i64 iteration_cap) {
    try {
        const Csr a = make_csr(n, ptr, col, val);
        Report rep{};
        std::unique_ptr<Precond> m;
        const double s0 = now_ms();
        if (precond == 0) {
            m.reset(new Jacobi(a));
        } else if (precond == 1) {
            size_t count = 0;
            const size_t nn = a.n / 2;
            std::vector<uint32_t> node_owner;
            if (split == 0) {
                node_owner = chunk_split(nn, static_cast<size_t>(nodes_per), &count);
            } else {
                std::vector<double> xs(nn), ys(nn);
                for (size_t k = 0; k < nn; ++k) {
                    xs[k] = xy[2 * k];
                    ys[k] = xy[2 * k + 1];
                }
                node_owner = rcb_split(xs, ys, static_cast<size_t>(nodes_per), &count);
            }
            std::vector<uint32_t> owner(a.n);
            for (size_t k = 0; k < nn; ++k) owner[2 * k] = owner[2 * k + 1] = node_owner[k];
            auto* bj = new BlockJacobi(a, owner, count);
            if (stats) {
                stats[0] = static_cast<double>(count);
                stats[1] = bj->capture;
                stats[2] = static_cast<double>(bj->degenerate);
            }
            m.reset(bj);
        } else {
            auto* ic = new Ic0(a);
            if (stats) stats[0] = static_cast<double>(ic->breakdowns);
            m.reset(ic);
        }
        const double setup_ms = now_ms() - s0;
        const size_t cap = static_cast<size_t>(iteration_cap);
        if (storage == 1) {
            const double c0 = now_ms();
            const Bsr bsr = Bsr::from_csr(a);
            const double convert_ms = now_ms() - c0;
            rep = pcg(bsr, *m, b, tol, static_cast<size_t>(maxit), x, cap);
            if (stats) stats[3] = convert_ms;
        } else {
            rep = pcg(a, *m, b, tol, static_cast<size_t>(maxit), x, cap);
        }
        if (stats) stats[4] = setup_ms;
        std::memcpy(report, &rep, sizeof rep);
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// Adjoint sensitivity of a per-element modulus (no reference counterpart; the
// restatement the GPU kernel is checked against): K_e is linear in E_e, so
// dJ/dE_e = -lambda_e^T K_e u_e / E_e with K_e from q4_stiffness above.
int lfo_adjoint_grad(const double* xy, i64 n_elem, const i64* nodes, const double* young, const double* poisson,
                     const double* thick, int plane_strain, const double* u, const double* lam, double* grad) {
    int bad = 0;
#pragma omp parallel for schedule(static)
    for (i64 e = 0; e < n_elem; ++e) {
        double c[8], k[64], ue[8], le[8];
        for (int a = 0; a < 4; ++a) {
            const i64 nd = nodes[4 * e + a];
            c[2 * a] = xy[2 * nd];
            c[2 * a + 1] = xy[2 * nd + 1];
            ue[2 * a] = u[2 * nd];
            ue[2 * a + 1] = u[2 * nd + 1];
            le[2 * a] = lam[2 * nd];
            le[2 * a + 1] = lam[2 * nd + 1];
        }
        if (!q4_stiffness(c, young[e], poisson[e], thick[e], plane_strain, k)) {
            bad = 1;
            continue;
        }
        double s = 0.0;
        for (int r = 0; r < 8; ++r) {
            double row = 0.0;
            for (int q = 0; q < 8; ++q) row += k[8 * r + q] * ue[q];
            s += le[r] * row;
        }
        grad[e] = -s / young[e];
    }
    return bad ? -1 : 0;
}

// reverse_cuthill_mckee, src/reordering.cpp:11-62: node adjacency through Q4
// elements, seeds and neighbours ordered by (degree, node ID), BFS, reversed.
// ids[] are node IDs (any order); elem[] holds node IDs.  order[] receives IDs.
// Element fields and nodal stress smoothing: q4_center_field and
// q4_gauss_point_fields (src/element.cpp:212-248) as postprocess calls them
// (src/solver.cpp:756-771), and smooth_nodal_stresses (src/solver.cpp:807-871).
// fields[35 e + 7 k + (0..6)] = strain (3), stress (3), von Mises for k = 0 the
// element centre and k = 1..4 the Gauss points (-g,-g), (g,-g), (g,g), (-g,g);
// nodal[4 i + (0..3)] = smoothed stress (3) and its von Mises.  Returns -1 for a
// non-positive Jacobian.
int lfo_postprocess(const double* xy, i64 n_nodes, i64 n_elem, const i64* nodes, const double* young,
                    const double* poisson, int plane_strain, const double* u, double* fields, double* nodal) {
    auto field = [](const double b[24], const double d[9], const double ue[8], double* out) {
        double strain[3] = {0.0, 0.0, 0.0}, stress[3] = {0.0, 0.0, 0.0};
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 8; ++c) strain[r] += b[8 * r + c] * ue[c];
        for (int r = 0; r < 3; ++r)
            for (int c = 0; c < 3; ++c) stress[r] += d[3 * r + c] * strain[c];
        const double sx = stress[0], sy = stress[1], txy = stress[2];
        out[0] = strain[0];
        out[1] = strain[1];
        out[2] = strain[2];
        out[3] = sx;
        out[4] = sy;
        out[5] = txy;
        out[6] = std::sqrt(std::max(0.0, sx * sx - sx * sy + sy * sy + 3.0 * txy * txy));
    };
    int bad = 0;
#pragma omp parallel for schedule(static)
    for (i64 e = 0; e < n_elem; ++e) {
        double exy[8], ue[8], d[9], b[24], det;
        for (int a = 0; a < 4; ++a) {
            const i64 nd = nodes[4 * e + a];
            exy[2 * a] = xy[2 * nd];
            exy[2 * a + 1] = xy[2 * nd + 1];
            ue[2 * a] = u[2 * nd];
            ue[2 * a + 1] = u[2 * nd + 1];
        }
        constitutive(young[e], poisson[e], plane_strain, d);
        double* out = fields + 35 * e;
        if (!kinematics(exy, 0.0, 0.0, b, &det)) {
#pragma omp atomic write
            bad = 1;
            continue;
        }
        field(b, d, ue, out);
        for (int g = 0; g < 4; ++g) {
            if (!kinematics(exy, kPoints[g][0], kPoints[g][1], b, &det)) {
#pragma omp atomic write
                bad = 1;
                break;
            }
            field(b, d, ue, out + 7 * (g + 1));
        }
    }
    if (bad) return -1;
    constexpr double root_three = 1.7320508075688772935;
    const double alpha = 0.5 * (1.0 + root_three);
    const double beta = 0.5 * (1.0 - root_three);
    const double ext[4][4] = {{alpha * alpha, alpha * beta, beta * beta, alpha * beta},
                              {alpha * beta, alpha * alpha, alpha * beta, beta * beta},
                              {beta * beta, alpha * beta, alpha * alpha, alpha * beta},
                              {alpha * beta, beta * beta, alpha * beta, alpha * alpha}};
    std::vector<double> sums(3 * static_cast<size_t>(n_nodes), 0.0);
    std::vector<i64> counts(static_cast<size_t>(n_nodes), 0);
    for (i64 e = 0; e < n_elem; ++e)
        for (int a = 0; a < 4; ++a) {
            const i64 nd = nodes[4 * e + a];
            for (int c = 0; c < 3; ++c)
                for (int g = 0; g < 4; ++g) sums[3 * nd + c] += ext[a][g] * fields[35 * e + 7 * (g + 1) + 3 + c];
            ++counts[nd];
        }
    for (i64 i = 0; i < n_nodes; ++i) {
        double* out = nodal + 4 * i;
        if (counts[i] == 0) {
            out[0] = out[1] = out[2] = out[3] = 0.0;
            continue;
        }
        for (int c = 0; c < 3; ++c) out[c] = sums[3 * i + c] / static_cast<double>(counts[i]);
        const double sx = out[0], sy = out[1], txy = out[2];
        out[3] = std::sqrt(std::max(0.0, sx * sx - sx * sy + sy * sy + 3.0 * txy * txy));
    }
    return 0;
}

void lfo_rcm(i64 n_nodes, const i64* ids, i64 n_elem, const i64* elem, i64* order) {
    std::vector<i64> sorted(ids, ids + n_nodes);
    std::sort(sorted.begin(), sorted.end());
    auto idx = [&](i64 id) { return std::lower_bound(sorted.begin(), sorted.end(), id) - sorted.begin(); };
    std::vector<std::vector<i64>> adj(static_cast<size_t>(n_nodes));
    for (i64 e = 0; e < n_elem; ++e)
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
                if (i != j) adj[idx(elem[4 * e + i])].push_back(elem[4 * e + j]);
    for (auto& v : adj) {
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    }
    auto before = [&](i64 a, i64 b) {
        const size_t da = adj[idx(a)].size(), db = adj[idx(b)].size();
        return da != db ? da < db : a < b;
    };
    std::vector<i64> seeds(sorted);
    std::sort(seeds.begin(), seeds.end(), before);
    std::vector<char> seen(static_cast<size_t>(n_nodes), 0);
    i64 out = 0;
    for (const i64 s : seeds) {
        if (seen[idx(s)]) continue;
        seen[idx(s)] = 1;
        std::queue<i64> todo;
        todo.push(s);
        while (!todo.empty()) {
            const i64 cur = todo.front();
            todo.pop();
            order[out++] = cur;
            std::vector<i64> nb = adj[idx(cur)];
            std::sort(nb.begin(), nb.end(), before);
            for (const i64 v : nb)
                if (!seen[idx(v)]) {
                    seen[idx(v)] = 1;
                    todo.push(v);
                }
        }
    }
    std::reverse(order, order + out);
}

}  // extern "C"
