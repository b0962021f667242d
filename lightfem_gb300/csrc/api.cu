// C ABI of liblfgpu (include/lfgpu.h): handle lifetime, host-side validation of
// every index that reaches a kernel, uploads, and the orchestration of the solve
// path stages on the handle's stream.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <thread>
#include <cstring>
#include <exception>
#include <new>
#include <numeric>
#include <string>
#include <vector>

#include "common.cuh"
#include "host_setup.hpp"
#include "kernels.hpp"

struct lfgpu_context : lfgpu::Context {};

namespace lfgpu {

void check_status(Context& c) {
    LF_CUDA(cudaStreamSynchronize(c.stream));
    DeviceStatus s{};
    LF_CUDA(cudaMemcpy(&s, c.status.p, sizeof(s), cudaMemcpyDeviceToHost));
    if (s.code == 0) return;
    c.fail_code = s.code;
    c.fail_index = s.bad_index;
    c.fail_values[0] = c.fail_values[1] = 0.0;
    if (s.code == LFGPU_ERR_TIMEOUT) c.fail_values[0] = s.abort != 0u ? 1.0 : 0.0;  // the abort flag it raised
    if (s.code == LFGPU_ERR_MECHANISM && s.bad_index >= 0 && s.bad_index < c.n) {
        // The sweep leaves a loaded zero pivot untouched: read its load and diagonal
        // for the reference's message (src/solver.cpp:926-936).
        int pos = 0;
        LF_CUDA(cudaMemcpy(&pos, c.diag.p + s.bad_index, sizeof(int), cudaMemcpyDeviceToHost));
        LF_CUDA(cudaMemcpy(&c.fail_values[0], c.f.p + s.bad_index, sizeof(double), cudaMemcpyDeviceToHost));
        if (pos >= 0 && pos < c.nnz)
            LF_CUDA(cudaMemcpy(&c.fail_values[1], c.K.p + pos, sizeof(double), cudaMemcpyDeviceToHost));
    }
    std::string msg;
    switch (s.code) {
        case LFGPU_ERR_JACOBIAN:
            msg = "Q4 stiffness evaluation received a non-positive Jacobian (element index " +
                  std::to_string(s.bad_index) + ")";
            break;
        case LFGPU_ERR_EDGE:
            msg = "Q4 edge load received a zero-length edge (element index " + std::to_string(s.bad_index) + ")";
            break;
        case LFGPU_ERR_MECHANISM:
            msg = "the structure is a mechanism: zero pivot carrying load [dof " + std::to_string(s.bad_index) + "]";
            break;
        case LFGPU_ERR_NONFINITE_DIAG:
            msg = "Jacobi preconditioner encountered a non-finite diagonal";
            break;
        case LFGPU_ERR_TIMEOUT:
            msg = "a device-side wait exceeded its time bound (CTA " + std::to_string(s.bad_index) + ")";
            break;
        default:
            msg = "device failure " + std::to_string(s.code);
    }
    reset_status(c);
    throw Error{s.code, msg};
}

void reset_status(Context& c) {
    DeviceStatus s{};
    s.bad_index = 0x7fffffff;
    s.wait_limit_ns = c.wait_limit_ns;
    LF_CUDA(cudaMemcpyAsync(c.status.p, &s, sizeof(s), cudaMemcpyHostToDevice, c.stream));
}

float elapsed_ms(Context& c) {
    LF_CUDA(cudaEventSynchronize(c.ev_b));
    float ms = 0.f;
    LF_CUDA(cudaEventElapsedTime(&ms, c.ev_a, c.ev_b));
    return ms;
}

double capture_ratio_2x2(Context& c);

namespace {

template <typename T>
void upload(Context& c, Buf<T>& dst, const T* src, size_t count) {
    dst.ensure(count);
    if (count) LF_CUDA(cudaMemcpyAsync(dst.p, src, count * sizeof(T), cudaMemcpyHostToDevice, c.stream));
}

template <typename F>
int guarded(lfgpu_t h, F&& f) {
    if (h == nullptr) return LFGPU_ERR_ARGUMENT;
    try {
        LF_CUDA(cudaSetDevice(h->device));
        f();
        h->error.clear();
        return LFGPU_OK;
    } catch (const Error& e) {
        h->error = e.message;
        return e.code;
    } catch (const std::bad_alloc&) {
        h->error = "host allocation failed";
        return LFGPU_ERR_NOMEM;
    } catch (const std::exception& e) {
        h->error = e.what();
        return LFGPU_ERR_ARGUMENT;
    }
}

void install_colors(Context& c, const int* colors, bool check = true);
void install_finish(Context& c);

// Host copies the map/colour validation needs; set on lfgpu_set_pattern.
void install_pattern(Context& c, i64 n, i64 nnz, const int64_t* rowptr64, const int* col, const int* map,
                     const int* colors) {
    LF_REQUIRE(c.n_elem > 0 || nnz >= 0, LFGPU_ERR_STATE, "set the mesh before the pattern");
    LF_REQUIRE(n == 2 * c.n_nodes, LFGPU_ERR_ARGUMENT, "pattern dimension must be 2 x nodes");
    LF_REQUIRE(nnz >= 0 && nnz < (1LL << 31), LFGPU_ERR_ARGUMENT, "pattern must have fewer than 2^31 nonzeros");
    LF_REQUIRE(rowptr64[0] == 0 && rowptr64[n] == nnz, LFGPU_ERR_ARGUMENT, "row offsets must run from 0 to nnz");
    std::vector<int> rp(static_cast<size_t>(n) + 1);
    bool paired = true;
    for (i64 r = 0; r < n; ++r) {
        const i64 b = rowptr64[r], e = rowptr64[r + 1];
        LF_REQUIRE(e >= b, LFGPU_ERR_ARGUMENT, "row offsets must not decrease");
        rp[r] = static_cast<int>(b);
        bool diag = false;
        for (i64 k = b; k < e; ++k) {
            LF_REQUIRE(col[k] >= 0 && col[k] < n, LFGPU_ERR_ARGUMENT, "column index out of range");
            LF_REQUIRE(k == b || col[k] > col[k - 1], LFGPU_ERR_ARGUMENT, "columns must ascend within a row");
            diag = diag || col[k] == r;
        }
        LF_REQUIRE(diag, LFGPU_ERR_ARGUMENT, "every row needs its diagonal entry");
        if ((e - b) % 2 != 0 || b % 2 != 0) paired = false;
        if (paired)
            for (i64 k = b; k < e; k += 2)
                if (col[k] % 2 != 0 || col[k + 1] != col[k] + 1) paired = false;
        if (paired && r % 2 == 1) {
            const i64 pb = rowptr64[r - 1];
            if (e - b != b - pb) paired = false;
            for (i64 k = 0; paired && k < e - b; ++k)
                if (col[b + k] != col[pb + k]) paired = false;
        }
    }
    rp[n] = static_cast<int>(nnz);
    // Every map entry must point at (dof_a, dof_b) of its element: this both bounds
    // the scatter and proves the map matches the mesh.
    const int* en = c.h_elem_nodes.data();
    for (i64 e = 0; e < c.n_elem; ++e) {
        for (int a = 0; a < 8; ++a) {
            const int row = 2 * en[4 * e + a / 2] + (a & 1);
            for (int b = 0; b < 8; ++b) {
                const int m = map[64 * e + 8 * a + b];
                const int want = 2 * en[4 * e + b / 2] + (b & 1);
                LF_REQUIRE(m >= rp[row] && m < rp[row + 1] && col[m] == want, LFGPU_ERR_ARGUMENT,
                           "element value map does not point at the element's (row, column) entry");
            }
        }
    }
    install_colors(c, colors);
    c.n = n;
    c.nnz = nnz;
    c.paired = paired;
    upload(c, c.rowptr, rp.data(), rp.size());
    upload(c, c.col, col, static_cast<size_t>(nnz));
    upload(c, c.map, map, static_cast<size_t>(c.n_elem) * 64);
    c.h_rowptr_cache = rp;
    install_finish(c);
}

// Colours: per-colour element lists; no two elements of a colour may share a node
// (checked unless the library coloured the mesh itself: check = false).
void install_colors(Context& c, const int* colors, bool check) {
    const int* en = c.h_elem_nodes.data();
    c.n_colors = 0;
    c.color_offsets.assign(1, 0);
    std::vector<int> order;
    if (colors) {
        int top = -1;
        for (i64 e = 0; e < c.n_elem; ++e) {
            LF_REQUIRE(colors[e] >= 0 && colors[e] < (1 << 20), LFGPU_ERR_ARGUMENT, "element colour out of range");
            top = std::max(top, colors[e]);
        }
        c.n_colors = top + 1;
        c.color_offsets.assign(static_cast<size_t>(c.n_colors) + 1, 0);
        for (i64 e = 0; e < c.n_elem; ++e) ++c.color_offsets[colors[e] + 1];
        for (int k = 0; k < c.n_colors; ++k) c.color_offsets[k + 1] += c.color_offsets[k];
        order.resize(static_cast<size_t>(c.n_elem));
        std::vector<int> fill(c.color_offsets.begin(), c.color_offsets.end() - 1);
        for (i64 e = 0; e < c.n_elem; ++e) order[fill[colors[e]]++] = static_cast<int>(e);
        std::vector<int> owner(check ? static_cast<size_t>(c.n_nodes) : 0, -1);
        for (int k = 0; check && k < c.n_colors; ++k)
            for (int s = c.color_offsets[k]; s < c.color_offsets[k + 1]; ++s)
                for (int a = 0; a < 4; ++a) {
                    const int nd = en[4 * static_cast<i64>(order[s]) + a];
                    LF_REQUIRE(owner[nd] != k, LFGPU_ERR_ARGUMENT,
                               "two elements of one colour share a node: the colouring is not race-free");
                    owner[nd] = k;
                }
        c.h_colors.assign(colors, colors + c.n_elem);
    } else {
        c.h_colors.clear();
    }
    upload(c, c.color_elems, order.data(), order.size());
}

// Device state that follows a new pattern (rowptr, col, map, n, nnz, paired and
// the host row-pointer copy are in place).
void install_finish(Context& c) {
    const i64 n = c.n, nnz = c.nnz;
    c.diag.ensure(static_cast<size_t>(n));
    launch_find_diagonal(c);
    c.K.ensure(nnz);
    c.K_full.ensure(nnz);
    c.f.ensure(n);
    c.f_full.ensure(n);
    c.u.ensure(n);
    c.R.ensure(n);
    c.fixed.ensure(n);
    c.prescribed.ensure(n);
    LF_CUDA(cudaMemsetAsync(c.u.p, 0, sizeof(double) * n, c.stream));
    if (c.n_constraints == 0) {
        LF_CUDA(cudaMemsetAsync(c.fixed.p, 0, n, c.stream));
        LF_CUDA(cudaMemsetAsync(c.prescribed.p, 0, sizeof(double) * n, c.stream));
    }
    c.h_brow.clear();
    c.have_pattern = true;
    c.assembled = c.constrained = c.solved = false;
    ++c.k_version;
    ++c.pattern_version;
    check_status(c);
}

}  // namespace
}  // namespace lfgpu

using namespace lfgpu;

extern "C" {

const char* lfgpu_version(void) { return "lfgpu 0.1 (sm_103a)"; }

int lfgpu_create(int device, lfgpu_t* out) {
    if (out == nullptr) return LFGPU_ERR_ARGUMENT;
    *out = nullptr;
    lfgpu_t h = new (std::nothrow) lfgpu_context();
    if (h == nullptr) return LFGPU_ERR_NOMEM;
    h->device = device;
    const int rc = guarded(h, [&] {
        LF_CUDA(cudaGetDeviceCount(&h->num_sms));
        LF_REQUIRE(device >= 0 && device < h->num_sms, LFGPU_ERR_ARGUMENT, "no such CUDA device");
        LF_CUDA(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device));
        LF_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        LF_CUDA(cudaEventCreate(&h->ev_a));
        LF_CUDA(cudaEventCreate(&h->ev_b));
        h->status.ensure(1);
        reset_status(*h);
        LF_CUDA(cudaStreamSynchronize(h->stream));
    });
    if (rc != LFGPU_OK) {
        delete h;
        return rc;
    }
    *out = h;
    return LFGPU_OK;
}

int lfgpu_destroy(lfgpu_t h) {
    if (h == nullptr) return LFGPU_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    for (auto* b : {&h->mat_young, &h->mat_nu, &h->mat_t, &h->f_nodal, &h->body_bx, &h->body_by, &h->edge_a,
                    &h->edge_b, &h->prescribed, &h->K, &h->K_full, &h->f, &h->f_full, &h->bval64, &h->inv_diag64,
                    &h->blk64, &h->u, &h->R, &h->partials, &h->scratch64, &h->ic0_val, &h->ic0_inv, &h->lam,
                    &h->adj_rhs})
        b->release();
    for (auto& b : h->v64) b.release();
    for (auto& b : h->v32) b.release();
    for (auto* b : {&h->bval32, &h->K32, &h->inv_diag32, &h->blk32, &h->diag_hi, &h->diag_lo})
        b->release();
    for (auto* b : {&h->elem_mat, &h->rowptr, &h->col, &h->map, &h->diag, &h->color_elems, &h->edge_ptr,
                    &h->edge_side, &h->edge_kind, &h->brow, &h->bcol, &h->ic0_mirror, &h->ic0_flags,
                    &h->ic0_level})
        b->release();
    h->xy.release();
    h->elem_nodes.release();
    h->fixed.release();
    h->bar.release();
    h->status.release();
    h->pcg_result.release();
    h->ic0_misc.release();
    h->ne_ptr.release();
    h->ne_list.release();
    h->post_fields.release();
    h->post_nodal.release();
    for (auto& b : h->zp) b.release();
    h->xhi.release();
    h->xlo.release();
    for (auto& sc : h->sched) {
        sc.tiles.release();
        sc.cta.release();
    }
    h->cg_state.release();
    for (auto& ev : h->user_ev)
        if (ev) cudaEventDestroy(ev);
    if (h->ev_a) cudaEventDestroy(h->ev_a);
    if (h->ev_b) cudaEventDestroy(h->ev_b);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return LFGPU_OK;
}

const char* lfgpu_last_error(lfgpu_t h) { return h ? h->error.c_str() : "null handle"; }

int lfgpu_failure_detail(lfgpu_t h, int32_t* status, int64_t* index, double* values) {
    if (h == nullptr) return LFGPU_ERR_ARGUMENT;
    if (status) *status = h->fail_code;
    if (index) *index = h->fail_index;
    if (values) {
        values[0] = h->fail_values[0];
        values[1] = h->fail_values[1];
    }
    return LFGPU_OK;
}

int lfgpu_set_option(lfgpu_t h, int32_t option, int64_t value) {
    return guarded(h, [&] {
        switch (option) {
            case LFGPU_OPTION_WAIT_LIMIT_NS:
                LF_REQUIRE(value > 0, LFGPU_ERR_ARGUMENT, "the wait limit must be positive");
                h->wait_limit_ns = static_cast<unsigned long long>(value);
                reset_status(*h);  // the limit travels in the device status word
                LF_CUDA(cudaStreamSynchronize(h->stream));
                break;
            case LFGPU_OPTION_IC0_SWEEP:
                LF_REQUIRE(value == LFGPU_IC0_SWEEP_AUTO || value == LFGPU_IC0_SWEEP_LEVELS ||
                               value == LFGPU_IC0_SWEEP_POLLED,
                           LFGPU_ERR_ARGUMENT, "ic0 sweep must be auto, levels or polled");
                h->ic0_sweep = static_cast<int>(value);
                break;
            default:
                throw Error{LFGPU_ERR_ARGUMENT, "unknown option"};
        }
    });
}

int lfgpu_set_mesh(lfgpu_t h, int64_t n_nodes, const double* xy, int64_t n_elements, const int32_t* element_nodes,
                   const int32_t* element_material, int64_t n_materials, const double* young, const double* poisson,
                   const double* thickness, int32_t plane_mode) {
    return guarded(h, [&] {
        LF_REQUIRE(n_nodes > 0 && n_nodes < (1LL << 29), LFGPU_ERR_ARGUMENT, "node count out of range");
        LF_REQUIRE(n_elements >= 0 && n_elements < (1LL << 29), LFGPU_ERR_ARGUMENT, "element count out of range");
        LF_REQUIRE(n_materials > 0, LFGPU_ERR_ARGUMENT, "at least one material is required");
        LF_REQUIRE(plane_mode == LFGPU_PLANE_STRESS || plane_mode == LFGPU_PLANE_STRAIN, LFGPU_ERR_ARGUMENT,
                   "plane_mode must be plane_stress or plane_strain");
        LF_REQUIRE(xy && young && poisson && thickness && (n_elements == 0 || (element_nodes && element_material)),
                   LFGPU_ERR_ARGUMENT, "null mesh array");
        for (int64_t k = 0; k < 4 * n_elements; ++k)
            LF_REQUIRE(element_nodes[k] >= 0 && element_nodes[k] < n_nodes, LFGPU_ERR_ARGUMENT,
                       "element references a node index out of range");
        for (int64_t e = 0; e < n_elements; ++e)
            LF_REQUIRE(element_material[e] >= 0 && element_material[e] < n_materials, LFGPU_ERR_ARGUMENT,
                       "element references a material index out of range");
        h->n_nodes = n_nodes;
        h->n_elem = n_elements;
        h->n_mat = n_materials;
        h->plane_mode = plane_mode;
        upload(*h, h->xy, reinterpret_cast<const double2*>(xy), static_cast<size_t>(n_nodes));
        upload(*h, h->elem_nodes, reinterpret_cast<const int4*>(element_nodes), static_cast<size_t>(n_elements));
        upload(*h, h->elem_mat, element_material, static_cast<size_t>(n_elements));
        upload(*h, h->mat_young, young, static_cast<size_t>(n_materials));
        upload(*h, h->mat_nu, poisson, static_cast<size_t>(n_materials));
        upload(*h, h->mat_t, thickness, static_cast<size_t>(n_materials));
        h->h_elem_nodes.assign(element_nodes, element_nodes + 4 * n_elements);
        h->have_pattern = h->assembled = h->constrained = h->solved = false;
        ++h->mesh_version;
        h->have_nodal = h->have_body = h->have_edges = false;
        h->n_constraints = 0;
        LF_CUDA(cudaStreamSynchronize(h->stream));
    });
}

int lfgpu_set_young(lfgpu_t h, const double* young) {
    return guarded(h, [&] {
        LF_REQUIRE(young && h->n_mat > 0, LFGPU_ERR_STATE, "set the mesh before the moduli");
        upload(*h, h->mat_young, young, static_cast<size_t>(h->n_mat));
        LF_CUDA(cudaStreamSynchronize(h->stream));
    });
}

int lfgpu_set_pattern(lfgpu_t h, int64_t n_dofs, int64_t nnz, const int64_t* row_offsets, const int32_t* columns,
                      const int32_t* element_value_index, const int32_t* element_color) {
    return guarded(h, [&] {
        LF_REQUIRE(row_offsets && columns && element_value_index, LFGPU_ERR_ARGUMENT, "null pattern array");
        install_pattern(*h, n_dofs, nnz, row_offsets, columns, element_value_index, element_color);
    });
}

int lfgpu_build_pattern(lfgpu_t h) {
    return guarded(h, [&] {
        LF_REQUIRE(h->n_nodes > 0, LFGPU_ERR_STATE, "set the mesh before building the pattern");
        const auto t0 = std::chrono::steady_clock::now();
        // The greedy colouring is sequential in element order; it runs on a host
        // thread while the device builds the pattern and the map.
        std::vector<int> colors;
        std::exception_ptr colouring_error;
        std::thread colouring([&] {
            try {
                greedy_colors(h->n_nodes, h->n_elem, h->h_elem_nodes.data(), colors);
            } catch (...) {
                colouring_error = std::current_exception();
            }
        });
        bool on_device = false;
        try {
            on_device = build_pattern_device(*h, h->h_rowptr_cache);
        } catch (...) {
            colouring.join();
            throw;
        }
        colouring.join();
        if (colouring_error) std::rethrow_exception(colouring_error);
        if (on_device) {
            install_colors(*h, colors.data(), false);  // first fit: race-free by construction
            install_finish(*h);
        } else {  // a node with more elements than the device build handles
            const HostPattern p = build_pattern(h->n_nodes, h->n_elem, h->h_elem_nodes.data());
            install_pattern(*h, p.n, p.nnz, p.rowptr.data(), p.col.data(), p.map.data(), colors.data());
        }
        h->pattern_on_device = on_device;
        h->timings.pattern_ms =
            std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    });
}

int lfgpu_pattern_info(lfgpu_t h, int64_t* n_dofs, int64_t* nnz, int64_t* n_colors) {
    return guarded(h, [&] {
        LF_REQUIRE(h->have_pattern, LFGPU_ERR_STATE, "no pattern");
        if (n_dofs) *n_dofs = h->n;
        if (nnz) *nnz = h->nnz;
        if (n_colors) *n_colors = h->n_colors;
    });
}

int lfgpu_download_pattern(lfgpu_t h, int64_t* row_offsets, int32_t* columns, int32_t* element_value_index,
                           int32_t* element_color) {
    return guarded(h, [&] {
        LF_REQUIRE(h->have_pattern, LFGPU_ERR_STATE, "no pattern");
        if (row_offsets)
            for (i64 r = 0; r <= h->n; ++r) row_offsets[r] = h->h_rowptr_cache[r];
        if (columns)
            LF_CUDA(cudaMemcpy(columns, h->col.p, sizeof(int) * h->nnz, cudaMemcpyDeviceToHost));
        if (element_value_index)
            LF_CUDA(cudaMemcpy(element_value_index, h->map.p, sizeof(int) * 64 * h->n_elem, cudaMemcpyDeviceToHost));
        if (element_color) {
            LF_REQUIRE(!h->h_colors.empty() || h->n_elem == 0, LFGPU_ERR_STATE, "no colouring");
            std::copy(h->h_colors.begin(), h->h_colors.end(), element_color);
        }
    });
}

int lfgpu_set_loads(lfgpu_t h, const double* nodal, int64_t n_body, const int32_t* body_element,
                    const double* body_bx, const double* body_by, int64_t n_edge, const int32_t* edge_element,
                    const int32_t* edge_side, const int32_t* edge_kind, const double* edge_first,
                    const double* edge_second) {
    return guarded(h, [&] {
        LF_REQUIRE(h->n_nodes > 0, LFGPU_ERR_STATE, "set the mesh before the loads");
        const i64 n = 2 * h->n_nodes, E = h->n_elem;
        h->have_nodal = nodal != nullptr;
        if (nodal) upload(*h, h->f_nodal, nodal, static_cast<size_t>(n));
        h->have_body = n_body > 0;
        if (n_body > 0) {
            std::vector<double> bx(static_cast<size_t>(E), 0.0), by(static_cast<size_t>(E), 0.0);
            for (i64 k = 0; k < n_body; ++k) {
                LF_REQUIRE(body_element[k] >= 0 && body_element[k] < E, LFGPU_ERR_ARGUMENT,
                           "body force references an element index out of range");
                bx[body_element[k]] += body_bx[k];
                by[body_element[k]] += body_by[k];
            }
            upload(*h, h->body_bx, bx.data(), bx.size());
            upload(*h, h->body_by, by.data(), by.size());
        }
        h->have_edges = n_edge > 0;
        if (n_edge > 0) {
            std::vector<int> ptr(static_cast<size_t>(E) + 1, 0), side(n_edge), kind(n_edge);
            std::vector<double> ea(n_edge), eb(n_edge);
            for (i64 k = 0; k < n_edge; ++k) {
                LF_REQUIRE(edge_element[k] >= 0 && edge_element[k] < E, LFGPU_ERR_ARGUMENT,
                           "edge load references an element index out of range");
                LF_REQUIRE(edge_side[k] >= 1 && edge_side[k] <= 4, LFGPU_ERR_ARGUMENT, "Q4 edge must be in [1, 4]");
                LF_REQUIRE(edge_kind[k] == LFGPU_EDGE_TRACTION || edge_kind[k] == LFGPU_EDGE_PRESSURE,
                           LFGPU_ERR_ARGUMENT, "edge load type must be traction or pressure");
                ++ptr[edge_element[k] + 1];
            }
            for (i64 e = 0; e < E; ++e) ptr[e + 1] += ptr[e];
            std::vector<int> fill(ptr.begin(), ptr.end() - 1);
            for (i64 k = 0; k < n_edge; ++k) {
                const int s = fill[edge_element[k]]++;
                side[s] = edge_side[k];
                kind[s] = edge_kind[k];
                ea[s] = edge_first[k];
                eb[s] = edge_second ? edge_second[k] : 0.0;
            }
            upload(*h, h->edge_ptr, ptr.data(), ptr.size());
            upload(*h, h->edge_side, side.data(), side.size());
            upload(*h, h->edge_kind, kind.data(), kind.size());
            upload(*h, h->edge_a, ea.data(), ea.size());
            upload(*h, h->edge_b, eb.data(), eb.size());
        }
        LF_CUDA(cudaStreamSynchronize(h->stream));
    });
}

int lfgpu_set_constraints(lfgpu_t h, int64_t count, const int64_t* dofs, const double* values) {
    return guarded(h, [&] {
        LF_REQUIRE(h->have_pattern, LFGPU_ERR_STATE, "set the pattern before the constraints");
        const i64 n = h->n;
        std::vector<unsigned char> fixed(static_cast<size_t>(n), 0);
        std::vector<double> pres(static_cast<size_t>(n), 0.0);
        for (i64 k = 0; k < count; ++k) {
            LF_REQUIRE(dofs[k] >= 0 && dofs[k] < n, LFGPU_ERR_ARGUMENT, "constrained DOF out of range");
            LF_REQUIRE(!fixed[dofs[k]], LFGPU_ERR_ARGUMENT, "duplicate constraint on one DOF");
            fixed[dofs[k]] = 1;
            pres[dofs[k]] = values[k];
        }
        upload(*h, h->fixed, fixed.data(), fixed.size());
        upload(*h, h->prescribed, pres.data(), pres.size());
        h->n_constraints = count;
        LF_CUDA(cudaStreamSynchronize(h->stream));
    });
}

int lfgpu_assemble(lfgpu_t h, int32_t strategy) {
    return guarded(h, [&] {
        LF_REQUIRE(h->have_pattern, LFGPU_ERR_STATE, "set the mesh and pattern before assembling");
        LF_REQUIRE(strategy == LFGPU_ASSEMBLY_COLORING || strategy == LFGPU_ASSEMBLY_ATOMIC, LFGPU_ERR_ARGUMENT,
                   "assembly strategy must be coloring or atomic");
        LF_REQUIRE(strategy != LFGPU_ASSEMBLY_COLORING || h->n_colors > 0 || h->n_elem == 0, LFGPU_ERR_STATE,
                   "the coloring strategy needs element colours");
        LF_CUDA(cudaEventRecord(h->ev_a, h->stream));
        LF_CUDA(cudaMemsetAsync(h->K.p, 0, sizeof(double) * h->nnz, h->stream));
        if (h->have_nodal)
            LF_CUDA(cudaMemcpyAsync(h->f.p, h->f_nodal.p, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->stream));
        else
            LF_CUDA(cudaMemsetAsync(h->f.p, 0, sizeof(double) * h->n, h->stream));
        launch_assembly(*h, strategy);
        LF_CUDA(cudaEventRecord(h->ev_b, h->stream));
        h->assembled = false;
        ++h->k_version;
        check_status(*h);
        h->timings.assembly_ms = elapsed_ms(*h);
        h->timings.coloring_count = strategy == LFGPU_ASSEMBLY_COLORING ? h->n_colors : 0;
        h->assembled = true;
        h->constrained = false;
        h->solved = false;
    });
}

int lfgpu_apply_dirichlet(lfgpu_t h) {
    return guarded(h, [&] {
        LF_REQUIRE(h->assembled, LFGPU_ERR_STATE, "assemble before applying boundary conditions");
        LF_REQUIRE(!h->constrained, LFGPU_ERR_STATE, "boundary conditions are already applied");
        LF_CUDA(cudaEventRecord(h->ev_a, h->stream));
        LF_CUDA(cudaMemcpyAsync(h->K_full.p, h->K.p, sizeof(double) * h->nnz, cudaMemcpyDeviceToDevice, h->stream));
        LF_CUDA(cudaMemcpyAsync(h->f_full.p, h->f.p, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->stream));
        launch_dirichlet(*h);
        LF_CUDA(cudaEventRecord(h->ev_b, h->stream));
        ++h->k_version;
        check_status(*h);
        h->timings.boundary_ms = elapsed_ms(*h);
        h->constrained = true;
    });
}

namespace {

// The FP32 inner solve of a mixed solve stopped making progress: finish with FP64
// PCG warm-started from its solution s.x.  Adds the device time to *ms.
lfgpu::PcgResult finish_in_fp64(lfgpu_t h, const lfgpu_solve_options* o, const lfgpu::SolveSetup& s,
                                lfgpu::i64 done_iterations, double* ms) {
    using namespace lfgpu;
    Buf<double>& x0 = h->v64[5];
    x0.ensure(h->n);
    LF_CUDA(cudaMemcpyAsync(x0.p, s.x, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, h->stream));
    SolveSetup f = s;
    f.mixed = 0;
    f.x0 = x0.p;
    f.max_iterations = std::max<i64>(1, s.max_iterations - done_iterations);
    float ms2 = 0.f;
    const bool separate = f.precond == LFGPU_PRECOND_SUBDOMAIN || f.precond == LFGPU_PRECOND_IC0;
    const PcgResult r2 = separate        ? run_pcg_separate(*h, f, &ms2, nullptr)
                         : o->persistent ? run_pcg(*h, f, &ms2)
                                         : run_cg_graph(*h, f, &ms2);
    *ms += ms2;
    return r2;
}

}  // namespace

int lfgpu_solve(lfgpu_t h, const lfgpu_solve_options* o, double* u_out, lfgpu_report* rep) {
    return guarded(h, [&] {
        LF_REQUIRE(o != nullptr, LFGPU_ERR_ARGUMENT, "null solve options");
        LF_REQUIRE(h->constrained, LFGPU_ERR_STATE, "apply boundary conditions before solving");
        LF_REQUIRE(o->tolerance > 0.0 && o->tolerance < 1.0, LFGPU_ERR_ARGUMENT,
                   "solver tolerance must satisfy 0 < tolerance < 1");
        LF_REQUIRE(o->max_iterations > 0, LFGPU_ERR_ARGUMENT, "max_iterations must be greater than zero");
        LF_REQUIRE(o->storage == LFGPU_STORAGE_CSR || o->storage == LFGPU_STORAGE_BSR, LFGPU_ERR_ARGUMENT,
                   "storage must be csr or bsr");
        LF_REQUIRE(o->preconditioner >= LFGPU_PRECOND_JACOBI && o->preconditioner <= LFGPU_PRECOND_SUBDOMAIN,
                   LFGPU_ERR_ARGUMENT, "preconditioner must be jacobi, block, ic0 or subdomain");
        LF_REQUIRE(o->precision == LFGPU_PRECISION_FP64 || o->precision == LFGPU_PRECISION_MIXED, LFGPU_ERR_ARGUMENT,
                   "precision must be fp64 or mixed");
        lfgpu_report r{};
        r.status = LFGPU_OK;
        const double fnorm = device_norm2(*h, h->f, h->n);
        const double target = o->tolerance * std::max(1.0, fnorm);
        SolveSetup s{};
        s.storage = o->storage;
        s.precond = o->preconditioner;
        s.tolerance = target;
        s.max_iterations = o->max_iterations;
        s.mixed = o->precision == LFGPU_PRECISION_MIXED;
        s.restart = o->refinement == LFGPU_REFINE_RESTART;
        s.inner_reduction = o->inner_reduction > 0.0 && o->inner_reduction < 1.0 ? o->inner_reduction
                                                                                 : (s.restart ? 1e-4 : 0.1);
        s.max_refinements = o->max_refinements > 0 ? o->max_refinements : 1000;
        s.unrolled = o->unrolled > 0 ? o->unrolled : 0;
        s.rhs = h->f;
        s.x = h->u;
        s.x0 = nullptr;
        const bool had_bsr = h->bsr_version == h->k_version;
        float ms = 0.f;
        double apply_ms = 0.0;
        PcgResult res{};
        LF_CUDA(cudaEventRecord(h->ev_a, h->stream));
        if (o->preconditioner == LFGPU_PRECOND_IC0) {
            LF_CUDA(cudaEventRecord(h->ev_a, h->stream));
            ensure_ic0(*h);
            // The level schedules (once per pattern) and the factor in their order.
            if (ic0_use_levels(*h, s.mixed)) ensure_ic0_sweep_values(*h, s.mixed);
            LF_CUDA(cudaEventRecord(h->ev_b, h->stream));
            r.preconditioner_setup_ms = elapsed_ms(*h);
            if (o->storage == LFGPU_STORAGE_BSR) ensure_bsr(*h);
            if (s.mixed) {
                res = run_cg_graph(*h, s, &ms);
            } else {
                res = run_pcg_separate(*h, s, &ms, &apply_ms);
                r.preconditioner_apply_ms = apply_ms;
            }
            r.ic0_breakdowns = h->ic0_breakdowns;
            r.ic0_levels = h->ic0_levels;
        } else if (o->preconditioner == LFGPU_PRECOND_SUBDOMAIN) {
            LF_CUDA(cudaEventRecord(h->ev_a, h->stream));
            if (s.mixed) ensure_subdomain_inverse(*h);  // factor, then the FP32 block inverses
            else ensure_subdomains(*h);
            LF_CUDA(cudaEventRecord(h->ev_b, h->stream));
            r.preconditioner_setup_ms = elapsed_ms(*h);
            if (o->storage == LFGPU_STORAGE_BSR) ensure_bsr(*h);
            if (s.mixed) {
                res = run_cg_graph(*h, s, &ms);
            } else {
                res = run_pcg_separate(*h, s, &ms, &apply_ms);
                r.preconditioner_apply_ms = apply_ms;
            }
            r.subdomains = h->sub_count;
            r.capture_ratio = h->sub_capture;
            r.degenerate_subdomains = h->sub_degenerate;
        } else {
            LF_CUDA(cudaEventRecord(h->ev_a, h->stream));
            ensure_preconditioners(*h, o->preconditioner);
            LF_CUDA(cudaEventRecord(h->ev_b, h->stream));
            r.preconditioner_setup_ms = elapsed_ms(*h);
            res = o->persistent ? run_pcg(*h, s, &ms) : run_cg_graph(*h, s, &ms);
            if (o->preconditioner == LFGPU_PRECOND_BLOCK2) {
                r.subdomains = h->n / 2;
                r.capture_ratio = capture_ratio_2x2(*h);
                r.degenerate_subdomains = h->degenerate_blocks;
            }
        }
        double total_ms = ms;
        r.iterations = res.iterations;
        r.refinements = res.refinements;
        r.initial_residual = res.initial_residual;
        r.final_residual = res.final_residual;
        r.converged = res.converged;
        r.status = res.status;
        for (int k = 0; k < 6; ++k) r.phase_ms[k] = static_cast<double>(res.phase_ns[k]) * 1e-6;
        r.matvec_ms = r.phase_ms[0];
        if (s.mixed && res.stagnated && res.status == LFGPU_OK) {
            const PcgResult r2 = finish_in_fp64(h, o, s, res.iterations, &total_ms);
            r.iterations += r2.iterations;
            r.final_residual = r2.final_residual;
            r.converged = r2.converged;
            r.status = r2.status;
            r.fallback_fp64 = 1;
        }
        r.solve_ms = total_ms;
        // The graph loop's FP32 copy of a paired CSR pattern is the BSR blocks.
        const bool blocks = o->storage == LFGPU_STORAGE_BSR || (s.mixed && !o->persistent && h->paired);
        r.storage_convert_ms = (blocks && !had_bsr && h->bsr_version == h->k_version) ? h->last_convert_ms : 0.0;
        r.matvec_calls = r.iterations + r.refinements;
        r.matrix_bytes_per_matvec =
            blocks
                ? h->nblocks * (s.mixed ? 4 * 4 + (h->bcol16_ok ? 2 : 4) : 4 * 8 + 4)
                : h->nnz * (s.mixed ? 4 + (h->col16_ok ? 2 : 4) : 8 + 4);
        // True residual ||f - K u|| in FP64.
        Buf<double>& tmp = h->v64[0];
        tmp.ensure(h->n);
        launch_spmv_csr64(*h, h->K, h->u, tmp, h->f);
        r.true_residual = device_norm2(*h, tmp, h->n);
        h->solved = true;
        if (u_out) LF_CUDA(cudaMemcpyAsync(u_out, h->u.p, sizeof(double) * h->n, cudaMemcpyDeviceToHost, h->stream));
        LF_CUDA(cudaStreamSynchronize(h->stream));
        if (rep) *rep = r;
        switch (r.status) {
            case LFGPU_OK:
                break;
            case LFGPU_ERR_NOT_SPD:
                throw Error{r.status, "PCG encountered non-positive curvature; system is not SPD"};
            case LFGPU_ERR_RHO_INITIAL:
                throw Error{r.status, "PCG failed to form a positive initial preconditioned residual"};
            case LFGPU_ERR_RHO:
                throw Error{r.status, "PCG preconditioned residual became non-positive or non-finite"};
            default:
                throw Error{r.status, "PCG stopped with device status " + std::to_string(r.status)};
        }
    });
}

int lfgpu_reactions(lfgpu_t h, double* r_out) {
    return guarded(h, [&] {
        LF_REQUIRE(h->solved, LFGPU_ERR_STATE, "solve before recovering reactions");
        LF_CUDA(cudaEventRecord(h->ev_a, h->stream));
        launch_spmv_csr64(*h, h->K_full, h->u, h->R, h->f_full);
        LF_CUDA(cudaEventRecord(h->ev_b, h->stream));
        h->timings.reactions_ms = elapsed_ms(*h);
        if (r_out) LF_CUDA(cudaMemcpyAsync(r_out, h->R.p, sizeof(double) * h->n, cudaMemcpyDeviceToHost, h->stream));
        LF_CUDA(cudaStreamSynchronize(h->stream));
    });
}

int lfgpu_download(lfgpu_t h, int32_t which, double* out) {
    return guarded(h, [&] {
        LF_REQUIRE(out != nullptr, LFGPU_ERR_ARGUMENT, "null output");
        const double* src = nullptr;
        i64 count = h->n;
        switch (which) {
            case LFGPU_K_FULL:
                LF_REQUIRE(h->assembled, LFGPU_ERR_STATE, "not assembled");
                src = h->constrained ? h->K_full.p : h->K.p;
                count = h->nnz;
                break;
            case LFGPU_K_CONSTRAINED:
                LF_REQUIRE(h->constrained, LFGPU_ERR_STATE, "boundary conditions not applied");
                src = h->K;
                count = h->nnz;
                break;
            case LFGPU_F_FULL:
                LF_REQUIRE(h->assembled, LFGPU_ERR_STATE, "not assembled");
                src = h->constrained ? h->f_full.p : h->f.p;
                break;
            case LFGPU_F_CONSTRAINED:
                LF_REQUIRE(h->constrained, LFGPU_ERR_STATE, "boundary conditions not applied");
                src = h->f;
                break;
            case LFGPU_U:
                LF_REQUIRE(h->solved, LFGPU_ERR_STATE, "not solved");
                src = h->u;
                break;
            case LFGPU_R:
                LF_REQUIRE(h->solved, LFGPU_ERR_STATE, "not solved");
                src = h->R;
                break;
            default:
                throw Error{LFGPU_ERR_ARGUMENT, "unknown array"};
        }
        LF_CUDA(cudaMemcpyAsync(out, src, sizeof(double) * count, cudaMemcpyDeviceToHost, h->stream));
        LF_CUDA(cudaStreamSynchronize(h->stream));
    });
}

int lfgpu_timings_get(lfgpu_t h, lfgpu_timings* out) {
    return guarded(h, [&] {
        LF_REQUIRE(out != nullptr, LFGPU_ERR_ARGUMENT, "null output");
        *out = h->timings;
        out->kernel_launches = h->launches;
    });
}

int lfgpu_event_record(lfgpu_t h, int32_t slot) {
    return guarded(h, [&] {
        LF_REQUIRE(slot >= 0 && slot < 8, LFGPU_ERR_ARGUMENT, "event slot must be in [0, 8)");
        if (!h->user_ev[slot]) LF_CUDA(cudaEventCreate(&h->user_ev[slot]));
        LF_CUDA(cudaEventRecord(h->user_ev[slot], h->stream));
    });
}

int lfgpu_event_elapsed(lfgpu_t h, int32_t slot_a, int32_t slot_b, double* ms) {
    return guarded(h, [&] {
        LF_REQUIRE(slot_a >= 0 && slot_a < 8 && slot_b >= 0 && slot_b < 8 && ms, LFGPU_ERR_ARGUMENT,
                   "bad event slots");
        LF_REQUIRE(h->user_ev[slot_a] && h->user_ev[slot_b], LFGPU_ERR_STATE, "event slot never recorded");
        LF_CUDA(cudaEventSynchronize(h->user_ev[slot_b]));
        float f = 0.f;
        LF_CUDA(cudaEventElapsedTime(&f, h->user_ev[slot_a], h->user_ev[slot_b]));
        *ms = f;
    });
}

int lfgpu_spmv(lfgpu_t h, int32_t which, int32_t storage, int32_t precision, const double* x, double* y,
               int32_t repeat, double* ms_per_call) {
    return guarded(h, [&] {
        LF_REQUIRE(h->assembled, LFGPU_ERR_STATE, "assemble before a product");
        LF_REQUIRE(which == 0 || which == 1, LFGPU_ERR_ARGUMENT, "which must be 0 (full) or 1 (constrained)");
        LF_REQUIRE(which == 0 || h->constrained, LFGPU_ERR_STATE, "boundary conditions not applied");
        LF_REQUIRE(storage == LFGPU_STORAGE_CSR || (storage == LFGPU_STORAGE_BSR && which == 1), LFGPU_ERR_ARGUMENT,
                   "BSR products are available for the constrained matrix");
        const i64 n = h->n;
        const double* val = (which == 0 && h->constrained) ? h->K_full.p : h->K.p;
        Buf<double>& xd = h->v64[4];
        Buf<double>& yd = h->v64[5];
        xd.ensure(n);
        yd.ensure(n);
        Buf<float>& xf = h->v32[4];
        Buf<float>& yf = h->v32[5];
        xf.ensure(n);
        yf.ensure(n);
        if (x) LF_CUDA(cudaMemcpyAsync(xd.p, x, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
        const bool f32 = precision == LFGPU_PRECISION_MIXED;
        if (f32) launch_to_float(*h, xd, xf, n);
        if (storage == LFGPU_STORAGE_BSR) {
            ensure_bsr(*h);
            if (f32) ensure_bsr32(*h);
        } else if (f32) {
            LF_REQUIRE(which == 1, LFGPU_ERR_ARGUMENT, "FP32 products use the constrained matrix");
            ensure_csr32(*h);
        }
        auto once = [&] {
            if (storage == LFGPU_STORAGE_CSR) {
                if (f32) launch_spmv_csr32(*h, h->K32, xf, yf);
                else launch_spmv_csr64(*h, val, xd, yd, nullptr);
            } else {
                if (f32) launch_spmv_bsr32(*h, xf, yf);
                else launch_spmv_bsr64(*h, xd, yd);
            }
        };
        once();
        const int reps = std::max(1, repeat);
        LF_CUDA(cudaEventRecord(h->ev_a, h->stream));
        for (int k = 0; k < reps; ++k) once();
        LF_CUDA(cudaEventRecord(h->ev_b, h->stream));
        const float ms = elapsed_ms(*h);
        if (ms_per_call) *ms_per_call = ms / reps;
        if (y) {
            if (f32) {
                std::vector<float> tmp(static_cast<size_t>(n));
                LF_CUDA(cudaMemcpyAsync(tmp.data(), yf.p, sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream));
                LF_CUDA(cudaStreamSynchronize(h->stream));
                for (i64 i = 0; i < n; ++i) y[i] = tmp[i];
            } else {
                LF_CUDA(cudaMemcpyAsync(y, yd.p, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
            }
        }
        check_status(*h);
    });
}

int lfgpu_postprocess(lfgpu_t h, double* element_fields, double* nodal_stress) {
    return guarded(h, [&] {
        LF_REQUIRE(h->solved, LFGPU_ERR_STATE, "solve before post-processing");
        h->post_fields.ensure(35 * static_cast<size_t>(h->n_elem) + 1);
        h->post_nodal.ensure(4 * static_cast<size_t>(h->n_nodes));
        LF_CUDA(cudaEventRecord(h->ev_a, h->stream));
        launch_postprocess(*h, h->u, h->post_fields, h->post_nodal);
        LF_CUDA(cudaEventRecord(h->ev_b, h->stream));
        h->timings.postprocess_ms = elapsed_ms(*h);
        check_status(*h);
        if (element_fields)
            LF_CUDA(cudaMemcpyAsync(element_fields, h->post_fields.p, sizeof(double) * 35 * h->n_elem,
                                    cudaMemcpyDeviceToHost, h->stream));
        if (nodal_stress)
            LF_CUDA(cudaMemcpyAsync(nodal_stress, h->post_nodal.p, sizeof(double) * 4 * h->n_nodes,
                                    cudaMemcpyDeviceToHost, h->stream));
        LF_CUDA(cudaStreamSynchronize(h->stream));
    });
}

int lfgpu_apply_preconditioner(lfgpu_t h, int32_t preconditioner, const double* r, double* z, double* ms) {
    return guarded(h, [&] {
        LF_REQUIRE(h->constrained, LFGPU_ERR_STATE, "apply boundary conditions before preconditioning");
        LF_REQUIRE(preconditioner >= LFGPU_PRECOND_JACOBI && preconditioner <= LFGPU_PRECOND_SUBDOMAIN,
                   LFGPU_ERR_ARGUMENT, "preconditioner must be jacobi, block, ic0 or subdomain");
        LF_REQUIRE(r != nullptr && z != nullptr, LFGPU_ERR_ARGUMENT, "null vector");
        const i64 n = h->n;
        for (auto& b : h->v64) b.ensure(n);
        Buf<double>& rd = h->v64[5];
        Buf<double>& zd = h->v64[3];
        LF_CUDA(cudaMemcpyAsync(rd.p, r, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
        if (preconditioner == LFGPU_PRECOND_IC0) ensure_ic0(*h);
        else if (preconditioner == LFGPU_PRECOND_SUBDOMAIN) ensure_subdomains(*h);
        else ensure_preconditioners(*h, preconditioner);
        LF_CUDA(cudaEventRecord(h->ev_a, h->stream));
        launch_precond_apply(*h, preconditioner, rd, zd);
        LF_CUDA(cudaEventRecord(h->ev_b, h->stream));
        const float t = elapsed_ms(*h);
        check_status(*h);
        if (ms) *ms = t;
        LF_CUDA(cudaMemcpyAsync(z, zd.p, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
        LF_CUDA(cudaStreamSynchronize(h->stream));
    });
}

int lfgpu_adjoint(lfgpu_t h, const double* dj_du, const lfgpu_solve_options* o, double* grad, lfgpu_report* rep) {
    return guarded(h, [&] {
        LF_REQUIRE(h->solved, LFGPU_ERR_STATE, "solve the forward problem before the adjoint");
        LF_REQUIRE(grad != nullptr, LFGPU_ERR_ARGUMENT, "null gradient output");
        const i64 n = h->n;
        Buf<double>& lam = h->lam;
        lam.ensure(n);
        Buf<double>& g = h->scratch64;
        lfgpu_report r{};
        if (dj_du == nullptr) {
            // Compliance: lambda = u.
            LF_CUDA(cudaMemcpyAsync(lam.p, h->u.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
        } else {
            LF_REQUIRE(o != nullptr, LFGPU_ERR_ARGUMENT, "the adjoint solve needs solve options");
            LF_REQUIRE(o->preconditioner >= LFGPU_PRECOND_JACOBI && o->preconditioner <= LFGPU_PRECOND_SUBDOMAIN,
                       LFGPU_ERR_ARGUMENT, "preconditioner must be jacobi, block, ic0 or subdomain");
            // Solve K lambda = dJ/du with dJ/du zeroed on the constrained DOFs: reuse the
            // solve machinery on the adjoint right-hand side.
            std::vector<double> rhs(dj_du, dj_du + n);
            std::vector<unsigned char> fixed(static_cast<size_t>(n));
            LF_CUDA(cudaMemcpy(fixed.data(), h->fixed.p, n, cudaMemcpyDeviceToHost));
            for (i64 i = 0; i < n; ++i)
                if (fixed[i]) rhs[i] = 0.0;
            Buf<double>& adj_rhs = h->adj_rhs;
            adj_rhs.ensure(n);
            LF_CUDA(cudaMemcpyAsync(adj_rhs.p, rhs.data(), sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
            const double rnorm = [&] {
                double s = 0.0;
                for (double v : rhs) s += v * v;
                return std::sqrt(s);
            }();
            SolveSetup s{};
            s.storage = o->storage;
            s.precond = o->preconditioner;
            s.tolerance = o->tolerance * std::max(1.0, rnorm);
            s.max_iterations = o->max_iterations;
            s.mixed = o->precision == LFGPU_PRECISION_MIXED;
            s.restart = o->refinement == LFGPU_REFINE_RESTART;
            s.inner_reduction = o->inner_reduction > 0.0 && o->inner_reduction < 1.0 ? o->inner_reduction
                                                                                     : (s.restart ? 1e-4 : 0.1);
            s.max_refinements = o->max_refinements > 0 ? o->max_refinements : 1000;
            s.rhs = adj_rhs.p;
            s.x = lam.p;
            float ms = 0.f;
            double apply_ms = 0.0;
            PcgResult res;
            if (o->preconditioner == LFGPU_PRECOND_IC0 || o->preconditioner == LFGPU_PRECOND_SUBDOMAIN) {
                if (o->preconditioner == LFGPU_PRECOND_IC0) ensure_ic0(*h);
                else if (s.mixed) ensure_subdomain_inverse(*h);
                else ensure_subdomains(*h);
                res = s.mixed ? run_cg_graph(*h, s, &ms) : run_pcg_separate(*h, s, &ms, &apply_ms);
            } else {
                ensure_preconditioners(*h, o->preconditioner);
                res = o->persistent ? run_pcg(*h, s, &ms) : run_cg_graph(*h, s, &ms);
            }
            double total_ms = ms;
            r.iterations = res.iterations;
            r.refinements = res.refinements;
            r.initial_residual = res.initial_residual;
            r.final_residual = res.final_residual;
            r.converged = res.converged;
            r.status = res.status;
            if (s.mixed && res.stagnated && res.status == LFGPU_OK) {
                const PcgResult r2 = finish_in_fp64(h, o, s, res.iterations, &total_ms);
                r.iterations += r2.iterations;
                r.final_residual = r2.final_residual;
                r.converged = r2.converged;
                r.status = r2.status;
                r.fallback_fp64 = 1;
            }
            r.solve_ms = total_ms;
            LF_REQUIRE(r.status == LFGPU_OK, r.status, "adjoint PCG failed");
            LF_REQUIRE(r.converged, LFGPU_ERR_STATE, "adjoint PCG did not converge");
        }
        g.ensure(64 + static_cast<size_t>(h->n_elem));
        double* gd = g.p + 64;
        LF_CUDA(cudaEventRecord(h->ev_a, h->stream));
        launch_adjoint_grad(*h, h->u, lam, gd);
        LF_CUDA(cudaEventRecord(h->ev_b, h->stream));
        LF_CUDA(cudaMemcpyAsync(grad, gd, sizeof(double) * h->n_elem, cudaMemcpyDeviceToHost, h->stream));
        check_status(*h);
        h->timings.adjoint_kernel_ms = elapsed_ms(*h);
        if (rep) *rep = r;
    });
}

int lfgpu_mesh_profile(lfgpu_t h, int64_t* profile_out) {
    return guarded(h, [&] {
        LF_REQUIRE(h->n_nodes > 0, LFGPU_ERR_STATE, "set the mesh first");
        LF_REQUIRE(profile_out != nullptr, LFGPU_ERR_ARGUMENT, "null profile output");
        long long p[3];
        if (!mesh_profile_device(*h, p)) {  // a node in too many elements: profile the host pattern
            const HostPattern hp = build_pattern(h->n_nodes, h->n_elem, h->h_elem_nodes.data());
            p[0] = hp.nnz;
            p[1] = p[2] = 0;
            for (i64 r = 0; r < hp.n; ++r) {
                const i64 b = hp.rowptr[r], e = hp.rowptr[r + 1];
                i64 lo = r;
                for (i64 k = b; k < e; ++k) {
                    const i64 col = hp.col[k];
                    p[1] = std::max<long long>(p[1], col > r ? col - r : r - col);
                    if (col <= r) lo = std::min<i64>(lo, col);
                }
                p[2] += r - lo;
            }
        }
        profile_out[0] = 2 * h->n_nodes;
        profile_out[1] = p[0];
        profile_out[2] = p[1];
        profile_out[3] = p[2];
    });
}

int lfgpu_rcm(lfgpu_t h, int64_t* order_out) {
    return guarded(h, [&] {
        LF_REQUIRE(h->n_nodes > 0, LFGPU_ERR_STATE, "set the mesh before ordering it");
        LF_REQUIRE(order_out != nullptr, LFGPU_ERR_ARGUMENT, "null order output");
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<int> order;
        if (rcm_device(*h, order)) {
            for (i64 k = 0; k < h->n_nodes; ++k) order_out[k] = order[static_cast<size_t>(k)];
        } else {  // a level or a node valence beyond the device search: order on the host
            std::vector<long long> ids(static_cast<size_t>(h->n_nodes));
            std::iota(ids.begin(), ids.end(), 0LL);
            std::vector<long long> en(h->h_elem_nodes.begin(), h->h_elem_nodes.end());
            rcm_order(h->n_nodes, ids.data(), h->n_elem, en.data(), reinterpret_cast<long long*>(order_out));
        }
        h->timings.rcm_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    });
}

int lfgpu_set_subdomains(lfgpu_t h, int64_t nodes_per_subdomain, int32_t split) {
    return guarded(h, [&] {
        LF_REQUIRE(nodes_per_subdomain >= 1, LFGPU_ERR_ARGUMENT, "subdomain_nodes must be at least 1");
        LF_REQUIRE(split == LFGPU_SPLIT_RCB || split == LFGPU_SPLIT_CHUNK, LFGPU_ERR_ARGUMENT,
                   "subdomain_split must be rcb or chunk");
        h->sub_nodes = nodes_per_subdomain;
        h->sub_split = split;
    });
}

int lfgpu_host_subdomains(int64_t n_nodes, const double* xy, int64_t nodes_per_subdomain, int32_t split,
                          uint32_t* owner_out, int64_t* count_out) {
    if (n_nodes < 0 || nodes_per_subdomain < 1 || (split != LFGPU_SPLIT_RCB && split != LFGPU_SPLIT_CHUNK) ||
        !count_out || (n_nodes > 0 && (!xy || !owner_out)))
        return LFGPU_ERR_ARGUMENT;
    try {
        std::vector<uint32_t> owner;
        *count_out = subdomain_split(n_nodes, xy, nodes_per_subdomain, split == LFGPU_SPLIT_RCB, owner);
        std::copy(owner.begin(), owner.end(), owner_out);
    } catch (...) {
        return LFGPU_ERR_NOMEM;
    }
    return LFGPU_OK;
}

int lfgpu_host_rcm(int64_t n_nodes, const int64_t* node_ids, int64_t n_elements, const int64_t* element_node_ids,
                   int64_t* order_out) {
    if (n_nodes < 0 || n_elements < 0 || (n_nodes > 0 && (!node_ids || !order_out)) ||
        (n_elements > 0 && !element_node_ids))
        return LFGPU_ERR_ARGUMENT;
    try {
        rcm_order(n_nodes, reinterpret_cast<const long long*>(node_ids), n_elements,
                  reinterpret_cast<const long long*>(element_node_ids), reinterpret_cast<long long*>(order_out));
    } catch (...) {
        return LFGPU_ERR_ARGUMENT;
    }
    return LFGPU_OK;
}

}  // extern "C"
