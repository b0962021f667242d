/*
 * lightfem_gpu_solve.hpp — LinearElasticSolver::solve on the GPU for C++ hosts,
 * over liblfgpu's C ABI (include/lfgpu.h).  Header-only; link with -llfgpu.
 *
 * lightfem_gpu::solve(model, result, device) is a template over the host's own
 * model and result types.  It reads and writes only members that the reference's
 * types have (Model, Node, Material, Q4Element, DirichletBC, NodalLoad,
 * BodyForce, EdgeLoad, SolverSettings in include/lightfem/model.hpp;
 * AnalysisResult, LinearSolverReport, PerformanceReport, ElementResult,
 * NodeResult in include/lightfem/solver.hpp), so src/solver.cpp can hand it
 * lightfem::Model and lightfem::AnalysisResult unchanged.  The one member it
 * cannot fill generically is the retained CSR stiffness: the host provides
 * assign_stiffness(CsrMatrix&, rows, row_offsets, columns, values), found by
 * argument-dependent lookup.
 *
 * The stages follow LinearElasticSolver::solve (src/solver.cpp:875-960): RCM
 * (:886-892), pattern + map + colours, element stiffness + assembly + loads
 * (assemble, :219-334), retained K and f, Dirichlet elimination and the
 * zero-pivot sweep (:908-940), solve_iterative (:675-747), the "PCG did not
 * converge" check (:948-950), reactions (:953-954), postprocess and nodal
 * smoothing (:955-957).  Failures raise the reference's exception kinds with its
 * messages: std::invalid_argument for a bad argument, std::logic_error for a
 * call-order error, std::runtime_error for everything the reference reports at
 * run time.
 *
 * Selection follows the .fem keys: settings.solver "gpu_mixed" runs the FP32-inner
 * PCG inside FP64 refinement, any other value FP64 PCG; settings.assembly
 * "atomic" or "gpu_atomic" scatters with atomics, any other value by colours;
 * preconditioner "block" with subdomain_nodes 1 is the fused 2x2 nodal form, any
 * other subdomain_nodes the general subdomain block-Jacobi.  The GPU path
 * assembles Q4 elements only: a model with truss bars is refused.
 */
#pragma once

#include "lfgpu.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <numeric>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <utility>
#include <vector>

namespace lightfem_gpu {

// A status and its message as the reference's exception kind: a bad argument or
// an option combination the library does not build is std::invalid_argument, a
// call-order error std::logic_error, every run-time failure std::runtime_error.
[[noreturn]] inline void raise(int status, const std::string& message) {
    if (status == LFGPU_ERR_ARGUMENT || status == LFGPU_ERR_UNSUPPORTED) throw std::invalid_argument(message);
    if (status == LFGPU_ERR_STATE) throw std::logic_error(message);
    throw std::runtime_error(message);
}

// One liblfgpu handle: one CUDA stream and the device copy of one model.
class Handle {
public:
    explicit Handle(int device) {
        const int rc = lfgpu_create(device, &h_);
        if (rc != LFGPU_OK)
            throw std::runtime_error("lfgpu_create failed with status " + std::to_string(rc) +
                                     " (is a CUDA device visible?)");
    }
    ~Handle() { lfgpu_destroy(h_); }
    Handle(const Handle&) = delete;
    Handle& operator=(const Handle&) = delete;

    [[nodiscard]] lfgpu_t get() const noexcept { return h_; }
    void check(int rc) const {
        if (rc != LFGPU_OK) raise(rc, lfgpu_last_error(h_));
    }

private:
    lfgpu_t h_{nullptr};
};

namespace detail {

inline double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

template <typename Entities>
std::unordered_map<int, int32_t> index_by_id(const Entities& v) {
    std::unordered_map<int, int32_t> m;
    m.reserve(v.size());
    for (std::size_t i = 0; i < v.size(); ++i) m.emplace(v[i].id, static_cast<int32_t>(i));
    return m;
}

inline int32_t find(const std::unordered_map<int, int32_t>& m, int id, const char* what) {
    const auto it = m.find(id);
    if (it == m.end()) throw std::logic_error(what);
    return it->second;
}

// Nodes (in the order `order` gives, or the model's own order when it is empty),
// elements and materials into the handle.
template <typename ModelT>
void set_mesh(const Handle& h, const ModelT& model, const std::vector<std::size_t>& order) {
    const std::size_t n_nodes = model.nodes.size();
    std::vector<double> xy(2 * n_nodes);
    std::unordered_map<int, int32_t> node;
    node.reserve(n_nodes);
    for (std::size_t k = 0; k < n_nodes; ++k) {
        const auto& nd = model.nodes[order.empty() ? k : order[k]];
        xy[2 * k] = nd.position.x;
        xy[2 * k + 1] = nd.position.y;
        node.emplace(nd.id, static_cast<int32_t>(k));
    }
    const auto material = index_by_id(model.materials);
    std::vector<int32_t> element_nodes(4 * model.elements.size()), element_material(model.elements.size());
    for (std::size_t e = 0; e < model.elements.size(); ++e) {
        for (int a = 0; a < 4; ++a)
            element_nodes[4 * e + a] =
                find(node, model.elements[e].node_ids[a], "validated Q4 element references an unknown node");
        element_material[e] =
            find(material, model.elements[e].material_id, "validated element references an unknown material");
    }
    std::vector<double> young, poisson, thickness;
    for (const auto& m : model.materials) {
        young.push_back(m.young_modulus);
        poisson.push_back(m.poisson_ratio);
        thickness.push_back(m.thickness);
    }
    using Mode = decltype(model.settings.plane_mode);
    const int32_t mode = model.settings.plane_mode == Mode::PlaneStrain ? LFGPU_PLANE_STRAIN : LFGPU_PLANE_STRESS;
    h.check(lfgpu_set_mesh(h.get(), static_cast<int64_t>(n_nodes), xy.data(),
                           static_cast<int64_t>(model.elements.size()), element_nodes.data(), element_material.data(),
                           static_cast<int64_t>(model.materials.size()), young.data(), poisson.data(),
                           thickness.data(), mode));
}

template <typename Profile>
Profile profile_of(const Handle& h) {
    int64_t p[4] = {0, 0, 0, 0};
    h.check(lfgpu_mesh_profile(h.get(), p));
    Profile out{};
    out.dimension = static_cast<std::size_t>(p[0]);
    out.nonzeros = static_cast<std::size_t>(p[1]);
    out.bandwidth = static_cast<std::size_t>(p[2]);
    out.profile = static_cast<std::size_t>(p[3]);
    return out;
}

// reverse_cuthill_mckee (src/reordering.cpp:11-62) on the device.  The
// reference ranks ties by node ID, so the mesh goes in in ascending-ID order.
template <typename ModelT>
std::vector<int> rcm_order(const Handle& h, const ModelT& model) {
    std::vector<std::size_t> by_id(model.nodes.size());
    std::iota(by_id.begin(), by_id.end(), std::size_t{0});
    std::stable_sort(by_id.begin(), by_id.end(),
                     [&](std::size_t a, std::size_t b) { return model.nodes[a].id < model.nodes[b].id; });
    set_mesh(h, model, by_id);
    std::vector<int64_t> order(model.nodes.size());
    h.check(lfgpu_rcm(h.get(), order.data()));
    std::vector<int> ids(order.size());
    for (std::size_t i = 0; i < order.size(); ++i) ids[i] = model.nodes[by_id[static_cast<std::size_t>(order[i])]].id;
    return ids;
}

// Loads in the reference's order (src/solver.cpp:303-332): nodal loads summed in
// record order, then body forces, then edge loads, element by element.
template <typename ModelT>
void set_loads(const Handle& h, const ModelT& model) {
    const auto node = index_by_id(model.nodes);
    const auto element = index_by_id(model.elements);
    std::vector<double> nodal(2 * model.nodes.size(), 0.0);
    for (const auto& load : model.loads) {
        const int32_t k = find(node, load.node_id, "validated load references an unknown node");
        nodal[2 * static_cast<std::size_t>(k)] += load.fx;
        nodal[2 * static_cast<std::size_t>(k) + 1] += load.fy;
    }
    std::vector<int32_t> body_e;
    std::vector<double> bx, by;
    for (const auto& f : model.body_forces) {
        body_e.push_back(find(element, f.element_id, "validated body force references an unknown element"));
        bx.push_back(f.bx);
        by.push_back(f.by);
    }
    std::vector<int32_t> edge_e, edge_side, edge_kind;
    std::vector<double> first, second;
    for (const auto& l : model.edge_loads) {
        using Type = decltype(l.type);
        edge_e.push_back(find(element, l.element_id, "validated edge load references an unknown element"));
        edge_side.push_back(static_cast<int32_t>(l.edge));
        edge_kind.push_back(l.type == Type::Pressure ? LFGPU_EDGE_PRESSURE : LFGPU_EDGE_TRACTION);
        first.push_back(l.first);
        second.push_back(l.second);
    }
    const auto ptr = [](auto& v) { return v.empty() ? nullptr : v.data(); };
    h.check(lfgpu_set_loads(h.get(), nodal.data(), static_cast<int64_t>(body_e.size()), ptr(body_e), ptr(bx),
                            ptr(by), static_cast<int64_t>(edge_e.size()), ptr(edge_e), ptr(edge_side),
                            ptr(edge_kind), ptr(first), ptr(second)));
}

// collect_constraints (src/solver.cpp:340-351): (DOF, value) pairs by DOF.
template <typename ModelT>
void set_constraints(const Handle& h, const ModelT& model) {
    const auto node = index_by_id(model.nodes);
    std::vector<std::pair<int64_t, double>> c;
    for (const auto& b : model.boundaries) {
        const int64_t k = find(node, b.node_id, "validated boundary references an unknown node");
        if (b.ux) c.emplace_back(2 * k, *b.ux);
        if (b.uy) c.emplace_back(2 * k + 1, *b.uy);
    }
    std::stable_sort(c.begin(), c.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    std::vector<int64_t> dofs(c.size());
    std::vector<double> values(c.size());
    for (std::size_t i = 0; i < c.size(); ++i) {
        dofs[i] = c[i].first;
        values[i] = c[i].second;
    }
    h.check(lfgpu_set_constraints(h.get(), static_cast<int64_t>(c.size()), dofs.empty() ? nullptr : dofs.data(),
                                  values.empty() ? nullptr : values.data()));
}

// Every ID the records name exists, checked on the host before a device is
// touched, with the reference's messages (q4_dof_indices src/element.cpp:120-123,
// assemble and collect_constraints src/solver.cpp:303-351).
template <typename ModelT>
void check_references(const ModelT& model) {
    const auto node = index_by_id(model.nodes);
    const auto material = index_by_id(model.materials);
    const auto element = index_by_id(model.elements);
    for (const auto& e : model.elements) {
        for (const int id : e.node_ids) find(node, id, "validated Q4 element references an unknown node");
        find(material, e.material_id, "validated element references an unknown material");
    }
    for (const auto& l : model.loads) find(node, l.node_id, "validated load references an unknown node");
    for (const auto& f : model.body_forces)
        find(element, f.element_id, "validated body force references an unknown element");
    for (const auto& l : model.edge_loads)
        find(element, l.element_id, "validated edge load references an unknown element");
    for (const auto& b : model.boundaries) find(node, b.node_id, "validated boundary references an unknown node");
}

// The failure a kernel reported during assembly or elimination, with the
// reference's message: q4_kinematics (src/element.cpp:52-54), the edge loads
// (:189, :206) and the zero-pivot sweep (src/solver.cpp:926-936).
template <typename ModelT>
void check_stage(const Handle& h, const ModelT& model, int rc) {
    if (rc == LFGPU_ERR_JACOBIAN) throw std::runtime_error("Q4 stiffness evaluation received a non-positive Jacobian");
    if (rc != LFGPU_ERR_EDGE && rc != LFGPU_ERR_MECHANISM) return h.check(rc);
    int32_t status = 0;
    int64_t index = -1;
    double values[2] = {0.0, 0.0};
    h.check(lfgpu_failure_detail(h.get(), &status, &index, values));
    if (rc == LFGPU_ERR_EDGE) {
        // The reference stops at the first zero-length loaded edge in record
        // order; its kind names the message.
        const auto node = index_by_id(model.nodes);
        const auto element = index_by_id(model.elements);
        for (const auto& l : model.edge_loads) {
            using Type = decltype(l.type);
            if (l.edge < 1 || l.edge > 4) continue;
            const auto& el = model.elements[static_cast<std::size_t>(
                find(element, l.element_id, "validated edge load references an unknown element"))];
            const auto& a = model.nodes[static_cast<std::size_t>(
                find(node, el.node_ids[l.edge - 1], "validated Q4 element references an unknown node"))];
            const auto& b = model.nodes[static_cast<std::size_t>(
                find(node, el.node_ids[l.edge % 4], "validated Q4 element references an unknown node"))];
            if (!(std::hypot(b.position.x - a.position.x, b.position.y - a.position.y) > 1.0e-14))
                throw std::runtime_error(l.type == Type::Pressure ? "Q4 edge pressure received a zero-length edge"
                                                                  : "Q4 edge traction received a zero-length edge");
        }
        h.check(rc);
    }
    if (index < 0 || static_cast<std::size_t>(index / 2) >= model.nodes.size()) h.check(rc);
    const auto& nd = model.nodes[static_cast<std::size_t>(index / 2)];
    throw std::runtime_error(
        "the structure is a mechanism: a bar end has no transverse stiffness but "
        "carries a transverse load; add a support there or load the bar along its axis [dof " +
        std::to_string(index) + " load " + std::to_string(values[0]) + " diag " + std::to_string(values[1]) +
        " node " + std::to_string(nd.id) + " xy " + std::to_string(nd.position.x) + "," +
        std::to_string(nd.position.y) + "]");
}

// The Jacobi setup's exception (inverse_diagonal_of, src/solver.cpp:656-661) and
// pcg_solve's (:579-581, :591-593, :616-618).
inline void check_solve(const Handle& h, int rc) {
    if (rc == LFGPU_ERR_NONFINITE_DIAG)
        throw std::runtime_error("Jacobi preconditioner encountered a non-finite diagonal");
    if (rc == LFGPU_ERR_RHO_INITIAL)
        throw std::runtime_error("PCG failed to form a positive initial preconditioned residual");
    if (rc == LFGPU_ERR_NOT_SPD) throw std::runtime_error("PCG encountered non-positive curvature; system is not SPD");
    if (rc == LFGPU_ERR_RHO)
        throw std::runtime_error("PCG preconditioned residual became non-positive or non-finite");
    h.check(rc);
}

template <typename SettingsT>
lfgpu_solve_options solve_options(const SettingsT& s) {
    if (s.storage != "csr" && s.storage != "bsr") throw std::invalid_argument("storage must be csr or bsr");
    if (s.preconditioner != "jacobi" && s.preconditioner != "block" && s.preconditioner != "ic0")
        throw std::invalid_argument("preconditioner must be jacobi, block or ic0");
    lfgpu_solve_options o{};
    o.tolerance = s.tolerance;
    o.max_iterations = static_cast<int64_t>(s.max_iterations);
    o.storage = s.storage == "bsr" ? LFGPU_STORAGE_BSR : LFGPU_STORAGE_CSR;
    o.preconditioner = s.preconditioner == "ic0" ? LFGPU_PRECOND_IC0 : LFGPU_PRECOND_JACOBI;
    if (s.preconditioner == "block")
        o.preconditioner = s.subdomain_nodes == 1 ? LFGPU_PRECOND_BLOCK2 : LFGPU_PRECOND_SUBDOMAIN;
    o.precision = s.solver == "gpu_mixed" ? LFGPU_PRECISION_MIXED : LFGPU_PRECISION_FP64;
    o.refinement = LFGPU_REFINE_RELIABLE;
    return o;
}

}  // namespace detail

// LinearElasticSolver::solve (src/solver.cpp:875-960) with every numeric stage
// on the GPU of `device`.  `model` must be indexed; with reordering "rcm" its
// nodes are put in the reverse Cuthill-McKee order, as the reference does.
template <typename ModelT, typename ResultT>
void solve(ModelT& model, ResultT& result, int device = 0) {
    if (!model.is_indexed()) throw std::logic_error("model must pass validation and sort_and_index before solving");
    if (!model.trusses.empty())
        throw std::invalid_argument("the GPU path assembles Q4 elements only: a model with truss bars needs the CPU path");
    detail::check_references(model);
    const auto t_start = std::chrono::steady_clock::now();
    const auto& s = model.settings;
    auto& perf = result.performance;
    using Profile = std::decay_t<decltype(perf.before)>;
    perf.reordering = s.reordering;
    Handle h(device);

    const bool reorder = s.reordering == "rcm";
    auto t0 = std::chrono::steady_clock::now();
    if (reorder) {
        detail::set_mesh(h, model, {});
        perf.before = detail::profile_of<Profile>(h);
        perf.profile_ms = detail::ms_since(t0);
        model.index_with_node_order(detail::rcm_order(h, model));
    }
    detail::set_mesh(h, model, {});
    h.check(lfgpu_build_pattern(h.get()));
    detail::set_loads(h, model);
    detail::set_constraints(h, model);
    t0 = std::chrono::steady_clock::now();
    perf.after = detail::profile_of<Profile>(h);
    perf.profile_ms += detail::ms_since(t0);
    if (!reorder) perf.before = perf.after;

    const bool atomic = s.assembly == "atomic" || s.assembly == "gpu_atomic";
    detail::check_stage(h, model, lfgpu_assemble(h.get(), atomic ? LFGPU_ASSEMBLY_ATOMIC : LFGPU_ASSEMBLY_COLORING));
    detail::check_stage(h, model, lfgpu_apply_dirichlet(h.get()));

    const lfgpu_solve_options o = detail::solve_options(s);
    if (o.preconditioner == LFGPU_PRECOND_SUBDOMAIN)
        h.check(lfgpu_set_subdomains(h.get(), static_cast<int64_t>(s.subdomain_nodes),
                                     s.subdomain_split == "chunk" ? LFGPU_SPLIT_CHUNK : LFGPU_SPLIT_RCB));
    const std::size_t n = 2 * model.nodes.size();
    result.displacement.assign(n, 0.0);
    lfgpu_report rep{};
    detail::check_solve(h, lfgpu_solve(h.get(), &o, result.displacement.data(), &rep));

    auto& r = result.solver;
    r.converged = rep.converged != 0;
    r.iterations = static_cast<std::size_t>(rep.iterations);
    r.initial_residual = rep.initial_residual;
    r.final_residual = rep.final_residual;
    r.message = !r.converged            ? "maximum iterations reached without convergence"
                : rep.iterations == 0 ? "initial residual satisfies tolerance"
                                      : "converged";
    r.preconditioner = s.preconditioner;
    r.solve_ms = rep.solve_ms;
    r.matvec_ms = rep.matvec_ms;
    r.matvec_calls = static_cast<std::size_t>(rep.matvec_calls);
    r.storage = s.storage;
    r.matrix_bytes_per_matvec = static_cast<std::size_t>(rep.matrix_bytes_per_matvec);
    r.storage_convert_ms = rep.storage_convert_ms;
    r.preconditioner_setup_ms = rep.preconditioner_setup_ms;
    r.preconditioner_apply_ms = rep.preconditioner_apply_ms;
    r.subdomains = static_cast<std::size_t>(rep.subdomains);
    r.capture_ratio = rep.capture_ratio;
    if (!r.converged) throw std::runtime_error("PCG did not converge: " + r.message);

    result.reaction.assign(n, 0.0);
    h.check(lfgpu_reactions(h.get(), result.reaction.data()));
    const std::size_t n_elem = model.elements.size();
    std::vector<double> fields(35 * n_elem), nodal(4 * model.nodes.size());
    h.check(lfgpu_postprocess(h.get(), fields.data(), nodal.data()));
    constexpr double g = 0.57735026918962576451;
    constexpr double xi[4] = {-g, g, g, -g}, eta[4] = {-g, -g, g, g};
    result.element_results.assign(n_elem, {});
    for (std::size_t e = 0; e < n_elem; ++e) {
        auto& er = result.element_results[e];
        const double* f = fields.data() + 35 * e;
        const auto put = [](auto& field, const double* v) {
            field.strain = {{v[0], v[1], v[2]}};
            field.stress = {{v[3], v[4], v[5]}};
            field.von_mises = v[6];
        };
        er.element_id = model.elements[e].id;
        put(er.field, f);
        for (int k = 0; k < 4; ++k) {
            er.gauss_points[k].xi = xi[k];
            er.gauss_points[k].eta = eta[k];
            put(er.gauss_points[k].field, f + 7 * (k + 1));
        }
    }
    result.node_results.assign(model.nodes.size(), {});
    for (std::size_t i = 0; i < model.nodes.size(); ++i) {
        auto& nr = result.node_results[i];
        nr.node_id = model.nodes[i].id;
        nr.stress = {{nodal[4 * i], nodal[4 * i + 1], nodal[4 * i + 2]}};
        nr.von_mises = nodal[4 * i + 3];
    }

    int64_t n_dofs = 0, nnz = 0, n_colors = 0;
    h.check(lfgpu_pattern_info(h.get(), &n_dofs, &nnz, &n_colors));
    std::vector<int64_t> row_offsets(static_cast<std::size_t>(n_dofs) + 1);
    std::vector<int32_t> columns(static_cast<std::size_t>(nnz));
    h.check(lfgpu_download_pattern(h.get(), row_offsets.data(), columns.data(), nullptr, nullptr));
    std::vector<double> values(static_cast<std::size_t>(nnz));
    h.check(lfgpu_download(h.get(), LFGPU_K_FULL, values.data()));
    assign_stiffness(result.stiffness, static_cast<std::size_t>(n_dofs), row_offsets, columns, std::move(values));
    result.load.assign(n, 0.0);
    h.check(lfgpu_download(h.get(), LFGPU_F_FULL, result.load.data()));

    lfgpu_timings t{};
    h.check(lfgpu_timings_get(h.get(), &t));
    perf.assembly = s.assembly;
    perf.requested_threads = s.threads;
    perf.coloring_count = static_cast<std::size_t>(t.coloring_count);
    perf.pattern_ms = t.pattern_ms;
    perf.assembly_ms = t.assembly_ms;
    perf.boundary_ms = t.boundary_ms;
    perf.postprocess_ms = t.reactions_ms + t.postprocess_ms;
    perf.total_ms = detail::ms_since(t_start);
}

}  // namespace lightfem_gpu
