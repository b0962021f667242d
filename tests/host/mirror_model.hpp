/*
 * mirror_model.hpp — test scaffolding: types with the reference's names and
 * members (Model, Node, Material, Q4Element, ... in include/lightfem/model.hpp;
 * AnalysisResult, LinearSolverReport, PerformanceReport, ... in
 * include/lightfem/solver.hpp) so that tests/host/solve_model.cpp can drive
 * lightfem_gpu::solve (lightfem_gb300/host/lightfem_gpu_solve.hpp) without the
 * reference's library.  Model::sort_and_index and index_with_node_order keep the
 * reference's checks and messages (src/model.cpp:13-92) so the tests can compare
 * the host-side errors too.  The product header is the template alone.
 */
#pragma once

#include "lfgpu.h"

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <optional>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

namespace lightfem_gpu {

// ---------------------------------------------------------------------------
// Mirror types: the reference's names and members.

enum class PlaneMode { PlaneStress, PlaneStrain };

struct Vec2 {
    double x{0.0};
    double y{0.0};
};

struct Node {
    int id{0};
    Vec2 position{};
    std::size_t dof_x{0};
    std::size_t dof_y{0};
};

struct Material {
    int id{0};
    double young_modulus{0.0};
    double poisson_ratio{0.0};
    double thickness{0.0};
};

struct Q4Element {
    int id{0};
    std::array<int, 4> node_ids{{0, 0, 0, 0}};
    int material_id{0};
};

struct TrussElement {
    int id{0};
    std::array<int, 2> node_ids{{0, 0}};
    int material_id{0};
    double area{0.0};
};

struct DirichletBC {
    int node_id{0};
    std::optional<double> ux{};
    std::optional<double> uy{};
};

struct NodalLoad {
    int node_id{0};
    double fx{0.0};
    double fy{0.0};
};

struct BodyForce {
    int element_id{0};
    double bx{0.0};
    double by{0.0};
};

enum class EdgeLoadType { Traction, Pressure };

struct EdgeLoad {
    int element_id{0};
    int edge{0};  // 1 = n1-n2, 2 = n2-n3, 3 = n3-n4, 4 = n4-n1
    EdgeLoadType type{EdgeLoadType::Traction};
    double first{0.0};   // tx or pressure
    double second{0.0};  // ty
};

struct SolverSettings {
    PlaneMode plane_mode{PlaneMode::PlaneStress};
    std::string solver{"gpu"};  // gpu | gpu_mixed
    double tolerance{1.0e-10};
    std::size_t max_iterations{5000};
    std::string reordering{"none"};
    std::string assembly{"gpu"};  // gpu (colouring) | atomic
    std::size_t threads{0};
    std::string storage{"csr"};
    std::string preconditioner{"jacobi"};
    std::string subdomain_split{"rcb"};
    std::size_t subdomain_nodes{64};
};

// Model::sort_and_index / index_with_node_order / rebuild_indices
// (src/model.cpp:24-92): entities sorted by ID, node k owning DOFs 2k and 2k+1.
class Model {
public:
    std::vector<Node> nodes;
    std::vector<Material> materials;
    std::vector<Q4Element> elements;
    std::vector<TrussElement> trusses;
    std::vector<DirichletBC> boundaries;
    std::vector<NodalLoad> loads;
    std::vector<BodyForce> body_forces;
    std::vector<EdgeLoad> edge_loads;
    SolverSettings settings;

    void sort_and_index() {
        sort_by_id(nodes);
        sort_by_id(materials);
        sort_by_id(elements);
        sort_by_id(trusses);
        require_unique_ids(nodes, "node");
        require_unique_ids(materials, "material");
        require_unique_ids(elements, "element");
        require_unique_ids(trusses, "truss");
        rebuild_indices();
    }

    void index_with_node_order(const std::vector<int>& node_order) {
        if (node_order.size() != nodes.size())
            throw std::invalid_argument("node reordering must contain every model node exactly once");
        sort_by_id(materials);
        sort_by_id(elements);
        sort_by_id(trusses);
        require_unique_ids(materials, "material");
        require_unique_ids(elements, "element");
        require_unique_ids(trusses, "truss");
        std::unordered_map<int, std::size_t> where;
        where.reserve(nodes.size());
        for (std::size_t i = 0; i < nodes.size(); ++i)
            if (!where.emplace(nodes[i].id, i).second)
                throw std::logic_error("duplicate node ID: " + std::to_string(nodes[i].id));
        std::vector<Node> reordered;
        reordered.reserve(nodes.size());
        for (const int id : node_order) {
            const auto it = where.find(id);
            if (it == where.end())
                throw std::invalid_argument("node reordering references an unknown or duplicate node ID");
            reordered.push_back(nodes[it->second]);
            where.erase(it);
        }
        nodes = std::move(reordered);
        rebuild_indices();
    }

    [[nodiscard]] bool is_indexed() const noexcept { return indexed_; }

private:
    template <typename T>
    static void sort_by_id(std::vector<T>& v) {
        std::sort(v.begin(), v.end(), [](const T& a, const T& b) { return a.id < b.id; });
    }
    template <typename T>
    static void require_unique_ids(const std::vector<T>& v, const char* label) {
        for (std::size_t i = 1; i < v.size(); ++i)
            if (v[i - 1].id == v[i].id)
                throw std::logic_error(std::string("duplicate ") + label + " ID: " + std::to_string(v[i].id));
    }
    void rebuild_indices() {
        for (std::size_t i = 0; i < nodes.size(); ++i) {
            nodes[i].dof_x = 2 * i;
            nodes[i].dof_y = 2 * i + 1;
        }
        indexed_ = true;
    }

    bool indexed_{false};
};

// The retained stiffness with public arrays (the reference's CsrMatrix keeps
// them private behind accessors of the same names).
struct CsrMatrix {
    std::vector<std::size_t> row_offsets{0};
    std::vector<std::size_t> column_indices;
    std::vector<double> values;
    [[nodiscard]] std::size_t rows() const noexcept { return row_offsets.size() - 1; }
    [[nodiscard]] std::size_t nonzeros() const noexcept { return values.size(); }
};

inline void assign_stiffness(CsrMatrix& m, std::size_t rows, const std::vector<int64_t>& row_offsets,
                             const std::vector<int32_t>& columns, std::vector<double>&& values) {
    m.row_offsets.assign(row_offsets.begin(), row_offsets.begin() + static_cast<std::ptrdiff_t>(rows + 1));
    m.column_indices.assign(columns.begin(), columns.end());
    m.values = std::move(values);
}

struct CsrProfile {
    std::size_t dimension{0};
    std::size_t nonzeros{0};
    std::size_t bandwidth{0};
    std::size_t profile{0};
};

struct ElementField {
    std::array<double, 3> strain{{0.0, 0.0, 0.0}};
    std::array<double, 3> stress{{0.0, 0.0, 0.0}};
    double von_mises{0.0};
};

struct GaussPointField {
    double xi{0.0};
    double eta{0.0};
    ElementField field{};
};

struct ElementResult {
    int element_id{0};
    ElementField field{};
    std::array<GaussPointField, 4> gauss_points{};
};

struct NodeResult {
    int node_id{0};
    std::array<double, 3> stress{{0.0, 0.0, 0.0}};
    double von_mises{0.0};
};

struct LinearSolverReport {
    bool converged{false};
    std::size_t iterations{0};
    double initial_residual{0.0};
    double final_residual{0.0};
    std::string message;
    std::string preconditioner{"jacobi"};
    double solve_ms{0.0};
    double matvec_ms{0.0};
    std::size_t matvec_calls{0};
    std::string storage{"csr"};
    std::size_t matrix_bytes_per_matvec{0};
    double storage_convert_ms{0.0};
    double preconditioner_setup_ms{0.0};
    double preconditioner_apply_ms{0.0};
    std::size_t subdomains{0};
    double capture_ratio{0.0};
};

struct PerformanceReport {
    std::string reordering{"none"};
    CsrProfile before;
    CsrProfile after;
    std::string assembly{"gpu"};
    std::size_t requested_threads{0};
    std::size_t threads_used{1};
    std::size_t coloring_count{0};
    double profile_ms{0.0};
    double pattern_ms{0.0};
    double element_stiffness_ms{0.0};
    double assembly_ms{0.0};
    double boundary_ms{0.0};
    double postprocess_ms{0.0};
    double retain_matrix_ms{0.0};
    double total_ms{0.0};
};

struct AnalysisResult {
    CsrMatrix stiffness;
    std::vector<double> load;
    std::vector<double> displacement;
    std::vector<double> reaction;
    std::vector<ElementResult> element_results;
    std::vector<NodeResult> node_results;
    LinearSolverReport solver;
    PerformanceReport performance;
};

}  // namespace lightfem_gpu

#include "lightfem_gpu_solve.hpp"
