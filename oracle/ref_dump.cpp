// ref_dump — golden-vector generator built from the reference's own, unmodified
// sources (test infrastructure only).
//
// The reference keeps its assembly, Dirichlet and colouring stages in an
// anonymous namespace inside src/solver.cpp, so this translation unit includes
// that file in place: every stage below runs the reference's own code, exactly
// as LinearElasticSolver::solve (src/solver.cpp:875-960) sequences it, and each
// intermediate is written out as a .npy array for the tests under tests/golden.
//
// Usage: ref_dump <model.fem> <outdir> [key=value ...]
//   setting overrides: assembly storage preconditioner subdomain_split
//                      subdomain_nodes tolerance max_iterations reordering threads
//   stages:  pattern=1 (pattern, map, colours, K, f, Kc, fc, BSR)
//            solve=1   (u, R, element fields, smoothed nodal stress and the solver
//                       report through the public solve())
//            precond=1 (M^-1 fc for jacobi / 2x2 block / ic0, and the ic0 report)
//            fd=<i,j,..> fd_step=<rel> tip_node=<id>  (central differences of the
//                      compliance f.u and of the tip uy w.r.t. element moduli)
//            ke=<count> (element matrices of the first <count> elements)
//            outcome=1 (the public solve() once: "converged" with its iterations
//                       and u, or the message of the exception it throws)
//   library-level inputs (the solver needs only an indexed model,
//   src/solver.cpp:876-878; the parser and validator refuse these values):
//            validate=0          skip ModelValidator
//            set_young=<id>:<v>  Young's modulus of material <id> after parsing
//            set_fy=<id>:<v>     fy of the nodal load at node <id> after parsing
//            (<v> is read with strtod, so nan and inf are accepted)
#include "src/solver.cpp"

#include "lightfem/input_parser.hpp"
#include "lightfem/validation.hpp"

#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

namespace {

using lightfem::Model;

void write_npy(const std::string& path, const char* descr, const void* data, std::size_t count,
               std::size_t item, std::size_t cols = 0) {
    std::string shape = cols == 0 ? "(" + std::to_string(count) + ",)"
                                  : "(" + std::to_string(count / cols) + ", " + std::to_string(cols) + ")";
    std::string header = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': " + shape + ", }";
    const std::size_t prefix = 10;
    std::size_t total = prefix + header.size() + 1;
    const std::size_t pad = (64 - total % 64) % 64;
    header.append(pad, ' ');
    header.push_back('\n');
    std::ofstream out(path, std::ios::binary);
    const unsigned char magic[8] = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
    out.write(reinterpret_cast<const char*>(magic), 8);
    const unsigned short len = static_cast<unsigned short>(header.size());
    out.put(static_cast<char>(len & 0xff));
    out.put(static_cast<char>(len >> 8));
    out.write(header.data(), static_cast<std::streamsize>(header.size()));
    out.write(static_cast<const char*>(data), static_cast<std::streamsize>(count * item));
}

void dump_f64(const std::string& dir, const std::string& name, const std::vector<double>& v, std::size_t cols = 0) {
    write_npy(dir + "/" + name + ".npy", "<f8", v.data(), v.size(), 8, cols);
}

void dump_i64(const std::string& dir, const std::string& name, const std::vector<long long>& v, std::size_t cols = 0) {
    write_npy(dir + "/" + name + ".npy", "<i8", v.data(), v.size(), 8, cols);
}

template <typename T>
std::vector<long long> as_i64(const std::vector<T>& v) {
    return std::vector<long long>(v.begin(), v.end());
}

Model load(const std::string& path, const std::map<std::string, std::string>& opt) {
    Model model = lightfem::InputParser{}.parse_file(path);
    auto& s = model.settings;
    for (const auto& [key, value] : opt) {
        if (key == "assembly") s.assembly = value;
        else if (key == "storage") s.storage = value;
        else if (key == "preconditioner") s.preconditioner = value;
        else if (key == "subdomain_split") s.subdomain_split = value;
        else if (key == "subdomain_nodes") s.subdomain_nodes = std::stoull(value);
        else if (key == "tolerance") s.tolerance = std::stod(value);
        else if (key == "max_iterations") s.max_iterations = std::stoull(value);
        else if (key == "reordering") s.reordering = value;
        else if (key == "threads") s.threads = std::stoull(value);
    }
    for (const auto& [key, value] : opt) {
        if (key != "set_young" && key != "set_fy") continue;
        const std::size_t colon = value.find(':');
        const int id = std::stoi(value.substr(0, colon));
        const double v = std::strtod(value.c_str() + colon + 1, nullptr);
        bool found = false;
        if (key == "set_young") {
            for (auto& m : model.materials) {
                if (m.id != id) continue;
                m.young_modulus = v;
                found = true;
            }
        } else {
            for (auto& l : model.loads) {
                if (l.node_id != id) continue;
                l.fy = v;
                found = true;
            }
        }
        if (!found) throw std::runtime_error(key + ": no record with id " + std::to_string(id));
    }
    if (!opt.count("validate") || opt.at("validate") != "0") {
        const lightfem::ValidationReport report = lightfem::ModelValidator{}.validate(model);
        if (!report.ok()) {
            for (const auto& d : report.diagnostics())
                std::fprintf(stderr, "%s: %s\n", d.code.c_str(), d.message.c_str());
            throw std::runtime_error("model did not pass the reference validation");
        }
    }
    model.sort_and_index();
    return model;
}

struct Json {
    std::ostringstream text;
    bool first = true;
    void key(const std::string& k) {
        text << (first ? "{" : ", ") << '"' << k << "\": ";
        first = false;
    }
    void num(const std::string& k, double v) {
        key(k);
        char buf[64];
        std::snprintf(buf, sizeof buf, "%.17g", v);
        text << buf;
    }
    void str(const std::string& k, const std::string& v) {
        key(k);
        text << '"' << v << '"';
    }
    std::string done() { return text.str() + (first ? "{}" : "}"); }
};

void stage_pattern(Model model, const std::string& dir, Json& json, std::size_t ke_count) {
    using namespace lightfem;
    if (model.settings.reordering == "rcm") model.index_with_node_order(reverse_cuthill_mckee(model));
    std::vector<long long> order;
    for (const Node& node : model.nodes) order.push_back(node.id);
    dump_i64(dir, "node_order", order);

    const ElementDofList element_dofs = element_dof_lists(model);
    std::vector<long long> dofs_flat;
    for (const auto& d : element_dofs) dofs_flat.insert(dofs_flat.end(), d.begin(), d.end());
    dump_i64(dir, "elem_dofs", dofs_flat, 8);

    const CsrAssemblyPattern pattern = build_csr_assembly_pattern(model.summary().dofs, element_dofs);
    dump_i64(dir, "rowptr", as_i64(pattern.matrix.row_offsets()));
    dump_i64(dir, "col", as_i64(pattern.matrix.column_indices()));
    std::vector<long long> map_flat;
    for (const auto& m : pattern.element_value_indices) map_flat.insert(map_flat.end(), m.begin(), m.end());
    dump_i64(dir, "map", map_flat, 64);

    const auto groups = element_colors(model);
    std::vector<long long> colors(element_dofs.size(), -1);
    for (std::size_t c = 0; c < groups.size(); ++c)
        for (const std::size_t e : groups[c]) colors[e] = static_cast<long long>(c);
    dump_i64(dir, "colors", colors);
    json.num("n_colors", static_cast<double>(groups.size()));

    AssembledSystem system = assemble(model);
    dump_f64(dir, "K", system.stiffness.values());
    dump_f64(dir, "f", system.load);
    json.num("coloring_count", static_cast<double>(system.coloring_count));

    CsrMatrix constrained = system.stiffness;
    std::vector<double> load = system.load;
    const auto constraints = collect_constraints(model);
    std::vector<long long> c_dofs;
    std::vector<double> c_vals;
    for (const auto& c : constraints) {
        c_dofs.push_back(static_cast<long long>(c.first));
        c_vals.push_back(c.second);
    }
    dump_i64(dir, "constraint_dofs", c_dofs);
    dump_f64(dir, "constraint_values", c_vals);
    apply_dirichlet(constrained, load, constraints);
    // Zero-pivot sweep exactly as LinearElasticSolver::solve runs it.
    {
        const std::vector<double> diagonal = constrained.diagonal();
        double load_scale = 0.0;
        for (const double value : load) load_scale = std::max(load_scale, std::abs(value));
        if (load_scale <= 0.0) load_scale = 1.0;
        for (std::size_t i = 0; i < diagonal.size(); ++i) {
            if (std::abs(diagonal[i]) > 1.0e-30) continue;
            if (std::abs(load[i]) > 1.0e-12 * load_scale) throw std::runtime_error("mechanism");
            constrained.set(i, i, 1.0);
            load[i] = 0.0;
        }
    }
    dump_f64(dir, "Kc", constrained.values());
    dump_f64(dir, "fc", load);

    if (constrained.rows() % 2 == 0) {
        const BsrMatrix bsr = BsrMatrix::from_csr(constrained);
        dump_i64(dir, "bsr_rowptr", as_i64(bsr.block_row_offsets()));
        dump_i64(dir, "bsr_col", as_i64(bsr.block_columns()));
        dump_f64(dir, "bsr_val", bsr.values(), 4);
        std::vector<double> y;
        bsr.multiply_into(load, y);
        dump_f64(dir, "bsr_Kc_fc", y);
    }
    std::vector<double> y(constrained.rows(), 0.0);
    constrained.multiply_into(load, y);
    dump_f64(dir, "csr_Kc_fc", y);

    if (ke_count > 0) {
        std::vector<double> ke;
        for (std::size_t e = 0; e < std::min(ke_count, model.elements.size()); ++e) {
            const Q4Element& element = model.elements[e];
            const ElementMatrix m = q4_stiffness(q4_coordinates(model, element),
                                                 *model.find_material(element.material_id),
                                                 model.settings.plane_mode);
            ke.insert(ke.end(), m.begin(), m.end());
        }
        dump_f64(dir, "Ke", ke, 64);
    }
}

void stage_precond(Model model, const std::string& dir, Json& json) {
    using namespace lightfem;
    if (model.settings.reordering == "rcm") model.index_with_node_order(reverse_cuthill_mckee(model));
    AssembledSystem system = assemble(model);
    CsrMatrix constrained = system.stiffness;
    std::vector<double> load = system.load;
    apply_dirichlet(constrained, load, collect_constraints(model));
    const std::vector<double> inv = inverse_diagonal_of(constrained.diagonal());
    std::vector<double> z(load.size(), 0.0);
    JacobiPreconditioner(inv).apply(load, z);
    dump_f64(dir, "z_jacobi", z);

    std::size_t count = 0;
    const auto owner = build_dof_subdomain(model, model.settings.subdomain_split,
                                           model.settings.subdomain_nodes, count);
    SubdomainBlockJacobi block(constrained, owner, count);
    std::vector<double> zb(load.size(), 0.0);
    block.apply(load, zb);
    dump_f64(dir, "z_block", zb);
    json.num("block_subdomains", static_cast<double>(block.stats().subdomains));
    json.num("block_capture_ratio", block.stats().capture_ratio);
    json.num("block_degenerate", static_cast<double>(block.stats().degenerate_subdomains));

    IncompleteCholesky0 ic(constrained);
    std::vector<double> zi(load.size(), 0.0);
    ic.apply(load, zi);
    dump_f64(dir, "z_ic0", zi);
    json.num("ic0_breakdowns", static_cast<double>(ic.stats().breakdowns));
    json.num("ic0_factor_entries", static_cast<double>(ic.stats().factor_entries));
}

void stage_solve(Model model, const std::string& dir, Json& json) {
    using namespace lightfem;
    const AnalysisResult result = LinearElasticSolver{}.solve(model);
    // Results are dumped in node-ID order so a reordered and a plain run compare
    // entry by entry: row 2k/2k+1 is the k-th node in ascending ID.
    std::vector<std::pair<int, std::size_t>> by_id;
    for (const Node& node : model.nodes) by_id.emplace_back(node.id, node.dof_x);
    std::sort(by_id.begin(), by_id.end());
    std::vector<double> u, r, u_raw = result.displacement;
    for (const auto& [id, dof] : by_id) {
        (void)id;
        u.push_back(result.displacement[dof]);
        u.push_back(result.displacement[dof + 1]);
        r.push_back(result.reaction[dof]);
        r.push_back(result.reaction[dof + 1]);
    }
    dump_f64(dir, "u", u);
    dump_f64(dir, "R", r);
    // Element fields (element-ID order): centre then the four Gauss points, each
    // strain[3], stress[3], von Mises; smoothed nodal stress[3] + von Mises in
    // node-ID order.
    std::vector<double> fields, nodal;
    for (const ElementResult& er : result.element_results) {
        auto put = [&](const ElementField& f) {
            fields.insert(fields.end(), f.strain.begin(), f.strain.end());
            fields.insert(fields.end(), f.stress.begin(), f.stress.end());
            fields.push_back(f.von_mises);
        };
        put(er.field);
        for (const auto& gp : er.gauss_points) put(gp.field);
    }
    std::vector<std::pair<int, const NodeResult*>> nodes_by_id;
    for (const NodeResult& nr : result.node_results) nodes_by_id.emplace_back(nr.node_id, &nr);
    std::sort(nodes_by_id.begin(), nodes_by_id.end());
    for (const auto& [id, nr] : nodes_by_id) {
        (void)id;
        nodal.insert(nodal.end(), nr->stress.begin(), nr->stress.end());
        nodal.push_back(nr->von_mises);
    }
    dump_f64(dir, "post_fields", fields);
    dump_f64(dir, "post_nodal", nodal);
    json.num("iterations", static_cast<double>(result.solver.iterations));
    json.num("initial_residual", result.solver.initial_residual);
    json.num("final_residual", result.solver.final_residual);
    json.num("converged", result.solver.converged ? 1.0 : 0.0);
    json.num("pcg_ms", result.solver.solve_ms);
    json.num("matvec_ms", result.solver.matvec_ms);
    json.num("matvec_calls", static_cast<double>(result.solver.matvec_calls));
    json.num("matrix_bytes_per_matvec", static_cast<double>(result.solver.matrix_bytes_per_matvec));
    json.num("subdomains", static_cast<double>(result.solver.subdomains));
    json.num("capture_ratio", result.solver.capture_ratio);
    json.num("nnz", static_cast<double>(result.stiffness.nonzeros()));
    json.num("dofs", static_cast<double>(result.displacement.size()));
    json.num("element_stiffness_ms", result.performance.element_stiffness_ms);
    json.num("assembly_ms", result.performance.assembly_ms);
    json.num("pattern_ms", result.performance.pattern_ms);
    json.num("boundary_ms", result.performance.boundary_ms);
    json.num("threads_used", static_cast<double>(result.performance.threads_used));
    json.num("perf_coloring_count", static_cast<double>(result.performance.coloring_count));
    json.num("bandwidth_before", static_cast<double>(result.performance.before.bandwidth));
    json.num("bandwidth_after", static_cast<double>(result.performance.after.bandwidth));
    json.num("profile_before", static_cast<double>(result.performance.before.profile));
    json.num("profile_after", static_cast<double>(result.performance.after.profile));
    double compliance = 0.0;
    for (std::size_t i = 0; i < result.load.size(); ++i) compliance += result.load[i] * result.displacement[i];
    json.num("compliance", compliance);
    json.str("storage", result.solver.storage);
    json.str("preconditioner", result.solver.preconditioner);
}

// Central differences of c = f.u and of the tip uy with respect to the modulus of
// single elements. Each listed element must own its material (one material per
// element), which is how the per-element-modulus meshes are written.
void stage_fd(const Model& base, const std::string& dir, const std::string& list, double step, int tip_node,
              Json& json) {
    using namespace lightfem;
    std::vector<long long> elems;
    std::stringstream ss(list);
    for (std::string item; std::getline(ss, item, ',');) elems.push_back(std::stoll(item));
    std::vector<double> dc, dtip;
    for (const long long e : elems) {
        double values[2][2] = {{0, 0}, {0, 0}};
        double modulus = 0.0;
        for (int side = 0; side < 2; ++side) {
            Model model = base;
            const int material_id = model.elements[static_cast<std::size_t>(e)].material_id;
            Material* material = nullptr;
            for (Material& m : model.materials)
                if (m.id == material_id) material = &m;
            modulus = material->young_modulus;
            material->young_modulus = modulus * (1.0 + (side == 0 ? step : -step));
            model.sort_and_index();
            const AnalysisResult result = LinearElasticSolver{}.solve(model);
            double c = 0.0;
            for (std::size_t i = 0; i < result.load.size(); ++i) c += result.load[i] * result.displacement[i];
            values[side][0] = c;
            values[side][1] = result.displacement[model.find_node(tip_node)->dof_y];
        }
        dc.push_back((values[0][0] - values[1][0]) / (2.0 * step * modulus));
        dtip.push_back((values[0][1] - values[1][1]) / (2.0 * step * modulus));
    }
    dump_i64(dir, "fd_elements", elems);
    dump_f64(dir, "fd_dc_dE", dc);
    dump_f64(dir, "fd_dtip_dE", dtip);
    json.num("fd_step", step);
    json.num("fd_tip_node", tip_node);
}

}  // namespace

// One public solve(): the outcome the GPU path's failure tests compare with.
void stage_outcome(Model model, const std::string& dir, Json& json) {
    using namespace lightfem;
    try {
        const AnalysisResult result = LinearElasticSolver{}.solve(model);
        json.str("outcome", "converged");
        json.num("iterations", static_cast<double>(result.solver.iterations));
        std::vector<std::pair<int, std::size_t>> by_id;
        for (const Node& node : model.nodes) by_id.emplace_back(node.id, node.dof_x);
        std::sort(by_id.begin(), by_id.end());
        std::vector<double> u;
        for (const auto& [id, dof] : by_id) {
            (void)id;
            u.push_back(result.displacement[dof]);
            u.push_back(result.displacement[dof + 1]);
        }
        dump_f64(dir, "u", u);
    } catch (const std::runtime_error& error) {
        json.str("outcome", error.what());
    }
}

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: ref_dump <model.fem> <outdir> [key=value ...]\n");
        return 1;
    }
    const std::string path = argv[1];
    const std::string dir = argv[2];
    std::map<std::string, std::string> opt;
    for (int i = 3; i < argc; ++i) {
        const char* eq = std::strchr(argv[i], '=');
        if (eq == nullptr) continue;
        opt[std::string(argv[i], static_cast<std::size_t>(eq - argv[i]))] = std::string(eq + 1);
    }
    try {
        const Model model = load(path, opt);
        Json json;
        if (opt.count("pattern")) stage_pattern(model, dir, json, opt.count("ke") ? std::stoull(opt["ke"]) : 0);
        if (opt.count("precond")) stage_precond(model, dir, json);
        if (opt.count("solve")) stage_solve(model, dir, json);
        if (opt.count("outcome")) stage_outcome(model, dir, json);
        if (opt.count("fd")) {
            stage_fd(model, dir, opt["fd"], opt.count("fd_step") ? std::stod(opt["fd_step"]) : 1e-6,
                     opt.count("tip_node") ? std::stoi(opt["tip_node"]) : 1, json);
        }
        std::ofstream(dir + "/report.json") << json.done() << '\n';
    } catch (const std::exception& error) {
        std::fprintf(stderr, "ref_dump: %s\n", error.what());
        return 4;
    }
    return 0;
}
