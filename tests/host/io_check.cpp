// Parity check of lightfem_gb300/host/lightfem_gpu_io.hpp against the reference's
// own parser and writers (src/input_parser.cpp, src/vtk_writer.cpp), compiled from
// the reference tree:
//
//   io_check <out_dir> <threads> <file.fem>...
//   io_check --time <out_dir> <threads> <file.fem>
//
// For each file: both parsers must give the same records (every field, in order)
// or fail with the same message; a file that parses and validates is solved with
// the reference's solver, and both writers must write the same VTK and CSV bytes.
// Prints one line per file ("ok ...") and exits non-zero on the first difference.
// --time skips the solve (a large model): it fills the result with seeded values
// of the right sizes, writes both ways, compares the bytes and prints the wall
// time of each parse and write.
#include "lightfem/input_parser.hpp"
#include "lightfem/model.hpp"
#include "lightfem/solver.hpp"
#include "lightfem/validation.hpp"
#include "lightfem/vtk_writer.hpp"
#include "lightfem_gpu_io.hpp"

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <fstream>
#include <iostream>
#include <iterator>
#include <sstream>
#include <string>

namespace {

int failures = 0;

void differ(const std::string& what) {
    std::cout << "DIFFER " << what << "\n";
    ++failures;
}

template <typename A>
bool same_opt(const std::optional<A>& a, const std::optional<A>& b) {
    return a.has_value() == b.has_value() && (!a || *a == *b);
}

void compare(const lightfem::Model& a, const lightfem::Model& b, const std::string& name) {
    bool ok = a.nodes.size() == b.nodes.size() && a.materials.size() == b.materials.size() &&
              a.elements.size() == b.elements.size() && a.trusses.size() == b.trusses.size() &&
              a.boundaries.size() == b.boundaries.size() && a.loads.size() == b.loads.size() &&
              a.body_forces.size() == b.body_forces.size() && a.edge_loads.size() == b.edge_loads.size() &&
              a.source_name == b.source_name;
    for (std::size_t i = 0; ok && i < a.nodes.size(); ++i) {
        const auto &x = a.nodes[i], &y = b.nodes[i];
        ok = x.id == y.id && x.position.x == y.position.x && x.position.y == y.position.y && x.dof_x == y.dof_x &&
             x.dof_y == y.dof_y && x.source_line == y.source_line;
    }
    for (std::size_t i = 0; ok && i < a.materials.size(); ++i) {
        const auto &x = a.materials[i], &y = b.materials[i];
        ok = x.id == y.id && x.young_modulus == y.young_modulus && x.poisson_ratio == y.poisson_ratio &&
             x.thickness == y.thickness && x.source_line == y.source_line;
    }
    for (std::size_t i = 0; ok && i < a.elements.size(); ++i) {
        const auto &x = a.elements[i], &y = b.elements[i];
        ok = x.id == y.id && x.node_ids == y.node_ids && x.material_id == y.material_id &&
             x.source_line == y.source_line;
    }
    for (std::size_t i = 0; ok && i < a.trusses.size(); ++i) {
        const auto &x = a.trusses[i], &y = b.trusses[i];
        ok = x.id == y.id && x.node_ids == y.node_ids && x.material_id == y.material_id && x.area == y.area &&
             x.source_line == y.source_line;
    }
    for (std::size_t i = 0; ok && i < a.boundaries.size(); ++i) {
        const auto &x = a.boundaries[i], &y = b.boundaries[i];
        ok = x.node_id == y.node_id && same_opt(x.ux, y.ux) && same_opt(x.uy, y.uy) && x.source_line == y.source_line;
    }
    for (std::size_t i = 0; ok && i < a.loads.size(); ++i) {
        const auto &x = a.loads[i], &y = b.loads[i];
        ok = x.node_id == y.node_id && x.fx == y.fx && x.fy == y.fy && x.source_line == y.source_line;
    }
    for (std::size_t i = 0; ok && i < a.body_forces.size(); ++i) {
        const auto &x = a.body_forces[i], &y = b.body_forces[i];
        ok = x.element_id == y.element_id && x.bx == y.bx && x.by == y.by && x.source_line == y.source_line;
    }
    for (std::size_t i = 0; ok && i < a.edge_loads.size(); ++i) {
        const auto &x = a.edge_loads[i], &y = b.edge_loads[i];
        ok = x.element_id == y.element_id && x.edge == y.edge && x.type == y.type && x.first == y.first &&
             x.second == y.second && x.source_line == y.source_line;
    }
    const auto &s = a.settings, &t = b.settings;
    ok = ok && s.plane_mode == t.plane_mode && s.solver == t.solver && s.tolerance == t.tolerance &&
         s.max_iterations == t.max_iterations && s.reordering == t.reordering && s.assembly == t.assembly &&
         s.threads == t.threads && s.storage == t.storage && s.preconditioner == t.preconditioner &&
         s.subdomain_split == t.subdomain_split && s.subdomain_nodes == t.subdomain_nodes &&
         s.output_file == t.output_file && s.deformation_scale == t.deformation_scale && s.csv_prefix == t.csv_prefix;
    if (!ok) differ(name + ": parsed records");
}

std::string slurp(const std::string& path) {
    std::ifstream in(path, std::ios::binary);
    return std::string((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
}

}  // namespace

double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

int time_io(const std::string& out, unsigned threads, const std::string& path) {
    auto t0 = std::chrono::steady_clock::now();
    lightfem::Model ref = lightfem::InputParser{}.parse_file(path);
    const double ref_parse = ms_since(t0);
    t0 = std::chrono::steady_clock::now();
    lightfem::Model ours = lightfem_gpu::parse_fem<lightfem::Model>(path, threads);
    const double our_parse = ms_since(t0);
    compare(ref, ours, path);
    ref.sort_and_index();
    lightfem::AnalysisResult r;
    const std::size_t n = ref.summary().dofs;
    std::mt19937_64 rng(7);
    std::normal_distribution<double> g(0.0, 1e-4);
    r.displacement.resize(n);
    r.reaction.resize(n);
    for (auto& v : r.displacement) v = g(rng);
    for (auto& v : r.reaction) v = g(rng) * 1e6;
    r.node_results.resize(ref.nodes.size());
    for (std::size_t i = 0; i < ref.nodes.size(); ++i) {
        r.node_results[i].node_id = ref.nodes[i].id;
        for (auto& v : r.node_results[i].stress) v = g(rng) * 1e10;
        r.node_results[i].von_mises = std::abs(g(rng)) * 1e10;
    }
    r.element_results.resize(ref.elements.size());
    for (std::size_t e = 0; e < ref.elements.size(); ++e) {
        auto& x = r.element_results[e];
        x.element_id = ref.elements[e].id;
        for (auto& v : x.field.strain) v = g(rng);
        for (auto& v : x.field.stress) v = g(rng) * 1e10;
        x.field.von_mises = std::abs(g(rng)) * 1e10;
        for (auto& p : x.gauss_points) {
            p.xi = g(rng);
            p.eta = g(rng);
            for (auto& v : p.field.strain) v = g(rng);
            for (auto& v : p.field.stress) v = g(rng) * 1e10;
            p.field.von_mises = std::abs(g(rng)) * 1e10;
        }
    }
    t0 = std::chrono::steady_clock::now();
    lightfem::write_vtk(ref, r, out + "/time_ref.vtk");
    const auto rp = lightfem::write_csv_results(ref, r, out + "/time_ref");
    const double ref_write = ms_since(t0);
    t0 = std::chrono::steady_clock::now();
    lightfem_gpu::write_vtk(ref, r, out + "/time_gpu.vtk", threads);
    const auto gp = lightfem_gpu::write_csv_results(ref, r, out + "/time_gpu", threads);
    const double our_write = ms_since(t0);
    if (slurp(out + "/time_ref.vtk") != slurp(out + "/time_gpu.vtk")) differ(path + ": VTK bytes");
    if (slurp(rp.nodes) != slurp(gp.first)) differ(path + ": nodes CSV bytes");
    if (slurp(rp.gauss_points) != slurp(gp.second)) differ(path + ": Gauss-point CSV bytes");
    std::printf("{\"nodes\": %zu, \"threads\": %u, \"parse_ms\": {\"reference\": %.1f, \"threaded\": %.1f}, "
                "\"write_ms\": {\"reference\": %.1f, \"threaded\": %.1f}, \"identical\": %s}\n",
                ref.nodes.size(), threads, ref_parse, our_parse, ref_write, our_write, failures ? "false" : "true");
    return failures == 0 ? 0 : 1;
}

int main(int argc, char** argv) {
    if (argc == 5 && std::string(argv[1]) == "--time")
        return time_io(argv[2], static_cast<unsigned>(std::atoi(argv[3])), argv[4]);
    if (argc < 4) {
        std::cerr << "usage: io_check <out_dir> <threads> <file.fem>...\n";
        return 2;
    }
    const std::string out = argv[1];
    const unsigned threads = static_cast<unsigned>(std::atoi(argv[2]));
    for (int k = 3; k < argc; ++k) {
        const std::string path = argv[k];
        std::string ref_error, our_error;
        lightfem::Model ref, ours;
        try {
            ref = lightfem::InputParser{}.parse_file(path);
        } catch (const std::exception& e) {
            ref_error = e.what();
        }
        try {
            ours = lightfem_gpu::parse_fem<lightfem::Model>(path, threads);
        } catch (const std::exception& e) {
            our_error = e.what();
        }
        if (ref_error != our_error) {
            differ(path + ": parse error '" + ref_error + "' vs '" + our_error + "'");
            continue;
        }
        if (!ref_error.empty()) {
            std::cout << "ok " << path << " (both fail: " << ref_error << ")\n";
            continue;
        }
        compare(ref, ours, path);
        const lightfem::ValidationReport report = lightfem::ModelValidator{}.validate(ref);
        if (!report.ok()) {
            std::cout << "ok " << path << " (parsed; invalid model, not solved)\n";
            continue;
        }
        ref.sort_and_index();
        const lightfem::AnalysisResult result = lightfem::LinearElasticSolver{}.solve(ref);
        const std::string base = out + "/" + std::to_string(k);
        lightfem::write_vtk(ref, result, base + "_ref.vtk");
        lightfem_gpu::write_vtk(ref, result, base + "_gpu.vtk", threads);
        const auto rp = lightfem::write_csv_results(ref, result, base + "_ref");
        const auto gp = lightfem_gpu::write_csv_results(ref, result, base + "_gpu", threads);
        if (slurp(base + "_ref.vtk") != slurp(base + "_gpu.vtk")) differ(path + ": VTK bytes");
        if (slurp(rp.nodes) != slurp(gp.first)) differ(path + ": nodes CSV bytes");
        if (slurp(rp.gauss_points) != slurp(gp.second)) differ(path + ": Gauss-point CSV bytes");
        std::cout << "ok " << path << " (" << ref.nodes.size() << " nodes, files identical)\n";
    }
    return failures == 0 ? 0 : 1;
}
