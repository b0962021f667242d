// Test driver of the C++ host layer (lightfem_gb300/host/lightfem_gpu_solve.hpp),
// over the mirror types of mirror_model.hpp.
//
//   solve_model <model.txt> <out_dir> [--no-index]
//
// Reads a model in the line format below, indexes it (Model::sort_and_index)
// unless --no-index, runs lightfem_gpu::solve on device 0 and writes into
// out_dir:
//   outcome.txt   "converged", or the exception kind (invalid_argument,
//                 logic_error, runtime_error), a tab and its message
//   report.txt    "key value" lines of LinearSolverReport and PerformanceReport
//   *.bin         raw little-endian arrays: node_ids (int64, index order),
//                 u, R, f, K (double), row_offsets, columns (uint64),
//                 element_fields (double, 35 per element), node_stress (4 per node)
//
// Model lines (numbers as printed by Python's repr, so they round-trip exactly):
//   setting <name> <value>
//   node <id> <x> <y>
//   material <id> <E> <nu> <t>
//   q4 <id> <n1> <n2> <n3> <n4> <material>
//   truss <id> <n1> <n2> <material> <area>
//   fix <node> <ux|-> <uy|->
//   load <node> <fx> <fy>
//   body <element> <bx> <by>
//   edge <element> <side> <traction|pressure> <first> <second>
#include "mirror_model.hpp"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

namespace {

using namespace lightfem_gpu;

double num(const std::string& s) { return std::strtod(s.c_str(), nullptr); }

Model read_model(const char* path) {
    std::ifstream in(path);
    if (!in) throw std::runtime_error(std::string("cannot open ") + path);
    Model m;
    std::string line;
    while (std::getline(in, line)) {
        std::istringstream ls(line);
        std::string kind;
        if (!(ls >> kind)) continue;
        std::vector<std::string> a;
        for (std::string t; ls >> t;) a.push_back(t);
        const auto i = [&](std::size_t k) { return std::stoi(a.at(k)); };
        const auto d = [&](std::size_t k) { return num(a.at(k)); };
        if (kind == "setting") {
            auto& s = m.settings;
            const std::string& key = a.at(0);
            const std::string& v = a.at(1);
            if (key == "plane_mode") s.plane_mode = v == "strain" ? PlaneMode::PlaneStrain : PlaneMode::PlaneStress;
            else if (key == "solver") s.solver = v;
            else if (key == "tolerance") s.tolerance = num(v);
            else if (key == "max_iterations") s.max_iterations = std::stoul(v);
            else if (key == "reordering") s.reordering = v;
            else if (key == "assembly") s.assembly = v;
            else if (key == "storage") s.storage = v;
            else if (key == "preconditioner") s.preconditioner = v;
            else if (key == "subdomain_split") s.subdomain_split = v;
            else if (key == "subdomain_nodes") s.subdomain_nodes = std::stoul(v);
            else throw std::runtime_error("unknown setting " + key);
        } else if (kind == "node") {
            Node n;
            n.id = i(0);
            n.position = {d(1), d(2)};
            m.nodes.push_back(n);
        } else if (kind == "material") {
            m.materials.push_back({i(0), d(1), d(2), d(3)});
        } else if (kind == "q4") {
            m.elements.push_back({i(0), {{i(1), i(2), i(3), i(4)}}, i(5)});
        } else if (kind == "truss") {
            m.trusses.push_back({i(0), {{i(1), i(2)}}, i(3), d(4)});
        } else if (kind == "fix") {
            DirichletBC b;
            b.node_id = i(0);
            if (a.at(1) != "-") b.ux = d(1);
            if (a.at(2) != "-") b.uy = d(2);
            m.boundaries.push_back(b);
        } else if (kind == "load") {
            m.loads.push_back({i(0), d(1), d(2)});
        } else if (kind == "body") {
            m.body_forces.push_back({i(0), d(1), d(2)});
        } else if (kind == "edge") {
            const EdgeLoadType type = a.at(2) == "pressure" ? EdgeLoadType::Pressure : EdgeLoadType::Traction;
            m.edge_loads.push_back({i(0), i(1), type, d(3), d(4)});
        } else {
            throw std::runtime_error("unknown record " + kind);
        }
    }
    return m;
}

template <typename T>
void write_bin(const std::string& dir, const char* name, const std::vector<T>& v) {
    std::FILE* f = std::fopen((dir + "/" + name + ".bin").c_str(), "wb");
    if (f == nullptr) throw std::runtime_error(std::string("cannot write ") + name);
    if (!v.empty()) std::fwrite(v.data(), sizeof(T), v.size(), f);
    std::fclose(f);
}

void write_outcome(const std::string& dir, const std::string& text) {
    std::ofstream(dir + "/outcome.txt") << text;
}

void write_result(const std::string& dir, const Model& m, const AnalysisResult& r) {
    std::vector<int64_t> ids;
    for (const auto& n : m.nodes) ids.push_back(n.id);
    write_bin(dir, "node_ids", ids);
    write_bin(dir, "u", r.displacement);
    write_bin(dir, "R", r.reaction);
    write_bin(dir, "f", r.load);
    write_bin(dir, "K", r.stiffness.values);
    std::vector<uint64_t> rp(r.stiffness.row_offsets.begin(), r.stiffness.row_offsets.end());
    std::vector<uint64_t> col(r.stiffness.column_indices.begin(), r.stiffness.column_indices.end());
    write_bin(dir, "row_offsets", rp);
    write_bin(dir, "columns", col);
    std::vector<double> fields, stress;
    for (const auto& e : r.element_results) {
        const auto put = [&](const ElementField& f) {
            fields.insert(fields.end(), f.strain.begin(), f.strain.end());
            fields.insert(fields.end(), f.stress.begin(), f.stress.end());
            fields.push_back(f.von_mises);
        };
        put(e.field);
        for (const auto& g : e.gauss_points) put(g.field);
    }
    for (const auto& n : r.node_results) {
        stress.insert(stress.end(), n.stress.begin(), n.stress.end());
        stress.push_back(n.von_mises);
    }
    write_bin(dir, "element_fields", fields);
    write_bin(dir, "node_stress", stress);
    std::ofstream rep(dir + "/report.txt");
    rep.precision(17);
    const auto& s = r.solver;
    const auto& p = r.performance;
    rep << "converged " << s.converged << "\niterations " << s.iterations << "\ninitial_residual "
        << s.initial_residual << "\nfinal_residual " << s.final_residual << "\nmessage " << s.message
        << "\npreconditioner " << s.preconditioner << "\nstorage " << s.storage << "\nsolve_ms " << s.solve_ms
        << "\nmatrix_bytes_per_matvec " << s.matrix_bytes_per_matvec << "\nsubdomains " << s.subdomains
        << "\ncapture_ratio " << s.capture_ratio << "\nreordering " << p.reordering << "\nbefore_bandwidth "
        << p.before.bandwidth << "\nbefore_profile " << p.before.profile << "\nafter_bandwidth "
        << p.after.bandwidth << "\nafter_profile " << p.after.profile << "\nafter_nonzeros " << p.after.nonzeros
        << "\ncoloring_count " << p.coloring_count << "\nassembly " << p.assembly << "\ntotal_ms " << p.total_ms
        << "\n";
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <model.txt> <out_dir> [--no-index]\n", argv[0]);
        return 2;
    }
    const std::string dir = argv[2];
    const bool index = !(argc > 3 && std::string(argv[3]) == "--no-index");
    Model model = read_model(argv[1]);
    try {
        if (index) model.sort_and_index();
        AnalysisResult result;
        lightfem_gpu::solve(model, result, 0);
        write_result(dir, model, result);
        write_outcome(dir, "converged");
    } catch (const std::invalid_argument& e) {
        write_outcome(dir, std::string("invalid_argument\t") + e.what());
    } catch (const std::logic_error& e) {
        write_outcome(dir, std::string("logic_error\t") + e.what());
    } catch (const std::runtime_error& e) {
        write_outcome(dir, std::string("runtime_error\t") + e.what());
    }
    return 0;
}
