/*
 * lightfem_gpu_io.hpp — the reference host's text I/O on all host cores: the .fem
 * parser (InputParser, src/input_parser.cpp:162-341) and the VTK / CSV result
 * writers (write_vtk, write_csv_results, src/vtk_writer.cpp:110-337).
 * Header-only C++17 with std::thread; no device code.
 *
 * Same results as the reference's serial code, byte for byte:
 *  - parse_fem_text / parse_fem fill the host's own Model type (the reference's
 *    lightfem::Model, or any type with its members) with the same records in the
 *    same order, and fail with the same message ("source:line: message") at the
 *    same line: the first failing line of the file.  The text is cut into one
 *    piece per thread at line ends; each thread strips comments and blanks and
 *    classifies its lines, the section each piece starts in comes from the
 *    headers of the pieces before it, and each thread then converts its own data
 *    lines with the reference's conversions (std::stoll, std::stoull, std::stod)
 *    and checks.  [settings] lines are applied afterwards in file order, because
 *    a repeated key is an error of the later line.
 *  - write_vtk / write_csv_results format each block of records (the nodes, the
 *    cells, one field) in one piece per thread, each number through std::to_chars
 *    (shortest round-trip form) as the reference's writer does, and write the
 *    pieces in order.  With LIGHTFEM_LEGACY_EXPORT set, numbers take the
 *    reference's legacy form (17 significant digits, as std::ostream prints them).
 *
 * threads == 0 uses std::thread::hardware_concurrency().
 */
#pragma once

#include <algorithm>
#include <array>
#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <functional>
#include <iterator>
#include <limits>
#include <optional>
#include <sstream>
#include <stdexcept>
#include <string>
#include <system_error>
#include <thread>
#include <type_traits>
#include <unordered_set>
#include <utility>
#include <vector>

namespace lightfem_gpu {

// A parse failure: what() is "source:line: message", as the reference's ParseError.
class ParseError : public std::runtime_error {
public:
    ParseError(std::string source, std::size_t line, const std::string& message)
        : std::runtime_error(source + ":" + std::to_string(line) + ": " + message),
          source_(std::move(source)),
          line_(line) {}
    const std::string& source() const noexcept { return source_; }
    std::size_t line() const noexcept { return line_; }

private:
    std::string source_;
    std::size_t line_ = 0;
};

namespace io_detail {

inline unsigned thread_count(unsigned requested, std::size_t work) {
    unsigned t = requested ? requested : std::max(1u, std::thread::hardware_concurrency());
    if (requested == 0 && work < 4096) t = 1;  // small inputs: not worth a thread
    return std::max(1u, std::min<unsigned>(t, 256u));
}

// Runs body(k, begin, end) over [0, n) cut into `parts` contiguous ranges, one thread each.
template <typename F>
void parallel_ranges(std::size_t n, unsigned parts, F&& body) {
    if (parts <= 1 || n == 0) {
        body(0u, std::size_t{0}, n);
        return;
    }
    std::vector<std::thread> pool;
    pool.reserve(parts - 1);
    for (unsigned k = 1; k < parts; ++k)
        pool.emplace_back([&, k] { body(k, n * k / parts, n * (k + 1) / parts); });
    body(0u, std::size_t{0}, n / parts);
    for (auto& t : pool) t.join();
}

inline bool space(char c) { return std::isspace(static_cast<unsigned char>(c)) != 0; }

inline std::string lower(std::string v) {
    for (char& c : v) c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
    return v;
}

// ----------------------------------------------------------------------- parser
enum class Section { None, Settings, Nodes, Materials, Elements, Trusses, Boundary, Loads, BodyForces, EdgeLoads };

// A failure found by a thread: the earliest line wins.
struct Failure {
    std::size_t line = std::numeric_limits<std::size_t>::max();
    std::string message;
    void note(std::size_t l, std::string m) {
        if (l < line) {
            line = l;
            message = std::move(m);
        }
    }
    bool any() const { return line != std::numeric_limits<std::size_t>::max(); }
};

// Thrown inside a line's conversion and caught by the thread that parses it.
struct LineFailure {
    std::string message;
};

inline int to_int(const std::string& token, const char* field) {
    try {
        std::size_t used = 0;
        const long long v = std::stoll(token, &used);
        if (used != token.size() || v < std::numeric_limits<int>::min() || v > std::numeric_limits<int>::max())
            throw LineFailure{std::string("invalid integer for ") + field + ": " + token};
        return static_cast<int>(v);
    } catch (const std::invalid_argument&) {
        throw LineFailure{std::string("invalid integer for ") + field + ": " + token};
    } catch (const std::out_of_range&) {
        throw LineFailure{std::string("integer out of range for ") + field + ": " + token};
    }
}

inline std::size_t to_size(const std::string& token, const char* field) {
    try {
        std::size_t used = 0;
        const unsigned long long v = std::stoull(token, &used);
        if (used != token.size() || v > std::numeric_limits<std::size_t>::max())
            throw LineFailure{std::string("invalid non-negative integer for ") + field + ": " + token};
        return static_cast<std::size_t>(v);
    } catch (const std::invalid_argument&) {
        throw LineFailure{std::string("invalid non-negative integer for ") + field + ": " + token};
    } catch (const std::out_of_range&) {
        throw LineFailure{std::string("integer out of range for ") + field + ": " + token};
    }
}

inline double to_double(const std::string& token, const char* field) {
    try {
        std::size_t used = 0;
        const double v = std::stod(token, &used);
        if (used != token.size() || !std::isfinite(v))
            throw LineFailure{std::string("invalid finite number for ") + field + ": " + token};
        return v;
    } catch (const std::invalid_argument&) {
        throw LineFailure{std::string("invalid number for ") + field + ": " + token};
    } catch (const std::out_of_range&) {
        throw LineFailure{std::string("number out of range for ") + field + ": " + token};
    }
}

inline std::optional<double> to_constraint(const std::string& token, const char* field) {
    const std::string t = lower(token);
    if (t == "free" || t == "none" || t == "-") return std::nullopt;
    return to_double(token, field);
}

inline void need(const std::vector<std::string>& tokens, std::size_t n, const char* format) {
    if (tokens.size() != n)
        throw LineFailure{std::string("expected ") + std::to_string(n) + " fields (" + format + "), got " +
                          std::to_string(tokens.size())};
}

// Section of a header's inner text, or a failure message.
inline bool section_of(const std::string& inner, Section& out, std::string& message) {
    std::size_t b = 0, e = inner.size();
    while (b < e && space(inner[b])) ++b;
    while (e > b && space(inner[e - 1])) --e;
    const std::string s = lower(inner.substr(b, e - b));
    if (s == "settings") out = Section::Settings;
    else if (s == "nodes") out = Section::Nodes;
    else if (s == "materials") out = Section::Materials;
    else if (s == "elements") out = Section::Elements;
    else if (s == "trusses" || s == "bars" || s == "rods" || s == "members") out = Section::Trusses;
    else if (s == "boundary" || s == "boundaries" || s == "dirichlet") out = Section::Boundary;
    else if (s == "loads" || s == "forces") out = Section::Loads;
    else if (s == "body_forces" || s == "body_loads") out = Section::BodyForces;
    else if (s == "edge_loads" || s == "surface_loads" || s == "tractions" || s == "pressures") out = Section::EdgeLoads;
    else {
        message = "unknown section [" + s + "]";
        return false;
    }
    return true;
}

// A non-empty line after comment stripping and trimming.
struct Line {
    std::size_t number;  // 1-based, counted as std::getline counts
    std::size_t begin, end;
    bool header;
};

template <typename Model>
struct Records {
    decltype(Model{}.nodes) nodes;
    decltype(Model{}.materials) materials;
    decltype(Model{}.elements) elements;
    decltype(Model{}.trusses) trusses;
    decltype(Model{}.boundaries) boundaries;
    decltype(Model{}.loads) loads;
    decltype(Model{}.body_forces) body_forces;
    decltype(Model{}.edge_loads) edge_loads;
};

template <typename V>
void append(V& to, V& from) {
    to.insert(to.end(), std::make_move_iterator(from.begin()), std::make_move_iterator(from.end()));
}

inline std::vector<std::string> tokens_of(const std::string& text, std::size_t b, std::size_t e) {
    std::vector<std::string> out;
    std::size_t i = b;
    while (i < e) {
        while (i < e && space(text[i])) ++i;
        const std::size_t s = i;
        while (i < e && !space(text[i])) ++i;
        if (i > s) out.emplace_back(text, s, i - s);
    }
    return out;
}

// One data line of a record section into `r` (throws LineFailure).
template <typename Model>
void parse_record(Section section, const std::vector<std::string>& t, std::size_t line, Records<Model>& r) {
    using Node = typename decltype(Model{}.nodes)::value_type;
    using Material = typename decltype(Model{}.materials)::value_type;
    using Q4 = typename decltype(Model{}.elements)::value_type;
    using Truss = typename decltype(Model{}.trusses)::value_type;
    using BC = typename decltype(Model{}.boundaries)::value_type;
    using Load = typename decltype(Model{}.loads)::value_type;
    using Body = typename decltype(Model{}.body_forces)::value_type;
    using Edge = typename decltype(Model{}.edge_loads)::value_type;
    using EdgeType = decltype(Edge{}.type);
    switch (section) {
        case Section::Nodes: {
            need(t, 3, "id x y");
            Node n{};
            n.id = to_int(t[0], "node id");
            n.position.x = to_double(t[1], "x");
            n.position.y = to_double(t[2], "y");
            n.dof_x = n.dof_y = std::numeric_limits<std::size_t>::max();
            n.source_line = line;
            r.nodes.push_back(n);
            break;
        }
        case Section::Materials: {
            need(t, 4, "id E nu thickness");
            Material m{};
            m.id = to_int(t[0], "material id");
            m.young_modulus = to_double(t[1], "E");
            m.poisson_ratio = to_double(t[2], "nu");
            m.thickness = to_double(t[3], "thickness");
            m.source_line = line;
            r.materials.push_back(m);
            break;
        }
        case Section::Elements: {
            need(t, 6, "id n1 n2 n3 n4 material_id");
            Q4 q{};
            q.id = to_int(t[0], "element id");
            q.node_ids[0] = to_int(t[1], "n1");
            q.node_ids[1] = to_int(t[2], "n2");
            q.node_ids[2] = to_int(t[3], "n3");
            q.node_ids[3] = to_int(t[4], "n4");
            q.material_id = to_int(t[5], "material id");
            q.source_line = line;
            r.elements.push_back(q);
            break;
        }
        case Section::Trusses: {
            need(t, 5, "id n1 n2 material_id area");
            Truss b{};
            b.id = to_int(t[0], "truss id");
            b.node_ids[0] = to_int(t[1], "n1");
            b.node_ids[1] = to_int(t[2], "n2");
            b.material_id = to_int(t[3], "material id");
            b.area = to_double(t[4], "area");
            b.source_line = line;
            r.trusses.push_back(b);
            break;
        }
        case Section::Boundary: {
            BC bc{};
            bc.source_line = line;
            if (t.size() == 2) {
                const std::string type = lower(t[1]);
                bc.node_id = to_int(t[0], "boundary node id");
                if (type == "fixed" || type == "pinned") {
                    bc.ux = 0.0;
                    bc.uy = 0.0;
                } else if (type == "roller_x" || type == "symmetry_x") {
                    bc.ux = 0.0;
                } else if (type == "roller_y" || type == "symmetry_y") {
                    bc.uy = 0.0;
                } else {
                    throw LineFailure{
                        "boundary type must be fixed, pinned, roller_x, roller_y, symmetry_x, or symmetry_y"};
                }
            } else {
                need(t, 3, "node_id ux uy or node_id boundary_type");
                bc.node_id = to_int(t[0], "boundary node id");
                bc.ux = to_constraint(t[1], "ux");
                bc.uy = to_constraint(t[2], "uy");
            }
            r.boundaries.push_back(bc);
            break;
        }
        case Section::Loads: {
            need(t, 3, "node_id fx fy");
            Load l{};
            l.node_id = to_int(t[0], "load node id");
            l.fx = to_double(t[1], "fx");
            l.fy = to_double(t[2], "fy");
            l.source_line = line;
            r.loads.push_back(l);
            break;
        }
        case Section::BodyForces: {
            need(t, 3, "element_id bx by");
            Body b{};
            b.element_id = to_int(t[0], "element id");
            b.bx = to_double(t[1], "bx");
            b.by = to_double(t[2], "by");
            b.source_line = line;
            r.body_forces.push_back(b);
            break;
        }
        case Section::EdgeLoads: {
            if (t.size() < 4)
                throw LineFailure{
                    "expected edge load: element_id edge traction tx ty or element_id edge pressure p"};
            Edge e{};
            e.element_id = to_int(t[0], "element id");
            e.edge = to_int(t[1], "edge");
            const std::string type = lower(t[2]);
            if (type == "traction") {
                need(t, 5, "element_id edge traction tx ty");
                e.type = EdgeType::Traction;
                e.first = to_double(t[3], "tx");
                e.second = to_double(t[4], "ty");
            } else if (type == "pressure") {
                need(t, 4, "element_id edge pressure p");
                e.type = EdgeType::Pressure;
                e.first = to_double(t[3], "pressure");
                e.second = 0.0;
            } else {
                throw LineFailure{"edge load type must be traction or pressure"};
            }
            e.source_line = line;
            r.edge_loads.push_back(e);
            break;
        }
        default:
            break;
    }
}

// One [settings] line into the model (throws LineFailure).
template <typename Model>
void apply_setting(Model& m, const std::vector<std::string>& t, std::unordered_set<std::string>& seen) {
    need(t, 2, "key value");
    const std::string key = lower(t[0]);
    if (!seen.insert(key).second) throw LineFailure{"duplicate setting: " + key};
    auto& s = m.settings;
    using Mode = decltype(s.plane_mode);
    if (key == "plane_mode") {
        const std::string mode = lower(t[1]);
        if (mode == "plane_stress") s.plane_mode = Mode::PlaneStress;
        else if (mode == "plane_strain") s.plane_mode = Mode::PlaneStrain;
        else throw LineFailure{"plane_mode must be plane_stress or plane_strain"};
    } else if (key == "solver") {
        s.solver = lower(t[1]);
    } else if (key == "tolerance") {
        s.tolerance = to_double(t[1], "tolerance");
    } else if (key == "max_iterations") {
        s.max_iterations = to_size(t[1], "max_iterations");
    } else if (key == "reordering") {
        s.reordering = lower(t[1]);
    } else if (key == "assembly") {
        s.assembly = lower(t[1]);
    } else if (key == "threads") {
        s.threads = to_size(t[1], "threads");
    } else if (key == "storage") {
        s.storage = lower(t[1]);
    } else if (key == "preconditioner") {
        s.preconditioner = lower(t[1]);
    } else if (key == "subdomain_split") {
        s.subdomain_split = lower(t[1]);
    } else if (key == "subdomain_nodes") {
        s.subdomain_nodes = to_size(t[1], "subdomain_nodes");
    } else if (key == "output") {
        s.output_file = t[1];
    } else if (key == "deformation_scale") {
        s.deformation_scale = to_double(t[1], "deformation_scale");
    } else if (key == "csv_prefix") {
        s.csv_prefix = t[1];
    } else {
        throw LineFailure{"unknown setting: " + key};
    }
}

// ------------------------------------------------------------------------ writers
inline bool legacy_export() {
    const char* v = std::getenv("LIGHTFEM_LEGACY_EXPORT");
    return v != nullptr && v[0] != '\0' && v[0] != '0';
}

// Text of one piece of a file, formatted the reference writer's way.
struct Text {
    std::string s;
    bool legacy = false;
    void text(const char* v) { s += v; }
    void ch(char c) { s += c; }
    template <typename I>
    void integer(I v) {
        char buf[24];
        const auto r = std::to_chars(buf, buf + sizeof buf, static_cast<long long>(v));
        s.append(buf, r.ptr);
    }
    void real(double v) {
        char buf[40];
        if (legacy) {
            std::ostringstream o;
            o.precision(17);
            o << v;
            s += o.str();
            return;
        }
        const auto r = std::to_chars(buf, buf + sizeof buf, v);
        if (r.ec != std::errc{}) throw std::runtime_error("failed to format a number");
        s.append(buf, r.ptr);
    }
};

// A file written block by block; each block's records are formatted in parallel pieces.
class BlockFile {
public:
    BlockFile(const std::string& path, unsigned threads)
        : path_(path), out_(std::fopen(path.c_str(), "wb")), threads_(threads), legacy_(legacy_export()) {
        if (!out_) throw std::runtime_error("cannot open output file: " + path);
    }
    ~BlockFile() {
        if (out_) std::fclose(out_);
    }
    BlockFile(const BlockFile&) = delete;
    BlockFile& operator=(const BlockFile&) = delete;

    // A fixed piece of text.
    void head(const std::function<void(Text&)>& f) {
        Text t;
        t.legacy = legacy_;
        f(t);
        put(t.s);
    }
    // n records, record(i, text) for each, formatted in parallel pieces and written in order.
    template <typename F>
    void records(std::size_t n, F&& record) {
        const unsigned parts = thread_count(threads_, n);
        std::vector<std::string> pieces(parts);
        parallel_ranges(n, parts, [&](unsigned k, std::size_t b, std::size_t e) {
            Text t;
            t.legacy = legacy_;
            t.s.reserve((e - b) * 24);
            for (std::size_t i = b; i < e; ++i) record(i, t);
            pieces[k] = std::move(t.s);
        });
        for (const std::string& p : pieces) put(p);
    }
    void finish() {
        if (std::fflush(out_) != 0 || std::ferror(out_)) throw std::runtime_error("failed while writing " + path_);
        const int rc = std::fclose(out_);
        out_ = nullptr;
        if (rc != 0) throw std::runtime_error("failed while closing " + path_);
    }

private:
    void put(const std::string& s) {
        if (!s.empty() && std::fwrite(s.data(), 1, s.size(), out_) != s.size())
            throw std::runtime_error("failed while writing " + path_);
    }
    std::string path_;
    std::FILE* out_;
    unsigned threads_;
    bool legacy_;
};

}  // namespace io_detail

// Parses .fem text (the reference's InputParser::parse, src/input_parser.cpp:162-341).
template <typename Model>
Model parse_fem_text(const std::string& text, const std::string& source_name, unsigned threads = 0) {
    using namespace io_detail;
    Model model;
    model.source_name = source_name;
    // Cut at line ends into one piece per thread.
    const unsigned parts = thread_count(threads, text.size() / 64);
    std::vector<std::size_t> cut(parts + 1, text.size());
    cut[0] = 0;
    for (unsigned k = 1; k < parts; ++k) {
        std::size_t c = std::max(cut[k - 1], text.size() * k / parts);
        while (c < text.size() && c > 0 && text[c - 1] != '\n') ++c;
        cut[k] = c;
    }
    // Pass 1, per piece: the non-empty lines and their kind; line counts per piece.
    std::vector<std::vector<Line>> lines(parts);
    std::vector<std::size_t> counted(parts, 0);
    parallel_ranges(parts, parts, [&](unsigned, std::size_t kb, std::size_t ke) {
        for (std::size_t k = kb; k < ke; ++k) {
            std::size_t i = cut[k], local = 0;
            while (i < cut[k + 1]) {
                std::size_t e = text.find('\n', i);
                if (e == std::string::npos || e > cut[k + 1]) e = cut[k + 1];
                ++local;
                // The comment starts at the line's first '#' (searched within the line only).
                const std::size_t stop0 =
                    static_cast<std::size_t>(std::find(text.begin() + static_cast<std::ptrdiff_t>(i),
                                                       text.begin() + static_cast<std::ptrdiff_t>(e), '#') -
                                             text.begin());
                std::size_t stop = stop0;
                std::size_t b = i;
                while (b < stop && space(text[b])) ++b;
                while (stop > b && space(text[stop - 1])) --stop;
                if (stop > b) lines[k].push_back(Line{local, b, stop, text[b] == '['});
                i = e + 1;
            }
            counted[k] = local;
        }
    });
    std::size_t base = 0;
    for (unsigned k = 0; k < parts; ++k) {
        for (Line& l : lines[k]) l.number += base;
        base += counted[k];
    }
    // The section each piece starts in, from the headers of the pieces before it.
    Failure failure;
    std::vector<Section> start(parts, Section::None);
    Section current = Section::None;
    for (unsigned k = 0; k < parts; ++k) {
        start[k] = current;
        for (const Line& l : lines[k]) {
            if (!l.header) continue;
            Section s;
            std::string message;
            if (text[l.end - 1] != ']') failure.note(l.number, "section header must end with ']'");
            else if (section_of(text.substr(l.begin + 1, l.end - l.begin - 2), s, message)) current = s;
            else failure.note(l.number, message);
            if (failure.any()) break;
        }
        if (failure.any()) break;
    }
    // Pass 2, per piece: the records; [settings] lines are kept for the ordered pass.
    std::vector<Records<Model>> records(parts);
    std::vector<Failure> failures(parts);
    std::vector<std::vector<const Line*>> settings(parts);
    parallel_ranges(parts, parts, [&](unsigned, std::size_t kb, std::size_t ke) {
        for (std::size_t k = kb; k < ke; ++k) {
            Section section = start[k];
            for (const Line& l : lines[k]) {
                if (l.header) {
                    Section s;
                    std::string message;
                    if (text[l.end - 1] != ']' ||
                        !section_of(text.substr(l.begin + 1, l.end - l.begin - 2), s, message))
                        break;  // the header's failure is in `failure`; nothing after it counts
                    section = s;
                    continue;
                }
                if (section == Section::None) {
                    failures[k].note(l.number, "data appears before the first section header");
                    break;
                }
                if (section == Section::Settings) {
                    settings[k].push_back(&l);
                    continue;
                }
                try {
                    parse_record<Model>(section, tokens_of(text, l.begin, l.end), l.number, records[k]);
                } catch (const LineFailure& f) {
                    failures[k].note(l.number, f.message);
                    break;
                }
            }
        }
    });
    for (const Failure& f : failures) failure.note(f.line, f.message);
    // Settings in file order, up to the first failure.
    std::unordered_set<std::string> seen;
    for (unsigned k = 0; k < parts; ++k) {
        for (const Line* l : settings[k]) {
            if (l->number > failure.line) break;
            try {
                apply_setting(model, tokens_of(text, l->begin, l->end), seen);
            } catch (const LineFailure& f) {
                failure.note(l->number, f.message);
                break;
            }
        }
    }
    if (failure.any()) throw ParseError(source_name, failure.line, failure.message);
    for (auto& r : records) {
        append(model.nodes, r.nodes);
        append(model.materials, r.materials);
        append(model.elements, r.elements);
        append(model.trusses, r.trusses);
        append(model.boundaries, r.boundaries);
        append(model.loads, r.loads);
        append(model.body_forces, r.body_forces);
        append(model.edge_loads, r.edge_loads);
    }
    return model;
}

// Parses a .fem file (InputParser::parse_file, src/input_parser.cpp:154-160).
template <typename Model>
Model parse_fem(const std::string& path, unsigned threads = 0) {
    std::ifstream in(path, std::ios::binary);
    if (!in) throw ParseError(path, 0, "cannot open input file");
    std::string text((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>());
    return parse_fem_text<Model>(text, path, threads);
}

// The VTK result file (write_vtk, src/vtk_writer.cpp:110-264).
template <typename Model, typename Result>
void write_vtk(const Model& model, const Result& result, const std::string& path, unsigned threads = 0) {
    if (!model.is_indexed()) throw std::logic_error("model must be indexed before VTK export");
    const std::size_t dofs = model.summary().dofs;
    if (result.displacement.size() != dofs)
        throw std::invalid_argument("VTK displacement size does not match model DOFs");
    if (result.reaction.size() != dofs) throw std::invalid_argument("VTK reaction size does not match model DOFs");
    const std::size_t cells = model.elements.size() + model.trusses.size();
    if (result.element_results.size() != cells)
        throw std::invalid_argument("VTK element result count does not match model elements");
    if (result.node_results.size() != model.nodes.size())
        throw std::invalid_argument("VTK nodal result count does not match model nodes");
    // Node indices of every cell, resolved before the parallel blocks (a missing
    // node is the reference's logic_error).
    std::vector<std::size_t> q4(4 * model.elements.size()), bars(2 * model.trusses.size());
    for (std::size_t e = 0; e < model.elements.size(); ++e)
        for (int a = 0; a < 4; ++a) {
            const auto* node = model.find_node(model.elements[e].node_ids[a]);
            if (node == nullptr) throw std::logic_error("validated element references an unknown node");
            q4[4 * e + a] = node->dof_x / 2;
        }
    for (std::size_t e = 0; e < model.trusses.size(); ++e)
        for (int a = 0; a < 2; ++a) {
            const auto* node = model.find_node(model.trusses[e].node_ids[a]);
            if (node == nullptr) throw std::logic_error("validated truss references an unknown node");
            bars[2 * e + a] = node->dof_x / 2;
        }
    const auto& u = result.displacement;
    const auto& R = result.reaction;
    const double scale = model.settings.deformation_scale;
    const std::size_t nn = model.nodes.size(), ne = model.elements.size(), nt = model.trusses.size();
    using io_detail::Text;
    io_detail::BlockFile f(path, threads);
    f.head([&](Text& t) {
        t.text("# vtk DataFile Version 3.0\nLightFEM linear static Q4 result\nASCII\nDATASET UNSTRUCTURED_GRID\n");
        t.text("POINTS ");
        t.integer(nn);
        t.text(" double\n");
    });
    f.records(nn, [&](std::size_t i, Text& t) {
        const auto& n = model.nodes[i];
        t.real(n.position.x + scale * u[n.dof_x]);
        t.ch(' ');
        t.real(n.position.y + scale * u[n.dof_y]);
        t.text(" 0\n");
    });
    f.head([&](Text& t) {
        t.text("CELLS ");
        t.integer(cells);
        t.ch(' ');
        t.integer(5 * ne + 3 * nt);
        t.ch('\n');
    });
    f.records(ne, [&](std::size_t e, Text& t) {
        t.ch('4');
        for (int a = 0; a < 4; ++a) {
            t.ch(' ');
            t.integer(q4[4 * e + a]);
        }
        t.ch('\n');
    });
    f.records(nt, [&](std::size_t e, Text& t) {
        t.ch('2');
        for (int a = 0; a < 2; ++a) {
            t.ch(' ');
            t.integer(bars[2 * e + a]);
        }
        t.ch('\n');
    });
    f.head([&](Text& t) {
        t.text("CELL_TYPES ");
        t.integer(cells);
        t.ch('\n');
    });
    f.records(ne, [&](std::size_t, Text& t) { t.text("9\n"); });  // VTK_QUAD
    f.records(nt, [&](std::size_t, Text& t) { t.text("3\n"); });  // VTK_LINE
    f.head([&](Text& t) {
        t.text("POINT_DATA ");
        t.integer(nn);
        t.text("\nVECTORS displacement double\n");
    });
    auto node_vector = [&](const std::vector<double>& v) {
        f.records(nn, [&](std::size_t i, Text& t) {
            const auto& n = model.nodes[i];
            t.real(v[n.dof_x]);
            t.ch(' ');
            t.real(v[n.dof_y]);
            t.text(" 0\n");
        });
    };
    node_vector(u);
    const std::array<const char*, 3> nodal{{"nodal_stress_xx", "nodal_stress_yy", "nodal_stress_xy"}};
    for (std::size_t c = 0; c < 3; ++c) {
        f.head([&](Text& t) {
            t.text("SCALARS ");
            t.text(nodal[c]);
            t.text(" double 1\nLOOKUP_TABLE default\n");
        });
        f.records(nn, [&](std::size_t i, Text& t) {
            t.real(result.node_results[i].stress[c]);
            t.ch('\n');
        });
    }
    f.head([&](Text& t) { t.text("SCALARS nodal_von_mises_in_plane double 1\nLOOKUP_TABLE default\n"); });
    f.records(nn, [&](std::size_t i, Text& t) {
        t.real(result.node_results[i].von_mises);
        t.ch('\n');
    });
    f.head([&](Text& t) { t.text("VECTORS reaction double\n"); });
    node_vector(R);
    f.head([&](Text& t) { t.text("SCALARS displacement_magnitude double 1\nLOOKUP_TABLE default\n"); });
    f.records(nn, [&](std::size_t i, Text& t) {
        const auto& n = model.nodes[i];
        t.real(std::hypot(u[n.dof_x], u[n.dof_y]));
        t.ch('\n');
    });
    const auto& er = result.element_results;
    f.head([&](Text& t) {
        t.text("CELL_DATA ");
        t.integer(cells);
        t.text("\nSCALARS element_id int 1\nLOOKUP_TABLE default\n");
    });
    f.records(cells, [&](std::size_t e, Text& t) {
        t.integer(er[e].element_id);
        t.ch('\n');
    });
    const std::array<const char*, 3> strain{{"strain_xx", "strain_yy", "strain_xy"}};
    const std::array<const char*, 3> stress{{"stress_xx", "stress_yy", "stress_xy"}};
    auto cell_scalar = [&](const std::string& name, auto&& value) {
        f.head([&](Text& t) {
            t.text("SCALARS ");
            t.text(name.c_str());
            t.text(" double 1\nLOOKUP_TABLE default\n");
        });
        f.records(cells, [&](std::size_t e, Text& t) {
            t.real(value(er[e]));
            t.ch('\n');
        });
    };
    for (std::size_t c = 0; c < 3; ++c) cell_scalar(strain[c], [c](const auto& x) { return x.field.strain[c]; });
    for (std::size_t c = 0; c < 3; ++c) cell_scalar(stress[c], [c](const auto& x) { return x.field.stress[c]; });
    cell_scalar("von_mises_in_plane", [](const auto& x) { return x.field.von_mises; });
    for (std::size_t gp = 0; gp < 4; ++gp) {
        for (std::size_t c = 0; c < 3; ++c)
            cell_scalar(std::string(stress[c]) + "_gp" + std::to_string(gp + 1),
                        [gp, c](const auto& x) { return x.gauss_points[gp].field.stress[c]; });
        cell_scalar("von_mises_gp" + std::to_string(gp + 1),
                    [gp](const auto& x) { return x.gauss_points[gp].field.von_mises; });
    }
    f.finish();
}

// The two CSV result files (write_csv_results, src/vtk_writer.cpp:266-337); returns
// the node and Gauss-point file names.
template <typename Model, typename Result>
std::pair<std::string, std::string> write_csv_results(const Model& model, const Result& result,
                                                      const std::string& prefix, unsigned threads = 0) {
    if (!model.is_indexed()) throw std::logic_error("model must be indexed before CSV export");
    if (prefix.empty()) throw std::invalid_argument("CSV prefix must not be empty");
    const std::size_t dofs = model.summary().dofs;
    if (result.displacement.size() != dofs)
        throw std::invalid_argument("VTK displacement size does not match model DOFs");
    if (result.reaction.size() != dofs) throw std::invalid_argument("VTK reaction size does not match model DOFs");
    if (result.node_results.size() != model.nodes.size() ||
        result.element_results.size() != model.elements.size() + model.trusses.size())
        throw std::invalid_argument("CSV result count does not match model");
    std::pair<std::string, std::string> paths{prefix + "_nodes.csv", prefix + "_gauss_points.csv"};
    using io_detail::Text;
    const auto& u = result.displacement;
    const auto& R = result.reaction;
    const double scale = model.settings.deformation_scale;
    {
        io_detail::BlockFile f(paths.first, threads);
        f.head([](Text& t) {
            t.text("node_id,x,y,deformed_x,deformed_y,ux,uy,reaction_x,reaction_y,stress_xx,stress_yy,stress_xy,"
                   "von_mises\n");
        });
        f.records(model.nodes.size(), [&](std::size_t i, Text& t) {
            const auto& n = model.nodes[i];
            const auto& field = result.node_results[i];
            t.integer(n.id);
            for (double v : {n.position.x, n.position.y, n.position.x + scale * u[n.dof_x],
                             n.position.y + scale * u[n.dof_y], u[n.dof_x], u[n.dof_y], R[n.dof_x], R[n.dof_y],
                             field.stress[0], field.stress[1], field.stress[2], field.von_mises}) {
                t.ch(',');
                t.real(v);
            }
            t.ch('\n');
        });
        f.finish();
    }
    {
        io_detail::BlockFile f(paths.second, threads);
        f.head([](Text& t) {
            t.text("element_id,gauss_point,xi,eta,strain_xx,strain_yy,strain_xy,stress_xx,stress_yy,stress_xy,"
                   "von_mises\n");
        });
        f.records(result.element_results.size(), [&](std::size_t e, Text& t) {
            const auto& el = result.element_results[e];
            for (std::size_t gp = 0; gp < 4; ++gp) {
                const auto& p = el.gauss_points[gp];
                t.integer(el.element_id);
                t.ch(',');
                t.integer(gp + 1);
                for (double v : {p.xi, p.eta, p.field.strain[0], p.field.strain[1], p.field.strain[2],
                                 p.field.stress[0], p.field.stress[1], p.field.stress[2], p.field.von_mises}) {
                    t.ch(',');
                    t.real(v);
                }
                t.ch('\n');
            }
        });
        f.finish();
    }
    return paths;
}

}  // namespace lightfem_gpu
