// openmps_gb300_main - the GB300 counterpart of OpenMps's executable (src/OpenMps/Main.cpp).
//
// Same input and output contract as the reference driver:
//   * input: an XML file <openmps> with <condition> (startTime, endTime, outputInterval,
//     eps), <environment> (l_0, minStepCountPerOutput, courant, g, rho, nu, r_eByl_0,
//     surfaceRatio, minX, minZ, maxX, maxZ) as value="..." attributes (Main.cpp:180-274)
//     and <particles type="csv"> holding CSV text with the header items Type, x, z, u, w,
//     p, n in any order (Main.cpp:63-170: spaces and tabs removed, blank lines skipped,
//     an unknown or missing header item is an error);
//   * output: result/particles_%05d.csv with the header "Type, x, z, u, w, p, n" and
//     default ostream formatting (Main.cpp:30-61), written at start and then every
//     outputInterval of simulated time, stepping with ForwardTime() (CFL time step, at
//     most outputInterval / minStepCountPerOutput) (Main.cpp:320-395);
//   * a Computer::Exception prints "!!!!ERROR!!!!" and stops the run (Main.cpp:380-388).
// With MPS_FLAG_PRESSURE_EXPLICIT among the flags, <environment> holds the sound speed c
// and <condition> needs no eps, as in the reference built with PRESSURE_EXPLICIT.
// A DIM3 input (minY < maxY in <environment>, or dim = 3) runs a three-dimensional
// scene: its CSV holds Type, x, y, z, u, v, w, p, n.
// Extensions (optional elements of <environment>): r_lapByl_0 (Laplacian radius),
// flags (method bit set, default the reference's stock set) and solver (cg64, mixed,
// mg, learned; default cg64 like the reference), weights (network file for "learned",
// raw FP32 blob).
// Usage: openmps_gb300_main [input.xml] [--parse-only]
#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/openmps_gb300.hpp"

namespace {

struct Xml {
    std::string text;

    // value="..." of the first <tag .../> inside <section>
    bool attr(const std::string& section, const std::string& tag, std::string* out) const {
        const size_t s0 = text.find("<" + section + ">");
        const size_t s1 = text.find("</" + section + ">");
        if (s0 == std::string::npos || s1 == std::string::npos) return false;
        size_t at = s0;
        const std::string open = "<" + tag;
        for (;;) {
            at = text.find(open, at);
            if (at == std::string::npos || at > s1) return false;
            const char c = text[at + open.size()];
            if (std::isspace(static_cast<unsigned char>(c)) || c == '/' || c == '>') break;
            at += open.size();
        }
        const size_t end = text.find('>', at);
        const size_t v = text.find("value=\"", at);
        if (v == std::string::npos || v > end) return false;
        const size_t q = text.find('"', v + 7);
        *out = text.substr(v + 7, q - (v + 7));
        return true;
    }
    double num(const std::string& section, const std::string& tag) const {
        std::string s;
        if (!attr(section, tag, &s)) throw std::runtime_error("missing " + section + "." + tag);
        return std::stod(s);
    }
    double num_or(const std::string& section, const std::string& tag, double dflt) const {
        std::string s;
        return attr(section, tag, &s) ? std::stod(s) : dflt;
    }
    // text content of <particles type="csv"> ... </particles>
    std::string particles_csv() const {
        const size_t a = text.find("<particles");
        if (a == std::string::npos) throw std::runtime_error("missing particles");
        const size_t gt = text.find('>', a);
        const std::string head = text.substr(a, gt - a);
        if (head.find("type=\"csv\"") == std::string::npos) throw std::runtime_error("Not Implemented!");
        const size_t b = text.find("</particles>", gt);
        return text.substr(gt + 1, b - gt - 1);
    }
};

std::vector<std::string> items(std::string line) {
    line.erase(std::remove_if(line.begin(), line.end(), [](char c) { return c == ' ' || c == '\t' || c == '\r'; }),
               line.end());
    std::vector<std::string> out;
    if (line.empty()) return out;
    std::stringstream ss(line);
    std::string it;
    while (std::getline(ss, it, ',')) out.push_back(it);
    if (!line.empty() && line.back() == ',') out.push_back("");
    return out;
}

// Particle columns of the CSV (y and v only in 3D).
struct Columns {
    std::vector<int32_t> type;
    std::vector<double> x, y, z, u, v, w, p, n;
};

// The header items Type, x, z, u, w, p, n (with y, v in 3D) in any order (Main.cpp:63-170).
Columns read_csv(const std::string& csv, int dim) {
    std::stringstream ss(csv);
    std::string line;
    std::vector<std::string> header;
    while (std::getline(ss, line)) {
        header = items(line);
        if (!header.empty()) break;
    }
    std::map<std::string, int> col = {{"Type", -1}, {"x", -1}, {"z", -1}, {"u", -1}, {"w", -1}, {"p", -1}, {"n", -1}};
    if (dim == 3) col.insert({{"y", -1}, {"v", -1}});
    for (size_t i = 0; i < header.size(); i++) {
        auto f = col.find(header[i]);
        if (f == col.end()) throw std::runtime_error("Illegal header item in input csv");
        f->second = static_cast<int>(i);
    }
    for (const auto& c : col)
        if (c.second < 0) throw std::runtime_error("Some header item doesn't exist");
    Columns out;
    while (std::getline(ss, line)) {
        const auto d = items(line);
        if (d.empty()) continue;
        out.type.push_back(static_cast<int32_t>(std::stoi(d.at(col["Type"]))));
        out.x.push_back(std::stod(d.at(col["x"])));
        out.z.push_back(std::stod(d.at(col["z"])));
        out.u.push_back(std::stod(d.at(col["u"])));
        out.w.push_back(std::stod(d.at(col["w"])));
        out.p.push_back(std::stod(d.at(col["p"])));
        out.n.push_back(std::stod(d.at(col["n"])));
        if (dim == 3) {
            out.y.push_back(std::stod(d.at(col["y"])));
            out.v.push_back(std::stod(d.at(col["v"])));
        }
    }
    std::cout << out.type.size() << " particles" << std::endl;
    return out;
}

void check_status(mps_handle* h, int rc) {
    if (rc != MPS_OK) throw openmps_gb300::Computer::Exception(rc, mps_last_error(h));
}

void add_columns(mps_handle* h, const Columns& c, int dim) {
    const int64_t n = static_cast<int64_t>(c.type.size());
    if (dim == 3)
        check_status(h, mps_add_particles3(h, n, c.type.data(), c.x.data(), c.y.data(), c.z.data(), c.u.data(),
                                           c.v.data(), c.w.data(), c.p.data(), c.n.data()));
    else
        check_status(h, mps_add_particles(h, n, c.type.data(), c.x.data(), c.z.data(), c.u.data(), c.w.data(),
                                          c.p.data(), c.n.data()));
}

// result/particles_%05d.csv with the reference's header and default ostream formatting
// (Main.cpp:30-61); returns the particles that are not disabled.
size_t write_csv(mps_handle* h, int dim, size_t count) {
    const int64_t n = mps_particle_count(h);
    Columns c;
    c.type.resize(static_cast<size_t>(n));
    for (auto* a : {&c.x, &c.y, &c.z, &c.u, &c.v, &c.w, &c.p, &c.n}) a->resize(static_cast<size_t>(n));
    if (dim == 3)
        check_status(h, mps_get_particles3(h, c.type.data(), c.x.data(), c.y.data(), c.z.data(), c.u.data(),
                                           c.v.data(), c.w.data(), c.p.data(), c.n.data()));
    else
        check_status(h, mps_get_particles(h, c.type.data(), c.x.data(), c.z.data(), c.u.data(), c.w.data(),
                                          c.p.data(), c.n.data()));
    char name[64];
    std::snprintf(name, sizeof(name), "result/particles_%05zu.csv", count);
    std::ofstream out(name);
    out << (dim == 3 ? "Type, x, y, z, u, v, w, p, n" : "Type, x, z, u, w, p, n") << std::endl;
    size_t alive = 0;
    for (size_t i = 0; i < static_cast<size_t>(n); i++) {
        out << c.type[i] << ", " << c.x[i] << ", ";
        if (dim == 3) out << c.y[i] << ", ";
        out << c.z[i] << ", " << c.u[i] << ", ";
        if (dim == 3) out << c.v[i] << ", ";
        out << c.w[i] << ", " << c.p[i] << ", " << c.n[i] << std::endl;
        if (c.type[i] != MPS_TYPE_DISABLED) alive++;
    }
    return alive;
}

int solver_code(const std::string& s) {
    if (s == "cg64") return MPS_SOLVER_CG64;
    if (s == "mixed") return MPS_SOLVER_MIXED;
    if (s == "mg") return MPS_SOLVER_MIXED_MG;
    if (s == "learned") return MPS_SOLVER_LEARNED;
    throw std::runtime_error("unknown solver " + s);
}

}  // namespace

int run(int argc, char** argv) {
    std::string file;
    bool parse_only = false;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        if (a == "--parse-only")
            parse_only = true;
        else
            file = a;
    }
    if (file.empty()) {
        std::cerr << "usage: openmps_gb300_main input.xml [--parse-only]" << std::endl;
        return 2;
    }
    std::cout << "Input XML file: " << file << std::endl;
    Xml xml;
    {
        std::ifstream in(file);
        if (!in) {
            std::cerr << "cannot read " << file << std::endl;
            return 2;
        }
        std::stringstream ss;
        ss << in.rdbuf();
        xml.text = ss.str();
    }
    const double start = xml.num("condition", "startTime");
    const double end = xml.num("condition", "endTime");
    const double interval = xml.num("condition", "outputInterval");
    const uint32_t flags = static_cast<uint32_t>(xml.num_or("environment", "flags", MPS_PRESET_REFERENCE));
    const bool explicit_pressure = (flags & MPS_FLAG_PRESSURE_EXPLICIT) != 0u;
    // with PRESSURE_EXPLICIT there is no eps and the sound speed c is read (Main.cpp:215-217, :263-265)
    const double eps = explicit_pressure ? xml.num_or("condition", "eps", 0.0) : xml.num("condition", "eps");
    const double steps_per_output = xml.num("environment", "minStepCountPerOutput");
    // the method set is read at run time, so the environment is built from mps_params
    // (the Environment(...) constructor takes the reference's compile-time argument list)
    mps_params prm;
    mps_default_params(&prm);
    prm.max_dt = interval / steps_per_output;
    prm.courant = xml.num("environment", "courant");
    prm.g = xml.num("environment", "g");
    prm.rho = xml.num("environment", "rho");
    prm.nu = xml.num("environment", "nu");
    prm.surface_ratio = xml.num_or("environment", "surfaceRatio", 0.97);
    prm.re_by_l0 = xml.num("environment", "r_eByl_0");
    prm.l0 = xml.num("environment", "l_0");
    prm.min_x = xml.num("environment", "minX");
    prm.min_z = xml.num("environment", "minZ");
    prm.max_x = xml.num("environment", "maxX");
    prm.max_z = xml.num("environment", "maxZ");
    prm.flags = flags;
    openmps_gb300::Environment env(prm);
    env.LaplacianRadius(xml.num_or("environment", "r_lapByl_0", 0.0));
    if (explicit_pressure) env.SoundSpeed(xml.num("environment", "c"));
    // A DIM3 input spans a y range (minY < maxY, Main.cpp:224-232); the reference's 2D
    // inputs may carry minY = maxY (Benchmark/Sample/Sample.xml), read only by DIM3 builds.
    const bool y_range = xml.num_or("environment", "maxY", 0.0) > xml.num_or("environment", "minY", 0.0);
    const int dim = static_cast<int>(xml.num_or("environment", "dim", y_range ? 3 : 2));
    if (dim == 3) {
        env.params.dim = 3;
        env.params.min_y = xml.num("environment", "minY");
        env.params.max_y = xml.num("environment", "maxY");
    }
    std::string solver = "cg64", weights;
    xml.attr("environment", "solver", &solver);
    xml.attr("environment", "weights", &weights);
    env.Solver(solver_code(solver));
    const Columns particles = read_csv(xml.particles_csv(), dim);
    if (parse_only) {
        const mps_params& p = env.params;
        std::printf("maxDt=%.17g courant=%.17g g=%.17g rho=%.17g nu=%.17g surfaceRatio=%.17g r_eByl_0=%.17g "
                    "l_0=%.17g min=(%.17g,%.17g) max=(%.17g,%.17g) flags=%u solver=%d eps=%.17g "
                    "start=%.17g end=%.17g interval=%.17g c=%.17g dim=%d minY=%.17g maxY=%.17g\n",
                    p.max_dt, p.courant, p.g, p.rho, p.nu, p.surface_ratio, p.re_by_l0, p.l0, p.min_x, p.min_z,
                    p.max_x, p.max_z, p.flags, p.solver, eps, start, end, interval, p.sound_speed, dim, p.min_y,
                    p.max_y);
        return 0;
    }
    mkdir("result", 0755);
    try {
        openmps_gb300::Computer computer(eps, env);
        if (solver == "learned") {
            std::ifstream w(weights, std::ios::binary);
            std::vector<float> blob(MPS_MLP_BLOB_FLOATS);
            if (!w.read(reinterpret_cast<char*>(blob.data()), sizeof(float) * blob.size()))
                throw std::runtime_error("cannot read weights " + weights);
            if (mps_learned_set_weights(computer.Handle(), blob.data(), MPS_MLP_BLOB_FLOATS) != MPS_OK)
                throw std::runtime_error(mps_last_error(computer.Handle()));
        }
        add_columns(computer.Handle(), particles, dim);
        const size_t offset = static_cast<size_t>(std::ceil(start / interval));
        size_t alive = write_csv(computer.Handle(), dim, offset);
        std::printf("#%05zu: t=%8.4f (%05d), %12zu particles\n", offset, start, 0, alive);
        double next = 0.0;
        size_t iteration = 0;
        const size_t end_count = static_cast<size_t>(std::ceil((end - start) / interval));
        for (size_t out = 1; out <= end_count; out++) {
            double t = computer.GetEnvironment().T();
            try {
                next += interval;
                while (t < next) {
                    computer.ForwardTime();
                    t = computer.GetEnvironment().T();
                    iteration++;
                }
                alive = write_csv(computer.Handle(), dim, out + offset);
                std::printf("#%05zu: t=%8.4f (%05zu), %12zu particles\n", out + offset, t + start, iteration, alive);
            } catch (const openmps_gb300::Computer::Exception& ex) {
                std::cout << "!!!!ERROR!!!!" << std::endl
                          << "#" << (out + offset) << ": t=" << t << " (" << iteration << ")" << std::endl
                          << ex.what() << std::endl;
                break;
            }
        }
    } catch (const std::exception& ex) {
        std::cerr << ex.what() << std::endl;
        return 1;
    }
    std::cout << "finished" << std::endl;
    return 0;
}

int main(int argc, char** argv) {
    try {
        return run(argc, argv);
    } catch (const std::exception& ex) {  // a malformed input (missing item, bad number)
        std::cerr << ex.what() << std::endl;
        return 1;
    }
}
