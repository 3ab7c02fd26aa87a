// shoccs -- the command line of the reference (src/app/shoccs.cpp) over the sm_103a library.
//
//   shoccs [--check] [--script "<lua>"] <input-file.lua>
//
// Runs the Lua input file (and then the --script text, whose assignments take precedence),
// reads the global table `simulation` section by section as the reference's from_lua
// readers do, and runs the simulation cycle on the GPU: the system log goes to
// <logging_dir>/system.csv (header line, then one line per step) and geometry.csv (the cut
// points, src/mesh/mesh.cpp:139-151), the field dumps to the io
// table's directory, the progress messages to standard output.  --check stops after the Lua
// has run, as the reference does.  As in the reference, a section that cannot be read is
// reported and the program still exits 0; a Lua error exits non-zero.
//
// Readers (reference file:line):
//   simulation.mesh            cartesian::from_lua          src/mesh/cartesian.cpp:47-100
//   simulation.shapes          object_geometry::from_lua    src/mesh/object_geometry.cpp:239-300
//                              (spheres; other shape types are rejected)
//   simulation.domain_boundaries, shapes[i].boundary_condition
//                              bcs::from_lua                src/operators/boundaries.cpp:7-90
//   simulation.scheme          stencil::from_lua            src/stencils/stencil.cpp:8-106
//                              (E2 / E4 second-derivative, E4 / E4u / E6u / E8u / E2-poly
//                              first-derivative)
//   simulation.system          system::from_lua, heat::from_lua, scalar_wave::from_lua
//                              src/systems/system.cpp:103-132, heat.cpp:78-104,
//                              scalar_wave.cpp:134-193
//   simulation.manufactured_solution
//                              manufactured_solution::from_lua  src/mms/mms.cpp:34-98
//   simulation.integrator      integrator::from_lua         src/temporal/integrator.cpp:27-49
//                              (rk4, euler for FP64 systems; none: the empty integrator)
//   simulation.step_controller step_controller::from_lua    src/temporal/step_controller.cpp:7-29
//   simulation.io              field_io::from_lua           src/io/field_io.cpp:71-103
//   simulation.logging, logging_dir
//                              simulation_cycle::from_lua   src/simulation/simulation_cycle.cpp:145-162
//
// Manufactured solutions: the reference's "gaussian" (terms {center, variance, amplitude,
// frequency} in the table's array part; FP64 heat systems) is evaluated on the device; its
// "lua" kind (Lua functions evaluated at every point for every stage) is not available.  A heat system without
// a manufactured solution uses the zero solution (homogeneous Dirichlet data, no source),
// where the reference requires one.
//
// Extensions (keys the reference does not read): system.precision = "fp64" (default) or
// "mixed" selects the arithmetic of the time stepping; manufactured_solution.type =
// "sinsin" with frequency = k is the closed form prod_d sin(2 pi k x_d) e^-t.
#include "lua_subset.hpp"
#include "shoccs_gb300.hpp"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <iostream>
#include <limits>
#include <optional>
#include <string>
#include <variant>

namespace
{
using namespace ccs;
using lua::value;

// ---- sol-style access: t[key], get_or ----------------------------------------------------
value at(const value& t, const char* key)
{
    auto tb = t.tbl();
    return tb ? tb->get(key) : value{};
}
value at(const value& t, long long i)
{
    auto tb = t.tbl();
    return tb ? tb->get(i) : value{};
}
bool valid(const value& v) { return !v.is_nil(); }
real num_or(const value& v, real d) { return v.number() ? *v.number() : d; }
int int_or(const value& v, int d) { return v.number() ? (int)*v.number() : d; }
std::string str_or(const value& v, const std::string& d) { return v.string() ? *v.string() : d; }
bool bool_or(const value& v, bool d) { return v.boolean() ? *v.boolean() : d; }

// the builder's messages (the reference's "builder" console logger)
struct logger {
    bool enable = true;
    void info(const std::string& m) const
    {
        if (enable) std::cout << "[builder] [info] " << m << "\n";
    }
    void warn(const std::string& m) const
    {
        if (enable) std::cout << "[builder] [warning] " << m << "\n";
    }
    void err(const std::string& m) const { std::cerr << "[builder] [error] " << m << "\n"; }
};

// ---- mesh: cartesian::from_lua + object_geometry::from_lua ---------------------------------
std::optional<mesh> read_mesh(const value& sim, const logger& log)
{
    const value m = at(sim, "mesh");
    if (!valid(m)) {
        log.err("simulation.mesh is required");
        return std::nullopt;
    }
    const value ie = at(m, "index_extents");
    if (!valid(ie)) {
        log.err("simulation.mesh.index_extents is required");
        return std::nullopt;
    }
    const value db = at(m, "domain_bounds");
    if (!valid(db)) {
        log.err("simulation.mesh.domain_bounds is required");
        return std::nullopt;
    }
    const int3 n{int_or(at(ie, 1), 1), int_or(at(ie, 2), 1), int_or(at(ie, 3), 1)};
    real3 lb{}, ub{};
    if (const value x = at(db, "min"); valid(x)) {
        lb = {num_or(at(x, 1), 0.0), num_or(at(x, 2), 0.0), num_or(at(x, 3), 0.0)};
    } else {
        log.info("No explicit domain lower bound set.  Assuming (0, 0, 0)");
    }
    if (const value x = at(db, "max"); valid(x)) {
        ub = {num_or(at(x, 1), lb[0]), num_or(at(x, 2), lb[1]), num_or(at(x, 3), lb[2])};
    } else if (valid(at(db, 1))) {
        ub = {num_or(at(db, 1), lb[0]), num_or(at(db, 2), lb[1]), num_or(at(db, 3), lb[2])};
    } else {
        log.err("domain_bounds.max = {...} or domain_bounds = {...} must be specified");
        return std::nullopt;
    }
    std::vector<shape> shapes;
    const value t = at(sim, "shapes");
    if (!valid(t)) log.info("No cut-cell shapes specified");
    for (long long i = 1; valid(at(t, i)); i++) {
        const value s = at(t, i);
        const std::string type = str_or(at(s, "type"), "");
        if (type != "sphere") {
            log.err("shape type '" + type + "' is not supported (spheres only)");
            return std::nullopt;
        }
        const value c = at(s, "center");
        const real3 center{num_or(at(c, 1), 0.0), num_or(at(c, 2), 0.0), num_or(at(c, 3), 0.0)};
        shapes.push_back(make_sphere((int)shapes.size(), center, num_or(at(s, "radius"), 0.0)));
    }
    return mesh{index_extents{n}, domain_extents{lb, ub}, shapes};
}

// ---- boundary conditions: bcs::from_lua -----------------------------------------------------
// get_bc: a missing side is Floating; Dirichlet / Neumann on an axis of one point is Floating
std::optional<bcs::type> get_bc(const value& tbl, const char* side, const logger& log, int n = 0)
{
    const value bc = at(tbl, side);
    if (!valid(bc)) return bcs::Floating;
    const std::string t = str_or(bc, "");
    auto check = [&](bcs::type success) {
        if (n == 1) {
            log.warn(std::string("ignoring bc specification on side ") + side + " due to domain extents.");
            return bcs::Floating;
        }
        return success;
    };
    if (t == "dirichlet") return check(bcs::Dirichlet);
    if (t == "floating") return bcs::Floating;
    if (t == "neumann") return check(bcs::Neumann);
    log.err("incorrect boundary condition");
    return std::nullopt;
}

std::optional<std::pair<bcs::Grid, bcs::Object>> read_bcs(const value& sim, const int3& ex, const logger& log)
{
    bcs::Grid g{bcs::ff, bcs::ff, bcs::ff};
    bcs::Object o;
    if (const value m = at(sim, "domain_boundaries"); valid(m)) {
        const char* sides[6] = {"xmin", "xmax", "ymin", "ymax", "zmin", "zmax"};
        for (int k = 0; k < 6; k++) {
            const auto d = get_bc(m, sides[k], log, ex[k / 2]);
            if (!d) return std::nullopt;
            (k % 2 ? g[k / 2].right : g[k / 2].left) = *d;
        }
    }
    const value m = at(sim, "shapes");
    for (long long i = 1; valid(at(m, i)); i++) {
        const auto d = get_bc(at(m, i), "boundary_condition", log);
        if (!d) return std::nullopt;
        o.push_back(*d);
    }
    return std::pair{g, o};
}

// a number as fmt's "{}" prints it (shortest representation that reads back the same)
std::string fmt_real(real v)
{
    char buf[40];
    for (int prec = 1; prec <= 17; prec++) {
        std::snprintf(buf, sizeof buf, "%.*g", prec, v);
        if (std::strtod(buf, nullptr) == v) break;
    }
    return buf;
}

// ---- scheme: stencil::from_lua ---------------------------------------------------------------
std::optional<stencil> read_stencil(const value& sim, const logger& log)
{
    const value m = at(sim, "scheme");
    if (!valid(m)) {
        log.err("simulation.scheme must be specified");
        return std::nullopt;
    }
    // the numeric arrays scheme.alpha, floating_alpha, dirichlet_alpha, interpolant_alpha
    // (stencil.cpp:10-30: read_alpha)
    auto read_alpha = [&](const char* key) {
        std::vector<real> a;
        if (const value as = at(m, key); valid(as))
            for (long long i = 1; valid(at(as, i)); ++i) {
                if (!at(as, i).number())
                    throw lua::error(std::string("scheme.") + key + " must hold numbers");
                a.push_back(*at(as, i).number());
            }
        return a;
    };
    std::vector<real> alpha = read_alpha("alpha");
    const int order = int_or(at(m, "order"), 1);
    const std::string type = str_or(at(m, "type"), "");
    if (order == 2 && type == "E2") {
        log.info("E2 scheme chosen");
        return stencils::make_E2_2();
    }
    if (order == 2 && type == "E4") {
        log.info("E4 scheme chosen");
        return stencils::make_E4_2();
    }
    if (order == 1 && type == "E4") {
        log.info("E4 cut-cell first scheme chosen");
        // copy_zero_padded semantics for short alpha arrays; throws std::invalid_argument
        // for alpha[1] < 197/288 as the reference's make_E4_1 does
        std::vector<real> a = alpha;
        a.resize(std::max<std::size_t>(a.size(), 2), 0.0);
        return stencils::make_E4_1(a);
    }
    if (order == 1 && type == "E4u") {
        log.info("E4 uniform first scheme chosen");
        return stencils::make_E4u_1(alpha);
    }
    if (order == 1 && type == "E2-poly") { // stencil.cpp:78-100
        log.info("E2-poly scheme chosen");
        auto join = [](const std::vector<real>& v) {
            std::string out;
            for (size_t i = 0; i < v.size(); i++) out += (i ? ", " : "") + fmt_real(v[i]);
            return out;
        };
        if (!alpha.empty()) {
            // one array holding the floating, dirichlet and interpolant alpha in turn
            log.info("alpha = " + join(alpha));
            std::vector<real> a = alpha;
            a.resize(std::max<std::size_t>(a.size(), 13), 0.0);
            const std::span<const real> sa{a};
            return stencils::make_polyE2_1(sa.subspan(0, 6), sa.subspan(6, 3), sa.subspan(9, 4));
        }
        const std::vector<real> fa = read_alpha("floating_alpha"), da = read_alpha("dirichlet_alpha"),
                                ia = read_alpha("interpolant_alpha");
        log.info("floating alpha = " + join(fa));
        log.info("dirichlet alpha = " + join(da));
        log.info("interpolant alpha = " + join(ia));
        return stencils::make_polyE2_1(fa, da, ia);
    }
    if (order == 1 && type == "E6u") {
        log.info("E6 uniform first scheme chosen");
        return stencils::make_E6u_1(alpha);
    }
    if (order == 1 && type == "E8u") {
        log.info("E8 uniform first scheme chosen");
        return stencils::make_E8u_1(alpha);
    }
    if (order == 1 && (type == "E2" || type == "tension_E4u" || type == "gaussian_E4u" ||
                       type == "multiquadric_E4u")) {
        log.err("scheme.order/type = 1 / " + type + " is not available in this build");
        return std::nullopt;
    }
    log.err("scheme.order/type = " + std::to_string(order) + " / " + type + " not recognized");
    return std::nullopt;
}

// ---- step controller: step_controller::from_lua --------------------------------------------
step_controller read_step_controller(const value& sim, const logger& log)
{
    const value c = at(sim, "step_controller");
    if (!valid(c)) {
        log.info("step_controller not specified.  using default");
        return step_controller(0, 0.0, 1.0, 1.0);
    }
    constexpr int int_max = std::numeric_limits<int>::max();
    constexpr real real_max = std::numeric_limits<real>::max();
    int max_step = int_or(at(c, "max_step"), int_max);
    const real max_time = num_or(at(c, "max_time"), real_max);
    const real min_dt = num_or(at(c, "min_dt"), 1e-6);
    const real h_cfl = num_or(at(at(c, "cfl"), "hyperbolic"), 1.0);
    const real p_cfl = num_or(at(at(c, "cfl"), "parabolic"), 1.0);
    if (max_step == int_max && max_time == real_max) max_step = 0;
    return step_controller(max_step, max_time, h_cfl, p_cfl, min_dt);
}

// ---- field output: field_io::from_lua ---------------------------------------------------------
std::optional<io_config> read_io(const value& sim, const logger& log)
{
    const value io = at(sim, "io");
    if (!valid(io)) return std::nullopt;
    io_config cfg;
    if (const value v = at(io, "write_every_step"); v.number()) cfg.write_every_step = (int)*v.number();
    if (const value v = at(io, "write_every_time"); v.number()) cfg.write_every_time = *v.number();
    cfg.dir = str_or(at(io, "dir"), "io");
    cfg.suffix_length = int_or(at(io, "suffix_length"), 6);
    cfg.xdmf_filename = str_or(at(io, "xdmf_filename"), "view.xmf");
    if (cfg.write_every_step)
        log.info("field io will write every " + std::to_string(*cfg.write_every_step) + " steps");
    else if (cfg.write_every_time)
        log.info("field io will write every " + detail::num(*cfg.write_every_time) + " time interval");
    else
        log.info("field io will not output data");
    return cfg;
}

// ---- manufactured solution: manufactured_solution::from_lua ------------------------------------
// nullopt when the section is absent; an error string when it names a kind not available here
std::variant<std::monostate, manufactured_solution, std::string> read_mms(const value& sim, const logger& log)
{
    const value ms = at(sim, "manufactured_solution");
    if (!valid(ms)) {
        log.info("manufactured_solution not specified.");
        return std::monostate{};
    }
    std::string t = str_or(at(ms, "type"), "");
    for (auto& ch : t) ch = (char)std::tolower((unsigned char)ch);
    if (t == "sinsin") return mms::sinsin(num_or(at(ms, "frequency"), 1.0));
    if (t == "gaussian") {
        log.info("building gaussian manufactured solution");
        std::vector<real3> center, variance;
        std::vector<real> amplitude, frequency;
        for (long long i = 1; valid(at(ms, i)); ++i) {
            const value g = at(ms, i);
            const value c = at(g, "center"), v = at(g, "variance");
            center.push_back({num_or(at(c, 1), 0.0), num_or(at(c, 2), 0.0), num_or(at(c, 3), 0.0)});
            variance.push_back({num_or(at(v, 1), 0.0), num_or(at(v, 2), 0.0), num_or(at(v, 3), 0.0)});
            amplitude.push_back(num_or(at(g, "amplitude"), 0.0));
            frequency.push_back(num_or(at(g, "frequency"), 0.0));
        }
        // no terms: the reference builds no solution either
        if (center.empty()) return std::monostate{};
        return mms::gaussian(center, variance, amplitude, frequency);
    }
    if (t == "lua")
        return "manufactured_solution.type = `lua` (Lua functions evaluated at every point for "
               "every stage) is not available here (use `gaussian` or `sinsin`)";
    return "Got manufactured_solution.type = `" + t + "`.  Expected one of: `gaussian, lua, sinsin`";
}

// ---- the whole simulation: simulation_cycle::from_lua + run ------------------------------------
int run_simulation(const value& sim)
{
    const bool enable_logging = bool_or(at(sim, "logging"), true);
    const std::string logging_dir = enable_logging ? str_or(at(sim, "logging_dir"), "logs") : "";
    const logger log{enable_logging};

    const value sys = at(sim, "system");
    if (!valid(sys)) {
        log.err("simulation.system must be specified");
        return 0;
    }
    const std::string type = str_or(at(sys, "type"), "");
    if (type != "heat" && type != "scalar wave") {
        log.err(type == "inviscid vortex" || type == "eigenvalues" ? "system.type `" + type + "` is not available in this build"
                                                                  : "unrecognized system.type");
        return 0;
    }
    const std::string prec_s = str_or(at(sys, "precision"), "fp64");
    if (prec_s != "fp64" && prec_s != "mixed") {
        log.err("system.precision must be fp64 or mixed");
        return 0;
    }
    const precision prec = prec_s == "mixed" ? precision::mixed : precision::fp64;

    auto m = read_mesh(sim, log);
    if (!m) return 0;
    auto bc = read_bcs(sim, m->extents().extents, log);
    auto st = read_stencil(sim, log);
    if (!bc || !st) return 0;

    // integrator::from_lua
    const value integ = at(sim, "integrator");
    integrators::integrator integrator{integrators::empty{}};
    if (!valid(integ)) {
        log.warn("simulation.integrator not specified.  Defaulting to empty");
    } else {
        const std::string it = str_or(at(integ, "type"), "");
        if (it != "rk4" && it != "euler") {
            log.err("integrator.type must be one of: [rk4, euler]");
            return 0;
        }
        log.info("building " + it + " integrator");
        integrator = it == "euler" ? integrators::integrator{integrators::euler{}}
                                   : integrators::integrator{integrators::rk4{}};
    }
    const step_controller ctrl = read_step_controller(sim, log);
    const auto io_cfg = read_io(sim, log);

    // the operators of the (mesh, stencil, bcs) triple, built once on the host; the mesh's
    // geometry log comes from them, and the system runs on them
    const problem prob{*m, *st, bc->first, bc->second};
    std::optional<std::ofstream> syslog;
    if (enable_logging) {
        std::filesystem::create_directories(logging_dir);
        std::ofstream geo(std::filesystem::path{logging_dir} / "geometry.csv", std::ios::trunc);
        write_geometry_log(geo, prob);
        syslog.emplace(std::filesystem::path{logging_dir} / "system.csv", std::ios::trunc);
        write_system_log_header(*syslog);
    }
    simulation_cycle cycle(ctrl, syslog ? &*syslog : nullptr, field_io::from_config(*m, io_cfg), integrator);
    cycle.set_console(enable_logging ? &std::cout : nullptr);

    real3 r{};
    if (type == "heat") {
        log.info("building heat system");
        const real diff = num_or(at(sys, "diffusivity"), 1.0);
        auto ms = read_mms(sim, log);
        if (auto e = std::get_if<std::string>(&ms)) {
            log.err(*e);
            return 0;
        }
        manufactured_solution sol = std::holds_alternative<manufactured_solution>(ms)
                                        ? std::get<manufactured_solution>(ms)
                                        : mms::zero();
        systems::heat h(prob, std::move(sol), diff, prec);
        r = cycle.run(h);
    } else {
        log.info("building scalar_wave system");
        const real max_error = num_or(at(sys, "max_error"), 100.0);
        real3 center{};
        real radius = 0.0;
        if (valid(at(sys, "center")) && valid(at(sys, "radius"))) {
            const value c = at(sys, "center");
            center = {num_or(at(c, 1), 0.0), num_or(at(c, 2), 0.0), num_or(at(c, 3), 0.0)};
            radius = num_or(at(sys, "radius"), 0.0);
        } else if (valid(at(sim, "shapes"))) {
            bool found = false;
            const value t = at(sim, "shapes");
            for (long long i = 1; valid(at(t, i)) && !found; i++) {
                found = str_or(at(at(t, i), "type"), "") == "sphere";
                if (found) {
                    const value c = at(at(t, i), "center");
                    center = {num_or(at(c, 1), 0.0), num_or(at(c, 2), 0.0), num_or(at(c, 3), 0.0)};
                    radius = num_or(at(at(t, i), "radius"), 0.0);
                }
            }
            if (!found) {
                log.err("No valid spheres found in simulation.shapes for scalar_wave");
                return 0;
            }
        } else {
            log.err("a system.center / system.radius must be specified for scalar_wave");
            return 0;
        }
        systems::scalar_wave w(prob, center, radius, max_error, prec);
        r = cycle.run(w);
    }
    std::cout << "result " << detail::num(r[0]) << " " << detail::num(r[1]) << " " << detail::num(r[2]) << "\n";
    return 0;
}

void usage(std::ostream& os)
{
    os << "Run the Stable High-Order Cut-Cell Solver with a given input\n"
          "Usage:\n"
          "  shoccs [OPTION...] input-file\n\n"
          "      --input-file arg  Main lua input file\n"
          "      --script arg      Supplementary lua options take precedence over file\n"
          "      --check           Check input file for errors and return\n"
          "      --help            Print usage\n";
}
} // namespace

int main(int argc, char** argv)
{
    std::optional<std::string> input, script;
    bool check = false, help = false;
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        auto value_of = [&](const char* opt) -> std::optional<std::string> {
            const std::string o = opt;
            if (a == o) {
                if (i + 1 >= argc) {
                    std::cerr << "option '" << o << "' requires an argument\n";
                    std::exit(2);
                }
                return std::string(argv[++i]);
            }
            if (a.rfind(o + "=", 0) == 0) return a.substr(o.size() + 1);
            return std::nullopt;
        };
        if (a == "--help" || a == "-h") help = true;
        else if (a == "--check") check = true;
        else if (auto v = value_of("--script")) script = v;
        else if (auto v = value_of("--input-file")) input = v;
        else if (a.size() > 1 && a[0] == '-') {
            std::cerr << "unrecognised option '" << a << "'\n";
            return 2;
        } else input = a;
    }
    if (help || argc == 1) {
        usage(std::cout);
        return 0;
    }
    lua::state L;
    try {
        if (input) L.script_file(*input);
        if (script) L.script(*script, "script");
    } catch (const lua::error& e) {
        std::cerr << "lua error: " << e.what() << "\n";
        return 1;
    }
    if (check) return 0;
    std::cout << "[info] Starting shoccs\n";
    try {
        const value sim = L.get("simulation");
        if (!sim.tbl()) {
            std::cerr << "[builder] [error] the global table `simulation` is required\n";
            return 0;
        }
        return run_simulation(sim);
    } catch (const lua::error& e) {
        std::cerr << "lua error: " << e.what() << "\n";
        return 1;
    } catch (const std::exception& e) {
        std::cerr << "error: " << e.what() << "\n";
        return 1;
    }
}
