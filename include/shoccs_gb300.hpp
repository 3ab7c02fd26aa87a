// shoccs_gb300.hpp -- C++20 classes with the reference's names over the C ABI (shoccs_gpu.h).
//
// pbrady/shoccs exposes its derivative-operator path as C++ classes; this header gives a
// caller of those classes the same names, constructor arguments, call shapes and error
// behaviour, backed by the sm_103a library:
//
//   ccs::mesh                 src/mesh/mesh.hpp:24-31 (index_extents, domain_extents, shapes)
//   ccs::make_sphere          src/mesh/shapes.hpp:123
//   ccs::stencils::make_E2_2 / make_E4_2 / make_E4_1 / make_E4u_1
//                             src/stencils/stencil.hpp:275-279
//   ccs::bcs::{type, Line, Grid, Object, dd, df, ...}   src/operators/boundaries.hpp:11-47
//   ccs::eq / ccs::plus_eq    src/types.hpp:69-86
//   ccs::derivative           src/operators/derivative.hpp:20-80
//   ccs::laplacian            src/operators/laplacian.hpp:10-33
//   ccs::gradient             src/operators/gradient.hpp:10-30
//   ccs::graph, build_graph / submit_graph / add_graph_nodes of the operators,
//   build_rhs_graph / submit_rhs_graph of the systems
//                             src/operators/derivative.hpp:71-151, laplacian.hpp:35-118,
//                             gradient.hpp:31-122, src/systems/system.cpp:57-69
//   ccs::systems::heat        src/systems/heat.hpp:16-70
//   ccs::systems::scalar_wave src/systems/scalar_wave.hpp:16-80
//   ccs::integrators::rk4, euler, integrator
//                             src/temporal/rk4.hpp:10-20, euler.cpp:11-27, integrator.hpp
//   ccs::step_controller      src/temporal/step_controller.hpp:10-50
//   ccs::simulation_cycle     src/simulation/simulation_cycle.cpp:31-143 (run)
//   ccs::interval, d_interval src/io/interval.hpp:9-97
//   ccs::xdmf, field_data, field_io
//                             src/io/xdmf.cpp:20-179, src/io/field_data.cpp:8-57,
//                             src/io/field_io.cpp:29-103
//
// Differences a caller sees.  Fields are device buffers (scalar_span / scalar_view hold
// device pointers and sizes), because the kernels run on the GPU; the reference's fields are
// host Kokkos views.  Systems own their state on the device (the reference keeps it in a
// sim_registry slot), so rk4 takes the system, the time and the step size.  Failures throw
// ccs::error (a std::runtime_error carrying the library's status and message) where the
// reference returns std::nullopt from from_lua or asserts; make_E4_1 throws
// std::invalid_argument for alpha[1] < 197/288 exactly as src/stencils/E4_1.cpp:37-40 does.
// Every call returns after the stream has finished, like the reference's Kokkos::fence.
#pragma once

#include "shoccs_gpu.h"

#include <array>
#include <charconv>
#include <chrono>
#include <concepts>
#include <cstdint>
#include <cstdio>
#include <ctime>
#include <filesystem>
#include <fstream>
#include <functional>
#include <iterator>
#include <limits>
#include <optional>
#include <ostream>
#include <memory>
#include <span>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace ccs
{
using real = double;
using real3 = std::array<real, 3>;
using int3 = std::array<int, 3>;
using integer = std::int64_t;

// thrown for every non-OK status of the C ABI
class error : public std::runtime_error
{
    shoccs_status status_;

public:
    error(shoccs_status s, const std::string& what) : std::runtime_error(what), status_{s} {}
    shoccs_status status() const { return status_; }
};

namespace detail
{
inline void check(shoccs_status s, const char* call)
{
    if (s == SHOCCS_OK) return;
    char buf[512] = {};
    shoccs_last_error(buf, sizeof(buf));
    throw error(s, std::string(call) + ": " + buf);
}
} // namespace detail

// ---- index / domain extents, shapes (src/index_extents.hpp:9-19, src/mesh/mesh_types.hpp:25-28)
struct index_extents {
    int3 extents;
    constexpr operator const int3&() const { return extents; }
    constexpr integer size() const { return (integer)extents[0] * extents[1] * extents[2]; }
};

struct domain_extents {
    real3 min;
    real3 max;
};

// the embedded shapes this path supports: spheres (circles in 2-D)
struct shape {
    int id;
    real3 origin;
    real radius;
};

inline shape make_sphere(int id, const real3& origin, real radius) { return {id, origin, radius}; }

// ---- boundary conditions (src/operators/boundaries.hpp:11-47) -------------------------------
namespace bcs
{
enum class type { Dirichlet, D = Dirichlet, Floating, F = Floating, Neumann, N = Neumann };

constexpr auto Dirichlet = type::Dirichlet;
constexpr auto Neumann = type::Neumann;
constexpr auto Floating = type::Floating;

struct Line {
    type left;
    type right;
    friend auto operator<=>(const Line&, const Line&) = default;
};

using X = Line;
using Y = Line;
using Z = Line;
using Grid = std::array<Line, 3>;
using Object = std::vector<type>;

constexpr auto dd = Line{type::D, type::D};
constexpr auto ff = Line{type::F, type::F};
constexpr auto nn = Line{type::N, type::N};
constexpr auto dn = Line{type::D, type::N};
constexpr auto nd = Line{type::N, type::D};
constexpr auto df = Line{type::D, type::F};
constexpr auto fd = Line{type::F, type::D};
constexpr auto fn = Line{type::F, type::N};
constexpr auto nf = Line{type::N, type::F};

// bcs::type -> SHOCCS_BC_* (same order as the enum)
constexpr int to_c(type t) { return static_cast<int>(t); }
} // namespace bcs

// ---- stencils (src/stencils/stencil.hpp:275-279) --------------------------------------------
namespace stencils
{
struct stencil {
    int scheme;                  // SHOCCS_SCHEME_*
    std::array<real, 2> alpha{}; // E4_1 / E4u_1 closure parameters
    // E2-poly: floating alpha[6], dirichlet alpha[3], interpolant alpha[4]; E6u: alpha[5];
    // E8u: alpha[7]
    std::array<real, 13> params{};
};

inline stencil make_E2_2() { return {SHOCCS_SCHEME_E2_2, {}}; }
inline stencil make_E4_2() { return {SHOCCS_SCHEME_E4_2, {}}; }

namespace detail
{
// src/stencils/E4_1.cpp:37-40: the closure is unstable below this bound
inline std::array<real, 2> e4_alpha(std::span<const real> a, const char* name)
{
    if (a.size() < 2) throw std::invalid_argument(std::string(name) + " needs two alpha values");
    if (a[1] < 197.0 / 288.0)
        throw std::invalid_argument(std::string(name) + ": alpha[1] must be >= 197/288");
    return {a[0], a[1]};
}
} // namespace detail

inline stencil make_E4_1(std::span<const real> alpha)
{
    return {SHOCCS_SCHEME_E4_1, detail::e4_alpha(alpha, "E4_1")};
}
inline stencil make_E4u_1(std::span<const real> alpha)
{
    return {SHOCCS_SCHEME_E4U_1, {alpha.size() > 0 ? alpha[0] : 0.0, alpha.size() > 1 ? alpha[1] : 0.0}};
}
// src/stencils/polyE2_1.cpp:260-265; each parameter span copied zero-padded to its length
// (polyE2_1.cpp:21-28)
inline stencil make_polyE2_1(std::span<const real> floating_alpha, std::span<const real> dirichlet_alpha,
                             std::span<const real> interpolant_alpha)
{
    stencil st{SHOCCS_SCHEME_POLYE2_1, {}};
    for (size_t i = 0; i < 6 && i < floating_alpha.size(); i++) st.params[i] = floating_alpha[i];
    for (size_t i = 0; i < 3 && i < dirichlet_alpha.size(); i++) st.params[6 + i] = dirichlet_alpha[i];
    for (size_t i = 0; i < 4 && i < interpolant_alpha.size(); i++) st.params[9 + i] = interpolant_alpha[i];
    return st;
}
// src/stencils/E6u_1.cpp:207, E8u_1.cpp:303; alpha copied zero-padded to 5 / 7 values
inline stencil make_E6u_1(std::span<const real> alpha)
{
    stencil st{SHOCCS_SCHEME_E6U_1, {}};
    for (size_t i = 0; i < 5 && i < alpha.size(); i++) st.params[i] = alpha[i];
    return st;
}
inline stencil make_E8u_1(std::span<const real> alpha)
{
    stencil st{SHOCCS_SCHEME_E8U_1, {}};
    for (size_t i = 0; i < 7 && i < alpha.size(); i++) st.params[i] = alpha[i];
    return st;
}
} // namespace stencils
using stencils::stencil;

// ---- mesh (src/mesh/mesh.hpp:24-31) ---------------------------------------------------------
// Geometry only; the cut points and line segments are built with the operators (by the
// library, bit-exact with the reference's mesh) the first time a problem is created.
class mesh
{
    index_extents ex_;
    domain_extents bounds_;
    std::vector<shape> shapes_;

public:
    mesh() = default;
    mesh(const index_extents& extents, const domain_extents& bounds) : ex_{extents}, bounds_{bounds} {}
    mesh(const index_extents& extents, const domain_extents& bounds, const std::vector<shape>& shapes)
        : ex_{extents}, bounds_{bounds}, shapes_{shapes}
    {
    }
    const index_extents& extents() const { return ex_; }
    const domain_extents& bounds() const { return bounds_; }
    const std::vector<shape>& shapes() const { return shapes_; }
    integer size() const { return ex_.size(); }
    int dims() const
    {
        return (ex_.extents[0] > 1) + (ex_.extents[1] > 1) + (ex_.extents[2] > 1);
    }
    real h(int i) const
    {
        return ex_.extents[i] > 1 ? (bounds_.max[i] - bounds_.min[i]) / (ex_.extents[i] - 1) : 0.0;
    }
    // flat index of (i, j, k), z fastest (src/mesh/mesh.hpp:64-68)
    integer ic(int3 ijk) const
    {
        const auto& n = ex_.extents;
        return (integer)ijk[0] * n[1] * n[2] + (integer)ijk[1] * n[2] + ijk[2];
    }
};

// ---- fields (src/fields/scalar.hpp:13-67) -----------------------------------------------------
// {D, Rx, Ry, Rz} as DEVICE pointers with their element counts.  The element type is double
// for FP64 operators and systems, float for mixed-precision operators.
template <typename T>
struct scalar_ref {
    std::span<T> D, Rx, Ry, Rz;
};
using scalar_span = scalar_ref<real>;
using scalar_view = scalar_ref<const real>;
using scalar_span_f = scalar_ref<float>;
using scalar_view_f = scalar_ref<const float>;

namespace detail
{
template <typename T>
shoccs_field field(const scalar_ref<T>& s)
{
    auto p = [](auto sp) { return (void*)sp.data(); };
    return {p(s.D), p(s.Rx), p(s.Ry), p(s.Rz)};
}
} // namespace detail

// ---- assignment operators (src/types.hpp:69-86) ---------------------------------------------
struct eq_t {
    constexpr void operator()(real& a, real b) const { a = b; }
};
struct plus_eq_t {
    constexpr void operator()(real& a, real b) const { a += b; }
};
inline constexpr eq_t eq{};
inline constexpr plus_eq_t plus_eq{};

// arithmetic of an operator or system (SHOCCS_PREC_*)
enum class precision { fp64 = SHOCCS_PREC_FP64, mixed = SHOCCS_PREC_MIXED };

// ---- the compiled operators of one (mesh, stencil, bcs) triple ------------------------------
// derivative(x), derivative(y), derivative(z), laplacian, gradient and the systems of the
// same triple share one library problem (the three axes' operators, built once).
class problem
{
    std::shared_ptr<shoccs_problem> p_;
    std::array<integer, 5> sizes_{};

public:
    problem() = default;
    problem(const mesh& m, const stencil& st, const bcs::Grid& grid_bcs, const bcs::Object& object_bcs)
    {
        shoccs_problem_desc d{};
        const auto& sh = m.shapes();
        if (object_bcs.size() < sh.size())
            throw std::invalid_argument("bcs::Object needs one boundary condition per shape");
        std::vector<real> centers;
        std::vector<real> radii;
        std::vector<int> sbc;
        for (std::size_t i = 0; i < sh.size(); i++) {
            centers.insert(centers.end(), sh[i].origin.begin(), sh[i].origin.end());
            radii.push_back(sh[i].radius);
            sbc.push_back(bcs::to_c(object_bcs[i]));
        }
        for (int a = 0; a < 3; a++) {
            d.n[a] = m.extents().extents[a];
            d.lo[a] = m.bounds().min[a];
            d.hi[a] = m.bounds().max[a];
            d.grid_bc[2 * a] = bcs::to_c(grid_bcs[a].left);
            d.grid_bc[2 * a + 1] = bcs::to_c(grid_bcs[a].right);
        }
        d.n_spheres = (int)sh.size();
        d.centers = centers.data();
        d.radii = radii.data();
        d.sphere_bc = sbc.data();
        d.scheme = st.scheme;
        d.alpha[0] = st.alpha[0];
        d.alpha[1] = st.alpha[1];
        for (int i = 0; i < 13; i++) d.scheme_alpha[i] = st.params[i];
        shoccs_problem* raw = nullptr;
        detail::check(shoccs_problem_create(&d, &raw), "shoccs_problem_create");
        p_.reset(raw, [](shoccs_problem* q) { shoccs_problem_destroy(q); });
        int64_t s[5];
        detail::check(shoccs_problem_sizes(raw, s), "shoccs_problem_sizes");
        for (int i = 0; i < 5; i++) sizes_[i] = s[i];
    }
    shoccs_problem* get() const { return p_.get(); }
    explicit operator bool() const { return (bool)p_; }
    // N_D, |Rx|, |Ry|, |Rz|, fluid points (mesh::size(), mesh::R(dir).size())
    integer size() const { return sizes_[0]; }
    integer R(int dir) const { return sizes_[1 + dir]; }
    integer fluid() const { return sizes_[4]; }
};

namespace detail
{
inline int plus(eq_t) { return 0; }
inline int plus(plus_eq_t) { return 1; }
} // namespace detail

// ---- graphs (Kokkos::Experimental::Graph as the reference builds them) -------------------------
// A graph records operator applies (add_graph_nodes) and system right-hand sides with their
// buffers baked in and replays them, in the order they were added, as one captured CUDA
// graph.  The reference chains graph nodes from a parent (add_graph_nodes(parent, ...)
// returns the node to chain from); here the parent is the graph itself and the recording
// order is the chain.  submit() runs the graph and returns after the stream has finished
// (derivative::submit_graph, src/operators/derivative.cpp:591-596); t is the time of its
// right-hand sides (heat::submit_rhs_graph fills the source at that time).
class graph
{
    std::shared_ptr<shoccs_graph> g_;
    void* stream_ = nullptr;

public:
    graph()
    {
        shoccs_graph* raw = nullptr;
        detail::check(shoccs_graph_create(&raw), "shoccs_graph_create");
        g_.reset(raw, [](shoccs_graph* q) { shoccs_graph_destroy(q); });
    }
    shoccs_graph* get() const { return g_.get(); }
    void set_stream(void* cuda_stream) { stream_ = cuda_stream; }
    void submit(real t = 0.0) const { detail::check(shoccs_graph_submit(g_.get(), t, stream_), "shoccs_graph_submit"); }
    // {recorded applies, kernel and memset nodes of the captured graph, captures so far}
    std::array<std::int64_t, 3> info() const
    {
        std::array<std::int64_t, 3> v{};
        detail::check(shoccs_graph_info(g_.get(), v.data()), "shoccs_graph_info");
        return v;
    }
};

// ---- derivative (src/operators/derivative.hpp:20-80) -------------------------------------------
// du (=|+=) D_dir u, with optional Neumann data nu (FP64 in both precisions).
// precision::mixed applies the FP32 operator to float fields (scalar_view_f / scalar_span_f).
class derivative
{
    int dir_ = 0;
    problem p_;
    precision prec_ = precision::fp64;
    void* stream_ = nullptr;

    template <typename V, typename S>
    void apply(const V& u, const scalar_view* nu, const S& du, int plus) const
    {
        shoccs_field fu = detail::field(u), fdu = detail::field(du), fnu{};
        if (nu) fnu = detail::field(*nu);
        detail::check(shoccs_derivative_apply(p_.get(), dir_, (int)prec_, &fu, nu ? &fnu : nullptr,
                                              &fdu, plus, stream_),
                      "shoccs_derivative_apply");
    }

public:
    derivative() = default;
    derivative(int dir, const mesh& m, const stencil& st, const bcs::Grid& grid_bcs,
               const bcs::Object& object_bcs, precision prec = precision::fp64)
        : dir_{dir}, p_{m, st, grid_bcs, object_bcs}, prec_{prec}
    {
    }
    // share the operators of an existing problem
    derivative(int dir, const problem& p, precision prec = precision::fp64) : dir_{dir}, p_{p}, prec_{prec} {}

    void set_stream(void* cuda_stream) { stream_ = cuda_stream; }
    const problem& get_problem() const { return p_; }

    template <typename Op = eq_t>
    void operator()(scalar_view u, scalar_span du, Op op = {}) const { apply(u, nullptr, du, detail::plus(op)); }
    template <typename Op = eq_t>
    void operator()(scalar_view u, scalar_view nu, scalar_span du, Op op = {}) const
    {
        apply(u, &nu, du, detail::plus(op));
    }
    template <typename Op = eq_t>
    void operator()(scalar_view_f u, scalar_span_f du, Op op = {}) const { apply(u, nullptr, du, detail::plus(op)); }
    template <typename Op = eq_t>
    void operator()(scalar_view_f u, scalar_view nu, scalar_span_f du, Op op = {}) const
    {
        apply(u, &nu, du, detail::plus(op));
    }

    // graph forms (src/operators/derivative.hpp:71-151): add_graph_nodes records the apply
    // in a graph; build_graph makes the operator's own graph of one apply, submit_graph runs it
    template <typename Op = eq_t>
    graph& add_graph_nodes(graph& g, scalar_view u, scalar_span du, Op op = {}) const
    {
        return record(g, u, nullptr, du, detail::plus(op));
    }
    template <typename Op = eq_t>
    graph& add_graph_nodes(graph& g, scalar_view u, scalar_view nu, scalar_span du, Op op = {}) const
    {
        return record(g, u, &nu, du, detail::plus(op));
    }
    template <typename Op = eq_t>
    graph& add_graph_nodes(graph& g, scalar_view_f u, scalar_span_f du, Op op = {}) const
    {
        return record(g, u, nullptr, du, detail::plus(op));
    }
    template <typename Op = eq_t>
    graph& add_graph_nodes(graph& g, scalar_view_f u, scalar_view nu, scalar_span_f du, Op op = {}) const
    {
        return record(g, u, &nu, du, detail::plus(op));
    }
    template <typename... A>
    void build_graph(A&&... a)
    {
        graph_ = graph{};
        add_graph_nodes(*graph_, std::forward<A>(a)...);
    }
    void submit_graph()
    {
        if (!graph_) throw error(SHOCCS_EINVAL, "derivative::submit_graph: no graph built");
        graph_->set_stream(stream_);
        graph_->submit();
    }

private:
    std::optional<graph> graph_;
    template <typename V, typename S>
    graph& record(graph& g, const V& u, const scalar_view* nu, const S& du, int plus) const
    {
        shoccs_field fu = detail::field(u), fdu = detail::field(du), fnu{};
        if (nu) fnu = detail::field(*nu);
        detail::check(shoccs_graph_add_derivative(g.get(), p_.get(), dir_, (int)prec_, &fu,
                                                  nu ? &fnu : nullptr, &fdu, plus),
                      "shoccs_graph_add_derivative");
        return g;
    }
};

// ---- laplacian (src/operators/laplacian.hpp:10-33) ---------------------------------------------
// operator()(u[, nu]) returns the apply as a callable, like the reference:  lap(u)(du).
class laplacian
{
    problem p_;
    precision prec_ = precision::fp64;
    void* stream_ = nullptr;

    template <typename V, typename S>
    void apply(const V& u, const scalar_view* nu, const S& du) const
    {
        shoccs_field fu = detail::field(u), fdu = detail::field(du), fnu{};
        if (nu) fnu = detail::field(*nu);
        detail::check(shoccs_laplacian_apply(p_.get(), (int)prec_, &fu, nu ? &fnu : nullptr, &fdu, stream_),
                      "shoccs_laplacian_apply");
    }

public:
    laplacian() = default;
    laplacian(const mesh& m, const stencil& st, const bcs::Grid& grid_bcs, const bcs::Object& object_bcs,
              precision prec = precision::fp64)
        : p_{m, st, grid_bcs, object_bcs}, prec_{prec}
    {
    }
    laplacian(const problem& p, precision prec = precision::fp64) : p_{p}, prec_{prec} {}
    void set_stream(void* cuda_stream) { stream_ = cuda_stream; }

    std::function<void(scalar_span)> operator()(scalar_view u) const
    {
        return [this, u](scalar_span du) { apply(u, nullptr, du); };
    }
    std::function<void(scalar_span)> operator()(scalar_view u, scalar_view nu) const
    {
        return [this, u, nu](scalar_span du) { apply(u, &nu, du); };
    }
    std::function<void(scalar_span_f)> operator()(scalar_view_f u) const
    {
        return [this, u](scalar_span_f du) { apply(u, nullptr, du); };
    }
    std::function<void(scalar_span_f)> operator()(scalar_view_f u, scalar_view nu) const
    {
        return [this, u, nu](scalar_span_f du) { apply(u, &nu, du); };
    }

    // graph forms (src/operators/laplacian.hpp:35-118)
    graph& add_graph_nodes(graph& g, scalar_view u, scalar_span du) const { return record(g, u, nullptr, du); }
    graph& add_graph_nodes(graph& g, scalar_view u, scalar_view nu, scalar_span du) const
    {
        return record(g, u, &nu, du);
    }
    graph& add_graph_nodes(graph& g, scalar_view_f u, scalar_span_f du) const { return record(g, u, nullptr, du); }
    graph& add_graph_nodes(graph& g, scalar_view_f u, scalar_view nu, scalar_span_f du) const
    {
        return record(g, u, &nu, du);
    }
    template <typename... A>
    void build_graph(A&&... a)
    {
        graph_ = graph{};
        add_graph_nodes(*graph_, std::forward<A>(a)...);
    }
    void submit_graph()
    {
        if (!graph_) throw error(SHOCCS_EINVAL, "laplacian::submit_graph: no graph built");
        graph_->set_stream(stream_);
        graph_->submit();
    }

private:
    std::optional<graph> graph_;
    template <typename V, typename S>
    graph& record(graph& g, const V& u, const scalar_view* nu, const S& du) const
    {
        shoccs_field fu = detail::field(u), fdu = detail::field(du), fnu{};
        if (nu) fnu = detail::field(*nu);
        detail::check(shoccs_graph_add_laplacian(g.get(), p_.get(), (int)prec_, &fu, nu ? &fnu : nullptr, &fdu),
                      "shoccs_graph_add_laplacian");
        return g;
    }
};

// ---- gradient (src/operators/gradient.hpp:10-30) -----------------------------------------------
class gradient
{
    problem p_;
    precision prec_ = precision::fp64;
    void* stream_ = nullptr;

    template <typename V, typename S>
    void apply(const V& u, const S& dx, const S& dy, const S& dz) const
    {
        shoccs_field fu = detail::field(u), fx = detail::field(dx), fy = detail::field(dy),
                     fz = detail::field(dz);
        detail::check(shoccs_gradient_apply(p_.get(), (int)prec_, &fu, &fx, &fy, &fz, stream_),
                      "shoccs_gradient_apply");
    }

public:
    gradient() = default;
    gradient(const mesh& m, const stencil& st, const bcs::Grid& grid_bcs, const bcs::Object& object_bcs,
             precision prec = precision::fp64)
        : p_{m, st, grid_bcs, object_bcs}, prec_{prec}
    {
    }
    gradient(const problem& p, precision prec = precision::fp64) : p_{p}, prec_{prec} {}
    void set_stream(void* cuda_stream) { stream_ = cuda_stream; }

    std::function<void(scalar_span, scalar_span, scalar_span)> operator()(scalar_view u) const
    {
        return [this, u](scalar_span dx, scalar_span dy, scalar_span dz) { apply(u, dx, dy, dz); };
    }
    std::function<void(scalar_span_f, scalar_span_f, scalar_span_f)> operator()(scalar_view_f u) const
    {
        return [this, u](scalar_span_f dx, scalar_span_f dy, scalar_span_f dz) { apply(u, dx, dy, dz); };
    }

    // graph form (src/operators/gradient.hpp:31-122): du_x, du_y, du_z of u
    graph& add_graph_nodes(graph& g, scalar_view u, scalar_span dx, scalar_span dy, scalar_span dz) const
    {
        return record(g, u, dx, dy, dz);
    }
    graph& add_graph_nodes(graph& g, scalar_view_f u, scalar_span_f dx, scalar_span_f dy, scalar_span_f dz) const
    {
        return record(g, u, dx, dy, dz);
    }

private:
    template <typename V, typename S>
    graph& record(graph& g, const V& u, const S& dx, const S& dy, const S& dz) const
    {
        shoccs_field fu = detail::field(u), fx = detail::field(dx), fy = detail::field(dy),
                     fz = detail::field(dz);
        detail::check(shoccs_graph_add_gradient(g.get(), p_.get(), (int)prec_, &fu, &fx, &fy, &fz),
                      "shoccs_graph_add_gradient");
        return g;
    }
};

// ---- statistics (src/types.hpp:57-60) ---------------------------------------------------------
// stats = {Linf, min, max, Linf_D, argmax_D, Linf_Rx, argmax_Rx, Linf_Ry, argmax_Ry, Linf_Rz,
//          argmax_Rz} of the state against the exact solution
struct system_stats {
    std::vector<real> stats;
    real wall_time_s = 0.0;
};

// ---- closed-form manufactured / exact solutions (the Dirichlet data, the heat source and
// the error reference; src/mms/manufactured_solutions.hpp) -------------------------------------
struct manufactured_solution {
    int kind = SHOCCS_SOL_ZERO;
    std::array<real, 8> params{};
    std::vector<real> terms; // SHOCCS_SOL_GAUSSIAN: 8 values per term
};
namespace mms
{
inline manufactured_solution zero() { return {}; }
// prod_d sin(2 pi k x_d) e^{-t}
inline manufactured_solution sinsin(real k) { return {SHOCCS_SOL_SINSIN, {k}, {}}; }
// exp(-|x - x0 - a t|^2 / (2 sigma^2)), the translated pulse of a constant velocity a
inline manufactured_solution gauss_pulse(const real3& x0, const real3& a, real sigma)
{
    return {SHOCCS_SOL_GAUSS_PULSE, {x0[0], x0[1], x0[2], a[0], a[1], a[2], sigma}, {}};
}
// sin(2 pi (|x - c| - r - t)), the reference's circular wave (src/systems/scalar_wave.cpp:28-40)
inline manufactured_solution radial_sin(const real3& c, real r)
{
    return {SHOCCS_SOL_RADIAL_SIN, {c[0], c[1], c[2], r}, {}};
}
// the reference's "gaussian" solution (build_ms_gauss, src/mms/mms.cpp:16-31): the sum over
// terms of amplitude cos(frequency t) exp(-1/2 sum_d (x_d - center_d)^2 / variance_d^2) over
// the mesh's dimensions; FP64 heat systems only
inline manufactured_solution gaussian(std::span<const real3> center, std::span<const real3> variance,
                                      std::span<const real> amplitude, std::span<const real> frequency)
{
    manufactured_solution m{SHOCCS_SOL_GAUSSIAN, {}, {}};
    for (std::size_t i = 0; i < center.size(); i++) {
        m.terms.insert(m.terms.end(), center[i].begin(), center[i].end());
        const real3 v = i < variance.size() ? variance[i] : real3{};
        m.terms.insert(m.terms.end(), v.begin(), v.end());
        m.terms.push_back(i < amplitude.size() ? amplitude[i] : 0.0);
        m.terms.push_back(i < frequency.size() ? frequency[i] : 0.0);
    }
    return m;
}
} // namespace mms

class field_io;
class step_controller;

namespace systems
{
// the state, the RK4 registers and the boundary data of a system live on the device
class scalar_system
{
protected:
    problem p_;
    std::shared_ptr<shoccs_system> s_;
    real max_error_ = 0.0;
    void* stream_ = nullptr;

    scalar_system(const mesh& m, const stencil& st, const bcs::Grid& g, const bcs::Object& o,
                  const shoccs_system_desc& d)
        : scalar_system(problem{m, st, g, o}, d)
    {
    }
    // on operators already built for the (mesh, stencil, bcs) triple
    scalar_system(const problem& p, const shoccs_system_desc& d) : p_{p}, max_error_{d.max_error}
    {
        shoccs_system* raw = nullptr;
        detail::check(shoccs_system_create(p_.get(), &d, &raw), "shoccs_system_create");
        s_.reset(raw, [](shoccs_system* q) { shoccs_system_destroy(q); });
    }

public:
    shoccs_system* get() const { return s_.get(); }
    const problem& get_problem() const { return p_; }
    void set_stream(void* cuda_stream) { stream_ = cuda_stream; }

    // u0 <- the exact solution at time t (system::initialize)
    void initialize(real t)
    {
        detail::check(shoccs_system_initialize(s_.get(), t, stream_), "shoccs_system_initialize");
    }
    // rhs of the current state at time t into du (FP64 device field)
    void rhs(real t, scalar_span du) const
    {
        shoccs_field f = detail::field(du);
        detail::check(shoccs_system_rhs(s_.get(), t, &f, stream_), "shoccs_system_rhs");
    }
    // the state as FP64: on_device selects device (true) or host (false) buffers
    void get_state(scalar_span u, bool on_device = true) const
    {
        shoccs_field f = detail::field(u);
        detail::check(shoccs_system_get_state(s_.get(), &f, on_device ? 1 : 0, stream_),
                      "shoccs_system_get_state");
    }
    void set_state(scalar_view u, bool on_device = true)
    {
        shoccs_field f = detail::field(u);
        detail::check(shoccs_system_set_state(s_.get(), &f, on_device ? 1 : 0, stream_),
                      "shoccs_system_set_state");
    }
    system_stats stats(real t) const
    {
        system_stats st;
        st.stats.resize(11);
        detail::check(shoccs_system_stats(s_.get(), t, st.stats.data(), stream_), "shoccs_system_stats");
        return st;
    }
    // system::valid: a finite max-norm error within the system's bound
    bool valid(const system_stats& st) const
    {
        const real v = st.stats.empty() ? 0.0 : st.stats[0];
        return v == v && v <= max_error_ && v >= -max_error_;
    }
    // system::timestep_size: heat p h_min^2 / (4k), wave c h_min
    real timestep_size(real cfl) const
    {
        real dt = 0.0;
        detail::check(shoccs_system_timestep(s_.get(), cfl, &dt), "shoccs_system_timestep");
        return dt;
    }
    // |u - exact(t)| at the fluid D points and the non-Dirichlet cut points, 0 elsewhere
    // (FP64; on_device selects device or host buffers)
    void error_field(real t, scalar_span err, bool on_device = true) const
    {
        shoccs_field f = detail::field(err);
        detail::check(shoccs_system_error_field(s_.get(), t, &f, on_device ? 1 : 0, stream_),
                      "shoccs_system_error_field");
    }
    // system::write: the fields "U" (the state) and "Error" through the field writer when
    // its schedule fires at this step (write_scalar_error,
    // src/systems/detail/scalar_system_utils.hpp:224-296); true when it wrote
    bool write(field_io& io, const step_controller& c, real dt) const;

    // graph forms (src/systems/system.cpp:57-69, heat.cpp:164-294): the right-hand side of
    // the current state into du as a graph, run at a given time
    graph& add_graph_nodes(graph& g, scalar_span du) const
    {
        shoccs_field f = detail::field(du);
        detail::check(shoccs_graph_add_rhs(g.get(), s_.get(), &f), "shoccs_graph_add_rhs");
        return g;
    }
    void build_rhs_graph(scalar_span du)
    {
        rhs_graph_ = graph{};
        add_graph_nodes(*rhs_graph_, du);
    }
    void submit_rhs_graph(real t)
    {
        if (!rhs_graph_) throw error(SHOCCS_EINVAL, "submit_rhs_graph: no graph built");
        rhs_graph_->set_stream(stream_);
        rhs_graph_->submit(t);
    }

private:
    std::optional<graph> rhs_graph_;
};

// dT/dt = k lap T + the manufactured source (src/systems/heat.hpp:16-70)
class heat : public scalar_system
{
    static shoccs_system_desc desc(const manufactured_solution& ms, real k, precision prec)
    {
        shoccs_system_desc d{};
        d.kind = SHOCCS_SYS_HEAT;
        d.prec = (int)prec;
        d.diffusivity = k;
        d.sol_kind = ms.kind;
        for (int i = 0; i < 8; i++) d.sol[i] = ms.params[i];
        d.sol_n_terms = (int)(ms.terms.size() / 8);
        d.sol_terms = ms.terms.empty() ? nullptr : ms.terms.data(); // copied by shoccs_system_create
        d.max_error = 1e6; // src/systems/heat.cpp:54-58
        return d;
    }

public:
    heat(mesh&& m, bcs::Grid&& grid_bcs, bcs::Object&& object_bcs, manufactured_solution&& m_sol,
         stencil st, real diffusivity, precision prec = precision::fp64)
        : scalar_system(m, st, grid_bcs, object_bcs, desc(m_sol, diffusivity, prec))
    {
    }
    // on a problem's operators (shared with derivative / laplacian / gradient of the same triple)
    heat(const problem& p, manufactured_solution&& m_sol, real diffusivity, precision prec = precision::fp64)
        : scalar_system(p, desc(m_sol, diffusivity, prec))
    {
    }
};

// u_t + a . grad u = 0 written as u_t = gG . grad u (src/systems/scalar_wave.hpp:16-80)
class scalar_wave : public scalar_system
{
    static shoccs_system_desc radial(const real3& center, real radius, real max_error, precision prec)
    {
        shoccs_system_desc d{};
        d.kind = SHOCCS_SYS_WAVE;
        d.prec = (int)prec;
        d.vel_kind = SHOCCS_VEL_RADIAL;
        for (int i = 0; i < 3; i++) d.center[i] = center[i];
        const auto ms = mms::radial_sin(center, radius);
        d.sol_kind = ms.kind;
        for (int i = 0; i < 8; i++) d.sol[i] = ms.params[i];
        d.max_error = max_error;
        return d;
    }
    static shoccs_system_desc constant(const real3& a, const manufactured_solution& ms, real max_error,
                                       precision prec)
    {
        shoccs_system_desc d{};
        d.kind = SHOCCS_SYS_WAVE;
        d.prec = (int)prec;
        d.vel_kind = SHOCCS_VEL_CONSTANT;
        for (int i = 0; i < 3; i++) d.vel[i] = a[i];
        d.sol_kind = ms.kind;
        for (int i = 0; i < 8; i++) d.sol[i] = ms.params[i];
        d.max_error = max_error;
        return d;
    }

public:
    // the reference's circular wave: gG = -(x - c)/|x - c|, exact sin(2 pi (|x - c| - r - t))
    scalar_wave(mesh&& m, bcs::Grid&& grid_bcs, bcs::Object&& object_bcs, stencil st, real3 center,
                real radius, real max_error = 100.0, precision prec = precision::fp64)
        : scalar_system(m, st, grid_bcs, object_bcs, radial(center, radius, max_error, prec))
    {
    }
    scalar_wave(const problem& p, real3 center, real radius, real max_error = 100.0,
                precision prec = precision::fp64)
        : scalar_system(p, radial(center, radius, max_error, prec))
    {
    }
    // extension: a constant velocity a with a closed-form exact solution (e.g. mms::gauss_pulse)
    scalar_wave(mesh&& m, bcs::Grid&& grid_bcs, bcs::Object&& object_bcs, stencil st, real3 velocity,
                manufactured_solution&& exact, real max_error = 100.0, precision prec = precision::fp64)
        : scalar_system(m, st, grid_bcs, object_bcs, constant(velocity, exact, max_error, prec))
    {
    }
};
} // namespace systems

// ---- integrators (src/temporal/rk4.hpp:10-20, src/temporal/rk4.cpp:11-48) ----------------------
namespace integrators
{
// classic RK4: one step of size dt from time t advances the system's state in place (the
// reference's rk4 writes u1 and simulation_cycle copies it back into u0)
class rk4
{
public:
    rk4() = default;
    void operator()(systems::scalar_system& sys, real t, real dt, void* stream = nullptr) const
    {
        run(sys, t, dt, 1, stream);
    }
    // nsteps steps in one call (the fused stage kernels stay on the device throughout)
    void run(systems::scalar_system& sys, real t0, real dt, int nsteps, void* stream = nullptr) const
    {
        detail::check(shoccs_system_rk4(sys.get(), t0, dt, nsteps, stream), "shoccs_system_rk4");
    }
};

// forward Euler (src/temporal/euler.cpp:11-27): u <- u + dt rhs(u, t), then the boundary
// data at t + dt; FP64 systems
class euler
{
public:
    euler() = default;
    void operator()(systems::scalar_system& sys, real t, real dt, void* stream = nullptr) const
    {
        run(sys, t, dt, 1, stream);
    }
    void run(systems::scalar_system& sys, real t0, real dt, int nsteps, void* stream = nullptr) const
    {
        detail::check(shoccs_system_euler(sys.get(), t0, dt, nsteps, stream), "shoccs_system_euler");
    }
};

// no time integration: the state keeps its value while the cycle advances the time
// (src/temporal/empty_integrator.hpp; integrator::operator() does nothing for it)
struct empty {
};

// the integrator of a simulation (src/temporal/integrator.hpp: a variant over the
// integrators), rk4 unless chosen otherwise
class integrator
{
    int kind_ = 0; // 0 rk4, 1 euler, 2 empty

public:
    integrator(rk4 = {}) {}
    integrator(euler) : kind_{1} {}
    integrator(empty) : kind_{2} {}
    bool is_euler() const { return kind_ == 1; }
    bool is_empty() const { return kind_ == 2; }
    void operator()(systems::scalar_system& sys, real t, real dt, void* stream = nullptr) const
    {
        if (kind_ == 1) euler{}(sys, t, dt, stream);
        else if (kind_ == 0) rk4{}(sys, t, dt, stream);
    }
};
} // namespace integrators

// ---- step controller and simulation cycle (src/temporal/step_controller.hpp,
// src/simulation/simulation_cycle.cpp:31-143) -------------------------------------------------
// The step and the time are bounded [min, max): the cycle runs while both are in bounds.
class step_controller
{
    int step_ = 0, max_step_ = 0;
    real time_ = 0.0, max_time_ = 0.0;
    real h_cfl_ = 0.0, p_cfl_ = 0.0, min_dt_ = 0.0;

public:
    step_controller() = default;
    step_controller(int max_step, real max_time, real hyperbolic_cfl, real parabolic_cfl,
                    real min_dt = 0.0, real start_time = 0.0)
        : max_step_{max_step}, time_{start_time}, max_time_{max_time}, h_cfl_{hyperbolic_cfl},
          p_cfl_{parabolic_cfl}, min_dt_{min_dt}
    {
    }
    explicit operator bool() const { return step_ < max_step_ && time_ < max_time_; }
    real simulation_time() const { return time_; }
    int simulation_step() const { return step_; }
    real hyperbolic_cfl() const { return h_cfl_; }
    real parabolic_cfl() const { return p_cfl_; }
    bool check_timestep_size(real dt) const { return dt >= min_dt_; }
    void advance(real dt)
    {
        time_ += dt;
        step_ += 1;
    }
};

namespace detail
{
inline real cfl_of(const systems::heat&, const step_controller& c) { return c.parabolic_cfl(); }
inline real cfl_of(const systems::scalar_wave&, const step_controller& c) { return c.hyperbolic_cfl(); }

// shortest round-trip text of a double, as fmt's "{}" prints it
inline std::string num(real v)
{
    char buf[64];
    const auto r = std::to_chars(buf, buf + sizeof buf, v);
    return std::string(buf, r.ptr);
}

// the system log line of heat::log / scalar_wave::log (heat.cpp:60-68) behind the
// "%Y-%m-%d %H:%M:%S.%f," pattern the systems set: time,step,stats...,wall ms
// "%Y-%m-%d %H:%M:%S.%f", the timestamp of the reference's log lines
inline std::string timestamp()
{
    const auto now = std::chrono::system_clock::now();
    const std::time_t tt = std::chrono::system_clock::to_time_t(now);
    const auto us = std::chrono::duration_cast<std::chrono::microseconds>(now.time_since_epoch()).count() % 1000000;
    std::tm tm{};
    localtime_r(&tt, &tm);
    char ts[64];
    std::strftime(ts, sizeof ts, "%Y-%m-%d %H:%M:%S", &tm);
    char frac[16];
    std::snprintf(frac, sizeof frac, ".%06lld", (long long)us);
    return std::string(ts) + frac;
}

inline void log_line(std::ostream& os, const step_controller& c, const system_stats& st)
{
    os << timestamp() << ',' << num(c.simulation_time()) << ',' << c.simulation_step();
    for (real v : st.stats) os << ',' << num(v);
    char wall[32];
    std::snprintf(wall, sizeof wall, "%.3f", st.wall_time_s * 1000.0);
    os << ',' << wall << '\n';
}
} // namespace detail

// ---- field output (src/io/interval.hpp, src/io/field_data.cpp, src/io/xdmf.cpp,
// src/io/field_io.cpp) ------------------------------------------------------------------------
// interval: true once a value has moved at least `distance` (less a tolerance) past the last
// accepted one; ++ accepts, so the next firing is measured from the last target, not from
// the value that fired (rollover).  A default interval never fires.
template <typename T>
class interval
{
    std::optional<T> distance_;
    T first_{};

public:
    interval() = default;
    interval(T distance, T first = T{}) : distance_{distance}, first_{first} {}
    bool operator()(T val, T tolerance = T{}) const
    {
        return distance_ && val - first_ >= *distance_ - tolerance;
    }
    explicit operator bool() const { return distance_.has_value(); }
    interval& operator++()
    {
        first_ += distance_.value_or(T{});
        return *this;
    }
    interval& operator--()
    {
        first_ -= distance_.value_or(T{});
        return *this;
    }
};

// the dump schedule: every so many steps and/or every so much simulation time (the time
// test allows one step size of slack), and always at step 0 when either is set
class d_interval
{
    interval<int> step_interval_;
    interval<real> time_interval_;
    int ndumps_ = 0;
    bool step_ready_ = false, time_ready_ = false;

public:
    d_interval() = default;
    d_interval(interval<int> step_interval, interval<real> time_interval)
        : step_interval_{step_interval}, time_interval_{time_interval}
    {
    }
    bool operator()(const step_controller& step, real dt);
    int current_dump() const { return ndumps_; }
    d_interval& operator++()
    {
        if (step_ready_) ++step_interval_;
        if (time_ready_) ++time_interval_;
        ++ndumps_;
        return *this;
    }
};

// cut-point positions of R(x), R(y), R(z) (mesh_object_info::position per cut point)
using cut_positions = std::array<std::span<const real3>, 3>;

namespace detail
{
// "%.17g": the text pugixml gives a double attribute
inline std::string num17(real v)
{
    char buf[40];
    std::snprintf(buf, sizeof buf, "%.17g", v);
    return buf;
}
inline std::string xml_escape(const std::string& s)
{
    std::string o;
    for (char c : s) {
        if (c == '&') o += "&amp;";
        else if (c == '<') o += "&lt;";
        else if (c == '>') o += "&gt;";
        else if (c == '"') o += "&quot;";
        else o += c;
    }
    return o;
}
template <typename R>
std::string join(const R& r)
{
    std::string o;
    for (auto v : r) {
        if (!o.empty()) o += ' ';
        o += num(v);
    }
    return o;
}
} // namespace detail

// xdmf: the XDMF 3.0 index of a run.  Grid 0 writes the outline (the co-rectilinear grid,
// its origin and spacing, one polyvertex geometry per cut-point axis read from the binary
// files rx, ry, rz, and an empty temporal collection); every grid appends one spatial
// collection to the temporal one: the grid F and the cut points RX, RY, RZ (those with
// points), each with one binary attribute per variable, the cut-point parts at the byte
// offset (Seek) where they follow D in the variable's file.  The file is written in the
// layout pugixml's default save gives the reference's document (tab indentation, empty
// elements as "<name ... />", doubles as %.17g attributes), and each write appends to the
// file on disk, as the reference reloads and saves it.
class xdmf
{
    std::string xmf_filename_;
    index_extents ix_;
    domain_extents bounds_;

    std::string header(const cut_positions& t) const
    {
        const auto& n = ix_.extents;
        real3 dxyz;
        for (int i = 0; i < 3; i++) dxyz[i] = (bounds_.max[i] - bounds_.min[i]) / std::max(n[i] - 1.0, 1.0);
        std::string h = "<?xml version=\"1.0\" encoding=\"utf-8\"?>\n"
                        "<!DOCTYPE Xdmf SYSTEM \"Xdmf.dtd\" []>\n"
                        "<Xdmf Version=\"3.0\">\n\t<Domain>\n";
        h += "\t\t<Topology TopologyType=\"3DCoRectMesh\" Dimensions=\"" + detail::join(n) + "\" />\n";
        h += "\t\t<Geometry GeometryType=\"Origin_DxDyDz\">\n";
        h += "\t\t\t<DataItem Format=\"XML\" NumberType=\"Float\" Dimensions=\"3\">" +
             detail::join(bounds_.min) + "</DataItem>\n";
        h += "\t\t\t<DataItem Format=\"XML\" NumberType=\"Float\" Dimensions=\"3\">" + detail::join(dxyz) +
             "</DataItem>\n\t\t</Geometry>\n";
        const char* names[3] = {"rx", "ry", "rz"};
        for (int d = 0; d < 3; d++) {
            const std::string c = std::to_string(t[d].size());
            h += "\t\t<Topology TopologyType=\"Polyvertex\" NumberOfElements=\"" + c + "\" />\n";
            h += "\t\t<Geometry GeometryType=\"XYZ\">\n";
            h += "\t\t\t<DataItem NumberType=\"Float\" Precision=\"8\" Format=\"Binary\" Dimensions=\"" + c +
                 " 3\">" + names[d] + "</DataItem>\n\t\t</Geometry>\n";
        }
        h += "\t\t<Grid Name=\"TimeSeries\" GridType=\"Collection\" CollectionType=\"Temporal\" />\n";
        h += "\t</Domain>\n</Xdmf>\n";
        return h;
    }

    std::string grid(int step, real time, std::span<const std::string> var_names,
                     std::span<const std::string> file_names, const cut_positions& t) const
    {
        std::string g = "\t\t\t<Grid Name=\"" + std::to_string(step) +
                        "\" GridType=\"Collection\" CollectionType=\"Spatial\">\n";
        g += "\t\t\t\t<Time Value=\"" + detail::num17(time) + "\" />\n";
        unsigned long offset = 0;
        auto sub = [&](unsigned long sz, const char* name, int topo, const std::string& dims) {
            if (sz == 0) return;
            g += std::string("\t\t\t\t<Grid Name=\"") + name + "\" GridType=\"Uniform\">\n";
            g += "\t\t\t\t\t<Topology Reference=\"/Xdmf/Domain/Topology[" + std::to_string(topo) + "]\" />\n";
            g += "\t\t\t\t\t<Geometry Reference=\"/Xdmf/Domain/Geometry[" + std::to_string(topo) + "]\" />\n";
            for (std::size_t i = 0; i < var_names.size(); ++i) {
                g += "\t\t\t\t\t<Attribute Name=\"" + detail::xml_escape(var_names[i]) + "\">\n";
                g += "\t\t\t\t\t\t<DataItem Dimensions=\"" + dims +
                     "\" NumberType=\"Float\" Precision=\"8\" Format=\"Binary\"";
                if (offset > 0) g += " Seek=\"" + std::to_string(offset) + "\"";
                g += ">" + detail::xml_escape(file_names[i]) + "</DataItem>\n\t\t\t\t\t</Attribute>\n";
            }
            g += "\t\t\t\t</Grid>\n";
            offset += sz * sizeof(real);
        };
        const auto& n = ix_.extents;
        sub((unsigned long)n[0] * n[1] * n[2], "F", 1, detail::join(n));
        const char* names[3] = {"RX", "RY", "RZ"};
        for (int d = 0; d < 3; d++)
            sub(t[d].size(), names[d], 2 + d, std::to_string(t[d].size()) + " 1");
        g += "\t\t\t</Grid>\n";
        return g;
    }

public:
    xdmf() = default;
    xdmf(std::string xmf_filename, index_extents ix, domain_extents bounds)
        : xmf_filename_{std::move(xmf_filename)}, ix_{ix}, bounds_{bounds}
    {
    }
    const std::string& filename() const { return xmf_filename_; }

    void write(int grid_number, real time, std::span<const std::string> var_names,
               std::span<const std::string> file_names, const cut_positions& t) const
    {
        if (grid_number == 0) {
            std::ofstream o(xmf_filename_, std::ios::binary | std::ios::trunc);
            o << header(t);
            if (!o) throw std::runtime_error("xdmf: cannot write " + xmf_filename_);
        }
        std::string doc;
        {
            std::ifstream i(xmf_filename_, std::ios::binary);
            if (!i) throw std::runtime_error("xdmf: cannot reload " + xmf_filename_);
            doc.assign(std::istreambuf_iterator<char>(i), std::istreambuf_iterator<char>());
        }
        const std::string g = grid(grid_number, time, var_names, file_names, t);
        const std::string empty =
            "\t\t<Grid Name=\"TimeSeries\" GridType=\"Collection\" CollectionType=\"Temporal\" />\n";
        const std::string close = "\t\t</Grid>\n\t</Domain>\n</Xdmf>\n";
        if (const auto at = doc.rfind(empty); at != std::string::npos) {
            doc.replace(at, empty.size(),
                        "\t\t<Grid Name=\"TimeSeries\" GridType=\"Collection\" CollectionType=\"Temporal\">\n" +
                            g + "\t\t</Grid>\n");
        } else if (doc.size() >= close.size() && doc.compare(doc.size() - close.size(), close.size(), close) == 0) {
            doc.insert(doc.size() - close.size(), g);
        } else {
            throw std::runtime_error("xdmf: " + xmf_filename_ + " has no temporal collection to append to");
        }
        std::ofstream o(xmf_filename_, std::ios::binary | std::ios::trunc);
        o << doc;
        if (!o) throw std::runtime_error("xdmf: cannot write " + xmf_filename_);
    }
};

// field_data: one raw binary file per variable: D (nx*ny*nz doubles, z fastest), then Rx,
// Ry, Rz where nonempty; and the cut-point positions (3 doubles per point, (z, y, x) on
// grids with nz == 1) in one file per axis.  The views hold HOST memory.
class field_data
{
    index_extents ix_;

public:
    field_data() = default;
    explicit field_data(index_extents ix) : ix_{ix} {}

    void write(std::span<const scalar_view> scalars, std::span<const std::string> filenames) const
    {
        const std::size_t sz = (std::size_t)ix_.extents[0] * ix_.extents[1] * ix_.extents[2];
        for (std::size_t k = 0; k < filenames.size(); ++k) {
            const auto& sc = scalars[k];
            if (sc.D.size() < sz) throw std::invalid_argument("field_data: D holds fewer than nx*ny*nz values");
            std::ofstream o(filenames[k], std::ios::binary | std::ios::trunc);
            o.write(reinterpret_cast<const char*>(sc.D.data()), (std::streamsize)(sz * sizeof(real)));
            for (auto r : {sc.Rx, sc.Ry, sc.Rz})
                if (!r.empty())
                    o.write(reinterpret_cast<const char*>(r.data()), (std::streamsize)(r.size() * sizeof(real)));
            if (!o) throw std::runtime_error("field_data: cannot write " + filenames[k]);
        }
    }

    void write_geom(std::span<const std::string> filenames, const cut_positions& t) const
    {
        for (int d = 0; d < 3; d++) {
            std::ofstream o(filenames[d], std::ios::binary | std::ios::trunc);
            for (const real3& p : t[d]) {
                const real3 q = ix_.extents[2] == 1 ? real3{p[2], p[1], p[0]} : p;
                o.write(reinterpret_cast<const char*>(q.data()), (std::streamsize)sizeof q);
            }
            if (!o) throw std::runtime_error("field_data: cannot write " + filenames[d]);
        }
    }
};

// the io table of a simulation (the keys of field_io::from_lua, src/io/field_io.cpp:71-103)
struct io_config {
    std::optional<int> write_every_step;
    std::optional<real> write_every_time;
    std::string dir = "io";
    int suffix_length = 6;
    std::string xdmf_filename = "view.xmf";
};

// field_io: on each dump (d_interval), the variables' binary files "<name>.<dump number>"
// (zero-padded to suffix_length digits) under dir, the cut-point geometry files rx, ry, rz
// with the first dump, and one grid appended to the xdmf index dir/xdmf_filename.  A
// default field_io writes nothing.
class field_io
{
    xdmf xdmf_w_;
    field_data field_data_w_;
    d_interval dump_interval_;
    std::string io_dir_;
    int suffix_length_ = 6;

public:
    field_io() = default;
    field_io(xdmf&& xdmf_w, field_data&& field_data_w, d_interval&& dump_interval, std::string&& io_dir,
             int suffix_length)
        : xdmf_w_{std::move(xdmf_w)}, field_data_w_{std::move(field_data_w)},
          dump_interval_{std::move(dump_interval)}, io_dir_{std::move(io_dir)}, suffix_length_{suffix_length}
    {
    }
    // field_io::from_lua over a parsed io table (none: a writer that never fires)
    static field_io from_config(const mesh& m, const std::optional<io_config>& cfg)
    {
        if (!cfg) return field_io{};
        const std::filesystem::path d{cfg->dir};
        const auto step = cfg->write_every_step ? interval<int>{*cfg->write_every_step} : interval<int>{};
        const auto time = cfg->write_every_time ? interval<real>{*cfg->write_every_time} : interval<real>{};
        return field_io{xdmf{(d / cfg->xdmf_filename).string(), m.extents(), m.bounds()},
                        field_data{m.extents()}, d_interval{step, time}, std::string{cfg->dir},
                        cfg->suffix_length};
    }
    // whether write() would fire at this step (the schedule is left unchanged)
    bool due(const step_controller& step, real dt) const
    {
        d_interval probe = dump_interval_;
        return probe(step, dt);
    }
    int current_dump() const { return dump_interval_.current_dump(); }
    const std::string& xdmf_filename() const { return xdmf_w_.filename(); }

    bool write(std::span<const std::string> names, std::span<const scalar_view> scalars,
               const step_controller& step, real dt, const cut_positions& r);
};

inline bool d_interval::operator()(const step_controller& step, real dt)
{
    if (!(step_interval_ || time_interval_)) return false;
    step_ready_ = step_interval_(step.simulation_step());
    time_ready_ = time_interval_(step.simulation_time(), dt);
    return step_ready_ || time_ready_ || step.simulation_step() == 0;
}

inline bool field_io::write(std::span<const std::string> names, std::span<const scalar_view> scalars,
                            const step_controller& step, real dt, const cut_positions& r)
{
    if (!dump_interval_(step, dt)) return false;
    const std::filesystem::path io{io_dir_};
    if (step.simulation_step() == 0) std::filesystem::create_directories(io);
    const int n = dump_interval_.current_dump();
    std::vector<std::string> xmf_names, data_names;
    for (const auto& name : names) {
        char suffix[48];
        std::snprintf(suffix, sizeof suffix, "%0*d", suffix_length_, n);
        xmf_names.push_back(name + "." + suffix);
        data_names.push_back((io / xmf_names.back()).string());
    }
    xdmf_w_.write(n, step.simulation_time(), names, xmf_names, r);
    if (n == 0) {
        const std::vector<std::string> geom{(io / "rx").string(), (io / "ry").string(), (io / "rz").string()};
        field_data_w_.write_geom(geom, r);
    }
    field_data_w_.write(scalars, data_names);
    ++dump_interval_;
    return true;
}

inline bool systems::scalar_system::write(field_io& io, const step_controller& c, real dt) const
{
    if (!io.due(c, dt)) return false;
    const integer N = p_.size();
    std::vector<real> u(N), err(N);
    std::array<std::vector<real>, 3> uR, eR;
    std::array<std::vector<real3>, 3> pos;
    for (int d = 0; d < 3; d++) {
        const integer n = p_.R(d);
        uR[d].resize(n);
        eR[d].resize(n);
        pos[d].resize(n);
        if (n)
            detail::check(shoccs_problem_cut_points(p_.get(), d, nullptr, pos[d].data()->data(), nullptr,
                                                    nullptr, nullptr, nullptr),
                          "shoccs_problem_cut_points");
    }
    get_state(scalar_span{u, uR[0], uR[1], uR[2]}, false);
    error_field(c.simulation_time(), scalar_span{err, eR[0], eR[1], eR[2]}, false);
    const std::array<std::string, 2> names{"U", "Error"};
    const std::array<scalar_view, 2> fields{scalar_view{u, uR[0], uR[1], uR[2]},
                                            scalar_view{err, eR[0], eR[1], eR[2]}};
    return io.write(names, fields, c, dt, cut_positions{pos[0], pos[1], pos[2]});
}

// simulation_cycle::run: initialize, then step while the controller is in bounds and the
// system's statistics are valid, logging the statistics of every step and handing the
// state to the field writer (which dumps on its own schedule).  Returns {time,
// error, error} when the run reached its bound in a valid state, {time, max, max} when it
// ended early in an invalid state, and {max, 0, 0} when the step size fell below the
// controller's minimum, as the reference does with null_v.
// the header line heat / scalar_wave write into system.csv before the first statistics line
// (src/systems/heat.cpp:44-48)
inline void write_system_log_header(std::ostream& os)
{
    os << "Timestamp,Time,Step,Linf,Min,Max,Domain_Linf,Domain_ic,Rx_Linf,Rx_ic,Ry_Linf,Ry_ic,Rz_Linf,"
          "Rz_ic,Wall_ms\n";
}

// the geometry log the mesh writes when it is built (src/mesh/mesh.cpp:139-151): a header
// line, then per cut point "timestamp,direction,index,psi,x, y, z,i, j, k" (position and
// the solid point's index triple each joined by ", ")
inline void write_geometry_log(std::ostream& os, const problem& p)
{
    os << "Timestamp,direction,ic,psi,x,y,z,i,j,k\n";
    for (int d = 0; d < 3; d++) {
        const integer n = p.R(d);
        if (!n) continue;
        std::vector<real> psi(n), pos(3 * n);
        std::vector<int> sc(3 * n);
        detail::check(shoccs_problem_cut_points(p.get(), d, psi.data(), pos.data(), nullptr, nullptr,
                                                sc.data(), nullptr),
                      "shoccs_problem_cut_points");
        for (integer i = 0; i < n; i++)
            os << detail::timestamp() << ',' << d << ',' << i << ',' << detail::num(psi[i]) << ','
               << detail::num(pos[3 * i]) << ", " << detail::num(pos[3 * i + 1]) << ", "
               << detail::num(pos[3 * i + 2]) << ',' << sc[3 * i] << ", " << sc[3 * i + 1] << ", "
               << sc[3 * i + 2] << '\n';
    }
}

class simulation_cycle
{
    step_controller ctrl_;
    std::ostream* log_ = nullptr;
    field_io io_;
    std::ostream* console_ = nullptr;
    integrators::integrator integ_;

public:
    simulation_cycle() = default;
    explicit simulation_cycle(const step_controller& c, std::ostream* system_log = nullptr,
                              field_io io = {}, integrators::integrator integ = integrators::rk4{})
        : ctrl_{c}, log_{system_log}, io_{std::move(io)}, integ_{integ}
    {
    }
    const step_controller& controller() const { return ctrl_; }
    const field_io& io() const { return io_; }
    // the cycle's progress messages (one per step, the cumulative wall time, an early end),
    // as the reference's simulation_cycle logger prints them (simulation_cycle.cpp:113-140)
    void set_console(std::ostream* console) { console_ = console; }

    template <typename System>
    real3 run(System& sys)
    {
        constexpr real null = std::numeric_limits<real>::max();
        sys.initialize(ctrl_.simulation_time());
        system_stats stats = sys.stats(ctrl_.simulation_time());
        if (log_) detail::log_line(*log_, ctrl_, stats);
        sys.write(io_, ctrl_, 0.0); // the initial dump
        const auto start = std::chrono::steady_clock::now();
        while (ctrl_ && sys.valid(stats)) {
            const real dt = sys.timestep_size(detail::cfl_of(sys, ctrl_));
            if (!ctrl_.check_timestep_size(dt)) {
                if (console_) *console_ << "required timestep too small\n";
                return {null, 0.0, 0.0};
            }
            const auto t0 = std::chrono::steady_clock::now();
            integ_(sys, ctrl_.simulation_time(), dt);
            ctrl_.advance(dt);
            stats = sys.stats(ctrl_.simulation_time());
            sys.write(io_, ctrl_, dt);
            stats.wall_time_s =
                std::chrono::duration<real>(std::chrono::steady_clock::now() - t0).count();
            if (log_) detail::log_line(*log_, ctrl_, stats);
            if (console_) {
                char wall[32];
                std::snprintf(wall, sizeof wall, "%.3f", stats.wall_time_s * 1000.0);
                *console_ << "time= " << detail::num(ctrl_.simulation_time())
                          << "  step=" << ctrl_.simulation_step() << ", dt=" << detail::num(dt)
                          << ", s0=" << detail::num(stats.stats[0]) << ", wall=" << wall << "ms\n";
            }
        }
        if (console_) {
            char total[32];
            std::snprintf(total, sizeof total, "%.3f",
                          std::chrono::duration<real>(std::chrono::steady_clock::now() - start).count());
            *console_ << "cumulative wall time: " << total << "s\n";
        }
        if (ctrl_) {
            if (console_)
                *console_ << "simulation ended prematurely at time/step  "
                          << detail::num(ctrl_.simulation_time()) << " / " << ctrl_.simulation_step() << "\n";
            return {ctrl_.simulation_time(), null, null};
        }
        return {ctrl_.simulation_time(), stats.stats[0], stats.stats[0]};
    }
};
} // namespace ccs
