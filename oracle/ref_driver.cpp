// ref_driver.cpp -- C entry points over the reference's OWN hot-path code.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.sh together with the reference's
// translation units taken unmodified from its source tree (stencils, mesh / object
// geometry / sphere / rect, operators/derivative + laplacian + gradient, matrices/csr +
// inner_block + circulant + dense, io/logging) and the serial Kokkos / sol / spdlog
// stand-ins under oracle/ref_stubs, into oracle/_ref/libshoccs_ref.so.  Used by the tests
// and tests/golden/make_golden.py to pin the oracle restatement (oracle/shoccs_oracle.cpp)
// to the reference's own setup and operator arithmetic.
//
// Problems are built exactly as the reference's from_lua readers build them
// (src/mesh/mesh.cpp:209-220, src/operators/boundaries.cpp:42-110,
// src/stencils/stencil.cpp:8-107), but through the C++ constructors: the mesh
// (mesh.hpp:29-33), one derivative per axis (derivative.hpp:42-47), the laplacian
// (laplacian.hpp:23-27) and the gradient (gradient.hpp:23-27).
#include "mesh/mesh.hpp"
#include "mesh/shapes.hpp"
#include "operators/derivative.hpp"
#include "operators/gradient.hpp"
#include "operators/laplacian.hpp"
#include "stencils/stencil.hpp"
#include "systems/system.hpp"
#include "temporal/rk4.hpp"

#include <cmath>
#include <numbers>
#include <cstring>
#include <limits>
#include <memory>
#include <vector>

using namespace ccs;
using namespace ccs::stencils;

namespace ccs
{
// defined in src/mms/mms.cpp:16-30 (declared in no header of the reference)
manufactured_solution build_ms_gauss(int dims,
                                     std::span<const real3> center,
                                     std::span<const real3> variance,
                                     std::span<const real> amplitude,
                                     std::span<const real> frequency);
} // namespace ccs

// ---------------------------------------------------------------------------
// Read access to private members.  An explicit instantiation may name a private member
// (the access check does not apply to the names in it), and the friend function it
// defines hands the member pointer out.  Nothing is modified through these pointers.
// ---------------------------------------------------------------------------
template <typename Tag, typename Tag::type M>
struct member_access {
    friend typename Tag::type get(Tag) { return M; }
};

#define REF_MEMBER(TAG, CLASS, TYPE, NAME)                                                 \
    struct TAG {                                                                           \
        using type = TYPE CLASS::*;                                                        \
        friend type get(TAG);                                                              \
    };                                                                                     \
    template struct member_access<TAG, &CLASS::NAME>;

REF_MEMBER(der_O, derivative, matrix::block, O)
REF_MEMBER(der_B, derivative, matrix::csr, B)
REF_MEMBER(der_N, derivative, matrix::csr, N)
REF_MEMBER(der_Bfx, derivative, matrix::csr, Bfx)
REF_MEMBER(der_Bfy, derivative, matrix::csr, Bfy)
REF_MEMBER(der_Bfz, derivative, matrix::csr, Bfz)
REF_MEMBER(der_Brx, derivative, matrix::csr, Brx)
REF_MEMBER(der_Bry, derivative, matrix::csr, Bry)
REF_MEMBER(der_Brz, derivative, matrix::csr, Brz)
REF_MEMBER(csr_w, matrix::csr, std::vector<real>, w)
REF_MEMBER(csr_v, matrix::csr, std::vector<integer>, v)
REF_MEMBER(csr_u, matrix::csr, std::vector<integer>, u)

// scheme: 0 E2_2, 1 E4_2, 2 E4_1, 3 E4u_1, 5 polyE2_1, 6 E6u_1, 7 E8u_1; alpha: 2 values,
// 13 for polyE2_1 (floating alpha[6], dirichlet alpha[3], interpolant alpha[4],
// stencil.cpp:79-87's order), 5 for E6u_1, 7 for E8u_1
static stencil make(int scheme, const double* alpha)
{
    if (scheme == 5) {
        std::vector<real> a(13, 0.0);
        if (alpha) std::copy(alpha, alpha + 13, a.begin());
        auto s = std::span<const real>{a};
        return make_polyE2_1(s.subspan(0, 6), s.subspan(6, 3), s.subspan(9, 4));
    }
    if (scheme == 6 || scheme == 7) {
        const int n = scheme == 6 ? 5 : 7;
        std::vector<real> a(n, 0.0);
        if (alpha) std::copy(alpha, alpha + n, a.begin());
        return scheme == 6 ? make_E6u_1(a) : make_E8u_1(a);
    }
    std::vector<real> a{alpha ? alpha[0] : 0.0, alpha ? alpha[1] : 0.0};
    switch (scheme) {
    case 0: return make_E2_2();
    case 1: return make_E4_2();
    case 3: return make_E4u_1(a);
    default: return make_E4_1(a);
    }
}

static bcs::type bc_of(int b)
{
    return b == 0 ? bcs::Dirichlet : b == 1 ? bcs::Floating : bcs::Neumann;
}

namespace
{
struct ref_problem {
    mesh m;
    std::array<derivative, 3> d;
    laplacian lap;
    gradient grad;
    std::array<int, 3> nR{};
};

scalar_view view(const ref_problem& p, const double* D, const double* rx, const double* ry,
                 const double* rz)
{
    return scalar_view{std::span<const real>(D, (std::size_t)p.m.size()),
                       std::span<const real>(rx, (std::size_t)p.nR[0]),
                       std::span<const real>(ry, (std::size_t)p.nR[1]),
                       std::span<const real>(rz, (std::size_t)p.nR[2])};
}

scalar_span span_of(const ref_problem& p, double* D, double* rx, double* ry, double* rz)
{
    return scalar_span{std::span<real>(D, (std::size_t)p.m.size()),
                       std::span<real>(rx, (std::size_t)p.nR[0]),
                       std::span<real>(ry, (std::size_t)p.nR[1]),
                       std::span<real>(rz, (std::size_t)p.nR[2])};
}

const matrix::csr& csr_of(const derivative& d, int which)
{
    switch (which) {
    case 0: return d.*get(der_B{});
    case 1: return d.*get(der_N{});
    case 2: return d.*get(der_Bfx{});
    case 3: return d.*get(der_Bfy{});
    case 4: return d.*get(der_Bfz{});
    case 5: return d.*get(der_Brx{});
    case 6: return d.*get(der_Bry{});
    default: return d.*get(der_Brz{});
    }
}
} // namespace

extern "C" {

// ---------------------------------------------------------------------------
// Problems: mesh + three derivatives + laplacian + gradient
// ---------------------------------------------------------------------------
void* ref_problem_create(const int n[3], const double lo[3], const double hi[3], int nsph,
                         const double* centers, const double* radii, const int* sphere_bc,
                         const int grid_bc[6], int scheme, const double alpha[2])
{
    std::vector<shape> shapes;
    bcs::Object obj;
    for (int i = 0; i < nsph; i++) {
        shapes.push_back(make_sphere(
            i, real3{centers[3 * i], centers[3 * i + 1], centers[3 * i + 2]}, radii[i]));
        obj.push_back(bc_of(sphere_bc[i]));
    }
    bcs::Grid grid{bcs::Line{bc_of(grid_bc[0]), bc_of(grid_bc[1])},
                   bcs::Line{bc_of(grid_bc[2]), bc_of(grid_bc[3])},
                   bcs::Line{bc_of(grid_bc[4]), bc_of(grid_bc[5])}};
    auto st = make(scheme, alpha);
    auto p = std::make_unique<ref_problem>();
    p->m = mesh{index_extents{int3{n[0], n[1], n[2]}},
                domain_extents{real3{lo[0], lo[1], lo[2]}, real3{hi[0], hi[1], hi[2]}},
                shapes};
    for (int k = 0; k < 3; k++) {
        p->d[k] = derivative{k, p->m, st, grid, obj};
        p->nR[k] = (int)p->m.R(k).size();
    }
    p->lap = laplacian{p->m, st, grid, obj};
    p->grad = gradient{p->m, st, grid, obj};
    return p.release();
}

void ref_problem_destroy(void* h) { delete static_cast<ref_problem*>(h); }

// which: 0 -> number of grid points, 1 + d -> number of cut points along axis d
long ref_problem_size(void* h, int which)
{
    auto* p = static_cast<ref_problem*>(h);
    return which == 0 ? (long)p->m.size() : (long)p->nR[which - 1];
}

void ref_cut_points(void* h, int dir, double* psi, double* pos, double* normal,
                    int* ray_outside, int* solid, int* shape_id)
{
    auto R = static_cast<ref_problem*>(h)->m.R(dir);
    for (std::size_t i = 0; i < R.size(); i++) {
        psi[i] = R[i].psi;
        for (int c = 0; c < 3; c++) {
            pos[3 * i + c] = R[i].position[c];
            normal[3 * i + c] = R[i].normal[c];
            solid[3 * i + c] = R[i].solid_coord[c];
        }
        ray_outside[i] = R[i].ray_outside;
        shape_id[i] = R[i].shape_id;
    }
}

// 8 ints per line: start ijk, start object's cut-point index (-1 at a wall), end ijk, end's
long ref_lines(void* h, int dir, int* out)
{
    const auto& L = static_cast<ref_problem*>(h)->m.lines(dir);
    if (out) {
        for (std::size_t i = 0; i < L.size(); i++) {
            int* q = out + 8 * i;
            for (int c = 0; c < 3; c++) q[c] = L[i].start.mesh_coordinate[c];
            q[3] = L[i].start.object ? (int)L[i].start.object->object_coordinate : -1;
            for (int c = 0; c < 3; c++) q[4 + c] = L[i].end.mesh_coordinate[c];
            q[7] = L[i].end.object ? (int)L[i].end.object->object_coordinate : -1;
        }
    }
    return (long)L.size();
}

long ref_fluid(void* h, long* idx)
{
    const auto& F = static_cast<ref_problem*>(h)->m.fluid_desc().indices_;
    if (idx)
        for (std::size_t i = 0; i < F.extent(0); i++) idx[i] = F(i);
    return (long)F.extent(0);
}

// block metadata (13 ints per line, inner_block_meta order) and the coefficient array
long ref_block(void* h, int dir, int* meta, double* coeffs, long* ncoeffs)
{
    const auto& O = static_cast<ref_problem*>(h)->d[dir].*get(der_O{});
    const auto& M = O.metadata_view();
    const auto& C = O.coefficients_view();
    if (meta) std::memcpy(meta, M.data(), M.extent(0) * sizeof(matrix::inner_block_meta));
    if (coeffs) std::copy(C.data(), C.data() + C.extent(0), coeffs);
    if (ncoeffs) *ncoeffs = (long)C.extent(0);
    return (long)M.extent(0);
}

// which: 0 B, 1 N, 2 + r Bf(r), 5 + r Br(r); returns nnz, fills the row offsets (rows + 1,
// or none for an empty matrix), column indices and values
long ref_csr(void* h, int dir, int which, long* nrows, long* u, long* v, double* w)
{
    const auto& c = csr_of(static_cast<ref_problem*>(h)->d[dir], which);
    const auto& W = c.*get(csr_w{});
    const auto& V = c.*get(csr_v{});
    const auto& U = c.*get(csr_u{});
    if (nrows) *nrows = (long)c.rows();
    if (u) std::copy(U.begin(), U.end(), u);
    if (v) std::copy(V.begin(), V.end(), v);
    if (w) std::copy(W.begin(), W.end(), w);
    return (long)W.size();
}

// derivative::operator() (derivative.cpp:501-519): du (op)= D_dir u, with the Neumann
// term N nu when nu_D is given
void ref_derivative(void* h, int dir, const double* uD, const double* uRx, const double* uRy,
                    const double* uRz, const double* nuD, double* dD, double* dRx, double* dRy,
                    double* dRz, int plus_eq)
{
    auto* p = static_cast<ref_problem*>(h);
    auto u = view(*p, uD, uRx, uRy, uRz);
    auto du = span_of(*p, dD, dRx, dRy, dRz);
    if (nuD) {
        std::vector<double> zr[3];
        for (int k = 0; k < 3; k++) zr[k].assign(p->nR[k], 0.0);
        auto nu = view(*p, nuD, zr[0].data(), zr[1].data(), zr[2].data());
        if (plus_eq)
            p->d[dir](u, nu, du, ccs::plus_eq);
        else
            p->d[dir](u, nu, du, ccs::eq);
    } else {
        if (plus_eq)
            p->d[dir](u, du, ccs::plus_eq);
        else
            p->d[dir](u, du, ccs::eq);
    }
}

// laplacian::operator() (laplacian.cpp:37-58)
void ref_laplacian(void* h, const double* uD, const double* uRx, const double* uRy,
                   const double* uRz, const double* nuD, double* dD, double* dRx, double* dRy,
                   double* dRz)
{
    auto* p = static_cast<ref_problem*>(h);
    auto u = view(*p, uD, uRx, uRy, uRz);
    auto du = span_of(*p, dD, dRx, dRy, dRz);
    if (nuD) {
        std::vector<double> zr[3];
        for (int k = 0; k < 3; k++) zr[k].assign(p->nR[k], 0.0);
        auto nu = view(*p, nuD, zr[0].data(), zr[1].data(), zr[2].data());
        p->lap(u, nu)(du);
    } else {
        p->lap(u)(du);
    }
}

// gradient::operator() (gradient.cpp:36-46); out = 12 pointers: (D, Rx, Ry, Rz) of du/dx,
// du/dy, du/dz
void ref_gradient(void* h, const double* uD, const double* uRx, const double* uRy,
                  const double* uRz, double** out)
{
    auto* p = static_cast<ref_problem*>(h);
    auto u = view(*p, uD, uRx, uRy, uRz);
    p->grad(u)(span_of(*p, out[0], out[1], out[2], out[3]),
               span_of(*p, out[4], out[5], out[6], out[7]),
               span_of(*p, out[8], out[9], out[10], out[11]));
}

// ---------------------------------------------------------------------------
// Systems: the reference's heat (src/systems/heat.cpp) and scalar wave
// (src/systems/scalar_wave.cpp) behind its system variant (src/systems/system.cpp), stepped
// by its rk4 integrator (src/temporal/rk4.cpp) in the loop of simulation_cycle::run
// (src/simulation/simulation_cycle.cpp:36-126): four registry slots u0, u1, rk, srhs, the
// right-hand-side graph built once on (u1, srhs), and u1 copied back to u0 after each step.
// ---------------------------------------------------------------------------
namespace
{
// sin(2 pi k x) sin(2 pi k y) [sin(2 pi k z)] e^-t with its time derivative, gradient and
// Laplacian written as the oracle writes them (this manufactured solution is a Lua function
// in the reference's inputs, so the reference holds no compiled form of it)
struct sinsin_mms {
    real k;
    int dims;
    real operator()(real t, const real3& x) const
    {
        constexpr real twoPI = 2 * 3.14159265358979323846;
        real v = std::sin(twoPI * k * x[0]) * std::sin(twoPI * k * x[1]);
        if (dims == 3) v = v * std::sin(twoPI * k * x[2]);
        return v * std::exp(-t);
    }
    real ddt(real t, const real3& x) const { return -(*this)(t, x); }
    real3 gradient(real t, const real3& x) const
    {
        constexpr real twoPI = 2 * 3.14159265358979323846;
        const real kk = twoPI * k;
        real3 g{};
        for (int dir = 0; dir < 3; dir++) {
            real v = 1.0;
            for (int d = 0; d < dims; d++)
                v = v * (d == dir ? kk * std::cos(kk * x[d]) : std::sin(kk * x[d]));
            g[dir] = dir < dims ? v * std::exp(-t) : 0.0;
        }
        return g;
    }
    real divergence(real, const real3&) const { return 0.0; }
    real laplacian(real t, const real3& x) const
    {
        constexpr real twoPI = 2 * 3.14159265358979323846;
        real kk = twoPI * k;
        return -(real)dims * kk * kk * (*this)(t, x);
    }
};

struct ref_system {
    ccs::system sys;
    sim_registry reg;
    field_ref u0{0}, u1{1}, rk{2}, srhs{3};
    std::array<int, 3> nR{};
    integer nD = 0;
    real p_cfl = 0.0, h_cfl = 0.0;
    bool graph_built = false;
};

step_controller controller_at(const ref_system& s, real t)
{
    return step_controller{bounded<int>{0, 0, std::numeric_limits<int>::max()},
                           bounded<real>{t, -std::numeric_limits<real>::max(),
                                         std::numeric_limits<real>::max()},
                           s.h_cfl, s.p_cfl, 0.0};
}

void load(ref_system& s, field_ref ref, const double* D, const double* rx, const double* ry,
          const double* rz)
{
    constexpr auto sh = scalar_handle{0};
    auto u = extract_scalar_span(s.reg, ref, sh);
    std::copy(D, D + s.nD, u.D.data());
    const double* R[3] = {rx, ry, rz};
    std::span<real> dst[3] = {u.Rx, u.Ry, u.Rz};
    for (int k = 0; k < 3; k++)
        if (s.nR[k]) std::copy(R[k], R[k] + s.nR[k], dst[k].data());
}

void store(ref_system& s, field_ref ref, double* D, double* rx, double* ry, double* rz)
{
    constexpr auto sh = scalar_handle{0};
    auto u = extract_scalar_span(s.reg, ref, sh);
    std::copy(u.D.begin(), u.D.end(), D);
    double* R[3] = {rx, ry, rz};
    std::span<real> src[3] = {u.Rx, u.Ry, u.Rz};
    for (int k = 0; k < 3; k++)
        if (s.nR[k] && R[k]) std::copy(src[k].begin(), src[k].end(), R[k]);
}

struct problem_parts {
    mesh m;
    bcs::Grid grid;
    bcs::Object obj;
    stencil st;
};

problem_parts make_parts(const int n[3], const double lo[3], const double hi[3], int nsph,
                         const double* centers, const double* radii, const int* sphere_bc,
                         const int grid_bc[6], int scheme, const double alpha[2])
{
    std::vector<shape> shapes;
    problem_parts p;
    for (int i = 0; i < nsph; i++) {
        shapes.push_back(make_sphere(
            i, real3{centers[3 * i], centers[3 * i + 1], centers[3 * i + 2]}, radii[i]));
        p.obj.push_back(bc_of(sphere_bc[i]));
    }
    p.grid = bcs::Grid{bcs::Line{bc_of(grid_bc[0]), bc_of(grid_bc[1])},
                       bcs::Line{bc_of(grid_bc[2]), bc_of(grid_bc[3])},
                       bcs::Line{bc_of(grid_bc[4]), bc_of(grid_bc[5])}};
    p.st = make(scheme, alpha);
    p.m = mesh{index_extents{int3{n[0], n[1], n[2]}},
               domain_extents{real3{lo[0], lo[1], lo[2]}, real3{hi[0], hi[1], hi[2]}},
               shapes};
    return p;
}

void* finish(std::unique_ptr<ref_system> s)
{
    auto sz = s->sys.size();
    s->nD = sz.d_size;
    s->nR = {(int)sz.rx_size, (int)sz.ry_size, (int)sz.rz_size};
    for (int c = 0; c < sz.nscalars; ++c) {
        s->u0 = s->reg.allocate_scalar(0, c, sz.d_size, sz.rx_size, sz.ry_size, sz.rz_size);
        s->u1 = s->reg.allocate_scalar(1, c, sz.d_size, sz.rx_size, sz.ry_size, sz.rz_size);
        s->rk = s->reg.allocate_scalar(2, c, sz.d_size, sz.rx_size, sz.ry_size, sz.rz_size);
        s->srhs = s->reg.allocate_scalar(3, c, sz.d_size, sz.rx_size, sz.ry_size, sz.rz_size);
    }
    return s.release();
}
} // namespace

// heat with diffusivity kappa; sol_kind 1: sin-sin (params[0] = k), 4: the reference's
// gaussian manufactured solution (build_ms_gauss, src/mms/mms.cpp:16-32) over `nterms`
// terms of 8 doubles (centre[3], variance[3], amplitude, frequency); p_cfl: cfl.parabolic
void* ref_heat_create(const int n[3], const double lo[3], const double hi[3], int nsph,
                      const double* centers, const double* radii, const int* sphere_bc,
                      const int grid_bc[6], int scheme, const double alpha[2], double kappa,
                      int sol_kind, const double* params, int nterms, const double* terms,
                      double p_cfl)
{
    auto parts = make_parts(n, lo, hi, nsph, centers, radii, sphere_bc, grid_bc, scheme, alpha);
    const int dims = parts.m.dims();
    manufactured_solution ms;
    if (sol_kind == 1) {
        ms = manufactured_solution{sinsin_mms{params[0], dims}};
    } else if (sol_kind == 4) {
        std::vector<real3> c, v;
        std::vector<real> a, f;
        for (int i = 0; i < nterms; i++) {
            const double* q = terms + 8 * i;
            c.push_back(real3{q[0], q[1], q[2]});
            v.push_back(real3{q[3], q[4], q[5]});
            a.push_back(q[6]);
            f.push_back(q[7]);
        }
        ms = build_ms_gauss(dims, c, v, a, f);
    } else {
        return nullptr;
    }
    auto s = std::make_unique<ref_system>();
    s->p_cfl = p_cfl;
    s->sys = ccs::system{systems::heat{std::move(parts.m), std::move(parts.grid),
                                       std::move(parts.obj), std::move(ms), parts.st, kappa}};
    return finish(std::move(s));
}

// the reference's scalar wave: radial velocity about `center`, exact solution
// sin(2 pi (|x - center| - radius - t)); h_cfl: cfl.hyperbolic
void* ref_wave_create(const int n[3], const double lo[3], const double hi[3], int nsph,
                      const double* centers, const double* radii, const int* sphere_bc,
                      const int grid_bc[6], int scheme, const double alpha[2],
                      const double center[3], double radius, double h_cfl)
{
    auto parts = make_parts(n, lo, hi, nsph, centers, radii, sphere_bc, grid_bc, scheme, alpha);
    auto s = std::make_unique<ref_system>();
    s->h_cfl = h_cfl;
    s->sys = ccs::system{systems::scalar_wave{std::move(parts.m), std::move(parts.grid),
                                              std::move(parts.obj), parts.st,
                                              real3{center[0], center[1], center[2]}, radius,
                                              1e300}};
    return finish(std::move(s));
}

void ref_system_destroy(void* h) { delete static_cast<ref_system*>(h); }

// system::initialize at time t (the solution at fluid points and at every cut point)
void ref_system_initialize(void* h, double t, double* D, double* rx, double* ry, double* rz)
{
    auto* s = static_cast<ref_system*>(h);
    auto c = controller_at(*s, t);
    s->sys.initialize(s->reg, s->u0, c);
    store(*s, s->u0, D, rx, ry, rz);
}

// system::update_boundary at time t on the given state (in place)
void ref_system_update_boundary(void* h, double t, double* D, double* rx, double* ry,
                                double* rz)
{
    auto* s = static_cast<ref_system*>(h);
    load(*s, s->u0, D, rx, ry, rz);
    s->sys.update_boundary(s->reg, s->u0, t);
    store(*s, s->u0, D, rx, ry, rz);
}

// system::rhs at time t (the eager form, heat.cpp:119-162 / scalar_wave.cpp)
void ref_system_rhs(void* h, double t, const double* uD, const double* urx, const double* ury,
                    const double* urz, double* dD, double* drx, double* dry, double* drz)
{
    auto* s = static_cast<ref_system*>(h);
    load(*s, s->u1, uD, urx, ury, urz);
    s->sys.rhs(s->reg, s->u1, s->reg, s->srhs, t);
    store(*s, s->srhs, dD, drx, dry, drz);
}

// nsteps RK4 steps of size dt from time t0, as simulation_cycle::run advances them: the
// boundary update at t0 that precedes its loop (simulation_cycle.cpp:64), then per step the
// integrator, the clock and the copy of u1 into u0
void ref_system_rk4(void* h, double t0, double dt, int nsteps, double* D, double* rx,
                    double* ry, double* rz)
{
    auto* s = static_cast<ref_system*>(h);
    load(*s, s->u0, D, rx, ry, rz);
    s->sys.update_boundary(s->reg, s->u0, t0);
    if (!s->graph_built) {
        s->sys.build_rhs_graph(s->reg, s->u1, s->reg, s->srhs);
        s->graph_built = true;
    }
    auto c = controller_at(*s, t0);
    integrators::rk4 integrate;
    for (int i = 0; i < nsteps; i++) {
        integrate(s->sys, s->reg, s->u0, s->u1, s->rk, s->srhs, c, dt);
        c.advance(dt);
        s->reg.deep_copy_slot(s->u0.slot, s->u1.slot);
    }
    store(*s, s->u0, D, rx, ry, rz);
}

// system::stats at time t: the reference's statistics vector (Linf, min, max, domain Linf
// and index, Rx/Ry/Rz Linf and index); returns the number of entries written
int ref_system_stats(void* h, double t, const double* D, const double* rx, const double* ry,
                     const double* rz, double* out)
{
    auto* s = static_cast<ref_system*>(h);
    load(*s, s->u1, D, rx, ry, rz);
    auto c = controller_at(*s, t);
    auto st = s->sys.stats(s->reg, s->u0, s->u1, c);
    for (std::size_t i = 0; i < st.stats.size(); i++) out[i] = st.stats[i];
    return (int)st.stats.size();
}

// system::timestep_size at the given state
double ref_system_timestep(void* h)
{
    auto* s = static_cast<ref_system*>(h);
    auto c = controller_at(*s, 0.0);
    auto dt = s->sys.timestep_size(s->reg, s->u0, c);
    return dt ? *dt : -1.0;
}

// ---------------------------------------------------------------------------
// Stencils and the sphere intersection
// ---------------------------------------------------------------------------
int ref_stencil_nbs(int scheme, const double* alpha, double h, int bc, double psi,
                    int right, double* c, double* x)
{
    auto st = make(scheme, alpha);
    auto q = st.query(bc_of(bc));
    auto mx = st.query_max();
    std::vector<real> cc(mx.r * mx.t, 0.0), xx(mx.nextra > 0 ? mx.nextra : 1, 0.0);
    st.nbs(h, bc_of(bc), psi, right != 0, cc, xx);
    for (int i = 0; i < q.r * q.t; i++) c[i] = cc[i];
    for (int i = 0; i < q.nextra; i++) x[i] = xx[i];
    return q.r * q.t;
}

int ref_stencil_interior(int scheme, const double* alpha, double h, double* c)
{
    auto st = make(scheme, alpha);
    auto mx = st.query_max();
    std::vector<real> cc(2 * mx.p + 1);
    st.interior(h, cc);
    for (int i = 0; i < 2 * mx.p + 1; i++) c[i] = cc[i];
    return 2 * mx.p + 1;
}

int ref_stencil_interp_wall(int scheme, const double* alpha, int i, double y, double psi,
                            int right, double* c)
{
    auto st = make(scheme, alpha);
    std::vector<real> cc(8, 0.0);
    auto s = st.interp_wall(i, y, psi, cc, right != 0);
    for (size_t k = 0; k < s.size(); k++) c[k] = s[k];
    return (int)s.size();
}

int ref_stencil_interp_interior(int scheme, double y, double* c)
{
    auto st = make(scheme, nullptr);
    std::vector<real> cc(8, 0.0);
    auto s = st.interp_interior(y, cc);
    for (size_t k = 0; k < s.size(); k++) c[k] = s[k];
    return (int)s.size();
}

// sphere::hit on the ray origin + t*direction (src/mesh/sphere.cpp:15-38); returns 1 on a
// hit and fills t, position, ray_outside and the outward normal at the hit point.
int ref_sphere_hit(const double* center, double radius, const double* origin,
                   const double* direction, double t_min, double t_max, double* t,
                   double* pos, int* ray_outside, double* normal)
{
    shape s = make_sphere(0, real3{center[0], center[1], center[2]}, radius);
    ray r{real3{origin[0], origin[1], origin[2]},
          real3{direction[0], direction[1], direction[2]}};
    auto hh = s.hit(r, t_min, t_max);
    if (!hh) return 0;
    *t = hh->t;
    for (int k = 0; k < 3; k++) pos[k] = hh->position[k];
    *ray_outside = hh->ray_outside;
    auto nn = s.normal(hh->position);
    for (int k = 0; k < 3; k++) normal[k] = nn[k];
    return 1;
}
}
