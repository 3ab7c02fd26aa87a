// shoccs_oracle.cpp -- CPU oracle for the SHOCCS derivative-operator / RHS / RK4 path.
//
// TEST INFRASTRUCTURE ONLY.  This file is a plain, serial-by-default restatement of the
// reference algorithm (pbrady/shoccs, C++20 on Kokkos host): the tests compare the CUDA
// product path with it, and it is the timed CPU baseline.  Nothing in the product
// library links, loads or calls it; only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg do.
//
// Every function follows the reference statement by statement, in the same floating-point
// operation order, and cites the reference file:line it restates.  It is compiled with
// -ffp-contract=off so that a*b+c is never fused on either host architecture (x86-64 or
// aarch64), which keeps the setup arithmetic (ray casts, closure coefficients) bit-exact
// with the product host code built the same way.
//
// Parity pins: see tests/test_oracle_golden.py (golden vectors read from the reference's
// own unit tests and from oracle/_ref, which compiles the reference's stencil and sphere
// translation units directly when the reference tree is present).

#include <algorithm>
#include <array>
#include <cassert>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <optional>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc
{
using real = double;
using integer = long;
using int3 = std::array<int, 3>;
using real3 = std::array<real, 3>;

enum bc_type { Dirichlet = 0, Floating = 1, Neumann = 2 };

// ---------------------------------------------------------------------------------------
// real3 helpers: src/real3_operators.hpp:49-84 (dot is a unary RIGHT fold:
// a0*b0 + (a1*b1 + a2*b2)).
// ---------------------------------------------------------------------------------------
static inline real dot3(const real3& a, const real3& b)
{
    return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]);
}
static inline real3 sub3(const real3& a, const real3& b)
{
    return {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
}
static inline real length3(const real3& a) { return std::sqrt(dot3(a, a)); }

// ---------------------------------------------------------------------------------------
// Shapes: src/mesh/sphere.cpp:15-38, src/mesh/shapes.hpp (hit_info)
// ---------------------------------------------------------------------------------------
struct hit_info {
    real t;
    real3 position;
    bool ray_outside;
    int shape_id;
};

struct sphere {
    real3 origin;
    real radius;
    int id;

    std::optional<hit_info>
    hit(const real3& ro, const real3& rd, real t_min, real t_max) const
    {
        const real3 oc = sub3(ro, origin);
        const real a = dot3(rd, rd);
        const real b = dot3(oc, rd);
        const real c = dot3(oc, oc) - radius * radius;
        const real discriminant = b * b - a * c;
        if (discriminant > 0) {
            const real sqr = std::sqrt(discriminant);
            if (real t = (-b - sqr) / a; t > t_min && t < t_max) {
                real3 p{ro[0] + t * rd[0], ro[1] + t * rd[1], ro[2] + t * rd[2]};
                return hit_info{t, p, dot3(rd, sub3(p, origin)) < 0, id};
            }
            if (real t = (-b + sqr) / a; t > t_min && t < t_max) {
                real3 p{ro[0] + t * rd[0], ro[1] + t * rd[1], ro[2] + t * rd[2]};
                return hit_info{t, p, dot3(rd, sub3(p, origin)) < 0, id};
            }
        }
        return std::nullopt;
    }

    real3 normal(const real3& pos) const
    {
        const real3 r = sub3(pos, origin);
        const real d = length3(r);
        return {r[0] / d, r[1] / d, r[2] / d};
    }
};

// src/mesh/mesh_types.hpp:31-38
struct mesh_object_info {
    real psi;
    real3 position;
    real3 normal;
    bool ray_outside;
    int3 solid_coord;
    int shape_id;
};

// src/mesh/mesh_types.hpp:8-23
struct object_boundary {
    integer object_coordinate;
    integer objectID;
    real psi;
};
struct boundary {
    int3 mesh_coordinate;
    std::optional<object_boundary> object;
};
struct line {
    integer stride;
    boundary start;
    boundary end;
};

// src/indexing.hpp:18-36: slow/fast index per direction
static inline int slow_of(int I) { return I == 0 ? 1 : 0; }
static inline int fast_of(int I) { return I == 2 ? 1 : 2; }

struct umesh_line {
    real min, max, h;
    int n;
};

// ---------------------------------------------------------------------------------------
// Mesh: src/mesh/cartesian.cpp:13-44, src/mesh/object_geometry.cpp:17-116,
// src/mesh/mesh.cpp:30-152, src/mesh/mesh.hpp:61-114
// ---------------------------------------------------------------------------------------
struct mesh {
    int3 n;
    real3 lo, hi, h;
    std::vector<real> xyz[3];
    std::vector<sphere> shapes;
    std::vector<mesh_object_info> R[3];
    std::vector<line> lines[3];
    std::vector<std::pair<integer, integer>> fluid_slices;
    std::vector<integer> fluid; // gather list of fluid D indices

    integer size() const { return (integer)n[0] * n[1] * n[2]; }
    integer ic(const int3& ijk) const
    {
        return (integer)ijk[0] * n[1] * n[2] + (integer)ijk[1] * n[2] + ijk[2];
    }
    integer stride(int dir) const
    {
        integer s = 1;
        for (int i = dir + 1; i < 3; i++) s *= n[i];
        return s;
    }
    umesh_line uline(int i) const { return {lo[i], hi[i], h[i], n[i]}; }
    real3 loc(integer idx) const
    {
        int i = (int)(idx / ((integer)n[1] * n[2]));
        int j = (int)((idx / n[2]) % n[1]);
        int k = (int)(idx % n[2]);
        return {xyz[0][i], xyz[1][j], xyz[2][k]};
    }
};

// src/mesh/object_geometry.cpp:17-30
static std::optional<hit_info> closest_hit(const std::vector<sphere>& shapes,
                                           const real3& ro,
                                           const real3& rd,
                                           real t_min,
                                           real t_max)
{
    std::optional<hit_info> global_hit{};
    for (auto&& s : shapes) {
        if (auto current_hit = s.hit(ro, rd, t_min, t_max); current_hit) {
            global_hit = current_hit;
            t_max = current_hit->t;
        }
    }
    return global_hit;
}

// src/mesh/object_geometry.cpp:32-116
static void ray_cast(int I, const std::vector<sphere>& shapes, const umesh_line lines[3],
                     std::vector<mesh_object_info>& info)
{
    const int S = slow_of(I), F = fast_of(I);
    const umesh_line& fline = lines[F];
    const umesh_line& sline = lines[S];
    const umesh_line& iline = lines[I];
    real3 origin{};
    int3 coord{};
    for (int s = 0; s < sline.n; s++) {
        origin[S] = sline.min + s * sline.h;
        coord[S] = s;
        for (int f = 0; f < fline.n; f++) {
            origin[F] = fline.min + f * fline.h;
            coord[F] = f;
            const real min = iline.min, max = iline.max, h = iline.h;
            real t_min{0};
            real t_max{max - min};
            origin[I] = min;
            real3 direction{};
            direction[I] = 1.0;
            while (auto hit = closest_hit(shapes, origin, direction, t_min, t_max)) {
                real t_over_h = hit->t / iline.h;
                int i_cell = static_cast<int>(std::round(t_over_h));
                constexpr real snap_tol = 1e-12;
                if (std::abs(t_over_h - i_cell) > snap_tol)
                    i_cell = static_cast<int>(t_over_h);
                coord[I] = i_cell + hit->ray_outside;
                int off = 1 - 2 * hit->ray_outside;
                real fluid_pos = min + h * (coord[I] + off);
                real psi = off * (fluid_pos - hit->position[I]) / h;
                psi = std::clamp(psi, snap_tol, 1.0 - snap_tol);
                const auto& shp = shapes[hit->shape_id];
                info.push_back(mesh_object_info{psi, hit->position, shp.normal(hit->position),
                                                hit->ray_outside, coord, hit->shape_id});
                t_min = std::nextafter(hit->t, t_max);
            }
        }
    }
}

static bool same_plane(int J, int K, const int3& x, const int3& y)
{
    return x[J] == y[J] && x[K] == y[K];
}

// src/mesh/mesh.cpp:29-87
static void init_lines(int I, std::vector<line>& v, const int3& extents,
                       const std::vector<mesh_object_info>& r, integer stride)
{
    if (extents[I] == 1) return;
    const int S = slow_of(I), F = fast_of(I);
    integer ns = extents[S], nf = extents[F];
    auto first = r.begin();
    auto last = r.end();
    int3 left{}, right{};
    for (integer s = 0; s < ns; s++) {
        left[S] = (int)s;
        right[S] = (int)s;
        for (integer f = 0; f < nf; f++) {
            left[F] = (int)f;
            right[F] = (int)f;
            left[I] = 0;
            right[I] = extents[I] - 1;
            std::optional<boundary> left_boundary = boundary{left, std::nullopt};
            while (first != last && same_plane(S, F, left, first->solid_coord)) {
                object_boundary ob{(integer)(first - r.begin()), first->shape_id, first->psi};
                if (first->ray_outside) {
                    v.push_back(line{stride, *left_boundary,
                                     boundary{first->solid_coord, ob}});
                    left_boundary.reset();
                } else {
                    left_boundary = boundary{first->solid_coord, ob};
                }
                ++first;
            }
            if (left_boundary)
                v.push_back(line{stride, *left_boundary, boundary{right, std::nullopt}});
        }
    }
}

static mesh make_mesh(const int n_in[3], const real lo_in[3], const real hi_in[3],
                      const std::vector<sphere>& shapes)
{
    mesh m;
    for (int i = 0; i < 3; i++) {
        m.n[i] = n_in[i] > 0 ? n_in[i] : 1;
        m.lo[i] = lo_in[i];
        m.hi[i] = hi_in[i];
        // src/mesh/cartesian.cpp:36-37
        m.h[i] = (m.n[i] - 1) ? (m.hi[i] - m.lo[i]) / (m.n[i] - 1)
                              : std::numeric_limits<real>::max();
        // src/fields/lazy_views.hpp:563-569 (linear_distribute)
        m.xyz[i].resize(m.n[i]);
        for (int k = 0; k < m.n[i]; ++k)
            m.xyz[i][k] = m.n[i] > 1 ? m.lo[i] + k * (m.hi[i] - m.lo[i]) / (m.n[i] - 1)
                                     : m.lo[i];
    }
    m.shapes = shapes;
    umesh_line ul[3] = {m.uline(0), m.uline(1), m.uline(2)};
    for (int d = 0; d < 3; d++) ray_cast(d, shapes, ul, m.R[d]);
    for (int d = 0; d < 3; d++) init_lines(d, m.lines[d], m.n, m.R[d], m.stride(d));

    // src/mesh/mesh.cpp:89-111, 134-137
    int fd = m.n[2] > 1 ? 2 : m.n[1] > 1 ? 1 : 0;
    for (auto&& ln : m.lines[fd]) {
        integer i0 = ln.start.object ? m.ic(ln.start.mesh_coordinate) + 1
                                     : m.ic(ln.start.mesh_coordinate);
        integer i1 = ln.end.object ? m.ic(ln.end.mesh_coordinate)
                                   : m.ic(ln.end.mesh_coordinate) + 1;
        if (m.fluid_slices.empty()) {
            m.fluid_slices.emplace_back(i0, i1);
        } else {
            auto& back = m.fluid_slices.back();
            if (back.second == i0)
                back.second = i1;
            else
                m.fluid_slices.emplace_back(i0, i1);
        }
    }
    for (auto&& [a, b] : m.fluid_slices)
        for (integer i = a; i < b; ++i) m.fluid.push_back(i);
    return m;
}

// src/mesh/mesh.cpp:154-168
static bool dirichlet_line(const mesh& m, const int3& start, int dir, const int gbc[3][2])
{
    bool result = false;
    auto f = [&](int i) {
        return (gbc[i][0] == Dirichlet && start[i] == 0) ||
               (gbc[i][1] == Dirichlet && start[i] == m.n[i] - 1);
    };
    for (int i = 0; i < dir; i++) result = result || f(i);
    for (int i = dir + 1; i < 3; i++) result = result || f(i);
    return result;
}

// src/mesh/mesh.cpp:170-207
static line interp_line(const mesh& m, int dir, int3 pt)
{
    int3 l{pt};
    l[dir] = 0;
    int3 r{pt};
    r[dir] = m.n[dir] - 1;
    boundary start{l, std::nullopt};
    boundary end{r, std::nullopt};
    // index::dirs(dir) returns {fast, slow}
    const int f = fast_of(dir), s = slow_of(dir);
    integer i = -1;
    for (auto&& o : m.R[dir]) {
        ++i;
        const auto& ijk = o.solid_coord;
        const auto& nrm = o.normal;
        if (ijk[s] > pt[s]) break;
        if (ijk[s] != pt[s] || ijk[f] != pt[f]) continue;
        if (nrm[dir] >= 0.0 && ijk[dir] <= pt[dir]) {
            if (ijk[dir] >= start.mesh_coordinate[dir])
                start = boundary{ijk, object_boundary{i, o.shape_id, o.psi}};
        } else if (nrm[dir] < 0.0 && ijk[dir] >= pt[dir]) {
            if (ijk[dir] <= end.mesh_coordinate[dir])
                end = boundary{ijk, object_boundary{i, o.shape_id, o.psi}};
        }
    }
    return {m.stride(dir), start, end};
}

// ---------------------------------------------------------------------------------------
// Stencils: src/stencils/stencil.hpp:22-270, E2_2.cpp, E4_2.cpp, E4_1.cpp
// ---------------------------------------------------------------------------------------
struct info {
    int p, r, t, nextra;
};
struct interp_info {
    int p, t;
};

struct stencil {
    int kind = 1; // 0: E2_2, 1: E4_2, 2: E4_1, 3: E4u_1, 5: polyE2_1 (type "E2-poly"),
                  // 6: E6u_1, 7: E8u_1
    real alpha[2] = {0, 0};
    // polyE2_1: floating alpha[6], dirichlet alpha[3], interpolant alpha[4]; E6u_1: alpha[5];
    // E8u_1: alpha[7]
    real pa[13] = {};

    info query_max() const
    {
        switch (kind) {
        case 0: return {1, 2, 4, 2};
        case 1: return {2, 3, 5, 3};
        case 3: return {2, 3, 5, 0};
        case 5: return {1, 3, 4, 0}; // polyE2_1.cpp:11-14
        case 6: return {3, 5, 8, 0};  // E6u_1.cpp:13-16
        case 7: return {4, 7, 11, 0}; // E8u_1.cpp:13-16
        default: return {2, 5, 7, 0};
        }
    }
    info query(int b) const
    {
        info mx = query_max();
        if ((kind == 2 || kind == 3 || kind >= 5) && b == Neumann) return {0, 0, 0, 0};
        switch (b) {
        case Dirichlet: return {mx.p, mx.r - 1, mx.t, 0};
        case Floating: return {mx.p, mx.r, mx.t, 0};
        default: return {mx.p, mx.r, mx.t, mx.nextra};
        }
    }
    interp_info query_interp() const
    {
        switch (kind) {
        case 0: return {2, 3};
        case 1: return {5, 5};
        case 5: return {2, 4}; // polyE2_1.cpp:44
        default: return {0, 0};
        }
    }

    // interior coefficients
    void interior(real h, real* c) const
    {
        if (kind == 0) { // E2_2.cpp:104-111
            c[0] = 1 / (h * h);
            c[1] = -2 / (h * h);
            c[2] = 1 / (h * h);
        } else if (kind == 1) { // E4_2.cpp:33-42
            c[0] = -1 / (12. * (h * h));
            c[1] = 4 / (3. * (h * h));
            c[2] = -5 / (2. * (h * h));
            c[3] = 4 / (3. * (h * h));
            c[4] = -1 / (12. * (h * h));
        } else if (kind == 5) {
            pe2_interior(h, c);
        } else if (kind == 6) { // E6u_1.cpp:49-60
            c[0] = -1 / (60 * h);
            c[1] = 3 / (20 * h);
            c[2] = -3 / (4 * h);
            c[3] = 0;
            c[4] = -c[2];
            c[5] = -c[1];
            c[6] = -c[0];
        } else if (kind == 7) { // E8u_1.cpp:48-61
            c[0] = 1 / (280 * h);
            c[1] = -4 / (105 * h);
            c[2] = 1 / (5 * h);
            c[3] = -4 / (5 * h);
            c[4] = 0;
            c[5] = -c[3];
            c[6] = -c[2];
            c[7] = -c[1];
            c[8] = -c[0];
        } else if (kind == 3) { // E4u_1.cpp:49-58
            c[0] = 1 / (12 * h);
            c[1] = -2 / (3 * h);
            c[2] = 0;
            c[3] = -c[1];
            c[4] = -c[0];
        } else { // E4_1.cpp:66-76
            c[0] = 0.083333333333333329;
            c[1] = -0.66666666666666663;
            c[2] = 0;
            c[3] = 0.66666666666666663;
            c[4] = -0.083333333333333329;
            for (int i = 0; i < 5; i++) c[i] /= h;
        }
    }

    // boundary closure: returns the number of coefficients written (r*t)
    void nbs(real h, int b, real psi, bool right, real* c, real* x) const
    {
        if (kind == 0) {
            if (b == Floating) e22_floating(h, psi, c, right);
            else if (b == Dirichlet) e22_dirichlet(h, psi, c, right);
            else e22_neumann(h, psi, c, x, right);
        } else if (kind == 1) {
            if (b == Floating) e42_floating(h, psi, c, right);
            else if (b == Dirichlet) e42_dirichlet(h, psi, c, right);
            else e42_neumann(h, psi, c, x, right);
        } else if (kind == 3) {
            if (b == Floating) e4u_floating(h, c, right);
            else if (b == Dirichlet) e4u_dirichlet(h, c, right);
        } else if (kind == 5) {
            if (b == Floating) pe2_floating(h, psi, c, right);
            else if (b == Dirichlet) pe2_dirichlet(h, psi, c, right);
        } else if (kind == 6) { // uniform-grid closures, psi ignored
            if (b == Floating) e6u_floating(h, c, right);
            else if (b == Dirichlet) e6u_dirichlet(h, c, right);
        } else if (kind == 7) {
            if (b == Floating) e8u_floating(h, c, right);
            else if (b == Dirichlet) e8u_dirichlet(h, c, right);
        } else {
            if (b == Floating) e41_floating(h, psi, c, right);
            else if (b == Dirichlet) e41_dirichlet(h, psi, c, right);
        }
    }

    // ---- polyE2_1 (type "E2-poly"): src/stencils/polyE2_1.cpp.  Parameters pa[13]: the
    // floating alpha fa = pa[0..5], the dirichlet alpha da = pa[6..8] and the interpolant
    // alpha ia = pa[9..12] (the reference's single-array order, stencil.cpp:79-87).  The
    // closed forms keep the reference's operation order term for term (bit-exact).
    void pe2_interior(real h, real* c) const // polyE2_1.cpp:169-177
    {
        c[0] = -0.5;
        c[1] = 0;
        c[2] = 0.5;
        for (int i = 0; i < 3; i++) c[i] /= h;
    }
    void pe2_floating(real h, real psi, real* c, bool right) const // polyE2_1.cpp:194-230
    {
        const real* fa = pa;
        const real a0 = fa[0], b0 = fa[1], a1 = fa[2], b1 = fa[3], a2 = fa[4], b2 = fa[5];
        const real inv = 1.0 / (1 + psi);
        const real p2 = 2 + psi;
        const real b0m = -1 + b0, b1m = -1 + b1, b2m = -1 + b2;
        c[0] = 0.5 * inv * b0m;
        c[1] = (-1 + a0) * 0.5;
        c[2] = -1 * a0 + -0.5 * p2 * inv * b0m;
        c[3] = (a0 + b0) * 0.5;
        c[4] = 0.5 * b1m * inv;
        c[5] = (-1 + a1) * 0.5;
        c[6] = -1 * a1 + -0.5 * p2 * b1m * inv;
        c[7] = (b1 + a1) * 0.5;
        c[8] = 0.5 * b2m * inv;
        c[9] = (-1 + a2) * 0.5;
        c[10] = -1 * a2 + -0.5 * p2 * b2m * inv;
        c[11] = (b2 + a2) * 0.5;
        for (int i = 0; i < 12; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 12; i++) c[i] *= -1;
            reverse(c, 12);
        }
    }
    void pe2_dirichlet(real h, real psi, real* c, bool right) const // polyE2_1.cpp:232-280
    {
        const real* da = pa + 6;
        const real d0 = da[0], d1 = da[1], d2 = da[2];
        const real inv = 1.0 / (1 + psi);
        const real d0m = -1 + d0;
        const real tp = 2 * psi;
        const real d2x3 = 3 * d2;
        const real tpd2 = 2 * psi * d2;
        const real den = 1.0 / (1 + tp + d2x3 + tpd2);
        const real tpd1 = 2 * psi * d1;
        const real d1d0x3 = 3 * d1 * d0;
        const real tpd1d0 = 2 * psi * d1 * d0;
        const real md1 = -1 * d1;
        const real p2 = 2 + psi;
        const real d2m = -1 + d2;
        c[0] = 0.5 * inv * d0m;
        c[1] = (-1 + -2 * psi + d1 + tpd1 + d1d0x3 + tpd1d0 + -3 * d0 + -2 * psi * d0) * 0.5 * den;
        c[2] = (-2 * psi * d1 + -3 * d2 + -2 * psi * d2 + md1 + 3 * d0 + 2 * psi * d0 +
                -3 * d1 * d0 + -2 * psi * d1 * d0) *
                   den +
               -0.5 * p2 * inv * d0m;
        c[3] = (d1 + tpd1 + d1d0x3 + tpd1d0 + d2x3 + tpd2 + -2 * d0 + 3 * d2 * d0 +
                2 * psi * d2 * d0) *
               0.5 * den;
        c[4] = 0.5 * d2m * inv;
        c[5] = (-1 + d1) * 0.5;
        c[6] = md1 + -0.5 * p2 * d2m * inv;
        c[7] = (d1 + d2) * 0.5;
        for (int i = 0; i < 8; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 8; i++) c[i] *= -1;
            reverse(c, 8);
        }
    }
    int pe2_interp_wall(int i, real y, real psi, real* c, bool right) const // polyE2_1.cpp:58-141
    {
        const real* fa = pa;
        const real* ia = pa + 9;
        const real inv = 1.0 / (1 + psi);
        const real my = -1 * y;
        if (right) {
            if (i == 0) {
                const real f0y = fa[0] * y, f1y = fa[1] * y;
                c[0] = (f0y + f1y + ia[0] + ia[1]) * 0.5;
                c[1] = (-1 * psi + my + (f0y + ia[0]) * -2 +
                        (my + -2 * ia[1] + -1 * psi * ia[1] + -2 * fa[1] * y + -1 * psi * fa[1] * y) *
                            inv) *
                       0.5;
                c[2] = (1 + psi + f0y + ia[0] + y) * 0.5;
                c[3] = (1 + psi + f1y + ia[1] + y) * 0.5 * inv;
            } else {
                const real f2y = fa[2] * y, f3y = fa[3] * y;
                c[0] = (ia[3] + f2y + f3y + ia[2]) * 0.5;
                c[1] = (my + (f2y + ia[2]) * -2 +
                        (psi + -2 * ia[3] + -1 * psi * ia[3] + my + -2 * fa[3] * y +
                         -1 * psi * fa[3] * y) *
                            inv) *
                       0.5;
                c[2] = (1 + f2y + ia[2] + y) * 0.5;
                c[3] = (1 + ia[3] + f3y + y) * 0.5 * inv;
            }
        } else {
            if (i == 0) {
                const real f0y = fa[0] * y, f1y = fa[1] * y;
                c[0] = (1 + psi + ia[1] + my + f1y) * 0.5 * inv;
                c[1] = (1 + psi + f0y + ia[0] + my) * 0.5;
                c[2] = (-1 * psi + (f0y + ia[0]) * -2 + y +
                        (-2 * ia[1] + -1 * psi * ia[1] + y + -2 * fa[1] * y + -1 * psi * fa[1] * y) *
                            inv) *
                       0.5;
                c[3] = (ia[1] + f0y + ia[0] + f1y) * 0.5;
            } else {
                const real f2y = fa[2] * y, f3y = fa[3] * y;
                c[0] = (1 + f3y + ia[3] + my) * 0.5 * inv;
                c[1] = (1 + f2y + ia[2] + my) * 0.5;
                c[2] = ((f2y + ia[2]) * -2 + y +
                        (psi + -2 * ia[3] + -1 * psi * ia[3] + y + -2 * fa[3] * y +
                         -1 * psi * fa[3] * y) *
                            inv) *
                       0.5;
                c[3] = (f3y + ia[3] + f2y + ia[2]) * 0.5;
            }
        }
        return 4;
    }

    // ---- E6u_1, E8u_1 (uniform-grid closures, psi ignored): src/stencils/E6u_1.cpp:78-205,
    // E8u_1.cpp:78-301, the generated expressions term for term
    void e6u_floating(real h, real* c, bool right) const // E6u_1.cpp nbs_floating
    {
        const real* alpha = pa;
        c[0] = (60 * alpha[0] - 137) / 60;
        c[1] = 5 - 6 * alpha[0];
        c[2] = 15 * alpha[0] - 5;
        c[3] = -(60 * alpha[0] - 10) / 3;
        c[4] = (60 * alpha[0] - 5) / 4;
        c[5] = -(30 * alpha[0] - 1) / 5;
        c[6] = alpha[0];
        c[7] = 0;
        c[8] = (5 * alpha[1] - 1) / 5;
        c[9] = -(72 * alpha[1] + 13) / 12;
        c[10] = 15 * alpha[1] + 2;
        c[11] = (-20 * alpha[1]) - 1;
        c[12] = (45 * alpha[1] + 1) / 3;
        c[13] = -(120 * alpha[1] + 1) / 20;
        c[14] = alpha[1];
        c[15] = 0;
        c[16] = (20 * alpha[2] + 1) / 20;
        c[17] = -(12 * alpha[2] + 1) / 2;
        c[18] = (45 * alpha[2] - 1) / 3;
        c[19] = 1 - 20 * alpha[2];
        c[20] = (60 * alpha[2] - 1) / 4;
        c[21] = -(180 * alpha[2] - 1) / 30;
        c[22] = alpha[2];
        c[23] = 0;
        c[24] = (180 * alpha[4] + 30 * alpha[3] - 1) / 30;
        c[25] = -(140 * alpha[4] + 24 * alpha[3] - 1) / 4;
        c[26] = 84 * alpha[4] + 15 * alpha[3] - 1;
        c[27] = -(315 * alpha[4] + 60 * alpha[3] - 1) / 3;
        c[28] = (140 * alpha[4] + 30 * alpha[3] + 1) / 2;
        c[29] = -(420 * alpha[4] + 120 * alpha[3] + 1) / 20;
        c[30] = alpha[3];
        c[31] = alpha[4];
        c[32] = -(190320 * alpha[4] + 31720 * alpha[3] + 22080 * alpha[2] + 38040 * alpha[1] + 9500 * alpha[0] - 453) / 28260;
        c[33] = (55510 * alpha[4] + 9516 * alpha[3] + 6624 * alpha[2] + 11412 * alpha[1] + 2850 * alpha[0] - 159) / 1413;
        c[34] = -(44408 * alpha[4] + 7930 * alpha[3] + 5520 * alpha[2] + 9510 * alpha[1] + 2375 * alpha[0] - 183) / 471;
        c[35] = (166530 * alpha[4] + 31720 * alpha[3] + 22080 * alpha[2] + 38040 * alpha[1] + 9500 * alpha[0] - 1506) / 1413;
        c[36] = -(444080 * alpha[4] + 95160 * alpha[3] + 66240 * alpha[2] + 114120 * alpha[1] + 28500 * alpha[0] - 1323) / 5652;
        c[37] = (55510 * alpha[4] + 15860 * alpha[3] + 11040 * alpha[2] + 19020 * alpha[1] + 4750 * alpha[0] + 1551) / 2355;
        c[38] = -(1586 * alpha[3] + 1104 * alpha[2] + 1902 * alpha[1] + 475 * alpha[0] + 192) / 1413;
        c[39] = -(1586 * alpha[4] - 24) / 1413;
        for (int i = 0; i < 40; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 40; i++) c[i] *= -1;
            reverse(c, 40);
        }
    }
    void e6u_dirichlet(real h, real* c, bool right) const // E6u_1.cpp nbs_dirichlet
    {
        const real* alpha = pa;
        c[0] = (5 * alpha[1] - 1) / 5;
        c[1] = -(72 * alpha[1] + 13) / 12;
        c[2] = 15 * alpha[1] + 2;
        c[3] = (-20 * alpha[1]) - 1;
        c[4] = (45 * alpha[1] + 1) / 3;
        c[5] = -(120 * alpha[1] + 1) / 20;
        c[6] = alpha[1];
        c[7] = 0;
        c[8] = (20 * alpha[2] + 1) / 20;
        c[9] = -(12 * alpha[2] + 1) / 2;
        c[10] = (45 * alpha[2] - 1) / 3;
        c[11] = 1 - 20 * alpha[2];
        c[12] = (60 * alpha[2] - 1) / 4;
        c[13] = -(180 * alpha[2] - 1) / 30;
        c[14] = alpha[2];
        c[15] = 0;
        c[16] = (180 * alpha[4] + 30 * alpha[3] - 1) / 30;
        c[17] = -(140 * alpha[4] + 24 * alpha[3] - 1) / 4;
        c[18] = 84 * alpha[4] + 15 * alpha[3] - 1;
        c[19] = -(315 * alpha[4] + 60 * alpha[3] - 1) / 3;
        c[20] = (140 * alpha[4] + 30 * alpha[3] + 1) / 2;
        c[21] = -(420 * alpha[4] + 120 * alpha[3] + 1) / 20;
        c[22] = alpha[3];
        c[23] = alpha[4];
        c[24] = -(190320 * alpha[4] + 31720 * alpha[3] + 22080 * alpha[2] + 38040 * alpha[1] + 9500 * alpha[0] - 453) / 28260;
        c[25] = (55510 * alpha[4] + 9516 * alpha[3] + 6624 * alpha[2] + 11412 * alpha[1] + 2850 * alpha[0] - 159) / 1413;
        c[26] = -(44408 * alpha[4] + 7930 * alpha[3] + 5520 * alpha[2] + 9510 * alpha[1] + 2375 * alpha[0] - 183) / 471;
        c[27] = (166530 * alpha[4] + 31720 * alpha[3] + 22080 * alpha[2] + 38040 * alpha[1] + 9500 * alpha[0] - 1506) / 1413;
        c[28] = -(444080 * alpha[4] + 95160 * alpha[3] + 66240 * alpha[2] + 114120 * alpha[1] + 28500 * alpha[0] - 1323) / 5652;
        c[29] = (55510 * alpha[4] + 15860 * alpha[3] + 11040 * alpha[2] + 19020 * alpha[1] + 4750 * alpha[0] + 1551) / 2355;
        c[30] = -(1586 * alpha[3] + 1104 * alpha[2] + 1902 * alpha[1] + 475 * alpha[0] + 192) / 1413;
        c[31] = -(1586 * alpha[4] - 24) / 1413;
        for (int i = 0; i < 32; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 32; i++) c[i] *= -1;
            reverse(c, 32);
        }
    }
    void e8u_floating(real h, real* c, bool right) const // E8u_1.cpp nbs_floating
    {
        const real* alpha = pa;
        c[0] = (140 * alpha[0] - 363) / 140;
        c[1] = 7 - 8 * alpha[0];
        c[2] = (56 * alpha[0] - 21) / 2;
        c[3] = -(168 * alpha[0] - 35) / 3;
        c[4] = (280 * alpha[0] - 35) / 4;
        c[5] = -(280 * alpha[0] - 21) / 5;
        c[6] = (168 * alpha[0] - 7) / 6;
        c[7] = -(56 * alpha[0] - 1) / 7;
        c[8] = alpha[0];
        c[9] = 0;
        c[10] = 0;
        c[11] = (7 * alpha[1] - 1) / 7;
        c[12] = -(160 * alpha[1] + 29) / 20;
        c[13] = 28 * alpha[1] + 3;
        c[14] = -(112 * alpha[1] + 5) / 2;
        c[15] = (210 * alpha[1] + 5) / 3;
        c[16] = -(224 * alpha[1] + 3) / 4;
        c[17] = (140 * alpha[1] + 1) / 5;
        c[18] = -(336 * alpha[1] + 1) / 42;
        c[19] = alpha[1];
        c[20] = 0;
        c[21] = 0;
        c[22] = (42 * alpha[2] + 1) / 42;
        c[23] = -(24 * alpha[2] + 1) / 3;
        c[24] = (1680 * alpha[2] - 47) / 60;
        c[25] = -(168 * alpha[2] - 5) / 3;
        c[26] = (420 * alpha[2] - 5) / 6;
        c[27] = -(168 * alpha[2] - 1) / 3;
        c[28] = (336 * alpha[2] - 1) / 12;
        c[29] = -(840 * alpha[2] - 1) / 105;
        c[30] = alpha[2];
        c[31] = 0;
        c[32] = 0;
        c[33] = (105 * alpha[3] - 1) / 105;
        c[34] = -(80 * alpha[3] - 1) / 10;
        c[35] = (140 * alpha[3] - 3) / 5;
        c[36] = -(224 * alpha[3] + 1) / 4;
        c[37] = 70 * alpha[3] + 1;
        c[38] = -(560 * alpha[3] + 3) / 10;
        c[39] = (420 * alpha[3] + 1) / 15;
        c[40] = -(1120 * alpha[3] + 1) / 140;
        c[41] = alpha[3];
        c[42] = 0;
        c[43] = 0;
        c[44] = (140 * alpha[4] + 1) / 140;
        c[45] = -(120 * alpha[4] + 1) / 15;
        c[46] = (280 * alpha[4] + 3) / 10;
        c[47] = (-56 * alpha[4]) - 1;
        c[48] = (280 * alpha[4] + 1) / 4;
        c[49] = -(280 * alpha[4] - 3) / 5;
        c[50] = (280 * alpha[4] - 1) / 10;
        c[51] = -(840 * alpha[4] - 1) / 105;
        c[52] = alpha[4];
        c[53] = 0;
        c[54] = 0;
        c[55] = (840 * alpha[6] + 105 * alpha[5] - 1) / 105;
        c[56] = -(756 * alpha[6] + 96 * alpha[5] - 1) / 12;
        c[57] = (648 * alpha[6] + 84 * alpha[5] - 1) / 3;
        c[58] = -(2520 * alpha[6] + 336 * alpha[5] - 5) / 6;
        c[59] = (1512 * alpha[6] + 210 * alpha[5] - 5) / 3;
        c[60] = -(22680 * alpha[6] + 3360 * alpha[5] - 47) / 60;
        c[61] = (504 * alpha[6] + 84 * alpha[5] + 1) / 3;
        c[62] = -(1512 * alpha[6] + 336 * alpha[5] + 1) / 42;
        c[63] = alpha[5];
        c[64] = alpha[6];
        c[65] = 0;
        c[66] = -(43994496 * alpha[6] + 5499312 * alpha[5] + 3756354 * alpha[4] + 7475328 * alpha[3] + 2303742 * alpha[2] + 7419216 * alpha[1] + 1545558 * alpha[0] - 28865) / 5022570;
        c[67] = (8248968 * alpha[6] + 1047488 * alpha[5] + 715496 * alpha[4] + 1423872 * alpha[3] + 438808 * alpha[2] + 1413184 * alpha[1] + 294392 * alpha[0] - 5917) / 119585;
        c[68] = -(113128704 * alpha[6] + 14664832 * alpha[5] + 10016944 * alpha[4] + 19934208 * alpha[3] + 6143312 * alpha[2] + 19784576 * alpha[1] + 4121488 * alpha[0] - 92067) / 478340;
        c[69] = (164979360 * alpha[6] + 21997248 * alpha[5] + 15025416 * alpha[4] + 29901312 * alpha[3] + 9214968 * alpha[2] + 29676864 * alpha[1] + 6182232 * alpha[0] - 164197) / 358755;
        c[70] = -(131983488 * alpha[6] + 18331040 * alpha[5] + 12521180 * alpha[4] + 24917760 * alpha[3] + 7679140 * alpha[2] + 24730720 * alpha[1] + 5151860 * alpha[0] - 190693) / 239170;
        c[71] = (49493808 * alpha[6] + 7332416 * alpha[5] + 5008472 * alpha[4] + 9967104 * alpha[3] + 3071656 * alpha[2] + 9892288 * alpha[1] + 2060744 * alpha[0] - 163203) / 119585;
        c[72] = -(87988992 * alpha[6] + 14664832 * alpha[5] + 10016944 * alpha[4] + 19934208 * alpha[3] + 6143312 * alpha[2] + 19784576 * alpha[1] + 4121488 * alpha[0] - 169433) / 478340;
        c[73] = (32995872 * alpha[6] + 7332416 * alpha[5] + 5008472 * alpha[4] + 9967104 * alpha[3] + 3071656 * alpha[2] + 9892288 * alpha[1] + 2060744 * alpha[0] + 551009) / 837095;
        c[74] = -(130936 * alpha[5] + 89437 * alpha[4] + 177984 * alpha[3] + 54851 * alpha[2] + 176648 * alpha[1] + 36799 * alpha[0] + 20016) / 119585;
        c[75] = -(130936 * alpha[6] - 4176) / 119585;
        c[76] = -432.0 / 119585;
        for (int i = 0; i < 77; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 77; i++) c[i] *= -1;
            reverse(c, 77);
        }
    }
    void e8u_dirichlet(real h, real* c, bool right) const // E8u_1.cpp nbs_dirichlet
    {
        const real* alpha = pa;
        c[0] = (7 * alpha[1] - 1) / 7;
        c[1] = -(160 * alpha[1] + 29) / 20;
        c[2] = 28 * alpha[1] + 3;
        c[3] = -(112 * alpha[1] + 5) / 2;
        c[4] = (210 * alpha[1] + 5) / 3;
        c[5] = -(224 * alpha[1] + 3) / 4;
        c[6] = (140 * alpha[1] + 1) / 5;
        c[7] = -(336 * alpha[1] + 1) / 42;
        c[8] = alpha[1];
        c[9] = 0;
        c[10] = 0;
        c[11] = (42 * alpha[2] + 1) / 42;
        c[12] = -(24 * alpha[2] + 1) / 3;
        c[13] = (1680 * alpha[2] - 47) / 60;
        c[14] = -(168 * alpha[2] - 5) / 3;
        c[15] = (420 * alpha[2] - 5) / 6;
        c[16] = -(168 * alpha[2] - 1) / 3;
        c[17] = (336 * alpha[2] - 1) / 12;
        c[18] = -(840 * alpha[2] - 1) / 105;
        c[19] = alpha[2];
        c[20] = 0;
        c[21] = 0;
        c[22] = (105 * alpha[3] - 1) / 105;
        c[23] = -(80 * alpha[3] - 1) / 10;
        c[24] = (140 * alpha[3] - 3) / 5;
        c[25] = -(224 * alpha[3] + 1) / 4;
        c[26] = 70 * alpha[3] + 1;
        c[27] = -(560 * alpha[3] + 3) / 10;
        c[28] = (420 * alpha[3] + 1) / 15;
        c[29] = -(1120 * alpha[3] + 1) / 140;
        c[30] = alpha[3];
        c[31] = 0;
        c[32] = 0;
        c[33] = (140 * alpha[4] + 1) / 140;
        c[34] = -(120 * alpha[4] + 1) / 15;
        c[35] = (280 * alpha[4] + 3) / 10;
        c[36] = (-56 * alpha[4]) - 1;
        c[37] = (280 * alpha[4] + 1) / 4;
        c[38] = -(280 * alpha[4] - 3) / 5;
        c[39] = (280 * alpha[4] - 1) / 10;
        c[40] = -(840 * alpha[4] - 1) / 105;
        c[41] = alpha[4];
        c[42] = 0;
        c[43] = 0;
        c[44] = (840 * alpha[6] + 105 * alpha[5] - 1) / 105;
        c[45] = -(756 * alpha[6] + 96 * alpha[5] - 1) / 12;
        c[46] = (648 * alpha[6] + 84 * alpha[5] - 1) / 3;
        c[47] = -(2520 * alpha[6] + 336 * alpha[5] - 5) / 6;
        c[48] = (1512 * alpha[6] + 210 * alpha[5] - 5) / 3;
        c[49] = -(22680 * alpha[6] + 3360 * alpha[5] - 47) / 60;
        c[50] = (504 * alpha[6] + 84 * alpha[5] + 1) / 3;
        c[51] = -(1512 * alpha[6] + 336 * alpha[5] + 1) / 42;
        c[52] = alpha[5];
        c[53] = alpha[6];
        c[54] = 0;
        c[55] = -(43994496 * alpha[6] + 5499312 * alpha[5] + 3756354 * alpha[4] + 7475328 * alpha[3] + 2303742 * alpha[2] + 7419216 * alpha[1] + 1545558 * alpha[0] - 28865) / 5022570;
        c[56] = (8248968 * alpha[6] + 1047488 * alpha[5] + 715496 * alpha[4] + 1423872 * alpha[3] + 438808 * alpha[2] + 1413184 * alpha[1] + 294392 * alpha[0] - 5917) / 119585;
        c[57] = -(113128704 * alpha[6] + 14664832 * alpha[5] + 10016944 * alpha[4] + 19934208 * alpha[3] + 6143312 * alpha[2] + 19784576 * alpha[1] + 4121488 * alpha[0] - 92067) / 478340;
        c[58] = (164979360 * alpha[6] + 21997248 * alpha[5] + 15025416 * alpha[4] + 29901312 * alpha[3] + 9214968 * alpha[2] + 29676864 * alpha[1] + 6182232 * alpha[0] - 164197) / 358755;
        c[59] = -(131983488 * alpha[6] + 18331040 * alpha[5] + 12521180 * alpha[4] + 24917760 * alpha[3] + 7679140 * alpha[2] + 24730720 * alpha[1] + 5151860 * alpha[0] - 190693) / 239170;
        c[60] = (49493808 * alpha[6] + 7332416 * alpha[5] + 5008472 * alpha[4] + 9967104 * alpha[3] + 3071656 * alpha[2] + 9892288 * alpha[1] + 2060744 * alpha[0] - 163203) / 119585;
        c[61] = -(87988992 * alpha[6] + 14664832 * alpha[5] + 10016944 * alpha[4] + 19934208 * alpha[3] + 6143312 * alpha[2] + 19784576 * alpha[1] + 4121488 * alpha[0] - 169433) / 478340;
        c[62] = (32995872 * alpha[6] + 7332416 * alpha[5] + 5008472 * alpha[4] + 9967104 * alpha[3] + 3071656 * alpha[2] + 9892288 * alpha[1] + 2060744 * alpha[0] + 551009) / 837095;
        c[63] = -(130936 * alpha[5] + 89437 * alpha[4] + 177984 * alpha[3] + 54851 * alpha[2] + 176648 * alpha[1] + 36799 * alpha[0] + 20016) / 119585;
        c[64] = -(130936 * alpha[6] - 4176) / 119585;
        c[65] = -432.0 / 119585;
        for (int i = 0; i < 66; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 66; i++) c[i] *= -1;
            reverse(c, 66);
        }
    }

    // ---- E4u_1 (uniform-grid closures, psi ignored): src/stencils/E4u_1.cpp:77-127
    void e4u_floating(real h, real* c, bool right) const
    {
        c[0] = (6 * alpha[0] - 11) / 6;
        c[1] = 3 - 4 * alpha[0];
        c[2] = (12 * alpha[0] - 3) / 2;
        c[3] = -(12 * alpha[0] - 1) / 3;
        c[4] = alpha[0];
        c[5] = (3 * alpha[1] - 1) / 3;
        c[6] = -(8 * alpha[1] + 1) / 2;
        c[7] = 6 * alpha[1] + 1;
        c[8] = -(24 * alpha[1] + 1) / 6;
        c[9] = alpha[1];
        c[10] = -(168 * alpha[1] + 54 * alpha[0] - 11) / 138;
        c[11] = (112 * alpha[1] + 36 * alpha[0] - 15) / 23;
        c[12] = -(336 * alpha[1] + 108 * alpha[0] + 1) / 46;
        c[13] = (336 * alpha[1] + 108 * alpha[0] + 47) / 69;
        c[14] = -(28 * alpha[1] + 9 * alpha[0] + 2) / 23;
        for (int i = 0; i < 15; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 15; i++) c[i] *= -1;
            reverse(c, 15);
        }
    }
    void e4u_dirichlet(real h, real* c, bool right) const
    {
        c[0] = (3 * alpha[1] - 1) / 3;
        c[1] = -(8 * alpha[1] + 1) / 2;
        c[2] = 6 * alpha[1] + 1;
        c[3] = -(24 * alpha[1] + 1) / 6;
        c[4] = alpha[1];
        c[5] = -(168 * alpha[1] + 54 * alpha[0] - 11) / 138;
        c[6] = (112 * alpha[1] + 36 * alpha[0] - 15) / 23;
        c[7] = -(336 * alpha[1] + 108 * alpha[0] + 1) / 46;
        c[8] = (336 * alpha[1] + 108 * alpha[0] + 47) / 69;
        c[9] = -(28 * alpha[1] + 9 * alpha[0] + 2) / 23;
        for (int i = 0; i < 10; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 10; i++) c[i] *= -1;
            reverse(c, 10);
        }
    }

    static void reverse(real* c, int n) { std::reverse(c, c + n); }

    // ---- E2_2: src/stencils/E2_2.cpp:113-186
    static void e22_floating(real h, real psi, real* c, bool right)
    {
        real t6 = psi * psi;
        real t8 = psi * psi * psi;
        real t9 = -1 * t8;
        real t5 = -2 * psi;
        c[0] = psi;
        c[1] = (2 + t5 + -3 * t6 + t9) * 0.5;
        c[2] = -2 + 2 * t6 + t8;
        c[3] = (2 + -1 * t6 + t9) * 0.5;
        c[4] = (2 + 4 * psi) * 1.0 / (2 + 3 * psi + t6);
        c[5] = t5;
        c[6] = (-2 + 4 * t6) * 1.0 / (1 + psi);
        c[7] = (2 + -2 * t6) * 1.0 / (2 + psi);
        for (int i = 0; i < 8; i++) c[i] /= (h * h);
        if (right) reverse(c, 8);
    }
    static void e22_dirichlet(real h, real psi, real* c, bool right)
    {
        real t6 = psi * psi;
        real t5 = -2 * psi;
        c[0] = (2 + 4 * psi) * 1.0 / (2 + 3 * psi + t6);
        c[1] = t5;
        c[2] = (-2 + 4 * t6) * 1.0 / (1 + psi);
        c[3] = (2 + -2 * t6) * 1.0 / (2 + psi);
        for (int i = 0; i < 4; i++) c[i] /= (h * h);
        if (right) reverse(c, 4);
    }
    static void e22_neumann(real h, real psi, real* c, real* x, bool right)
    {
        real t5 = 2 * psi;
        real t9 = psi * psi;
        real t18 = -1 + psi;
        real t23 = psi * psi * psi;
        x[0] = -2;
        x[1] = 2 * t18;
        c[0] = (4 + 8 * psi) * -1 * 1.0 / (2 + 3 * psi + t9);
        c[1] = t5;
        c[2] = (2 + t5 + -4 * t9) * 1.0 / (1 + psi);
        c[3] = 2 * psi * 1.0 / (2 + psi) * t18;
        c[4] = psi;
        c[5] = (-4 + -1 * t23 + t9) * 0.5;
        c[6] = 2 + t23 + -2 * t9;
        c[7] = (2 + -3 * psi + t9) * -0.5 * psi;
        for (int i = 0; i < 8; i++) c[i] /= (h * h);
        for (int i = 0; i < 2; i++) x[i] /= h;
        if (right) {
            reverse(c, 8);
            reverse(x, 2);
            for (int i = 0; i < 2; i++) x[i] *= -1;
        }
    }

    // ---- E4_2: src/stencils/E4_2.cpp:204-311
    static void e42_floating(real h, real psi, real* c, bool right)
    {
        double t6 = -3 * psi;
        double t7 = psi * psi;
        double t9 = t7 * psi;
        double t11 = t7 * t7;
        double t12 = -t11;
        double t18 = 3 * psi;
        double t33 = -1 + psi;
        double t5 = 2 * psi;
        double t31 = 6 * psi;
        c[0] = t5;
        c[1] = (6 + t12 + t6 - 11 * t7 - 6 * t9) / 3.;
        c[2] = -5 + t11 + t6 + 6 * t7 + 5 * t9;
        c[3] = 4 + t12 + t18 - 3 * t7 - 4 * t9;
        c[4] = (-3 + t11 + t6 + 2 * t7 + 3 * t9) / 3.;
        c[5] = 12 / (6 + 5 * psi + t7);
        c[6] = -2 * psi;
        c[7] = -5 + t31;
        c[8] = (-2 * (4 + t18) * t33) / (2 + psi);
        c[9] = (t33 * (3 + t5)) / (3 + psi);
        c[10] = -psi / 12.;
        c[11] = (72 + t11 + t31 + 11 * t7 + 6 * t9) / 72.;
        c[12] = (-48 + t12 - 6 * t7 - 5 * t9) / 24.;
        c[13] = (24 + t11 + 3 * t7 + 4 * t9) / 24.;
        c[14] = -(t7 * (2 + t18 + t7)) / 72.;
        for (int i = 0; i < 15; i++) c[i] /= (h * h);
        if (right) reverse(c, 15);
    }
    static void e42_dirichlet(real h, real psi, real* c, bool right)
    {
        double t7 = psi * psi;
        double t9 = t7 * psi;
        double t11 = t7 * t7;
        double t12 = -t11;
        double t18 = 3 * psi;
        double t33 = -1 + psi;
        double t5 = 2 * psi;
        double t31 = 6 * psi;
        c[0] = 12 / (6 + 5 * psi + t7);
        c[1] = -2 * psi;
        c[2] = -5 + t31;
        c[3] = (-2 * (4 + t18) * t33) / (2 + psi);
        c[4] = (t33 * (3 + t5)) / (3 + psi);
        c[5] = -psi / 12.;
        c[6] = (72 + t11 + t31 + 11 * t7 + 6 * t9) / 72.;
        c[7] = (-48 + t12 - 6 * t7 - 5 * t9) / 24.;
        c[8] = (24 + t11 + 3 * t7 + 4 * t9) / 24.;
        c[9] = -(t7 * (2 + t18 + t7)) / 72.;
        for (int i = 0; i < 10; i++) c[i] /= (h * h);
        if (right) reverse(c, 10);
    }
    static void e42_neumann(real h, real psi, real* c, real* x, bool right)
    {
        double t7 = psi * psi;
        double t10 = 11 * psi;
        double t28 = -1 + psi;
        double t12 = t7 * psi;
        double t36 = t7 * t7;
        double t37 = -t36;
        double t51 = -6 * t7;
        double t8 = 3 * t7;
        x[0] = -3;
        x[1] = 3 * t28;
        x[2] = 0;
        c[0] = (-3 * (7 + 18 * psi + t8)) / (6 + t10 + t12 + 6 * t7);
        c[1] = 4 * psi;
        c[2] = (8 + t10 - 21 * t7) / (2 + 2 * psi);
        c[3] = (-1 - 8 * psi + 9 * t7) / (2 + psi);
        c[4] = (-5 * psi * t28) / (2. * (3 + psi));
        c[5] = psi;
        c[6] = (-21 - 9 * psi + 3 * t12 + t37 + 16 * t7) / 6.;
        c[7] = (8 + 12 * psi - 4 * t12 + t36 - 15 * t7) / 2.;
        c[8] = (-1 - 15 * psi + 5 * t12 + t37 + 12 * t7) / 2.;
        c[9] = (psi * (12 - 7 * psi + t12 + t51)) / 6.;
        c[10] = -psi / 12.;
        c[11] = (72 + 6 * psi + 6 * t12 + t36 + 11 * t7) / 72.;
        c[12] = (-48 - 5 * t12 + t37 + t51) / 24.;
        c[13] = (24 + 4 * t12 + t36 + t8) / 24.;
        c[14] = -(t7 * (2 + 3 * psi + t7)) / 72.;
        for (int i = 0; i < 15; i++) c[i] /= (h * h);
        for (int i = 0; i < 3; i++) x[i] /= h;
        if (right) {
            reverse(c, 15);
            reverse(x, 3);
            for (int i = 0; i < 3; i++) x[i] *= -1;
        }
    }

    // ---- E4_1: src/stencils/E4_1.cpp:95-342
    void e41_floating(real h, real psi, real* c, bool right) const
    {
        constexpr real psi_eps = 1e-4;
        psi = std::clamp(psi, psi_eps, 1.0 - psi_eps);
        real t5 = alpha[1]*psi;
        real t6 = psi * psi;
        real t7 = psi * psi * psi;
        real t8 = std::pow(psi, 4);
        real t9 = std::pow(psi, 5);
        real t10 = std::pow(psi, 6);
        real t11 = std::pow(psi, 7);
        real t12 = alpha[1]*t6;
        real t13 = alpha[1]*t7;
        real t14 = alpha[1]*t8;
        real t15 = alpha[1]*t9;
        real t16 = alpha[1]*t10;
        real t17 = alpha[1]*t11;
        real t18 = alpha[1]*std::pow(psi, 8);
        real t19 = alpha[1] * alpha[1];
        real t20 = psi*t19;
        real t21 = alpha[0]*t12;
        real t22 = alpha[0]*t13;
        real t23 = alpha[0]*t14;
        real t24 = alpha[0]*t15;
        real t25 = alpha[0]*t16;
        real t26 = t19*t6;
        real t27 = 99360*t19;
        real t28 = t19*t9;
        real t29 = alpha[0]*t26;
        real t30 = alpha[0]*t19;
        real t31 = 17280*t30;
        real t32 = 2484*alpha[0]*t17 + 216*alpha[0]*t18 + 3456*alpha[0]*t28 + 10368*alpha[1] + 13872*psi - 414*t10 - 36*t11 + 314677*t12 + 1282709*t13 - 182437*t14 - 496397*t15 - 169230*t16 - 21558*t17 - 1716*t18 + 276480*t20 + 20394*t21 - 94806*t22 + 14166*t23 + 41670*t24 + 15876*t25 + 218592*t26 - t27*t7 - t27*t8 - 19872*t28 - 38016*t29 + t31*t7 + t31*t8 - 184800*t5 + 33753*t6 + 9060*t7 - 6339*t8 - 2988*t9 - 7092;
        real t33 = 1.0 / (alpha[1]);
        real t34 = 1.0 / (psi - 1);
        real t35 = 1.0 / (1728*alpha[1] + 1721*psi + 12*t10 + 864*t12 + 144*t13 + 1584*t5 + 8070*t6 + 5617*t7 + 1464*t8 + 162*t9 - 1182);
        real t36 = t33*t34*t35;
        real t37 = t32*t36;
        real t38 = (1.0 / 6)*t37;
        real t39 = 1.0 / (psi);
        real t40 = t38*t39;
        real t41 = -t40;
        real t42 = -2.0 / 3*t32*t33*t34*t35*t39;
        real t43 = t37*t6;
        real t44 = psi*t37;
        real t45 = t37*t7;
        real t46 = (1.0 / 36)*t45 + (11.0 / 36)*t8;
        real t47 = (7.0 / 12)*t6;
        real t48 = (1.0 / 12)*t45 + (11.0 / 12)*t8;
        real t49 = (5.0 / 36)*t6;
        real t50 = alpha[0]*psi;
        real t51 = 6*alpha[0];
        real t52 = 168*alpha[0]*alpha[1] - 832*alpha[1]*t50 + 342*alpha[1] - 288*psi - 10194*t12 + 4350*t13 + 4671*t14 + 1032*t15 + 33*t16 + t17*t51 + 3*t17 - 756*t19*t50 + 330*t19*t7 + 66*t19*t8 + 5034*t20 - 770*t21 + 274*t22 + 752*t23 + 336*t24 + 66*t25 + 330*t26 + 540*t29 + 540*t30*t7 + 108*t30*t8 - 432*t30 - 5565*t5 - 18*t6 + 72*t7 + 18*t8 - 216;
        real t53 = t36*t52;
        real t54 = 4*t53;
        real t55 = psi*t54;
        real t56 = (1.0 / 3)*psi;
        real t57 = t56 - 1.0 / 3;
        real t58 = t53*t8;
        real t59 = -2.0 / 3*t58;
        real t60 = 16*t53;
        real t61 = psi*t53;
        real t62 = (1.0 / 18)*t8;
        real t63 = -13.0 / 9*psi + (17.0 / 18)*t6 + t62 + (4.0 / 9)*t7;
        real t64 = 24*t53;
        real t65 = t53*t6;
        real t66 = t53*t7;
        real t67 = -2*t58;
        real t68 = (1.0 / 6)*t8;
        real t69 = -19.0 / 6*psi + (11.0 / 6)*t6 + t68 + (7.0 / 6)*t7;
        real t70 = -7.0 / 3*psi + (7.0 / 6)*t6 + t68 + t7;
        real t71 = -11.0 / 18*psi + (5.0 / 18)*t6 + t62 + (5.0 / 18)*t7;
        real t72 = -alpha[0];
        real t73 = -4*alpha[0];
        real t74 = alpha[0]*t7;
        real t75 = alpha[0]*t6;
        real t76 = alpha[0]*t68 + (1.0 / 36)*t8;
        real t77 = (1.0 / 2)*alpha[0]*t8 + (1.0 / 12)*t8;
        real t78 = 6*t50;
        real t79 = psi*t64;
        real t80 = -1.0 / 6*t32*t33*t34*t35;
        real t81 = 2*psi;
        real t82 = (4.0 / 3)*t37;
        real t83 = 8*psi;
        real t84 = t51*t6 + t6*t64 - 149*t6;

        c[0] = (11.0 / 6)*psi + t38 + t41 - 11.0 / 6;
        c[1] = psi*(-t40 - 11.0 / 6);
        c[2] = (143.0 / 18)*psi + (13.0 / 18)*t32*t33*t34*t35 - t42 - 2.0 / 9*t43 - 17.0 / 36*t44 - t46 - 187.0 / 36*t6 - 22.0 / 9*t7 + 3;
        c[3] = -209.0 / 12*psi - t37*t39 + t37*t47 - 19.0 / 12*t37 + (11.0 / 12)*t44 + t48 + (121.0 / 12)*t6 + (77.0 / 12)*t7 - 3.0 / 2;
        c[4] = (77.0 / 6)*psi + (7.0 / 6)*t32*t33*t34*t35 - t42 - 1.0 / 2*t43 - 7.0 / 12*t44 - t48 - 77.0 / 12*t6 - 11.0 / 2*t7 + 1.0 / 3;
        c[5] = -121.0 / 36*psi + t37*t49 - 11.0 / 36*t37 + t41 + (5.0 / 36)*t44 + t46 + (55.0 / 36)*t6 + (55.0 / 36)*t7;
        c[6] = 0;
        c[7] = t54 - t55 + t57;
        c[8] = psi*(t54 - 1.0 / 3);
        c[9] = (34.0 / 3)*t33*t34*t35*t52*t6 + (16.0 / 3)*t33*t34*t35*t52*t7 - t59 - t60 - 52.0 / 3*t61 - t63 - 1.0 / 2;
        c[10] = 38*t61 + t64 - 22*t65 - 14*t66 + t67 + t69 + 1;
        c[11] = 14*t33*t34*t35*t52*t6 + 12*t33*t34*t35*t52*t7 - t60 - 28*t61 - t67 - t70 - 1.0 / 6;
        c[12] = t54 + t59 + (22.0 / 3)*t61 - 10.0 / 3*t65 - 10.0 / 3*t66 + t71;
        c[13] = 0;
        c[14] = -1.0 / 6*psi - t50 - t72 + 1.0 / 6;
        c[15] = psi*(alpha[0] + 1.0 / 6);
        c[16] = -13.0 / 18*psi - 13.0 / 3*t50 + (17.0 / 36)*t6 + (2.0 / 9)*t7 + t73 + (4.0 / 3)*t74 + (17.0 / 6)*t75 + t76 - 1;
        c[17] = (19.0 / 2)*alpha[0]*psi + (19.0 / 12)*psi + t51 - 11.0 / 12*t6 - 7.0 / 12*t7 - 7.0 / 2*t74 - 11.0 / 2*t75 - t77 + 1.0 / 2;
        c[18] = -7.0 / 6*psi + t47 - 7*t50 + (1.0 / 2)*t7 + t73 + 3*t74 + (7.0 / 2)*t75 + t77 + 1.0 / 3;
        c[19] = (11.0 / 6)*alpha[0]*psi + (11.0 / 36)*psi - t49 - 5.0 / 36*t7 - t72 - 5.0 / 6*t74 - 5.0 / 6*t75 - t76;
        c[20] = 0;
        c[21] = t57;
        c[22] = -t56;
        c[23] = 3.0 / 2 - t63;
        c[24] = t69 - 3;
        c[25] = 11.0 / 6 - t70;
        c[26] = t71;
        c[27] = 0;
        c[28] = (-149*psi - t51 - t64 + t78 + t79 - 11)/(11*psi + 6*t6 + t7 + 6);
        c[29] = (149.0 / 6)*psi - t50 - t55 - t80;
        c[30] = (8*alpha[0] - psi*t82 + 3*psi + 2*t50 + t53*t83 + 32*t53 - t82 + t84 + 14)/(t81 + 2);
        c[31] = (-24*alpha[0] + 2*psi*t32*t33*t34*t35 + 4*t32*t33*t34*t35 - 96*t53 - t78 - t79 - t83 - t84 - 38)/(t81 + 4);
        c[32] = (72*alpha[0] - 4*psi*t37 + 15*psi - 12*t37 + 18*t50 + 288*t53 + 72*t61 + t84 + 78)/(6*psi + 18);
        c[33] = -alpha[0] - t54 - t80;
        c[34] = 0;

        for (int i = 0; i < 35; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 35; i++) c[i] *= -1;
            reverse(c, 35);
        }
    }

    void e41_dirichlet(real h, real psi, real* c, bool right) const
    {
        constexpr real psi_eps = 1e-4;
        psi = std::clamp(psi, psi_eps, 1.0 - psi_eps);
        real t5 = alpha[0]*alpha[1];
        real t6 = alpha[1]*psi;
        real t7 = psi * psi;
        real t8 = psi * psi * psi;
        real t9 = std::pow(psi, 4);
        real t10 = alpha[0]*psi;
        real t11 = alpha[1] * alpha[1];
        real t12 = alpha[0]*t11;
        real t13 = alpha[1]*t7;
        real t14 = alpha[1]*t8;
        real t15 = alpha[1]*t9;
        real t16 = std::pow(psi, 5);
        real t17 = alpha[1]*t16;
        real t18 = std::pow(psi, 6);
        real t19 = alpha[1]*t18;
        real t20 = std::pow(psi, 7);
        real t21 = alpha[1]*t20;
        real t22 = psi*t11;
        real t23 = alpha[0]*t13;
        real t24 = alpha[0]*t14;
        real t25 = t5*t9;
        real t26 = t16*t5;
        real t27 = alpha[0]*t19;
        real t28 = 6*alpha[0];
        real t29 = 330*t11;
        real t30 = t11*t9;
        real t31 = 540*t12;
        real t32 = t12*t9;
        real t33 = -832*alpha[1]*t10 + 342*alpha[1] - 288*psi - 756*t10*t11 - 432*t12 - 10194*t13 + 4350*t14 + 4671*t15 + 1032*t17 + 33*t19 + t21*t28 + 3*t21 + 5034*t22 - 770*t23 + 274*t24 + 752*t25 + 336*t26 + 66*t27 + t29*t7 + t29*t8 + 66*t30 + t31*t7 + t31*t8 + 108*t32 + 168*t5 - 5565*t6 - 18*t7 + 72*t8 + 18*t9 - 216;
        real t34 = 1.0 / (alpha[1]);
        real t35 = 1.0 / (psi - 1);
        real t36 = 1.0 / (1728*alpha[1] + 1721*psi + 864*t13 + 144*t14 + 162*t16 + 12*t18 + 1584*t6 + 8070*t7 + 5617*t8 + 1464*t9 - 1182);
        real t37 = t34*t35*t36;
        real t38 = t33*t37;
        real t39 = 4*t38;
        real t40 = psi*t39;
        real t41 = (1.0 / 3)*psi;
        real t42 = t41 - 1.0 / 3;
        real t43 = t38*t9;
        real t44 = -2.0 / 3*t43;
        real t45 = 16*t38;
        real t46 = psi*t38;
        real t47 = (1.0 / 18)*t9;
        real t48 = -13.0 / 9*psi + t47 + (17.0 / 18)*t7 + (4.0 / 9)*t8;
        real t49 = 24*t38;
        real t50 = t38*t7;
        real t51 = t38*t8;
        real t52 = -2*t43;
        real t53 = (1.0 / 6)*t9;
        real t54 = -19.0 / 6*psi + t53 + (11.0 / 6)*t7 + (7.0 / 6)*t8;
        real t55 = -7.0 / 3*psi + t53 + (7.0 / 6)*t7 + t8;
        real t56 = -11.0 / 18*psi + t47 + (5.0 / 18)*t7 + (5.0 / 18)*t8;
        real t57 = -alpha[0];
        real t58 = -4*alpha[0];
        real t59 = alpha[0]*t8;
        real t60 = alpha[0]*t7;
        real t61 = alpha[0]*t53 + (1.0 / 36)*t9;
        real t62 = (1.0 / 2)*alpha[0]*t9 + (1.0 / 12)*t9;
        real t63 = 6*t10;
        real t64 = psi*t49;
        real t65 = std::pow(psi, 8);
        real t66 = 2484*alpha[0]*t21 - 1716*alpha[1]*t65 + 10368*alpha[1] + 13872*psi - 19872*t11*t16 + 218592*t11*t7 - 99360*t11*t8 + 3456*t12*t16 - 38016*t12*t7 + 17280*t12*t8 + 314677*t13 + 1282709*t14 - 182437*t15 - 2988*t16 - 496397*t17 - 414*t18 - 169230*t19 - 36*t20 - 21558*t21 + 276480*t22 + 20394*t23 - 94806*t24 + 14166*t25 + 41670*t26 + 15876*t27 - 99360*t30 + 17280*t32 + 216*t5*t65 - 184800*t6 + 33753*t7 + 9060*t8 - 6339*t9 - 7092;
        real t67 = -1.0 / 6*t34*t35*t36*t66;
        real t68 = 2*psi;
        real t69 = t37*t66;
        real t70 = (4.0 / 3)*t69;
        real t71 = 8*psi;
        real t72 = t28*t7 + t49*t7 - 149*t7;

        c[0] = t39 - t40 + t42;
        c[1] = psi*(t39 - 1.0 / 3);
        c[2] = (34.0 / 3)*t33*t34*t35*t36*t7 + (16.0 / 3)*t33*t34*t35*t36*t8 - t44 - t45 - 52.0 / 3*t46 - t48 - 1.0 / 2;
        c[3] = 38*t46 + t49 - 22*t50 - 14*t51 + t52 + t54 + 1;
        c[4] = 14*t33*t34*t35*t36*t7 + 12*t33*t34*t35*t36*t8 - t45 - 28*t46 - t52 - t55 - 1.0 / 6;
        c[5] = t39 + t44 + (22.0 / 3)*t46 - 10.0 / 3*t50 - 10.0 / 3*t51 + t56;
        c[6] = 0;
        c[7] = -1.0 / 6*psi - t10 - t57 + 1.0 / 6;
        c[8] = psi*(alpha[0] + 1.0 / 6);
        c[9] = -13.0 / 18*psi - 13.0 / 3*t10 + t58 + (4.0 / 3)*t59 + (17.0 / 6)*t60 + t61 + (17.0 / 36)*t7 + (2.0 / 9)*t8 - 1;
        c[10] = (19.0 / 2)*alpha[0]*psi + (19.0 / 12)*psi + t28 - 7.0 / 2*t59 - 11.0 / 2*t60 - t62 - 11.0 / 12*t7 - 7.0 / 12*t8 + 1.0 / 2;
        c[11] = -7.0 / 6*psi - 7*t10 + t58 + 3*t59 + (7.0 / 2)*t60 + t62 + (7.0 / 12)*t7 + (1.0 / 2)*t8 + 1.0 / 3;
        c[12] = (11.0 / 6)*alpha[0]*psi + (11.0 / 36)*psi - t57 - 5.0 / 6*t59 - 5.0 / 6*t60 - t61 - 5.0 / 36*t7 - 5.0 / 36*t8;
        c[13] = 0;
        c[14] = t42;
        c[15] = -t41;
        c[16] = 3.0 / 2 - t48;
        c[17] = t54 - 3;
        c[18] = 11.0 / 6 - t55;
        c[19] = t56;
        c[20] = 0;
        c[21] = (-149*psi - t28 - t49 + t63 + t64 - 11)/(11*psi + 6*t7 + t8 + 6);
        c[22] = (149.0 / 6)*psi - t10 - t40 - t67;
        c[23] = (8*alpha[0] - psi*t70 + 3*psi + 2*t10 + t38*t71 + 32*t38 - t70 + t72 + 14)/(t68 + 2);
        c[24] = (-24*alpha[0] + 2*psi*t34*t35*t36*t66 + 4*t34*t35*t36*t66 - 96*t38 - t63 - t64 - t71 - t72 - 38)/(t68 + 4);
        c[25] = (72*alpha[0] - 4*psi*t69 + 15*psi + 18*t10 + 288*t38 + 72*t46 - 12*t69 + t72 + 78)/(6*psi + 18);
        c[26] = -alpha[0] - t39 - t67;
        c[27] = 0;

        for (int i = 0; i < 28; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 28; i++) c[i] *= -1;
            reverse(c, 28);
        }
    }

    // interpolants: E2_2.cpp:32-102, E4_2.cpp:44-185
    int interp_interior(real y, real* c) const
    {
        if (kind == 0 || kind == 5) { // polyE2_1.cpp:46-56: E2_2's
            if (y > 0) {
                c[0] = 1 + -1 * y;
                c[1] = y;
            } else {
                c[0] = -1 * y;
                c[1] = 1 + y;
            }
            return 2;
        }
        real y2 = y * y;
        real y3 = y * y * y;
        real y4 = y2 * y2;
        c[0] = (y * (2 - y - 2 * y2 + y3)) / 24.;
        c[1] = (y * (-4 + 4 * y + y2 - y3)) / 6.;
        c[2] = (4 - 5 * y2 + y4) / 4.;
        c[3] = -(y * (-4 - 4 * y + y2 + y3)) / 6.;
        c[4] = (y * (-2 - y + 2 * y2 + y3)) / 24.;
        return 5;
    }

    int interp_wall(int i, real y, real psi, real* c, bool right) const
    {
        if (kind == 5) return pe2_interp_wall(i, y, psi, c, right);
        if (kind == 0) {
            if (right) {
                const real t6 = 1 + psi;
                const real t7 = 1.0 / (t6);
                const real t8 = -1 + y;
                const real t9 = psi * t8;
                const real t5 = -1 + psi;
                const real t12 = -1 * psi * y;
                const real t20 = 1 + y;
                switch (i) {
                case 0:
                    c[0] = (psi + y + psi * y) * t5;
                    c[1] = 1 + t12 + -1 * psi * psi * t20 + y;
                    c[2] = psi * t20;
                    break;
                case 1:
                    c[0] = (t9 + y) * t5 * t7;
                    c[1] = psi + t12;
                    c[2] = (1 + t9 + y) * t7;
                    break;
                }
            } else {
                const real t8 = -1 + y;
                const real t11 = psi * y;
                const real t13 = -1 + psi;
                const real t17 = 1 + psi;
                const real t18 = 1.0 / (t17);
                switch (i) {
                case 0:
                    c[0] = psi + -1 * psi * y;
                    c[1] = 1 + t11 + psi * psi * t8 + -1 * y;
                    c[2] = (psi * t8 + y) * -1 * t13;
                    break;
                case 1:
                    c[0] = (-1 + psi + t11 + y) * -1 * t18;
                    c[1] = (1 + y) * psi;
                    c[2] = (psi + t11 + y) * -1 * t13 * t18;
                    break;
                }
            }
            return 3;
        }
        real y2 = y * y;
        real y3 = y2 * y;
        real psi2 = psi * psi;
        real psi3 = psi2 * psi;
        real psi4 = psi2 * psi2;
        if (right) {
            switch (i) {
            case 0:
                c[0] = ((-1 + psi) *
                        (6 * y * (2 + 3 * y + y2) + 6 * psi * (2 + 8 * y + 6 * y2 + y3) +
                         psi3 * (6 + 11 * y + 6 * y2 + y3) +
                         2 * psi2 * (9 + 22 * y + 12 * y2 + 2 * y3))) /
                       36.;
                c[1] = (6 * y * (3 + 4 * y + y2) + 6 * psi * (3 + 8 * y + 3 * y2) -
                        3 * psi2 * (-2 + 5 * y + 6 * y2 + y3) -
                        psi4 * (6 + 11 * y + 6 * y2 + y3) -
                        2 * psi3 * (9 + 22 * y + 12 * y2 + 2 * y3)) /
                       12.;
                c[2] = (-6 * y * (6 + 5 * y + y2) - 6 * psi * (6 + 10 * y + 3 * y2) +
                        6 * psi2 * (1 + 8 * y + 6 * y2 + y3) +
                        psi4 * (6 + 11 * y + 6 * y2 + y3) +
                        psi3 * (24 + 55 * y + 30 * y2 + 5 * y3)) /
                       12.;
                c[3] =
                    (-6 * psi * (-5 - y + 3 * y2 + y3) -
                     6 * psi3 * (5 + 11 * y + 6 * y2 + y3) +
                     6 * (6 + 11 * y + 6 * y2 + y3) - psi4 * (6 + 11 * y + 6 * y2 + y3) -
                     psi2 * (30 + 103 * y + 66 * y2 + 11 * y3)) /
                    36.;
                c[4] = (psi * (6 + 11 * y + 6 * y2 + y3)) / 6.;
                break;
            case 1:
                c[0] = ((-1 + psi) * (psi * (-1 + y) + y) * (2 + 3 * y + y2)) /
                       (2. * (3 + psi));
                c[1] = -((1 + y) * (2 * psi * (3 + y) - 2 * y * (3 + y) +
                                    3 * psi2 * (-2 + y + y2))) /
                       (2. * (2 + psi));
                c[2] = ((2 + y) * (psi * (3 + y) - y * (3 + y) + 3 * psi2 * (-1 + y2))) /
                       (2. * (1 + psi));
                c[3] = (psi * (2 + y - 2 * y2 - y3)) / 2.;
                c[4] = ((3 + 3 * psi * (-1 + y) + y) * (2 + 3 * y + y2)) /
                       (6 + 11 * psi + 6 * psi2 + psi3);
                break;
            default:
                c[0] = (y * (-24 * (-1 + y2) + 2 * psi2 * (-2 - y + 2 * y2 + y3) +
                             3 * psi3 * (-2 - y + 2 * y2 + y3) +
                             psi4 * (-2 - y + 2 * y2 + y3))) /
                       144.;
                c[1] = (y * (24 * (-2 + y + y2) + psi4 * (2 + y - 2 * y2 - y3) -
                             3 * psi2 * (-2 - y + 2 * y2 + y3) -
                             4 * psi3 * (-2 - y + 2 * y2 + y3))) /
                       48.;
                c[2] = ((-24 + 6 * psi2 * y + 5 * psi3 * y + psi4 * y) *
                        (-2 - y + 2 * y2 + y3)) /
                       48.;
                c[3] = -(y * (-24 * (2 + 3 * y + y2) + 6 * psi * (-2 - y + 2 * y2 + y3) +
                              11 * psi2 * (-2 - y + 2 * y2 + y3) +
                              6 * psi3 * (-2 - y + 2 * y2 + y3) +
                              psi4 * (-2 - y + 2 * y2 + y3))) /
                       144.;
                c[4] = (psi * y * (-2 - y + 2 * y2 + y3)) / 24.;
            }
        } else {
            switch (i) {
            case 0:
                c[0] = -(psi * (-6 + 11 * y - 6 * y2 + y3)) / 6.;
                c[1] = (-6 * (-6 + 11 * y - 6 * y2 + y3) +
                        psi4 * (-6 + 11 * y - 6 * y2 + y3) +
                        6 * psi3 * (-5 + 11 * y - 6 * y2 + y3) +
                        6 * psi * (5 - y - 3 * y2 + y3) +
                        psi2 * (-30 + 103 * y - 66 * y2 + 11 * y3)) /
                       36.;
                c[2] = (6 * y * (6 - 5 * y + y2) - 6 * psi * (6 - 10 * y + 3 * y2) +
                        psi3 * (24 - 55 * y + 30 * y2 - 5 * y3) -
                        6 * psi2 * (-1 + 8 * y - 6 * y2 + y3) -
                        psi4 * (-6 + 11 * y - 6 * y2 + y3)) /
                       12.;
                c[3] = (-6 * y * (3 - 4 * y + y2) + 6 * psi * (3 - 8 * y + 3 * y2) +
                        3 * psi2 * (2 + 5 * y - 6 * y2 + y3) +
                        psi4 * (-6 + 11 * y - 6 * y2 + y3) +
                        2 * psi3 * (-9 + 22 * y - 12 * y2 + 2 * y3)) /
                       12.;
                c[4] = -((-1 + psi) * (6 * y * (2 - 3 * y + y2) +
                                       6 * psi * (-2 + 8 * y - 6 * y2 + y3) +
                                       psi3 * (-6 + 11 * y - 6 * y2 + y3) +
                                       2 * psi2 * (-9 + 22 * y - 12 * y2 + 2 * y3))) /
                       36.;
                break;
            case 1:
                c[0] = -(((2 - 3 * y + y2) * (-3 + y + 3 * psi * (1 + y))) /
                         ((1 + psi) * (2 + psi) * (3 + psi)));
                c[1] = (psi * (2 - y - 2 * y2 + y3)) / 2.;
                c[2] = -((-2 + y) *
                         (-(psi * (-3 + y)) - (-3 + y) * y + 3 * psi2 * (-1 + y2))) /
                       (2. * (1 + psi));
                c[3] = ((-1 + y) * (-2 * psi * (-3 + y) - 2 * (-3 + y) * y +
                                    3 * psi2 * (-2 - y + y2))) /
                       (2. * (2 + psi));
                c[4] = -((-1 + psi) * (psi + y + psi * y) * (2 - 3 * y + y2)) /
                       (2. * (3 + psi));
                break;
            default:
                c[0] = (psi * y * (2 - y - 2 * y2 + y3)) / 24.;
                c[1] = -(y * (24 * (2 - 3 * y + y2) + 6 * psi * (2 - y - 2 * y2 + y3) +
                              11 * psi2 * (2 - y - 2 * y2 + y3) +
                              6 * psi3 * (2 - y - 2 * y2 + y3) +
                              psi4 * (2 - y - 2 * y2 + y3))) /
                       144.;
                c[2] = ((24 + 6 * psi2 * y + 5 * psi3 * y + psi4 * y) *
                        (2 - y - 2 * y2 + y3)) /
                       48.;
                c[3] = (y * (24 * (2 + y - y2) + psi4 * (-2 + y + 2 * y2 - y3) -
                             3 * psi2 * (2 - y - 2 * y2 + y3) -
                             4 * psi3 * (2 - y - 2 * y2 + y3))) /
                       48.;
                c[4] = (y * (24 * (-1 + y2) + 2 * psi2 * (2 - y - 2 * y2 + y3) +
                             3 * psi3 * (2 - y - 2 * y2 + y3) +
                             psi4 * (2 - y - 2 * y2 + y3))) /
                       144.;
            }
        }
        return 5;
    }

    // src/stencils/stencil.hpp:213-270
    struct interp_line_t {
        std::vector<real> v;
        boundary left, right;
    };
    interp_line_t interp(int dir, int3 closest, real y, const boundary& left,
                         const boundary& right) const
    {
        const auto [p, t] = query_interp();
        real c[8];
        const int ic = closest[dir];
        const int lc = left.mesh_coordinate[dir];
        const int rc = right.mesh_coordinate[dir];
        int st1 = p & 1 ? (p - 1) / 2 : p / 2;
        int st2 = (p - 1) / 2;
        if (y > 0) std::swap(st1, st2);
        if ((ic - lc > st1 || (ic - lc == st1 && !left.object)) &&
            (rc - ic > st2 || (rc - ic == st2 && !right.object))) {
            int3 l{closest}, r{closest};
            l[dir] -= st1;
            r[dir] += st2;
            int nn = interp_interior(y, c);
            return {std::vector<real>(c, c + nn), boundary{l, std::nullopt},
                    boundary{r, std::nullopt}};
        } else if (ic - lc < rc - ic) {
            int3 r{left.mesh_coordinate};
            r[dir] += t - 1;
            const auto& obj = left.object;
            real psi = obj ? obj->psi : 1.0;
            if (obj && lc == ic) y += psi - 1;
            int nn = interp_wall(ic - lc, y, psi, c, false);
            return {std::vector<real>(c, c + nn), left, boundary{r, std::nullopt}};
        } else {
            int3 l{right.mesh_coordinate};
            l[dir] -= t - 1;
            const auto& obj = right.object;
            real psi = obj ? obj->psi : 1.0;
            if (obj && rc == ic) y += 1 - psi;
            int nn = interp_wall(rc - ic, y, psi, c, true);
            return {std::vector<real>(c, c + nn), boundary{l, std::nullopt}, right};
        }
    }
};

// ---------------------------------------------------------------------------------------
// Matrices: src/matrices/csr.{hpp,cpp}, src/matrices/block.hpp, inner_block.cpp
// ---------------------------------------------------------------------------------------
struct csr {
    std::vector<real> w;
    std::vector<integer> v;
    std::vector<integer> u;
    integer rows() const { return u.size() ? (integer)u.size() - 1 : 0; }

    // src/matrices/csr.cpp:37-51 (always +=)
    void apply(const real* x, real* b) const
    {
        const integer nr = rows();
#pragma omp parallel for schedule(static) if (nr > 65536)
        for (integer row = 0; row < nr; ++row)
            for (integer i = u[row]; i < u[row + 1]; i++) b[row] += w[i] * x[v[i]];
    }
};

struct csr_builder {
    struct pts {
        integer row, col;
        real v;
        bool operator<(const pts& o) const
        {
            if (row != o.row) return row < o.row;
            if (col != o.col) return col < o.col;
            return v < o.v;
        }
    };
    std::vector<pts> p;
    void add_point(integer row, integer col, real v) { p.push_back({row, col, v}); }

    // src/matrices/csr.cpp:10-35 (sort by (row, col, v); defaulted <=>)
    csr to_csr(integer nrows)
    {
        std::vector<integer> u(nrows + 1);
        std::sort(p.begin(), p.end());
        auto first = p.begin();
        auto last = p.end();
        for (integer i = 0; i < nrows; i++) {
            u[i + 1] = u[i];
            while (first != last && first->row == i) {
                ++u[i + 1];
                ++first;
            }
        }
        csr c;
        for (auto& pt : p) {
            c.w.push_back(pt.v);
            c.v.push_back(pt.col);
        }
        c.u = std::move(u);
        return c;
    }
};

// src/matrices/inner_block_meta.hpp:9-23
struct inner_block_meta {
    int row_offset, col_offset, stride, left_rows, left_cols, left_coeff_offset,
        interior_rows, interior_coeff_offset, stencil_width, right_rows, right_cols,
        right_coeff_offset, right_col_offset;
};

struct dense {
    integer rows = 0, cols = 0;
    std::vector<real> v;
};

struct block {
    std::vector<inner_block_meta> meta;
    std::vector<real> coeffs;

    // one line's block: inner_block ctor (src/matrices/inner_block.cpp:73-96) and its
    // entry in block::build_device_arrays (src/matrices/block.hpp:30-94)
    void append_line(integer columns, integer row_offset, integer col_offset, integer stride,
                     const dense& L, integer n_interior, const std::vector<real>& interior,
                     const dense& R)
    {
        inner_block_meta mt{};
        mt.row_offset = (int)row_offset;
        mt.col_offset = (int)col_offset;
        mt.stride = (int)stride;
        mt.left_rows = (int)L.rows;
        mt.left_cols = (int)L.cols;
        mt.left_coeff_offset = (int)coeffs.size();
        coeffs.insert(coeffs.end(), L.v.begin(), L.v.end());
        mt.interior_rows = (int)n_interior;
        mt.interior_coeff_offset = (int)coeffs.size();
        mt.stencil_width = (int)interior.size();
        coeffs.insert(coeffs.end(), interior.begin(), interior.end());
        mt.right_rows = (int)R.rows;
        mt.right_cols = (int)R.cols;
        mt.right_coeff_offset = (int)coeffs.size();
        mt.right_col_offset = (int)(col_offset + stride * (columns - R.cols));
        coeffs.insert(coeffs.end(), R.v.begin(), R.v.end());
        meta.push_back(mt);
    }

    // src/matrices/block.hpp:118-178 with the TeamPolicy flattened to one line per
    // iteration; each row's dot is a sequential j-loop starting from 0.
    template <bool PlusEq>
    void apply(const real* x, real* b) const
    {
        const int n = (int)meta.size();
#pragma omp parallel for schedule(dynamic, 64) if (n > 1024)
        for (int l = 0; l < n; ++l) {
            const auto m = meta[l];
            const int total_rows = m.left_rows + m.interior_rows + m.right_rows;
            for (int local_row = 0; local_row < total_rows; ++local_row) {
                long out_idx;
                real dot = 0;
                if (local_row < m.left_rows) {
                    int r = local_row;
                    out_idx = m.row_offset + (long)r * m.stride;
                    for (int j = 0; j < m.left_cols; ++j)
                        dot += coeffs[m.left_coeff_offset + r * m.left_cols + j] *
                               x[m.col_offset + (long)j * m.stride];
                } else if (local_row < m.left_rows + m.interior_rows) {
                    int r = local_row - m.left_rows;
                    out_idx = m.row_offset + (long)(m.left_rows + r) * m.stride;
                    const int half_w = m.stencil_width / 2;
                    for (int j = 0; j < m.stencil_width; ++j)
                        dot += coeffs[m.interior_coeff_offset + j] *
                               x[out_idx + (long)(j - half_w) * m.stride];
                } else {
                    int r = local_row - m.left_rows - m.interior_rows;
                    out_idx = m.row_offset +
                              (long)(m.left_rows + m.interior_rows + r) * m.stride;
                    for (int j = 0; j < m.right_cols; ++j)
                        dot += coeffs[m.right_coeff_offset + r * m.right_cols + j] *
                               x[m.right_col_offset + (long)j * m.stride];
                }
                if (PlusEq)
                    b[out_idx] += dot;
                else
                    b[out_idx] = dot;
            }
        }
    }
};

// ---------------------------------------------------------------------------------------
// Derivative: src/operators/derivative.cpp:22-473
// ---------------------------------------------------------------------------------------
struct derivative {
    int dir = 0;
    bool active = false;
    block O;
    csr B, N;
    csr Bf[3], Br[3];
};

struct submatrix_size {
    integer rows, columns, row_offset, col_offset, stride, last_row;
    void remove_left_row() { --rows; row_offset += stride; }
    void remove_left_row_col() { remove_left_row(); --columns; col_offset += stride; }
    void remove_right_row() { --rows; }
    void remove_right_row_col() { remove_right_row(); --columns; }
    integer left_row(integer row = 0) const { return row_offset + stride * row; }
    integer right_row(integer row = 0) const { return last_row + stride * row; }
};

// src/operators/derivative.cpp:305-449
static void domain_discretization(int dir, const mesh& m, const stencil& st,
                                  const int gbc[3][2], const std::vector<int>& obc,
                                  derivative& D, const std::vector<real>& interior)
{
    auto mx = st.query_max();
    const real h = m.h[dir];
    std::vector<real> left(mx.r * mx.t), right(mx.r * mx.t), extra(std::max(mx.nextra, 1));
    csr_builder B_builder, N_builder;

    for (auto&& ln : m.lines[dir]) {
        const auto& start = ln.start;
        const auto& end = ln.end;
        const integer stride = ln.stride;
        if (dirichlet_line(m, start.mesh_coordinate, dir, gbc)) continue;

        submatrix_size sub;
        sub.rows = end.mesh_coordinate[dir] - start.mesh_coordinate[dir] + 1;
        sub.columns = sub.rows;
        sub.row_offset = m.ic(start.mesh_coordinate);
        sub.col_offset = sub.row_offset;
        sub.stride = stride;
        sub.last_row = m.ic(end.mesh_coordinate);

        dense leftMat{}, rightMat{};
        if (const auto& obj = start.object; obj) {
            const int bc_t = obc[obj->objectID];
            auto q = st.query(bc_t);
            st.nbs(h, bc_t, obj->psi, false, left.data(), extra.data());
            int s = bc_t != Dirichlet;
            int rL = q.r - s;
            const real* lc = left.data() + s * q.t;
            leftMat.rows = rL;
            leftMat.cols = q.t - 1;
            for (int row = 0; row < rL; ++row)
                for (int j = 1; j < q.t; ++j) leftMat.v.push_back(lc[row * q.t + j]);
            sub.remove_left_row_col();
            for (int row = 0; row < rL; ++row)
                B_builder.add_point(sub.left_row(row), obj->object_coordinate, lc[row * q.t]);
        } else {
            const int bc = gbc[dir][0];
            auto q = st.query(bc);
            st.nbs(h, bc, 1.0, false, left.data(), extra.data());
            leftMat.rows = q.r;
            leftMat.cols = q.t;
            leftMat.v.assign(left.begin(), left.begin() + q.r * q.t);
            if (bc == Dirichlet) {
                sub.remove_left_row();
            } else if (bc == Neumann) {
                for (int row = 0; row < q.nextra; row++)
                    N_builder.add_point(sub.left_row(row), sub.left_row(), extra[row]);
            }
        }

        if (const auto& obj = end.object; obj) {
            const int bc_t = obc[obj->objectID];
            auto q = st.query(bc_t);
            st.nbs(h, bc_t, obj->psi, true, right.data(), extra.data());
            integer s = bc_t != Dirichlet;
            int rR = q.r - (int)s;
            const real* rc = right.data();
            rightMat.rows = rR;
            rightMat.cols = q.t - 1;
            for (int row = 0; row < rR; ++row)
                for (int j = 0; j < q.t - 1; ++j) rightMat.v.push_back(rc[row * q.t + j]);
            sub.remove_right_row_col();
            for (int row = 0; row < rR; ++row)
                B_builder.add_point(sub.right_row(row - rR), obj->object_coordinate,
                                    rc[row * q.t + q.t - 1]);
        } else {
            const int bc = gbc[dir][1];
            auto q = st.query(bc);
            st.nbs(h, bc, 1.0, true, right.data(), extra.data());
            rightMat.rows = q.r;
            rightMat.cols = q.t;
            rightMat.v.assign(right.begin(), right.begin() + q.r * q.t);
            if (bc == Dirichlet) {
                sub.remove_right_row();
            } else if (bc == Neumann) {
                for (int row = 0; row < q.nextra; row++)
                    N_builder.add_point(sub.right_row(row - q.nextra + 1), sub.right_row(),
                                        extra[row]);
            }
        }
        const integer n_interior = sub.rows - leftMat.rows - rightMat.rows;
        D.O.append_line(sub.columns, sub.row_offset, sub.col_offset, stride, leftMat,
                        n_interior, interior, rightMat);
    }
    D.B = B_builder.to_csr(m.size());
    D.N = N_builder.to_csr(m.size());
}

// src/operators/derivative.cpp:22-70
struct interp_deriv_info {
    std::vector<real> c;
    int offset;
};
static interp_deriv_info interp_deriv_coefficients(int dir, int n, real h,
                                                   const mesh_object_info& obj, int bc,
                                                   const stencil& st)
{
    auto q = st.query(bc);
    const int p = q.p, r = q.r, t = q.t;
    std::vector<real> c(128), ex(8);
    if (std::abs(obj.normal[dir]) > 1e-12) {
        const bool right_interp_wall = obj.normal[dir] < 0.0;
        st.nbs(h, bc, 1.0, right_interp_wall, c.data(), ex.data());
        if (right_interp_wall)
            return {std::vector<real>(c.begin() + (r - 1) * t, c.begin() + r * t), 1 - t};
        else
            return {std::vector<real>(c.begin(), c.begin() + t), 0};
    } else {
        auto right_dist = n - obj.solid_coord[dir];
        auto left_dist = obj.solid_coord[dir];
        if (right_dist >= p && left_dist >= p) {
            st.interior(h, c.data());
            return {std::vector<real>(c.begin(), c.begin() + 2 * p + 1), -p};
        } else {
            const bool right_interp_wall = right_dist < left_dist;
            st.nbs(h, bc, 1.0, right_interp_wall, c.data(), ex.data());
            if (right_interp_wall) {
                auto qq = 1 + right_dist;
                return {std::vector<real>(c.begin() + (r - qq) * t,
                                          c.begin() + (r - qq) * t + t),
                        qq - t};
            } else {
                auto qq = left_dist;
                return {std::vector<real>(c.begin() + qq * t, c.begin() + qq * t + t), -qq};
            }
        }
    }
}

// src/operators/derivative.cpp:159-257
static void cut_discretization(int r, int dir, const mesh& m, const stencil& st,
                               const std::vector<int>& obc, csr& O, csr& B)
{
    const auto& shapes = m.R[r];
    const integer sz = (integer)shapes.size();
    bool all_dir = std::all_of(obc.begin(), obc.end(), [](int b) { return b == Dirichlet; });
    if (sz == 0 || all_dir) return;

    auto mx = st.query_max();
    const real h = m.h[dir];
    csr_builder Ob, Bb;
    std::vector<real> c(mx.r * mx.t), extra(std::max(mx.nextra, 1));
    const integer stride = m.stride(dir);

    if (dir == r) {
        for (integer shape_row = 0; shape_row < sz; ++shape_row) {
            const auto& obj = shapes[shape_row];
            int bc_t = obc[obj.shape_id];
            if (bc_t == Dirichlet) continue;
            auto q = st.query(bc_t);
            st.nbs(h, bc_t, obj.psi, obj.ray_outside, c.data(), extra.data());
            std::vector<real> rng;
            integer sgn;
            if (obj.ray_outside) {
                rng.assign(c.begin() + (q.r - 1) * q.t, c.begin() + q.r * q.t);
                std::reverse(rng.begin(), rng.end());
                sgn = -stride;
            } else {
                rng.assign(c.begin(), c.begin() + q.t);
                sgn = stride;
            }
            // OB_builder::add_cut_row: derivative.cpp:76-82
            const integer solid_ic = m.ic(obj.solid_coord);
            Bb.add_point(shape_row, shape_row, rng[0]);
            for (int i = 1; i < (int)rng.size(); ++i)
                Ob.add_point(shape_row, solid_ic + i * sgn, rng[i]);
        }
    } else {
        for (integer shape_row = 0; shape_row < sz; ++shape_row) {
            const auto& obj = shapes[shape_row];
            int bc_t = obc[obj.shape_id];
            if (bc_t == Dirichlet) continue;
            auto idc = interp_deriv_coefficients(dir, m.n[dir] - 1, h, obj, bc_t, st);
            int3 cp = obj.solid_coord;
            if (obj.psi <= 0.5) cp[r] += 1 - 2 * obj.ray_outside;
            cp[dir] += idc.offset;
            const real y = (obj.ray_outside ? 1.0 : -1.0) *
                           (obj.psi <= 0.5 ? obj.psi : obj.psi - 1);
            for (auto&& v : idc.c) {
                if (cp[dir] == obj.solid_coord[dir]) {
                    Bb.add_point(shape_row, shape_row, v);
                } else {
                    line il = interp_line(m, r, cp);
                    auto itp = st.interp(r, cp, y, il.start, il.end);
                    // OB_builder::add_interp_row: derivative.cpp:91-135
                    const integer left_ic = m.ic(itp.left.mesh_coordinate);
                    const integer right_ic = m.ic(itp.right.mesh_coordinate);
                    auto it = itp.v.begin();
                    if (const auto& o = itp.left.object; o)
                        Bb.add_point(shape_row, o->object_coordinate, v * *it);
                    else
                        Ob.add_point(shape_row, left_ic, v * *it);
                    ++it;
                    for (integer ic = left_ic + il.stride; ic < right_ic; ic += il.stride) {
                        Ob.add_point(shape_row, ic, v * *it);
                        ++it;
                    }
                    if (const auto& o = itp.right.object; o)
                        Bb.add_point(shape_row, o->object_coordinate, v * *it);
                    else
                        Ob.add_point(shape_row, right_ic, v * *it);
                }
                ++cp[dir];
            }
        }
    }
    O = Ob.to_csr(sz);
    B = Bb.to_csr(sz);
}

static derivative make_derivative(int dir, const mesh& m, const stencil& st,
                                  const int gbc[3][2], const std::vector<int>& obc)
{
    derivative D;
    D.dir = dir;
    if (m.n[dir] < 2) return D;
    D.active = true;
    auto mx = st.query_max();
    std::vector<real> interior(2 * mx.p + 1);
    st.interior(m.h[dir], interior.data());
    domain_discretization(dir, m, st, gbc, obc, D, interior);
    for (int r = 0; r < 3; r++) cut_discretization(r, dir, m, st, obc, D.Bf[r], D.Br[r]);
    return D;
}

// a scalar field {D, Rx, Ry, Rz}: src/fields/scalar.hpp:13-67
struct sfield {
    real* D;
    real* R[3];
};
struct cfield {
    const real* D;
    const real* R[3];
};

// src/operators/derivative.cpp:475-519
template <bool PlusEq>
static void apply_derivative(const derivative& Dv, cfield u, const real* nuD, sfield du)
{
    if (!Dv.active) return;
    for (int r = 0; r < 3; r++) Dv.Bf[r].apply(u.D, du.R[r]);
    for (int r = 0; r < 3; r++) Dv.Br[r].apply(u.R[r], du.R[r]);
    Dv.O.apply<PlusEq>(u.D, du.D);
    Dv.B.apply(u.R[Dv.dir], du.D);
    if (nuD) Dv.N.apply(nuD, du.D);
}

// ---------------------------------------------------------------------------------------
// Exact solutions / MMS (closed forms).  gaussian: src/mms/gauss{1,2,3}d.cpp; the
// remaining kinds are the restated extensions needed by the benchmark configurations.
// ---------------------------------------------------------------------------------------
enum sol_kind {
    SOL_ZERO = 0,        // u = 0
    SOL_SINSIN = 1,      // u = prod_d sin(2 pi k x_d) * exp(-t) over the active dims
    SOL_GAUSS_PULSE = 2, // u = exp(-|x - x0 - a t|^2 / (2 sigma^2))
    SOL_RADIAL_SIN = 3,  // u = sin(2 pi (|x - c| - r - t))   (scalar_wave.cpp:35-40)
    SOL_GAUSSIAN = 4,    // u = sum_i A_i cos(f_i t) exp(-1/2 sum_{d<D} (x_d - c_id)^2 / s_id^2)
                         //   (src/mms/gauss1d.cpp:10-68, gauss2d.cpp:10-87, gauss3d.cpp:10-122)
};

// the Gaussian sum of SOL_GAUSSIAN and its derivatives at (t, x): D = the mesh's dimension
// count, term i = G[8i..8i+7] = centre[3], variance[3], amplitude A, frequency f.  The
// reference's gauss{1,2,3}d spell the same functions out per dimension count.
struct gauss_terms {
    real u = 0, ddt = 0, lap = 0, grad[3] = {0, 0, 0};
};
static gauss_terms gauss_eval(const std::vector<real>& G, int D, real t, const real3& x)
{
    gauss_terms r;
    for (size_t i = 0; i + 8 <= G.size(); i += 8) {
        const real* g = G.data() + i;
        real e = 0.0, lp = 0.0, dv[3] = {0.0, 0.0, 0.0};
        for (int d = 0; d < D; d++) {
            const real dx = x[d] - g[d];
            const real is2 = 1.0 / (g[3 + d] * g[3 + d]);
            e = e - 0.5 * (dx * dx) * is2;
            dv[d] = dx * is2;
            lp = lp + (dv[d] * dv[d] - is2);
        }
        const real E = std::exp(e);
        const real ac = g[6] * std::cos(g[7] * t) * E;
        r.u = r.u + ac;
        r.ddt = r.ddt - g[6] * g[7] * std::sin(g[7] * t) * E;
        r.lap = r.lap + ac * lp;
        for (int d = 0; d < 3; d++) r.grad[d] = r.grad[d] - ac * dv[d];
    }
    return r;
}

struct solution {
    int kind = SOL_ZERO;
    int dims = 3;
    real p[8] = {0};
    std::vector<real> G; // SOL_GAUSSIAN terms
    int gdims = 0;       // SOL_GAUSSIAN: the mesh's dimension count
    // SINSIN: p[0] = k ; GAUSS_PULSE: p[0..2] = x0, p[3..5] = a, p[6] = sigma;
    // RADIAL_SIN: p[0..2] = c, p[3] = r

    real operator()(real t, const real3& x) const
    {
        constexpr real twoPI = 2 * 3.14159265358979323846;
        switch (kind) {
        case SOL_SINSIN: {
            real v = std::sin(twoPI * p[0] * x[0]) * std::sin(twoPI * p[0] * x[1]);
            if (dims == 3) v = v * std::sin(twoPI * p[0] * x[2]);
            return v * std::exp(-t);
        }
        case SOL_GAUSS_PULSE: {
            real d0 = x[0] - p[0] - p[3] * t;
            real d1 = x[1] - p[1] - p[4] * t;
            real d2 = x[2] - p[2] - p[5] * t;
            real r2 = d0 * d0 + d1 * d1 + d2 * d2;
            return std::exp(-r2 / (2 * p[6] * p[6]));
        }
        case SOL_RADIAL_SIN: {
            real3 d{x[0] - p[0], x[1] - p[1], x[2] - p[2]};
            return std::sin(twoPI * (length3(d) - p[3] - t));
        }
        case SOL_GAUSSIAN: return gauss_eval(G, gdims, t, x).u;
        default: return 0.0;
        }
    }
    real ddt(real t, const real3& x) const
    {
        if (kind == SOL_SINSIN) return -(*this)(t, x);
        if (kind == SOL_GAUSSIAN) return gauss_eval(G, gdims, t, x).ddt;
        return 0.0;
    }
    real laplacian(real t, const real3& x) const
    {
        if (kind == SOL_GAUSSIAN) return gauss_eval(G, gdims, t, x).lap;
        if (kind == SOL_SINSIN) {
            constexpr real twoPI = 2 * 3.14159265358979323846;
            real kk = twoPI * p[0];
            return -(real)dims * kk * kk * (*this)(t, x);
        }
        return 0.0;
    }
    // component dir of the gradient (manufactured_solution::gradient, the Neumann data of
    // heat::update_boundary, src/systems/heat.cpp:324-352); the heat systems here use the
    // sin-sin solution or zero
    real gradient(real t, const real3& x, int dir) const
    {
        if (kind == SOL_GAUSSIAN) return gauss_eval(G, gdims, t, x).grad[dir];
        if (kind != SOL_SINSIN) return 0.0;
        constexpr real twoPI = 2 * 3.14159265358979323846;
        const real kk = twoPI * p[0];
        real v = 1.0;
        for (int d = 0; d < dims; d++)
            v = v * (d == dir ? kk * std::cos(kk * x[d]) : std::sin(kk * x[d]));
        return v * std::exp(-t);
    }
};

// ---------------------------------------------------------------------------------------
// Systems: heat (src/systems/heat.cpp) and scalar_wave (src/systems/scalar_wave.cpp)
// ---------------------------------------------------------------------------------------
struct problem {
    mesh m;
    stencil st;
    int gbc[3][2];
    std::vector<int> obc;
    derivative D[3];
};

struct field_buf {
    std::vector<real> D, R[3];
    void resize(const mesh& m)
    {
        D.assign(m.size(), 0.0);
        for (int d = 0; d < 3; d++) R[d].assign(m.R[d].size(), 0.0);
    }
    sfield span() { return {D.data(), {R[0].data(), R[1].data(), R[2].data()}}; }
    cfield view() const { return {D.data(), {R[0].data(), R[1].data(), R[2].data()}}; }
    void zero()
    {
        std::fill(D.begin(), D.end(), 0.0);
        for (int d = 0; d < 3; d++) std::fill(R[d].begin(), R[d].end(), 0.0);
    }
};

// src/fields/selection_desc.hpp:211-222 (for_each_grid_bc_desc)
template <typename F>
static void for_each_dirichlet_face(const problem& P, F&& fn)
{
    const auto& n = P.m.n;
    for (int d = 0; d < 3; d++) {
        for (int side = 0; side < 2; side++) {
            if (P.gbc[d][side] != Dirichlet) continue;
            int face = side == 0 ? 0 : n[d] - 1;
            for (int i = 0; i < n[0]; i++)
                for (int j = 0; j < n[1]; j++)
                    for (int k = 0; k < n[2]; k++) {
                        int3 ijk{i, j, k};
                        if (ijk[d] == face) fn(P.m.ic(ijk));
                    }
        }
    }
}

// eval_at_locations: src/systems/detail/scalar_system_utils.hpp:16-73
template <typename F>
static void eval_at_locations(const mesh& m, F&& f, field_buf& out)
{
    const integer N = m.size();
#pragma omp parallel for schedule(static) if (N > 65536)
    for (integer idx = 0; idx < N; ++idx) out.D[idx] = f(m.loc(idx));
    for (int d = 0; d < 3; d++)
        for (size_t i = 0; i < m.R[d].size(); ++i) out.R[d][i] = f(m.R[d][i].position);
}

struct heat_sys {
    problem* P;
    real k;
    solution sol;
    field_buf neu, src;

    // Neumann data of heat::update_boundary (heat.cpp:324-352): the gradient component of
    // the axis on that axis' Neumann faces, axes in order, so at an edge shared with a later
    // axis' Neumann face the later axis' value stays.  update_boundary runs at every stage
    // time before the right-hand side (and simulation_cycle runs it once after initialize),
    // so the data a right-hand side sees is the one at its own time.
    void fill_neumann(real time)
    {
        const mesh& m = P->m;
        const auto& n = m.n;
        if ((integer)neu.D.size() != m.size()) neu.resize(m);
        for (int d = 0; d < 3; d++)
            for (int side = 0; side < 2; side++) {
                if (P->gbc[d][side] != Neumann) continue;
                const int face = side == 0 ? 0 : n[d] - 1;
                for (int i = 0; i < n[0]; i++)
                    for (int j = 0; j < n[1]; j++)
                        for (int k = 0; k < n[2]; k++) {
                            const int3 ijk{i, j, k};
                            if (ijk[d] != face) continue;
                            const integer idx = m.ic(ijk);
                            neu.D[idx] = sol.gradient(time, m.loc(idx), d);
                        }
            }
    }

    // heat::build_rhs_graph order: src/systems/heat.cpp:164-288
    void rhs(cfield u, sfield du, real time)
    {
        const mesh& m = P->m;
        fill_neumann(time);
        // fill_source: heat.cpp:111-117
        eval_at_locations(m, [&](const real3& loc) {
            return sol.ddt(time, loc) - k * sol.laplacian(time, loc);
        }, src);
        // laplacian with Neumann data: laplacian.cpp:48-58
        std::fill(du.D, du.D + m.size(), 0.0);
        for (int d = 0; d < 3; d++) std::fill(du.R[d], du.R[d] + m.R[d].size(), 0.0);
        for (int d = 0; d < 3; d++)
            if (m.n[d] > 1) apply_derivative<true>(P->D[d], u, neu.D.data(), du);
        const integer N = m.size();
        for (integer i = 0; i < N; i++) du.D[i] *= k;
        for (int d = 0; d < 3; d++)
            for (size_t i = 0; i < m.R[d].size(); i++) du.R[d][i] *= k;
        for (integer i : m.fluid) du.D[i] += src.D[i];
        for (int d = 0; d < 3; d++)
            for (size_t i = 0; i < m.R[d].size(); i++)
                if (P->obc[m.R[d][i].shape_id] != Dirichlet) du.R[d][i] += src.R[d][i];
        for_each_dirichlet_face(*P, [&](integer i) { du.D[i] = 0; });
        for (int d = 0; d < 3; d++)
            for (size_t i = 0; i < m.R[d].size(); i++)
                if (P->obc[m.R[d][i].shape_id] == Dirichlet) du.R[d][i] = 0;
    }

    // heat::update_boundary: src/systems/heat.cpp:296-354
    void update_boundary(sfield u, real time)
    {
        const mesh& m = P->m;
        for_each_dirichlet_face(*P, [&](integer i) { u.D[i] = sol(time, m.loc(i)); });
        for (int d = 0; d < 3; d++)
            for (size_t i = 0; i < m.R[d].size(); i++)
                if (P->obc[m.R[d][i].shape_id] == Dirichlet)
                    u.R[d][i] = sol(time, m.R[d][i].position);
        // Neumann faces are not exercised by the closed-form solutions supported here.
    }
};

struct wave_sys {
    problem* P;
    int vel_kind = 0; // 0: constant velocity a (gG = -a), 1: radial (scalar_wave.cpp:28-33)
    real vel[3] = {0, 0, 0};
    real3 center{0, 0, 0};
    solution sol;
    field_buf gG[3], dux, duy, duz;

    void init()
    {
        const mesh& m = P->m;
        for (int c = 0; c < 3; c++) {
            gG[c].resize(m);
            if (vel_kind == 1) {
                real3 cc = center;
                eval_at_locations(m, [&](const real3& loc) {
                    return -(loc[c] - cc[c]) / length3(sub3(loc, cc));
                }, gG[c]);
            } else {
                real a = vel[c];
                eval_at_locations(m, [&](const real3&) { return -a; }, gG[c]);
            }
            // scalar_wave.cpp:79-95
            for_each_dirichlet_face(*P, [&](integer i) { gG[c].D[i] = 0.0; });
            for (int d = 0; d < 3; d++)
                for (size_t i = 0; i < m.R[d].size(); i++)
                    if (P->obc[m.R[d][i].shape_id] == Dirichlet) gG[c].R[d][i] = 0.0;
        }
        dux.resize(m);
        duy.resize(m);
        duz.resize(m);
    }

    // scalar_wave::build_rhs_graph: src/systems/scalar_wave.cpp:241-321
    void rhs(cfield u, sfield du, real)
    {
        const mesh& m = P->m;
        dux.zero();
        duy.zero();
        duz.zero();
        if (m.n[0] > 1) apply_derivative<false>(P->D[0], u, nullptr, dux.span());
        if (m.n[1] > 1) apply_derivative<false>(P->D[1], u, nullptr, duy.span());
        if (m.n[2] > 1) apply_derivative<false>(P->D[2], u, nullptr, duz.span());
        const integer N = m.size();
#pragma omp parallel for schedule(static) if (N > 65536)
        for (integer i = 0; i < N; i++)
            du.D[i] = gG[0].D[i] * dux.D[i] + gG[1].D[i] * duy.D[i] + gG[2].D[i] * duz.D[i];
        for (int d = 0; d < 3; d++)
            for (size_t i = 0; i < m.R[d].size(); i++)
                du.R[d][i] = gG[0].R[d][i] * dux.R[d][i] + gG[1].R[d][i] * duy.R[d][i] +
                             gG[2].R[d][i] * duz.R[d][i];
    }

    // scalar_wave::update_boundary: src/systems/scalar_wave.cpp:329-355
    void update_boundary(sfield u, real time)
    {
        const mesh& m = P->m;
        for_each_dirichlet_face(*P, [&](integer i) { u.D[i] = sol(time, m.loc(i)); });
        for (int d = 0; d < 3; d++)
            for (size_t i = 0; i < m.R[d].size(); i++)
                if (P->obc[m.R[d][i].shape_id] == Dirichlet)
                    u.R[d][i] = sol(time, m.R[d][i].position);
    }
};

// slot ops: src/temporal/slot_ops.hpp:11-61
static void lc_assign(field_buf& d, const field_buf& s0, real coeff, const field_buf& r)
{
    const integer N = (integer)d.D.size();
#pragma omp parallel for schedule(static) if (N > 65536)
    for (integer i = 0; i < N; i++) d.D[i] = s0.D[i] + coeff * r.D[i];
    for (int c = 0; c < 3; c++)
        for (size_t i = 0; i < d.R[c].size(); i++) d.R[c][i] = s0.R[c][i] + coeff * r.R[c][i];
}
static void accumulate(field_buf& d, real coeff, const field_buf& r)
{
    const integer N = (integer)d.D.size();
#pragma omp parallel for schedule(static) if (N > 65536)
    for (integer i = 0; i < N; i++) d.D[i] += coeff * r.D[i];
    for (int c = 0; c < 3; c++)
        for (size_t i = 0; i < d.R[c].size(); i++) d.R[c][i] += coeff * r.R[c][i];
}

// rk4::operator(): src/temporal/rk4.cpp:11-48
template <typename Sys>
static void rk4_step(Sys& sys, field_buf& u0, field_buf& u1, field_buf& rk, field_buf& srhs,
                     real time, real dt)
{
    constexpr real rki[4] = {0.0, 0.5, 0.5, 1.0};
    constexpr real rkf[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
    rk.zero();
    srhs.zero();
    u1 = u0;
    for (int i = 0; i < 4; ++i) {
        if (i > 0) {
            lc_assign(u1, u0, dt * rki[i], srhs);
            sys.update_boundary(u1.span(), time + dt * rki[i]);
        }
        sys.rhs(u1.view(), srhs.span(), time + dt * rki[i]);
        accumulate(rk, dt * rkf[i], srhs);
    }
    lc_assign(u1, u0, 1.0, rk);
    sys.update_boundary(u1.span(), time + dt);
}

// integrators::euler::operator(): src/temporal/euler.cpp:11-27 -- output <- u0, the right-hand
// side of output at `time`, output <- u0 + dt rhs, then the boundary data at time + dt
template <typename Sys>
static void euler_step(Sys& sys, field_buf& u0, field_buf& u1, field_buf& srhs, real time, real dt)
{
    u1 = u0;
    srhs.zero();
    sys.rhs(u1.view(), srhs.span(), time);
    lc_assign(u1, u0, dt, srhs);
    sys.update_boundary(u1.span(), time + dt);
}

} // namespace orc

// =======================================================================================
// C API used by the tests (ctypes) and by bench.py's CPU-baseline leg.
// =======================================================================================
using namespace orc;

struct orc_problem {
    problem P;
    std::vector<real> gauss; // SOL_GAUSSIAN terms (orc_set_gaussian)
};

extern "C" {

int orc_num_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

// grid_bc: xmin,xmax,ymin,ymax,zmin,zmax (0 Dirichlet, 1 Floating, 2 Neumann)
// scheme: 0 E2_2, 1 E4_2, 2 E4_1, 3 E4u_1, 5 polyE2_1, 6 E6u_1, 7 E8u_1; alpha: 2 values
// (E4_1, E4u_1), 13 for polyE2_1 (floating alpha[6], dirichlet alpha[3], interpolant
// alpha[4]), 5 for E6u_1, 7 for E8u_1
static void set_params(stencil& st, int scheme, const double* alpha)
{
    st.kind = scheme;
    if (!alpha) return;
    if (scheme >= 5) { // polyE2_1: 13 values; E6u_1: 5; E8u_1: 7
        const int n = scheme == 5 ? 13 : (scheme == 6 ? 5 : 7);
        for (int i = 0; i < n; i++) st.pa[i] = alpha[i];
    } else {
        st.alpha[0] = alpha[0];
        st.alpha[1] = alpha[1];
    }
}

orc_problem* orc_create(const int n[3], const double lo[3], const double hi[3], int nsph,
                        const double* centers, const double* radii, const int* obj_bc,
                        const int grid_bc[6], int scheme, const double* alpha)
{
    auto* o = new orc_problem;
    std::vector<sphere> shapes;
    for (int i = 0; i < nsph; i++)
        shapes.push_back(sphere{{centers[3 * i], centers[3 * i + 1], centers[3 * i + 2]},
                                radii[i], i});
    o->P.m = make_mesh(n, lo, hi, shapes);
    set_params(o->P.st, scheme, alpha);
    // src/operators/boundaries.cpp:11-38: Dirichlet/Neumann on a trivial axis -> Floating
    for (int d = 0; d < 3; d++)
        for (int s = 0; s < 2; s++) {
            int b = grid_bc[2 * d + s];
            if (o->P.m.n[d] == 1 && b != Floating) b = Floating;
            o->P.gbc[d][s] = b;
        }
    o->P.obc.assign(obj_bc, obj_bc + nsph);
    for (int d = 0; d < 3; d++)
        o->P.D[d] = make_derivative(d, o->P.m, o->P.st, o->P.gbc, o->P.obc);
    return o;
}

void orc_destroy(orc_problem* o) { delete o; }

long orc_size(orc_problem* o, int which)
{
    if (which == 0) return o->P.m.size();
    return (long)o->P.m.R[which - 1].size();
}

void orc_cut_points(orc_problem* o, int dir, double* psi, double* pos, double* normal,
                    int* ray_outside, int* solid, int* shape_id)
{
    const auto& R = o->P.m.R[dir];
    for (size_t i = 0; i < R.size(); i++) {
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

// lines: 8 ints per line: start ijk, start object index (-1 if wall), end ijk, end object
long orc_lines(orc_problem* o, int dir, int* out)
{
    const auto& L = o->P.m.lines[dir];
    if (out) {
        for (size_t i = 0; i < L.size(); i++) {
            int* q = out + 8 * i;
            for (int c = 0; c < 3; c++) q[c] = L[i].start.mesh_coordinate[c];
            q[3] = L[i].start.object ? (int)L[i].start.object->object_coordinate : -1;
            for (int c = 0; c < 3; c++) q[4 + c] = L[i].end.mesh_coordinate[c];
            q[7] = L[i].end.object ? (int)L[i].end.object->object_coordinate : -1;
        }
    }
    return (long)L.size();
}

long orc_fluid(orc_problem* o, long* idx)
{
    const auto& F = o->P.m.fluid;
    if (idx) std::copy(F.begin(), F.end(), idx);
    return (long)F.size();
}

// block metadata (13 ints per line) and coefficient array
long orc_block(orc_problem* o, int dir, int* meta, double* coeffs, long* ncoeffs)
{
    const auto& O = o->P.D[dir].O;
    if (meta) std::memcpy(meta, O.meta.data(), O.meta.size() * sizeof(inner_block_meta));
    if (coeffs) std::copy(O.coeffs.begin(), O.coeffs.end(), coeffs);
    if (ncoeffs) *ncoeffs = (long)O.coeffs.size();
    return (long)O.meta.size();
}

// block layout of hand-built lines (the known-answer cases of src/matrices/block.t.cpp):
// 9 longs per line: columns, row offset, column offset, stride, left rows, left columns,
// interior rows, stencil width, right rows, right columns (coefficients are zeros); writes
// 13 ints of metadata per line
void orc_block_layout(int nlines, const long* spec, int* meta)
{
    block O;
    for (int l = 0; l < nlines; l++) {
        const long* q = spec + 10 * l;
        dense L{q[4], q[5], std::vector<real>(q[4] * q[5], 0.0)};
        dense R{q[8], q[9], std::vector<real>(q[8] * q[9], 0.0)};
        O.append_line(q[0], q[1], q[2], q[3], L, q[6], std::vector<real>(q[7], 0.0), R);
    }
    std::memcpy(meta, O.meta.data(), O.meta.size() * sizeof(inner_block_meta));
}

// which: 0 B, 1 N, 2+r Bf[r], 5+r Br[r]; returns nnz, fills rows+1 offsets, cols, vals
long orc_csr(orc_problem* o, int dir, int which, long* nrows, long* u, long* v, double* w)
{
    const auto& D = o->P.D[dir];
    const csr* c = which == 0 ? &D.B : which == 1 ? &D.N : which < 5 ? &D.Bf[which - 2]
                                                                     : &D.Br[which - 5];
    if (nrows) *nrows = c->rows();
    if (u) std::copy(c->u.begin(), c->u.end(), u);
    if (v) std::copy(c->v.begin(), c->v.end(), v);
    if (w) std::copy(c->w.begin(), c->w.end(), w);
    return (long)c->w.size();
}

// stencil coefficients (for golden-vector pinning)
void orc_stencil_nbs(int scheme, const double* alpha, double h, int bc, double psi,
                     int right, double* c, double* x)
{
    stencil st;
    set_params(st, scheme, alpha);
    st.nbs(h, bc, psi, right != 0, c, x);
}
void orc_stencil_interior(int scheme, double h, double* c)
{
    stencil st;
    st.kind = scheme;
    st.interior(h, c);
}
int orc_stencil_interp_wall(int scheme, const double* alpha, int i, double y, double psi,
                            int right, double* c)
{
    stencil st;
    set_params(st, scheme, alpha);
    return st.interp_wall(i, y, psi, c, right != 0);
}
int orc_stencil_interp_interior(int scheme, double y, double* c)
{
    stencil st;
    st.kind = scheme;
    return st.interp_interior(y, c);
}

// derivative apply (eq or plus_eq); nu may be null (no Neumann overload)
void orc_derivative(orc_problem* o, int dir, const double* uD, const double* uRx,
                    const double* uRy, const double* uRz, const double* nuD, double* dD,
                    double* dRx, double* dRy, double* dRz, int plus_eq)
{
    cfield u{uD, {uRx, uRy, uRz}};
    sfield du{dD, {dRx, dRy, dRz}};
    if (plus_eq)
        apply_derivative<true>(o->P.D[dir], u, nuD, du);
    else
        apply_derivative<false>(o->P.D[dir], u, nuD, du);
}

// laplacian: src/operators/laplacian.cpp:37-58
void orc_laplacian(orc_problem* o, const double* uD, const double* uRx, const double* uRy,
                   const double* uRz, const double* nuD, double* dD, double* dRx,
                   double* dRy, double* dRz)
{
    const auto& m = o->P.m;
    cfield u{uD, {uRx, uRy, uRz}};
    sfield du{dD, {dRx, dRy, dRz}};
    std::fill(dD, dD + m.size(), 0.0);
    for (int d = 0; d < 3; d++) std::fill(du.R[d], du.R[d] + m.R[d].size(), 0.0);
    for (int d = 0; d < 3; d++)
        if (m.n[d] > 1) apply_derivative<true>(o->P.D[d], u, nuD, du);
}

// gradient: src/operators/gradient.cpp:35-46; out = 3 fields of 4 buffers each
void orc_gradient(orc_problem* o, const double* uD, const double* uRx, const double* uRy,
                  const double* uRz, double* const* out)
{
    const auto& m = o->P.m;
    cfield u{uD, {uRx, uRy, uRz}};
    for (int d = 0; d < 3; d++) {
        sfield du{out[4 * d], {out[4 * d + 1], out[4 * d + 2], out[4 * d + 3]}};
        std::fill(du.D, du.D + m.size(), 0.0);
        for (int c = 0; c < 3; c++) std::fill(du.R[c], du.R[c] + m.R[c].size(), 0.0);
    }
    for (int d = 0; d < 3; d++) {
        sfield du{out[4 * d], {out[4 * d + 1], out[4 * d + 2], out[4 * d + 3]}};
        if (m.n[d] > 1) apply_derivative<false>(o->P.D[d], u, nullptr, du);
    }
}

static solution make_solution(const orc_problem* o, int kind, const double* params)
{
    solution s;
    s.kind = kind;
    s.dims = o->P.m.n[2] > 1 ? 3 : 2;
    for (int i = 0; i < 8 && params; i++) s.p[i] = params[i];
    if (kind == SOL_GAUSSIAN) {
        // manufactured_solution::from_lua picks gauss1d/2d/3d by mesh::dims (mms.cpp:16-31)
        s.G = o->gauss;
        s.gdims = (o->P.m.n[0] > 1) + (o->P.m.n[1] > 1) + (o->P.m.n[2] > 1);
    }
    return s;
}

extern "C" void orc_set_gaussian(orc_problem* o, int n_terms, const double* terms)
{
    o->gauss.assign(terms, terms + 8 * (size_t)n_terms);
}

static void load_field(field_buf& f, const orc_problem* o, const double* D, const double* Rx,
                       const double* Ry, const double* Rz)
{
    f.resize(o->P.m);
    std::copy(D, D + f.D.size(), f.D.begin());
    const double* R[3] = {Rx, Ry, Rz};
    for (int d = 0; d < 3; d++)
        if (R[d]) std::copy(R[d], R[d] + f.R[d].size(), f.R[d].begin());
}
static void store_field(const field_buf& f, double* D, double* Rx, double* Ry, double* Rz)
{
    std::copy(f.D.begin(), f.D.end(), D);
    double* R[3] = {Rx, Ry, Rz};
    for (int d = 0; d < 3; d++)
        if (R[d]) std::copy(f.R[d].begin(), f.R[d].end(), R[d]);
}

// initialize_scalar_field: src/systems/detail/scalar_system_utils.hpp:186-219
void orc_initialize(orc_problem* o, int sol_kind, const double* params, double t, double* D,
                    double* Rx, double* Ry, double* Rz)
{
    solution s = make_solution(o, sol_kind, params);
    field_buf sol;
    sol.resize(o->P.m);
    eval_at_locations(o->P.m, [&](const real3& loc) { return s(t, loc); }, sol);
    std::fill(D, D + o->P.m.size(), 0.0);
    for (integer i : o->P.m.fluid) D[i] = sol.D[i];
    double* R[3] = {Rx, Ry, Rz};
    for (int d = 0; d < 3; d++)
        if (R[d]) std::copy(sol.R[d].begin(), sol.R[d].end(), R[d]);
}

// exact solution at every D point and R point (for error measurements)
void orc_exact(orc_problem* o, int sol_kind, const double* params, double t, double* D,
               double* Rx, double* Ry, double* Rz)
{
    solution s = make_solution(o, sol_kind, params);
    field_buf sol;
    sol.resize(o->P.m);
    eval_at_locations(o->P.m, [&](const real3& loc) { return s(t, loc); }, sol);
    store_field(sol, D, Rx, Ry, Rz);
}

// heat RHS (one evaluation) and heat RK4 time stepping
void orc_heat_rhs(orc_problem* o, double kappa, int sol_kind, const double* params,
                  double t, const double* uD, const double* uRx, const double* uRy,
                  const double* uRz, double* dD, double* dRx, double* dRy, double* dRz)
{
    heat_sys H{&o->P, kappa, make_solution(o, sol_kind, params), {}, {}};
    H.neu.resize(o->P.m);
    H.src.resize(o->P.m);
    H.rhs(cfield{uD, {uRx, uRy, uRz}}, sfield{dD, {dRx, dRy, dRz}}, t);
}

void orc_heat_rk4(orc_problem* o, double kappa, int sol_kind, const double* params,
                  double t0, double dt, int nsteps, double* D, double* Rx, double* Ry,
                  double* Rz)
{
    heat_sys H{&o->P, kappa, make_solution(o, sol_kind, params), {}, {}};
    H.neu.resize(o->P.m);
    H.src.resize(o->P.m);
    field_buf u0, u1, rk, srhs;
    load_field(u0, o, D, Rx, Ry, Rz);
    u1.resize(o->P.m);
    rk.resize(o->P.m);
    srhs.resize(o->P.m);
    real t = t0;
    for (int s = 0; s < nsteps; s++) {
        rk4_step(H, u0, u1, rk, srhs, t, dt);
        u0 = u1; // simulation_cycle.cpp:125 deep_copy_slot
        t += dt;
    }
    store_field(u0, D, Rx, Ry, Rz);
}

void orc_heat_euler(orc_problem* o, double kappa, int sol_kind, const double* params,
                    double t0, double dt, int nsteps, double* D, double* Rx, double* Ry,
                    double* Rz)
{
    heat_sys H{&o->P, kappa, make_solution(o, sol_kind, params), {}, {}};
    H.neu.resize(o->P.m);
    H.src.resize(o->P.m);
    field_buf u0, u1, srhs;
    load_field(u0, o, D, Rx, Ry, Rz);
    u1.resize(o->P.m);
    srhs.resize(o->P.m);
    real t = t0;
    for (int s = 0; s < nsteps; s++) {
        euler_step(H, u0, u1, srhs, t, dt);
        u0 = u1;
        t += dt;
    }
    store_field(u0, D, Rx, Ry, Rz);
}

// wave: vel_kind 0 -> constant velocity a = vel (u_t + a.grad u = 0, gG = -a);
//       vel_kind 1 -> radial velocity about `center` (scalar_wave.cpp:28-33)
void orc_wave_rhs(orc_problem* o, int vel_kind, const double* vel, const double* center,
                  const double* uD, const double* uRx, const double* uRy, const double* uRz,
                  double* dD, double* dRx, double* dRy, double* dRz)
{
    wave_sys W;
    W.P = &o->P;
    W.vel_kind = vel_kind;
    for (int c = 0; c < 3; c++) {
        W.vel[c] = vel ? vel[c] : 0.0;
        W.center[c] = center ? center[c] : 0.0;
    }
    W.init();
    W.rhs(cfield{uD, {uRx, uRy, uRz}}, sfield{dD, {dRx, dRy, dRz}}, 0.0);
}

void orc_wave_rk4(orc_problem* o, int vel_kind, const double* vel, const double* center,
                  int sol_kind, const double* params, double t0, double dt, int nsteps,
                  double* D, double* Rx, double* Ry, double* Rz)
{
    wave_sys W;
    W.P = &o->P;
    W.vel_kind = vel_kind;
    for (int c = 0; c < 3; c++) {
        W.vel[c] = vel ? vel[c] : 0.0;
        W.center[c] = center ? center[c] : 0.0;
    }
    W.sol = make_solution(o, sol_kind, params);
    W.init();
    field_buf u0, u1, rk, srhs;
    load_field(u0, o, D, Rx, Ry, Rz);
    u1.resize(o->P.m);
    rk.resize(o->P.m);
    srhs.resize(o->P.m);
    real t = t0;
    for (int s = 0; s < nsteps; s++) {
        rk4_step(W, u0, u1, rk, srhs, t, dt);
        u0 = u1;
        t += dt;
    }
    store_field(u0, D, Rx, Ry, Rz);
}

void orc_wave_euler(orc_problem* o, int vel_kind, const double* vel, const double* center,
                    int sol_kind, const double* params, double t0, double dt, int nsteps,
                    double* D, double* Rx, double* Ry, double* Rz)
{
    wave_sys W;
    W.P = &o->P;
    W.vel_kind = vel_kind;
    for (int c = 0; c < 3; c++) {
        W.vel[c] = vel ? vel[c] : 0.0;
        W.center[c] = center ? center[c] : 0.0;
    }
    W.sol = make_solution(o, sol_kind, params);
    W.init();
    field_buf u0, u1, srhs;
    load_field(u0, o, D, Rx, Ry, Rz);
    u1.resize(o->P.m);
    srhs.resize(o->P.m);
    real t = t0;
    for (int s = 0; s < nsteps; s++) {
        euler_step(W, u0, u1, srhs, t, dt);
        u0 = u1;
        t += dt;
    }
    store_field(u0, D, Rx, Ry, Rz);
}

// compute_scalar_stats: src/systems/detail/scalar_system_utils.hpp:77-181
// out[11] = {err, min, max, err_d, err_d_idx, err_rx, idx_rx, err_ry, idx_ry, err_rz, idx_rz}
void orc_stats(orc_problem* o, int sol_kind, const double* params, double t,
               const double* uD, const double* uRx, const double* uRy, const double* uRz,
               double* out)
{
    const auto& m = o->P.m;
    solution s = make_solution(o, sol_kind, params);
    real umin = std::numeric_limits<real>::max(), umax = -std::numeric_limits<real>::max();
    real err_d = 0;
    long err_idx = 0;
    bool have = false;
    for (integer i : m.fluid) {
        real v = uD[i];
        umin = std::min(umin, v);
        umax = std::max(umax, v);
        real e = std::abs(v - s(t, m.loc(i)));
        if (!have || e > err_d) {
            err_d = e;
            err_idx = i;
        }
        have = true;
    }
    if (!have) umin = umax = 0;
    real ce[3] = {0, 0, 0}, ci[3] = {0, 0, 0};
    const double* uR[3] = {uRx, uRy, uRz};
    for (int d = 0; d < 3; d++) {
        bool any = false;
        real e_best = 0;
        long i_best = 0;
        for (size_t i = 0; i < m.R[d].size(); i++) {
            if (o->P.obc[m.R[d][i].shape_id] == Dirichlet) continue;
            real v = uR[d][i];
            umin = std::min(umin, v);
            umax = std::max(umax, v);
            real e = std::abs(v - s(t, m.R[d][i].position));
            if (!any || e > e_best) {
                e_best = e;
                i_best = (long)i;
            }
            any = true;
        }
        ce[d] = e_best;
        ci[d] = (real)i_best;
    }
    out[0] = std::max({err_d, ce[0], ce[1], ce[2]});
    out[1] = umin;
    out[2] = umax;
    out[3] = err_d;
    out[4] = (real)err_idx;
    out[5] = ce[0];
    out[6] = ci[0];
    out[7] = ce[1];
    out[8] = ci[1];
    out[9] = ce[2];
    out[10] = ci[2];
}

// write_scalar_error: src/systems/detail/scalar_system_utils.hpp:224-296 -- zero the error
// field, |u - sol| at the fluid D points and at the non-Dirichlet cut points, then zero the
// Dirichlet grid faces and the Dirichlet cut points
void orc_error_field(orc_problem* o, int sol_kind, const double* params, double t,
                     const double* uD, const double* uRx, const double* uRy, const double* uRz,
                     double* eD, double* eRx, double* eRy, double* eRz)
{
    const auto& m = o->P.m;
    solution s = make_solution(o, sol_kind, params);
    std::fill(eD, eD + m.size(), 0.0);
    for (integer i : m.fluid) eD[i] = std::abs(uD[i] - s(t, m.loc(i)));
    const double* uR[3] = {uRx, uRy, uRz};
    double* eR[3] = {eRx, eRy, eRz};
    for (int d = 0; d < 3; d++)
        for (size_t i = 0; i < m.R[d].size(); i++)
            eR[d][i] = o->P.obc[m.R[d][i].shape_id] == Dirichlet
                           ? 0.0
                           : std::abs(uR[d][i] - s(t, m.R[d][i].position));
    for_each_dirichlet_face(o->P, [&](integer i) { eD[i] = 0.0; });
}

} // extern "C"

extern "C" int orc_sphere_hit(const double* center, double radius, const double* origin,
                              const double* direction, double t_min, double t_max, double* t,
                              double* pos, int* ray_outside, double* normal)
{
    orc::sphere s{{center[0], center[1], center[2]}, radius, 0};
    auto h = s.hit({origin[0], origin[1], origin[2]},
                   {direction[0], direction[1], direction[2]}, t_min, t_max);
    if (!h) return 0;
    *t = h->t;
    for (int k = 0; k < 3; k++) pos[k] = h->position[k];
    *ray_outside = h->ray_outside;
    auto n = s.normal(h->position);
    for (int k = 0; k < 3; k++) normal[k] = n[k];
    return 1;
}
