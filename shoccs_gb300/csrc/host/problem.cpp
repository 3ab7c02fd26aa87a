// problem.cpp -- mesh, cut points, operator assembly and compilation into device tables.
// See problem.hpp for the reference files each part follows.
#include "problem.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <map>
#include <optional>
#include <stdexcept>
#include <string>
#include <unordered_map>

namespace sgb
{
namespace
{
// indexing: src/indexing.hpp:18-36 -- slow/fast axes of a line direction
inline int slow_of(int I) { return I == 0 ? 1 : 0; }
inline int fast_of(int I) { return I == 2 ? 1 : 2; }

// dot of two 3-vectors as the reference folds it: a0*b0 + (a1*b1 + a2*b2)
// (src/real3_operators.hpp:56-65)
inline real dot3(const real* a, const real* b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }

struct Hit {
    real t;
    real pos[3];
    int ray_outside;
    int shape;
};

// src/mesh/sphere.cpp:15-38
bool sphere_hit(const Sphere& s, const real* o, const real* d, real t_min, real t_max, Hit& out)
{
    const real oc[3] = {o[0] - s.c[0], o[1] - s.c[1], o[2] - s.c[2]};
    const real a = dot3(d, d);
    const real b = dot3(oc, d);
    const real c = dot3(oc, oc) - s.r * s.r;
    const real disc = b * b - a * c;
    if (!(disc > 0)) return false;
    const real sq = std::sqrt(disc);
    for (int root = 0; root < 2; ++root) {
        const real t = root == 0 ? (-b - sq) / a : (-b + sq) / a;
        if (t > t_min && t < t_max) {
            out.t = t;
            for (int k = 0; k < 3; k++) out.pos[k] = o[k] + t * d[k];
            const real pc[3] = {out.pos[0] - s.c[0], out.pos[1] - s.c[1], out.pos[2] - s.c[2]};
            out.ray_outside = dot3(d, pc) < 0;
            out.shape = s.id;
            return true;
        }
    }
    return false;
}

void sphere_normal(const Sphere& s, const real* pos, real* nrm)
{
    const real r[3] = {pos[0] - s.c[0], pos[1] - s.c[1], pos[2] - s.c[2]};
    const real len = std::sqrt(dot3(r, r));
    for (int k = 0; k < 3; k++) nrm[k] = r[k] / len;
}

// closest hit over all shapes, later shapes winning only when strictly closer
// (src/mesh/object_geometry.cpp:17-30)
bool closest_hit(const std::vector<Sphere>& shapes, const real* o, const real* d, real t_min,
                 real t_max, Hit& out)
{
    bool any = false;
    Hit h;
    for (const auto& s : shapes) {
        if (sphere_hit(s, o, d, t_min, t_max, h)) {
            out = h;
            any = true;
            t_max = h.t;
        }
    }
    return any;
}

// ray cast along axis I from the domain minimum of every grid line
// (src/mesh/object_geometry.cpp:32-116)
void cast_axis(int I, const Mesh& m, std::vector<CutPoint>& out)
{
    const int S = slow_of(I), F = fast_of(I);
    const real min = m.lo[I], max = m.hi[I], h = m.h[I];
    real origin[3] = {0, 0, 0};
    int coord[3] = {0, 0, 0};
    for (int s = 0; s < m.n[S]; s++) {
        origin[S] = m.lo[S] + s * m.h[S];
        coord[S] = s;
        for (int f = 0; f < m.n[F]; f++) {
            origin[F] = m.lo[F] + f * m.h[F];
            coord[F] = f;
            real t_min = 0, t_max = max - min;
            origin[I] = min;
            real dir[3] = {0, 0, 0};
            dir[I] = 1.0;
            Hit hit;
            while (closest_hit(m.shapes, origin, dir, t_min, t_max, hit)) {
                const real t_over_h = hit.t / h;
                int i_cell = static_cast<int>(std::round(t_over_h));
                constexpr real snap_tol = 1e-12;
                if (std::abs(t_over_h - i_cell) > snap_tol) i_cell = static_cast<int>(t_over_h);
                coord[I] = i_cell + hit.ray_outside;
                const int off = 1 - 2 * hit.ray_outside;
                const real fluid_pos = min + h * (coord[I] + off);
                real psi = off * (fluid_pos - hit.pos[I]) / h;
                psi = std::clamp(psi, snap_tol, 1.0 - snap_tol);
                CutPoint cp{};
                cp.psi = psi;
                std::memcpy(cp.pos, hit.pos, sizeof cp.pos);
                sphere_normal(m.shapes[hit.shape], hit.pos, cp.nrm);
                cp.ray_outside = hit.ray_outside;
                std::memcpy(cp.solid, coord, sizeof cp.solid);
                cp.shape_id = hit.shape;
                out.push_back(cp);
                t_min = std::nextafter(hit.t, t_max);
            }
        }
    }
}

// split every grid line along I into fluid segments at its cut points
// (src/mesh/mesh.cpp:29-87)
void segment_axis(int I, Mesh& m)
{
    if (m.n[I] == 1) return;
    const int S = slow_of(I), F = fast_of(I);
    const auto& r = m.R[I];
    size_t q = 0;
    const i64 stride = m.stride(I);
    auto& v = m.lines[I];
    v.reserve((size_t)m.n[S] * m.n[F] + r.size());
    for (int s = 0; s < m.n[S]; s++) {
        for (int f = 0; f < m.n[F]; f++) {
            Bnd left{};
            left.ijk[S] = s;
            left.ijk[F] = f;
            left.ijk[I] = 0;
            bool have_left = true;
            while (q < r.size() && r[q].solid[S] == s && r[q].solid[F] == f) {
                Bnd b{};
                std::memcpy(b.ijk, r[q].solid, sizeof b.ijk);
                b.obj = (i64)q;
                b.obj_id = r[q].shape_id;
                b.psi = r[q].psi;
                if (r[q].ray_outside) {
                    if (!have_left) throw std::runtime_error("non-convex or overlapping shapes");
                    v.push_back(Line{stride, left, b});
                    have_left = false;
                } else {
                    left = b;
                    have_left = true;
                }
                ++q;
            }
            if (have_left) {
                Bnd right{};
                right.ijk[S] = s;
                right.ijk[F] = f;
                right.ijk[I] = m.n[I] - 1;
                v.push_back(Line{stride, left, right});
            }
        }
    }
}

} // namespace

Mesh build_mesh(const int n[3], const real lo[3], const real hi[3],
                const std::vector<Sphere>& shapes)
{
    Mesh m{};
    for (int i = 0; i < 3; i++) {
        m.n[i] = n[i] > 0 ? n[i] : 1;
        m.lo[i] = lo[i];
        m.hi[i] = hi[i];
        m.h[i] = (m.n[i] - 1) ? (m.hi[i] - m.lo[i]) / (m.n[i] - 1)
                              : std::numeric_limits<real>::max();
        m.x[i].resize(m.n[i]);
        for (int k = 0; k < m.n[i]; ++k)
            m.x[i][k] = m.n[i] > 1 ? m.lo[i] + k * (m.hi[i] - m.lo[i]) / (m.n[i] - 1) : m.lo[i];
    }
    m.shapes = shapes;
    for (int d = 0; d < 3; d++) cast_axis(d, m, m.R[d]);
    for (int d = 0; d < 3; d++) segment_axis(d, m);
    // fluid slices along the highest non-trivial axis (src/mesh/mesh.cpp:89-111, 134-137)
    const int fd = m.n[2] > 1 ? 2 : m.n[1] > 1 ? 1 : 0;
    for (const auto& ln : m.lines[fd]) {
        const i64 i0 = ln.s.obj >= 0 ? m.ic(ln.s.ijk) + 1 : m.ic(ln.s.ijk);
        const i64 i1 = ln.e.obj >= 0 ? m.ic(ln.e.ijk) : m.ic(ln.e.ijk) + 1;
        if (!m.fluid_slices.empty() && m.fluid_slices.back().second == i0)
            m.fluid_slices.back().second = i1;
        else
            m.fluid_slices.emplace_back(i0, i1);
    }
    return m;
}

bool on_dirichlet_face(const Mesh& m, const Bcs& bcs, const int ijk[3])
{
    for (int d = 0; d < 3; d++) {
        if (bcs.grid[d][0] == Dirichlet && ijk[d] == 0) return true;
        if (bcs.grid[d][1] == Dirichlet && ijk[d] == m.n[d] - 1) return true;
    }
    return false;
}

namespace
{
// src/mesh/mesh.cpp:154-168: lines lying on another axis's Dirichlet face carry no rows
bool dirichlet_line(const Mesh& m, const int* start, int dir, const Bcs& bcs)
{
    for (int i = 0; i < 3; i++) {
        if (i == dir) continue;
        if ((bcs.grid[i][0] == Dirichlet && start[i] == 0) ||
            (bcs.grid[i][1] == Dirichlet && start[i] == m.n[i] - 1))
            return true;
    }
    return false;
}

struct Coo {
    i64 row, col;
    real v;
    bool operator<(const Coo& o) const
    {
        if (row != o.row) return row < o.row;
        if (col != o.col) return col < o.col;
        return v < o.v;
    }
};

// src/matrices/csr.cpp:10-35 (stable (row, col, value) order)
Csr to_csr(std::vector<Coo> p, i64 nrows)
{
    std::sort(p.begin(), p.end());
    Csr c;
    c.rows = nrows;
    c.u.assign(nrows + 1, 0);
    size_t q = 0;
    for (i64 i = 0; i < nrows; i++) {
        c.u[i + 1] = c.u[i];
        while (q < p.size() && p[q].row == i) {
            ++c.u[i + 1];
            ++q;
        }
    }
    for (auto& e : p) {
        c.v.push_back(e.col);
        c.w.push_back(e.v);
    }
    return c;
}

// src/mesh/mesh.cpp:170-207 -- nearest boundaries of the line through pt along dir
Line interp_line(const Mesh& m, int dir, const int* pt)
{
    Line ln{};
    ln.stride = m.stride(dir);
    std::memcpy(ln.s.ijk, pt, sizeof ln.s.ijk);
    std::memcpy(ln.e.ijk, pt, sizeof ln.e.ijk);
    ln.s.ijk[dir] = 0;
    ln.e.ijk[dir] = m.n[dir] - 1;
    const int f = fast_of(dir), s = slow_of(dir);
    for (size_t i = 0; i < m.R[dir].size(); i++) {
        const auto& o = m.R[dir][i];
        if (o.solid[s] > pt[s]) break;
        if (o.solid[s] != pt[s] || o.solid[f] != pt[f]) continue;
        if (o.nrm[dir] >= 0.0 && o.solid[dir] <= pt[dir]) {
            if (o.solid[dir] >= ln.s.ijk[dir]) {
                std::memcpy(ln.s.ijk, o.solid, sizeof ln.s.ijk);
                ln.s.obj = (i64)i;
                ln.s.obj_id = o.shape_id;
                ln.s.psi = o.psi;
            }
        } else if (o.nrm[dir] < 0.0 && o.solid[dir] >= pt[dir]) {
            if (o.solid[dir] <= ln.e.ijk[dir]) {
                std::memcpy(ln.e.ijk, o.solid, sizeof ln.e.ijk);
                ln.e.obj = (i64)i;
                ln.e.obj_id = o.shape_id;
                ln.e.psi = o.psi;
            }
        }
    }
    return ln;
}

// src/stencils/stencil.hpp:213-270 -- cross-direction interpolant through `closest`
struct Interp {
    int n;
    real c[8];
    Bnd left, right;
};
Interp interp(const Stencil& st, int dir, const int* closest, real y, const Bnd& left,
              const Bnd& right)
{
    const auto q = st.query_interp();
    const int p = q.p, t = q.t;
    Interp out{};
    const int ic = closest[dir], lc = left.ijk[dir], rc = right.ijk[dir];
    int st1 = p & 1 ? (p - 1) / 2 : p / 2;
    int st2 = (p - 1) / 2;
    if (y > 0) std::swap(st1, st2);
    const bool lo = left.obj >= 0, ro = right.obj >= 0;
    if ((ic - lc > st1 || (ic - lc == st1 && !lo)) && (rc - ic > st2 || (rc - ic == st2 && !ro))) {
        Bnd l{}, r{};
        std::memcpy(l.ijk, closest, sizeof l.ijk);
        std::memcpy(r.ijk, closest, sizeof r.ijk);
        l.ijk[dir] -= st1;
        r.ijk[dir] += st2;
        out.n = st.interp_interior(y, out.c);
        out.left = l;
        out.right = r;
    } else if (ic - lc < rc - ic) {
        Bnd r{};
        std::memcpy(r.ijk, left.ijk, sizeof r.ijk);
        r.ijk[dir] += t - 1;
        const real psi = lo ? left.psi : 1.0;
        if (lo && lc == ic) y += psi - 1;
        out.n = st.interp_wall(ic - lc, y, psi, out.c, false);
        out.left = left;
        out.right = r;
    } else {
        Bnd l{};
        std::memcpy(l.ijk, right.ijk, sizeof l.ijk);
        l.ijk[dir] -= t - 1;
        const real psi = ro ? right.psi : 1.0;
        if (ro && rc == ic) y += 1 - psi;
        out.n = st.interp_wall(rc - ic, y, psi, out.c, true);
        out.left = l;
        out.right = right;
    }
    return out;
}

// src/operators/derivative.cpp:22-70
struct DerivRow {
    std::vector<real> c;
    int offset;
};
DerivRow interp_deriv_coefficients(int dir, int n, real h, const CutPoint& obj, int bc,
                                   const Stencil& st)
{
    const auto q = st.query(bc);
    const int p = q.p, r = q.r, t = q.t;
    real c[128], ex[8];
    if (std::abs(obj.nrm[dir]) > 1e-12) {
        const bool right_wall = obj.nrm[dir] < 0.0;
        st.nbs(h, bc, 1.0, right_wall, c, ex);
        if (right_wall) return {std::vector<real>(c + (r - 1) * t, c + r * t), 1 - t};
        return {std::vector<real>(c, c + t), 0};
    }
    const int right_dist = n - obj.solid[dir];
    const int left_dist = obj.solid[dir];
    if (right_dist >= p && left_dist >= p) {
        st.interior(h, c);
        return {std::vector<real>(c, c + 2 * p + 1), -p};
    }
    const bool right_wall = right_dist < left_dist;
    st.nbs(h, bc, 1.0, right_wall, c, ex);
    if (right_wall) {
        const int qq = 1 + right_dist;
        return {std::vector<real>(c + (r - qq) * t, c + (r - qq) * t + t), qq - t};
    }
    const int qq = left_dist;
    return {std::vector<real>(c + qq * t, c + qq * t + t), -qq};
}

// src/operators/derivative.cpp:159-257 -- rows of R(r) for non-Dirichlet objects
void cut_rows(int r, int dir, const Mesh& m, const Stencil& st, const Bcs& bcs, Csr& Bf,
              Csr& Br)
{
    const auto& cps = m.R[r];
    const i64 sz = (i64)cps.size();
    const bool all_dirichlet =
        std::all_of(bcs.obj.begin(), bcs.obj.end(), [](int b) { return b == Dirichlet; });
    if (sz == 0 || all_dirichlet) return;
    const real h = m.h[dir];
    const i64 stride = m.stride(dir);
    std::vector<Coo> O, B;
    real c[128], ex[8];
    for (i64 row = 0; row < sz; ++row) {
        const auto& obj = cps[row];
        const int bc = bcs.obj[obj.shape_id];
        if (bc == Dirichlet) continue;
        if (dir == r) {
            const auto q = st.query(bc);
            st.nbs(h, bc, obj.psi, obj.ray_outside != 0, c, ex);
            std::vector<real> rng;
            i64 sgn;
            if (obj.ray_outside) {
                rng.assign(c + (q.r - 1) * q.t, c + q.r * q.t);
                std::reverse(rng.begin(), rng.end());
                sgn = -stride;
            } else {
                rng.assign(c, c + q.t);
                sgn = stride;
            }
            const i64 solid_ic = m.ic(obj.solid);
            B.push_back({row, row, rng[0]});
            for (int i = 1; i < (int)rng.size(); ++i) O.push_back({row, solid_ic + i * sgn, rng[i]});
        } else {
            const auto dr = interp_deriv_coefficients(dir, m.n[dir] - 1, h, obj, bc, st);
            int cp[3] = {obj.solid[0], obj.solid[1], obj.solid[2]};
            if (obj.psi <= 0.5) cp[r] += 1 - 2 * obj.ray_outside;
            cp[dir] += dr.offset;
            const real y =
                (obj.ray_outside ? 1.0 : -1.0) * (obj.psi <= 0.5 ? obj.psi : obj.psi - 1);
            for (real v : dr.c) {
                if (cp[dir] == obj.solid[dir]) {
                    B.push_back({row, row, v});
                } else {
                    const Line il = interp_line(m, r, cp);
                    const Interp it = interp(st, r, cp, y, il.s, il.e);
                    const i64 left_ic = m.ic(it.left.ijk), right_ic = m.ic(it.right.ijk);
                    int k = 0;
                    if (it.left.obj >= 0)
                        B.push_back({row, it.left.obj, v * it.c[k]});
                    else
                        O.push_back({row, left_ic, v * it.c[k]});
                    ++k;
                    for (i64 ic = left_ic + il.stride; ic < right_ic; ic += il.stride)
                        O.push_back({row, ic, v * it.c[k++]});
                    if (it.right.obj >= 0)
                        B.push_back({row, it.right.obj, v * it.c[k]});
                    else
                        O.push_back({row, right_ic, v * it.c[k]});
                }
                ++cp[dir];
            }
        }
    }
    Bf = to_csr(std::move(O), sz);
    Br = to_csr(std::move(B), sz);
}
} // namespace

AxisOp assemble_axis(int dir, const Mesh& m, const Stencil& st, const Bcs& bcs)
{
    AxisOp A;
    A.dir = dir;
    A.stride = m.stride(dir);
    if (m.n[dir] < 2) return A;
    A.active = true;
    const auto mx = st.query_max();
    const real h = m.h[dir];
    A.interior.resize(2 * mx.p + 1);
    st.interior(h, A.interior.data());

    real left[128], right[128], extra[8];
    std::vector<Coo> B, N;
    for (const auto& ln : m.lines[dir]) {
        if (dirichlet_line(m, ln.s.ijk, dir, bcs)) continue;
        const i64 stride = ln.stride;
        // submatrix_size: src/operators/derivative.cpp:259-303
        i64 rows = ln.e.ijk[dir] - ln.s.ijk[dir] + 1;
        i64 cols = rows;
        i64 row_offset = m.ic(ln.s.ijk);
        i64 col_offset = row_offset;
        const i64 last_row = m.ic(ln.e.ijk);
        int lrows, lcols, rrows, rcols;
        std::vector<real> lv, rv;

        if (ln.s.obj >= 0) {
            const int bc = bcs.obj[ln.s.obj_id];
            const auto q = st.query(bc);
            st.nbs(h, bc, ln.s.psi, false, left, extra);
            const int s = bc != Dirichlet;
            lrows = q.r - s;
            lcols = q.t - 1;
            const real* lc = left + s * q.t;
            for (int row = 0; row < lrows; ++row)
                for (int j = 1; j < q.t; ++j) lv.push_back(lc[row * q.t + j]);
            --rows;
            row_offset += stride;
            --cols;
            col_offset += stride;
            for (int row = 0; row < lrows; ++row)
                B.push_back({row_offset + stride * row, ln.s.obj, lc[row * q.t]});
        } else {
            const int bc = bcs.grid[dir][0];
            const auto q = st.query(bc);
            st.nbs(h, bc, 1.0, false, left, extra);
            lrows = q.r;
            lcols = q.t;
            lv.assign(left, left + q.r * q.t);
            if (bc == Dirichlet) {
                --rows;
                row_offset += stride;
            } else if (bc == Neumann) {
                for (int row = 0; row < q.nextra; row++)
                    N.push_back({row_offset + stride * row, row_offset, extra[row]});
            }
        }

        if (ln.e.obj >= 0) {
            const int bc = bcs.obj[ln.e.obj_id];
            const auto q = st.query(bc);
            st.nbs(h, bc, ln.e.psi, true, right, extra);
            const int s = bc != Dirichlet;
            rrows = q.r - s;
            rcols = q.t - 1;
            for (int row = 0; row < rrows; ++row)
                for (int j = 0; j < q.t - 1; ++j) rv.push_back(right[row * q.t + j]);
            --rows;
            --cols;
            for (int row = 0; row < rrows; ++row)
                B.push_back({last_row + stride * (row - rrows), ln.e.obj,
                             right[row * q.t + q.t - 1]});
        } else {
            const int bc = bcs.grid[dir][1];
            const auto q = st.query(bc);
            st.nbs(h, bc, 1.0, true, right, extra);
            rrows = q.r;
            rcols = q.t;
            rv.assign(right, right + q.r * q.t);
            if (bc == Dirichlet) {
                --rows;
            } else if (bc == Neumann) {
                for (int row = 0; row < q.nextra; row++)
                    N.push_back({last_row + stride * (row - q.nextra + 1), last_row, extra[row]});
            }
        }
        const i64 n_interior = rows - lrows - rrows;
        if (n_interior < 0)
            throw std::runtime_error(
                "line segment along axis " + std::to_string(dir) + " starting at (" +
                std::to_string(ln.s.ijk[0]) + "," + std::to_string(ln.s.ijk[1]) + "," +
                std::to_string(ln.s.ijk[2]) + ") has " + std::to_string(rows) +
                " rows, fewer than its two boundary closures (" + std::to_string(lrows) +
                " + " + std::to_string(rrows) +
                "); the closure blocks would overlap (refine the grid or separate the shapes)");

        // inner_block / block::build_device_arrays: src/matrices/inner_block.cpp:73-96,
        // src/matrices/block.hpp:30-94
        BlockMeta bm{};
        bm.row_offset = (int)row_offset;
        bm.col_offset = (int)col_offset;
        bm.stride = (int)stride;
        bm.left_rows = lrows;
        bm.left_cols = lcols;
        bm.left_coeff_offset = (int)A.coeffs.size();
        A.coeffs.insert(A.coeffs.end(), lv.begin(), lv.end());
        bm.interior_rows = (int)n_interior;
        bm.interior_coeff_offset = (int)A.coeffs.size();
        bm.stencil_width = (int)A.interior.size();
        A.coeffs.insert(A.coeffs.end(), A.interior.begin(), A.interior.end());
        bm.right_rows = rrows;
        bm.right_cols = rcols;
        bm.right_coeff_offset = (int)A.coeffs.size();
        bm.right_col_offset = (int)(col_offset + stride * (cols - rcols));
        A.coeffs.insert(A.coeffs.end(), rv.begin(), rv.end());
        A.meta.push_back(bm);
        A.block_wall.push_back((uint8_t)((ln.s.obj < 0 ? 1 : 0) | (ln.e.obj < 0 ? 2 : 0)));
    }
    A.B = to_csr(std::move(B), m.size());
    A.N = to_csr(std::move(N), m.size());
    for (int r = 0; r < 3; r++) cut_rows(r, dir, m, st, bcs, A.Bf[r], A.Br[r]);
    return A;
}

// ---------------------------------------------------------------------------------------
// compile into the device format (gpu_layout.hpp)
// ---------------------------------------------------------------------------------------
namespace
{
struct RowKey {
    std::string bytes;
    bool operator==(const RowKey& o) const { return bytes == o.bytes; }
};
struct RowKeyHash {
    size_t operator()(const RowKey& k) const { return std::hash<std::string>{}(k.bytes); }
};
} // namespace

Compiled compile_operators(const Mesh& m, const AxisOp ops[3], const Bcs& bcs)
{
    Compiled C{};
    // iteration space: squeeze trivial axes to the front so the contiguous axis is wide
    {
        int k = 2;
        int it[3] = {1, 1, 1}, phys[3] = {-1, -1, -1};
        for (int d = 2; d >= 0; --d)
            if (m.n[d] > 1) {
                it[k] = m.n[d];
                phys[k] = d;
                --k;
            }
        if (k == 2) { // zero-dimensional: a single point
            it[2] = 1;
            phys[2] = 2;
        }
        for (int i = 0; i < 3; i++) {
            C.it[i] = it[i];
            C.phys_of_it[i] = phys[i];
        }
        C.nzc = (C.it[2] + 31) / 32;
    }
    const i64 N = m.size();
    C.cls.assign(N, 0);

    // fluid and Dirichlet-face flags
    for (const auto& [a, b] : m.fluid_slices)
        for (i64 i = a; i < b; ++i) C.cls[i] |= CLS_FLUID;
    C.n_fluid = 0;
    for (i64 i = 0; i < N; i++) C.n_fluid += (C.cls[i] & CLS_FLUID) != 0;
    for (int i = 0; i < m.n[0]; i++)
        for (int j = 0; j < m.n[1]; j++)
            for (int k = 0; k < m.n[2]; k++) {
                const int ijk[3] = {i, j, k};
                if (on_dirichlet_face(m, bcs, ijk)) C.cls[m.ic(ijk)] |= CLS_DIRFACE;
            }

    const i64 n_chunks = (i64)C.it[0] * C.it[1] * C.nzc;
    for (int d = 0; d < 3; d++) {
        const AxisOp& A = ops[d];
        AxisTables& T = C.ax[d];
        T.active = A.active;
        T.stride = A.stride;
        if (!A.active) continue;
        T.width = (int)A.interior.size();
        for (int j = 0; j < T.width; j++) T.interior[j] = A.interior[j];

        struct Pending {
            i64 out;
            std::vector<real> c;
            int col0;
            i64 b_idx = -1, n_idx = -1;
            real b = 0, nn = 0;
        };
        std::vector<Pending> pend;
        const int shift = 2 * d;
        const i64 sd = m.stride(d);
        auto axis_coord = [&](i64 flat) { return (int)((flat / sd) % m.n[d]); };
        // a wall row joins its side's shared block; the first line defines the block and
        // every other line must reproduce it exactly
        std::vector<std::vector<std::vector<real>>> wall_rows(2);
        std::vector<int> wall_col0(2, -1), wall_first(2, -1), wall_cols(2, 0);
        auto wall_row = [&](int side, int r, int nrows, int ncols, const real* c, i64 out,
                            i64 col_start) {
            const int coord = axis_coord(out);
            const int col0 = axis_coord(col_start);
            auto& rows = wall_rows[side];
            if (rows.empty()) {
                rows.assign(nrows, {});
                wall_col0[side] = col0;
                wall_first[side] = coord - r;
                wall_cols[side] = ncols;
            }
            if ((int)rows.size() != nrows || wall_first[side] != coord - r ||
                wall_col0[side] != col0 || wall_cols[side] != ncols)
                throw std::runtime_error("domain-wall closure blocks differ between lines");
            std::vector<real> v(c, c + ncols);
            if (rows[r].empty())
                rows[r] = v;
            else if (rows[r] != v)
                throw std::runtime_error("domain-wall closure rows differ between lines");
            C.cls[out] |= (uint8_t)(ROW_WALL << shift);
        };
        for (size_t b = 0; b < A.meta.size(); b++) {
            const auto& bm = A.meta[b];
            // a domain-wall block is stored once per axis and side when it fits the 5 x 7
            // WallBlock (E6u_1's and E8u_1's do not); otherwise its rows are per-row records
            // like the cut-cell rows
            const bool lwall = (A.block_wall[b] & 1) && bm.left_rows <= 5 && bm.left_cols <= 7;
            const bool rwall = (A.block_wall[b] & 2) && bm.right_rows <= 5 && bm.right_cols <= 7;
            const i64 st = bm.stride;
            for (int r = 0; r < bm.left_rows; r++) {
                const i64 out = bm.row_offset + (i64)r * st;
                const real* c = A.coeffs.data() + bm.left_coeff_offset + r * bm.left_cols;
                if (lwall) {
                    wall_row(0, r, bm.left_rows, bm.left_cols, c, out, bm.col_offset);
                    continue;
                }
                Pending p;
                p.out = out;
                p.c.assign(c, c + bm.left_cols);
                p.col0 = (int)((bm.col_offset - out) / st);
                pend.push_back(std::move(p));
                C.cls[out] |= (uint8_t)(ROW_CLOSURE << shift);
            }
            for (int r = 0; r < bm.interior_rows; r++) {
                const i64 out = bm.row_offset + (i64)(bm.left_rows + r) * st;
                C.cls[out] |= (uint8_t)(ROW_INTERIOR << shift);
            }
            for (int r = 0; r < bm.right_rows; r++) {
                const i64 out = bm.row_offset + (i64)(bm.left_rows + bm.interior_rows + r) * st;
                const real* c = A.coeffs.data() + bm.right_coeff_offset + r * bm.right_cols;
                if (rwall) {
                    wall_row(1, r, bm.right_rows, bm.right_cols, c, out, bm.right_col_offset);
                    continue;
                }
                Pending p;
                p.out = out;
                p.c.assign(c, c + bm.right_cols);
                p.col0 = (int)((bm.right_col_offset - out) / st);
                pend.push_back(std::move(p));
                C.cls[out] |= (uint8_t)(ROW_CLOSURE << shift);
            }
        }
        for (int side = 0; side < 2; side++) {
            WallBlock& W = T.wall[side];
            W = WallBlock{};
            W.wall = side == 0 ? 0 : m.n[d] - 1;
            if (wall_rows[side].empty()) continue;
            W.rows = (int)wall_rows[side].size();
            W.cols = wall_cols[side];
            W.first_row = wall_first[side];
            W.col0 = wall_col0[side];
            if (W.rows > 5 || W.cols > 7) throw std::runtime_error("wall block exceeds 5 x 7");
            for (int r = 0; r < W.rows; r++) {
                real sum = 0.0;
                for (int j = 0; j < W.cols; j++) {
                    W.c[r * 7 + j] = wall_rows[side][r][j];
                    W.cf[r * 7 + j] = (float)wall_rows[side][r][j];
                    sum += wall_rows[side][r][j];
                }
                const int self = W.first_row + r - W.col0;
                if (self < 0 || self >= W.cols)
                    throw std::runtime_error("wall closure row without its own point as a column");
                W.sf[r] = (float)sum;
            }
        }
        std::sort(pend.begin(), pend.end(),
                  [](const Pending& a, const Pending& b) { return a.out < b.out; });
        // attach B and N entries (one per closure row in the reference's assembly)
        auto find_row = [&](i64 out) -> Pending& {
            auto it = std::lower_bound(pend.begin(), pend.end(), out,
                                       [](const Pending& a, i64 o) { return a.out < o; });
            if (it == pend.end() || it->out != out)
                throw std::runtime_error("closure B/N entry on a row without a closure block");
            return *it;
        };
        for (i64 row = 0; row < A.B.rows; row++) {
            const i64 nnz = A.B.u[row + 1] - A.B.u[row];
            if (nnz == 0) continue;
            if (nnz > 1) throw std::runtime_error("more than one B entry on a closure row");
            auto& p = find_row(row);
            p.b_idx = A.B.v[A.B.u[row]];
            p.b = A.B.w[A.B.u[row]];
        }
        bool n_set[2][5] = {};
        for (i64 row = 0; row < A.N.rows; row++) {
            const i64 nnz = A.N.u[row + 1] - A.N.u[row];
            if (nnz == 0) continue;
            if (nnz > 1) throw std::runtime_error("more than one N entry on a closure row");
            if (((C.cls[row] >> shift) & 3u) == ROW_WALL) {
                // Neumann data of a wall row: coefficient on the wall point of its line
                const int coord = axis_coord(row);
                const int side = coord < m.n[d] / 2 ? 0 : 1;
                WallBlock& W = T.wall[side];
                const int r = coord - W.first_row;
                const i64 col = A.N.v[A.N.u[row]];
                if (r < 0 || r >= W.rows || axis_coord(col) != W.wall ||
                    col != row + (i64)(W.wall - coord) * sd)
                    throw std::runtime_error("Neumann entry off its wall row");
                const real v = A.N.w[A.N.u[row]];
                if (n_set[side][r] && W.n[r] != v)
                    throw std::runtime_error("Neumann wall rows differ between lines");
                W.n[r] = v;
                W.has_n = 1;
                n_set[side][r] = true;
                continue;
            }
            auto& p = find_row(row);
            p.n_idx = A.N.v[A.N.u[row]];
            p.nn = A.N.w[A.N.u[row]];
        }
        // emit rows with a deduplicated coefficient pool
        std::unordered_map<RowKey, int, RowKeyHash> pool;
        for (const auto& p : pend) {
            std::vector<real> blk = p.c;
            if (p.b_idx >= 0) blk.push_back(p.b);
            if (p.n_idx >= 0) blk.push_back(p.nn);
            RowKey key{std::string(reinterpret_cast<const char*>(blk.data()),
                                   blk.size() * sizeof(real))};
            auto it = pool.find(key);
            int off;
            if (it == pool.end()) {
                // blocks start at even offsets, so the FP32-pair copy of the pool is read two
                // coefficients (16 bytes) at a time; the pool ends with a zero pad for that
                if (T.coef.size() % 2) T.coef.push_back(0.0);
                off = (int)T.coef.size();
                T.coef.insert(T.coef.end(), blk.begin(), blk.end());
                pool.emplace(std::move(key), off);
            } else {
                off = it->second;
            }
            ClosureRow cr{};
            cr.coef_off = off;
            cr.col0 = (int16_t)p.col0;
            cr.ncol = (uint8_t)p.c.size();
            cr.flags = (uint8_t)((p.b_idx >= 0 ? ROWF_B : 0) | (p.n_idx >= 0 ? ROWF_N : 0));
            cr.b_idx = (int32_t)p.b_idx;
            cr.n_idx = (int32_t)p.n_idx;
            T.rows.push_back(cr);
            T.row_out.push_back(p.out);
        }
        T.coef.push_back(0.0);
        if (T.coef.size() % 2) T.coef.push_back(0.0);
        // chunk prefix counts over the iteration space
        T.chunk_base.assign(n_chunks + 1, 0);
        const i64 it2 = C.it[2];
        for (i64 out : T.row_out) {
            const i64 ch = (out / it2) * C.nzc + (out % it2) / 32;
            T.chunk_base[ch + 1]++;
        }
        for (i64 c = 0; c < n_chunks; c++) T.chunk_base[c + 1] += T.chunk_base[c];

        // R-space rows
        for (int r = 0; r < 3; r++) {
            const Csr& Bf = A.Bf[r];
            const Csr& Br = A.Br[r];
            const i64 nr = (i64)m.R[r].size();
            if (Bf.w.empty() && Br.w.empty()) continue;
            T.rr_u[r].assign(nr + 1, 0);
            for (i64 row = 0; row < nr; row++) {
                if (row < Bf.rows)
                    for (i64 q = Bf.u[row]; q < Bf.u[row + 1]; q++) {
                        T.rr_col[r].push_back((int)Bf.v[q]);
                        T.rr_src[r].push_back(0);
                        T.rr_w[r].push_back(Bf.w[q]);
                    }
                if (row < Br.rows)
                    for (i64 q = Br.u[row]; q < Br.u[row + 1]; q++) {
                        T.rr_col[r].push_back((int)Br.v[q]);
                        T.rr_src[r].push_back(1);
                        T.rr_w[r].push_back(Br.w[q]);
                    }
                T.rr_u[r][row + 1] = (int)T.rr_col[r].size();
            }
        }
    }
    return C;
}

} // namespace sgb
