// ref_driver.cpp -- C entry points over the reference's OWN stencil and sphere code.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.sh together with the reference
// translation units src/stencils/{E2_2,E4_2,E4_1,E4u_1}.cpp and src/mesh/sphere.cpp taken
// unmodified from the reference tree, into oracle/_ref/libshoccs_ref.so.  Used only by
// tests/golden/make_golden.py to pin the oracle restatement bit-for-bit.
#include "mesh/shapes.hpp"
#include "stencils/stencil.hpp"

#include <cmath>
#include <vector>

using namespace ccs;
using namespace ccs::stencils;

static stencil make(int scheme, const double* alpha)
{
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

extern "C" {

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

int ref_stencil_interp_wall(int scheme, int i, double y, double psi, int right, double* c)
{
    auto st = make(scheme, nullptr);
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
    auto h = s.hit(r, t_min, t_max);
    if (!h) return 0;
    *t = h->t;
    for (int k = 0; k < 3; k++) pos[k] = h->position[k];
    *ray_outside = h->ray_outside;
    auto n = s.normal(h->position);
    for (int k = 0; k < 3; k++) normal[k] = n[k];
    return 1;
}
}
