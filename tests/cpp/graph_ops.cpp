// Graph forms of the operators and systems (include/shoccs_gb300.hpp) against their eager
// applies, the pattern of the reference's "graph matches eager" tests
// (src/operators/derivative.t.cpp:423-513): every output of a submitted graph must equal the
// eager apply's output bit for bit, a resubmitted graph must give the same result again, a
// plus_eq graph must accumulate on each submit, and a right-hand-side graph must follow the
// system's state and the submit's time.  Cases: a 3-D grid around a Dirichlet sphere with
// Neumann z faces (E4_2: FP64 operators and the vectorised FP32 operators, nz a multiple of
// 4), a 3-D grid with a Floating sphere (R-space rows), the 2-D heat configuration.
// Prints one line per check and exits 0 when every check holds.
#include "shoccs_gb300.hpp"

#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace
{
int failures = 0;

void cuda(cudaError_t e)
{
    if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
}

template <typename T>
struct device_field {
    std::array<std::size_t, 4> n{};
    std::array<T*, 4> p{};
    explicit device_field(const std::array<std::size_t, 4>& sizes) : n{sizes}
    {
        for (int i = 0; i < 4; i++) {
            cuda(cudaMalloc(&p[i], std::max<std::size_t>(n[i], 1) * sizeof(T)));
            cuda(cudaMemset(p[i], 0, std::max<std::size_t>(n[i], 1) * sizeof(T)));
        }
    }
    ~device_field()
    {
        for (auto q : p) cudaFree(q);
    }
    device_field(const device_field&) = delete;
    device_field& operator=(const device_field&) = delete;
    ccs::scalar_ref<T> span() { return {{p[0], n[0]}, {p[1], n[1]}, {p[2], n[2]}, {p[3], n[3]}}; }
    ccs::scalar_ref<const T> view() const { return {{p[0], n[0]}, {p[1], n[1]}, {p[2], n[2]}, {p[3], n[3]}}; }
    void upload(const std::vector<T>& h)
    {
        std::size_t off = 0;
        for (int i = 0; i < 4; i++) {
            if (n[i]) cuda(cudaMemcpy(p[i], h.data() + off, n[i] * sizeof(T), cudaMemcpyHostToDevice));
            off += n[i];
        }
    }
    std::vector<T> download() const
    {
        std::vector<T> h(n[0] + n[1] + n[2] + n[3]);
        std::size_t off = 0;
        for (int i = 0; i < 4; i++) {
            if (n[i]) cuda(cudaMemcpy(h.data() + off, p[i], n[i] * sizeof(T), cudaMemcpyDeviceToHost));
            off += n[i];
        }
        return h;
    }
    void fill(T v)
    {
        upload(std::vector<T>(n[0] + n[1] + n[2] + n[3], v));
    }
};

// deterministic values in [-1, 1]
template <typename T>
std::vector<T> seeded(std::size_t n, unsigned long long seed)
{
    std::vector<T> v(n);
    unsigned long long x = seed * 6364136223846793005ULL + 1442695040888963407ULL;
    for (auto& e : v) {
        x = x * 6364136223846793005ULL + 1442695040888963407ULL;
        e = (T)((double)(x >> 11) / (double)(1ULL << 53) * 2.0 - 1.0);
    }
    return v;
}

template <typename T>
void same(const std::string& what, const std::vector<T>& a, const std::vector<T>& b)
{
    const bool ok = a.size() == b.size() && std::memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0;
    double d = 0.0;
    if (!ok && a.size() == b.size())
        for (std::size_t i = 0; i < a.size(); i++) d = std::max(d, std::fabs((double)a[i] - (double)b[i]));
    std::printf("%s %s%s\n", ok ? "OK  " : "FAIL", what.c_str(),
                ok ? "" : (" max diff " + std::to_string(d)).c_str());
    if (!ok) ++failures;
}

template <typename T>
void operators(const std::string& name, const ccs::problem& p, std::array<int, 3> ext,
               ccs::precision prec, bool neumann)
{
    using namespace ccs;
    const std::array<std::size_t, 4> n{(std::size_t)p.size(), (std::size_t)p.R(0), (std::size_t)p.R(1),
                                       (std::size_t)p.R(2)};
    const std::size_t tot = n[0] + n[1] + n[2] + n[3];
    device_field<T> u(n), e(n), g(n);
    device_field<double> nu(n);
    u.upload(seeded<T>(tot, 7));
    nu.upload(seeded<double>(tot, 11));
    const std::string tag = name + (prec == precision::mixed ? " mixed" : " fp64");
    for (int dir = 0; dir < 3; dir++) {
        if (ext[dir] < 2) continue;
        derivative d(dir, p, prec);
        // eq (which writes the rows of the axis and, like the reference's csr matvecs, adds the
        // R-space rows of Floating objects), then the same again from the same start
        e.fill(0.5);
        g.fill(0.5);
        d(u.view(), e.span());
        d.build_graph(u.view(), g.span());
        d.submit_graph();
        same(tag + " derivative " + std::to_string(dir) + " eq", e.download(), g.download());
        e.fill(0.5);
        g.fill(0.5);
        d(u.view(), e.span());
        d.submit_graph();
        same(tag + " derivative " + std::to_string(dir) + " resubmit", e.download(), g.download());
        // plus_eq accumulates on every submit
        e.fill(1);
        g.fill(1);
        d(u.view(), e.span(), plus_eq);
        d(u.view(), e.span(), plus_eq);
        d.build_graph(u.view(), g.span(), plus_eq);
        d.submit_graph();
        d.submit_graph();
        same(tag + " derivative " + std::to_string(dir) + " plus_eq twice", e.download(), g.download());
        if (neumann) {
            e.fill(0.5);
            g.fill(0.5);
            d(u.view(), nu.view(), e.span());
            d.build_graph(u.view(), nu.view(), g.span());
            d.submit_graph();
            same(tag + " derivative " + std::to_string(dir) + " with Neumann data", e.download(),
                 g.download());
        }
    }
    laplacian L(p, prec);
    L(u.view())(e.span());
    L.build_graph(u.view(), g.span());
    L.submit_graph();
    same(tag + " laplacian", e.download(), g.download());
    if (neumann) {
        L(u.view(), nu.view())(e.span());
        L.build_graph(u.view(), nu.view(), g.span());
        L.submit_graph();
        same(tag + " laplacian with Neumann data", e.download(), g.download());
    }
    // one graph holding a derivative, the Laplacian and the gradient
    device_field<T> ex(n), ey(n), ez(n), gx(n), gy(n), gz(n), e2(n), g2(n);
    const gradient G(p, prec);
    G(u.view())(ex.span(), ey.span(), ez.span());
    const derivative d0(0, p, prec);
    d0(u.view(), e2.span()); // applied twice, as the graph is submitted twice
    d0(u.view(), e2.span());
    L(u.view())(e.span());
    graph all;
    d0.add_graph_nodes(all, u.view(), g2.span());
    L.add_graph_nodes(all, u.view(), g.span());
    G.add_graph_nodes(all, u.view(), gx.span(), gy.span(), gz.span());
    all.submit();
    all.submit();
    same(tag + " composite graph: derivative", e2.download(), g2.download());
    same(tag + " composite graph: laplacian", e.download(), g.download());
    same(tag + " composite graph: gradient x", ex.download(), gx.download());
    same(tag + " composite graph: gradient y", ey.download(), gy.download());
    same(tag + " composite graph: gradient z", ez.download(), gz.download());
    const auto info = all.info();
    std::printf("     %s composite graph: %lld applies, %lld nodes, %lld captures\n", tag.c_str(),
                (long long)info[0], (long long)info[1], (long long)info[2]);
    if (info[0] != 3 || info[1] < 3 || info[2] != 1) {
        std::printf("FAIL %s composite graph info\n", tag.c_str());
        ++failures;
    }
}

void rhs_graph(const std::string& name, const ccs::problem& p, ccs::precision prec)
{
    using namespace ccs;
    const std::array<std::size_t, 4> n{(std::size_t)p.size(), (std::size_t)p.R(0), (std::size_t)p.R(1),
                                       (std::size_t)p.R(2)};
    device_field<double> e(n), g(n), state(n);
    systems::heat h(p, mms::sinsin(1.0), 0.7, prec);
    const std::string tag = name + (prec == precision::mixed ? " mixed" : " fp64");
    h.initialize(0.0);
    h.build_rhs_graph(g.span());
    for (const real t : {0.0, 0.013, 0.013, 0.02}) {
        h.rhs(t, e.span());
        h.submit_rhs_graph(t);
        same(tag + " heat rhs graph at t = " + std::to_string(t), e.download(), g.download());
    }
    // the graph reads the state the system holds when it runs
    integrators::rk4{}.run(h, 0.0, 1e-5, 3);
    h.rhs(0.02, e.span());
    h.submit_rhs_graph(0.02);
    same(tag + " heat rhs graph after RK4 steps", e.download(), g.download());
}
} // namespace

int main()
{
    try {
        using namespace ccs;
        const stencil st = stencils::make_E4_2();
        {
            // 3-D, Dirichlet sphere, Dirichlet x faces, Floating y, Neumann z (nz % 4 == 0)
            const mesh m{index_extents{{34, 30, 40}}, domain_extents{{0, 0, 0}, {1, 1, 1}},
                         {make_sphere(0, {0.48, 0.52, 0.5}, 0.22)}};
            const problem p{m, st, bcs::Grid{bcs::dd, bcs::ff, bcs::nn}, bcs::Object{bcs::Dirichlet}};
            operators<double>("sphere3d", p, {34, 30, 40}, precision::fp64, true);
            operators<float>("sphere3d", p, {34, 30, 40}, precision::mixed, true);
        }
        {
            // 3-D, Floating sphere: R-space rows (Bf, Br) in every apply
            const mesh m{index_extents{{26, 24, 28}}, domain_extents{{0, 0, 0}, {1, 1, 1}},
                         {make_sphere(0, {0.5, 0.47, 0.52}, 0.24)}};
            const problem p{m, st, bcs::Grid{bcs::dd, bcs::df, bcs::ff}, bcs::Object{bcs::Floating}};
            operators<double>("floating3d", p, {26, 24, 28}, precision::fp64, false);
            rhs_graph("floating3d", p, precision::fp64);
        }
        {
            // the 2-D heat configuration: 65^2, circle, Dirichlet walls
            const mesh m{index_extents{{65, 65, 1}}, domain_extents{{0, 0, 0}, {1, 1, 0}},
                         {make_sphere(0, {0.51, 0.49, 0.0}, 0.2)}};
            const problem p{m, st, bcs::Grid{bcs::dd, bcs::dd, bcs::ff}, bcs::Object{bcs::Dirichlet}};
            operators<double>("circle2d", p, {65, 65, 1}, precision::fp64, false);
            rhs_graph("circle2d", p, precision::fp64);
            rhs_graph("circle2d", p, precision::mixed);
        }
    } catch (const std::exception& ex) {
        std::printf("FAIL exception: %s\n", ex.what());
        return 1;
    }
    std::printf("%d failure(s)\n", failures);
    return failures ? 1 : 0;
}
