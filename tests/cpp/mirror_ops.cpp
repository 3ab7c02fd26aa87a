// Drives the library through the C++ classes of include/shoccs_gb300.hpp the way a caller of
// the reference's classes would: a 2-D mesh with one circle, derivative / laplacian /
// gradient applies, and a heat system stepped by integrators::rk4.  Inputs and outputs are
// raw binary files in the directory given as argv[1] (written and read by
// tests/test_cpp_mirror.py, which runs the same cases through the Python binding and
// compares the bits):
//   in:  u.f64 (D then Rx, Ry, Rz of the problem; FP64)
//   out: dx.f64, dx_plus.f64, lap.f64, gx.f64, gy.f64, lap_mixed.f32, heat_fp64.f64,
//        heat_mixed.f64 (the state after 100 steps), stats.txt, system.csv, and the field
//        writer's output of two simulation cycles under io2d/ and io3d/
#include "shoccs_gb300.hpp"

#include <cuda_runtime.h>

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

namespace
{
template <typename T>
std::vector<T> read_file(const std::string& path, std::size_t n)
{
    std::vector<T> v(n);
    std::ifstream f(path, std::ios::binary);
    if (!f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T))))
        throw std::runtime_error("cannot read " + path);
    return v;
}

template <typename T>
void write_file(const std::string& path, const std::vector<T>& v)
{
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(v.data()), (std::streamsize)(v.size() * sizeof(T)));
}

void cuda(cudaError_t e)
{
    if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e));
}

// a device copy of a {D, Rx, Ry, Rz} field
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
    ccs::scalar_ref<const T> view() const
    {
        return {{p[0], n[0]}, {p[1], n[1]}, {p[2], n[2]}, {p[3], n[3]}};
    }
    void upload(const std::vector<T>& host)
    {
        std::size_t off = 0;
        for (int i = 0; i < 4; i++) {
            if (n[i]) cuda(cudaMemcpy(p[i], host.data() + off, n[i] * sizeof(T), cudaMemcpyHostToDevice));
            off += n[i];
        }
    }
    std::vector<T> download() const
    {
        std::vector<T> host(n[0] + n[1] + n[2] + n[3]);
        std::size_t off = 0;
        for (int i = 0; i < 4; i++) {
            if (n[i]) cuda(cudaMemcpy(host.data() + off, p[i], n[i] * sizeof(T), cudaMemcpyDeviceToHost));
            off += n[i];
        }
        return host;
    }
};
} // namespace

int main(int argc, char** argv)
{
    if (argc < 2) {
        std::fprintf(stderr, "usage: mirror_ops <dir>\n");
        return 2;
    }
    try {
        using namespace ccs;
        const std::string dir = argv[1];
        // the 2-D heat case: 65^2 on [0,1]^2, circle (0.51, 0.49) r = 0.2, E4_2
        const mesh m{index_extents{{65, 65, 1}}, domain_extents{{0, 0, 0}, {1, 1, 0}},
                     {make_sphere(0, {0.51, 0.49, 0.0}, 0.2)}};
        const bcs::Grid g{bcs::dd, bcs::dd, bcs::ff};
        const bcs::Object o{bcs::Dirichlet};
        const stencil st = stencils::make_E4_2();

        const problem p{m, st, g, o};
        const std::array<std::size_t, 4> n{(std::size_t)p.size(), (std::size_t)p.R(0),
                                           (std::size_t)p.R(1), (std::size_t)p.R(2)};
        device_field<double> u(n), du(n), lap(n), gx(n), gy(n), gz(n);
        u.upload(read_file<double>(dir + "/u.f64", n[0] + n[1] + n[2] + n[3]));

        const derivative dx(0, p);
        dx(u.view(), du.span());
        write_file(dir + "/dx.f64", du.download());
        dx(u.view(), du.span(), plus_eq);
        write_file(dir + "/dx_plus.f64", du.download());

        const laplacian L(p);
        L(u.view())(lap.span());
        write_file(dir + "/lap.f64", lap.download());

        const gradient G(p);
        G(u.view())(gx.span(), gy.span(), gz.span());
        write_file(dir + "/gx.f64", gx.download());
        write_file(dir + "/gy.f64", gy.download());

        // the mixed-precision Laplacian on the FP32 copy of u
        device_field<float> uf(n), lapf(n);
        {
            const auto h = u.download();
            uf.upload(std::vector<float>(h.begin(), h.end()));
        }
        const laplacian Lm(p, precision::mixed);
        Lm(uf.view())(lapf.span());
        write_file(dir + "/lap_mixed.f32", lapf.download());

        // heat with the manufactured sin-sin solution, 100 RK4 steps at dt = 0.1 h^2
        std::FILE* out = std::fopen((dir + "/stats.txt").c_str(), "w");
        if (!out) throw std::runtime_error("cannot write stats.txt");
        for (const precision prec : {precision::fp64, precision::mixed}) {
            systems::heat h(mesh{m}, bcs::Grid{g}, bcs::Object{o}, mms::sinsin(1.0), st, 1.0, prec);
            h.initialize(0.0);
            const real dt = h.timestep_size(0.4);
            integrators::rk4{}.run(h, 0.0, dt, 100);
            const auto s = h.stats(100 * dt);
            device_field<double> state(n);
            h.get_state(state.span());
            const bool mixed = prec == precision::mixed;
            write_file(dir + (mixed ? "/heat_mixed.f64" : "/heat_fp64.f64"), state.download());
            std::fprintf(out, "%s linf %.17g valid %d dt %.17g\n", mixed ? "mixed" : "fp64", s.stats[0],
                         (int)h.valid(s), dt);
        }
        // the reference's per-step call shape: rk4(system, t, dt) once per step
        {
            systems::heat h(mesh{m}, bcs::Grid{g}, bcs::Object{o}, mms::sinsin(1.0), st, 1.0);
            h.initialize(0.0);
            const real dt = h.timestep_size(0.4);
            const integrators::rk4 step;
            for (int i = 0; i < 100; i++) step(h, i * dt, dt);
            std::fprintf(out, "stepwise linf %.17g\n", h.stats(100 * dt).stats[0]);
        }
        // the simulation cycle: 100 steps of the heat case, the system log to a file
        {
            systems::heat h(mesh{m}, bcs::Grid{g}, bcs::Object{o}, mms::sinsin(1.0), st, 1.0);
            std::ofstream log(dir + "/system.csv");
            io_config cfg;
            cfg.write_every_step = 40;
            cfg.dir = dir + "/io2d";
            simulation_cycle cycle(step_controller(100, 1e9, 0.5, 0.4), &log, field_io::from_config(m, cfg));
            const real3 r = cycle.run(h);
            std::fprintf(out, "cycle %.17g %.17g %d\n", r[0], r[1], cycle.controller().simulation_step());
            std::fprintf(out, "io2d_dumps %d\n", cycle.io().current_dump());
        }
        // field output on a time schedule: FP64 heat around a Floating sphere (cut-point values
        // are state, so the Error field has nonzero cut-point parts), 10 steps, a dump every
        // 3 dt of simulation time
        {
            const mesh m3{index_extents{{24, 24, 24}}, domain_extents{{0, 0, 0}, {1, 1, 1}},
                          {make_sphere(0, {0.5, 0.5, 0.5}, 0.25)}};
            systems::heat h(mesh{m3}, bcs::Grid{bcs::dd, bcs::dd, bcs::dd}, bcs::Object{bcs::Floating},
                            mms::sinsin(1.0), stencils::make_E4_2(), 1.0);
            const real dt = h.timestep_size(0.4);
            io_config cfg;
            cfg.write_every_time = 3 * dt;
            cfg.dir = dir + "/io3d";
            cfg.suffix_length = 4;
            cfg.xdmf_filename = "floating.xmf";
            simulation_cycle cycle(step_controller(10, 1e9, 0.5, 0.4), nullptr, field_io::from_config(m3, cfg));
            const real3 r = cycle.run(h);
            std::fprintf(out, "io3d %.17g %d %d %.17g\n", r[0], cycle.controller().simulation_step(),
                         cycle.io().current_dump(), dt);
        }
        // error behaviour: E4_1's alpha bound, and a status the library refuses
        try {
            const real bad[2] = {0.1, 0.5};
            (void)stencils::make_E4_1(bad);
            std::fprintf(out, "e4_1_bound none\n");
        } catch (const std::invalid_argument&) {
            std::fprintf(out, "e4_1_bound invalid_argument\n");
        }
        try {
            const mesh m3{index_extents{{24, 24, 24}}, domain_extents{{0, 0, 0}, {1, 1, 1}},
                          {make_sphere(0, {0.5, 0.5, 0.5}, 0.25)}};
            // a Floating object's cut-point values are state (the unfused step, FP64 state in
            // either precision); the forward Euler integrator steps FP64 systems only
            systems::heat h(mesh{m3}, bcs::Grid{bcs::dd, bcs::dd, bcs::dd}, bcs::Object{bcs::Floating},
                            mms::zero(), stencils::make_E4_2(), 1.0, precision::mixed);
            h.initialize(0.0);
            integrators::rk4{}.run(h, 0.0, 1e-4, 1);
            integrators::euler{}.run(h, 0.0, 1e-4, 1);
            std::fprintf(out, "floating_object none\n");
        } catch (const ccs::error& e) {
            std::fprintf(out, "floating_object status %d\n", (int)e.status());
        }
        std::fclose(out);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
