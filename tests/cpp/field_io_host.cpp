// The field writer of include/shoccs_gb300.hpp on the host (no GPU, no library calls): the
// cases of the reference's src/io/interval.t.cpp, field_io.t.cpp and xdmf.t.cpp, plus a time
// schedule and cut-point geometry.  Writes under the directory given as argv[1]; prints one
// "name value..." line per check for tests/test_field_io.py.
#include "shoccs_gb300.hpp"

#include <cstdio>
#include <string>
#include <vector>

using namespace ccs;

int main(int argc, char** argv)
{
    if (argc < 2) return 2;
    const std::string dir = argv[1];

    // interval.t.cpp "Never fire"
    {
        interval<double> it;
        bool ok = !it;
        for (int i = 0; i < 50; ++i) ok = ok && !it(i);
        std::printf("never_fire %d\n", (int)ok);
    }
    // "No rollover": distance 1.5, values 0.5 i, fires at every third value
    {
        interval<double> it(1.5);
        bool ok = true;
        for (int i = 0; i < 50; ++i) {
            const double val = i * 0.5;
            if (i > 0 && i % 3 == 0) {
                ok = ok && it(val, 1e-6);
                ++it;
            } else {
                ok = ok && !it(val, 1e-6);
            }
        }
        std::printf("no_rollover %d\n", (int)ok);
    }
    // "Rollover": distance 4.5 over the integers 0..45 fires 10 times, at 5 and at 45
    {
        interval<double> it(4.5);
        int fires = 0;
        bool ok = true;
        for (int i = 0; i < 46; ++i) {
            const bool ready = it(i, 1e-6);
            if (i == 5) ok = ok && ready;
            if (i == 45) ok = ok && ready;
            if (ready) {
                ++fires;
                ++it;
            }
        }
        std::printf("rollover %d %d\n", (int)ok, fires);
    }
    // field_io.t.cpp "default": no io table, nothing is written
    {
        const mesh m{index_extents{{31, 1, 1}}, domain_extents{{0, 0, 0}, {2, 0, 0}}};
        field_io io = field_io::from_config(m, std::nullopt);
        const std::vector<std::string> names;
        const std::vector<scalar_view> fields;
        std::printf("default_writes %d\n", (int)io.write(names, fields, step_controller{}, 0.1, {}));
    }
    // field_io.t.cpp "data": 2x3x4, U = 0..23, V = 24..47, every step, dir io_test
    {
        const mesh m{index_extents{{2, 3, 4}}, domain_extents{{0.1, 0.2, 0.3}, {0.3, 0.5, 0.7}}};
        io_config cfg;
        cfg.write_every_step = 1;
        cfg.dir = dir + "/io_test";
        field_io io = field_io::from_config(m, cfg);
        std::vector<real> u(24), v(24);
        for (int i = 0; i < 24; i++) {
            u[i] = i;
            v[i] = 24 + i;
        }
        const std::vector<std::string> names{"U", "V"};
        const std::vector<scalar_view> fields{scalar_view{u, {}, {}, {}}, scalar_view{v, {}, {}, {}}};
        const bool w = io.write(names, fields, step_controller{}, 0.0, {});
        std::printf("data_writes %d %d\n", (int)w, io.current_dump());
    }
    // xdmf.t.cpp "header": two grids of U and V on 3x4x5, [0.1, 1.1] x [0.2, 1.2] x [0.3, 1.3]
    {
        const xdmf writer{dir + "/headertest.xmf", index_extents{{3, 4, 5}},
                          domain_extents{{0.1, 0.2, 0.3}, {1.1, 1.2, 1.3}}};
        const std::vector<std::string> var_names{"U", "V"};
        std::vector<std::string> file_names{"U.00000", "V.00000"};
        writer.write(0, 0.0, var_names, file_names, {});
        file_names = {"U.00001", "V.00001"};
        writer.write(1, 0.1, var_names, file_names, {});
        std::printf("header_written 1\n");
    }
    // a time schedule with cut points: every 0.25 of simulation time with dt = 0.1 (the
    // step size is the tolerance), 2-D grid (nz = 1: positions written as (z, y, x)),
    // three cut points in x, none in y, one in z; steps advance until t = 1
    {
        const mesh m{index_extents{{5, 4, 1}}, domain_extents{{0, 0, 0}, {1, 1, 0}}};
        io_config cfg;
        cfg.write_every_time = 0.25;
        cfg.dir = dir + "/io_time";
        cfg.suffix_length = 3;
        cfg.xdmf_filename = "t.xmf";
        field_io io = field_io::from_config(m, cfg);
        const std::vector<real3> rx{{0.1, 0.2, 0.0}, {0.3, 0.4, 0.0}, {0.5, 0.6, 0.0}};
        const std::vector<real3> rz{{0.7, 0.8, 0.0}};
        std::vector<real> d(20), ex(3), ez(1);
        const std::vector<std::string> names{"U"};
        step_controller c(100, 1e9, 0.5, 0.5);
        const real dt = 0.1;
        std::printf("time_dumps");
        for (int s = 0; s <= 10; s++) {
            for (int i = 0; i < 20; i++) d[i] = 100 * s + i;
            for (int i = 0; i < 3; i++) ex[i] = -(100 * s + i);
            ez[0] = 0.5 + s;
            const std::vector<scalar_view> fields{scalar_view{d, ex, {}, ez}};
            if (io.write(names, fields, c, s == 0 ? 0.0 : dt, cut_positions{rx, {}, rz}))
                std::printf(" %d", s);
            c.advance(dt);
        }
        std::printf("\n");
    }
    return 0;
}
