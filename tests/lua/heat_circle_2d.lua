-- Heat equation on the unit square around a Dirichlet circle, E4 second-derivative scheme,
-- manufactured solution sin(2 pi x) sin(2 pi y) e^-t (the "sinsin" closed form), 60 steps,
-- field dumps on a simulation-time schedule, the system log under mylogs/.
local h = 1 / 64
local dt = 0.4 * h ^ 2 / 4

simulation = {
    mesh = {
        index_extents = {65, 65},
        domain_bounds = {min = {0, 0}, max = {1, 1}}
    },
    domain_boundaries = {
        xmin = "dirichlet", xmax = "dirichlet",
        ymin = "dirichlet", ymax = "dirichlet"
    },
    shapes = {
        {type = "sphere", center = {0.51, 0.49}, radius = 0.2, boundary_condition = "dirichlet"}
    },
    scheme = {order = 2, type = "E4"},
    system = {type = "heat", diffusivity = 1.0},
    manufactured_solution = {type = "sinsin", frequency = 1},
    integrator = {type = "rk4"},
    step_controller = {
        max_step = 60,
        cfl = {parabolic = 0.4}
    },
    io = {write_every_time = 7 * dt, dir = "fields", suffix_length = 4, xdmf_filename = "heat.xmf"},
    logging_dir = "mylogs"
}
