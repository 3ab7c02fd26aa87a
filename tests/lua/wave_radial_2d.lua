-- Radial scalar wave on a 2-D box without embedded shapes: the velocity points away from a
-- centre outside the box and the exact solution is sin(2 pi (|x - c| - r - t)).  Dirichlet
-- data on the inflow sides, E4u first-derivative scheme, field dumps every 4 steps.
local n = 41
local side = 1.25

simulation = {
    mesh = {
        index_extents = {n, n},
        domain_bounds = {side, side}
    },
    domain_boundaries = {
        xmin = "dirichlet",
        ymin = "dirichlet",
    },
    shapes = {},
    scheme = {order = 1, type = "E4u", alpha = {-0.7733323791884821, 0.1623961700641681}},
    system = {
        type = "scalar wave",
        center = {-0.3, -0.2, 0},
        radius = 0,
        max_error = 10.0
    },
    integrator = {type = "rk4"},
    step_controller = {
        max_time = 0.25,
        cfl = {hyperbolic = 0.5}
    },
    io = {write_every_step = 4, dir = "out"}
}
