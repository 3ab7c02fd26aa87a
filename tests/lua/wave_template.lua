-- Template in the form a driver script fills in by plain text substitution: the three
-- markers (N, T_FINAL and SCHEME_TABLE between double braces, inside Lua line comments) are
-- replaced before the file is run, so this file is not runnable as it stands.

simulation = {
    mesh = {
        index_extents = {--{{N}}--, --{{N}}--},
        domain_bounds = {1, 1}
    },
    domain_boundaries = {
        xmin = "dirichlet",
        ymin = "dirichlet"
    },
    shapes = {},
    scheme = --{{SCHEME_TABLE}}--,
    system = {
        type = "scalar wave",
        center = {-0.25, -0.25, 0},
        radius = 0,
        max_error = 10.0
    },
    integrator = {
        type = "rk4"
    },
    step_controller = {
        max_time = --{{T_FINAL}}--,
        cfl = {
            hyperbolic = 0.5
        }
    },
    io = {
        write_every_step = 10
    }
}
