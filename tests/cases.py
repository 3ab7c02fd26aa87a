"""Problem configurations shared by the parity tests.

Each case is a dict accepted by both shoccs_gb300.Problem and oracle.OracleProblem.
"""
import numpy as np

DIR, FLT, NEU = "dirichlet", "floating", "neumann"


def random_spheres(n_spheres, seed, lo=0.15, hi=0.85, rmin=0.03, rmax=0.08, gap=0.0, bcs=(DIR,)):
    """Seeded non-overlapping spheres (rejection sampling with a clearance `gap`)."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n_spheres:
        c = rng.uniform(lo, hi, 3)
        r = rng.uniform(rmin, rmax)
        if all(np.linalg.norm(c - np.array(c2)) > r + r2 + gap for c2, r2, _ in out):
            out.append((tuple(float(v) for v in c), float(r), bcs[len(out) % len(bcs)]))
    return out


# E2-poly (polyE2_1) parameters of the reference's scalar_wave.lua: floating alpha[6],
# dirichlet alpha[3], interpolant alpha[4] (the single-array order of stencil.cpp:79-87)
POLY_ALPHA_LUA = (0.7039278390946743, 0.5390086175376538, -0.647109821986589, 0.2051508287133347,
                  0.6062051039572746, 0.8148425279273044, -0.10739761225713096,
                  0.8736492896991024, 0.40413606410467495, 0.01, -0.01, 0.01, 0.04)


# the alpha of the reference's own E6u_1 and E8u_1 tests (src/stencils/E6u_1.t.cpp:25,
# E8u_1.t.cpp:25-31)
E6U_ALPHA = (0.1, 0.2, 0.3, 0.4, 0.5)
E8U_ALPHA = (-0.6484343281044554, 0.1546307245964576, -0.0024361150534464, -0.0767677234359209,
             0.0395245547501803, -0.25779890216368, 0.0527307049447768)


def cases():
    from shoccs_gb300 import workloads as W
    return {
        # the uniform-grid 6th- and 8th-order first derivatives: a Dirichlet sphere (their
        # closures have no cross-direction interpolant, so objects are Dirichlet)
        "e6u_sphere_3d": dict(n=(30, 28, 32), lo=(0, 0, 0), hi=(1, 1, 1),
                              spheres=[((0.5, 0.48, 0.52), 0.16, DIR)],
                              grid_bc=(DIR, FLT) * 3, scheme="E6u_1", alpha=E6U_ALPHA),
        "e8u_circle_2d": dict(n=(61, 57, 1), lo=(0, 0, 0), hi=(1, 1, 0),
                              spheres=[((0.52, 0.47, 0.0), 0.17, DIR)],
                              grid_bc=(DIR, FLT, DIR, FLT, FLT, FLT), scheme="E8u_1", alpha=E8U_ALPHA),
        # E2-poly on the geometry of the reference's scalar_wave.lua: a Dirichlet quarter
        # circle at (0, 0) and a Floating one at (2, 2) on [0, 2]^2, inflow faces Dirichlet
        "poly_scalar_wave_2d": dict(n=(71, 71, 1), lo=(0, 0, 0), hi=(2, 2, 0),
                                    spheres=[((0.0, 0.0, 0.0), np.pi / 10, DIR),
                                             ((2.0, 2.0, 0.0), np.pi / 10, FLT)],
                                    grid_bc=(DIR, FLT, DIR, FLT, FLT, FLT), scheme="polyE2_1",
                                    alpha=POLY_ALPHA_LUA),
        # E2-poly in 3-D: a Floating and a Dirichlet sphere
        "poly_spheres_3d": dict(n=(28, 26, 30), lo=(0, 0, 0), hi=(1, 1, 1),
                                spheres=[((0.35, 0.37, 0.4), 0.14, FLT),
                                         ((0.66, 0.64, 0.62), 0.12, DIR)],
                                grid_bc=(DIR, FLT) * 3, scheme="polyE2_1", alpha=POLY_ALPHA_LUA),
        # the operator microbenchmark's generator (8 seeded spheres, gap >= 8h) at 96^3:
        # E4_1 derivative with Dirichlet spheres, E4_2 Laplacian with Dirichlet and Floating
        "micro_e41_96": W.micro_case(96, "E4_1", (DIR,)),
        "micro_e42_96": W.micro_case(96, "E4_2", (DIR, FLT)),
        # the adjoint configuration's geometry at 24^3
        "adjoint_24": W.adjoint_case(24),
        # Neumann walls on both z faces (the z-wall rows of the vectorised operators carry
        # the Neumann term), Floating sphere
        "neumann_z_e42": dict(n=(20, 18, 24), lo=(0, 0, 0), hi=(1, 1, 1),
                              spheres=[((0.5, 0.52, 0.47), 0.22, FLT)],
                              grid_bc=(DIR, FLT, FLT, DIR, NEU, NEU), scheme="E4_2"),
        # configuration 0 of the benchmark: 2-D heat, circle, E4_2, Dirichlet walls
        "c0_circle_2d": dict(n=(65, 65, 1), lo=(0, 0, 0), hi=(1, 1, 0),
                             spheres=[((0.51, 0.49, 0.0), 0.2, DIR)],
                             grid_bc=(DIR, DIR, DIR, DIR, FLT, FLT), scheme="E4_2"),
        # small copy of the 3-D wave configuration: sphere r=0.3, inflow faces Dirichlet
        "wave_sphere_3d": dict(n=(40, 38, 42), lo=(0, 0, 0), hi=(1, 1, 1),
                               spheres=[((0.5, 0.5, 0.5), 0.22, DIR)],
                               grid_bc=(DIR, FLT, DIR, FLT, DIR, FLT), scheme="E4_1",
                               alpha=(0.1, 0.7)),
        # the domain and sphere of the reference's geometry test (object_geometry.t.cpp:16-31)
        # on a finer grid, so that the wall-to-sphere segments hold both closures
        "ref_geometry_mesh": dict(n=(41, 44, 61), lo=(-1, -1, 0), hi=(1, 2, 2.2),
                                  spheres=[((0.01, -0.01, 0.5), 0.25, DIR)],
                                  grid_bc=(DIR, DIR, FLT, FLT, DIR, FLT), scheme="E4_2"),
        # Floating object: cross-direction interpolation rows (E4_2)
        "floating_sphere_e42": dict(n=(21, 19, 23), lo=(-1, -1, -1), hi=(1, 1, 1),
                                    spheres=[((0.1, -0.05, 0.02), 0.45, FLT)],
                                    grid_bc=(FLT, DIR, DIR, FLT, FLT, FLT), scheme="E4_2"),
        # E2_2 with Neumann faces and a Floating object
        "neumann_e22": dict(n=(17, 18, 16), lo=(0, 0, 0), hi=(1, 1, 1),
                            spheres=[((0.45, 0.52, 0.5), 0.27, FLT)],
                            grid_bc=(NEU, FLT, FLT, NEU, DIR, FLT), scheme="E2_2"),
        # a Neumann sphere beside a Dirichlet one (E4_2): the object's Neumann closure rows
        # keep its cut point as a column and carry no Neumann data; one Neumann face
        "neumann_objects_e42": dict(n=(26, 24, 28), lo=(0, 0, 0), hi=(1, 1, 1),
                                    spheres=[((0.3, 0.33, 0.36), 0.14, NEU),
                                             ((0.66, 0.64, 0.62), 0.14, DIR)],
                                    grid_bc=(DIR, FLT, NEU, DIR, FLT, DIR), scheme="E4_2"),
        # several seeded spheres, E4_1 (Dirichlet objects)
        "multi_sphere_e41": dict(n=(64, 60, 66), lo=(0, 0, 0), hi=(1, 1, 1),
                                 spheres=random_spheres(5, 20261204, lo=0.3, hi=0.7,
                                                        rmin=0.04, rmax=0.07, gap=0.18),
                                 grid_bc=(FLT, FLT, DIR, FLT, FLT, DIR), scheme="E4_1",
                                 alpha=(0.1, 0.7)),
        # several seeded spheres, E4_2, Dirichlet and Floating objects
        "multi_sphere_e42": dict(n=(48, 44, 50), lo=(0, 0, 0), hi=(1, 1, 1),
                                 spheres=random_spheres(5, 7, lo=0.25, hi=0.75, rmin=0.05,
                                                        rmax=0.09, gap=0.12, bcs=(DIR, FLT)),
                                 grid_bc=(DIR, DIR, FLT, FLT, DIR, DIR), scheme="E4_2"),
        # no objects at all, all-Floating walls
        "plain_box_e42": dict(n=(12, 9, 40), lo=(0, 0, 0), hi=(1, 2, 3), spheres=[],
                              grid_bc=(FLT,) * 6, scheme="E4_2"),
        # uniform-grid first-derivative scheme (E4u_1), Dirichlet inflow / Floating outflow
        "box_e4u": dict(n=(34, 30, 36), lo=(0, 0, 0), hi=(1, 1, 1), spheres=[],
                        grid_bc=(DIR, FLT, DIR, FLT, DIR, FLT), scheme="E4u_1",
                        alpha=(-0.7733323791884821, 0.1623961700641681)),
        # 1-D line
        "line_1d_e41": dict(n=(64, 1, 1), lo=(0, 0, 0), hi=(1, 0, 0), spheres=[],
                            grid_bc=(DIR, FLT, FLT, FLT, FLT, FLT), scheme="E4_1",
                            alpha=(0.1, 0.7)),
    }
