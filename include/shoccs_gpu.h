/* shoccs_gpu.h -- C ABI of the GB300 (sm_103a) SHOCCS derivative-operator hot path.
 *
 * The reference (pbrady/shoccs) exposes this path only as C++ classes; each entry point
 * below replaces one of them and keeps its argument meaning:
 *
 *   shoccs_problem_create   ccs::mesh(index_extents, domain_extents, shapes)
 *                             src/mesh/mesh.hpp:24-31, src/mesh/mesh.cpp:121-152
 *                           + bcs::Grid / bcs::Object   src/operators/boundaries.hpp:37-38
 *                           + stencil::from_lua         src/stencils/stencil.cpp:8-106
 *                           + derivative ctor (x, y, z) src/operators/derivative.cpp:452-473
 *   shoccs_problem_sizes    mesh::size(), mesh::R(dir).size()   src/mesh/mesh.hpp:35,71-97
 *   shoccs_problem_cut_points  mesh::R(dir) (mesh_object_info)  src/mesh/mesh_types.hpp:31-38
 *   shoccs_problem_block_meta  block::metadata_view()/coefficients_view()
 *                                                   src/matrices/block.hpp:30-113
 *   shoccs_problem_csr      derivative's B / N / Bf / Br csr matrices
 *                                                   src/operators/derivative.hpp:20-40
 *   shoccs_derivative_apply derivative::operator()(u[, nu], du, eq|plus_eq)
 *                                                   src/operators/derivative.cpp:502-519
 *   shoccs_laplacian_apply  laplacian::operator()(u[, nu])(du)  src/operators/laplacian.cpp:37-58
 *   shoccs_gradient_apply   gradient::operator()(u)(dx, dy, dz)  src/operators/gradient.cpp:35-46
 *   shoccs_system_create    systems::heat / systems::scalar_wave ctors
 *                                                   src/systems/heat.cpp:22-51,
 *                                                   src/systems/scalar_wave.cpp:44-102
 *   shoccs_system_initialize  system::initialize    src/systems/detail/scalar_system_utils.hpp:186-219
 *   shoccs_system_rk4       integrators::rk4::operator() applied nsteps times with the
 *                           simulation_cycle u0 <- u1 copy   src/temporal/rk4.cpp:16-47,
 *                                                   src/simulation/simulation_cycle.cpp:79-126
 *   shoccs_system_euler     integrators::euler::operator() applied nsteps times
 *                                                   src/temporal/euler.cpp:11-27
 *   shoccs_system_rhs       system::rhs             src/systems/heat.cpp:119-162,
 *                                                   src/systems/scalar_wave.cpp:195-239
 *   shoccs_system_stats     system::stats           src/systems/detail/scalar_system_utils.hpp:77-181
 *   shoccs_system_error_field  the Error field of system::write
 *                                                   src/systems/detail/scalar_system_utils.hpp:224-296
 *   shoccs_system_timestep  system::timestep_size   src/systems/heat.cpp:356-361,
 *                                                   src/systems/scalar_wave.cpp:357-362
 *   shoccs_graph_*          derivative / laplacian / gradient add_graph_nodes, build_graph,
 *                           submit_graph; system::build_rhs_graph / submit_rhs_graph
 *                                                   src/operators/derivative.hpp:71-151,
 *                                                   src/systems/system.cpp:57-69
 *
 * Conventions.  Fields are the reference's scalar {D, Rx, Ry, Rz} (src/fields/scalar.hpp:13-67):
 * D is the full nx*ny*nz grid (z fastest, solid points included), Rx/Ry/Rz hold one value
 * per cut point.  Pointers in shoccs_field are DEVICE pointers owned by the caller unless an
 * entry point says otherwise.  Every entry point returns a shoccs_status; on failure
 * shoccs_last_error() gives a one-line reason (the reference logs and returns std::nullopt
 * from from_lua, or asserts).  Handles are not thread-safe; use one per host thread.
 * Work is issued on the given CUDA stream (NULL = legacy default stream) and every entry
 * point returns after the stream has finished, like the reference's Kokkos::fence.
 */
#ifndef SHOCCS_GPU_H
#define SHOCCS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SHOCCS_OK = 0,
    SHOCCS_EINVAL = 1,      /* bad argument or configuration */
    SHOCCS_ENOMEM = 2,      /* device or host allocation failed */
    SHOCCS_ECUDA = 3,       /* a CUDA runtime call failed */
    SHOCCS_ETIMEOUT = 4,    /* a bounded device-side wait gave up */
    SHOCCS_ENONFINITE = 5,  /* the solution became non-finite or exceeded its bound */
    SHOCCS_EUNSUPPORTED = 6 /* valid in the reference but not provided by this path */
} shoccs_status;

/* boundary condition types, in the order of bcs::type (src/operators/boundaries.hpp:13-20) */
enum { SHOCCS_BC_DIRICHLET = 0, SHOCCS_BC_FLOATING = 1, SHOCCS_BC_NEUMANN = 2 };

/* schemes: scheme.order/type of stencil::from_lua (src/stencils/stencil.cpp:35-50) */
enum { SHOCCS_SCHEME_E2_2 = 0, SHOCCS_SCHEME_E4_2 = 1, SHOCCS_SCHEME_E4_1 = 2,
       SHOCCS_SCHEME_E4U_1 = 3 /* type "E4u" (src/stencils/stencil.cpp:51-53) */,
       SHOCCS_SCHEME_POLYE2_1 = 5 /* type "E2-poly" (src/stencils/stencil.cpp:78-100) */,
       SHOCCS_SCHEME_E6U_1 = 6 /* type "E6u" (src/stencils/stencil.cpp:54-56) */,
       SHOCCS_SCHEME_E8U_1 = 7 /* type "E8u" (src/stencils/stencil.cpp:57-59) */ };

/* arithmetic of the operator and system kernels */
enum {
    SHOCCS_PREC_FP64 = 0,  /* every value and coefficient in FP64 */
    SHOCCS_PREC_MIXED = 1  /* FP32 stage fields, interior and wall rows; cut-cell rows in
                              compensated FP32 over FP32-pair coefficients (FP64 with
                              SHOCCS_CUT_ROWS_FP64=1); FP32 stage accumulator; the solution a
                              compensated FP32 pair (~2^-46), updated by an error-free
                              two-sum -- FP64 on the unfused whole-field step, whose cut-point
                              stage values and rows are FP64 too */
};

typedef struct {
    int n[3];                 /* index_extents (1 for a trivial axis) */
    double lo[3], hi[3];      /* domain_bounds min / max */
    int n_spheres;
    const double* centers;    /* 3 * n_spheres */
    const double* radii;      /* n_spheres */
    const int* sphere_bc;     /* n_spheres: boundary_condition of each shape */
    int grid_bc[6];           /* xmin, xmax, ymin, ymax, zmin, zmax */
    int scheme;               /* SHOCCS_SCHEME_* */
    double alpha[2];          /* scheme.alpha (E4_1, E4u_1) */
    double scheme_alpha[13];  /* E2-poly: floating_alpha[6], dirichlet_alpha[3],
                                 interpolant_alpha[4] (src/stencils/polyE2_1.cpp:16-28);
                                 E6u: alpha[5]; E8u: alpha[7] (E6u_1.cpp:18, E8u_1.cpp:18) */
} shoccs_problem_desc;

typedef struct shoccs_problem shoccs_problem;
typedef struct shoccs_system shoccs_system;

/* A scalar field: device pointers to D, Rx, Ry, Rz; element type double (FP64) or float
 * (MIXED operators).  R pointers may be NULL when the matching R(dir) is empty. */
typedef struct {
    void* D;
    void* Rx;
    void* Ry;
    void* Rz;
} shoccs_field;

/* ---- problem (mesh + stencil + boundary conditions + compiled operators) ---- */
shoccs_status shoccs_problem_create(const shoccs_problem_desc* desc, shoccs_problem** out);
shoccs_status shoccs_problem_destroy(shoccs_problem* p);
/* sizes[0] = nx*ny*nz, sizes[1..3] = |Rx|, |Ry|, |Rz|, sizes[4] = fluid points */
shoccs_status shoccs_problem_sizes(const shoccs_problem* p, int64_t sizes[5]);
/* cut points of R(dir): psi[n], position[3n], normal[3n], ray_outside[n], solid_coord[3n],
 * shape_id[n] (any output may be NULL) */
shoccs_status shoccs_problem_cut_points(const shoccs_problem* p, int dir, double* psi,
                                        double* position, double* normal, int* ray_outside,
                                        int* solid_coord, int* shape_id);
/* per-line block metadata (13 ints per line, inner_block_meta order) and coefficients;
 * call with NULL buffers to query n_lines / n_coeffs */
shoccs_status shoccs_problem_block_meta(const shoccs_problem* p, int dir, int* meta,
                                        int64_t* n_lines, double* coeffs, int64_t* n_coeffs);
/* which: 0 B, 1 N, 2..4 Bf(r=0..2), 5..7 Br(r=0..2); row offsets have rows+1 entries */
shoccs_status shoccs_problem_csr(const shoccs_problem* p, int dir, int which, int64_t* rows,
                                 int64_t* nnz, int64_t* row_offsets, int64_t* cols,
                                 double* vals);
/* per-point class bytes of the compiled operator (host copy, nx*ny*nz bytes) */
shoccs_status shoccs_problem_classes(const shoccs_problem* p, uint8_t* cls);
/* upload the compiled operator to the current device (done lazily by apply calls) */
shoccs_status shoccs_problem_upload(shoccs_problem* p, void* stream);

/* ---- operators (device fields; prec selects double or float element type) ---- */
shoccs_status shoccs_derivative_apply(shoccs_problem* p, int dir, int prec,
                                      const shoccs_field* u, const shoccs_field* nu,
                                      shoccs_field* du, int plus_eq, void* stream);
shoccs_status shoccs_laplacian_apply(shoccs_problem* p, int prec, const shoccs_field* u,
                                     const shoccs_field* nu, shoccs_field* du, void* stream);
shoccs_status shoccs_gradient_apply(shoccs_problem* p, int prec, const shoccs_field* u,
                                    shoccs_field* dx, shoccs_field* dy, shoccs_field* dz,
                                    void* stream);

/* ---- systems ---- */
enum { SHOCCS_SYS_HEAT = 0, SHOCCS_SYS_WAVE = 1 };
/* exact / manufactured solutions with closed forms (params in shoccs_system_desc.sol) */
enum {
    SHOCCS_SOL_ZERO = 0,        /* u = 0 */
    SHOCCS_SOL_SINSIN = 1,      /* prod_d sin(2 pi k x_d) exp(-t); sol[0] = k */
    SHOCCS_SOL_GAUSS_PULSE = 2, /* exp(-|x - x0 - a t|^2 / (2 s^2)); sol = x0[3], a[3], s */
    SHOCCS_SOL_RADIAL_SIN = 3,  /* sin(2 pi (|x - c| - r - t)); sol = c[3], r */
    SHOCCS_SOL_GAUSSIAN = 4     /* the reference's "gaussian" manufactured solution
                                 * (src/mms/gauss1d.cpp, gauss2d.cpp, gauss3d.cpp):
                                 * sum_i A_i cos(f_i t) exp(-1/2 sum_{d<D} (x_d - c_id)^2 / s_id^2),
                                 * D the mesh's dimension count; terms in sol_terms.  Heat
                                 * systems only (stepped on the unfused whole-field path) */
};
enum { SHOCCS_VEL_CONSTANT = 0, SHOCCS_VEL_RADIAL = 1 };

typedef struct {
    int kind;          /* SHOCCS_SYS_* */
    int prec;          /* SHOCCS_PREC_* */
    double diffusivity;/* heat */
    int vel_kind;      /* wave: SHOCCS_VEL_* */
    double vel[3];     /* wave constant velocity a (u_t + a.grad u = 0) */
    double center[3];  /* wave radial velocity centre */
    int sol_kind;      /* SHOCCS_SOL_*: Dirichlet data, heat source and error reference */
    double sol[8];
    double max_error;  /* validity bound on the max-norm error (heat uses 1e6) */
    int sol_n_terms;   /* SHOCCS_SOL_GAUSSIAN: number of terms */
    const double* sol_terms; /* SHOCCS_SOL_GAUSSIAN: 8 doubles per term: centre[3],
                              * variance[3], amplitude, frequency (copied at create) */
} shoccs_system_desc;

shoccs_status shoccs_system_create(shoccs_problem* p, const shoccs_system_desc* desc,
                                   shoccs_system** out);
shoccs_status shoccs_system_destroy(shoccs_system* s);
/* Time stepping takes Dirichlet and Floating faces and Dirichlet objects; a heat system
 * also takes Floating objects, whose cut-point values are then state that evolves through
 * the Laplacian's R-space rows (rk4 advances the whole field {D, Rx, Ry, Rz}, as
 * src/temporal/rk4.cpp:16-47 does), and Neumann faces, whose Neumann data is the solution's
 * gradient at each right-hand side's time (heat::update_boundary,
 * src/systems/heat.cpp:324-352).  Neumann objects step like Floating ones (heat::rhs adds
 * the source at every non-Dirichlet cut point and assigns no Neumann data to objects).  A
 * wave system takes Floating objects (the gradient's R-space rows).  These systems step
 * the whole field unfused; their state is FP64 in either precision, and a SHOCCS_PREC_MIXED
 * system computes each step in FP32 (stage inputs, right-hand sides, stage accumulator;
 * the mixed operators' rows) and adds the step's increment to the FP64 state. */
/* u0 <- exact solution at time t on fluid D points, 0 on solid points, exact on R */
shoccs_status shoccs_system_initialize(shoccs_system* s, double t, void* stream);
/* copy the state in/out as FP64; where = 0 host pointers, 1 device pointers */
shoccs_status shoccs_system_set_state(shoccs_system* s, const shoccs_field* u, int where,
                                      void* stream);
shoccs_status shoccs_system_get_state(shoccs_system* s, shoccs_field* u, int where,
                                      void* stream);
/* nsteps classic RK4 steps of size dt from time t0 (fused stage kernels) */
shoccs_status shoccs_system_rk4(shoccs_system* s, double t0, double dt, int nsteps,
                                void* stream);
/* as shoccs_system_rk4, with CUDA events recorded on `stream` around the fused stage
 * kernels; kernel_ms[1..4] = total time of the main kernels of RK4 stages 0..3,
 * kernel_ms[0] = everything else (boundary-value and cut-cell row kernels),
 * kernel_ms[5] = elapsed time of the whole run */
shoccs_status shoccs_system_rk4_timed(shoccs_system* s, double t0, double dt, int nsteps,
                                      void* stream, double kernel_ms[6]);
/* one right-hand-side evaluation of the current state at time t into rhs (FP64, device) */
/* integrators::euler::operator() applied nsteps times (src/temporal/euler.cpp:11-27): the
 * state u <- u + dt * rhs(u, t), then the boundary data at t + dt.  FP64 systems. */
shoccs_status shoccs_system_euler(shoccs_system* s, double t0, double dt, int nsteps,
                                  void* stream);
shoccs_status shoccs_system_rhs(shoccs_system* s, double t, shoccs_field* rhs, void* stream);
/* out[11] = {Linf, min, max, Linf_D, argmax_D, Linf_Rx, argmax_Rx, Linf_Ry, argmax_Ry,
 *            Linf_Rz, argmax_Rz} of the current state against the exact solution at t */
shoccs_status shoccs_system_stats(shoccs_system* s, double t, double out[11], void* stream);
/* err <- |u - exact(t)| (FP64) at the fluid D points and at the non-Dirichlet cut points, 0
 * on the Dirichlet faces, the solid points and the Dirichlet cut points: the "Error" field
 * system::write hands to the field writer (write_scalar_error,
 * src/systems/detail/scalar_system_utils.hpp:224-296).  where = 0 host pointers, 1 device
 * pointers; every cut-point buffer of a nonempty R(dir) must be given. */
shoccs_status shoccs_system_error_field(shoccs_system* s, double t, shoccs_field* err, int where,
                                        void* stream);
/* Allocation-free variant of shoccs_system_stats; it has no counterpart in the reference.
 * Some callers cannot allocate device memory while they call in: an application that has
 * handed the whole device memory to its own pool allocator, or a time loop that must never
 * block in (or fail in) the CUDA allocator between steps.  This entry point allocates
 * nothing: its scratch is one fixed array inside the library's device image, sized for
 * 65536 tiles of 256 grid points (16.7 M points, 2 MB), which every GPU that loads the
 * library keeps until the process exits.  Larger grids are rejected with SHOCCS_EINVAL.
 * The first call on a device looks up the array's device address (with that device
 * current), so make that first call before any stream capture.  The address is kept per
 * device for the life of the process: it assumes the device's primary context is not reset
 * (cudaDeviceReset) in between.  Every call copies the eleven statistics to `out` and
 * synchronizes `stream` before it returns.  All calls share the array and it keeps the last
 * call's contents (each call writes every slot it reads); calls that overlap on the GPU race
 * on it.  Results equal shoccs_system_stats. */
shoccs_status shoccs_system_stats_noalloc(shoccs_system* s, double t, double out[11],
                                          void* stream);
/* dt from the CFL number: heat p*h_min^2/(4k), wave c*h_min */
shoccs_status shoccs_system_timestep(const shoccs_system* s, double cfl, double* dt);
/* Stage-kernel variant of the system's RK4 path, chosen at creation by timing the
 * candidates on the system's own grid (the SHOCCS_STAGE_KERNEL environment variable --
 * point, tma, col1, col2, col4, vec, vec3, vecx2, vecx4 -- forces one):
 * 0 per-point kernel, 1 TMA plane-marching, 2/3/4 column-blocked with 1/2/4 planes per
 * thread, 5/6 vectorised (four z points per thread; nz a multiple of 4) with 4/3 resident
 * blocks per SM, 7 unfused whole-field step (systems with non-Dirichlet objects, whose
 * cut-point values are state, Neumann faces or the Gaussian solution), 8/9 vectorised marching over 2/4 x planes per thread
 * (the x stencil's planes kept in registers).  Variants 0-6, 8 and 9 give the same bits.
 * FP64 systems and 2-D / 1-D grids otherwise use the per-point kernel. */
shoccs_status shoccs_system_path(const shoccs_system* s, int* kernel);
/* ---- batched heat solves ---------------------------------------------------------------
 * Many independent heat systems (each with the manufactured sin-sin solution, Dirichlet
 * objects, one precision for the whole batch) advance together: per RK4 stage one launch
 * evaluates the cut-cell rows of every instance and one persistent launch updates every
 * instance, and the whole nsteps-step loop is captured once as a CUDA graph and replayed.
 * Each instance gets the bits shoccs_system_rk4 would give it alone.  The reference runs
 * such solves one after another through integrators::rk4 (src/temporal/rk4.cpp:16-47);
 * the batch itself has no counterpart there. */
typedef struct shoccs_batch shoccs_batch;
/* the systems stay owned by the caller and must outlive the batch.  Mixed 2-D instances take
 * the split stage (uniform tiles and special points, two kernels per stage on parallel graph
 * branches), in groups of instances of about 48 MB of fields advanced one group after
 * another (SHOCCS_BATCH_GROUP_MB; 0: the whole batch at once), or with SHOCCS_BATCH_PERSIST=1
 * the whole solve as one persistent launch of thread-block clusters; FP64 batches take the
 * per-point stage, whose tile shape creation picks by timing the candidates on the batch
 * (SHOCCS_BATCH_KERNEL=point|flat|split overrides the choice of stage).  Every form gives each
 * instance the bits of its single-system solve. */
shoccs_status shoccs_batch_create(shoccs_system* const* systems, int n, shoccs_batch** out);
shoccs_status shoccs_batch_destroy(shoccs_batch* b);
/* nsteps RK4 steps of instance i from t0[i] with step dt[i]; afterwards each system holds
 * its state as after shoccs_system_rk4(system_i, t0[i], dt[i], nsteps) */
shoccs_status shoccs_batch_rk4(shoccs_batch* b, const double* t0, const double* dt, int nsteps,
                               void* stream);
/* info[6] = {instances, tiles (per-point, flat and uniform tiles), cut-cell rows of the row
 *            pass, tile warps (autotuned), grid (blocks of the per-point stage, or of the
 *            persistent launch), kernel nodes of the captured graph (0 before the first run)} */
shoccs_status shoccs_batch_info(const shoccs_batch* b, int64_t info[6]);

/* ---- discrete adjoint (FP64 heat systems) ------------------------------------------------
 * An autograd-shaped pair: shoccs_system_forward advances the system like shoccs_system_rk4
 * and records a tape (the step size, the step count and a copy of the state every
 * checkpoint_every steps); shoccs_system_backward maps the gradient of a loss with respect
 * to the final state to its gradient with respect to the state the forward run started from
 * (the vector-Jacobian product of the nsteps RK4 steps: the reverse stage sweep with the
 * transposed operator).  The heat right-hand side is linear in the state, so the reverse
 * sweep reads no forward state; the checkpoints make the tape self-contained (the states a
 * caller may want to inspect or restart from) and are not recomputed.  R entries of the
 * gradients are zero (cut-point values are boundary data, not state).  The reference has no
 * adjoint; its operators' transposes are what shoccs_system_rhs_transpose applies. */
typedef struct shoccs_tape shoccs_tape;
/* y = A^T x with A the linear part of system::rhs (src/systems/heat.cpp:119-162): the
 * transposed interior sweeps plus the transposed closure rows */
shoccs_status shoccs_system_rhs_transpose(shoccs_system* s, const shoccs_field* x,
                                          shoccs_field* y, void* stream);
shoccs_status shoccs_system_forward(shoccs_system* s, double t0, double dt, int nsteps,
                                    int checkpoint_every, shoccs_tape** tape, void* stream);
shoccs_status shoccs_system_backward(shoccs_system* s, const shoccs_tape* tape,
                                     const shoccs_field* grad_uT, shoccs_field* grad_u0,
                                     void* stream);
/* number of checkpoints in the tape and, with state != NULL, a copy of checkpoint i (the D
 * array, FP64, device pointer) */
shoccs_status shoccs_tape_checkpoint(const shoccs_tape* tape, int i, double* state,
                                     int* count, void* stream);
shoccs_status shoccs_tape_destroy(shoccs_tape* tape);

/* ---- captured graphs ----------------------------------------------------------------------
 * The reference's graph forms: derivative::build_graph / submit_graph / add_graph_nodes
 * (src/operators/derivative.hpp:71-151, derivative.cpp:521-596), laplacian and gradient
 * add_graph_nodes (src/operators/laplacian.hpp:35-118, gradient.hpp:31-122) and
 * system::build_rhs_graph / submit_rhs_graph (src/systems/system.cpp:57-69,
 * heat.cpp:164-294).  A graph records operator applies and system right-hand sides with
 * their buffers (pointers are baked in, as in the reference: the buffers must stay where they
 * are) and runs them in the order they were added.  On its first submit -- and, when it holds
 * a right-hand side, on a submit at another time than the last or after the system's RK4
 * steps have moved its state buffers -- the graph's kernels are captured into a CUDA graph
 * (instantiated once, later captures update the instantiated graph in place); every submit
 * replays it on `stream` and returns after the stream has finished (the reference's
 * submit_graph fences).  A right-hand side takes the system's
 * current state as its input, like shoccs_system_rhs.  Results equal the eager entry points'
 * bit for bit.  A graph is not re-entrant, and two graphs over the same problem must not run
 * at the same time (the mixed-precision operators share the problem's scratch). */
typedef struct shoccs_graph shoccs_graph;
shoccs_status shoccs_graph_create(shoccs_graph** out);
shoccs_status shoccs_graph_destroy(shoccs_graph* g);
/* derivative::add_graph_nodes(parent, u[, nu], du, eq|plus_eq) */
shoccs_status shoccs_graph_add_derivative(shoccs_graph* g, shoccs_problem* p, int dir, int prec,
                                          const shoccs_field* u, const shoccs_field* nu,
                                          shoccs_field* du, int plus_eq);
/* laplacian::add_graph_nodes(parent, u[, nu], du) */
shoccs_status shoccs_graph_add_laplacian(shoccs_graph* g, shoccs_problem* p, int prec,
                                         const shoccs_field* u, const shoccs_field* nu,
                                         shoccs_field* du);
/* gradient::add_graph_nodes(parent, u, du_x, du_y, du_z) */
shoccs_status shoccs_graph_add_gradient(shoccs_graph* g, shoccs_problem* p, int prec,
                                        const shoccs_field* u, shoccs_field* dx, shoccs_field* dy,
                                        shoccs_field* dz);
/* system::build_rhs_graph: the right-hand side of the system's state at the submit's time
 * into rhs (FP64 device field) */
shoccs_status shoccs_graph_add_rhs(shoccs_graph* g, shoccs_system* s, shoccs_field* rhs);
/* submit_graph / submit_rhs_graph(time): t is the time of the graph's right-hand sides (the
 * operators ignore it) */
shoccs_status shoccs_graph_submit(shoccs_graph* g, double t, void* stream);
/* info[3] = {recorded applies, kernel launches and memsets in the captured graph (0 before
 *            the first submit), captures so far} */
shoccs_status shoccs_graph_info(const shoccs_graph* g, int64_t info[3]);

/* kernels launched by this library since load (for launch-count accounting) */
int64_t shoccs_kernel_launches(void);

/* last error message of the calling thread */
size_t shoccs_last_error(char* buf, size_t len);

#ifdef __cplusplus
}
#endif

#endif /* SHOCCS_GPU_H */
