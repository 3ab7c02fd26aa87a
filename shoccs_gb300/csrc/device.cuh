// device.cuh -- device-side view of a compiled cut-cell operator and of the closed-form
// solutions, shared by kernels.cu and the host API (capi.cpp).
#pragma once

#include "host/gpu_layout.hpp"

#include <cstdint>
#include <cuda.h>
#include <cuda_runtime.h>

namespace sgb
{

struct DevAxis {
    int active;
    int width;   // 2p+1 interior stencil width (3, 5, 7 or 9)
    int antisym; // interior coefficients are antisymmetric with a zero centre (E4_1, E4u_1)
    int n;       // grid points along the axis
    long long stride;
    double ic[9];   // interior coefficients, 2p+1 <= 9 (E8u_1)
    float icf[9];
    WallBlock wall[2]; // rows shared by every line ending at the left / right wall
    // cut-cell closure rows, sorted by output index
    int n_rows;
    int row_base; // offset of this axis's rows in the concatenated cut-row value array
    const ClosureRow* rows;
    const long long* row_out; // output flat index of each row
    const double* coef;
    const float2* coef_ff; // the same pool as FP32 pairs (hi, lo = coef - hi)
    const int* chunk_base;
    // R-space rows (non-Dirichlet objects) per target r: CSR with source flag
    const int* rr_u[3];
    const int* rr_col[3];
    const unsigned char* rr_src[3];
    const double* rr_w[3];
    int rr_rows[3];
};

struct DevOp {
    int it0, it1, it2, nzc; // iteration space (it2 contiguous) and 32-point chunks of it2
    long long N;            // nx*ny*nz
    long long nR[3];
    int n[3];
    int phys_of_it[3];
    const uint8_t* cls;
    const double* xc[3]; // grid coordinates per physical axis
    int n_faces;         // Dirichlet-face points
    const long long* faces;
    int n_cut_rows;      // cut-cell rows of all axes
    DevAxis ax[3];
    // scratch of the vectorised FP32 operators (3-D grids, nz a multiple of 4): cut-cell row
    // values at their points (3 x N floats, axis-major) and the z-wall rows of every z line
    // (16-word records: words 0..5 the left block's rows, 8..13 the right block's);
    // allocated on the first mixed-precision apply, null before
    float* op_rowv = nullptr;
    float* op_zw = nullptr;
    int op_form = 0; // FORM_* of the interior rows; 0 before the first mixed apply, -1 when
                     // the vectorised operators do not apply to this grid
};

// closed-form exact / manufactured solution evaluated on the device
struct DevSol {
    int kind; // SHOCCS_SOL_*
    int dims;
    double p[8];
    const double* S[3];  // SINSIN: sin(2 pi k x) tables per physical axis
    const float* Sf[3];  // SINSIN: the same tables rounded to FP32 (mixed heat source)
    const double* SR[3]; // SINSIN: product of sines at the cut points of R(d)
    const double* C[3];  // SINSIN: cos(2 pi k x) tables (the gradient, Neumann data)
    double lapfac;       // SINSIN: -(dims) (2 pi k)^2
    const double* G;     // GAUSSIAN: nG terms of 8 doubles (centre[3], variance[3], A, f)
    int nG;
    int gdims;           // GAUSSIAN: the mesh's dimension count (axes with more than one point)
};

struct DevR {
    const double* pos[3];        // cut-point positions (3 per point)
    const uint8_t* dirichlet[3]; // 1 where the cut point's shape is Dirichlet
};

// a whole FP64 scalar field {D, Rx, Ry, Rz} on the device
struct FieldF64 {
    double* D;
    double* R[3];
};

// Neumann domain faces of a system: bit 2a + side per face, and the D-size array of the
// Neumann data (the gradient component of the face's axis at the face points), or none
struct NeumannFaces {
    int mask;
    double* nu;
};

// a whole scalar field of the mixed unfused step: FP32 D values, FP64 cut-point values
struct FieldMx {
    float* D;
    double* R[3];
};

// what the unfused whole-field step needs beyond the state: the Neumann face data (heat) and
// the gradient's three components over the whole field (wave).  With mixed set the step
// computes at the D points in FP32 (interior and wall rows) and at the cut points in FP64
// (cut-cell and R-space rows; stage input y_mx, right-hand side k_mx, stage accumulator
// acc_mx, gradient grad_mx) and adds the accumulated increment to the FP64 state once per
// step.
struct UnfusedAux {
    NeumannFaces nf{};
    FieldF64 grad[3]{};
    int mixed = 0;
    FieldMx y_mx{}, k_mx{}, acc_mx{}, grad_mx[3]{};
};

// launch helpers implemented in kernels.cu -----------------------------------------------
enum { PREC_FP64 = 0, PREC_MIXED = 1 };
// interior stencil shared by every active axis: 5-point antisymmetric (first derivative),
// 5-point symmetric, 3-point; FORM_ANY when the axes differ
enum { FORM_ANY = 0, FORM_ANTI5 = 1, FORM_SYM5 = 2, FORM_W3 = 3 };

cudaError_t launch_derivative(const DevOp& op, int dir, int prec, const void* uD,
                              const void* uR, const double* nuD, void* duD, void* const duR[3],
                              const void* const uRall[3], int plus_eq, cudaStream_t s);
cudaError_t launch_laplacian(const DevOp& op, int prec, const void* uD, const void* const uR[3],
                             const double* nuD, void* duD, void* const duR[3], cudaStream_t s);
cudaError_t launch_gradient(const DevOp& op, int prec, const void* uD, const void* const uR[3],
                            void* const out[3][4], cudaStream_t s);

struct SysParams {
    int kind;      // 0 heat, 1 wave
    double k;      // heat diffusivity
    float kf;
    int vel_kind;  // wave 0 constant, 1 radial
    double vel[3];
    float gf[3];   // -vel in FP32
    double center[3];
    float centerf[3];
    DevSol sol;
};

// words of a z line's record for the vectorised mixed stage (kernels.cu, k_cut_rows)
constexpr int LREC_WORDS = 20;

struct StepBuffers {
    void* u0;      // double (FP64), or the hi plane then the lo plane of FP32 pairs (MIXED)
    void* acc;     // double (FP64) or float (MIXED)
    void* sa;      // stage fields: double or float
    void* sb;
    void* cval;    // cut-cell row values of the current stage: double or float
    double* R[3];      // state R values (time t)
    double* Rhalf[3];  // Dirichlet R values at t + dt/2
    double* Rfull[3];  // Dirichlet R values at t + dt
    // TMA plane-marching path of the mixed stages (3-D grids): tensor maps of the stage
    // inputs, planes per block, and the device error flag of its bounded waits
    int tma = 0;
    // column-blocked mixed stages (3-D grids): planes per thread, 0 = per-point kernel
    int col_nx = 0;
    // vectorised mixed stages (3-D grids, nz a multiple of 4): the cut-cell row values they
    // read, at their points (3 x N floats, axis-major), and the line records (z-wall rows
    // and z-face values of every z line, 16 floats per line)
    int vec = 0;      // stencil form (FORM_*) of the vectorised kernel, 0 = not used
    // mixed path: the cut-cell rows in FP64 arithmetic (their FP32 stage inputs and FP64
    // coefficients, rounded to FP32 at the end) instead of compensated FP32; chosen at
    // creation by SHOCCS_CUT_ROWS_FP64=1
    int cut_fp64 = 0;
    int vec_minb = 4; // its resident blocks per SM (4: 64 registers, 3: 85 registers)
    int vec_px = 1;   // its x planes per thread (1, 2 or 4; 64 registers when above 1)
    float* rowv = nullptr;
    float* lrec = nullptr;
    unsigned* err = nullptr;
    // exact values on the Dirichlet domain faces (mixed path): per face (x lo, x hi, y lo,
    // y hi, z lo, z hi; null where the face is not Dirichlet) a plane of {FP32 value at
    // t+dt/2, FP32 value at t+dt, hi and lo words of the value at t+dt}, in the face's two
    // other axes (lower axis slower); filled each step together with the cut-point values
    float4* fplane[6] = {};
    // side stream of those per-step boundary evaluations and its fork / join events.  With
    // a side stream, each step also evaluates the next step's boundary values into a second
    // set (the *_next buffers, swapped in when that step starts), so the FP64-heavy boundary
    // kernel overlaps a whole step instead of delaying the first stage.
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    double* Rhalf_next[3] = {};
    double* Rfull_next[3] = {};
    float4* fplane_next[6] = {};
    cudaEvent_t join_next = nullptr;
    bool next_pending = false; // the *_next set holds the step starting at next_t, next_dt
    double next_t = 0.0, next_dt = 0.0;
    CUtensorMap tm_u0, tm_sa, tm_sb;     // stage inputs (u0: hi plane): one plane tile plus halo
    CUtensorMap tm_u0t, tm_u0l, tm_acct; // hi and lo planes of u0, accumulator: one tile, no halo
    CUtensorMap tm_cls;              // class bytes: one plane tile
};

// one RK4 step; prefetch_next: also start the next step's (t + dt, same dt) boundary values
// ---- batched heat solves ------------------------------------------------------------------
// One instance of a batch: its operator, system parameters and RK4 registers (the
// instance's own system's buffers), the RK4 weights of its time step, and where its tiles
// and cut-cell rows start in the batch's flattened lists.
struct BatchInst {
    DevOp op;
    SysParams sp;
    void* u0;
    void* acc;
    void* sa;
    void* sb;
    void* cval;
    void* rowv;              // 2-D instances: cut-cell row values at their points (3 x N), else null
    const float* s2f;        // mixed x-y instances of the split stage: the sin-sin tables'
                             // FP32 product Sf_x[i] * Sf_y[j] at every point, else null
    double* R[3];
    double cf[4], ci[4];     // dt*rkf[s], dt*rki[s+1] (ci[3] unused)
    float2 cf_ff[4], ci_ff[4];
    int row0;                // first cut-cell row of the instance in the batch's row list
};
// the three time points of one RK4 step of one instance (t, t+dt/2, t+dt) and e^-t of each,
// computed on the host exactly as the single-system path computes them
struct BatchTime {
    double t[3];
    double et[3];
};
// tile shapes of the batched stage kernel: warps per block (tile = 32 x warps points)
constexpr int BATCH_TILE_WARPS[4] = {1, 2, 4, 8};
// one RK4 step of every instance: per stage, the cut-cell rows of all instances, then the
// stage update of all instances (persistent blocks over the (instance, tile) list)
// the split 2-D stage's work lists: uniform tiles (instance, first point; BATCH_UTILE points
// each, a multiple of BATCH2D_TILE) and special points (instance, point, cut-cell row along
// it1, along it2; -1: none)
constexpr int BATCH_UTILE = 128;
struct BatchSplit {
    const int2* ut = nullptr;
    int n_ut = 0;
    const int4* sp = nullptr;
    int n_sp = 0;
    // stream and events of the special points' branch (null: both on the launch stream)
    cudaStream_t aux = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
};
// per stage: the cut-cell rows of every instance, then the per-point stage over `tiles`
// (instances that are not 2-D) and the flat 2-D stage over the warp tiles `wtiles`
// (instance, first point; BATCH2D_TILE points each), or the split 2-D stage, which needs no
// cut-cell row pass
// out[i n2 + j] = fl(sx[i] * sy[j]) over an n1 x n2 grid
cudaError_t launch_sinsin_xy(const float* sx, const float* sy, int n1, int n2, float* out,
                             cudaStream_t s);
cudaError_t launch_batch_step(const BatchInst* inst, const int* row_inst, int n_rows,
                              const int4* tiles, int n_tiles, int tile_cfg, int grid,
                              const int2* wtiles, int n_wtiles, int grid2d, const BatchSplit& sp,
                              const BatchTime* times, int prec, cudaStream_t s);
// persistent grid of the flat 2-D batched stage (128-thread blocks), and the points of one
// of its warp tiles
int batch_stage2d_grid(int prec, int n_wtiles);
// the whole solve of a batch of 2-D instances in one persistent launch of the split stage:
// clusters of BATCH_CLUSTER blocks, cluster c owning whole instances -- ctab[c] = its ranges
// of the special-point list psp and of the uniform-tile list put
constexpr int BATCH_CLUSTER = 8;
int batch_persist_clusters(int prec); // clusters resident at once (0: unavailable)
cudaError_t launch_batch_persist(const BatchInst* inst, const int4* psp, const int2* put,
                                 const int4* ctab, int n_clusters, const BatchTime* times,
                                 int n_inst, int nsteps, int prec, cudaStream_t s);
constexpr int BATCH2D_PPL = 4;                // points per lane
constexpr int BATCH2D_TILE = 32 * BATCH2D_PPL; // points per warp tile
int batch2d_tile_points();
// one stage-1 pass (timing probe of a tile shape for the autotuner)
cudaError_t launch_batch_probe(const BatchInst* inst, const int4* tiles, int n_tiles,
                               int tile_cfg, int grid, const BatchTime* times, int prec,
                               cudaStream_t s);
// persistent grid size of the batched stage kernel for a tile shape
int batch_stage_grid(int tile_cfg, int prec, int n_tiles);
// state R arrays (Dirichlet cut points) of every instance at the end of a run
cudaError_t launch_batch_finish(const BatchInst* inst, int n_inst, const BatchTime* last,
                                const int* r_inst, int n_r, cudaStream_t s);

// ---- discrete adjoint of the heat RK4 path (FP64) -----------------------------------------
// The heat right-hand side is linear in the state: rhs = A u + (boundary and source terms),
// A = k (sum over axes of the derivative rows of evolving points -- fluid points with a row
// that are not on a Dirichlet face).  A^T splits into the transposed interior sweep (a point
// gathers from the neighbours whose interior rows reference it) and the transposed closure
// rows (cut-cell and wall rows), a CSR grouped by column built once on the host.
struct AdjClosure {
    int n_tgt = 0;
    const long long* tgt = nullptr; // column points that closure rows reference
    const int* ptr = nullptr;       // entries of target t: [ptr[t], ptr[t+1])
    const long long* src = nullptr; // output point of the row
    const double* w = nullptr;      // coefficient
};
// one reverse RK4 stage S (4..1), or mode 0: out = A^T z (the transposed operator alone).
// The vectors are FP64 (PREC_FP64) or FP32 (PREC_MIXED: the reverse sweep of a mixed system)
struct AdjArgs {
    const void* z;     // stencil input: the stage adjoint z_S (lam for S = 4, scaled by zscale)
    double zscale;
    const void* lam;   // adjoint of the step's end state
    void* acc;         // sum of the stage adjoints of the step
    void* out;         // z_{S-1} (S = 4..2), the step's start adjoint (S = 1), A^T z (mode 0)
    double bl, ay;     // out = bl * lam + ay * (A^T z) for S = 4..2
    int first_step;    // S = 1 of the solve's first step: the adjoint of the caller's
                       // Dirichlet-face values (read by its first stage) is kept
    double k;          // diffusivity
};
cudaError_t launch_adjoint_stage(const DevOp& op, const AdjClosure& cl, int S, const AdjArgs& a,
                                 int prec, cudaStream_t s);
// zero lam on the Dirichlet-face points
cudaError_t launch_adjoint_mask_faces(const DevOp& op, void* lam, int prec, cudaStream_t s);
// n values between FP64 and FP32 (to_f32: double -> float, else float -> double)
cudaError_t launch_cast(long long n, int to_f32, const void* in, void* out, cudaStream_t s);

cudaError_t launch_rk4_step(const DevOp& op, const DevR& dr, const SysParams& sp, int prec,
                            StepBuffers& b, double t, double dt, cudaStream_t s,
                            cudaEvent_t* ev = nullptr, bool prefetch_next = false);
// FP64 systems whose objects are not all Dirichlet (heat: also Neumann faces and the Gaussian
// manufactured solution): rhs of the whole field, and one RK4 step of the whole field U with
// the scratch fields Y, K, ACC
cudaError_t launch_rhs_unfused(const DevOp& op, const DevR& dr, const SysParams& sp,
                               const UnfusedAux& ux, FieldF64 u, double t, FieldF64 out,
                               cudaStream_t s);
cudaError_t launch_step_unfused(const DevOp& op, const DevR& dr, const SysParams& sp,
                                const UnfusedAux& ux, FieldF64 U, FieldF64 Y, FieldF64 K,
                                FieldF64 ACC, double t, double dt, cudaStream_t s);
// statistics of the non-Dirichlet cut points: out12[4d..4d+3] = {err, index (-1: none),
// min, max} per axis
cudaError_t launch_stats_r(const DevOp& op, const DevR& dr, const DevSol& sol, double* const R[3],
                           double t, double* out12, cudaStream_t s);
// err <- |u - exact(t)| at the fluid D points and the non-Dirichlet cut points, 0 elsewhere
cudaError_t launch_error_field(const DevOp& op, const DevR& dr, const DevSol& sol, int prec,
                               const void* u0, double* const R[3], double t, FieldF64 err,
                               cudaStream_t s);
// one forward Euler step of an FP64 system (fused: U = {b.u0, b.R}; unfused: the whole
// field); K is scratch for the right-hand side
cudaError_t launch_euler_fp64(const DevOp& op, const DevR& dr, const SysParams& sp, const UnfusedAux& ux,
                              bool unfused, const StepBuffers& b, FieldF64 U, FieldF64 K, double t,
                              double dt, cudaStream_t s);
cudaError_t launch_rhs(const DevOp& op, const SysParams& sp, int prec, const StepBuffers& b,
                       double t, double* out, double* const outR[3], cudaStream_t s);
cudaError_t launch_initialize(const DevOp& op, const DevR& dr, const DevSol& sol, int prec,
                              double t, void* u0, double* const R[3], cudaStream_t s);
cudaError_t launch_state_convert(long long n, int to_mixed, const double* in_d, void* out,
                                 const void* in_m, double* out_d, cudaStream_t s);
cudaError_t launch_stats(const DevOp& op, const DevR& dr, const DevSol& sol, int prec,
                         const void* u0, double* const R[3], double t, double* dev_out,
                         cudaStream_t s);
cudaError_t launch_stats_noalloc(const DevOp& op, const DevSol& sol, int prec, const void* u0,
                                 double t, double host_out[4], cudaStream_t s);
long long stats_noalloc_max_tiles();
long long kernel_launch_count();

} // namespace sgb
