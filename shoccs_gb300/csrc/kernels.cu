// kernels.cu -- sm_103a kernels of the SHOCCS derivative-operator hot path.
//
// One thread per grid point; a warp covers 32 consecutive points of the contiguous axis,
// so the z (unit-stride) neighbours of a stencil are coalesced and the strided neighbours
// of the x / y sweeps are served by L1/L2.  Every point reads its class byte (gpu_layout.hpp):
// interior rows apply the constant 2p+1 point stencil, closure rows (walls and cut cells)
// apply their dense row in FP64, with the record found by a warp ballot over the 32-point
// chunk.  The RK4 stage kernels fuse the whole right-hand side (all three axes, closures,
// heat source or wave advection, Dirichlet rows) with the RK4 register update, so each
// stage reads the stage field, u0 and the accumulator once and writes them once.
//
// Reference operations replaced here:
//   block::matvec_functor            src/matrices/block.hpp:118-178
//   csr matvec (B, N, Bf, Br)        src/matrices/csr.cpp:37-51
//   derivative::apply_kernels        src/operators/derivative.cpp:475-519
//   laplacian / gradient             src/operators/laplacian.cpp:37-58, gradient.cpp:35-46
//   heat rhs graph                   src/systems/heat.cpp:164-288
//   scalar_wave rhs graph            src/systems/scalar_wave.cpp:241-321
//   update_boundary                  src/systems/heat.cpp:296-354, scalar_wave.cpp:329-355
//   rk4 + slot ops                   src/temporal/rk4.cpp:11-48, slot_ops.hpp:11-61
//   compute_scalar_stats             src/systems/detail/scalar_system_utils.hpp:77-181
#include "device.cuh"

#include <cooperative_groups.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <type_traits>
#include <cmath>
#include <cstdio>

namespace sgb
{
namespace cg = cooperative_groups;
namespace
{
std::atomic<long long> g_launches{0};

constexpr unsigned FULL = 0xffffffffu;
constexpr int BY = 8; // warps per block along the second iteration axis

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// ---- programmatic dependent launch -------------------------------------------------------
// Kernels of the mixed stage chain (cut-cell rows -> stage -> cut-cell rows ...) are launched
// with programmatic stream serialisation: a kernel's blocks may be scheduled while the
// previous kernel drains, and wait here until its writes are visible.  Without that launch
// attribute both instructions return at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }

// ---- loads -----------------------------------------------------------------------------
__device__ __forceinline__ double ldd(const double* p, long long i) { return __ldg(p + i); }
__device__ __forceinline__ double ldd(const float* p, long long i) { return (double)__ldg(p + i); }
__device__ __forceinline__ float ldf(const float* p, long long i) { return __ldg(p + i); }

// The solution of the mixed path is a compensated FP32 pair held as two planes: the hi
// words at [0, n) and the lo words at [n, 2n), so the hi plane doubles as the FP32 input
// field of the first RK4 stage.  As a row input it reads as hi + lo (ldd) or hi (ldf).
struct PairU {
    const float* hi;
    long long n;
};
__device__ __forceinline__ double ldd(const PairU& u, long long i)
{
    return (double)__ldg(u.hi + i) + (double)__ldg(u.hi + u.n + i);
}

// launch with programmatic stream serialisation when pdl is set (see pdl_wait)
template <class... KArgs, class... Args>
cudaError_t launch_ex(void (*kern)(KArgs...), dim3 grid, dim3 block, cudaStream_t s, bool pdl,
                      Args&&... args)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = pdl ? at : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}
__device__ __forceinline__ float ldf(const PairU& u, long long i) { return __ldg(u.hi + i); }
// Loads of values that other blocks wrote earlier in the same launch (the persistent batched
// solve, whose stages follow one another inside one kernel): from L2 (ld.global.cg), never
// through the read-only non-coherent path that __ldg takes.
struct CgF {
    const float* p;
};
struct CgD {
    const double* p;
};
struct CgPair {
    const float* hi;
    long long n;
};
__device__ __forceinline__ float ldf(const CgF& u, long long i) { return __ldcg(u.p + i); }
__device__ __forceinline__ double ldd(const CgF& u, long long i) { return (double)__ldcg(u.p + i); }
__device__ __forceinline__ double ldd(const CgD& u, long long i) { return __ldcg(u.p + i); }
__device__ __forceinline__ float ldf(const CgPair& u, long long i) { return __ldcg(u.hi + i); }
__device__ __forceinline__ double ldd(const CgPair& u, long long i)
{
    return (double)__ldcg(u.hi + i) + (double)__ldcg(u.hi + u.n + i);
}
__device__ __forceinline__ float2 ld_pair(const void* u0, long long n, long long i)
{
    const float* h = (const float*)u0;
    return make_float2(h[i], h[n + i]);
}
// The u0 words a mixed RK4 stage reads: stages 0-2 form the next FP32 stage field from the
// hi word alone (one FP32 rounding of hi + c dt rhs; the lo word is below half an ulp of hi),
// only stage 3, which adds the step's increment to the pair, reads the lo word.
template <int STAGE>
__device__ __forceinline__ float2 ld_u0(const void* u0, long long n, long long i)
{
    if constexpr (STAGE == 3)
        return ld_pair(u0, n, i);
    else
        return make_float2(((const float*)u0)[i], 0.f);
}
__device__ __forceinline__ void st_pair(void* u0, long long n, long long i, float2 v)
{
    float* h = (float*)u0;
    h[i] = v.x;
    h[n + i] = v.y;
}

// ---- point indexing ----------------------------------------------------------------------
struct Pt {
    long long p;
    long long chunk;
    int a, b, c;
    bool valid;
};

__device__ __forceinline__ Pt point_of(const DevOp& op)
{
    Pt q;
    q.c = blockIdx.x * 32 + threadIdx.x;
    q.b = blockIdx.y * blockDim.y + threadIdx.y;
    q.a = blockIdx.z;
    q.valid = (q.b < op.it1) && (q.c < op.it2);
    const long long line = (long long)q.a * op.it1 + q.b;
    q.p = line * op.it2 + q.c;
    q.chunk = line * op.nzc + blockIdx.x;
    return q;
}

__device__ __forceinline__ void phys_ijk(const DevOp& op, const Pt& q, int ijk[3])
{
    ijk[0] = ijk[1] = ijk[2] = 0;
    if (op.phys_of_it[0] >= 0) ijk[op.phys_of_it[0]] = q.a;
    if (op.phys_of_it[1] >= 0) ijk[op.phys_of_it[1]] = q.b;
    if (op.phys_of_it[2] >= 0) ijk[op.phys_of_it[2]] = q.c;
}

// record index of this lane's closure row (all 32 lanes of the warp must call it)
__device__ __forceinline__ int closure_row(const DevAxis& A, bool is_closure, long long chunk)
{
    const unsigned m = __ballot_sync(FULL, is_closure);
    int base = 0;
    if (m) {
        if (threadIdx.x == 0) base = A.chunk_base[chunk];
        base = __shfl_sync(FULL, base, 0);
    }
    return base + __popc(m & lanemask_lt());
}

// ---- interior stencils -------------------------------------------------------------------
template <class TIN>
__device__ __forceinline__ double interior64(const DevAxis& A, TIN u, long long p)
{
    const long long s = A.stride;
    if (A.width > 5) { // 7- and 9-point interiors (E6u_1, E8u_1), width 5's order
        const int hw = A.width / 2;
        double r = A.ic[0] * ldd(u, p - hw * s);
        for (int k = 1; k < A.width; k++) r = fma(A.ic[k], ldd(u, p + (k - hw) * s), r);
        return r;
    }
    if (A.width == 5) {
        if (A.antisym) {
            const double d1 = ldd(u, p + s) - ldd(u, p - s);
            const double d2 = ldd(u, p + 2 * s) - ldd(u, p - 2 * s);
            return fma(A.ic[3], d1, A.ic[4] * d2);
        }
        double r = A.ic[0] * ldd(u, p - 2 * s);
        r = fma(A.ic[1], ldd(u, p - s), r);
        r = fma(A.ic[2], ldd(u, p), r);
        r = fma(A.ic[3], ldd(u, p + s), r);
        return fma(A.ic[4], ldd(u, p + 2 * s), r);
    }
    double r = A.ic[0] * ldd(u, p - s);
    r = fma(A.ic[1], ldd(u, p), r);
    return fma(A.ic[2], ldd(u, p + s), r);
}

// ---- FP32 rows in difference form (mixed path) -------------------------------------------
// Every row of a derivative operator sums to zero (the derivative of a constant vanishes), so
// sum_j c_j x_j = sum_j c_j (x_j - x_s) + x_s sum_j c_j for any x_s.  With x_s the row's own
// point, the differences of neighbouring values are exact or nearly so in FP32 (Sterbenz),
// and the row's rounding error is relative to its result instead of to the cancelling
// products c_j x_j ~ |u| / h^2 (at h = 1/128 that is the difference between 6e-8 |Lu| and
// 1e-3 absolute); the FP32 rounding of the coefficients cancels the same way.  The
// symmetric second-derivative interiors (E2_2, E4_2: a0 = -2 (a1 + a2)) take
// a1 ((m1 - c0) + (p1 - c0)) + a2 ((m2 - c0) + (p2 - c0)); the antisymmetric first-derivative
// interiors are already differences.  Roundings are explicit, so every kernel that calls
// these helpers gets the same bits.
__device__ __forceinline__ float sym5(float a1, float a2, float m2, float m1, float c0, float p1,
                                      float p2)
{
    const float d1 = __fadd_rn(__fsub_rn(m1, c0), __fsub_rn(p1, c0));
    const float d2 = __fadd_rn(__fsub_rn(m2, c0), __fsub_rn(p2, c0));
    return fmaf(a1, d1, __fmul_rn(a2, d2));
}
__device__ __forceinline__ float sym3(float a1, float m1, float c0, float p1)
{
    return __fmul_rn(a1, __fadd_rn(__fsub_rn(m1, c0), __fsub_rn(p1, c0)));
}

template <class TIN>
__device__ __forceinline__ float interior32(const DevAxis& A, TIN u, long long p)
{
    const long long s = A.stride;
    if (A.width > 5) { // 7- and 9-point antisymmetric interiors (E6u_1, E8u_1): differences
        const int hw = A.width / 2;
        float r = A.icf[2 * hw] * (ldf(u, p + hw * s) - ldf(u, p - hw * s));
        for (int k = hw - 1; k >= 1; k--) r = fmaf(A.icf[hw + k], ldf(u, p + k * s) - ldf(u, p - k * s), r);
        return r;
    }
    if (A.width == 5) {
        if (A.antisym) {
            const float d1 = ldf(u, p + s) - ldf(u, p - s);
            const float d2 = ldf(u, p + 2 * s) - ldf(u, p - 2 * s);
            return fmaf(A.icf[3], d1, A.icf[4] * d2);
        }
        return sym5(A.icf[1], A.icf[0], ldf(u, p - 2 * s), ldf(u, p - s), ldf(u, p),
                    ldf(u, p + s), ldf(u, p + 2 * s));
    }
    if (A.antisym) return A.icf[2] * (ldf(u, p + s) - ldf(u, p - s)); // 3-point, zero centre
    return sym3(A.icf[0], ldf(u, p - s), ldf(u, p), ldf(u, p + s));
}

// ---- closure rows (always FP64) ----------------------------------------------------------
// R values of a cut-cell row's boundary term: an array, or -- for a manufactured solution
// whose value at a cut point is a fixed table entry times e^{-t} -- that product formed on
// the fly (the batched solves use it; the product is the one the array would hold).
struct RScaled {
    const double* tab;
    double et;
};
__device__ __forceinline__ double ldr(const double* R, long long i) { return __ldg(R + i); }
__device__ __forceinline__ double ldr(const float* R, long long i) { return (double)__ldg(R + i); }
__device__ __forceinline__ double ldr(const RScaled& R, long long i) { return __ldg(R.tab + i) * R.et; }
__device__ __forceinline__ double ldr(const CgD& R, long long i) { return __ldcg(R.p + i); }
// v = (first ? 0 : acc) + sum_j c_j x_j ; v += b * R[b_idx] ; v += n * nu[n_idx]
// in the order of derivative::apply_kernels (O, then B, then N).
template <class TIN, class TR>
__device__ __forceinline__ double closure64(const DevAxis& A, int row, long long p,
                                            TIN u, TR Rd, const double* nu,
                                            double acc, bool first)
{
    const ClosureRow cr = A.rows[row];
    const double* c = A.coef + cr.coef_off;
    double s = 0.0;
    long long q = p + (long long)cr.col0 * A.stride;
    for (int j = 0; j < cr.ncol; ++j) {
        s = fma(__ldg(c + j), ldd(u, q), s);
        q += A.stride;
    }
    double v = first ? s : acc + s;
    int k = cr.ncol;
    if (cr.flags & ROWF_B) {
        v = fma(__ldg(c + k), ldr(Rd, cr.b_idx), v);
        ++k;
    }
    if ((cr.flags & ROWF_N) && nu) v = fma(__ldg(c + k), __ldg(nu + cr.n_idx), v);
    return v;
}

// ---- closure rows in compensated FP32 (mixed path) --------------------------------------
// The mixed path's row inputs are FP32 (stage fields) or FP32 pairs (the solution), so a
// cut-cell row needs no FP64 arithmetic to be evaluated well: every product of an FP32-pair
// coefficient with an input is formed exactly to ~2^-48 (the leading product's rounding
// error recovered by an FMA) and accumulated as an unevaluated FP32 pair (two-sum), which
// keeps ~44 bits of the sum of terms as large as 1e7 x |u| -- far below the FP32 rounding
// of the inputs themselves, and at FP32 rather than FP64 throughput.  All roundings are
// explicit (__f*_rn), so no step is contracted into an FMA.
__device__ __forceinline__ float2 ldff(const float* u, long long i) { return make_float2(__ldg(u + i), 0.f); }
__device__ __forceinline__ float2 ldff(const CgF& u, long long i) { return make_float2(__ldcg(u.p + i), 0.f); }
__device__ __forceinline__ float2 ldff(const CgPair& u, long long i)
{
    return make_float2(__ldcg(u.hi + i), __ldcg(u.hi + u.n + i));
}
__device__ __forceinline__ float2 ldff(const PairU& u, long long i)
{
    return make_float2(__ldg(u.hi + i), __ldg(u.hi + u.n + i));
}

// (sh, sl) += (c.x + c.y) * (x.x + x.y), the term c.y * x.y (~2^-48 relative) dropped
__device__ __forceinline__ void ff_mac(float& sh, float& sl, float2 c, float2 x)
{
    const float ph = __fmul_rn(c.x, x.x);
    const float pe = fmaf(c.x, x.x, -ph); // exact rounding error of ph
    const float pl = __fadd_rn(pe, fmaf(c.x, x.y, __fmul_rn(c.y, x.x)));
    const float s = __fadd_rn(sh, ph);
    const float bb = __fsub_rn(s, sh);
    const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(ph, bb));
    const float t = __fadd_rn(__fadd_rn(e, sl), pl);
    sh = __fadd_rn(s, t);
    sl = __fsub_rn(t, __fsub_rn(sh, s));
}

// cut-cell row of the mixed path: sum_j c_j u_j + b R_d[b] (no Neumann term: systems have
// no Neumann faces or objects)
// (PF: terms whose loads are issued before the first use; the sum's order does not depend on it)
template <class TIN, class TR, int PF = 8>
__device__ __forceinline__ float closure_ff(const DevAxis& A, int row, long long p, TIN u, TR Rd)
{
    const ClosureRow cr = A.rows[row];
    const float2* c = A.coef_ff + cr.coef_off;
    const long long q0 = p + (long long)cr.col0 * A.stride;
    // issue every load of the row before the first use, so the gathers overlap; the
    // coefficients come two at a time (a block starts at an even offset of the pool, and the
    // pool has a pad after its last coefficient)
    static_assert(PF % 2 == 0, "coefficients are loaded in pairs");
    float2 cv[PF], xv[PF];
    const float4* c4 = reinterpret_cast<const float4*>(c);
#pragma unroll
    for (int m = 0; m < PF / 2; ++m)
        if (2 * m < cr.ncol) {
            const float4 v = __ldg(c4 + m);
            cv[2 * m] = make_float2(v.x, v.y);
            cv[2 * m + 1] = make_float2(v.z, v.w);
        }
#pragma unroll
    for (int j = 0; j < PF; ++j)
        if (j < cr.ncol) xv[j] = ldff(u, q0 + j * A.stride);
    double r = 0.0;
    float2 cb = make_float2(0.f, 0.f);
    if (cr.flags & ROWF_B) {
        r = ldr(Rd, cr.b_idx);
        cb = __ldg(c + cr.ncol);
    }
    float sh = 0.f, sl = 0.f;
#pragma unroll
    for (int j = 0; j < PF; ++j)
        if (j < cr.ncol) ff_mac(sh, sl, cv[j], xv[j]);
    for (int j = PF; j < cr.ncol; ++j) ff_mac(sh, sl, __ldg(c + j), ldff(u, q0 + j * A.stride));
    if (cr.flags & ROWF_B) {
        const float rh = (float)r;
        ff_mac(sh, sl, cb, make_float2(rh, (float)(r - (double)rh)));
    }
    return __fadd_rn(sh, sl);
}

// ---- domain-wall closure rows (shared per axis and side) ---------------------------------
// row r of the block at axis coordinate `coord`: sum_j c[r][j] * x[col0 + j] along the axis
__device__ __forceinline__ int wall_side(const DevAxis& A, int coord) { return coord * 2 < A.n ? 0 : 1; }

template <class TIN>
__device__ __forceinline__ double wall64(const DevAxis& A, long long p, int coord, TIN u,
                                         const double* nu, double acc, bool first)
{
    const WallBlock& W = A.wall[wall_side(A, coord)];
    const int r = coord - W.first_row;
    long long q = p + (long long)(W.col0 - coord) * A.stride;
    double s = 0.0;
    for (int j = 0; j < W.cols; ++j) {
        s = fma(W.c[r * 7 + j], ldd(u, q), s);
        q += A.stride;
    }
    double v = first ? s : acc + s;
    if (W.has_n && nu) v = fma(W.n[r], __ldg(nu + p + (long long)(W.wall - coord) * A.stride), v);
    return v;
}

// row r of a wall block over its columns x[0 .. cols-1] in difference form (see sym5):
// S_r x_s + sum_j c_j (x_j - x_s), x_s the row's own point (column first_row + r - col0),
// S_r the row sum of the FP64 coefficients rounded to FP32 (zero up to rounding)
__device__ __forceinline__ float wall_row_diff(const WallBlock& W, int r, const float (&x)[7])
{
    const int self = W.first_row + r - W.col0;
    float xs = 0.f;
#pragma unroll
    for (int j = 0; j < 7; ++j)
        if (j == self) xs = x[j];
    float s = __fmul_rn(W.sf[r], xs);
#pragma unroll
    for (int j = 0; j < 7; ++j)
        if (j < W.cols) s = fmaf(W.cf[r * 7 + j], __fsub_rn(x[j], xs), s);
    return s;
}

template <class TIN>
__device__ __forceinline__ float wall32(const DevAxis& A, long long p, int coord, TIN u)
{
    const WallBlock& W = A.wall[wall_side(A, coord)];
    const int r = coord - W.first_row;
    const long long q = p + (long long)(W.col0 - coord) * A.stride;
    float x[7]; // a wall block has at most 7 columns; all loads issued before the first use
#pragma unroll
    for (int j = 0; j < 7; ++j) x[j] = j < W.cols ? ldf(u, q + j * A.stride) : 0.f;
    return wall_row_diff(W, r, x);
}

// the Neumann term of a wall row (FP64 data, FP64 product) added to an FP32 row value
__device__ __forceinline__ float wall_neumann32(const DevAxis& A, long long p, int coord,
                                                const double* nu, float v)
{
    const WallBlock& W = A.wall[wall_side(A, coord)];
    if (!W.has_n || !nu) return v;
    const double t = fma(W.n[coord - W.first_row],
                         __ldg(nu + p + (long long)(W.wall - coord) * A.stride), (double)v);
    return (float)t;
}

// ---- closed-form solutions -------------------------------------------------------------
enum { SOL_ZERO = 0, SOL_SINSIN = 1, SOL_GAUSS_PULSE = 2, SOL_RADIAL_SIN = 3, SOL_GAUSSIAN = 4 };

// the sin-sin solution at a grid point from its per-axis table values s0, s1, s2 (physical
// axis order; s2 read only in 3-D): (s0 s1 [s2]) e^-t
__device__ __forceinline__ double sinsin_value(double s0, double s1, double s2, bool dims3, double et)
{
    double v = s0 * s1;
    if (dims3) v = v * s2;
    return v * et;
}
// the mixed heat path's manufactured source -u - k lapfac u, u = (s0 s1 [s2]) e^-t in FP32;
// s01 = fl(s0 s1)
__device__ __forceinline__ float sinsin_heat_src_p(float s01, float s2, bool dims3, float etf,
                                                   float kf, float lapff)
{
    float u = s01;
    if (dims3) u = __fmul_rn(u, s2);
    u = __fmul_rn(u, etf);
    return __fsub_rn(-u, __fmul_rn(kf, __fmul_rn(lapff, u)));
}
__device__ __forceinline__ float sinsin_heat_src_f(float s0, float s1, float s2, bool dims3,
                                                   float etf, float kf, float lapff)
{
    return sinsin_heat_src_p(__fmul_rn(s0, s1), s2, dims3, etf, kf, lapff);
}

__device__ __forceinline__ double sol_at(const DevSol& s, double t, double et, const double x[3],
                                         const int* ijk, int rdir, long long ridx)
{
    switch (s.kind) {
    case SOL_SINSIN: {
        if (ijk)
            return sinsin_value(s.S[0][ijk[0]], s.S[1][ijk[1]], s.dims == 3 ? s.S[2][ijk[2]] : 0.0,
                                s.dims == 3, et);
        return s.SR[rdir][ridx] * et;
    }
    case SOL_GAUSS_PULSE: {
        const double d0 = (x[0] - s.p[0]) - s.p[3] * t;
        const double d1 = (x[1] - s.p[1]) - s.p[4] * t;
        const double d2 = (x[2] - s.p[2]) - s.p[5] * t;
        const double r2 = d0 * d0 + d1 * d1 + d2 * d2;
        return exp(-r2 / (2 * s.p[6] * s.p[6]));
    }
    case SOL_RADIAL_SIN: {
        const double d0 = x[0] - s.p[0], d1 = x[1] - s.p[1], d2 = x[2] - s.p[2];
        const double len = sqrt(d0 * d0 + (d1 * d1 + d2 * d2));
        return sin(2 * 3.14159265358979323846 * (len - s.p[3] - t));
    }
    default: return 0.0;
    }
}

__device__ __forceinline__ double sol_at_point(const DevOp& op, const DevSol& s, double t,
                                               double et, const int ijk[3])
{
    const double x[3] = {op.xc[0][ijk[0]], op.xc[1][ijk[1]], op.xc[2][ijk[2]]};
    return sol_at(s, t, et, x, ijk, 0, 0);
}

// A sum of separable Gaussians, the reference's "gaussian" manufactured solution
// (src/mms/gauss1d.cpp, gauss2d.cpp, gauss3d.cpp): with D the mesh's dimension count and term
// i = (centre c_i, variance s_i, amplitude A_i, frequency f_i),
//   u = sum_i A_i cos(f_i t) E_i,  E_i = exp(-1/2 sum_{d<D} (x_d - c_id)^2 / s_id^2),
// so du/dt = -sum_i A_i f_i sin(f_i t) E_i, du/dx_d = -sum_i A_i cos(f_i t) E_i (x_d - c_id) / s_id^2
// and lap u = sum_i A_i cos(f_i t) E_i sum_{d<D} ((x_d - c_id)^2 / s_id^4 - 1 / s_id^2).
// Only the generic kernels (unfused heat step, initialisation, statistics, boundary data)
// evaluate it; the fused stage kernels never see this kind.
struct GaussEval {
    double u, ddt, lap, grad[3];
};
__device__ __forceinline__ GaussEval gauss_eval(const DevSol& s, double t, const double x[3])
{
    GaussEval r{0.0, 0.0, 0.0, {0.0, 0.0, 0.0}};
    for (int i = 0; i < s.nG; i++) {
        const double* g = s.G + 8 * i; // c[3], s[3], A, f
        double e = 0.0, lp = 0.0, dv[3] = {0.0, 0.0, 0.0};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            if (d < s.gdims) {
                const double dx = x[d] - g[d];
                const double is2 = 1.0 / (g[3 + d] * g[3 + d]);
                e = e - 0.5 * (dx * dx) * is2;
                dv[d] = dx * is2;
                lp = lp + (dv[d] * dv[d] - is2);
            }
        }
        const double E = exp(e);
        const double ac = g[6] * cos(g[7] * t) * E;
        r.u = r.u + ac;
        r.ddt = r.ddt - g[6] * g[7] * sin(g[7] * t) * E;
        r.lap = r.lap + ac * lp;
#pragma unroll
        for (int d = 0; d < 3; d++) r.grad[d] = r.grad[d] - ac * dv[d];
    }
    return r;
}

// sol_at / sol_at_point for the generic kernels: every solution kind, the Gaussian sum too
__device__ __forceinline__ double sol_any(const DevSol& s, double t, double et, const double x[3],
                                          const int* ijk, int rdir, long long ridx)
{
    if (s.kind == SOL_GAUSSIAN) return gauss_eval(s, t, x).u;
    return sol_at(s, t, et, x, ijk, rdir, ridx);
}
__device__ __forceinline__ double sol_point_any(const DevOp& op, const DevSol& s, double t,
                                                double et, const int ijk[3])
{
    const double x[3] = {op.xc[0][ijk[0]], op.xc[1][ijk[1]], op.xc[2][ijk[2]]};
    return sol_any(s, t, et, x, ijk, 0, 0);
}

// ---- compensated FP32 pairs ("float-float", ~2^-46 relative) ------------------------------
__device__ __forceinline__ float2 two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    const float e = (a - (s - bb)) + (b - bb);
    return make_float2(s, e);
}
__device__ __forceinline__ float2 fast_two_sum(float a, float b)
{
    const float s = a + b;
    const float e = b - (s - a);
    return make_float2(s, e);
}
__device__ __forceinline__ float2 ff_from_double(double d)
{
    const float hi = (float)d;
    return make_float2(hi, (float)(d - (double)hi));
}

inline float2 ff_host(double d)
{
    const float hi = (float)d;
    return make_float2(hi, (float)(d - (double)hi));
}

inline dim3 point_grid(const DevOp& op)
{
    return dim3(op.nzc, (op.it1 + BY - 1) / BY, op.it0);
}

// ===========================================================================================
// Standalone operators (derivative / Laplacian / gradient)
// ===========================================================================================
// value of axis d's row at point q (kind != ROW_NONE); FP64 fields compute in FP64, FP32
// fields compute interior and wall rows in FP32 and cut-cell rows in FP64
template <class T, class TR = T>
__device__ __forceinline__ T op_row(const DevAxis& A, unsigned kind, int row, long long p,
                                    int coord, const T* u, const TR* Rd, const double* nu,
                                    T acc, bool first)
{
    if constexpr (sizeof(T) == 8) {
        if (kind == ROW_INTERIOR) {
            const double v = interior64(A, (const double*)u, p);
            return first ? v : acc + v;
        }
        if (kind == ROW_WALL) return wall64(A, p, coord, (const double*)u, nu, acc, first);
        return closure64(A, row, p, (const double*)u, (const double*)Rd, nu, acc, first);
    } else {
        if (kind == ROW_INTERIOR) {
            const float v = interior32(A, (const float*)u, p);
            return first ? v : acc + v;
        }
        if (kind == ROW_WALL) {
            float v = wall32(A, p, coord, (const float*)u);
            v = wall_neumann32(A, p, coord, nu, v);
            return first ? v : acc + v;
        }
        return (float)closure64(A, row, p, (const float*)u, Rd, nu, (double)acc, first);
    }
}

template <class T, bool PLUS>
__global__ void __launch_bounds__(256) k_derivative(DevOp op, int dir, const T* __restrict__ u,
                                                    const T* __restrict__ Rd,
                                                    const double* __restrict__ nu,
                                                    T* __restrict__ du)
{
    const Pt q = point_of(op);
    const DevAxis& A = op.ax[dir];
    const unsigned kind = q.valid ? (op.cls[q.p] >> (2 * dir)) & 3u : 0u;
    const int row = closure_row(A, kind == ROW_CLOSURE, q.chunk);
    if (kind == ROW_NONE) return;
    int ijk[3];
    phys_ijk(op, q, ijk);
    const T prev = PLUS ? du[q.p] : (T)0;
    du[q.p] = op_row<T>(A, kind, row, q.p, ijk[dir], u, Rd, nu, prev, !PLUS);
}

template <class T, class TR = T> // TR: the R values' type (FP64 R with FP32 D: mixed unfused step)
__global__ void __launch_bounds__(256) k_laplacian(DevOp op, const T* __restrict__ u,
                                                   const TR* R0, const TR* R1, const TR* R2,
                                                   const double* __restrict__ nu,
                                                   T* __restrict__ du)
{
    const Pt q = point_of(op);
    const unsigned c = q.valid ? op.cls[q.p] : 0u;
    const TR* R[3] = {R0, R1, R2};
    int ijk[3];
    phys_ijk(op, q, ijk);
    T acc = 0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const DevAxis& A = op.ax[d];
        if (!A.active) continue;
        const unsigned kind = (c >> (2 * d)) & 3u;
        const int row = closure_row(A, kind == ROW_CLOSURE, q.chunk);
        if (kind != ROW_NONE) acc = op_row<T, TR>(A, kind, row, q.p, ijk[d], u, R[d], nu, acc, false);
    }
    if (q.valid) du[q.p] = acc;
}

template <class T, class TR = T>
__global__ void __launch_bounds__(256) k_gradient(DevOp op, const T* __restrict__ u,
                                                  const TR* R0, const TR* R1, const TR* R2,
                                                  T* o0, T* o1, T* o2)
{
    const Pt q = point_of(op);
    const unsigned c = q.valid ? op.cls[q.p] : 0u;
    const TR* R[3] = {R0, R1, R2};
    T* out[3] = {o0, o1, o2};
    int ijk[3];
    phys_ijk(op, q, ijk);
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const DevAxis& A = op.ax[d];
        if (!A.active) {
            if (q.valid && out[d]) out[d][q.p] = 0;
            continue;
        }
        const unsigned kind = (c >> (2 * d)) & 3u;
        const int row = closure_row(A, kind == ROW_CLOSURE, q.chunk);
        T v = 0;
        if (kind != ROW_NONE)
            v = op_row<T, TR>(A, kind, row, q.p, ijk[d], u, R[d], (const double*)nullptr, (T)0, true);
        if (q.valid) out[d][q.p] = v;
    }
}

// R-space rows (Bf then Br of each derivative) accumulated into du.R_r (always +=): one
// launch for every target r and every axis in dmask.  A thread owns one row of one target
// and adds the axes in order, rounding to T after each axis -- what one launch per (axis,
// target) in that order stores -- so the result does not depend on how the rows are grouped.
struct RspaceAll {
    const int* u[3][3]; // [axis][target]
    const int* col[3][3];
    const unsigned char* src[3][3];
    const double* w[3][3];
    int n[3]; // rows of each target (0 where no axis in the mask has rows for it)
};

template <class T, class TR = T> // TR: the R values' type, in and out
__global__ void k_rspace_all(RspaceAll ra, int dmask, const T* __restrict__ uD,
                             const TR* __restrict__ uR0, const TR* __restrict__ uR1,
                             const TR* __restrict__ uR2, TR* __restrict__ du0,
                             TR* __restrict__ du1, TR* __restrict__ du2)
{
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    int r = 0;
    while (r < 3 && row >= ra.n[r]) row -= ra.n[r++];
    if (r == 3) return;
    const TR* __restrict__ uR = r == 0 ? uR0 : (r == 1 ? uR1 : uR2);
    TR* __restrict__ duR = r == 0 ? du0 : (r == 1 ? du1 : du2);
    double t = (double)duR[row];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        if (!((dmask >> d) & 1) || !ra.u[d][r]) continue;
        const int* __restrict__ ru = ra.u[d][r];
        for (int q = ru[row]; q < ru[row + 1]; q++) {
            const double x = ra.src[d][r][q] ? (double)uR[ra.col[d][r][q]] : (double)uD[ra.col[d][r][q]];
            t = fma(ra.w[d][r][q], x, t);
        }
        t = (double)(TR)t;
    }
    duR[row] = (TR)t;
}

// the R-space rows of the axes in dmask (active axes only), one launch
template <class T, class TR = T>
cudaError_t rspace_axes(const DevOp& op, int dmask, const void* uD, const void* const uR[3],
                        void* const duR[3], cudaStream_t s)
{
    RspaceAll ra{};
    long long total = 0;
    for (int r = 0; r < 3; r++) {
        for (int d = 0; d < 3; d++) {
            const DevAxis& A = op.ax[d];
            if (!((dmask >> d) & 1) || !A.active || A.rr_rows[r] == 0 || !A.rr_u[r]) continue;
            ra.u[d][r] = A.rr_u[r];
            ra.col[d][r] = A.rr_col[r];
            ra.src[d][r] = A.rr_src[r];
            ra.w[d][r] = A.rr_w[r];
            ra.n[r] = A.rr_rows[r];
        }
        total += ra.n[r];
    }
    if (!total) return cudaSuccess;
    k_rspace_all<T, TR><<<(unsigned)((total + 127) / 128), 128, 0, s>>>(
        ra, dmask, (const T*)uD, (const TR*)uR[0], (const TR*)uR[1], (const TR*)uR[2],
        (TR*)duR[0], (TR*)duR[1], (TR*)duR[2]);
    ++g_launches;
    return cudaGetLastError();
}

template <class T, class TR = T>
cudaError_t rspace_for(const DevOp& op, int d, const void* uD, const void* const uR[3],
                       void* const duR[3], cudaStream_t s)
{
    return rspace_axes<T, TR>(op, 1 << d, uD, uR, duR, s);
}

// ===========================================================================================
// Fused RK4 stages
//
// Per stage: k_cut_rows evaluates every cut-cell closure row (FP64, one thread per row, so
// warps stay full), the main kernel applies interior and wall rows (FP32 in the mixed
// path, FP64 in the FP64 path), reads the cut-row values, forms the right-hand side and
// updates the RK4 registers, and k_faces writes the Dirichlet face values.
// ===========================================================================================
struct StageArgs {
    const void* s_in;
    void* u0;
    void* acc;
    void* s_out;
    const void* cval;
    float* rowv;            // vectorised mixed stages: cut-cell row values of the stage at
                            // their points, axis-major (3 x N), or null
    float* lrec;            // and the line records (LREC_WORDS per z line, k_cut_rows)
    const float4* fplane[6]; // Dirichlet face values of the step (mixed path), see StepBuffers
    const double* R[3];
    double cf, ci;          // dt*rkf[s], dt*rki[s+1]
    float2 cf_ff, ci_ff;    // same as compensated FP32 pairs
    double t_stage, t_next; // RHS time and Dirichlet time of the stage output
    double et_stage, et_next;
    float etf_stage;
    int cut_fp64; // mixed path: cut-cell rows in FP64 arithmetic instead of compensated FP32
};

enum { SYS_HEAT = 0, SYS_WAVE = 1 };

// cut-cell rows of all axes: value = sum_j c_j u_j + b R_d[b] (FP64 path: FP64; mixed path:
// compensated FP32, closure_ff), stored compacted in row order (cval) or -- for the
// vectorised mixed stage -- scattered to their points in rowv (3 x N, axis-major), where a
// lane finds its value with one load at its own index.
//
// With line records (lrec), the first threads of the grid each fill the record of one z line
// for the vectorised stage, in the point order of the lanes that use it: words 0..7 the
// z-wall row values at z = 0..7 (wall32's arithmetic; 0 where z holds no wall row), 8..15
// the same at z = nz-8 .. nz-1, 16..17 and 18..19 the stage output's value (hi, lo words) at
// the line's first and last point where that point is on a Dirichlet face (face_entry,
// face_pick).  The record is written as five aligned float4s; a warp holding either end of
// the line reads it with one load on each of its lanes 0..19, and a lane takes the word of
// each of its points by a shuffle from a fixed lane (its coordinate's place in the record).
// plane entry of the face point (i, j, k): the first Dirichlet face that holds it (every
// face holding it has the same values)
__device__ __forceinline__ const float4* face_entry(const StageArgs& sa, const DevOp& op, int i,
                                                    int j, int k)
{
    const int ijk[3] = {i, j, k};
#pragma unroll
    for (int f = 0; f < 6; f++) {
        const int a = f >> 1;
        if (!sa.fplane[f] || ijk[a] != ((f & 1) ? op.n[a] - 1 : 0)) continue;
        const int b = a == 0 ? 1 : 0, c = a == 2 ? 1 : 2;
        return sa.fplane[f] + (ijk[b] * op.n[c] + ijk[c]);
    }
    return nullptr;
}

// the words of a face entry that the stage output takes: the FP32 value at t+dt/2 (stages 0,
// 1), at t+dt (stage 2), the hi and lo words of the value at t+dt (stage 3, the solution)
template <int STAGE>
__device__ __forceinline__ float2 face_pick(const float4* f)
{
    if constexpr (STAGE < 2)
        return make_float2(f->x, 0.f);
    else if constexpr (STAGE == 2)
        return make_float2(f->y, 0.f);
    else
        return make_float2(f->z, f->w);
}

// the FP32 plane of a mixed-path row input: the stage field, or the hi words of the solution
__device__ __forceinline__ const float* fp32_plane(const CgF& u) { return u.p; }
__device__ __forceinline__ const float* fp32_plane(const CgPair& u) { return u.hi; }

// The row inputs of k_cut_rows were written by the kernel it follows by programmatic
// dependent launch, and the boundary values by the side stream: every load of them goes to
// L2 (TIN is CgD, CgF or CgPair; the R arrays are read through CgD), never through the
// non-coherent read-only path.

template <class TIN, class TOUT>
__global__ void k_cut_rows(DevOp op, TIN u, const double* R0,
                           const double* R1, const double* R2, TOUT* __restrict__ cval,
                           float* __restrict__ rowv, StageArgs sa, int stage)
{
    pdl_wait();
    pdl_trigger();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if constexpr (!std::is_same<TIN, CgD>::value) {
        // the line records come first in the grid, so their threads run beside the cut-cell
        // rows instead of after them
        const int nlines = sa.lrec ? op.it0 * op.it1 : 0;
        if (i < nlines) {
            const int line = i;
            const DevAxis& A = op.ax[2];
            const int nz = op.it2;
            const long long base = (long long)line * nz;
            const float* __restrict__ hi = fp32_plane(u);
            // the face values and the two line ends (the left block's columns start at the
            // wall, the right block's end there: eight values at each end, two float4s each)
            const int li = line / op.it1, lj = line - li * op.it1;
            const float4* f0 = face_entry(sa, op, li, lj, 0);
            const float4* f1 = face_entry(sa, op, li, lj, nz - 1);
            const float4 fa = f0 ? __ldcg(f0) : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 fb = f1 ? __ldcg(f1) : make_float4(0.f, 0.f, 0.f, 0.f);
            const float4 l0 = __ldcg((const float4*)(hi + base)), l1 = __ldcg((const float4*)(hi + base + 4));
            const float4 r0 = __ldcg((const float4*)(hi + base + nz - 8)),
                         r1 = __ldcg((const float4*)(hi + base + nz - 4));
            const float xl[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
            const float xr[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
            float w[LREC_WORDS];
#pragma unroll
            for (int m = 0; m < LREC_WORDS; m++) w[m] = 0.f;
            {
                const WallBlock& W = A.wall[0]; // columns 0 .. cols-1
                const float x[7] = {xl[0], xl[1], xl[2], xl[3], xl[4], xl[5], xl[6]};
#pragma unroll
                for (int z = 0; z < 8; z++) {
                    const int r = z - W.first_row;
                    if (r >= 0 && r < W.rows) w[z] = wall_row_diff(W, r, x); // wall32's arithmetic
                }
            }
            {
                const WallBlock& W = A.wall[1]; // columns nz-cols .. nz-1: xr[8-cols ..]
                const int sh = 8 - W.cols;
                float x[7];
#pragma unroll
                for (int jj = 0; jj < 7; jj++) {
                    x[jj] = 0.f;
#pragma unroll
                    for (int m = 1; m < 8; m++)
                        if (m == sh + jj) x[jj] = xr[m];
                }
#pragma unroll
                for (int m = 0; m < 8; m++) {
                    const int r = nz - 8 + m - W.first_row;
                    if (r >= 0 && r < W.rows) w[8 + m] = wall_row_diff(W, r, x);
                }
            }
            auto pick = [stage](const float4& f) {
                return stage < 2 ? make_float2(f.x, 0.f)
                                 : (stage == 2 ? make_float2(f.y, 0.f) : make_float2(f.z, f.w));
            };
            if (f0) {
                const float2 v = pick(fa);
                w[16] = v.x;
                w[17] = v.y;
            }
            if (f1) {
                const float2 v = pick(fb);
                w[18] = v.x;
                w[19] = v.y;
            }
            float4* o = (float4*)(sa.lrec + (long long)line * LREC_WORDS);
#pragma unroll
            for (int m = 0; m < LREC_WORDS / 4; m++)
                o[m] = make_float4(w[4 * m], w[4 * m + 1], w[4 * m + 2], w[4 * m + 3]);
            return;
        }
        i -= nlines;
    }
    if (i >= op.n_cut_rows) return;
    const int d = i < op.ax[1].row_base ? 0 : (i < op.ax[2].row_base ? 1 : 2);
    const CgD Rd{d == 0 ? R0 : (d == 1 ? R1 : R2)}; // a select, not an indexed local array
    const DevAxis& A = op.ax[d];
    const int row = i - A.row_base;
    const long long p = A.row_out[row];
    if constexpr (std::is_same<TOUT, double>::value) {
        cval[i] = closure64(A, row, p, u, Rd, (const double*)nullptr, 0.0, true);
    } else {
        const float v = sa.cut_fp64 ? (float)closure64(A, row, p, u, Rd, (const double*)nullptr, 0.0, true)
                                    : closure_ff(A, row, p, u, Rd);
        if (rowv)
            rowv[d * op.N + p] = v;
        else
            cval[i] = v;
    }
}


// Index arithmetic of the stage kernels runs in IDX (int when the grid has fewer than 2^31
// points, which keeps every address a single 32-bit add).
template <class IDX>
struct StagePt {
    IDX p;
    long long chunk;
    int a, b, c;
    bool valid;
};

template <class IDX>
__device__ __forceinline__ StagePt<IDX> stage_point(const DevOp& op)
{
    StagePt<IDX> q;
    q.c = blockIdx.x * 32 + threadIdx.x;
    q.b = blockIdx.y * blockDim.y + threadIdx.y;
    q.a = blockIdx.z;
    q.valid = (q.b < op.it1) && (q.c < op.it2);
    const IDX line = (IDX)q.a * op.it1 + q.b;
    q.p = line * op.it2 + q.c;
    q.chunk = (long long)line * op.nzc + blockIdx.x;
    return q;
}

template <class IDX>
__device__ __forceinline__ void stage_ijk(const DevOp& op, const StagePt<IDX>& q, int ijk[3])
{
    ijk[0] = ijk[1] = ijk[2] = 0;
    if (op.phys_of_it[0] >= 0) ijk[op.phys_of_it[0]] = q.a;
    if (op.phys_of_it[1] >= 0) ijk[op.phys_of_it[1]] = q.b;
    if (op.phys_of_it[2] >= 0) ijk[op.phys_of_it[2]] = q.c;
}

template <class T, class IDX>
__device__ __forceinline__ T ld_in(const T* u, IDX i) { return __ldg(u + i); }

// interior row with IDX addressing, FP32 (mixed) field
template <class IDX>
__device__ __forceinline__ float interior_f(const DevAxis& A, const float* u, IDX p, IDX s)
{
    auto L = [&](IDX i) -> float { return __ldg(u + i); };
    if (A.width > 5) { // 7- and 9-point antisymmetric interiors (E6u_1, E8u_1), interior32's order
        const int hw = A.width / 2;
        float r = A.icf[2 * hw] * (L(p + hw * s) - L(p - hw * s));
        for (int k = hw - 1; k >= 1; k--) r = fmaf(A.icf[hw + k], L(p + k * s) - L(p - k * s), r);
        return r;
    }
    if (A.width == 5) {
        if (A.antisym) {
            const float d1 = L(p + s) - L(p - s);
            const float d2 = L(p + 2 * s) - L(p - 2 * s);
            return fmaf(A.icf[3], d1, A.icf[4] * d2);
        }
        return sym5(A.icf[1], A.icf[0], L(p - 2 * s), L(p - s), L(p), L(p + s), L(p + 2 * s));
    }
    if (A.antisym) return A.icf[2] * (L(p + s) - L(p - s)); // 3-point, zero centre
    return sym3(A.icf[0], L(p - s), L(p), L(p + s));
}

template <class IDX>
__device__ __forceinline__ double interior_d(const DevAxis& A, const double* u, IDX p, IDX s)
{
    if (A.width > 5) { // 7- and 9-point interiors (E6u_1, E8u_1), interior64's order
        const int hw = A.width / 2;
        double r = A.ic[0] * __ldg(u + p - hw * s);
        for (int k = 1; k < A.width; k++) r = fma(A.ic[k], __ldg(u + p + (k - hw) * s), r);
        return r;
    }
    if (A.width == 5) {
        if (A.antisym) {
            const double d1 = __ldg(u + p + s) - __ldg(u + p - s);
            const double d2 = __ldg(u + p + 2 * s) - __ldg(u + p - 2 * s);
            return fma(A.ic[3], d1, A.ic[4] * d2);
        }
        double r = A.ic[0] * __ldg(u + p - 2 * s);
        r = fma(A.ic[1], __ldg(u + p - s), r);
        r = fma(A.ic[2], __ldg(u + p), r);
        r = fma(A.ic[3], __ldg(u + p + s), r);
        return fma(A.ic[4], __ldg(u + p + 2 * s), r);
    }
    double r = A.ic[0] * __ldg(u + p - s);
    r = fma(A.ic[1], __ldg(u + p), r);
    return fma(A.ic[2], __ldg(u + p + s), r);
}

__device__ __forceinline__ void radial_g64(const SysParams& sp, const DevOp& op, const int ijk[3],
                                           double g[3])
{
    const double x[3] = {op.xc[0][ijk[0]], op.xc[1][ijk[1]], op.xc[2][ijk[2]]};
    const double r[3] = {x[0] - sp.center[0], x[1] - sp.center[1], x[2] - sp.center[2]};
    const double len = sqrt(r[0] * r[0] + (r[1] * r[1] + r[2] * r[2]));
    g[0] = -r[0] / len;
    g[1] = -r[1] / len;
    g[2] = -r[2] / len;
}

// FP64 stage: interior and wall rows in FP64, cut-cell rows from k_cut_rows.  The source
// term is written with explicit rounding so that every kernel that inlines this body (the
// single-system and the batched stages) rounds it the same way.
template <int STAGE, int SYS, class IDX>
__device__ __forceinline__ void stage64_at(const DevOp& op, const SysParams& sp,
                                           const StageArgs& sa, const StagePt<IDX>& q)
{
    const unsigned c = q.valid ? op.cls[q.p] : 0u;
    const double* __restrict__ in =
        STAGE == 0 ? (const double*)sa.u0 : (const double*)sa.s_in;
    const double* __restrict__ cval = (const double*)sa.cval;
    double lap = 0.0;
    double dd[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const DevAxis& A = op.ax[d];
        if (!A.active) continue;
        const unsigned kind = (c >> (2 * d)) & 3u;
        const IDX s = (IDX)A.stride;
        double v;
        if (__all_sync(FULL, kind == ROW_INTERIOR)) {
            v = interior_d<IDX>(A, in, q.p, s);
        } else {
            const int row = closure_row(A, kind == ROW_CLOSURE, q.chunk);
            v = 0.0;
            if (kind == ROW_INTERIOR) {
                v = interior_d<IDX>(A, in, q.p, s);
            } else if (kind == ROW_WALL) {
                int ijk[3];
                stage_ijk(op, q, ijk);
                v = wall64(A, (long long)q.p, ijk[d], in, (const double*)nullptr, 0.0, true);
            } else if (kind == ROW_CLOSURE) {
                v = __ldcg(cval + A.row_base + row); // k_cut_rows, the dependent-launch predecessor
            }
        }
        if (SYS == SYS_HEAT)
            lap = lap + v;
        else
            dd[d] = v;
    }
    if (!q.valid) return;
    double rhs = 0.0;
    if (c & 0x3Fu) {
        if (SYS == SYS_HEAT) {
            double src = 0.0;
            if (sp.sol.kind == SOL_SINSIN) {
                int ijk[3];
                stage_ijk(op, q, ijk);
                const double u = sol_at_point(op, sp.sol, sa.t_stage, sa.et_stage, ijk);
                src = __dsub_rn(-u, __dmul_rn(sp.k, __dmul_rn(sp.sol.lapfac, u)));
            }
            rhs = fma(lap, sp.k, src);
        } else {
            double g[3] = {-sp.vel[0], -sp.vel[1], -sp.vel[2]};
            if (sp.vel_kind != 0) {
                int ijk[3];
                stage_ijk(op, q, ijk);
                radial_g64(sp, op, ijk, g);
            }
            rhs = fma(g[2], dd[2], fma(g[1], dd[1], g[0] * dd[0]));
        }
    }
    double* __restrict__ u0 = (double*)sa.u0;
    double* __restrict__ acc = (double*)sa.acc;
    if (STAGE < 3) {
        if (STAGE == 0)
            acc[q.p] = sa.cf * rhs;
        else
            acc[q.p] = fma(sa.cf, rhs, acc[q.p]);
        ((double*)sa.s_out)[q.p] = fma(sa.ci, rhs, u0[q.p]);
    } else {
        u0[q.p] = u0[q.p] + fma(sa.cf, rhs, acc[q.p]);
    }
}

template <int STAGE, int SYS, class IDX>
__global__ void __launch_bounds__(256) k_stage64(DevOp op, SysParams sp, StageArgs sa)
{
    pdl_wait();
    pdl_trigger();
    stage64_at<STAGE, SYS, IDX>(op, sp, sa, stage_point<IDX>(op));
}

// Right-hand side of one point of the mixed path from its axis values (heat: lap, the sum
// of the second-derivative rows; wave: d0..d2, the first-derivative rows).  Products are
// written with explicit rounding (__fmul_rn never fuses into an FMA), so every stage-kernel
// variant yields the same bits from the same inputs.
template <int SYS, int VK = -1> // VK: velocity field of the wave, -1 from sp, 0 constant, 1 radial
__device__ __forceinline__ float rhs_mixed(const DevOp& op, const SysParams& sp, float etf, int i,
                                           int j, int k, float lap, float d0, float d1, float d2)
{
    if constexpr (SYS == SYS_HEAT) {
        float src = 0.f;
        if (sp.sol.kind == SOL_SINSIN) {
            const bool d3 = sp.sol.dims == 3;
            src = sinsin_heat_src_f(sp.sol.Sf[0][i], sp.sol.Sf[1][j], d3 ? sp.sol.Sf[2][k] : 0.f, d3,
                                    etf, sp.kf, (float)sp.sol.lapfac);
        }
        return fmaf(lap, sp.kf, src);
    } else {
        float g0 = sp.gf[0], g1 = sp.gf[1], g2 = sp.gf[2];
        if (VK == 1 || (VK < 0 && sp.vel_kind != 0)) {
            const float r0 = __fsub_rn((float)op.xc[0][i], sp.centerf[0]);
            const float r1 = __fsub_rn((float)op.xc[1][j], sp.centerf[1]);
            const float r2 = __fsub_rn((float)op.xc[2][k], sp.centerf[2]);
            const float il = rsqrtf(fmaf(r2, r2, fmaf(r1, r1, __fmul_rn(r0, r0))));
            g0 = __fmul_rn(-r0, il);
            g1 = __fmul_rn(-r1, il);
            g2 = __fmul_rn(-r2, il);
        }
        return fmaf(g2, d2, fmaf(g1, d1, __fmul_rn(g0, d0)));
    }
}

// RK4 register update of one point of the mixed path: the increment dt*b_s*rhs with the
// weight held as an FP32 pair; stages 0-2 write the accumulator and the next stage field
// fl(hi + c dt rhs) (one rounding; u.y is not read), stage 3 adds the accumulated increment
// to the (hi, lo) solution by an error-free two-sum.
template <int STAGE>
__device__ __forceinline__ void rk_mixed(const StageArgs& sa, float rhs, float2 u, float accv,
                                         float& acc_out, float& s_out, float2& u_out)
{
    const float inc = fmaf(sa.cf_ff.x, rhs, __fmul_rn(sa.cf_ff.y, rhs));
    if constexpr (STAGE < 3) {
        acc_out = STAGE == 0 ? inc : __fadd_rn(accv, inc);
        s_out = fmaf(sa.ci_ff.x, rhs, u.x);
    } else {
        const float a = __fadd_rn(accv, inc);
        const float2 t = two_sum(u.x, a);
        u_out = fast_two_sum(t.x, __fadd_rn(t.y, u.y));
    }
}

// Mixed stage: FP32 stage field, interior and wall rows, FP32 stage accumulator; FP64
// cut-cell rows (k_cut_rows); the solution u0 is a compensated FP32 pair (hi, lo) and
// receives the step's accumulated increment through an error-free two-sum.  Stage 0 reads
// u0 (hi word) as its input field.  The 32 lanes of a warp hold 32 consecutive points of
// one 32-point chunk (q.chunk), which the cut-cell row lookup relies on.
template <int STAGE, int SYS, class IDX>
__device__ __forceinline__ void stage_mixed_at(const DevOp& op, const SysParams& sp,
                                               const StageArgs& sa, const StagePt<IDX>& q)
{
    const unsigned c = q.valid ? op.cls[q.p] : 0u;
    const float* __restrict__ cval = (const float*)sa.cval;
    const float* __restrict__ in = STAGE == 0 ? (const float*)sa.u0 : (const float*)sa.s_in;
    float lap = 0.f;
    float dd[3] = {0.f, 0.f, 0.f};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const DevAxis& A = op.ax[d];
        if (!A.active) continue;
        const unsigned kind = (c >> (2 * d)) & 3u;
        const IDX s = (IDX)A.stride;
        float v;
        if (__all_sync(FULL, kind == ROW_INTERIOR)) {
            v = interior_f<IDX>(A, in, q.p, s);
        } else {
            const int row = closure_row(A, kind == ROW_CLOSURE, q.chunk);
            v = 0.f;
            if (kind == ROW_INTERIOR) {
                v = interior_f<IDX>(A, in, q.p, s);
            } else if (kind == ROW_WALL) {
                int ijk[3];
                stage_ijk(op, q, ijk);
                v = wall32(A, (long long)q.p, ijk[d], in);
            } else if (kind == ROW_CLOSURE) {
                v = cval[A.row_base + row];
            }
        }
        if (SYS == SYS_HEAT)
            lap = __fadd_rn(lap, v);
        else
            dd[d] = v;
    }
    if (!q.valid) return;
    float rhs = 0.f;
    if (c & 0x3Fu) {
        int ijk[3];
        stage_ijk(op, q, ijk);
        rhs = rhs_mixed<SYS>(op, sp, sa.etf_stage, ijk[0], ijk[1], ijk[2], lap, dd[0], dd[1],
                             dd[2]);
    }
    float* __restrict__ acc = (float*)sa.acc;
    float a_out = 0.f, s_out = 0.f;
    float2 u_out;
    rk_mixed<STAGE>(sa, rhs, ld_u0<STAGE>(sa.u0, op.N, q.p), STAGE == 0 ? 0.f : acc[q.p], a_out,
                    s_out, u_out);
    if constexpr (STAGE < 3) {
        acc[q.p] = a_out;
        ((float*)sa.s_out)[q.p] = s_out;
    } else {
        st_pair(sa.u0, op.N, q.p, u_out);
    }
}

template <int STAGE, int SYS, class IDX>
__global__ void __launch_bounds__(256) k_stage_mixed(DevOp op, SysParams sp, StageArgs sa)
{
    stage_mixed_at<STAGE, SYS, IDX>(op, sp, sa, stage_point<IDX>(op));
}

// interior row from five register values (m2 .. p2 along the axis); the operation order is
// interior_f's.  AX: DevAxis, or a register copy of its interior fields (IRow)
template <class AX>
__device__ __forceinline__ float interior_row(const AX& A, float m2, float m1, float c0,
                                              float p1, float p2)
{
    if (A.width == 5) {
        if (A.antisym) return fmaf(A.icf[3], p1 - m1, A.icf[4] * (p2 - m2));
        return sym5(A.icf[1], A.icf[0], m2, m1, c0, p1, p2);
    }
    if (A.antisym) return A.icf[2] * (p1 - m1); // 3-point, zero centre
    return sym3(A.icf[0], m1, c0, p1);
}

// ---- column-blocked mixed stage (3-D grids) ------------------------------------------------
// Each thread owns NX consecutive x-planes of one (y, z) column.  The x-stencil values of
// the column come from a register window of NX + 4 loads; the y / z stencil values, the
// class bytes, u0 and the accumulator of all NX points are issued together, before any
// class byte is decoded, with neighbour coordinates clamped into the grid so every
// speculative load stays in bounds (values of rows that turn out not to be interior are
// simply not used).  Per axis every lane evaluates the interior row from these registers
// and keeps it where its row is interior (points without a row contribute 0); only warps
// that hold a cut-cell or wall row along that axis branch to read the cut-row values and
// evaluate the wall rows.
template <int STAGE, int SYS, int NX>
__global__ void __launch_bounds__(256) k_stage_mixed_col(DevOp op, SysParams sp, StageArgs sa)
{
    const float* __restrict__ in = STAGE == 0 ? (const float*)sa.u0 : (const float*)sa.s_in;
    auto L = [&](int idx) -> float { return __ldg(in + idx); };
    const int nx = op.it0, ny = op.it1, nz = op.it2;
    const int k = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * BY + threadIdx.y;
    const int i0 = blockIdx.z * NX;
    const bool col_valid = (j < ny) && (k < nz);
    const int plane = ny * nz;
    const int jc = min(j, ny - 1), kc = min(k, nz - 1);
    const int col = jc * nz + kc;
    // clamped neighbour offsets within a plane
    const int ym2 = (max(jc - 2, 0) - jc) * nz, ym1 = (max(jc - 1, 0) - jc) * nz;
    const int yp1 = (min(jc + 1, ny - 1) - jc) * nz, yp2 = (min(jc + 2, ny - 1) - jc) * nz;
    const int zm2 = max(kc - 2, 0) - kc, zm1 = max(kc - 1, 0) - kc;
    const int zp1 = min(kc + 1, nz - 1) - kc, zp2 = min(kc + 2, nz - 1) - kc;

    float w[NX + 4]; // x window: planes i0-2 .. i0+NX+1 of this column
#pragma unroll
    for (int m = 0; m < NX + 4; m++) w[m] = L(min(max(i0 - 2 + m, 0), nx - 1) * plane + col);
    unsigned c[NX];
    float yv[NX][4], zv[NX][4];
    float2 uu[NX];
    float av[NX];
#pragma unroll
    for (int t = 0; t < NX; t++) {
        const int ic = min(i0 + t, nx - 1);
        const int p = ic * plane + col;
        const bool valid = col_valid && (i0 + t < nx);
        c[t] = valid ? (unsigned)op.cls[p] : 0u;
        yv[t][0] = L(p + ym2); yv[t][1] = L(p + ym1); yv[t][2] = L(p + yp1); yv[t][3] = L(p + yp2);
        zv[t][0] = L(p + zm2); zv[t][1] = L(p + zm1); zv[t][2] = L(p + zp1); zv[t][3] = L(p + zp2);
        if constexpr (STAGE > 0) {
            uu[t] = ld_u0<STAGE>(sa.u0, op.N, p);
            av[t] = ((const float*)sa.acc)[p];
        }
    }
    const float* __restrict__ cval = (const float*)sa.cval;
#pragma unroll
    for (int t = 0; t < NX; t++) {
        const int i = i0 + t;
        const int p = min(i, nx - 1) * plane + col;
        float lap = 0.f;
        float dd[3] = {0.f, 0.f, 0.f};
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const DevAxis& A = op.ax[d];
            const unsigned kind = (c[t] >> (2 * d)) & 3u;
            // the interior row from the registers, kept where the point has one (the
            // speculative loads are exact for such points); no-row points contribute 0
            float xm2, xm1, x0v, xp1, xp2;
            if (d == 0) {
                xm2 = w[t]; xm1 = w[t + 1]; x0v = w[t + 2]; xp1 = w[t + 3]; xp2 = w[t + 4];
            } else if (d == 1) {
                xm2 = yv[t][0]; xm1 = yv[t][1]; x0v = w[t + 2]; xp1 = yv[t][2]; xp2 = yv[t][3];
            } else {
                xm2 = zv[t][0]; xm1 = zv[t][1]; x0v = w[t + 2]; xp1 = zv[t][2]; xp2 = zv[t][3];
            }
            const float s_int = interior_row(A, xm2, xm1, x0v, xp1, xp2);
            float v = kind == ROW_INTERIOR ? s_int : 0.f;
            // cut-cell and wall rows: only warps that hold one take this branch
            if (__any_sync(FULL, kind >= ROW_CLOSURE)) {
                const long long chunk = ((long long)min(i, nx - 1) * ny + j) * op.nzc + blockIdx.x;
                const int row = closure_row(A, kind == ROW_CLOSURE, chunk);
                if (kind == ROW_WALL) {
                    const int coord = d == 0 ? i : (d == 1 ? j : k);
                    v = wall32(A, (long long)p, coord, in);
                } else if (kind == ROW_CLOSURE) {
                    v = cval[A.row_base + row];
                }
            }
            if (SYS == SYS_HEAT)
                lap = __fadd_rn(lap, v);
            else
                dd[d] = v;
        }
        if (!(col_valid && i < nx)) continue;
        const float rhs = (c[t] & 0x3Fu) ? rhs_mixed<SYS>(op, sp, sa.etf_stage, i, j, k, lap,
                                                          dd[0], dd[1], dd[2])
                                         : 0.f;
        float a_out = 0.f, s_out = 0.f;
        float2 u_out;
        if constexpr (STAGE == 0)
            rk_mixed<STAGE>(sa, rhs, ld_u0<STAGE>(sa.u0, op.N, p), 0.f, a_out, s_out, u_out);
        else
            rk_mixed<STAGE>(sa, rhs, uu[t], av[t], a_out, s_out, u_out);
        if constexpr (STAGE < 3) {
            ((float*)sa.acc)[p] = a_out;
            ((float*)sa.s_out)[p] = s_out;
        } else {
            st_pair(sa.u0, op.N, p, u_out);
        }
    }
}

// ---- Dirichlet face values of the mixed path ------------------------------------------------
// The exact solution on the Dirichlet domain faces depends only on the time, so each RK4
// step evaluates it once, for every face point, into per-face planes (StepBuffers::fplane):
// the FP32 stage fields take the value computed in FP32 arithmetic at t+dt/2 (stages 0, 1)
// and t+dt (stage 2), the solution takes the compensated pair of the FP64 value at t+dt.
inline int face_plane_size_host(const DevOp& op, int f)
{
    const int a = f >> 1;
    return a == 0 ? op.n[1] * op.n[2] : (a == 1 ? op.n[0] * op.n[2] : op.n[0] * op.n[1]);
}

// the exact value in FP32 arithmetic (the stage fields' precision)
__device__ float face_f32(const DevOp& op, const DevSol& sol, double t, double et,
                          const int ijk[3])
{
    if (sol.kind == SOL_GAUSS_PULSE || sol.kind == SOL_RADIAL_SIN) {
        const float x0 = (float)op.xc[0][ijk[0]], x1 = (float)op.xc[1][ijk[1]],
                    x2 = (float)op.xc[2][ijk[2]];
        const float tf = (float)t;
        if (sol.kind == SOL_GAUSS_PULSE) {
            const float d0 = (x0 - (float)sol.p[0]) - (float)sol.p[3] * tf;
            const float d1 = (x1 - (float)sol.p[1]) - (float)sol.p[4] * tf;
            const float d2 = (x2 - (float)sol.p[2]) - (float)sol.p[5] * tf;
            const float sg = (float)sol.p[6];
            return expf(-(d0 * d0 + d1 * d1 + d2 * d2) / (2.f * sg * sg));
        }
        const float d0 = x0 - (float)sol.p[0], d1 = x1 - (float)sol.p[1],
                    d2 = x2 - (float)sol.p[2];
        return sinf(6.283185307179586f * (sqrtf(d0 * d0 + d1 * d1 + d2 * d2) -
                                          (float)sol.p[3] - tf));
    }
    return (float)sol_at_point(op, sol, t, et, ijk);
}

// face values of the stage output from the planes, for the stage kernels without the
// face write fused in
template <int STAGE>
__global__ void k_faces_mixed(DevOp op, StageArgs sa)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= op.n_faces) return;
    const long long p = op.faces[e];
    const long long nyz = (long long)op.n[1] * op.n[2];
    const int i = (int)(p / nyz), j = (int)((p / op.n[2]) % op.n[1]), k = (int)(p % op.n[2]);
    const float4* f = face_entry(sa, op, i, j, k);
    if (!f) return;
    const float4 v = *f;
    if constexpr (STAGE < 2)
        ((float*)sa.s_out)[p] = v.x;
    else if constexpr (STAGE == 2)
        ((float*)sa.s_out)[p] = v.y;
    else
        st_pair(sa.u0, op.N, p, make_float2(v.z, v.w));
}

// ---- vectorised mixed stage (3-D grids, nz a multiple of 4) --------------------------------
// A thread owns four consecutive z points of one x plane, so a warp covers 128 points of one
// z line and every field moves as float4 (stage input, class bytes as one 32-bit word, the
// hi plane of u0 and, in stage 3, its lo plane, accumulator).  The z neighbours come from
// the float4s on either side, the y neighbours from the float4s of rows j-2..j+2, the x
// neighbours from those of planes i-2..i+2; all loads are issued before any class byte is
// decoded, with coordinates clamped into the grid so they stay in bounds.  Per axis every
// point evaluates the interior row from these registers, and the points whose row is a
// closure or wall row replace it.  A point without a row along some axis is a solid point
// (right-hand side 0) or a Dirichlet face point (value replaced by the face's): the host
// offers this kernel only when no other point lacks a row, so stages 0-2 test no row kind on
// the common path (stage 3 keeps a select per row kind: without it its registers spill).
// The rows that are not interior cost each warp at most one extra round trip to memory,
// overlapped with the stencil loads where the position alone says what is needed:
//  * cut-cell rows: one load at the point's own index of the dense per-axis value array that
//    k_cut_rows fills, issued as soon as the class word arrives;
//  * x- and y-wall rows (whole planes / rows, uniform across a warp): the wall block's
//    columns of the four points as float4s, all in one round trip;
//  * z-wall rows and Dirichlet z-face points (the lanes at either end of every line): from
//    the line record, one word per lane loaded at entry and moved by shuffles; x- and y-face
//    planes (uniform across a warp) after the update.
// FORM fixes the interior stencil (5-point antisymmetric, 5-point symmetric, 3-point) and VK
// the velocity field of the wave system (constant or radial), so the per-point code has no
// run-time branch on either.  The arithmetic of each point is the per-point kernel's,
// operation for operation.
template <int FORM>
__device__ __forceinline__ float interior_row_t(const DevAxis& A, float m2, float m1, float c0,
                                                float p1, float p2)
{
    if constexpr (FORM == FORM_ANTI5) {
        return fmaf(A.icf[3], p1 - m1, A.icf[4] * (p2 - m2));
    } else if constexpr (FORM == FORM_SYM5) {
        return sym5(A.icf[1], A.icf[0], m2, m1, c0, p1, p2);
    } else if constexpr (FORM == FORM_W3) {
        return sym3(A.icf[0], m1, c0, p1);
    } else {
        return interior_row(A, m2, m1, c0, p1, p2);
    }
}

__device__ __forceinline__ float4 ld4(const float* base, int idx)
{
    return __ldg((const float4*)(base + idx));
}
// the same from L2, for data the dependent-launch predecessor wrote
__device__ __forceinline__ float4 ld4cg(const float* base, int idx)
{
    return __ldcg((const float4*)(base + idx));
}

__device__ __forceinline__ float f4(const float4& v, int q)
{
    return q == 0 ? v.x : (q == 1 ? v.y : (q == 2 ? v.z : v.w));
}

// the loads of one thread's four points of plane i (stage input at the point and its y / z
// neighbours, class bytes, u0 hi word and accumulator); the x neighbours are the caller's
struct VecLoads {
    float4 C, ya, yb, yc, yd, zL, zR, uh, av;
    unsigned c4;
};

// C: the stage input at the four points (loaded by the caller)
template <int STAGE>
__device__ __forceinline__ VecLoads vec_loads(const DevOp& op, const StageArgs& sa, const float* in,
                                              int i, int j, int k, float4 C)
{
    const int ny = op.it1, nz = op.it2;
    const int plane = ny * nz;
    const int kc = min(k, nz - 4);
    const int p = i * plane + j * nz + kc;
    const int ym2 = (max(j - 2, 0) - j) * nz, ym1 = (max(j - 1, 0) - j) * nz;
    const int yp1 = (min(j + 1, ny - 1) - j) * nz, yp2 = (min(j + 2, ny - 1) - j) * nz;
    const int zl = kc >= 4 ? -4 : 0, zr = kc + 8 <= nz ? 4 : 0;
    VecLoads L;
    L.c4 = k < nz ? __ldg((const unsigned*)(op.cls + p)) : 0u;
    L.C = C;
    L.ya = ld4(in, p + ym2);
    L.yb = ld4(in, p + ym1);
    L.yc = ld4(in, p + yp1);
    L.yd = ld4(in, p + yp2);
    L.zL = ld4(in, p + zl);
    L.zR = ld4(in, p + zr);
    const float* __restrict__ u0 = (const float*)sa.u0;
    L.uh = STAGE == 0 ? L.C : *(const float4*)(u0 + p);
    L.av = make_float4(0.f, 0.f, 0.f, 0.f);
    if constexpr (STAGE > 0) L.av = *((const float4*)((const float*)sa.acc + p));
    return L;
}

// Everything of one thread's four points of plane i after the loads: interior rows from the
// registers, cut-cell rows (rowv), z-wall rows and z-face values (the line record, word
// `lane` of it in rec), x / y wall rows, the right-hand side, the RK4 registers, Dirichlet
// faces, the stores.
template <int STAGE, int SYS, int FORM, int VK>
__device__ __forceinline__ void vec_stage_points(const DevOp& op, const SysParams& sp,
                                                 const StageArgs& sa, const float* in, int i,
                                                 int j, int k, int lane, const VecLoads& L,
                                                 const float4 xa, const float4 xb,
                                                 const float4 xc, const float4 xd, float rec)
{
    const int nz = op.it2;
    const int plane = op.it1 * nz;
    const bool kvalid = k < nz;
    const int p = i * plane + j * nz + min(k, nz - 4);
    const float4 C = L.C, ya = L.ya, yb = L.yb, yc = L.yc, yd = L.yd, uh = L.uh, av = L.av;
    const unsigned c4 = L.c4;
    const float zz[8] = {L.zL.z, L.zL.w, C.x, C.y, C.z, C.w, L.zR.x, L.zR.y};
    const float* __restrict__ u0 = (const float*)sa.u0;
    float v[3][4];
    // the kind of row d of point q (2-bit fields, bits 0-5 of each class byte): decoded where
    // it is used in stages 0-2, held in registers in stage 3 (each the faster form measured)
    unsigned kqa[3][4];
    auto kq = [&kqa, c4](int d, int q) -> unsigned {
        if constexpr (STAGE == 3)
            return kqa[d][q];
        else
            return (c4 >> (8 * q + 2 * d)) & 3u;
    };
    // the twelve row kinds tested at once: hb holds each field's high bit, lb its low bit
    // moved to the high bit's position
    const unsigned hb = c4 & 0x2A2A2A2Au, lb = (c4 << 1) & 0x2A2A2A2Au;
    const bool cut = (hb & ~lb) != 0u;                      // cut-cell rows (kind 2)
    const bool zwall = (hb & lb & 0x20202020u) != 0u;       // z-wall rows (kind 3)
    const bool xywall = (hb & lb & 0x0A0A0A0Au) != 0u;      // x / y wall rows
#pragma unroll
    for (int q = 0; q < 4; q++) {
        if constexpr (STAGE == 3) {
#pragma unroll
            for (int d = 0; d < 3; d++) kqa[d][q] = (c4 >> (8 * q + 2 * d)) & 3u;
        }
        const float sx = interior_row_t<FORM>(op.ax[0], f4(xa, q), f4(xb, q), f4(C, q), f4(xc, q), f4(xd, q));
        const float sy = interior_row_t<FORM>(op.ax[1], f4(ya, q), f4(yb, q), f4(C, q), f4(yc, q), f4(yd, q));
        const float sz = interior_row_t<FORM>(op.ax[2], zz[q], zz[q + 1], zz[q + 2], zz[q + 3], zz[q + 4]);
        if constexpr (STAGE < 3) {
            v[0][q] = sx;
            v[1][q] = sy;
            v[2][q] = sz;
        } else {
            // stage 3 keeps only the interior rows here: without these selects the
            // compiler's schedule of its u0 and accumulator registers spills (measured slower)
            v[0][q] = kqa[0][q] == ROW_INTERIOR ? sx : 0.f;
            v[1][q] = kqa[1][q] == ROW_INTERIOR ? sy : 0.f;
            v[2][q] = kqa[2][q] == ROW_INTERIOR ? sz : 0.f;
        }
    }
    // the lo plane of u0 (stage 3 only) is loaded here, after the stencil registers are
    // free: issued before it, it pushed stage 3 past the 64-register budget
    const float4 ul = STAGE == 3 ? *(const float4*)(u0 + op.N + p) : make_float4(0.f, 0.f, 0.f, 0.f);
    if (cut) { // cut-cell rows: one load each, at the point's own index
        const float* rv = sa.rowv + p; // written by k_cut_rows, the dependent-launch predecessor
#pragma unroll
        for (int d = 0; d < 3; d++)
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (kq(d, q) == ROW_CLOSURE) v[d][q] = __ldcg(rv + d * op.N + q);
    }
    if (__any_sync(FULL, zwall)) { // z-wall rows: the record words of the four points
        const int w0 = k < 8 ? k : 8 + k - (nz - 8);
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const float val = __shfl_sync(FULL, rec, (w0 + q) & 31);
            if (kq(2, q) == ROW_WALL) v[2][q] = val;
        }
    }
    if (__any_sync(FULL, xywall)) { // whole x / y wall planes: uniform across the warp
#pragma unroll
        for (int d = 0; d < 2; d++) {
            const bool wd = kq(d, 0) == ROW_WALL || kq(d, 1) == ROW_WALL ||
                            kq(d, 2) == ROW_WALL || kq(d, 3) == ROW_WALL;
            if (!__any_sync(FULL, wd)) continue;
            // the block's columns for the four points as float4s, in two groups of at most
            // four (two round trips, at most 16 registers of loads in flight); wall32's order
            const DevAxis& A = op.ax[d];
            const int coord = d == 0 ? i : j;
            const WallBlock& W = A.wall[wall_side(A, coord)];
            const int r = coord - W.first_row;
            const int stride = d == 0 ? plane : nz;
            const int q0 = p + (W.col0 - coord) * stride;
            // wall_row_diff's arithmetic: the points' own values (the row's column
            // first_row + r - col0) are the differences' reference
            const float4 xs = ld4(in, p);
            float sw[4];
#pragma unroll
            for (int q = 0; q < 4; q++) sw[q] = __fmul_rn(W.sf[r], f4(xs, q));
#pragma unroll
            for (int g = 0; g < 2; g++) {
                float4 xw[4];
#pragma unroll
                for (int jj = 0; jj < 4; jj++) {
                    const int col = 4 * g + jj;
                    xw[jj] = col < W.cols ? ld4(in, q0 + col * stride) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int jj = 0; jj < 4; jj++) {
                    const int col = 4 * g + jj;
                    if (col < W.cols)
#pragma unroll
                        for (int q = 0; q < 4; q++)
                            sw[q] = fmaf(W.cf[r * 7 + col], __fsub_rn(f4(xw[jj], q), f4(xs, q)), sw[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (kq(d, q) == ROW_WALL) v[d][q] = sw[q];
        }
    }
    float ao[4], so[4];
    float2 uo[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float lap = 0.f;
        if constexpr (SYS == SYS_HEAT) {
            lap = __fadd_rn(lap, v[0][q]);
            lap = __fadd_rn(lap, v[1][q]);
            lap = __fadd_rn(lap, v[2][q]);
        }
        const float rhs = ((c4 >> (8 * q)) & 0x3Fu)
                              ? rhs_mixed<SYS, VK>(op, sp, sa.etf_stage, i, j, k + q, lap,
                                                   v[0][q], v[1][q], v[2][q])
                              : 0.f;
        rk_mixed<STAGE>(sa, rhs, make_float2(f4(uh, q), f4(ul, q)), f4(av, q), ao[q], so[q],
                        uo[q]);
    }
    // the z-face values of the line's first and last point (record words 16, 17 and 18, 19);
    // every lane takes part in the shuffles, lanes past the line's end store nothing
    const int fw = k == 0 ? 16 : 18;
    const float fa = __shfl_sync(FULL, rec, fw);
    const float fb = STAGE == 3 ? __shfl_sync(FULL, rec, fw + 1) : 0.f;
    if (!kvalid) return;
    if (c4 & 0x40404040u) { // Dirichlet face points (whole planes, or one lane of a line)
#pragma unroll
        for (int q = 0; q < 4; q++) {
            if (!((c4 >> (8 * q)) & CLS_DIRFACE)) continue;
            float2 fv;
            if ((q == 0 && k == 0) || (q == 3 && k + 4 == nz)) {
                fv = make_float2(fa, fb); // z faces: from the line record
            } else {                      // x / y face planes, uniform across the warp
                const float4* f = face_entry(sa, op, i, j, k + q);
                if (!f) continue;
                fv = face_pick<STAGE>(f);
            }
            if constexpr (STAGE < 3)
                so[q] = fv.x;
            else
                uo[q] = fv;
        }
    }
    if constexpr (STAGE < 3) {
        *((float4*)((float*)sa.acc + p)) = make_float4(ao[0], ao[1], ao[2], ao[3]);
        *((float4*)((float*)sa.s_out + p)) = make_float4(so[0], so[1], so[2], so[3]);
    } else {
        float* __restrict__ w0 = (float*)sa.u0;
        *((float4*)(w0 + p)) = make_float4(uo[0].x, uo[1].x, uo[2].x, uo[3].x);
        *((float4*)(w0 + op.N + p)) = make_float4(uo[0].y, uo[1].y, uo[2].y, uo[3].y);
    }
}

// PX > 1: a thread marches over PX consecutive x planes at its (j, k) and keeps the five
// planes of the x stencil in registers, so each further plane costs one x load instead of
// five (the window shifts by one plane per step); the per-point arithmetic is unchanged.
// VEC_BY warps (z lines) per block: a block's slot frees when its slowest warp -- one with
// cut-cell or wall rows -- finishes, so small blocks keep more warp slots busy; MINB counts
// resident 256-thread blocks per SM (4: 64 registers, 3: 85 registers)
constexpr int VEC_BY = 4;
template <int STAGE, int SYS, int FORM, int VK, int MINB, int PX = 1>
__global__ void __launch_bounds__(32 * VEC_BY, MINB * 8 / VEC_BY) k_stage_mixed_vec(DevOp op, SysParams sp, StageArgs sa)
{
    // The stage input, u0 and the accumulator were complete before the cut-row kernel that
    // precedes this one could let it start, so their loads go out before the dependent-launch
    // wait; what that kernel writes (line records, cut-cell values) is read after it.
    pdl_trigger();
    const float* __restrict__ in = STAGE == 0 ? (const float*)sa.u0 : (const float*)sa.s_in;
    const int nx = op.it0, ny = op.it1, nz = op.it2;
    const int lane = threadIdx.x;
    const int j = blockIdx.y * VEC_BY + threadIdx.y;
    if (j >= ny) return; // whole warp
    const int k = blockIdx.x * 128 + 4 * lane;
    const int plane = ny * nz;
    const int pj = j * nz + min(k, nz - 4); // the four points' offset within a plane
    // plane ii of the stage input at the thread's four points, ii clamped into the grid (the
    // clamped planes only feed rows that are not interior)
    auto ldx = [&](int ii) { return ld4(in, min(max(ii, 0), nx - 1) * plane + pj); };
    const int kw = blockIdx.x * 128;
    const bool rec_lane = lane < LREC_WORDS && (kw < 8 || kw + 128 > nz - 8);
    const int i0 = blockIdx.z * PX;
    float4 xa = ldx(i0 - 2), xb = ldx(i0 - 1), C = ldx(i0), xc = ldx(i0 + 1), xd = ldx(i0 + 2);
    VecLoads L = vec_loads<STAGE>(op, sa, in, i0, j, k, C);
    // the line record (k_cut_rows): word `lane` on lanes 0..19 of a warp that holds either
    // end of the line
    pdl_wait();
    const int i1 = min(i0 + PX, nx);
    for (int i = i0;;) {
        const float rec = rec_lane ? __ldcg(sa.lrec + (long long)(i * ny + j) * LREC_WORDS + lane) : 0.f;
        vec_stage_points<STAGE, SYS, FORM, VK>(op, sp, sa, in, i, j, k, lane, L, xa, xb, xc, xd, rec);
        if constexpr (PX == 1) {
            break;
        } else {
            if (++i >= i1) break;
            xa = xb;
            xb = L.C;
            C = xc;
            xc = xd;
            xd = ldx(i + 2);
            L = vec_loads<STAGE>(op, sa, in, i, j, k, C);
        }
    }
}

// ---- TMA plane-marching mixed stage (3-D grids) -----------------------------------------
// A block owns a TY x TZ column tile of the (y, z) plane and marches along x over `px`
// planes.  Stage-field planes (tile + 2-point y halo + 4-point z halo, the z start rounded to
// a 16-byte boundary) arrive in shared memory by cp.async.bulk.tensor into a ring of NS
// slots, each guarded by an mbarrier; the ring keeps planes i-2 .. i+5 so four planes are in
// flight while plane i is computed.  Interior rows read their 5-point stencils from shared
// memory; wall and cut-cell rows (rare, and not warp-uniform) use the global-memory path.
// Every mbarrier wait is bounded: on time-out the block records an error flag, stops issuing
// copies and drains the ones in flight before it returns.
constexpr int TMA_TY = 8, TMA_TZ = 32, TMA_HY = 2, TMA_HZ = 4, TMA_NS = 8;
constexpr int TMA_BY = TMA_TY + 2 * TMA_HY; // 12
constexpr int TMA_BZ = TMA_TZ + 2 * TMA_HZ; // 40
constexpr unsigned TMA_WAIT_LIMIT = 1u << 20;

__device__ __forceinline__ unsigned smem_u32(const void* ptr)
{
    return (unsigned)__cvta_generic_to_shared(ptr);
}
__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)),
                 "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, unsigned parity)
{
    unsigned done;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(done)
                 : "r"(smem_u32(b)), "r"(parity)
                 : "memory");
    return done != 0;
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* b, unsigned parity)
{
    for (unsigned it = 0; it < TMA_WAIT_LIMIT; ++it)
        if (mbar_try_wait(b, parity)) return true;
    return false;
}
__device__ __forceinline__ void fence_proxy_async()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, int c0, int c1,
                                            int c2, uint64_t* bar)
{
    asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
                 " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
                 "l"((unsigned long long)tm), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* b)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}

// Warp-specialised persistent stage.  Work is the list of (tile, plane) pairs in
// tile-major order; CTA b owns the contiguous range [b*W/G, (b+1)*W/G), cut at tile
// boundaries into segments, so one wave of CTAs covers the grid evenly.  Per segment the
// producer warp (warp 8, lane 0) streams planes x_a-2 .. x_b+1 of its tile into a ring of
// TMA_NS slots: each slot gets the stage-field plane with its halo and, for computed
// planes, the class bytes, u0 and accumulator tiles of that plane.  full[s] completes when
// a slot's copies have landed; empty[s] when all eight consumer warps are done with it.
// Consumers (warps 0..7, one tile row each, one point per lane) read only shared memory on
// the interior fast path.  Every wait is bounded; on time-out the CTA records an error
// flag, stops issuing copies, and drains the ones in flight before it returns.
//
// Slot layout: stage-field plane with halo (FP32; the hi plane of u0 in stage 0), class
// bytes, hi tile of u0 (stages 1-3; stage 0 has it in the halo plane), lo tile of u0
// (stage 3), accumulator tile (stages 1-3).
template <int STAGE>
struct TmaSlot {
    static constexpr unsigned S = TMA_BY * TMA_BZ * 4u;
    static constexpr unsigned C = TMA_TY * TMA_TZ;
    static constexpr unsigned UH = STAGE == 0 ? 0u : TMA_TY * TMA_TZ * 4u;
    static constexpr unsigned UL = STAGE == 3 ? TMA_TY * TMA_TZ * 4u : 0u;
    static constexpr unsigned A = STAGE == 0 ? 0u : TMA_TY * TMA_TZ * 4u;
    static constexpr unsigned BYTES = S + C + UH + UL + A;
    static_assert(BYTES % 128 == 0 && S % 128 == 0 && C % 128 == 0 && UH % 128 == 0 &&
                      UL % 128 == 0,
                  "TMA destinations stay 128-byte aligned");
};

template <int STAGE, int SYS>
__global__ void __launch_bounds__(288) k_stage_mixed_tma(const __grid_constant__ CUtensorMap tm_in,
                                                         const __grid_constant__ CUtensorMap tm_u0h,
                                                         const __grid_constant__ CUtensorMap tm_u0l,
                                                         const __grid_constant__ CUtensorMap tm_acc,
                                                         const __grid_constant__ CUtensorMap tm_cls,
                                                         DevOp op, SysParams sp, StageArgs sa,
                                                         unsigned* err)
{
    using L = TmaSlot<STAGE>;
    constexpr unsigned S_BYTES = L::S, C_BYTES = L::C, SLOT = L::BYTES;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw + TMA_NS * SLOT);
    uint64_t* empty = full + TMA_NS;

    const int lane = threadIdx.x, warp = threadIdx.y;
    const int nx = op.it0, ny = op.it1, nz = op.it2;
    const int tiles_z = (nz + TMA_TZ - 1) / TMA_TZ;
    const long long work = (long long)tiles_z * ((ny + TMA_TY - 1) / TMA_TY) * nx;
    const long long w_begin = work * blockIdx.x / gridDim.x;
    const long long w_end = work * (blockIdx.x + 1) / gridDim.x;

    if (warp == 0 && lane == 0) {
        for (int s2 = 0; s2 < TMA_NS; s2++) {
            mbar_init(&full[s2], 1);
            mbar_init(&empty[s2], TMA_TY);
        }
        mbar_fence_init();
    }
    __syncthreads();

    if (warp == TMA_TY) {
        // ---- producer ----
        if (lane != 0) return;
        bool ok = true;
        unsigned r = 0; // stream index of the next plane
        for (long long w = w_begin; ok && w < w_end;) {
            const long long tile = w / nx;
            const int xa = (int)(w % nx);
            const int xb = (int)min((long long)nx, xa + (w_end - w));
            const int k0 = (int)(tile % tiles_z) * TMA_TZ, j0 = (int)(tile / tiles_z) * TMA_TY;
            for (int pl = xa - 2; pl <= xb + 1; ++pl, ++r) {
                const unsigned slot = r % TMA_NS;
                if (r >= TMA_NS && !mbar_wait_bounded(&empty[slot], ((r / TMA_NS) - 1) & 1u)) {
                    ok = false;
                    atomicOr(err, 1u);
                    break;
                }
                unsigned char* base = smem_raw + slot * SLOT;
                const bool own = pl >= xa && pl < xb;
                mbar_expect_tx(&full[slot], own ? SLOT : S_BYTES);
                tma_load_3d(base, &tm_in, k0 - TMA_HZ, j0 - TMA_HY, pl, &full[slot]);
                if (own) {
                    tma_load_3d(base + S_BYTES, &tm_cls, k0, j0, pl, &full[slot]);
                    if (STAGE > 0)
                        tma_load_3d(base + S_BYTES + C_BYTES, &tm_u0h, k0, j0, pl, &full[slot]);
                    if (STAGE == 3)
                        tma_load_3d(base + S_BYTES + C_BYTES + L::UH, &tm_u0l, k0, j0, pl,
                                    &full[slot]);
                    if (STAGE > 0)
                        tma_load_3d(base + S_BYTES + C_BYTES + L::UH + L::UL, &tm_acc, k0, j0,
                                    pl, &full[slot]);
                }
            }
            w += xb - xa;
        }
        if (!ok) {
            // drain the copies that may still be in flight before returning
            const unsigned lo = r >= TMA_NS ? r - TMA_NS : 0u;
            for (unsigned q = lo; q < r; ++q) mbar_wait_bounded(&full[q % TMA_NS], (q / TMA_NS) & 1u);
        }
        return;
    }

    // ---- consumers: warp = tile row, lane = column ----
    const int tz = lane, ty = warp;
    const int s_off = (TMA_HY + ty) * TMA_BZ + (TMA_HZ + tz);
    const int t_off = ty * TMA_TZ + tz;
    const float* __restrict__ cval = (const float*)sa.cval;
    float* __restrict__ accg = (float*)sa.acc;
    const float* __restrict__ gin = STAGE == 0 ? (const float*)sa.u0 : (const float*)sa.s_in;
    const int plane = ny * nz;
    bool ok = true;
    auto wait_full = [&](unsigned q) {
        if (ok && !mbar_wait_bounded(&full[q % TMA_NS], (q / TMA_NS) & 1u)) {
            ok = false;
            atomicOr(err, 1u);
        }
    };
    auto release = [&](unsigned q) {
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[q % TMA_NS]);
    };
    unsigned r0 = 0; // stream index of the segment's first (halo) plane
    for (long long w = w_begin; w < w_end;) {
        const long long tile = w / nx;
        const int xa = (int)(w % nx);
        const int xb = (int)min((long long)nx, xa + (w_end - w));
        const int k = (int)(tile % tiles_z) * TMA_TZ + tz, j = (int)(tile / tiles_z) * TMA_TY + ty;
        const bool col_valid = (j < ny) && (k < nz);
        const long long chunk0 = (long long)j * op.nzc + (tile % tiles_z);
        for (unsigned q = r0; q < r0 + 4; ++q) wait_full(q); // planes xa-2 .. xa+1
        int p = (xa * ny + j) * nz + k;
        for (int i = xa; i < xb; ++i, p += plane) {
            const unsigned r = r0 + 2 + (unsigned)(i - xa); // stream index of plane i
            wait_full(r + 2);
            const unsigned char* cur = smem_raw + (r % TMA_NS) * SLOT;
            const float* Sc = reinterpret_cast<const float*>(cur) + s_off;
            auto Sx = [&](int m) -> float { // plane i-2+m, this column
                return reinterpret_cast<const float*>(smem_raw + ((r - 2 + m) % TMA_NS) * SLOT)[s_off];
            };
            auto Sp = [&](int off) -> float { return Sc[off]; };
            const unsigned c = (col_valid && ok) ? (unsigned)cur[S_BYTES + t_off] : 0u;
            float2 u;
            float accv = 0.f;
            u.x = STAGE == 0 ? Sc[0] : reinterpret_cast<const float*>(cur + S_BYTES + C_BYTES)[t_off];
            u.y = STAGE == 3 ? reinterpret_cast<const float*>(cur + S_BYTES + C_BYTES + L::UH)[t_off] : 0.f;
            if constexpr (STAGE > 0)
                accv = reinterpret_cast<const float*>(cur + S_BYTES + C_BYTES + L::UH + L::UL)[t_off];
            float lap = 0.f;
            float dd[3] = {0.f, 0.f, 0.f};
#pragma unroll
            for (int d = 0; d < 3; d++) {
                const DevAxis& A = op.ax[d];
                const unsigned kind = (c >> (2 * d)) & 3u;
                float v;
                if (__all_sync(FULL, kind == ROW_INTERIOR)) {
                    float xm2, xm1, x0v, xp1, xp2;
                    if (d == 0) {
                        xm2 = Sx(0); xm1 = Sx(1); x0v = Sp(0); xp1 = Sx(3); xp2 = Sx(4);
                    } else if (d == 1) {
                        xm2 = Sp(-2 * TMA_BZ); xm1 = Sp(-TMA_BZ); x0v = Sp(0);
                        xp1 = Sp(TMA_BZ); xp2 = Sp(2 * TMA_BZ);
                    } else {
                        xm2 = Sp(-2); xm1 = Sp(-1); x0v = Sp(0); xp1 = Sp(1); xp2 = Sp(2);
                    }
                    if (A.antisym) {
                        v = fmaf(A.icf[3], xp1 - xm1, A.icf[4] * (xp2 - xm2));
                    } else {
                        v = sym5(A.icf[1], A.icf[0], xm2, xm1, x0v, xp1, xp2);
                    }
                } else {
                    const long long chunk = (long long)i * ny * op.nzc + chunk0;
                    const int row = closure_row(A, kind == ROW_CLOSURE, chunk);
                    v = 0.f;
                    if (kind == ROW_INTERIOR) {
                        v = interior_f<int>(A, gin, p, (int)A.stride);
                    } else if (kind == ROW_WALL) {
                        const int coord = d == 0 ? i : (d == 1 ? j : k);
                        v = wall32(A, (long long)p, coord, gin);
                    } else if (kind == ROW_CLOSURE) {
                        v = cval[A.row_base + row];
                    }
                }
                if (SYS == SYS_HEAT)
                    lap = __fadd_rn(lap, v);
                else
                    dd[d] = v;
            }
            release(r - 2); // plane i-2 is no longer read by this warp
            if (!(col_valid && ok)) continue;
            const float rhs = (c & 0x3Fu) ? rhs_mixed<SYS>(op, sp, sa.etf_stage, i, j, k, lap,
                                                           dd[0], dd[1], dd[2])
                                          : 0.f;
            float a_out = 0.f, s_out = 0.f;
            float2 u_out;
            rk_mixed<STAGE>(sa, rhs, u, accv, a_out, s_out, u_out);
            if constexpr (STAGE < 3) {
                accg[p] = a_out;
                ((float*)sa.s_out)[p] = s_out;
            } else {
                st_pair(sa.u0, op.N, p, u_out);
            }
        }
        // the segment's last four planes (xb-2 .. xb+1) are no longer needed
        const unsigned rend = r0 + 4 + (unsigned)(xb - xa);
        for (unsigned q = rend - 4; q < rend; ++q) release(q);
        r0 = rend;
        w += xb - xa;
    }
}

// Dirichlet face values of the stage output (update_boundary on D), FP64 path
__global__ void k_faces64(DevOp op, DevSol sol, double t, double et, double* out)
{
    pdl_wait();
    pdl_trigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= op.n_faces) return;
    const long long p = op.faces[i];
    const long long nyz = (long long)op.n[1] * op.n[2];
    const int ijk[3] = {(int)(p / nyz), (int)((p / op.n[2]) % op.n[1]), (int)(p % op.n[2])};
    out[p] = sol_at_point(op, sol, t, et, ijk);
}

// Dirichlet cut-point values at t+dt/2 and t+dt of all three R arrays (update_boundary on R)
struct BcRArgs {
    int n[3];
    double* out1[3];
    double* out2[3];
    const double* keep[3];
    float4* fplane[6]; // face planes to fill (mixed path), null where not Dirichlet
    int fn[6];         // points per face plane (0 where not filled)
};
// threads past the cut points fill the Dirichlet face planes of the mixed path
// One item (a cut point or a face point) per iteration of a grid-stride loop: on the side
// stream the kernel runs on a small grid, a step ahead of the stage kernels it feeds, so that
// it holds few of the warp slots those occupancy-bound kernels run in.
__device__ __forceinline__ void bc_r_item(const DevOp& op, const DevR& dr, const DevSol& sol,
                                          const BcRArgs& ra, int i, double t1, double et1,
                                          double t2, double et2);
__global__ void k_bc_r(DevOp op, DevR dr, DevSol sol, BcRArgs ra, int total, double t1,
                       double et1, double t2, double et2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x)
        bc_r_item(op, dr, sol, ra, i, t1, et1, t2, et2);
}
__device__ __forceinline__ void bc_r_item(const DevOp& op, const DevR& dr, const DevSol& sol,
                                          const BcRArgs& ra, int i, double t1, double et1,
                                          double t2, double et2)
{
    int d = 0;
    while (d < 3 && i >= ra.n[d]) i -= ra.n[d++];
    if (d == 3) {
        int f = 0;
        while (f < 6 && i >= ra.fn[f]) i -= ra.fn[f++];
        if (f == 6) return;
        const int a = f >> 1, c = a == 2 ? 1 : 2;
        // the face's fixed coordinate and its two running ones (b, c = the other axes in
        // order), placed by selects: indexed writes would put ijk in local memory
        const int fixed = (f & 1) ? op.n[a] - 1 : 0;
        const int vb = i / op.n[c], vc = i - vb * op.n[c];
        const int ijk[3] = {a == 0 ? fixed : vb, a == 1 ? fixed : (a == 0 ? vb : vc),
                            a == 2 ? fixed : vc};
        const float2 u = ff_from_double(sol_at_point(op, sol, t2, et2, ijk));
        ra.fplane[f][i] = make_float4(face_f32(op, sol, t1, et1, ijk),
                                      face_f32(op, sol, t2, et2, ijk), u.x, u.y);
        return;
    }
    double* out1 = ra.out1[d];
    double* out2 = ra.out2[d];
    const double* keep = ra.keep[d];
    if (dr.dirichlet[d][i]) {
        const double* x = dr.pos[d] + 3 * (long long)i;
        out1[i] = sol_at(sol, t1, et1, x, nullptr, d, i);
        out2[i] = sol_at(sol, t2, et2, x, nullptr, d, i);
    } else {
        out1[i] = keep[i];
        out2[i] = keep[i];
    }
}

// one RHS evaluation into an FP64 field (system::rhs)
template <int SYS, bool MIXED>
__global__ void __launch_bounds__(256) k_rhs(DevOp op, SysParams sp, const void* uin,
                                             const double* R0, const double* R1,
                                             const double* R2, double t, double et,
                                             double* out)
{
    const Pt q = point_of(op);
    const unsigned c = q.valid ? op.cls[q.p] : 0u;
    const double* R[3] = {R0, R1, R2};
    int ijk[3];
    phys_ijk(op, q, ijk);
    double lap = 0.0, dd[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const DevAxis& A = op.ax[d];
        if (!A.active) continue;
        const unsigned kind = (c >> (2 * d)) & 3u;
        const int row = closure_row(A, kind == ROW_CLOSURE, q.chunk);
        double v = 0.0;
        if (MIXED) {
            const PairU in{(const float*)uin, op.N};
            if (kind == ROW_INTERIOR) v = (double)interior32(A, in, q.p);
            else if (kind == ROW_WALL) v = (double)wall32(A, q.p, ijk[d], in);
            else if (kind == ROW_CLOSURE)
                v = closure64(A, row, q.p, in, R[d], (const double*)nullptr, 0.0, true);
        } else {
            const double* in = (const double*)uin;
            if (kind == ROW_INTERIOR) v = interior64(A, in, q.p);
            else if (kind == ROW_WALL) v = wall64(A, q.p, ijk[d], in, nullptr, 0.0, true);
            else if (kind == ROW_CLOSURE)
                v = closure64(A, row, q.p, in, R[d], (const double*)nullptr, 0.0, true);
        }
        if (SYS == SYS_HEAT)
            lap = lap + v;
        else
            dd[d] = v;
    }
    if (!q.valid) return;
    double rhs = 0.0;
    if (c & 0x3Fu) {
        if (SYS == SYS_HEAT) {
            double src = 0.0;
            if (sp.sol.kind == SOL_SINSIN) {
                const double u = sol_at_point(op, sp.sol, t, et, ijk);
                src = (-u) - sp.k * (sp.sol.lapfac * u);
            }
            rhs = fma(lap, sp.k, src);
        } else {
            double g[3] = {-sp.vel[0], -sp.vel[1], -sp.vel[2]};
            if (sp.vel_kind != 0) radial_g64(sp, op, ijk, g);
            rhs = fma(g[2], dd[2], fma(g[1], dd[1], g[0] * dd[0]));
        }
    }
    out[q.p] = rhs;
}

// initialize_scalar_field: 0 on non-fluid D points, exact on fluid D points
__global__ void __launch_bounds__(256) k_init(DevOp op, DevSol sol, double t, double et,
                                              int mixed, void* u0)
{
    const Pt q = point_of(op);
    if (!q.valid) return;
    const unsigned c = op.cls[q.p];
    double v = 0.0;
    if (c & CLS_FLUID) {
        int ijk[3];
        phys_ijk(op, q, ijk);
        v = sol_point_any(op, sol, t, et, ijk);
    }
    if (mixed)
        st_pair(u0, op.N, q.p, ff_from_double(v));
    else
        ((double*)u0)[q.p] = v;
}

__global__ void k_init_r(DevR dr, DevSol sol, int n, int d, double t, double et, double* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = sol_any(sol, t, et, dr.pos[d] + 3 * (long long)i, nullptr, d, i);
}

__global__ void k_convert(long long n, int to_mixed, const double* in_d, float* out_m,
                          const float* in_m, double* out_d)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (to_mixed) {
        st_pair(out_m, n, i, ff_from_double(in_d[i]));
    } else {
        const float2 v = ld_pair(in_m, n, i);
        out_d[i] = (double)v.x + (double)v.y;
    }
}

// stats over fluid D points: per block max error (+index), min, max
struct StatPart {
    double err;
    long long idx;
    double mn, mx;
};

__device__ __forceinline__ void stat_merge(StatPart& m, const StatPart& o)
{
    if (o.err > m.err || (o.err == m.err && o.err >= 0 && o.idx < m.idx)) {
        m.err = o.err;
        m.idx = o.idx;
    }
    m.mn = fmin(m.mn, o.mn);
    m.mx = fmax(m.mx, o.mx);
}

__global__ void __launch_bounds__(256) k_stats(DevOp op, DevSol sol, double t, double et,
                                               int mixed, const void* u0, StatPart* parts)
{
    const Pt q = point_of(op);
    StatPart s{-1.0, 0, 1e308, -1e308};
    if (q.valid && (op.cls[q.p] & CLS_FLUID)) {
        const double u = mixed ? ldd(PairU{(const float*)u0, op.N}, q.p) : ((const double*)u0)[q.p];
        int ijk[3];
        phys_ijk(op, q, ijk);
        double e = fabs(u - sol_point_any(op, sol, t, et, ijk));
        // a non-finite value counts as an infinite error so that system validity trips
        if (!(e <= 1.7976931348623157e308)) e = __longlong_as_double(0x7ff0000000000000LL);
        s = StatPart{e, q.p, isnan(u) ? 0.0 : u, isnan(u) ? 0.0 : u};
    }
    __shared__ StatPart sh[256];
    const int tid = threadIdx.y * 32 + threadIdx.x;
    sh[tid] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (tid < w) stat_merge(sh[tid], sh[tid + w]);
        __syncthreads();
    }
    if (tid == 0) {
        const long long b =
            ((long long)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
        parts[b] = sh[0];
    }
}

__global__ void k_stats_final(long long nparts, const StatPart* parts, double* out)
{
    __shared__ StatPart sh[256];
    StatPart s{-1.0, 0, 1e308, -1e308};
    for (long long i = threadIdx.x; i < nparts; i += 256) stat_merge(s, parts[i]);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) stat_merge(sh[threadIdx.x], sh[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sh[0].err < 0 ? 0.0 : sh[0].err;
        out[1] = (double)sh[0].idx;
        out[2] = sh[0].mn;
        out[3] = sh[0].mx;
    }
}

} // namespace

long long kernel_launch_count() { return g_launches.load(); }

// ===========================================================================================
// launchers
// ===========================================================================================
// ---- vectorised FP32 operators (3-D grids, nz a multiple of 4) -----------------------------
// The layout of k_stage_mixed_vec: four z points per thread, float4 loads of the field at
// the points and their stencil neighbours, interior rows from registers kept where the class
// says "interior".  Cut-cell rows (FP64 arithmetic as op_row, Neumann-aware) and the z-wall
// rows are evaluated first by k_op_rows into the problem's scratch: cut-cell rows at their
// points, z-wall rows as one 16-word record per z line (words 0..5 the left block's rows,
// 8..13 the right block's) that lanes 0..15 of the warps at the line's ends load at entry and
// hand to the lanes holding those rows by warp shuffles; x- and y-wall rows (whole planes,
// uniform across a warp) inline.
// MODE 0..2: derivative along x, y, z (eq or, PLUS, plus_eq: only points with a row are
// written); 3: Laplacian (every point, 0 where no axis has a row); 4: gradient (three
// outputs, 0 where the axis has no row).
namespace
{
template <class TR> // the R values' type: FP32, or FP64 (the mixed unfused step)
__global__ void k_op_rows(DevOp op, int d0, int d1, const float* __restrict__ u,
                          const TR* R0, const TR* R1, const TR* R2,
                          const double* __restrict__ nu)
{
    pdl_trigger(); // the operator kernel after it may start and issue its stencil loads
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int r0 = op.ax[d0].row_base, r1 = d1 < 3 ? op.ax[d1].row_base : op.n_cut_rows;
    if (i < r1 - r0) {
        const int g = r0 + i;
        const int d = g < op.ax[1].row_base ? 0 : (g < op.ax[2].row_base ? 1 : 2);
        const DevAxis& A = op.ax[d];
        const int row = g - A.row_base;
        const long long p = A.row_out[row];
        const TR* Rd = d == 0 ? R0 : (d == 1 ? R1 : R2);
        op.op_rowv[d * op.N + p] = (float)closure64(A, row, p, u, Rd, nu, 0.0, true);
        return;
    }
    i -= r1 - r0;
    const int nlines = op.it0 * op.it1;
    if (d1 < 3 || i >= nlines) return; // z walls only with the z axis
    const DevAxis& A = op.ax[2];
    const long long base = (long long)i * op.it2;
    float w[16];
#pragma unroll
    for (int m = 0; m < 16; m++) w[m] = 0.f;
#pragma unroll
    for (int side = 0; side < 2; side++) {
        const WallBlock& W = A.wall[side];
        float x[7];
#pragma unroll
        for (int jj = 0; jj < 7; jj++) x[jj] = jj < W.cols ? __ldg(u + base + W.col0 + jj) : 0.f;
#pragma unroll
        for (int r = 0; r < 6; r++) {
            if (r >= W.rows) continue;
            float acc = wall_row_diff(W, r, x); // wall32's arithmetic
            if (W.has_n && nu) acc = (float)fma(W.n[r], __ldg(nu + base + W.wall), (double)acc);
            w[side * 8 + r] = acc;
        }
    }
    float4* o = reinterpret_cast<float4*>(op.op_zw + (long long)i * 16);
#pragma unroll
    for (int m = 0; m < 4; m++) o[m] = make_float4(w[4 * m], w[4 * m + 1], w[4 * m + 2], w[4 * m + 3]);
}

// z lines per block: four for the Laplacian (its 13 float4 loads a lane make the block's
// slowest warp matter most), eight for a derivative or the gradient (measured each way)
template <int MODE>
__host__ __device__ constexpr int op_vec_by() { return MODE == 3 ? 4 : 8; }

template <int MODE, bool PLUS, int FORM>
__global__ void __launch_bounds__(32 * op_vec_by<MODE>(), 32 / op_vec_by<MODE>()) k_op_vec(DevOp op, const float* __restrict__ u,
                                                   const double* __restrict__ nu,
                                                   float* __restrict__ o0, float* __restrict__ o1,
                                                   float* __restrict__ o2)
{
    pdl_trigger();
    constexpr bool NX = MODE == 0 || MODE >= 3, NY = MODE == 1 || MODE >= 3,
                   NZ = MODE == 2 || MODE >= 3;
    const int nx = op.it0, ny = op.it1, nz = op.it2;
    const int j = blockIdx.y * op_vec_by<MODE>() + threadIdx.y;
    if (j >= ny) return; // whole warp
    const int i = blockIdx.z;
    const int k = blockIdx.x * 128 + 4 * threadIdx.x;
    const bool kvalid = k < nz;
    const int plane = ny * nz;
    const int kc = min(k, nz - 4);
    const int p = i * plane + j * nz + kc;
    const unsigned c4 = kvalid ? __ldg((const unsigned*)(op.cls + p)) : 0u;
    const float4 C = ld4(u, p);
    float4 xa{}, xb{}, xc{}, xd{}, ya{}, yb{}, yc{}, yd{}, zL{}, zR{};
    if constexpr (NX) {
        xa = ld4(u, p + (max(i - 2, 0) - i) * plane);
        xb = ld4(u, p + (max(i - 1, 0) - i) * plane);
        xc = ld4(u, p + (min(i + 1, nx - 1) - i) * plane);
        xd = ld4(u, p + (min(i + 2, nx - 1) - i) * plane);
    }
    if constexpr (NY) {
        ya = ld4(u, p + (max(j - 2, 0) - j) * nz);
        yb = ld4(u, p + (max(j - 1, 0) - j) * nz);
        yc = ld4(u, p + (min(j + 1, ny - 1) - j) * nz);
        yd = ld4(u, p + (min(j + 2, ny - 1) - j) * nz);
    }
    if constexpr (NZ) {
        zL = ld4(u, p + (kc >= 4 ? -4 : 0));
        zR = ld4(u, p + (kc + 8 <= nz ? 4 : 0));
    }
    const float zz[8] = {zL.z, zL.w, C.x, C.y, C.z, C.w, zR.x, zR.y};
    pdl_wait(); // what k_op_rows wrote is read below
    float rec = 0.f; // the line's z-wall record word of this lane (k_op_rows)
    if constexpr (NZ) {
        const int lane = threadIdx.x;
        if (lane < 8 ? blockIdx.x == 0 : (lane < 16 && blockIdx.x + 1 == gridDim.x))
            rec = __ldcg(op.op_zw + (long long)(i * ny + j) * 16 + lane);
    }
    float v[3][4] = {};
    unsigned kq[3][4];
    bool cut = false, zwall = false, xywall = false;
#pragma unroll
    for (int q = 0; q < 4; q++) {
#pragma unroll
        for (int d = 0; d < 3; d++) {
            kq[d][q] = (c4 >> (8 * q + 2 * d)) & 3u;
            const bool need = d == 0 ? NX : (d == 1 ? NY : NZ);
            if (!need) continue;
            cut = cut || kq[d][q] == ROW_CLOSURE;
            if (d == 2)
                zwall = zwall || kq[d][q] == ROW_WALL;
            else
                xywall = xywall || kq[d][q] == ROW_WALL;
        }
        if constexpr (NX)
            v[0][q] = kq[0][q] == ROW_INTERIOR
                          ? interior_row_t<FORM>(op.ax[0], f4(xa, q), f4(xb, q), f4(C, q), f4(xc, q), f4(xd, q))
                          : 0.f;
        if constexpr (NY)
            v[1][q] = kq[1][q] == ROW_INTERIOR
                          ? interior_row_t<FORM>(op.ax[1], f4(ya, q), f4(yb, q), f4(C, q), f4(yc, q), f4(yd, q))
                          : 0.f;
        if constexpr (NZ)
            v[2][q] = kq[2][q] == ROW_INTERIOR
                          ? interior_row_t<FORM>(op.ax[2], zz[q], zz[q + 1], zz[q + 2], zz[q + 3], zz[q + 4])
                          : 0.f;
    }
    if (cut) {
        const float* rv = op.op_rowv + p; // written by k_op_rows, the dependent-launch predecessor
#pragma unroll
        for (int d = 0; d < 3; d++)
#pragma unroll
            for (int q = 0; q < 4; q++)
                if ((d == 0 ? NX : (d == 1 ? NY : NZ)) && kq[d][q] == ROW_CLOSURE)
                    v[d][q] = __ldcg(rv + d * op.N + q);
    }
    if constexpr (NZ) {
        if (__any_sync(FULL, zwall)) { // the record word of each z-wall row to its lane
            const DevAxis& A = op.ax[2];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int kk = k + q;
                const bool use = kq[2][q] == ROW_WALL;
                const int w = kk * 2 < nz ? kk - A.wall[0].first_row : 8 + kk - A.wall[1].first_row;
                const float val = __shfl_sync(FULL, rec, use ? w : 0);
                if (use) v[2][q] = val;
            }
        }
    }
    if constexpr (NX || NY) {
        if (__any_sync(FULL, xywall)) {
#pragma unroll
            for (int d = 0; d < 2; d++) {
                if (!(d == 0 ? NX : NY)) continue;
#pragma unroll
                for (int q = 0; q < 4; q++)
                    if (kq[d][q] == ROW_WALL) {
                        const int coord = d == 0 ? i : j;
                        const float w = wall32(op.ax[d], (long long)(p + q), coord, u);
                        v[d][q] = wall_neumann32(op.ax[d], (long long)(p + q), coord, nu, w);
                    }
            }
        }
    }
    if (!kvalid) return;
    if constexpr (MODE <= 2) {
        constexpr int d = MODE;
        const bool all = kq[d][0] && kq[d][1] && kq[d][2] && kq[d][3];
        if (all) {
            float4 r = make_float4(v[d][0], v[d][1], v[d][2], v[d][3]);
            if constexpr (PLUS) {
                const float4 o = *(const float4*)(o0 + p);
                r = make_float4(o.x + r.x, o.y + r.y, o.z + r.z, o.w + r.w);
            }
            *(float4*)(o0 + p) = r;
        } else {
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (kq[d][q] != ROW_NONE) o0[p + q] = PLUS ? o0[p + q] + v[d][q] : v[d][q];
        }
    } else if constexpr (MODE == 3) {
        float lap[4];
#pragma unroll
        for (int q = 0; q < 4; q++) {
            float a = 0.f; // op_row's order: axes x, y, z, only those with a row
#pragma unroll
            for (int d = 0; d < 3; d++)
                if (kq[d][q] != ROW_NONE) a = a + v[d][q];
            lap[q] = a;
        }
        *(float4*)(o0 + p) = make_float4(lap[0], lap[1], lap[2], lap[3]);
    } else {
        float* outs[3] = {o0, o1, o2};
#pragma unroll
        for (int d = 0; d < 3; d++)
            *(float4*)(outs[d] + p) = make_float4(v[d][0], v[d][1], v[d][2], v[d][3]);
    }
}

template <int MODE, bool PLUS>
void op_vec(const DevOp& op, const float* u, const double* nu, float* o0, float* o1, float* o2,
            cudaStream_t s)
{
    // dependent launch after k_op_rows: the kernel issues its stencil loads and waits for
    // the prepass before it reads the cut-cell values and the z-wall records
    constexpr int by = op_vec_by<MODE>();
    const dim3 grid((op.it2 + 127) / 128, (op.it1 + by - 1) / by, op.it0), block(32, by);
    if (op.op_form == FORM_ANTI5)
        launch_ex(k_op_vec<MODE, PLUS, FORM_ANTI5>, grid, block, s, true, op, u, nu, o0, o1, o2);
    else if (op.op_form == FORM_SYM5)
        launch_ex(k_op_vec<MODE, PLUS, FORM_SYM5>, grid, block, s, true, op, u, nu, o0, o1, o2);
    else
        launch_ex(k_op_vec<MODE, PLUS, FORM_W3>, grid, block, s, true, op, u, nu, o0, o1, o2);
    ++g_launches;
}

void op_rows(const DevOp& op, int d0, int d1, const float* u, const void* const R[3],
             const double* nu, cudaStream_t s, bool r64 = false)
{
    const int r0 = op.ax[d0].row_base, r1 = d1 < 3 ? op.ax[d1].row_base : op.n_cut_rows;
    const long long n = (long long)(r1 - r0) + (d1 == 3 ? (long long)op.it0 * op.it1 : 0);
    if (n <= 0) return;
    const unsigned nb = (unsigned)((n + 127) / 128);
    if (r64)
        k_op_rows<double><<<nb, 128, 0, s>>>(op, d0, d1, u, (const double*)R[0],
                                             (const double*)R[1], (const double*)R[2], nu);
    else
        k_op_rows<float><<<nb, 128, 0, s>>>(op, d0, d1, u, (const float*)R[0],
                                            (const float*)R[1], (const float*)R[2], nu);
    ++g_launches;
}

bool op_vec_ok(const DevOp& op)
{
    return op.op_form > 0 && op.op_rowv && op.op_zw;
}
} // namespace

cudaError_t launch_derivative(const DevOp& op, int dir, int prec, const void* uD,
                              const void* uR, const double* nuD, void* duD, void* const duR[3],
                              const void* const uRall[3], int plus_eq, cudaStream_t s)
{
    const dim3 grid = point_grid(op), block(32, BY);
    if (!op.ax[dir].active) return cudaSuccess;
    if (prec == PREC_FP64) {
        if (plus_eq)
            k_derivative<double, true><<<grid, block, 0, s>>>(op, dir, (const double*)uD,
                                                              (const double*)uR, nuD,
                                                              (double*)duD);
        else
            k_derivative<double, false><<<grid, block, 0, s>>>(op, dir, (const double*)uD,
                                                               (const double*)uR, nuD,
                                                               (double*)duD);
        ++g_launches;
        return rspace_for<double>(op, dir, uD, uRall, duR, s);
    }
    if (op_vec_ok(op)) {
        const void* Rs[3] = {nullptr, nullptr, nullptr};
        Rs[dir] = uR;
        op_rows(op, dir, dir + 1, (const float*)uD, Rs, nuD, s);
        float* o = (float*)duD;
        const float* u = (const float*)uD;
        if (plus_eq) {
            if (dir == 0) op_vec<0, true>(op, u, nuD, o, nullptr, nullptr, s);
            else if (dir == 1) op_vec<1, true>(op, u, nuD, o, nullptr, nullptr, s);
            else op_vec<2, true>(op, u, nuD, o, nullptr, nullptr, s);
        } else {
            if (dir == 0) op_vec<0, false>(op, u, nuD, o, nullptr, nullptr, s);
            else if (dir == 1) op_vec<1, false>(op, u, nuD, o, nullptr, nullptr, s);
            else op_vec<2, false>(op, u, nuD, o, nullptr, nullptr, s);
        }
        return rspace_for<float>(op, dir, uD, uRall, duR, s);
    }
    if (plus_eq)
        k_derivative<float, true><<<grid, block, 0, s>>>(op, dir, (const float*)uD,
                                                         (const float*)uR, nuD, (float*)duD);
    else
        k_derivative<float, false><<<grid, block, 0, s>>>(op, dir, (const float*)uD,
                                                          (const float*)uR, nuD, (float*)duD);
    ++g_launches;
    return rspace_for<float>(op, dir, uD, uRall, duR, s);
}

cudaError_t launch_laplacian(const DevOp& op, int prec, const void* uD, const void* const uR[3],
                             const double* nuD, void* duD, void* const duR[3], cudaStream_t s)
{
    const dim3 grid = point_grid(op), block(32, BY);
    const size_t es = prec == PREC_FP64 ? 8 : 4;
    for (int r = 0; r < 3; r++)
        if (op.nR[r] && duR[r]) cudaMemsetAsync(duR[r], 0, op.nR[r] * es, s);
    if (prec == PREC_FP64) {
        k_laplacian<double><<<grid, block, 0, s>>>(op, (const double*)uD, (const double*)uR[0],
                                                   (const double*)uR[1], (const double*)uR[2],
                                                   nuD, (double*)duD);
        ++g_launches;
        rspace_axes<double>(op, 7, uD, uR, duR, s);
    } else if (op_vec_ok(op)) {
        op_rows(op, 0, 3, (const float*)uD, uR, nuD, s);
        op_vec<3, false>(op, (const float*)uD, nuD, (float*)duD, nullptr, nullptr, s);
        rspace_axes<float>(op, 7, uD, uR, duR, s);
    } else {
        k_laplacian<float><<<grid, block, 0, s>>>(op, (const float*)uD, (const float*)uR[0],
                                                  (const float*)uR[1], (const float*)uR[2], nuD,
                                                  (float*)duD);
        ++g_launches;
        rspace_axes<float>(op, 7, uD, uR, duR, s);
    }
    return cudaGetLastError();
}

cudaError_t launch_gradient(const DevOp& op, int prec, const void* uD, const void* const uR[3],
                            void* const out[3][4], cudaStream_t s)
{
    const dim3 grid = point_grid(op), block(32, BY);
    const size_t es = prec == PREC_FP64 ? 8 : 4;
    for (int d = 0; d < 3; d++)
        for (int r = 0; r < 3; r++)
            if (op.nR[r] && out[d][r + 1]) cudaMemsetAsync(out[d][r + 1], 0, op.nR[r] * es, s);
    if (prec == PREC_FP64) {
        k_gradient<double><<<grid, block, 0, s>>>(
            op, (const double*)uD, (const double*)uR[0], (const double*)uR[1],
            (const double*)uR[2], (double*)out[0][0], (double*)out[1][0], (double*)out[2][0]);
        ++g_launches;
        for (int d = 0; d < 3; d++) {
            void* const dR[3] = {out[d][1], out[d][2], out[d][3]};
            if (op.ax[d].active) rspace_for<double>(op, d, uD, uR, dR, s);
        }
    } else if (op_vec_ok(op) && out[0][0] && out[1][0] && out[2][0]) {
        op_rows(op, 0, 3, (const float*)uD, uR, nullptr, s);
        op_vec<4, false>(op, (const float*)uD, nullptr, (float*)out[0][0], (float*)out[1][0],
                         (float*)out[2][0], s);
        for (int d = 0; d < 3; d++) {
            void* const dR[3] = {out[d][1], out[d][2], out[d][3]};
            if (op.ax[d].active) rspace_for<float>(op, d, uD, uR, dR, s);
        }
    } else {
        k_gradient<float><<<grid, block, 0, s>>>(
            op, (const float*)uD, (const float*)uR[0], (const float*)uR[1], (const float*)uR[2],
            (float*)out[0][0], (float*)out[1][0], (float*)out[2][0]);
        ++g_launches;
        for (int d = 0; d < 3; d++) {
            void* const dR[3] = {out[d][1], out[d][2], out[d][3]};
            if (op.ax[d].active) rspace_for<float>(op, d, uD, uR, dR, s);
        }
    }
    return cudaGetLastError();
}

namespace
{
// The mixed Laplacian and gradient with FP32 D values and FP64 R values in and out (the
// mixed unfused step, whose cut-point values are state): interior and wall rows in FP32,
// cut-cell rows in FP64 from the FP64 cut-point values, R-space rows accumulated and stored
// in FP64.
cudaError_t laplacian_mixed_r64(const DevOp& op, const float* uD, double* const uR[3],
                                const double* nuD, float* duD, double* const duR[3], cudaStream_t s)
{
    for (int r = 0; r < 3; r++)
        if (op.nR[r] && duR[r]) cudaMemsetAsync(duR[r], 0, op.nR[r] * sizeof(double), s);
    const void* uRv[3] = {uR[0], uR[1], uR[2]};
    void* const duRv[3] = {duR[0], duR[1], duR[2]};
    if (op_vec_ok(op)) {
        op_rows(op, 0, 3, uD, uRv, nuD, s, true);
        op_vec<3, false>(op, uD, nuD, duD, nullptr, nullptr, s);
    } else {
        k_laplacian<float, double><<<point_grid(op), dim3(32, BY), 0, s>>>(op, uD, uR[0], uR[1],
                                                                           uR[2], nuD, duD);
        ++g_launches;
    }
    rspace_axes<float, double>(op, 7, uD, uRv, duRv, s);
    return cudaGetLastError();
}

cudaError_t gradient_mixed_r64(const DevOp& op, const float* uD, double* const uR[3],
                               float* const outD[3], double* const outR[3][3], cudaStream_t s)
{
    for (int d = 0; d < 3; d++)
        for (int r = 0; r < 3; r++)
            if (op.nR[r] && outR[d][r]) cudaMemsetAsync(outR[d][r], 0, op.nR[r] * sizeof(double), s);
    const void* uRv[3] = {uR[0], uR[1], uR[2]};
    if (op_vec_ok(op)) {
        op_rows(op, 0, 3, uD, uRv, nullptr, s, true);
        op_vec<4, false>(op, uD, nullptr, outD[0], outD[1], outD[2], s);
    } else {
        k_gradient<float, double><<<point_grid(op), dim3(32, BY), 0, s>>>(
            op, uD, uR[0], uR[1], uR[2], outD[0], outD[1], outD[2]);
        ++g_launches;
    }
    for (int d = 0; d < 3; d++) {
        void* const dR[3] = {outR[d][0], outR[d][1], outR[d][2]};
        if (op.ax[d].active) rspace_for<float, double>(op, d, uD, uRv, dR, s);
    }
    return cudaGetLastError();
}
} // namespace

namespace
{

template <int STAGE, int SYS>
void launch_stage(const DevOp& op, const SysParams& sp, int prec, const StageArgs& a,
                  const StepBuffers& b, cudaStream_t s, cudaEvent_t* ev, cudaEvent_t join)
{
    const dim3 grid = point_grid(op), block(32, BY);
    const bool mixed = prec == PREC_MIXED;
    float* rowv = mixed && b.vec ? a.rowv : nullptr;
    // the vectorised stage's line records (one thread per z line after the cut-cell rows);
    // they hold face values, so the boundary values of the step must be ready first
    StageArgs ca = a;
    ca.lrec = mixed && b.vec ? a.lrec : nullptr;
    const long long n_lines = ca.lrec ? (long long)op.it0 * op.it1 : 0;
    if (join) cudaStreamWaitEvent(s, join, 0); // boundary values of the step are ready
    if (op.n_cut_rows || n_lines) {
        const int nb = (int)((op.n_cut_rows + n_lines + 127) / 128);
        const double* const* R = a.R;
        if (!mixed)
            launch_ex(k_cut_rows<CgD, double>, dim3(nb), dim3(128), s, true, op,
                      CgD{(const double*)(STAGE == 0 ? a.u0 : a.s_in)}, R[0], R[1], R[2],
                      (double*)a.cval, nullptr, ca, STAGE);
        else if (STAGE == 0)
            launch_ex(k_cut_rows<CgPair, float>, dim3(nb), dim3(128), s, b.vec != 0, op,
                      CgPair{(const float*)a.u0, op.N}, R[0], R[1], R[2], (float*)a.cval, rowv,
                      ca, STAGE);
        else
            launch_ex(k_cut_rows<CgF, float>, dim3(nb), dim3(128), s, b.vec != 0, op,
                      CgF{(const float*)a.s_in}, R[0], R[1], R[2], (float*)a.cval, rowv, ca, STAGE);
        ++g_launches;
    }
    if (ev) cudaEventRecord(ev[0], s);
    const bool small = op.N < (1LL << 31) - 64;
    if (mixed && b.tma) {
        const CUtensorMap& tm = STAGE == 0 ? b.tm_u0 : (STAGE == 2 ? b.tm_sb : b.tm_sa);
        const size_t smem = TMA_NS * TmaSlot<STAGE>::BYTES + 2 * TMA_NS * 8;
        static int grid_n[4] = {0, 0, 0, 0};
        if (!grid_n[STAGE]) {
            cudaFuncSetAttribute(k_stage_mixed_tma<STAGE, SYS>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
            int per_sm = 0, dev = 0, sms = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_stage_mixed_tma<STAGE, SYS>,
                                                          32 * (TMA_TY + 1), smem);
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            grid_n[STAGE] = std::max(1, per_sm) * std::max(1, sms);
        }
        const long long work = (long long)((op.it2 + TMA_TZ - 1) / TMA_TZ) *
                               ((op.it1 + TMA_TY - 1) / TMA_TY) * op.it0;
        const int grid = (int)std::min<long long>(grid_n[STAGE], work);
        k_stage_mixed_tma<STAGE, SYS><<<grid, dim3(32, TMA_TY + 1), smem, s>>>(
            tm, b.tm_u0t, b.tm_u0l, b.tm_acct, b.tm_cls, op, sp, a, b.err);
    } else if (mixed && b.vec) {
        const int px = b.vec_px;
        const dim3 vgrid((op.it2 + 127) / 128, (op.it1 + VEC_BY - 1) / VEC_BY, (op.it0 + px - 1) / px);
        // 4 or 3 resident blocks per SM (64 or 85 registers per thread); 1, 2 or 4 x planes
        // per thread
        auto go = [&](auto kern) { launch_ex(kern, vgrid, dim3(32, VEC_BY), s, true, op, sp, a); };
        auto pick = [&](auto form, auto vk) {
            constexpr int F = decltype(form)::value, V = decltype(vk)::value;
            if (px == 4)
                go(k_stage_mixed_vec<STAGE, SYS, F, V, 3, 4>);
            else if (px == 2)
                go(k_stage_mixed_vec<STAGE, SYS, F, V, 3, 2>);
            else if (b.vec_minb == 4)
                go(k_stage_mixed_vec<STAGE, SYS, F, V, 4, 1>);
            else
                go(k_stage_mixed_vec<STAGE, SYS, F, V, 3, 1>);
        };
        using I0 = std::integral_constant<int, 0>;
        using I1 = std::integral_constant<int, 1>;
        if constexpr (SYS == SYS_WAVE) {
            if (sp.vel_kind)
                pick(std::integral_constant<int, FORM_ANTI5>{}, I1{});
            else
                pick(std::integral_constant<int, FORM_ANTI5>{}, I0{});
        } else {
            if (b.vec == FORM_SYM5)
                pick(std::integral_constant<int, FORM_SYM5>{}, I0{});
            else
                pick(std::integral_constant<int, FORM_W3>{}, I0{});
        }
    } else if (mixed && b.col_nx) {
        const dim3 cgrid(op.nzc, (op.it1 + BY - 1) / BY, (op.it0 + b.col_nx - 1) / b.col_nx);
        if (b.col_nx == 2)
            k_stage_mixed_col<STAGE, SYS, 2><<<cgrid, block, 0, s>>>(op, sp, a);
        else if (b.col_nx == 4)
            k_stage_mixed_col<STAGE, SYS, 4><<<cgrid, block, 0, s>>>(op, sp, a);
        else
            k_stage_mixed_col<STAGE, SYS, 1><<<cgrid, block, 0, s>>>(op, sp, a);
    } else if (mixed) {
        if (small)
            k_stage_mixed<STAGE, SYS, int><<<grid, block, 0, s>>>(op, sp, a);
        else
            k_stage_mixed<STAGE, SYS, long long><<<grid, block, 0, s>>>(op, sp, a);
    } else {
        if (small)
            launch_ex(k_stage64<STAGE, SYS, int>, grid, block, s, true, op, sp, a);
        else
            launch_ex(k_stage64<STAGE, SYS, long long>, grid, block, s, true, op, sp, a);
    }
    ++g_launches;
    if (ev) cudaEventRecord(ev[1], s);
    // Dirichlet faces: the vectorised kernel writes them itself
    if (op.n_faces && !(mixed && b.vec)) {
        const int nb = (op.n_faces + 255) / 256;
        if (mixed)
            k_faces_mixed<STAGE><<<nb, 256, 0, s>>>(op, a);
        else
            launch_ex(k_faces64, dim3(nb), dim3(256), s, true, op, sp.sol, a.t_next, a.et_next,
                      (double*)(STAGE == 3 ? a.u0 : a.s_out));
        ++g_launches;
    }
}

template <int SYS>
void launch_stages(const DevOp& op, const SysParams& sp, int prec, StageArgs sa[4],
                   const StepBuffers& b, cudaStream_t s, cudaEvent_t* ev)
{
    // the boundary values of the step come from the side stream when there is one
    launch_stage<0, SYS>(op, sp, prec, sa[0], b, s, ev ? ev + 2 : nullptr, b.side ? b.join : nullptr);
    launch_stage<1, SYS>(op, sp, prec, sa[1], b, s, ev ? ev + 4 : nullptr, nullptr);
    launch_stage<2, SYS>(op, sp, prec, sa[2], b, s, ev ? ev + 6 : nullptr, nullptr);
    launch_stage<3, SYS>(op, sp, prec, sa[3], b, s, ev ? ev + 8 : nullptr, nullptr);
}
} // namespace

// ev (optional): 10 events -- [0] step start, [1] after the cut-point BC kernel,
// [2+2i], [3+2i] around the main kernel of stage i
cudaError_t launch_rk4_step(const DevOp& op, const DevR& dr, const SysParams& sp, int prec,
                            StepBuffers& b, double t, double dt, cudaStream_t s,
                            cudaEvent_t* ev, bool prefetch_next)
{
    // src/temporal/rk4.cpp:11-12
    constexpr double rki[4] = {0.0, 0.5, 0.5, 1.0};
    constexpr double rkf[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
    const bool sinsin = sp.sol.kind == SOL_SINSIN;
    auto et = [&](double tt) { return sinsin ? std::exp(-tt) : 0.0; };

    // Dirichlet values of the step starting at tt on the cut points (tt+dt/2, tt+dt) and,
    // in the mixed path, on the domain faces.  keep: the R values at tt (kept where the
    // cut point is not Dirichlet).
    auto launch_bc = [&](double tt, double* const keep[3], double* const rh[3],
                         double* const rf[3], float4* const fp[6], cudaStream_t bs) {
        const double h = tt + dt * rki[1], f = tt + dt * rki[3];
        BcRArgs ra;
        long long tot = 0;
        for (int d = 0; d < 3; d++) {
            ra.n[d] = (int)op.nR[d];
            ra.out1[d] = rh[d];
            ra.out2[d] = rf[d];
            ra.keep[d] = keep[d];
            tot += ra.n[d];
        }
        for (int k = 0; k < 6; k++) {
            ra.fplane[k] = fp[k];
            ra.fn[k] = fp[k] ? face_plane_size_host(op, k) : 0;
            tot += ra.fn[k];
        }
        if (tot) {
            // inline (no side stream): one thread per item; on the side stream: two blocks
            // per SM, looping, a step ahead of the stage kernels
            static int sms = 0;
            if (!sms) {
                int dev = 0;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            }
            const long long full = (tot + 127) / 128;
            const unsigned nb = (unsigned)(bs == s ? full : std::min<long long>(full, 2LL * std::max(sms, 1)));
            k_bc_r<<<nb, 128, 0, bs>>>(op, dr, sp.sol, ra, (int)tot, h, et(h), f, et(f));
            ++g_launches;
        }
    };

    if (ev) cudaEventRecord(ev[0], s);
    if (!b.side) {
        launch_bc(t, b.R, b.Rhalf, b.Rfull, b.fplane, s);
    } else {
        // the side stream starts after everything issued so far on s (the previous step,
        // the last reader of the buffers it overwrites)
        cudaEventRecord(b.fork, s);
        cudaStreamWaitEvent(b.side, b.fork, 0);
        if (b.next_pending && b.next_t == t && b.next_dt == dt) {
            // evaluated during the previous step: make that set the current one
            for (int d = 0; d < 3; d++) {
                std::swap(b.Rhalf[d], b.Rhalf_next[d]);
                std::swap(b.Rfull[d], b.Rfull_next[d]);
            }
            for (int k = 0; k < 6; k++) std::swap(b.fplane[k], b.fplane_next[k]);
            std::swap(b.join, b.join_next);
        } else {
            launch_bc(t, b.R, b.Rhalf, b.Rfull, b.fplane, b.side);
            cudaEventRecord(b.join, b.side);
        }
        b.next_pending = false;
        if (prefetch_next) {
            // the next step starts from this step's R at t + dt (Rfull)
            launch_bc(t + dt, b.Rfull, b.Rhalf_next, b.Rfull_next, b.fplane_next, b.side);
            cudaEventRecord(b.join_next, b.side);
            b.next_pending = true;
            b.next_t = t + dt;
            b.next_dt = dt;
        }
    }
    if (ev) cudaEventRecord(ev[1], s);
    StageArgs sa[4];
    for (int i = 0; i < 4; i++) {
        StageArgs& a = sa[i];
        a.u0 = b.u0;
        a.acc = b.acc;
        a.cval = b.cval;
        a.rowv = b.rowv;
        a.lrec = b.lrec;
        for (int f = 0; f < 6; f++) a.fplane[f] = b.fplane[f];
        a.s_in = i == 0 ? b.u0 : (i == 2 ? b.sb : b.sa);
        a.s_out = i == 1 ? b.sb : b.sa;
        for (int d = 0; d < 3; d++)
            a.R[d] = i == 0 ? b.R[d] : (i == 3 ? b.Rfull[d] : b.Rhalf[d]);
        a.cf = dt * rkf[i];
        a.ci = i < 3 ? dt * rki[i + 1] : 1.0;
        a.cf_ff = ff_host(a.cf);
        a.ci_ff = ff_host(a.ci);
        a.t_stage = t + dt * rki[i];
        a.t_next = i < 3 ? t + dt * rki[i + 1] : t + dt;
        a.et_stage = et(a.t_stage);
        a.et_next = et(a.t_next);
        a.etf_stage = (float)a.et_stage;
        a.cut_fp64 = b.cut_fp64;
    }
    if (sp.kind == SYS_HEAT)
        launch_stages<SYS_HEAT>(op, sp, prec, sa, b, s, ev);
    else
        launch_stages<SYS_WAVE>(op, sp, prec, sa, b, s, ev);
    for (int d = 0; d < 3; d++) std::swap(b.R[d], b.Rfull[d]);
    return cudaGetLastError();
}

// ===========================================================================================
// Unfused FP64 heat step, for systems whose objects are not all Dirichlet.  The values at the
// cut points of Floating objects are state: the reference's rk4::operator()
// (src/temporal/rk4.cpp:16-47) advances the whole scalar field {D, Rx, Ry, Rz}, the
// Laplacian's R-space rows (Bf, Br) give their right-hand side, and heat::update_boundary
// (src/systems/heat.cpp:296-354) resets the Dirichlet faces and the Dirichlet cut points to
// the exact solution after every stage.  Each stage here is the standalone Laplacian (which
// evaluates those rows), one kernel forming k*lap + source, and whole-field axpys.
// ===========================================================================================
namespace
{
// flat index over {D, Rx, Ry, Rz} -> (part 0..3, index within the part)
__device__ __forceinline__ int field_part(const DevOp& op, long long g, long long& i)
{
    if (g < op.N) {
        i = g;
        return 0;
    }
    g -= op.N;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        if (g < op.nR[d]) {
            i = g;
            return 1 + d;
        }
        g -= op.nR[d];
    }
    return -1;
}

__device__ __forceinline__ double heat_source(const SysParams& sp, double u)
{
    return __dsub_rn(-u, __dmul_rn(sp.k, __dmul_rn(sp.sol.lapfac, u)));
}

__device__ __forceinline__ void phys_of_point(const DevOp& op, long long p, int ijk[3])
{
    const long long nyz = (long long)op.n[1] * op.n[2];
    ijk[0] = (int)(p / nyz);
    ijk[1] = (int)((p / op.n[2]) % op.n[1]);
    ijk[2] = (int)(p % op.n[2]);
}

// The RK4 bookkeeping folded into the right-hand side's last pass (an unfused stage):
// instead of storing the right-hand side v, acc <- acc + c_acc v and, before the last
// stage, y <- u + c_y v (the next stage's input), with the arithmetic of k_field_lc.
struct StageFold {
    int on;
    FieldF64 acc;
    double c_acc;
    int has_y;
    FieldF64 y;
    FieldF64 u;
    double c_y;
};

// K <- k * lap + source (heat::build_rhs_graph, heat.cpp:164-288): the source at fluid D
// points and at non-Dirichlet cut points; 0 on Dirichlet faces and at Dirichlet cut points.
// With f.on the value goes into the RK4 registers instead (StageFold).
__global__ void k_heat_rhs_finish(DevOp op, DevR dr, SysParams sp, double t, double et, FieldF64 K,
                                  StageFold f)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long i = 0;
    const int part = field_part(op, g, i);
    if (part < 0) return;
    const bool sinsin = sp.sol.kind == SOL_SINSIN;
    const bool gauss = sp.sol.kind == SOL_GAUSSIAN;
    auto put = [&](double* k, double* acc, double* y, const double* u, long long j, double v) {
        if (!f.on) {
            k[j] = v;
            return;
        }
        acc[j] = __dadd_rn(acc[j], __dmul_rn(f.c_acc, v));
        if (f.has_y) y[j] = __dadd_rn(u[j], __dmul_rn(f.c_y, v));
    };
    // the source ddt - k lap of the Gaussian sum at x
    auto gauss_source = [&](const double x[3]) {
        const GaussEval ge = gauss_eval(sp.sol, t, x);
        return __dsub_rn(ge.ddt, __dmul_rn(sp.k, ge.lap));
    };
    if (part == 0) {
        const unsigned c = op.cls[i];
        double v = __dmul_rn(K.D[i], sp.k);
        if ((c & CLS_FLUID) && (sinsin || gauss)) {
            int ijk[3];
            phys_of_point(op, i, ijk);
            if (sinsin) {
                v = __dadd_rn(v, heat_source(sp, sol_at_point(op, sp.sol, t, et, ijk)));
            } else {
                const double x[3] = {op.xc[0][ijk[0]], op.xc[1][ijk[1]], op.xc[2][ijk[2]]};
                v = __dadd_rn(v, gauss_source(x));
            }
        }
        if (c & CLS_DIRFACE) v = 0.0;
        put(K.D, f.acc.D, f.y.D, f.u.D, i, v);
    } else {
        const int d = part - 1;
        double v = __dmul_rn(K.R[d][i], sp.k);
        if (dr.dirichlet[d][i])
            v = 0.0;
        else if (sinsin)
            v = __dadd_rn(v, heat_source(sp, sol_at(sp.sol, t, et, dr.pos[d] + 3 * i, nullptr, d, (int)i)));
        else if (gauss)
            v = __dadd_rn(v, gauss_source(dr.pos[d] + 3 * i));
        put(K.R[d], f.acc.R[d], f.y.R[d], f.u.R[d], i, v);
    }
}

// out <- a + c * k over the whole field (slot_assign_lc / slot_accumulate, slot_ops.hpp:11-61)
__global__ void k_field_lc(DevOp op, FieldF64 out, FieldF64 a, double c, FieldF64 k)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long i = 0;
    const int part = field_part(op, g, i);
    if (part < 0) return;
    if (part == 0)
        out.D[i] = __dadd_rn(a.D[i], __dmul_rn(c, k.D[i]));
    else
        out.R[part - 1][i] = __dadd_rn(a.R[part - 1][i], __dmul_rn(c, k.R[part - 1][i]));
}

// heat::update_boundary: Dirichlet faces and Dirichlet cut points take the exact solution
__global__ void k_update_boundary(DevOp op, DevR dr, DevSol sol, double t, double et, FieldF64 u)
{
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < op.n_faces) {
        const long long p = op.faces[g];
        int ijk[3];
        phys_of_point(op, p, ijk);
        u.D[p] = sol_point_any(op, sol, t, et, ijk);
        return;
    }
    g -= op.n_faces;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        if (g < op.nR[d]) {
            if (dr.dirichlet[d][g]) u.R[d][g] = sol_any(sol, t, et, dr.pos[d] + 3 * g, nullptr, d, (int)g);
            return;
        }
        g -= op.nR[d];
    }
}

// Neumann data of heat::update_boundary (heat.cpp:324-352) at time t: on each Neumann face
// of axis a, the gradient component a of the solution (sin-sin: 2 pi k cos(2 pi k x_a) times
// the other axes' sines, times e^-t; the Gaussian sum's gradient; zero otherwise), axes in
// order, so at an edge shared with a later axis' Neumann face the later axis' value is the
// one written.
__global__ void k_neumann_faces(DevOp op, DevSol sol, int mask, double t, double et, double* nu)
{
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    for (int f = 0; f < 6; f++) {
        const int a = f >> 1, b = a == 0 ? 1 : 0, c = a == 2 ? 1 : 2;
        const long long fn = (mask >> f) & 1 ? (long long)op.n[b] * op.n[c] : 0;
        if (i >= fn) {
            i -= fn;
            continue;
        }
        int ijk[3];
        ijk[a] = (f & 1) ? op.n[a] - 1 : 0;
        ijk[b] = (int)(i / op.n[c]);
        ijk[c] = (int)(i - (long long)ijk[b] * op.n[c]);
        for (int a2 = a + 1; a2 < 3; a2++) // a later axis' Neumann face holds this point
            if (((mask >> (2 * a2)) & 1 && ijk[a2] == 0) ||
                ((mask >> (2 * a2 + 1)) & 1 && ijk[a2] == op.n[a2] - 1))
                return;
        double v = 0.0;
        if (sol.kind == SOL_SINSIN) {
            const double kk = 2 * 3.14159265358979323846 * sol.p[0];
            v = 1.0;
            for (int d = 0; d < sol.dims; d++)
                v = __dmul_rn(v, d == a ? __dmul_rn(kk, sol.C[d][ijk[d]]) : sol.S[d][ijk[d]]);
            v = __dmul_rn(v, et);
        } else if (sol.kind == SOL_GAUSSIAN) {
            const double x[3] = {op.xc[0][ijk[0]], op.xc[1][ijk[1]], op.xc[2][ijk[2]]};
            v = gauss_eval(sol, t, x).grad[a];
        }
        const long long nyz = (long long)op.n[1] * op.n[2];
        nu[ijk[0] * nyz + (long long)ijk[1] * op.n[2] + ijk[2]] = v;
        return;
    }
}

long long field_size(const DevOp& op) { return op.N + op.nR[0] + op.nR[1] + op.nR[2]; }

cudaError_t heat_rhs_unfused(const DevOp& op, const DevR& dr, const SysParams& sp, NeumannFaces nf,
                             FieldF64 u, double t, FieldF64 K, cudaStream_t s, StageFold fold = {})
{
    const double et = sp.sol.kind == SOL_SINSIN ? std::exp(-t) : 0.0;
    if (nf.mask) {
        long long nface = 0;
        for (int f = 0; f < 6; f++)
            if ((nf.mask >> f) & 1) {
                const int a = f >> 1, b = a == 0 ? 1 : 0, c = a == 2 ? 1 : 2;
                nface += (long long)op.n[b] * op.n[c];
            }
        k_neumann_faces<<<(unsigned)((nface + 255) / 256), 256, 0, s>>>(op, sp.sol, nf.mask, t, et, nf.nu);
        ++g_launches;
    }
    const void* uR[3] = {u.R[0], u.R[1], u.R[2]};
    void* kR[3] = {K.R[0], K.R[1], K.R[2]};
    cudaError_t e = launch_laplacian(op, PREC_FP64, u.D, uR, nf.mask ? nf.nu : nullptr, K.D, kR, s);
    if (e != cudaSuccess) return e;
    const long long n = field_size(op);
    k_heat_rhs_finish<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(op, dr, sp, t, et, K, fold);
    ++g_launches;
    return cudaGetLastError();
}
} // namespace

namespace
{
// the radial velocity field's -(x - c) / |x - c| at a point x (scalar_wave.cpp:28-33), in
// radial_g64's operation order
__device__ __forceinline__ void radial_g64x(const SysParams& sp, const double x[3], double g[3])
{
    const double r[3] = {x[0] - sp.center[0], x[1] - sp.center[1], x[2] - sp.center[2]};
    const double len = sqrt(r[0] * r[0] + (r[1] * r[1] + r[2] * r[2]));
    g[0] = -r[0] / len;
    g[1] = -r[1] / len;
    g[2] = -r[2] / len;
}

// scalar_wave::build_rhs_graph on the whole field (src/systems/scalar_wave.cpp:241-321):
// K <- gG . grad u with gG = -a (constant velocity) or the radial field, and gG zero on
// Dirichlet faces and at Dirichlet cut points (scalar_wave.cpp:79-95).  G0..G2: the
// gradient's components over the whole field (D rows, then the R-space rows at the cut
// points).  Points without a row (solid points) take 0, as in the fused stage kernels; the
// dot product is the fused kernels' (fma(g2, d2, fma(g1, d1, g0 d0))).  With f.on the value
// goes into the RK4 registers instead (StageFold).
__global__ void k_wave_rhs_finish(DevOp op, DevR dr, SysParams sp, FieldF64 G0, FieldF64 G1,
                                  FieldF64 G2, FieldF64 K, StageFold f)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long i = 0;
    const int part = field_part(op, g, i);
    if (part < 0) return;
    auto put = [&](double* k, double* acc, double* y, const double* u, long long j, double v) {
        if (!f.on) {
            k[j] = v;
            return;
        }
        acc[j] = __dadd_rn(acc[j], __dmul_rn(f.c_acc, v));
        if (f.has_y) y[j] = __dadd_rn(u[j], __dmul_rn(f.c_y, v));
    };
    double gv[3] = {-sp.vel[0], -sp.vel[1], -sp.vel[2]};
    if (part == 0) {
        const unsigned c = op.cls[i];
        double v = 0.0;
        if ((c & 0x3Fu) && !(c & CLS_DIRFACE)) {
            if (sp.vel_kind != 0) {
                int ijk[3];
                phys_of_point(op, i, ijk);
                radial_g64(sp, op, ijk, gv);
            }
            v = fma(gv[2], G2.D[i], fma(gv[1], G1.D[i], gv[0] * G0.D[i]));
        }
        put(K.D, f.acc.D, f.y.D, f.u.D, i, v);
    } else {
        const int d = part - 1;
        double v = 0.0;
        if (!dr.dirichlet[d][i]) {
            if (sp.vel_kind != 0) radial_g64x(sp, dr.pos[d] + 3 * i, gv);
            v = fma(gv[2], G2.R[d][i], fma(gv[1], G1.R[d][i], gv[0] * G0.R[d][i]));
        }
        put(K.R[d], f.acc.R[d], f.y.R[d], f.u.R[d], i, v);
    }
}

cudaError_t wave_rhs_unfused(const DevOp& op, const DevR& dr, const SysParams& sp,
                             const UnfusedAux& ux, FieldF64 u, double t, FieldF64 K, cudaStream_t s,
                             StageFold fold = {})
{
    (void)t; // the wave's right-hand side has no time-dependent term
    const void* uR[3] = {u.R[0], u.R[1], u.R[2]};
    void* const out[3][4] = {
        {ux.grad[0].D, ux.grad[0].R[0], ux.grad[0].R[1], ux.grad[0].R[2]},
        {ux.grad[1].D, ux.grad[1].R[0], ux.grad[1].R[1], ux.grad[1].R[2]},
        {ux.grad[2].D, ux.grad[2].R[0], ux.grad[2].R[1], ux.grad[2].R[2]}};
    cudaError_t e = launch_gradient(op, PREC_FP64, u.D, uR, out, s);
    if (e != cudaSuccess) return e;
    const long long n = field_size(op);
    k_wave_rhs_finish<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(op, dr, sp, ux.grad[0], ux.grad[1],
                                                                  ux.grad[2], K, fold);
    ++g_launches;
    return cudaGetLastError();
}

cudaError_t rhs_unfused(const DevOp& op, const DevR& dr, const SysParams& sp, const UnfusedAux& ux,
                        FieldF64 u, double t, FieldF64 K, cudaStream_t s, StageFold fold = {})
{
    if (sp.kind == SYS_WAVE) return wave_rhs_unfused(op, dr, sp, ux, u, t, K, s, fold);
    return heat_rhs_unfused(op, dr, sp, ux.nf, u, t, K, s, fold);
}

// ---- the unfused whole-field step in mixed precision ------------------------------------
// FP32 stage input, right-hand side and stage accumulator at the D points, FP64 at the cut
// points (whose values are state and enter cut-cell rows with large coefficients); the
// operators are the mixed ones with FP64 R values (FP32 interior and wall rows, FP64
// cut-cell and R-space rows); the state stays FP64 and receives the step's accumulated
// increment once.  The D points' arithmetic of the right-hand side and of the RK4 registers
// is the fused mixed stage's (rhs_mixed, rk_mixed); the cut points' is the FP64 step's.
struct StageFoldMx {
    int on;
    FieldMx acc;
    float2 c_acc_f; // dt rkf[i] as a compensated FP32 pair (D points)
    double c_acc;   // and in FP64 (cut points)
    int has_y;
    FieldMx y;
    FieldF64 u;
    float c_y_f; // dt rki[i+1]
    double c_y;
};

__device__ __forceinline__ void fold_d(const StageFoldMx& f, float* k, long long j, float v,
                                       const FieldF64& u)
{
    if (!f.on) {
        k[j] = v;
        return;
    }
    f.acc.D[j] = __fadd_rn(f.acc.D[j], fmaf(f.c_acc_f.x, v, __fmul_rn(f.c_acc_f.y, v)));
    if (f.has_y) f.y.D[j] = fmaf(f.c_y_f, v, (float)u.D[j]);
}

__device__ __forceinline__ void fold_r(const StageFoldMx& f, double* k, int d, long long j, double v)
{
    if (!f.on) {
        k[j] = v;
        return;
    }
    f.acc.R[d][j] = __dadd_rn(f.acc.R[d][j], __dmul_rn(f.c_acc, v));
    if (f.has_y) f.y.R[d][j] = __dadd_rn(f.u.R[d][j], __dmul_rn(f.c_y, v));
}

// K <- k lap + source: FP32 at the D points (rhs_mixed's arithmetic: the sin-sin source from
// the FP32 sine tables; the Gaussian source evaluated in FP64 and rounded), FP64 at the cut
// points (k_heat_rhs_finish's arithmetic); 0 on Dirichlet faces and at Dirichlet cut points
__global__ void k_heat_rhs_finish_mx(DevOp op, DevR dr, SysParams sp, double t, double et, float etf,
                                     FieldMx K, StageFoldMx f)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long i = 0;
    const int part = field_part(op, g, i);
    if (part < 0) return;
    const bool sinsin = sp.sol.kind == SOL_SINSIN;
    const bool gauss = sp.sol.kind == SOL_GAUSSIAN;
    auto gauss_source = [&](const double x[3]) {
        const GaussEval ge = gauss_eval(sp.sol, t, x);
        return __dsub_rn(ge.ddt, __dmul_rn(sp.k, ge.lap));
    };
    if (part == 0) {
        const unsigned c = op.cls[i];
        float src = 0.f;
        if ((c & CLS_FLUID) && (sinsin || gauss)) {
            int ijk[3];
            phys_of_point(op, i, ijk);
            if (sinsin) {
                const bool d3 = sp.sol.dims == 3;
                src = sinsin_heat_src_f(sp.sol.Sf[0][ijk[0]], sp.sol.Sf[1][ijk[1]],
                                        d3 ? sp.sol.Sf[2][ijk[2]] : 0.f, d3, etf, sp.kf,
                                        (float)sp.sol.lapfac);
            } else {
                const double x[3] = {op.xc[0][ijk[0]], op.xc[1][ijk[1]], op.xc[2][ijk[2]]};
                src = (float)gauss_source(x);
            }
        }
        float v = fmaf(K.D[i], sp.kf, src);
        if (c & CLS_DIRFACE) v = 0.f;
        fold_d(f, K.D, i, v, f.u);
    } else {
        const int d = part - 1;
        double v = __dmul_rn(K.R[d][i], sp.k);
        if (dr.dirichlet[d][i])
            v = 0.0;
        else if (sinsin)
            v = __dadd_rn(v, heat_source(sp, sol_at(sp.sol, t, et, dr.pos[d] + 3 * i, nullptr, d, (int)i)));
        else if (gauss)
            v = __dadd_rn(v, gauss_source(dr.pos[d] + 3 * i));
        fold_r(f, K.R[d], d, i, v);
    }
}

// K <- gG . grad u: rhs_mixed's FP32 arithmetic at the D points, k_wave_rhs_finish's FP64
// arithmetic at the cut points; 0 at points without a row, on Dirichlet faces and at
// Dirichlet cut points
__global__ void k_wave_rhs_finish_mx(DevOp op, DevR dr, SysParams sp, FieldMx G0, FieldMx G1,
                                     FieldMx G2, FieldMx K, StageFoldMx f)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long i = 0;
    const int part = field_part(op, g, i);
    if (part < 0) return;
    if (part == 0) {
        const unsigned c = op.cls[i];
        float v = 0.f;
        if ((c & 0x3Fu) && !(c & CLS_DIRFACE)) {
            float g0 = sp.gf[0], g1 = sp.gf[1], g2 = sp.gf[2];
            if (sp.vel_kind != 0) {
                int ijk[3];
                phys_of_point(op, i, ijk);
                const float r0 = __fsub_rn((float)op.xc[0][ijk[0]], sp.centerf[0]);
                const float r1 = __fsub_rn((float)op.xc[1][ijk[1]], sp.centerf[1]);
                const float r2 = __fsub_rn((float)op.xc[2][ijk[2]], sp.centerf[2]);
                const float il = rsqrtf(fmaf(r2, r2, fmaf(r1, r1, __fmul_rn(r0, r0))));
                g0 = __fmul_rn(-r0, il);
                g1 = __fmul_rn(-r1, il);
                g2 = __fmul_rn(-r2, il);
            }
            v = fmaf(g2, G2.D[i], fmaf(g1, G1.D[i], __fmul_rn(g0, G0.D[i])));
        }
        fold_d(f, K.D, i, v, f.u);
    } else {
        const int d = part - 1;
        double v = 0.0;
        if (!dr.dirichlet[d][i]) {
            double gv[3] = {-sp.vel[0], -sp.vel[1], -sp.vel[2]};
            if (sp.vel_kind != 0) radial_g64x(sp, dr.pos[d] + 3 * i, gv);
            v = fma(gv[2], G2.R[d][i], fma(gv[1], G1.R[d][i], gv[0] * G0.R[d][i]));
        }
        fold_r(f, K.R[d], d, i, v);
    }
}

// Dirichlet faces (FP32) and Dirichlet cut points (FP64) of a stage input take the exact
// solution
__global__ void k_update_boundary_mx(DevOp op, DevR dr, DevSol sol, double t, double et, FieldMx u)
{
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < op.n_faces) {
        const long long p = op.faces[g];
        int ijk[3];
        phys_of_point(op, p, ijk);
        u.D[p] = (float)sol_point_any(op, sol, t, et, ijk);
        return;
    }
    g -= op.n_faces;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        if (g < op.nR[d]) {
            if (dr.dirichlet[d][g]) u.R[d][g] = sol_any(sol, t, et, dr.pos[d] + 3 * g, nullptr, d, (int)g);
            return;
        }
        g -= op.nR[d];
    }
}

// out <- the state with its D values rounded to FP32; out <- in widened; u <- u + acc (the
// step's increment)
__global__ void k_field_to_mx(DevOp op, FieldMx out, FieldF64 in)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long i = 0;
    const int part = field_part(op, g, i);
    if (part == 0)
        out.D[i] = (float)in.D[i];
    else if (part > 0)
        out.R[part - 1][i] = in.R[part - 1][i];
}

__global__ void k_field_from_mx(DevOp op, FieldF64 out, FieldMx in)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long i = 0;
    const int part = field_part(op, g, i);
    if (part == 0)
        out.D[i] = (double)in.D[i];
    else if (part > 0)
        out.R[part - 1][i] = in.R[part - 1][i];
}

__global__ void k_field_acc_mx(DevOp op, FieldF64 u, FieldMx acc)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long i = 0;
    const int part = field_part(op, g, i);
    if (part == 0)
        u.D[i] = __dadd_rn(u.D[i], (double)acc.D[i]);
    else if (part > 0)
        u.R[part - 1][i] = __dadd_rn(u.R[part - 1][i], acc.R[part - 1][i]);
}

cudaError_t rhs_unfused_mx(const DevOp& op, const DevR& dr, const SysParams& sp, const UnfusedAux& ux,
                           FieldMx u, double t, FieldMx K, cudaStream_t s, StageFoldMx fold = {})
{
    const long long n = field_size(op);
    const unsigned nb = (unsigned)((n + 255) / 256);
    if (sp.kind == SYS_WAVE) {
        const FieldMx* G = ux.grad_mx;
        float* const outD[3] = {G[0].D, G[1].D, G[2].D};
        double* const outR[3][3] = {{G[0].R[0], G[0].R[1], G[0].R[2]},
                                    {G[1].R[0], G[1].R[1], G[1].R[2]},
                                    {G[2].R[0], G[2].R[1], G[2].R[2]}};
        cudaError_t e = gradient_mixed_r64(op, u.D, u.R, outD, outR, s);
        if (e != cudaSuccess) return e;
        k_wave_rhs_finish_mx<<<nb, 256, 0, s>>>(op, dr, sp, G[0], G[1], G[2], K, fold);
        ++g_launches;
        return cudaGetLastError();
    }
    const double et = sp.sol.kind == SOL_SINSIN ? std::exp(-t) : 0.0;
    const NeumannFaces& nf = ux.nf;
    if (nf.mask) {
        long long nface = 0;
        for (int f = 0; f < 6; f++)
            if ((nf.mask >> f) & 1) {
                const int a = f >> 1, b = a == 0 ? 1 : 0, c = a == 2 ? 1 : 2;
                nface += (long long)op.n[b] * op.n[c];
            }
        k_neumann_faces<<<(unsigned)((nface + 255) / 256), 256, 0, s>>>(op, sp.sol, nf.mask, t, et, nf.nu);
        ++g_launches;
    }
    cudaError_t e = laplacian_mixed_r64(op, u.D, u.R, nf.mask ? nf.nu : nullptr, K.D, K.R, s);
    if (e != cudaSuccess) return e;
    k_heat_rhs_finish_mx<<<nb, 256, 0, s>>>(op, dr, sp, t, et, (float)et, K, fold);
    ++g_launches;
    return cudaGetLastError();
}

cudaError_t step_unfused_mx(const DevOp& op, const DevR& dr, const SysParams& sp, const UnfusedAux& ux,
                            FieldF64 U, double t, double dt, cudaStream_t s)
{
    constexpr double rki[4] = {0.0, 0.5, 0.5, 1.0};
    constexpr double rkf[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
    const long long n = field_size(op);
    const unsigned nb = (unsigned)((n + 255) / 256);
    const long long nbnd = op.n_faces + op.nR[0] + op.nR[1] + op.nR[2];
    const unsigned bb = (unsigned)std::max(1LL, (nbnd + 255) / 256);
    auto et = [&](double tt) { return sp.sol.kind == SOL_SINSIN ? std::exp(-tt) : 0.0; };
    const FieldMx Y = ux.y_mx, K = ux.k_mx, ACC = ux.acc_mx;
    cudaError_t e = cudaMemsetAsync(ACC.D, 0, op.N * sizeof(float), s);
    for (int d = 0; d < 3 && e == cudaSuccess; d++)
        if (op.nR[d]) e = cudaMemsetAsync(ACC.R[d], 0, op.nR[d] * sizeof(double), s);
    if (e != cudaSuccess) return e;
    // stage 0's input: the state, its D values rounded to FP32 (the fused mixed stage reads
    // the hi words)
    k_field_to_mx<<<nb, 256, 0, s>>>(op, Y, U);
    ++g_launches;
    // stage i: K <- rhs(Y); its last pass adds dt rkf[i] k_i into ACC and (i < 3) writes the
    // next stage's input Y <- U + dt rki[i+1] k_i after the operators have finished reading Y
    for (int i = 0; i < 4 && e == cudaSuccess; i++) {
        const double ti = t + dt * rki[i];
        const double ca = dt * rkf[i];
        const float cah = (float)ca;
        const double cy = i < 3 ? dt * rki[i + 1] : 0.0;
        const StageFoldMx fold{1, ACC, make_float2(cah, (float)(ca - (double)cah)), ca, i < 3, Y, U,
                               (float)cy, cy};
        e = rhs_unfused_mx(op, dr, sp, ux, Y, ti, K, s, fold);
        if (e != cudaSuccess) break;
        if (i < 3) {
            const double tn = t + dt * rki[i + 1];
            k_update_boundary_mx<<<bb, 256, 0, s>>>(op, dr, sp.sol, tn, et(tn), Y);
            ++g_launches;
        }
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
    k_field_acc_mx<<<nb, 256, 0, s>>>(op, U, ACC);
    k_update_boundary<<<bb, 256, 0, s>>>(op, dr, sp.sol, t + dt, et(t + dt), U);
    g_launches += 2;
    return cudaGetLastError();
}
} // namespace

cudaError_t launch_rhs_unfused(const DevOp& op, const DevR& dr, const SysParams& sp,
                               const UnfusedAux& ux, FieldF64 u, double t, FieldF64 out,
                               cudaStream_t s)
{
    if (!ux.mixed) return rhs_unfused(op, dr, sp, ux, u, t, out, s);
    // mixed: the state with its D values rounded to FP32, the mixed right-hand side, widened
    // into out
    const unsigned nb = (unsigned)((field_size(op) + 255) / 256);
    k_field_to_mx<<<nb, 256, 0, s>>>(op, ux.y_mx, u);
    ++g_launches;
    cudaError_t e = rhs_unfused_mx(op, dr, sp, ux, ux.y_mx, t, ux.k_mx, s);
    if (e != cudaSuccess) return e;
    k_field_from_mx<<<nb, 256, 0, s>>>(op, out, ux.k_mx);
    ++g_launches;
    return cudaGetLastError();
}

// one RK4 step of the whole field U (rk4.cpp:16-47) with the scratch fields Y, K, ACC; the
// boundary data of each stage input and of the result are the exact solution on Dirichlet
// faces and at Dirichlet cut points (heat::update_boundary and scalar_wave::update_boundary
// set the same values there)
cudaError_t launch_step_unfused(const DevOp& op, const DevR& dr, const SysParams& sp,
                                const UnfusedAux& ux, FieldF64 U, FieldF64 Y, FieldF64 K,
                                FieldF64 ACC, double t, double dt, cudaStream_t s)
{
    if (ux.mixed) return step_unfused_mx(op, dr, sp, ux, U, t, dt, s);
    constexpr double rki[4] = {0.0, 0.5, 0.5, 1.0};
    constexpr double rkf[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
    const long long n = field_size(op);
    const unsigned nb = (unsigned)((n + 255) / 256);
    const long long nbnd = op.n_faces + op.nR[0] + op.nR[1] + op.nR[2];
    const unsigned bb = (unsigned)std::max(1LL, (nbnd + 255) / 256);
    auto et = [&](double tt) { return sp.sol.kind == SOL_SINSIN ? std::exp(-tt) : 0.0; };
    // rk_rhs <- 0, then += dt rkf[i] k_i (rk4.cpp:21, 40)
    cudaError_t e = cudaMemsetAsync(ACC.D, 0, op.N * sizeof(double), s);
    for (int d = 0; d < 3 && e == cudaSuccess; d++)
        if (op.nR[d]) e = cudaMemsetAsync(ACC.R[d], 0, op.nR[d] * sizeof(double), s);
    // stage i: K <- lap(in), then the last pass adds dt rkf[i] k_i into ACC and (i < 3)
    // writes the next stage's input Y <- U + dt rki[i+1] k_i, whose boundary data is then
    // set at its time; the input of stage i > 0 is Y, which the Laplacian has finished
    // reading before that pass overwrites it
    for (int i = 0; i < 4 && e == cudaSuccess; i++) {
        const double ti = t + dt * rki[i];
        const StageFold fold{1, ACC, dt * rkf[i], i < 3, Y, U, i < 3 ? dt * rki[i + 1] : 0.0};
        e = rhs_unfused(op, dr, sp, ux, i == 0 ? U : Y, ti, K, s, fold);
        if (e != cudaSuccess) break;
        if (i < 3) {
            const double tn = t + dt * rki[i + 1];
            k_update_boundary<<<bb, 256, 0, s>>>(op, dr, sp.sol, tn, et(tn), Y);
            ++g_launches;
        }
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) return e;
    k_field_lc<<<nb, 256, 0, s>>>(op, U, U, 1.0, ACC);
    k_update_boundary<<<bb, 256, 0, s>>>(op, dr, sp.sol, t + dt, et(t + dt), U);
    g_launches += 2;
    return cudaGetLastError();
}

// One forward Euler step of an FP64 system (integrators::euler, src/temporal/euler.cpp:11-27):
// K <- rhs(U, t) (the unfused heat right-hand side, or the fused systems' k_rhs with a zero
// right-hand side at the Dirichlet cut points), U <- U + dt K, then the boundary data at
// t + dt (Dirichlet faces and Dirichlet cut points).  For fused systems U.D is b.u0 and U.R
// the state's cut-point values b.R.
cudaError_t launch_euler_fp64(const DevOp& op, const DevR& dr, const SysParams& sp, const UnfusedAux& ux,
                              bool unfused, const StepBuffers& b, FieldF64 U, FieldF64 K, double t,
                              double dt, cudaStream_t s)
{
    cudaError_t e = unfused ? rhs_unfused(op, dr, sp, ux, U, t, K, s)
                            : launch_rhs(op, sp, PREC_FP64, b, t, K.D, K.R, s);
    if (e != cudaSuccess) return e;
    const long long n = field_size(op);
    const long long nbnd = op.n_faces + op.nR[0] + op.nR[1] + op.nR[2];
    const double t1 = t + dt;
    k_field_lc<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(op, U, U, dt, K);
    k_update_boundary<<<(unsigned)std::max(1LL, (nbnd + 255) / 256), 256, 0, s>>>(
        op, dr, sp.sol, t1, sp.sol.kind == SOL_SINSIN ? std::exp(-t1) : 0.0, U);
    g_launches += 2;
    return cudaGetLastError();
}

cudaError_t launch_rhs(const DevOp& op, const SysParams& sp, int prec, const StepBuffers& b,
                       double t, double* out, double* const outR[3], cudaStream_t s)
{
    const dim3 grid = point_grid(op), block(32, BY);
    const double et = sp.sol.kind == SOL_SINSIN ? std::exp(-t) : 0.0;
    if (sp.kind == SYS_HEAT) {
        if (prec == PREC_FP64)
            k_rhs<SYS_HEAT, false><<<grid, block, 0, s>>>(op, sp, b.u0, b.R[0], b.R[1], b.R[2], t,
                                                          et, out);
        else
            k_rhs<SYS_HEAT, true><<<grid, block, 0, s>>>(op, sp, b.u0, b.R[0], b.R[1], b.R[2], t,
                                                         et, out);
    } else {
        if (prec == PREC_FP64)
            k_rhs<SYS_WAVE, false><<<grid, block, 0, s>>>(op, sp, b.u0, b.R[0], b.R[1], b.R[2], t,
                                                          et, out);
        else
            k_rhs<SYS_WAVE, true><<<grid, block, 0, s>>>(op, sp, b.u0, b.R[0], b.R[1], b.R[2], t,
                                                         et, out);
    }
    ++g_launches;
    // Dirichlet cut points carry a zero right-hand side (heat.cpp:269-284; the wave's gG
    // is zeroed there, scalar_wave.cpp:86-95)
    for (int d = 0; d < 3; d++)
        if (op.nR[d] && outR[d]) cudaMemsetAsync(outR[d], 0, op.nR[d] * sizeof(double), s);
    return cudaGetLastError();
}

cudaError_t launch_initialize(const DevOp& op, const DevR& dr, const DevSol& sol, int prec,
                              double t, void* u0, double* const R[3], cudaStream_t s)
{
    const dim3 grid = point_grid(op), block(32, BY);
    const double et = sol.kind == SOL_SINSIN ? std::exp(-t) : 0.0;
    k_init<<<grid, block, 0, s>>>(op, sol, t, et, prec == PREC_MIXED, u0);
    ++g_launches;
    for (int d = 0; d < 3; d++) {
        const int n = (int)op.nR[d];
        if (!n) continue;
        k_init_r<<<(n + 127) / 128, 128, 0, s>>>(dr, sol, n, d, t, et, R[d]);
        ++g_launches;
    }
    return cudaGetLastError();
}

cudaError_t launch_state_convert(long long n, int to_mixed, const double* in_d, void* out,
                                 const void* in_m, double* out_d, cudaStream_t s)
{
    const int bs = 256;
    const long long nb = (n + bs - 1) / bs;
    k_convert<<<(unsigned)nb, bs, 0, s>>>(n, to_mixed, in_d, (float*)out, (const float*)in_m,
                                          out_d);
    ++g_launches;
    return cudaGetLastError();
}

// errors at the non-Dirichlet cut points (compute_scalar_stats,
// src/systems/detail/scalar_system_utils.hpp:77-181): per axis (one block each) the largest
// |u - exact| with its first index, and the min / max of the values; out[4d..4d+3] =
// {err, index, min, max}, index -1 where the axis has no such point.  A non-finite value
// counts as an infinite error, as in the D statistics.
__global__ void __launch_bounds__(256) k_stats_r(DevOp op, DevR dr, DevSol sol, double t, double et,
                                                 const double* R0, const double* R1,
                                                 const double* R2, double* out)
{
    const int d = blockIdx.x;
    const double* R = d == 0 ? R0 : (d == 1 ? R1 : R2);
    const long long n = op.nR[d];
    double be = -1.0, vmin = 1.0 / 0.0, vmax = -1.0 / 0.0;
    long long bi = -1;
    for (long long i = threadIdx.x; i < n; i += blockDim.x) {
        if (dr.dirichlet[d][i]) continue;
        const double v = R[i];
        double e = fabs(v - sol_any(sol, t, et, dr.pos[d] + 3 * i, nullptr, d, i));
        if (!(e <= 1.0e300)) e = 1.0 / 0.0;
        if (e > be) { // i grows along the loop, so the first index of a tie is kept
            be = e;
            bi = i;
        }
        vmin = fmin(vmin, v);
        vmax = fmax(vmax, v);
    }
    __shared__ double se[256], smn[256], smx[256];
    __shared__ long long si[256];
    se[threadIdx.x] = be;
    si[threadIdx.x] = bi;
    smn[threadIdx.x] = vmin;
    smx[threadIdx.x] = vmax;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            const int o = threadIdx.x + w;
            if (si[o] >= 0 && (si[threadIdx.x] < 0 || se[o] > se[threadIdx.x] ||
                               (se[o] == se[threadIdx.x] && si[o] < si[threadIdx.x]))) {
                se[threadIdx.x] = se[o];
                si[threadIdx.x] = si[o];
            }
            smn[threadIdx.x] = fmin(smn[threadIdx.x], smn[o]);
            smx[threadIdx.x] = fmax(smx[threadIdx.x], smx[o]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[4 * d] = si[0] >= 0 ? se[0] : 0.0;
        out[4 * d + 1] = (double)si[0];
        out[4 * d + 2] = smn[0];
        out[4 * d + 3] = smx[0];
    }
}

cudaError_t launch_stats_r(const DevOp& op, const DevR& dr, const DevSol& sol, double* const R[3],
                           double t, double* out12, cudaStream_t s)
{
    const double et = sol.kind == SOL_SINSIN ? std::exp(-t) : 0.0;
    k_stats_r<<<3, 256, 0, s>>>(op, dr, sol, t, et, R[0], R[1], R[2], out12);
    ++g_launches;
    return cudaGetLastError();
}

// err <- |u - exact(t)| at the fluid D points and at the non-Dirichlet cut points, 0 on the
// Dirichlet faces, the solid points and the Dirichlet cut points: the "Error" field that
// write_scalar_error (src/systems/detail/scalar_system_utils.hpp:224-296) hands to the field
// writer.  u0 is the D state (FP64, or the FP32 hi/lo pair of a mixed system); R is the
// FP64 cut-point state (read only at non-Dirichlet cut points).
__global__ void __launch_bounds__(256) k_error_field(DevOp op, DevR dr, DevSol sol, double t, double et,
                                                     int mixed, const void* u0, const double* R0,
                                                     const double* R1, const double* R2, FieldF64 err)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long i = 0;
    const int part = field_part(op, g, i);
    if (part < 0) return;
    if (part == 0) {
        const unsigned c = op.cls[i];
        double e = 0.0;
        if ((c & CLS_FLUID) && !(c & CLS_DIRFACE)) {
            const double u = mixed ? ldd(PairU{(const float*)u0, op.N}, i) : ((const double*)u0)[i];
            int ijk[3];
            phys_of_point(op, i, ijk);
            e = fabs(u - sol_point_any(op, sol, t, et, ijk));
        }
        err.D[i] = e;
    } else {
        const int d = part - 1;
        const double* R = d == 0 ? R0 : (d == 1 ? R1 : R2);
        err.R[d][i] = dr.dirichlet[d][i]
                          ? 0.0
                          : fabs(R[i] - sol_any(sol, t, et, dr.pos[d] + 3 * i, nullptr, d, (int)i));
    }
}

cudaError_t launch_error_field(const DevOp& op, const DevR& dr, const DevSol& sol, int prec,
                               const void* u0, double* const R[3], double t, FieldF64 err,
                               cudaStream_t s)
{
    const long long n = op.N + op.nR[0] + op.nR[1] + op.nR[2];
    if (n == 0) return cudaSuccess;
    const double et = sol.kind == SOL_SINSIN ? std::exp(-t) : 0.0;
    k_error_field<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(op, dr, sol, t, et, prec == PREC_MIXED,
                                                             u0, R[0], R[1], R[2], err);
    ++g_launches;
    return cudaGetLastError();
}

cudaError_t launch_stats(const DevOp& op, const DevR&, const DevSol& sol, int prec,
                         const void* u0, double* const*, double t, double* dev_out,
                         cudaStream_t s)
{
    const dim3 grid = point_grid(op), block(32, BY);
    const long long nparts = (long long)grid.x * grid.y * grid.z;
    StatPart* parts = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&parts, nparts * sizeof(StatPart), s);
    if (e != cudaSuccess) return e;
    const double et = sol.kind == SOL_SINSIN ? std::exp(-t) : 0.0;
    k_stats<<<grid, block, 0, s>>>(op, sol, t, et, prec == PREC_MIXED, u0, parts);
    k_stats_final<<<1, 256, 0, s>>>(nparts, parts, dev_out);
    g_launches += 2;
    cudaFreeAsync(parts, s);
    return cudaGetLastError();
}

// ---- allocation-free statistics ------------------------------------------------------------
// Some callers cannot allocate device memory while they call in: an application that has
// handed the whole device memory to its own pool allocator, or a time loop that must never
// block in (or fail in) the CUDA allocator between its steps.  For them the statistics
// reduction can run out of one fixed scratch array that lives in the library's own device
// image: the per-tile partial results (one per 256-point tile, 4 doubles each) followed by
// the four results.  Every GPU that loads the library holds the array until the process
// exits.  All calls share it and it keeps the last call's contents; every slot a call
// reads is written earlier in the same call, so nothing has to be cleared first, but two
// calls that overlap on the GPU (different streams, or different host threads on one
// device) race on it.
namespace
{
constexpr long long STATS_NOALLOC_MAX_TILES = 65536; // 16.7 M points (256^3), 2 MB
static_assert(sizeof(StatPart) == 4 * sizeof(double), "StatPart is four 8-byte words");
static __device__ __align__(256) double g_stats_scratch[4 * STATS_NOALLOC_MAX_TILES + 4];

// device address of g_stats_scratch on each device, looked up once per device with that
// device current (in host code the array's name is a host-side stand-in, not a device
// address)
constexpr int MAX_DEVICES = 64;
double* g_scratch_addr[MAX_DEVICES] = {};
std::mutex g_scratch_mutex;
} // namespace

long long stats_noalloc_max_tiles() { return STATS_NOALLOC_MAX_TILES; }

cudaError_t launch_stats_noalloc(const DevOp& op, const DevSol& sol, int prec, const void* u0,
                                 double t, double host_out[4], cudaStream_t s)
{
    const dim3 grid = point_grid(op), block(32, BY);
    const long long nparts = (long long)grid.x * grid.y * grid.z;
    if (nparts > STATS_NOALLOC_MAX_TILES) return cudaErrorInvalidValue;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
    double* scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mutex);
        if (!g_scratch_addr[dev]) {
            void* ptr = nullptr;
            e = cudaGetSymbolAddress(&ptr, g_stats_scratch);
            if (e != cudaSuccess) return e;
            g_scratch_addr[dev] = static_cast<double*>(ptr);
        }
        scratch = g_scratch_addr[dev];
    }
    StatPart* parts = reinterpret_cast<StatPart*>(scratch);
    double* out = scratch + 4 * STATS_NOALLOC_MAX_TILES;
    const double et = sol.kind == SOL_SINSIN ? std::exp(-t) : 0.0;
    k_stats<<<grid, block, 0, s>>>(op, sol, t, et, prec == PREC_MIXED, u0, parts);
    k_stats_final<<<1, 256, 0, s>>>(nparts, parts, out);
    g_launches += 2;
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    e = cudaMemcpyAsync(host_out, out, 4 * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return e;
    return cudaStreamSynchronize(s);
}

// ===========================================================================================
// Batched heat solves (the manufactured sin-sin solution): many independent systems of
// different grids and cut geometries advance together, one launch per kernel kind and
// stage for the whole batch.  Boundary values are the solution's tables times e^{-t}, formed
// inline (RScaled, face values) rather than stored, with the same products the single-system
// path stores; the per-point stage bodies are the single-system ones, so every instance
// gets the bits it would get alone.
// ===========================================================================================
namespace
{
// cut-cell row g of the batch's row list; COH: inputs written earlier in the same launch
template <bool MIXED, int STAGE, bool COH>
__device__ __forceinline__ void batch_cut_row(const BatchInst* __restrict__ B,
                                              const int* __restrict__ row_inst, int g,
                                              const BatchTime* __restrict__ bt)
{
    const int ii = row_inst[g];
    const BatchInst& I = B[ii];
    const DevOp& op = I.op;
    const int i = g - I.row0;
    const int d = i < op.ax[1].row_base ? 0 : (i < op.ax[2].row_base ? 1 : 2);
    const DevAxis& A = op.ax[d];
    const int row = i - A.row_base;
    const long long p = A.row_out[row];
    const int tp = STAGE == 0 ? 0 : (STAGE == 3 ? 2 : 1); // R at t, t+dt/2, t+dt
    const RScaled R{I.sp.sol.SR[d], bt[ii].et[tp]};
    const void* in = STAGE == 0 ? I.u0 : (STAGE == 2 ? I.sb : I.sa);
    // compacted in row order (the per-point stage) and, for the 2-D stage, at the point
    if constexpr (MIXED) {
        float v;
        if constexpr (COH)
            v = STAGE == 0 ? closure_ff<CgPair, RScaled, 4>(A, row, p, CgPair{(const float*)in, op.N}, R)
                           : closure_ff<CgF, RScaled, 4>(A, row, p, CgF{(const float*)in}, R);
        else
            v = STAGE == 0 ? closure_ff(A, row, p, PairU{(const float*)in, op.N}, R)
                           : closure_ff(A, row, p, (const float*)in, R);
        ((float*)I.cval)[i] = v;
        if (I.rowv) ((float*)I.rowv)[(long long)d * op.N + p] = v;
    } else {
        double v;
        if constexpr (COH)
            v = closure64(A, row, p, CgD{(const double*)in}, R, (const double*)nullptr, 0.0, true);
        else
            v = closure64(A, row, p, (const double*)in, R, (const double*)nullptr, 0.0, true);
        ((double*)I.cval)[i] = v;
        if (I.rowv) ((double*)I.rowv)[(long long)d * op.N + p] = v;
    }
}

template <bool MIXED, int STAGE>
__global__ void __launch_bounds__(128) k_batch_cut_rows(const BatchInst* __restrict__ B,
                                                        const int* __restrict__ row_inst,
                                                        int n_rows, const BatchTime* __restrict__ bt)
{
    pdl_wait();
    pdl_trigger();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_rows) return;
    batch_cut_row<MIXED, STAGE, false>(B, row_inst, g, bt);
}

template <int STAGE, bool MIXED, int WARPS>
__global__ void __launch_bounds__(32 * WARPS) k_batch_stage(const BatchInst* __restrict__ B,
                                                            const int4* __restrict__ tiles,
                                                            int n_tiles,
                                                            const BatchTime* __restrict__ bt)
{
    pdl_wait();
    pdl_trigger();
    for (int T = blockIdx.x; T < n_tiles; T += gridDim.x) {
        const int4 tl = __ldg(tiles + T); // (instance, it0 index, first it1 index, it2 chunk)
        const BatchInst& I = B[tl.x];
        const DevOp& op = I.op;
        const int bx = tl.w;
        StagePt<int> q;
        q.c = bx * 32 + threadIdx.x;
        q.b = tl.z + threadIdx.y;
        q.a = tl.y;
        q.valid = (q.b < op.it1) && (q.c < op.it2);
        const int line = q.a * op.it1 + q.b;
        q.p = line * op.it2 + q.c;
        q.chunk = (long long)line * op.nzc + bx;
        const BatchTime& tm = bt[tl.x];
        const int ts = STAGE == 0 ? 0 : (STAGE == 3 ? 2 : 1); // stage time
        const int tn = STAGE < 2 ? 1 : 2;                      // time of the stage output
        StageArgs sa{};
        sa.u0 = I.u0;
        sa.acc = I.acc;
        sa.cval = I.cval;
        sa.s_in = STAGE == 0 ? I.u0 : (STAGE == 2 ? I.sb : I.sa);
        sa.s_out = STAGE == 1 ? I.sb : I.sa;
        sa.cf = I.cf[STAGE];
        sa.ci = I.ci[STAGE];
        sa.cf_ff = I.cf_ff[STAGE];
        sa.ci_ff = I.ci_ff[STAGE];
        sa.t_stage = tm.t[ts];
        sa.t_next = tm.t[tn];
        sa.et_stage = tm.et[ts];
        sa.et_next = tm.et[tn];
        sa.etf_stage = (float)tm.et[ts];
        if constexpr (MIXED)
            stage_mixed_at<STAGE, SYS_HEAT, int>(op, I.sp, sa, q);
        else
            stage64_at<STAGE, SYS_HEAT, int>(op, I.sp, sa, q);
        // Dirichlet faces: the exact value at the stage output's time
        if (q.valid && (op.cls[q.p] & CLS_DIRFACE)) {
            int ijk[3];
            stage_ijk(op, q, ijk);
            const double v = sol_at_point(op, I.sp.sol, sa.t_next, sa.et_next, ijk);
            if constexpr (!MIXED)
                ((double*)(STAGE == 3 ? sa.u0 : sa.s_out))[q.p] = v;
            else if constexpr (STAGE < 3)
                ((float*)sa.s_out)[q.p] = (float)v;
            else
                st_pair(sa.u0, op.N, q.p, ff_from_double(v));
        }
    }
}

// interior row of the FP64 path from register values, in interior_d's operation order
template <class AX>
__device__ __forceinline__ double interior_row64(const AX& A, double m2, double m1, double c0,
                                                double p1, double p2)
{
    if (A.width == 5) {
        if (A.antisym) return fma(A.ic[3], p1 - m1, A.ic[4] * (p2 - m2));
        double r = A.ic[0] * m2;
        r = fma(A.ic[1], m1, r);
        r = fma(A.ic[2], c0, r);
        r = fma(A.ic[3], p1, r);
        return fma(A.ic[4], p2, r);
    }
    double r = A.ic[0] * m1;
    r = fma(A.ic[1], c0, r);
    return fma(A.ic[2], p1, r);
}

// Batched stage of the 2-D heat instances (iteration space (1, n1, n2), it2 contiguous).  A
// warp takes BATCH2D_TILE consecutive points of one instance's flat array, BATCH2D_PPL per
// lane, running
// across the ends of the it2 lines: a point within two points of a line end has no interior
// row along it2, so the flat neighbours read for it there are never used, and every lane of
// the warp has work.  All of a lane's loads are issued before any class byte is decoded
// (coordinates clamped into the array); the instance's parameters are read once per warp
// tile.  Per point the arithmetic is the per-point stage body's, with the same helpers in the
// same order (interior_row / interior_row64, wall32 / wall64, rhs_mixed or the FP64 source,
// rk_mixed or the FP64 update, the exact face values), so every instance gets the bits a
// single-system solve gives it.  Cut-cell row values come from the dense per-point array
// (BatchInst::rowv) that k_batch_cut_rows fills.  No warp-collective operation is used, so
// lanes past an instance's last point simply skip the tile.
// One warp tile (instance, first point) of the flat 2-D batched stage, PPL points per lane
// in BATCH2D_TILE / (32 PPL) passes.  COH: the stage input and the cut-cell row values were written earlier in the
// same launch by other blocks (the persistent solve), so they are loaded from L2.
template <int STAGE, bool MIXED, bool COH, int PPL = BATCH2D_PPL>
__device__ __forceinline__ void batch2d_tile(const BatchInst* __restrict__ B, int2 tl,
                                             const BatchTime* __restrict__ bt, int lane)
{
    using T = typename std::conditional<MIXED, float, double>::type;
    const BatchInst& I = B[tl.x];
    const DevOp& op = I.op;
    const int n2 = op.it2, N = (int)op.N;
    const int da = op.phys_of_it[1], db = op.phys_of_it[2]; // physical axes of it1, it2
    const DevAxis& Aa = op.ax[da];
    const DevAxis& Ab = op.ax[db];
    const T* __restrict__ in = (const T*)(STAGE == 0 ? I.u0 : (STAGE == 2 ? I.sb : I.sa));
    auto cl = [N](int x) { return min(max(x, 0), N - 1); };
    auto LD = [in](int x) -> T { return COH ? __ldcg(in + x) : __ldg(in + x); };
    const BatchTime& tm = bt[tl.x];
    const int ts = STAGE == 0 ? 0 : (STAGE == 3 ? 2 : 1); // stage time
    const int tn = STAGE < 2 ? 1 : 2;                      // time of the stage output
    StageArgs sa{};
    sa.u0 = I.u0;
    sa.acc = I.acc;
    sa.s_out = STAGE == 1 ? I.sb : I.sa;
    sa.cf = I.cf[STAGE];
    sa.ci = I.ci[STAGE];
    sa.cf_ff = I.cf_ff[STAGE];
    sa.ci_ff = I.ci_ff[STAGE];
    sa.t_stage = tm.t[ts];
    sa.t_next = tm.t[tn];
    sa.et_stage = tm.et[ts];
    sa.et_next = tm.et[tn];
    sa.etf_stage = (float)tm.et[ts];
    const T* __restrict__ rowv = (const T*)I.rowv;
    auto RV = [rowv](long long x) -> T { return COH ? __ldcg(rowv + x) : rowv[x]; };
    // the parameters above are read once per tile
    for (int sub = 0; sub < BATCH2D_TILE / (32 * PPL); sub++) {
        const int p0 = tl.y + sub * (32 * PPL) + PPL * lane;
        if (p0 >= N) break;
        T wv[PPL + 4]; // it2 neighbours: points p0-2 .. p0+PPL+1
#pragma unroll
        for (int m = 0; m < PPL + 4; m++) wv[m] = LD(cl(p0 - 2 + m));
        T am2[PPL], am1[PPL], ap1[PPL], ap2[PPL]; // it1 neighbours
        unsigned c[PPL];
#pragma unroll
        for (int q = 0; q < PPL; q++) {
            const int p = p0 + q;
            am2[q] = LD(cl(p - 2 * n2));
            am1[q] = LD(cl(p - n2));
            ap1[q] = LD(cl(p + n2));
            ap2[q] = LD(cl(p + 2 * n2));
            c[q] = p < N ? (unsigned)op.cls[p] : 0u;
        }
        const int i0 = p0 / n2;
        int ja = i0, jb = p0 - i0 * n2; // iteration coordinates (it1, it2) of the point
#pragma unroll
        for (int q = 0; q < PPL; q++) {
            const int p = p0 + q;
            if (p >= N) break;
            if (q > 0 && ++jb == n2) {
                jb = 0;
                ++ja;
            }
            const unsigned ka = (c[q] >> (2 * da)) & 3u, kb = (c[q] >> (2 * db)) & 3u;
            T va = 0, vb = 0;
            if constexpr (MIXED) {
                if (ka == ROW_INTERIOR) va = interior_row(Aa, am2[q], am1[q], wv[q + 2], ap1[q], ap2[q]);
                if (kb == ROW_INTERIOR) vb = interior_row(Ab, wv[q], wv[q + 1], wv[q + 2], wv[q + 3], wv[q + 4]);
                if (ka == ROW_WALL) va = COH ? wall32(Aa, (long long)p, ja, CgF{(const float*)in}) : wall32(Aa, (long long)p, ja, in);
                if (kb == ROW_WALL) vb = COH ? wall32(Ab, (long long)p, jb, CgF{(const float*)in}) : wall32(Ab, (long long)p, jb, in);
            } else {
                if (ka == ROW_INTERIOR) va = interior_row64(Aa, am2[q], am1[q], wv[q + 2], ap1[q], ap2[q]);
                if (kb == ROW_INTERIOR) vb = interior_row64(Ab, wv[q], wv[q + 1], wv[q + 2], wv[q + 3], wv[q + 4]);
                if (ka == ROW_WALL)
                    va = COH ? wall64(Aa, (long long)p, ja, CgD{(const double*)in}, (const double*)nullptr, 0.0, true)
                             : wall64(Aa, (long long)p, ja, in, (const double*)nullptr, 0.0, true);
                if (kb == ROW_WALL)
                    vb = COH ? wall64(Ab, (long long)p, jb, CgD{(const double*)in}, (const double*)nullptr, 0.0, true)
                             : wall64(Ab, (long long)p, jb, in, (const double*)nullptr, 0.0, true);
            }
            if (ka == ROW_CLOSURE) va = RV((long long)da * N + p);
            if (kb == ROW_CLOSURE) vb = RV((long long)db * N + p);
            // physical coordinates (da < db; the third axis has extent 1)
            const int ijk[3] = {da == 0 ? ja : 0, da == 1 ? ja : (db == 1 ? jb : 0), db == 2 ? jb : 0};
            const bool face = (c[q] & CLS_DIRFACE) != 0;
            if constexpr (MIXED) {
                const float lap = __fadd_rn(__fadd_rn(0.f, va), vb);
                const float rhs = (c[q] & 0x3Fu) ? rhs_mixed<SYS_HEAT>(op, I.sp, sa.etf_stage, ijk[0],
                                                                      ijk[1], ijk[2], lap, 0.f, 0.f, 0.f)
                                                 : 0.f;
                float a_out = 0.f, s_out = 0.f;
                float2 u_out;
                rk_mixed<STAGE>(sa, rhs, ld_u0<STAGE>(I.u0, N, p),
                                STAGE == 0 ? 0.f : ((const float*)I.acc)[p], a_out, s_out, u_out);
                if (face) { // the exact value at the stage output's time
                    const double v = sol_at_point(op, I.sp.sol, sa.t_next, sa.et_next, ijk);
                    if constexpr (STAGE < 3)
                        s_out = (float)v;
                    else
                        u_out = ff_from_double(v);
                }
                if constexpr (STAGE < 3) {
                    ((float*)I.acc)[p] = a_out;
                    ((float*)sa.s_out)[p] = s_out;
                } else {
                    st_pair(I.u0, N, p, u_out);
                }
            } else {
                const double lap = (0.0 + va) + vb;
                double rhs = 0.0;
                if (c[q] & 0x3Fu) {
                    double src = 0.0;
                    if (I.sp.sol.kind == SOL_SINSIN) {
                        const double u = sol_at_point(op, I.sp.sol, sa.t_stage, sa.et_stage, ijk);
                        src = __dsub_rn(-u, __dmul_rn(I.sp.k, __dmul_rn(I.sp.sol.lapfac, u)));
                    }
                    rhs = fma(lap, I.sp.k, src);
                }
                double* __restrict__ u0 = (double*)I.u0;
                double* __restrict__ acc = (double*)I.acc;
                if constexpr (STAGE < 3) {
                    acc[p] = STAGE == 0 ? sa.cf * rhs : fma(sa.cf, rhs, acc[p]);
                    double so = fma(sa.ci, rhs, u0[p]);
                    if (face) so = sol_at_point(op, I.sp.sol, sa.t_next, sa.et_next, ijk);
                    ((double*)sa.s_out)[p] = so;
                } else {
                    double un = u0[p] + fma(sa.cf, rhs, acc[p]);
                    if (face) un = sol_at_point(op, I.sp.sol, sa.t_next, sa.et_next, ijk);
                    u0[p] = un;
                }
            }
        }
    }
}

template <int STAGE, bool MIXED>
__global__ void __launch_bounds__(128) k_batch_stage2d(const BatchInst* __restrict__ B,
                                                       const int2* __restrict__ wt, int n_wt,
                                                       const BatchTime* __restrict__ bt)
{
    pdl_wait();
    pdl_trigger();
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int w = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); w < n_wt; w += nwarps)
        batch2d_tile<STAGE, MIXED, false>(B, __ldg(wt + w), bt, lane);
}

// ---- split 2-D batched stage -------------------------------------------------------------
// The points of a 2-D instance fall in two sets.  Uniform points have along each axis an
// interior row or no row and are not on a Dirichlet face: their update is the same short
// branch-free sequence everywhere.  Special points (a domain-wall or cut-cell row along
// either axis, or a Dirichlet face) take the general path, each on a thread of its own, with
// the cut-cell rows evaluated at the point (no separate row pass).  Warp tiles of
// BATCH2D_TILE consecutive points cover every point and write the uniform ones; a list of
// special points (instance, point, cut-cell row along it1, along it2) covers the rest.
// Every value is formed by the same helpers, in the same order, as in the single-system
// stage, so each instance gets its bits.

// the interior fields of an axis in registers
struct IRow {
    int width, antisym;
    float icf[5];
    double ic[5];
};
__device__ __forceinline__ IRow irow_of(const DevAxis& A)
{
    IRow r;
    r.width = A.width;
    r.antisym = A.antisym;
#pragma unroll
    for (int m = 0; m < 5; m++) {
        r.icf[m] = A.icf[m];
        r.ic[m] = A.ic[m];
    }
    return r;
}
// values a, b, t at the physical axes da < db and the third axis 3 - da - db, in physical order
template <class T>
__device__ __forceinline__ void phys_order(int dt3, T a, T b, T t, T& s0, T& s1, T& s2)
{
    s0 = dt3 == 0 ? t : a;
    s1 = dt3 == 0 ? a : (dt3 == 1 ? t : b);
    s2 = dt3 == 2 ? t : b;
}

// What a point update reads of its instance, loaded once per tile or point: the update's
// stores could alias the instance record as far as the compiler knows, so fields read after
// a store would be re-loaded.
template <int STAGE, bool MIXED>
struct BatchPt {
    using T = typename std::conditional<MIXED, float, double>::type;
    int N, n2, da, db, dt3;
    bool sinsin, d3;
    const float* Sfa;
    const float* Sfb;
    float Sft;
    const double* Sda;
    const double* Sdb;
    double Sdt;
    float kf, lapff;
    double kd, lapfac;
    double et_stage, et_next;
    void* u0;
    T* acc;
    T* sout;
    StageArgs sa;
};
template <int STAGE, bool MIXED>
__device__ __forceinline__ BatchPt<STAGE, MIXED> batch_pt_of(const BatchInst& I, const BatchTime& tm)
{
    using T = typename BatchPt<STAGE, MIXED>::T;
    BatchPt<STAGE, MIXED> P;
    const DevOp& op = I.op;
    P.N = (int)op.N;
    P.n2 = op.it2;
    P.da = op.phys_of_it[1];
    P.db = op.phys_of_it[2];
    P.dt3 = 3 - P.da - P.db;
    const DevSol& sol = I.sp.sol;
    P.sinsin = sol.kind == SOL_SINSIN;
    P.d3 = sol.dims == 3;
    const bool need_t = P.sinsin && (P.dt3 < 2 || P.d3);
    P.Sfa = sol.Sf[P.da];
    P.Sfb = sol.Sf[P.db];
    P.Sft = MIXED && need_t ? sol.Sf[P.dt3][0] : 0.f;
    P.Sda = sol.S[P.da];
    P.Sdb = sol.S[P.db];
    P.Sdt = need_t ? sol.S[P.dt3][0] : 0.0;
    P.kf = I.sp.kf;
    P.lapff = (float)sol.lapfac;
    P.kd = I.sp.k;
    P.lapfac = sol.lapfac;
    const int ts = STAGE == 0 ? 0 : (STAGE == 3 ? 2 : 1); // stage time
    const int tn = STAGE < 2 ? 1 : 2;                      // time of the stage output
    P.et_stage = tm.et[ts];
    P.et_next = tm.et[tn];
    P.u0 = I.u0;
    P.acc = (T*)I.acc;
    P.sout = (T*)(STAGE == 1 ? I.sb : I.sa);
    P.sa = StageArgs{};
    P.sa.cf = I.cf[STAGE];
    P.sa.ci = I.ci[STAGE];
    P.sa.cf_ff = I.cf_ff[STAGE];
    P.sa.ci_ff = I.ci_ff[STAGE];
    P.sa.etf_stage = (float)tm.et[ts];
    return P;
}

// the update of point p = (ia, ib) from its two axis values: right-hand side, RK4 stage,
// the exact value on a Dirichlet face, stores
template <int STAGE, bool MIXED, int DA = -1, int DB = -1>
__device__ __forceinline__ void batch_point_update(const BatchPt<STAGE, MIXED>& P, int p, int ia,
                                                   int ib, unsigned c,
                                                   typename BatchPt<STAGE, MIXED>::T va,
                                                   typename BatchPt<STAGE, MIXED>::T vb)
{
    const int dt3 = DA >= 0 ? 3 - DA - DB : P.dt3, db = DB >= 0 ? DB : P.db;
    const bool face = (c & CLS_DIRFACE) != 0;
    auto face_value = [&]() {
        double s0, s1, s2;
        phys_order(dt3, P.Sda[ia], P.d3 || db < 2 ? P.Sdb[ib] : 0.0, P.Sdt, s0, s1, s2);
        return sinsin_value(s0, s1, s2, P.d3, P.et_next);
    };
    if constexpr (MIXED) {
        const float lap = __fadd_rn(__fadd_rn(0.f, va), vb);
        float rhs = 0.f;
        if (c & 0x3Fu) {
            float src = 0.f;
            if (P.sinsin) {
                float s0, s1, s2;
                phys_order(dt3, P.Sfa[ia], P.d3 || db < 2 ? P.Sfb[ib] : 0.f, P.Sft, s0, s1, s2);
                src = sinsin_heat_src_f(s0, s1, s2, P.d3, P.sa.etf_stage, P.kf, P.lapff);
            }
            rhs = fmaf(lap, P.kf, src);
        }
        float a_out = 0.f, s_out = 0.f;
        float2 u_out;
        rk_mixed<STAGE>(P.sa, rhs, ld_u0<STAGE>(P.u0, P.N, p), STAGE == 0 ? 0.f : P.acc[p], a_out,
                        s_out, u_out);
        if (face) {
            const double v = P.sinsin ? face_value() : 0.0;
            if constexpr (STAGE < 3)
                s_out = (float)v;
            else
                u_out = ff_from_double(v);
        }
        if constexpr (STAGE < 3) {
            P.acc[p] = a_out;
            P.sout[p] = s_out;
        } else {
            st_pair(P.u0, P.N, p, u_out);
        }
    } else {
        const double lap = (0.0 + va) + vb;
        double rhs = 0.0;
        if (c & 0x3Fu) {
            double src = 0.0;
            if (P.sinsin) {
                double s0, s1, s2;
                phys_order(dt3, P.Sda[ia], P.d3 || db < 2 ? P.Sdb[ib] : 0.0, P.Sdt, s0, s1, s2);
                const double u = sinsin_value(s0, s1, s2, P.d3, P.et_stage);
                src = __dsub_rn(-u, __dmul_rn(P.kd, __dmul_rn(P.lapfac, u)));
            }
            rhs = fma(lap, P.kd, src);
        }
        double* const ud = (double*)P.u0;
        if constexpr (STAGE < 3) {
            P.acc[p] = STAGE == 0 ? P.sa.cf * rhs : fma(P.sa.cf, rhs, P.acc[p]);
            double so = fma(P.sa.ci, rhs, ud[p]);
            if (face) so = P.sinsin ? face_value() : 0.0;
            P.sout[p] = so;
        } else {
            double un = ud[p] + fma(P.sa.cf, rhs, P.acc[p]);
            if (face) un = P.sinsin ? face_value() : 0.0;
            ud[p] = un;
        }
    }
}

// BATCH2D_TILE consecutive points of one instance, BATCH2D_PPL per lane; writes the uniform
// points only.  DA, DB: the physical axes of it1, it2 when known at compile time (-1: read
// from the instance).  CLAMP: neighbour loads that may fall outside the grid are clamped
// into it (their values reach only points that are not written); tiles at least two it1
// lines away from both ends of the grid load without clamping.  COH: inputs written
// earlier in the same launch.
template <int STAGE, bool MIXED, bool COH, int DA, int DB, bool CLAMP>
__device__ __forceinline__ void uniform_tile_body(const BatchInst& I,
                                                  const BatchPt<STAGE, MIXED>& P, int2 tl, int lane)
{
    using T = typename std::conditional<MIXED, float, double>::type;
    constexpr int PPL = BATCH2D_PPL;
    const DevOp& op = I.op;
    const int da = DA >= 0 ? DA : P.da, db = DB >= 0 ? DB : P.db;
    const IRow ra = irow_of(op.ax[da]), rb = irow_of(op.ax[db]);
    const uint8_t* __restrict__ cls = op.cls;
    const T* __restrict__ in = (const T*)(STAGE == 0 ? I.u0 : (STAGE == 2 ? I.sb : I.sa));
    const int N = P.n2 * op.it1, n2 = P.n2;
    auto LD = [in, N](int x) -> T {
        if (CLAMP) x = min(max(x, 0), N - 1);
        return COH ? __ldcg(in + x) : __ldg(in + x);
    };
    const int p0 = tl.y + PPL * lane;
    if (CLAMP && p0 >= N) return;
    T wv[PPL + 4]; // it2 neighbours: points p0-2 .. p0+PPL+1
#pragma unroll
    for (int m = 0; m < PPL + 4; m++) wv[m] = LD(p0 - 2 + m);
    T am2[PPL], am1[PPL], ap1[PPL], ap2[PPL]; // it1 neighbours
    unsigned c[PPL];
#pragma unroll
    for (int q = 0; q < PPL; q++) {
        const int p = p0 + q;
        am2[q] = LD(p - 2 * n2);
        am1[q] = LD(p - n2);
        ap1[q] = LD(p + n2);
        ap2[q] = LD(p + 2 * n2);
        c[q] = !CLAMP || p < N ? (unsigned)cls[p] : 0u;
    }
    const int i0 = p0 / n2;
    int ia = i0, ib = p0 - i0 * n2; // iteration coordinates (it1, it2) of the point
#pragma unroll
    for (int q = 0; q < PPL; q++) {
        const int p = p0 + q;
        if (CLAMP && p >= N) break;
        if (q > 0 && ++ib == n2) {
            ib = 0;
            ++ia;
        }
        const unsigned ka = (c[q] >> (2 * da)) & 3u, kb = (c[q] >> (2 * db)) & 3u;
        if (ka >= ROW_CLOSURE || kb >= ROW_CLOSURE || (c[q] & CLS_DIRFACE)) continue;
        T va = 0, vb = 0;
        if constexpr (MIXED) {
            if (ka == ROW_INTERIOR) va = interior_row(ra, am2[q], am1[q], wv[q + 2], ap1[q], ap2[q]);
            if (kb == ROW_INTERIOR) vb = interior_row(rb, wv[q], wv[q + 1], wv[q + 2], wv[q + 3], wv[q + 4]);
        } else {
            if (ka == ROW_INTERIOR) va = interior_row64(ra, am2[q], am1[q], wv[q + 2], ap1[q], ap2[q]);
            if (kb == ROW_INTERIOR) vb = interior_row64(rb, wv[q], wv[q + 1], wv[q + 2], wv[q + 3], wv[q + 4]);
        }
        batch_point_update<STAGE, MIXED, DA, DB>(P, p, ia, ib, c[q], va, vb);
    }
}

// four consecutive floats at p (a multiple of four points from a field's start): one float4
// access when the field is 16-byte aligned (`al`, warp-uniform), else four scalar ones
template <bool COH>
__device__ __forceinline__ float4 ld_quad(const float* p, bool al)
{
    if (al) return COH ? __ldcg((const float4*)p) : __ldg((const float4*)p);
    if (COH) return make_float4(__ldcg(p), __ldcg(p + 1), __ldcg(p + 2), __ldcg(p + 3));
    return make_float4(__ldg(p), __ldg(p + 1), __ldg(p + 2), __ldg(p + 3));
}
// the same for a field this thread wrote itself (plain loads)
__device__ __forceinline__ float4 ld_quad_own(const float* p, bool al)
{
    if (al) return *(const float4*)p;
    return make_float4(p[0], p[1], p[2], p[3]);
}
__device__ __forceinline__ void st_quad(float* p, bool al, float4 v)
{
    if (al) {
        *(float4*)p = v;
    } else {
        p[0] = v.x;
        p[1] = v.y;
        p[2] = v.z;
        p[3] = v.w;
    }
}
__device__ __forceinline__ bool al16(const void* p) { return ((unsigned long long)p & 15u) == 0; }

// The mixed uniform tile in the x-y plane (sin-sin solution), away from the grid's first and
// last two lines: four consecutive points per lane (a quad starting at a multiple of four),
// each field read and written as float4 where it is 16-byte aligned, and the source's
// spatial factor read from the instance's product table s2f.  A quad whose four points are uniform is
// stored whole, any other point by point (the special points are written by the other
// kernel).
template <int STAGE, bool COH, bool SYM5>
__device__ __forceinline__ void uniform_quads_xy(const BatchInst& I, const BatchPt<STAGE, true>& P,
                                                 int2 tl, int lane)
{
    const DevOp& op = I.op;
    const IRow ra = irow_of(op.ax[0]), rb = irow_of(op.ax[1]);
    // the interior rows: five-point symmetric ones (E4_2) inline, any other through interior_row
    auto row = [](const IRow& r, float m2, float m1, float c0, float p1, float p2) {
        return SYM5 ? sym5(r.icf[1], r.icf[0], m2, m1, c0, p1, p2) : interior_row(r, m2, m1, c0, p1, p2);
    };
    const float* __restrict__ in = (const float*)(STAGE == 0 ? I.u0 : (STAGE == 2 ? I.sb : I.sa));
    const int n2 = P.n2, N = P.N;
    float* const hi = (float*)P.u0;
    float* const lo = hi + N;
    const bool ain = al16(in), a1 = ain && (n2 & 3) == 0, aout = al16(P.sout), alo = al16(lo);
#pragma unroll 1
    for (int pass = 0; pass < BATCH_UTILE / 128; pass++) {
        const int p0 = tl.y + pass * 128 + 4 * lane;
        const float4 cw = ld_quad<COH>(in + p0, ain);
        const float4 lw = ld_quad<COH>(in + p0 - 4, ain), rw = ld_quad<COH>(in + p0 + 4, ain);
        const float4 m2 = ld_quad<COH>(in + p0 - 2 * n2, a1), m1 = ld_quad<COH>(in + p0 - n2, a1);
        const float4 q1 = ld_quad<COH>(in + p0 + n2, a1), q2 = ld_quad<COH>(in + p0 + 2 * n2, a1);
        const unsigned c4 = __ldg((const unsigned*)(op.cls + p0));
        const float4 acc4 = STAGE == 0 ? make_float4(0.f, 0.f, 0.f, 0.f) : ld_quad_own(P.acc + p0, true);
        const float4 uh4 = STAGE == 0 ? cw : ld_quad_own(hi + p0, true);
        float4 ul4 = make_float4(0.f, 0.f, 0.f, 0.f);
        if constexpr (STAGE == 3) ul4 = ld_quad_own(lo + p0, alo);
        const float wv[8] = {lw.z, lw.w, cw.x, cw.y, cw.z, cw.w, rw.x, rw.y};
        const float am2[4] = {m2.x, m2.y, m2.z, m2.w}, am1[4] = {m1.x, m1.y, m1.z, m1.w};
        const float ap1[4] = {q1.x, q1.y, q1.z, q1.w}, ap2[4] = {q2.x, q2.y, q2.z, q2.w};
        const float av[4] = {acc4.x, acc4.y, acc4.z, acc4.w};
        const float uh[4] = {uh4.x, uh4.y, uh4.z, uh4.w}, ul[4] = {ul4.x, ul4.y, ul4.z, ul4.w};
        const float4 s24 = __ldg((const float4*)(I.s2f + p0));
        const float s2[4] = {s24.x, s24.y, s24.z, s24.w};
        float ao[4], so[4];
        float2 uo[4];
        unsigned wmask = 0;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const unsigned c = (c4 >> (8 * q)) & 0xFFu;
            const unsigned ka = c & 3u, kb = (c >> 2) & 3u;
            ao[q] = so[q] = 0.f;
            uo[q] = make_float2(0.f, 0.f);
            if (ka >= ROW_CLOSURE || kb >= ROW_CLOSURE || (c & CLS_DIRFACE)) continue;
            wmask |= 1u << q;
            float va = 0.f, vb = 0.f;
            if (ka == ROW_INTERIOR) va = row(ra, am2[q], am1[q], wv[q + 2], ap1[q], ap2[q]);
            if (kb == ROW_INTERIOR) vb = row(rb, wv[q], wv[q + 1], wv[q + 2], wv[q + 3], wv[q + 4]);
            const float lap = __fadd_rn(__fadd_rn(0.f, va), vb);
            float rhs = 0.f;
            if (c & 0x3Fu)
                rhs = fmaf(lap, P.kf, sinsin_heat_src_p(s2[q], 0.f, false, P.sa.etf_stage, P.kf, P.lapff));
            rk_mixed<STAGE>(P.sa, rhs, make_float2(uh[q], ul[q]), av[q], ao[q], so[q], uo[q]);
        }
        if (wmask == 15u) {
            if constexpr (STAGE < 3) {
                st_quad(P.acc + p0, true, make_float4(ao[0], ao[1], ao[2], ao[3]));
                st_quad(P.sout + p0, aout, make_float4(so[0], so[1], so[2], so[3]));
            } else {
                st_quad(hi + p0, true, make_float4(uo[0].x, uo[1].x, uo[2].x, uo[3].x));
                st_quad(lo + p0, alo, make_float4(uo[0].y, uo[1].y, uo[2].y, uo[3].y));
            }
        } else {
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (wmask >> q & 1u) {
                    if constexpr (STAGE < 3) {
                        P.acc[p0 + q] = ao[q];
                        P.sout[p0 + q] = so[q];
                    } else {
                        hi[p0 + q] = uo[q].x;
                        lo[p0 + q] = uo[q].y;
                    }
                }
        }
    }
}

template <int STAGE, bool MIXED, bool COH>
__device__ __forceinline__ void batch_uniform_tile(const BatchInst* __restrict__ B, int2 tl,
                                                   const BatchTime* __restrict__ bt, int lane)
{
    const BatchInst& I = B[tl.x];
    const BatchPt<STAGE, MIXED> P = batch_pt_of<STAGE, MIXED>(I, bt[tl.x]);
    const int N = P.n2 * I.op.it1, n2 = P.n2;
    // the x-y plane (the batched configuration's instances), away from the first and last
    // two lines: no clamping, and quads in the mixed path
    if (MIXED && I.s2f && P.da == 0 && P.db == 1 && tl.y >= 2 * n2 && tl.y + BATCH_UTILE + 2 * n2 <= N) {
        if constexpr (MIXED) {
            const DevAxis& A0 = I.op.ax[0];
            const DevAxis& A1 = I.op.ax[1];
            if (A0.width == 5 && !A0.antisym && A1.width == 5 && !A1.antisym)
                uniform_quads_xy<STAGE, COH, true>(I, P, tl, lane);
            else
                uniform_quads_xy<STAGE, COH, false>(I, P, tl, lane);
        }
        return;
    }
#pragma unroll 1
    for (int pass = 0; pass < BATCH_UTILE / BATCH2D_TILE; pass++) {
        const int2 t = make_int2(tl.x, tl.y + pass * BATCH2D_TILE);
        if (t.y >= N) return;
        if (P.da == 0 && P.db == 1) {
            if (t.y >= 2 * n2 && t.y + BATCH2D_TILE + 2 * n2 <= N)
                uniform_tile_body<STAGE, MIXED, COH, 0, 1, false>(I, P, t, lane);
            else
                uniform_tile_body<STAGE, MIXED, COH, 0, 1, true>(I, P, t, lane);
        } else {
            uniform_tile_body<STAGE, MIXED, COH, -1, -1, true>(I, P, t, lane);
        }
    }
}

// one special point: item (instance, point, cut-cell row along it1, along it2; -1 for none)
template <int STAGE, bool MIXED, bool COH>
__device__ __forceinline__ void batch_special_point(const BatchInst* __restrict__ B, int4 it,
                                                    const BatchTime* __restrict__ bt)
{
    using T = typename std::conditional<MIXED, float, double>::type;
    const BatchInst& I = B[it.x];
    const DevOp& op = I.op;
    const BatchTime& tm = bt[it.x];
    const BatchPt<STAGE, MIXED> P = batch_pt_of<STAGE, MIXED>(I, tm);
    const int p = it.y, n2 = P.n2;
    const int ia = p / n2, ib = p - ia * n2;
    const T* __restrict__ in = (const T*)(STAGE == 0 ? I.u0 : (STAGE == 2 ? I.sb : I.sa));
    const unsigned c = op.cls[p];
    // R at the stage time (t, t + dt/2, t + dt), as the cut-cell row pass forms it
    const double etR = tm.et[STAGE == 0 ? 0 : (STAGE == 3 ? 2 : 1)];
    T v[2];
#pragma unroll
    for (int a = 0; a < 2; a++) {
        const int d = a == 0 ? P.da : P.db;
        const DevAxis& A = op.ax[d];
        const unsigned k = (c >> (2 * d)) & 3u;
        const int coord = a == 0 ? ia : ib;
        const int s = a == 0 ? n2 : 1;
        T x = 0;
        if (k == ROW_INTERIOR) {
            auto L = [&](int q) -> T { return COH ? __ldcg(in + q) : __ldg(in + q); };
            if constexpr (MIXED)
                x = interior_row(A, L(p - 2 * s), L(p - s), L(p), L(p + s), L(p + 2 * s));
            else
                x = interior_row64(A, L(p - 2 * s), L(p - s), L(p), L(p + s), L(p + 2 * s));
        } else if (k == ROW_WALL) {
            if constexpr (MIXED)
                x = COH ? wall32(A, (long long)p, coord, CgF{(const float*)in}) : wall32(A, (long long)p, coord, in);
            else
                x = COH ? wall64(A, (long long)p, coord, CgD{(const double*)in}, (const double*)nullptr, 0.0, true)
                        : wall64(A, (long long)p, coord, in, (const double*)nullptr, 0.0, true);
        } else if (k == ROW_CLOSURE) {
            const int row = a == 0 ? it.z : it.w;
            const RScaled R{I.sp.sol.SR[d], etR};
            if constexpr (MIXED) {
                if constexpr (COH)
                    x = STAGE == 0 ? closure_ff<CgPair, RScaled, 4>(A, row, p, CgPair{(const float*)in, op.N}, R)
                                   : closure_ff<CgF, RScaled, 4>(A, row, p, CgF{(const float*)in}, R);
                else
                    x = STAGE == 0 ? closure_ff(A, row, p, PairU{(const float*)in, op.N}, R)
                                   : closure_ff(A, row, p, (const float*)in, R);
            } else {
                if constexpr (COH)
                    x = closure64(A, row, p, CgD{(const double*)in}, R, (const double*)nullptr, 0.0, true);
                else
                    x = closure64(A, row, p, (const double*)in, R, (const double*)nullptr, 0.0, true);
            }
        }
        v[a] = x;
    }
    batch_point_update<STAGE, MIXED>(P, p, ia, ib, c, v[0], v[1]);
}

// one stage of the split form: the uniform tiles (a warp each) and the special points (a
// thread each), two kernels with disjoint outputs that may run concurrently
// (mixed: 64 registers, measured faster than the unbounded 80-94 at 128-point tiles)
template <int STAGE, bool MIXED>
__global__ void __launch_bounds__(128, MIXED ? 8 : 1) k_batch_uniform(const BatchInst* __restrict__ B,
                                                       const int2* __restrict__ ut, int n_ut,
                                                       const BatchTime* __restrict__ bt)
{
    pdl_wait();
    pdl_trigger();
    const int w = (int)blockIdx.x * 4 + (int)(threadIdx.x >> 5);
    if (w < n_ut) batch_uniform_tile<STAGE, MIXED, false>(B, __ldg(ut + w), bt, threadIdx.x & 31);
}

template <int STAGE, bool MIXED>
__global__ void __launch_bounds__(128) k_batch_special(const BatchInst* __restrict__ B,
                                                       const int4* __restrict__ sp, int n_sp,
                                                       const BatchTime* __restrict__ bt)
{
    pdl_wait();
    pdl_trigger();
    const int g = blockIdx.x * 128 + threadIdx.x;
    if (g < n_sp) batch_special_point<STAGE, MIXED, false>(B, __ldg(sp + g), bt);
}

// ---- the whole batched solve in one persistent launch -------------------------------------
// Thread-block clusters of BATCH_CLUSTER blocks; each cluster owns a set of whole instances
// (ctab[c] = its ranges of the special-point list psp and of the uniform-tile list put, the
// instances balanced over the clusters by their work).  A cluster runs every RK4 step of its
// instances, a stage at a time with a cluster barrier after each.  Instances are independent,
// so no block ever waits for another cluster; the barrier is the hardware cluster barrier
// (release / acquire at cluster scope), which every block reaches the same number of times.
// Inputs written by other blocks of the cluster are loaded from L2 (the COH forms); the
// arithmetic is the split stage's, so each instance gets the single-system bits.
template <int STAGE, bool MIXED>
__device__ __forceinline__ void persist_stage(cg::cluster_group& cl, const BatchInst* __restrict__ B,
                                              const int4* __restrict__ psp,
                                              const int2* __restrict__ put, int4 W,
                                              const BatchTime* __restrict__ bt, int tid, int nth,
                                              int warp, int nwarp, int lane)
{
#pragma unroll 1
    for (int g = W.x + tid; g < W.y; g += nth) batch_special_point<STAGE, MIXED, true>(B, __ldg(psp + g), bt);
#pragma unroll 1
    for (int w = W.z + warp; w < W.w; w += nwarp) batch_uniform_tile<STAGE, MIXED, true>(B, __ldg(put + w), bt, lane);
    cl.sync();
}

template <bool MIXED>
__global__ void __launch_bounds__(256, 2) k_batch_persist(const BatchInst* __restrict__ B,
                                                          const int4* __restrict__ psp,
                                                          const int2* __restrict__ put,
                                                          const int4* __restrict__ ctab,
                                                          const BatchTime* __restrict__ times,
                                                          int n_inst, int nsteps)
{
    cg::cluster_group cl = cg::this_cluster();
    const int cs = (int)cl.num_blocks();
    const int4 W = __ldg(ctab + blockIdx.x / cs);
    const int tid = (int)cl.block_rank() * blockDim.x + threadIdx.x, nth = cs * blockDim.x;
    const int lane = threadIdx.x & 31, warp = tid >> 5, nwarp = nth >> 5;
#pragma unroll 1
    for (int k = 0; k < nsteps; k++) {
        const BatchTime* bt = times + (long long)k * n_inst;
        persist_stage<0, MIXED>(cl, B, psp, put, W, bt, tid, nth, warp, nwarp, lane);
        persist_stage<1, MIXED>(cl, B, psp, put, W, bt, tid, nth, warp, nwarp, lane);
        persist_stage<2, MIXED>(cl, B, psp, put, W, bt, tid, nth, warp, nwarp, lane);
        persist_stage<3, MIXED>(cl, B, psp, put, W, bt, tid, nth, warp, nwarp, lane);
    }
}

__global__ void k_sinsin_xy(const float* __restrict__ sx, const float* __restrict__ sy, int n1,
                            int n2, float* __restrict__ out)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n1 * n2) return;
    const int i = p / n2;
    out[p] = __fmul_rn(sx[i], sy[p - i * n2]);
}

__global__ void k_batch_finish(const BatchInst* __restrict__ B, const BatchTime* __restrict__ last,
                               const int* __restrict__ r_inst, int n_r)
{
    // r_inst: instance of each cut point of the batch, axis-major within an instance
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_r) return;
    const int ii = r_inst[3 * g], d = r_inst[3 * g + 1], k = r_inst[3 * g + 2];
    const BatchInst& I = B[ii];
    I.R[d][k] = __ldg(I.sp.sol.SR[d] + k) * last[ii].et[2];
}

template <int STAGE, bool MIXED>
void batch_stage(const BatchInst* inst, const int4* tiles, int n_tiles, int cfg, int grid,
                 const BatchTime* times, cudaStream_t s)
{
    switch (cfg) {
    case 0: k_batch_stage<STAGE, MIXED, 1><<<grid, dim3(32, 1), 0, s>>>(inst, tiles, n_tiles, times); break;
    case 1: k_batch_stage<STAGE, MIXED, 2><<<grid, dim3(32, 2), 0, s>>>(inst, tiles, n_tiles, times); break;
    case 2: k_batch_stage<STAGE, MIXED, 4><<<grid, dim3(32, 4), 0, s>>>(inst, tiles, n_tiles, times); break;
    default: k_batch_stage<STAGE, MIXED, 8><<<grid, dim3(32, 8), 0, s>>>(inst, tiles, n_tiles, times); break;
    }
    ++g_launches;
}

template <int STAGE, bool MIXED>
void batch_stage_all(const BatchInst* inst, const int* row_inst, int n_rows, const int4* tiles,
                     int n_tiles, int cfg, int grid, const int2* wt, int n_wt, int grid2d,
                     const BatchSplit& sp, const BatchTime* times, cudaStream_t s)
{
    if (n_rows) {
        k_batch_cut_rows<MIXED, STAGE><<<(n_rows + 127) / 128, 128, 0, s>>>(inst, row_inst, n_rows, times);
        ++g_launches;
    }
    if (n_tiles) batch_stage<STAGE, MIXED>(inst, tiles, n_tiles, cfg, grid, times, s);
    if (n_wt) {
        k_batch_stage2d<STAGE, MIXED><<<grid2d, 128, 0, s>>>(inst, wt, n_wt, times);
        ++g_launches;
    }
    // the special points on a forked stream (a parallel branch when captured), the uniform
    // tiles on s; s waits for both
    const bool fork = sp.n_sp && sp.n_ut && sp.aux;
    cudaStream_t ss = fork ? sp.aux : s;
    if (fork) {
        cudaEventRecord(sp.fork, s);
        cudaStreamWaitEvent(sp.aux, sp.fork, 0);
    }
    if (sp.n_sp) {
        k_batch_special<STAGE, MIXED><<<(sp.n_sp + 127) / 128, 128, 0, ss>>>(inst, sp.sp, sp.n_sp, times);
        ++g_launches;
    }
    if (sp.n_ut) {
        k_batch_uniform<STAGE, MIXED><<<(sp.n_ut + 3) / 4, 128, 0, s>>>(inst, sp.ut, sp.n_ut, times);
        ++g_launches;
    }
    if (fork) {
        cudaEventRecord(sp.join, sp.aux);
        cudaStreamWaitEvent(s, sp.join, 0);
    }
}

template <bool MIXED>
void batch_step(const BatchInst* inst, const int* row_inst, int n_rows, const int4* tiles,
                int n_tiles, int cfg, int grid, const int2* wt, int n_wt, int grid2d,
                const BatchSplit& sp, const BatchTime* times, cudaStream_t s)
{
    batch_stage_all<0, MIXED>(inst, row_inst, n_rows, tiles, n_tiles, cfg, grid, wt, n_wt, grid2d, sp, times, s);
    batch_stage_all<1, MIXED>(inst, row_inst, n_rows, tiles, n_tiles, cfg, grid, wt, n_wt, grid2d, sp, times, s);
    batch_stage_all<2, MIXED>(inst, row_inst, n_rows, tiles, n_tiles, cfg, grid, wt, n_wt, grid2d, sp, times, s);
    batch_stage_all<3, MIXED>(inst, row_inst, n_rows, tiles, n_tiles, cfg, grid, wt, n_wt, grid2d, sp, times, s);
}
} // namespace

cudaError_t launch_batch_step(const BatchInst* inst, const int* row_inst, int n_rows,
                              const int4* tiles, int n_tiles, int tile_cfg, int grid,
                              const int2* wtiles, int n_wtiles, int grid2d, const BatchSplit& sp,
                              const BatchTime* times, int prec, cudaStream_t s)
{
    if (prec == PREC_MIXED)
        batch_step<true>(inst, row_inst, n_rows, tiles, n_tiles, tile_cfg, grid, wtiles, n_wtiles,
                         grid2d, sp, times, s);
    else
        batch_step<false>(inst, row_inst, n_rows, tiles, n_tiles, tile_cfg, grid, wtiles, n_wtiles,
                          grid2d, sp, times, s);
    return cudaGetLastError();
}

namespace
{
template <bool MIXED>
cudaLaunchConfig_t persist_config(int n_clusters, cudaStream_t s, cudaLaunchAttribute* at)
{
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(n_clusters * BATCH_CLUSTER);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = BATCH_CLUSTER;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cfg;
}
} // namespace

int batch_persist_clusters(int prec)
{
    cudaLaunchAttribute at[1];
    int n = 0;
    cudaError_t e;
    if (prec == PREC_MIXED) {
        auto cfg = persist_config<true>(1, nullptr, at);
        e = cudaOccupancyMaxActiveClusters(&n, k_batch_persist<true>, &cfg);
    } else {
        auto cfg = persist_config<false>(1, nullptr, at);
        e = cudaOccupancyMaxActiveClusters(&n, k_batch_persist<false>, &cfg);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

cudaError_t launch_batch_persist(const BatchInst* inst, const int4* psp, const int2* put,
                                 const int4* ctab, int n_clusters, const BatchTime* times,
                                 int n_inst, int nsteps, int prec, cudaStream_t s)
{
    cudaLaunchAttribute at[1];
    ++g_launches;
    if (prec == PREC_MIXED) {
        auto cfg = persist_config<true>(n_clusters, s, at);
        return cudaLaunchKernelEx(&cfg, k_batch_persist<true>, inst, psp, put, ctab,
                                  times, n_inst, nsteps);
    }
    auto cfg = persist_config<false>(n_clusters, s, at);
    return cudaLaunchKernelEx(&cfg, k_batch_persist<false>, inst, psp, put, ctab, times,
                              n_inst, nsteps);
}

int batch_stage2d_grid(int prec, int n_wtiles)
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const void* fn = prec == PREC_MIXED ? (const void*)k_batch_stage2d<1, true>
                                        : (const void*)k_batch_stage2d<1, false>;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 128, 0);
    const long long g = (long long)std::max(1, per_sm) * std::max(1, sms);
    return (int)std::max(1LL, std::min<long long>(g, ((long long)n_wtiles + 3) / 4));
}

int batch2d_tile_points() { return BATCH2D_TILE;
}

cudaError_t launch_batch_probe(const BatchInst* inst, const int4* tiles, int n_tiles,
                               int tile_cfg, int grid, const BatchTime* times, int prec,
                               cudaStream_t s)
{
    if (prec == PREC_MIXED)
        batch_stage<1, true>(inst, tiles, n_tiles, tile_cfg, grid, times, s);
    else
        batch_stage<1, false>(inst, tiles, n_tiles, tile_cfg, grid, times, s);
    return cudaGetLastError();
}

int batch_stage_grid(int tile_cfg, int prec, int n_tiles)
{
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int warps = BATCH_TILE_WARPS[tile_cfg & 3];
    const void* fn = nullptr;
    if (prec == PREC_MIXED) {
        const void* f[4] = {(const void*)k_batch_stage<1, true, 1>, (const void*)k_batch_stage<1, true, 2>,
                            (const void*)k_batch_stage<1, true, 4>, (const void*)k_batch_stage<1, true, 8>};
        fn = f[tile_cfg & 3];
    } else {
        const void* f[4] = {(const void*)k_batch_stage<1, false, 1>, (const void*)k_batch_stage<1, false, 2>,
                            (const void*)k_batch_stage<1, false, 4>, (const void*)k_batch_stage<1, false, 8>};
        fn = f[tile_cfg & 3];
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * warps, 0);
    const long long g = (long long)std::max(1, per_sm) * std::max(1, sms);
    return (int)std::max(1LL, std::min<long long>(g, n_tiles));
}

cudaError_t launch_sinsin_xy(const float* sx, const float* sy, int n1, int n2, float* out,
                             cudaStream_t s)
{
    const long long n = (long long)n1 * n2;
    if (n > 0) {
        k_sinsin_xy<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(sx, sy, n1, n2, out);
        ++g_launches;
    }
    return cudaGetLastError();
}

cudaError_t launch_batch_finish(const BatchInst* inst, int n_inst, const BatchTime* last,
                                const int* r_inst, int n_r, cudaStream_t s)
{
    (void)n_inst;
    if (n_r) {
        k_batch_finish<<<(n_r + 127) / 128, 128, 0, s>>>(inst, last, r_inst, n_r);
        ++g_launches;
    }
    return cudaGetLastError();
}

// ===========================================================================================
// Discrete adjoint of the heat RK4 path (FP64).  Forward step (rk4.cpp:16-47):
//   Y1 = u, k_s = A Y_s, Y_{s+1} = u + dt a_s k_s, u' = u + dt sum_s b_s k_s,
// with Dirichlet faces reset after every stage.  Reverse step, given lam = adjoint of u':
//   z4 = dt b4 lam; for S = 4..1: Ybar_S = A^T z_S, z_{S-1} = dt b_{S-1} lam + dt a_{S-1} Ybar_S;
//   lam <- lam + sum_S Ybar_S,
// all restricted to the evolving points E; solid points keep their adjoint (their value never
// changes), Dirichlet-face points get one only from the solve's first stage, which reads the
// caller's face values.
// ===========================================================================================
namespace
{
__device__ __forceinline__ bool evolves(unsigned c) { return (c & 0x3Fu) && !(c & CLS_DIRFACE); }

// transposed interior rows at point p (coordinates ijk): sum over axes and offsets of the
// neighbours i = p - m s whose interior row (an evolving point's) reads p with weight c_m
template <class T>
__device__ __forceinline__ T interior_t(const DevOp& op, long long p, const int ijk[3],
                                        const T* __restrict__ z)
{
    T y = 0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const DevAxis& A = op.ax[d];
        if (!A.active) continue;
        const int half = A.width / 2;
        for (int m = -half; m <= half; m++) {
            const int ci = ijk[d] - m;
            if (ci < 0 || ci >= A.n) continue;
            const long long i = p - (long long)m * A.stride;
            const unsigned c = op.cls[i];
            if (((c >> (2 * d)) & 3u) != ROW_INTERIOR || (c & CLS_DIRFACE)) continue;
            if constexpr (sizeof(T) == 8)
                y = fma(A.ic[half + m], __ldcg(z + i), y); // row i's weight on offset m
            else
                y = fmaf(A.icf[half + m], __ldcg(z + i), y);
        }
    }
    return y;
}

template <class T>
__global__ void __launch_bounds__(256) k_adj_stage(DevOp op, int S, AdjArgs a)
{
    pdl_wait();
    pdl_trigger();
    const Pt q = point_of(op);
    if (!q.valid) return;
    const unsigned c = op.cls[q.p];
    int ijk[3];
    phys_ijk(op, q, ijk);
    const T* z = (const T*)a.z;
    const T* lam = (const T*)a.lam;
    T* acc = (T*)a.acc;
    T* out = (T*)a.out;
    const T y = (T)a.k * (interior_t<T>(op, q.p, ijk, z) * (T)a.zscale);
    const bool e = evolves(c);
    if (S == 0) {
        out[q.p] = y;
    } else if (S > 1) {
        const T ac = S == 4 ? T(0) : acc[q.p];
        acc[q.p] = e ? ac + y : T(0);
        out[q.p] = e ? (T)a.ay * y + (T)a.bl * lam[q.p] : T(0);
    } else {
        const T l = lam[q.p];
        out[q.p] = e ? l + acc[q.p] + y : ((c & CLS_DIRFACE) ? (a.first_step ? y : T(0)) : l);
    }
}

// transposed closure rows, added after k_adj_stage: target t gets k sum w z[src] (FP64 sum)
template <class T>
__global__ void k_adj_closure(DevOp op, AdjClosure cl, int S, AdjArgs a)
{
    pdl_wait();
    pdl_trigger();
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= cl.n_tgt) return;
    const T* z = (const T*)a.z;
    T* acc = (T*)a.acc;
    T* out = (T*)a.out;
    double yd = 0.0;
    for (int e = cl.ptr[t]; e < cl.ptr[t + 1]; e++)
        yd = fma(cl.w[e], (double)__ldcg(z + cl.src[e]), yd);
    const T y = (T)(a.k * (yd * a.zscale));
    const long long p = cl.tgt[t];
    const unsigned c = op.cls[p];
    if (S == 0) {
        out[p] += y;
    } else if (S > 1) {
        if (evolves(c)) {
            acc[p] += y;
            out[p] += (T)a.ay * y;
        }
    } else if (evolves(c) || ((c & CLS_DIRFACE) && a.first_step)) {
        out[p] += y;
    }
}

// FP32 reverse stage in the vectorised layout (3-D grids, nz a multiple of 4): four z points
// per thread; the stage adjoint and the class words of the 12 stencil neighbours arrive as
// float4 / 32-bit loads, and each point gathers from the neighbour rows that read it (their
// class says interior, not on a Dirichlet face, and they lie in the grid).  The closure part
// follows in k_adj_closure as in the per-point path.
__device__ __forceinline__ unsigned cbyte(unsigned w, int q) { return (w >> (8 * q)) & 0xFFu; }
__device__ __forceinline__ bool row_reads(unsigned c, int d)
{
    return ((c >> (2 * d)) & 3u) == ROW_INTERIOR && !(c & CLS_DIRFACE);
}

__global__ void __launch_bounds__(256, 4) k_adj_stage_vec(DevOp op, int S, AdjArgs a)
{
    pdl_wait();
    pdl_trigger();
    const int nx = op.it0, ny = op.it1, nz = op.it2;
    const int j = blockIdx.y * BY + threadIdx.y;
    if (j >= ny) return;
    const int i = blockIdx.z;
    const int k = blockIdx.x * 128 + 4 * threadIdx.x;
    if (k >= nz) return;
    const int plane = ny * nz;
    const int p = i * plane + j * nz + k;
    const float* __restrict__ z = (const float*)a.z;
    const unsigned* __restrict__ cw = (const unsigned*)op.cls;
    auto C4 = [&](int idx) { return __ldg(cw + idx / 4); };
    // neighbours along x and y: offsets of planes / rows i-2 .. i+2 (clamped; the range
    // checks below drop the clamped ones)
    const int ox[5] = {(max(i - 2, 0) - i) * plane, (max(i - 1, 0) - i) * plane, 0,
                       (min(i + 1, nx - 1) - i) * plane, (min(i + 2, nx - 1) - i) * plane};
    const int oy[5] = {(max(j - 2, 0) - j) * nz, (max(j - 1, 0) - j) * nz, 0,
                       (min(j + 1, ny - 1) - j) * nz, (min(j + 2, ny - 1) - j) * nz};
    const bool inx[5] = {i >= 2, i >= 1, true, i + 1 < nx, i + 2 < nx};
    const bool iny[5] = {j >= 2, j >= 1, true, j + 1 < ny, j + 2 < ny};
    float4 zx[5], zy[5];
    unsigned cx[5], cy[5];
#pragma unroll
    for (int m = 0; m < 5; m++) {
        zx[m] = ld4cg(z, p + ox[m]);
        cx[m] = C4(p + ox[m]);
        zy[m] = ld4cg(z, p + oy[m]);
        cy[m] = C4(p + oy[m]);
    }
    const int zl = k >= 4 ? -4 : 0, zr = k + 8 <= nz ? 4 : 0;
    const float4 zL = ld4cg(z, p + zl), zR = ld4cg(z, p + zr);
    const unsigned cL = C4(p + zl), cR = C4(p + zr);
    const float4 zc = zx[2];
    const unsigned cc = cx[2];
    const float zz[12] = {zL.x, zL.y, zL.z, zL.w, zc.x, zc.y, zc.z, zc.w, zR.x, zR.y, zR.z, zR.w};
    const unsigned czw[3] = {cL, cc, cR};
    float y[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        float t = 0.f;
        // x: the row at plane i - (m - 2) reads this point with weight icf[half + (m - 2)]
#pragma unroll
        for (int m = 0; m < 5; m++) {
            const DevAxis& A = op.ax[0];
            const int off = 2 - m; // this point's offset in that row
            const int half = A.width / 2;
            if (off < -half || off > half || !inx[m]) continue;
            if (row_reads(cbyte(cx[m], q), 0)) t = fmaf(A.icf[half + off], f4(zx[m], q), t);
        }
#pragma unroll
        for (int m = 0; m < 5; m++) {
            const DevAxis& A = op.ax[1];
            const int off = 2 - m;
            const int half = A.width / 2;
            if (off < -half || off > half || !iny[m]) continue;
            if (row_reads(cbyte(cy[m], q), 1)) t = fmaf(A.icf[half + off], f4(zy[m], q), t);
        }
#pragma unroll
        for (int m = 0; m < 5; m++) {
            const DevAxis& A = op.ax[2];
            const int off = 2 - m;
            const int half = A.width / 2;
            const int kk = k + q - off; // the row's point
            if (off < -half || off > half || kk < 0 || kk >= nz) continue;
            const int w = 4 + q - off; // position in the 12-value window
            if (row_reads(cbyte(czw[w >> 2], w & 3), 2)) t = fmaf(A.icf[half + off], zz[w], t);
        }
        y[q] = (float)a.k * (t * (float)a.zscale);
    }
    const float* __restrict__ lam = (const float*)a.lam;
    float* __restrict__ acc = (float*)a.acc;
    float* __restrict__ out = (float*)a.out;
    float o[4], ac[4];
    const float4 l4 = *(const float4*)(lam + p);
    const float4 a4 = S == 4 ? make_float4(0.f, 0.f, 0.f, 0.f) : *(const float4*)(acc + p);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const unsigned c = cbyte(cc, q);
        const bool e = evolves(c);
        const float l = f4(l4, q);
        if (S > 1) {
            ac[q] = e ? f4(a4, q) + y[q] : 0.f;
            o[q] = e ? (float)a.ay * y[q] + (float)a.bl * l : 0.f;
        } else {
            o[q] = e ? l + f4(a4, q) + y[q] : ((c & CLS_DIRFACE) ? (a.first_step ? y[q] : 0.f) : l);
        }
    }
    if (S > 1) *(float4*)(acc + p) = make_float4(ac[0], ac[1], ac[2], ac[3]);
    *(float4*)(out + p) = make_float4(o[0], o[1], o[2], o[3]);
}

template <class T>
__global__ void k_adj_mask_faces(DevOp op, T* lam)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < op.n_faces) lam[op.faces[e]] = T(0);
}

__global__ void k_cast(long long n, int to_f32, const void* in, void* out)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (to_f32)
        ((float*)out)[i] = (float)((const double*)in)[i];
    else
        ((double*)out)[i] = (double)((const float*)in)[i];
}
} // namespace

cudaError_t launch_adjoint_mask_faces(const DevOp& op, void* lam, int prec, cudaStream_t s)
{
    if (op.n_faces) {
        if (prec == PREC_MIXED)
            k_adj_mask_faces<float><<<(op.n_faces + 255) / 256, 256, 0, s>>>(op, (float*)lam);
        else
            k_adj_mask_faces<double><<<(op.n_faces + 255) / 256, 256, 0, s>>>(op, (double*)lam);
        ++g_launches;
    }
    return cudaGetLastError();
}

cudaError_t launch_cast(long long n, int to_f32, const void* in, void* out, cudaStream_t s)
{
    if (n > 0) {
        k_cast<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, to_f32, in, out);
        ++g_launches;
    }
    return cudaGetLastError();
}

cudaError_t launch_adjoint_stage(const DevOp& op, const AdjClosure& cl, int S, const AdjArgs& a,
                                 int prec, cudaStream_t s)
{
    const bool vec = prec == PREC_MIXED && S > 0 && op.it0 > 1 && op.it1 > 1 && op.it2 > 1 &&
                     op.it2 % 4 == 0 && op.N < (1LL << 31) - 64;
    // every kernel of the reverse sweep waits for its predecessor before it reads anything,
    // so each is launched to start while the previous one drains (dependent launch)
    cudaError_t e;
    if (vec)
        e = launch_ex(k_adj_stage_vec, dim3((op.it2 + 127) / 128, (op.it1 + BY - 1) / BY, op.it0),
                      dim3(32, BY), s, true, op, S, a);
    else if (prec == PREC_MIXED)
        e = launch_ex(k_adj_stage<float>, point_grid(op), dim3(32, BY), s, true, op, S, a);
    else
        e = launch_ex(k_adj_stage<double>, point_grid(op), dim3(32, BY), s, true, op, S, a);
    ++g_launches;
    if (e != cudaSuccess) return e;
    if (cl.n_tgt) {
        const dim3 g((cl.n_tgt + 127) / 128);
        if (prec == PREC_MIXED)
            e = launch_ex(k_adj_closure<float>, g, dim3(128), s, true, op, cl, S, a);
        else
            e = launch_ex(k_adj_closure<double>, g, dim3(128), s, true, op, cl, S, a);
        ++g_launches;
        if (e != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

} // namespace sgb
