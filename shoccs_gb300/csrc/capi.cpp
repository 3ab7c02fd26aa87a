// capi.cpp -- implementation of include/shoccs_gpu.h.
//
// A shoccs_problem owns the host setup (mesh, stencil, per-axis operators in the reference's
// own decomposition) and, once uploaded, the compiled device tables.  A shoccs_system owns
// the RK4 registers of one heat or scalar-wave solve.  Errors are reported as status codes
// with a thread-local message; nothing here falls back to host arithmetic.
#include "../../include/shoccs_gpu.h"
#include "device.cuh"
#include "host/problem.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

using namespace sgb;

namespace
{
thread_local std::string g_err;

shoccs_status fail(shoccs_status s, const std::string& msg)
{
    g_err = msg;
    return s;
}

#define SH_CUDA(call)                                                                       \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess)                                                              \
            return fail(e_ == cudaErrorMemoryAllocation ? SHOCCS_ENOMEM : SHOCCS_ECUDA,     \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                \
    } while (0)

template <class T>
cudaError_t upload(const std::vector<T>& h, T** d, cudaStream_t s)
{
    *d = nullptr;
    if (h.empty()) return cudaSuccess;
    cudaError_t e = cudaMalloc((void**)d, h.size() * sizeof(T));
    if (e != cudaSuccess) return e;
    return cudaMemcpyAsync(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s);
}

struct DeviceAlloc {
    std::vector<void*> ptrs;
    ~DeviceAlloc()
    {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    cudaError_t put(const std::vector<T>& h, const T** d, cudaStream_t s)
    {
        T* p = nullptr;
        cudaError_t e = upload(h, &p, s);
        if (p) ptrs.push_back(p);
        *d = p;
        return e;
    }
    cudaError_t alloc(size_t bytes, void** d)
    {
        *d = nullptr;
        if (!bytes) return cudaSuccess;
        cudaError_t e = cudaMalloc(d, bytes);
        if (e == cudaSuccess) ptrs.push_back(*d);
        return e;
    }
};
} // namespace

struct shoccs_problem {
    Mesh mesh;
    Stencil st;
    Bcs bcs;
    AxisOp ops[3];
    Compiled comp;
    // every point with a row and not on a Dirichlet face has a row along every active axis
    // (the vectorised stage kernel evaluates the interior row everywhere and relies on it)
    bool rows_complete = false;
    // device side
    bool uploaded = false;
    int device = -1;
    DeviceAlloc mem;
    DevOp op{};
    DevR dr{};
};

// adjoint state of a system, built on first use
struct AdjointState {
    bool built = false;
    DeviceAlloc mem;
    AdjClosure cl{};
    void* lam = nullptr; // adjoint of the current state (FP64, or FP32 for a mixed system)
    void* acc = nullptr;
    void* za = nullptr;
    void* zb = nullptr;
};

struct shoccs_system {
    shoccs_problem* P;
    shoccs_system_desc desc;
    SysParams sp{};
    DeviceAlloc mem;
    StepBuffers b{};
    double t = 0.0;
    AdjointState adj;
    // heat systems with non-Dirichlet objects step the whole field {D, R} unfused (FP64):
    // stage field, right-hand side and accumulator (D parts: b.sa, b.sb, b.acc)
    bool unfused = false;
    FieldF64 fy{}, fk{}, facc{};
    UnfusedAux ux{}; // Neumann domain faces (unfused heat), gradient scratch (unfused wave)
    FieldF64 state() const { return {(double*)b.u0, {b.R[0], b.R[1], b.R[2]}}; }
    ~shoccs_system()
    {
        if (b.side) cudaStreamDestroy(b.side);
        if (b.fork) cudaEventDestroy(b.fork);
        if (b.join) cudaEventDestroy(b.join);
        if (b.join_next) cudaEventDestroy(b.join_next);
    }
};

namespace
{
shoccs_status do_upload(shoccs_problem* p, cudaStream_t s)
{
    int dev = 0;
    SH_CUDA(cudaGetDevice(&dev));
    if (p->uploaded) {
        if (dev != p->device)
            return fail(SHOCCS_EINVAL, "problem was uploaded to another device");
        return SHOCCS_OK;
    }
    const Compiled& C = p->comp;
    DevOp& op = p->op;
    op = DevOp{};
    op.it0 = C.it[0];
    op.it1 = C.it[1];
    op.it2 = C.it[2];
    op.nzc = C.nzc;
    op.N = p->mesh.size();
    for (int d = 0; d < 3; d++) {
        op.nR[d] = (long long)p->mesh.R[d].size();
        op.n[d] = p->mesh.n[d];
        op.phys_of_it[d] = C.phys_of_it[d];
    }
    if (op.it0 > 65535) return fail(SHOCCS_EINVAL, "grid too large along the slowest axis");
    SH_CUDA(p->mem.put(C.cls, &op.cls, s));
    {
        std::vector<long long> faces;
        for (long long i = 0; i < (long long)C.cls.size(); i++)
            if (C.cls[i] & CLS_DIRFACE) faces.push_back(i);
        if (faces.size() > 0x7fffffff) return fail(SHOCCS_EINVAL, "too many face points");
        op.n_faces = (int)faces.size();
        SH_CUDA(p->mem.put(faces, &op.faces, s));
    }
    for (int d = 0; d < 3; d++) SH_CUDA(p->mem.put(p->mesh.x[d], &op.xc[d], s));
    for (int d = 0; d < 3; d++) {
        const AxisTables& T = C.ax[d];
        DevAxis& A = op.ax[d];
        A.active = T.active;
        A.stride = T.stride;
        A.width = T.width;
        A.n = p->mesh.n[d];
        A.wall[0] = T.wall[0];
        A.wall[1] = T.wall[1];
        A.row_base = op.n_cut_rows;
        A.n_rows = (int)T.rows.size();
        op.n_cut_rows += A.n_rows;
        for (int j = 0; j < 9; j++) {
            A.ic[j] = T.interior[j];
            A.icf[j] = (float)T.interior[j];
        }
        // antisymmetric (first derivative, zero centre) or symmetric interior rows
        const int hw = T.width / 2;
        bool anti = T.width >= 3 && T.interior[hw] == 0.0, sym = T.width >= 3;
        for (int k = 1; k <= hw; k++) {
            anti = anti && T.interior[hw - k] == -T.interior[hw + k];
            sym = sym && T.interior[hw - k] == T.interior[hw + k];
        }
        A.antisym = anti;
        if (!T.active) continue;
        // the FP32 kernels evaluate a non-antisymmetric interior as a symmetric zero-sum
        // second-derivative row in difference form (sym5 / sym3: 3- and 5-point rows only)
        if (!A.antisym && !(sym && T.width <= 5))
            return fail(SHOCCS_EINVAL, "interior stencil neither symmetric nor antisymmetric");
        SH_CUDA(p->mem.put(T.rows, &A.rows, s));
        SH_CUDA(p->mem.put(T.row_out, (const long long**)&A.row_out, s));
        SH_CUDA(p->mem.put(T.coef, &A.coef, s));
        {
            std::vector<float2> ff(T.coef.size());
            for (size_t m = 0; m < ff.size(); m++) {
                const float hi = (float)T.coef[m];
                ff[m] = make_float2(hi, (float)(T.coef[m] - (double)hi));
            }
            SH_CUDA(p->mem.put(ff, &A.coef_ff, s));
        }
        SH_CUDA(p->mem.put(T.chunk_base, &A.chunk_base, s));
        for (int r = 0; r < 3; r++) {
            if (T.rr_u[r].empty()) continue;
            A.rr_rows[r] = (int)T.rr_u[r].size() - 1;
            SH_CUDA(p->mem.put(T.rr_u[r], &A.rr_u[r], s));
            SH_CUDA(p->mem.put(T.rr_col[r], &A.rr_col[r], s));
            SH_CUDA(p->mem.put(T.rr_src[r], &A.rr_src[r], s));
            SH_CUDA(p->mem.put(T.rr_w[r], &A.rr_w[r], s));
        }
    }
    for (int d = 0; d < 3; d++) {
        std::vector<double> pos;
        std::vector<uint8_t> dir;
        for (const auto& cp : p->mesh.R[d]) {
            pos.insert(pos.end(), cp.pos, cp.pos + 3);
            dir.push_back(p->bcs.obj[cp.shape_id] == Dirichlet ? 1 : 0);
        }
        SH_CUDA(p->mem.put(pos, &p->dr.pos[d], s));
        SH_CUDA(p->mem.put(dir, &p->dr.dirichlet[d], s));
    }
    SH_CUDA(cudaStreamSynchronize(s));
    p->uploaded = true;
    p->device = dev;
    return SHOCCS_OK;
}

bool bad_bc(int b) { return b < 0 || b > 2; }

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                 const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                 const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn()
{
    static EncodeTiled fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* ptr = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(ptr);
    }
    return fn;
}

// 3-D tensor map over a field of nx x ny x nz elements (z fastest): boxes of one plane of
// (32 + 8) x (8 + 4) elements (the tile of k_stage_mixed_tma plus its halo) or, with
// halo = false, of the 32 x 8 tile alone
bool make_plane_map(CUtensorMap* m, void* base, int esz, const int it[3], bool halo = true)
{
    EncodeTiled enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)it[2], (cuuint64_t)it[1], (cuuint64_t)it[0]};
    const cuuint64_t strides[2] = {(cuuint64_t)it[2] * esz, (cuuint64_t)it[2] * it[1] * esz};
    const cuuint32_t box[3] = {halo ? 40u : 32u, halo ? 12u : 8u, 1u};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUtensorMapDataType ty = esz == 1   ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                                   : esz == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                              : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    return enc(m, ty, 3,
               base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
               CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
// scratch of the vectorised FP32 operators, allocated on the first mixed-precision apply of
// a 3-D grid whose z extent is a multiple of 4 and whose axes share one interior stencil
shoccs_status ensure_op_scratch(shoccs_problem* p)
{
    DevOp& op = p->op;
    if (op.op_rowv || op.op_form == -1) return SHOCCS_OK;
    const int* it = p->comp.it;
    auto f = [](const DevAxis& A) {
        return A.width == 5 ? (A.antisym ? FORM_ANTI5 : FORM_SYM5)
                            : (A.width == 3 && !A.antisym ? FORM_W3 : FORM_ANY);
    };
    int form = f(op.ax[0]);
    for (int d = 1; d < 3; d++)
        if (f(op.ax[d]) != form) form = FORM_ANY;
    // z-wall rows travel in 16-word line records: at most 6 rows per wall block, and the
    // line's first and last points in different lanes
    const WallBlock* Wz = op.ax[2].wall;
    const bool ok = it[0] > 1 && it[1] > 1 && it[2] >= 8 && it[2] % 4 == 0 && form != FORM_ANY &&
                    Wz[0].rows <= 6 && Wz[1].rows <= 6 && op.N < (1LL << 31) - 64 &&
                    (long long)op.n_cut_rows + (long long)it[0] * it[1] < (1LL << 31) - 256;
    if (!ok) {
        op.op_form = -1; // not applicable: the per-point kernels serve this problem
        return SHOCCS_OK;
    }
    void* r = nullptr;
    SH_CUDA(p->mem.alloc((size_t)3 * op.N * sizeof(float), &r));
    const size_t nzw = (size_t)it[0] * it[1] * 16; // one 16-word record per z line
    void* z = nullptr;
    SH_CUDA(p->mem.alloc(nzw * sizeof(float), &z));
    op.op_rowv = (float*)r;
    op.op_zw = (float*)z;
    op.op_form = form;
    return SHOCCS_OK;
}
} // namespace

extern "C" {

size_t shoccs_last_error(char* buf, size_t len)
{
    if (buf && len) {
        std::snprintf(buf, len, "%s", g_err.c_str());
    }
    return g_err.size();
}

int64_t shoccs_kernel_launches(void) { return kernel_launch_count(); }

shoccs_status shoccs_problem_create(const shoccs_problem_desc* d, shoccs_problem** out)
{
    if (!d || !out) return fail(SHOCCS_EINVAL, "null descriptor or output");
    *out = nullptr;
    for (int i = 0; i < 3; i++)
        if (d->n[i] < 1) return fail(SHOCCS_EINVAL, "index_extents must be >= 1");
    if (d->scheme < 0 || d->scheme > 7 || d->scheme == 4) return fail(SHOCCS_EINVAL, "unknown scheme");
    if (d->n_spheres < 0 || (d->n_spheres && (!d->centers || !d->radii || !d->sphere_bc)))
        return fail(SHOCCS_EINVAL, "sphere arrays missing");
    for (int i = 0; i < 6; i++)
        if (bad_bc(d->grid_bc[i])) return fail(SHOCCS_EINVAL, "bad grid boundary condition");
    for (int i = 0; i < d->n_spheres; i++)
        if (bad_bc(d->sphere_bc[i])) return fail(SHOCCS_EINVAL, "bad shape boundary condition");
    if (d->scheme == SHOCCS_SCHEME_POLYE2_1) {
        for (int i = 0; i < 13; i++)
            if (!std::isfinite(d->scheme_alpha[i])) return fail(SHOCCS_EINVAL, "E2-poly: non-finite alpha");
        for (int i = 0; i < 6; i++)
            if (d->grid_bc[i] == SHOCCS_BC_NEUMANN && d->n[i / 2] > 1)
                return fail(SHOCCS_EUNSUPPORTED, "first-derivative schemes have no Neumann closure");
        for (int i = 0; i < d->n_spheres; i++)
            if (d->sphere_bc[i] == SHOCCS_BC_NEUMANN)
                return fail(SHOCCS_EUNSUPPORTED, "first-derivative schemes have no Neumann closure");
    }
    if (d->scheme == SHOCCS_SCHEME_E4_1 || d->scheme == SHOCCS_SCHEME_E4U_1 ||
        d->scheme == SHOCCS_SCHEME_E6U_1 || d->scheme == SHOCCS_SCHEME_E8U_1) {
        // src/stencils/E4_1.cpp:34-41
        if (d->scheme == SHOCCS_SCHEME_E4_1 && d->alpha[1] < 197.0 / 288.0)
            return fail(SHOCCS_EINVAL,
                        "E4_1: alpha[1] must be >= 197/288 to avoid the interior "
                        "denominator singularity");
        for (int i = 0; i < 6; i++)
            if (d->grid_bc[i] == SHOCCS_BC_NEUMANN && d->n[i / 2] > 1)
                return fail(SHOCCS_EUNSUPPORTED, "first-derivative schemes have no Neumann closure");
        for (int i = 0; i < d->n_spheres; i++)
            if (d->sphere_bc[i] != SHOCCS_BC_DIRICHLET)
                return fail(SHOCCS_EUNSUPPORTED,
                            "first-derivative schemes have no cross-direction interpolant; "
                            "objects must be Dirichlet");
    }
    try {
        auto p = std::make_unique<shoccs_problem>();
        std::vector<Sphere> shapes;
        for (int i = 0; i < d->n_spheres; i++) {
            if (!(d->radii[i] > 0)) return fail(SHOCCS_EINVAL, "sphere radius must be > 0");
            shapes.push_back(Sphere{{d->centers[3 * i], d->centers[3 * i + 1],
                                     d->centers[3 * i + 2]},
                                    d->radii[i], i});
        }
        p->mesh = build_mesh(d->n, d->lo, d->hi, shapes);
        p->st.kind = d->scheme;
        p->st.alpha[0] = d->alpha[0];
        p->st.alpha[1] = d->alpha[1];
        for (int i = 0; i < 13; i++) p->st.pa[i] = d->scheme_alpha[i];
        // a boundary condition on a trivial axis is Floating (src/operators/boundaries.cpp:15-24)
        for (int a = 0; a < 3; a++)
            for (int side = 0; side < 2; side++) {
                int b = d->grid_bc[2 * a + side];
                if (p->mesh.n[a] == 1 && b != Floating) b = Floating;
                p->bcs.grid[a][side] = b;
            }
        p->bcs.obj.assign(d->sphere_bc, d->sphere_bc + d->n_spheres);
        for (int a = 0; a < 3; a++) p->ops[a] = assemble_axis(a, p->mesh, p->st, p->bcs);
        p->comp = compile_operators(p->mesh, p->ops, p->bcs);
        p->rows_complete = true;
        for (const uint8_t c : p->comp.cls) {
            if (!(c & 0x3F) || (c & CLS_DIRFACE)) continue;
            for (int a = 0; a < 3; a++)
                if (p->ops[a].active && ((c >> (2 * a)) & 3) == 0) p->rows_complete = false;
        }
        *out = p.release();
        return SHOCCS_OK;
    } catch (const std::bad_alloc&) {
        return fail(SHOCCS_ENOMEM, "host allocation failed during setup");
    } catch (const std::exception& e) {
        return fail(SHOCCS_EINVAL, e.what());
    }
}

shoccs_status shoccs_problem_destroy(shoccs_problem* p)
{
    delete p;
    return SHOCCS_OK;
}

shoccs_status shoccs_problem_sizes(const shoccs_problem* p, int64_t sizes[5])
{
    if (!p || !sizes) return fail(SHOCCS_EINVAL, "null argument");
    sizes[0] = p->mesh.size();
    for (int d = 0; d < 3; d++) sizes[d + 1] = (int64_t)p->mesh.R[d].size();
    sizes[4] = p->comp.n_fluid;
    return SHOCCS_OK;
}

shoccs_status shoccs_problem_cut_points(const shoccs_problem* p, int dir, double* psi,
                                        double* position, double* normal, int* ray_outside,
                                        int* solid_coord, int* shape_id)
{
    if (!p || dir < 0 || dir > 2) return fail(SHOCCS_EINVAL, "bad problem or direction");
    const auto& R = p->mesh.R[dir];
    for (size_t i = 0; i < R.size(); i++) {
        if (psi) psi[i] = R[i].psi;
        for (int c = 0; c < 3; c++) {
            if (position) position[3 * i + c] = R[i].pos[c];
            if (normal) normal[3 * i + c] = R[i].nrm[c];
            if (solid_coord) solid_coord[3 * i + c] = R[i].solid[c];
        }
        if (ray_outside) ray_outside[i] = R[i].ray_outside;
        if (shape_id) shape_id[i] = R[i].shape_id;
    }
    return SHOCCS_OK;
}

shoccs_status shoccs_problem_block_meta(const shoccs_problem* p, int dir, int* meta,
                                        int64_t* n_lines, double* coeffs, int64_t* n_coeffs)
{
    if (!p || dir < 0 || dir > 2) return fail(SHOCCS_EINVAL, "bad problem or direction");
    const AxisOp& A = p->ops[dir];
    if (n_lines) *n_lines = (int64_t)A.meta.size();
    if (n_coeffs) *n_coeffs = (int64_t)A.coeffs.size();
    if (meta) std::memcpy(meta, A.meta.data(), A.meta.size() * sizeof(BlockMeta));
    if (coeffs) std::memcpy(coeffs, A.coeffs.data(), A.coeffs.size() * sizeof(double));
    return SHOCCS_OK;
}

shoccs_status shoccs_problem_csr(const shoccs_problem* p, int dir, int which, int64_t* rows,
                                 int64_t* nnz, int64_t* row_offsets, int64_t* cols,
                                 double* vals)
{
    if (!p || dir < 0 || dir > 2 || which < 0 || which > 7)
        return fail(SHOCCS_EINVAL, "bad problem, direction or matrix");
    const AxisOp& A = p->ops[dir];
    const Csr& c = which == 0 ? A.B : which == 1 ? A.N : which < 5 ? A.Bf[which - 2]
                                                                   : A.Br[which - 5];
    if (rows) *rows = c.rows;
    if (nnz) *nnz = (int64_t)c.w.size();
    if (row_offsets)
        for (size_t i = 0; i < c.u.size(); i++) row_offsets[i] = c.u[i];
    if (cols)
        for (size_t i = 0; i < c.v.size(); i++) cols[i] = c.v[i];
    if (vals) std::memcpy(vals, c.w.data(), c.w.size() * sizeof(double));
    return SHOCCS_OK;
}

shoccs_status shoccs_problem_classes(const shoccs_problem* p, uint8_t* cls)
{
    if (!p || !cls) return fail(SHOCCS_EINVAL, "null argument");
    std::memcpy(cls, p->comp.cls.data(), p->comp.cls.size());
    return SHOCCS_OK;
}

shoccs_status shoccs_problem_upload(shoccs_problem* p, void* stream)
{
    if (!p) return fail(SHOCCS_EINVAL, "null problem");
    return do_upload(p, (cudaStream_t)stream);
}

shoccs_status shoccs_derivative_apply(shoccs_problem* p, int dir, int prec,
                                      const shoccs_field* u, const shoccs_field* nu,
                                      shoccs_field* du, int plus_eq, void* stream)
{
    if (!p || !u || !du || dir < 0 || dir > 2 || (prec != 0 && prec != 1))
        return fail(SHOCCS_EINVAL, "bad argument");
    const cudaStream_t s = (cudaStream_t)stream;
    if (auto st = do_upload(p, s); st != SHOCCS_OK) return st;
    if (prec == PREC_MIXED)
        if (auto st = ensure_op_scratch(p); st != SHOCCS_OK) return st;
    const void* uR[3] = {u->Rx, u->Ry, u->Rz};
    void* duR[3] = {du->Rx, du->Ry, du->Rz};
    SH_CUDA(launch_derivative(p->op, dir, prec, u->D, uR[dir], nu ? (const double*)nu->D : nullptr,
                              du->D, duR, uR, plus_eq, s));
    SH_CUDA(cudaStreamSynchronize(s));
    return SHOCCS_OK;
}

shoccs_status shoccs_laplacian_apply(shoccs_problem* p, int prec, const shoccs_field* u,
                                     const shoccs_field* nu, shoccs_field* du, void* stream)
{
    if (!p || !u || !du || (prec != 0 && prec != 1)) return fail(SHOCCS_EINVAL, "bad argument");
    const cudaStream_t s = (cudaStream_t)stream;
    if (auto st = do_upload(p, s); st != SHOCCS_OK) return st;
    if (prec == PREC_MIXED)
        if (auto st = ensure_op_scratch(p); st != SHOCCS_OK) return st;
    const void* uR[3] = {u->Rx, u->Ry, u->Rz};
    void* duR[3] = {du->Rx, du->Ry, du->Rz};
    SH_CUDA(launch_laplacian(p->op, prec, u->D, uR, nu ? (const double*)nu->D : nullptr, du->D,
                             duR, s));
    SH_CUDA(cudaStreamSynchronize(s));
    return SHOCCS_OK;
}

shoccs_status shoccs_gradient_apply(shoccs_problem* p, int prec, const shoccs_field* u,
                                    shoccs_field* dx, shoccs_field* dy, shoccs_field* dz,
                                    void* stream)
{
    if (!p || !u || !dx || !dy || !dz || (prec != 0 && prec != 1))
        return fail(SHOCCS_EINVAL, "bad argument");
    const cudaStream_t s = (cudaStream_t)stream;
    if (auto st = do_upload(p, s); st != SHOCCS_OK) return st;
    if (prec == PREC_MIXED)
        if (auto st = ensure_op_scratch(p); st != SHOCCS_OK) return st;
    const void* uR[3] = {u->Rx, u->Ry, u->Rz};
    void* const out[3][4] = {{dx->D, dx->Rx, dx->Ry, dx->Rz},
                             {dy->D, dy->Rx, dy->Ry, dy->Rz},
                             {dz->D, dz->Rx, dz->Ry, dz->Rz}};
    SH_CUDA(launch_gradient(p->op, prec, u->D, uR, out, s));
    SH_CUDA(cudaStreamSynchronize(s));
    return SHOCCS_OK;
}

// ---------------------------------------------------------------------------------------
// systems
// ---------------------------------------------------------------------------------------
// The vectorised stage kernels take the z-wall rows of a line from its 16-word record
// (k_cut_rows): at most 6 rows per wall block (words 0..5 and 8..13), each block entirely on
// its side of the line's middle (wall_side), the left block's columns starting at the wall
// and the right block's ending there (the record threads read the eight points at each end
// of the line), no Neumann term, and nz >= 8 so that the first and last points of a line sit
// in different lanes.
static bool line_records_fit(const DevOp& op)
{
    const int nz = op.it2;
    const WallBlock& L = op.ax[2].wall[0];
    const WallBlock& R = op.ax[2].wall[1];
    // the record holds the wall rows of z = 0..7 and nz-8 .. nz-1
    if (nz < 16) return false;
    if (L.rows && (L.has_n || L.cols > 7 || L.col0 != 0 || L.first_row < 0 ||
                   L.first_row + L.rows > 8))
        return false;
    if (R.rows && (R.has_n || R.cols > 7 || R.col0 + R.cols != nz || R.first_row < nz - 8 ||
                   R.first_row + R.rows > nz))
        return false;
    return true;
}

// Pick the mixed stage kernel for this system: every candidate runs a few RK4 steps on the
// system's own buffers (timed with CUDA events), the fastest is kept, and the state is reset.
// All candidates compute the same values; they differ only in data movement.
static shoccs_status autotune_stage_kernel(shoccs_system* S, cudaStream_t s)
{
    struct Cand {
        const char* name;
        int tma, col, vec, minb = 4, px = 1;
    };
    std::vector<Cand> cands;
    if (S->b.tma) cands.push_back({"tma", 1, 0, 0});
    // the vectorised kernel is compiled for the stencil of each system: 5-point
    // antisymmetric rows for the wave, 5- or 3-point symmetric rows for the heat equation
    int form = FORM_ANY;
    {
        const DevOp& op = S->P->op;
        auto f = [](const DevAxis& A) {
            return A.width == 5 ? (A.antisym ? FORM_ANTI5 : FORM_SYM5)
                                : (A.width == 3 && !A.antisym ? FORM_W3 : FORM_ANY);
        };
        form = f(op.ax[0]);
        for (int d = 1; d < 3; d++)
            if (f(op.ax[d]) != form) form = FORM_ANY;
        const bool wave = S->desc.kind == SHOCCS_SYS_WAVE;
        if (wave ? form != FORM_ANTI5 : (form != FORM_SYM5 && form != FORM_W3)) form = FORM_ANY;
    }
    if (S->P->comp.it[2] % 4 == 0 && S->b.rowv && S->b.lrec && form != FORM_ANY &&
        S->P->rows_complete) {
        cands.push_back({"vec", 0, 0, form, 4});
        cands.push_back({"vec3", 0, 0, form, 3});
        cands.push_back({"vecx2", 0, 0, form, 4, 2});
        cands.push_back({"vecx4", 0, 0, form, 4, 4});
    }
    // the column kernels keep a five-point window along each axis: interiors of up to 5 points
    bool w5 = true;
    for (int a = 0; a < 3; a++) w5 = w5 && (!S->P->op.ax[a].active || S->P->op.ax[a].width <= 5);
    if (w5) {
        cands.push_back({"col1", 0, 1, 0});
        cands.push_back({"col2", 0, 2, 0});
        cands.push_back({"col4", 0, 4, 0});
    }
    cands.push_back({"point", 0, 0, 0});
    auto use = [&](const Cand& c) {
        S->b.tma = c.tma;
        S->b.col_nx = c.col;
        S->b.vec = c.vec;
        S->b.vec_minb = c.minb;
        S->b.vec_px = c.px;
    };
    if (const char* force = std::getenv("SHOCCS_STAGE_KERNEL")) {
        for (const auto& c : cands)
            if (std::string(force) == c.name) {
                use(c);
                return SHOCCS_OK;
            }
        return fail(SHOCCS_EINVAL, std::string("SHOCCS_STAGE_KERNEL: unknown or unavailable ") +
                                       force);
    }
    const long long N = S->P->mesh.size();
    const double h = std::min(S->P->mesh.h[0], std::min(S->P->mesh.h[1], S->P->mesh.h[2]));
    const double dt = 1e-3 * h;
    cudaEvent_t e0, e1;
    SH_CUDA(cudaEventCreate(&e0));
    SH_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    Cand pick = cands.back();
    const int reps = N > (1 << 22) ? 3 : 2;
    for (const auto& c : cands) {
        use(c);
        SH_CUDA(launch_rk4_step(S->P->op, S->P->dr, S->sp, S->desc.prec, S->b, 0.0, dt, s));
        SH_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < reps; r++)
            SH_CUDA(launch_rk4_step(S->P->op, S->P->dr, S->sp, S->desc.prec, S->b, 0.0, dt, s));
        SH_CUDA(cudaEventRecord(e1, s));
        SH_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        SH_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            pick = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    use(pick);
    // reset the registers the trial steps touched
    SH_CUDA(cudaMemsetAsync(S->b.u0, 0, N * 8, s));
    SH_CUDA(cudaMemsetAsync(S->b.acc, 0, N * 4, s));
    for (int r = 0; r < 3; r++)
        if (!S->P->mesh.R[r].empty())
            SH_CUDA(cudaMemsetAsync(S->b.R[r], 0, S->P->mesh.R[r].size() * 8, s));
    if (S->b.err) SH_CUDA(cudaMemsetAsync(S->b.err, 0, sizeof(unsigned), s));
    SH_CUDA(cudaStreamSynchronize(s));
    return SHOCCS_OK;
}

shoccs_status shoccs_system_create(shoccs_problem* p, const shoccs_system_desc* d,
                                   shoccs_system** out)
{
    if (!p || !d || !out) return fail(SHOCCS_EINVAL, "null argument");
    *out = nullptr;
    if (d->kind != SHOCCS_SYS_HEAT && d->kind != SHOCCS_SYS_WAVE)
        return fail(SHOCCS_EINVAL, "unknown system kind");
    if (d->prec != 0 && d->prec != 1) return fail(SHOCCS_EINVAL, "unknown precision");
    if (d->sol_kind < 0 || d->sol_kind > 4) return fail(SHOCCS_EINVAL, "unknown solution kind");
    const bool gaussian = d->sol_kind == SHOCCS_SOL_GAUSSIAN;
    if (gaussian) {
        if (d->kind != SHOCCS_SYS_HEAT)
            return fail(SHOCCS_EUNSUPPORTED, "the gaussian manufactured solution is time-stepped by the "
                                             "heat system only");
        if (d->sol_n_terms < 0 || (d->sol_n_terms > 0 && !d->sol_terms))
            return fail(SHOCCS_EINVAL, "gaussian manufactured solution: bad term list");
        for (int i = 0; i < 8 * d->sol_n_terms; i++)
            if (!std::isfinite(d->sol_terms[i]))
                return fail(SHOCCS_EINVAL, "gaussian manufactured solution: non-finite parameter");
    }
    // Neumann objects step like Floating ones: heat::rhs adds the source at every
    // non-Dirichlet cut point (heat.cpp:143-149) and the object part of the Neumann data
    // (neumann_rx/ry/rz) is never assigned, so their closures carry no data term
    bool non_dirichlet_objects = false;
    for (int b : p->bcs.obj) non_dirichlet_objects = non_dirichlet_objects || b != Dirichlet;
    if (non_dirichlet_objects && d->kind == SHOCCS_SYS_WAVE) {
        for (int b : p->bcs.obj)
            if (b == Neumann)
                return fail(SHOCCS_EUNSUPPORTED, "Neumann objects in the wave system: the reference's "
                                                 "first-derivative schemes have no Neumann closures");
    }
    int neumann_mask = 0;
    for (int a = 0; a < 3; a++)
        for (int side = 0; side < 2; side++)
            if (p->bcs.grid[a][side] == Neumann) neumann_mask |= 1 << (2 * a + side);
    if (neumann_mask && d->kind != SHOCCS_SYS_HEAT)
        return fail(SHOCCS_EUNSUPPORTED, "Neumann faces are time-stepped by the heat system only");
    // Non-Dirichlet objects (whose cut-point values are state), Neumann faces and the
    // Gaussian solution step the whole field unfused.  Its state is FP64 in either
    // precision; a mixed system computes the step in FP32 (UnfusedAux::mixed) and is
    // otherwise handled as an FP64 one (initialisation, state access, statistics).
    const bool unfused = non_dirichlet_objects || neumann_mask || gaussian;
    const bool mixed_step = unfused && d->prec == PREC_MIXED;
    const int prec = unfused ? PREC_FP64 : d->prec;
    if (d->kind == SHOCCS_SYS_HEAT && !(d->diffusivity > 0))
        return fail(SHOCCS_EINVAL, "diffusivity must be > 0");
    const cudaStream_t s = nullptr;
    if (auto st = do_upload(p, s); st != SHOCCS_OK) return st;

    auto S = std::make_unique<shoccs_system>();
    S->P = p;
    S->desc = *d;
    S->desc.prec = prec;
    SysParams& sp = S->sp;
    sp.kind = d->kind;
    sp.k = d->diffusivity;
    sp.kf = (float)d->diffusivity;
    sp.vel_kind = d->vel_kind;
    for (int c = 0; c < 3; c++) {
        sp.vel[c] = d->vel[c];
        sp.gf[c] = (float)(-d->vel[c]);
        sp.center[c] = d->center[c];
        sp.centerf[c] = (float)d->center[c];
    }
    DevSol& sol = sp.sol;
    sol.kind = d->sol_kind;
    sol.dims = p->mesh.n[2] > 1 ? 3 : 2;
    for (int i = 0; i < 8; i++) sol.p[i] = d->sol[i];
    if (sol.kind == SHOCCS_SOL_SINSIN) {
        // sin tables evaluated with the host libm, as the reference evaluates its MMS
        constexpr double twoPI = 2 * 3.14159265358979323846;
        const double k = d->sol[0];
        for (int a = 0; a < 3; a++) {
            std::vector<double> tab(p->mesh.n[a]);
            for (int i = 0; i < p->mesh.n[a]; i++) tab[i] = std::sin(twoPI * k * p->mesh.x[a][i]);
            SH_CUDA(S->mem.put(tab, &sol.S[a], s));
            std::vector<float> tabf(tab.begin(), tab.end());
            SH_CUDA(S->mem.put(tabf, &sol.Sf[a], s));
            std::vector<double> ctab(p->mesh.n[a]);
            for (int i = 0; i < p->mesh.n[a]; i++) ctab[i] = std::cos(twoPI * k * p->mesh.x[a][i]);
            SH_CUDA(S->mem.put(ctab, &sol.C[a], s));
        }
        for (int r = 0; r < 3; r++) {
            std::vector<double> tab;
            for (const auto& cp : p->mesh.R[r]) {
                double v = std::sin(twoPI * k * cp.pos[0]) * std::sin(twoPI * k * cp.pos[1]);
                if (sol.dims == 3) v = v * std::sin(twoPI * k * cp.pos[2]);
                tab.push_back(v);
            }
            SH_CUDA(S->mem.put(tab, &sol.SR[r], s));
        }
        const double kk = twoPI * k;
        sol.lapfac = -(double)sol.dims * kk * kk;
    }
    if (gaussian) {
        // gauss1d / gauss2d / gauss3d by the mesh's dimension count (mms.cpp:16-31)
        sol.gdims = (p->mesh.n[0] > 1) + (p->mesh.n[1] > 1) + (p->mesh.n[2] > 1);
        sol.nG = d->sol_n_terms;
        if (sol.nG > 0) {
            std::vector<double> terms(d->sol_terms, d->sol_terms + 8 * sol.nG);
            SH_CUDA(S->mem.put(terms, &sol.G, s));
        }
    }
    const long long N = p->mesh.size();
    const size_t es_u = 8; // double or float2
    const size_t es_s = prec == PREC_FP64 ? 8 : 4;
    SH_CUDA(S->mem.alloc(N * es_u, &S->b.u0));
    // the mixed path keeps its stage accumulator in FP32 (the increments are FP32-accurate)
    SH_CUDA(S->mem.alloc(N * (prec == PREC_FP64 ? 8 : 4), &S->b.acc));
    if (prec == PREC_FP64) {
        SH_CUDA(S->mem.alloc(N * es_s, &S->b.sa));
        SH_CUDA(S->mem.alloc(N * es_s, &S->b.sb));
    } else {
        // both FP32 stage fields in one N x 8-byte block, which also stages FP64 state
        // conversions in set_state / get_state
        void* base = nullptr;
        SH_CUDA(S->mem.alloc(N * 2 * es_s, &base));
        S->b.sa = base;
        S->b.sb = (char*)base + N * es_s;
    }
    SH_CUDA(S->mem.alloc((size_t)p->op.n_cut_rows * 8, &S->b.cval));
    {
        void* e = nullptr;
        SH_CUDA(S->mem.alloc(sizeof(unsigned), &e));
        S->b.err = (unsigned*)e;
        SH_CUDA(cudaMemsetAsync(e, 0, sizeof(unsigned), s));
    }
    SH_CUDA(cudaMemsetAsync(S->b.u0, 0, N * es_u, s));
    SH_CUDA(cudaMemsetAsync(S->b.acc, 0, N * (prec == PREC_FP64 ? 8 : 4), s));
    for (int r = 0; r < 3; r++) {
        const size_t n = p->mesh.R[r].size();
        void *a, *h, *f;
        SH_CUDA(S->mem.alloc(n * 8, &a));
        SH_CUDA(S->mem.alloc(n * 8, &h));
        SH_CUDA(S->mem.alloc(n * 8, &f));
        S->b.R[r] = (double*)a;
        S->b.Rhalf[r] = (double*)h;
        S->b.Rfull[r] = (double*)f;
        if (n) SH_CUDA(cudaMemsetAsync(a, 0, n * 8, s));
    }
    if (unfused) {
        S->unfused = true;
        if (neumann_mask) {
            void* nu = nullptr;
            SH_CUDA(S->mem.alloc((size_t)N * 8, &nu));
            SH_CUDA(cudaMemsetAsync(nu, 0, (size_t)N * 8, s));
            S->ux.nf = NeumannFaces{neumann_mask, (double*)nu};
        }
        S->fy.D = (double*)S->b.sa;
        S->fk.D = (double*)S->b.sb;
        S->facc.D = (double*)S->b.acc;
        for (int r = 0; r < 3; r++) {
            void* a = nullptr;
            SH_CUDA(S->mem.alloc(p->mesh.R[r].size() * 8, &a));
            S->fy.R[r] = S->b.Rhalf[r];
            S->fk.R[r] = S->b.Rfull[r];
            S->facc.R[r] = (double*)a;
        }
        if (d->kind == SHOCCS_SYS_WAVE && !mixed_step) { // the gradient over the whole field
            for (int c = 0; c < 3; c++) {
                void* g = nullptr;
                SH_CUDA(S->mem.alloc((size_t)N * 8, &g));
                S->ux.grad[c].D = (double*)g;
                for (int r = 0; r < 3; r++) {
                    void* a = nullptr;
                    SH_CUDA(S->mem.alloc(p->mesh.R[r].size() * 8, &a));
                    S->ux.grad[c].R[r] = (double*)a;
                }
            }
        }
        if (mixed_step) { // stage input, right-hand side, accumulator (and gradient): FP32 D
            S->ux.mixed = 1;  // values, FP64 cut-point values
            auto field_mx = [&](FieldMx& f) -> shoccs_status {
                void* a = nullptr;
                SH_CUDA(S->mem.alloc((size_t)N * sizeof(float), &a));
                f.D = (float*)a;
                for (int r = 0; r < 3; r++) {
                    SH_CUDA(S->mem.alloc(std::max<size_t>(1, p->mesh.R[r].size()) * sizeof(double), &a));
                    f.R[r] = (double*)a;
                }
                return SHOCCS_OK;
            };
            for (FieldMx* f : {&S->ux.y_mx, &S->ux.k_mx, &S->ux.acc_mx})
                if (auto st = field_mx(*f); st != SHOCCS_OK) return st;
            if (d->kind == SHOCCS_SYS_WAVE)
                for (int c = 0; c < 3; c++)
                    if (auto st = field_mx(S->ux.grad_mx[c]); st != SHOCCS_OK) return st;
        }
    }
    if (prec == PREC_MIXED) {
        // exact values on the Dirichlet faces, evaluated once per step on a side stream
        for (int f = 0; f < 6; f++) {
            if (p->bcs.grid[f / 2][f % 2] != Dirichlet) continue;
            const int a = f / 2;
            const size_t n = a == 0   ? (size_t)p->mesh.n[1] * p->mesh.n[2]
                             : a == 1 ? (size_t)p->mesh.n[0] * p->mesh.n[2]
                                      : (size_t)p->mesh.n[0] * p->mesh.n[1];
            void* fp = nullptr;
            SH_CUDA(S->mem.alloc(n * sizeof(float4), &fp));
            S->b.fplane[f] = (float4*)fp;
            SH_CUDA(S->mem.alloc(n * sizeof(float4), &fp));
            S->b.fplane_next[f] = (float4*)fp;
        }
        // second set of cut-point boundary values (the next step's, evaluated ahead)
        for (int r = 0; r < 3; r++) {
            const size_t n = p->mesh.R[r].size();
            void *h = nullptr, *f = nullptr;
            SH_CUDA(S->mem.alloc(n * 8, &h));
            SH_CUDA(S->mem.alloc(n * 8, &f));
            S->b.Rhalf_next[r] = (double*)h;
            S->b.Rfull_next[r] = (double*)f;
        }
        int lo = 0, hi = 0;
        SH_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        // normal priority: its work is needed a step later, so the stage kernels go first
        SH_CUDA(cudaStreamCreateWithPriority(&S->b.side, cudaStreamNonBlocking, lo));
        SH_CUDA(cudaEventCreateWithFlags(&S->b.fork, cudaEventDisableTiming));
        SH_CUDA(cudaEventCreateWithFlags(&S->b.join, cudaEventDisableTiming));
        SH_CUDA(cudaEventCreateWithFlags(&S->b.join_next, cudaEventDisableTiming));
    }
    // TMA plane-marching stages for 3-D mixed solves whose planes are 16-byte aligned
    {
        const int* it = p->comp.it;
        const bool three_d = it[0] > 1 && it[1] > 1 && it[2] > 1;
        // its interior rows are the 5-point ones (sym5, or antisymmetric)
        bool w5 = true;
        for (int a = 0; a < 3; a++) w5 = w5 && (!p->op.ax[a].active || p->op.ax[a].width == 5);
        if (prec == PREC_MIXED && three_d && w5 && it[2] % 16 == 0 && N < (1LL << 31) - 64 &&
            !std::getenv("SHOCCS_DISABLE_TMA")) {
            float* hi = (float*)S->b.u0;
            S->b.tma = make_plane_map(&S->b.tm_u0, hi, 4, it) &&
                       make_plane_map(&S->b.tm_sa, S->b.sa, 4, it) &&
                       make_plane_map(&S->b.tm_sb, S->b.sb, 4, it) &&
                       make_plane_map(&S->b.tm_u0t, hi, 4, it, false) &&
                       make_plane_map(&S->b.tm_u0l, hi + N, 4, it, false) &&
                       make_plane_map(&S->b.tm_acct, S->b.acc, 4, it, false) &&
                       make_plane_map(&S->b.tm_cls, (void*)p->op.cls, 1, it, false);
        }
        // the trial steps of the autotuner need every register allocated and zeroed; the
        // column and vectorised kernels index with 32-bit integers
        if (const char* f = std::getenv("SHOCCS_CUT_ROWS_FP64")) S->b.cut_fp64 = std::atoi(f) != 0;
        if (prec == PREC_MIXED && three_d && N < (1LL << 31) - 64) {
            // the vectorised stage: cut-cell row values at their points, line records; the
            // cut-row kernel runs one thread per cut-cell row and per z line
            const long long nthreads = (long long)it[0] * it[1] + p->op.n_cut_rows;
            if (it[2] % 4 == 0 && line_records_fit(p->op) && nthreads < (1LL << 31) - 256) {
                void* z = nullptr;
                SH_CUDA(S->mem.alloc((size_t)3 * N * sizeof(float), &z));
                S->b.rowv = (float*)z;
                SH_CUDA(S->mem.alloc((size_t)it[0] * it[1] * LREC_WORDS * sizeof(float), &z));
                S->b.lrec = (float*)z;
            }
            if (auto st = autotune_stage_kernel(S.get(), s); st != SHOCCS_OK) return st;
        }
    }
    SH_CUDA(cudaStreamSynchronize(s));
    *out = S.release();
    return SHOCCS_OK;
}

shoccs_status shoccs_system_destroy(shoccs_system* s)
{
    delete s;
    return SHOCCS_OK;
}

shoccs_status shoccs_system_initialize(shoccs_system* S, double t, void* stream)
{
    if (!S) return fail(SHOCCS_EINVAL, "null system");
    const cudaStream_t s = (cudaStream_t)stream;
    SH_CUDA(launch_initialize(S->P->op, S->P->dr, S->sp.sol, S->desc.prec, t, S->b.u0, S->b.R, s));
    SH_CUDA(cudaStreamSynchronize(s));
    S->t = t;
    return SHOCCS_OK;
}

shoccs_status shoccs_system_set_state(shoccs_system* S, const shoccs_field* u, int where,
                                      void* stream)
{
    if (!S || !u || !u->D) return fail(SHOCCS_EINVAL, "null argument");
    const cudaStream_t s = (cudaStream_t)stream;
    const long long N = S->P->mesh.size();
    const cudaMemcpyKind kind = where == 0 ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    if (S->desc.prec == PREC_FP64) {
        SH_CUDA(cudaMemcpyAsync(S->b.u0, u->D, N * 8, kind, s));
    } else {
        // stage the FP64 input through the stage-field block (2 x N x 4 bytes = N doubles)
        void* tmp = S->b.sa;
        SH_CUDA(cudaMemcpyAsync(tmp, u->D, N * 8, kind, s));
        SH_CUDA(launch_state_convert(N, 1, (const double*)tmp, S->b.u0, nullptr, nullptr, s));
    }
    const void* R[3] = {u->Rx, u->Ry, u->Rz};
    for (int r = 0; r < 3; r++) {
        const size_t n = S->P->mesh.R[r].size();
        if (n && R[r]) SH_CUDA(cudaMemcpyAsync(S->b.R[r], R[r], n * 8, kind, s));
    }
    SH_CUDA(cudaStreamSynchronize(s));
    return SHOCCS_OK;
}

shoccs_status shoccs_system_get_state(shoccs_system* S, shoccs_field* u, int where,
                                      void* stream)
{
    if (!S || !u || !u->D) return fail(SHOCCS_EINVAL, "null argument");
    const cudaStream_t s = (cudaStream_t)stream;
    const long long N = S->P->mesh.size();
    const cudaMemcpyKind kind = where == 0 ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
    if (S->desc.prec == PREC_FP64) {
        SH_CUDA(cudaMemcpyAsync(u->D, S->b.u0, N * 8, kind, s));
    } else {
        void* tmp = S->b.sa;
        SH_CUDA(launch_state_convert(N, 0, nullptr, nullptr, S->b.u0, (double*)tmp, s));
        SH_CUDA(cudaMemcpyAsync(u->D, tmp, N * 8, kind, s));
    }
    void* R[3] = {u->Rx, u->Ry, u->Rz};
    for (int r = 0; r < 3; r++) {
        const size_t n = S->P->mesh.R[r].size();
        if (n && R[r]) SH_CUDA(cudaMemcpyAsync(R[r], S->b.R[r], n * 8, kind, s));
    }
    SH_CUDA(cudaStreamSynchronize(s));
    return SHOCCS_OK;
}

shoccs_status shoccs_system_error_field(shoccs_system* S, double t, shoccs_field* err, int where,
                                        void* stream)
{
    if (!S || !err || !err->D) return fail(SHOCCS_EINVAL, "null argument");
    if (where != 0 && where != 1) return fail(SHOCCS_EINVAL, "where must be 0 (host) or 1 (device)");
    const cudaStream_t s = (cudaStream_t)stream;
    const long long N = S->P->mesh.size();
    long long nR[3], total = N;
    void* out[4] = {err->D, err->Rx, err->Ry, err->Rz};
    for (int r = 0; r < 3; r++) {
        nR[r] = (long long)S->P->mesh.R[r].size();
        if (nR[r] && !out[1 + r]) return fail(SHOCCS_EINVAL, "null cut-point buffer");
        total += nR[r];
    }
    double* tmp = nullptr;
    FieldF64 f{};
    if (where == 1) {
        f = FieldF64{(double*)err->D, {(double*)err->Rx, (double*)err->Ry, (double*)err->Rz}};
    } else {
        SH_CUDA(cudaMallocAsync((void**)&tmp, total * sizeof(double), s));
        f.D = tmp;
        long long off = N;
        for (int r = 0; r < 3; r++) {
            f.R[r] = tmp + off;
            off += nR[r];
        }
    }
    cudaError_t e = launch_error_field(S->P->op, S->P->dr, S->sp.sol, S->desc.prec, S->b.u0, S->b.R,
                                       t, f, s);
    if (where == 0) {
        if (e == cudaSuccess) e = cudaMemcpyAsync(out[0], f.D, N * 8, cudaMemcpyDeviceToHost, s);
        for (int r = 0; r < 3; r++)
            if (e == cudaSuccess && nR[r])
                e = cudaMemcpyAsync(out[1 + r], f.R[r], nR[r] * 8, cudaMemcpyDeviceToHost, s);
        cudaFreeAsync(tmp, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(SHOCCS_ECUDA, std::string("error field: ") + cudaGetErrorString(e));
    return SHOCCS_OK;
}

static shoccs_status check_wait_flag(shoccs_system* S, cudaStream_t s)
{
    if (!S->b.tma) return SHOCCS_OK;
    unsigned flag = 0;
    SH_CUDA(cudaMemcpyAsync(&flag, S->b.err, sizeof flag, cudaMemcpyDeviceToHost, s));
    SH_CUDA(cudaStreamSynchronize(s));
    if (flag) {
        SH_CUDA(cudaMemsetAsync(S->b.err, 0, sizeof flag, s));
        return fail(SHOCCS_ETIMEOUT, "a stage kernel's bounded wait for its TMA copies gave up");
    }
    return SHOCCS_OK;
}

shoccs_status shoccs_system_rk4(shoccs_system* S, double t0, double dt, int nsteps,
                                void* stream)
{
    if (!S || nsteps < 0 || !(dt > 0)) return fail(SHOCCS_EINVAL, "bad argument");
    const cudaStream_t s = (cudaStream_t)stream;
    double t = t0;
    for (int i = 0; i < nsteps; i++) {
        if (S->unfused)
            SH_CUDA(launch_step_unfused(S->P->op, S->P->dr, S->sp, S->ux, S->state(), S->fy,
                                             S->fk, S->facc, t, dt, s));
        else
            SH_CUDA(launch_rk4_step(S->P->op, S->P->dr, S->sp, S->desc.prec, S->b, t, dt, s,
                                    nullptr, i + 1 < nsteps));
        t += dt; // step_controller advance (src/simulation/simulation_cycle.cpp:97)
    }
    SH_CUDA(cudaStreamSynchronize(s));
    S->t = t;
    return check_wait_flag(S, s);
}

shoccs_status shoccs_system_euler(shoccs_system* S, double t0, double dt, int nsteps,
                                  void* stream)
{
    if (!S || nsteps < 0 || !(dt > 0)) return fail(SHOCCS_EINVAL, "bad argument");
    if (S->desc.prec != PREC_FP64 || S->ux.mixed)
        return fail(SHOCCS_EUNSUPPORTED, "the forward Euler integrator steps FP64 systems");
    const cudaStream_t s = (cudaStream_t)stream;
    // the right-hand side's scratch: the unfused step's whole-field register, or (fused
    // systems) the stage field sa and the Rhalf arrays, which every RK4 step rewrites
    const FieldF64 K = S->unfused ? S->fk
                                  : FieldF64{(double*)S->b.sa, {S->b.Rhalf[0], S->b.Rhalf[1], S->b.Rhalf[2]}};
    double t = t0;
    for (int i = 0; i < nsteps; i++) {
        SH_CUDA(launch_euler_fp64(S->P->op, S->P->dr, S->sp, S->ux, S->unfused, S->b, S->state(), K, t, dt, s));
        t += dt;
    }
    SH_CUDA(cudaStreamSynchronize(s));
    S->t = t;
    return SHOCCS_OK;
}

shoccs_status shoccs_system_rk4_timed(shoccs_system* S, double t0, double dt, int nsteps,
                                      void* stream, double kernel_ms[6])
{
    if (!S || nsteps < 1 || !(dt > 0) || !kernel_ms) return fail(SHOCCS_EINVAL, "bad argument");
    const cudaStream_t s = (cudaStream_t)stream;
    if (S->unfused) { // no fused stage kernels to time: the whole run is kernel_ms[0]
        cudaEvent_t a, z;
        SH_CUDA(cudaEventCreate(&a));
        SH_CUDA(cudaEventCreate(&z));
        SH_CUDA(cudaEventRecord(a, s));
        const shoccs_status st = shoccs_system_rk4(S, t0, dt, nsteps, stream);
        float ms = 0.f;
        if (st == SHOCCS_OK) {
            cudaEventRecord(z, s);
            cudaEventSynchronize(z);
            cudaEventElapsedTime(&ms, a, z);
        }
        cudaEventDestroy(a);
        cudaEventDestroy(z);
        for (int k = 0; k < 6; k++) kernel_ms[k] = 0.0;
        kernel_ms[0] = kernel_ms[5] = ms;
        return st;
    }
    constexpr int EV = 10;
    std::vector<cudaEvent_t> ev(EV * (size_t)nsteps, nullptr);
    shoccs_status st = SHOCCS_OK;
    for (auto& e : ev)
        if (cudaEventCreate(&e) != cudaSuccess) {
            st = fail(SHOCCS_ECUDA, "cudaEventCreate failed");
            break;
        }
    double t = t0;
    for (int i = 0; st == SHOCCS_OK && i < nsteps; i++) {
        cudaError_t e = launch_rk4_step(S->P->op, S->P->dr, S->sp, S->desc.prec, S->b, t, dt,
                                        s, ev.data() + EV * (size_t)i, i + 1 < nsteps);
        if (e != cudaSuccess) st = fail(SHOCCS_ECUDA, cudaGetErrorString(e));
        t += dt;
    }
    if (st == SHOCCS_OK && cudaStreamSynchronize(s) != cudaSuccess)
        st = fail(SHOCCS_ECUDA, "stream synchronize failed");
    if (st == SHOCCS_OK) {
        for (int k = 0; k < 6; k++) kernel_ms[k] = 0.0;
        for (int i = 0; i < nsteps; i++) {
            cudaEvent_t* e = ev.data() + EV * (size_t)i;
            for (int k = 0; k < 4; k++) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e[2 + 2 * k], e[3 + 2 * k]);
                kernel_ms[1 + k] += ms;
            }
        }
        // the run ends with the last stage's face kernel: time it up to the run's end
        cudaEvent_t end;
        float all = 0.f;
        if (cudaEventCreate(&end) == cudaSuccess) {
            cudaEventRecord(end, s);
            cudaEventSynchronize(end);
            cudaEventElapsedTime(&all, ev.front(), end);
            cudaEventDestroy(end);
        }
        kernel_ms[5] = all;
        kernel_ms[0] = all - (kernel_ms[1] + kernel_ms[2] + kernel_ms[3] + kernel_ms[4]);
        S->t = t;
    }
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    if (st == SHOCCS_OK) st = check_wait_flag(S, s);
    return st;
}

shoccs_status shoccs_system_rhs(shoccs_system* S, double t, shoccs_field* rhs, void* stream)
{
    if (!S || !rhs || !rhs->D) return fail(SHOCCS_EINVAL, "null argument");
    const cudaStream_t s = (cudaStream_t)stream;
    double* outR[3] = {(double*)rhs->Rx, (double*)rhs->Ry, (double*)rhs->Rz};
    if (S->unfused)
        SH_CUDA(launch_rhs_unfused(S->P->op, S->P->dr, S->sp, S->ux, S->state(), t,
                                        FieldF64{(double*)rhs->D, {outR[0], outR[1], outR[2]}}, s));
    else
        SH_CUDA(launch_rhs(S->P->op, S->sp, S->desc.prec, S->b, t, (double*)rhs->D, outR, s));
    SH_CUDA(cudaStreamSynchronize(s));
    return SHOCCS_OK;
}

shoccs_status shoccs_system_stats(shoccs_system* S, double t, double out[11], void* stream)
{
    if (!S || !out) return fail(SHOCCS_EINVAL, "null argument");
    const cudaStream_t s = (cudaStream_t)stream;
    double* dev = nullptr;
    SH_CUDA(cudaMallocAsync((void**)&dev, 16 * sizeof(double), s));
    cudaError_t e = launch_stats(S->P->op, S->P->dr, S->sp.sol, S->desc.prec, S->b.u0, S->b.R, t,
                                 dev, s);
    if (e == cudaSuccess && S->unfused) e = launch_stats_r(S->P->op, S->P->dr, S->sp.sol, S->b.R, t, dev + 4, s);
    double h[16] = {};
    if (e == cudaSuccess) e = cudaMemcpyAsync(h, dev, sizeof h, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(dev, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return fail(SHOCCS_ECUDA, std::string("stats: ") + cudaGetErrorString(e));
    // compute_scalar_stats visits the fluid D points and the non-Dirichlet cut points; a
    // system whose objects are all Dirichlet has no such cut point, so its R statistics are 0
    const bool fluid = S->P->comp.n_fluid > 0;
    out[0] = h[0];
    out[1] = fluid ? h[2] : 0.0;
    out[2] = fluid ? h[3] : 0.0;
    out[3] = h[0];
    out[4] = h[1];
    for (int i = 5; i < 11; i++) out[i] = 0.0;
    if (S->unfused) {
        bool any = fluid;
        for (int d = 0; d < 3; d++) {
            const double* r = h + 4 + 4 * d; // {err, index (-1: none), min, max}
            if (r[1] < 0) continue;
            out[5 + 2 * d] = r[0];
            out[6 + 2 * d] = r[1];
            out[0] = std::max(out[0], r[0]);
            out[1] = any ? std::min(out[1], r[2]) : r[2];
            out[2] = any ? std::max(out[2], r[3]) : r[3];
            any = true;
        }
    }
    const double bound = S->desc.kind == SHOCCS_SYS_HEAT ? 1e6 : S->desc.max_error;
    if (!std::isfinite(out[0]) || std::abs(out[0]) > bound)
        return fail(SHOCCS_ENONFINITE, "solution error is non-finite or above its bound");
    return SHOCCS_OK;
}

shoccs_status shoccs_system_stats_noalloc(shoccs_system* S, double t, double out[11],
                                          void* stream)
{
    if (!S || !out) return fail(SHOCCS_EINVAL, "null argument");
    if (S->unfused)
        return fail(SHOCCS_EUNSUPPORTED, "shoccs_system_stats_noalloc covers systems whose "
                                         "objects are all Dirichlet; use shoccs_system_stats");
    const DevOp& op = S->P->op;
    const long long tiles = (long long)op.nzc * ((op.it1 + 7) / 8) * op.it0;
    if (tiles > stats_noalloc_max_tiles())
        return fail(SHOCCS_EINVAL,
                    "shoccs_system_stats_noalloc: the grid has " + std::to_string(tiles) +
                        " tiles of 256 points; its fixed scratch holds at most " +
                        std::to_string(stats_noalloc_max_tiles()) +
                        " (16.7 M points); use shoccs_system_stats");
    double h[4] = {0, 0, 0, 0};
    const cudaError_t e = launch_stats_noalloc(op, S->sp.sol, S->desc.prec, S->b.u0, t, h,
                                               (cudaStream_t)stream);
    if (e != cudaSuccess)
        return fail(SHOCCS_ECUDA, std::string("stats_noalloc: ") + cudaGetErrorString(e));
    out[0] = h[0];
    out[1] = S->P->comp.n_fluid ? h[2] : 0.0;
    out[2] = S->P->comp.n_fluid ? h[3] : 0.0;
    out[3] = h[0];
    out[4] = h[1];
    for (int i = 5; i < 11; i++) out[i] = 0.0;
    const double bound = S->desc.kind == SHOCCS_SYS_HEAT ? 1e6 : S->desc.max_error;
    if (!std::isfinite(out[0]) || std::abs(out[0]) > bound)
        return fail(SHOCCS_ENONFINITE, "solution error is non-finite or above its bound");
    return SHOCCS_OK;
}

// ---------------------------------------------------------------------------------------
// captured graphs: the recorded applies are launched, in order, on a private capturing
// stream (the launchers below issue kernels and memsets only; every allocation and upload
// happens when an apply is added), and the capture is instantiated -- or, after the first
// capture, applied to the instantiated graph with cudaGraphExecUpdate.
// ---------------------------------------------------------------------------------------
struct shoccs_graph {
    struct op {
        bool timed; // depends on the submit's time (a system right-hand side)
        std::function<cudaError_t(cudaStream_t, double)> run;
        // the buffers the op reads that may move between submits (a system's state and its
        // cut-point values, which its RK4 steps exchange with their next-step copies)
        std::function<std::array<const void*, 4>()> inputs;
        std::array<const void*, 4> captured{};
    };
    std::vector<op> ops;
    cudaStream_t cap = nullptr;
    cudaGraphExec_t exec = nullptr;
    double t_captured = 0.0;
    bool stale = true;
    int64_t nodes = 0, captures = 0;
    ~shoccs_graph()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (cap) cudaStreamDestroy(cap);
    }
};

shoccs_status shoccs_graph_create(shoccs_graph** out)
{
    if (!out) return fail(SHOCCS_EINVAL, "null argument");
    *out = nullptr;
    auto g = std::make_unique<shoccs_graph>();
    SH_CUDA(cudaStreamCreateWithFlags(&g->cap, cudaStreamNonBlocking));
    *out = g.release();
    return SHOCCS_OK;
}

shoccs_status shoccs_graph_destroy(shoccs_graph* g)
{
    delete g;
    return SHOCCS_OK;
}

namespace
{
// the problem's device tables (and, for the FP32 operators, their scratch) before capture
shoccs_status graph_prepare(shoccs_graph* g, shoccs_problem* p, int prec)
{
    if (auto st = do_upload(p, g->cap); st != SHOCCS_OK) return st;
    if (prec == PREC_MIXED)
        if (auto st = ensure_op_scratch(p); st != SHOCCS_OK) return st;
    g->stale = true;
    return SHOCCS_OK;
}
struct field_ptrs {
    void* D;
    void* R[3];
    explicit field_ptrs(const shoccs_field* f) : D{f ? f->D : nullptr}, R{nullptr, nullptr, nullptr}
    {
        if (f) {
            R[0] = f->Rx;
            R[1] = f->Ry;
            R[2] = f->Rz;
        }
    }
};
} // namespace

shoccs_status shoccs_graph_add_derivative(shoccs_graph* g, shoccs_problem* p, int dir, int prec,
                                          const shoccs_field* u, const shoccs_field* nu,
                                          shoccs_field* du, int plus_eq)
{
    if (!g || !p || !u || !du || dir < 0 || dir > 2 || (prec != 0 && prec != 1))
        return fail(SHOCCS_EINVAL, "bad argument");
    if (auto st = graph_prepare(g, p, prec); st != SHOCCS_OK) return st;
    const field_ptrs fu{u}, fdu{du};
    const double* nuD = nu ? (const double*)nu->D : nullptr;
    g->ops.push_back({false, [p, dir, prec, fu, fdu, nuD, plus_eq](cudaStream_t s, double) {
                          const void* uR[3] = {fu.R[0], fu.R[1], fu.R[2]};
                          void* duR[3] = {fdu.R[0], fdu.R[1], fdu.R[2]};
                          return launch_derivative(p->op, dir, prec, fu.D, uR[dir], nuD, fdu.D, duR,
                                                   uR, plus_eq, s);
                      },
                      {},
                      {}});
    return SHOCCS_OK;
}

shoccs_status shoccs_graph_add_laplacian(shoccs_graph* g, shoccs_problem* p, int prec,
                                         const shoccs_field* u, const shoccs_field* nu,
                                         shoccs_field* du)
{
    if (!g || !p || !u || !du || (prec != 0 && prec != 1)) return fail(SHOCCS_EINVAL, "bad argument");
    if (auto st = graph_prepare(g, p, prec); st != SHOCCS_OK) return st;
    const field_ptrs fu{u}, fdu{du};
    const double* nuD = nu ? (const double*)nu->D : nullptr;
    g->ops.push_back({false, [p, prec, fu, fdu, nuD](cudaStream_t s, double) {
                          const void* uR[3] = {fu.R[0], fu.R[1], fu.R[2]};
                          void* duR[3] = {fdu.R[0], fdu.R[1], fdu.R[2]};
                          return launch_laplacian(p->op, prec, fu.D, uR, nuD, fdu.D, duR, s);
                      },
                      {},
                      {}});
    return SHOCCS_OK;
}

shoccs_status shoccs_graph_add_gradient(shoccs_graph* g, shoccs_problem* p, int prec,
                                        const shoccs_field* u, shoccs_field* dx, shoccs_field* dy,
                                        shoccs_field* dz)
{
    if (!g || !p || !u || !dx || !dy || !dz || (prec != 0 && prec != 1))
        return fail(SHOCCS_EINVAL, "bad argument");
    if (auto st = graph_prepare(g, p, prec); st != SHOCCS_OK) return st;
    const field_ptrs fu{u}, fx{dx}, fy{dy}, fz{dz};
    g->ops.push_back({false, [p, prec, fu, fx, fy, fz](cudaStream_t s, double) {
                          const void* uR[3] = {fu.R[0], fu.R[1], fu.R[2]};
                          void* const out[3][4] = {{fx.D, fx.R[0], fx.R[1], fx.R[2]},
                                                   {fy.D, fy.R[0], fy.R[1], fy.R[2]},
                                                   {fz.D, fz.R[0], fz.R[1], fz.R[2]}};
                          return launch_gradient(p->op, prec, fu.D, uR, out, s);
                      },
                      {},
                      {}});
    return SHOCCS_OK;
}

shoccs_status shoccs_graph_add_rhs(shoccs_graph* g, shoccs_system* S, shoccs_field* rhs)
{
    if (!g || !S || !rhs || !rhs->D) return fail(SHOCCS_EINVAL, "null argument");
    const field_ptrs fr{rhs};
    g->stale = true;
    g->ops.push_back({true,
                      [S, fr](cudaStream_t s, double t) {
                          double* outR[3] = {(double*)fr.R[0], (double*)fr.R[1], (double*)fr.R[2]};
                          if (S->unfused)
                              return launch_rhs_unfused(S->P->op, S->P->dr, S->sp, S->ux, S->state(), t,
                                                             FieldF64{(double*)fr.D, {outR[0], outR[1], outR[2]}},
                                                             s);
                          return launch_rhs(S->P->op, S->sp, S->desc.prec, S->b, t, (double*)fr.D, outR, s);
                      },
                      [S]() {
                          return std::array<const void*, 4>{S->b.u0, S->b.R[0], S->b.R[1], S->b.R[2]};
                      },
                      {}});
    return SHOCCS_OK;
}

shoccs_status shoccs_graph_submit(shoccs_graph* g, double t, void* stream)
{
    if (!g) return fail(SHOCCS_EINVAL, "null graph");
    const cudaStream_t s = (cudaStream_t)stream;
    bool timed = false, moved = false;
    for (const auto& o : g->ops) {
        timed = timed || o.timed;
        if (o.inputs) moved = moved || o.inputs() != o.captured;
    }
    if (g->stale || !g->exec || moved || (timed && t != g->t_captured)) {
        for (auto& o : g->ops)
            if (o.inputs) o.captured = o.inputs();
        SH_CUDA(cudaStreamBeginCapture(g->cap, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        for (const auto& o : g->ops) {
            e = o.run(g->cap, t);
            if (e != cudaSuccess) break;
        }
        cudaGraph_t graph = nullptr;
        const cudaError_t e_end = cudaStreamEndCapture(g->cap, &graph);
        if (e == cudaSuccess) e = e_end;
        if (e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            return fail(SHOCCS_ECUDA, std::string("graph capture: ") + cudaGetErrorString(e));
        }
        size_t n = 0;
        cudaGraphGetNodes(graph, nullptr, &n);
        bool updated = false;
        if (g->exec) {
            cudaGraphExecUpdateResultInfo info{};
            updated = cudaGraphExecUpdate(g->exec, graph, &info) == cudaSuccess;
            if (!updated) {
                cudaGetLastError();
                cudaGraphExecDestroy(g->exec);
                g->exec = nullptr;
            }
        }
        if (!updated) e = cudaGraphInstantiate(&g->exec, graph, 0);
        cudaGraphDestroy(graph);
        SH_CUDA(e);
        g->nodes = (int64_t)n;
        g->t_captured = t;
        g->stale = false;
        g->captures++;
    }
    SH_CUDA(cudaGraphLaunch(g->exec, s));
    SH_CUDA(cudaStreamSynchronize(s));
    return SHOCCS_OK;
}

shoccs_status shoccs_graph_info(const shoccs_graph* g, int64_t info[3])
{
    if (!g || !info) return fail(SHOCCS_EINVAL, "null argument");
    info[0] = (int64_t)g->ops.size();
    info[1] = g->nodes;
    info[2] = g->captures;
    return SHOCCS_OK;
}

shoccs_status shoccs_system_path(const shoccs_system* S, int* kernel)
{
    if (!S || !kernel) return fail(SHOCCS_EINVAL, "null argument");
    const StepBuffers& b = S->b;
    *kernel = S->unfused           ? 7
              : b.tma              ? 1
              : b.col_nx == 1      ? 2
              : b.col_nx == 2      ? 3
              : b.col_nx == 4      ? 4
              : b.vec_px == 2      ? 8
              : b.vec_px == 4      ? 9
              : b.vec              ? (b.vec_minb == 4 ? 5 : 6)
                                   : 0;
    return SHOCCS_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------------------
// batched heat solves
// ---------------------------------------------------------------------------------------
struct shoccs_batch {
    std::vector<shoccs_system*> sys;
    int prec = 0;
    DeviceAlloc mem;
    std::vector<BatchInst> h_inst;
    BatchInst* d_inst = nullptr;
    const int* d_row_inst = nullptr;
    int n_rows = 0;
    const int4* d_tiles[4] = {}; // (instance, it0 index, first it1 index, it2 chunk)
    int n_tiles[4] = {};
    // 2-D instances go to the flat stage: warp tiles (instance, first point) of BATCH2D_TILE points
    const int2* d_wtiles = nullptr;
    int n_wtiles = 0, grid2d = 1;
    // or to the split stage (uniform tiles, special points; no cut-cell row pass)
    BatchSplit split;
    // every instance split: groups of consecutive instances whose fields fit well inside L2
    // (SHOCCS_BATCH_GROUP_MB), each advanced through all its steps before the next, so that
    // a group's stages find their inputs in L2 (instances are independent: the order of
    // their work does not matter)
    std::vector<BatchSplit> groups;
    // every instance split 2-D and SHOCCS_BATCH_PERSIST=1: the whole solve in one persistent
    // launch of n_clusters clusters (kernels.cu k_batch_persist), cluster c owning the
    // instances of ctab[c]
    bool persist = false;
    int n_clusters = 0;
    const int4* d_psp = nullptr;
    const int2* d_put = nullptr;
    const int4* d_ctab = nullptr;
    const int* d_r_inst = nullptr;
    int n_r = 0;
    int cfg = 3, grid = 1;
    BatchTime* d_times = nullptr;
    long long times_cap = 0; // steps the time table holds
    cudaStream_t cap = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_steps = 0;
    int64_t graph_nodes = 0;
    ~shoccs_batch()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (cap) cudaStreamDestroy(cap);
        if (split.aux) cudaStreamDestroy(split.aux);
        if (split.fork) cudaEventDestroy(split.fork);
        if (split.join) cudaEventDestroy(split.join);
    }
};

namespace
{
constexpr double RKI[4] = {0.0, 0.5, 0.5, 1.0}; // src/temporal/rk4.cpp:11-12
constexpr double RKF[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};

shoccs_status batch_set_steps(shoccs_batch* B, const double* t0, const double* dt, int nsteps,
                              cudaStream_t s)
{
    const int n = (int)B->sys.size();
    // the time points and e^-t of every step, as shoccs_system_rk4 forms them
    std::vector<BatchTime> h((size_t)nsteps * n);
    for (int i = 0; i < n; i++) {
        double t = t0[i];
        for (int k = 0; k < nsteps; k++) {
            BatchTime& bt = h[(size_t)k * n + i];
            bt.t[0] = t + dt[i] * RKI[0];
            bt.t[1] = t + dt[i] * RKI[1];
            bt.t[2] = t + dt[i] * RKI[3];
            for (int m = 0; m < 3; m++) bt.et[m] = std::exp(-bt.t[m]);
            t += dt[i];
        }
        BatchInst& I = B->h_inst[i];
        for (int st = 0; st < 4; st++) {
            I.cf[st] = dt[i] * RKF[st];
            I.ci[st] = st < 3 ? dt[i] * RKI[st + 1] : 1.0;
            const float ch = (float)I.cf[st], ih = (float)I.ci[st];
            I.cf_ff[st] = make_float2(ch, (float)(I.cf[st] - (double)ch));
            I.ci_ff[st] = make_float2(ih, (float)(I.ci[st] - (double)ih));
        }
    }
    if ((long long)nsteps > B->times_cap) {
        void* p = nullptr;
        SH_CUDA(B->mem.alloc(h.size() * sizeof(BatchTime), &p));
        B->d_times = (BatchTime*)p;
        B->times_cap = nsteps;
        if (B->exec) { // the captured graph points at the old table
            cudaGraphExecDestroy(B->exec);
            B->exec = nullptr;
            B->graph_steps = 0;
        }
    }
    SH_CUDA(cudaMemcpyAsync(B->d_times, h.data(), h.size() * sizeof(BatchTime),
                            cudaMemcpyHostToDevice, s));
    SH_CUDA(cudaMemcpyAsync(B->d_inst, B->h_inst.data(), n * sizeof(BatchInst),
                            cudaMemcpyHostToDevice, s));
    return SHOCCS_OK;
}

// pick the tile shape: time a stage-1 pass of every candidate (stage 1 writes only the
// accumulator and a stage field, which hold nothing between runs)
shoccs_status batch_autotune(shoccs_batch* B, cudaStream_t s)
{
    const int n = (int)B->sys.size();
    std::vector<double> t0(n, 0.0), dt(n, 1e-6);
    if (auto st = batch_set_steps(B, t0.data(), dt.data(), 1, s); st != SHOCCS_OK) return st;
    if (const char* f = std::getenv("SHOCCS_BATCH_TILE_WARPS")) {
        for (int c = 0; c < 4; c++)
            if (std::atoi(f) == BATCH_TILE_WARPS[c]) {
                B->cfg = c;
                B->grid = batch_stage_grid(c, B->prec, B->n_tiles[c]);
                return SHOCCS_OK;
            }
        return fail(SHOCCS_EINVAL, "SHOCCS_BATCH_TILE_WARPS must be 1, 2, 4 or 8");
    }
    if (B->n_tiles[0] == 0) return SHOCCS_OK; // every instance takes the flat 2-D stage
    cudaEvent_t e0, e1;
    SH_CUDA(cudaEventCreate(&e0));
    SH_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int c = 0; c < 4; c++) {
        const int grid = batch_stage_grid(c, B->prec, B->n_tiles[c]);
        SH_CUDA(launch_batch_probe(B->d_inst, B->d_tiles[c], B->n_tiles[c], c, grid,
                                   B->d_times, B->prec, s));
        SH_CUDA(cudaEventRecord(e0, s));
        for (int r = 0; r < 5; r++)
            SH_CUDA(launch_batch_probe(B->d_inst, B->d_tiles[c], B->n_tiles[c], c, grid,
                                       B->d_times, B->prec, s));
        SH_CUDA(cudaEventRecord(e1, s));
        SH_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        SH_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) {
            best = ms;
            B->cfg = c;
            B->grid = grid;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return SHOCCS_OK;
}
} // namespace

extern "C" {

shoccs_status shoccs_batch_create(shoccs_system* const* systems, int n, shoccs_batch** out)
{
    if (!systems || n < 1 || !out) return fail(SHOCCS_EINVAL, "bad argument");
    *out = nullptr;
    auto B = std::make_unique<shoccs_batch>();
    B->prec = systems[0] ? systems[0]->desc.prec : 0;
    int dev = 0;
    SH_CUDA(cudaGetDevice(&dev));
    std::vector<int> row_inst, r_inst;
    std::vector<int4> tiles[4];
    std::vector<int2> wtiles;
    std::vector<int2> ut;
    std::vector<int4> sp;
    std::vector<int> sp_kind; // row kinds along it1, it2 and the face bit of each special point
    std::vector<std::pair<int, int>> inst_ut(n), inst_sp(n); // (begin, end) of each instance
    bool all2d = true;
    // SHOCCS_BATCH_KERNEL=point sends every instance through the per-point stage, =flat the
    // 2-D instances through the flat stage, =split through the split stage.  By default the
    // 2-D instances of a mixed batch take the split stage and FP64 batches the per-point
    // stage (with FP64 arithmetic at a small fraction of the FP32 rate, the 2-D forms'
    // register-heavy bodies measured slower there: 212 ms against 164 ms for the batched
    // configuration's 200 steps)
    const char* kenv = std::getenv("SHOCCS_BATCH_KERNEL");
    const std::string kname =
        kenv ? std::string(kenv) : std::string(B->prec == PREC_MIXED ? "split" : "point");
    const bool allow2d = kname == "flat" || kname == "split";
    const bool use_split = kname == "split";
    for (int i = 0; i < n; i++) {
        shoccs_system* S = systems[i];
        if (!S) return fail(SHOCCS_EINVAL, "null system");
        for (int k = 0; k < i; k++)
            if (systems[k] == S) return fail(SHOCCS_EINVAL, "a system appears twice in the batch");
        if (S->desc.kind != SHOCCS_SYS_HEAT || S->desc.sol_kind != SHOCCS_SOL_SINSIN)
            return fail(SHOCCS_EUNSUPPORTED,
                        "batched solves take heat systems with the sin-sin manufactured solution");
        if (S->desc.prec != B->prec) return fail(SHOCCS_EINVAL, "mixed precisions in one batch");
        if (S->unfused)
            return fail(SHOCCS_EUNSUPPORTED, "batched solves take systems whose objects are all Dirichlet");
        if (S->P->device != dev) return fail(SHOCCS_EINVAL, "systems on different devices");
        for (int a = 0; a < 3; a++)
            if (S->P->op.ax[a].active && S->P->op.ax[a].width > 5)
                return fail(SHOCCS_EUNSUPPORTED, "batched solves take interiors of up to 5 points");
        const DevOp& op = S->P->op;
        if (op.N >= (1LL << 31) - 64) return fail(SHOCCS_EUNSUPPORTED, "instance above 2^31 points");
        B->sys.push_back(S);
        BatchInst I{};
        I.op = op;
        I.sp = S->sp;
        I.u0 = S->b.u0;
        I.acc = S->b.acc;
        I.sa = S->b.sa;
        I.sb = S->b.sb;
        I.cval = S->b.cval;
        for (int d = 0; d < 3; d++) I.R[d] = S->b.R[d];
        I.row0 = (int)row_inst.size();
        const bool flat2d = allow2d && op.it0 == 1 && op.it1 > 1 && op.phys_of_it[1] >= 0 &&
                            op.phys_of_it[2] >= 0 && op.N < (1LL << 31) - 256;
        all2d = all2d && flat2d;
        if (flat2d && !use_split) {
            // cut-cell row values at their points, per axis (3 x N, the batch's own buffer)
            void* rv = nullptr;
            const size_t elem = B->prec == PREC_MIXED ? sizeof(float) : sizeof(double);
            SH_CUDA(B->mem.alloc((size_t)3 * op.N * elem, &rv));
            SH_CUDA(cudaMemset(rv, 0, (size_t)3 * op.N * elem));
            I.rowv = rv;
        }
        if (flat2d && use_split && B->prec == PREC_MIXED && op.phys_of_it[1] == 0 &&
            op.phys_of_it[2] == 1 && S->sp.sol.kind == SHOCCS_SOL_SINSIN && S->sp.sol.dims != 3) {
            // the source's spatial factor at every point (the batch's own buffer)
            void* s2 = nullptr;
            SH_CUDA(B->mem.alloc((size_t)op.N * sizeof(float), &s2));
            SH_CUDA(launch_sinsin_xy(S->sp.sol.Sf[0], S->sp.sol.Sf[1], op.it1, op.it2, (float*)s2, nullptr));
            I.s2f = (const float*)s2;
        }
        if (flat2d) {
            if ((long long)wtiles.size() + op.N / BATCH2D_TILE + 1 >= (1LL << 31))
                return fail(SHOCCS_EUNSUPPORTED, "batch above 2^31 tiles");
            if (use_split) {
                inst_ut[i].first = (int)ut.size();
                for (long long t = 0; t < op.N; t += BATCH_UTILE) ut.push_back(make_int2(i, (int)t));
                inst_ut[i].second = (int)ut.size();
                // special points: a wall or cut-cell row along either axis, or a Dirichlet face
                const Compiled& cp = S->P->comp;
                const int da = op.phys_of_it[1], db = op.phys_of_it[2];
                auto row_of = [&](int d, long long q) {
                    const auto& ro = cp.ax[d].row_out;
                    const auto it = std::lower_bound(ro.begin(), ro.end(), (i64)q);
                    return it != ro.end() && *it == q ? (int)(it - ro.begin()) : -1;
                };
                inst_sp[i].first = (int)sp.size();
                for (long long q = 0; q < op.N; q++) {
                    const unsigned c = cp.cls[q];
                    const unsigned ka = (c >> (2 * da)) & 3u, kb = (c >> (2 * db)) & 3u;
                    if (ka < ROW_CLOSURE && kb < ROW_CLOSURE && !(c & CLS_DIRFACE)) continue;
                    const int ra = ka == ROW_CLOSURE ? row_of(da, q) : -1;
                    const int rb = kb == ROW_CLOSURE ? row_of(db, q) : -1;
                    if ((ka == ROW_CLOSURE && ra < 0) || (kb == ROW_CLOSURE && rb < 0))
                        return fail(SHOCCS_EINVAL, "cut-cell point without its row");
                    sp.push_back(make_int4(i, (int)q, ra, rb));
                    sp_kind.push_back((int)(((ka << 2 | kb) << 1) | ((c & CLS_DIRFACE) ? 1u : 0u)));
                }
                inst_sp[i].second = (int)sp.size();
            } else {
                for (long long t = 0; t < op.N; t += BATCH2D_TILE) wtiles.push_back(make_int2(i, (int)t));
            }
        }
        if ((long long)row_inst.size() + op.n_cut_rows >= (1LL << 31))
            return fail(SHOCCS_EUNSUPPORTED, "batch above 2^31 cut-cell rows");
        // the split stage evaluates its cut-cell rows at their points: no row pass
        if (!(flat2d && use_split)) row_inst.insert(row_inst.end(), op.n_cut_rows, i);
        for (int c = 0; c < 4 && !flat2d; c++) {
            const int w = BATCH_TILE_WARPS[c];
            const int nyb = (op.it1 + w - 1) / w;
            const long long nt = (long long)op.nzc * nyb * op.it0;
            if ((long long)tiles[c].size() + nt >= (1LL << 31))
                return fail(SHOCCS_EUNSUPPORTED, "batch above 2^31 tiles");
            // tile t of the instance: it2 chunk t % nzc, it1 block of w rows, it0 index
            for (long long t = 0; t < nt; t++) {
                const long long rest = t / op.nzc;
                tiles[c].push_back(make_int4(i, (int)(rest / nyb), (int)(rest % nyb) * w,
                                             (int)(t % op.nzc)));
            }
        }
        for (int d = 0; d < 3; d++)
            for (long long k = 0; k < op.nR[d]; k++) {
                r_inst.push_back(i);
                r_inst.push_back(d);
                r_inst.push_back((int)k);
            }
        B->h_inst.push_back(I);
    }
    const cudaStream_t s = nullptr;
    void* p = nullptr;
    SH_CUDA(B->mem.alloc(n * sizeof(BatchInst), &p));
    B->d_inst = (BatchInst*)p;
    SH_CUDA(B->mem.put(row_inst, &B->d_row_inst, s));
    B->n_rows = (int)row_inst.size();
    for (int c = 0; c < 4; c++) {
        SH_CUDA(B->mem.put(tiles[c], &B->d_tiles[c], s));
        B->n_tiles[c] = (int)tiles[c].size();
    }
    SH_CUDA(B->mem.put(wtiles, &B->d_wtiles, s));
    B->n_wtiles = (int)wtiles.size();
    B->grid2d = batch_stage2d_grid(B->prec, B->n_wtiles);
    if ((long long)sp.size() + ((long long)ut.size() + 3) / 4 * 128 >= (1LL << 31))
        return fail(SHOCCS_EUNSUPPORTED, "batch above 2^31 points");
    // special points grouped by their kinds of rows, so that the threads of a warp mostly
    // take the same path (instance and point order within a group)
    auto by_kind = [&](std::vector<int4>& v, std::vector<int>& kind, size_t b, size_t e) {
        std::vector<size_t> ord(e - b);
        for (size_t k = 0; k < ord.size(); k++) ord[k] = b + k;
        std::stable_sort(ord.begin(), ord.end(), [&](size_t x, size_t y) { return kind[x] < kind[y]; });
        std::vector<int4> tmp(ord.size());
        std::vector<int> tk(ord.size());
        for (size_t k = 0; k < ord.size(); k++) {
            tmp[k] = v[ord[k]];
            tk[k] = kind[ord[k]];
        }
        std::copy(tmp.begin(), tmp.end(), v.begin() + b);
        std::copy(tk.begin(), tk.end(), kind.begin() + b);
    };
    // groups (every instance split): consecutive instances up to the byte budget
    std::vector<std::pair<int, int>> grp; // (first, end) instance of each group
    if (all2d && use_split && n > 1) {
        const char* genv = std::getenv("SHOCCS_BATCH_GROUP_MB");
        const double budget = (genv ? std::atof(genv) : 48.0) * 1048576.0;
        const double per_pt = B->prec == PREC_MIXED ? 25.0 : 33.0; // field bytes per point
        int first = 0;
        double bytes = 0.0;
        for (int i = 0; i < n; i++) {
            const double b = per_pt * (double)B->h_inst[i].op.N;
            if (i > first && bytes + b > budget) {
                grp.emplace_back(first, i);
                first = i;
                bytes = 0.0;
            }
            bytes += b;
        }
        grp.emplace_back(first, n);
        if (budget <= 0.0 || grp.size() < 2) grp.clear();
    }
    {
        std::vector<int4> sps = sp;
        std::vector<int> spk = sp_kind;
        if (grp.empty()) {
            by_kind(sps, spk, 0, sps.size());
        } else {
            for (const auto& g : grp)
                by_kind(sps, spk, (size_t)inst_sp[g.first].first, (size_t)inst_sp[g.second - 1].second);
        }
        SH_CUDA(B->mem.put(sps, &B->split.sp, s));
    }
    SH_CUDA(B->mem.put(ut, &B->split.ut, s));
    B->split.n_ut = (int)ut.size();
    B->split.n_sp = (int)sp.size();

    for (const auto& g : grp) {
        BatchSplit G;
        const int u0 = inst_ut[g.first].first, u1 = inst_ut[g.second - 1].second;
        const int s0 = inst_sp[g.first].first, s1 = inst_sp[g.second - 1].second;
        G.ut = B->split.ut + u0;
        G.n_ut = u1 - u0;
        G.sp = B->split.sp + s0;
        G.n_sp = s1 - s0;
        B->groups.push_back(G);
    }
    SH_CUDA(B->mem.put(r_inst, &B->d_r_inst, s));
    B->n_r = (int)(r_inst.size() / 3);
    // SHOCCS_BATCH_PERSIST=0 keeps a batch of 2-D instances on the launch-per-stage kernels
    const char* penv = std::getenv("SHOCCS_BATCH_PERSIST");
    if (all2d && use_split && penv && std::string(penv) == "1") {
        const int maxc = batch_persist_clusters(B->prec);
        if (maxc > 0) {
            // instances to clusters by their work (points, plus a cut-cell row as 8 points),
            // the largest first, each to the least loaded cluster
            const int C = std::min(maxc, n);
            std::vector<int> order(n);
            std::vector<double> work(n);
            for (int i = 0; i < n; i++) {
                order[i] = i;
                work[i] = (double)B->h_inst[i].op.N + 8.0 * B->h_inst[i].op.n_cut_rows;
            }
            std::stable_sort(order.begin(), order.end(),
                             [&](int a, int b) { return work[a] > work[b]; });
            std::vector<double> load(C, 0.0);
            std::vector<std::vector<int>> own(C);
            for (int i : order) {
                const int c = (int)(std::min_element(load.begin(), load.end()) - load.begin());
                load[c] += work[i];
                own[c].push_back(i);
            }
            std::vector<int4> psp;
            std::vector<int> pspk;
            std::vector<int2> put;
            std::vector<int4> ctab(C);
            for (int c = 0; c < C; c++) {
                std::sort(own[c].begin(), own[c].end());
                ctab[c].x = (int)psp.size();
                ctab[c].z = (int)put.size();
                for (int i : own[c]) {
                    psp.insert(psp.end(), sp.begin() + inst_sp[i].first, sp.begin() + inst_sp[i].second);
                    pspk.insert(pspk.end(), sp_kind.begin() + inst_sp[i].first, sp_kind.begin() + inst_sp[i].second);
                    put.insert(put.end(), ut.begin() + inst_ut[i].first, ut.begin() + inst_ut[i].second);
                }
                ctab[c].y = (int)psp.size();
                ctab[c].w = (int)put.size();
                by_kind(psp, pspk, ctab[c].x, ctab[c].y);
            }
            SH_CUDA(B->mem.put(psp, &B->d_psp, s));
            SH_CUDA(B->mem.put(put, &B->d_put, s));
            SH_CUDA(B->mem.put(ctab, &B->d_ctab, s));
            B->persist = true;
            B->n_clusters = C;
        }
    }
    SH_CUDA(cudaStreamCreateWithFlags(&B->cap, cudaStreamNonBlocking));
    if (B->split.n_sp && B->split.n_ut) {
        SH_CUDA(cudaStreamCreateWithFlags(&B->split.aux, cudaStreamNonBlocking));
        SH_CUDA(cudaEventCreateWithFlags(&B->split.fork, cudaEventDisableTiming));
        SH_CUDA(cudaEventCreateWithFlags(&B->split.join, cudaEventDisableTiming));
        for (auto& G : B->groups) {
            G.aux = B->split.aux;
            G.fork = B->split.fork;
            G.join = B->split.join;
        }
    }
    if (auto st = batch_autotune(B.get(), s); st != SHOCCS_OK) return st;
    SH_CUDA(cudaStreamSynchronize(s));
    *out = B.release();
    return SHOCCS_OK;
}

shoccs_status shoccs_batch_destroy(shoccs_batch* b)
{
    delete b;
    return SHOCCS_OK;
}

shoccs_status shoccs_batch_rk4(shoccs_batch* B, const double* t0, const double* dt, int nsteps,
                               void* stream)
{
    if (!B || !t0 || !dt || nsteps < 0) return fail(SHOCCS_EINVAL, "bad argument");
    const int n = (int)B->sys.size();
    for (int i = 0; i < n; i++)
        if (!(dt[i] > 0)) return fail(SHOCCS_EINVAL, "dt must be > 0");
    if (nsteps == 0) return SHOCCS_OK;
    const cudaStream_t s = (cudaStream_t)stream;
    if (auto st = batch_set_steps(B, t0, dt, nsteps, s); st != SHOCCS_OK) return st;
    if (!B->exec || B->graph_steps != nsteps) {
        // capture the whole loop once; later runs of the same length replay it (the time
        // table and the RK4 weights it reads are refreshed above)
        if (B->exec) {
            cudaGraphExecDestroy(B->exec);
            B->exec = nullptr;
        }
        SH_CUDA(cudaStreamBeginCapture(B->cap, cudaStreamCaptureModeThreadLocal));
        cudaError_t e = cudaSuccess;
        if (B->persist)
            e = launch_batch_persist(B->d_inst, B->d_psp, B->d_put, B->d_ctab, B->n_clusters,
                                     B->d_times, n, nsteps, B->prec, B->cap);
        for (size_t g = 0; g < B->groups.size() && !B->persist; g++)
            for (int k = 0; k < nsteps && e == cudaSuccess; k++)
                e = launch_batch_step(B->d_inst, B->d_row_inst, 0, nullptr, 0, B->cfg, B->grid,
                                      nullptr, 0, B->grid2d, B->groups[g],
                                      B->d_times + (size_t)k * n, B->prec, B->cap);
        for (int k = 0; k < nsteps && e == cudaSuccess && !B->persist && B->groups.empty(); k++)
            e = launch_batch_step(B->d_inst, B->d_row_inst, B->n_rows, B->d_tiles[B->cfg],
                                  B->n_tiles[B->cfg], B->cfg, B->grid, B->d_wtiles,
                                  B->n_wtiles, B->grid2d, B->split, B->d_times + (size_t)k * n,
                                  B->prec, B->cap);
        cudaGraph_t g = nullptr;
        const cudaError_t e2 = cudaStreamEndCapture(B->cap, &g);
        if (e != cudaSuccess || e2 != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return fail(SHOCCS_ECUDA, std::string("graph capture: ") +
                                          cudaGetErrorString(e != cudaSuccess ? e : e2));
        }
        size_t nn = 0;
        cudaGraphGetNodes(g, nullptr, &nn);
        const cudaError_t e3 = cudaGraphInstantiate(&B->exec, g, 0);
        cudaGraphDestroy(g);
        SH_CUDA(e3);
        B->graph_steps = nsteps;
        B->graph_nodes = (int64_t)nn;
    }
    SH_CUDA(cudaGraphLaunch(B->exec, s));
    SH_CUDA(launch_batch_finish(B->d_inst, n, B->d_times + (size_t)(nsteps - 1) * n,
                                B->d_r_inst, B->n_r, s));
    SH_CUDA(cudaStreamSynchronize(s));
    for (int i = 0; i < n; i++) {
        double t = t0[i];
        for (int k = 0; k < nsteps; k++) t += dt[i];
        B->sys[i]->t = t;
    }
    return SHOCCS_OK;
}

shoccs_status shoccs_batch_info(const shoccs_batch* B, int64_t info[6])
{
    if (!B || !info) return fail(SHOCCS_EINVAL, "null argument");
    info[0] = (int64_t)B->sys.size();
    info[1] = B->n_tiles[B->cfg] + B->n_wtiles + B->split.n_ut;
    info[2] = B->n_rows;
    info[3] = BATCH_TILE_WARPS[B->cfg];
    info[4] = B->persist ? B->n_clusters * BATCH_CLUSTER : B->grid;
    info[5] = B->graph_nodes;
    return SHOCCS_OK;
}

} // extern "C"

// ---------------------------------------------------------------------------------------
// discrete adjoint
// ---------------------------------------------------------------------------------------
struct shoccs_tape {
    double t0 = 0.0, dt = 0.0;
    int nsteps = 0, every = 0;
    long long n = 0;
    std::vector<double*> ckpt;
    DeviceAlloc mem;
};

namespace
{
// transposed closure rows: for each column point of a cut-cell or wall row whose output point
// evolves (fluid, has a row, not on a Dirichlet face), the (output point, coefficient) pairs
shoccs_status build_adjoint(shoccs_system* S, cudaStream_t s)
{
    AdjointState& A = S->adj;
    if (A.built) return SHOCCS_OK;
    const shoccs_problem* P = S->P;
    const Compiled& C = P->comp;
    const Mesh& m = P->mesh;
    const i64 N = m.size();
    auto evolves = [&](i64 p) {
        const uint8_t c = C.cls[p];
        return (c & 0x3F) && !(c & CLS_DIRFACE);
    };
    struct Trip {
        i64 tgt, src;
        double w;
    };
    std::vector<Trip> trip;
    for (int d = 0; d < 3; d++) {
        const AxisTables& T = C.ax[d];
        if (!T.active) continue;
        const i64 sd = T.stride;
        for (size_t r = 0; r < T.rows.size(); r++) {
            const i64 p = T.row_out[r];
            if (!evolves(p)) continue;
            const ClosureRow& cr = T.rows[r];
            for (int j = 0; j < cr.ncol; j++)
                trip.push_back({p + (i64)(cr.col0 + j) * sd, p, T.coef[cr.coef_off + j]});
        }
        const i64 nyz = (i64)m.n[1] * m.n[2];
        for (i64 p = 0; p < N; p++) {
            if (((C.cls[p] >> (2 * d)) & 3) != ROW_WALL || !evolves(p)) continue;
            const int coord = d == 0 ? (int)(p / nyz) : (d == 1 ? (int)((p / m.n[2]) % m.n[1])
                                                                : (int)(p % m.n[2]));
            const WallBlock& W = T.wall[coord * 2 < m.n[d] ? 0 : 1];
            const int r = coord - W.first_row;
            for (int j = 0; j < W.cols; j++)
                trip.push_back({p + (i64)(W.col0 - coord + j) * sd, p, W.c[r * 7 + j]});
        }
    }
    std::sort(trip.begin(), trip.end(), [](const Trip& a, const Trip& b) {
        return a.tgt != b.tgt ? a.tgt < b.tgt : a.src < b.src;
    });
    std::vector<long long> tgt, src;
    std::vector<int> ptr{0};
    std::vector<double> w;
    for (size_t e = 0; e < trip.size(); e++) {
        if (e == 0 || trip[e].tgt != trip[e - 1].tgt) {
            if (e) ptr.push_back((int)e);
            tgt.push_back(trip[e].tgt);
        }
        src.push_back(trip[e].src);
        w.push_back(trip[e].w);
    }
    if (!trip.empty()) ptr.push_back((int)trip.size());
    if (trip.size() >= (size_t)INT32_MAX) return fail(SHOCCS_EUNSUPPORTED, "closure too large");
    SH_CUDA(A.mem.put(tgt, &A.cl.tgt, s));
    SH_CUDA(A.mem.put(ptr, &A.cl.ptr, s));
    SH_CUDA(A.mem.put(src, &A.cl.src, s));
    SH_CUDA(A.mem.put(w, &A.cl.w, s));
    A.cl.n_tgt = (int)tgt.size();
    const size_t es = S->desc.prec == PREC_MIXED ? sizeof(float) : sizeof(double);
    for (void** b : {&A.lam, &A.acc, &A.za, &A.zb})
        SH_CUDA(A.mem.alloc(N * es, b));
    A.built = true;
    return SHOCCS_OK;
}

shoccs_status adjoint_supported(const shoccs_system* S)
{
    if (S->desc.kind != SHOCCS_SYS_HEAT)
        return fail(SHOCCS_EUNSUPPORTED, "the adjoint is implemented for heat systems");
    if (S->unfused)
        return fail(SHOCCS_EUNSUPPORTED, "the adjoint covers systems whose objects are all Dirichlet");
    return SHOCCS_OK;
}
} // namespace

extern "C" {

shoccs_status shoccs_system_rhs_transpose(shoccs_system* S, const shoccs_field* x,
                                          shoccs_field* y, void* stream)
{
    if (!S || !x || !y || !x->D || !y->D) return fail(SHOCCS_EINVAL, "null argument");
    if (auto st = adjoint_supported(S); st != SHOCCS_OK) return st;
    if (S->desc.prec != PREC_FP64)
        return fail(SHOCCS_EUNSUPPORTED, "the transposed operator takes FP64 fields");
    const cudaStream_t s = (cudaStream_t)stream;
    if (auto st = build_adjoint(S, s); st != SHOCCS_OK) return st;
    AdjArgs a{};
    a.z = (const double*)x->D;
    a.zscale = 1.0;
    a.out = (double*)y->D;
    a.k = S->desc.diffusivity;
    SH_CUDA(launch_adjoint_stage(S->P->op, S->adj.cl, 0, a, PREC_FP64, s));
    for (int r = 0; r < 3; r++) {
        void* yr = r == 0 ? y->Rx : (r == 1 ? y->Ry : y->Rz);
        if (yr && S->P->mesh.R[r].size())
            SH_CUDA(cudaMemsetAsync(yr, 0, S->P->mesh.R[r].size() * 8, s));
    }
    SH_CUDA(cudaStreamSynchronize(s));
    return SHOCCS_OK;
}

shoccs_status shoccs_system_forward(shoccs_system* S, double t0, double dt, int nsteps,
                                    int checkpoint_every, shoccs_tape** tape, void* stream)
{
    if (!S || !tape || nsteps < 0 || !(dt > 0) || checkpoint_every < 0)
        return fail(SHOCCS_EINVAL, "bad argument");
    *tape = nullptr;
    if (auto st = adjoint_supported(S); st != SHOCCS_OK) return st;
    const cudaStream_t s = (cudaStream_t)stream;
    auto T = std::make_unique<shoccs_tape>();
    T->t0 = t0;
    T->dt = dt;
    T->nsteps = nsteps;
    T->every = checkpoint_every;
    T->n = S->P->mesh.size();
    auto save = [&]() -> shoccs_status { // checkpoints hold the state in FP64
        void* q = nullptr;
        SH_CUDA(T->mem.alloc(T->n * sizeof(double), &q));
        if (S->desc.prec == PREC_MIXED)
            SH_CUDA(launch_state_convert(T->n, 0, nullptr, nullptr, S->b.u0, (double*)q, s));
        else
            SH_CUDA(cudaMemcpyAsync(q, S->b.u0, T->n * sizeof(double), cudaMemcpyDeviceToDevice, s));
        T->ckpt.push_back((double*)q);
        return SHOCCS_OK;
    };
    if (checkpoint_every > 0)
        if (auto st = save(); st != SHOCCS_OK) return st;
    double t = t0;
    int done = 0;
    while (done < nsteps) {
        const int k = checkpoint_every > 0 ? std::min(checkpoint_every, nsteps - done)
                                           : nsteps - done;
        for (int i = 0; i < k; i++) {
            SH_CUDA(launch_rk4_step(S->P->op, S->P->dr, S->sp, S->desc.prec, S->b, t, dt, s,
                                    nullptr, i + 1 < k));
            t += dt;
        }
        done += k;
        if (checkpoint_every > 0)
            if (auto st = save(); st != SHOCCS_OK) return st;
    }
    SH_CUDA(cudaStreamSynchronize(s));
    S->t = t;
    *tape = T.release();
    return check_wait_flag(S, s);
}

shoccs_status shoccs_system_backward(shoccs_system* S, const shoccs_tape* T,
                                     const shoccs_field* g, shoccs_field* out, void* stream)
{
    if (!S || !T || !g || !out || !g->D || !out->D) return fail(SHOCCS_EINVAL, "null argument");
    if (auto st = adjoint_supported(S); st != SHOCCS_OK) return st;
    if (T->n != S->P->mesh.size()) return fail(SHOCCS_EINVAL, "tape of another system");
    const cudaStream_t s = (cudaStream_t)stream;
    if (auto st = build_adjoint(S, s); st != SHOCCS_OK) return st;
    AdjointState& A = S->adj;
    const long long N = T->n;
    constexpr double rki[4] = {0.0, 0.5, 0.5, 1.0}; // src/temporal/rk4.cpp:11-12
    constexpr double rkf[4] = {1.0 / 6.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 6.0};
    const double dt = T->dt;
    const int prec = S->desc.prec;
    // lam = dJ/du(T); its Dirichlet-face entries are dropped (the last stage resets faces).
    // A mixed system runs the reverse sweep in FP32 (the forward's stage precision).
    if (prec == PREC_MIXED) {
        SH_CUDA(launch_cast(N, 1, g->D, A.lam, s)); // field pointers are device pointers
    } else {
        SH_CUDA(cudaMemcpyAsync(A.lam, g->D, N * sizeof(double), cudaMemcpyDefault, s));
    }
    SH_CUDA(launch_adjoint_mask_faces(S->P->op, A.lam, prec, s));
    for (int n = T->nsteps - 1; n >= 0; n--) {
        void* zin = nullptr;
        for (int st = 4; st >= 1; st--) {
            AdjArgs a{};
            a.k = S->desc.diffusivity;
            a.lam = A.lam;
            a.acc = A.acc;
            a.z = st == 4 ? A.lam : zin;
            a.zscale = st == 4 ? dt * rkf[3] : 1.0;
            if (st > 1) {
                a.out = (st % 2 == 0) ? A.za : A.zb;
                a.bl = dt * rkf[st - 2];
                a.ay = dt * rki[st - 1];
            } else {
                a.out = A.lam; // in place: S = 1 reads lam only at the point it writes
                a.first_step = n == 0;
            }
            SH_CUDA(launch_adjoint_stage(S->P->op, A.cl, st, a, prec, s));
            zin = a.out;
        }
    }
    if (prec == PREC_MIXED)
        SH_CUDA(launch_cast(N, 0, A.lam, out->D, s));
    else
        SH_CUDA(cudaMemcpyAsync(out->D, A.lam, N * sizeof(double), cudaMemcpyDefault, s));
    for (int r = 0; r < 3; r++) {
        void* yr = r == 0 ? out->Rx : (r == 1 ? out->Ry : out->Rz);
        if (yr && S->P->mesh.R[r].size())
            SH_CUDA(cudaMemsetAsync(yr, 0, S->P->mesh.R[r].size() * 8, s));
    }
    SH_CUDA(cudaStreamSynchronize(s));
    return SHOCCS_OK;
}

shoccs_status shoccs_tape_checkpoint(const shoccs_tape* T, int i, double* state, int* count,
                                     void* stream)
{
    if (!T) return fail(SHOCCS_EINVAL, "null tape");
    if (count) *count = (int)T->ckpt.size();
    if (!state) return SHOCCS_OK;
    if (i < 0 || i >= (int)T->ckpt.size()) return fail(SHOCCS_EINVAL, "no such checkpoint");
    const cudaStream_t s = (cudaStream_t)stream;
    SH_CUDA(cudaMemcpyAsync(state, T->ckpt[i], T->n * sizeof(double), cudaMemcpyDefault, s));
    SH_CUDA(cudaStreamSynchronize(s));
    return SHOCCS_OK;
}

shoccs_status shoccs_tape_destroy(shoccs_tape* T)
{
    delete T;
    return SHOCCS_OK;
}

shoccs_status shoccs_system_timestep(const shoccs_system* S, double cfl, double* dt)
{
    if (!S || !dt) return fail(SHOCCS_EINVAL, "null argument");
    const auto& h = S->P->mesh.h;
    const double hmin = std::min(h[0], std::min(h[1], h[2]));
    if (S->desc.kind == SHOCCS_SYS_HEAT)
        *dt = cfl * hmin * hmin / (4 * S->desc.diffusivity); // heat.cpp:356-361
    else
        *dt = cfl * hmin; // scalar_wave.cpp:357-362
    return SHOCCS_OK;
}

} // extern "C"
