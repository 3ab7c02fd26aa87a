// problem.hpp -- host-side setup of the cut-cell operators and their compilation into the
// GPU layout used by the sm_103a kernels.
//
// Setup mirrors the reference's construction so that the cut-point sets, line segments,
// per-line block metadata and closure sparsity are bit-identical:
//   * cartesian grid            src/mesh/cartesian.cpp:13-44
//   * ray-cast cut points       src/mesh/object_geometry.cpp:17-116, src/mesh/sphere.cpp:15-38
//   * fluid line segments       src/mesh/mesh.cpp:29-111
//   * per-axis operator O/B/N   src/operators/derivative.cpp:305-449
//   * R-space rows Bf/Br        src/operators/derivative.cpp:22-257
// and then compiles them (compile_axis) into the device format described in gpu_layout.hpp.
#pragma once

#include "gpu_layout.hpp"
#include "stencils.hpp"

#include <array>
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

namespace sgb
{
using i64 = long long;

struct Sphere {
    real c[3];
    real r;
    int id;
};

// one ray/shape intersection (src/mesh/mesh_types.hpp:31-38)
struct CutPoint {
    real psi;
    real pos[3];
    real nrm[3];
    int ray_outside;
    int solid[3];
    int shape_id;
};

// end of a fluid line segment; obj >= 0 is the index of the cut point in R(dir)
struct Bnd {
    int ijk[3];
    i64 obj = -1;
    int obj_id = -1;
    real psi = 1.0;
};

struct Line {
    i64 stride;
    Bnd s, e;
};

struct Mesh {
    int n[3];
    real lo[3], hi[3], h[3];
    std::vector<real> x[3];
    std::vector<Sphere> shapes;
    std::vector<CutPoint> R[3];
    std::vector<Line> lines[3];
    std::vector<std::pair<i64, i64>> fluid_slices;

    i64 size() const { return (i64)n[0] * n[1] * n[2]; }
    i64 ic(const int* ijk) const
    {
        return (i64)ijk[0] * n[1] * n[2] + (i64)ijk[1] * n[2] + ijk[2];
    }
    i64 stride(int d) const
    {
        i64 s = 1;
        for (int i = d + 1; i < 3; i++) s *= n[i];
        return s;
    }
};

Mesh build_mesh(const int n[3], const real lo[3], const real hi[3],
                const std::vector<Sphere>& shapes);

// grid_bc[d][side] (0 left / 1 right) and per-shape bc
struct Bcs {
    int grid[3][2];
    std::vector<int> obj;
};

// reference-shaped per-line block metadata (src/matrices/inner_block_meta.hpp:9-23)
struct BlockMeta {
    int row_offset, col_offset, stride, left_rows, left_cols, left_coeff_offset,
        interior_rows, interior_coeff_offset, stencil_width, right_rows, right_cols,
        right_coeff_offset, right_col_offset;
};

struct Csr {
    i64 rows = 0;
    std::vector<i64> u{0};
    std::vector<i64> v;
    std::vector<real> w;
};

// one derivative direction, in the reference's own decomposition
struct AxisOp {
    bool active = false;
    int dir = 0;
    i64 stride = 1;
    std::vector<real> interior;
    std::vector<BlockMeta> meta;
    std::vector<uint8_t> block_wall; // per block: bit0 left end is a wall, bit1 right end
    std::vector<real> coeffs;
    Csr B, N;
    Csr Bf[3], Br[3];
};

AxisOp assemble_axis(int dir, const Mesh& m, const Stencil& st, const Bcs& bcs);

// ---------------------------------------------------------------------------------------
// Compiled device tables (host copies; gpu_layout.hpp defines the records)
// ---------------------------------------------------------------------------------------
struct AxisTables {
    bool active = false;
    i64 stride = 1;
    int width = 0;
    real interior[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}; // 2p+1 <= 9 (E8u_1)
    WallBlock wall[2] = {};       // left / right domain-wall closure blocks
    std::vector<ClosureRow> rows; // cut-cell closure rows, sorted by output index
    std::vector<i64> row_out;     // output flat index of each row
    std::vector<real> coef;       // deduplicated coefficient pool
    std::vector<int> chunk_base;  // exclusive prefix of closure rows per 32-point chunk
    // R-space rows (non-Dirichlet objects): per target r, Bf (cols in D) then Br (cols in R_r)
    std::vector<int> rr_u[3];
    std::vector<int> rr_col[3];
    std::vector<unsigned char> rr_src[3]; // 0: column in D, 1: column in R_r
    std::vector<real> rr_w[3];
};

struct Compiled {
    int it[3];  // iteration extents (canonical: last one contiguous)
    int nzc;    // chunks of 32 along the contiguous iteration axis
    int phys_of_it[3]; // physical axis of each iteration axis (-1 when trivial)
    std::vector<uint8_t> cls;
    AxisTables ax[3];
    i64 n_fluid = 0;
};

Compiled compile_operators(const Mesh& m, const AxisOp ops[3], const Bcs& bcs);

// Dirichlet domain faces as flat indices (src/fields/selection_desc.hpp:211-222)
bool on_dirichlet_face(const Mesh& m, const Bcs& bcs, const int ijk[3]);

} // namespace sgb
