// gpu_layout.hpp -- device-side layout of a compiled cut-cell operator.
//
// For every grid point p (flat index i*ny*nz + j*nz + k, z fastest, as the reference's
// index_extents, src/index_extents.hpp:15-19) one class byte cls[p] holds, for each axis d,
// the kind of row the reference's block operator has at p along d:
//     bits 2d..2d+1 : ROW_NONE (no row: solid point or removed Dirichlet row),
//                     ROW_INTERIOR (circulant interior row, 2p+1 point centred stencil),
//                     ROW_CLOSURE (dense closure row next to a cut cell: per-row record),
//                     ROW_WALL (dense closure row next to a domain wall: the rows of every
//                               line at a given wall are identical, so they are stored once
//                               per axis and side in kernel-parameter space)
//     bit 6         : point lies on a Dirichlet domain face
//     bit 7         : point is a fluid point (the reference's fluid_desc)
// Cut-cell closure rows of axis d are stored once, sorted by output index, as ClosureRow
// records;
// a kernel finds the record of point p from a per-chunk exclusive prefix count
// (chunk = 32 consecutive points along the contiguous iteration axis) plus the rank of p
// among the closure points of its warp (ballot/popc).  Coefficients live in a deduplicated
// pool, so the identical wall-closure rows of all lines share one coefficient block.
#pragma once
#include <cstdint>

namespace sgb
{
enum : unsigned { ROW_NONE = 0, ROW_INTERIOR = 1, ROW_CLOSURE = 2, ROW_WALL = 3 };

// the closure block shared by every line that ends at one domain wall of one axis
struct WallBlock {
    int rows;      // closure rows (0: no line ends at this wall)
    int cols;      // columns of each row
    int first_row; // axis coordinate of row 0
    int col0;      // axis coordinate of column 0
    int has_n;     // Neumann wall: row r adds n[r] * nu[wall point]
    int wall;      // axis coordinate of the wall point
    double c[5 * 7];
    double n[5];
    float cf[5 * 7];
    float sf[5]; // row sums of c, rounded to FP32 (zero up to rounding; difference form)
};
enum : unsigned { CLS_DIRFACE = 0x40, CLS_FLUID = 0x80 };

// one dense closure row: out[p] (op)= sum_j coef[coef_off+j] * x[p + (col0+j)*stride]
//                                    + coef[coef_off+ncol]   * R_d[b_idx]   (flags & 1)
//                                    + coef[coef_off+ncol+b] * nu[n_idx]    (flags & 2)
struct ClosureRow {
    int32_t coef_off;
    int16_t col0;
    uint8_t ncol;
    uint8_t flags;
    int32_t b_idx;
    int32_t n_idx;
};
static_assert(sizeof(ClosureRow) == 16, "ClosureRow must stay 16 bytes");

enum : uint8_t { ROWF_B = 1, ROWF_N = 2 };
} // namespace sgb
