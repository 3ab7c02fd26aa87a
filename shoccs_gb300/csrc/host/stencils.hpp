// stencils.hpp -- closed-form stencil coefficients for the cut-cell schemes E2_2, E4_2
// (second derivative), E4_1 (cut-cell first derivative) and E4u_1 (uniform-grid first
// derivative).
//
// Setup-time host code.  The formulas restate src/stencils/E2_2.cpp, src/stencils/E4_2.cpp,
// src/stencils/E4_1.cpp and src/stencils/E4u_1.cpp of the reference (query / interior /
// nbs / interp_interior / interp_wall), statement by statement so that the coefficients are bit-identical when
// compiled with -ffp-contract=off.  They are mathematics that must be alike; the closure
// rows they produce are compiled into GPU tables by problem.cpp.
#pragma once
#include <algorithm>
#include <cmath>

namespace sgb
{
using real = double;
enum bc_type { Dirichlet = 0, Floating = 1, Neumann = 2 };

struct info {
    int p, r, t, nextra;
};
struct interp_info {
    int p, t;
};

struct Stencil {
    int kind = 1; // 0: E2_2, 1: E4_2, 2: E4_1, 3: E4u_1, 5: polyE2_1 (type "E2-poly"),
                  // 6: E6u_1, 7: E8u_1
    real alpha[2] = {0, 0};
    // polyE2_1: floating alpha[6], dirichlet alpha[3], interpolant alpha[4]; E6u_1: alpha[5];
    // E8u_1: alpha[7]
    real pa[13] = {};

    info query_max() const
    {
        switch (kind) {
        case 0: return {1, 2, 4, 2};
        case 1: return {2, 3, 5, 3};
        case 3: return {2, 3, 5, 0};
        case 5: return {1, 3, 4, 0}; // polyE2_1.cpp:11-14
        case 6: return {3, 5, 8, 0};  // E6u_1.cpp:13-16
        case 7: return {4, 7, 11, 0}; // E8u_1.cpp:13-16
        default: return {2, 5, 7, 0};
        }
    }
    info query(int b) const
    {
        info mx = query_max();
        if ((kind == 2 || kind == 3 || kind >= 5) && b == Neumann) return {0, 0, 0, 0};
        switch (b) {
        case Dirichlet: return {mx.p, mx.r - 1, mx.t, 0};
        case Floating: return {mx.p, mx.r, mx.t, 0};
        default: return {mx.p, mx.r, mx.t, mx.nextra};
        }
    }
    interp_info query_interp() const
    {
        switch (kind) {
        case 0: return {2, 3};
        case 1: return {5, 5};
        case 5: return {2, 4}; // polyE2_1.cpp:44
        default: return {0, 0};
        }
    }

    // interior coefficients
    void interior(real h, real* c) const
    {
        if (kind == 0) { // E2_2.cpp:104-111
            c[0] = 1 / (h * h);
            c[1] = -2 / (h * h);
            c[2] = 1 / (h * h);
        } else if (kind == 1) { // E4_2.cpp:33-42
            c[0] = -1 / (12. * (h * h));
            c[1] = 4 / (3. * (h * h));
            c[2] = -5 / (2. * (h * h));
            c[3] = 4 / (3. * (h * h));
            c[4] = -1 / (12. * (h * h));
        } else if (kind == 5) {
            pe2_interior(h, c);
        } else if (kind == 6) { // E6u_1.cpp:49-60
            c[0] = -1 / (60 * h);
            c[1] = 3 / (20 * h);
            c[2] = -3 / (4 * h);
            c[3] = 0;
            c[4] = -c[2];
            c[5] = -c[1];
            c[6] = -c[0];
        } else if (kind == 7) { // E8u_1.cpp:48-61
            c[0] = 1 / (280 * h);
            c[1] = -4 / (105 * h);
            c[2] = 1 / (5 * h);
            c[3] = -4 / (5 * h);
            c[4] = 0;
            c[5] = -c[3];
            c[6] = -c[2];
            c[7] = -c[1];
            c[8] = -c[0];
        } else if (kind == 3) { // E4u_1.cpp:49-58
            c[0] = 1 / (12 * h);
            c[1] = -2 / (3 * h);
            c[2] = 0;
            c[3] = -c[1];
            c[4] = -c[0];
        } else { // E4_1.cpp:66-76
            c[0] = 0.083333333333333329;
            c[1] = -0.66666666666666663;
            c[2] = 0;
            c[3] = 0.66666666666666663;
            c[4] = -0.083333333333333329;
            for (int i = 0; i < 5; i++) c[i] /= h;
        }
    }

    // boundary closure: returns the number of coefficients written (r*t)
    void nbs(real h, int b, real psi, bool right, real* c, real* x) const
    {
        if (kind == 0) {
            if (b == Floating) e22_floating(h, psi, c, right);
            else if (b == Dirichlet) e22_dirichlet(h, psi, c, right);
            else e22_neumann(h, psi, c, x, right);
        } else if (kind == 1) {
            if (b == Floating) e42_floating(h, psi, c, right);
            else if (b == Dirichlet) e42_dirichlet(h, psi, c, right);
            else e42_neumann(h, psi, c, x, right);
        } else if (kind == 3) {
            if (b == Floating) e4u_floating(h, c, right);
            else if (b == Dirichlet) e4u_dirichlet(h, c, right);
        } else if (kind == 5) {
            if (b == Floating) pe2_floating(h, psi, c, right);
            else if (b == Dirichlet) pe2_dirichlet(h, psi, c, right);
        } else if (kind == 6) { // uniform-grid closures, psi ignored
            if (b == Floating) e6u_floating(h, c, right);
            else if (b == Dirichlet) e6u_dirichlet(h, c, right);
        } else if (kind == 7) {
            if (b == Floating) e8u_floating(h, c, right);
            else if (b == Dirichlet) e8u_dirichlet(h, c, right);
        } else {
            if (b == Floating) e41_floating(h, psi, c, right);
            else if (b == Dirichlet) e41_dirichlet(h, psi, c, right);
        }
    }

    // ---- polyE2_1 (type "E2-poly"): src/stencils/polyE2_1.cpp.  Parameters pa[13]: the
    // floating alpha fa = pa[0..5], the dirichlet alpha da = pa[6..8] and the interpolant
    // alpha ia = pa[9..12] (the reference's single-array order, stencil.cpp:79-87).  The
    // closed forms keep the reference's operation order term for term (bit-exact).
    void pe2_interior(real h, real* c) const // polyE2_1.cpp:169-177
    {
        c[0] = -0.5;
        c[1] = 0;
        c[2] = 0.5;
        for (int i = 0; i < 3; i++) c[i] /= h;
    }
    void pe2_floating(real h, real psi, real* c, bool right) const // polyE2_1.cpp:194-230
    {
        const real* fa = pa;
        const real a0 = fa[0], b0 = fa[1], a1 = fa[2], b1 = fa[3], a2 = fa[4], b2 = fa[5];
        const real inv = 1.0 / (1 + psi);
        const real p2 = 2 + psi;
        const real b0m = -1 + b0, b1m = -1 + b1, b2m = -1 + b2;
        c[0] = 0.5 * inv * b0m;
        c[1] = (-1 + a0) * 0.5;
        c[2] = -1 * a0 + -0.5 * p2 * inv * b0m;
        c[3] = (a0 + b0) * 0.5;
        c[4] = 0.5 * b1m * inv;
        c[5] = (-1 + a1) * 0.5;
        c[6] = -1 * a1 + -0.5 * p2 * b1m * inv;
        c[7] = (b1 + a1) * 0.5;
        c[8] = 0.5 * b2m * inv;
        c[9] = (-1 + a2) * 0.5;
        c[10] = -1 * a2 + -0.5 * p2 * b2m * inv;
        c[11] = (b2 + a2) * 0.5;
        for (int i = 0; i < 12; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 12; i++) c[i] *= -1;
            reverse(c, 12);
        }
    }
    void pe2_dirichlet(real h, real psi, real* c, bool right) const // polyE2_1.cpp:232-280
    {
        const real* da = pa + 6;
        const real d0 = da[0], d1 = da[1], d2 = da[2];
        const real inv = 1.0 / (1 + psi);
        const real d0m = -1 + d0;
        const real tp = 2 * psi;
        const real d2x3 = 3 * d2;
        const real tpd2 = 2 * psi * d2;
        const real den = 1.0 / (1 + tp + d2x3 + tpd2);
        const real tpd1 = 2 * psi * d1;
        const real d1d0x3 = 3 * d1 * d0;
        const real tpd1d0 = 2 * psi * d1 * d0;
        const real md1 = -1 * d1;
        const real p2 = 2 + psi;
        const real d2m = -1 + d2;
        c[0] = 0.5 * inv * d0m;
        c[1] = (-1 + -2 * psi + d1 + tpd1 + d1d0x3 + tpd1d0 + -3 * d0 + -2 * psi * d0) * 0.5 * den;
        c[2] = (-2 * psi * d1 + -3 * d2 + -2 * psi * d2 + md1 + 3 * d0 + 2 * psi * d0 +
                -3 * d1 * d0 + -2 * psi * d1 * d0) *
                   den +
               -0.5 * p2 * inv * d0m;
        c[3] = (d1 + tpd1 + d1d0x3 + tpd1d0 + d2x3 + tpd2 + -2 * d0 + 3 * d2 * d0 +
                2 * psi * d2 * d0) *
               0.5 * den;
        c[4] = 0.5 * d2m * inv;
        c[5] = (-1 + d1) * 0.5;
        c[6] = md1 + -0.5 * p2 * d2m * inv;
        c[7] = (d1 + d2) * 0.5;
        for (int i = 0; i < 8; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 8; i++) c[i] *= -1;
            reverse(c, 8);
        }
    }
    int pe2_interp_wall(int i, real y, real psi, real* c, bool right) const // polyE2_1.cpp:58-141
    {
        const real* fa = pa;
        const real* ia = pa + 9;
        const real inv = 1.0 / (1 + psi);
        const real my = -1 * y;
        if (right) {
            if (i == 0) {
                const real f0y = fa[0] * y, f1y = fa[1] * y;
                c[0] = (f0y + f1y + ia[0] + ia[1]) * 0.5;
                c[1] = (-1 * psi + my + (f0y + ia[0]) * -2 +
                        (my + -2 * ia[1] + -1 * psi * ia[1] + -2 * fa[1] * y + -1 * psi * fa[1] * y) *
                            inv) *
                       0.5;
                c[2] = (1 + psi + f0y + ia[0] + y) * 0.5;
                c[3] = (1 + psi + f1y + ia[1] + y) * 0.5 * inv;
            } else {
                const real f2y = fa[2] * y, f3y = fa[3] * y;
                c[0] = (ia[3] + f2y + f3y + ia[2]) * 0.5;
                c[1] = (my + (f2y + ia[2]) * -2 +
                        (psi + -2 * ia[3] + -1 * psi * ia[3] + my + -2 * fa[3] * y +
                         -1 * psi * fa[3] * y) *
                            inv) *
                       0.5;
                c[2] = (1 + f2y + ia[2] + y) * 0.5;
                c[3] = (1 + ia[3] + f3y + y) * 0.5 * inv;
            }
        } else {
            if (i == 0) {
                const real f0y = fa[0] * y, f1y = fa[1] * y;
                c[0] = (1 + psi + ia[1] + my + f1y) * 0.5 * inv;
                c[1] = (1 + psi + f0y + ia[0] + my) * 0.5;
                c[2] = (-1 * psi + (f0y + ia[0]) * -2 + y +
                        (-2 * ia[1] + -1 * psi * ia[1] + y + -2 * fa[1] * y + -1 * psi * fa[1] * y) *
                            inv) *
                       0.5;
                c[3] = (ia[1] + f0y + ia[0] + f1y) * 0.5;
            } else {
                const real f2y = fa[2] * y, f3y = fa[3] * y;
                c[0] = (1 + f3y + ia[3] + my) * 0.5 * inv;
                c[1] = (1 + f2y + ia[2] + my) * 0.5;
                c[2] = ((f2y + ia[2]) * -2 + y +
                        (psi + -2 * ia[3] + -1 * psi * ia[3] + y + -2 * fa[3] * y +
                         -1 * psi * fa[3] * y) *
                            inv) *
                       0.5;
                c[3] = (f3y + ia[3] + f2y + ia[2]) * 0.5;
            }
        }
        return 4;
    }

    // ---- E6u_1, E8u_1 (uniform-grid closures, psi ignored): src/stencils/E6u_1.cpp:78-205,
    // E8u_1.cpp:78-301, the generated expressions term for term
    void e6u_floating(real h, real* c, bool right) const // E6u_1.cpp nbs_floating
    {
        const real* alpha = pa;
        c[0] = (60 * alpha[0] - 137) / 60;
        c[1] = 5 - 6 * alpha[0];
        c[2] = 15 * alpha[0] - 5;
        c[3] = -(60 * alpha[0] - 10) / 3;
        c[4] = (60 * alpha[0] - 5) / 4;
        c[5] = -(30 * alpha[0] - 1) / 5;
        c[6] = alpha[0];
        c[7] = 0;
        c[8] = (5 * alpha[1] - 1) / 5;
        c[9] = -(72 * alpha[1] + 13) / 12;
        c[10] = 15 * alpha[1] + 2;
        c[11] = (-20 * alpha[1]) - 1;
        c[12] = (45 * alpha[1] + 1) / 3;
        c[13] = -(120 * alpha[1] + 1) / 20;
        c[14] = alpha[1];
        c[15] = 0;
        c[16] = (20 * alpha[2] + 1) / 20;
        c[17] = -(12 * alpha[2] + 1) / 2;
        c[18] = (45 * alpha[2] - 1) / 3;
        c[19] = 1 - 20 * alpha[2];
        c[20] = (60 * alpha[2] - 1) / 4;
        c[21] = -(180 * alpha[2] - 1) / 30;
        c[22] = alpha[2];
        c[23] = 0;
        c[24] = (180 * alpha[4] + 30 * alpha[3] - 1) / 30;
        c[25] = -(140 * alpha[4] + 24 * alpha[3] - 1) / 4;
        c[26] = 84 * alpha[4] + 15 * alpha[3] - 1;
        c[27] = -(315 * alpha[4] + 60 * alpha[3] - 1) / 3;
        c[28] = (140 * alpha[4] + 30 * alpha[3] + 1) / 2;
        c[29] = -(420 * alpha[4] + 120 * alpha[3] + 1) / 20;
        c[30] = alpha[3];
        c[31] = alpha[4];
        c[32] = -(190320 * alpha[4] + 31720 * alpha[3] + 22080 * alpha[2] + 38040 * alpha[1] + 9500 * alpha[0] - 453) / 28260;
        c[33] = (55510 * alpha[4] + 9516 * alpha[3] + 6624 * alpha[2] + 11412 * alpha[1] + 2850 * alpha[0] - 159) / 1413;
        c[34] = -(44408 * alpha[4] + 7930 * alpha[3] + 5520 * alpha[2] + 9510 * alpha[1] + 2375 * alpha[0] - 183) / 471;
        c[35] = (166530 * alpha[4] + 31720 * alpha[3] + 22080 * alpha[2] + 38040 * alpha[1] + 9500 * alpha[0] - 1506) / 1413;
        c[36] = -(444080 * alpha[4] + 95160 * alpha[3] + 66240 * alpha[2] + 114120 * alpha[1] + 28500 * alpha[0] - 1323) / 5652;
        c[37] = (55510 * alpha[4] + 15860 * alpha[3] + 11040 * alpha[2] + 19020 * alpha[1] + 4750 * alpha[0] + 1551) / 2355;
        c[38] = -(1586 * alpha[3] + 1104 * alpha[2] + 1902 * alpha[1] + 475 * alpha[0] + 192) / 1413;
        c[39] = -(1586 * alpha[4] - 24) / 1413;
        for (int i = 0; i < 40; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 40; i++) c[i] *= -1;
            reverse(c, 40);
        }
    }
    void e6u_dirichlet(real h, real* c, bool right) const // E6u_1.cpp nbs_dirichlet
    {
        const real* alpha = pa;
        c[0] = (5 * alpha[1] - 1) / 5;
        c[1] = -(72 * alpha[1] + 13) / 12;
        c[2] = 15 * alpha[1] + 2;
        c[3] = (-20 * alpha[1]) - 1;
        c[4] = (45 * alpha[1] + 1) / 3;
        c[5] = -(120 * alpha[1] + 1) / 20;
        c[6] = alpha[1];
        c[7] = 0;
        c[8] = (20 * alpha[2] + 1) / 20;
        c[9] = -(12 * alpha[2] + 1) / 2;
        c[10] = (45 * alpha[2] - 1) / 3;
        c[11] = 1 - 20 * alpha[2];
        c[12] = (60 * alpha[2] - 1) / 4;
        c[13] = -(180 * alpha[2] - 1) / 30;
        c[14] = alpha[2];
        c[15] = 0;
        c[16] = (180 * alpha[4] + 30 * alpha[3] - 1) / 30;
        c[17] = -(140 * alpha[4] + 24 * alpha[3] - 1) / 4;
        c[18] = 84 * alpha[4] + 15 * alpha[3] - 1;
        c[19] = -(315 * alpha[4] + 60 * alpha[3] - 1) / 3;
        c[20] = (140 * alpha[4] + 30 * alpha[3] + 1) / 2;
        c[21] = -(420 * alpha[4] + 120 * alpha[3] + 1) / 20;
        c[22] = alpha[3];
        c[23] = alpha[4];
        c[24] = -(190320 * alpha[4] + 31720 * alpha[3] + 22080 * alpha[2] + 38040 * alpha[1] + 9500 * alpha[0] - 453) / 28260;
        c[25] = (55510 * alpha[4] + 9516 * alpha[3] + 6624 * alpha[2] + 11412 * alpha[1] + 2850 * alpha[0] - 159) / 1413;
        c[26] = -(44408 * alpha[4] + 7930 * alpha[3] + 5520 * alpha[2] + 9510 * alpha[1] + 2375 * alpha[0] - 183) / 471;
        c[27] = (166530 * alpha[4] + 31720 * alpha[3] + 22080 * alpha[2] + 38040 * alpha[1] + 9500 * alpha[0] - 1506) / 1413;
        c[28] = -(444080 * alpha[4] + 95160 * alpha[3] + 66240 * alpha[2] + 114120 * alpha[1] + 28500 * alpha[0] - 1323) / 5652;
        c[29] = (55510 * alpha[4] + 15860 * alpha[3] + 11040 * alpha[2] + 19020 * alpha[1] + 4750 * alpha[0] + 1551) / 2355;
        c[30] = -(1586 * alpha[3] + 1104 * alpha[2] + 1902 * alpha[1] + 475 * alpha[0] + 192) / 1413;
        c[31] = -(1586 * alpha[4] - 24) / 1413;
        for (int i = 0; i < 32; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 32; i++) c[i] *= -1;
            reverse(c, 32);
        }
    }
    void e8u_floating(real h, real* c, bool right) const // E8u_1.cpp nbs_floating
    {
        const real* alpha = pa;
        c[0] = (140 * alpha[0] - 363) / 140;
        c[1] = 7 - 8 * alpha[0];
        c[2] = (56 * alpha[0] - 21) / 2;
        c[3] = -(168 * alpha[0] - 35) / 3;
        c[4] = (280 * alpha[0] - 35) / 4;
        c[5] = -(280 * alpha[0] - 21) / 5;
        c[6] = (168 * alpha[0] - 7) / 6;
        c[7] = -(56 * alpha[0] - 1) / 7;
        c[8] = alpha[0];
        c[9] = 0;
        c[10] = 0;
        c[11] = (7 * alpha[1] - 1) / 7;
        c[12] = -(160 * alpha[1] + 29) / 20;
        c[13] = 28 * alpha[1] + 3;
        c[14] = -(112 * alpha[1] + 5) / 2;
        c[15] = (210 * alpha[1] + 5) / 3;
        c[16] = -(224 * alpha[1] + 3) / 4;
        c[17] = (140 * alpha[1] + 1) / 5;
        c[18] = -(336 * alpha[1] + 1) / 42;
        c[19] = alpha[1];
        c[20] = 0;
        c[21] = 0;
        c[22] = (42 * alpha[2] + 1) / 42;
        c[23] = -(24 * alpha[2] + 1) / 3;
        c[24] = (1680 * alpha[2] - 47) / 60;
        c[25] = -(168 * alpha[2] - 5) / 3;
        c[26] = (420 * alpha[2] - 5) / 6;
        c[27] = -(168 * alpha[2] - 1) / 3;
        c[28] = (336 * alpha[2] - 1) / 12;
        c[29] = -(840 * alpha[2] - 1) / 105;
        c[30] = alpha[2];
        c[31] = 0;
        c[32] = 0;
        c[33] = (105 * alpha[3] - 1) / 105;
        c[34] = -(80 * alpha[3] - 1) / 10;
        c[35] = (140 * alpha[3] - 3) / 5;
        c[36] = -(224 * alpha[3] + 1) / 4;
        c[37] = 70 * alpha[3] + 1;
        c[38] = -(560 * alpha[3] + 3) / 10;
        c[39] = (420 * alpha[3] + 1) / 15;
        c[40] = -(1120 * alpha[3] + 1) / 140;
        c[41] = alpha[3];
        c[42] = 0;
        c[43] = 0;
        c[44] = (140 * alpha[4] + 1) / 140;
        c[45] = -(120 * alpha[4] + 1) / 15;
        c[46] = (280 * alpha[4] + 3) / 10;
        c[47] = (-56 * alpha[4]) - 1;
        c[48] = (280 * alpha[4] + 1) / 4;
        c[49] = -(280 * alpha[4] - 3) / 5;
        c[50] = (280 * alpha[4] - 1) / 10;
        c[51] = -(840 * alpha[4] - 1) / 105;
        c[52] = alpha[4];
        c[53] = 0;
        c[54] = 0;
        c[55] = (840 * alpha[6] + 105 * alpha[5] - 1) / 105;
        c[56] = -(756 * alpha[6] + 96 * alpha[5] - 1) / 12;
        c[57] = (648 * alpha[6] + 84 * alpha[5] - 1) / 3;
        c[58] = -(2520 * alpha[6] + 336 * alpha[5] - 5) / 6;
        c[59] = (1512 * alpha[6] + 210 * alpha[5] - 5) / 3;
        c[60] = -(22680 * alpha[6] + 3360 * alpha[5] - 47) / 60;
        c[61] = (504 * alpha[6] + 84 * alpha[5] + 1) / 3;
        c[62] = -(1512 * alpha[6] + 336 * alpha[5] + 1) / 42;
        c[63] = alpha[5];
        c[64] = alpha[6];
        c[65] = 0;
        c[66] = -(43994496 * alpha[6] + 5499312 * alpha[5] + 3756354 * alpha[4] + 7475328 * alpha[3] + 2303742 * alpha[2] + 7419216 * alpha[1] + 1545558 * alpha[0] - 28865) / 5022570;
        c[67] = (8248968 * alpha[6] + 1047488 * alpha[5] + 715496 * alpha[4] + 1423872 * alpha[3] + 438808 * alpha[2] + 1413184 * alpha[1] + 294392 * alpha[0] - 5917) / 119585;
        c[68] = -(113128704 * alpha[6] + 14664832 * alpha[5] + 10016944 * alpha[4] + 19934208 * alpha[3] + 6143312 * alpha[2] + 19784576 * alpha[1] + 4121488 * alpha[0] - 92067) / 478340;
        c[69] = (164979360 * alpha[6] + 21997248 * alpha[5] + 15025416 * alpha[4] + 29901312 * alpha[3] + 9214968 * alpha[2] + 29676864 * alpha[1] + 6182232 * alpha[0] - 164197) / 358755;
        c[70] = -(131983488 * alpha[6] + 18331040 * alpha[5] + 12521180 * alpha[4] + 24917760 * alpha[3] + 7679140 * alpha[2] + 24730720 * alpha[1] + 5151860 * alpha[0] - 190693) / 239170;
        c[71] = (49493808 * alpha[6] + 7332416 * alpha[5] + 5008472 * alpha[4] + 9967104 * alpha[3] + 3071656 * alpha[2] + 9892288 * alpha[1] + 2060744 * alpha[0] - 163203) / 119585;
        c[72] = -(87988992 * alpha[6] + 14664832 * alpha[5] + 10016944 * alpha[4] + 19934208 * alpha[3] + 6143312 * alpha[2] + 19784576 * alpha[1] + 4121488 * alpha[0] - 169433) / 478340;
        c[73] = (32995872 * alpha[6] + 7332416 * alpha[5] + 5008472 * alpha[4] + 9967104 * alpha[3] + 3071656 * alpha[2] + 9892288 * alpha[1] + 2060744 * alpha[0] + 551009) / 837095;
        c[74] = -(130936 * alpha[5] + 89437 * alpha[4] + 177984 * alpha[3] + 54851 * alpha[2] + 176648 * alpha[1] + 36799 * alpha[0] + 20016) / 119585;
        c[75] = -(130936 * alpha[6] - 4176) / 119585;
        c[76] = -432.0 / 119585;
        for (int i = 0; i < 77; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 77; i++) c[i] *= -1;
            reverse(c, 77);
        }
    }
    void e8u_dirichlet(real h, real* c, bool right) const // E8u_1.cpp nbs_dirichlet
    {
        const real* alpha = pa;
        c[0] = (7 * alpha[1] - 1) / 7;
        c[1] = -(160 * alpha[1] + 29) / 20;
        c[2] = 28 * alpha[1] + 3;
        c[3] = -(112 * alpha[1] + 5) / 2;
        c[4] = (210 * alpha[1] + 5) / 3;
        c[5] = -(224 * alpha[1] + 3) / 4;
        c[6] = (140 * alpha[1] + 1) / 5;
        c[7] = -(336 * alpha[1] + 1) / 42;
        c[8] = alpha[1];
        c[9] = 0;
        c[10] = 0;
        c[11] = (42 * alpha[2] + 1) / 42;
        c[12] = -(24 * alpha[2] + 1) / 3;
        c[13] = (1680 * alpha[2] - 47) / 60;
        c[14] = -(168 * alpha[2] - 5) / 3;
        c[15] = (420 * alpha[2] - 5) / 6;
        c[16] = -(168 * alpha[2] - 1) / 3;
        c[17] = (336 * alpha[2] - 1) / 12;
        c[18] = -(840 * alpha[2] - 1) / 105;
        c[19] = alpha[2];
        c[20] = 0;
        c[21] = 0;
        c[22] = (105 * alpha[3] - 1) / 105;
        c[23] = -(80 * alpha[3] - 1) / 10;
        c[24] = (140 * alpha[3] - 3) / 5;
        c[25] = -(224 * alpha[3] + 1) / 4;
        c[26] = 70 * alpha[3] + 1;
        c[27] = -(560 * alpha[3] + 3) / 10;
        c[28] = (420 * alpha[3] + 1) / 15;
        c[29] = -(1120 * alpha[3] + 1) / 140;
        c[30] = alpha[3];
        c[31] = 0;
        c[32] = 0;
        c[33] = (140 * alpha[4] + 1) / 140;
        c[34] = -(120 * alpha[4] + 1) / 15;
        c[35] = (280 * alpha[4] + 3) / 10;
        c[36] = (-56 * alpha[4]) - 1;
        c[37] = (280 * alpha[4] + 1) / 4;
        c[38] = -(280 * alpha[4] - 3) / 5;
        c[39] = (280 * alpha[4] - 1) / 10;
        c[40] = -(840 * alpha[4] - 1) / 105;
        c[41] = alpha[4];
        c[42] = 0;
        c[43] = 0;
        c[44] = (840 * alpha[6] + 105 * alpha[5] - 1) / 105;
        c[45] = -(756 * alpha[6] + 96 * alpha[5] - 1) / 12;
        c[46] = (648 * alpha[6] + 84 * alpha[5] - 1) / 3;
        c[47] = -(2520 * alpha[6] + 336 * alpha[5] - 5) / 6;
        c[48] = (1512 * alpha[6] + 210 * alpha[5] - 5) / 3;
        c[49] = -(22680 * alpha[6] + 3360 * alpha[5] - 47) / 60;
        c[50] = (504 * alpha[6] + 84 * alpha[5] + 1) / 3;
        c[51] = -(1512 * alpha[6] + 336 * alpha[5] + 1) / 42;
        c[52] = alpha[5];
        c[53] = alpha[6];
        c[54] = 0;
        c[55] = -(43994496 * alpha[6] + 5499312 * alpha[5] + 3756354 * alpha[4] + 7475328 * alpha[3] + 2303742 * alpha[2] + 7419216 * alpha[1] + 1545558 * alpha[0] - 28865) / 5022570;
        c[56] = (8248968 * alpha[6] + 1047488 * alpha[5] + 715496 * alpha[4] + 1423872 * alpha[3] + 438808 * alpha[2] + 1413184 * alpha[1] + 294392 * alpha[0] - 5917) / 119585;
        c[57] = -(113128704 * alpha[6] + 14664832 * alpha[5] + 10016944 * alpha[4] + 19934208 * alpha[3] + 6143312 * alpha[2] + 19784576 * alpha[1] + 4121488 * alpha[0] - 92067) / 478340;
        c[58] = (164979360 * alpha[6] + 21997248 * alpha[5] + 15025416 * alpha[4] + 29901312 * alpha[3] + 9214968 * alpha[2] + 29676864 * alpha[1] + 6182232 * alpha[0] - 164197) / 358755;
        c[59] = -(131983488 * alpha[6] + 18331040 * alpha[5] + 12521180 * alpha[4] + 24917760 * alpha[3] + 7679140 * alpha[2] + 24730720 * alpha[1] + 5151860 * alpha[0] - 190693) / 239170;
        c[60] = (49493808 * alpha[6] + 7332416 * alpha[5] + 5008472 * alpha[4] + 9967104 * alpha[3] + 3071656 * alpha[2] + 9892288 * alpha[1] + 2060744 * alpha[0] - 163203) / 119585;
        c[61] = -(87988992 * alpha[6] + 14664832 * alpha[5] + 10016944 * alpha[4] + 19934208 * alpha[3] + 6143312 * alpha[2] + 19784576 * alpha[1] + 4121488 * alpha[0] - 169433) / 478340;
        c[62] = (32995872 * alpha[6] + 7332416 * alpha[5] + 5008472 * alpha[4] + 9967104 * alpha[3] + 3071656 * alpha[2] + 9892288 * alpha[1] + 2060744 * alpha[0] + 551009) / 837095;
        c[63] = -(130936 * alpha[5] + 89437 * alpha[4] + 177984 * alpha[3] + 54851 * alpha[2] + 176648 * alpha[1] + 36799 * alpha[0] + 20016) / 119585;
        c[64] = -(130936 * alpha[6] - 4176) / 119585;
        c[65] = -432.0 / 119585;
        for (int i = 0; i < 66; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 66; i++) c[i] *= -1;
            reverse(c, 66);
        }
    }

    // ---- E4u_1 (uniform-grid closures, psi ignored): src/stencils/E4u_1.cpp:77-127
    void e4u_floating(real h, real* c, bool right) const
    {
        c[0] = (6 * alpha[0] - 11) / 6;
        c[1] = 3 - 4 * alpha[0];
        c[2] = (12 * alpha[0] - 3) / 2;
        c[3] = -(12 * alpha[0] - 1) / 3;
        c[4] = alpha[0];
        c[5] = (3 * alpha[1] - 1) / 3;
        c[6] = -(8 * alpha[1] + 1) / 2;
        c[7] = 6 * alpha[1] + 1;
        c[8] = -(24 * alpha[1] + 1) / 6;
        c[9] = alpha[1];
        c[10] = -(168 * alpha[1] + 54 * alpha[0] - 11) / 138;
        c[11] = (112 * alpha[1] + 36 * alpha[0] - 15) / 23;
        c[12] = -(336 * alpha[1] + 108 * alpha[0] + 1) / 46;
        c[13] = (336 * alpha[1] + 108 * alpha[0] + 47) / 69;
        c[14] = -(28 * alpha[1] + 9 * alpha[0] + 2) / 23;
        for (int i = 0; i < 15; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 15; i++) c[i] *= -1;
            reverse(c, 15);
        }
    }
    void e4u_dirichlet(real h, real* c, bool right) const
    {
        c[0] = (3 * alpha[1] - 1) / 3;
        c[1] = -(8 * alpha[1] + 1) / 2;
        c[2] = 6 * alpha[1] + 1;
        c[3] = -(24 * alpha[1] + 1) / 6;
        c[4] = alpha[1];
        c[5] = -(168 * alpha[1] + 54 * alpha[0] - 11) / 138;
        c[6] = (112 * alpha[1] + 36 * alpha[0] - 15) / 23;
        c[7] = -(336 * alpha[1] + 108 * alpha[0] + 1) / 46;
        c[8] = (336 * alpha[1] + 108 * alpha[0] + 47) / 69;
        c[9] = -(28 * alpha[1] + 9 * alpha[0] + 2) / 23;
        for (int i = 0; i < 10; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 10; i++) c[i] *= -1;
            reverse(c, 10);
        }
    }

    static void reverse(real* c, int n) { std::reverse(c, c + n); }

    // ---- E2_2: src/stencils/E2_2.cpp:113-186
    static void e22_floating(real h, real psi, real* c, bool right)
    {
        real t6 = psi * psi;
        real t8 = psi * psi * psi;
        real t9 = -1 * t8;
        real t5 = -2 * psi;
        c[0] = psi;
        c[1] = (2 + t5 + -3 * t6 + t9) * 0.5;
        c[2] = -2 + 2 * t6 + t8;
        c[3] = (2 + -1 * t6 + t9) * 0.5;
        c[4] = (2 + 4 * psi) * 1.0 / (2 + 3 * psi + t6);
        c[5] = t5;
        c[6] = (-2 + 4 * t6) * 1.0 / (1 + psi);
        c[7] = (2 + -2 * t6) * 1.0 / (2 + psi);
        for (int i = 0; i < 8; i++) c[i] /= (h * h);
        if (right) reverse(c, 8);
    }
    static void e22_dirichlet(real h, real psi, real* c, bool right)
    {
        real t6 = psi * psi;
        real t5 = -2 * psi;
        c[0] = (2 + 4 * psi) * 1.0 / (2 + 3 * psi + t6);
        c[1] = t5;
        c[2] = (-2 + 4 * t6) * 1.0 / (1 + psi);
        c[3] = (2 + -2 * t6) * 1.0 / (2 + psi);
        for (int i = 0; i < 4; i++) c[i] /= (h * h);
        if (right) reverse(c, 4);
    }
    static void e22_neumann(real h, real psi, real* c, real* x, bool right)
    {
        real t5 = 2 * psi;
        real t9 = psi * psi;
        real t18 = -1 + psi;
        real t23 = psi * psi * psi;
        x[0] = -2;
        x[1] = 2 * t18;
        c[0] = (4 + 8 * psi) * -1 * 1.0 / (2 + 3 * psi + t9);
        c[1] = t5;
        c[2] = (2 + t5 + -4 * t9) * 1.0 / (1 + psi);
        c[3] = 2 * psi * 1.0 / (2 + psi) * t18;
        c[4] = psi;
        c[5] = (-4 + -1 * t23 + t9) * 0.5;
        c[6] = 2 + t23 + -2 * t9;
        c[7] = (2 + -3 * psi + t9) * -0.5 * psi;
        for (int i = 0; i < 8; i++) c[i] /= (h * h);
        for (int i = 0; i < 2; i++) x[i] /= h;
        if (right) {
            reverse(c, 8);
            reverse(x, 2);
            for (int i = 0; i < 2; i++) x[i] *= -1;
        }
    }

    // ---- E4_2: src/stencils/E4_2.cpp:204-311
    static void e42_floating(real h, real psi, real* c, bool right)
    {
        double t6 = -3 * psi;
        double t7 = psi * psi;
        double t9 = t7 * psi;
        double t11 = t7 * t7;
        double t12 = -t11;
        double t18 = 3 * psi;
        double t33 = -1 + psi;
        double t5 = 2 * psi;
        double t31 = 6 * psi;
        c[0] = t5;
        c[1] = (6 + t12 + t6 - 11 * t7 - 6 * t9) / 3.;
        c[2] = -5 + t11 + t6 + 6 * t7 + 5 * t9;
        c[3] = 4 + t12 + t18 - 3 * t7 - 4 * t9;
        c[4] = (-3 + t11 + t6 + 2 * t7 + 3 * t9) / 3.;
        c[5] = 12 / (6 + 5 * psi + t7);
        c[6] = -2 * psi;
        c[7] = -5 + t31;
        c[8] = (-2 * (4 + t18) * t33) / (2 + psi);
        c[9] = (t33 * (3 + t5)) / (3 + psi);
        c[10] = -psi / 12.;
        c[11] = (72 + t11 + t31 + 11 * t7 + 6 * t9) / 72.;
        c[12] = (-48 + t12 - 6 * t7 - 5 * t9) / 24.;
        c[13] = (24 + t11 + 3 * t7 + 4 * t9) / 24.;
        c[14] = -(t7 * (2 + t18 + t7)) / 72.;
        for (int i = 0; i < 15; i++) c[i] /= (h * h);
        if (right) reverse(c, 15);
    }
    static void e42_dirichlet(real h, real psi, real* c, bool right)
    {
        double t7 = psi * psi;
        double t9 = t7 * psi;
        double t11 = t7 * t7;
        double t12 = -t11;
        double t18 = 3 * psi;
        double t33 = -1 + psi;
        double t5 = 2 * psi;
        double t31 = 6 * psi;
        c[0] = 12 / (6 + 5 * psi + t7);
        c[1] = -2 * psi;
        c[2] = -5 + t31;
        c[3] = (-2 * (4 + t18) * t33) / (2 + psi);
        c[4] = (t33 * (3 + t5)) / (3 + psi);
        c[5] = -psi / 12.;
        c[6] = (72 + t11 + t31 + 11 * t7 + 6 * t9) / 72.;
        c[7] = (-48 + t12 - 6 * t7 - 5 * t9) / 24.;
        c[8] = (24 + t11 + 3 * t7 + 4 * t9) / 24.;
        c[9] = -(t7 * (2 + t18 + t7)) / 72.;
        for (int i = 0; i < 10; i++) c[i] /= (h * h);
        if (right) reverse(c, 10);
    }
    static void e42_neumann(real h, real psi, real* c, real* x, bool right)
    {
        double t7 = psi * psi;
        double t10 = 11 * psi;
        double t28 = -1 + psi;
        double t12 = t7 * psi;
        double t36 = t7 * t7;
        double t37 = -t36;
        double t51 = -6 * t7;
        double t8 = 3 * t7;
        x[0] = -3;
        x[1] = 3 * t28;
        x[2] = 0;
        c[0] = (-3 * (7 + 18 * psi + t8)) / (6 + t10 + t12 + 6 * t7);
        c[1] = 4 * psi;
        c[2] = (8 + t10 - 21 * t7) / (2 + 2 * psi);
        c[3] = (-1 - 8 * psi + 9 * t7) / (2 + psi);
        c[4] = (-5 * psi * t28) / (2. * (3 + psi));
        c[5] = psi;
        c[6] = (-21 - 9 * psi + 3 * t12 + t37 + 16 * t7) / 6.;
        c[7] = (8 + 12 * psi - 4 * t12 + t36 - 15 * t7) / 2.;
        c[8] = (-1 - 15 * psi + 5 * t12 + t37 + 12 * t7) / 2.;
        c[9] = (psi * (12 - 7 * psi + t12 + t51)) / 6.;
        c[10] = -psi / 12.;
        c[11] = (72 + 6 * psi + 6 * t12 + t36 + 11 * t7) / 72.;
        c[12] = (-48 - 5 * t12 + t37 + t51) / 24.;
        c[13] = (24 + 4 * t12 + t36 + t8) / 24.;
        c[14] = -(t7 * (2 + 3 * psi + t7)) / 72.;
        for (int i = 0; i < 15; i++) c[i] /= (h * h);
        for (int i = 0; i < 3; i++) x[i] /= h;
        if (right) {
            reverse(c, 15);
            reverse(x, 3);
            for (int i = 0; i < 3; i++) x[i] *= -1;
        }
    }

    // ---- E4_1: src/stencils/E4_1.cpp:95-342
    void e41_floating(real h, real psi, real* c, bool right) const
    {
        constexpr real psi_eps = 1e-4;
        psi = std::clamp(psi, psi_eps, 1.0 - psi_eps);
        real t5 = alpha[1]*psi;
        real t6 = psi * psi;
        real t7 = psi * psi * psi;
        real t8 = std::pow(psi, 4);
        real t9 = std::pow(psi, 5);
        real t10 = std::pow(psi, 6);
        real t11 = std::pow(psi, 7);
        real t12 = alpha[1]*t6;
        real t13 = alpha[1]*t7;
        real t14 = alpha[1]*t8;
        real t15 = alpha[1]*t9;
        real t16 = alpha[1]*t10;
        real t17 = alpha[1]*t11;
        real t18 = alpha[1]*std::pow(psi, 8);
        real t19 = alpha[1] * alpha[1];
        real t20 = psi*t19;
        real t21 = alpha[0]*t12;
        real t22 = alpha[0]*t13;
        real t23 = alpha[0]*t14;
        real t24 = alpha[0]*t15;
        real t25 = alpha[0]*t16;
        real t26 = t19*t6;
        real t27 = 99360*t19;
        real t28 = t19*t9;
        real t29 = alpha[0]*t26;
        real t30 = alpha[0]*t19;
        real t31 = 17280*t30;
        real t32 = 2484*alpha[0]*t17 + 216*alpha[0]*t18 + 3456*alpha[0]*t28 + 10368*alpha[1] + 13872*psi - 414*t10 - 36*t11 + 314677*t12 + 1282709*t13 - 182437*t14 - 496397*t15 - 169230*t16 - 21558*t17 - 1716*t18 + 276480*t20 + 20394*t21 - 94806*t22 + 14166*t23 + 41670*t24 + 15876*t25 + 218592*t26 - t27*t7 - t27*t8 - 19872*t28 - 38016*t29 + t31*t7 + t31*t8 - 184800*t5 + 33753*t6 + 9060*t7 - 6339*t8 - 2988*t9 - 7092;
        real t33 = 1.0 / (alpha[1]);
        real t34 = 1.0 / (psi - 1);
        real t35 = 1.0 / (1728*alpha[1] + 1721*psi + 12*t10 + 864*t12 + 144*t13 + 1584*t5 + 8070*t6 + 5617*t7 + 1464*t8 + 162*t9 - 1182);
        real t36 = t33*t34*t35;
        real t37 = t32*t36;
        real t38 = (1.0 / 6)*t37;
        real t39 = 1.0 / (psi);
        real t40 = t38*t39;
        real t41 = -t40;
        real t42 = -2.0 / 3*t32*t33*t34*t35*t39;
        real t43 = t37*t6;
        real t44 = psi*t37;
        real t45 = t37*t7;
        real t46 = (1.0 / 36)*t45 + (11.0 / 36)*t8;
        real t47 = (7.0 / 12)*t6;
        real t48 = (1.0 / 12)*t45 + (11.0 / 12)*t8;
        real t49 = (5.0 / 36)*t6;
        real t50 = alpha[0]*psi;
        real t51 = 6*alpha[0];
        real t52 = 168*alpha[0]*alpha[1] - 832*alpha[1]*t50 + 342*alpha[1] - 288*psi - 10194*t12 + 4350*t13 + 4671*t14 + 1032*t15 + 33*t16 + t17*t51 + 3*t17 - 756*t19*t50 + 330*t19*t7 + 66*t19*t8 + 5034*t20 - 770*t21 + 274*t22 + 752*t23 + 336*t24 + 66*t25 + 330*t26 + 540*t29 + 540*t30*t7 + 108*t30*t8 - 432*t30 - 5565*t5 - 18*t6 + 72*t7 + 18*t8 - 216;
        real t53 = t36*t52;
        real t54 = 4*t53;
        real t55 = psi*t54;
        real t56 = (1.0 / 3)*psi;
        real t57 = t56 - 1.0 / 3;
        real t58 = t53*t8;
        real t59 = -2.0 / 3*t58;
        real t60 = 16*t53;
        real t61 = psi*t53;
        real t62 = (1.0 / 18)*t8;
        real t63 = -13.0 / 9*psi + (17.0 / 18)*t6 + t62 + (4.0 / 9)*t7;
        real t64 = 24*t53;
        real t65 = t53*t6;
        real t66 = t53*t7;
        real t67 = -2*t58;
        real t68 = (1.0 / 6)*t8;
        real t69 = -19.0 / 6*psi + (11.0 / 6)*t6 + t68 + (7.0 / 6)*t7;
        real t70 = -7.0 / 3*psi + (7.0 / 6)*t6 + t68 + t7;
        real t71 = -11.0 / 18*psi + (5.0 / 18)*t6 + t62 + (5.0 / 18)*t7;
        real t72 = -alpha[0];
        real t73 = -4*alpha[0];
        real t74 = alpha[0]*t7;
        real t75 = alpha[0]*t6;
        real t76 = alpha[0]*t68 + (1.0 / 36)*t8;
        real t77 = (1.0 / 2)*alpha[0]*t8 + (1.0 / 12)*t8;
        real t78 = 6*t50;
        real t79 = psi*t64;
        real t80 = -1.0 / 6*t32*t33*t34*t35;
        real t81 = 2*psi;
        real t82 = (4.0 / 3)*t37;
        real t83 = 8*psi;
        real t84 = t51*t6 + t6*t64 - 149*t6;

        c[0] = (11.0 / 6)*psi + t38 + t41 - 11.0 / 6;
        c[1] = psi*(-t40 - 11.0 / 6);
        c[2] = (143.0 / 18)*psi + (13.0 / 18)*t32*t33*t34*t35 - t42 - 2.0 / 9*t43 - 17.0 / 36*t44 - t46 - 187.0 / 36*t6 - 22.0 / 9*t7 + 3;
        c[3] = -209.0 / 12*psi - t37*t39 + t37*t47 - 19.0 / 12*t37 + (11.0 / 12)*t44 + t48 + (121.0 / 12)*t6 + (77.0 / 12)*t7 - 3.0 / 2;
        c[4] = (77.0 / 6)*psi + (7.0 / 6)*t32*t33*t34*t35 - t42 - 1.0 / 2*t43 - 7.0 / 12*t44 - t48 - 77.0 / 12*t6 - 11.0 / 2*t7 + 1.0 / 3;
        c[5] = -121.0 / 36*psi + t37*t49 - 11.0 / 36*t37 + t41 + (5.0 / 36)*t44 + t46 + (55.0 / 36)*t6 + (55.0 / 36)*t7;
        c[6] = 0;
        c[7] = t54 - t55 + t57;
        c[8] = psi*(t54 - 1.0 / 3);
        c[9] = (34.0 / 3)*t33*t34*t35*t52*t6 + (16.0 / 3)*t33*t34*t35*t52*t7 - t59 - t60 - 52.0 / 3*t61 - t63 - 1.0 / 2;
        c[10] = 38*t61 + t64 - 22*t65 - 14*t66 + t67 + t69 + 1;
        c[11] = 14*t33*t34*t35*t52*t6 + 12*t33*t34*t35*t52*t7 - t60 - 28*t61 - t67 - t70 - 1.0 / 6;
        c[12] = t54 + t59 + (22.0 / 3)*t61 - 10.0 / 3*t65 - 10.0 / 3*t66 + t71;
        c[13] = 0;
        c[14] = -1.0 / 6*psi - t50 - t72 + 1.0 / 6;
        c[15] = psi*(alpha[0] + 1.0 / 6);
        c[16] = -13.0 / 18*psi - 13.0 / 3*t50 + (17.0 / 36)*t6 + (2.0 / 9)*t7 + t73 + (4.0 / 3)*t74 + (17.0 / 6)*t75 + t76 - 1;
        c[17] = (19.0 / 2)*alpha[0]*psi + (19.0 / 12)*psi + t51 - 11.0 / 12*t6 - 7.0 / 12*t7 - 7.0 / 2*t74 - 11.0 / 2*t75 - t77 + 1.0 / 2;
        c[18] = -7.0 / 6*psi + t47 - 7*t50 + (1.0 / 2)*t7 + t73 + 3*t74 + (7.0 / 2)*t75 + t77 + 1.0 / 3;
        c[19] = (11.0 / 6)*alpha[0]*psi + (11.0 / 36)*psi - t49 - 5.0 / 36*t7 - t72 - 5.0 / 6*t74 - 5.0 / 6*t75 - t76;
        c[20] = 0;
        c[21] = t57;
        c[22] = -t56;
        c[23] = 3.0 / 2 - t63;
        c[24] = t69 - 3;
        c[25] = 11.0 / 6 - t70;
        c[26] = t71;
        c[27] = 0;
        c[28] = (-149*psi - t51 - t64 + t78 + t79 - 11)/(11*psi + 6*t6 + t7 + 6);
        c[29] = (149.0 / 6)*psi - t50 - t55 - t80;
        c[30] = (8*alpha[0] - psi*t82 + 3*psi + 2*t50 + t53*t83 + 32*t53 - t82 + t84 + 14)/(t81 + 2);
        c[31] = (-24*alpha[0] + 2*psi*t32*t33*t34*t35 + 4*t32*t33*t34*t35 - 96*t53 - t78 - t79 - t83 - t84 - 38)/(t81 + 4);
        c[32] = (72*alpha[0] - 4*psi*t37 + 15*psi - 12*t37 + 18*t50 + 288*t53 + 72*t61 + t84 + 78)/(6*psi + 18);
        c[33] = -alpha[0] - t54 - t80;
        c[34] = 0;

        for (int i = 0; i < 35; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 35; i++) c[i] *= -1;
            reverse(c, 35);
        }
    }

    void e41_dirichlet(real h, real psi, real* c, bool right) const
    {
        constexpr real psi_eps = 1e-4;
        psi = std::clamp(psi, psi_eps, 1.0 - psi_eps);
        real t5 = alpha[0]*alpha[1];
        real t6 = alpha[1]*psi;
        real t7 = psi * psi;
        real t8 = psi * psi * psi;
        real t9 = std::pow(psi, 4);
        real t10 = alpha[0]*psi;
        real t11 = alpha[1] * alpha[1];
        real t12 = alpha[0]*t11;
        real t13 = alpha[1]*t7;
        real t14 = alpha[1]*t8;
        real t15 = alpha[1]*t9;
        real t16 = std::pow(psi, 5);
        real t17 = alpha[1]*t16;
        real t18 = std::pow(psi, 6);
        real t19 = alpha[1]*t18;
        real t20 = std::pow(psi, 7);
        real t21 = alpha[1]*t20;
        real t22 = psi*t11;
        real t23 = alpha[0]*t13;
        real t24 = alpha[0]*t14;
        real t25 = t5*t9;
        real t26 = t16*t5;
        real t27 = alpha[0]*t19;
        real t28 = 6*alpha[0];
        real t29 = 330*t11;
        real t30 = t11*t9;
        real t31 = 540*t12;
        real t32 = t12*t9;
        real t33 = -832*alpha[1]*t10 + 342*alpha[1] - 288*psi - 756*t10*t11 - 432*t12 - 10194*t13 + 4350*t14 + 4671*t15 + 1032*t17 + 33*t19 + t21*t28 + 3*t21 + 5034*t22 - 770*t23 + 274*t24 + 752*t25 + 336*t26 + 66*t27 + t29*t7 + t29*t8 + 66*t30 + t31*t7 + t31*t8 + 108*t32 + 168*t5 - 5565*t6 - 18*t7 + 72*t8 + 18*t9 - 216;
        real t34 = 1.0 / (alpha[1]);
        real t35 = 1.0 / (psi - 1);
        real t36 = 1.0 / (1728*alpha[1] + 1721*psi + 864*t13 + 144*t14 + 162*t16 + 12*t18 + 1584*t6 + 8070*t7 + 5617*t8 + 1464*t9 - 1182);
        real t37 = t34*t35*t36;
        real t38 = t33*t37;
        real t39 = 4*t38;
        real t40 = psi*t39;
        real t41 = (1.0 / 3)*psi;
        real t42 = t41 - 1.0 / 3;
        real t43 = t38*t9;
        real t44 = -2.0 / 3*t43;
        real t45 = 16*t38;
        real t46 = psi*t38;
        real t47 = (1.0 / 18)*t9;
        real t48 = -13.0 / 9*psi + t47 + (17.0 / 18)*t7 + (4.0 / 9)*t8;
        real t49 = 24*t38;
        real t50 = t38*t7;
        real t51 = t38*t8;
        real t52 = -2*t43;
        real t53 = (1.0 / 6)*t9;
        real t54 = -19.0 / 6*psi + t53 + (11.0 / 6)*t7 + (7.0 / 6)*t8;
        real t55 = -7.0 / 3*psi + t53 + (7.0 / 6)*t7 + t8;
        real t56 = -11.0 / 18*psi + t47 + (5.0 / 18)*t7 + (5.0 / 18)*t8;
        real t57 = -alpha[0];
        real t58 = -4*alpha[0];
        real t59 = alpha[0]*t8;
        real t60 = alpha[0]*t7;
        real t61 = alpha[0]*t53 + (1.0 / 36)*t9;
        real t62 = (1.0 / 2)*alpha[0]*t9 + (1.0 / 12)*t9;
        real t63 = 6*t10;
        real t64 = psi*t49;
        real t65 = std::pow(psi, 8);
        real t66 = 2484*alpha[0]*t21 - 1716*alpha[1]*t65 + 10368*alpha[1] + 13872*psi - 19872*t11*t16 + 218592*t11*t7 - 99360*t11*t8 + 3456*t12*t16 - 38016*t12*t7 + 17280*t12*t8 + 314677*t13 + 1282709*t14 - 182437*t15 - 2988*t16 - 496397*t17 - 414*t18 - 169230*t19 - 36*t20 - 21558*t21 + 276480*t22 + 20394*t23 - 94806*t24 + 14166*t25 + 41670*t26 + 15876*t27 - 99360*t30 + 17280*t32 + 216*t5*t65 - 184800*t6 + 33753*t7 + 9060*t8 - 6339*t9 - 7092;
        real t67 = -1.0 / 6*t34*t35*t36*t66;
        real t68 = 2*psi;
        real t69 = t37*t66;
        real t70 = (4.0 / 3)*t69;
        real t71 = 8*psi;
        real t72 = t28*t7 + t49*t7 - 149*t7;

        c[0] = t39 - t40 + t42;
        c[1] = psi*(t39 - 1.0 / 3);
        c[2] = (34.0 / 3)*t33*t34*t35*t36*t7 + (16.0 / 3)*t33*t34*t35*t36*t8 - t44 - t45 - 52.0 / 3*t46 - t48 - 1.0 / 2;
        c[3] = 38*t46 + t49 - 22*t50 - 14*t51 + t52 + t54 + 1;
        c[4] = 14*t33*t34*t35*t36*t7 + 12*t33*t34*t35*t36*t8 - t45 - 28*t46 - t52 - t55 - 1.0 / 6;
        c[5] = t39 + t44 + (22.0 / 3)*t46 - 10.0 / 3*t50 - 10.0 / 3*t51 + t56;
        c[6] = 0;
        c[7] = -1.0 / 6*psi - t10 - t57 + 1.0 / 6;
        c[8] = psi*(alpha[0] + 1.0 / 6);
        c[9] = -13.0 / 18*psi - 13.0 / 3*t10 + t58 + (4.0 / 3)*t59 + (17.0 / 6)*t60 + t61 + (17.0 / 36)*t7 + (2.0 / 9)*t8 - 1;
        c[10] = (19.0 / 2)*alpha[0]*psi + (19.0 / 12)*psi + t28 - 7.0 / 2*t59 - 11.0 / 2*t60 - t62 - 11.0 / 12*t7 - 7.0 / 12*t8 + 1.0 / 2;
        c[11] = -7.0 / 6*psi - 7*t10 + t58 + 3*t59 + (7.0 / 2)*t60 + t62 + (7.0 / 12)*t7 + (1.0 / 2)*t8 + 1.0 / 3;
        c[12] = (11.0 / 6)*alpha[0]*psi + (11.0 / 36)*psi - t57 - 5.0 / 6*t59 - 5.0 / 6*t60 - t61 - 5.0 / 36*t7 - 5.0 / 36*t8;
        c[13] = 0;
        c[14] = t42;
        c[15] = -t41;
        c[16] = 3.0 / 2 - t48;
        c[17] = t54 - 3;
        c[18] = 11.0 / 6 - t55;
        c[19] = t56;
        c[20] = 0;
        c[21] = (-149*psi - t28 - t49 + t63 + t64 - 11)/(11*psi + 6*t7 + t8 + 6);
        c[22] = (149.0 / 6)*psi - t10 - t40 - t67;
        c[23] = (8*alpha[0] - psi*t70 + 3*psi + 2*t10 + t38*t71 + 32*t38 - t70 + t72 + 14)/(t68 + 2);
        c[24] = (-24*alpha[0] + 2*psi*t34*t35*t36*t66 + 4*t34*t35*t36*t66 - 96*t38 - t63 - t64 - t71 - t72 - 38)/(t68 + 4);
        c[25] = (72*alpha[0] - 4*psi*t69 + 15*psi + 18*t10 + 288*t38 + 72*t46 - 12*t69 + t72 + 78)/(6*psi + 18);
        c[26] = -alpha[0] - t39 - t67;
        c[27] = 0;

        for (int i = 0; i < 28; i++) c[i] /= h;
        if (right) {
            for (int i = 0; i < 28; i++) c[i] *= -1;
            reverse(c, 28);
        }
    }

    // interpolants: E2_2.cpp:32-102, E4_2.cpp:44-185
    int interp_interior(real y, real* c) const
    {
        if (kind == 0 || kind == 5) { // polyE2_1.cpp:46-56: E2_2's
            if (y > 0) {
                c[0] = 1 + -1 * y;
                c[1] = y;
            } else {
                c[0] = -1 * y;
                c[1] = 1 + y;
            }
            return 2;
        }
        real y2 = y * y;
        real y3 = y * y * y;
        real y4 = y2 * y2;
        c[0] = (y * (2 - y - 2 * y2 + y3)) / 24.;
        c[1] = (y * (-4 + 4 * y + y2 - y3)) / 6.;
        c[2] = (4 - 5 * y2 + y4) / 4.;
        c[3] = -(y * (-4 - 4 * y + y2 + y3)) / 6.;
        c[4] = (y * (-2 - y + 2 * y2 + y3)) / 24.;
        return 5;
    }

    int interp_wall(int i, real y, real psi, real* c, bool right) const
    {
        if (kind == 5) return pe2_interp_wall(i, y, psi, c, right);
        if (kind == 0) {
            if (right) {
                const real t6 = 1 + psi;
                const real t7 = 1.0 / (t6);
                const real t8 = -1 + y;
                const real t9 = psi * t8;
                const real t5 = -1 + psi;
                const real t12 = -1 * psi * y;
                const real t20 = 1 + y;
                switch (i) {
                case 0:
                    c[0] = (psi + y + psi * y) * t5;
                    c[1] = 1 + t12 + -1 * psi * psi * t20 + y;
                    c[2] = psi * t20;
                    break;
                case 1:
                    c[0] = (t9 + y) * t5 * t7;
                    c[1] = psi + t12;
                    c[2] = (1 + t9 + y) * t7;
                    break;
                }
            } else {
                const real t8 = -1 + y;
                const real t11 = psi * y;
                const real t13 = -1 + psi;
                const real t17 = 1 + psi;
                const real t18 = 1.0 / (t17);
                switch (i) {
                case 0:
                    c[0] = psi + -1 * psi * y;
                    c[1] = 1 + t11 + psi * psi * t8 + -1 * y;
                    c[2] = (psi * t8 + y) * -1 * t13;
                    break;
                case 1:
                    c[0] = (-1 + psi + t11 + y) * -1 * t18;
                    c[1] = (1 + y) * psi;
                    c[2] = (psi + t11 + y) * -1 * t13 * t18;
                    break;
                }
            }
            return 3;
        }
        real y2 = y * y;
        real y3 = y2 * y;
        real psi2 = psi * psi;
        real psi3 = psi2 * psi;
        real psi4 = psi2 * psi2;
        if (right) {
            switch (i) {
            case 0:
                c[0] = ((-1 + psi) *
                        (6 * y * (2 + 3 * y + y2) + 6 * psi * (2 + 8 * y + 6 * y2 + y3) +
                         psi3 * (6 + 11 * y + 6 * y2 + y3) +
                         2 * psi2 * (9 + 22 * y + 12 * y2 + 2 * y3))) /
                       36.;
                c[1] = (6 * y * (3 + 4 * y + y2) + 6 * psi * (3 + 8 * y + 3 * y2) -
                        3 * psi2 * (-2 + 5 * y + 6 * y2 + y3) -
                        psi4 * (6 + 11 * y + 6 * y2 + y3) -
                        2 * psi3 * (9 + 22 * y + 12 * y2 + 2 * y3)) /
                       12.;
                c[2] = (-6 * y * (6 + 5 * y + y2) - 6 * psi * (6 + 10 * y + 3 * y2) +
                        6 * psi2 * (1 + 8 * y + 6 * y2 + y3) +
                        psi4 * (6 + 11 * y + 6 * y2 + y3) +
                        psi3 * (24 + 55 * y + 30 * y2 + 5 * y3)) /
                       12.;
                c[3] =
                    (-6 * psi * (-5 - y + 3 * y2 + y3) -
                     6 * psi3 * (5 + 11 * y + 6 * y2 + y3) +
                     6 * (6 + 11 * y + 6 * y2 + y3) - psi4 * (6 + 11 * y + 6 * y2 + y3) -
                     psi2 * (30 + 103 * y + 66 * y2 + 11 * y3)) /
                    36.;
                c[4] = (psi * (6 + 11 * y + 6 * y2 + y3)) / 6.;
                break;
            case 1:
                c[0] = ((-1 + psi) * (psi * (-1 + y) + y) * (2 + 3 * y + y2)) /
                       (2. * (3 + psi));
                c[1] = -((1 + y) * (2 * psi * (3 + y) - 2 * y * (3 + y) +
                                    3 * psi2 * (-2 + y + y2))) /
                       (2. * (2 + psi));
                c[2] = ((2 + y) * (psi * (3 + y) - y * (3 + y) + 3 * psi2 * (-1 + y2))) /
                       (2. * (1 + psi));
                c[3] = (psi * (2 + y - 2 * y2 - y3)) / 2.;
                c[4] = ((3 + 3 * psi * (-1 + y) + y) * (2 + 3 * y + y2)) /
                       (6 + 11 * psi + 6 * psi2 + psi3);
                break;
            default:
                c[0] = (y * (-24 * (-1 + y2) + 2 * psi2 * (-2 - y + 2 * y2 + y3) +
                             3 * psi3 * (-2 - y + 2 * y2 + y3) +
                             psi4 * (-2 - y + 2 * y2 + y3))) /
                       144.;
                c[1] = (y * (24 * (-2 + y + y2) + psi4 * (2 + y - 2 * y2 - y3) -
                             3 * psi2 * (-2 - y + 2 * y2 + y3) -
                             4 * psi3 * (-2 - y + 2 * y2 + y3))) /
                       48.;
                c[2] = ((-24 + 6 * psi2 * y + 5 * psi3 * y + psi4 * y) *
                        (-2 - y + 2 * y2 + y3)) /
                       48.;
                c[3] = -(y * (-24 * (2 + 3 * y + y2) + 6 * psi * (-2 - y + 2 * y2 + y3) +
                              11 * psi2 * (-2 - y + 2 * y2 + y3) +
                              6 * psi3 * (-2 - y + 2 * y2 + y3) +
                              psi4 * (-2 - y + 2 * y2 + y3))) /
                       144.;
                c[4] = (psi * y * (-2 - y + 2 * y2 + y3)) / 24.;
            }
        } else {
            switch (i) {
            case 0:
                c[0] = -(psi * (-6 + 11 * y - 6 * y2 + y3)) / 6.;
                c[1] = (-6 * (-6 + 11 * y - 6 * y2 + y3) +
                        psi4 * (-6 + 11 * y - 6 * y2 + y3) +
                        6 * psi3 * (-5 + 11 * y - 6 * y2 + y3) +
                        6 * psi * (5 - y - 3 * y2 + y3) +
                        psi2 * (-30 + 103 * y - 66 * y2 + 11 * y3)) /
                       36.;
                c[2] = (6 * y * (6 - 5 * y + y2) - 6 * psi * (6 - 10 * y + 3 * y2) +
                        psi3 * (24 - 55 * y + 30 * y2 - 5 * y3) -
                        6 * psi2 * (-1 + 8 * y - 6 * y2 + y3) -
                        psi4 * (-6 + 11 * y - 6 * y2 + y3)) /
                       12.;
                c[3] = (-6 * y * (3 - 4 * y + y2) + 6 * psi * (3 - 8 * y + 3 * y2) +
                        3 * psi2 * (2 + 5 * y - 6 * y2 + y3) +
                        psi4 * (-6 + 11 * y - 6 * y2 + y3) +
                        2 * psi3 * (-9 + 22 * y - 12 * y2 + 2 * y3)) /
                       12.;
                c[4] = -((-1 + psi) * (6 * y * (2 - 3 * y + y2) +
                                       6 * psi * (-2 + 8 * y - 6 * y2 + y3) +
                                       psi3 * (-6 + 11 * y - 6 * y2 + y3) +
                                       2 * psi2 * (-9 + 22 * y - 12 * y2 + 2 * y3))) /
                       36.;
                break;
            case 1:
                c[0] = -(((2 - 3 * y + y2) * (-3 + y + 3 * psi * (1 + y))) /
                         ((1 + psi) * (2 + psi) * (3 + psi)));
                c[1] = (psi * (2 - y - 2 * y2 + y3)) / 2.;
                c[2] = -((-2 + y) *
                         (-(psi * (-3 + y)) - (-3 + y) * y + 3 * psi2 * (-1 + y2))) /
                       (2. * (1 + psi));
                c[3] = ((-1 + y) * (-2 * psi * (-3 + y) - 2 * (-3 + y) * y +
                                    3 * psi2 * (-2 - y + y2))) /
                       (2. * (2 + psi));
                c[4] = -((-1 + psi) * (psi + y + psi * y) * (2 - 3 * y + y2)) /
                       (2. * (3 + psi));
                break;
            default:
                c[0] = (psi * y * (2 - y - 2 * y2 + y3)) / 24.;
                c[1] = -(y * (24 * (2 - 3 * y + y2) + 6 * psi * (2 - y - 2 * y2 + y3) +
                              11 * psi2 * (2 - y - 2 * y2 + y3) +
                              6 * psi3 * (2 - y - 2 * y2 + y3) +
                              psi4 * (2 - y - 2 * y2 + y3))) /
                       144.;
                c[2] = ((24 + 6 * psi2 * y + 5 * psi3 * y + psi4 * y) *
                        (2 - y - 2 * y2 + y3)) /
                       48.;
                c[3] = (y * (24 * (2 + y - y2) + psi4 * (-2 + y + 2 * y2 - y3) -
                             3 * psi2 * (2 - y - 2 * y2 + y3) -
                             4 * psi3 * (2 - y - 2 * y2 + y3))) /
                       48.;
                c[4] = (y * (24 * (-1 + y2) + 2 * psi2 * (2 - y - 2 * y2 + y3) +
                             3 * psi3 * (2 - y - 2 * y2 + y3) +
                             psi4 * (2 - y - 2 * y2 + y3))) /
                       144.;
            }
        }
        return 5;
    }

    // src/stencils/stencil.hpp:213-270
};

} // namespace sgb
