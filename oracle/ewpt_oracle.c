/*
 * ewpt_oracle.c -- CPU FP64 oracle for the EWPT-GPU RK4 lattice evolution.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is linked by the
 * tests, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg, never
 * by the product library.  It restates, in plain C and in the reference's own
 * floating-point evaluation order, the Julia routines of Teerthal/EWPT-GPU:
 *
 *   stencils            gpu-kernels-rk4/diff_scheme.jl:157-311
 *   covariant derivs    gpu-kernels-rk4/cov_derivs_temporal.jl:23-130
 *   field strengths     gpu-kernels-rk4/field_strengths.jl:34-311
 *   RK4 stage kernel    gpu-kernels-rk4/main_rk4.jl:52-661   (rk4_step!)
 *   RK4 combination     gpu-kernels-rk4/main_rk4.jl:6146-6437
 *   J_ext / damp        gpu-kernels-rk4/main_rk4.jl:5154-5172
 *   energies            gpu-kernels-rk4/main_rk4.jl:1334-2301, sums :6451-6560
 *   B, B_2, A fields    gpu-kernels-rk4/main_rk4.jl:2303-2822, 3718-4250, 3012-3528
 *   snapshot table      gpu-kernels-rk4/main_rk4.jl:6790-6805
 *   spectrum            gpu-kernels-rk4/spec_routines.jl:6-77
 *
 * Compile with -ffp-contract=off (no FMA contraction): Julia does not
 * contract a*b+c, so the expression order below reproduces its rounding.
 *
 * Parity pin: tests/golden/make_golden.py executes the reference's own Julia
 * source text (mechanically translated, evaluated in Python) on seeded 8^3
 * lattices; tests/test_oracle_golden.py checks this oracle against those
 * fixtures.
 *
 * Layout: 36 arrays of nx*ny*nz doubles, linear index i + nx*(j + ny*k)
 * (Julia column-major, x fastest), in the order
 *   0-3 phi_1..4 | 4-12 W_a_i (a=1..3 outer, i=x,y,z inner) | 13-15 Y_x,y,z |
 *   16-18 Gamma_1..3 | 19 Sigma | 20-23 dphi_dt | 24-32 dW_dt | 33-35 dY_dt
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define NARR 36

/* order: finite-difference order of every stencil (0 or 6: the driver's
 * `differentiations`, diff_scheme.jl:157-311; 2, 8, 10, 12: the modules
 * differentiations_{2nd,8th,10th,12th}_order, diff_scheme.jl:370-1438);
 * -2: the 2nd-order module exactly as written, whose branches miss the
 * planes i = 2 and i = N-1 (1-based), where it returns the caller's
 * placeholder 0 (every call site passes 0.). */
typedef struct or_params {
    int32_t nx, ny, nz, order;
    double dx, gw, gy, gp2, lambda, vev, beta_w, beta_y, theta_w;
} or_params;

/* ---------------------------------------------------------------- stencils */
/* diff_scheme.jl:157-233 (and 376-1403 for the other orders).  The
 * branches of each function there are a periodic wrap of one stencil; the
 * formula is identical in every branch, so the neighbours below are wrapped
 * indices and each formula keeps the written evaluation order. */
typedef struct {
    int64_t p[6], m[6]; /* +1..+6, -1..-6 */
    int gap;            /* order -2 at 1-based index 2 or N-1: the reference returns 0 */
} nbr_t;

static int g_order = 6; /* the stencil order in force (or_params.order, 0 -> 6) */

static inline int wrap(int i, int n) { i %= n; return i < 0 ? i + n : i; }

static void use_order(const or_params* p) { g_order = p->order ? p->order : 6; }

#define P_(d) A[s->p[(d) - 1]]
#define M_(d) A[s->m[(d) - 1]]
static inline double d1(const double* A, int64_t c, const nbr_t* s, double dx) {
    (void)c;
    switch (g_order) {
        case 2:
        case -2: /* diff_scheme.jl:1372-1381 */
            if (s->gap) return 0.;
            return (-M_(1) + P_(1)) / (2.0 * dx);
        case 8: /* diff_scheme.jl:376-415 */
            return (3 * M_(4) - 32 * M_(3) + 168 * M_(2) - 672 * M_(1) + 672 * P_(1) - 168 * P_(2) + 32 * P_(3) -
                    3 * P_(4)) / (840 * dx);
        case 10: /* diff_scheme.jl:633-680 */
            return (-2 * M_(5) + 25 * M_(4) - 150 * M_(3) + 600 * M_(2) - 2100 * M_(1) + 2100 * P_(1) - 600 * P_(2) +
                    150 * P_(3) - 25 * P_(4) + 2 * P_(5)) / (2520 * dx);
        case 12: /* diff_scheme.jl:939-1007 */
            return (5 * M_(6) - 72 * M_(5) + 495 * M_(4) - 2200 * M_(3) + 7425 * M_(2) - 23760 * M_(1) +
                    23760 * P_(1) - 7425 * P_(2) + 2200 * P_(3) - 495 * P_(4) + 72 * P_(5) - 5 * P_(6)) / (27720 * dx);
        default: /* diff_scheme.jl:157-181 */
            return (P_(3) - 9. * P_(2) + 45. * P_(1) - 45. * M_(1) + 9. * M_(2) - M_(3)) / (60 * dx);
    }
}
static inline double d2(const double* A, int64_t c, const nbr_t* s, double dx) {
    switch (g_order) {
        case 2:
        case -2: /* diff_scheme.jl:1405-1414 */
            if (s->gap) return 0.;
            return (M_(1) - 2.0 * A[c] + P_(1)) / (dx * dx);
        case 8: /* diff_scheme.jl:499-538 */
            return (-9 * M_(4) + 128 * M_(3) - 1008 * M_(2) + 8064 * M_(1) - 14350 * A[c] + 8064 * P_(1) -
                    1008 * P_(2) + 128 * P_(3) - 9 * P_(4)) / (5040 * dx * dx);
        case 10: /* diff_scheme.jl:780-827 */
            return (8 * M_(5) - 125 * M_(4) + 1000 * M_(3) - 6000 * M_(2) + 42000 * M_(1) - 73766 * A[c] +
                    42000 * P_(1) - 6000 * P_(2) + 1000 * P_(3) - 125 * P_(4) + 8 * P_(5)) / (25200 * dx * dx);
        case 12: /* diff_scheme.jl:1149-1217 */
            return (-50 * M_(6) + 864 * M_(5) - 7425 * M_(4) + 44000 * M_(3) - 222750 * M_(2) + 1425600 * M_(1) -
                    2480478 * A[c] + 1425600 * P_(1) - 222750 * P_(2) + 44000 * P_(3) - 7425 * P_(4) +
                    864 * P_(5) - 50 * P_(6)) / (831600 * dx * dx);
        default: /* diff_scheme.jl:235-259 */
            return (P_(3) / 90. - 3. * P_(2) / 20. + 3. * P_(1) / 2. - 49. * A[c] / 18. + 3. * M_(1) / 2. -
                    3. * M_(2) / 20. + M_(3) / 90.) / (dx * dx);
    }
}
#undef P_
#undef M_

typedef struct {
    int64_t c;
    nbr_t x, y, z;
} site_t;

static inline void make_site(const or_params* p, int i, int j, int k, site_t* s) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    const int64_t base_yz = (int64_t)j * sy + (int64_t)k * sz;
    const int64_t base_xz = (int64_t)i + (int64_t)k * sz;
    const int64_t base_xy = (int64_t)i + (int64_t)j * sy;
    s->c = i + base_yz;
    for (int d = 1; d <= 6; ++d) {
        s->x.p[d - 1] = wrap(i + d, nx) + base_yz;
        s->x.m[d - 1] = wrap(i - d, nx) + base_yz;
        s->y.p[d - 1] = wrap(j + d, ny) * sy + base_xz;
        s->y.m[d - 1] = wrap(j - d, ny) * sy + base_xz;
        s->z.p[d - 1] = wrap(k + d, nz) * sz + base_xy;
        s->z.m[d - 1] = wrap(k - d, nz) * sz + base_xy;
    }
    const int g2 = g_order == -2;
    s->x.gap = g2 && (i == 1 || i == nx - 2);
    s->y.gap = g2 && (j == 1 || j == ny - 2);
    s->z.gap = g2 && (k == 1 || k == nz - 2);
}

#define DX(A) d1((A), s.c, &s.x, dx)
#define DY(A) d1((A), s.c, &s.y, dx)
#define DZ(A) d1((A), s.c, &s.z, dx)
#define D2X(A) d2((A), s.c, &s.x, dx)
#define D2Y(A) d2((A), s.c, &s.y, dx)
#define D2Z(A) d2((A), s.c, &s.z, dx)

/* ----------------------------------------------- covariant derivatives */
/* cov_derivs_temporal.jl:23-130: D_iphi_a for i = x (W_a_2, Y_2), y, z. */
static inline double Dphi1(double dphi1, double p2, double p3, double p4,
                           double W1, double W2, double W3, double Y, double gw, double gy) {
    return (dphi1 + 0.5 * gw * ((W1) * (p4) - (W2) * (p3) + (W3) * (p2)) + 0.5 * gy * ((Y) * (p2)));
}
static inline double Dphi2(double dphi2, double p1, double p3, double p4,
                           double W1, double W2, double W3, double Y, double gw, double gy) {
    return (dphi2 - 0.5 * gw * ((W1) * (p3) + (W2) * (p4) + (W3) * (p1)) - 0.5 * gy * ((Y) * (p1)));
}
static inline double Dphi3(double dphi3, double p1, double p2, double p4,
                           double W1, double W2, double W3, double Y, double gw, double gy) {
    return (dphi3 + 0.5 * gw * ((W1) * (p2) + (W2) * (p1) - (W3) * (p4)) + 0.5 * gy * ((Y) * (p4)));
}
static inline double Dphi4(double dphi4, double p1, double p2, double p3,
                           double W1, double W2, double W3, double Y, double gw, double gy) {
    return (dphi4 - 0.5 * gw * ((W1) * (p1) - (W2) * (p2) - (W3) * (p3)) - 0.5 * gy * ((Y) * (p3)));
}

/* All per-site derivative quantities shared by the stage kernel and the
 * diagnostics (main_rk4.jl:84-330). */
typedef struct {
    double dphi[4][3];      /* d phi_a / d x_i */
    double dW[3][3][3];     /* d W_a_j / d x_i : [a][j][i] */
    double dY[3][3];        /* d Y_j / d x_i : [j][i] */
    double Dp[3][4];        /* D_i phi_a : [i][a] */
    double F[3][3];         /* W_a_{23,24,34} : [a][xy,xz,yz] */
    double FY[3];           /* Y_23, Y_24, Y_34 */
} derivs_t;

static void site_derivs(const or_params* p, const double* const* y, const site_t* sp, derivs_t* d) {
    const site_t s = *sp;
    const double dx = p->dx, gw = p->gw, gy = p->gy;
    const int64_t c = s.c;
    for (int a = 0; a < 4; ++a) {
        d->dphi[a][0] = DX(y[a]);
        d->dphi[a][1] = DY(y[a]);
        d->dphi[a][2] = DZ(y[a]);
    }
    for (int a = 0; a < 3; ++a)
        for (int jj = 0; jj < 3; ++jj) {
            const double* A = y[4 + 3 * a + jj];
            d->dW[a][jj][0] = DX(A);
            d->dW[a][jj][1] = DY(A);
            d->dW[a][jj][2] = DZ(A);
        }
    for (int jj = 0; jj < 3; ++jj) {
        d->dY[jj][0] = DX(y[13 + jj]);
        d->dY[jj][1] = DY(y[13 + jj]);
        d->dY[jj][2] = DZ(y[13 + jj]);
    }
    const double p1 = y[0][c], p2 = y[1][c], p3 = y[2][c], p4 = y[3][c];
    for (int i = 0; i < 3; ++i) {
        const double W1 = y[4 + i][c], W2 = y[7 + i][c], W3 = y[10 + i][c], Yi = y[13 + i][c];
        d->Dp[i][0] = Dphi1(d->dphi[0][i], p2, p3, p4, W1, W2, W3, Yi, gw, gy);
        d->Dp[i][1] = Dphi2(d->dphi[1][i], p1, p3, p4, W1, W2, W3, Yi, gw, gy);
        d->Dp[i][2] = Dphi3(d->dphi[2][i], p1, p2, p4, W1, W2, W3, Yi, gw, gy);
        d->Dp[i][3] = Dphi4(d->dphi[3][i], p1, p2, p3, W1, W2, W3, Yi, gw, gy);
    }
    /* field_strengths.jl:34-62,115-143,196-224: W_a_xy = dW_a_3_dx - dW_a_2_dy + gw*(W_b_2*W_c_3 - W_b_3*W_c_2) */
    const double W12 = y[4][c], W13 = y[5][c], W14 = y[6][c];
    const double W22 = y[7][c], W23 = y[8][c], W24 = y[9][c];
    const double W32 = y[10][c], W33 = y[11][c], W34 = y[12][c];
    d->F[0][0] = d->dW[0][1][0] - d->dW[0][0][1] + gw * (W22 * W33 - W23 * W32);
    d->F[0][1] = d->dW[0][2][0] - d->dW[0][0][2] + gw * (W22 * W34 - W24 * W32);
    d->F[0][2] = d->dW[0][2][1] - d->dW[0][1][2] + gw * (W23 * W34 - W24 * W33);
    d->F[1][0] = d->dW[1][1][0] - d->dW[1][0][1] + gw * (W32 * W13 - W33 * W12);
    d->F[1][1] = d->dW[1][2][0] - d->dW[1][0][2] + gw * (W32 * W14 - W34 * W12);
    d->F[1][2] = d->dW[1][2][1] - d->dW[1][1][2] + gw * (W33 * W14 - W34 * W13);
    d->F[2][0] = d->dW[2][1][0] - d->dW[2][0][1] + gw * (W12 * W23 - W13 * W22);
    d->F[2][1] = d->dW[2][2][0] - d->dW[2][0][2] + gw * (W12 * W24 - W14 * W22);
    d->F[2][2] = d->dW[2][2][1] - d->dW[2][1][2] + gw * (W13 * W24 - W14 * W23);
    /* field_strengths.jl:281-311 */
    d->FY[0] = d->dY[1][0] - d->dY[0][1];
    d->FY[1] = d->dY[2][0] - d->dY[0][2];
    d->FY[2] = d->dY[2][1] - d->dY[1][2];
}

/* ------------------------------------------------------ stage kernel */
/* main_rk4.jl:52-661 (rk4_step!) for one site.  r[0..19] = k outputs,
 * r[20..35] = kt outputs. */
static void site_rates(const or_params* p, const double* const* y, double* const* r,
                       int i, int j, int k, double Jex, double gam) {
    site_t s;
    make_site(p, i, j, k, &s);
    const int64_t c = s.c;
    const double dx = p->dx, gw = p->gw, gy = p->gy, gp2 = p->gp2;
    const double lambda = p->lambda, vev = p->vev, bW = p->beta_w, bY = p->beta_y;
    derivs_t d;
    site_derivs(p, y, &s, &d);

    const double p1 = y[0][c], p2 = y[1][c], p3 = y[2][c], p4 = y[3][c];
    const double W12 = y[4][c], W13 = y[5][c], W14 = y[6][c];
    const double W22 = y[7][c], W23 = y[8][c], W24 = y[9][c];
    const double W32 = y[10][c], W33 = y[11][c], W34 = y[12][c];
    const double Y2 = y[13][c], Y3 = y[14][c], Y4 = y[15][c];
    const double G1 = y[16][c], G2 = y[17][c], G3 = y[18][c], S = y[19][c];
    const double pt1 = y[20][c], pt2 = y[21][c], pt3 = y[22][c], pt4 = y[23][c];
    const double Wt12 = y[24][c], Wt13 = y[25][c], Wt14 = y[26][c];
    const double Wt22 = y[27][c], Wt23 = y[28][c], Wt24 = y[29][c];
    const double Wt32 = y[30][c], Wt33 = y[31][c], Wt34 = y[32][c];
    const double Yt2 = y[33][c], Yt3 = y[34][c], Yt4 = y[35][c];

    const double dp1x = d.dphi[0][0], dp1y = d.dphi[0][1], dp1z = d.dphi[0][2];
    const double dp2x = d.dphi[1][0], dp2y = d.dphi[1][1], dp2z = d.dphi[1][2];
    const double dp3x = d.dphi[2][0], dp3y = d.dphi[2][1], dp3z = d.dphi[2][2];
    const double dp4x = d.dphi[3][0], dp4y = d.dphi[3][1], dp4z = d.dphi[3][2];
    /* dW_a_j_d{x,y,z}: names follow main_rk4.jl:100-146 */
    const double dW12x = d.dW[0][0][0], dW12y = d.dW[0][0][1], dW12z = d.dW[0][0][2];
    const double dW13x = d.dW[0][1][0], dW13y = d.dW[0][1][1], dW13z = d.dW[0][1][2];
    const double dW14x = d.dW[0][2][0], dW14y = d.dW[0][2][1], dW14z = d.dW[0][2][2];
    const double dW22x = d.dW[1][0][0], dW22y = d.dW[1][0][1], dW22z = d.dW[1][0][2];
    const double dW23x = d.dW[1][1][0], dW23y = d.dW[1][1][1], dW23z = d.dW[1][1][2];
    const double dW24x = d.dW[1][2][0], dW24y = d.dW[1][2][1], dW24z = d.dW[1][2][2];
    const double dW32x = d.dW[2][0][0], dW32y = d.dW[2][0][1], dW32z = d.dW[2][0][2];
    const double dW33x = d.dW[2][1][0], dW33y = d.dW[2][1][1], dW33z = d.dW[2][1][2];
    const double dW34x = d.dW[2][2][0], dW34y = d.dW[2][2][1], dW34z = d.dW[2][2][2];

    const double dG1x = DX(y[16]), dG1y = DY(y[16]), dG1z = DZ(y[16]);
    const double dG2x = DX(y[17]), dG2y = DY(y[17]), dG2z = DZ(y[17]);
    const double dG3x = DX(y[18]), dG3y = DY(y[18]), dG3z = DZ(y[18]);
    const double dSx = DX(y[19]), dSy = DY(y[19]), dSz = DZ(y[19]);

    double lap[16];
    for (int a = 0; a < 16; ++a) {
        const double* A = y[a];
        /* d2f_dx2 + d2f_dy2 + d2f_dz2, main_rk4.jl:177-250 then :337 et seq. */
        lap[a] = D2X(A) + D2Y(A) + D2Z(A);
    }

    const double Dxp1 = d.Dp[0][0], Dxp2 = d.Dp[0][1], Dxp3 = d.Dp[0][2], Dxp4 = d.Dp[0][3];
    const double Dyp1 = d.Dp[1][0], Dyp2 = d.Dp[1][1], Dyp3 = d.Dp[1][2], Dyp4 = d.Dp[1][3];
    const double Dzp1 = d.Dp[2][0], Dzp2 = d.Dp[2][1], Dzp3 = d.Dp[2][2], Dzp4 = d.Dp[2][3];
    const double W1_23 = d.F[0][0], W1_24 = d.F[0][1], W1_34 = d.F[0][2];
    const double W2_23 = d.F[1][0], W2_24 = d.F[1][1], W2_34 = d.F[1][2];
    const double W3_23 = d.F[2][0], W3_24 = d.F[2][1], W3_34 = d.F[2][2];
    const double Y_23 = d.FY[0], Y_24 = d.FY[1], Y_34 = d.FY[2];

    const double mag = (p1 * p1 + p2 * p2 + p3 * p3 + p4 * p4);
    /* main_rk4.jl:350-352: the beta_W bracket as written (dW_1_3_dt, dW_1_4_dt
     * in all three rows) is shared by all four kt_phi rows. */
    const double bWterm = (Wt12 * W1_34 + Wt13 * (-W1_24) + Wt14 * W1_23 +
                           Wt22 * W2_34 + Wt13 * (-W2_24) + Wt14 * W2_23 +
                           Wt32 * W3_34 + Wt13 * (-W3_24) + Wt14 * W3_23);
    const double bYterm = (Yt2 * Y_34 + Yt3 * (-Y_24) + Yt4 * Y_23);

    /* kt_phi_1  main_rk4.jl:337-353 */
    r[20][c] = (lap[0] -
        0.5 * gw * (((-W12 * dp4x) - (W13 * dp4y) - (W14 * dp4z)) -
                    ((-W22 * dp3x) - (W23 * dp3y) - (W24 * dp3z)) +
                    ((-W32 * dp2x) - (W33 * dp2y) - (W34 * dp2z))) -
        0.5 * gy * (-Y2 * dp2x - Y3 * dp2y - Y4 * dp2z) -
        0.5 * gw * ((-W12 * Dxp4 - W13 * Dyp4 - W14 * Dzp4) -
                    (-W22 * Dxp3 - W23 * Dyp3 - W24 * Dzp3) +
                    (-W32 * Dxp2 - W33 * Dyp2 - W34 * Dzp2)) -
        0.5 * gy * (-Y2 * Dxp2 - Y3 * Dyp2 - Y4 * Dzp2) -
        2.0 * lambda * (p1 * p1 + p2 * p2 + p3 * p3 + p4 * p4 - vev * vev) * p1 +
        0.5 * ((gw * G3 + gy * S) * p2 - gw * G2 * p3 + gw * G1 * p4) -
        0.5 * Jex * p1 -
        gam * p1 * (p1 * pt1) / mag +
        bW * bWterm * p1 +
        bY * bYterm * p1);

    /* kt_phi_2  main_rk4.jl:355-371 */
    r[21][c] = (lap[1] +
        0.5 * gw * ((-W12 * dp3x - W13 * dp3y - W14 * dp3z) +
                    (-W22 * dp4x - W23 * dp4y - W24 * dp4z) +
                    (-W32 * dp1x - W33 * dp1y - W34 * dp1z)) +
        0.5 * gy * (-Y2 * dp1x - Y3 * dp1y - Y4 * dp1z) +
        0.5 * gw * ((-W12 * Dxp3 - W13 * Dyp3 - W14 * Dzp3) +
                    (-W22 * Dxp4 - W23 * Dyp4 - W24 * Dzp4) +
                    (-W32 * Dxp1 - W33 * Dyp1 - W34 * Dzp1)) +
        0.5 * gy * (-Y2 * Dxp1 - Y3 * Dyp1 - Y4 * Dzp1) -
        2.0 * lambda * (p1 * p1 + p2 * p2 + p3 * p3 + p4 * p4 - vev * vev) * p2 -
        0.5 * ((gw * G3 + gy * S) * p1 + gw * G1 * p3 + gw * G2 * p4) -
        0.5 * Jex * p2 -
        gam * p2 * (p2 * pt2) / mag +
        bW * bWterm * p2 +
        bY * bYterm * p2);

    /* kt_phi_3  main_rk4.jl:373-389 */
    r[22][c] = (lap[2] -
        0.5 * gw * ((-W12 * dp2x - W13 * dp2y - W14 * dp2z) +
                    (-W22 * dp1x - W23 * dp1y - W24 * dp1z) -
                    (-W32 * dp4x - W33 * dp4y - W34 * dp4z)) -
        0.5 * gy * (-Y2 * dp4x - Y3 * dp4y - Y4 * dp4z) -
        0.5 * gw * ((-W12 * Dxp2 - W13 * Dyp2 - W14 * Dzp2) +
                    (-W22 * Dxp1 - W23 * Dyp1 - W24 * Dzp1) -
                    (-W32 * Dxp4 - W33 * Dyp4 - W34 * Dzp4)) -
        0.5 * gy * (-Y2 * Dxp4 - Y3 * Dyp4 - Y4 * Dzp4) -
        2.0 * lambda * (p1 * p1 + p2 * p2 + p3 * p3 + p4 * p4 - vev * vev) * p3 +
        0.5 * ((-gw * G3 + gy * S) * p4 + gw * G2 * p1 + gw * G1 * p2) -
        0.5 * Jex * p3 -
        gam * p3 * (p3 * pt3) / mag +
        bW * bWterm * p3 +
        bY * bYterm * p3);

    /* kt_phi_4  main_rk4.jl:391-407 */
    r[23][c] = (lap[3] +
        0.5 * gw * ((-W12 * dp1x - W13 * dp1y - W14 * dp1z) -
                    (-W22 * dp2x - W23 * dp2y - W24 * dp2z) -
                    (-W32 * dp3x - W33 * dp3y - W34 * dp3z)) +
        0.5 * gy * (-Y2 * dp3x - Y3 * dp3y - Y4 * dp3z) +
        0.5 * gw * ((-W12 * Dxp1 - W13 * Dyp1 - W14 * Dzp1) -
                    (-W22 * Dxp2 - W23 * Dyp2 - W24 * Dzp2) -
                    (-W32 * Dxp3 - W33 * Dyp3 - W34 * Dzp3)) +
        0.5 * gy * (-Y2 * Dxp3 - Y3 * Dyp3 - Y4 * Dzp3) -
        2.0 * lambda * (p1 * p1 + p2 * p2 + p3 * p3 + p4 * p4 - vev * vev) * p4 -
        0.5 * ((-gw * G3 + gy * S) * p3 + gw * G1 * p1 - gw * G2 * p2) -
        0.5 * Jex * p4 -
        gam * p4 * (p4 * pt4) / mag +
        bW * bWterm * p4 +
        bY * bYterm * p4);

    /* Contractions shared by the beta terms of kt_W and kt_Y. */
    const double pdot = (pt1 * p1 + pt2 * p2 + pt3 * p3 + pt4 * p4);
    const double cx = (dp1x * p1 + dp2x * p2 + dp3x * p3 + dp4x * p4);
    const double cy = (dp1y * p1 + dp2y * p2 + dp3y * p3 + dp4y * p4);
    const double cz = (dp1z * p1 + dp2z * p2 + dp3z * p3 + dp4z * p4);

    /* kt_W_1_2  main_rk4.jl:409-424 */
    r[24][c] = (lap[4] +
        gw * (-(dW22x * W32 - dW32x * W22) -
              (dW22y * W33 - dW32y * W23) -
              (dW22z * W34 - dW32z * W24) -
              (W23 * W3_23 - W33 * W2_23) -
              (W24 * W3_24 - W34 * W2_24)) +
        gw * (p1 * Dxp4 - p2 * Dxp3 + p3 * Dxp2 - p4 * Dxp1) -
        dG1x - gw * (W22 * G3 - W32 * G2) -
        bW * pdot * 2.0 * W1_34 +
        2.0 * bW * (cy * Wt14 - cz * Wt13));
    /* kt_W_1_3  main_rk4.jl:426-441 */
    r[25][c] = (lap[5] +
        gw * (-(dW23x * W32 - dW33x * W22) -
              (dW23y * W33 - dW33y * W23) -
              (dW23z * W34 - dW33z * W24) -
              (W22 * (-W3_23) - W32 * (-W2_23)) -
              (W24 * W3_34 - W34 * W2_34)) +
        gw * (p1 * Dyp4 - p2 * Dyp3 + p3 * Dyp2 - p4 * Dyp1) -
        dG1y - gw * (W23 * G3 - W33 * G2) -
        bW * pdot * 2.0 * (-W1_24) +
        2.0 * bW * (cz * Wt12 - cx * Wt14));
    /* kt_W_1_4  main_rk4.jl:443-458 */
    r[26][c] = (lap[6] +
        gw * (-(dW24x * W32 - dW34x * W22) -
              (dW24y * W33 - dW34y * W23) -
              (dW24z * W34 - dW34z * W24) -
              (W22 * (-W3_24) - W32 * (-W2_24)) -
              (W23 * (-W3_34) - W33 * (-W2_34))) +
        gw * (p1 * Dzp4 - p2 * Dzp3 + p3 * Dzp2 - p4 * Dzp1) -
        dG1z - gw * (W24 * G3 - W34 * G2) -
        bW * pdot * 2.0 * W1_23 +
        2.0 * bW * (cx * Wt13 - cy * Wt12));
    /* kt_W_2_2  main_rk4.jl:460-475 */
    r[27][c] = (lap[7] +
        gw * (-(dW32x * W12 - dW12x * W32) -
              (dW32y * W13 - dW12y * W33) -
              (dW32z * W14 - dW12z * W34) -
              (W33 * W1_23 - W13 * W3_23) -
              (W34 * W1_24 - W14 * W3_24)) +
        gw * (-p1 * Dxp3 - p2 * Dxp4 + p3 * Dxp1 + p4 * Dxp2) -
        dG2x - gw * (W32 * G1 - W12 * G3) -
        bW * pdot * 2.0 * W2_34 +
        2.0 * bW * (cy * Wt24 - cz * Wt23));
    /* kt_W_2_3  main_rk4.jl:477-492 */
    r[28][c] = (lap[8] +
        gw * (-(dW33x * W12 - dW13x * W32) -
              (dW33y * W13 - dW13y * W33) -
              (dW33z * W14 - dW13z * W34) -
              (W32 * (-W1_23) - W12 * (-W3_23)) -
              (W34 * (W1_34) - W14 * W3_34)) +
        gw * (-p1 * Dyp3 - p2 * Dyp4 + p3 * Dyp1 + p4 * Dyp2) -
        dG2y - gw * (W33 * G1 - W13 * G3) -
        bW * pdot * 2.0 * (-W2_24) +
        2.0 * bW * (cz * Wt22 - cx * Wt24));
    /* kt_W_2_4  main_rk4.jl:494-509 */
    r[29][c] = (lap[9] +
        gw * (-(dW34x * W12 - dW14x * W32) -
              (dW34y * W13 - dW14y * W33) -
              (dW34z * W14 - dW14z * W34) -
              (W32 * (-W1_24) - W12 * (-W3_24)) -
              (W33 * (-W1_34) - W13 * (-W3_34))) +
        gw * (-p1 * Dzp3 - p2 * Dzp4 + p3 * Dzp1 + p4 * Dzp2) -
        dG2z - gw * (W34 * G1 - W14 * G3) -
        bW * pdot * 2.0 * W2_23 +
        2.0 * bW * (cx * Wt23 - cy * Wt22));
    /* kt_W_3_2  main_rk4.jl:511-526 */
    r[30][c] = (lap[10] +
        gw * (-(dW12x * W22 - dW22x * W12) -
              (dW12y * W23 - dW22y * W13) -
              (dW12z * W24 - dW22z * W14) -
              (W13 * W2_23 - W23 * W1_23) -
              (W14 * W2_24 - W24 * W1_24)) +
        gw * (p1 * Dxp2 - p2 * Dxp1 - p3 * Dxp4 + p4 * Dxp3) -
        dG3x - gw * (W12 * G2 - W22 * G1) -
        bW * pdot * 2.0 * W3_34 +
        2.0 * bW * (cy * Wt34 - cz * Wt33));
    /* kt_W_3_3  main_rk4.jl:528-543 */
    r[31][c] = (lap[11] +
        gw * (-(dW13x * W22 - dW23x * W12) -
              (dW13y * W23 - dW23y * W13) -
              (dW13z * W24 - dW23z * W14) -
              (W12 * (-W2_23) - W22 * (-W1_23)) -
              (W14 * W2_34 - W24 * (W1_34))) +
        gw * (p1 * Dyp2 - p2 * Dyp1 - p3 * Dyp4 + p4 * Dyp3) -
        dG3y - gw * (W13 * G2 - W23 * G1) -
        bW * pdot * 2.0 * (-W3_24) +
        2.0 * bW * (cz * Wt32 - cx * Wt34));
    /* kt_W_3_4  main_rk4.jl:545-560 */
    r[32][c] = (lap[12] +
        gw * (-(dW14x * W22 - dW24x * W12) -
              (dW14y * W23 - dW24y * W13) -
              (dW14z * W24 - dW24z * W14) -
              (W12 * (-W2_24) - W22 * (-W1_24)) -
              (W13 * (-W2_34) - W23 * (-W1_34))) +
        gw * (p1 * Dzp2 - p2 * Dzp1 - p3 * Dzp4 + p4 * Dzp3) -
        dG3z - gw * (W14 * G2 - W24 * G1) -
        bW * pdot * 2.0 * W3_23 +
        2.0 * bW * (cx * Wt33 - cy * Wt32));
    /* kt_Y_2..4  main_rk4.jl:562-581 */
    r[33][c] = ((lap[13] +
        gy * (p1 * Dxp2 - p2 * Dxp1 + p3 * Dxp4 - p4 * Dxp3) - dSx) -
        bY * pdot * 2.0 * Y_34 +
        2.0 * bY * (cy * Yt4 - cz * Yt3));
    r[34][c] = ((lap[14] +
        gy * (p1 * Dyp2 - p2 * Dyp1 + p3 * Dyp4 - p4 * Dyp3) - dSy) -
        bY * pdot * 2.0 * (-Y_24) +
        2.0 * bY * (cz * Yt2 - cx * Yt4));
    r[35][c] = ((lap[15] +
        gy * (p1 * Dzp2 - p2 * Dzp1 + p3 * Dzp4 - p4 * Dzp3) - dSz) -
        bY * pdot * 2.0 * Y_23 +
        2.0 * bY * (cx * Yt3 - cy * Yt2));

    /* k_field = momentum  main_rk4.jl:585-600 */
    for (int a = 0; a < 16; ++a) r[a][c] = y[20 + a][c];

    /* k_Gamma_a, k_Sigma  main_rk4.jl:603-655 */
    const double dvW1 = (DX(y[24]) + DY(y[25]) + DZ(y[26]));
    const double dvW2 = (DX(y[27]) + DY(y[28]) + DZ(y[29]));
    const double dvW3 = (DX(y[30]) + DY(y[31]) + DZ(y[32]));
    const double dvY = (DX(y[33]) + DY(y[34]) + DZ(y[35]));
    r[16][c] = ((1.0 - gp2) * dvW1 +
        gp2 * gw * (-((W22) * (Wt32) - (W32) * (Wt22)) -
                    ((W23) * (Wt33) - (W33) * (Wt23)) -
                    ((W24) * (Wt34) - (W34) * (Wt24))) +
        gp2 * gw * ((p1) * ((pt4)) - (p4) * ((pt1)) + (p3) * ((pt2)) - (p2) * ((pt3))));
    r[17][c] = ((1.0 - gp2) * dvW2 +
        gp2 * gw * (-((W32) * (Wt12) - (W12) * (Wt32)) -
                    ((W33) * (Wt13) - (W13) * (Wt33)) -
                    ((W34) * (Wt14) - (W14) * (Wt34))) +
        gp2 * gw * ((p3) * ((pt1)) - (p1) * ((pt3)) + (p4) * ((pt2)) - (p2) * ((pt4))));
    r[18][c] = ((1.0 - gp2) * dvW3 +
        gp2 * gw * (-((W12) * (Wt22) - (W22) * (Wt12)) -
                    ((W13) * (Wt23) - (W23) * (Wt13)) -
                    ((W14) * (Wt24) - (W24) * (Wt14))) +
        gp2 * gw * ((p1) * ((pt2)) - (p2) * ((pt1)) + (p4) * ((pt3)) - (p3) * ((pt4))));
    r[19][c] = ((1.0 - gp2) * dvY +
        gp2 * gy * ((p1) * ((pt2)) - (p2) * ((pt1)) + (p3) * ((pt4)) - (p4) * ((pt3))));
}

static inline int64_t nsites(const or_params* p) { return (int64_t)p->nx * p->ny * p->nz; }

static void split(const or_params* p, const double* base, const double** v) {
    const int64_t S = nsites(p);
    for (int a = 0; a < NARR; ++a) v[a] = base + a * S;
}
static void splitw(const or_params* p, double* base, double** v) {
    const int64_t S = nsites(p);
    for (int a = 0; a < NARR; ++a) v[a] = base + a * S;
}

/* Rates of the 36 arrays: one application of rk4_step!.  y and r are
 * contiguous [36][S] buffers and must not alias. */
int or_rates(const or_params* p, const double* y, double* r, double Jex, double gam) {
    use_order(p);
    if (!p || !y || !r || p->nx < 7 || p->ny < 7 || p->nz < 7) return 1;
    const double* yv[NARR];
    double* rv[NARR];
    split(p, y, yv);
    splitw(p, r, rv);
    const int nx = p->nx, ny = p->ny, nz = p->nz;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i)
                site_rates(p, yv, rv, i, j, k, Jex, gam);
    return 0;
}

/* J_ext and damp, main_rk4.jl:5154-5172. */
double or_jext(int64_t it, double dt, double mH, double t_sat, int thermal) {
    return (((double)it * dt * mH <= t_sat) && thermal) ? mH * mH : 0.0;
}
double or_damp(int64_t it, double dt, double mH, double t_sat, int thermal, double gamma_inp) {
    return (((double)it * dt * mH < t_sat) && thermal) ? 0.0 : gamma_inp;
}

/* One classical RK4 step, main_rk4.jl:6146-6437, with the reference's
 * broadcast rounding order: X_n = k*(dt/6) + X; X_n = k*(dt/3) + X_n (x2);
 * X = k*(dt/6) + X_n; stage arguments X + k*(dt/2), X + k*(dt/2), X + k*dt.
 * work must hold 3*36*S doubles. */
int or_rk4_step(const or_params* p, double* y, double* work, double dt, double Jex, double gam) {
    use_order(p);
    if (!p || !y || !work) return 1;
    const int64_t n = NARR * nsites(p);
    double* kk = work;
    double* yn = work + n;
    double* tmp = work + 2 * n;
    const double c6 = dt / 6., c3 = dt / 3., c2 = dt / 2.;
    int rc = or_rates(p, y, kk, Jex, gam);
    if (rc) return rc;
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < n; ++q) { yn[q] = kk[q] * c6 + y[q]; tmp[q] = y[q] + kk[q] * c2; }
    or_rates(p, tmp, kk, Jex, gam);
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < n; ++q) { yn[q] = kk[q] * c3 + yn[q]; tmp[q] = y[q] + kk[q] * c2; }
    or_rates(p, tmp, kk, Jex, gam);
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < n; ++q) { yn[q] = kk[q] * c3 + yn[q]; tmp[q] = y[q] + kk[q] * dt; }
    or_rates(p, tmp, kk, Jex, gam);
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < n; ++q) { y[q] = kk[q] * c6 + yn[q]; }
    return 0;
}

/* -------------------------------------------------------- diagnostics */
/* Per-site densities; out[q*S + c] for q in the order of or_field_* below. */
enum {
    DEN_PE = 0, DEN_KE, DEN_GE, DEN_EEW, DEN_MEW, DEN_EEY, DEN_MEY,
    DEN_BX, DEN_BY, DEN_BZ, DEN_B2X, DEN_B2Y, DEN_B2Z, DEN_AX, DEN_AY, DEN_AZ,
    DEN_MODPHI, DEN_GW1, DEN_GW2, DEN_GW3, DEN_GY, DEN_CW1, DEN_CW2, DEN_CW3, DEN_CY,
    NDEN
};

static void site_densities(const or_params* p, const double* const* y, double* const* o, int i, int j, int k) {
    site_t s;
    make_site(p, i, j, k, &s);
    const int64_t c = s.c;
    const double dx = p->dx, gw = p->gw, gy = p->gy, lambda = p->lambda, vev = p->vev, th = p->theta_w;
    derivs_t d;
    site_derivs(p, y, &s, &d);
    const double p1 = y[0][c], p2 = y[1][c], p3 = y[2][c], p4 = y[3][c];
    /* compute_PE!  main_rk4.jl:1340-1341 */
    {
        const double sdev = ((p1 * p1) + (p2 * p2) + (p3 * p3) + (p4 * p4) - vev * vev);
        o[DEN_PE][c] = (lambda * (sdev * sdev));
    }
    /* compute_KE!  main_rk4.jl:1659 */
    const double t1 = y[20][c], t2 = y[21][c], t3 = y[22][c], t4 = y[23][c];
    o[DEN_KE][c] = (t1 * t1 + t2 * t2 + t3 * t3 + t4 * t4);
    /* compute_GE!  main_rk4.jl:1498-1501 */
    const double (*D)[4] = d.Dp;
    o[DEN_GE][c] = (D[0][0] * D[0][0] + D[1][0] * D[1][0] + D[2][0] * D[2][0] +
                    D[0][1] * D[0][1] + D[1][1] * D[1][1] + D[2][1] * D[2][1] +
                    D[0][2] * D[0][2] + D[1][2] * D[1][2] + D[2][2] * D[2][2] +
                    D[0][3] * D[0][3] + D[1][3] * D[1][3] + D[2][3] * D[2][3]);
    /* compute_EEW!  main_rk4.jl:1817-1820 */
    {
        double e = 0;
        const double w0 = y[24][c], w1 = y[25][c], w2 = y[26][c], w3 = y[27][c], w4 = y[28][c],
                     w5 = y[29][c], w6 = y[30][c], w7 = y[31][c], w8 = y[32][c];
        e = (0.5 * ((w0 * w0) + (w1 * w1) + (w2 * w2) + (w3 * w3) + (w4 * w4) + (w5 * w5) +
                    (w6 * w6) + (w7 * w7) + (w8 * w8)));
        o[DEN_EEW][c] = e;
    }
    /* compute_MEW!  main_rk4.jl:1978-1981 */
    const double (*F)[3] = d.F;
    o[DEN_MEW][c] = (0.5 * (F[0][0] * F[0][0] + F[0][1] * F[0][1] + F[0][2] * F[0][2] +
                            F[1][0] * F[1][0] + F[1][1] * F[1][1] + F[1][2] * F[1][2] +
                            F[2][0] * F[2][0] + F[2][1] * F[2][1] + F[2][2] * F[2][2]));
    /* compute_EEY!  main_rk4.jl:2139-2140 */
    {
        const double a = y[33][c], b = y[34][c], e = y[35][c];
        o[DEN_EEY][c] = (0.5 * ((a * a) + (b * b) + (e * e)));
    }
    /* compute_MEY!  main_rk4.jl:2298 */
    o[DEN_MEY][c] = (0.5 * (d.FY[0] * d.FY[0] + d.FY[1] * d.FY[1] + d.FY[2] * d.FY[2]));

    /* compute_Bx!/By!/Bz!  main_rk4.jl:2455-2471, 2629-2645, 2803-2819 */
    const double mag = (p1 * p1 + p2 * p2 + p3 * p3 + p4 * p4);
    double n1, n2, n3;
    if (mag == 0.0) {
        n1 = 0.0; n2 = 0.0; n3 = 0.0;
    } else {
        n1 = -2. * (p1 * p3 + p2 * p4) / mag;
        n2 = +2. * (p2 * p3 - p1 * p4) / mag;
        n3 = (-(p1 * p1) - (p2 * p2) + (p3 * p3) + (p4 * p4)) / mag;
    }
    const double sw = sin(th), cw = cos(th);
    const double Dxp1 = D[0][0], Dxp2 = D[0][1], Dxp3 = D[0][2], Dxp4 = D[0][3];
    const double Dyp1 = D[1][0], Dyp2 = D[1][1], Dyp3 = D[1][2], Dyp4 = D[1][3];
    const double Dzp1 = D[2][0], Dzp2 = D[2][1], Dzp3 = D[2][2], Dzp4 = D[2][3];
    const double W1_23 = F[0][0], W1_24 = F[0][1], W1_34 = F[0][2];
    const double W2_23 = F[1][0], W2_24 = F[1][1], W2_34 = F[1][2];
    const double W3_23 = F[2][0], W3_24 = F[2][1], W3_34 = F[2][2];
    const double Y_23 = d.FY[0], Y_24 = d.FY[1], Y_34 = d.FY[2];
    const double hx = (Dyp1 * Dzp2 - Dyp2 * Dzp1 + Dyp3 * Dzp4 - Dyp4 * Dzp3);
    const double hy = (Dzp1 * Dxp2 - Dzp2 * Dxp1 + Dzp3 * Dxp4 - Dzp4 * Dxp3);
    const double hz = (Dxp1 * Dyp2 - Dxp2 * Dyp1 + Dxp3 * Dyp4 - Dxp4 * Dyp3);
    o[DEN_BX][c] = -(sw * (n1 * W1_34 + n2 * W2_34 + n3 * W3_34) + cw * Y_34 + (4. * sw / (gw * (vev * vev))) * hx);
    o[DEN_BY][c] = -(sw * (n1 * (-W1_24) + n2 * (-W2_24) + n3 * (-W3_24)) + cw * (-Y_24) + (4. * sw / (gw * (vev * vev))) * hy);
    o[DEN_BZ][c] = -(sw * (n1 * (W1_23) + n2 * W2_23 + n3 * W3_23) + cw * Y_23 + (4. * sw / (gw * (vev * vev))) * hz);
    /* compute_B_2_x/y/z!  main_rk4.jl:3883-3892 et seq. */
    if (mag == 0.0) {
        o[DEN_B2X][c] = 0.0; o[DEN_B2Y][c] = 0.0; o[DEN_B2Z][c] = 0.0;
    } else {
        o[DEN_B2X][c] = -(sw * (n1 * W1_34 + n2 * W2_34 + n3 * W3_34) + cw * Y_34 + (4. * sw / (gw * (mag * mag))) * hx);
        o[DEN_B2Y][c] = -(sw * (n1 * (-W1_24) + n2 * (-W2_24) + n3 * (-W3_24)) + cw * (-Y_24) + (4. * sw / (gw * (mag * mag))) * hy);
        o[DEN_B2Z][c] = -(sw * (n1 * (W1_23) + n2 * W2_23 + n3 * W3_23) + cw * Y_23 + (4. * sw / (gw * (mag * mag))) * hz);
    }
    /* compute_Ax/Ay/Az!  main_rk4.jl:3179, 3352, 3525 */
    o[DEN_AX][c] = (sw * (n1 * y[4][c] + n2 * y[7][c] + n3 * y[10][c]) + cw * y[13][c]);
    o[DEN_AY][c] = (sw * (n1 * (y[5][c]) + n2 * (y[8][c]) + n3 * (y[11][c])) + cw * (y[14][c]));
    o[DEN_AZ][c] = (sw * (n1 * (y[6][c]) + n2 * y[9][c] + n3 * y[12][c]) + cw * y[15][c]);
    o[DEN_MODPHI][c] = sqrt(p1 * p1 + p2 * p2 + p3 * p3 + p4 * p4);

    /* Gauss-constraint residuals: divergence of the electric field minus the
     * charge that multiplies gp2 in k_Gamma / k_Sigma (main_rk4.jl:603-655). */
    const double W12 = y[4][c], W13 = y[5][c], W14 = y[6][c];
    const double W22 = y[7][c], W23 = y[8][c], W24 = y[9][c];
    const double W32 = y[10][c], W33 = y[11][c], W34 = y[12][c];
    const double Wt12 = y[24][c], Wt13 = y[25][c], Wt14 = y[26][c];
    const double Wt22 = y[27][c], Wt23 = y[28][c], Wt24 = y[29][c];
    const double Wt32 = y[30][c], Wt33 = y[31][c], Wt34 = y[32][c];
    const double dvW1 = (DX(y[24]) + DY(y[25]) + DZ(y[26]));
    const double dvW2 = (DX(y[27]) + DY(y[28]) + DZ(y[29]));
    const double dvW3 = (DX(y[30]) + DY(y[31]) + DZ(y[32]));
    const double dvY = (DX(y[33]) + DY(y[34]) + DZ(y[35]));
    const double q1 = gw * (-((W22) * (Wt32) - (W32) * (Wt22)) - ((W23) * (Wt33) - (W33) * (Wt23)) -
                            ((W24) * (Wt34) - (W34) * (Wt24))) +
                      gw * ((p1) * (t4) - (p4) * (t1) + (p3) * (t2) - (p2) * (t3));
    const double q2 = gw * (-((W32) * (Wt12) - (W12) * (Wt32)) - ((W33) * (Wt13) - (W13) * (Wt33)) -
                            ((W34) * (Wt14) - (W14) * (Wt34))) +
                      gw * ((p3) * (t1) - (p1) * (t3) + (p4) * (t2) - (p2) * (t4));
    const double q3 = gw * (-((W12) * (Wt22) - (W22) * (Wt12)) - ((W13) * (Wt23) - (W23) * (Wt13)) -
                            ((W14) * (Wt24) - (W24) * (Wt14))) +
                      gw * ((p1) * (t2) - (p2) * (t1) + (p4) * (t3) - (p3) * (t4));
    const double qY = gy * ((p1) * (t2) - (p2) * (t1) + (p3) * (t4) - (p4) * (t3));
    o[DEN_GW1][c] = dvW1 - q1;
    o[DEN_GW2][c] = dvW2 - q2;
    o[DEN_GW3][c] = dvW3 - q3;
    o[DEN_GY][c] = dvY - qY;
    /* Auxiliary-field consistency: Gamma_a - d_i W_a_i, Sigma - d_i Y_i. */
    o[DEN_CW1][c] = y[16][c] - (d.dW[0][0][0] + d.dW[0][1][1] + d.dW[0][2][2]);
    o[DEN_CW2][c] = y[17][c] - (d.dW[1][0][0] + d.dW[1][1][1] + d.dW[1][2][2]);
    o[DEN_CW3][c] = y[18][c] - (d.dW[2][0][0] + d.dW[2][1][1] + d.dW[2][2][2]);
    o[DEN_CY][c] = y[19][c] - (d.dY[0][0] + d.dY[1][1] + d.dY[2][2]);
}

int or_ndensities(void) { return NDEN; }

/* Per-site density fields, [NDEN][S]. */
int or_densities(const or_params* p, const double* y, double* out) {
    use_order(p);
    if (!p || !y || !out || p->nx < 7 || p->ny < 7 || p->nz < 7) return 1;
    const double* yv[NARR];
    split(p, y, yv);
    const int64_t S = nsites(p);
    double* ov[NDEN];
    for (int q = 0; q < NDEN; ++q) ov[q] = out + q * S;
    const int nx = p->nx, ny = p->ny, nz = p->nz;
#pragma omp parallel for collapse(2) schedule(static)
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) site_densities(p, yv, ov, i, j, k);
    return 0;
}

/* Snapshot table (main_rk4.jl:6790-6805) plus Gauss-constraint columns.
 *  0 PE  1 KE  2 GE  3 EEW  4 MEW  5 EEY  6 MEY   (sum * dx^3)
 *  7 0.5*sum(B^2)*dx^3   8 0.5*sum(B_2^2)*dx^3   9 min|Phi|  10 0.0
 * 11 mean|Phi|  12 sum(B_2 . A)*dx^3  13 total energy = sum of 0..6
 * 14 sqrt(sum_a sum G_a^2 dx^3)  15 max|G_a|  16 sqrt(sum G_Y^2 dx^3)  17 max|G_Y|
 * 18 sqrt(sum_a sum (Gamma_a - div W_a)^2 dx^3)  19 sqrt(sum (Sigma - div Y)^2 dx^3) */
#define NDIAG 20
int or_ndiag(void) { return NDIAG; }

int or_diagnostics(const or_params* p, const double* y, double* out) {
    use_order(p);
    const int64_t S = nsites(p);
    double* den = (double*)malloc(sizeof(double) * NDEN * S);
    if (!den) return 2;
    int rc = or_densities(p, y, den);
    if (rc) { free(den); return rc; }
    const double vol = p->dx * p->dx * p->dx;
    double acc[NDIAG];
    for (int q = 0; q < NDIAG; ++q) acc[q] = 0.0;
    double minphi = INFINITY, maxgw = 0.0, maxgy = 0.0;
    double bsq[6] = {0, 0, 0, 0, 0, 0};
    for (int64_t c = 0; c < S; ++c) {
        for (int q = 0; q < 7; ++q) acc[q] += den[q * S + c];
        const double bx = den[DEN_BX * S + c], by = den[DEN_BY * S + c], bz = den[DEN_BZ * S + c];
        bsq[0] += bx * bx; bsq[1] += by * by; bsq[2] += bz * bz;
        const double b2x = den[DEN_B2X * S + c], b2y = den[DEN_B2Y * S + c], b2z = den[DEN_B2Z * S + c];
        bsq[3] += b2x * b2x; bsq[4] += b2y * b2y; bsq[5] += b2z * b2z;
        const double m = den[DEN_MODPHI * S + c];
        if (m < minphi) minphi = m;
        acc[11] += m;
        acc[12] += b2x * den[DEN_AX * S + c] + b2y * den[DEN_AY * S + c] + b2z * den[DEN_AZ * S + c];
        for (int a = 0; a < 3; ++a) {
            const double g = den[(DEN_GW1 + a) * S + c];
            acc[14] += g * g;
            if (fabs(g) > maxgw) maxgw = fabs(g);
            const double cc = den[(DEN_CW1 + a) * S + c];
            acc[18] += cc * cc;
        }
        const double gyv = den[DEN_GY * S + c];
        acc[16] += gyv * gyv;
        if (fabs(gyv) > maxgy) maxgy = fabs(gyv);
        const double cy = den[DEN_CY * S + c];
        acc[19] += cy * cy;
    }
    free(den);
    for (int q = 0; q < 7; ++q) out[q] = acc[q] * vol;
    /* main_rk4.jl:6797-6798: (0.5*(bxe+bye+bze))*Vol */
    out[7] = (0.5 * (bsq[0] + bsq[1] + bsq[2])) * vol;
    out[8] = (0.5 * (bsq[3] + bsq[4] + bsq[5])) * vol;
    out[9] = minphi;
    out[10] = 0.0;
    out[11] = acc[11] / (double)S;
    out[12] = acc[12] * vol;
    out[13] = out[0] + out[1] + out[2] + out[3] + out[4] + out[5] + out[6];
    out[14] = sqrt(acc[14] * vol);
    out[15] = maxgw;
    out[16] = sqrt(acc[16] * vol);
    out[17] = maxgy;
    out[18] = sqrt(acc[18] * vol);
    out[19] = sqrt(acc[19] * vol);
    return 0;
}

/* ------------------------------------------------------------ spectra */
/* K_c_mag squared, spec_routines.jl:6-30 (0-based index here). */
static inline int64_t kc2(int x, int n) {
    const int K = (x <= n / 2) ? x : x - n;
    return (int64_t)K * K;
}

static int cmp_i64(const void* a, const void* b) {
    const int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
    return (x > y) - (x < y);
}

/* Number of distinct |K| on a cut^3 index lattice, spec_routines.jl:32-43. */
int64_t or_kc_bin_nums(int cx, int cy, int cz) {
    const int64_t n = (int64_t)cx * cy * cz;
    int64_t* v = (int64_t*)malloc(sizeof(int64_t) * n);
    if (!v) return -1;
    int64_t q = 0;
    for (int i = 0; i < cx; ++i)
        for (int j = 0; j < cy; ++j)
            for (int k = 0; k < cz; ++k) v[q++] = kc2(i, cx) + kc2(j, cy) + kc2(k, cz);
    qsort(v, n, sizeof(int64_t), cmp_i64);
    int64_t u = 0;
    for (int64_t t = 0; t < n; ++t)
        if (t == 0 || v[t] != v[t - 1]) ++u;
    free(v);
    return u;
}

/* convolve_1d, spec_routines.jl:47-77: mean of P over all sites of the full
 * lattice that share the same |K|, for the first nbins distinct |K| in
 * increasing order (nbins = or_kc_bin_nums(cut)).  P is [S] in column-major
 * order.  kout[b] = |K|, pout[b] = mean.  Returns nbins. */
int64_t or_convolve_1d(const or_params* p, const double* P, int cx, int cy, int cz,
                       double* kout, double* pout, int64_t maxbins) {
    const int64_t nb = or_kc_bin_nums(cx, cy, cz);
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const int64_t kmax = (int64_t)(nx / 2) * (nx / 2) + (int64_t)(ny / 2) * (ny / 2) + (int64_t)(nz / 2) * (nz / 2);
    double* sum = (double*)calloc(kmax + 1, sizeof(double));
    int64_t* cnt = (int64_t*)calloc(kmax + 1, sizeof(int64_t));
    if (!sum || !cnt) { free(sum); free(cnt); return -1; }
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int64_t m = kc2(i, nx) + kc2(j, ny) + kc2(k, nz);
                sum[m] += P[i + (int64_t)nx * (j + (int64_t)ny * k)];
                cnt[m] += 1;
            }
    int64_t b = 0;
    for (int64_t m = 0; m <= kmax && b < nb && b < maxbins; ++m) {
        if (!cnt[m]) continue;
        kout[b] = sqrt((double)m);
        pout[b] = sum[m] / (double)cnt[m];
        ++b;
    }
    free(sum);
    free(cnt);
    return b;
}

/* Integer |n|^2 thresholds of nshell log-spaced shells over |n| in [1, nmax]:
 * mode m = |n|^2 is in shell b when thr[b] <= m < thr[b+1]; thr[0] = 1,
 * thr[nshell] = nmax^2 + 1.  thr[b] is the smallest m with sqrt(m) >= e_b,
 * e_b = exp(log(nmax) b / nshell). */
void or_shell_thresholds(int nmax, int nshell, int64_t* thr) {
    const double lmax = log((double)nmax);
    for (int b = 0; b <= nshell; ++b) {
        if (b == 0) { thr[b] = 1; continue; }
        if (b == nshell) { thr[b] = (int64_t)nmax * nmax + 1; continue; }
        const double e = exp(lmax * (double)b / (double)nshell);
        int64_t m = (int64_t)ceil(e * e);
        while (m > 1 && sqrt((double)(m - 1)) >= e) --m;
        while (sqrt((double)m) < e) ++m;
        thr[b] = m;
    }
}

/* Log-spaced shell spectrum over the full lattice: nshell shells in |n| over
 * [1, nmax], nmax = min(nx,ny,nz)/2, DC and |n| > nmax excluded.  Outputs
 * per-shell sum, count, mean and the geometric shell centre. */
int or_shell_spectrum(const or_params* p, const double* P, int nshell,
                      double* ssum, double* scount, double* smean, double* kcenter) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    int nm = nx < ny ? nx : ny;
    nm = nm < nz ? nm : nz;
    const int nmax = nm / 2;
    int64_t* thr = (int64_t*)malloc(sizeof(int64_t) * (nshell + 1));
    if (!thr) return 2;
    or_shell_thresholds(nmax, nshell, thr);
    const double lmax = log((double)nmax);
    for (int b = 0; b < nshell; ++b) {
        ssum[b] = 0; scount[b] = 0; smean[b] = 0;
        kcenter[b] = exp(lmax * (b + 0.5) / nshell);
    }
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int64_t m = kc2(i, nx) + kc2(j, ny) + kc2(k, nz);
                if (m == 0 || m >= thr[nshell]) continue;
                int b = 0;
                while (b + 1 < nshell && thr[b + 1] <= m) ++b;
                ssum[b] += P[i + (int64_t)nx * (j + (int64_t)ny * k)];
                scount[b] += 1;
            }
    for (int b = 0; b < nshell; ++b) smean[b] = scount[b] > 0 ? ssum[b] / scount[b] : 0.0;
    free(thr);
    return 0;
}

/* ---------------------------------------------------- initial conditions */
/* initializer!, main_rk4.jl:4930-4946: add one bubble's rmag profile times
 * (p1..p4) to phi.  ib, jb, kb are the reference's 1-based centre indices. */
int or_bubble_rmag(const or_params* p, double* y, double ib, double jb, double kb,
                   double q1, double q2, double q3, double q4, double mH) {
    const int nx = p->nx, ny = p->ny, nz = p->nz;
    const double dx = p->dx;
    const double rkx = M_PI / ((nx - 1) * dx), rky = M_PI / ((ny - 1) * dx), rkz = M_PI / ((nz - 1) * dx);
    const int64_t S = nsites(p);
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                /* 1-based (i-1) == 0-based i */
                const double sx = sin(rkx * ((i) - (ib - 0.5)) * dx);
                const double sy = sin(rky * ((j) - (jb - 0.5)) * dx);
                const double sz = sin(rkz * ((k) - (kb - 0.5)) * dx);
                const double rb = sqrt((1.0 / (rkx * rkx)) * (sx * sx) + (1.0 / (rky * rky)) * (sy * sy) +
                                       (1.0 / (rkz * rkz)) * (sz * sz));
                const double s2 = sqrt(2.0);
                const double rmag = (1.0 + (s2 - 1.0) * (s2 - 1.0)) * exp(-mH * rb / s2) /
                                    (1.0 + ((s2 - 1.0) * (s2 - 1.0)) * exp(-s2 * mH * rb));
                const int64_t c = i + (int64_t)nx * (j + (int64_t)ny * k);
                y[0 * S + c] = y[0 * S + c] + rmag * q1;
                y[1 * S + c] = y[1 * S + c] + rmag * q2;
                y[2 * S + c] = y[2 * S + c] + rmag * q3;
                y[3 * S + c] = y[3 * S + c] + rmag * q4;
            }
    return 0;
}

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void or_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
