// devphys.cu -- the stage kernels' per-site arithmetic compiled for the host
// (test and measurement infrastructure, never linked into libewpt).
//
// The per-site arithmetic of the stage kernels is the template site_rates
// (csrc/physics.cuh) over the accessor SiteAcc (csrc/accessors.cuh).  This
// file compiles those same templates for the host (EWPT_ARITH = inline) and
// instantiates them twice:
//
//  * with double: dp_rates() evaluates all 36 rates at every site of a
//    periodic lattice, so the tests compare the kernels' own equations with
//    the oracle's restatement of rk4_step! on the CPU;
//  * with an operator-counting scalar type: dp_count() counts every
//    addition, subtraction, multiplication and division the kernels' source
//    performs for one site, exactly.  The epilogue of each stage (the RK4
//    combination of stage.cu's Fp64Sink: two fused multiply-adds per array in
//    stages 1-3, one in stage 4) is counted from its formulas.
//
// FLOPs are counted as the source writes them: an addition, subtraction or
// multiplication is 1 FLOP and a fused multiply-add 2, so the total does not
// depend on which products the compiler contracts.  Negations are free
// (operand modifiers) and counted apart, divisions too (one per site and
// stage, 1/|Phi|^2).  The FP64 pipe instruction figure is an estimate: it
// fuses a product into the addition that consumes it, as the compiler's
// contraction does, and counts every other operation as one instruction.
//
// Build: nvcc -shared -Xcompiler -fPIC -std=c++17 --expt-relaxed-constexpr
//        -gencode arch=compute_103a,code=sm_103a -I include -I csrc
//        oracle/devphys.cu -o oracle/build/libdevphys.so   (oracle/devphys.py)
#define EWPT_ARITH inline
#include <cstdio>
#include <cstring>

#include "accessors.cuh"

namespace {

struct Tally {
    long long add = 0, mul = 0, div = 0, neg = 0;
    long long inst = 0;  // FP64 pipe instructions with single-use products fused into FMAs
};
Tally g_t;
int g_section = 0;  // 0 = physics, 1 = stencils
Tally g_sec[2];

inline void bump(long long Tally::*f, int n = 1) {
    g_t.*f += n;
    g_sec[g_section].*f += n;
}

// A value, or a product not yet issued (`pend`): a product meeting an
// addition becomes one fused multiply-add, as the compiler contracts it;
// a product used any other way is issued as a multiplication first.
struct Op {
    double v;
    bool pend;
    Op() : v(0), pend(false) {}
    Op(double x) : v(x), pend(false) {}
};
inline Op issued(Op a) {
    if (a.pend) {
        bump(&Tally::inst);
        a.pend = false;
    }
    return a;
}
inline Op addsub(Op a, Op b, double v) {
    bump(&Tally::add);
    if (a.pend && b.pend) a = issued(a);
    bump(&Tally::inst);  // DADD, or the DFMA that absorbs the pending product
    Op r(v);
    return r;
}
inline Op operator+(Op a, Op b) { return addsub(a, b, a.v + b.v); }
inline Op operator-(Op a, Op b) { return addsub(a, b, a.v - b.v); }
inline Op operator*(Op a, Op b) {
    bump(&Tally::mul);
    a = issued(a);
    b = issued(b);
    Op r(a.v * b.v);
    r.pend = true;
    return r;
}
inline Op operator/(Op a, Op b) {
    bump(&Tally::div);
    a = issued(a);
    b = issued(b);
    return Op(a.v / b.v);
}
inline Op operator-(Op a) {
    bump(&Tally::neg);
    Op r = a;
    r.v = -a.v;
    return r;
}
inline Op& operator+=(Op& a, Op b) { a = a + b; return a; }
inline Op& operator-=(Op& a, Op b) { a = a - b; return a; }

// The accessor the kernels use, with the stencil work attributed to its own
// section of the tally.
struct CountAcc {
    SiteAcc<double, Op, SrcPtr36<double>> A;
    Op v(int a) const { return A.v(a); }
    void grad(int a, Op& x, Op& y, Op& z) const {
        g_section = 1;
        A.grad(a, x, y, z);
        g_section = 0;
    }
    void grad_lap(int a, Op& x, Op& y, Op& z, Op& l) const {
        g_section = 1;
        A.grad_lap(a, x, y, z, l);
        g_section = 0;
    }
    Op div3(int a) const {
        g_section = 1;
        const Op r = A.div3(a);
        g_section = 0;
        return r;
    }
};

struct NullSink {
    int got = 0;
    void operator()(int, Op r) {
        issued(r);  // a rate that is a bare product is issued before the epilogue
        ++got;
    }
};

// One site's rates on a 7^3 periodic box of arbitrary values.
template <bool BETA>
Tally count_rates(int* rates) {
    const int n = 7, S = n * n * n;
    static double buf[36 * 343];
    for (int q = 0; q < 36 * S; ++q) buf[q] = 0.1 + 1e-3 * (q % 97);
    Ptr36 P;
    for (int a = 0; a < 36; ++a) P.p[a] = buf + a * S;
    SrcPtr36<double> src{P};
    CountAcc acc{{src}};
    acc.A.c = 3 + n * (3 + n * 3);
    for (int d = 0; d < 3; ++d) {
        const int sx[3] = {1, n, n * n};
        for (int ax = 0; ax < 3; ++ax) {
            int* o = ax == 0 ? acc.A.ox : ax == 1 ? acc.A.oy : acc.A.oz;
            o[d] = (d + 1) * sx[ax];
            o[d + 3] = -(d + 1) * sx[ax];
        }
    }
    acc.A.s = make_stencil<Op>(0.25);
    ewpt_params p{};
    p.gw = 0.65;
    p.gy = 0.35;
    p.gp2 = 0.99;
    p.lambda = 0.129;
    p.vev = 1.0;
    p.beta_w = BETA ? 0.1 : 0.0;
    p.beta_y = BETA ? 0.1 : 0.0;
    const PhysCoef<Op> pc = make_phys<Op>(p, 0.3, 0.2);
    g_t = Tally{};
    g_sec[0] = g_sec[1] = Tally{};
    NullSink out;
    site_rates<Op, BETA>(acc, pc, out);
    *rates = out.got;
    return g_t;
}

struct RateSink {
    double* const* r;
    int64_t c;
    void operator()(int a, double v) { r[a][c] = v; }
};

}  // namespace

extern "C" {

// counts[0..7]: add_sub, mul, div, neg, fp64 instruction estimate, stencil
// FLOPs, stencil instruction estimate, rates delivered; for the stage
// without (beta = 0) or with (beta = 1) the CP-odd terms.
int dp_count(int beta, long long* counts) {
    int rates = 0;
    const Tally t = beta ? count_rates<true>(&rates) : count_rates<false>(&rates);
    const Tally st = g_sec[1];
    counts[0] = t.add;
    counts[1] = t.mul;
    counts[2] = t.div;
    counts[3] = t.neg;
    counts[4] = t.inst;
    counts[5] = st.add + st.mul;
    counts[6] = st.inst;
    counts[7] = rates;
    return rates == 36 ? 0 : 1;
}

// All 36 rates at every site of a periodic nx x ny x nz lattice (6th-order
// stencils), y and r [36][S] (S = nx ny nz, x fastest).  cp: gw, gy, gp2,
// lambda, vev, beta_w, beta_y, dx.
int dp_rates(int nx, int ny, int nz, const double* cp, const double* y, double* r, double Jex, double gam) {
    if (nx < 7 || ny < 7 || nz < 7) return 1;
    const int64_t S = (int64_t)nx * ny * nz;
    ewpt_params p{};
    p.gw = cp[0];
    p.gy = cp[1];
    p.gp2 = cp[2];
    p.lambda = cp[3];
    p.vev = cp[4];
    p.beta_w = cp[5];
    p.beta_y = cp[6];
    const PhysCoef<double> pc = make_phys<double>(p, Jex, gam);
    const StencilCoef<double> sc = make_stencil<double>(cp[7]);
    const bool beta = p.beta_w != 0.0 || p.beta_y != 0.0;
    Ptr36 P;
    double* R[36];
    for (int a = 0; a < 36; ++a) {
        P.p[a] = y + a * S;
        R[a] = r + a * S;
    }
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                SiteAcc<double, double, SrcPtr36<double>> A{{P}};
                A.c = (int)(i + (int64_t)nx * (j + (int64_t)ny * k));
                const int idx[3] = {i, j, k}, n[3] = {nx, ny, nz}, st[3] = {1, nx, nx * ny};
                for (int ax = 0; ax < 3; ++ax) {
                    int* o = ax == 0 ? A.ox : ax == 1 ? A.oy : A.oz;
                    for (int d = 1; d <= 3; ++d) {
                        o[d - 1] = (idx[ax] + d < n[ax] ? d : d - n[ax]) * st[ax];
                        o[d + 2] = (idx[ax] - d >= 0 ? -d : n[ax] - d) * st[ax];
                    }
                }
                A.s = sc;
                RateSink out{R, A.c};
                if (beta)
                    site_rates<double, true>(A, pc, out);
                else
                    site_rates<double, false>(A, pc, out);
            }
    return 0;
}

}  // extern "C"
