// Operator definitions for the PadeOps compact line operators (see operators.h).
//
// Each def_* function states one reference operator as data: the RHS rows as linear
// forms in the input line and the LHS as a band.  The formulas follow the cited
// reference lines; X/Y/Z variants in the reference are the same 1-D formulas, so one
// definition serves every direction.  Rows are written with 1-based indices F(i) to
// read like the Fortran they state.
#include "operators.h"

#include <algorithm>
#include <cmath>

namespace pade {

LinForm operator+(const LinForm& a, const LinForm& b) {
    LinForm r = a;
    r.t.insert(r.t.end(), b.t.begin(), b.t.end());
    return r;
}
LinForm operator-(const LinForm& a) {
    LinForm r = a;
    for (auto& p : r.t) p.second = -p.second;
    return r;
}
LinForm operator-(const LinForm& a, const LinForm& b) { return a + (-b); }
LinForm operator*(double c, const LinForm& a) {
    LinForm r = a;
    for (auto& p : r.t) p.second *= c;
    return r;
}

namespace {

struct Line {
    int n;            // logical length used by reflections
    int bc1 = 0, bcn = 0;
    // 1-based direct access
    LinForm F(int i) const { return LinForm(i - 1, 1.0); }
    // periodic access with period n
    LinForm P(int i) const { return LinForm(((i - 1) % n + n) % n, 1.0); }
    // symmetric (bc=1) / antisymmetric (bc=-1) reflection about the end points: the form
    // that the bc=+-1 rows of cd10/cf90/gaussian write out term by term
    LinForm G(int i) const {
        if (i < 1) return (bc1 == -1 ? -1.0 : 1.0) * F(2 - i);
        if (i > n) return (bcn == -1 ? -1.0 : 1.0) * F(2 * n - i);
        return F(i);
    }
};

void lhs_row(OpDef& o, int i1, double m2, double m1, double d, double p1, double p2) {
    o.lhs[i1 - 1] = {m2, m1, d, p1, p2};
}

bool bc_ok(int bc) { return bc == 0 || bc == 1 || bc == -1; }

// ---- cd06 constants (cd06.F90:14-59) ----
const double alpha06d1 = 1.0 / 3.0, a06d1 = (14.0 / 9.0) / 2.0, b06d1 = (1.0 / 9.0) / 4.0;
const double alpha06d2 = 2.0 / 11.0, a06d2 = (12.0 / 11.0) / 1.0, b06d2 = (3.0 / 11.0) / 4.0;
struct Cd06B {
    double alpha = 3.0, p = 17.0 / 6.0, q = 3.0 / 2.0, r = 3.0 / 2.0, s = -1.0 / 6.0;
    double alpha_hat = alpha06d1, q_p = 3.0 / 4.0, alpha_p = 1.0 / 4.0;
    double alpha_pp, q_pp, r_pp, w1, w2, w3;
    Cd06B() {
        alpha_pp = ((40 * alpha_hat - 1) * q + 7 * (4 * alpha_hat - 1) * s) /
                   (16 * (alpha_hat + 2) * q + 8 * (1 - 4 * alpha_hat) * s);
        q_pp = (1.0 / 3.0) * (alpha_pp + 2);
        r_pp = (1.0 / 12.0) * (4 * alpha_pp - 1);
        w1 = (2 * alpha_hat + 1) / (2 * (q + s));
        w2 = ((8 * alpha_hat + 7) * q - 6 * (2 * alpha_hat + 1) * r + (8 * alpha_hat + 7) * s) / (9 * (q + s));
        w3 = (4 * (alpha_hat + 2) * q + 2 * (1 - 4 * alpha_hat) * s) / (9 * (q + s));
    }
};

// ---- cd10 constants (cd10.F90:16-104) ----
const double alpha10d1 = 1.0 / 2.0, beta10d1 = 1.0 / 20.0, a10d1 = (17.0 / 12.0) / 2.0,
             b10d1 = (101.0 / 150.0) / 4.0, c10d1 = (1.0 / 100.0) / 6.0;
const double alpha10d2 = 334.0 / 899.0, beta10d2 = 43.0 / 1798.0, a10d2 = (1065.0 / 1798.0) / 1.0,
             b10d2 = (1038.0 / 899.0) / 4.0, c10d2 = (79.0 / 1798.0) / 9.0;
struct Cd10B {
    double alpha = 3.0, p = -17.0 / 6.0, q = 3.0 / 2.0, r = 3.0 / 2.0, s = -1.0 / 6.0;
    double q_hat = a10d1, r_hat = b10d1, s_hat = c10d1, alpha_hat = alpha10d1, beta_hat = beta10d1;
    double q_p = 3.0 / 4.0, alpha_p = 1.0 / 4.0;
    double alpha_ppp, beta_ppp, q_ppp, r_ppp, s_ppp, alpha_pp, beta_pp, q_pp, r_pp, w1, w2, w3, w4;
    double b1_alpha = 11.0, b1_a, b1_b, b1_c, b1_d, b1_e, b2_alpha = 1.0 / 10.0, b2_a;
    double b3_alpha = 344.0 / 1179.0, b3_beta, b3_a, b3_b;
    Cd10B() {
        alpha_ppp = (8 * r_hat - 175 * s_hat) / (18 * r_hat - 550 * s_hat);
        beta_ppp = (1.0 / 20.0) * (-3 + 8 * alpha_ppp);
        q_ppp = (1.0 / 12.0) * (12 - 7 * alpha_ppp);
        r_ppp = (1.0 / 600.0) * (568 * alpha_ppp - 183);
        s_ppp = (1.0 / 300.0) * (9 * alpha_ppp - 4);
        double t = (q_hat + r_hat - s_hat * (q_ppp / s_ppp - 1));
        double u = s * (r_hat + 2 * s_hat) - q * (q_hat + r_hat + s_hat);
        alpha_pp = ((17 * u) / (72 * (q + s) * t) - 8.0 / 9.0) / ((19 * u) / (24 * (q + s) * t) - 1.0 / 3);
        beta_pp = (1.0 / 12.0) * (-1 + 3 * alpha_pp);
        q_pp = (2.0 / 18.0) * (8 - 3 * alpha_pp);
        r_pp = (1.0 / 72.0) * (-17 + 57 * alpha_pp);
        w1 = (q_hat + 2 * r_hat + 3 * s_hat) / (q + s);
        w2 = (1 / q_p) * (r_hat + s_hat * (1 + q_ppp / s_ppp) - r * (q_hat + 2 * r_hat + 3 * s_hat) / (q + s));
        w3 = (q_hat + r_hat + s_hat * (1 - q_ppp / s_ppp)) / (r_pp);
        w4 = s_hat / s_ppp;
        b1_a = (11 * b1_alpha + 35) / 12;
        b1_b = -(5 * b1_alpha + 26) / 3;
        b1_c = (b1_alpha + 19) / 2;
        b1_d = (b1_alpha - 14) / 3;
        b1_e = (11 - b1_alpha) / 12;
        b2_a = (4 * (1 - b2_alpha) / 3) / 1.0;
        b3_beta = (38.0 * b3_alpha - 9.0) / 214.0;
        b3_a = ((696 - 1191 * b3_alpha) / 428) / 1.0;
        b3_b = ((2454 * b3_alpha - 294) / 535) / 4.0;
    }
};

// ---- cf90 / gaussian constants (cf90.F90:16-48, gaussian.F90:16-43) ----
const double alpha90 = 6.6624e-1, beta90 = 1.6688e-1, a90 = 9.9965e-1, b90 = 6.6652e-1, c90 = 1.6674e-1,
             d90 = 4.0e-5, e90 = -5.0e-6;
const double b2_alpha90 = 4.997e-1, b2_a90 = 9.997e-1, b2_b90 = 4.9985e-1;
const double b3_alpha90 = 6.6624e-1, b3_beta90 = 1.6688e-1, b3_a90 = 9.9952e-1, b3_b90 = 6.6656e-1,
             b3_c90 = 1.668e-1;
const double b4_alpha90 = 6.6624e-1, b4_beta90 = 1.6688e-1, b4_a90 = 9.9968e-1, b4_b90 = 6.6652e-1,
             b4_c90 = 1.6672e-1, b4_d90 = 4.0e-5;
const double agf = 3565.0 / 10368.0, bgf = 3091.0 / 12960.0, cgf = 1997.0 / 25920.0, dgf = 149.0 / 12960.0,
             egf = 107.0 / 103680.0;
const double b1_agf = 5.0 / 6.0, b1_bgf = 1.0 / 6.0, b2_agf = 2.0 / 3.0, b2_bgf = 1.0 / 6.0;
const double b3_agf = 31.0 / 64.0, b3_bgf = 7.0 / 32.0, b3_cgf = 5.0 / 128.0;
const double b4_agf = 17.0 / 48.0, b4_bgf = 15.0 / 64.0, b4_cgf = 7.0 / 96.0, b4_dgf = 1.0 / 64.0;

void init_square(OpDef& o, int n, int q, bool cyclic) {
    o.m = o.nout = o.ns = n;
    o.q = q;
    o.cyclic = cyclic;
    o.rhs.assign(n, LinForm());
    o.lhs.assign(n, {0, 0, 1, 0, 0});
}

void zero_op(OpDef& o, int n, bool identity) {
    o = OpDef();
    o.m = o.nout = o.ns = n;
    if (identity) o.identity = true;
    else o.zero = true;
}

// symmetric 9-point filter row a f(i) + sum_k c_k (f(i+k) + f(i-k)) with the access rule acc
template <class Acc>
LinForm sym9(const Acc& G, int i, double a, double b, double c, double d, double e) {
    return a * G(i) + b * (G(i + 1) + G(i - 1)) + c * (G(i + 2) + G(i - 2)) + d * (G(i + 3) + G(i - 3)) +
           e * (G(i + 4) + G(i - 4));
}

}  // namespace

// cd06 (cd06.F90:129-201 init, 264-327 ComputeTri1, 515-592 D1 RHS, 745-773 D2 RHS)
int def_cd06(int n, double dx, bool periodic, int bc1, int bcn, int order, OpDef& o) {
    if (periodic) {
        if (n == 1) return zero_op(o, n, false), PS_OK;
        if (n < 6) return PS_EREF_PERIODIC_N;
    } else {
        if (n == 1) return zero_op(o, n, false), PS_OK;
        if (n < 8) return PS_EREF_NONPERIODIC_N;
        // the reference's non-periodic second derivative is incomplete (cd06.F90:330-343, 492-513)
        if (order == 2) return PS_ENOTSUP;
    }
    o = OpDef();
    init_square(o, n, 1, periodic);
    Line L{n, bc1, bcn};
    const double obdx = 1.0 / dx;
    if (order == 2) {
        // periodic D2 (cd06.F90:745-773), completed with the 1/dx^2 factor and the LU2 solve
        const double a = a06d2 * obdx * obdx, b = b06d2 * obdx * obdx;
        for (int i = 1; i <= n; i++) {
            o.rhs[i - 1] = a * (L.P(i + 1) - 2.0 * L.P(i) + L.P(i - 1)) + b * (L.P(i + 2) - 2.0 * L.P(i) + L.P(i - 2));
            lhs_row(o, i, 0, alpha06d2, 1.0, alpha06d2, 0);
        }
        o.io = {-2, -1, 0, 1, 2};
        o.ic = {b, a, -2.0 * a - 2.0 * b, a, b};
        return PS_OK;
    }
    const double a06 = a06d1 * obdx, b06 = b06d1 * obdx;
    o.io = {-2, -1, 1, 2};
    o.ic = {-b06, -a06, a06, b06};
    if (periodic) {
        for (int i = 1; i <= n; i++) {
            o.rhs[i - 1] = a06 * (L.P(i + 1) - L.P(i - 1)) + b06 * (L.P(i + 2) - L.P(i - 2));
            lhs_row(o, i, 0, alpha06d1, 1.0, alpha06d1, 0);
        }
        return PS_OK;
    }
    Cd06B k;
    const double a_np_3 = k.w3 * k.q_pp * obdx, b_np_3 = k.w3 * k.r_pp * obdx, a_np_2 = k.w2 * k.q_p * obdx;
    const double a_np_1 = k.w1 * (-k.p * obdx), b_np_1 = k.w1 * (k.q * obdx), c_np_1 = k.w1 * (k.r * obdx),
                 d_np_1 = k.w1 * (k.s * obdx);
    for (int i = 1; i <= n; i++) lhs_row(o, i, 0, k.alpha_hat, 1.0, k.alpha_hat, 0);
    o.rhs[0] = a_np_1 * L.F(1) + b_np_1 * L.F(2) + c_np_1 * L.F(3) + d_np_1 * L.F(4);
    o.rhs[1] = a_np_2 * (L.F(3) - L.F(1));
    o.rhs[2] = a_np_3 * (L.F(4) - L.F(2)) + b_np_3 * (L.F(5) - L.F(1));
    for (int i = 4; i <= n - 3; i++) o.rhs[i - 1] = b06 * (L.F(i + 2) - L.F(i - 2)) + a06 * (L.F(i + 1) - L.F(i - 1));
    o.rhs[n - 3] = a_np_3 * (L.F(n - 1) - L.F(n - 3)) + b_np_3 * (L.F(n) - L.F(n - 4));
    o.rhs[n - 2] = a_np_2 * (L.F(n) - L.F(n - 2));
    o.rhs[n - 1] = -a_np_1 * L.F(n) - b_np_1 * L.F(n - 1) - c_np_1 * L.F(n - 2) - d_np_1 * L.F(n - 3);
    // ComputeTri1: only bc == 0 modifies the matrix (bc == 1 is "Incomplete" upstream)
    if (bc1 == 0) {
        lhs_row(o, 1, 0, k.w1 * 0.0, k.w1 * 1.0, k.w1 * k.alpha, 0);
        lhs_row(o, 2, 0, k.w2 * k.alpha_p, k.w2 * 1.0, k.w2 * k.alpha_p, 0);
        lhs_row(o, 3, 0, k.w3 * k.alpha_pp, k.w3 * 1.0, k.w3 * k.alpha_pp, 0);
    }
    if (bcn == 0) {
        lhs_row(o, n, 0, k.w1 * k.alpha, k.w1 * 1.0, k.w1 * 0.0, 0);
        lhs_row(o, n - 1, 0, k.w2 * k.alpha_p, k.w2 * 1.0, k.w2 * k.alpha_p, 0);
        lhs_row(o, n - 2, 0, k.w3 * k.alpha_pp, k.w3 * 1.0, k.w3 * k.alpha_pp, 0);
    }
    // the tridiagonal Thomas sweep never reads the sub-diagonal of row 1 or the
    // super-diagonal of row n (cd06.F90:441-448)
    o.lhs[0][1] = 0.0;
    o.lhs[n - 1][3] = 0.0;
    return PS_OK;
}

// cd10 (cd10.F90:195-315 init, 429-709 ComputePenta1/2, 1098-1263 D1 RHS, 1587-1736 D2 RHS)
int def_cd10(int n, double dx, bool periodic, int bc1, int bcn, int order, OpDef& o) {
    if (!bc_ok(bc1) || !bc_ok(bcn)) return PS_EREF_BC;
    if (n == 1) return zero_op(o, n, false), PS_OK;
    if (n < 8) return PS_EREF_NONPERIODIC_N;
    o = OpDef();
    init_square(o, n, 2, periodic);
    Line L{n, bc1, bcn};
    Cd10B k;
    const double obdx = 1.0 / dx, obdx2 = obdx / dx;
    if (order == 1) {
        const double a10 = a10d1 * obdx, b10 = b10d1 * obdx, c10 = c10d1 * obdx;
        o.io = {-3, -2, -1, 1, 2, 3};
        o.ic = {-c10, -b10, -a10, a10, b10, c10};
        if (periodic) {
            for (int i = 1; i <= n; i++) {
                o.rhs[i - 1] = a10 * (L.P(i + 1) - L.P(i - 1)) + b10 * (L.P(i + 2) - L.P(i - 2)) +
                               c10 * (L.P(i + 3) - L.P(i - 3));
                lhs_row(o, i, beta10d1, alpha10d1, 1.0, alpha10d1, beta10d1);
            }
            return PS_OK;
        }
        const double a_np_4 = k.w4 * k.q_ppp * obdx, b_np_4 = k.w4 * k.r_ppp * obdx, c_np_4 = k.w4 * k.s_ppp * obdx;
        const double a_np_3 = k.w3 * k.q_pp * obdx, b_np_3 = k.w3 * k.r_pp * obdx, a_np_2 = k.w2 * k.q_p * obdx;
        const double a_np_1 = k.w1 * (k.p * obdx), b_np_1 = k.w1 * (k.q * obdx), c_np_1 = k.w1 * (k.r * obdx),
                     d_np_1 = k.w1 * (k.s * obdx);
        auto row = [&](int i) {
            return a10 * (L.G(i + 1) - L.G(i - 1)) + b10 * (L.G(i + 2) - L.G(i - 2)) + c10 * (L.G(i + 3) - L.G(i - 3));
        };
        for (int i = 1; i <= n; i++) {
            o.rhs[i - 1] = row(i);
            lhs_row(o, i, k.beta_hat, k.alpha_hat, 1.0, k.alpha_hat, k.beta_hat);
        }
        if (bc1 == 0) {
            o.rhs[0] = a_np_1 * L.F(1) + b_np_1 * L.F(2) + c_np_1 * L.F(3) + d_np_1 * L.F(4);
            o.rhs[1] = a_np_2 * (L.F(3) - L.F(1));
            o.rhs[2] = a_np_3 * (L.F(4) - L.F(2)) + b_np_3 * (L.F(5) - L.F(1));
            o.rhs[3] = a_np_4 * (L.F(5) - L.F(3)) + b_np_4 * (L.F(6) - L.F(2)) + c_np_4 * (L.F(7) - L.F(1));
            lhs_row(o, 1, k.w1 * 0.0, k.w1 * 0.0, k.w1 * 1.0, k.w1 * k.alpha, k.w1 * 0.0);
            lhs_row(o, 2, k.w2 * 0.0, k.w2 * k.alpha_p, k.w2 * 1.0, k.w2 * k.alpha_p, k.w2 * 0.0);
            lhs_row(o, 3, k.w3 * k.beta_pp, k.w3 * k.alpha_pp, k.w3 * 1.0, k.w3 * k.alpha_pp, k.w3 * k.beta_pp);
            lhs_row(o, 4, k.w4 * k.beta_ppp, k.w4 * k.alpha_ppp, k.w4 * 1.0, k.w4 * k.alpha_ppp, k.w4 * k.beta_ppp);
        } else if (bc1 == 1) {
            o.rhs[0] = LinForm();
            lhs_row(o, 1, 0.0, 0.0, 1.0, 0.0, 0.0);
            lhs_row(o, 2, 0.0, k.alpha_hat, 1.0 - k.beta_hat, k.alpha_hat, k.beta_hat);
        } else {
            lhs_row(o, 1, 0.0, 0.0, 1.0, 2.0 * k.alpha_hat, 2.0 * k.beta_hat);
            lhs_row(o, 2, 0.0, k.alpha_hat, 1.0 + k.beta_hat, k.alpha_hat, k.beta_hat);
        }
        if (bcn == 0) {
            o.rhs[n - 4] = a_np_4 * (L.F(n - 2) - L.F(n - 4)) + b_np_4 * (L.F(n - 1) - L.F(n - 5)) +
                           c_np_4 * (L.F(n) - L.F(n - 6));
            o.rhs[n - 3] = a_np_3 * (L.F(n - 1) - L.F(n - 3)) + b_np_3 * (L.F(n) - L.F(n - 4));
            o.rhs[n - 2] = a_np_2 * (L.F(n) - L.F(n - 2));
            o.rhs[n - 1] = -a_np_1 * L.F(n) - b_np_1 * L.F(n - 1) - c_np_1 * L.F(n - 2) - d_np_1 * L.F(n - 3);
            lhs_row(o, n, k.w1 * 0.0, k.w1 * k.alpha, k.w1 * 1.0, k.w1 * 0.0, k.w1 * 0.0);
            lhs_row(o, n - 1, k.w2 * 0.0, k.w2 * k.alpha_p, k.w2 * 1.0, k.w2 * k.alpha_p, k.w2 * 0.0);
            lhs_row(o, n - 2, k.w3 * k.beta_pp, k.w3 * k.alpha_pp, k.w3 * 1.0, k.w3 * k.alpha_pp, k.w3 * k.beta_pp);
            lhs_row(o, n - 3, k.w4 * k.beta_ppp, k.w4 * k.alpha_ppp, k.w4 * 1.0, k.w4 * k.alpha_ppp, k.w4 * k.beta_ppp);
        } else if (bcn == 1) {
            o.rhs[n - 1] = LinForm();
            lhs_row(o, n, 0.0, 0.0, 1.0, 0.0, 0.0);
            lhs_row(o, n - 1, k.beta_hat, k.alpha_hat, 1.0 - k.beta_hat, k.alpha_hat, 0.0);
        } else {
            lhs_row(o, n, 2.0 * k.beta_hat, 2.0 * k.alpha_hat, 1.0, 0.0, 0.0);
            lhs_row(o, n - 1, k.beta_hat, k.alpha_hat, 1.0 + k.beta_hat, k.alpha_hat, 0.0);
        }
    } else {
        const double a10 = a10d2 * obdx2, b10 = b10d2 * obdx2, c10 = c10d2 * obdx2;
        o.io = {-3, -2, -1, 0, 1, 2, 3};
        o.ic = {c10, b10, a10, -2.0 * a10 - 2.0 * b10 - 2.0 * c10, a10, b10, c10};
        auto rowP = [&](int i) {
            return a10 * (L.P(i + 1) - 2.0 * L.P(i) + L.P(i - 1)) + b10 * (L.P(i + 2) - 2.0 * L.P(i) + L.P(i - 2)) +
                   c10 * (L.P(i + 3) - 2.0 * L.P(i) + L.P(i - 3));
        };
        auto rowG = [&](int i) {
            return a10 * (L.G(i + 1) - 2.0 * L.G(i) + L.G(i - 1)) + b10 * (L.G(i + 2) - 2.0 * L.G(i) + L.G(i - 2)) +
                   c10 * (L.G(i + 3) - 2.0 * L.G(i) + L.G(i - 3));
        };
        if (periodic) {
            for (int i = 1; i <= n; i++) {
                o.rhs[i - 1] = rowP(i);
                lhs_row(o, i, beta10d2, alpha10d2, 1.0, alpha10d2, beta10d2);
            }
            return PS_OK;
        }
        const double a_np_3 = k.b3_a * obdx2, b_np_3 = k.b3_b * obdx2, a_np_2 = k.b2_a * obdx2;
        const double a_np_1 = k.b1_a * obdx2, b_np_1 = k.b1_b * obdx2, c_np_1 = k.b1_c * obdx2,
                     d_np_1 = k.b1_d * obdx2, e_np_1 = k.b1_e * obdx2;
        for (int i = 1; i <= n; i++) {
            o.rhs[i - 1] = rowG(i);
            lhs_row(o, i, beta10d2, alpha10d2, 1.0, alpha10d2, beta10d2);
        }
        if (bc1 == 0) {
            o.rhs[0] = a_np_1 * L.F(1) + b_np_1 * L.F(2) + c_np_1 * L.F(3) + d_np_1 * L.F(4) + e_np_1 * L.F(5);
            o.rhs[1] = a_np_2 * (L.F(3) - 2.0 * L.F(2) + L.F(1));
            o.rhs[2] = a_np_3 * (L.F(4) - 2.0 * L.F(3) + L.F(2)) + b_np_3 * (L.F(5) - 2.0 * L.F(3) + L.F(1));
            lhs_row(o, 1, 0.0, 0.0, 1.0, k.b1_alpha, 0.0);
            lhs_row(o, 2, 0.0, k.b2_alpha, 1.0, k.b2_alpha, 0.0);
            lhs_row(o, 3, k.b3_beta, k.b3_alpha, 1.0, k.b3_alpha, k.b3_beta);
        } else if (bc1 == 1) {
            lhs_row(o, 1, 0.0, 0.0, 1.0, 2.0 * alpha10d2, 2.0 * beta10d2);
            lhs_row(o, 2, 0.0, alpha10d2, 1.0 + beta10d2, alpha10d2, beta10d2);
        } else {
            lhs_row(o, 1, 0.0, 0.0, 1.0, 0.0, 0.0);
            lhs_row(o, 2, 0.0, alpha10d2, 1.0 - beta10d2, alpha10d2, beta10d2);
        }
        if (bcn == 0) {
            o.rhs[n - 3] = a_np_3 * (L.F(n - 1) - 2.0 * L.F(n - 2) + L.F(n - 3)) +
                           b_np_3 * (L.F(n) - 2.0 * L.F(n - 2) + L.F(n - 4));
            o.rhs[n - 2] = a_np_2 * (L.F(n) - 2.0 * L.F(n - 1) + L.F(n - 2));
            o.rhs[n - 1] = a_np_1 * L.F(n) + b_np_1 * L.F(n - 1) + c_np_1 * L.F(n - 2) + d_np_1 * L.F(n - 3) +
                           e_np_1 * L.F(n - 4);
            lhs_row(o, n - 2, k.b3_beta, k.b3_alpha, 1.0, k.b3_alpha, k.b3_beta);
            lhs_row(o, n - 1, 0.0, k.b2_alpha, 1.0, k.b2_alpha, 0.0);
            lhs_row(o, n, 0.0, k.b1_alpha, 1.0, 0.0, 0.0);
        } else if (bcn == 1) {
            lhs_row(o, n - 1, beta10d2, alpha10d2, 1.0 + beta10d2, alpha10d2, 0.0);
            lhs_row(o, n, 2.0 * beta10d2, 2.0 * alpha10d2, 1.0, 0.0, 0.0);
        } else {
            lhs_row(o, n - 1, beta10d2, alpha10d2, 1.0 - beta10d2, alpha10d2, 0.0);
            lhs_row(o, n, 0.0, 0.0, 1.0, 0.0, 0.0);
        }
    }
    // entries that fall outside the matrix are never read by the pentadiagonal sweep
    o.lhs[0][0] = o.lhs[0][1] = o.lhs[1][0] = 0.0;
    o.lhs[n - 1][3] = o.lhs[n - 1][4] = o.lhs[n - 2][4] = 0.0;
    return PS_OK;
}

namespace {
// shared row layout of cf90 and gaussian (cf90.F90:610-994, gaussian.F90:137-330)
void sym_filter_rhs(OpDef& o, int n, bool periodic, int bc1, int bcn, const double* c, const double* r1,
                    const double* r2, const double* r3, const double* r4) {
    Line L{n, bc1, bcn};
    auto Pa = [&](int i) { return L.P(i); };
    auto Ga = [&](int i) { return L.G(i); };
    auto Fa = [&](int i) { return L.F(i); };
    o.io = {-4, -3, -2, -1, 0, 1, 2, 3, 4};
    o.ic = {c[4], c[3], c[2], c[1], c[0], c[1], c[2], c[3], c[4]};
    for (int i = 1; i <= n; i++) o.rhs[i - 1] = periodic ? sym9(Pa, i, c[0], c[1], c[2], c[3], c[4])
                                                         : sym9(Ga, i, c[0], c[1], c[2], c[3], c[4]);
    if (periodic) return;
    if (bc1 == 0) {
        o.rhs[0] = r1[0] * Fa(1) + r1[1] * Fa(2);
        o.rhs[1] = r2[0] * Fa(2) + r2[1] * (Fa(3) + Fa(1));
        o.rhs[2] = r3[0] * Fa(3) + r3[1] * (Fa(4) + Fa(2)) + r3[2] * (Fa(5) + Fa(1));
        o.rhs[3] = r4[0] * Fa(4) + r4[1] * (Fa(5) + Fa(3)) + r4[2] * (Fa(6) + Fa(2)) + r4[3] * (Fa(7) + Fa(1));
    }
    if (bcn == 0) {
        o.rhs[n - 4] = r4[0] * Fa(n - 3) + r4[1] * (Fa(n - 2) + Fa(n - 4)) + r4[2] * (Fa(n - 1) + Fa(n - 5)) +
                       r4[3] * (Fa(n) + Fa(n - 6));
        o.rhs[n - 3] = r3[0] * Fa(n - 2) + r3[1] * (Fa(n - 1) + Fa(n - 3)) + r3[2] * (Fa(n) + Fa(n - 4));
        o.rhs[n - 2] = r2[0] * Fa(n - 1) + r2[1] * (Fa(n) + Fa(n - 2));
        o.rhs[n - 1] = r1[0] * Fa(n) + r1[1] * Fa(n - 1);
    }
}
}  // namespace

// cf90 (cf90.F90:107-175 init, 276-418 ComputePenta, 610-994 RHS)
int def_cf90(int n, bool periodic, int bc1, int bcn, OpDef& o) {
    if (!bc_ok(bc1) || !bc_ok(bcn)) return PS_EREF_BC;
    if (n == 1) return zero_op(o, n, true), PS_OK;
    if (n < 10) return PS_EREF_FILTER_N;
    o = OpDef();
    init_square(o, n, 2, periodic);
    const double c[5] = {a90, b90, c90, d90, e90};
    const double r1[2] = {1.0, 0.0}, r2[2] = {b2_a90, b2_b90}, r3[3] = {b3_a90, b3_b90, b3_c90},
                 r4[4] = {b4_a90, b4_b90, b4_c90, b4_d90};
    sym_filter_rhs(o, n, periodic, bc1, bcn, c, r1, r2, r3, r4);
    for (int i = 1; i <= n; i++) lhs_row(o, i, beta90, alpha90, 1.0, alpha90, beta90);
    if (!periodic) {
        if (bc1 == 0) {
            lhs_row(o, 1, 0.0, 0.0, 1.0, 0.0, 0.0);
            lhs_row(o, 2, 0.0, b2_alpha90, 1.0, b2_alpha90, 0.0);
            lhs_row(o, 3, b3_beta90, b3_alpha90, 1.0, b3_alpha90, b3_beta90);
            lhs_row(o, 4, b4_beta90, b4_alpha90, 1.0, b4_alpha90, b4_beta90);
        } else if (bc1 == 1) {
            lhs_row(o, 1, 0.0, 0.0, 1.0, 2.0 * alpha90, 2.0 * beta90);
            lhs_row(o, 2, 0.0, alpha90, 1.0 + beta90, alpha90, beta90);
        } else {
            lhs_row(o, 1, 0.0, 0.0, 1.0, 0.0, 0.0);
            lhs_row(o, 2, 0.0, alpha90, 1.0 - beta90, alpha90, beta90);
        }
        if (bcn == 0) {
            lhs_row(o, n, 0.0, 0.0, 1.0, 0.0, 0.0);
            lhs_row(o, n - 1, 0.0, b2_alpha90, 1.0, b2_alpha90, 0.0);
            lhs_row(o, n - 2, b3_beta90, b3_alpha90, 1.0, b3_alpha90, b3_beta90);
            lhs_row(o, n - 3, b4_beta90, b4_alpha90, 1.0, b4_alpha90, b4_beta90);
        } else if (bcn == 1) {
            lhs_row(o, n, 2.0 * beta90, 2.0 * alpha90, 1.0, 0.0, 0.0);
            lhs_row(o, n - 1, beta90, alpha90, 1.0 + beta90, alpha90, 0.0);
        } else {
            lhs_row(o, n, 0.0, 0.0, 1.0, 0.0, 0.0);
            lhs_row(o, n - 1, beta90, alpha90, 1.0 - beta90, alpha90, 0.0);
        }
        o.lhs[0][0] = o.lhs[0][1] = o.lhs[1][0] = 0.0;
        o.lhs[n - 1][3] = o.lhs[n - 1][4] = o.lhs[n - 2][4] = 0.0;
    }
    o.resid = true;
    return PS_OK;
}

// gaussian (gaussian.F90:74-334): explicit, no LHS
int def_gaussian(int n, bool periodic, int bc1, int bcn, OpDef& o) {
    if (!bc_ok(bc1) || !bc_ok(bcn)) return PS_EREF_BC;
    if (n == 1) return zero_op(o, n, true), PS_OK;
    // the reference filter rows address f(i-4..i+4), so n < 9 would read outside the line
    if (n < 9) return PS_EINVAL;
    o = OpDef();
    init_square(o, n, 0, false);
    const double c[5] = {agf, bgf, cgf, dgf, egf};
    const double r1[2] = {b1_agf, b1_bgf}, r2[2] = {b2_agf, b2_bgf}, r3[3] = {b3_agf, b3_bgf, b3_cgf},
                 r4[4] = {b4_agf, b4_bgf, b4_cgf, b4_dgf};
    sym_filter_rhs(o, n, periodic, bc1, bcn, c, r1, r2, r3, r4);
    o.cyclic = periodic;  // periodic wrap of the explicit stencil (q = 0: nothing to solve)
    return PS_OK;
}

// cd06stagg (cd06stagg.F90:170-232 init, 301-629 periodic RHS, STAGG_CD06_files/*)
int def_stagg(const StaggCfg& c, int op, OpDef& o) {
    if (op < 0 || op >= STAGG_NOPS) return PS_EINVAL;
    const int n = c.n, nE = n + 1;
    if (n <= 4) return PS_EREF_STAGG_N;
    const bool inE = (op == D1_E2C || op == D1_E2E || op == D2_E2E || op == I_E2C);
    const bool outE = (op == D1_C2E || op == D1_E2E || op == D2_E2E || op == I_C2E);
    o = OpDef();
    o.m = inE ? nE : n;
    o.nout = outE ? nE : n;
    o.q = 1;
    o.cyclic = c.periodic;
    o.ns = c.periodic ? n : o.nout;
    o.rhs.assign(o.ns, LinForm());
    o.lhs.assign(o.ns, {0, 0, 1, 0, 0});
    Line L{n};
    const double dxi = 1.0 / c.dx, dxi2 = dxi / c.dx;
    auto F = [&](int i) { return L.F(i); };
    auto P = [&](int i) { return L.P(i); };
    auto R = [&](int i) -> LinForm& { return o.rhs[i - 1]; };
    const double w0s = 223.0 / 186.0, w1s = 61.0 / 62.0;
    double alpha;
    switch (op) {
    case D1_E2C: case D1_C2E: alpha = 9.0 / 62.0; break;
    case D1_C2C: case D1_E2E: alpha = 1.0 / 3.0; break;
    case D2_C2C: case D2_E2E: alpha = 2.0 / 11.0; break;
    default: alpha = 3.0 / 10.0; break;
    }
    if (c.periodic) {
        for (int i = 1; i <= n; i++) lhs_row(o, i, 0, alpha, 1.0, alpha, 0);
        if (op == D1_E2C || op == I_E2C) {  // 301-322, 526-547: the (n+1)-th edge is read as given
            double a06, b06, s;
            if (op == D1_E2C) { a06 = (63.0 / 62.0) * dxi; b06 = ((17.0 / 62.0) / 3.0) * dxi; s = -1; }
            else { a06 = (3.0 / 2.0) * (1.0 / 2.0); b06 = (1.0 / 10.0) * (1.0 / 2.0); s = 1; }
            R(1) = a06 * (F(2) + s * F(1)) + b06 * (F(3) + s * F(n));
            for (int i = 2; i <= n - 1; i++) R(i) = a06 * (F(i + 1) + s * F(i)) + b06 * (F(i + 2) + s * F(i - 1));
            R(n) = a06 * (F(n + 1) + s * F(n)) + b06 * (F(2) + s * F(n - 1));
            o.io = {-1, 0, 1, 2};
            o.ic = {s * b06, s * a06, a06, b06};
        } else if (op == D1_C2E || op == I_C2E) {  // 349-375, 573-600; row n+1 is a copy of row 1
            double a06, b06, s;
            if (op == D1_C2E) { a06 = (63.0 / 62.0) * dxi; b06 = ((17.0 / 62.0) / 3.0) * dxi; s = -1; }
            else { a06 = (3.0 / 2.0) * (1.0 / 2.0); b06 = (1.0 / 10.0) * (1.0 / 2.0); s = 1; }
            for (int i = 1; i <= n; i++) R(i) = a06 * (P(i) + s * P(i - 1)) + b06 * (P(i + 1) + s * P(i - 2));
            o.io = {-2, -1, 0, 1};
            o.ic = {s * b06, s * a06, a06, b06};
        } else if (op == D2_C2C || op == D2_E2E) {  // 405-432, 465-495: rows 1..n use the cell period
            const double a06 = (12.0 / 11.0) * (dxi * dxi), b06 = ((3.0 / 11.0) / 4.0) * (dxi * dxi);
            for (int i = 1; i <= n; i++)
                R(i) = a06 * (P(i + 1) - 2.0 * P(i) + P(i - 1)) + b06 * (P(i + 2) - 2.0 * P(i) + P(i - 2));
            o.io = {-2, -1, 0, 1, 2};
            o.ic = {b06, a06, -2.0 * a06 - 2.0 * b06, a06, b06};
        } else {
            return PS_ENOTSUP;  // C2C/E2E first derivatives have no periodic form upstream (cd06stagg.F90:883-925)
        }
        return PS_OK;
    }
    // ---------------- non-periodic ----------------
    const int no = o.nout;
    for (int i = 1; i <= no; i++) lhs_row(o, i, 0, alpha, 1.0, alpha, 0);
    auto lrow = [&](int i, double dn, double dg, double up) { o.lhs[i - 1][1] = dn; o.lhs[i - 1][2] = dg; o.lhs[i - 1][3] = up; };
    auto& lh = o.lhs;
    if (op == D1_E2C) {  // D1RHS_E2C_common.F90, ComputeTri_allRoutines.F90:1-47
        const double a = (63.0 / 62.0) / 1.0, b = (17.0 / 62.0) / 3.0, alpha1 = 37.0 / 183.0, alpha0 = -1.0;
        const double a0 = (1.0 / 24.0) * (alpha0 - 23.0), b0 = (1.0 / 8.0) * (-9.0 * alpha0 + 7.0);
        const double c0 = (1.0 / 8.0) * (9.0 * alpha0 + 1.0), d0 = -(1.0 / 24.0) * (alpha0 + 1.0);
        const double a1 = (3.0 / 8.0) * (3.0 - 2.0 * alpha1), b1 = (1.0 / 8.0) * (-1.0 + 22.0 * alpha1);
        const double a06 = a * dxi, b06 = b * dxi;
        for (int i = 2; i <= n - 1; i++) R(i) = b06 * (F(i + 2) - F(i - 1)) + a06 * (F(i + 1) - F(i));
        if (c.botSided) {
            R(1) = (w0s * dxi) * (a0 * F(1) + b0 * F(2) + c0 * F(3) + d0 * F(4));
            R(2) = (w1s * dxi) * ((-b1 / 3.0) * F(1) + (-a1) * F(2) + (a1)*F(3) + (b1 / 3.0) * F(4));
        } else if (c.botEven) R(1) = b06 * (F(3) - F(2)) + a06 * (F(2) - F(1));
        else R(1) = b06 * (F(3) + F(2)) + a06 * (F(2) - F(1));
        if (c.topSided) {
            R(n) = (-w0s * dxi) * (a0 * F(nE) + b0 * F(nE - 1) + c0 * F(nE - 2) + d0 * F(nE - 3));
            R(n - 1) = (w1s * dxi) * ((-b1 / 3.0) * F(nE - 3) + (-a1) * F(nE - 2) + (a1)*F(nE - 1) + (b1 / 3.0) * F(nE));
        } else if (c.topEven) R(n) = b06 * (F(nE - 1) - F(nE - 2)) + a06 * (F(nE) - F(nE - 1));
        else R(n) = -b06 * (F(nE - 1) + F(nE - 2)) + a06 * (F(nE) - F(nE - 1));
        o.io = {-1, 0, 1, 2};
        o.ic = {-b06, -a06, a06, b06};
        if (c.topSided) { lh[n - 1][1] = w0s * alpha0; lh[n - 1][2] = w0s; lrow(n - 1, w1s * alpha1, w1s, w1s * alpha1); }
        else if (c.topEven) { lh[n - 1][3] = 0.0; lh[n - 1][2] = 1.0 - alpha; }
        else { lh[n - 1][2] = 1.0 + alpha; lh[n - 1][3] = 0.0; }
        if (c.botSided) { lh[0][3] = w0s * alpha0; lh[0][2] = w0s; lrow(2, w1s * alpha1, w1s, w1s * alpha1); }
        else if (c.botEven) { lh[0][1] = 0.0; lh[0][2] = 1.0 - alpha; }
        else { lh[0][1] = 0.0; lh[0][2] = 1.0 + alpha; }
    } else if (op == D1_C2E) {  // D1RHS_C2E_common.F90, ComputeTri_allRoutines.F90:49-94
        const double a = (63.0 / 62.0) / 1.0, b = (17.0 / 62.0) / 3.0;
        const double a0 = -71.0 / 24.0, b0 = 47.0 / 8.0, c0 = -31.0 / 8.0, d0 = 23.0 / 24.0, a1 = 12.0 / 11.0;
        const double a06 = a * dxi, b06 = b * dxi;
        for (int i = 2; i <= nE - 1; i++) R(i) = a06 * (F(i) - F(i - 1));
        for (int i = 3; i <= nE - 2; i++) R(i) = R(i) + b06 * (F(i + 1) - F(i - 2));
        if (c.botSided) {
            R(1) = dxi * (a0 * F(1) + b0 * F(2) + c0 * F(3) + d0 * F(4));
            R(2) = (a1 * dxi) * (F(2) - F(1));
        } else if (c.botEven) { R(1) = LinForm(); R(2) = R(2) + b06 * (F(3) - F(1)); }
        else { R(1) = 2.0 * b06 * F(2) + 2.0 * a06 * F(1); R(2) = R(2) + b06 * (F(3) + F(1)); }
        if (c.topSided) {
            R(nE - 1) = (a1 * dxi) * (F(n) - F(n - 1));
            R(nE) = (-dxi) * (a0 * F(n) + b0 * F(n - 1) + c0 * F(n - 2) + d0 * F(n - 3));
        } else if (c.topEven) { R(nE - 1) = R(nE - 1) + b06 * (F(n) - F(n - 2)); R(nE) = LinForm(); }
        else { R(nE - 1) = R(nE - 1) - b06 * (F(n) + F(n - 2)); R(nE) = -2.0 * b06 * F(n - 1) - 2.0 * a06 * F(n); }
        o.io = {-2, -1, 0, 1};
        o.ic = {-b06, -a06, a06, b06};
        if (c.topSided) { lh[nE - 1][1] = 0.0; lh[nE - 1][3] = 0.0; lrow(nE - 1, 1.0 / 22.0, 1.0, 1.0 / 22.0); }
        else if (c.topEven) { lh[nE - 1][3] = 0.0; lh[nE - 1][1] = 0.0; }
        else { lh[nE - 1][1] = 2.0 * alpha; lh[nE - 1][3] = 0.0; }
        if (c.botSided) { lh[0][3] = 0.0; lh[0][1] = 0.0; lrow(2, 1.0 / 22.0, 1.0, 1.0 / 22.0); }
        else if (c.botEven) { lh[0][1] = 0.0; lh[0][3] = 0.0; }
        else { lh[0][1] = 0.0; lh[0][3] = 2.0 * alpha; }
    } else if (op == D1_C2C) {  // D1RHS_C2C_common.F90, ComputeTri_allRoutines.F90:96-160
        Cd06B k;
        const double a06 = ((14.0 / 9.0) / 2.0) * dxi, b06 = ((1.0 / 9.0) / 4.0) * dxi;
        const double a_np_3 = k.w3 * k.q_pp * dxi, b_np_3 = k.w3 * k.r_pp * dxi, a_np_2 = k.w2 * k.q_p * dxi;
        const double a_np_1 = k.w1 * (-k.p * dxi), b_np_1 = k.w1 * (k.q * dxi), c_np_1 = k.w1 * (k.r * dxi),
                     d_np_1 = k.w1 * (k.s * dxi);
        if (c.botSided) {
            R(1) = a_np_1 * F(1) + b_np_1 * F(2) + c_np_1 * F(3) + d_np_1 * F(4);
            R(2) = a_np_2 * (F(3) - F(1));
            R(3) = a_np_3 * (F(4) - F(2)) + b_np_3 * (F(5) - F(1));
        } else if (c.botEven) {
            R(1) = b06 * (F(3) - F(2)) + a06 * (F(2) - F(1));
            R(2) = b06 * (F(4) - F(1)) + a06 * (F(3) - F(1));
            R(3) = b06 * (F(5) - F(1)) + a06 * (F(4) - F(2));
        } else {
            R(1) = b06 * (F(3) + F(2)) + a06 * (F(2) + F(1));
            R(2) = b06 * (F(4) + F(1)) + a06 * (F(3) - F(1));
            R(3) = b06 * (F(5) - F(1)) + a06 * (F(4) - F(2));
        }
        for (int i = 4; i <= n - 3; i++) R(i) = b06 * (F(i + 2) - F(i - 2)) + a06 * (F(i + 1) - F(i - 1));
        if (c.topSided) {
            R(n - 2) = a_np_3 * (F(n - 1) - F(n - 3)) + b_np_3 * (F(n) - F(n - 4));
            R(n - 1) = a_np_2 * (F(n) - F(n - 2));
            R(n) = -a_np_1 * F(n) - b_np_1 * F(n - 1) - c_np_1 * F(n - 2) - d_np_1 * F(n - 3);
        } else if (c.topEven) {
            R(n - 2) = b06 * (F(n) - F(n - 4)) + a06 * (F(n - 1) - F(n - 3));
            R(n - 1) = b06 * (F(n) - F(n - 3)) + a06 * (F(n) - F(n - 2));
            R(n) = b06 * (F(n - 1) - F(n - 2)) + a06 * (F(n) - F(n - 1));
        } else {
            R(n - 2) = b06 * (F(n) - F(n - 4)) + a06 * (F(n - 1) - F(n - 3));
            R(n - 1) = -b06 * (F(n) + F(n - 3)) + a06 * (F(n) - F(n - 2));
            R(n) = -b06 * (F(n - 1) + F(n - 2)) - a06 * (F(n) + F(n - 1));
        }
        o.io = {-2, -1, 1, 2};
        o.ic = {-b06, -a06, a06, b06};
        const double alphaLOW = 3.0;
        if (c.topSided) {
            lrow(n, k.w1 * alphaLOW, k.w1 * 1.0, k.w1 * 0.0);
            lrow(n - 1, k.w2 * k.alpha_p, k.w2 * 1.0, k.w2 * k.alpha_p);
            lrow(n - 2, k.w3 * k.alpha_pp, k.w3 * 1.0, k.w3 * k.alpha_pp);
        } else lh[n - 1][2] = c.topEven ? (1.0 - alpha) : (1.0 + alpha);
        if (c.botSided) {
            lrow(1, k.w1 * 0.0, k.w1 * 1.0, k.w1 * alphaLOW);
            lrow(2, k.w2 * k.alpha_p, k.w2 * 1.0, k.w2 * k.alpha_p);
            lrow(3, k.w3 * k.alpha_pp, k.w3 * 1.0, k.w3 * k.alpha_pp);
        } else lh[0][2] = c.botEven ? (1.0 - alpha) : (1.0 + alpha);
    } else if (op == D1_E2E) {  // D1RHS_E2E_common.F90, ComputeTri_allRoutines.F90:162-197
        const double a06 = ((14.0 / 9.0) / 2.0) * dxi, b06 = ((1.0 / 9.0) / 4.0) * dxi;
        for (int i = 2; i <= nE - 1; i++) R(i) = a06 * (F(i + 1) - F(i - 1));
        for (int i = 3; i <= nE - 2; i++) R(i) = R(i) + b06 * (F(i + 2) - F(i - 2));
        if (c.botEven) { R(1) = LinForm(); R(2) = R(2) + b06 * (F(4) - F(2)); }
        else { R(1) = b06 * (F(3) + F(3)) + a06 * (F(2) + F(2)); R(2) = R(2) + b06 * (F(4) + F(2)); }
        if (c.topEven) { R(nE) = LinForm(); R(nE - 1) = R(nE - 1) + b06 * (F(nE - 1) - F(nE - 3)); }
        else {
            R(nE) = -b06 * (F(nE - 2) + F(nE - 2)) - a06 * (F(nE - 1) + F(nE - 1));
            R(nE - 1) = R(nE - 1) - b06 * (F(nE - 1) + F(nE - 3));
        }
        o.io = {-2, -1, 1, 2};
        o.ic = {-b06, -a06, a06, b06};
        lh[nE - 1][2] = 1.0; lh[nE - 1][1] = c.topEven ? 0.0 : 2.0 * alpha;
        lh[0][2] = 1.0; lh[0][3] = c.botEven ? 0.0 : 2.0 * alpha;
    } else if (op == D2_C2C || op == D2_E2E) {  // D2RHS_C2C/E2E_common.F90, ComputeTri_allRoutines.F90:294-366
        const double a06 = (12.0 / 11.0) * dxi2, b06 = ((3.0 / 11.0) / 4.0) * dxi2;
        const int m = (op == D2_C2C) ? n : nE;
        for (int i = 2; i <= m - 1; i++) R(i) = a06 * (F(i + 1) + F(i - 1));
        for (int i = 3; i <= m - 2; i++) R(i) = R(i) + b06 * (F(i + 2) + F(i - 2));
        if (op == D2_C2C) {
            if (c.botEven) { R(1) = b06 * (F(3) + F(2)) + a06 * (F(2) + F(1)); R(2) = R(2) + b06 * (F(4) + F(1)); }
            else { R(1) = b06 * (F(3) - F(2)) + a06 * (F(2) - F(1)); R(2) = R(2) + b06 * (F(4) - F(1)); }
            if (c.topEven) {
                R(n) = b06 * (F(n - 1) + F(n - 2)) + a06 * (F(n) + F(n - 1));
                R(n - 1) = R(n - 1) + b06 * (F(n) + F(n - 3));
            } else {
                R(n) = b06 * (-F(n - 1) + F(n - 2)) + a06 * (-F(n) + F(n - 1));
                R(n - 1) = R(n - 1) + b06 * (-F(n) + F(n - 3));
            }
            lh[n - 1][2] = c.topEven ? 1.0 + alpha : 1.0 - alpha;
            lh[0][2] = c.botEven ? 1.0 + alpha : 1.0 - alpha;
        } else {
            if (c.botEven) { R(1) = b06 * (F(3) + F(3)) + a06 * (F(2) + F(2)); R(2) = R(2) + b06 * (F(4) + F(2)); }
            else { R(1) = LinForm(); R(2) = R(2) + b06 * (F(4) - F(2)); }
            if (c.topEven) {
                R(nE) = 2.0 * b06 * F(nE - 2) + 2.0 * a06 * F(nE - 1);
                R(nE - 1) = R(nE - 1) + b06 * (F(nE - 1) + F(nE - 3));
            } else {
                R(nE) = LinForm();
                R(nE - 1) = R(nE - 1) + b06 * (-F(nE - 1) + F(nE - 3));
            }
            lh[nE - 1][2] = 1.0; lh[nE - 1][1] = c.topEven ? 2.0 * alpha : 0.0;
            lh[0][2] = 1.0; lh[0][3] = c.botEven ? 2.0 * alpha : 0.0;
        }
        for (int i = 1; i <= m; i++) R(i) = R(i) - (2.0 * (b06 + a06)) * F(i);
        o.io = {-2, -1, 0, 1, 2};
        o.ic = {b06, a06, -2.0 * (b06 + a06), a06, b06};
    } else if (op == I_C2E) {  // InterpRHS_C2E_common.F90, ComputeTri_allRoutines.F90:199-244
        const double b = (1.0 / 10.0) / 2.0, a = (3.0 / 2.0) / 2.0;
        const double a0 = 15.0 / 8.0, b0 = -5.0 / 4.0, c0 = 3.0 / 8.0, alpha1 = 1.0 / 6.0,
                     a1 = (1.0 / 8.0) * (9.0 + 10.0 * alpha1);
        for (int i = 2; i <= nE - 1; i++) R(i) = (a) * (F(i) + F(i - 1));
        for (int i = 3; i <= nE - 2; i++) R(i) = R(i) + (b) * (F(i + 1) + F(i - 2));
        if (c.botSided) { R(1) = a0 * F(1) + b0 * F(2) + c0 * F(3); R(2) = (a1 / 2.0) * (F(2) + F(1)); }
        else if (c.botEven) { R(1) = 2.0 * b * F(2) + 2.0 * a * F(1); R(2) = R(2) + (b) * (F(3) + F(1)); }
        else { R(1) = LinForm(); R(2) = R(2) + (b) * (F(3) - F(1)); }
        if (c.topSided) { R(nE) = a0 * F(n) + b0 * F(n - 1) + c0 * F(n - 2); R(nE - 1) = (a1 / 2.0) * (F(n) + F(n - 1)); }
        else if (c.topEven) { R(nE) = 2.0 * b * F(n - 1) + 2.0 * a * F(n); R(nE - 1) = R(nE - 1) + (b) * (F(n) + F(n - 2)); }
        else { R(nE) = LinForm(); R(nE - 1) = R(nE - 1) + (b) * (-F(n) + F(n - 2)); }
        o.io = {-2, -1, 0, 1};
        o.ic = {b, a, a, b};
        if (c.topSided) { lh[nE - 1][3] = 0.0; lh[nE - 1][1] = 0.0; lrow(nE - 1, alpha1, 1.0, alpha1); }
        else if (c.topEven) { lh[nE - 1][1] = 2.0 * alpha; lh[nE - 1][2] = 1.0; }
        else { lh[nE - 1][1] = 0.0; lh[nE - 1][2] = 1.0; }
        if (c.botSided) { lrow(1, 0.0, 1.0, 0.0); lrow(2, alpha1, 1.0, alpha1); }
        else if (c.botEven) { lh[0][3] = 2.0 * alpha; lh[0][2] = 1.0; }
        else { lh[0][3] = 0.0; lh[0][2] = 1.0; }
    } else {  // I_E2C: InterpRHS_E2C_common.F90, ComputeTri_allRoutines.F90:247-291
        const double b = (1.0 / 10.0) / 2.0, a = (3.0 / 2.0) / 2.0, alpha0 = 1.0;
        const double a0 = (1.0 / 16.0) * (5.0 - alpha0), b0 = (1.0 / 16.0) * (9.0 * alpha0 + 15.0);
        const double c0 = (1.0 / 16.0) * (9.0 * alpha0 - 5.0), d0 = (1.0 / 16.0) * (1.0 - alpha0);
        if (c.botSided) R(1) = a0 * F(1) + b0 * F(2) + c0 * F(3) + d0 * F(4);
        else if (c.botEven) R(1) = (b) * (F(3) + F(2)) + (a) * (F(2) + F(1));
        else R(1) = (b) * (F(3) - F(2)) + (a) * (F(2) + F(1));
        for (int i = 2; i <= n - 1; i++) R(i) = (b) * (F(i + 2) + F(i - 1)) + (a) * (F(i + 1) + F(i));
        if (c.topSided) R(n) = a0 * F(nE) + b0 * F(nE - 1) + c0 * F(nE - 2) + d0 * F(nE - 3);
        else if (c.topEven) R(n) = (b) * (F(nE - 1) + F(nE - 2)) + (a) * (F(nE) + F(nE - 1));
        else R(n) = (b) * (-F(nE - 1) + F(nE - 2)) + (a) * (F(nE) + F(nE - 1));
        o.io = {-1, 0, 1, 2};
        o.ic = {b, a, a, b};
        if (c.topSided) { lh[n - 1][1] = alpha0; lh[n - 1][3] = 0.0; }
        else lh[n - 1][2] = c.topEven ? (1.0 + alpha) : (1.0 - alpha);
        if (c.botSided) { lh[0][3] = alpha0; lh[0][1] = 0.0; }
        else lh[0][2] = c.botEven ? (1.0 + alpha) : (1.0 - alpha);
    }
    o.lhs[0][1] = 0.0;
    o.lhs[no - 1][3] = 0.0;
    return PS_OK;
}

// Dense nout x m matrix of the operator (A^-1 B with copied rows), by band elimination in
// long double on the dense B.  Host-side only; O(ns * q * m).
// Pade6stagg fd02 (PadeDerOps.F90:146-995, fd02 branches) over staggOps (staggOps.F90:54-448).
// Every operator is explicit (q = 0), written row by row on the true input/output lengths
// (cells n, edges n + 1), the periodic wrap as explicit column indices.
int def_fd02(int n, double dz, bool periodic, int bot, int top, int op, OpDef& o) {
    if (n < 3) return PS_EINVAL;
    const bool inE = (op == D1_E2C || op == D2_E2E || op == I_E2C);
    const bool outE = (op == D1_C2E || op == D2_E2E || op == I_C2E);
    if (op != D1_E2C && op != D1_C2E && op != D2_C2C && op != D2_E2E && op != I_E2C && op != I_C2E) return PS_ENOTSUP;
    o = OpDef();
    o.m = inE ? n + 1 : n;
    o.nout = outE ? n + 1 : n;
    o.ns = o.nout;
    o.q = 0;
    o.cyclic = false;
    o.rhs.assign(o.ns, LinForm());
    o.lhs.assign(o.ns, {0, 0, 1, 0, 0});
    auto F = [](int i) { return LinForm(i - 1, 1.0); };  // 1-based
    auto R = [&](int i) -> LinForm& { return o.rhs[i - 1]; };
    const double dzi = 1.0 / dz, dzi2 = 1.0 / (dz * dz);
    const bool codes = bot >= -1 && bot <= 1 && top >= -1 && top <= 1;
    switch (op) {
    case D1_E2C:  // staggOps.F90:54-64; the same operator for every (bot, top) (PadeDerOps.F90:583-585)
        for (int i = 1; i <= n; i++) R(i) = dzi * (F(i + 1) - F(i));
        o.io = {0, 1};
        o.ic = {-dzi, dzi};
        break;
    case I_E2C:  // staggOps.F90:390-399
        for (int i = 1; i <= n; i++) R(i) = 0.5 * (F(i) + F(i + 1));
        o.io = {0, 1};
        o.ic = {0.5, 0.5};
        break;
    case D1_C2E: {  // staggOps.F90:78-107; evenness flags of PadeDerOps.F90:419-445
        for (int i = 2; i <= n; i++) R(i) = dzi * (F(i) - F(i - 1));
        if (periodic) {
            R(1) = dzi * (F(1) - F(n));
            R(n + 1) = R(1);
        } else {
            if (!codes) return zero_op(o, n, false), o.m = n, o.nout = n + 1, o.ns = n + 1, PS_OK;
            const bool be = bot != -1, te = top == 1 || (top == 0 && bot == -1);
            R(1) = be ? LinForm() : (2.0 * dzi) * F(1);
            R(n + 1) = te ? LinForm() : (-2.0 * dzi) * F(n);
        }
        o.io = {-1, 0};
        o.ic = {-dzi, dzi};
        break;
    }
    case I_C2E: {  // staggOps.F90:431-448 with the overrides of PadeDerOps.F90:703-738
        for (int i = 2; i <= n; i++) R(i) = 0.5 * (F(i - 1) + F(i));
        if (periodic) {
            R(1) = 0.5 * (F(1) + F(n));
            R(n + 1) = R(1);
        } else {
            if (!codes) return zero_op(o, n, false), o.m = n, o.nout = n + 1, o.ns = n + 1, PS_OK;
            // bottom: -1 the zero BotVal, 0 2 f1 - e2 (one-sided), 1 f1; top likewise
            R(1) = bot == -1 ? LinForm() : (bot == 0 ? 2.0 * F(1) - 0.5 * (F(1) + F(2)) : F(1));
            R(n + 1) = top == -1 ? LinForm() : (top == 0 ? 2.0 * F(n) - 0.5 * (F(n - 1) + F(n)) : F(n));
        }
        o.io = {-1, 0};
        o.ic = {0.5, 0.5};
        break;
    }
    case D2_C2C: {  // staggOps.F90:235-264 (the interior reads f(k-1), f(k), f(k+1)); PadeDerOps.F90:159-183
        for (int i = 2; i <= n - 1; i++) R(i) = dzi2 * (F(i + 1) - 2.0 * F(i) + F(i - 1));
        if (periodic) {
            R(1) = dzi2 * (F(2) - 2.0 * F(1) + F(n));
            R(n) = dzi2 * (F(1) - 2.0 * F(n) + F(n - 1));
        } else {
            if (!codes || bot == 0 || top == 0) return zero_op(o, n, false), PS_OK;
            R(1) = dzi2 * (bot == 1 ? F(2) - F(1) : F(2) - 3.0 * F(1));
            R(n) = dzi2 * (top == 1 ? F(n - 1) - F(n) : F(n - 1) - 3.0 * F(n));
        }
        o.io = {-1, 0, 1};
        o.ic = {dzi2, -2.0 * dzi2, dzi2};
        break;
    }
    case D2_E2E: {  // staggOps.F90:297-326; PadeDerOps.F90:283-312
        const int nE = n + 1;
        for (int i = 2; i <= nE - 1; i++) R(i) = dzi2 * (F(i + 1) - 2.0 * F(i) + F(i - 1));
        if (periodic) {
            R(1) = dzi2 * (F(2) - 2.0 * F(1) + F(nE - 1));
            R(nE) = dzi2 * (F(2) - 2.0 * F(nE) + F(nE - 1));
        } else {
            if (!codes || bot == 0 || top == 0) return zero_op(o, nE, false), PS_OK;
            R(1) = bot == 1 ? (2.0 * dzi2) * (F(2) - F(1)) : LinForm();
            R(nE) = top == 1 ? (2.0 * dzi2) * (F(nE - 1) - F(nE)) : LinForm();
        }
        o.io = {-1, 0, 1};
        o.ic = {dzi2, -2.0 * dzi2, dzi2};
        break;
    }
    }
    return PS_OK;
}

int dense_operator(const OpDef& d, std::vector<double>& M) {
    M.assign((size_t)d.nout * d.m, 0.0);
    if (d.zero) return PS_OK;
    if (d.identity) {
        for (int i = 0; i < d.nout; i++) M[(size_t)i * d.m + i] = 1.0;
        return PS_OK;
    }
    const int ns = d.ns, m = d.m;
    std::vector<long double> A((size_t)ns * ns, 0.0L), B((size_t)ns * m, 0.0L);
    for (int i = 0; i < ns; i++) {
        for (auto& p : d.rhs[i].t) B[(size_t)i * m + p.first] += p.second;
        for (int o = -2; o <= 2; o++) {
            double v = d.lhs[i][o + 2];
            if (v == 0.0) continue;
            int j = i + o;
            if (d.cyclic) j = ((j % ns) + ns) % ns;
            else if (j < 0 || j >= ns) continue;
            A[(size_t)i * ns + j] += v;
        }
    }
    if (d.q == 0) {
        for (int i = 0; i < ns; i++)
            for (int j = 0; j < m; j++) M[(size_t)i * m + j] = (double)B[(size_t)i * m + j];
    } else {
        // Gaussian elimination with partial pivoting on the dense system (small n only)
        std::vector<int> piv(ns);
        for (int c = 0; c < ns; c++) {
            int p = c;
            for (int r = c + 1; r < ns; r++)
                if (fabsl(A[(size_t)r * ns + c]) > fabsl(A[(size_t)p * ns + c])) p = r;
            if (A[(size_t)p * ns + c] == 0.0L) return PS_EINVAL;
            if (p != c) {
                for (int j = 0; j < ns; j++) std::swap(A[(size_t)p * ns + j], A[(size_t)c * ns + j]);
                for (int j = 0; j < m; j++) std::swap(B[(size_t)p * m + j], B[(size_t)c * m + j]);
            }
            for (int r = c + 1; r < ns; r++) {
                long double l = A[(size_t)r * ns + c] / A[(size_t)c * ns + c];
                if (l == 0.0L) continue;
                for (int j = c; j < ns; j++) A[(size_t)r * ns + j] -= l * A[(size_t)c * ns + j];
                for (int j = 0; j < m; j++) B[(size_t)r * m + j] -= l * B[(size_t)c * m + j];
            }
        }
        for (int c = ns - 1; c >= 0; c--) {
            for (int j = 0; j < m; j++) {
                long double s = B[(size_t)c * m + j];
                for (int k = c + 1; k < ns; k++) s -= A[(size_t)c * ns + k] * B[(size_t)k * m + j];
                B[(size_t)c * m + j] = s / A[(size_t)c * ns + c];
            }
        }
        for (int i = 0; i < ns; i++)
            for (int j = 0; j < m; j++) M[(size_t)i * m + j] = (double)B[(size_t)i * m + j];
    }
    for (int i = ns; i < d.nout; i++)
        for (int j = 0; j < m; j++) M[(size_t)i * m + j] = M[(size_t)(i - ns) * m + j];
    return PS_OK;
}

}  // namespace pade
