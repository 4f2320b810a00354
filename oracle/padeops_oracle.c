/*
 * padeops_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C, FP64 restatement of the PadeOps (FPAL-Stanford-University/PadeOps)
 * compact-difference and compact-filter line algorithms.  It exists to check the
 * GPU library: only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark may load it.  The product library never links or calls it.
 *
 * Every routine works on ONE line of a 3-D column-major array, addressed as
 * p[(i-1)*s] for the 1-based index i, so one restatement serves the reference's
 * X, Y and Z variants (which were checked to be the same formulas after index
 * normalisation).  Loop order, factorisation arrays and the order of the
 * floating-point operations follow the cited Fortran lines, so the results agree
 * with the reference to rounding (the reference's Release build uses
 * -ffast-math, so agreement is to ~1e-15 relative, not bitwise).
 *
 * Parity status: the Fortran cannot be compiled here (no Fortran compiler on
 * either machine), and the reference ships no stored output vectors.  The
 * restatement is pinned by the reference's own known-answer tests (analytic
 * derivatives, filter transfer function, modified wavenumbers) and by an
 * independent dense-matrix restatement in the tests.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_API __attribute__((visibility("default")))

/* ------------------------------------------------------------------------- */
/* accessors                                                                  */
/* ------------------------------------------------------------------------- */
/* column-major (i,c) element of an n x ncol coefficient table, 1-based */
#define T(a, i, c) (a)[((long)(c) - 1) * (long)n + ((long)(i) - 1)]

/* ------------------------------------------------------------------------- */
/* cd06: 6th-order collocated compact first derivative (src/derivatives/cd06.F90) */
/* ------------------------------------------------------------------------- */

/* cd06.F90:14-21 */
static const double alpha06d1 = 1.0 / 3.0;
static const double a06d1 = (14.0 / 9.0) / 2.0;
static const double b06d1 = (1.0 / 9.0) / 4.0;
static const double alpha06d2 = 2.0 / 11.0;
static const double a06d2 = (12.0 / 11.0) / 1.0;
static const double b06d2 = (3.0 / 11.0) / 4.0;

/* cd06.F90:29-59 one-sided closure constants (computed like the Fortran parameters) */
typedef struct {
    double alpha, p, q, r, s, qhat, rhat, alpha_hat, q_p, alpha_p, alpha_pp, q_pp, r_pp, w1, w2, w3;
} cd06_bnd_t;

static cd06_bnd_t cd06_bnd(void) {
    cd06_bnd_t k;
    k.alpha = 3.0;
    k.p = 17.0 / 6.0;
    k.q = 3.0 / 2.0;
    k.r = 3.0 / 2.0;
    k.s = -1.0 / 6.0;
    k.qhat = a06d1;
    k.rhat = b06d1;
    k.alpha_hat = alpha06d1;
    k.q_p = 3.0 / 4.0;
    k.alpha_p = 1.0 / 4.0;
    k.alpha_pp = ((40 * k.alpha_hat - 1) * k.q + 7 * (4 * k.alpha_hat - 1) * k.s) /
                 (16 * (k.alpha_hat + 2) * k.q + 8 * (1 - 4 * k.alpha_hat) * k.s);
    k.q_pp = (1.0 / 3.0) * (k.alpha_pp + 2);
    k.r_pp = (1.0 / 12.0) * (4 * k.alpha_pp - 1);
    k.w1 = (2 * k.alpha_hat + 1) / (2 * (k.q + k.s));
    k.w2 = ((8 * k.alpha_hat + 7) * k.q - 6 * (2 * k.alpha_hat + 1) * k.r + (8 * k.alpha_hat + 7) * k.s) /
           (9 * (k.q + k.s));
    k.w3 = (4 * (k.alpha_hat + 2) * k.q + 2 * (1 - 4 * k.alpha_hat) * k.s) / (9 * (k.q + k.s));
    return k;
}

/* Periodic cyclic-tridiagonal LU after Neossi Nguetchue & Abelman (cd06.F90:221-262;
 * identical routine in cd06stagg.F90:631-672).  LU is n x 5: bc,h,c,aa,v. */
static void tri_cyclic_lu(double *LU, int n, double b, double d, double a) {
    memset(LU, 0, sizeof(double) * 5 * (size_t)n);
#define bc(i) T(LU, i, 1)
#define h(i) T(LU, i, 2)
#define c(i) T(LU, i, 3)
#define aa(i) T(LU, i, 4)
#define v(i) T(LU, i, 5)
    c(1) = d;
    v(1) = b;
    h(1) = a / c(1);
    for (int i = 2; i <= n - 1; i++) c(i) = d - (b / c(i - 1)) * a;
    for (int i = 2; i <= n - 2; i++) {
        v(i) = -(b / c(i - 1)) * v(i - 1);
        h(i) = -(a / c(i)) * h(i - 1);
    }
    v(n - 1) = a - (b / c(n - 2)) * v(n - 2);
    h(n - 1) = (b - h(n - 2) * a) / c(n - 1);
    double sum = 0.0;
    for (int i = 1; i <= n - 1; i++) sum += h(i) * v(i);
    c(n) = d - sum;
    for (int i = 2; i <= n - 1; i++) bc(i) = b / c(i - 1);
    for (int i = 1; i <= n - 2; i++) aa(i) = a;
    for (int i = 1; i <= n; i++) c(i) = 1.0 / c(i);
    for (int i = 1; i <= n; i++) aa(i) = aa(i) * c(i);
    for (int i = 1; i <= n; i++) v(i) = v(i) * c(i);
#undef bc
#undef h
#undef c
#undef aa
#undef v
}

/* Cyclic-tridiagonal solve (cd06.F90:345-373 SolveXLU1; cd06stagg.F90:248-273 SolveZLU) */
static void tri_cyclic_solve(const double *LU, int n, double *y, long ys) {
#define Y(i) y[((long)(i) - 1) * ys]
    double sum1 = T(LU, 1, 2) * Y(1);
    for (int i = 2; i <= n - 1; i++) {
        Y(i) = Y(i) - T(LU, i, 1) * Y(i - 1);
        sum1 = sum1 + T(LU, i, 2) * Y(i);
    }
    Y(n) = Y(n) - sum1;
    Y(n) = Y(n) * T(LU, n, 3);
    Y(n - 1) = Y(n - 1) * T(LU, n - 1, 3) - Y(n) * T(LU, n - 1, 5);
    for (int i = n - 2; i >= 1; i--) Y(i) = Y(i) * T(LU, i, 3) - Y(i + 1) * T(LU, i, 4) - Y(n) * T(LU, i, 5);
#undef Y
}

/* Thomas factorisation shared by cd06 ComputeTri1 (cd06.F90:315-325) and every
 * cd06stagg ComputeTri* routine (STAGG_CD06_files/ComputeTri_common.F90). Tri is n x 3. */
static void tri_factor(double *Tri, int n, const double *ddn, const double *dg, const double *dup) {
    double *cp = calloc((size_t)n, sizeof(double)), *den = calloc((size_t)n, sizeof(double));
    cp[0] = dup[0] / dg[0];
    for (int i = 2; i <= n - 1; i++) cp[i - 1] = dup[i - 1] / (dg[i - 1] - ddn[i - 1] * cp[i - 2]);
    den[0] = 1.0 / dg[0];
    for (int i = 2; i <= n; i++) den[i - 1] = 1.0 / (dg[i - 1] - ddn[i - 1] * cp[i - 2]);
    for (int i = 1; i <= n; i++) {
        T(Tri, i, 1) = ddn[i - 1] * den[i - 1];
        T(Tri, i, 2) = den[i - 1];
        T(Tri, i, 3) = cp[i - 1];
    }
    free(cp);
    free(den);
}

/* Thomas solve (cd06.F90:432-452 SolveXTri1; STAGG_CD06_files/TridiagSolver_allRoutines.F90:1-16) */
static void tri_solve(const double *Tri, int n, double *y, long ys) {
#define Y(i) y[((long)(i) - 1) * ys]
    Y(1) = Y(1) * T(Tri, 1, 2);
    for (int i = 2; i <= n; i++) Y(i) = Y(i) * T(Tri, i, 2) - Y(i - 1) * T(Tri, i, 1);
    for (int i = n - 1; i >= 1; i--) Y(i) = Y(i) - T(Tri, i, 3) * Y(i + 1);
#undef Y
}

typedef struct {
    int n, periodic, bc1, bcn;
    double dx, onebydx, onebydx2;
    double *LU1, *LU2, *Tri1;
} cd06_t;

/* cd06.F90:129-201 */
static int cd06_init(cd06_t *o, int n, double dx, int periodic, int bc1, int bcn) {
    memset(o, 0, sizeof(*o));
    o->n = n;
    o->dx = dx;
    o->onebydx = 1.0 / dx;
    o->onebydx2 = o->onebydx / dx;
    o->periodic = periodic;
    o->bc1 = bc1;
    o->bcn = bcn;
    if (periodic) {
        if (n >= 6) {
            o->LU1 = malloc(sizeof(double) * 5 * n);
            o->LU2 = malloc(sizeof(double) * 5 * n);
            tri_cyclic_lu(o->LU1, n, alpha06d1, 1.0, alpha06d1);
            tri_cyclic_lu(o->LU2, n, alpha06d2, 1.0, alpha06d2);
        } else if (n != 1) {
            return 3;
        }
    } else {
        if (n >= 8) {
            cd06_bnd_t k = cd06_bnd();
            double *a = malloc(sizeof(double) * n), *b = malloc(sizeof(double) * n), *c = malloc(sizeof(double) * n);
            for (int i = 0; i < n; i++) {
                a[i] = k.alpha_hat;
                b[i] = 1.0;
                c[i] = k.alpha_hat;
            }
            /* cd06.F90:274-313: only bc=0 modifies the matrix ("1" is incomplete upstream) */
            if (bc1 == 0) {
                a[0] = k.w1 * 0.0; a[1] = k.w2 * k.alpha_p; a[2] = k.w3 * k.alpha_pp;
                b[0] = k.w1 * 1.0; b[1] = k.w2 * 1.0;       b[2] = k.w3 * 1.0;
                c[0] = k.w1 * k.alpha; c[1] = k.w2 * k.alpha_p; c[2] = k.w3 * k.alpha_pp;
            }
            if (bcn == 0) {
                c[n - 1] = k.w1 * 0.0; c[n - 2] = k.w2 * k.alpha_p; c[n - 3] = k.w3 * k.alpha_pp;
                b[n - 1] = k.w1 * 1.0; b[n - 2] = k.w2 * 1.0;       b[n - 3] = k.w3 * 1.0;
                a[n - 1] = k.w1 * k.alpha; a[n - 2] = k.w2 * k.alpha_p; a[n - 3] = k.w3 * k.alpha_pp;
            }
            o->Tri1 = malloc(sizeof(double) * 3 * n);
            tri_factor(o->Tri1, n, a, b, c);
            free(a);
            free(b);
            free(c);
        } else if (n != 1) {
            return 2;
        }
    }
    return 0;
}

static void cd06_free(cd06_t *o) {
    free(o->LU1);
    free(o->LU2);
    free(o->Tri1);
}

/* First-derivative RHS (cd06.F90:515-592) */
static void cd06_rhs_d1(const cd06_t *o, const double *f, long fs, double *r, long rs) {
#define F(i) f[((long)(i) - 1) * fs]
#define R(i) r[((long)(i) - 1) * rs]
    const int n = o->n;
    double a06 = a06d1 * o->onebydx, b06 = b06d1 * o->onebydx;
    if (o->periodic) {
        R(1) = a06 * (F(2) - F(n)) + b06 * (F(3) - F(n - 1));
        R(2) = a06 * (F(3) - F(1)) + b06 * (F(4) - F(n));
        for (int i = 3; i <= n - 2; i++) R(i) = a06 * (F(i + 1) - F(i - 1)) + b06 * (F(i + 2) - F(i - 2));
        R(n - 1) = a06 * (F(n) - F(n - 2)) + b06 * (F(1) - F(n - 3));
        R(n) = a06 * (F(1) - F(n - 1)) + b06 * (F(2) - F(n - 2));
    } else {
        cd06_bnd_t k = cd06_bnd();
        double a_np_3 = k.w3 * k.q_pp * o->onebydx, b_np_3 = k.w3 * k.r_pp * o->onebydx;
        double a_np_2 = k.w2 * k.q_p * o->onebydx;
        double a_np_1 = k.w1 * (-k.p * o->onebydx), b_np_1 = k.w1 * (k.q * o->onebydx);
        double c_np_1 = k.w1 * (k.r * o->onebydx), d_np_1 = k.w1 * (k.s * o->onebydx);
        R(1) = a_np_1 * F(1) + b_np_1 * F(2) + c_np_1 * F(3) + d_np_1 * F(4);
        R(2) = a_np_2 * (F(3) - F(1));
        R(3) = a_np_3 * (F(4) - F(2)) + b_np_3 * (F(5) - F(1));
        for (int i = 4; i <= n - 3; i++) R(i) = b06 * (F(i + 2) - F(i - 2)) + a06 * (F(i + 1) - F(i - 1));
        R(n - 2) = a_np_3 * (F(n - 1) - F(n - 3)) + b_np_3 * (F(n) - F(n - 4));
        R(n - 1) = a_np_2 * (F(n) - F(n - 2));
        R(n) = -a_np_1 * F(n) - b_np_1 * F(n - 1) - c_np_1 * F(n - 2) - d_np_1 * F(n - 3);
    }
#undef F
#undef R
}

/* Periodic second-derivative RHS (cd06.F90:745-773).  Upstream this routine omits the
 * 1/dx^2 factor and the second derivative is never solved ("Incomplete"); the restatement
 * completes it by applying 1/dx^2 and the cyclic solve with LU2 (cd06.F90:163-170).  This
 * completed operator has no reference output to pin it beyond the analytic symbol. */
static void cd06_rhs_d2_periodic(const cd06_t *o, const double *f, long fs, double *r, long rs) {
#define F(i) f[((long)(i) - 1) * fs]
#define R(i) r[((long)(i) - 1) * rs]
    const int n = o->n;
    R(1) = a06d2 * (F(2) - 2.0 * F(1) + F(n)) + b06d2 * (F(3) - 2.0 * F(1) + F(n - 1));
    R(2) = a06d2 * (F(3) - 2.0 * F(2) + F(1)) + b06d2 * (F(4) - 2.0 * F(2) + F(n));
    for (int i = 3; i <= n - 2; i++)
        R(i) = a06d2 * (F(i + 1) - 2.0 * F(i) + F(i - 1)) + b06d2 * (F(i + 2) - 2.0 * F(i) + F(i - 2));
    R(n - 1) = a06d2 * (F(n) - 2.0 * F(n - 1) + F(n - 2)) + b06d2 * (F(1) - 2.0 * F(n - 1) + F(n - 3));
    R(n) = a06d2 * (F(1) - 2.0 * F(n) + F(n - 1)) + b06d2 * (F(2) - 2.0 * F(n) + F(n - 2));
    for (int i = 1; i <= n; i++) R(i) = R(i) * o->onebydx2;
#undef F
#undef R
}

/* dd1/dd2/dd3 on one line (cd06.F90:775-839) */
static void cd06_d1_line(const cd06_t *o, const double *f, long fs, double *df, long dfs) {
    if (o->n == 1) {
        df[0] = 0.0;
        return;
    }
    cd06_rhs_d1(o, f, fs, df, dfs);
    if (o->periodic) tri_cyclic_solve(o->LU1, o->n, df, dfs);
    else tri_solve(o->Tri1, o->n, df, dfs);
}

static void cd06_d2_line(const cd06_t *o, const double *f, long fs, double *df, long dfs) {
    if (o->n == 1) {
        df[0] = 0.0;
        return;
    }
    cd06_rhs_d2_periodic(o, f, fs, df, dfs);
    tri_cyclic_solve(o->LU2, o->n, df, dfs);
}

/* ------------------------------------------------------------------------- */
/* cd10: 10th-order collocated compact first/second derivative (cd10.F90)       */
/* ------------------------------------------------------------------------- */

/* cd10.F90:16-27 */
static const double alpha10d1 = 1.0 / 2.0;
static const double beta10d1 = 1.0 / 20.0;
static const double a10d1 = (17.0 / 12.0) / 2.0;
static const double b10d1 = (101.0 / 150.0) / 4.0;
static const double c10d1 = (1.0 / 100.0) / 6.0;
static const double alpha10d2 = 334.0 / 899.0;
static const double beta10d2 = 43.0 / 1798.0;
static const double a10d2 = (1065.0 / 1798.0) / 1.0;
static const double b10d2 = (1038.0 / 899.0) / 4.0;
static const double c10d2 = (79.0 / 1798.0) / 9.0;

typedef struct {
    double alpha, p, q, r, s, q_hat, r_hat, s_hat, alpha_hat, beta_hat, q_p, alpha_p;
    double alpha_ppp, beta_ppp, q_ppp, r_ppp, s_ppp, alpha_pp, beta_pp, q_pp, r_pp, w1, w2, w3, w4;
    double b1_alpha, b1_a, b1_b, b1_c, b1_d, b1_e, b2_alpha, b2_a, b3_alpha, b3_beta, b3_a, b3_b;
} cd10_bnd_t;

/* cd10.F90:35-104 */
static cd10_bnd_t cd10_bnd(void) {
    cd10_bnd_t k;
    k.alpha = 3.0;
    k.p = -17.0 / 6.0;
    k.q = 3.0 / 2.0;
    k.r = 3.0 / 2.0;
    k.s = -1.0 / 6.0;
    k.q_hat = a10d1;
    k.r_hat = b10d1;
    k.s_hat = c10d1;
    k.alpha_hat = alpha10d1;
    k.beta_hat = beta10d1;
    k.q_p = 3.0 / 4.0;
    k.alpha_p = 1.0 / 4.0;
    k.alpha_ppp = (8 * k.r_hat - 175 * k.s_hat) / (18 * k.r_hat - 550 * k.s_hat);
    k.beta_ppp = (1.0 / 20.0) * (-3 + 8 * k.alpha_ppp);
    k.q_ppp = (1.0 / 12.0) * (12 - 7 * k.alpha_ppp);
    k.r_ppp = (1.0 / 600.0) * (568 * k.alpha_ppp - 183);
    k.s_ppp = (1.0 / 300.0) * (9 * k.alpha_ppp - 4);
    {
        double qh = k.q_hat, rh = k.r_hat, sh = k.s_hat, q = k.q, s = k.s;
        double t = (qh + rh - sh * (k.q_ppp / k.s_ppp - 1));
        k.alpha_pp = ((17 * (s * (rh + 2 * sh) - q * (qh + rh + sh))) / (72 * (q + s) * t) - 8.0 / 9.0) /
                     ((19 * (s * (rh + 2 * sh) - q * (qh + rh + sh))) / (24 * (q + s) * t) - 1.0 / 3);
    }
    k.beta_pp = (1.0 / 12.0) * (-1 + 3 * k.alpha_pp);
    k.q_pp = (2.0 / 18.0) * (8 - 3 * k.alpha_pp);
    k.r_pp = (1.0 / 72.0) * (-17 + 57 * k.alpha_pp);
    k.w1 = (k.q_hat + 2 * k.r_hat + 3 * k.s_hat) / (k.q + k.s);
    k.w2 = (1 / k.q_p) * (k.r_hat + k.s_hat * (1 + k.q_ppp / k.s_ppp) -
                          k.r * (k.q_hat + 2 * k.r_hat + 3 * k.s_hat) / (k.q + k.s));
    k.w3 = (k.q_hat + k.r_hat + k.s_hat * (1 - k.q_ppp / k.s_ppp)) / (k.r_pp);
    k.w4 = k.s_hat / k.s_ppp;
    k.b1_alpha = 11.0;
    k.b1_a = (11 * k.b1_alpha + 35) / 12;
    k.b1_b = -(5 * k.b1_alpha + 26) / 3;
    k.b1_c = (k.b1_alpha + 19) / 2;
    k.b1_d = (k.b1_alpha - 14) / 3;
    k.b1_e = (11 - k.b1_alpha) / 12;
    k.b2_alpha = 1.0 / 10.0;
    k.b2_a = (4 * (1 - k.b2_alpha) / 3) / 1.0;
    k.b3_alpha = 344.0 / 1179.0;
    k.b3_beta = (38.0 * k.b3_alpha - 9.0) / 214.0;
    k.b3_a = ((696 - 1191 * k.b3_alpha) / 428) / 1.0;
    k.b3_b = ((2454 * k.b3_alpha - 294) / 535) / 4.0;
    return k;
}

/* Periodic cyclic-pentadiagonal LU (cd10.F90:351-427; identical in cf90.F90:198-274).
 * LU is n x 9: b,eg,k,l,g,h,ff,v,w. */
static void penta_cyclic_lu(double *LU, int n, double e, double a, double d, double c, double f) {
    memset(LU, 0, sizeof(double) * 9 * (size_t)n);
#define b(i) T(LU, i, 1)
#define eg(i) T(LU, i, 2)
#define k(i) T(LU, i, 3)
#define l(i) T(LU, i, 4)
#define g(i) T(LU, i, 5)
#define h(i) T(LU, i, 6)
#define ff(i) T(LU, i, 7)
#define v(i) T(LU, i, 8)
#define w(i) T(LU, i, 9)
    g(1) = d;
    b(2) = a / g(1);
    h(1) = c;
    k(1) = f / g(1);
    w(1) = a;
    v(1) = e;
    l(1) = c / g(1);
    g(2) = d - b(2) * h(1);
    k(2) = -k(1) * h(1) / g(2);
    w(2) = e - b(2) * w(1);
    v(2) = -b(2) * v(1);
    l(2) = (f - l(1) * h(1)) / g(2);
    h(2) = c - b(2) * f;
    for (int i = 3; i <= n - 3; i++) {
        b(i) = (a - (e / g(i - 2)) * h(i - 2)) / g(i - 1);
        h(i) = c - b(i) * f;
        g(i) = d - (e / g(i - 2)) * f - b(i) * h(i - 1);
    }
    b(n - 2) = (a - (e / g(n - 4)) * h(n - 4)) / g(n - 3);
    g(n - 2) = d - (e / g(n - 4)) * f - b(n - 2) * h(n - 3);
    for (int i = 3; i <= n - 4; i++) {
        k(i) = -(k(i - 2) * f + k(i - 1) * h(i - 1)) / g(i);
        v(i) = -(e / g(i - 2)) * v(i - 2) - b(i) * v(i - 1);
    }
    k(n - 3) = (e - k(n - 5) * f - k(n - 4) * h(n - 4)) / g(n - 3);
    k(n - 2) = (a - k(n - 4) * f - k(n - 3) * h(n - 3)) / g(n - 2);
    v(n - 3) = f - (e / g(n - 5)) * v(n - 5) - b(n - 3) * v(n - 4);
    v(n - 2) = c - (e / g(n - 4)) * v(n - 4) - b(n - 2) * v(n - 3);
    double s = 0.0;
    for (int i = 1; i <= n - 2; i++) s += k(i) * v(i);
    g(n - 1) = d - s;
    for (int i = 3; i <= n - 3; i++) {
        w(i) = -(e / g(i - 2)) * w(i - 2) - b(i) * w(i - 1);
        l(i) = -(l(i - 2) * f + l(i - 1) * h(i - 1)) / g(i);
    }
    w(n - 2) = f - (e / g(n - 4)) * w(n - 4) - b(n - 2) * w(n - 3);
    s = 0.0;
    for (int i = 1; i <= n - 2; i++) s += k(i) * w(i);
    w(n - 1) = c - s;
    l(n - 2) = (e - l(n - 4) * f - l(n - 3) * h(n - 3)) / g(n - 2);
    s = 0.0;
    for (int i = 1; i <= n - 2; i++) s += l(i) * v(i);
    l(n - 1) = (a - s) / g(n - 1);
    s = 0.0;
    for (int i = 1; i <= n - 1; i++) s += l(i) * w(i);
    g(n) = d - s;
    for (int i = 3; i <= n - 2; i++) eg(i) = e / g(i - 2);
    for (int i = 1; i <= n - 4; i++) ff(i) = f;
    for (int i = 1; i <= n; i++) g(i) = 1.0 / g(i);
#undef b
#undef eg
#undef k
#undef l
#undef g
#undef h
#undef ff
#undef v
#undef w
}

/* Cyclic-pentadiagonal solve (cd10.F90:712-749 SolveXLU1; cf90.F90:421-458 SolveXLU) */
static void penta_cyclic_solve(const double *LU, int n, double *y, long ys) {
#define Y(i) y[((long)(i) - 1) * ys]
    Y(2) = Y(2) - T(LU, 2, 1) * Y(1);
    double sum1 = T(LU, 1, 3) * Y(1) + T(LU, 2, 3) * Y(2);
    double sum2 = T(LU, 1, 4) * Y(1) + T(LU, 2, 4) * Y(2);
    for (int i = 3; i <= n - 2; i++) {
        Y(i) = Y(i) - T(LU, i, 1) * Y(i - 1) - T(LU, i, 2) * Y(i - 2);
        sum1 = sum1 + T(LU, i, 3) * Y(i);
        sum2 = sum2 + T(LU, i, 4) * Y(i);
    }
    Y(n - 1) = Y(n - 1) - sum1;
    Y(n) = (Y(n) - sum2 - T(LU, n - 1, 4) * Y(n - 1)) * T(LU, n, 5);
    Y(n - 1) = (Y(n - 1) - T(LU, n - 1, 9) * Y(n)) * T(LU, n - 1, 5);
    Y(n - 2) = (Y(n - 2) - T(LU, n - 2, 8) * Y(n - 1) - T(LU, n - 2, 9) * Y(n)) * T(LU, n - 2, 5);
    Y(n - 3) = (Y(n - 3) - T(LU, n - 3, 6) * Y(n - 2) - T(LU, n - 3, 8) * Y(n - 1) - T(LU, n - 3, 9) * Y(n)) *
               T(LU, n - 3, 5);
    for (int i = n - 4; i >= 1; i--)
        Y(i) = (Y(i) - T(LU, i, 6) * Y(i + 1) - T(LU, i, 7) * Y(i + 2) - T(LU, i, 8) * Y(n - 1) -
                T(LU, i, 9) * Y(n)) *
               T(LU, i, 5);
#undef Y
}

/* Pentadiagonal factorisation from the five diagonals (the common tail of
 * cd10.F90:558-575 ComputePenta1, 689-706 ComputePenta2 and cf90.F90:398-415).
 * penta is n x 11: bt,b,d,a,at,e,obc,f,g,eobc,(unused). */
static void penta_factor(double *P, int n) {
#define bt(i) T(P, i, 1)
#define b(i) T(P, i, 2)
#define d(i) T(P, i, 3)
#define a(i) T(P, i, 4)
#define at(i) T(P, i, 5)
#define e(i) T(P, i, 6)
#define obc(i) T(P, i, 7)
#define f(i) T(P, i, 8)
#define g(i) T(P, i, 9)
#define eobc(i) T(P, i, 10)
    obc(1) = 1.0 / d(1);
    obc(2) = 1.0 / (d(2) - b(2) * a(1) * obc(1));
    e(1) = a(1);
    f(2) = b(2) * obc(1);
    for (int i = 3; i <= n; i++) {
        g(i) = bt(i) * obc(i - 2);
        e(i - 1) = a(i - 1) - f(i - 1) * at(i - 2);
        f(i) = (b(i) - g(i) * e(i - 2)) * obc(i - 1);
        obc(i) = 1.0 / (d(i) - f(i) * e(i - 1) - g(i) * at(i - 2));
    }
    for (int i = 1; i <= n; i++) eobc(i) = e(i) * obc(i);
#undef bt
#undef b
#undef d
#undef a
#undef at
#undef e
#undef obc
#undef f
#undef g
#undef eobc
}

/* Pentadiagonal solve (cd10.F90:823-851 SolveXPenta1 = 1016-1045 SolveXPenta2;
 * cf90.F90:532-558 SolveXPenta) */
static void penta_solve(const double *P, int n, double *y, long ys) {
#define Y(i) y[((long)(i) - 1) * ys]
    Y(2) = Y(2) - T(P, 2, 8) * Y(1);
    for (int i = 3; i <= n; i++) Y(i) = Y(i) - T(P, i, 9) * Y(i - 2) - T(P, i, 8) * Y(i - 1);
    Y(n) = Y(n) * T(P, n, 7);
    Y(n - 1) = Y(n - 1) * T(P, n - 1, 7) - T(P, n - 1, 10) * Y(n);
    for (int i = n - 2; i >= 1; i--)
        Y(i) = Y(i) * T(P, i, 7) - Y(i + 2) * T(P, i, 5) * T(P, i, 7) - Y(i + 1) * T(P, i, 10);
#undef Y
}

/* The same two solves on nb lines at once: line j of the block at y + j, rows ys apart.  The
 * reference's y and z solves (SolveYPenta1/2, SolveZPenta1/2, SolveYLU*, cd10.F90:751-899,
 * 951-1090; cf90.F90:460-600) run each statement over a whole row of lines (array syntax over
 * x); this restatement does the same, with every line's operations in the per-line order,
 * so the results equal penta_solve / penta_cyclic_solve bit for bit. */
enum { ORACLE_BLOCK = 16 };

static void penta_solve_blk(const double *P, int n, double *y, long ys, int nb) {
#define Y(i) y[((long)(i) - 1) * ys + j]
    for (int j = 0; j < nb; j++) Y(2) = Y(2) - T(P, 2, 8) * Y(1);
    for (int i = 3; i <= n; i++)
        for (int j = 0; j < nb; j++) Y(i) = Y(i) - T(P, i, 9) * Y(i - 2) - T(P, i, 8) * Y(i - 1);
    for (int j = 0; j < nb; j++) Y(n) = Y(n) * T(P, n, 7);
    for (int j = 0; j < nb; j++) Y(n - 1) = Y(n - 1) * T(P, n - 1, 7) - T(P, n - 1, 10) * Y(n);
    for (int i = n - 2; i >= 1; i--)
        for (int j = 0; j < nb; j++)
            Y(i) = Y(i) * T(P, i, 7) - Y(i + 2) * T(P, i, 5) * T(P, i, 7) - Y(i + 1) * T(P, i, 10);
#undef Y
}

static void penta_cyclic_solve_blk(const double *LU, int n, double *y, long ys, int nb) {
#define Y(i) y[((long)(i) - 1) * ys + j]
    double sum1[ORACLE_BLOCK], sum2[ORACLE_BLOCK];
    for (int j = 0; j < nb; j++) {
        Y(2) = Y(2) - T(LU, 2, 1) * Y(1);
        sum1[j] = T(LU, 1, 3) * Y(1) + T(LU, 2, 3) * Y(2);
        sum2[j] = T(LU, 1, 4) * Y(1) + T(LU, 2, 4) * Y(2);
    }
    for (int i = 3; i <= n - 2; i++)
        for (int j = 0; j < nb; j++) {
            Y(i) = Y(i) - T(LU, i, 1) * Y(i - 1) - T(LU, i, 2) * Y(i - 2);
            sum1[j] = sum1[j] + T(LU, i, 3) * Y(i);
            sum2[j] = sum2[j] + T(LU, i, 4) * Y(i);
        }
    for (int j = 0; j < nb; j++) {
        Y(n - 1) = Y(n - 1) - sum1[j];
        Y(n) = (Y(n) - sum2[j] - T(LU, n - 1, 4) * Y(n - 1)) * T(LU, n, 5);
        Y(n - 1) = (Y(n - 1) - T(LU, n - 1, 9) * Y(n)) * T(LU, n - 1, 5);
        Y(n - 2) = (Y(n - 2) - T(LU, n - 2, 8) * Y(n - 1) - T(LU, n - 2, 9) * Y(n)) * T(LU, n - 2, 5);
        Y(n - 3) = (Y(n - 3) - T(LU, n - 3, 6) * Y(n - 2) - T(LU, n - 3, 8) * Y(n - 1) - T(LU, n - 3, 9) * Y(n)) *
                   T(LU, n - 3, 5);
    }
    for (int i = n - 4; i >= 1; i--)
        for (int j = 0; j < nb; j++)
            Y(i) = (Y(i) - T(LU, i, 6) * Y(i + 1) - T(LU, i, 7) * Y(i + 2) - T(LU, i, 8) * Y(n - 1) -
                    T(LU, i, 9) * Y(n)) *
                   T(LU, i, 5);
#undef Y
}

/* index of bc in {0, 1, -1} -> 0..2, used to address the 9 precomputed factorisations */
static int bcidx(int bc) { return bc == 0 ? 0 : (bc == 1 ? 1 : 2); }
static int bc_ok(int bc) { return bc == 0 || bc == 1 || bc == -1; }

typedef struct {
    int n, periodic;
    double dx, onebydx, onebydx2;
    double *LU1, *LU2;
    double *penta1[9], *penta2[9];
} cd10_t;

/* ComputePenta1 diagonals (cd10.F90:441-556) */
static void cd10_penta1_diags(double *P, int n, int bc1, int bcn) {
    cd10_bnd_t k = cd10_bnd();
#define bt(i) T(P, i, 1)
#define b(i) T(P, i, 2)
#define d(i) T(P, i, 3)
#define a(i) T(P, i, 4)
#define at(i) T(P, i, 5)
    for (int i = 1; i <= n; i++) {
        at(i) = k.beta_hat;
        bt(i) = k.beta_hat;
        a(i) = k.alpha_hat;
        b(i) = k.alpha_hat;
        d(i) = 1.0;
    }
    if (bc1 == 0) {
        bt(1) = k.w1 * 0.0; b(1) = k.w1 * 0.0; d(1) = k.w1 * 1.0; a(1) = k.w1 * k.alpha; at(1) = k.w1 * 0.0;
        bt(2) = k.w2 * 0.0; b(2) = k.w2 * k.alpha_p; d(2) = k.w2 * 1.0; a(2) = k.w2 * k.alpha_p; at(2) = k.w2 * 0.0;
        bt(3) = k.w3 * k.beta_pp; b(3) = k.w3 * k.alpha_pp; d(3) = k.w3 * 1.0; a(3) = k.w3 * k.alpha_pp; at(3) = k.w3 * k.beta_pp;
        bt(4) = k.w4 * k.beta_ppp; b(4) = k.w4 * k.alpha_ppp; d(4) = k.w4 * 1.0; a(4) = k.w4 * k.alpha_ppp; at(4) = k.w4 * k.beta_ppp;
    } else if (bc1 == 1) {
        bt(1) = 0.0; b(1) = 0.0; d(1) = 1.0; a(1) = 0.0; at(1) = 0.0;
        bt(2) = 0.0; b(2) = k.alpha_hat; d(2) = 1.0 - k.beta_hat; a(2) = k.alpha_hat; at(2) = k.beta_hat;
    } else {
        bt(1) = 0.0; b(1) = 0.0; d(1) = 1.0; a(1) = 2.0 * k.alpha_hat; at(1) = 2.0 * k.beta_hat;
        bt(2) = 0.0; b(2) = k.alpha_hat; d(2) = 1.0 + k.beta_hat; a(2) = k.alpha_hat; at(2) = k.beta_hat;
    }
    if (bcn == 0) {
        bt(n) = k.w1 * 0.0; b(n) = k.w1 * k.alpha; d(n) = k.w1 * 1.0; a(n) = k.w1 * 0.0; at(n) = k.w1 * 0.0;
        bt(n - 1) = k.w2 * 0.0; b(n - 1) = k.w2 * k.alpha_p; d(n - 1) = k.w2 * 1.0; a(n - 1) = k.w2 * k.alpha_p; at(n - 1) = k.w2 * 0.0;
        bt(n - 2) = k.w3 * k.beta_pp; b(n - 2) = k.w3 * k.alpha_pp; d(n - 2) = k.w3 * 1.0; a(n - 2) = k.w3 * k.alpha_pp; at(n - 2) = k.w3 * k.beta_pp;
        bt(n - 3) = k.w4 * k.beta_ppp; b(n - 3) = k.w4 * k.alpha_ppp; d(n - 3) = k.w4 * 1.0; a(n - 3) = k.w4 * k.alpha_ppp; at(n - 3) = k.w4 * k.beta_ppp;
    } else if (bcn == 1) {
        bt(n) = 0.0; b(n) = 0.0; d(n) = 1.0; a(n) = 0.0; at(n) = 0.0;
        bt(n - 1) = k.beta_hat; b(n - 1) = k.alpha_hat; d(n - 1) = 1.0 - k.beta_hat; a(n - 1) = k.alpha_hat; at(n - 1) = 0.0;
    } else {
        bt(n) = 2.0 * k.beta_hat; b(n) = 2.0 * k.alpha_hat; d(n) = 1.0; a(n) = 0.0; at(n) = 0.0;
        bt(n - 1) = k.beta_hat; b(n - 1) = k.alpha_hat; d(n - 1) = 1.0 + k.beta_hat; a(n - 1) = k.alpha_hat; at(n - 1) = 0.0;
    }
#undef bt
#undef b
#undef d
#undef a
#undef at
}

/* ComputePenta2 diagonals (cd10.F90:592-686) */
static void cd10_penta2_diags(double *P, int n, int bc1, int bcn) {
    cd10_bnd_t k = cd10_bnd();
#define bt(i) T(P, i, 1)
#define b(i) T(P, i, 2)
#define d(i) T(P, i, 3)
#define a(i) T(P, i, 4)
#define at(i) T(P, i, 5)
    for (int i = 1; i <= n; i++) {
        at(i) = beta10d2;
        bt(i) = beta10d2;
        d(i) = 1.0;
        a(i) = alpha10d2;
        b(i) = alpha10d2;
    }
    if (bc1 == 0) {
        bt(1) = 0.0; b(1) = 0.0; d(1) = 1.0; a(1) = k.b1_alpha; at(1) = 0.0;
        bt(2) = 0.0; b(2) = k.b2_alpha; d(2) = 1.0; a(2) = k.b2_alpha; at(2) = 0.0;
        bt(3) = k.b3_beta; b(3) = k.b3_alpha; d(3) = 1.0; a(3) = k.b3_alpha; at(3) = k.b3_beta;
    } else if (bc1 == 1) {
        bt(1) = 0.0; b(1) = 0.0; d(1) = 1.0; a(1) = 2.0 * alpha10d2; at(1) = 2.0 * beta10d2;
        bt(2) = 0.0; b(2) = alpha10d2; d(2) = 1.0 + beta10d2; a(2) = alpha10d2; at(2) = beta10d2;
    } else {
        bt(1) = 0.0; b(1) = 0.0; d(1) = 1.0; a(1) = 0.0; at(1) = 0.0;
        bt(2) = 0.0; b(2) = alpha10d2; d(2) = 1.0 - beta10d2; a(2) = alpha10d2; at(2) = beta10d2;
    }
    if (bcn == 0) {
        bt(n - 2) = k.b3_beta; b(n - 2) = k.b3_alpha; d(n - 2) = 1.0; a(n - 2) = k.b3_alpha; at(n - 2) = k.b3_beta;
        bt(n - 1) = 0.0; b(n - 1) = k.b2_alpha; d(n - 1) = 1.0; a(n - 1) = k.b2_alpha; at(n - 1) = 0.0;
        bt(n) = 0.0; b(n) = k.b1_alpha; d(n) = 1.0; a(n) = 0.0; at(n) = 0.0;
    } else if (bcn == 1) {
        bt(n - 1) = beta10d2; b(n - 1) = alpha10d2; d(n - 1) = 1.0 + beta10d2; a(n - 1) = alpha10d2; at(n - 1) = 0.0;
        bt(n) = 2.0 * beta10d2; b(n) = 2.0 * alpha10d2; d(n) = 1.0; a(n) = 0.0; at(n) = 0.0;
    } else {
        bt(n - 1) = beta10d2; b(n - 1) = alpha10d2; d(n - 1) = 1.0 - beta10d2; a(n - 1) = alpha10d2; at(n - 1) = 0.0;
        bt(n) = 0.0; b(n) = 0.0; d(n) = 1.0; a(n) = 0.0; at(n) = 0.0;
    }
#undef bt
#undef b
#undef d
#undef a
#undef at
}

static const int BCS[3] = {0, 1, -1};

/* cd10.F90:195-315 */
static int cd10_init(cd10_t *o, int n, double dx, int periodic) {
    memset(o, 0, sizeof(*o));
    o->n = n;
    o->dx = dx;
    o->onebydx = 1.0 / dx;
    o->onebydx2 = o->onebydx / dx;
    o->periodic = periodic;
    if (n == 1) return 0;
    if (n < 8) return 2;
    if (periodic) {
        o->LU1 = malloc(sizeof(double) * 9 * n);
        o->LU2 = malloc(sizeof(double) * 9 * n);
        penta_cyclic_lu(o->LU1, n, beta10d1, alpha10d1, 1.0, alpha10d1, beta10d1);
        penta_cyclic_lu(o->LU2, n, beta10d2, alpha10d2, 1.0, alpha10d2, beta10d2);
    } else {
        for (int i1 = 0; i1 < 3; i1++)
            for (int in = 0; in < 3; in++) {
                int id = i1 * 3 + in;
                o->penta1[id] = calloc((size_t)11 * n, sizeof(double));
                o->penta2[id] = calloc((size_t)11 * n, sizeof(double));
                cd10_penta1_diags(o->penta1[id], n, BCS[i1], BCS[in]);
                penta_factor(o->penta1[id], n);
                cd10_penta2_diags(o->penta2[id], n, BCS[i1], BCS[in]);
                penta_factor(o->penta2[id], n);
            }
    }
    return 0;
}

static void cd10_free(cd10_t *o) {
    free(o->LU1);
    free(o->LU2);
    for (int i = 0; i < 9; i++) {
        free(o->penta1[i]);
        free(o->penta2[i]);
    }
}

/* Virtual index with symmetric (bc=1) / antisymmetric (bc=-1) reflection about the end
 * points, reproducing the reflected terms written out in the bc=+-1 rows of the
 * reference RHS routines (e.g. cd10.F90:1177-1206, 1666-1689; cf90.F90:691-732). */
static inline double fref(const double *f, long fs, int n, int i, int bc1, int bcn) {
    if (i < 1) {
        double v = f[(long)(2 - i - 1) * fs];
        return bc1 == -1 ? -v : v;
    }
    if (i > n) {
        double v = f[(long)(2 * n - i - 1) * fs];
        return bcn == -1 ? -v : v;
    }
    return f[(long)(i - 1) * fs];
}

/* First-derivative RHS (cd10.F90:1098-1263) */
static void cd10_rhs_d1(const cd10_t *o, const double *f, long fs, double *r, long rs, int bc1, int bcn) {
#define F(i) f[((long)(i) - 1) * fs]
#define G(i) fref(f, fs, n, (i), bc1, bcn)
#define R(i) r[((long)(i) - 1) * rs]
    const int n = o->n;
    if (o->periodic) {
        double a10 = a10d1 * o->onebydx, b10 = b10d1 * o->onebydx, c10 = c10d1 * o->onebydx;
#define P(i) F((((i) - 1 + 4 * n) % n) + 1)
        for (int i = 1; i <= n; i++)
            R(i) = a10 * (P(i + 1) - P(i - 1)) + b10 * (P(i + 2) - P(i - 2)) + c10 * (P(i + 3) - P(i - 3));
#undef P
        return;
    }
    cd10_bnd_t k = cd10_bnd();
    double a10 = k.q_hat * o->onebydx, b10 = k.r_hat * o->onebydx, c10 = k.s_hat * o->onebydx;
    double a_np_4 = k.w4 * k.q_ppp * o->onebydx, b_np_4 = k.w4 * k.r_ppp * o->onebydx, c_np_4 = k.w4 * k.s_ppp * o->onebydx;
    double a_np_3 = k.w3 * k.q_pp * o->onebydx, b_np_3 = k.w3 * k.r_pp * o->onebydx;
    double a_np_2 = k.w2 * k.q_p * o->onebydx;
    double a_np_1 = k.w1 * (k.p * o->onebydx), b_np_1 = k.w1 * (k.q * o->onebydx);
    double c_np_1 = k.w1 * (k.r * o->onebydx), d_np_1 = k.w1 * (k.s * o->onebydx);
    if (bc1 == 0) {
        R(1) = a_np_1 * F(1) + b_np_1 * F(2) + c_np_1 * F(3) + d_np_1 * F(4);
        R(2) = a_np_2 * (F(3) - F(1));
        R(3) = a_np_3 * (F(4) - F(2)) + b_np_3 * (F(5) - F(1));
        R(4) = a_np_4 * (F(5) - F(3)) + b_np_4 * (F(6) - F(2)) + c_np_4 * (F(7) - F(1));
    } else {
        for (int i = 1; i <= 4; i++)
            R(i) = a10 * (G(i + 1) - G(i - 1)) + b10 * (G(i + 2) - G(i - 2)) + c10 * (G(i + 3) - G(i - 3));
        if (bc1 == 1) R(1) = 0.0;
    }
    for (int i = 5; i <= n - 4; i++)
        R(i) = a10 * (F(i + 1) - F(i - 1)) + b10 * (F(i + 2) - F(i - 2)) + c10 * (F(i + 3) - F(i - 3));
    if (bcn == 0) {
        R(n - 3) = a_np_4 * (F(n - 2) - F(n - 4)) + b_np_4 * (F(n - 1) - F(n - 5)) + c_np_4 * (F(n) - F(n - 6));
        R(n - 2) = a_np_3 * (F(n - 1) - F(n - 3)) + b_np_3 * (F(n) - F(n - 4));
        R(n - 1) = a_np_2 * (F(n) - F(n - 2));
        R(n) = -a_np_1 * F(n) - b_np_1 * F(n - 1) - c_np_1 * F(n - 2) - d_np_1 * F(n - 3);
    } else {
        for (int i = n - 3; i <= n; i++)
            R(i) = a10 * (G(i + 1) - G(i - 1)) + b10 * (G(i + 2) - G(i - 2)) + c10 * (G(i + 3) - G(i - 3));
        if (bcn == 1) R(n) = 0.0;
    }
#undef F
#undef G
#undef R
}

/* Second-derivative RHS (cd10.F90:1587-1736) */
static void cd10_rhs_d2(const cd10_t *o, const double *f, long fs, double *r, long rs, int bc1, int bcn) {
#define F(i) f[((long)(i) - 1) * fs]
#define G(i) fref(f, fs, n, (i), bc1, bcn)
#define R(i) r[((long)(i) - 1) * rs]
    const int n = o->n;
    double a10 = a10d2 * o->onebydx2, b10 = b10d2 * o->onebydx2, c10 = c10d2 * o->onebydx2;
    if (o->periodic) {
#define P(i) F((((i) - 1 + 4 * n) % n) + 1)
        for (int i = 1; i <= n; i++)
            R(i) = a10 * (P(i + 1) - 2.0 * P(i) + P(i - 1)) + b10 * (P(i + 2) - 2.0 * P(i) + P(i - 2)) +
                   c10 * (P(i + 3) - 2.0 * P(i) + P(i - 3));
#undef P
        return;
    }
    cd10_bnd_t k = cd10_bnd();
    double a_np_3 = k.b3_a * o->onebydx2, b_np_3 = k.b3_b * o->onebydx2;
    double a_np_2 = k.b2_a * o->onebydx2;
    double a_np_1 = k.b1_a * o->onebydx2, b_np_1 = k.b1_b * o->onebydx2, c_np_1 = k.b1_c * o->onebydx2;
    double d_np_1 = k.b1_d * o->onebydx2, e_np_1 = k.b1_e * o->onebydx2;
    if (bc1 == 0) {
        R(1) = a_np_1 * F(1) + b_np_1 * F(2) + c_np_1 * F(3) + d_np_1 * F(4) + e_np_1 * F(5);
        R(2) = a_np_2 * (F(3) - 2.0 * F(2) + F(1));
        R(3) = a_np_3 * (F(4) - 2.0 * F(3) + F(2)) + b_np_3 * (F(5) - 2.0 * F(3) + F(1));
    } else {
        for (int i = 1; i <= 3; i++)
            R(i) = a10 * (G(i + 1) - 2.0 * G(i) + G(i - 1)) + b10 * (G(i + 2) - 2.0 * G(i) + G(i - 2)) +
                   c10 * (G(i + 3) - 2.0 * G(i) + G(i - 3));
    }
    for (int i = 4; i <= n - 3; i++)
        R(i) = a10 * (F(i + 1) - 2.0 * F(i) + F(i - 1)) + b10 * (F(i + 2) - 2.0 * F(i) + F(i - 2)) +
               c10 * (F(i + 3) - 2.0 * F(i) + F(i - 3));
    if (bcn == 0) {
        R(n - 2) = a_np_3 * (F(n - 1) - 2.0 * F(n - 2) + F(n - 3)) + b_np_3 * (F(n) - 2.0 * F(n - 2) + F(n - 4));
        R(n - 1) = a_np_2 * (F(n) - 2.0 * F(n - 1) + F(n - 2));
        R(n) = a_np_1 * F(n) + b_np_1 * F(n - 1) + c_np_1 * F(n - 2) + d_np_1 * F(n - 3) + e_np_1 * F(n - 4);
    } else {
        for (int i = n - 2; i <= n; i++)
            R(i) = a10 * (G(i + 1) - 2.0 * G(i) + G(i - 1)) + b10 * (G(i + 2) - 2.0 * G(i) + G(i - 2)) +
                   c10 * (G(i + 3) - 2.0 * G(i) + G(i - 3));
    }
#undef F
#undef G
#undef R
}

/* dd1..dd3 (cd10.F90:2029-2237) and d2d1..d2d3 (cd10.F90:2239-2447) on one line */
static void cd10_line(const cd10_t *o, int order, const double *f, long fs, double *df, long dfs, int bc1, int bcn) {
    if (o->n == 1) {
        df[0] = 0.0;
        return;
    }
    if (order == 1) cd10_rhs_d1(o, f, fs, df, dfs, bc1, bcn);
    else cd10_rhs_d2(o, f, fs, df, dfs, bc1, bcn);
    if (o->periodic) {
        penta_cyclic_solve(order == 1 ? o->LU1 : o->LU2, o->n, df, dfs);
    } else {
        int id = bcidx(bc1) * 3 + bcidx(bcn);
        penta_solve(order == 1 ? o->penta1[id] : o->penta2[id], o->n, df, dfs);
    }
}

/* ------------------------------------------------------------------------- */
/* cf90 (src/filters/cf90.F90) and gaussian (src/filters/gaussian.F90)          */
/* ------------------------------------------------------------------------- */

/* cf90.F90:16-48 */
static const double alpha90 = 6.6624e-1, beta90 = 1.6688e-1;
static const double a90 = 9.9965e-1, b90 = 6.6652e-1, c90 = 1.6674e-1, d90 = 4.0e-5, e90 = -5.0e-6;
static const double b2_alpha90 = 4.997e-1, b2_a90 = 9.997e-1, b2_b90 = 4.9985e-1;
static const double b3_alpha90 = 6.6624e-1, b3_beta90 = 1.6688e-1, b3_a90 = 9.9952e-1, b3_b90 = 6.6656e-1,
                    b3_c90 = 1.668e-1;
static const double b4_alpha90 = 6.6624e-1, b4_beta90 = 1.6688e-1, b4_a90 = 9.9968e-1, b4_b90 = 6.6652e-1,
                    b4_c90 = 1.6672e-1, b4_d90 = 4.0e-5;

/* gaussian.F90:16-43 */
static const double agf = 3565.0 / 10368.0, bgf = 3091.0 / 12960.0, cgf = 1997.0 / 25920.0,
                    dgf = 149.0 / 12960.0, egf = 107.0 / 103680.0;
static const double b1_agf = 5.0 / 6.0, b1_bgf = 1.0 / 6.0, b2_agf = 2.0 / 3.0, b2_bgf = 1.0 / 6.0;
static const double b3_agf = 31.0 / 64.0, b3_bgf = 7.0 / 32.0, b3_cgf = 5.0 / 128.0;
static const double b4_agf = 17.0 / 48.0, b4_bgf = 15.0 / 64.0, b4_cgf = 7.0 / 96.0, b4_dgf = 1.0 / 64.0;

/* ComputePenta diagonals (cf90.F90:288-396) */
static void cf90_penta_diags(double *P, int n, int bc1, int bcn) {
#define bt(i) T(P, i, 1)
#define b(i) T(P, i, 2)
#define d(i) T(P, i, 3)
#define a(i) T(P, i, 4)
#define at(i) T(P, i, 5)
    for (int i = 1; i <= n; i++) {
        at(i) = beta90;
        bt(i) = beta90;
        a(i) = alpha90;
        b(i) = alpha90;
        d(i) = 1.0;
    }
    if (bc1 == 0) {
        bt(1) = 0.0; b(1) = 0.0; d(1) = 1.0; a(1) = 0.0; at(1) = 0.0;
        bt(2) = 0.0; b(2) = b2_alpha90; d(2) = 1.0; a(2) = b2_alpha90; at(2) = 0.0;
        bt(3) = b3_beta90; b(3) = b3_alpha90; d(3) = 1.0; a(3) = b3_alpha90; at(3) = b3_beta90;
        bt(4) = b4_beta90; b(4) = b4_alpha90; d(4) = 1.0; a(4) = b4_alpha90; at(4) = b4_beta90;
    } else if (bc1 == 1) {
        bt(1) = 0.0; b(1) = 0.0; d(1) = 1.0; a(1) = 2.0 * alpha90; at(1) = 2.0 * beta90;
        bt(2) = 0.0; b(2) = alpha90; d(2) = 1.0 + beta90; a(2) = alpha90; at(2) = beta90;
    } else {
        bt(1) = 0.0; b(1) = 0.0; d(1) = 1.0; a(1) = 0.0; at(1) = 0.0;
        bt(2) = 0.0; b(2) = alpha90; d(2) = 1.0 - beta90; a(2) = alpha90; at(2) = beta90;
    }
    if (bcn == 0) {
        bt(n) = 0.0; b(n) = 0.0; d(n) = 1.0; a(n) = 0.0; at(n) = 0.0;
        bt(n - 1) = 0.0; b(n - 1) = b2_alpha90; d(n - 1) = 1.0; a(n - 1) = b2_alpha90; at(n - 1) = 0.0;
        bt(n - 2) = b3_beta90; b(n - 2) = b3_alpha90; d(n - 2) = 1.0; a(n - 2) = b3_alpha90; at(n - 2) = b3_beta90;
        bt(n - 3) = b4_beta90; b(n - 3) = b4_alpha90; d(n - 3) = 1.0; a(n - 3) = b4_alpha90; at(n - 3) = b4_beta90;
    } else if (bcn == 1) {
        bt(n) = 2.0 * beta90; b(n) = 2.0 * alpha90; d(n) = 1.0; a(n) = 0.0; at(n) = 0.0;
        bt(n - 1) = beta90; b(n - 1) = alpha90; d(n - 1) = 1.0 + beta90; a(n - 1) = alpha90; at(n - 1) = 0.0;
    } else {
        bt(n) = 0.0; b(n) = 0.0; d(n) = 1.0; a(n) = 0.0; at(n) = 0.0;
        bt(n - 1) = beta90; b(n - 1) = alpha90; d(n - 1) = 1.0 - beta90; a(n - 1) = alpha90; at(n - 1) = 0.0;
    }
#undef bt
#undef b
#undef d
#undef a
#undef at
}

typedef struct {
    int n, periodic;
    double *LU;
    double *penta[9];
} cf90_t;

/* cf90.F90:107-175 */
static int cf90_init(cf90_t *o, int n, int periodic) {
    memset(o, 0, sizeof(*o));
    o->n = n;
    o->periodic = periodic;
    if (n == 1) return 0;
    if (n < 10) return 7;
    if (periodic) {
        o->LU = malloc(sizeof(double) * 9 * n);
        penta_cyclic_lu(o->LU, n, beta90, alpha90, 1.0, alpha90, beta90);
    } else {
        for (int i1 = 0; i1 < 3; i1++)
            for (int in = 0; in < 3; in++) {
                int id = i1 * 3 + in;
                o->penta[id] = calloc((size_t)11 * n, sizeof(double));
                cf90_penta_diags(o->penta[id], n, BCS[i1], BCS[in]);
                penta_factor(o->penta[id], n);
            }
    }
    return 0;
}

static void cf90_free(cf90_t *o) {
    free(o->LU);
    for (int i = 0; i < 9; i++) free(o->penta[i]);
}

/* Symmetric 9-point filter row a*f(i) + sum_k c_k*(f(i+k)+f(i-k)) with virtual reflected
 * indices: the periodic, interior and bc=+-1 rows of cf90 ComputeXRHS (cf90.F90:619-797) and
 * gaussian filter1 (gaussian.F90:137-330) all have this form. */
static inline double sym9(const double *f, long fs, int n, int i, int bc1, int bcn, int periodic, double a,
                          double b, double c, double d, double e) {
#define G(j) (periodic ? f[(long)((((j) - 1) % n + n) % n) * fs] : fref(f, fs, n, (j), bc1, bcn))
    return a * (G(i)) + b * (G(i + 1) + G(i - 1)) + c * (G(i + 2) + G(i - 2)) + d * (G(i + 3) + G(i - 3)) +
           e * (G(i + 4) + G(i - 4));
#undef G
}

/* cf90 ComputeXRHS (cf90.F90:610-994) */
static void cf90_rhs(const cf90_t *o, const double *f, long fs, double *r, long rs, int bc1, int bcn) {
#define F(i) f[((long)(i) - 1) * fs]
#define R(i) r[((long)(i) - 1) * rs]
    const int n = o->n;
    if (o->periodic) {
        for (int i = 1; i <= n; i++) R(i) = sym9(f, fs, n, i, 0, 0, 1, a90, b90, c90, d90, e90);
        return;
    }
    if (bc1 == 0) {
        R(1) = 1.0 * (F(1));
        R(2) = b2_a90 * (F(2)) + b2_b90 * (F(3) + F(1));
        R(3) = b3_a90 * (F(3)) + b3_b90 * (F(4) + F(2)) + b3_c90 * (F(5) + F(1));
        R(4) = b4_a90 * (F(4)) + b4_b90 * (F(5) + F(3)) + b4_c90 * (F(6) + F(2)) + b4_d90 * (F(7) + F(1));
    } else {
        for (int i = 1; i <= 4; i++) R(i) = sym9(f, fs, n, i, bc1, bcn, 0, a90, b90, c90, d90, e90);
    }
    for (int i = 5; i <= n - 4; i++) R(i) = sym9(f, fs, n, i, bc1, bcn, 0, a90, b90, c90, d90, e90);
    if (bcn == 0) {
        R(n - 3) = b4_a90 * (F(n - 3)) + b4_b90 * (F(n - 2) + F(n - 4)) + b4_c90 * (F(n - 1) + F(n - 5)) +
                   b4_d90 * (F(n) + F(n - 6));
        R(n - 2) = b3_a90 * (F(n - 2)) + b3_b90 * (F(n - 1) + F(n - 3)) + b3_c90 * (F(n) + F(n - 4));
        R(n - 1) = b2_a90 * (F(n - 1)) + b2_b90 * (F(n) + F(n - 2));
        R(n) = 1.0 * (F(n));
    } else {
        for (int i = n - 3; i <= n; i++) R(i) = sym9(f, fs, n, i, bc1, bcn, 0, a90, b90, c90, d90, e90);
    }
#undef F
#undef R
}

/* filter1/filter2/filter3 on one line (cf90.F90:1020-1228) */
static void cf90_line(const cf90_t *o, const double *f, long fs, double *ff, long ffs, int bc1, int bcn) {
    if (o->n == 1) {
        ff[0] = f[0];
        return;
    }
    cf90_rhs(o, f, fs, ff, ffs, bc1, bcn);
    if (o->periodic) penta_cyclic_solve(o->LU, o->n, ff, ffs);
    else penta_solve(o->penta[bcidx(bc1) * 3 + bcidx(bcn)], o->n, ff, ffs);
}

/* gaussian filter1/2/3 on one line (gaussian.F90:104-334) */
static void gaussian_line(int n, int periodic, const double *f, long fs, double *g, long gs, int bc1, int bcn) {
#define F(i) f[((long)(i) - 1) * fs]
#define R(i) g[((long)(i) - 1) * gs]
    if (n == 1) {
        g[0] = f[0];
        return;
    }
    if (periodic) {
        for (int i = 1; i <= n; i++) R(i) = sym9(f, fs, n, i, 0, 0, 1, agf, bgf, cgf, dgf, egf);
        return;
    }
    if (bc1 == 0) {
        R(1) = b1_agf * (F(1)) + b1_bgf * (F(2));
        R(2) = b2_agf * (F(2)) + b2_bgf * (F(3) + F(1));
        R(3) = b3_agf * (F(3)) + b3_bgf * (F(4) + F(2)) + b3_cgf * (F(5) + F(1));
        R(4) = b4_agf * (F(4)) + b4_bgf * (F(5) + F(3)) + b4_cgf * (F(6) + F(2)) + b4_dgf * (F(7) + F(1));
    } else {
        for (int i = 1; i <= 4; i++) R(i) = sym9(f, fs, n, i, bc1, bcn, 0, agf, bgf, cgf, dgf, egf);
    }
    for (int i = 5; i <= n - 4; i++) R(i) = sym9(f, fs, n, i, bc1, bcn, 0, agf, bgf, cgf, dgf, egf);
    if (bcn == 0) {
        R(n - 3) = b4_agf * (F(n - 3)) + b4_bgf * (F(n - 2) + F(n - 4)) + b4_cgf * (F(n - 1) + F(n - 5)) +
                   b4_dgf * (F(n) + F(n - 6));
        R(n - 2) = b3_agf * (F(n - 2)) + b3_bgf * (F(n - 1) + F(n - 3)) + b3_cgf * (F(n) + F(n - 4));
        R(n - 1) = b2_agf * (F(n - 1)) + b2_bgf * (F(n) + F(n - 2));
        R(n) = b1_agf * (F(n)) + b1_bgf * (F(n - 1));
    } else {
        for (int i = n - 3; i <= n; i++) R(i) = sym9(f, fs, n, i, bc1, bcn, 0, agf, bgf, cgf, dgf, egf);
    }
#undef F
#undef R
}

/* ------------------------------------------------------------------------- */
/* cd06stagg (src/derivatives/cd06stagg.F90 + STAGG_CD06_files)                 */
/* ------------------------------------------------------------------------- */

enum { ST_D1_E2C = 0, ST_D1_C2E, ST_D1_C2C, ST_D1_E2E, ST_D2_C2C, ST_D2_E2E, ST_I_E2C, ST_I_C2E, ST_NOPS };

typedef struct {
    int n, nE, periodic, topEven, botEven, topSided, botSided;
    double dx, onebydx, onebydx2;
    double *LU_D1, *LU_D2, *LU_interp;
    double *tri[ST_NOPS];
} stagg_t;

static const double w0s = 223.0 / 186.0, w1s = 61.0 / 62.0; /* cd06stagg.F90:56 */

/* ComputeTri* routines (STAGG_CD06_files/ComputeTri_allRoutines.F90:1-366): build the
 * three diagonals for one operator, then factor with tri_factor. */
static void stagg_tri(stagg_t *o, int op) {
    cd06_bnd_t k = cd06_bnd();
    int n = (op == ST_D1_C2E || op == ST_D1_E2E || op == ST_D2_E2E || op == ST_I_C2E) ? o->nE : o->n;
    double *ddn = malloc(sizeof(double) * n), *dg = malloc(sizeof(double) * n), *dup = malloc(sizeof(double) * n);
    double alpha = 0;
    switch (op) {
    case ST_D1_E2C: case ST_D1_C2E: alpha = 9.0 / 62.0; break;
    case ST_D1_C2C: case ST_D1_E2E: alpha = 1.0 / 3.0; break;
    case ST_D2_C2C: case ST_D2_E2E: alpha = 2.0 / 11.0; break;
    default: alpha = 3.0 / 10.0; break;
    }
    for (int i = 0; i < n; i++) {
        ddn[i] = alpha;
        dg[i] = 1.0;
        dup[i] = alpha;
    }
#define DDN(i) ddn[(i) - 1]
#define DG(i) dg[(i) - 1]
#define DUP(i) dup[(i) - 1]
    if (op == ST_D1_E2C) { /* 1-47 */
        const double alpha1 = 37.0 / 183.0, alpha0 = -1.0;
        if (o->topSided) {
            DDN(n) = w0s * alpha0; DG(n) = w0s;
            DDN(n - 1) = w1s * alpha1; DUP(n - 1) = w1s * alpha1; DG(n - 1) = w1s;
        } else if (o->topEven) {
            DUP(n) = 0.0; DG(n) = (1.0 - alpha);
        } else {
            DG(n) = (1.0 + alpha); DUP(n) = 0.0;
        }
        if (o->botSided) {
            DUP(1) = w0s * alpha0; DG(1) = w0s;
            DDN(2) = w1s * alpha1; DUP(2) = w1s * alpha1; DG(2) = w1s;
        } else if (o->botEven) {
            DDN(1) = 0.0; DG(1) = (1.0 - alpha);
        } else {
            DDN(1) = 0.0; DG(1) = (1.0 + alpha);
        }
    } else if (op == ST_D1_C2E) { /* 49-94 */
        if (o->topSided) {
            DDN(n) = 0.0; DUP(n) = 0.0;
            DDN(n - 1) = 1.0 / 22.0; DUP(n - 1) = 1.0 / 22.0;
        } else if (o->topEven) {
            DUP(n) = 0.0; DDN(n) = 0.0;
        } else {
            DDN(n) = 2.0 * alpha; DUP(n) = 0.0;
        }
        if (o->botSided) {
            DUP(1) = 0.0; DDN(1) = 0.0;
            DUP(2) = 1.0 / 22.0; DDN(2) = 1.0 / 22.0;
        } else if (o->botEven) {
            DDN(1) = 0.0; DUP(1) = 0.0;
        } else {
            DDN(1) = 0.0; DUP(1) = 2.0 * alpha;
        }
    } else if (op == ST_D1_C2C) { /* 96-160 */
        const double alphaLOW = 3.0;
        if (o->topSided) {
            DUP(n) = k.w1 * 0.0; DUP(n - 1) = k.w2 * k.alpha_p; DUP(n - 2) = k.w3 * k.alpha_pp;
            DG(n) = k.w1 * 1.0; DG(n - 1) = k.w2 * 1.0; DG(n - 2) = k.w3 * 1.0;
            DDN(n) = k.w1 * alphaLOW; DDN(n - 1) = k.w2 * k.alpha_p; DDN(n - 2) = k.w3 * k.alpha_pp;
        } else if (o->topEven) {
            DG(n) = (1.0 - alpha);
        } else {
            DG(n) = (1.0 + alpha);
        }
        if (o->botSided) {
            DDN(1) = k.w1 * 0.0; DDN(2) = k.w2 * k.alpha_p; DDN(3) = k.w3 * k.alpha_pp;
            DG(1) = k.w1 * 1.0; DG(2) = k.w2 * 1.0; DG(3) = k.w3 * 1.0;
            DUP(1) = k.w1 * alphaLOW; DUP(2) = k.w2 * k.alpha_p; DUP(3) = k.w3 * k.alpha_pp;
        } else if (o->botEven) {
            DG(1) = (1.0 - alpha);
        } else {
            DG(1) = (1.0 + alpha);
        }
    } else if (op == ST_D1_E2E) { /* 162-197 */
        if (o->topEven) { DG(n) = 1.0; DDN(n) = 0.0; }
        else { DG(n) = 1.0; DDN(n) = 2.0 * alpha; }
        if (o->botEven) { DG(1) = 1.0; DUP(1) = 0.0; }
        else { DG(1) = 1.0; DUP(1) = 2.0 * alpha; }
    } else if (op == ST_I_C2E) { /* 199-244 */
        const double alpha1 = 1.0 / 6.0;
        if (o->topSided) {
            DUP(n) = 0.0; DDN(n) = 0.0;
            DUP(n - 1) = alpha1; DDN(n - 1) = alpha1;
        } else if (o->topEven) {
            DDN(n) = 2.0 * alpha; DG(n) = 1.0;
        } else {
            DDN(n) = 0.0; DG(n) = 1.0;
        }
        if (o->botSided) {
            DUP(1) = 0.0; DDN(1) = 0.0; DG(1) = 1.0;
            DUP(2) = alpha1; DDN(2) = alpha1; DG(2) = 1.0;
        } else if (o->botEven) {
            DUP(1) = 2.0 * alpha; DG(1) = 1.0;
        } else {
            DUP(1) = 0.0; DG(1) = 1.0;
        }
    } else if (op == ST_I_E2C) { /* 247-291 */
        const double alpha0 = 1.0;
        if (o->topSided) {
            DDN(n) = alpha0; DUP(n) = 0.0;
        } else if (o->topEven) {
            DG(n) = (1.0 + alpha);
        } else {
            DG(n) = (1.0 - alpha);
        }
        if (o->botSided) {
            DUP(1) = alpha0; DDN(1) = 0.0;
        } else if (o->botEven) {
            DG(1) = (1.0 + alpha);
        } else {
            DG(1) = (1.0 - alpha);
        }
    } else if (op == ST_D2_E2E) { /* 294-329 */
        if (o->topEven) { DG(n) = 1.0; DDN(n) = 2.0 * alpha; }
        else { DG(n) = 1.0; DDN(n) = 0.0; }
        if (o->botEven) { DG(1) = 1.0; DUP(1) = 2.0 * alpha; }
        else { DG(1) = 1.0; DUP(1) = 0.0; }
    } else { /* ST_D2_C2C 331-366 */
        if (o->topEven) DG(n) = 1.0 + alpha;
        else DG(n) = 1.0 - alpha;
        if (o->botEven) DG(1) = 1.0 + alpha;
        else DG(1) = 1.0 - alpha;
    }
#undef DDN
#undef DG
#undef DUP
    o->tri[op] = malloc(sizeof(double) * 3 * n);
    tri_factor(o->tri[op], n, ddn, dg, dup);
    free(ddn);
    free(dg);
    free(dup);
}

/* init_periodic (cd06stagg.F90:170-195) and init_nonperiodic (197-232) */
static int stagg_init(stagg_t *o, int n, double dx, int periodic, int topEven, int botEven, int topSided,
                      int botSided) {
    memset(o, 0, sizeof(*o));
    o->n = n;
    o->nE = n + 1;
    o->dx = dx;
    o->onebydx = 1.0 / dx;
    o->onebydx2 = o->onebydx / dx;
    o->periodic = periodic;
    o->topEven = topEven;
    o->botEven = botEven;
    o->topSided = topSided;
    o->botSided = botSided;
    if (n <= 4) return 21; /* GracefulExit("CD06_stagg requires at least 4 points",21) */
    if (periodic) {
        o->LU_D1 = malloc(sizeof(double) * 5 * n);
        o->LU_D2 = malloc(sizeof(double) * 5 * n);
        o->LU_interp = malloc(sizeof(double) * 5 * n);
        tri_cyclic_lu(o->LU_D1, n, 9.0 / 62.0, 1.0, 9.0 / 62.0);
        tri_cyclic_lu(o->LU_D2, n, 2.0 / 11.0, 1.0, 2.0 / 11.0);
        tri_cyclic_lu(o->LU_interp, n, 3.0 / 10.0, 1.0, 3.0 / 10.0);
    } else {
        for (int op = 0; op < ST_NOPS; op++) stagg_tri(o, op);
    }
    return 0;
}

static void stagg_free(stagg_t *o) {
    free(o->LU_D1);
    free(o->LU_D2);
    free(o->LU_interp);
    for (int i = 0; i < ST_NOPS; i++) free(o->tri[i]);
}

static int stagg_in_len(const stagg_t *o, int op) {
    return (op == ST_D1_E2C || op == ST_D1_E2E || op == ST_D2_E2E || op == ST_I_E2C) ? o->nE : o->n;
}
static int stagg_out_len(const stagg_t *o, int op) {
    return (op == ST_D1_C2E || op == ST_D1_E2E || op == ST_D2_E2E || op == ST_I_C2E) ? o->nE : o->n;
}

/* Periodic RHS routines (cd06stagg.F90:301-629).  Input f has the length the Fortran
 * dummy declares (nE for E-grid inputs: the n+1-th edge value is read as given). */
static void stagg_rhs_periodic(const stagg_t *o, int op, const double *f, long fs, double *r, long rs) {
#define F(i) f[((long)(i) - 1) * fs]
#define R(i) r[((long)(i) - 1) * rs]
    const int n = o->n;
    if (op == ST_D1_E2C || op == ST_I_E2C) { /* 301-322, 526-547 */
        double a06, b06;
        if (op == ST_D1_E2C) {
            a06 = (63.0 / 62.0) * o->onebydx;
            b06 = ((17.0 / 62.0) / 3.0) * o->onebydx;
            R(1) = a06 * (F(2) - F(1)) + b06 * (F(3) - F(n));
            for (int i = 2; i <= n - 1; i++) R(i) = a06 * (F(i + 1) - F(i)) + b06 * (F(i + 2) - F(i - 1));
            R(n) = a06 * (F(n + 1) - F(n)) + b06 * (F(2) - F(n - 1));
        } else {
            a06 = (3.0 / 2.0) * (1.0 / 2.0);
            b06 = (1.0 / 10.0) * (1.0 / 2.0);
            R(1) = a06 * (F(2) + F(1)) + b06 * (F(3) + F(n));
            for (int i = 2; i <= n - 1; i++) R(i) = a06 * (F(i + 1) + F(i)) + b06 * (F(i + 2) + F(i - 1));
            R(n) = a06 * (F(n + 1) + F(n)) + b06 * (F(2) + F(n - 1));
        }
    } else if (op == ST_D1_C2E || op == ST_I_C2E) { /* 349-375, 573-600 */
        double a06, b06;
        int sgn;
        if (op == ST_D1_C2E) {
            a06 = (63.0 / 62.0) * o->onebydx;
            b06 = ((17.0 / 62.0) / 3.0) * o->onebydx;
            sgn = -1;
        } else {
            a06 = (3.0 / 2.0) * (1.0 / 2.0);
            b06 = (1.0 / 10.0) * (1.0 / 2.0);
            sgn = 1;
        }
#define C(x, y) (sgn < 0 ? ((x) - (y)) : ((x) + (y)))
        R(1) = a06 * C(F(1), F(n)) + b06 * C(F(2), F(n - 1));
        R(2) = a06 * C(F(2), F(1)) + b06 * C(F(3), F(n));
        for (int i = 3; i <= n - 1; i++) R(i) = a06 * C(F(i), F(i - 1)) + b06 * C(F(i + 1), F(i - 2));
        R(n) = a06 * C(F(n), F(n - 1)) + b06 * C(F(1), F(n - 2));
        R(n + 1) = a06 * C(F(1), F(n)) + b06 * C(F(2), F(n - 1));
#undef C
    } else { /* D2 C2C 405-432, D2 E2E 465-495 */
        double a06 = (12.0 / 11.0) * (o->onebydx * o->onebydx);
        double b06 = ((3.0 / 11.0) / 4.0) * (o->onebydx * o->onebydx);
        R(1) = a06 * (F(2) - 2.0 * F(1) + F(n)) + b06 * (F(3) - 2.0 * F(1) + F(n - 1));
        R(2) = a06 * (F(3) - 2.0 * F(2) + F(1)) + b06 * (F(4) - 2.0 * F(2) + F(n));
        for (int i = 3; i <= n - 2; i++)
            R(i) = a06 * (F(i + 1) - 2.0 * F(i) + F(i - 1)) + b06 * (F(i + 2) - 2.0 * F(i) + F(i - 2));
        R(n - 1) = a06 * (F(n) - 2.0 * F(n - 1) + F(n - 2)) + b06 * (F(1) - 2.0 * F(n - 1) + F(n - 3));
        R(n) = a06 * (F(1) - 2.0 * F(n) + F(n - 1)) + b06 * (F(2) - 2.0 * F(n) + F(n - 2));
        if (op == ST_D2_E2E)
            R(n + 1) = a06 * (F(2) - 2.0 * F(n + 1) + F(n)) + b06 * (F(3) - 2.0 * F(n + 1) + F(n - 1));
    }
#undef F
#undef R
}

/* Non-periodic RHS include files (STAGG_CD06_files/D1RHS_*, D2RHS_*, InterpRHS_*) */
static void stagg_rhs_nonperiodic(const stagg_t *o, int op, const double *f, long fs, double *r, long rs) {
#define F(i) f[((long)(i) - 1) * fs]
#define R(i) r[((long)(i) - 1) * rs]
    const int n = o->n, nE = o->nE;
    const double dxi = o->onebydx;
    if (op == ST_D1_E2C) { /* D1RHS_E2C_common.F90 */
        const double a = (63.0 / 62.0) / 1.0, b = (17.0 / 62.0) / 3.0;
        const double alpha1 = 37.0 / 183.0, alpha0 = -1.0;
        const double a0 = (1.0 / 24.0) * (alpha0 - 23.0), b0 = (1.0 / 8.0) * (-9.0 * alpha0 + 7.0);
        const double c0 = (1.0 / 8.0) * (9.0 * alpha0 + 1.0), d0 = -(1.0 / 24.0) * (alpha0 + 1.0);
        const double a1 = (3.0 / 8.0) * (3.0 - 2.0 * alpha1), b1 = (1.0 / 8.0) * (-1.0 + 22.0 * alpha1);
        double a06 = a * dxi, b06 = b * dxi;
        for (int i = 2; i <= n - 1; i++) R(i) = b06 * (F(i + 2) - F(i - 1)) + a06 * (F(i + 1) - F(i));
        if (o->botSided) {
            R(1) = w0s * dxi * (a0 * F(1) + b0 * F(2) + c0 * F(3) + d0 * F(4));
            R(2) = w1s * dxi * ((-b1 / 3.0) * F(1) + (-a1) * F(2) + (a1)*F(3) + (b1 / 3.0) * F(4));
        } else if (o->botEven) {
            R(1) = b06 * (F(3) - F(2)) + a06 * (F(2) - F(1));
        } else {
            R(1) = b06 * (F(3) + F(2)) + a06 * (F(2) - F(1));
        }
        if (o->topSided) {
            R(n) = -w0s * dxi * (a0 * F(nE) + b0 * F(nE - 1) + c0 * F(nE - 2) + d0 * F(nE - 3));
            R(n - 1) = w1s * dxi * ((-b1 / 3.0) * F(nE - 3) + (-a1) * F(nE - 2) + (a1)*F(nE - 1) + (b1 / 3.0) * F(nE));
        } else if (o->topEven) {
            R(n) = b06 * (F(nE - 1) - F(nE - 2)) + a06 * (F(nE) - F(nE - 1));
        } else {
            R(n) = -b06 * (F(nE - 1) + F(nE - 2)) + a06 * (F(nE) - F(nE - 1));
        }
    } else if (op == ST_D1_C2E) { /* D1RHS_C2E_common.F90 */
        const double a = (63.0 / 62.0) / 1.0, b = (17.0 / 62.0) / 3.0;
        const double a0 = -71.0 / 24.0, b0 = 47.0 / 8.0, c0 = -31.0 / 8.0, d0 = 23.0 / 24.0, a1 = 12.0 / 11.0;
        double a06 = a * dxi, b06 = b * dxi;
        for (int i = 2; i <= nE - 1; i++) R(i) = a06 * (F(i) - F(i - 1));
        for (int i = 3; i <= nE - 2; i++) R(i) = R(i) + b06 * (F(i + 1) - F(i - 2));
        if (o->botSided) {
            R(1) = (a0 * F(1) + b0 * F(2) + c0 * F(3) + d0 * F(4)) * dxi;
            R(2) = (F(2) - F(1)) * (a1 * dxi);
        } else if (o->botEven) {
            R(1) = 0.0;
            R(2) = R(2) + b06 * (F(3) - F(1));
        } else {
            R(1) = 2.0 * b06 * F(2) + 2.0 * a06 * F(1);
            R(2) = R(2) + b06 * (F(3) + F(1));
        }
        if (o->topSided) {
            R(nE - 1) = (F(n) - F(n - 1)) * (a1 * dxi);
            R(nE) = (a0 * F(n) + b0 * F(n - 1) + c0 * F(n - 2) + d0 * F(n - 3)) * (-dxi);
        } else if (o->topEven) {
            R(nE - 1) = R(nE - 1) + b06 * (F(n) - F(n - 2));
            R(nE) = 0.0;
        } else {
            R(nE - 1) = R(nE - 1) - b06 * (F(n) + F(n - 2));
            R(nE) = -2.0 * b06 * (F(n - 1)) - 2.0 * a06 * (F(n));
        }
    } else if (op == ST_D1_C2C) { /* D1RHS_C2C_common.F90 */
        cd06_bnd_t k = cd06_bnd();
        double a06 = ((14.0 / 9.0) / 2.0) * dxi, b06 = ((1.0 / 9.0) / 4.0) * dxi;
        double a_np_3 = k.w3 * k.q_pp * dxi, b_np_3 = k.w3 * k.r_pp * dxi, a_np_2 = k.w2 * k.q_p * dxi;
        double a_np_1 = k.w1 * (-k.p * dxi), b_np_1 = k.w1 * (k.q * dxi), c_np_1 = k.w1 * (k.r * dxi),
               d_np_1 = k.w1 * (k.s * dxi);
        if (o->botSided) {
            R(1) = a_np_1 * F(1) + b_np_1 * F(2) + c_np_1 * F(3) + d_np_1 * F(4);
            R(2) = a_np_2 * (F(3) - F(1));
            R(3) = a_np_3 * (F(4) - F(2)) + b_np_3 * (F(5) - F(1));
        } else if (o->botEven) {
            R(1) = b06 * (F(3) - F(2)) + a06 * (F(2) - F(1));
            R(2) = b06 * (F(4) - F(1)) + a06 * (F(3) - F(1));
            R(3) = b06 * (F(5) - F(1)) + a06 * (F(4) - F(2));
        } else {
            R(1) = b06 * (F(3) + F(2)) + a06 * (F(2) + F(1));
            R(2) = b06 * (F(4) + F(1)) + a06 * (F(3) - F(1));
            R(3) = b06 * (F(5) - F(1)) + a06 * (F(4) - F(2));
        }
        for (int i = 4; i <= n - 3; i++) R(i) = b06 * (F(i + 2) - F(i - 2)) + a06 * (F(i + 1) - F(i - 1));
        if (o->topSided) {
            R(n - 2) = a_np_3 * (F(n - 1) - F(n - 3)) + b_np_3 * (F(n) - F(n - 4));
            R(n - 1) = a_np_2 * (F(n) - F(n - 2));
            R(n) = -a_np_1 * F(n) - b_np_1 * F(n - 1) - c_np_1 * F(n - 2) - d_np_1 * F(n - 3);
        } else if (o->topEven) {
            R(n - 2) = b06 * (F(n) - F(n - 4)) + a06 * (F(n - 1) - F(n - 3));
            R(n - 1) = b06 * (F(n) - F(n - 3)) + a06 * (F(n) - F(n - 2));
            R(n) = b06 * (F(n - 1) - F(n - 2)) + a06 * (F(n) - F(n - 1));
        } else {
            R(n - 2) = b06 * (F(n) - F(n - 4)) + a06 * (F(n - 1) - F(n - 3));
            R(n - 1) = -b06 * (F(n) + F(n - 3)) + a06 * (F(n) - F(n - 2));
            R(n) = -b06 * (F(n - 1) + F(n - 2)) - a06 * (F(n) + F(n - 1));
        }
    } else if (op == ST_D1_E2E) { /* D1RHS_E2E_common.F90 */
        double a06 = ((14.0 / 9.0) / 2.0) * dxi, b06 = ((1.0 / 9.0) / 4.0) * dxi;
        for (int i = 2; i <= nE - 1; i++) R(i) = a06 * (F(i + 1) - F(i - 1));
        for (int i = 3; i <= nE - 2; i++) R(i) = R(i) + b06 * (F(i + 2) - F(i - 2));
        if (o->botEven) {
            R(1) = 0;
            R(2) = R(2) + b06 * (F(4) - F(2));
        } else {
            R(1) = b06 * (F(3) + F(3)) + a06 * (F(2) + F(2));
            R(2) = R(2) + b06 * (F(4) + F(2));
        }
        if (o->topEven) {
            R(nE) = 0;
            R(nE - 1) = R(nE - 1) + b06 * (F(nE - 1) - F(nE - 3));
        } else {
            R(nE) = -b06 * (F(nE - 2) + F(nE - 2)) - a06 * (F(nE - 1) + F(nE - 1));
            R(nE - 1) = R(nE - 1) - b06 * (F(nE - 1) + F(nE - 3));
        }
    } else if (op == ST_D2_C2C || op == ST_D2_E2E) { /* D2RHS_C2C_common.F90, D2RHS_E2E_common.F90 */
        double a06 = (12.0 / 11.0) * o->onebydx2, b06 = ((3.0 / 11.0) / 4.0) * o->onebydx2;
        int m = (op == ST_D2_C2C) ? n : nE;
        for (int i = 2; i <= m - 1; i++) R(i) = a06 * (F(i + 1) + F(i - 1));
        for (int i = 3; i <= m - 2; i++) R(i) = R(i) + b06 * (F(i + 2) + F(i - 2));
        if (op == ST_D2_C2C) {
            if (o->botEven) {
                R(1) = b06 * (F(3) + F(2)) + a06 * (F(2) + F(1));
                R(2) = R(2) + b06 * (F(4) + F(1));
            } else {
                R(1) = b06 * (F(3) - F(2)) + a06 * (F(2) - F(1));
                R(2) = R(2) + b06 * (F(4) - F(1));
            }
            if (o->topEven) {
                R(n) = b06 * (F(n - 1) + F(n - 2)) + a06 * (F(n) + F(n - 1));
                R(n - 1) = R(n - 1) + b06 * (F(n) + F(n - 3));
            } else {
                R(n) = b06 * (-F(n - 1) + F(n - 2)) + a06 * (-F(n) + F(n - 1));
                R(n - 1) = R(n - 1) + b06 * (-F(n) + F(n - 3));
            }
        } else {
            if (o->botEven) {
                R(1) = b06 * (F(3) + F(3)) + a06 * (F(2) + F(2));
                R(2) = R(2) + b06 * (F(4) + F(2));
            } else {
                R(1) = 0.0;
                R(2) = R(2) + b06 * (F(4) - F(2));
            }
            if (o->topEven) {
                R(nE) = 2.0 * b06 * F(nE - 2) + 2.0 * a06 * F(nE - 1);
                R(nE - 1) = R(nE - 1) + b06 * (F(nE - 1) + F(nE - 3));
            } else {
                R(nE) = 0.0;
                R(nE - 1) = R(nE - 1) + b06 * (-F(nE - 1) + F(nE - 3));
            }
        }
        for (int i = 1; i <= m; i++) R(i) = R(i) - 2.0 * (b06 + a06) * F(i);
    } else if (op == ST_I_C2E) { /* InterpRHS_C2E_common.F90 */
        const double b = (1.0 / 10.0) / 2.0, a = (3.0 / 2.0) / 2.0;
        const double a0 = 15.0 / 8.0, b0 = -5.0 / 4.0, c0 = 3.0 / 8.0;
        const double alpha1 = 1.0 / 6.0, a1 = (1.0 / 8.0) * (9.0 + 10.0 * alpha1);
        for (int i = 2; i <= nE - 1; i++) R(i) = (a) * (F(i) + F(i - 1));
        for (int i = 3; i <= nE - 2; i++) R(i) = R(i) + (b) * (F(i + 1) + F(i - 2));
        if (o->botSided) {
            R(1) = a0 * F(1) + b0 * F(2) + c0 * F(3);
            R(2) = (a1 / 2.0) * (F(2) + F(1));
        } else if (o->botEven) {
            R(1) = 2.0 * b * F(2) + 2.0 * a * F(1);
            R(2) = R(2) + (b) * (F(3) + F(1));
        } else {
            R(1) = 0.0;
            R(2) = R(2) + (b) * (F(3) - F(1));
        }
        if (o->topSided) {
            R(nE) = a0 * F(n) + b0 * F(n - 1) + c0 * F(n - 2);
            R(nE - 1) = (a1 / 2.0) * (F(n) + F(n - 1));
        } else if (o->topEven) {
            R(nE) = 2.0 * b * F(n - 1) + 2.0 * a * F(n);
            R(nE - 1) = R(nE - 1) + (b) * (F(n) + F(n - 2));
        } else {
            R(nE) = 0.0;
            R(nE - 1) = R(nE - 1) + (b) * (-F(n) + F(n - 2));
        }
    } else { /* ST_I_E2C: InterpRHS_E2C_common.F90 */
        const double b = (1.0 / 10.0) / 2.0, a = (3.0 / 2.0) / 2.0;
        const double alpha0 = 1.0;
        const double a0 = (1.0 / 16.0) * (5.0 - alpha0), b0 = (1.0 / 16.0) * (9.0 * alpha0 + 15.0);
        const double c0 = (1.0 / 16.0) * (9.0 * alpha0 - 5.0), d0 = (1.0 / 16.0) * (1.0 - alpha0);
        if (o->botSided) R(1) = a0 * F(1) + b0 * F(2) + c0 * F(3) + d0 * F(4);
        else if (o->botEven) R(1) = (b) * (F(3) + F(2)) + (a) * (F(2) + F(1));
        else R(1) = (b) * (F(3) - F(2)) + (a) * (F(2) + F(1));
        for (int i = 2; i <= n - 1; i++) R(i) = (b) * (F(i + 2) + F(i - 1)) + (a) * (F(i + 1) + F(i));
        if (o->topSided) R(n) = a0 * F(nE) + b0 * F(nE - 1) + c0 * F(nE - 2) + d0 * F(nE - 3);
        else if (o->topEven) R(n) = (b) * (F(nE - 1) + F(nE - 2)) + (a) * (F(nE) + F(nE - 1));
        else R(n) = (b) * (-F(nE - 1) + F(nE - 2)) + (a) * (F(nE) + F(nE - 1));
    }
#undef F
#undef R
}

/* ddz_* / InterpZ_* / d2dz2_* on one line (cd06stagg.F90:820-1059) */
static void stagg_line(const stagg_t *o, int op, const double *f, long fs, double *df, long dfs) {
    const int n = o->n;
    if (o->periodic) {
        stagg_rhs_periodic(o, op, f, fs, df, dfs);
        const double *LU = (op == ST_D1_E2C || op == ST_D1_C2E || op == ST_D1_C2C || op == ST_D1_E2E)
                               ? o->LU_D1
                               : ((op == ST_D2_C2C || op == ST_D2_E2E) ? o->LU_D2 : o->LU_interp);
        tri_cyclic_solve(LU, n, df, dfs);
        if (stagg_out_len(o, op) == o->nE) df[(long)n * dfs] = df[0];
    } else {
        stagg_rhs_nonperiodic(o, op, f, fs, df, dfs);
        tri_solve(o->tri[op], stagg_out_len(o, op), df, dfs);
    }
}

/* ------------------------------------------------------------------------- */
/* 3-D drivers exported for ctypes                                             */
/* ------------------------------------------------------------------------- */

/* Line addressing for a column-major (n1,n2,n3) array along direction dir (1,2,3).
 * len is the line length of that array; returns the number of lines. */
static long lines_of(int dir, int n1, int n2, int n3, long *pstride, long *la_n, long *la_s, long *lb_s) {
    if (dir == 1) { *pstride = 1; *la_n = n2; *la_s = n1; *lb_s = (long)n1 * n2; return (long)n2 * n3; }
    if (dir == 2) { *pstride = n1; *la_n = n1; *la_s = 1; *lb_s = (long)n1 * n2; return (long)n1 * n3; }
    *pstride = (long)n1 * n2; *la_n = n1; *la_s = 1; *lb_s = n1; return (long)n1 * n2;
}

typedef void (*line_fn)(const void *ctx, const double *f, long fs, double *g, long gs);

/* Apply a line routine to every line of f (shape sin) producing g (shape sout); the two
 * shapes differ only along dir. */
static void for_lines(int dir, const int *sin, const int *sout, const double *f, double *g, line_fn fn,
                      const void *ctx) {
    long fps, las, lbs, gps, glas, glbs, fla_n, gla_n;
    long nl = lines_of(dir, sin[0], sin[1], sin[2], &fps, &fla_n, &las, &lbs);
    lines_of(dir, sout[0], sout[1], sout[2], &gps, &gla_n, &glas, &glbs);
    /* lines are independent: threads over lines mirror the reference's pencil ranks */
#pragma omp parallel for schedule(static)
    for (long l = 0; l < nl; l++) {
        long a = l % fla_n, b = l / fla_n;
        fn(ctx, f + a * las + b * lbs, fps, g + a * glas + b * glbs, gps);
    }
}

/* Blocks of nb lines that are consecutive in memory (y and z lines: consecutive x), for the
 * blocked solves: right-hand sides line by line (the block's rows stay in cache), then one
 * solve over the whole block. */
typedef void (*block_fn)(const void *ctx, const double *f, long fs, double *g, long gs, int nb);

static void for_line_blocks(int dir, const int *s, const double *f, double *g, block_fn fn, const void *ctx) {
    long fps, las, lbs, fla_n;
    long nl = lines_of(dir, s[0], s[1], s[2], &fps, &fla_n, &las, &lbs);
    if (nl <= 0 || fla_n <= 0) return;
    const long nbpa = (fla_n + ORACLE_BLOCK - 1) / ORACLE_BLOCK, nblk = nbpa * (nl / fla_n);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < nblk; k++) {
        const long b = k / nbpa, a0 = (k % nbpa) * ORACLE_BLOCK;
        const int nb = (int)(fla_n - a0 < ORACLE_BLOCK ? fla_n - a0 : ORACLE_BLOCK);
        fn(ctx, f + a0 * las + b * lbs, fps, g + a0 * las + b * lbs, fps, nb);
    }
}

typedef struct { const cd06_t *o; int order; } cd06_ctx;
static void cd06_fn(const void *c, const double *f, long fs, double *g, long gs) {
    const cd06_ctx *x = c;
    if (x->order == 1) cd06_d1_line(x->o, f, fs, g, gs);
    else cd06_d2_line(x->o, f, fs, g, gs);
}

/* returns 0, the reference's init ierr, or 99 for an unsupported combination */
ORACLE_API int oracle_cd06(int n, double dx, int periodic, int bc1, int bcn, int order, int dir, const double *f,
                           double *df, int n1, int n2, int n3) {
    cd06_t o;
    int ierr = cd06_init(&o, n, dx, periodic, bc1, bcn);
    if (ierr) { cd06_free(&o); return ierr; }
    if (order == 2 && !periodic && n != 1) { cd06_free(&o); return 99; }
    int s[3] = {n1, n2, n3};
    cd06_ctx c = {&o, order};
    for_lines(dir, s, s, f, df, cd06_fn, &c);
    cd06_free(&o);
    return 0;
}

typedef struct { const cd10_t *o; int order, bc1, bcn; } cd10_ctx;
static void cd10_fn(const void *c, const double *f, long fs, double *g, long gs) {
    const cd10_ctx *x = c;
    cd10_line(x->o, x->order, f, fs, g, gs, x->bc1, x->bcn);
}

/* cd10 on a block of nb consecutive lines (y, z): the reference's SolveY* / SolveZ* shape */
static void cd10_blk_fn(const void *c, const double *f, long fs, double *g, long gs, int nb) {
    const cd10_ctx *x = c;
    const cd10_t *o = x->o;
    if (o->n == 1) {
        for (int j = 0; j < nb; j++) g[j] = 0.0;
        return;
    }
    for (int j = 0; j < nb; j++) {
        if (x->order == 1) cd10_rhs_d1(o, f + j, fs, g + j, gs, x->bc1, x->bcn);
        else cd10_rhs_d2(o, f + j, fs, g + j, gs, x->bc1, x->bcn);
    }
    if (o->periodic) {
        penta_cyclic_solve_blk(x->order == 1 ? o->LU1 : o->LU2, o->n, g, gs, nb);
    } else {
        const int id = bcidx(x->bc1) * 3 + bcidx(x->bcn);
        penta_solve_blk(x->order == 1 ? o->penta1[id] : o->penta2[id], o->n, g, gs, nb);
    }
}

ORACLE_API int oracle_cd10(int n, double dx, int periodic, int bc1, int bcn, int order, int dir, const double *f,
                           double *df, int n1, int n2, int n3) {
    if (!bc_ok(bc1) || !bc_ok(bcn)) return 324;
    cd10_t o;
    int ierr = cd10_init(&o, n, dx, periodic);
    if (ierr) { cd10_free(&o); return ierr; }
    int s[3] = {n1, n2, n3};
    cd10_ctx c = {&o, order, bc1, bcn};
    if (dir == 1) for_lines(dir, s, s, f, df, cd10_fn, &c);
    else for_line_blocks(dir, s, f, df, cd10_blk_fn, &c);
    cd10_free(&o);
    return 0;
}

typedef struct { const cf90_t *o; int bc1, bcn; } cf90_ctx;
static void cf90_fn(const void *c, const double *f, long fs, double *g, long gs) {
    const cf90_ctx *x = c;
    cf90_line(x->o, f, fs, g, gs, x->bc1, x->bcn);
}

/* cf90 on a block of nb consecutive lines (y, z) */
static void cf90_blk_fn(const void *c, const double *f, long fs, double *g, long gs, int nb) {
    const cf90_ctx *x = c;
    const cf90_t *o = x->o;
    if (o->n == 1) {
        for (int j = 0; j < nb; j++) g[j] = f[j];
        return;
    }
    for (int j = 0; j < nb; j++) cf90_rhs(o, f + j, fs, g + j, gs, x->bc1, x->bcn);
    if (o->periodic) penta_cyclic_solve_blk(o->LU, o->n, g, gs, nb);
    else penta_solve_blk(o->penta[bcidx(x->bc1) * 3 + bcidx(x->bcn)], o->n, g, gs, nb);
}

ORACLE_API int oracle_cf90(int n, int periodic, int bc1, int bcn, int dir, const double *f, double *ff, int n1,
                           int n2, int n3) {
    if (!bc_ok(bc1) || !bc_ok(bcn)) return 324;
    cf90_t o;
    int ierr = cf90_init(&o, n, periodic);
    if (ierr) { cf90_free(&o); return ierr; }
    int s[3] = {n1, n2, n3};
    cf90_ctx c = {&o, bc1, bcn};
    if (dir == 1) for_lines(dir, s, s, f, ff, cf90_fn, &c);
    else for_line_blocks(dir, s, f, ff, cf90_blk_fn, &c);
    cf90_free(&o);
    return 0;
}

typedef struct { int n, periodic, bc1, bcn; } gauss_ctx;
static void gauss_fn(const void *c, const double *f, long fs, double *g, long gs) {
    const gauss_ctx *x = c;
    gaussian_line(x->n, x->periodic, f, fs, g, gs, x->bc1, x->bcn);
}

ORACLE_API int oracle_gaussian(int n, int periodic, int bc1, int bcn, int dir, const double *f, double *g,
                               int n1, int n2, int n3) {
    if (!bc_ok(bc1) || !bc_ok(bcn)) return 324;
    int s[3] = {n1, n2, n3};
    gauss_ctx c = {n, periodic, bc1, bcn};
    for_lines(dir, s, s, f, g, gauss_fn, &c);
    return 0;
}

typedef struct { const stagg_t *o; int op; } stagg_ctx;
static void stagg_fn(const void *c, const double *f, long fs, double *g, long gs) {
    const stagg_ctx *x = c;
    stagg_line(x->o, x->op, f, fs, g, gs);
}

/* op: 0 ddz_E2C, 1 ddz_C2E, 2 ddz_C2C, 3 ddz_E2E, 4 d2dz2_C2C, 5 d2dz2_E2E, 6 InterpZ_E2C,
 * 7 InterpZ_C2E.  f is (n1,n2,in_len) and df (n1,n2,out_len) for dir=3; the line length
 * sits in the dir-th extent of each shape. */
/* number of host threads the oracle drivers use */
ORACLE_API int oracle_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

ORACLE_API int oracle_stagg(int n, double dx, int periodic, int topEven, int botEven, int topSided, int botSided,
                            int op, int dir, const double *f, double *df, int n1, int n2, int n3) {
    if (op < 0 || op >= ST_NOPS) return 99;
    stagg_t o;
    int ierr = stagg_init(&o, n, dx, periodic, topEven, botEven, topSided, botSided);
    if (ierr) { stagg_free(&o); return ierr; }
    int sin[3] = {n1, n2, n3}, sout[3] = {n1, n2, n3};
    sin[dir - 1] = stagg_in_len(&o, op);
    sout[dir - 1] = stagg_out_len(&o, op);
    stagg_ctx c = {&o, op};
    for_lines(dir, sin, sout, f, df, stagg_fn, &c);
    stagg_free(&o);
    return 0;
}
