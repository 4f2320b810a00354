// Operator definitions for the PadeOps compact line operators.
//
// Every PadeOps operator on one grid line is   A x = B f   with B a banded explicit
// stencil (boundary rows special) and A tri- or pentadiagonal, cyclic for periodic
// grids.  This header describes one such operator as data (an OpDef); the device
// plan (banded LU + cyclic Woodbury correction) is derived from it in plan.cpp.
#pragma once
#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace pade {

// A linear form sum_t c_t * f[j_t] over 0-based input indices.
struct LinForm {
    std::vector<std::pair<int, double>> t;
    LinForm() = default;
    LinForm(int j, double c) { t.push_back({j, c}); }
};
LinForm operator+(const LinForm& a, const LinForm& b);
LinForm operator-(const LinForm& a, const LinForm& b);
LinForm operator-(const LinForm& a);
LinForm operator*(double c, const LinForm& a);
inline LinForm operator*(const LinForm& a, double c) { return c * a; }

struct OpDef {
    int m = 0;       // input line length
    int nout = 0;    // output line length
    int ns = 0;      // rows solved; rows ns..nout-1 copy row (i - ns) (periodic edge grids)
    int q = 0;       // LHS half bandwidth: 0 explicit, 1 tridiagonal, 2 pentadiagonal
    bool cyclic = false;
    bool zero = false;      // n == 1 derivative: output is zero
    bool identity = false;  // n == 1 filter: output equals input
    // residual form: out = f - A^-1 ((A - B) f), identical to A^-1 B f for square operators.
    // Used for near-identity filters (cf90): (A - B) has coefficients ~1e-4, so the
    // rounding that the solve amplifies at the poorly conditioned Nyquist mode shrinks by
    // the same factor.
    bool resid = false;
    std::vector<LinForm> rhs;                 // ns rows
    std::vector<std::array<double, 5>> lhs;   // ns rows, coefficients at offsets -2..2
    // Interior stencil used by the device fast path: out_i = sum_t ic[t] * f[i + io[t]]
    // with f extended periodically (period ns) outside [0, m) when cyclic.
    std::vector<int> io;
    std::vector<double> ic;
};

// Families and operator codes.  Error codes mirror the reference's init ierr values and
// GracefulExit codes so a Fortran shim can forward them unchanged.
enum Status : int {
    PS_OK = 0,
    PS_EREF_NONPERIODIC_N = 2,  // cd06/cd10 init: n too small (cd06.F90:181, cd10.F90:224)
    PS_EREF_PERIODIC_N = 3,     // cd06 init periodic n < 6 (cd06.F90:158)
    PS_EREF_FILTER_N = 7,       // cf90 init n < 10 (cf90.F90:128)
    PS_EREF_STAGG_N = 21,       // cd06stagg init n <= 4 (cd06stagg.F90:183)
    PS_EREF_BC = 324,           // bc outside {0,1,-1} (cd10.F90:2045)
    PS_EINVAL = 1001,
    PS_ENOMEM = 1002,
    PS_ECUDA = 1003,
    PS_ENOTSUP = 1004,
    PS_ETIMEOUT = 1005,
    PS_ERANGE = 1006,  // an input left the double-float range
};

// cd06 (cd06.F90): order 1 (periodic or bc 0 closures), order 2 (periodic only).
int def_cd06(int n, double dx, bool periodic, int bc1, int bcn, int order, OpDef& out);
// cd10 (cd10.F90): order 1/2, bc1/bcn in {0,1,-1} for non-periodic.
int def_cd10(int n, double dx, bool periodic, int bc1, int bcn, int order, OpDef& out);
// cf90 (cf90.F90)
int def_cf90(int n, bool periodic, int bc1, int bcn, OpDef& out);
// gaussian (gaussian.F90)
int def_gaussian(int n, bool periodic, int bc1, int bcn, OpDef& out);

// cd06stagg operators (cd06stagg.F90)
enum StaggOp { D1_E2C = 0, D1_C2E, D1_C2C, D1_E2E, D2_C2C, D2_E2E, I_E2C, I_C2E, STAGG_NOPS };
struct StaggCfg {
    int n = 0;
    double dx = 1.0;
    bool periodic = true, topEven = false, botEven = false, topSided = false, botSided = false;
};
int def_stagg(const StaggCfg& cfg, int op, OpDef& out);
// Pade6stagg's second-order staggered scheme (fd02: staggOps.F90 operators selected as
// PadeDerOps.F90 does per boundary-code pair (bot, top), each -1, 0 or 1; periodic lines
// ignore the codes).  op: D1_E2C, D1_C2E, D2_C2C, D2_E2E, I_E2C, I_C2E (StaggOp numbering);
// combinations the reference has no operator for give the zero operator.
int def_fd02(int n, double dz, bool periodic, int bot, int top, int op, OpDef& out);

// Dense restatement of an operator (nout x m matrix of A^-1 B including copied rows),
// used by host-side tests and by the dense tensor-core path.  Returns 0 on success.
int dense_operator(const OpDef& d, std::vector<double>& M);

}  // namespace pade
