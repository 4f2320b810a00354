// Device plan of one compact line operator, derived from an OpDef.
//
// The line solve A x = B f is executed as
//   r = B f                      interior stencil (io, ic) + explicit edge rows (table)
//   y = L^-1 r, x0 = U^-1 y      no-pivot band LU of the non-cyclic part A0
//   x = x0 - Z Cinv (W^T x0)     Woodbury correction for the cyclic corner entries
//   x[i] = x[i - ns], i >= ns    copied rows of periodic edge grids
#pragma once
#include <vector>

#include "operators.h"

namespace pade {

constexpr int kMaxTap = 12;  // interior stencil taps
constexpr int kMaxNc = 4;    // cyclic corner rows (2q)

// Plain-old-data view passed to kernels by value.  Coefficient arrays are of type C.
template <class C>
struct PlanView {
    int m, nout, ns, q, cyclic, zero, identity, resid;
    int ntap, nlo, nhi, tw, nc;
    int io[kMaxTap];
    C ic[kMaxTap];
    const int* tidx;   // (nlo + nhi) x tw
    const C* tc;       // (nlo + nhi) x tw
    const C* lu;       // ns x 5 : L1, L2, U1, U2, Dinv
    const C* Z;        // ns x nc
    const C* Cinv;     // nc x nc
    const int* wcol;   // nc x q
    const C* wc;       // nc x q
};

struct HostPlan {
    OpDef def;
    int ntap = 0, nlo = 0, nhi = 0, tw = 0, nc = 0;
    std::vector<int> io;
    std::vector<double> ic;
    std::vector<int> tidx;
    std::vector<double> tc;
    std::vector<double> lu;    // ns x 5
    std::vector<double> Z;     // ns x nc
    std::vector<double> Cinv;  // nc x nc
    std::vector<int> wcol;     // nc x q
    std::vector<double> wc;    // nc x q
};

// Build the host plan; returns PS_OK or an error status.
int build_plan(const OpDef& d, HostPlan& p);

// Apply the host plan to one line on the CPU in FP64 (used to validate plans on machines
// without a GPU; not on any product path).
void host_apply_line(const HostPlan& p, const double* f, long fs, double* out, long os);

}  // namespace pade
