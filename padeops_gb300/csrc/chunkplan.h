// Plan of the chunked line engine (the fast path).
//
// A line of ns rows is cut into P chunks of M rows, one chunk per lane; the P lanes of a
// line sit next to each other in a warp.  The solve A x = r is written as two
// second-order (or first-order) linear recurrences,
//   forward   y_i = g_i r_i - a1_i y_{i-1} - a2_i y_{i-2}
//   backward  x_i = y_i     - b1_i x_{i+1} - b2_i x_{i+2}
// taken from the no-pivot LU of A (non-periodic) or from the symmetric spectral
// factorisation A = c (I + l1 S^-1 + l2 S^-2)(I + l1 S + l2 S^2) of a circulant A
// (periodic; then the coefficients are constants and the recurrences wrap around the
// ring).  Each lane runs its chunk from a zero state, the lanes combine the chunk end
// states with a log-step shuffle scan of the affine chunk transfers (precomputed here),
// and each lane adds the response of its rows to the exact incoming state (precomputed
// fundamental solutions, phf/phb).  No step truncates.
#pragma once
#include <vector>

#include "plan.h"

namespace pade {

constexpr int kMaxPairs = 6;
constexpr int kMaxLanes = 32;
constexpr int kMaxSteps = 5;  // log2(32)

// Coefficients as the kernel consumes them: (hi, lo) float pairs for the double-float
// path, (value, 0) for the FP32 path.
struct F2 {
    float h, l;
};

struct ChunkPlanHost {
    int ok = 0;         // 1 if the chunked engine can run this operator
    int M = 16, P = 1, Pp = 1, nsteps = 0, L = 16;
    int Q = 0;          // 0 explicit, 1 tri, 2 penta
    int circ = 0;       // circulant (constant coefficients, ring wrap)
    int m = 0, nout = 0, ns = 0, resid = 0;
    int LS = 0;         // shared-memory line stride in elements (odd)
    // interior stencil as center + (antisymmetric or symmetric) pairs
    int has_center = 0, center_off = 0;
    int npair = 0;
    int pair_op[kMaxPairs] = {0}, pair_om[kMaxPairs] = {0}, pair_sign[kMaxPairs] = {0};
    double center_c = 0.0, pair_c[kMaxPairs] = {0};
    int use_pairs = 0;  // 0: generic taps
    int ntap = 0, io[kMaxTap] = {0};
    double ic[kMaxTap] = {0};
    // table rows (explicit) at both ends
    int nlo = 0, nhi = 0, tw = 1;
    std::vector<int> tidx;
    std::vector<double> tc;
    // per-row recurrence coefficients (non-circulant), ns rows: g, a1, a2, b1, b2
    std::vector<double> rc;
    // circulant constants
    double cg = 1.0, ca1 = 0.0, ca2 = 0.0;
    // scan matrices: fwd/bwd [lane][step] 2x2 (row-major), cyclic wrap [lane] 2x2
    std::vector<double> fscan, bscan, fwrap, bwrap;
    // fundamental solutions inside a chunk: the response of row i to a unit incoming state,
    // (phi1, phi2) per row (non-circulant, ns rows) or per position in the chunk counted
    // from the chunk start (forward) / end (backward) (circulant, M positions)
    std::vector<double> phf, phb;
};

int build_chunk_plan(const HostPlan& hp, int M, ChunkPlanHost& cp);

}  // namespace pade
