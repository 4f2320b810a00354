// Device side of the compact line operators: plan upload and kernel launchers.
#pragma once
#include <cuda_runtime.h>

#include "chunkplan.h"
#include "plan.h"

namespace pade {

// Arithmetic path used for an operator application.
enum Path : int {
    PATH_DF = 0,      // double-float arithmetic on the FP32 pipes, FP64 in/out (default)
    PATH_NATIVE = 1,  // native FP64 arithmetic, one thread per line (reference-order baseline)
    PATH_FP32 = 2,    // FP32 in/out, FP32 arithmetic, chunked engine
};

// Strided description of the lines of one array: line l = a + na*b, element i of line l at
// a*fa + b*fb + i*fp (input) and a*oa + b*ob + i*op (output), in elements.
struct LineSet {
    long nlines, na;
    long fa, fb, fp;
    long oa, ob, op;
};

// Parameters of the chunked kernel, passed by value.
struct ChunkParams {
    int m, nout, ns, P, Pp, nsteps, L, LS;
    int has_center, center_off, npair, nlo, nhi, tw, resid;
    int pair_op[kMaxPairs], pair_om[kMaxPairs], pair_sign[kMaxPairs];
    F2 center_c, pair_c[kMaxPairs];
    F2 ca1, ca2;
    const int* tidx;
    const F2* tc;
    const F2* rc;  // ns x 5 : g, a1, a2, b1, b2
    const F2* fscan;
    const F2* bscan;
    const F2* fwrap;
    const F2* bwrap;
    const F2* phf;  // fundamental solutions (see ChunkPlanHost)
    const F2* phb;
};

// Operators with an instantiated fixed-stencil kernel (stencil_kernel.cuh): chunk length,
// threads per CTA (NT / Pp lines each), and the stencil shapes (Q = LHS half bandwidth,
// NP pairs at offsets +-1..NP), each for circulant (periodic) and banded lines.
constexpr int kLineM = 16;
constexpr int kLineThreadsCirc = 128;
constexpr int kLineThreadsBand = 256;
enum LineShape : int {
    SHAPE_NONE = -1,
    SHAPE_T2A = 0,  // tridiagonal, 2 antisymmetric pairs (cd06 first derivative)
    SHAPE_T2S = 1,  // tridiagonal, centre + 2 symmetric pairs (cd06 second derivative)
    SHAPE_P3A = 2,  // pentadiagonal, 3 antisymmetric pairs (cd10 first derivative)
    SHAPE_P3S = 3,  // pentadiagonal, centre + 3 symmetric pairs (cd10 second derivative)
    SHAPE_P4S = 4,  // pentadiagonal, centre + 4 symmetric pairs (cf90, residual form)
    // staggered (cd06stagg, periodic, chunks of 32): tridiagonal, 2 pairs about the half point
    // i + 1/2 (edges to cells: offsets (m, 1 - m)) or i - 1/2 (cells to edges: (m - 1, -m))
    SHAPE_T2A_E2C = 5,  // derivative, edges to cells
    SHAPE_T2S_E2C = 6,  // interpolation, edges to cells
    SHAPE_T2A_C2E = 7,  // derivative, cells to edges
    SHAPE_T2S_C2E = 8,  // interpolation, cells to edges
};

struct StencilParams {
    int M;            // chunk length (16 or 32)
    int alias;        // work rows overwrite the input window (operators without residual form)
    int ns, nout, P, Pp, nsteps, L, resid;
    int xdup;         // edges to cells, periodic: the line's stored row ns (edge n + 1) is the
                      // first row above the top, as the reference reads it (not row 0)
    int circ;         // circulant line (ring wrap, constant coefficients)
    int nlo, nhi, tw; // banded: edge rows at both ends, taps per edge row
    F2 c0;            // centre coefficient (symmetric stencils; 0 when absent)
    F2 c[kMaxPairs];  // pair coefficients: pair k (k = 1..NP) at offsets +-k, in c[k-1]
    F2 ca1, ca2;      // circulant recurrence constants (forward and backward)
    const int* tidx;  // banded edge rows: tap rows and coefficients (nlo + nhi rows x tw)
    const F2* tc;
    const double* tcd;  // the same coefficients in FP64 (the double-float path evaluates the edge
                        // rows in FP64 from the FP64 input: their one-sided sums cancel)
    const F2* rc;     // banded: ns x 5 (g, a1, a2, b1, b2)
    const F2* fscan;
    const F2* bscan;
    const F2* fwrap;
    const F2* bwrap;
    const F2* phf;    // circulant: kLineM x 2 per chunk position; banded: ns x 2 per row
    const F2* phb;
    const void* hpair;  // banded half-chunk kernel: the leading lanes', last lane's and interior tables (float4)
    int hnf;            // banded half-chunk kernel: leading lanes with tables of their own
};

struct RegParams;  // reg_kernel.cuh

class DevicePlan {
   public:
    DevicePlan() = default;
    DevicePlan(const DevicePlan&) = delete;
    DevicePlan& operator=(const DevicePlan&) = delete;
    ~DevicePlan();
    int upload(const HostPlan& hp);  // allocates device memory (not graph-capturable)
    const HostPlan& host() const { return hp_; }
    PlanView<double> view_d() const { return vd_; }
    bool chunk_ok() const { return cok_; }
    const ChunkPlanHost& chunk_host() const { return ch_; }
    ChunkParams chunk_df() const { return cdf_; }
    ChunkParams chunk_f32() const { return cf32_; }
    int chunk_M() const { return ch_.M; }
    int line_shape() const { return line_shape_; }
    const StencilParams& line_params() const { return cline_; }
    // the line kernel's parameters on the 16-row chunk plan when line_params() is a 32-row
    // plan (null otherwise): the half-chunk kernel can take either
    const StencilParams* half16_params() const { return half16_ ? &chalf16_ : nullptr; }
    // 32-row chunk parameters of a residual-form filter whose line_params() keep 16-row
    // chunks for k_line (null otherwise)
    const StencilParams* half32_params() const { return half32_ ? &chalf32_ : nullptr; }
    // banded lines whose per-row tables are one interior pattern between the two end lanes:
    // the banded half-chunk kernel's parameters (null otherwise)
    const StencilParams* half_band_params() const { return halfb_ ? &chalfb_ : nullptr; }
    // register-resident periodic kernel (chunks of 32 rows), when the line shape allows it
    bool reg_ok() const { return reg_ok_; }
    const RegParams& reg_params() const { return *creg_; }

   private:
    HostPlan hp_;
    ChunkPlanHost ch_;
    bool cok_ = false;
    void* dev_ = nullptr;
    PlanView<double> vd_{};
    ChunkParams cdf_{}, cf32_{};
    int line_shape_ = SHAPE_NONE;
    StencilParams cline_{};
    StencilParams chalf16_{};
    StencilParams chalf32_{};
    StencilParams chalfb_{};
    bool half16_ = false;
    bool half32_ = false;
    bool halfb_ = false;
    bool reg_ok_ = false;
    RegParams* creg_ = nullptr;
};

// Fixed-stencil kernel for a plan with line_shape() != SHAPE_NONE: double-float (FP64 in
// and out) or FP32 (the centred shapes, SHAPE_T2A .. SHAPE_P4S).
int launch_line(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls, unsigned* status,
                cudaStream_t s);
int launch_line_f32(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                    unsigned* status, cudaStream_t s);
// Half-chunk periodic line kernel (half_kernel.cuh), double-float: PS_ENOTSUP for the
// shapes and sizes it does not take.
int launch_line_half(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                     unsigned* status, cudaStream_t s);
// Banded half-chunk line kernel (half_kernel.cuh), double-float: PS_ENOTSUP for the shapes
// and sizes it does not take.
int launch_line_half_band(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                          unsigned* status, cudaStream_t s);
// Register-resident periodic line kernel (reg_kernel.cuh): double-float (fp32 = 0, FP64
// in and out) or FP32.  PS_ENOTSUP for shapes it does not instantiate.
int launch_line_reg(int shape, const RegParams& c, int fp32, const void* f, void* out, const LineSet& ls,
                    unsigned* status, cudaStream_t s);

// Launch the operator on a set of lines.  f/out are device pointers to double (FP64 paths)
// or float (PATH_FP32).  status (device word) collects out-of-range flags of the df path.
int launch_lines(const DevicePlan& p, int path, const void* f, void* out, const LineSet& ls, unsigned* status,
                 cudaStream_t s);

}  // namespace pade
