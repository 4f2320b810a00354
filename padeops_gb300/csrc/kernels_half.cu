// Instantiations of the half-chunk line kernel (half_kernel.cuh) and its dispatcher.
#include <algorithm>
#include <cstdlib>

#include "half_kernel.cuh"

namespace pade {

// Periodic lines of whole chunks (32 rows, or 16 with the 16-row plan's parameters): the
// centred derivatives (window reused), cf90 in residual form and (32-row chunks) the
// staggered cd06stagg shapes; PS_ENOTSUP for the rest (k_line runs those).
template <int M>
static int launch_half_m(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                         unsigned* status, cudaStream_t s) {
    switch (shape) {
        case SHAPE_T2A: return launch_lhalf_t<1, 2, false, M>(c, f, out, ls, status, s);
        case SHAPE_T2S: return launch_lhalf_t<1, 2, true, M>(c, f, out, ls, status, s);
        case SHAPE_P3A: return launch_lhalf_t<2, 3, false, M>(c, f, out, ls, status, s);
        case SHAPE_P3S: return launch_lhalf_t<2, 3, true, M>(c, f, out, ls, status, s);
        case SHAPE_P4S: return c.resid ? launch_lhalf_t<2, 4, true, M, true>(c, f, out, ls, status, s) : PS_ENOTSUP;
        default: break;
    }
    if constexpr (M == 32) {  // the staggered shapes run in chunks of 32 only
        switch (shape) {
            case SHAPE_T2A_E2C: return launch_lhalf_t<1, 2, false, 32, false, 1>(c, f, out, ls, status, s);
            case SHAPE_T2S_E2C: return launch_lhalf_t<1, 2, true, 32, false, 1>(c, f, out, ls, status, s);
            case SHAPE_T2A_C2E: return launch_lhalf_t<1, 2, false, 32, false, -1>(c, f, out, ls, status, s);
            case SHAPE_T2S_C2E: return launch_lhalf_t<1, 2, true, 32, false, -1>(c, f, out, ls, status, s);
            default: break;
        }
    }
    return PS_ENOTSUP;
}

// The half-chunk kernels address the rows of strided lines with 32-bit offsets.
static bool half_offsets_fit(const StencilParams& c, const LineSet& ls) {
    const long rows = (long)std::max(c.ns, c.nout) + 1;
    const long st = std::max(std::labs(ls.fp), std::labs(ls.op));
    return rows * st <= 2147483647L;
}

int launch_line_half(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                     unsigned* status, cudaStream_t s) {
    if (!half_offsets_fit(c, ls)) return PS_ENOTSUP;
    const bool stagg = shape >= SHAPE_T2A_E2C && shape <= SHAPE_T2S_C2E;
    if (!c.circ || (c.M != 32 && c.M != 16) || (c.xdup && !(shape == SHAPE_T2A_E2C || shape == SHAPE_T2S_E2C)) ||
        c.ns % c.M != 0 || c.L < 1 || (stagg && c.M != 32))
        return PS_ENOTSUP;
    if (c.alias == (shape == SHAPE_P4S) || (shape == SHAPE_P4S && (!c.resid || c.nout != c.ns))) return PS_ENOTSUP;
    if (ls.fp == 1) {
        if ((c.ns + 31) / 32 > kHalfRowsContig) return PS_ENOTSUP;
    } else {
        const int pstep = kLineThreadsCirc / c.L;
        if ((c.ns + pstep - 1) / pstep > c.M) return PS_ENOTSUP;
    }
    return c.M == 32 ? launch_half_m<32>(shape, c, f, out, ls, status, s)
                     : launch_half_m<16>(shape, c, f, out, ls, status, s);
}

// Banded lines of whole 32-row chunks (two 16-row chunks of the plan per lane) whose tables
// passed the plan's interior check (hpair set).
int launch_line_half_band(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                          unsigned* status, cudaStream_t s) {
    if (!half_offsets_fit(c, ls)) return PS_ENOTSUP;
    if (c.circ || c.M != 16 || !c.hpair || c.hnf < 1 || c.hnf > 3 || c.ns % 32 != 0 || c.nout != c.ns || c.L < 1 ||
        c.nlo > 16 || c.nhi > 16)
        return PS_ENOTSUP;
    if (c.alias == (shape == SHAPE_P4S) || (shape == SHAPE_P4S && !c.resid)) return PS_ENOTSUP;
    if (ls.fp == 1) {
        if ((c.ns + 31) / 32 > kHalfRowsContig) return PS_ENOTSUP;
    } else {
        const int pstep = kLineThreadsCirc / c.L;
        if ((c.ns + pstep - 1) / pstep > 32) return PS_ENOTSUP;
    }
    switch (shape) {
        case SHAPE_T2A: return launch_lhalf_band_t<1, 2, false>(c, f, out, ls, status, s);
        case SHAPE_T2S: return launch_lhalf_band_t<1, 2, true>(c, f, out, ls, status, s);
        case SHAPE_P3A: return launch_lhalf_band_t<2, 3, false>(c, f, out, ls, status, s);
        case SHAPE_P3S: return launch_lhalf_band_t<2, 3, true>(c, f, out, ls, status, s);
        case SHAPE_P4S: return launch_lhalf_band_t<2, 4, true, true>(c, f, out, ls, status, s);
        default: return PS_ENOTSUP;
    }
}

}  // namespace pade
