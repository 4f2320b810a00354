// Instantiations of the fixed-stencil kernel (stencil_kernel.cuh) for the staggered
// cd06stagg operators on periodic lines: derivative and interpolation, edges to cells and
// cells to edges (double-float, chunks of 32 rows, input window reused).
#include "stencil_kernel.cuh"

namespace pade {

int launch_line_stagg(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                      unsigned* status, cudaStream_t s) {
    if (c.M != 32 || !c.circ) return PS_ENOTSUP;
    switch (shape) {
        case SHAPE_T2A_E2C: return launch_line_t<ArDF, 1, 2, false, true, 32, true, 1>(c, f, out, ls, status, s);
        case SHAPE_T2S_E2C: return launch_line_t<ArDF, 1, 2, true, true, 32, true, 1>(c, f, out, ls, status, s);
        case SHAPE_T2A_C2E: return launch_line_t<ArDF, 1, 2, false, true, 32, true, -1>(c, f, out, ls, status, s);
        case SHAPE_T2S_C2E: return launch_line_t<ArDF, 1, 2, true, true, 32, true, -1>(c, f, out, ls, status, s);
        default: return PS_ENOTSUP;
    }
}

}  // namespace pade
