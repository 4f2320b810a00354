// Instantiations of the fixed-stencil kernel (stencil_kernel.cuh).
#include "stencil_kernel.cuh"

namespace pade {

template <bool CIRC>
int launch_line_c(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls, unsigned* status,
                  cudaStream_t s) {
    switch (shape) {
        case SHAPE_T2A: return launch_line_t<1, 2, false, CIRC>(c, f, out, ls, status, s);
        case SHAPE_T2S: return launch_line_t<1, 2, true, CIRC>(c, f, out, ls, status, s);
        case SHAPE_P3A: return launch_line_t<2, 3, false, CIRC>(c, f, out, ls, status, s);
        case SHAPE_P3S: return launch_line_t<2, 3, true, CIRC>(c, f, out, ls, status, s);
        case SHAPE_P4S: return launch_line_t<2, 4, true, CIRC>(c, f, out, ls, status, s);
        default: return PS_ENOTSUP;
    }
}

int launch_line(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls, unsigned* status,
                cudaStream_t s) {
    return c.circ ? launch_line_c<true>(shape, c, f, out, ls, status, s)
                  : launch_line_c<false>(shape, c, f, out, ls, status, s);
}

}  // namespace pade
