// Instantiations of the fixed-stencil kernel (stencil_kernel.cuh) for circulant lines, and
// the dispatcher.
#include "stencil_kernel.cuh"

namespace pade {

int launch_line_circ(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                     unsigned* status, cudaStream_t s) {
    if (shape >= SHAPE_T2A_E2C) return launch_line_stagg(shape, c, f, out, ls, status, s);
    return launch_line_shapes<ArDF, true>(shape, c, f, out, ls, status, s);
}

int launch_line_f32(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                    unsigned* status, cudaStream_t s) {
    return c.circ ? launch_line_f32_circ(shape, c, f, out, ls, status, s)
                  : launch_line_f32_band(shape, c, f, out, ls, status, s);
}

int launch_line(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls, unsigned* status,
                cudaStream_t s) {
    return c.circ ? launch_line_circ(shape, c, f, out, ls, status, s)
                  : launch_line_band(shape, c, f, out, ls, status, s);
}

}  // namespace pade
