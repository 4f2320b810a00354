// Instantiations of the fixed-stencil kernel (stencil_kernel.cuh) for the FP32 path.
#include "stencil_kernel.cuh"

namespace pade {

int launch_line_f32_circ(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                         unsigned* status, cudaStream_t s) {
    return launch_line_shapes<ArF32, true>(shape, c, f, out, ls, status, s);
}

int launch_line_f32_band(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                         unsigned* status, cudaStream_t s) {
    return launch_line_shapes<ArF32, false>(shape, c, f, out, ls, status, s);
}

}  // namespace pade
