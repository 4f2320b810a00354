// Instantiations of the fixed-stencil kernel (stencil_kernel.cuh) for banded lines.
#include "stencil_kernel.cuh"

namespace pade {

int launch_line_band(int shape, const StencilParams& c, const void* f, void* out, const LineSet& ls,
                     unsigned* status, cudaStream_t s) {
    return launch_line_shapes<ArDF, false>(shape, c, f, out, ls, status, s);
}

}  // namespace pade
