// Explicit instantiations of the chunked kernel (compiled in parallel with the others).
#include "chunk_kernel.cuh"

namespace pade {
template int launch_chunk_m<ArDF, 16>(const ChunkPlanHost&, const ChunkParams&, const void*, void*,
                                         const LineSet&, unsigned*, cudaStream_t);
}  // namespace pade
