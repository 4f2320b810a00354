// Explicit instantiations of the chunked kernel (compiled in parallel with the others).
#include "chunk_kernel.cuh"

namespace pade {
template int launch_chunk_m<ArF32, 16>(const ChunkPlanHost&, const ChunkParams&, const void*, void*,
                                         const LineSet&, unsigned*, cudaStream_t);
template int launch_chunk_m<ArF32, 32>(const ChunkPlanHost&, const ChunkParams&, const void*, void*,
                                         const LineSet&, unsigned*, cudaStream_t);
}  // namespace pade
