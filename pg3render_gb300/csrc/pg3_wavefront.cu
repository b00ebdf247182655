// Wavefront pipeline (stage kernels over SoA ray/hit/shadow queues).
#include "pg3_kernels.h"

namespace pg3 {

size_t wavefrontBytes(uint64_t capacity) { return 64 * capacity; }

cudaError_t launchWavefront(const SceneView &, bool, uint32_t, uint64_t, uint32_t, float *, float *, float *,
                            DevStats *, void *, uint64_t, int, cudaStream_t)
{
    return cudaErrorNotSupported;
}

}  // namespace pg3
