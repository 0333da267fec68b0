// Backward pass of the closest-hit triangle test (placeholder until the
// differentiable path lands).
#include "lib_internal.h"

namespace rtbvh {

cudaError_t launch_intersect_backward(const float*, size_t, const float*, const float4*, const float*, size_t,
                                      float*, float*, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // namespace rtbvh
