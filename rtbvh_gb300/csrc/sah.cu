// Binned SAH build (placeholder until the device builder lands).
#include "lib_internal.h"

namespace rtbvh {

ResultCode build_binned_sah(const DAabb*, const float4*, size_t n, size_t, cudaStream_t, BuildOutput*) {
  if (n == 0) return NoPrimitives;
  return Error;
}

}  // namespace rtbvh
