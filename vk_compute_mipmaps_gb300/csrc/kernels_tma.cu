// kernels_tma.cu -- sRGBA8 fast pipeline with TMA tile loads (placeholder:
// the portable kernels run every dispatch until this family is enabled).
#include "device_common.cuh"

namespace nvpyr {

bool tmaFastSupported(const DispatchParams&) { return false; }

cudaError_t launchTmaFast(const DispatchParams&, const DispatchParams*, uint32_t, cudaStream_t, const Scratch&,
                          uint32_t*) {
  return cudaErrorNotSupported;
}

}  // namespace nvpyr
