// stage2d.cu - placeholder until the 2D kernel lands.
#include <cuda_runtime.h>

#include "hrw_internal.h"

namespace hrw {
cudaError_t launch_stage2d(const StageArgs&, int, int, bool, cudaStream_t) { return cudaErrorNotSupported; }
}  // namespace hrw
