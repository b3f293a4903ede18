// FP32 instantiation of the engine kernels.
#include "mpcmd_kernels.cuh"

namespace mpcmd {
template struct Launch<float>;
}  // namespace mpcmd
