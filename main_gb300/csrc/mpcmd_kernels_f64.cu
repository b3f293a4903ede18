// FP64 (compiled without FMA contraction for parity with the FP64 oracle) instantiation of the engine kernels.
#include "mpcmd_kernels.cuh"

namespace mpcmd {
template struct Launch<double>;
}  // namespace mpcmd
