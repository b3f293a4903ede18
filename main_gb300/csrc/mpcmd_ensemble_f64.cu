// FP64 instantiation of the batched ensemble (parity build, compiled without
// FMA contraction like the engine's FP64 kernels).
#include "mpcmd_ensemble_impl.cuh"

namespace mpcmd {
EnsembleBase* make_ensemble_f64(const mpcmd_ensemble_config& cfg, const mpcmd_replica* reps, int* status) {
  return ens::make_ensemble<double>(cfg, reps, status);
}
}  // namespace mpcmd
