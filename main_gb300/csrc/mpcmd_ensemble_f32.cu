// FP32 instantiation of the batched ensemble (production build).
#include "mpcmd_ensemble_impl.cuh"

namespace mpcmd {
EnsembleBase* make_ensemble_f32(const mpcmd_ensemble_config& cfg, const mpcmd_replica* reps, int* status) {
  return ens::make_ensemble<float>(cfg, reps, status);
}
}  // namespace mpcmd
