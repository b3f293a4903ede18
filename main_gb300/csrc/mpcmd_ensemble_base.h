// Precision-independent interface of a batched ensemble (the C ABI and the
// autotuner in mpcmd_ensemble.cu drive it; mpcmd_ensemble_impl.cuh implements
// it for float and double).
#pragma once
#include <cstdint>
#include <string>

#include "mpcmd.h"

namespace mpcmd {

struct EnsembleBase {
  virtual ~EnsembleBase() {}
  virtual int initial() = 0;
  virtual int upload(int r, const double* x, const double* y, const double* z, const double* vx,
                     const double* vy, const double* vz, const int32_t* flag, const double* dpos,
                     const double* dvel, const double* dforce) = 0;
  virtual int download(int r, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                       int32_t* flag, double* dpos, double* dvel, double* dforce) = 0;
  virtual int prepare() = 0;
  virtual int run(int64_t nsteps) = 0;
  virtual int observables(mpcmd_obs* out) = 0;
  virtual int reset_samples(int history) = 0;
  virtual int samples(double* mean, int64_t* count, float* axes) = 0;
  virtual int field_accumulate(int nz, int nr, double zmax, double rmax) = 0;
  virtual int field_read(uint32_t* counts, int64_t* samples) = 0;
  virtual int set_schedule(int particle_tile, int block, int shell_block) = 0;
  virtual void get_schedule(int* sched) const = 0;
  // tuner support: keep (save = true) or bring back (save = false) a copy of
  // the whole mutable state; release() frees the copy
  virtual int snapshot(bool save) = 0;
  virtual void release_snapshot() = 0;
  virtual bool at_period_boundary() const = 0;
  virtual int mpc_every() const = 0;
  virtual std::string shape_class() const = 0;
  virtual int counters(int64_t* c, int n) = 0;
  virtual int event_record(int slot) = 0;
  virtual int event_elapsed(int a, int b, double* ms) = 0;
  virtual int synchronize() = 0;
  int64_t bytes = 0;
};

EnsembleBase* make_ensemble_f32(const mpcmd_ensemble_config& cfg, const mpcmd_replica* reps, int* status);
EnsembleBase* make_ensemble_f64(const mpcmd_ensemble_config& cfg, const mpcmd_replica* reps, int* status);

}  // namespace mpcmd
