// C ABI of the batched ensemble (include/mpcmd.h, mpcmd_ens_*) and its
// autotuner.
//
// The autotuner picks the work schedule (particles per tile, threads per
// block of the particle kernels, shell entries per tile of the shell kernels)
// by timing collision periods of the ensemble itself: it keeps a snapshot of
// the state, runs each candidate from that snapshot with CUDA events around
// the timed periods, restores the snapshot and keeps the fastest.  The
// candidates are searched one coordinate at a time (tile and block with the
// default shell tile, then the shell tile).  Results are cached per shape
// class (precision, replica count and total particle count rounded to powers
// of two) in a plain text file, one line per class:
//   <class> <particle_tile> <block> <shell_block> <ms per period>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "mpcmd.h"
#include "mpcmd_ensemble_base.h"

using namespace mpcmd;

struct mpcmd_ens {
  EnsembleBase* e = nullptr;
};

#define ENS_OK(p)                                   \
  do {                                              \
    if (!(p) || !(p)->e) return MPCMD_ERR_STATE;    \
  } while (0)

namespace {

bool cache_lookup(const char* path, const std::string& cls, int* sched) {
  if (!path) return false;
  std::ifstream f(path);
  std::string line;
  bool found = false;
  while (std::getline(f, line)) {
    std::istringstream is(line);
    std::string c;
    int a, b, s;
    double ms;
    if (is >> c >> a >> b >> s >> ms && c == cls) {
      sched[0] = a; sched[1] = b; sched[2] = s;
      found = true;   // the last line of a class wins
    }
  }
  return found;
}

void cache_store(const char* path, const std::string& cls, const int* sched, double ms) {
  if (!path) return;
  std::FILE* f = std::fopen(path, "a");
  if (!f) return;
  std::fprintf(f, "%s %d %d %d %.6f\n", cls.c_str(), sched[0], sched[1], sched[2], ms);
  std::fclose(f);
}

// Mean ms per collision period of the current schedule, from the snapshot:
// one untimed period (graph capture, caches), then `periods` timed ones.
int time_schedule(EnsembleBase* e, int periods, double* ms) {
  int r = e->snapshot(false);
  if (r) return r;
  const int P = e->mpc_every();
  if ((r = e->run(P))) return r;
  if ((r = e->event_record(6))) return r;
  if ((r = e->run((int64_t)periods * P))) return r;
  if ((r = e->event_record(7))) return r;
  double t = 0;
  if ((r = e->event_elapsed(6, 7, &t))) return r;
  *ms = t / periods;
  return MPCMD_OK;
}

}  // namespace

extern "C" {

int mpcmd_ens_create(const mpcmd_ensemble_config* cfg, const mpcmd_replica* replicas, mpcmd_ens** out) {
  if (!cfg || !replicas || !out) return MPCMD_ERR_CONFIG;
  *out = nullptr;
  int st = MPCMD_OK;
  EnsembleBase* e = nullptr;
  if (cfg->precision == MPCMD_PREC_FP32 || cfg->precision == 0) e = make_ensemble_f32(*cfg, replicas, &st);
  else if (cfg->precision == MPCMD_PREC_FP64) e = make_ensemble_f64(*cfg, replicas, &st);
  else return MPCMD_ERR_CONFIG;
  if (!e) return st;
  *out = new mpcmd_ens{e};
  return MPCMD_OK;
}

int mpcmd_ens_destroy(mpcmd_ens* ens) {
  if (!ens) return MPCMD_OK;
  delete ens->e;
  delete ens;
  return MPCMD_OK;
}

int mpcmd_ens_device_bytes(const mpcmd_ens* ens, int64_t* bytes) {
  ENS_OK(ens);
  if (!bytes) return MPCMD_ERR_CONFIG;
  *bytes = ens->e->bytes;
  return MPCMD_OK;
}

int mpcmd_ens_initial(mpcmd_ens* ens) { ENS_OK(ens); return ens->e->initial(); }

int mpcmd_ens_upload(mpcmd_ens* ens, int32_t r, const double* x, const double* y, const double* z,
                     const double* vx, const double* vy, const double* vz, const int32_t* flag,
                     const double* dpos, const double* dvel, const double* dforce) {
  ENS_OK(ens);
  return ens->e->upload(r, x, y, z, vx, vy, vz, flag, dpos, dvel, dforce);
}

int mpcmd_ens_download(mpcmd_ens* ens, int32_t r, double* x, double* y, double* z, double* vx,
                       double* vy, double* vz, int32_t* flag, double* dpos, double* dvel,
                       double* dforce) {
  ENS_OK(ens);
  return ens->e->download(r, x, y, z, vx, vy, vz, flag, dpos, dvel, dforce);
}

int mpcmd_ens_prepare(mpcmd_ens* ens) { ENS_OK(ens); return ens->e->prepare(); }
int mpcmd_ens_run(mpcmd_ens* ens, int64_t nsteps) { ENS_OK(ens); return ens->e->run(nsteps); }
int mpcmd_ens_observables(mpcmd_ens* ens, mpcmd_obs* out) { ENS_OK(ens); return ens->e->observables(out); }
int mpcmd_ens_reset_samples(mpcmd_ens* ens, int32_t history) { ENS_OK(ens); return ens->e->reset_samples(history); }
int mpcmd_ens_samples(mpcmd_ens* ens, double* mean_speed, int64_t* count, float* axes) {
  ENS_OK(ens);
  return ens->e->samples(mean_speed, count, axes);
}
int mpcmd_ens_field_accumulate(mpcmd_ens* ens, int32_t nz, int32_t nr, double zmax, double rmax) {
  ENS_OK(ens);
  return ens->e->field_accumulate(nz, nr, zmax, rmax);
}
int mpcmd_ens_field_read(mpcmd_ens* ens, uint32_t* counts, int64_t* samples) {
  ENS_OK(ens);
  return ens->e->field_read(counts, samples);
}
int mpcmd_ens_set_schedule(mpcmd_ens* ens, int32_t particle_tile, int32_t block, int32_t shell_block) {
  ENS_OK(ens);
  return ens->e->set_schedule(particle_tile, block, shell_block);
}
int mpcmd_ens_get_schedule(mpcmd_ens* ens, int32_t* sched) {
  ENS_OK(ens);
  if (!sched) return MPCMD_ERR_CONFIG;
  int s[3];
  ens->e->get_schedule(s);
  for (int k = 0; k < 3; ++k) sched[k] = s[k];
  return MPCMD_OK;
}

int mpcmd_ens_autotune(mpcmd_ens* ens, const char* cache_path, int32_t periods) {
  ENS_OK(ens);
  EnsembleBase* e = ens->e;
  if (!e->at_period_boundary()) return MPCMD_ERR_STATE;
  if (periods <= 0) periods = 2;
  const std::string cls = e->shape_class();
  int sched[3];
  if (cache_lookup(cache_path, cls, sched)) return e->set_schedule(sched[0], sched[1], sched[2]);
  int r = e->snapshot(true);
  if (r) return r;
  int best[3];
  e->get_schedule(best);
  double best_ms = 1e300;
  const int tiles[] = {1024, 2048, 4096};
  const int blocks[] = {128, 256};
  const int shell_blocks[] = {128, 256};
  auto trial = [&](int a, int b, int s) -> int {
    int rr = e->set_schedule(a, b, s);
    if (rr) return rr;
    double ms = 0;
    rr = time_schedule(e, periods, &ms);
    if (rr) return rr;
    if (ms < best_ms) { best_ms = ms; best[0] = a; best[1] = b; best[2] = s; }
    return MPCMD_OK;
  };
  for (int a : tiles)
    for (int b : blocks)
      if (!r) r = trial(a, b, 256);
  const int ba = best[0], bb = best[1];
  for (int s : shell_blocks)
    if (!r && s != 256) r = trial(ba, bb, s);
  if (!r) r = e->set_schedule(best[0], best[1], best[2]);
  if (!r) r = e->snapshot(false);
  e->release_snapshot();
  if (!r) cache_store(cache_path, cls, best, best_ms);
  return r;
}

int mpcmd_ens_counters(mpcmd_ens* ens, int64_t* counters, int32_t n) {
  ENS_OK(ens);
  if (!counters || n < 0) return MPCMD_ERR_CONFIG;
  return ens->e->counters(counters, n);
}
int mpcmd_ens_event_record(mpcmd_ens* ens, int slot) { ENS_OK(ens); return ens->e->event_record(slot); }
int mpcmd_ens_event_elapsed(mpcmd_ens* ens, int a, int b, double* ms) {
  ENS_OK(ens);
  return ens->e->event_elapsed(a, b, ms);
}
int mpcmd_ens_synchronize(mpcmd_ens* ens) { ENS_OK(ens); return ens->e->synchronize(); }

}  // extern "C"
