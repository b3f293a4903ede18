/*
 * A plain-C driver of the mpcmd C ABI: the call sequence of
 * collective_code/main_pattern.f95 (initial state, prepare as :168-187, then
 * per step evolve, and on collision steps distribute, mpc_rotation and
 * reaction_simple as :203-225), compiled with gcc against include/mpcmd.h and
 * linked to libmpcmd.so.  It is what a Fortran driver built with the modules
 * of this directory does through iso_c_binding, and it shows that the header
 * and the library agree outside Python.
 *
 *   mpcmd_driver <out file> <geometry 0 walls | 1 periodic> <edge> <steps> <seed>
 *
 * The run is the collective input deck's physics in an edge^3 box (edge x
 * edge x 8 with walls) at density 10 with one dimer, FP64.  The output file
 * holds, in native byte order: int64 n, int64 n_spheres, int64 n_cells, the
 * cell order (int32[n_cells]), the initial state and the final state (each
 * x, y, z, vx, vy, vz as double[n], flag as int32[n], dpos, dvel as
 * double[3 n_spheres]), and the final species counts (int64[4]).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mpcmd.h"

static void check(int st, const char* what) {
  if (st != MPCMD_OK) {
    fprintf(stderr, "mpcmd_driver: %s failed: %s (%d)\n", what, mpcmd_error_string(st), st);
    exit(1);
  }
}

static void write_state(FILE* f, mpcmd_ctx* ctx, int64_t n, int64_t ns) {
  double* v[6];
  for (int c = 0; c < 6; ++c) v[c] = (double*)malloc(sizeof(double) * (size_t)n);
  int32_t* flag = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
  double* dpos = (double*)malloc(sizeof(double) * 3 * (size_t)ns);
  double* dvel = (double*)malloc(sizeof(double) * 3 * (size_t)ns);
  double* dfrc = (double*)malloc(sizeof(double) * 3 * (size_t)ns);
  check(mpcmd_download_state(ctx, v[0], v[1], v[2], v[3], v[4], v[5], flag, dpos, dvel, dfrc), "download_state");
  for (int c = 0; c < 6; ++c) fwrite(v[c], sizeof(double), (size_t)n, f);
  fwrite(flag, sizeof(int32_t), (size_t)n, f);
  fwrite(dpos, sizeof(double), 3 * (size_t)ns, f);
  fwrite(dvel, sizeof(double), 3 * (size_t)ns, f);
  for (int c = 0; c < 6; ++c) free(v[c]);
  free(flag); free(dpos); free(dvel); free(dfrc);
}

int main(int argc, char** argv) {
  if (argc != 6) {
    fprintf(stderr, "usage: %s <out> <geometry> <edge> <steps> <seed>\n", argv[0]);
    return 2;
  }
  const int geometry = atoi(argv[2]), edge = atoi(argv[3]);
  const long steps = atol(argv[4]);
  const double pi = 3.141592653589793;
  mpcmd_config c;
  memset(&c, 0, sizeof(c));
  c.lx = edge; c.ly = edge; c.lz = geometry == MPCMD_GEOM_WALLS ? 8 : edge;
  c.geometry = geometry;
  c.n_dimers = 1;
  c.kinetics = MPCMD_KIN_SIMPLE;
  c.exclusion = MPCMD_EXCL_PARTICLE;
  c.catalysis = MPCMD_CAT_DETERMINISTIC;
  c.rotation_sense = 1;
  c.md_dt = 0.01; c.mpc_dt = 0.5;
  c.mpc_every = 50;
  c.sort_every = 10000;
  c.react_box_type = 6; c.react_dir = 0;
  c.cell_capacity = 100; c.max_neighbour = 30000; c.rattle_max_iter = 100000;
  c.init_plane = geometry == MPCMD_GEOM_WALLS;
  c.n_solvent = 10LL * c.lx * c.ly * c.lz;
  c.seed = (uint64_t)strtoull(argv[5], NULL, 10);
  c.init_count[0] = c.n_solvent;
  for (int s = 0; s < 4; ++s) { c.mass[s] = 1.0; c.eps_c[s] = 1.0; c.eps_n[s] = 1.0; }
  c.eps_n[1] = 0.1;
  c.rc = 4.0; c.rn = 2.0; c.dcn = 6.5;
  /* main_pattern.f95:118-119 */
  const double rho = (double)c.n_solvent / ((double)c.lx * c.ly * c.lz);
  c.mc = rho * (4.0 * pi / 3.0) * c.rc * c.rc * c.rc;
  c.mn = rho * (4.0 * pi / 3.0) * c.rn * c.rn * c.rn;
  c.rw = 1.0; c.ew = 1.0; c.rm_delta = 1.0; c.em = 1.0;
  c.rp_ab = 1.0; c.rp_ba = 0.0;
  c.kT = 1.0 / 6.0; c.skin = 1.5; c.rot_angle = 2.0 * pi / 3.0;
  c.k[0] = 0.05;
  c.precision = MPCMD_PREC_FP64;

  mpcmd_ctx* ctx = NULL;
  check(mpcmd_create(&c, &ctx), "create");
  FILE* f = fopen(argv[1], "wb");
  if (!f) { perror(argv[1]); return 1; }
  const int64_t n = c.n_solvent, ns = 2 * c.n_dimers, nc = (int64_t)c.lx * c.ly * c.lz;
  fwrite(&n, sizeof(n), 1, f);
  fwrite(&ns, sizeof(ns), 1, f);
  fwrite(&nc, sizeof(nc), 1, f);
  int32_t* order = (int32_t*)malloc(sizeof(int32_t) * (size_t)nc);
  check(mpcmd_cell_order(ctx, order), "cell_order");
  fwrite(order, sizeof(int32_t), (size_t)nc, f);
  free(order);

  check(mpcmd_initial(ctx), "initial");
  write_state(f, ctx, n, ns);
  check(mpcmd_prepare(ctx), "prepare");
  for (long s = 1; s <= steps; ++s) {
    check(mpcmd_evolve(ctx), "evolve");
    if (s % c.mpc_every == 0) {
      check(mpcmd_distribute(ctx), "distribute");
      check(mpcmd_mpc_rotation(ctx), "mpc_rotation");
      check(mpcmd_reaction(ctx), "reaction");
    }
  }
  write_state(f, ctx, n, ns);
  mpcmd_obs o;
  check(mpcmd_observables(ctx, &o), "observables");
  fwrite(o.species_count, sizeof(int64_t), 4, f);
  fclose(f);
  check(mpcmd_destroy(ctx), "destroy");
  printf("mpcmd_driver: %ld steps of %lld particles\n", steps, (long long)n);
  return 0;
}
