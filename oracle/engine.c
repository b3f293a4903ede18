/*
 * Oracle engine: FP64 restatement of the collective_code time step
 * (main_pattern.f95 and the modules it calls) with the selkov_code kinetics,
 * catalysis, exclusion and collision forms as options.  Test infrastructure
 * only (see oracle.h).  Every routine cites the reference lines it follows.
 *
 * Deliberate, documented differences from the Fortran:
 *  - pair forces of the neighbour lists are cleared for the lists in use
 *    after a rebuild (evolve_mod.f95:441-452 clears them for the previous
 *    lists, which leaves stale forces in list slots that grew in the rebuild);
 *  - per-cell lists keep only the counts and the first member of each species,
 *    the only parts reaction_mod.f95 / RMPC_SelkovDimer.f90 read; a count above
 *    cell_capacity is an error instead of a silent overflow;
 *  - RATTLE iteration caps report ORC_ERR_RATTLE instead of continuing;
 *  - random draws come from the counter-based contract generator unless the
 *    MT19937 mode is selected (serial reference draw order, one thread).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "oracle.h"
#include "engine.h"

int orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

/* ------------------------------------------------------------------ RNG -- */
double orc_draw(orc_t* o, uint32_t tag, uint32_t index, uint32_t extra,
                uint32_t step, int which) {
  if (o->rng_mode == ORC_RNG_MT) {
    if (o->mt_kind == 2002) return orc_mt_real1(o->mt, &o->mti);
    return orc_mt_grnd(o->mt, &o->mti);
  }
  return orc_contract_u01(o->p.seed, tag, index, extra, step, which);
}

int orc_set_rng(orc_t* o, int mode, uint32_t mt_seed) {
  o->rng_mode = mode;
  if (mode == ORC_RNG_MT) {
    /* kind 1998: collective mtmod.f90 sgrnd; kind 2002: selkov mt95.f90 */
    if (o->mt_kind == 2002) { orc_mt2002_init(mt_seed, o->mt); o->mti = 624; }
    else { orc_mt1998_sgrnd(mt_seed, o->mt); o->mti = 624; }
  }
  return ORC_OK;
}

/* -------------------------------------------------------------- helpers -- */
static inline double pbc_d(double d, double L) {
  /* forces_mod.f95:68-74 minimum image, single shift */
  if (d > 0.5 * L) d -= L;
  else if (d < -0.5 * L) d += L;
  return d;
}

static inline double wrap_single(double x, double L) {
  /* evolve_mod.f95:260-264 */
  if (x >= L) x -= L;
  else if (x < 0.) x += L;
  return x;
}

static inline double wrap_floor(double x, double L) {
  /* evolve_mod.f95:360-361 */
  return x - L * floor(x / L);
}

void orc_lj_consts(double r, double* R6, double* R12, double* r6R6, double* r12R12) {
  double r2 = r * r;
  *R6 = r2 * r2 * r2;
  *R12 = (*R6) * (*R6);
  *r6R6 = 6.0 * (*R6);
  *r12R12 = 12.0 * (*R12);
}

/* Squared distance from particle i to sphere s with the geometry's images. */
static inline double sol_sphere_d(const orc_t* o, int64_t i, int s, double dR[3]) {
  dR[0] = o->x[i] - o->dpos[3 * s + 0];
  dR[1] = o->y[i] - o->dpos[3 * s + 1];
  dR[2] = o->z[i] - o->dpos[3 * s + 2];
  dR[0] = pbc_d(dR[0], o->L[0]);
  dR[1] = pbc_d(dR[1], o->L[1]);
  if (o->p.geometry == ORC_GEOM_PERIODIC) dR[2] = pbc_d(dR[2], o->L[2]);
  return dR[0] * dR[0] + dR[1] * dR[1] + dR[2] * dR[2];
}

/* ------------------------------------------------------------- lifetime -- */
orc_t* orc_create(const orc_params* p) {
  if (!p || p->lx <= 0 || p->ly <= 0 || p->lz <= 0 || p->n_solvent <= 0 ||
      p->n_dimers < 0 || p->mpc_every <= 0)
    return NULL;
  orc_t* o = (orc_t*)calloc(1, sizeof(orc_t));
  if (!o) return NULL;
  o->p = *p;
  o->nt = p->n_solvent;
  o->nd = p->n_dimers;
  o->ns = 2 * p->n_dimers;
  o->L[0] = p->lx; o->L[1] = p->ly; o->L[2] = p->lz;
  o->ncell = (int64_t)p->lx * p->ly * p->lz;
  o->ncell_shift = (p->geometry == ORC_GEOM_WALLS) ? (int64_t)p->lx * p->ly * (p->lz + 1) : o->ncell;
  o->maxnb = p->max_neighbour > 0 ? p->max_neighbour : 30000;
  o->mt_kind = (p->rotation_sense < 0) ? 2002 : 1998;
  int64_t n = o->nt, ns = o->ns > 0 ? o->ns : 1;
  o->x = calloc(n, 8); o->y = calloc(n, 8); o->z = calloc(n, 8);
  o->vx = calloc(n, 8); o->vy = calloc(n, 8); o->vz = calloc(n, 8);
  o->flag = calloc(n, 4);
  o->msd = calloc(n, 8);
  o->dpos = calloc(3 * ns, 8); o->dvel = calloc(3 * ns, 8); o->dfrc = calloc(3 * ns, 8);
  o->q = calloc(3 * ns, 8);
  o->anchor = calloc(3 * ns, 8);
  o->owner = calloc(n, 4);
  o->inc = calloc(n, 1);
  o->cnow = calloc(n, 1);
  o->nbnum = calloc(ns, 8);
  o->nb = calloc(ns * o->maxnb, 8);
  o->fpair = calloc(ns * o->maxnb * 3, 8);
  o->pot = calloc(ns * o->maxnb, 8);
  o->in_list = calloc(n, 8); o->out_list = calloc(n, 8);
  o->newcell = calloc(n, 8);
  o->cm = calloc(3 * o->ncell_shift, 8);
  o->axis = calloc(3 * o->ncell_shift, 8);
  o->ccount = calloc(o->ncell_shift, 4);
  o->dcount = calloc(4 * o->ncell, 4);
  o->dfirst = calloc(4 * o->ncell, 8);
  o->affected = calloc(o->ncell, 4);
  o->react_box = calloc((size_t)p->lx * p->ly, 4);
  o->fsx = calloc(n, 8); o->fsy = calloc(n, 8); o->fsz = calloc(n, 8);
  o->pfx = calloc(n, 8); o->pfy = calloc(n, 8); o->pfz = calloc(n, 8);
  o->spair = calloc(n * 2 * 3, 8);
  o->spot = calloc(n, 8);
  if (!o->x || !o->y || !o->z || !o->vx || !o->vy || !o->vz || !o->flag || !o->msd ||
      !o->dpos || !o->dvel || !o->dfrc || !o->q || !o->anchor || !o->owner || !o->inc || !o->cnow || !o->nbnum || !o->nb || !o->fpair ||
      !o->pot || !o->in_list || !o->out_list || !o->newcell || !o->cm || !o->axis ||
      !o->ccount || !o->dcount || !o->dfirst || !o->affected || !o->react_box ||
      !o->fsx || !o->fsy || !o->fsz || !o->pfx || !o->pfy || !o->pfz || !o->spair || !o->spot) {
    orc_destroy(o);
    return NULL;
  }
  o->rng_mode = ORC_RNG_CONTRACT;
  o->status = ORC_OK;
  return o;
}

void orc_destroy(orc_t* o) {
  if (!o) return;
  free(o->x); free(o->y); free(o->z); free(o->vx); free(o->vy); free(o->vz);
  free(o->flag); free(o->msd); free(o->dpos); free(o->dvel); free(o->dfrc); free(o->q); free(o->anchor); free(o->owner); free(o->inc); free(o->cnow);
  free(o->nbnum); free(o->nb); free(o->fpair); free(o->pot); free(o->in_list);
  free(o->out_list); free(o->newcell); free(o->cm); free(o->axis); free(o->ccount);
  free(o->dcount); free(o->dfirst); free(o->affected); free(o->react_box); free(o->order);
  free(o->fsx); free(o->fsy); free(o->fsz); free(o->pfx); free(o->pfy); free(o->pfz);
  free(o->spair); free(o->spot);
  free(o);
}

int orc_status(const orc_t* o) { return o ? o->status : ORC_ERR_STATE; }

/* motorCM(k,:) = 0.5 * (X(k,1) + X(k,2)) on the positions as stored
 * (rotational_code/2d_array/initial_mod.f95:86-88). */
static void set_midpoint_anchors(orc_t* o) {
  for (int k = 0; k < o->nd; ++k)
    for (int c = 0; c < 3; ++c)
      o->anchor[3 * k + c] = 0.5 * (o->dpos[3 * (2 * k) + c] + o->dpos[3 * (2 * k + 1) + c]);
}

int orc_set_state(orc_t* o, const double* x, const double* y, const double* z,
                  const double* vx, const double* vy, const double* vz,
                  const int32_t* flag, const double* dpos, const double* dvel,
                  const double* dforce) {
  int64_t n = o->nt;
  memcpy(o->x, x, n * 8); memcpy(o->y, y, n * 8); memcpy(o->z, z, n * 8);
  memcpy(o->vx, vx, n * 8); memcpy(o->vy, vy, n * 8); memcpy(o->vz, vz, n * 8);
  memcpy(o->flag, flag, n * 4);
  memset(o->owner, 0, n * 4);
  memset(o->inc, 0, n);
  if (o->ns > 0) {
    if (dpos) memcpy(o->dpos, dpos, 3 * o->ns * 8);
    if (dvel) memcpy(o->dvel, dvel, 3 * o->ns * 8);
    if (dforce) memcpy(o->dfrc, dforce, 3 * o->ns * 8);
    else memset(o->dfrc, 0, 3 * o->ns * 8);
    set_midpoint_anchors(o);
  }
  return ORC_OK;
}

int orc_set_anchors(orc_t* o, const double* anchors) {
  if (o->nd > 0) memcpy(o->anchor, anchors, 3 * (size_t)o->nd * 8);
  return ORC_OK;
}

int orc_get_anchors(const orc_t* o, double* anchors) {
  if (o->nd > 0) memcpy(anchors, o->anchor, 3 * (size_t)o->nd * 8);
  return ORC_OK;
}

int orc_set_owner(orc_t* o, const int32_t* owner) {
  memcpy(o->owner, owner, (size_t)o->nt * 4);
  return ORC_OK;
}

int orc_get_owner(const orc_t* o, int32_t* owner) {
  memcpy(owner, o->owner, (size_t)o->nt * 4);
  return ORC_OK;
}

int orc_get_state(const orc_t* o, double* x, double* y, double* z,
                  double* vx, double* vy, double* vz, int32_t* flag,
                  double* dpos, double* dvel, double* dforce) {
  int64_t n = o->nt;
  if (x) memcpy(x, o->x, n * 8);
  if (y) memcpy(y, o->y, n * 8);
  if (z) memcpy(z, o->z, n * 8);
  if (vx) memcpy(vx, o->vx, n * 8);
  if (vy) memcpy(vy, o->vy, n * 8);
  if (vz) memcpy(vz, o->vz, n * 8);
  if (flag) memcpy(flag, o->flag, n * 4);
  if (o->ns > 0) {
    if (dpos) memcpy(dpos, o->dpos, 3 * o->ns * 8);
    if (dvel) memcpy(dvel, o->dvel, 3 * o->ns * 8);
    if (dforce) memcpy(dforce, o->dfrc, 3 * o->ns * 8);
  }
  return ORC_OK;
}

int orc_set_cell_order(orc_t* o, const int32_t* order, int64_t n) {
  if (n != o->ncell) return ORC_ERR_CONFIG;
  free(o->order);
  o->order = malloc(n * 4);
  if (!o->order) return ORC_ERR_ALLOC;
  memcpy(o->order, order, n * 4);
  return ORC_OK;
}

int orc_set_cstep(orc_t* o, int64_t cstep, int32_t time_count) {
  o->cstep = cstep;
  o->time_count = time_count;
  return ORC_OK;
}

/* ------------------------------------------------------- reactive grid -- */
/* reactive_grid_mod.f95:8-99 (1-based patch index i as in the Fortran). */
static void reactive_grid_setup(orc_t* o) {
  const double b1 = o->L[0], b2 = o->L[1];
  const int ib1 = o->p.lx;
  const int64_t nbox = (int64_t)o->p.lx * o->p.ly;
  const int type = o->p.react_box_type;
  const double sixth = (double)(1.0f / 6.0f), fivesixth = (double)(5.0f / 6.0f);
  for (int64_t k = 0; k < nbox; ++k) o->react_box[k] = 0;
  for (int64_t i = 1; i <= nbox; ++i) {
    int set = 0;
    if (type == 1) {
      int64_t m = i % ib1;
      set = (m > 0 && m <= (int64_t)(0.5 * b1));
    } else if (type == 2) {
      int64_t f = (int64_t)floor((double)i / b2);
      set = ((i + f) % 2 == 0);
    } else if (type == 3) {
      double a = 0.5 * b1 - (double)((i - 1) % ib1) + 0.5;
      double c = 0.5 * b2 - (double)(int64_t)floor((double)i / b1) + 0.5;
      set = (a * a + c * c < 400.0);
    } else if (type == 4) {
      double xm = (double)((i - 1) % ib1), yf = (double)(int64_t)floor((double)i / b1);
      double cx[3] = {sixth * b1, 0.5 * b1, fivesixth * b1};
      double cy[2] = {0.25 * b2, 0.75 * b2};
      set = 1;
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 2; ++b) {
          double u = cx[a] - xm + 0.5, v = cy[b] - yf + 0.5;
          if (!(u * u + v * v < 100.0)) set = 0;
        }
    } else if (type == 5) {
      int64_t m = i % ib1;
      set = (m > (int64_t)floor(0.5 * b1 - 4) && m <= (int64_t)floor(0.5 * b1 + 4));
    } else if (type == 6) {
      set = 1;
    }
    if (set) o->react_box[i - 1] = 1;
  }
}

int orc_reactive_grid_table(const orc_t* o, int32_t* table) {
  memcpy(table, o->react_box, (size_t)o->p.lx * o->p.ly * 4);
  return ORC_OK;
}

/* reactive_grid_mod.f95:103-151: back-project to the floor hit point. */
static inline void reactive_grid(const orc_t* o, double x, double y, double vx, double vy,
                                 int32_t* flag, double t) {
  double ax = x - vx * t, ay = y - vy * t;
  ax = wrap_single(ax, o->L[0]);
  ay = wrap_single(ay, o->L[1]);
  int64_t hit = (int64_t)(floor(ax) + o->L[0] * floor(ay));
  if (hit < 0 || hit >= (int64_t)o->p.lx * o->p.ly) return;
  if (o->react_box[hit] == 1) {
    if (o->p.react_dir == 0 && *flag == 0) *flag = 1;
    else if (o->p.react_dir == 1 && *flag == 1) *flag = 0;
  }
}

/* evolve_mod.f95:258-314 (inside, lazy=0) and :473-527 (outside, lazy=1). */
static inline void stream_particle(orc_t* o, int64_t i, double dt, int tc, int lazy) {
  const double Lx = o->L[0], Ly = o->L[1], Lz = o->L[2];
  double dx = lazy ? (o->vx[i] * dt) * (double)tc : o->vx[i] * dt;
  double dy = lazy ? (o->vy[i] * dt) * (double)tc : o->vy[i] * dt;
  double dz = lazy ? (o->vz[i] * dt) * (double)tc : o->vz[i] * dt;
  double x = wrap_single(o->x[i] + dx, Lx);
  double y = wrap_single(o->y[i] + dy, Ly);
  double z = o->z[i] + dz;
  if (o->p.geometry == ORC_GEOM_WALLS) {
    if (z < 0.) {
      double t = z / o->vz[i];
      reactive_grid(o, x, y, o->vx[i], o->vy[i], &o->flag[i], t);
      o->vx[i] = -1. * o->vx[i];
      o->vy[i] = -1. * o->vy[i];
      o->vz[i] = -1. * o->vz[i];
      x = x + 2. * o->vx[i] * t;
      y = y + 2. * o->vy[i] * t;
      z = z + 2. * o->vz[i] * t;
      x = wrap_single(x, Lx);
      y = wrap_single(y, Ly);
    } else if (z > Lz) {
      double t = (z - Lz) / o->vz[i];
      o->vx[i] = -1. * o->vx[i];
      o->vy[i] = -1. * o->vy[i];
      o->vz[i] = -1. * o->vz[i];
      x = x + 2. * o->vx[i] * t;
      y = y + 2. * o->vy[i] * t;
      z = z + 2. * o->vz[i] * t;
      x = wrap_single(x, Lx);
      y = wrap_single(y, Ly);
    }
  } else {
    z = wrap_single(z, Lz);
  }
  o->x[i] = x; o->y[i] = y; o->z[i] = z;
}

/* ---------------------------------------------------------------- sort -- */
static inline int64_t cell_of(const orc_t* o, double x, double y, double z) {
  /* sort_hilbert_mod.f95:51, distribute_mod.f95:101 (0-based) */
  return (int64_t)(floor(x) + o->L[0] * floor(y) + o->L[0] * o->L[1] * floor(z));
}

static inline int64_t clamp_cell(const orc_t* o, int64_t c) {
  /* a particle exactly on the upper wall (z == Lz) is counted in the top layer */
  if (c >= o->ncell) c -= (int64_t)o->p.lx * o->p.ly;
  return c;
}

/* sort_hilbert_mod.f95:6-98: stable bin by unshifted cell, then gather the
 * cells in the given order (hilbert.txt in the reference; row-major when no
 * order was supplied). */
int orc_sort(orc_t* o) {
  int64_t n = o->nt, C = o->ncell;
  int64_t* cnt = calloc(C + 1, 8);
  int64_t* start = calloc(C + 1, 8);
  int64_t* cellid = malloc(n * 8);
  int64_t* perm = malloc(n * 8);
  double* tmp = malloc(n * 8);
  int32_t* tmpi = malloc(n * 4);
  if (!cnt || !start || !cellid || !perm || !tmp || !tmpi) {
    free(cnt); free(start); free(cellid); free(perm); free(tmp); free(tmpi);
    return o->status = ORC_ERR_ALLOC;
  }
  for (int64_t i = 0; i < n; ++i) {
    int64_t c = clamp_cell(o, cell_of(o, o->x[i], o->y[i], o->z[i]));
    cellid[i] = c;
    cnt[c]++;
  }
  /* prefix over cells in visiting order */
  int64_t acc = 0;
  for (int64_t k = 0; k < C; ++k) {
    int64_t c = o->order ? o->order[k] : k;
    start[c] = acc;
    acc += cnt[c];
  }
  for (int64_t i = 0; i < n; ++i) perm[start[cellid[i]]++] = i;  /* new <- old */
#define PERMUTE_D(a) do { for (int64_t j = 0; j < n; ++j) tmp[j] = a[perm[j]]; memcpy(a, tmp, n * 8); } while (0)
  PERMUTE_D(o->x); PERMUTE_D(o->y); PERMUTE_D(o->z);
  PERMUTE_D(o->vx); PERMUTE_D(o->vy); PERMUTE_D(o->vz);
#undef PERMUTE_D
  for (int64_t j = 0; j < n; ++j) tmpi[j] = o->flag[perm[j]];
  memcpy(o->flag, tmpi, n * 4);
  /* linear_periodic_no_ci/sort_hilbert_mod.f95:75,92 carries type_B along */
  for (int64_t j = 0; j < n; ++j) tmpi[j] = o->owner[perm[j]];
  memcpy(o->owner, tmpi, n * 4);
  /* the inside-a-C-cutoff record of the on-exit catalysis follows the particles */
  for (int64_t j = 0; j < n; ++j) tmpi[j] = o->inc[perm[j]];
  for (int64_t j = 0; j < n; ++j) o->inc[j] = (uint8_t)tmpi[j];
  free(cnt); free(start); free(cellid); free(perm); free(tmp); free(tmpi);
  return ORC_OK;
}

/* --------------------------------------------------------- neighbours -- */
/* neighbour_list_mod.f95:6-59 for every sphere, then :63-184 inout split. */
int orc_set_list_mode(orc_t* o, int mode) {
  if (mode != ORC_LISTS_ALL_PAIRS && mode != ORC_LISTS_CELLS) return ORC_ERR_CONFIG;
  o->list_mode = mode;
  return ORC_OK;
}

/* The lists of orc_rebuild_lists through cell bins: the particles are binned
 * by cell once, each sphere visits the cells its list radius reaches and
 * sorts what it finds by index, and the inside list is the particles found
 * by any sphere, in index order: the same lists, in the same order, as the
 * all-pairs search, without its N x spheres distance tests. */
static int cmp_i64(const void* a, const void* b) {
  const int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
  return (x > y) - (x < y);
}

static int rebuild_lists_cells(orc_t* o, double fullC2, double fullN2) {
  const int64_t n = o->nt, C = o->ncell;
  const int lx = o->p.lx, ly = o->p.ly, lz = o->p.lz;
  const int periodic = o->p.geometry == ORC_GEOM_PERIODIC;
  int64_t* start = calloc(C + 1, 8);
  int64_t* fill = malloc((C + 1) * 8);
  int64_t* byc = malloc(n * 8);
  uint8_t* in = calloc(n, 1);
  if (!start || !fill || !byc || !in) {
    free(start); free(fill); free(byc); free(in);
    return o->status = ORC_ERR_ALLOC;
  }
  for (int64_t i = 0; i < n; ++i) start[clamp_cell(o, cell_of(o, o->x[i], o->y[i], o->z[i])) + 1]++;
  for (int64_t c = 0; c < C; ++c) start[c + 1] += start[c];
  memcpy(fill, start, (C + 1) * 8);
  for (int64_t i = 0; i < n; ++i) byc[fill[clamp_cell(o, cell_of(o, o->x[i], o->y[i], o->z[i]))]++] = i;
  int overflow = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(|:overflow)
  for (int s = 0; s < o->ns; ++s) {
    const double full2 = (s % 2 == 0) ? fullC2 : fullN2, R = sqrt(full2);
    const double* P = o->dpos + 3 * s;
    int64_t cntl = 0;
    int64_t* list = o->nb + (int64_t)s * o->maxnb;
    const int x0 = (int)floor(P[0] - R) - 1, x1 = (int)floor(P[0] + R) + 1;
    const int y0 = (int)floor(P[1] - R) - 1, y1 = (int)floor(P[1] + R) + 1;
    int z0 = (int)floor(P[2] - R) - 1, z1 = (int)floor(P[2] + R) + 1;
    if (!periodic) { if (z0 < 0) z0 = 0; if (z1 > lz - 1) z1 = lz - 1; }
    /* a range as wide as the box visits every cell of that axis once */
    int xa = x0, xb = x1, ya = y0, yb = y1;
    if (xb - xa + 1 >= lx) { xa = 0; xb = lx - 1; }
    if (yb - ya + 1 >= ly) { ya = 0; yb = ly - 1; }
    if (periodic && z1 - z0 + 1 >= lz) { z0 = 0; z1 = lz - 1; }
    for (int cz = z0; cz <= z1; ++cz)
      for (int cy = ya; cy <= yb; ++cy)
        for (int cx = xa; cx <= xb; ++cx) {
          const int wx = ((cx % lx) + lx) % lx, wy = ((cy % ly) + ly) % ly;
          const int wz = periodic ? ((cz % lz) + lz) % lz : cz;
          const int64_t c = wx + (int64_t)lx * (wy + (int64_t)ly * wz);
          for (int64_t q = start[c]; q < start[c + 1]; ++q) {
            const int64_t i = byc[q];
            double dR[3];
            if (sol_sphere_d(o, i, s, dR) <= full2) {
              if (cntl < o->maxnb) list[cntl] = i;
              else overflow = 1;
              cntl++;
            }
          }
        }
    const int64_t m = cntl < o->maxnb ? cntl : o->maxnb;
    /* index order, as the all-pairs loop finds them */
    qsort(list, (size_t)m, sizeof(int64_t), cmp_i64);
    o->nbnum[s] = m;
  }
  if (overflow) o->status = ORC_ERR_NEIGHBOUR_OVERFLOW;
  for (int s = 0; s < o->ns; ++s)
    for (int64_t q = 0; q < o->nbnum[s]; ++q) in[o->nb[(int64_t)s * o->maxnb + q]] = 1;
  int64_t nin = 0, nout = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (in[i]) o->in_list[nin++] = i;
    else o->out_list[nout++] = i;
  }
  o->n_in = nin;
  o->n_out = nout;
  free(start); free(fill); free(byc); free(in);
  return o->status;
}

int orc_rebuild_lists(orc_t* o) {
  const double cut = pow(2.0, 1.0 / 6.0);
  const double cutC = o->p.rc * cut, cutN = o->p.rn * cut;
  const double fullC2 = (cutC + o->p.skin) * (cutC + o->p.skin);
  const double fullN2 = (cutN + o->p.skin) * (cutN + o->p.skin);
  if (o->list_mode == ORC_LISTS_CELLS) return rebuild_lists_cells(o, fullC2, fullN2);
  const int64_t n = o->nt;
  int overflow = 0;
#pragma omp parallel for schedule(static) reduction(|:overflow)
  for (int s = 0; s < o->ns; ++s) {
    double full2 = (s % 2 == 0) ? fullC2 : fullN2;
    int64_t cntl = 0;
    int64_t* list = o->nb + (int64_t)s * o->maxnb;
    for (int64_t i = 0; i < n; ++i) {
      double dR[3];
      if (sol_sphere_d(o, i, s, dR) <= full2) {
        if (cntl < o->maxnb) list[cntl] = i;
        else overflow = 1;
        cntl++;
      }
    }
    o->nbnum[s] = cntl < o->maxnb ? cntl : o->maxnb;
  }
  if (overflow) o->status = ORC_ERR_NEIGHBOUR_OVERFLOW;
  /* inside / outside split in particle order (one-thread order of :129-177) */
  int64_t nin = 0, nout = 0;
  for (int64_t i = 0; i < n; ++i) {
    int bulk = 0;
    for (int k = 0; k < o->nd && !bulk; ++k) {
      double dR[3];
      if (sol_sphere_d(o, i, 2 * k, dR) <= fullC2 || sol_sphere_d(o, i, 2 * k + 1, dR) <= fullN2)
        bulk = 1;
    }
    if (bulk) o->in_list[nin++] = i;
    else o->out_list[nout++] = i;
  }
  o->n_in = nin;
  o->n_out = nout;
  return o->status;
}

int64_t orc_neighbour_count(const orc_t* o, int sphere) {
  if (sphere < 0 || sphere >= o->ns) return -1;
  return o->nbnum[sphere];
}

int orc_get_neighbours(const orc_t* o, int sphere, int64_t* idx) {
  if (sphere < 0 || sphere >= o->ns) return ORC_ERR_CONFIG;
  memcpy(idx, o->nb + (int64_t)sphere * o->maxnb, o->nbnum[sphere] * 8);
  return ORC_OK;
}

int orc_get_pair_forces(const orc_t* o, int sphere, double* f, double* pot) {
  if (sphere < 0 || sphere >= o->ns) return ORC_ERR_CONFIG;
  int64_t base = (int64_t)sphere * o->maxnb;
  for (int64_t j = 0; j < o->nbnum[sphere]; ++j) {
    f[3 * j + 0] = o->fpair[3 * (base + j) + 0];
    f[3 * j + 1] = o->fpair[3 * (base + j) + 1];
    f[3 * j + 2] = o->fpair[3 * (base + j) + 2];
    pot[j] = o->pot[base + j];
  }
  return ORC_OK;
}

int orc_get_inside(const orc_t* o, int64_t* n_in, int64_t* idx) {
  *n_in = o->n_in;
  if (idx) memcpy(idx, o->in_list, o->n_in * 8);
  return ORC_OK;
}

/* ----------------------------------------------------------- initial -- */
/* initial_mod.f95:6-355.  Contract draws: dimer k attempt a uses
 * (INIT_DIMER, k, a, step 0..2); particle i attempt a uses (INIT_POS, i, a,
 * step 0..1); velocity of particle i component c uses (INIT_VEL, i, c, 0). */
int orc_initial(orc_t* o) {
  const double pi = 4.0 * atan(1.0);
  const double cut = pow(2.0, 1.0 / 6.0);
  const double rc = o->p.rc, rn = o->p.rn, dcn = o->p.dcn;
  const double cutC2 = (rc * cut) * (rc * cut), cutN2 = (rn * cut) * (rn * cut);
  const double w3 = pow(3.0, (double)(1.0f / 6.0f));
  const double wcC2 = ((o->p.rw + rc) * w3) * ((o->p.rw + rc) * w3);
  const double wcN2 = ((o->p.rw + rn) * w3) * ((o->p.rw + rn) * w3);
  const int periodic = o->p.geometry == ORC_GEOM_PERIODIC;
  const int mt = o->rng_mode == ORC_RNG_MT;
  const int64_t max_attempts = 100000000;

  if (o->p.layout != ORC_LAYOUT_RANDOM) {
    /* rotational_code/2d_array/initial_mod.f95:68-90 (grid, row-major over
     * numrows x numcols) and linear_periodic_ci/initial_mod.f95:72-88 (line
     * along x): motor centres on a lattice of pitch Dcn + 2 Rc 2^(1/6) + sep
     * in the plane z = zdimeq, each with a uniform in-plane orientation */
    const int grid = o->p.layout == ORC_LAYOUT_GRID;
    const double cutoff = pow(2.0, 1.0 / 6.0), sep = o->p.layout_sep;
    const double rows = o->p.layout_rows, cols = o->p.layout_cols;
    if (grid ? (o->p.layout_rows * o->p.layout_cols != o->nd) : o->p.layout != ORC_LAYOUT_LINE)
      return o->status = ORC_ERR_CONFIG;
    for (int i = 0; i < o->nd; ++i) {
      double theta = orc_draw(o, ORC_TAG_INIT_DIMER, i, 0, 0, 0);
      theta = 2. * pi * theta;
      const double w = dcn + 2. * rc * cutoff;
      double cx, cy;
      if (grid) {
        const int64_t j = i / o->p.layout_cols + 1, k = i % o->p.layout_cols + 1;
        cx = 0.5 * (o->L[0] - w * cols - sep * (cols - 1)) + 0.5 * w + (double)(k - 1) * (w + sep);
        cy = 0.5 * (o->L[1] - (w + sep) * (rows - 1) - w) + 0.5 * w + (double)(j - 1) * (w + sep);
      } else {
        cx = 0.5 * sep + 0.5 * w + (double)i * (w + sep);
        cy = o->L[1] * 0.5;
      }
      double* X1 = o->dpos + 3 * (2 * i);
      double* X2 = o->dpos + 3 * (2 * i + 1);
      X1[0] = cx + 0.5 * dcn * cos(theta); X1[1] = cy + 0.5 * dcn * sin(theta); X1[2] = o->p.tether_z;
      X2[0] = cx - 0.5 * dcn * cos(theta); X2[1] = cy - 0.5 * dcn * sin(theta); X2[2] = o->p.tether_z;
    }
  }
  for (int i = 0; i < o->nd && o->p.layout == ORC_LAYOUT_RANDOM; ++i) {
    int64_t a;
    for (a = 0; a < max_attempts; ++a) {
      double ux = orc_draw(o, ORC_TAG_INIT_DIMER, i, (uint32_t)a, 0, 0);
      double uy = orc_draw(o, ORC_TAG_INIT_DIMER, i, (uint32_t)a, 0, 1);
      double uz = orc_draw(o, ORC_TAG_INIT_DIMER, i, (uint32_t)a, 1, 0);
      double uphi = orc_draw(o, ORC_TAG_INIT_DIMER, i, (uint32_t)a, 1, 1);
      double uth = orc_draw(o, ORC_TAG_INIT_DIMER, i, (uint32_t)a, 2, 0);
      double phi = 2.0 * pi * uphi;
      double theta = 2.0 * uth - 1.0;
      if (o->p.init_plane) { uz = 0.5; theta = 0.0; }
      double s = sqrt(1.0 - theta * theta);
      double X1 = o->L[0] * ux + 0.5 * dcn * (s * cos(phi));
      double Y1 = o->L[1] * uy + 0.5 * dcn * (s * sin(phi));
      double Z1 = o->L[2] * uz + 0.5 * dcn * theta;
      double X2 = o->L[0] * ux - 0.5 * dcn * (s * cos(phi));
      double Y2 = o->L[1] * uy - 0.5 * dcn * (s * sin(phi));
      double Z2 = o->L[2] * uz - 0.5 * dcn * theta;
      X1 = wrap_floor(X1, o->L[0]); Y1 = wrap_floor(Y1, o->L[1]);
      X2 = wrap_floor(X2, o->L[0]); Y2 = wrap_floor(Y2, o->L[1]);
      if (periodic) { Z1 = wrap_floor(Z1, o->L[2]); Z2 = wrap_floor(Z2, o->L[2]); }
      double P[2][3] = {{X1, Y1, Z1}, {X2, Y2, Z2}};
      int bad = 0;
      if (!periodic && !o->p.init_plane) {
        bad = Z1 < sqrt(wcC2) + rc * cut || Z1 > o->L[2] - sqrt(wcC2) - rc * cut ||
              Z2 < sqrt(wcN2) + rn * cut || Z2 > o->L[2] - sqrt(wcN2) - rn * cut;
      }
      for (int j = 0; j < i && !bad; ++j) {
        for (int u = 0; u < 2 && !bad; ++u)
          for (int v = 0; v < 2 && !bad; ++v) {
            double d[3];
            for (int c = 0; c < 3; ++c) d[c] = P[u][c] - o->dpos[3 * (2 * j + v) + c];
            /* minimum image in the periodic directions (initial_mod.f95:108-111
             * compares raw differences, which lets dimers overlap across the
             * periodic x/y boundary) */
            for (int c = 0; c < (periodic ? 3 : 2); ++c) d[c] = pbc_d(d[c], o->L[c]);
            double r = (u == 0 ? rc : rn) + (v == 0 ? rc : rn);
            double lim = (r * cut) * (r * cut);
            if (u == 0 && v == 0) lim = (2. * rc * cut) * (2. * rc * cut);
            if (u == 1 && v == 1) lim = (2. * rn * cut) * (2. * rn * cut);
            if (d[0] * d[0] + d[1] * d[1] + d[2] * d[2] < lim) bad = 1;
          }
      }
      if (!bad) {
        for (int c = 0; c < 3; ++c) {
          o->dpos[3 * (2 * i) + c] = P[0][c];
          o->dpos[3 * (2 * i + 1) + c] = P[1][c];
        }
        break;
      }
    }
    if (a == max_attempts) return o->status = ORC_ERR_INIT;
  }

  /* species blocks in index order, positions rejected inside sphere cutoffs */
  int64_t bound[4], acc = 0;
  for (int c = 0; c < 4; ++c) { acc += o->p.init_count[c]; bound[c] = acc; }
  if (acc != o->nt) return o->status = ORC_ERR_CONFIG;
  int err = 0;
#pragma omp parallel for schedule(static) reduction(|:err) if (!mt)
  for (int64_t i = 0; i < o->nt; ++i) {
    int code = 0;
    while (code < 3 && i >= bound[code]) code++;
    o->flag[i] = code;
    int64_t a;
    for (a = 0; a < 1000000; ++a) {
      double ux = orc_draw(o, ORC_TAG_INIT_POS, (uint32_t)i, (uint32_t)a, 0, 0);
      double uy = orc_draw(o, ORC_TAG_INIT_POS, (uint32_t)i, (uint32_t)a, 0, 1);
      double uz = orc_draw(o, ORC_TAG_INIT_POS, (uint32_t)i, (uint32_t)a, 1, 0);
      o->x[i] = o->L[0] * ux;
      o->y[i] = o->L[1] * uy;
      o->z[i] = o->L[2] * uz;
      int bad = 0;
      for (int k = 0; k < o->nd && !bad; ++k) {
        double dR[3];
        if (sol_sphere_d(o, i, 2 * k, dR) < cutC2) bad = 1;
        else if (sol_sphere_d(o, i, 2 * k + 1, dR) < cutN2) bad = 1;
      }
      if (!bad) break;
    }
    if (a == 1000000) err = 1;
  }
  if (err) return o->status = ORC_ERR_INIT;

  for (int s = 0; s < 3 * o->ns; ++s) { o->dvel[s] = 0.; o->dfrc[s] = 0.; }
  set_midpoint_anchors(o);
  memset(o->owner, 0, (size_t)o->nt * 4);   /* linear_periodic_no_ci/initial_mod.f95:95,146 */
  memset(o->inc, 0, (size_t)o->nt);
  double* vel[3] = {o->vx, o->vy, o->vz};
  double sum[3] = {0., 0., 0.};
  if (mt) {
    /* reference draw order: per species block, component x, y, z */
    int64_t lo = 0;
    for (int c = 0; c < 4; ++c) {
      int64_t hi = bound[c];
      double var = o->p.kT / o->p.mass[c];
      for (int comp = 0; comp < 3; ++comp)
        for (int64_t i = lo; i < hi; ++i) {
          double xx = orc_draw(o, 0, 0, 0, 0, 0), yy = orc_draw(o, 0, 0, 0, 0, 0);
          double th = 2 * pi * xx, R = sqrt(-2 * log(yy));
          vel[comp][i] = sqrt(var) * (R * cos(th)) + 0.0;
        }
      lo = hi;
    }
  } else {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < o->nt; ++i) {
      double var = o->p.kT / o->p.mass[o->flag[i]];
      for (int comp = 0; comp < 3; ++comp) {
        double xx = orc_contract_u01(o->p.seed, ORC_TAG_INIT_VEL, (uint32_t)i, comp, 0, 0);
        double yy = 1.0 - orc_contract_u01(o->p.seed, ORC_TAG_INIT_VEL, (uint32_t)i, comp, 0, 1);
        double th = 2 * pi * xx, R = sqrt(-2 * log(yy));
        vel[comp][i] = sqrt(var) * (R * cos(th)) + 0.0;
      }
    }
  }
  for (int comp = 0; comp < 3; ++comp) {
    for (int64_t i = 0; i < o->nt; ++i) sum[comp] += vel[comp][i];
    sum[comp] = sum[comp] / (double)o->nt;
    for (int64_t i = 0; i < o->nt; ++i) vel[comp][i] = vel[comp][i] - sum[comp];
  }
  return ORC_OK;
}

/* ------------------------------------------------------------ prepare -- */
static void compute_time_penetrate(orc_t* o) {
  /* main_pattern.f95:187, evolve_mod.f95:555-563 */
  double maxt = o->vx[0] * o->vx[0] + o->vy[0] * o->vy[0] + o->vz[0] * o->vz[0];
  for (int64_t i = 0; i < o->nt; ++i) {
    double v = o->vx[i] * o->vx[i] + o->vy[i] * o->vy[i] + o->vz[i] * o->vz[i];
    if (v > maxt) maxt = v;
  }
  o->time_penetrate = (int32_t)floor((0.5 * o->p.skin / sqrt(maxt)) / o->p.md_dt);
}

int orc_prepare(orc_t* o) {
  /* main_pattern.f95:168-187 */
  reactive_grid_setup(o);
  if (o->p.sort_every > 0 && o->cstep % o->p.sort_every == 0) orc_sort(o);
  orc_rebuild_lists(o);
  for (int64_t i = 0; i < o->nt; ++i) o->msd[i] = 0.;
  for (int64_t j = 0; j < o->ns * o->maxnb * 3; ++j) o->fpair[j] = 0.;
  for (int64_t j = 0; j < o->ns * o->maxnb; ++j) o->pot[j] = 0.;
  compute_time_penetrate(o);
  o->time_count = 0;
  o->prepared = 1;
  return o->status;
}

/* restart_mod.f95:415-528: after the lists of a restart, the forces of the
 * restart state (pair forces for the first half kick, catalysis, sphere
 * totals); no kick. */
static void compute_forces(orc_t* o, int restart);
int orc_restart_forces(orc_t* o) {
  if (!o->prepared) return o->status = ORC_ERR_STATE;
  compute_forces(o, 1);
  return o->status;
}

/* ---------------------------------------------------------------- forces -- */
/* forces_mod.f95:6-140 (LJ_mot_sol) for sphere s over its list, with the
 * catalytic rule of the run (collective :79-92 or ForcesMD_SelkovDimer:302-339). */
static void lj_mot_sol(orc_t* o, int s) {
  const double cut = pow(2.0, 1.0 / 6.0);
  const int isC = (s % 2 == 0);
  const double R = isC ? o->p.rc : o->p.rn;
  const double cutoff2 = (R * cut) * (R * cut);
  double R6, R12, r6R6, r12R12;
  orc_lj_consts(R, &R6, &R12, &r6R6, &r12R12);
  const double* eps = isC ? o->p.eps_c : o->p.eps_n;
  int64_t base = (int64_t)s * o->maxnb;
  int64_t nn = o->nbnum[s];
  const int prob = o->p.catalysis == ORC_CAT_PROBABILISTIC;
  /* owner tags (linear_periodic_no_ci/forces_mod.f95:79-121): the C sphere
   * of motor k makes every particle in its cutoff a B of motor k; a B acts
   * as B only on the spheres of its own motor and as A on all others */
  const int tags = o->p.owner_tags;
  const int32_t motor = s / 2 + 1;
  for (int64_t j = 0; j < nn; ++j) {
    int64_t i = o->nb[base + j];
    double dR[3];
    double dRsq = sol_sphere_d(o, i, s, dR);
    if (dRsq <= cutoff2) {
      int f = o->flag[i];
      double E = eps[f & 3];
      if (tags && !isC && f == 1 && o->owner[i] != motor) E = eps[0];
      if (isC) {
        if (o->p.catalysis == ORC_CAT_ON_EXIT) {
          o->cnow[i] = 1;   /* converted, if at all, after every sphere's pairs (compute_forces) */
        } else if (!prob && tags) {
          o->flag[i] = 1; o->owner[i] = motor; E = eps[1];
        } else if (!prob) {
          if (f == 0) { o->flag[i] = 1; E = eps[1]; }
        } else {
          if (f == 0) {
            double u = orc_draw(o, ORC_TAG_CAT, (uint32_t)i, (uint32_t)s, (uint32_t)o->cstep, 0);
            if (o->p.rp_ab > u) o->flag[i] = 1;
            E = eps[0];
          } else if (f == 1) {
            double u = orc_draw(o, ORC_TAG_CAT, (uint32_t)i, (uint32_t)s, (uint32_t)o->cstep, 0);
            if (o->p.rp_ba > u) o->flag[i] = 0;
            E = eps[1];
          }
        }
      }
      double IdRsq = 1.0 / dRsq;
      double IdR6 = IdRsq * IdRsq * IdRsq;
      double IdR8 = IdR6 * IdRsq;
      double IdR12 = IdR6 * IdR6;
      double IdR14 = IdR12 * IdRsq;
      double Fbrack = 4.0 * (r12R12 * IdR14 - r6R6 * IdR8);
      double Ubrack = 4.0 * (R12 * IdR12 - R6 * IdR6) + 1.0;
      o->fpair[3 * (base + j) + 0] = E * Fbrack * dR[0];
      o->fpair[3 * (base + j) + 1] = E * Fbrack * dR[1];
      o->fpair[3 * (base + j) + 2] = E * Fbrack * dR[2];
      o->pot[base + j] = o->pot[base + j] + E * Ubrack;
    }
  }
}

/* forces_mod.f95:144-210 */
static void lj_mot_mot(const orc_t* o, int s1, int s2, double cutoff2, double Rx,
                       double F[3], double* pot) {
  double R6, R12, r6R6, r12R12;
  orc_lj_consts(Rx, &R6, &R12, &r6R6, &r12R12);
  double dR[3];
  for (int c = 0; c < 3; ++c) dR[c] = o->dpos[3 * s1 + c] - o->dpos[3 * s2 + c];
  dR[0] = pbc_d(dR[0], o->L[0]);
  dR[1] = pbc_d(dR[1], o->L[1]);
  if (o->p.geometry == ORC_GEOM_PERIODIC) dR[2] = pbc_d(dR[2], o->L[2]);
  double dRsq = dR[0] * dR[0] + dR[1] * dR[1] + dR[2] * dR[2];
  F[0] = F[1] = F[2] = 0.;
  *pot = 0.;
  if (dRsq <= cutoff2) {
    double IdRsq = 1.0 / dRsq;
    double IdR6 = IdRsq * IdRsq * IdRsq;
    double IdR8 = IdR6 * IdRsq;
    double IdR12 = IdR6 * IdR6;
    double IdR14 = IdR12 * IdRsq;
    double Fbrack = 4.0 * (r12R12 * IdR14 - r6R6 * IdR8);
    double Ubrack = 4.0 * (R12 * IdR12 - R6 * IdR6) + 1.0;
    F[0] = o->p.em * Fbrack * dR[0];
    F[1] = o->p.em * Fbrack * dR[1];
    F[2] = o->p.em * Fbrack * dR[2];
    *pot = o->p.em * Ubrack;
  }
}

/* forces_mod.f95:273-335 LJ_mot_wall, called as at evolve_mod.f95:597,600:
 * the actual arguments (R3, R9, 3R^3, 9R^9) bind to the dummies
 * (R3, R9, r9R9, r3R3), so the force uses 3R^3 where the dummy is named 9R^9
 * and vice versa.  The oracle keeps that binding. */
void orc_lj_mot_wall(double Lz, double zdim, double Ew, double Rw_plus_R,
                     double* fwallz, double* potential) {
  const double w3 = pow(3.0, (double)(1.0f / 6.0f));
  const double cutoff2 = (Rw_plus_R * w3) * (Rw_plus_R * w3);
  const double R3 = Rw_plus_R * Rw_plus_R * Rw_plus_R;
  const double R9 = R3 * R3 * R3;
  const double r9R9 = 3.0 * R3;  /* bound from the actual r3Rwc3 */
  const double r3R3 = 9.0 * R9;  /* bound from the actual r9Rwc9 */
  const double pref = 0.5 * 3. * sqrt(3.0);
  double dR = Lz - zdim;
  if (dR * dR < cutoff2) {
    double IdRsq = 1. / (dR * dR);
    double IdR3 = pow(IdRsq, 1.5);
    double IdR9 = IdR3 * IdR3 * IdR3;
    double IdR5 = IdR3 * IdRsq;
    double IdR11 = IdR9 * IdRsq;
    double Fbrack = pref * Ew * (r9R9 * IdR11 - r3R3 * IdR5);
    *fwallz = Fbrack * dR;
    *potential = pref * Ew * (R9 * IdR9 - R3 * IdR3) + 1.0;
  }
  dR = 0. - zdim;
  if (dR * dR < cutoff2) {
    double IdRsq = 1. / (dR * dR);
    double IdR3 = pow(IdRsq, 1.5);
    double IdR9 = IdR3 * IdR3 * IdR3;
    double IdR5 = IdR3 * IdRsq;
    double IdR11 = IdR9 * IdRsq;
    double Fbrack = pref * Ew * (r9R9 * IdR11 - r3R3 * IdR5);
    *fwallz = *fwallz + Fbrack * dR;
    *potential = *potential + pref * Ew * (R9 * IdR9 - R3 * IdR3) + 1.0;
  }
}

/* ------------------------------------------------------------- RATTLE -- */
/* evolve_mod.f95:325-415 for dimer k. */
static void rattle_positions(orc_t* o, int k) {
  const double dt = o->p.md_dt, Mc = o->p.mc, Mn = o->p.mn, Dcn = o->p.dcn;
  const double hIMc = (0.5 * dt) / Mc, hIMn = (0.5 * dt) / Mn;
  const double IIM = 1.0 / ((1.0 / Mc) + (1.0 / Mn));
  const int per = o->p.geometry == ORC_GEOM_PERIODIC;
  double* X1 = o->dpos + 3 * (2 * k);
  double* X2 = o->dpos + 3 * (2 * k + 1);
  double* V1 = o->dvel + 3 * (2 * k);
  double* V2 = o->dvel + 3 * (2 * k + 1);
  double* F1 = o->dfrc + 3 * (2 * k);
  double* F2 = o->dfrc + 3 * (2 * k + 1);
  double* Q1 = o->q + 3 * (2 * k);
  double* Q2 = o->q + 3 * (2 * k + 1);
  double pr1[3], pr2[3], dP[3];
  for (int c = 0; c < 3; ++c) { pr1[c] = X1[c]; pr2[c] = X2[c]; dP[c] = X1[c] - X2[c]; }
  for (int c = 0; c < (per ? 3 : 2); ++c) dP[c] = pbc_d(dP[c], o->L[c]);
  for (int c = 0; c < 3; ++c) { Q1[c] = V1[c] + hIMc * F1[c]; Q2[c] = V2[c] + hIMn * F2[c]; }
  for (int c = 0; c < 3; ++c) { X1[c] = X1[c] + dt * Q1[c]; X2[c] = X2[c] + dt * Q2[c]; }
  for (int c = 0; c < (per ? 3 : 2); ++c) {
    X1[c] = wrap_floor(X1[c], o->L[c]);
    X2[c] = wrap_floor(X2[c], o->L[c]);
  }
  int64_t acc = 0;
  for (;;) {
    double d[3];
    for (int c = 0; c < 3; ++c) d[c] = X1[c] - X2[c];
    for (int c = 0; c < (per ? 3 : 2); ++c) d[c] = pbc_d(d[c], o->L[c]);
    double Con1diff = (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) - Dcn * Dcn;
    if (fabs(Con1diff) < 1.e-6) break;
    if (acc == o->p.rattle_max_iter) { o->status = ORC_ERR_RATTLE; break; }
    double G = -(0.25 * Con1diff * IIM / (d[0] * dP[0] + d[1] * dP[1] + d[2] * dP[2]));
    for (int c = 0; c < 3; ++c) {
      X1[c] = pr1[c] + Q1[c] * dt + 2.0 * G * dP[c] / Mc;
      X2[c] = pr2[c] + Q2[c] * dt - 2.0 * G * dP[c] / Mn;
    }
    for (int c = 0; c < (per ? 3 : 2); ++c) {
      X1[c] = wrap_floor(X1[c], o->L[c]);
      X2[c] = wrap_floor(X2[c], o->L[c]);
    }
    for (int c = 0; c < 3; ++c) {
      Q1[c] = Q1[c] + 2.0 * G * dP[c] / (Mc * dt);
      Q2[c] = Q2[c] - 2.0 * G * dP[c] / (Mn * dt);
    }
    acc++;
  }
}

/* rotational_code/2d_array/evolve_mod.f95:283-391: RATTLE positions of an
 * anchored rotor.  Besides the bond, the midpoint 0.5 (X1 + X2) (wrapped
 * into the box in x and y) is held at the anchor motorCM(k): each iteration
 * adds the bond correction G dP / M and the anchor correction H / (2 M),
 * H = -4 IIM (midpoint - anchor), and wraps all three coordinates. */
static void rattle_positions_rotor(orc_t* o, int k) {
  const double dt = o->p.md_dt, Mc = o->p.mc, Mn = o->p.mn, Dcn = o->p.dcn;
  const double hIMc = (0.5 * dt) / Mc, hIMn = (0.5 * dt) / Mn;
  const double IIM = 1.0 / ((1.0 / Mc) + (1.0 / Mn));
  const int per = o->p.geometry == ORC_GEOM_PERIODIC;
  const double* A = o->anchor + 3 * k;
  double* X1 = o->dpos + 3 * (2 * k);
  double* X2 = o->dpos + 3 * (2 * k + 1);
  double* V1 = o->dvel + 3 * (2 * k);
  double* V2 = o->dvel + 3 * (2 * k + 1);
  double* F1 = o->dfrc + 3 * (2 * k);
  double* F2 = o->dfrc + 3 * (2 * k + 1);
  double* Q1 = o->q + 3 * (2 * k);
  double* Q2 = o->q + 3 * (2 * k + 1);
  double pr1[3], pr2[3], dP[3];
  for (int c = 0; c < 3; ++c) { pr1[c] = X1[c]; pr2[c] = X2[c]; dP[c] = X1[c] - X2[c]; }
  for (int c = 0; c < (per ? 3 : 2); ++c) dP[c] = pbc_d(dP[c], o->L[c]);
  for (int c = 0; c < 3; ++c) { Q1[c] = V1[c] + hIMc * F1[c]; Q2[c] = V2[c] + hIMn * F2[c]; }
  for (int c = 0; c < 3; ++c) { X1[c] = X1[c] + dt * Q1[c]; X2[c] = X2[c] + dt * Q2[c]; }
  for (int c = 0; c < (per ? 3 : 2); ++c) {
    X1[c] = wrap_floor(X1[c], o->L[c]);
    X2[c] = wrap_floor(X2[c], o->L[c]);
  }
  int64_t acc = 0;
  for (;;) {
    double d[3], D[3];
    for (int c = 0; c < 3; ++c) d[c] = X1[c] - X2[c];
    for (int c = 0; c < (per ? 3 : 2); ++c) d[c] = pbc_d(d[c], o->L[c]);
    for (int c = 0; c < 3; ++c) {
      double m = 0.5 * (X1[c] + X2[c]);
      if (c < 2) {
        if (m >= o->L[c]) m = m - o->L[c];
        else if (m < 0.) m = m + o->L[c];
      }
      D[c] = m - A[c];
    }
    double Con1diff = (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) - Dcn * Dcn;
    if ((fabs(Con1diff) < 1.e-6 && fabs(D[0]) < 1.e-6 && fabs(D[1]) < 1.e-6 && fabs(D[2]) < 1.e-6))
      break;
    if (acc == o->p.rattle_max_iter) { o->status = ORC_ERR_RATTLE; break; }
    double G = -(0.25 * Con1diff * IIM / (d[0] * dP[0] + d[1] * dP[1] + d[2] * dP[2]));
    double H[3];
    for (int c = 0; c < 3; ++c) H[c] = -(4.0 * IIM * D[c]);
    for (int c = 0; c < 3; ++c) {
      X1[c] = pr1[c] + Q1[c] * dt + G * dP[c] / Mc + 0.5 * H[c] / Mc;
      X2[c] = pr2[c] + Q2[c] * dt - G * dP[c] / Mn + 0.5 * H[c] / Mn;
    }
    for (int c = 0; c < 3; ++c) {
      X1[c] = wrap_floor(X1[c], o->L[c]);
      X2[c] = wrap_floor(X2[c], o->L[c]);
    }
    for (int c = 0; c < 3; ++c) {
      Q1[c] = Q1[c] + G * dP[c] / (Mc * dt) + 0.5 * H[c] / (Mc * dt);
      Q2[c] = Q2[c] - G * dP[c] / (Mn * dt) + 0.5 * H[c] / (Mn * dt);
    }
    acc++;
  }
}

/* rotational_code/2d_array/evolve_mod.f95:596-650: RATTLE velocities of an
 * anchored rotor: the bond constraint (without the factor 2 of the motor
 * form) and a zero midpoint velocity, P = -4 IIM (V1 + V2) / 2. */
static void rattle_velocities_rotor(orc_t* o, int k) {
  const double dt = o->p.md_dt, Mc = o->p.mc, Mn = o->p.mn, Dcn = o->p.dcn;
  const double hIMc = (0.5 * dt) / Mc, hIMn = (0.5 * dt) / Mn;
  const double IIM = 1.0 / ((1.0 / Mc) + (1.0 / Mn));
  const int per = o->p.geometry == ORC_GEOM_PERIODIC;
  double* X1 = o->dpos + 3 * (2 * k);
  double* X2 = o->dpos + 3 * (2 * k + 1);
  double* V1 = o->dvel + 3 * (2 * k);
  double* V2 = o->dvel + 3 * (2 * k + 1);
  double* F1 = o->dfrc + 3 * (2 * k);
  double* F2 = o->dfrc + 3 * (2 * k + 1);
  double* Q1 = o->q + 3 * (2 * k);
  double* Q2 = o->q + 3 * (2 * k + 1);
  for (int c = 0; c < 3; ++c) { V1[c] = Q1[c] + hIMc * F1[c]; V2[c] = Q2[c] + hIMn * F2[c]; }
  int64_t acc = 0;
  for (;;) {
    double dV[3], d[3], Vm[3];
    for (int c = 0; c < 3; ++c) { dV[c] = V1[c] - V2[c]; d[c] = X1[c] - X2[c]; }
    for (int c = 0; c < (per ? 3 : 2); ++c) d[c] = pbc_d(d[c], o->L[c]);
    double Con2diff = dV[0] * d[0] + dV[1] * d[1] + dV[2] * d[2];
    for (int c = 0; c < 3; ++c) Vm[c] = 0.5 * (V1[c] + V2[c]);
    if (fabs(Con2diff) < 1.e-8 && fabs(Vm[0]) < 1.e-8 && fabs(Vm[1]) < 1.e-8 && fabs(Vm[2]) < 1.e-8) break;
    if (acc == o->p.rattle_max_iter) { o->status = ORC_ERR_RATTLE; break; }
    double O = -(0.25 * (IIM * Con2diff) / (Dcn * Dcn));
    double P[3];
    for (int c = 0; c < 3; ++c) P[c] = -(4.0 * Vm[c] * IIM);
    for (int c = 0; c < 3; ++c) {
      V1[c] = V1[c] + O * d[c] / Mc + 0.5 * P[c] / Mc;
      V2[c] = V2[c] - O * d[c] / Mn + 0.5 * P[c] / Mn;
    }
    acc++;
  }
}

/* rotational_code/2d_array/forces_mod.f95:177-201: harmonic z tether. */
void orc_harmonic_tether(double zdim, double zdimeq, double k_harm, double* f, double* pot) {
  const double zdiff = zdim - zdimeq;
  *f = -1. * k_harm * zdiff;
  *pot = 0.5 * k_harm * (zdiff * zdiff);
}

/* evolve_mod.f95:679-724 for dimer k. */
static void rattle_velocities(orc_t* o, int k) {
  const double dt = o->p.md_dt, Mc = o->p.mc, Mn = o->p.mn, Dcn = o->p.dcn;
  const double hIMc = (0.5 * dt) / Mc, hIMn = (0.5 * dt) / Mn;
  const double IIM = 1.0 / ((1.0 / Mc) + (1.0 / Mn));
  const int per = o->p.geometry == ORC_GEOM_PERIODIC;
  double* X1 = o->dpos + 3 * (2 * k);
  double* X2 = o->dpos + 3 * (2 * k + 1);
  double* V1 = o->dvel + 3 * (2 * k);
  double* V2 = o->dvel + 3 * (2 * k + 1);
  double* F1 = o->dfrc + 3 * (2 * k);
  double* F2 = o->dfrc + 3 * (2 * k + 1);
  double* Q1 = o->q + 3 * (2 * k);
  double* Q2 = o->q + 3 * (2 * k + 1);
  for (int c = 0; c < 3; ++c) { V1[c] = Q1[c] + hIMc * F1[c]; V2[c] = Q2[c] + hIMn * F2[c]; }
  int64_t acc = 0;
  for (;;) {
    double dV[3], d[3];
    for (int c = 0; c < 3; ++c) { dV[c] = V1[c] - V2[c]; d[c] = X1[c] - X2[c]; }
    for (int c = 0; c < (per ? 3 : 2); ++c) d[c] = pbc_d(d[c], o->L[c]);
    double Con2diff = 2.0 * (dV[0] * d[0] + dV[1] * d[1] + dV[2] * d[2]);
    if (fabs(Con2diff) < 1.e-8) break;
    if (acc == o->p.rattle_max_iter) { o->status = ORC_ERR_RATTLE; break; }
    double O = -(0.25 * (IIM * Con2diff) / (Dcn * Dcn));
    for (int c = 0; c < 3; ++c) {
      V1[c] = V1[c] + 2.0 * O * d[c] / Mc;
      V2[c] = V2[c] - 2.0 * O * d[c] / Mn;
    }
    acc++;
  }
}

/* ---------------------------------------------------------------- evolve -- */
static void kick_lists(orc_t* o) {
  /* evolve_mod.f95:225-250 and :645-670 */
  double hIM[4];
  for (int c = 0; c < 4; ++c) hIM[c] = (0.5 * o->p.md_dt) / o->p.mass[c];
  for (int s = 0; s < o->ns; ++s) {
    int64_t base = (int64_t)s * o->maxnb;
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < o->nbnum[s]; ++j) {
      int64_t i = o->nb[base + j];
      double h = hIM[o->flag[i] & 3];
      o->vx[i] = o->vx[i] + h * o->fpair[3 * (base + j) + 0];
      o->vy[i] = o->vy[i] + h * o->fpair[3 * (base + j) + 1];
      o->vz[i] = o->vz[i] + h * o->fpair[3 * (base + j) + 2];
    }
  }
}

/* evolve_mod.f95:441-452 (pair forces of the lists in use cleared), :567-602
 * (sphere-solvent LJ with catalysis, motor-motor LJ, the wall, or the rotor
 * tether of rotational_code/2d_array/evolve_mod.f95:515-531) and :605-636
 * (sphere totals and the potential); restart_mod.f95:415-528 runs the same
 * evaluation at a restart. */
static void compute_forces(orc_t* o, int restart) {
  const double cut = pow(2.0, 1.0 / 6.0);
  const int rotor = o->p.variant == ORC_VARIANT_ROTOR;
  for (int j = 0; j < 3 * o->ns; ++j) o->dfrc[j] = 0.;
  o->tpot = 0.;
  /* clear pair forces for the lists in use */
  for (int s = 0; s < o->ns; ++s) {
    int64_t base = (int64_t)s * o->maxnb;
    for (int64_t j = 0; j < o->nbnum[s]; ++j) {
      o->fpair[3 * (base + j) + 0] = 0.;
      o->fpair[3 * (base + j) + 1] = 0.;
      o->fpair[3 * (base + j) + 2] = 0.;
      o->pot[base + j] = 0.;
    }
  }
  /* forces :567-602 */
  const double mcc2 = ((o->p.rc + o->p.rc + o->p.rm_delta) * cut) * ((o->p.rc + o->p.rc + o->p.rm_delta) * cut);
  const double mcn2 = ((o->p.rc + o->p.rn + o->p.rm_delta) * cut) * ((o->p.rc + o->p.rn + o->p.rm_delta) * cut);
  const double mnn2 = ((o->p.rn + o->p.rn + o->p.rm_delta) * cut) * ((o->p.rn + o->p.rn + o->p.rm_delta) * cut);
  double* fmot = calloc((size_t)o->ns * o->ns * 3 + 1, 8);
  double* fmotpot = calloc((size_t)o->ns * o->ns + 1, 8);
  double* fwall = calloc((size_t)o->ns + 1, 8);
  double* wpot = calloc((size_t)o->ns + 1, 8);
  for (int k = 0; k < o->nd; ++k) {
    lj_mot_sol(o, 2 * k);
    lj_mot_sol(o, 2 * k + 1);
    /* the rotor variant has no motor-motor LJ and a harmonic tether in place
     * of the wall (rotational_code/2d_array/evolve_mod.f95:515-531) */
    if (rotor) {
      orc_harmonic_tether(o->dpos[3 * (2 * k) + 2], o->p.tether_z, o->p.tether_k, &fwall[2 * k], &wpot[2 * k]);
      orc_harmonic_tether(o->dpos[3 * (2 * k + 1) + 2], o->p.tether_z, o->p.tether_k, &fwall[2 * k + 1],
                          &wpot[2 * k + 1]);
      continue;
    }
    for (int j = 0; j < o->nd; ++j) {
      if (j == k) continue;
      for (int i = 0; i < 2; ++i)
        for (int l = 0; l < 2; ++l) {
          int sa = 2 * k + i, sb = 2 * j + l;
          double c2 = (i == 0 && l == 0) ? mcc2 : ((i == 1 && l == 1) ? mnn2 : mcn2);
          double Rx = (i == 0 ? o->p.rc : o->p.rn) + (l == 0 ? o->p.rc : o->p.rn) + o->p.rm_delta;
          lj_mot_mot(o, sa, sb, c2, Rx, fmot + 3 * ((size_t)sa * o->ns + sb), fmotpot + (size_t)sa * o->ns + sb);
        }
    }
    if (o->p.geometry == ORC_GEOM_WALLS) {
      orc_lj_mot_wall(o->L[2], o->dpos[3 * (2 * k) + 2], o->p.ew, o->p.rw + o->p.rc, &fwall[2 * k], &wpot[2 * k]);
      orc_lj_mot_wall(o->L[2], o->dpos[3 * (2 * k + 1) + 2], o->p.ew, o->p.rw + o->p.rn, &fwall[2 * k + 1], &wpot[2 * k + 1]);
    }
  }
  /* catalysis on exit: an A inside a C cutoff at the last evaluation and
   * outside every C cutoff at this one becomes a B (each C-list member once;
   * a restart's evaluation records the state only) */
  if (o->p.catalysis == ORC_CAT_ON_EXIT) {
    for (int s = 0; s < o->ns; s += 2) {
      const int64_t base = (int64_t)s * o->maxnb;
      for (int64_t j = 0; j < o->nbnum[s]; ++j) {
        const int64_t i = o->nb[base + j];
        if (o->cnow[i] == 2) continue;
        if (!restart && o->inc[i] && o->cnow[i] == 0 && (o->flag[i] & 3) == 0) o->flag[i] = 1;
        o->inc[i] = o->cnow[i] == 1;
        o->cnow[i] = 2;
      }
    }
    for (int s = 0; s < o->ns; s += 2) {
      const int64_t base = (int64_t)s * o->maxnb;
      for (int64_t j = 0; j < o->nbnum[s]; ++j) o->cnow[o->nb[base + j]] = 0;
    }
  }
  /* totals :605-636 */
  for (int k = 0; k < o->nd; ++k)
    for (int i = 0; i < 2; ++i) {
      int s = 2 * k + i;
      int64_t base = (int64_t)s * o->maxnb;
      double tp = 0.;
      double* F = o->dfrc + 3 * s;
      for (int64_t j = 0; j < o->nbnum[s]; ++j) {
        tp = tp + o->pot[base + j];
        F[0] = F[0] - o->fpair[3 * (base + j) + 0];
        F[1] = F[1] - o->fpair[3 * (base + j) + 1];
        F[2] = F[2] - o->fpair[3 * (base + j) + 2];
      }
      for (int j = 0; j < o->nd; ++j)
        for (int l = 0; l < 2; ++l) {
          int sb = 2 * j + l;
          const double* fm = fmot + 3 * ((size_t)s * o->ns + sb);
          F[0] = F[0] + fm[0];
          F[1] = F[1] + fm[1];
          F[2] = F[2] + fm[2];
          if (j < k) tp = tp + fmotpot[(size_t)s * o->ns + sb];
        }
      F[2] = F[2] + fwall[s];
      tp = tp + wpot[s];
      o->tpot += tp;
    }
  free(fmot); free(fmotpot); free(fwall); free(wpot);
}

static void evolve(orc_t* o) {
  const double dt = o->p.md_dt;
  const double cut = pow(2.0, 1.0 / 6.0);
  kick_lists(o);
  /* stream inside particles :258-315 */
#pragma omp parallel for schedule(static)
  for (int64_t j = 0; j < o->n_in; ++j) {
    int64_t i = o->in_list[j];
    stream_particle(o, i, dt, 1, 0);
    o->msd[i] = o->msd[i] + (o->vx[i] * o->vx[i] + o->vy[i] * o->vy[i] + o->vz[i] * o->vz[i]) * (dt * dt);
  }
  /* RATTLE positions :320-417 */
  const int rotor = o->p.variant == ORC_VARIANT_ROTOR;
  for (int k = 0; k < o->nd; ++k) {
    if (rotor) rattle_positions_rotor(o, k);
    else rattle_positions(o, k);
  }
  /* (sphere forces :424-455 are zeroed by compute_forces) */
  /* rebuild test :457-465 */
  double maxv = o->msd[0];
  for (int64_t i = 0; i < o->nt; ++i) if (o->msd[i] > maxv) maxv = o->msd[i];
  int mpc_step = (o->cstep % o->p.mpc_every) == 0;
  if (maxv > (0.5 * o->p.skin) * (0.5 * o->p.skin) || o->time_count == o->time_penetrate || mpc_step) {
#pragma omp parallel for schedule(static)
    for (int64_t j = 0; j < o->n_out; ++j) stream_particle(o, o->out_list[j], dt, o->time_count, 1);
    if (o->p.sort_every > 0 && o->cstep % o->p.sort_every == 0) orc_sort(o);
    orc_rebuild_lists(o);
    for (int64_t i = 0; i < o->nt; ++i) o->msd[i] = 0.;
    compute_time_penetrate(o);
    o->time_count = 0;
    o->n_rebuilds++;
  }
  compute_forces(o, 0);
  kick_lists(o);
  for (int k = 0; k < o->nd; ++k) {
    if (rotor) rattle_velocities_rotor(o, k);
    else rattle_velocities(o, k);
  }
}

/* ------------------------------------------------------------ distribute -- */
/* Affected_Cell.f90:7-101 for every sphere (C with the C cutoff, N with N). */
static void affected_cells(orc_t* o) {
  const double cut = pow(2.0, 1.0 / 6.0);
  for (int64_t c = 0; c < o->ncell; ++c) o->affected[c] = 0;
  const int iB[3] = {o->p.lx, o->p.ly, o->p.lz};
  for (int s = 0; s < o->ns; ++s) {
    double R = (s % 2 == 0) ? o->p.rc : o->p.rn;
    double co = R * cut, co2 = co * co;
    const double* X = o->dpos + 3 * s;
    int lo[3], up[3];
    for (int c = 0; c < 3; ++c) {
      lo[c] = (int)ceil(X[c] - (co + 1.0));
      up[c] = (int)floor(X[c] + (co + 1.0));
    }
    for (int i = lo[0]; i <= up[0]; ++i)
      for (int j = lo[1]; j <= up[1]; ++j)
        for (int k = lo[2]; k <= up[2]; ++k) {
          double a = fabs((double)(float)i - X[0]) - 1.0;
          double b = fabs((double)(float)j - X[1]) - 1.0;
          double d = fabs((double)(float)k - X[2]) - 1.0;
          if (a * a + b * b + d * d < co2) {
            int cc[3] = {i, j, k};
            for (int q = 0; q < 3; ++q) {
              if (cc[q] < 0) cc[q] += iB[q];
              else if (cc[q] >= iB[q]) cc[q] -= iB[q];
            }
            o->affected[cc[0] + (int64_t)iB[0] * cc[1] + (int64_t)iB[0] * iB[1] * cc[2]] = 1;
          }
        }
  }
}

static inline int bin_particle(orc_t* o, int64_t i) {
  int64_t c = clamp_cell(o, cell_of(o, o->x[i], o->y[i], o->z[i]));
  int sp = o->flag[i] & 3;
  int32_t* cnt = &o->dcount[4 * c + sp];
  if (*cnt == 0) o->dfirst[4 * c + sp] = i;
  (*cnt)++;
  return *cnt > o->p.cell_capacity;
}

/* distribute_mod.f95:6-205 (exclusion PARTICLE: outside list then bulk members
 * of the inside list) or Distribute_SelkovDimer.f90:7-37 + Affected_Cell.f90
 * (exclusion CELLS: every particle in index order). */
int orc_distribute(orc_t* o) {
  const double cut = pow(2.0, 1.0 / 6.0);
  const double cutC2 = (o->p.rc * cut) * (o->p.rc * cut);
  const double cutN2 = (o->p.rn * cut) * (o->p.rn * cut);
  for (int64_t j = 0; j < 4 * o->ncell; ++j) { o->dcount[j] = 0; o->dfirst[j] = -1; }
  int over = 0;
  if (o->p.exclusion == ORC_EXCL_CELLS) {
    for (int64_t i = 0; i < o->nt; ++i) over |= bin_particle(o, i);
    affected_cells(o);
  } else {
    for (int64_t j = 0; j < o->n_out; ++j) over |= bin_particle(o, o->out_list[j]);
    for (int64_t j = 0; j < o->n_in; ++j) {
      int64_t i = o->in_list[j];
      int bulk = 1;
      for (int k = 0; k < o->nd; ++k) {
        double dR[3];
        if (sol_sphere_d(o, i, 2 * k, dR) <= cutC2 || sol_sphere_d(o, i, 2 * k + 1, dR) <= cutN2) bulk = 0;
      }
      if (bulk) over |= bin_particle(o, i);
    }
    for (int64_t c = 0; c < o->ncell; ++c) o->affected[c] = 0;
  }
  if (over) o->status = ORC_ERR_CELL_OVERFLOW;
  return o->status;
}

int orc_get_distribute(const orc_t* o, int32_t* counts, int64_t* first) {
  if (counts) memcpy(counts, o->dcount, 4 * o->ncell * 4);
  if (first) memcpy(first, o->dfirst, 4 * o->ncell * 8);
  return ORC_OK;
}

int orc_get_affected(const orc_t* o, int32_t* affected) {
  memcpy(affected, o->affected, o->ncell * 4);
  return ORC_OK;
}

/* ------------------------------------------------------- mpc rotation -- */
/* mpc_rotation_mod.f95:6-239 (rotation_sense +1) or RMPC_SelkovDimer.f90:15-120
 * (rotation_sense -1: periodic shift, reciprocal CM, projection form). */
int orc_mpc_rotation(orc_t* o) {
  const double pi = 4.0 * atan(1.0);
  const double sinrot = sin(o->p.rot_angle), cosrot = cos(o->p.rot_angle);
  const double Lx = o->L[0], Ly = o->L[1], Lz = o->L[2];
  const int64_t C = o->ncell_shift;
  const uint32_t step = (uint32_t)o->cstep;
  const int walls = o->p.geometry == ORC_GEOM_WALLS;
  const int selkov = o->p.rotation_sense < 0;
  double* sx = calloc(C, 8);
  double* sy = calloc(C, 8);
  double* sz = calloc(C, 8);
  if (!sx || !sy || !sz) { free(sx); free(sy); free(sz); return o->status = ORC_ERR_ALLOC; }
  double a0 = 1.0;
  double Xs = o->shift[0] = a0 * (orc_draw(o, ORC_TAG_SHIFT, 0, 0, step, 0) - 0.5);
  double Ys = o->shift[1] = a0 * (orc_draw(o, ORC_TAG_SHIFT, 0, 0, step, 1) - 0.5);
  double Zs = o->shift[2] = a0 * (orc_draw(o, ORC_TAG_SHIFT, 0, 1, step, 0) - 0.5);
  for (int64_t c = 0; c < C; ++c) o->ccount[c] = 0;
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < o->nt; ++i) {
    double xs = o->x[i] + Xs;
    xs = xs - Lx * floor(xs / Lx);
    double ys = o->y[i] + Ys;
    ys = ys - Ly * floor(ys / Ly);
    double zs = o->z[i] + Zs;
    double cell;
    if (walls) {
      if (Zs < 0) cell = floor(xs) + Lx * floor(ys) + Lx * Ly * floor(zs + 1);
      else cell = floor(xs) + Lx * floor(ys) + Lx * Ly * floor(zs);
    } else {
      zs = zs - Lz * floor(zs / Lz);
      cell = floor(xs) + Lx * floor(ys) + Lx * Ly * floor(zs);
    }
    o->newcell[i] = (int64_t)cell;
  }
  for (int64_t i = 0; i < o->nt; ++i) {
    int64_t c = o->newcell[i];
    o->ccount[c]++;
    sx[c] = sx[c] + o->vx[i];
    sy[c] = sy[c] + o->vy[i];
    sz[c] = sz[c] + o->vz[i];
  }
#pragma omp parallel for schedule(static)
  for (int64_t c = 0; c < C; ++c) {
    double vx = sx[c], vy = sy[c], vz = sz[c];
    if (o->ccount[c] != 0) {
      if (selkov) {
        double inv = 1.0 / (double)o->ccount[c];
        vx = vx * inv; vy = vy * inv; vz = vz * inv;
      } else {
        vx = vx / (double)o->ccount[c];
        vy = vy / (double)o->ccount[c];
        vz = vz / (double)o->ccount[c];
      }
    }
    o->cm[3 * c + 0] = vx; o->cm[3 * c + 1] = vy; o->cm[3 * c + 2] = vz;
    if (o->rng_mode != ORC_RNG_MT) {
      double u1 = orc_contract_u01(o->p.seed, ORC_TAG_AXIS, (uint32_t)c, 0, step, 0);
      double u2 = orc_contract_u01(o->p.seed, ORC_TAG_AXIS, (uint32_t)c, 0, step, 1);
      double phi = 2.0 * pi * u1;
      double theta = 2.0 * u2 - 1.0;
      o->axis[3 * c + 0] = sqrt(1.0 - theta * theta) * cos(phi);
      o->axis[3 * c + 1] = sqrt(1.0 - theta * theta) * sin(phi);
      o->axis[3 * c + 2] = theta;
    }
  }
  if (o->rng_mode == ORC_RNG_MT) {
    for (int64_t c = 0; c < C; ++c) {
      double u1 = orc_draw(o, 0, 0, 0, 0, 0), u2 = orc_draw(o, 0, 0, 0, 0, 0);
      double phi = 2.0 * pi * u1, theta = 2.0 * u2 - 1.0;
      o->axis[3 * c + 0] = sqrt(1.0 - theta * theta) * cos(phi);
      o->axis[3 * c + 1] = sqrt(1.0 - theta * theta) * sin(phi);
      o->axis[3 * c + 2] = theta;
    }
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < o->nt; ++i) {
    int64_t c = o->newcell[i];
    const double* cm = o->cm + 3 * c;
    const double ux = o->axis[3 * c + 0], uy = o->axis[3 * c + 1], uz = o->axis[3 * c + 2];
    double dx = o->vx[i] - cm[0], dy = o->vy[i] - cm[1], dz = o->vz[i] - cm[2];
    double rx, ry, rz;
    if (!selkov) {
      rx = dx * (cosrot + ux * ux * (1.0 - cosrot)) + dy * (ux * uy * (1.0 - cosrot) - uz * sinrot) +
           dz * (ux * uz * (1.0 - cosrot) + uy * sinrot);
      ry = dx * (ux * uy * (1.0 - cosrot) + uz * sinrot) + dy * (cosrot + uy * uy * (1.0 - cosrot)) +
           dz * (uy * uz * (1.0 - cosrot) - ux * sinrot);
      rz = dx * (ux * uz * (1.0 - cosrot) - uy * sinrot) + dy * (uy * uz * (1.0 - cosrot) + ux * sinrot) +
           dz * (cosrot + uz * uz * (1.0 - cosrot));
    } else {
      double P = dx * ux + dy * uy + dz * uz;
      double px = P * ux, py = P * uy, pz = P * uz;
      double ox = dx - px, oy = dy - py, oz = dz - pz;
      double qx = (oy * uz) - (oz * uy);
      double qy = (oz * ux) - (ox * uz);
      double qz = (ox * uy) - (oy * ux);
      rx = px + ox * cosrot + qx * sinrot;
      ry = py + oy * cosrot + qy * sinrot;
      rz = pz + oz * cosrot + qz * sinrot;
    }
    o->vx[i] = cm[0] + rx;
    o->vy[i] = cm[1] + ry;
    o->vz[i] = cm[2] + rz;
  }
  free(sx); free(sy); free(sz);
  return ORC_OK;
}

int64_t orc_n_cells_shifted(const orc_t* o) { return o->ncell_shift; }

int orc_get_new_cell(const orc_t* o, int64_t* newcell) {
  memcpy(newcell, o->newcell, o->nt * 8);
  return ORC_OK;
}

int orc_get_cell_rotation(const orc_t* o, double* cm, double* axis, int32_t* count) {
  if (cm) memcpy(cm, o->cm, 3 * o->ncell_shift * 8);
  if (axis) memcpy(axis, o->axis, 3 * o->ncell_shift * 8);
  if (count) memcpy(count, o->ccount, o->ncell_shift * 4);
  return ORC_OK;
}

int orc_get_shift(const orc_t* o, double* shift) {
  shift[0] = o->shift[0]; shift[1] = o->shift[1]; shift[2] = o->shift[2];
  return ORC_OK;
}

/* ------------------------------------------------------------- reaction -- */
/* Selkov six-channel RKMPC for one cell, RMPC_SelkovDimer.f90:132-321, written
 * as the first cumulative propensity interval containing a00*x1 (zero
 * channels leave the running sums unchanged, which reproduces the nested
 * branches of the Fortran exactly). */
void orc_selkov_cell(const double k[6], double tau, int32_t nF, int32_t nG, int32_t nI,
                     double x1, double x2, int* channel) {
  double a1 = k[0];
  double a2 = k[1] * (double)nF;
  double a5 = k[4] * (double)nG;
  double a6 = k[5];
  double a3 = (nG == 0) ? 0. : k[2] * (double)nF * (double)nG * (double)(nG - 1);
  double a4 = (nG <= 1) ? 0. : k[3] * (double)nG * (double)(nG - 1) * (double)(nG - 2);
  if (nI == 0) { a1 = 0.; a6 = 0.; }
  double a00 = a1 + a2 + a3 + a4 + a5 + a6;
  double prob = 1 - exp(-a00 * tau);
  double a0rand = a00 * x1;
  *channel = 0;
  if (!(prob > x2)) return;
  if (nI == 0 && nF == 0 && nG == 0) return;
  double a[6] = {a1, a2, a3, a4, a5, a6};
  double cum = 0.;
  for (int c = 0; c < 6; ++c) {
    cum = cum + a[c];
    if (a[c] != 0. && a0rand < cum) { *channel = c + 1; return; }
  }
}

int orc_reaction(orc_t* o) {
  const uint32_t step = (uint32_t)o->cstep;
  const double tau = o->p.mpc_dt;
  if (o->p.kinetics == ORC_KIN_SIMPLE) {
    /* reaction_mod.f95:8-66 */
    for (int64_t c = 0; c < o->ncell; ++c) {
      int32_t nB = o->dcount[4 * c + 1];
      double a1 = (nB == 0) ? 0. : o->p.k[0] * (double)nB;
      double a00 = a1;
      double prob1 = 1.0 - exp(-a00 * tau);
      double u = orc_draw(o, ORC_TAG_RXN, (uint32_t)c, 0, step, 0);
      if (0. < u && u <= prob1) {
        o->flag[o->dfirst[4 * c + 1]] = 0;
        o->owner[o->dfirst[4 * c + 1]] = 0;   /* linear_periodic_no_ci/reaction_simple_mod.f95:55 */
      }
    }
  } else if (o->p.kinetics == ORC_KIN_SELKOV) {
    static const int target_species[7] = {-1, 3, 0, 0, 1, 1, 3};
    static const int new_code[7] = {-1, 0, 3, 1, 0, 3, 1};
    for (int64_t c = 0; c < o->ncell; ++c) {
      if (o->affected[c] != 0) continue;
      double x1 = orc_draw(o, ORC_TAG_RXN, (uint32_t)c, 0, step, 0);
      double x2 = orc_draw(o, ORC_TAG_RXN, (uint32_t)c, 0, step, 1);
      int ch;
      orc_selkov_cell(o->p.k, tau, o->dcount[4 * c + 0], o->dcount[4 * c + 1],
                      o->dcount[4 * c + 3], x1, x2, &ch);
      if (ch > 0) {
        int64_t who = o->dfirst[4 * c + target_species[ch]];
        if (who >= 0) o->flag[who] = new_code[ch];
      }
    }
  }
  return o->status;
}

/* ----------------------------------------------------------- the driver -- */
int orc_step(orc_t* o) {
  /* main_pattern.f95:203-225 */
  if (!o->prepared) return o->status = ORC_ERR_STATE;
  o->cstep = o->cstep + 1;
  o->time_count = o->time_count + 1;
  evolve(o);
  if (o->cstep % o->p.mpc_every == 0) {
    orc_distribute(o);
    orc_mpc_rotation(o);
    orc_reaction(o);
  }
  return o->status;
}

int orc_run(orc_t* o, int64_t nsteps) {
  for (int64_t s = 0; s < nsteps; ++s) {
    int st = orc_step(o);
    if (st != ORC_OK) return st;
  }
  return o->status;
}

/* ----------------------------------------------------------- observables -- */
int orc_observables(const orc_t* o, orc_obs* out) {
  memset(out, 0, sizeof(*out));
  double p[3] = {0, 0, 0}, ke = 0;
  for (int64_t i = 0; i < o->nt; ++i) {
    double m = o->p.mass[o->flag[i] & 3];
    p[0] += m * o->vx[i]; p[1] += m * o->vy[i]; p[2] += m * o->vz[i];
    ke += 0.5 * m * (o->vx[i] * o->vx[i] + o->vy[i] * o->vy[i] + o->vz[i] * o->vz[i]);
    out->species_count[o->flag[i] & 3]++;
  }
  double pd[3] = {0, 0, 0}, ked = 0;
  for (int s = 0; s < o->ns; ++s) {
    double m = (s % 2 == 0) ? o->p.mc : o->p.mn;
    for (int c = 0; c < 3; ++c) {
      pd[c] += m * o->dvel[3 * s + c];
      ked += 0.5 * m * o->dvel[3 * s + c] * o->dvel[3 * s + c];
    }
  }
  for (int c = 0; c < 3; ++c) { out->solvent_momentum[c] = p[c]; out->momentum[c] = p[c] + pd[c]; }
  out->kinetic_solvent = ke;
  out->kinetic_dimer = ked;
  out->potential = o->tpot;
  out->n_inside = o->n_in;
  int64_t np = 0;
  for (int s = 0; s < o->ns; ++s) np += o->nbnum[s];
  out->n_pairs = np;
  out->time_count = o->time_count;
  out->time_penetrate = o->time_penetrate;
  out->cstep = o->cstep;
  return ORC_OK;
}

/* ------------------------------------------------- concentration fields -- */
/* output_mod.f95:482-575: TotA/TotB over the whole box, then A and B counted
 * in a z slab (1D along x, 2D in x-y), a y slab (x-z) and an x slab (y-z) of
 * half thickness prm[3] around prm[0..2], bin = ceiling(u / width), divided
 * by the bin volume.  A coordinate of exactly 0 (bin 0 in the reference,
 * outside its arrays) is counted in bin 1; indices above the last bin are
 * clamped to it. */
static int64_t conc_bin(double u, double w, int64_t nb) {
  int64_t j = (int64_t)ceil(u / w);
  if (j < 1) j = 1;
  if (j > nb) j = nb;
  return j - 1;
}

int orc_concentration(int64_t n, const double* x, const double* y, const double* z,
                      const int32_t* flag, const double* box, const double* prm, double* totals,
                      double* c1d_a, double* c1d_b, double* xy_a, double* xy_b,
                      double* xz_a, double* xz_b, double* yz_a, double* yz_b) {
  const double xs = prm[0], ys = prm[1], zs = prm[2], hw = prm[3];
  const double xw = prm[4], yw = prm[5], zw = prm[6];
  if (!(xw > 0 && yw > 0 && zw > 0 && hw >= 0)) return ORC_ERR_CONFIG;
  const int64_t nx = (int64_t)(box[0] / xw), ny = (int64_t)(box[1] / yw), nz = (int64_t)(box[2] / zw);
  if (nx < 1 || ny < 1 || nz < 1) return ORC_ERR_CONFIG;
  double* a1 = calloc((size_t)nx, sizeof(double));
  double* b1 = calloc((size_t)nx, sizeof(double));
  double* axy = calloc((size_t)(nx * ny), sizeof(double));
  double* bxy = calloc((size_t)(nx * ny), sizeof(double));
  double* axz = calloc((size_t)(nx * nz), sizeof(double));
  double* bxz = calloc((size_t)(nx * nz), sizeof(double));
  double* ayz = calloc((size_t)(ny * nz), sizeof(double));
  double* byz = calloc((size_t)(ny * nz), sizeof(double));
  if (!a1 || !b1 || !axy || !bxy || !axz || !bxz || !ayz || !byz) {
    free(a1); free(b1); free(axy); free(bxy); free(axz); free(bxz); free(ayz); free(byz);
    return ORC_ERR_ALLOC;
  }
  double tota = 0, totb = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int32_t f = flag[i];
    if (f != 0 && f != 1) continue;
    if (f == 0) tota += 1.; else totb += 1.;
    if (z[i] <= zs + hw && z[i] >= zs - hw) {
      const int64_t j = conc_bin(x[i], xw, nx), k = conc_bin(y[i], yw, ny);
      if (f == 0) { a1[j] += 1.; axy[j + nx * k] += 1.; } else { b1[j] += 1.; bxy[j + nx * k] += 1.; }
    }
    if (y[i] <= ys + hw && y[i] >= ys - hw) {
      const int64_t j = conc_bin(x[i], xw, nx), k = conc_bin(z[i], zw, nz);
      if (f == 0) axz[j + nx * k] += 1.; else bxz[j + nx * k] += 1.;
    }
    if (x[i] <= xs + hw && x[i] >= xs - hw) {
      const int64_t j = conc_bin(y[i], yw, ny), k = conc_bin(z[i], zw, nz);
      if (f == 0) ayz[j + ny * k] += 1.; else byz[j + ny * k] += 1.;
    }
  }
  const double vol = (double)(int64_t)(box[0] * box[1] * box[2]);
  const double v1 = xw * box[1] * (2. * hw), vxy = xw * yw * (2. * hw);
  const double vxz = xw * zw * (2. * hw), vyz = yw * zw * (2. * hw);
  if (totals) { totals[0] = tota; totals[1] = totb; totals[2] = tota / vol; totals[3] = totb / vol; }
  for (int64_t j = 0; j < nx; ++j) {
    if (c1d_a) c1d_a[j] = a1[j] / v1;
    if (c1d_b) c1d_b[j] = b1[j] / v1;
  }
  for (int64_t q = 0; q < nx * ny; ++q) {
    if (xy_a) xy_a[q] = axy[q] / vxy;
    if (xy_b) xy_b[q] = bxy[q] / vxy;
  }
  for (int64_t q = 0; q < nx * nz; ++q) {
    if (xz_a) xz_a[q] = axz[q] / vxz;
    if (xz_b) xz_b[q] = bxz[q] / vxz;
  }
  for (int64_t q = 0; q < ny * nz; ++q) {
    if (yz_a) yz_a[q] = ayz[q] / vyz;
    if (yz_b) yz_b[q] = byz[q] / vyz;
  }
  free(a1); free(b1); free(axy); free(bxy); free(axz); free(bxz); free(ayz); free(byz);
  return ORC_OK;
}
