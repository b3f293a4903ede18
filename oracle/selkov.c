/*
 * Faithful selkov_code driver of the oracle (test infrastructure; see
 * oracle.h): Main_SelkovDimer.f90:125-149 with Motion_SelkovDimer.f90,
 * ForcesMD_SelkovDimer.f90, Distribute_SelkovDimer.f90, Affected_Cell.f90,
 * RMPC_SelkovDimer.f90 and Sort.f90, for the reference's single dimer.  Every
 * particle is integrated each MD step (no neighbour lists), solvent forces are
 * stored per particle and the catalytic sphere overwrites the non-catalytic
 * one (ForcesMD_SelkovDimer.f90:318-320).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "oracle.h"
#include "engine.h"

static inline double hpbc(double d, double L) {
  if (d > 0.5 * L) d -= L;
  else if (d < -0.5 * L) d += L;
  return d;
}

static inline double fwrap(double x, double L) { return x - L * floor(x / L); }

/* Sort.f90:7-183: cells in row-major order, F then G then I inside a cell. */
static int selkov_sort(orc_t* o) {
  const int64_t n = o->nt, C = o->ncell;
  int64_t* cnt = calloc(4 * C + 1, 8);
  int64_t* start = calloc(4 * C + 1, 8);
  int64_t* perm = malloc(n * 8);
  int64_t* key = malloc(n * 8);
  double* tmp = malloc(n * 8);
  int32_t* tmpi = malloc(n * 4);
  if (!cnt || !start || !perm || !key || !tmp || !tmpi) {
    free(cnt); free(start); free(perm); free(key); free(tmp); free(tmpi);
    return o->status = ORC_ERR_ALLOC;
  }
  static const int slot[4] = {0, 1, -1, 2};
  int64_t kept = 0;
  for (int64_t i = 0; i < n; ++i) {
    int s = slot[o->flag[i] & 3];
    if (s < 0) { key[i] = -1; continue; }
    int64_t c = (int64_t)(floor(o->x[i]) + o->L[0] * floor(o->y[i]) + o->L[0] * o->L[1] * floor(o->z[i]));
    key[i] = 4 * c + s;
    cnt[key[i]]++;
    kept++;
  }
  int64_t acc = 0;
  for (int64_t k = 0; k < 4 * C; ++k) { start[k] = acc; acc += cnt[k]; }
  for (int64_t i = 0; i < n; ++i) if (key[i] >= 0) perm[start[key[i]]++] = i;
#define PERM(a) do {                                          \
    for (int64_t j = 0; j < kept; ++j) tmp[j] = a[perm[j]];   \
    for (int64_t j = kept; j < n; ++j) tmp[j] = 0.;           \
    memcpy(a, tmp, n * 8);                                    \
  } while (0)
  PERM(o->x); PERM(o->y); PERM(o->z); PERM(o->vx); PERM(o->vy); PERM(o->vz);
  PERM(o->fsx); PERM(o->fsy); PERM(o->fsz); PERM(o->pfx); PERM(o->pfy); PERM(o->pfz);
#undef PERM
  for (int64_t j = 0; j < kept; ++j) tmpi[j] = o->flag[perm[j]];
  for (int64_t j = kept; j < n; ++j) tmpi[j] = 2;
  memcpy(o->flag, tmpi, n * 4);
  free(cnt); free(start); free(perm); free(key); free(tmp); free(tmpi);
  return ORC_OK;
}

/* Motion_SelkovDimer.f90:7-159 */
static void selkov_motion(orc_t* o) {
  const double dt = o->p.md_dt, Mc = o->p.mc, Mn = o->p.mn, Dcn = o->p.dcn;
  double h2[4];
  for (int c = 0; c < 4; ++c) h2[c] = (0.5 * dt * dt) / o->p.mass[c];
  const double hIMc = (0.5 * dt) / Mc, hIMn = (0.5 * dt) / Mn;
  const double IMc = 1.0 / Mc, IMn = 1.0 / Mn, IIM = 1.0 / (IMc + IMn), IMDt = 1.0 / dt;
  for (int64_t i = 0; i < o->nt; ++i) { o->pfx[i] = o->fsx[i]; o->pfy[i] = o->fsy[i]; o->pfz[i] = o->fsz[i]; }
  double pF[2][3], pr[2][3], prV[2][3];
  for (int s = 0; s < 2; ++s)
    for (int c = 0; c < 3; ++c) {
      pF[s][c] = o->dfrc[3 * s + c];
      pr[s][c] = o->dpos[3 * s + c];
      prV[s][c] = o->dvel[3 * s + c];
    }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < o->nt; ++i) {
    int f = o->flag[i];
    if (f == 0 || f == 1 || f == 3) {
      o->x[i] = o->x[i] + o->vx[i] * dt + o->pfx[i] * h2[f];
      o->y[i] = o->y[i] + o->vy[i] * dt + o->pfy[i] * h2[f];
      o->z[i] = o->z[i] + o->vz[i] * dt + o->pfz[i] * h2[f];
    }
    o->x[i] = fwrap(o->x[i], o->L[0]);
    o->y[i] = fwrap(o->y[i], o->L[1]);
    o->z[i] = fwrap(o->z[i], o->L[2]);
  }
  double dP[3];
  for (int c = 0; c < 3; ++c) dP[c] = hpbc(pr[0][c] - pr[1][c], o->L[c]);
  double* Q = o->q;
  for (int c = 0; c < 3; ++c) {
    Q[c] = prV[0][c] + hIMc * pF[0][c];
    Q[3 + c] = prV[1][c] + hIMn * pF[1][c];
  }
  for (int s = 0; s < 2; ++s)
    for (int c = 0; c < 3; ++c) o->dpos[3 * s + c] = fwrap(pr[s][c] + dt * Q[3 * s + c], o->L[c]);
  int64_t acc = 0;
  for (;;) {
    double d[3];
    for (int c = 0; c < 3; ++c) d[c] = hpbc(o->dpos[c] - o->dpos[3 + c], o->L[c]);
    o->sd[0] = d[0]; o->sd[1] = d[1]; o->sd[2] = d[2];
    double dXYZ2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    double Con1diff = dXYZ2 - Dcn * Dcn;
    if (fabs(Con1diff) < 1.e-6) break;
    if (acc == o->p.rattle_max_iter) { o->status = ORC_ERR_RATTLE; break; }
    double G = (0.5 * Con1diff * IMDt * IIM) / (d[0] * dP[0] + d[1] * dP[1] + d[2] * dP[2]);
    for (int c = 0; c < 3; ++c) {
      Q[c] = Q[c] - G * IMc * dP[c];
      Q[3 + c] = Q[3 + c] + G * IMn * dP[c];
    }
    for (int s = 0; s < 2; ++s)
      for (int c = 0; c < 3; ++c) o->dpos[3 * s + c] = fwrap(pr[s][c] + dt * Q[3 * s + c], o->L[c]);
    acc++;
  }
}

/* ForcesMD_SelkovDimer.f90:169-464 */
static void selkov_forces(orc_t* o) {
  const double cut = pow(2.0, 1.0 / 6.0);
  const double dt = o->p.md_dt, Mc = o->p.mc, Mn = o->p.mn, Dcn = o->p.dcn;
  const double IMc = 1.0 / Mc, IMn = 1.0 / Mn, IIM = 1.0 / (IMc + IMn);
  const double hIMc = (0.5 * dt) / Mc, hIMn = (0.5 * dt) / Mn;
  double hIM[4];
  for (int c = 0; c < 4; ++c) hIM[c] = (0.5 * dt) / o->p.mass[c];
  o->tpot = 0.;
  memset(o->fsx, 0, o->nt * 8); memset(o->fsy, 0, o->nt * 8); memset(o->fsz, 0, o->nt * 8);
  memset(o->spot, 0, o->nt * 8);
  memset(o->spair, 0, o->nt * 6 * 8);
  for (int c = 0; c < 6; ++c) o->dfrc[c] = 0.;
  for (int pass = 0; pass < 2; ++pass) {
    /* pass 0: non-catalytic sphere (index 1), pass 1: catalytic sphere (0) */
    int s = pass == 0 ? 1 : 0;
    double R = s == 0 ? o->p.rc : o->p.rn;
    double cutoff2 = (R * cut) * (R * cut);
    double R6, R12, r6R6, r12R12;
    orc_lj_consts(R, &R6, &R12, &r6R6, &r12R12);
    const double* eps = s == 0 ? o->p.eps_c : o->p.eps_n;
    const double* X = o->dpos + 3 * s;
    for (int64_t i = 0; i < o->nt; ++i) {
      double dR[3] = {hpbc(o->x[i] - X[0], o->L[0]), hpbc(o->y[i] - X[1], o->L[1]),
                      hpbc(o->z[i] - X[2], o->L[2])};
      double dRsq = dR[0] * dR[0] + dR[1] * dR[1] + dR[2] * dR[2];
      if (dRsq > cutoff2) continue;
      int f = o->flag[i];
      if (!(f == 0 || f == 1 || f == 3)) continue;
      double E = eps[f];
      int newf = f;
      if (s == 0 && (f == 0 || f == 1)) {
        double u = orc_draw(o, ORC_TAG_CAT, (uint32_t)i, 0, (uint32_t)o->cstep, 0);
        if (f == 0 && o->p.rp_ab > u) newf = 1;
        if (f == 1 && o->p.rp_ba > u) newf = 0;
      }
      double IdRsq = 1.0 / dRsq;
      double IdR6 = IdRsq * IdRsq * IdRsq;
      double IdR8 = IdR6 * IdRsq;
      double IdR12 = IdR6 * IdR6;
      double IdR14 = IdR12 * IdRsq;
      double Fbrack = 4.0 * (r12R12 * IdR14 - r6R6 * IdR8);
      double Ubrack = 4.0 * (R12 * IdR12 - R6 * IdR6) + 1.0;
      double* fp = o->spair + 6 * i + 3 * s;
      fp[0] = E * Fbrack * dR[0];
      fp[1] = E * Fbrack * dR[1];
      fp[2] = E * Fbrack * dR[2];
      o->spot[i] = E * Ubrack;
      o->fsx[i] = fp[0]; o->fsy[i] = fp[1]; o->fsz[i] = fp[2];
      o->flag[i] = newf;
    }
  }
  for (int64_t i = 0; i < o->nt; ++i) {
    int f = o->flag[i];
    if (f == 0 || f == 1 || f == 3) {
      o->tpot = o->tpot + o->spot[i];
      for (int j = 0; j < 2; ++j)
        for (int c = 0; c < 3; ++c) o->dfrc[3 * j + c] = o->dfrc[3 * j + c] - o->spair[6 * i + 3 * j + c];
    }
  }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < o->nt; ++i) {
    int f = o->flag[i];
    if (f == 0 || f == 1 || f == 3) {
      o->vx[i] = o->vx[i] + (o->pfx[i] + o->fsx[i]) * hIM[f];
      o->vy[i] = o->vy[i] + (o->pfy[i] + o->fsy[i]) * hIM[f];
      o->vz[i] = o->vz[i] + (o->pfz[i] + o->fsz[i]) * hIM[f];
    }
  }
  double* V1 = o->dvel;
  double* V2 = o->dvel + 3;
  for (int c = 0; c < 3; ++c) {
    V1[c] = o->q[c] + hIMc * o->dfrc[c];
    V2[c] = o->q[3 + c] + hIMn * o->dfrc[3 + c];
  }
  int64_t acc = 0;
  for (;;) {
    double dV[3] = {V1[0] - V2[0], V1[1] - V2[1], V1[2] - V2[2]};
    double Con2diff = dV[0] * o->sd[0] + dV[1] * o->sd[1] + dV[2] * o->sd[2];
    if (fabs(Con2diff) < 1.e-8) break;
    if (acc == o->p.rattle_max_iter) { o->status = ORC_ERR_RATTLE; break; }
    double O = (IIM * Con2diff) / (Dcn * Dcn);
    for (int c = 0; c < 3; ++c) {
      V1[c] = V1[c] - O * o->sd[c] * IMc;
      V2[c] = V2[c] + O * o->sd[c] * IMn;
    }
    acc++;
  }
}

int orc_selkov_prepare(orc_t* o) {
  if (o->nd != 1 || o->p.geometry != ORC_GEOM_PERIODIC) return o->status = ORC_ERR_CONFIG;
  memset(o->fsx, 0, o->nt * 8); memset(o->fsy, 0, o->nt * 8); memset(o->fsz, 0, o->nt * 8);
  memset(o->pfx, 0, o->nt * 8); memset(o->pfy, 0, o->nt * 8); memset(o->pfz, 0, o->nt * 8);
  o->prepared = 2;
  return ORC_OK;
}

int orc_selkov_step(orc_t* o) {
  if (o->prepared != 2) return o->status = ORC_ERR_STATE;
  o->cstep = o->cstep + 1;
  if (o->cstep % o->p.mpc_every != 0) {
    selkov_motion(o);
    selkov_forces(o);
  } else {
    if (o->p.sort_every > 0 && o->cstep % o->p.sort_every == 0) selkov_sort(o);
    selkov_motion(o);
    orc_distribute(o);     /* Distribute_SelkovDimer + Affected_Cell (positions fixed) */
    selkov_forces(o);
    orc_mpc_rotation(o);
    orc_reaction(o);
  }
  return o->status;
}
