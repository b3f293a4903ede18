/* Internal state of the oracle (test infrastructure; see oracle.h). */
#ifndef MPCMD_ORACLE_ENGINE_H
#define MPCMD_ORACLE_ENGINE_H
#include <stdint.h>
#include "oracle.h"

struct orc {
  orc_params p;
  int64_t nt;                 /* solvent particles                                 */
  int nd, ns;                 /* dimers, spheres (2*nd)                            */
  double L[3];
  double *x, *y, *z, *vx, *vy, *vz;
  int32_t* flag;
  double* msd;                /* max_solvent_dist                                  */
  double *dpos, *dvel, *dfrc; /* [ns*3]                                            */
  double* q;                  /* RATTLE q vectors [ns*3]                           */
  double* anchor;             /* rotor anchors motorCM [nd*3]                      */
  int32_t* owner;             /* owner tags type_B [nt]                            */
  uint8_t* inc;               /* inside a C cutoff at the last force evaluation [nt] (catalysis on exit) */
  uint8_t* cnow;              /* scratch of one force evaluation [nt]              */
  int64_t maxnb;
  int64_t* nbnum;             /* [ns]                                              */
  int64_t* nb;                /* [ns*maxnb]                                        */
  double* fpair;              /* [ns*maxnb*3]                                      */
  double* pot;                /* [ns*maxnb]                                        */
  int64_t n_in, n_out;
  int64_t *in_list, *out_list;
  int32_t time_count, time_penetrate;
  int64_t cstep;
  int64_t n_rebuilds;
  double tpot;
  int prepared;
  int64_t ncell, ncell_shift;
  int64_t* newcell;           /* NewCellN [nt]                                     */
  double *cm, *axis;          /* [ncell_shift*3]                                   */
  int32_t* ccount;            /* tCellshift [ncell_shift]                          */
  double shift[3];
  int32_t* dcount;            /* distribute counts [ncell*4]                       */
  int64_t* dfirst;            /* first member per species [ncell*4], -1 if none    */
  int32_t* affected;          /* affectedCellN [ncell]                             */
  int32_t* react_box;         /* [lx*ly]                                           */
  int32_t* order;             /* cell visiting order of the sort, NULL = row-major  */
  int rng_mode, mt_kind;
  int list_mode;              /* ORC_LISTS_*: how orc_rebuild_lists finds the pairs  */
  uint32_t mt[624];
  int32_t mti;
  int status;
  /* selkov_code faithful driver state */
  double *fsx, *fsy, *fsz;    /* FXsol  [nt]                                       */
  double *pfx, *pfy, *pfz;    /* pFXsol [nt]                                       */
  double* spair;              /* FpairX(i,j) [nt*2*3]                              */
  double* spot;               /* Potential(i) [nt]                                 */
  double sd[3];               /* dXdim (last RATTLE-x separation)                  */
};

double orc_draw(orc_t* o, uint32_t tag, uint32_t index, uint32_t extra, uint32_t step, int which);
void orc_lj_consts(double r, double* R6, double* R12, double* r6R6, double* r12R12);
void orc_lj_mot_wall(double Lz, double zdim, double Ew, double Rw_plus_R, double* fwallz, double* potential);
void orc_harmonic_tether(double zdim, double zdimeq, double k_harm, double* f, double* pot);
void orc_selkov_cell(const double k[6], double tau, int32_t nF, int32_t nG, int32_t nI,
                     double x1, double x2, int* channel);
#endif
