/*
 * mf_oracle.h - CPU restatement of the MHDAM per-patch Godunov update.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the GPU
 * path and the timed CPU baseline; it is never linked into, called by or
 * shipped with the product library.  Parity status: "parity unpinned" - the
 * reference publishes no test vectors and cannot be built here (no Fortran
 * compiler, no Chombo), so this restatement is pinned by known-answer and
 * invariant tests instead of reference outputs.
 *
 * Entry points mirror include/mf_patch.h with host pointers.
 */
#ifndef MF_ORACLE_H
#define MF_ORACLE_H

#include "../include/mf_patch.h"

#ifdef __cplusplus
extern "C" {
#endif

/* PatchMHDAM::updateState (src/PatchMHDAM.cpp:1192-1317) on one host patch. */
/* updateState with the edge field output of constrained transport: E = the
   EdgeBox on valid (3 fabs in 3D, 1 nodal fab in 2D; NULL = not wanted) */
int mf_oracle_patch_update_e(const mf_params* p, double time, mf_fab* U, const mf_box* valid,
                             double dt, mf_fab* F, mf_fab* divB, mf_fab* E, double* new_dt,
                             int min_cell[3]);
/* PatchMHDMF::recalculateMagneticField (srcIdeal/PatchMHDMF.cpp:1461-1484) */
int mf_oracle_recalculate_b(const mf_params* p, mf_fab* U, const mf_fab* Uold, mf_fab* E,
                            double dt, const mf_box* box);
int mf_oracle_patch_update(const mf_params* p, double time, mf_fab* U, const mf_box* valid,
                           double dt, mf_fab* F, mf_fab* divB, double* new_dt, int min_cell[3]);

/* PatchMHDMF::computeDt (srcIdeal/PatchMHDMF.cpp:66-146). */
int mf_oracle_compute_dt(const mf_params* p, const mf_fab* U, const mf_box* box, double* dt,
                         int min_cell[3]);

/* LevelData::exchange: copy valid data of every patch into the ghost cells of
   every other patch (and its own periodic images). */
int mf_oracle_level_exchange(const mf_params* p, int npatch, mf_fab* U, const mf_box* valid);

/* One level step: exchange then updateState on every patch (OpenMP over
   patches, as AMRLevelIdealMHD::stepOMP) and the level minimum of new dt. */
int mf_oracle_level_step(const mf_params* p, double time, int npatch, mf_fab* U,
                         const mf_box* valid, double dt, int nthreads, double* new_dt,
                         int* min_patch, int min_cell[3]);

/* A level of a hierarchy: its parameters (dx and domain in the level's own
   index space), patches (host fabs with ghosts) and valid boxes. */
typedef struct {
  const mf_params* p;
  int npatch;
  mf_fab* U;
  const mf_box* valid;
} mf_oracle_level;

/* One time step of the coarsest level of a subcycled hierarchy
   (AMR_MHDAM::timeStep srcIdeal/AMR_MHDAM.cpp:1707-1880 with
   AMRLevelIdealMHD::advance / postTimeStep): level l steps ratio[l-1] times
   per step of level l-1 with dt0 / prod(ratio); fine ghosts are interpolated
   from the coarse level in space and time, coarse cells next to the fine
   region are refluxed and covered coarse cells are averaged from the fine
   level.  time[l] is advanced; new_dt = min over levels of the level's new dt
   times the level's refinement; dedner (nullable) receives Ch, Cp as the base
   level leaves them. */
int mf_oracle_hier_step(int nlev, const mf_oracle_level* lev, const int* ratio, double* time,
                        double dt0, int nthreads, double* new_dt, double* dedner);

/* PiecewiseLinearFillPatchMHDAM::fillInterp on its own (alpha: time
   fraction between the old and new coarse states). */
int mf_oracle_cf_fill(const mf_params* pc, const mf_params* pf, int ratio, int ncoarse,
                      mf_fab* Uc_old, mf_fab* Uc_new, const mf_box* vc, int nfine, mf_fab* Uf,
                      const mf_box* vf, double alpha);

/* CoarseAverageExt::averageToCoarse on its own. */
int mf_oracle_average_down(const mf_params* pc, const mf_params* pf, int ratio, int ncoarse,
                           mf_fab* Uc, const mf_box* vc, int nfine, mf_fab* Uf,
                           const mf_box* vf);

/* Single-face and single-cell kernels exposed for known-answer tests.
   wl / wr: primitive states (nprim entries, W layout); f: fluxes (ncons). */
int mf_oracle_face_flux(const mf_params* p, int dir, const double* wl, const double* wr,
                        double* f);
/* One limiter on one cell: *FACEVALUES from W(i-1), W(i), W(i+1) (lo: value
   on the low face, hi: on the high face), and *FACESLOPES in place on the
   left / right differences (src/reconstructionF.ChF). */
int mf_oracle_face_values(int lim, double wm1, double wp, double wp1, double* lo, double* hi);
int mf_oracle_face_slopes(int lim, double* sleft, double* sright);
int mf_oracle_cons_to_prim(const mf_params* p, const double* u, double* w);
/* HELIOBC (swlism/HeliosphericF.ChF:221-910) on one face of the domain
   boundary: the face fluxes of (wl, wr) by the configured solvers, then the
   heliosphere's boundary fluxes over them (side 0: low face, wl is the ghost
   side; 1: high face, wr is the ghost side); bn: the face-normal B. */
int mf_oracle_helio_bc_face(const mf_params* p, int dir, int side, const double* wl,
                            const double* wr, double* f, double* bn);
int mf_oracle_charge_exchange(const mf_params* p, const double* w, int reg, double dt,
                              double* s);
int mf_oracle_region(const mf_params* p, int i, int j, int k, const double* w);

/* Orszag-Tang initial state (problems/OrszagF.ChF:4-79). */
int mf_oracle_init_orszag(const mf_params* p, mf_fab* U, const mf_box* box);
/* The synthetic heliosphere's initial state: uniform inflow (primitive
   states wp, wn through PRIMTOCONS_MF), tracking surfaces, the inner sphere
   reset at time 0. */
int mf_oracle_init_helio(const mf_params* p, const double* wp, const double* wn, mf_fab* U,
                         const mf_box* box);

/* Number of OpenMP threads available to the oracle (1 without OpenMP). */
int mf_oracle_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
