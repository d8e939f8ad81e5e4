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

/* Single-face and single-cell kernels exposed for known-answer tests.
   wl / wr: primitive states (nprim entries, W layout); f: fluxes (ncons). */
int mf_oracle_face_flux(const mf_params* p, int dir, const double* wl, const double* wr,
                        double* f);
int mf_oracle_cons_to_prim(const mf_params* p, const double* u, double* w);
int mf_oracle_charge_exchange(const mf_params* p, const double* w, int reg, double dt,
                              double* s);
int mf_oracle_region(const mf_params* p, int i, int j, int k, const double* w);

/* Orszag-Tang initial state (problems/OrszagF.ChF:4-79). */
int mf_oracle_init_orszag(const mf_params* p, mf_fab* U, const mf_box* box);

/* Number of OpenMP threads available to the oracle (1 without OpenMP). */
int mf_oracle_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
