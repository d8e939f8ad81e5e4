/*
 * mf_oracle.c - CPU restatement of the MHDAM / MS-FLUKSS per-patch Godunov
 * update (PatchMHDAM::updateState for the multi-fluid MHD model).
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker of the GPU path and the timed
 * CPU baseline.  Nothing in the product links or calls this file.
 *
 * Parity status: "parity unpinned".  The reference ships no tests, golden
 * vectors or benchmark outputs, and it cannot be compiled here (no Fortran
 * compiler, Chombo 3.2.4 not vendored).  Every routine below restates the
 * cited Fortran/C++ literally, including the order in which each expression is
 * evaluated (Fortran evaluates a+b+c left to right; x**2 is x*x), and it is
 * pinned by the known-answer and invariant tests under tests/.
 *
 * Citations are paths inside the MHDAM-3.2.4 tree.
 * Compile with -ffp-contract=off so that no multiply-add is fused.
 */
#include "mf_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* srcIdeal/EosCommon.fh:13-27 */
#define D_1_4PI 0.079577471545947667884441881686257181
#define D_1_8PI 0.039788735772973833942220940843128591
#define D_SQRT_2 0.707106781186547524400844362104849039
#define D_PI 3.14159265358979323846264338327950288
#define D_2PI 6.28318530717958647692528676655900576
#define D_PI_2 1.57079632679489661923132169163975144
/* srcIdeal/EosCommon.fh:31-37 */
#define NETF2_DENS 1.0e-6
#define NETF2_PRES 1.0e-8
#define NETF3_DENS 1.0e-7
#define NETF3_PRES 1.0e-9

/* ------------------------------------------------------------------------ */
/* boxes and FArrayBox-like arrays                                           */
/* ------------------------------------------------------------------------ */

typedef struct {
  double* p;
  mf_box b;
  int nc;
  long n0, n1, n2, csz;
  int owned;
} Fab;

static Fab fab_wrap(double* p, mf_box b, int nc) {
  Fab f;
  f.p = p;
  f.b = b;
  f.nc = nc;
  f.n0 = b.hi[0] - b.lo[0] + 1;
  f.n1 = b.hi[1] - b.lo[1] + 1;
  f.n2 = b.hi[2] - b.lo[2] + 1;
  f.csz = f.n0 * f.n1 * f.n2;
  f.owned = 0;
  return f;
}

static Fab fab_alloc(mf_box b, int nc) {
  Fab f = fab_wrap(NULL, b, nc);
  long n = f.csz * (long)nc;
  f.p = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  /* FArrayBox storage is uninitialised; NaN makes any read of an unset
     entry visible in the results. */
  for (long q = 0; q < n; ++q) f.p[q] = NAN;
  f.owned = 1;
  return f;
}

static void fab_free(Fab* f) {
  if (f->owned && f->p) free(f->p);
  f->p = NULL;
}

static inline long fab_off(const Fab* f, int i, int j, int k) {
  return (i - f->b.lo[0]) + f->n0 * ((j - f->b.lo[1]) + f->n1 * (long)(k - f->b.lo[2]));
}
#define AT(f, i, j, k, c) ((f)->p[fab_off((f), (i), (j), (k)) + (long)(c) * (f)->csz])

static mf_box box_grow(mf_box b, int n, int sd) {
  for (int d = 0; d < sd; ++d) {
    b.lo[d] -= n;
    b.hi[d] += n;
  }
  return b;
}

/* Box & ProblemDomain: clip the non-periodic directions only. */
static mf_box box_and_domain(mf_box b, const mf_params* p) {
  for (int d = 0; d < p->space_dim; ++d) {
    if (p->periodic[d]) continue;
    if (b.lo[d] < p->domain_lo[d]) b.lo[d] = p->domain_lo[d];
    if (b.hi[d] > p->domain_hi[d]) b.hi[d] = p->domain_hi[d];
  }
  return b;
}

static mf_box box_nodes(mf_box b, int d) {
  b.hi[d] += 1;
  return b;
}

static int box_in(const mf_box* b, int i, int j, int k) {
  return i >= b->lo[0] && i <= b->hi[0] && j >= b->lo[1] && j <= b->hi[1] && k >= b->lo[2] &&
         k <= b->hi[2];
}

static int box_contains(const mf_box* outer, const mf_box* inner) {
  for (int d = 0; d < 3; ++d)
    if (inner->lo[d] < outer->lo[d] || inner->hi[d] > outer->hi[d]) return 0;
  return 1;
}

#define FOR_BOX(bx, i, j, k)                               \
  for (int k = (bx).lo[2]; k <= (bx).hi[2]; ++k)           \
    for (int j = (bx).lo[1]; j <= (bx).hi[1]; ++j)         \
      for (int i = (bx).lo[0]; i <= (bx).hi[0]; ++i)

/* ------------------------------------------------------------------------ */
/* model constants                                                           */
/* ------------------------------------------------------------------------ */

enum { RS_ROE8 = 0, RS_ROE7 = 1, RS_RUSANOV = 2, RS_VFROE = 3 };

typedef struct {
  const mf_params* p;
  int sd, nf, glm, nc, nprim, irhon, ipsi;
  int ils, nls; /* tracking surfaces: components ils .. nc-1 after the fluids */
  int ct;       /* constrained transport: 0 off, 1 Balsara-Spicer, 2/3 Gardiner-Stone 1/2 */
  int rs, aver;
  double gamma, hgamma, invhgamma, smallr, smallp, del2, smallB;
  double dCh, dCp;
  /* inner-sphere field: monopolar (sunBmonopolar == 1) or bipolar with the
     current-sheet surface ihcs (-1: none) and the sheet's tilt */
  int monopolar, ihcs;
  double sin_tilt, cos_tilt;
} Ctx;

/* EqSysMHDMF ctor (srcIdeal/EqSysMHDMF.cpp:11-48) and RiemannSolver::make
   (src/RiemannSolver.cpp:13-112). */
static int ctx_init(Ctx* c, const mf_params* p) {
  if (p->space_dim < 2 || p->space_dim > 3) return MF_ERR_BAD_ARG;
  if (p->n_fluids < 1 || p->n_fluids > MF_MAX_FLUIDS) return MF_ERR_BAD_ARG;
  c->p = p;
  c->sd = p->space_dim;
  c->nf = p->n_fluids;
  /* eDivergenceCleaning (src/PatchMHDAM.H:43-50): 1-3 constrained transport,
     5 GLM; 4 (projection) needs an elliptic solver and is not restated */
  if (!(p->divb_cleaning == 0 || (p->divb_cleaning >= 1 && p->divb_cleaning <= 3) ||
        p->divb_cleaning == 5))
    return MF_ERR_UNSUPPORTED;
  c->glm = (p->divb_cleaning == 5) ? 1 : 0;
  c->ct = (p->divb_cleaning >= 1 && p->divb_cleaning <= 3) ? p->divb_cleaning : 0;
  /* electricFieldGS0/GS1 in 3D store the z-edge field into EX over the EZ
     index range (srcIdeal/DivCleaningF.ChF:478-566, :700-852): EZ is left
     unset and EX is written outside its box; nothing defined to restate */
  if (c->ct >= 2 && p->space_dim == 3) return MF_ERR_UNSUPPORTED;
  /* lvlsStateInterval after consStateInterval; the primitive interval is
     the same (srcIdeal/EqSysMHDMF.cpp:32-42) */
  c->ils = 8 + c->glm + (c->nf - 1) * 5;
  c->nls = p->num_tracking_surfaces;
  if (c->nls < 0) return MF_ERR_BAD_ARG;
  if (c->nls > 2 || c->ils + c->nls > MF_MAX_COMP) return MF_ERR_UNSUPPORTED;
  if (p->region_tracer && c->nls < 1) return MF_ERR_BAD_ARG;
  c->nc = c->ils + c->nls;
  c->nprim = c->nc;
  c->irhon = 8 + c->glm;
  c->ipsi = c->glm ? 8 : -1;
  c->gamma = p->gamma;
  c->hgamma = p->gamma - 1.0;
  c->invhgamma = 1.0 / c->hgamma;
  c->smallr = p->smallr;
  c->smallp = p->smallp;
  c->del2 = p->entropy_fix;
  c->smallB = p->small_b;
  c->dCh = p->dedner_ch;
  c->dCp = p->dedner_cp;
  /* HeliosphericProblem (swlism/HeliosphericProblem.cpp:156, 616-631):
     every sunBmonopolar but 1 means bipolar; iHCS is the first tracking
     surface (the first of two with the region tracer) */
  c->monopolar = (p->sun_b_monopolar == 1);
  c->ihcs = -1;
  if (!c->monopolar && c->nls > (p->region_tracer ? 1 : 0)) c->ihcs = c->ils;
  {
    /* SETHELIOS: sunTILT in radians (swlism/HeliosphericF.ChF:66) */
    double tilt = p->sun_tilt * (D_PI / 180.0);
    c->sin_tilt = sin(tilt);
    c->cos_tilt = cos(tilt);
  }
  int f = p->flux;
  if (c->glm) {
    if (!(f == 1 || f == 3)) return MF_ERR_UNSUPPORTED;
    if (p->use_8wave) return MF_ERR_UNSUPPORTED;
    c->rs = RS_ROE7;
    c->aver = (f == 3);
  } else {
    switch (f) {
      case 2: c->rs = RS_RUSANOV; c->aver = 0; break;
      case 3: c->rs = RS_ROE8; c->aver = 1; break;
      case 4: c->rs = RS_RUSANOV; c->aver = 1; break;
      case 5: c->rs = RS_VFROE; c->aver = 0; break; /* VFRoeRS, arithmetic averaging */
      case 11: c->rs = RS_ROE7; c->aver = 0; break;
      case 13: c->rs = RS_ROE7; c->aver = 1; break;
      default: c->rs = RS_ROE8; c->aver = 0; break;
    }
  }
  if (p->time_approximation != MF_TA_FIRST_ORDER && p->time_approximation != MF_TA_RK2 &&
      p->time_approximation != MF_TA_HANCOCK)
    return MF_ERR_UNSUPPORTED;
  return MF_OK;
}

static int num_ghost(const mf_params* p) {
  if (p->time_approximation == MF_TA_RK2) return 4;
  if (p->time_approximation == MF_TA_HANCOCK) return 3;
  return 2;
}

/* ------------------------------------------------------------------------ */
/* conserved -> primitive                                                    */
/* ------------------------------------------------------------------------ */

/* CONSTOPRIM (srcIdeal/PatchIdealMHDF.ChF:143-189) and CONSTOPRIM_MF
   (srcIdeal/PatchMHDMFF.ChF:5-80), then the psi copy of
   EqSysMHDMF::stateToPrim (srcIdeal/EqSysMHDMF.cpp:169-212). */
static void cons_to_prim_cell(const Ctx* c, const double* U, double* W) {
  double rho, ru, rv, rw, invrho, uu, vv, ww, ke, bx, by, bz, b, p;
  if (c->nf == 1)
    rho = U[0];
  else
    rho = fmax(U[0], c->smallr);
  ru = U[1];
  rv = U[2];
  rw = U[3];
  invrho = 1.0 / rho;
  uu = ru * invrho;
  vv = rv * invrho;
  ww = rw * invrho;
  ke = ru * uu + rv * vv + rw * ww;
  bx = U[5];
  by = U[6];
  bz = U[7];
  b = D_1_4PI * (bx * bx + by * by + bz * bz);
  p = c->hgamma * (U[4] - 0.5 * (ke + b));
  p = fmax(p, c->smallp);
  W[1] = uu;
  W[2] = vv;
  W[3] = ww;
  W[0] = rho;
  W[4] = p;
  W[5] = bx;
  W[6] = by;
  W[7] = bz;
  for (int f = 1; f < c->nf; ++f) {
    int s = c->irhon + (f - 1) * 5;
    rho = fmax(U[s], c->smallr);
    ru = U[s + 1];
    rv = U[s + 2];
    rw = U[s + 3];
    invrho = 1.0 / rho;
    uu = ru * invrho;
    vv = rv * invrho;
    ww = rw * invrho;
    ke = ru * uu + rv * vv + rw * ww;
    p = c->hgamma * (U[s + 4] - 0.5 * ke);
    p = fmax(p, c->smallp);
    W[s + 1] = uu;
    W[s + 2] = vv;
    W[s + 3] = ww;
    W[s] = rho;
    W[s + 4] = p;
  }
  if (c->glm) W[8] = U[8];
  /* EqSysMHDMF::stateToPrim copies the tracking surfaces (:207-210) */
  for (int q = c->ils; q < c->nc; ++q) W[q] = U[q];
}

/* ------------------------------------------------------------------------ */
/* limited face values                                                       */
/* ------------------------------------------------------------------------ */

/* minmod (src/reconstructionF.ChF:5-13); sign(one,A) is copysign. */
static double minmod(double A, double B) {
  double signA = copysign(1.0, A);
  return signA * fmax(0.0, fmin(fabs(A), signA * B));
}

/* One cell, one variable: returns Wleft (value on the low face) and Wright
   (value on the high face) from W(i-1), W(i), W(i+1).
   MINMODFACEVALUES :126-155, SUPERBEEFACEVALUES :258-301,
   HYPERBEEFACEVALUES :430-464, VANALBADAFACEVALUES :550-589,
   MCFACEVALUES :622-661, HARMONICFACEVALUES :492-524,
   VANLEERFACEVALUES :794-841, KORENFACEVALUES :883-918,
   VENKATAKRISHNANFACEVALUES :950-988, CDFACEVALUES :1056-1079,
   WENO3FACEVALUES :1096-1136, WENO3YCFACEVALUES :1169-1212; dispatch of
   limiter1D::make (src/limiter1D.cpp:21-63). */
static void face_values(int lim, double Wm1, double WP, double Wp1, double* WL, double* WR) {
  double dWR = Wp1 - WP;
  double dWL = WP - Wm1;
  double SLOPE;
  switch (lim) {
    case MF_LIM_CD:
      *WL = 0.5 * (WP + Wp1);
      *WR = 0.5 * (WP + Wm1);
      return;
    case MF_LIM_SUPERBEE:
      if (dWL * dWR <= 0.0) {
        *WL = WP;
        *WR = WP;
        return;
      } else {
        double AR = fabs(dWR), AL = fabs(dWL);
        if (AL <= 0.5 * AR)
          SLOPE = dWL;
        else if (AL <= AR)
          SLOPE = 0.5 * dWR;
        else if (AL <= AR + AR)
          SLOPE = 0.5 * dWL;
        else
          SLOPE = dWR;
      }
      break;
    case MF_LIM_VANALBADA: {
      const double dSave = 1.0e-6, dSaveS = dSave + dSave;
      if (dWL * dWR <= 0.0) {
        *WL = WP;
        *WR = WP;
        return;
      }
      SLOPE = 0.5 * (dWR * dWL + dSave) * (dWR + dWL) / (dWR * dWR + dWL * dWL + dSaveS);
      break;
    }
    case MF_LIM_MC:
      if (dWL * dWR <= 0.0) {
        *WL = WP;
        *WR = WP;
        return;
      } else {
        double AR = fabs(dWR), AL = fabs(dWL);
        if (3.0 * AL <= AR)
          SLOPE = dWL;
        else if (AL <= 3.0 * AR)
          SLOPE = 0.25 * (dWR + dWL);
        else
          SLOPE = dWR;
      }
      break;
    case MF_LIM_HARMONIC:
      if (dWL * dWR <= 0.0) {
        *WL = WP;
        *WR = WP;
        return;
      }
      SLOPE = dWR / (1.0 + dWR / dWL);
      break;
    case MF_LIM_HYPERBEE: {
      double A;
      if (dWL * dWR <= 0.0) {
        *WL = WP;
        *WR = WP;
        return;
      }
      A = 1.0 + sqrt(dWR / dWL);
      SLOPE = dWR / (A * A);
      SLOPE = SLOPE + SLOPE;
      break;
    }
    case MF_LIM_KOREN: {
      const double dSave = 1.0e-10;
      double H;
      if (dWL * dWR <= 0.0) {
        *WL = WP;
        *WR = WP;
        return;
      }
      H = dWL * dWR / (2.0 * (dWL * dWL + dWR * dWR + dSave) - dWL * dWR);
      *WL = WP - (dWL + 0.5 * dWR) * H;
      *WR = WP + (dWR + 0.5 * dWL) * H;
      return;
    }
    case MF_LIM_VENKATAKRISHNAN: {
      const double dSave = 1.0e-10, dSave2 = dSave * dSave;
      double H;
      if (dWL * dWR <= 0.0) {
        *WL = WP;
        *WR = WP;
        return;
      }
      H = (dWR + dWL) / (6.0 * (dWR * dWR + dWL * dWL + dSave2));
      *WL = WP - (dWR + 2.0 * dWL) * (dWL + dSave) * H;
      *WR = WP + (dWL + 2.0 * dWR) * (dWR + dSave) * H;
      return;
    }
    case MF_LIM_WENO3: {
      const double dSave = 1.0e-6;
      double BR = dWR * dWR + dSave, AR = 1.0 / (BR * BR);
      double BL = dWL * dWL + dSave, AL = 1.0 / (BL * BL);
      double H = AR / (AR + 2.0 * AL);
      *WL = WP - 0.5 * (dWL + H * (dWR - dWL));
      H = AL / (AL + 2.0 * AR);
      *WR = WP + 0.5 * (dWR - H * (dWR - dWL));
      return;
    }
    case MF_LIM_WENO3YC: {
      const double dSave = 1.0e-6;
      double BR = dWR * dWR + dSave, BL = dWL * dWL + dSave;
      double D2P = dWR - dWL, AL, AR, H;
      D2P = D2P * D2P;
      AL = 1.0 + D2P / BL;
      AR = 1.0 + D2P / BR;
      H = AR / (AR + 2.0 * AL);
      *WL = WP - 0.5 * (dWL + H * (dWR - dWL));
      H = AL / (AL + 2.0 * AR);
      *WR = WP + 0.5 * (dWR - H * (dWR - dWL));
      return;
    }
    case MF_LIM_VANLEER: {
      const double dSLim = 1.0 / 3.0;
      const double BT = (3.0 - dSLim) / (1.0 - dSLim);
      const double SL1 = 0.25 * (1.0 - dSLim);
      const double SL2 = 0.25 * (1.0 + dSLim);
      if (dWL * dWR <= 0.0) {
        *WL = WP;
        *WR = WP;
        return;
      } else {
        double SL = fmin(fabs(dWR), fabs(BT * dWL));
        double SR = fmin(fabs(dWL), fabs(BT * dWR));
        double SLOPL = SL1 * SL + SL2 * SR;
        double SLOPR = SL1 * SR + SL2 * SL;
        if (dWR < 0.0) {
          SLOPL = -SLOPL;
          SLOPR = -SLOPR;
        }
        *WL = WP - SLOPL;
        *WR = WP + SLOPR;
        return;
      }
    }
    case MF_LIM_MINMOD:
    default:
      SLOPE = 0.5 * minmod(dWR, dWL);
      break;
  }
  *WL = WP - SLOPE;
  *WR = WP + SLOPE;
}

/* Limiter of primitive variable v: the driver sets minmod for every slope and
   then the per-variable limiters of the plasma variables
   (main/MHDAM.cpp:927-1009). */
static int limiter_of(const Ctx* c, int v) {
  if (v < 8) return c->p->limiter[v];
  if (v >= c->ils) return c->p->limiter_ls; /* main/MHDAM.cpp:1005-1006 */
  return MF_LIM_MINMOD;
}


/* ------------------------------------------------------------------------ */
/* characteristic reconstruction                                             */
/* ------------------------------------------------------------------------ */

/* minmod3 (src/reconstructionF.ChF:15-22) */
static double minmod3(double A, double B, double C) {
  double signA = copysign(1.0, A);
  return signA * fmax(0.0, fmin(fabs(A), fmin(signA * B, signA * C)));
}

/* *FACESLOPES: limited slopes of one variable from the left and right
   differences (src/reconstructionF.ChF: MINMODFACESLOPES :157-178,
   SUPERBEEFACESLOPES :356-392, HYPERBEEFACESLOPES :466-490,
   HARMONICFACESLOPES :526-550, VANALBADAFACESLOPES :591-622,
   MCFACESLOPES :664-697, VANLEERFACESLOPES :843-880, KORENFACESLOPES
   :920-948, VENKATAKRISHNANFACESLOPES :990-1021, CDFACESLOPES :1081-1096,
   WENO3FACESLOPES :1138-1167, WENO3YCFACESLOPES :1214-1246). */
static void face_slopes(int lim, double* Sleft, double* Sright) {
  double dSR = *Sright, dSL = *Sleft, SLOPE = 0.0;
  switch (lim) {
    case MF_LIM_CD:
      *Sleft = 0.5 * *Sleft;
      *Sright = 0.5 * *Sright;
      return;
    case MF_LIM_SUPERBEE:
      if (dSL * dSR > 0.0) {
        double AR = fabs(dSR), AL = fabs(dSL);
        if (AL <= 0.5 * AR)
          SLOPE = dSL;
        else if (AL <= AR)
          SLOPE = 0.5 * dSR;
        else if (AL <= AR + AR)
          SLOPE = 0.5 * dSL;
        else
          SLOPE = dSR;
      }
      break;
    case MF_LIM_HARMONIC:
      if (dSL * dSR > 0.0) SLOPE = dSR * dSL / (dSL + dSR);
      break;
    case MF_LIM_VANALBADA: {
      const double dSave = 1.0e-6, dSaveS = dSave + dSave;
      if (dSL * dSR > 0.0)
        SLOPE = 0.5 * (dSR * dSL + dSave) * (dSR + dSL) / (dSR * dSR + dSL * dSL + dSaveS);
      break;
    }
    case MF_LIM_MC:
      if (dSL * dSR > 0.0) {
        double AR = fabs(dSR), AL = fabs(dSL);
        if (3.0 * AL <= AR)
          SLOPE = dSL;
        else if (AL <= 3.0 * AR)
          SLOPE = 0.25 * (dSR + dSL);
        else
          SLOPE = dSR;
      }
      break;
    case MF_LIM_HYPERBEE:
      if (dSL * dSR > 0.0) {
        double A = 1.0 + sqrt(dSR / dSL);
        SLOPE = dSR / (A * A);
        SLOPE = SLOPE + SLOPE;
      }
      break;
    case MF_LIM_KOREN: {
      const double dSave = 1.0e-10;
      double SLOPL = 0.0, SLOPR = 0.0;
      if (dSL * dSR > 0.0) {
        double H = dSL * dSR / (2.0 * (dSL * dSL + dSR * dSR + dSave) - dSL * dSR);
        SLOPL = (dSL + 0.5 * dSR) * H;
        SLOPR = (dSR + 0.5 * dSL) * H;
      }
      *Sleft = SLOPL;
      *Sright = SLOPR;
      return;
    }
    case MF_LIM_VENKATAKRISHNAN: {
      const double dSave = 1.0e-10, dSave2 = dSave * dSave;
      double SLOPL = 0.0, SLOPR = 0.0;
      if (dSL * dSR > 0.0) {
        double H = (dSR + dSL) / (6.0 * (dSR * dSR + dSL * dSL + dSave2));
        SLOPL = (dSR + 2.0 * dSL) * (dSL + dSave) * H;
        SLOPR = (dSL + 2.0 * dSR) * (dSR + dSave) * H;
      }
      *Sleft = SLOPL;
      *Sright = SLOPR;
      return;
    }
    case MF_LIM_WENO3: {
      const double dSave = 1.0e-6;
      double BR = dSR * dSR + dSave, AR = 1.0 / (BR * BR);
      double BL = dSL * dSL + dSave, AL = 1.0 / (BL * BL);
      double H = AR / (AR + 2.0 * AL);
      *Sleft = 0.5 * (dSL + H * (dSR - dSL));
      H = AL / (AL + 2.0 * AR);
      *Sright = 0.5 * (dSR - H * (dSR - dSL));
      return;
    }
    case MF_LIM_WENO3YC: {
      const double dSave = 1.0e-6;
      double BR = dSR * dSR + dSave, BL = dSL * dSL + dSave;
      double D2P = dSR - dSL, AL, AR, H;
      D2P = D2P * D2P;
      AL = 1.0 + D2P / BL;
      AR = 1.0 + D2P / BR;
      H = AR / (AR + 2.0 * AL);
      *Sleft = 0.5 * (dSL + H * (dSR - dSL));
      H = AL / (AL + 2.0 * AR);
      *Sright = 0.5 * (dSR - H * (dSR - dSL));
      return;
    }
    case MF_LIM_VANLEER: {
      const double dSLim = 1.0 / 3.0;
      const double BT = (3.0 - dSLim) / (1.0 - dSLim);
      const double SL1 = 0.25 * (1.0 - dSLim);
      const double SL2 = 0.25 * (1.0 + dSLim);
      double SLOPL = 0.0, SLOPR = 0.0;
      if (dSL * dSR > 0.0) {
        double SL = fmin(fabs(dSR), fabs(BT * dSL));
        double SR = fmin(fabs(dSL), fabs(BT * dSR));
        SLOPL = SL1 * SL + SL2 * SR;
        SLOPR = SL1 * SR + SL2 * SL;
        if (dSR < 0.0) {
          SLOPL = -SLOPL;
          SLOPR = -SLOPR;
        }
      }
      *Sleft = SLOPL;
      *Sright = SLOPR;
      return;
    }
    case MF_LIM_MINMOD:
    default:
      SLOPE = 0.5 * minmod(dSR, dSL);
      break;
  }
  *Sleft = SLOPE;
  *Sright = SLOPE;
}

/* Wave speeds and mixing coefficients of CHARANALYSISF / CHARSYNTHESISF at
   a cell state (the two routines differ only in the dfs cut-off). */
typedef struct {
  double Rho, cc, c, as, af, alphaF, alphaS, betaY, betaZ, BX;
} CharState;

static void char_state(const Ctx* c, int d, const double* w, double dfs_cut, CharState* s) {
  const int inB = 5 + d, itB1 = 5 + (d + 1) % 3, itB2 = 5 + (d + 2) % 3;
  double PGas = w[4] > c->smallp ? w[4] : c->smallp;
  double Rho = w[0] > c->smallr ? w[0] : c->smallr;
  double BX = w[inB], BY = w[itB1], BZ = w[itB2];
  double cc = c->gamma * PGas / Rho;
  double cs = sqrt(cc);
  double BX2 = BX * BX, BY2 = BY * BY, BZ2 = BZ * BZ;
  double BYZ2 = BY2 + BZ2;
  double BxBH = D_1_8PI * (BX2 + BYZ2);
  double bb = D_1_4PI * BX2 / Rho;
  double b = sqrt(bb);
  double betaY, betaZ, aaf, aas, af, as;
  if (BYZ2 < c->smallB * c->smallB) {
    betaY = D_SQRT_2;
    betaZ = D_SQRT_2;
    if (bb > cc) {
      aaf = bb; aas = cc; af = b; as = cs;
    } else {
      aaf = cc; aas = bb; af = cs; as = b;
    }
  } else {
    double hyz = sqrt(BYZ2);
    betaY = BY / hyz;
    betaZ = BZ / hyz;
    double szb = cc + (BxBH + BxBH) / Rho;
    double h = sqrt(szb * szb - 4.0 * cc * bb);
    aas = 0.5 * (szb - h);
    as = sqrt(aas);
    aaf = 0.5 * (szb + h);
    af = sqrt(aaf);
  }
  double dfs = aaf - aas, alphaF, alphaS;
  if (dfs < dfs_cut) {
    alphaF = 1.0; alphaS = 0.0;
  } else if ((cc - aas) <= 0.0) {
    alphaF = 0.0; alphaS = 1.0;
  } else if ((aaf - cc) <= 0.0) {
    alphaF = 1.0; alphaS = 0.0;
  } else {
    alphaF = sqrt((cc - aas) / dfs);
    alphaS = sqrt((aaf - cc) / dfs);
  }
  s->Rho = Rho; s->cc = cc; s->c = cs; s->as = as; s->af = af;
  s->alphaF = alphaF; s->alphaS = alphaS; s->betaY = betaY; s->betaZ = betaZ; s->BX = BX;
}

/* CHARANALYSISF (srcIdeal/PatchIdealMHDF.ChF:1167-1328) on one slope vector
   dW (plasma primitives, global frame), in place. */
static void char_analysis1(const CharState* s, int d, double* dW) {
  const int in = 1 + d, it1 = 1 + (d + 1) % 3, it2 = 1 + (d + 2) % 3;
  const int inB = 5 + d, itB1 = 5 + (d + 1) % 3, itB2 = 5 + (d + 2) % 3;
  double siBX = copysign(1.0, s->BX);
  double dP = dW[4], dRho = dW[0], dUn = dW[in], dUt1 = dW[it1], dUt2 = dW[it2];
  double dBn = dW[inB], dBt1 = dW[itB1], dBt2 = dW[itB2];
  double Rho = s->Rho, cc = s->cc, betaY = s->betaY, betaZ = s->betaZ;
  dW[0] = dRho - dP / cc;
  dW[1] = dBn;
  double h1 = D_SQRT_2 * (betaY * dUt2 - betaZ * dUt1);
  double h2 = siBX * (betaZ * dBt1 - betaY * dBt2) / (2.0 * sqrt(2.0 * D_PI * Rho));
  dW[2] = h1 + h2;
  dW[3] = h1 - h2;
  h1 = dP / (2.0 * Rho * cc);
  h2 = dUn / (2.0 * cc);
  double h3 = (betaY * dBt1 + betaZ * dBt2) / (4.0 * s->c * sqrt(D_PI * Rho));
  double h4 = siBX * (betaY * dUt1 + betaZ * dUt2) / (2.0 * cc);
  double aF = s->alphaF, aS = s->alphaS, af = s->af, as = s->as;
  dW[4] = aF * (h1 + af * h2) + aS * (h3 - as * h4);
  dW[5] = aF * (h1 - af * h2) + aS * (h3 + as * h4);
  dW[6] = aS * (h1 + as * h2) - aF * (h3 - af * h4);
  dW[7] = aS * (h1 - as * h2) - aF * (h3 + af * h4);
}

/* CHARSYNTHESISF (srcIdeal/PatchIdealMHDF.ChF:1330-1500) on one vector of
   wave amplitudes, in place (back to primitive slopes, global frame). */
static void char_synthesis1(const CharState* s, int d, double* dW) {
  const int in = 1 + d, it1 = 1 + (d + 1) % 3, it2 = 1 + (d + 2) % 3;
  const int inB = 5 + d, itB1 = 5 + (d + 1) % 3, itB2 = 5 + (d + 2) % 3;
  double betaY = s->betaY, betaZ = s->betaZ, betaYX = betaY, betaZX = betaZ;
  if (s->BX < 0.0) {
    betaYX = -betaY;
    betaZX = -betaZ;
  }
  double alpha1 = dW[0], alpha2 = dW[1], alpha3 = dW[2], alpha4 = dW[3];
  double alpha5 = dW[4], alpha6 = dW[5], alpha7 = dW[6], alpha8 = dW[7];
  alpha3 = D_SQRT_2 * alpha3;
  alpha4 = D_SQRT_2 * alpha4;
  double alph3p4 = alpha3 + alpha4, alph3m4 = alpha3 - alpha4;
  double alph5p6 = alpha5 + alpha6, alph5m6 = alpha5 - alpha6;
  double alph7p8 = alpha7 + alpha8, alph7m8 = alpha7 - alpha8;
  double aF = s->alphaF, aS = s->alphaS, af = s->af, as = s->as;
  double DN = 2.0 * sqrt(D_PI * s->Rho);
  double HRho = s->Rho * (aF * alph5p6 + aS * alph7p8);
  double HU = aS * as * alph5m6 - aF * af * alph7m8;
  double HB = s->c * (aS * alph5p6 - aF * alph7p8);
  dW[0] = alpha1 + HRho;
  dW[in] = aF * af * alph5m6 + aS * as * alph7m8;
  dW[it1] = -betaZ * alph3p4 - betaYX * HU;
  dW[it2] = betaY * alph3p4 - betaZX * HU;
  dW[4] = s->cc * HRho;
  dW[inB] = alpha2;
  dW[itB1] = DN * (betaZX * alph3m4 + betaY * HB);
  dW[itB2] = DN * (-betaYX * alph3m4 + betaZ * HB);
}

/* One cell of Reconstruction::faceValues with characteristic limiting
   (src/Reconstruction.cpp:178-203): INITIALSLOPES, CHARANALYSISF on the
   plasma variables, the FACESLOPES of every variable, CHARSYNTHESISF,
   FROMSLOPESTOVALUES, then CHECKTVD on the variables main/MHDAM.cpp:939-968
   selects (check_tvd 1: the 8 plasma variables, 2: density and pressure). */
static void char_face_values(const Ctx* c, int d, const double* wm1, const double* w0,
                             const double* wp1, double* lo, double* hi) {
  const int np = c->nprim;
  double SL[MF_MAX_COMP], SR[MF_MAX_COMP];
  for (int v = 0; v < np; ++v) {
    SL[v] = w0[v] - wm1[v];
    SR[v] = wp1[v] - w0[v];
  }
  CharState sa, ss;
  char_state(c, d, w0, 1.0e-12, &sa);
  char_analysis1(&sa, d, SL);
  char_analysis1(&sa, d, SR);
  for (int v = 0; v < np; ++v) face_slopes(limiter_of(c, v), &SL[v], &SR[v]);
  char_state(c, d, w0, 1.0e-8, &ss);
  char_synthesis1(&ss, d, SL);
  char_synthesis1(&ss, d, SR);
  for (int v = 0; v < np; ++v) {
    lo[v] = w0[v] - SL[v];
    hi[v] = w0[v] + SR[v];
  }
  const int tvd = c->p->check_tvd;
  for (int v = 0; v < 8; ++v) {
    if (!(tvd == 1 || (tvd == 2 && (v == 0 || v == 4)))) continue;
    double WP = w0[v];
    double dWR = wp1[v] - WP, dWL = WP - wm1[v];
    double dSL = WP - lo[v], dSR = hi[v] - WP;
    lo[v] = WP - minmod3(dWL, dWR, dSL);
    hi[v] = WP + minmod3(dWL, dWR, dSR);
  }
}

/* ------------------------------------------------------------------------ */
/* Riemann solvers                                                           */
/* ------------------------------------------------------------------------ */

/* RIEMANNF, Roe 8-wave (src/Roe8WaveF.ChF:5-601), one face.  wl, wr are the
   left and right primitive states; g receives the fluxes at the prim indices
   (iRho = 0). */
static void roe8_face(const Ctx* c, int idir, const double* wl, const double* wr, double* g) {
  const double gamma = c->gamma, hgamma = c->hgamma, smallp = c->smallp, smallr = c->smallr;
  const double del2 = c->del2, smallB = c->smallB;
  const int inorm = 1 + idir, itan1 = 1 + (idir + 1) % 3, itan2 = 1 + (idir + 2) % 3;
  const int inormB = 5 + idir, itanB1 = 5 + (idir + 1) % 3, itanB2 = 5 + (idir + 2) % 3;
  double PGasL, RhoL, UL, VL, WL, RUL, RVL, RWL, BXL, BYL, BZL;
  double PGasR, RhoR, UR, VR, WR, RUR, RVR, RWR, BXR, BYR, BZR;
  double PGas, Rho, U, V, W, BX, BY, BZ;
  double BxBL, RUxUL, PL, EL, AL2, HL, coefRL, BxBR, RUxUR, PR, ER, AR2, HR, coefRR;
  double BxBH, P, HAV, BXAV, DBX, DBY, DBZ;
  double aas, as, aaf, af, alf, als, cc, c_, ccmi, ccma, dfs, X;
  double hyy = 0, hyz, hzz = 0, szb, h, kk, sih, z, del, dell2;
  double b, bb, BX2, BY2, BZ2, BYZ2, sqPiRho, sq2PiRho;
  double Ae[9], eig[9], eigmax;
  double fl[9], fr[9], du[9], lu[9], ra[9];
  double sp[9][9], so[9][9];

  PGasL = fmax(smallp, wl[4]);
  RhoL = fmax(smallr, wl[0]);
  UL = wl[inorm];
  VL = wl[itan1];
  WL = wl[itan2];
  BXL = wl[inormB];
  BYL = wl[itanB1];
  BZL = wl[itanB2];
  PGasR = fmax(smallp, wr[4]);
  RhoR = fmax(smallr, wr[0]);
  UR = wr[inorm];
  VR = wr[itan1];
  WR = wr[itan2];
  BXR = wr[inormB];
  BYR = wr[itanB1];
  BZR = wr[itanB2];

  RUL = RhoL * UL;
  RVL = RhoL * VL;
  RWL = RhoL * WL;
  BxBL = D_1_8PI * (BXL * BXL + BYL * BYL + BZL * BZL);
  RUxUL = 0.5 * (RUL * UL + RVL * VL + RWL * WL);
  PL = PGasL + BxBL;
  EL = PGasL / hgamma + RUxUL + BxBL;
  AL2 = gamma * PGasL / RhoL;

  RUR = RhoR * UR;
  RVR = RhoR * VR;
  RWR = RhoR * WR;
  BxBR = D_1_8PI * (BXR * BXR + BYR * BYR + BZR * BZR);
  RUxUR = 0.5 * (RUR * UR + RVR * VR + RWR * WR);
  PR = PGasR + BxBR;
  ER = PGasR / hgamma + RUxUR + BxBR;
  AR2 = gamma * PGasR / RhoR;

  if (AL2 > AR2) {
    ccmi = AR2;
    ccma = AL2;
  } else {
    ccmi = AL2;
    ccma = AR2;
  }

  if (c->aver == 1) {
    HL = (EL + PL) / RhoL;
    HR = (ER + PR) / RhoR;
    coefRL = 1.0 / (1.0 + sqrt(RhoR / RhoL));
    coefRR = 1.0 - coefRL;
    Rho = RhoR * coefRL + RhoL * coefRR;
    U = UL * coefRL + UR * coefRR;
    V = VL * coefRL + VR * coefRR;
    W = WL * coefRL + WR * coefRR;
    HAV = HL * coefRL + HR * coefRR;
    BX = BXR * coefRL + BXL * coefRR;
    BY = BYR * coefRL + BYL * coefRR;
    BZ = BZR * coefRL + BZL * coefRR;
    BXAV = 0.5 * (BXL + BXR);
    BX2 = BXAV * BXAV;
    BY2 = BY * BY;
    BZ2 = BZ * BZ;
    BYZ2 = BY2 + BZ2;
    BxBH = D_1_8PI * (BX2 + BYZ2);
    kk = 0.5 * (U * U + V * V + W * W);
    DBX = BXR - BXL;
    DBY = BYR - BYL;
    DBZ = BZR - BZL;
    X = D_1_8PI * (DBX * DBX + DBY * DBY + DBZ * DBZ) * coefRL * coefRL / RhoL;
    cc = hgamma * (HAV - kk - D_1_4PI * (BX * BXAV + BYZ2) / Rho) + (2.0 - gamma) * X;
  } else {
    Rho = 0.5 * (RhoL + RhoR);
    U = 0.5 * (UL + UR);
    V = 0.5 * (VL + VR);
    W = 0.5 * (WL + WR);
    BX = 0.5 * (BXL + BXR);
    BY = 0.5 * (BYL + BYR);
    BZ = 0.5 * (BZL + BZR);
    P = 0.5 * (PL + PR);
    BX2 = BX * BX;
    BY2 = BY * BY;
    BZ2 = BZ * BZ;
    BYZ2 = BY2 + BZ2;
    BxBH = D_1_8PI * (BX2 + BYZ2);
    kk = 0.5 * (U * U + V * V + W * W);
    PGas = P - BxBH;
    cc = gamma * PGas / Rho;
  }

  bb = D_1_4PI * BX2 / Rho;
  b = sqrt(bb);
  if (cc < ccmi) cc = ccmi;
  if (cc > ccma) cc = ccma;
  c_ = sqrt(cc);

  if (BYZ2 < smallB * smallB) {
    hyy = D_SQRT_2;
    hzz = D_SQRT_2;
    if (bb > cc) {
      aaf = bb;
      aas = cc;
      af = b;
      as = c_;
    } else {
      aaf = cc;
      aas = bb;
      af = c_;
      as = b;
    }
  } else {
    hyz = sqrt(BYZ2);
    hyy = BY / hyz;
    hzz = BZ / hyz;
    szb = cc + (BxBH + BxBH) / Rho;
    h = sqrt(szb * szb - 4.0 * cc * bb);
    aas = 0.5 * (szb - h);
    if (aas <= 0.0) {
      aas = 0.0;
      as = 0.0;
    } else if (aas >= cc) {
      aas = cc;
      as = c_;
    } else {
      as = sqrt(aas);
    }
    aaf = 0.5 * (szb + h);
    if (aaf <= cc) {
      aaf = cc;
      af = c_;
    } else {
      af = sqrt(aaf);
    }
  }

  eig[1] = U;
  eig[2] = U;
  eig[3] = U + b;
  eig[4] = U - b;
  eig[5] = U + af;
  eig[6] = U - af;
  eig[7] = U + as;
  eig[8] = U - as;
  eigmax = fabs(U) + fabs(V) + fabs(W) + af;
  del = del2 * eigmax;
  dell2 = del * del;
  for (int q = 1; q <= 8; ++q) {
    z = fabs(eig[q]);
    if (z >= del)
      Ae[q] = z;
    else
      Ae[q] = 0.5 * (z * z + dell2) / del;
  }

  dfs = aaf - aas;
  if (dfs < 1.0e-8) {
    alf = 1.0;
    als = 0.0;
  } else if ((cc - aas) <= 0.0) {
    alf = 0.0;
    als = 1.0;
  } else if ((aaf - cc) <= 0.0) {
    alf = 1.0;
    als = 0.0;
  } else {
    alf = sqrt((cc - aas) / dfs);
    als = sqrt((aaf - cc) / dfs);
  }

  sih = -1.0;
  if (BX >= 0.0) sih = 1.0;

  fl[1] = RUL;
  fl[2] = UL * RUL - BXL * BXL * D_1_4PI + PL;
  fl[3] = UL * RVL - BXL * BYL * D_1_4PI;
  fl[4] = UL * RWL - BXL * BZL * D_1_4PI;
  fl[5] = UL * (EL + PL) - BXL * (UL * BXL + VL * BYL + WL * BZL) * D_1_4PI;
  fl[6] = 0.0;
  fl[7] = UL * BYL - BXL * VL;
  fl[8] = UL * BZL - BXL * WL;

  fr[1] = RUR;
  fr[2] = UR * RUR - BXR * BXR * D_1_4PI + PR;
  fr[3] = UR * RVR - BXR * BYR * D_1_4PI;
  fr[4] = UR * RWR - BXR * BZR * D_1_4PI;
  fr[5] = UR * (ER + PR) - BXR * (UR * BXR + VR * BYR + WR * BZR) * D_1_4PI;
  fr[6] = 0.0;
  fr[7] = UR * BYR - BXR * VR;
  fr[8] = UR * BZR - BXR * WR;

  du[1] = RhoL - RhoR;
  du[2] = RUL - RUR;
  du[3] = RVL - RVR;
  du[4] = RWL - RWR;
  du[5] = EL - ER;
  du[6] = BXL - BXR;
  du[7] = BYL - BYR;
  du[8] = BZL - BZR;

  du[5] = -hgamma * (-kk * du[1] + U * du[2] + V * du[3] + W * du[4] - du[5] +
                     (BX * du[6] + BY * du[7] + BZ * du[8]) * D_1_4PI);
  du[2] = (-U * du[1] + du[2]) / Rho;
  du[3] = (-V * du[1] + du[3]) / Rho;
  du[4] = (-W * du[1] + du[4]) / Rho;

  sqPiRho = sqrt(D_PI * Rho);
  sq2PiRho = sqrt(D_2PI * Rho);

  sp[1][1] = 1.0; sp[1][2] = 0.0; sp[1][3] = 0.0; sp[1][4] = 0.0;
  sp[1][5] = Rho * alf; sp[1][6] = Rho * alf; sp[1][7] = Rho * als; sp[1][8] = Rho * als;

  sp[2][1] = 0.0; sp[2][2] = 0.0; sp[2][3] = 0.0; sp[2][4] = 0.0;
  sp[2][5] = alf * af; sp[2][6] = -alf * af; sp[2][7] = als * as; sp[2][8] = -als * as;

  sp[3][1] = 0.0; sp[3][2] = 0.0;
  sp[3][3] = -hzz * D_SQRT_2; sp[3][4] = -hzz * D_SQRT_2;
  sp[3][5] = -als * as * hyy * sih; sp[3][6] = als * as * hyy * sih;
  sp[3][7] = alf * af * hyy * sih; sp[3][8] = -alf * af * hyy * sih;

  sp[4][1] = 0.0; sp[4][2] = 0.0;
  sp[4][3] = hyy * D_SQRT_2; sp[4][4] = hyy * D_SQRT_2;
  sp[4][5] = -als * as * hzz * sih; sp[4][6] = als * as * hzz * sih;
  sp[4][7] = alf * af * hzz * sih; sp[4][8] = -alf * af * hzz * sih;

  sp[5][1] = 0.0; sp[5][2] = 0.0; sp[5][3] = 0.0; sp[5][4] = 0.0;
  sp[5][5] = alf * Rho * cc; sp[5][6] = alf * Rho * cc;
  sp[5][7] = als * Rho * cc; sp[5][8] = als * Rho * cc;

  sp[6][1] = 0.0; sp[6][2] = 1.0; sp[6][3] = 0.0; sp[6][4] = 0.0;
  sp[6][5] = 0.0; sp[6][6] = 0.0; sp[6][7] = 0.0; sp[6][8] = 0.0;

  sp[7][1] = 0.0; sp[7][2] = 0.0;
  sp[7][3] = hzz * sq2PiRho * sih; sp[7][4] = -hzz * sq2PiRho * sih;
  sp[7][5] = 2.0 * als * sqPiRho * c_ * hyy; sp[7][6] = 2.0 * als * sqPiRho * c_ * hyy;
  sp[7][7] = -2.0 * alf * sqPiRho * c_ * hyy; sp[7][8] = -2.0 * alf * sqPiRho * c_ * hyy;

  sp[8][1] = 0.0; sp[8][2] = 0.0;
  sp[8][3] = -hyy * sq2PiRho * sih; sp[8][4] = hyy * sq2PiRho * sih;
  sp[8][5] = 2.0 * als * sqPiRho * c_ * hzz; sp[8][6] = 2.0 * als * sqPiRho * c_ * hzz;
  sp[8][7] = -2.0 * alf * sqPiRho * c_ * hzz; sp[8][8] = -2.0 * alf * sqPiRho * c_ * hzz;

  so[1][1] = 1.0; so[1][2] = 0.0; so[1][3] = 0.0; so[1][4] = 0.0;
  so[1][5] = -1.0 / cc; so[1][6] = 0.0; so[1][7] = 0.0; so[1][8] = 0.0;

  so[2][1] = 0.0; so[2][2] = 0.0; so[2][3] = 0.0; so[2][4] = 0.0;
  so[2][5] = 0.0; so[2][6] = 1.0; so[2][7] = 0.0; so[2][8] = 0.0;

  so[3][1] = 0.0; so[3][2] = 0.0;
  so[3][3] = -hzz * D_SQRT_2; so[3][4] = hyy * D_SQRT_2;
  so[3][5] = 0.0; so[3][6] = 0.0;
  so[3][7] = 0.5 * hzz * sih / sq2PiRho; so[3][8] = -0.5 * hyy * sih / sq2PiRho;

  so[4][1] = 0.0; so[4][2] = 0.0;
  so[4][3] = -hzz * D_SQRT_2; so[4][4] = hyy * D_SQRT_2;
  so[4][5] = 0.0; so[4][6] = 0.0;
  so[4][7] = -0.5 * hzz * sih / sq2PiRho; so[4][8] = 0.5 * hyy * sih / sq2PiRho;

  so[5][1] = 0.0;
  so[5][2] = 0.5 * alf * af / cc;
  so[5][3] = -0.5 * als * as * hyy * sih / cc;
  so[5][4] = -0.5 * als * as * hzz * sih / cc;
  so[5][5] = 0.5 * alf / (cc * Rho);
  so[5][6] = 0.0;
  so[5][7] = 0.25 * als * hyy / (c_ * sqPiRho);
  so[5][8] = 0.25 * als * hzz / (c_ * sqPiRho);

  so[6][1] = 0.0;
  so[6][2] = -0.5 * alf * af / cc;
  so[6][3] = 0.5 * als * as * hyy * sih / cc;
  so[6][4] = 0.5 * als * as * hzz * sih / cc;
  so[6][5] = 0.5 * alf / (cc * Rho);
  so[6][6] = 0.0;
  so[6][7] = 0.25 * als * hyy / (c_ * sqPiRho);
  so[6][8] = 0.25 * als * hzz / (c_ * sqPiRho);

  so[7][1] = 0.0;
  so[7][2] = 0.5 * als * as / cc;
  so[7][3] = 0.5 * alf * af * hyy * sih / cc;
  so[7][4] = 0.5 * alf * af * hzz * sih / cc;
  so[7][5] = 0.5 * als / (Rho * cc);
  so[7][6] = 0.0;
  so[7][7] = -0.25 * alf * hyy / (c_ * sqPiRho);
  so[7][8] = -0.25 * alf * hzz / (c_ * sqPiRho);

  so[8][1] = 0.0;
  so[8][2] = -0.5 * als * as / cc;
  so[8][3] = -0.5 * alf * af * hyy * sih / cc;
  so[8][4] = -0.5 * alf * af * hzz * sih / cc;
  so[8][5] = 0.5 * als / (Rho * cc);
  so[8][6] = 0.0;
  so[8][7] = -0.25 * alf * hyy / (c_ * sqPiRho);
  so[8][8] = -0.25 * alf * hzz / (c_ * sqPiRho);

  for (int r = 1; r <= 8; ++r) {
    double s = so[r][1] * du[1];
    for (int q = 2; q <= 8; ++q) s = s + so[r][q] * du[q];
    lu[r] = Ae[r] * s;
  }
  for (int r = 1; r <= 8; ++r) {
    double s = sp[r][1] * lu[1];
    for (int q = 2; q <= 8; ++q) s = s + sp[r][q] * lu[q];
    ra[r] = s;
  }
  ra[5] = ra[1] * kk + Rho * (U * ra[2] + V * ra[3] + W * ra[4]) + ra[5] / hgamma +
          D_1_4PI * (BX * ra[6] + BY * ra[7] + BZ * ra[8]);
  ra[2] = U * ra[1] + Rho * ra[2];
  ra[3] = V * ra[1] + Rho * ra[3];
  ra[4] = W * ra[1] + Rho * ra[4];

  g[0] = 0.5 * (fl[1] + fr[1] + ra[1]);
  g[inorm] = 0.5 * (fl[2] + fr[2] + ra[2]);
  g[itan1] = 0.5 * (fl[3] + fr[3] + ra[3]);
  g[itan2] = 0.5 * (fl[4] + fr[4] + ra[4]);
  g[4] = 0.5 * (fl[5] + fr[5] + ra[5]);
  g[inormB] = 0.5 * (fl[6] + fr[6] + ra[6]);
  g[itanB1] = 0.5 * (fl[7] + fr[7] + ra[7]);
  g[itanB2] = 0.5 * (fl[8] + fr[8] + ra[8]);
}

/* RIEMANN7F, Roe 7-wave (src/Roe7WaveF.ChF:5-558), one face.  Identical to
   RIEMANNF up to the speeds; the normal-B wave is removed and the normal-B
   flux is zero (:522). */
static void roe7_face(const Ctx* c, int idir, const double* wl, const double* wr, double* g) {
  const double gamma = c->gamma, hgamma = c->hgamma, smallp = c->smallp, smallr = c->smallr;
  const double del2 = c->del2, smallB = c->smallB;
  const int inorm = 1 + idir, itan1 = 1 + (idir + 1) % 3, itan2 = 1 + (idir + 2) % 3;
  const int inormB = 5 + idir, itanB1 = 5 + (idir + 1) % 3, itanB2 = 5 + (idir + 2) % 3;
  double PGasL, RhoL, UL, VL, WL, RUL, RVL, RWL, BXL, BYL, BZL;
  double PGasR, RhoR, UR, VR, WR, RUR, RVR, RWR, BXR, BYR, BZR;
  double PGas, Rho, U, V, W, BX, BY, BZ;
  double BxBL, RUxUL, PL, EL, AL2, HL, coefRL, BxBR, RUxUR, PR, ER, AR2, HR, coefRR;
  double BxBH, P, HAV, BXAV, DBX, DBY, DBZ;
  double aas, as, aaf, af, alf, als, cc, c_, ccmi, ccma, dfs, X;
  double hyy = 0, hyz, hzz = 0, szb, h, kk, sih, z, del, dell2;
  double b, bb, BX2, BY2, BZ2, BYZ2, sqPiRho, sq2PiRho;
  double Ae[8], eig[8], eigmax;
  double fl[8], fr[8], du[8], lu[8], ra[8];
  double sp[8][8], so[8][8];

  PGasL = fmax(smallp, wl[4]);
  RhoL = fmax(smallr, wl[0]);
  UL = wl[inorm];
  VL = wl[itan1];
  WL = wl[itan2];
  BXL = wl[inormB];
  BYL = wl[itanB1];
  BZL = wl[itanB2];
  PGasR = fmax(smallp, wr[4]);
  RhoR = fmax(smallr, wr[0]);
  UR = wr[inorm];
  VR = wr[itan1];
  WR = wr[itan2];
  BXR = wr[inormB];
  BYR = wr[itanB1];
  BZR = wr[itanB2];

  RUL = RhoL * UL;
  RVL = RhoL * VL;
  RWL = RhoL * WL;
  BxBL = D_1_8PI * (BXL * BXL + BYL * BYL + BZL * BZL);
  RUxUL = 0.5 * (RUL * UL + RVL * VL + RWL * WL);
  PL = PGasL + BxBL;
  EL = PGasL / hgamma + RUxUL + BxBL;
  AL2 = gamma * PGasL / RhoL;

  RUR = RhoR * UR;
  RVR = RhoR * VR;
  RWR = RhoR * WR;
  BxBR = D_1_8PI * (BXR * BXR + BYR * BYR + BZR * BZR);
  RUxUR = 0.5 * (RUR * UR + RVR * VR + RWR * WR);
  PR = PGasR + BxBR;
  ER = PGasR / hgamma + RUxUR + BxBR;
  AR2 = gamma * PGasR / RhoR;

  if (AL2 > AR2) {
    ccmi = AR2;
    ccma = AL2;
  } else {
    ccmi = AL2;
    ccma = AR2;
  }

  if (c->aver == 1) {
    HL = (EL + PL) / RhoL;
    HR = (ER + PR) / RhoR;
    coefRL = 1.0 / (1.0 + sqrt(RhoR / RhoL));
    coefRR = 1.0 - coefRL;
    Rho = RhoR * coefRL + RhoL * coefRR;
    U = UL * coefRL + UR * coefRR;
    V = VL * coefRL + VR * coefRR;
    W = WL * coefRL + WR * coefRR;
    HAV = HL * coefRL + HR * coefRR;
    BX = BXR * coefRL + BXL * coefRR;
    BY = BYR * coefRL + BYL * coefRR;
    BZ = BZR * coefRL + BZL * coefRR;
    BXAV = 0.5 * (BXL + BXR);
    BX2 = BXAV * BXAV;
    BY2 = BY * BY;
    BZ2 = BZ * BZ;
    BYZ2 = BY2 + BZ2;
    BxBH = D_1_8PI * (BX2 + BYZ2);
    kk = 0.5 * (U * U + V * V + W * W);
    DBX = BXR - BXL;
    DBY = BYR - BYL;
    DBZ = BZR - BZL;
    X = D_1_8PI * (DBX * DBX + DBY * DBY + DBZ * DBZ) * coefRL * coefRL / RhoL;
    cc = hgamma * (HAV - kk - D_1_4PI * (BX * BXAV + BYZ2) / Rho) + (2.0 - gamma) * X;
  } else {
    Rho = 0.5 * (RhoL + RhoR);
    U = 0.5 * (UL + UR);
    V = 0.5 * (VL + VR);
    W = 0.5 * (WL + WR);
    BX = 0.5 * (BXL + BXR);
    BY = 0.5 * (BYL + BYR);
    BZ = 0.5 * (BZL + BZR);
    P = 0.5 * (PL + PR);
    BX2 = BX * BX;
    BY2 = BY * BY;
    BZ2 = BZ * BZ;
    BYZ2 = BY2 + BZ2;
    BxBH = D_1_8PI * (BX2 + BYZ2);
    kk = 0.5 * (U * U + V * V + W * W);
    PGas = P - BxBH;
    cc = gamma * PGas / Rho;
  }

  bb = D_1_4PI * BX2 / Rho;
  b = sqrt(bb);
  if (cc < ccmi) cc = ccmi;
  if (cc > ccma) cc = ccma;
  c_ = sqrt(cc);

  if (BYZ2 < smallB * smallB) {
    hyy = D_SQRT_2;
    hzz = D_SQRT_2;
    if (bb > cc) {
      aaf = bb;
      aas = cc;
      af = b;
      as = c_;
    } else {
      aaf = cc;
      aas = bb;
      af = c_;
      as = b;
    }
  } else {
    hyz = sqrt(BYZ2);
    hyy = BY / hyz;
    hzz = BZ / hyz;
    szb = cc + (BxBH + BxBH) / Rho;
    h = sqrt(szb * szb - 4.0 * cc * bb);
    aas = 0.5 * (szb - h);
    if (aas <= 0.0) {
      aas = 0.0;
      as = 0.0;
    } else if (aas >= cc) {
      aas = cc;
      as = c_;
    } else {
      as = sqrt(aas);
    }
    aaf = 0.5 * (szb + h);
    if (aaf <= cc) {
      aaf = cc;
      af = c_;
    } else {
      af = sqrt(aaf);
    }
  }

  eig[1] = U;
  eig[2] = U + b;
  eig[3] = U - b;
  eig[4] = U + af;
  eig[5] = U - af;
  eig[6] = U + as;
  eig[7] = U - as;
  eigmax = fabs(U) + fabs(V) + fabs(W) + af;
  del = del2 * eigmax;
  dell2 = del * del;
  for (int q = 1; q <= 7; ++q) {
    z = fabs(eig[q]);
    if (z >= del)
      Ae[q] = z;
    else
      Ae[q] = 0.5 * (z * z + dell2) / del;
  }

  dfs = aaf - aas;
  if (dfs < 1.0e-8) {
    alf = 1.0;
    als = 0.0;
  } else if ((cc - aas) <= 0.0) {
    alf = 0.0;
    als = 1.0;
  } else if ((aaf - cc) <= 0.0) {
    alf = 1.0;
    als = 0.0;
  } else {
    alf = sqrt((cc - aas) / dfs);
    als = sqrt((aaf - cc) / dfs);
  }

  sih = -1.0;
  if (BX >= 0.0) sih = 1.0;

  fl[1] = RUL;
  fl[2] = UL * RUL - BXL * BXL * D_1_4PI + PL;
  fl[3] = UL * RVL - BXL * BYL * D_1_4PI;
  fl[4] = UL * RWL - BXL * BZL * D_1_4PI;
  fl[5] = UL * (EL + PL) - BXL * (UL * BXL + VL * BYL + WL * BZL) * D_1_4PI;
  fl[6] = UL * BYL - BXL * VL;
  fl[7] = UL * BZL - BXL * WL;

  fr[1] = RUR;
  fr[2] = UR * RUR - BXR * BXR * D_1_4PI + PR;
  fr[3] = UR * RVR - BXR * BYR * D_1_4PI;
  fr[4] = UR * RWR - BXR * BZR * D_1_4PI;
  fr[5] = UR * (ER + PR) - BXR * (UR * BXR + VR * BYR + WR * BZR) * D_1_4PI;
  fr[6] = UR * BYR - BXR * VR;
  fr[7] = UR * BZR - BXR * WR;

  du[1] = RhoL - RhoR;
  du[2] = RUL - RUR;
  du[3] = RVL - RVR;
  du[4] = RWL - RWR;
  du[5] = EL - ER;
  du[6] = BYL - BYR;
  du[7] = BZL - BZR;

  du[5] = -hgamma * (-kk * du[1] + U * du[2] + V * du[3] + W * du[4] - du[5] +
                     (BY * du[6] + BZ * du[7]) * D_1_4PI);
  du[2] = (-U * du[1] + du[2]) / Rho;
  du[3] = (-V * du[1] + du[3]) / Rho;
  du[4] = (-W * du[1] + du[4]) / Rho;

  sqPiRho = sqrt(D_PI * Rho);
  sq2PiRho = sqrt(D_2PI * Rho);

  sp[1][1] = 1.0; sp[1][2] = 0.0; sp[1][3] = 0.0;
  sp[1][4] = Rho * alf; sp[1][5] = Rho * alf; sp[1][6] = Rho * als; sp[1][7] = Rho * als;

  sp[2][1] = 0.0; sp[2][2] = 0.0; sp[2][3] = 0.0;
  sp[2][4] = alf * af; sp[2][5] = -alf * af; sp[2][6] = als * as; sp[2][7] = -als * as;

  sp[3][1] = 0.0;
  sp[3][2] = -hzz * D_SQRT_2; sp[3][3] = -hzz * D_SQRT_2;
  sp[3][4] = -als * as * hyy * sih; sp[3][5] = als * as * hyy * sih;
  sp[3][6] = alf * af * hyy * sih; sp[3][7] = -alf * af * hyy * sih;

  sp[4][1] = 0.0;
  sp[4][2] = hyy * D_SQRT_2; sp[4][3] = hyy * D_SQRT_2;
  sp[4][4] = -als * as * hzz * sih; sp[4][5] = als * as * hzz * sih;
  sp[4][6] = alf * af * hzz * sih; sp[4][7] = -alf * af * hzz * sih;

  sp[5][1] = 0.0; sp[5][2] = 0.0; sp[5][3] = 0.0;
  sp[5][4] = alf * Rho * cc; sp[5][5] = alf * Rho * cc;
  sp[5][6] = als * Rho * cc; sp[5][7] = als * Rho * cc;

  sp[6][1] = 0.0;
  sp[6][2] = hzz * sq2PiRho * sih; sp[6][3] = -hzz * sq2PiRho * sih;
  sp[6][4] = 2.0 * als * sqPiRho * c_ * hyy; sp[6][5] = 2.0 * als * sqPiRho * c_ * hyy;
  sp[6][6] = -2.0 * alf * sqPiRho * c_ * hyy; sp[6][7] = -2.0 * alf * sqPiRho * c_ * hyy;

  sp[7][1] = 0.0;
  sp[7][2] = -hyy * sq2PiRho * sih; sp[7][3] = hyy * sq2PiRho * sih;
  sp[7][4] = 2.0 * als * sqPiRho * c_ * hzz; sp[7][5] = 2.0 * als * sqPiRho * c_ * hzz;
  sp[7][6] = -2.0 * alf * sqPiRho * c_ * hzz; sp[7][7] = -2.0 * alf * sqPiRho * c_ * hzz;

  so[1][1] = 1.0; so[1][2] = 0.0; so[1][3] = 0.0; so[1][4] = 0.0;
  so[1][5] = -1.0 / cc; so[1][6] = 0.0; so[1][7] = 0.0;

  so[2][1] = 0.0; so[2][2] = 0.0;
  so[2][3] = -hzz * D_SQRT_2; so[2][4] = hyy * D_SQRT_2; so[2][5] = 0.0;
  so[2][6] = 0.5 * hzz * sih / sq2PiRho; so[2][7] = -0.5 * hyy * sih / sq2PiRho;

  so[3][1] = 0.0; so[3][2] = 0.0;
  so[3][3] = -hzz * D_SQRT_2; so[3][4] = hyy * D_SQRT_2; so[3][5] = 0.0;
  so[3][6] = -0.5 * hzz * sih / sq2PiRho; so[3][7] = 0.5 * hyy * sih / sq2PiRho;

  so[4][1] = 0.0;
  so[4][2] = 0.5 * alf * af / cc;
  so[4][3] = -0.5 * als * as * hyy * sih / cc;
  so[4][4] = -0.5 * als * as * hzz * sih / cc;
  so[4][5] = 0.5 * alf / (cc * Rho);
  so[4][6] = 0.25 * als * hyy / (c_ * sqPiRho);
  so[4][7] = 0.25 * als * hzz / (c_ * sqPiRho);

  so[5][1] = 0.0;
  so[5][2] = -0.5 * alf * af / cc;
  so[5][3] = 0.5 * als * as * hyy * sih / cc;
  so[5][4] = 0.5 * als * as * hzz * sih / cc;
  so[5][5] = 0.5 * alf / (cc * Rho);
  so[5][6] = 0.25 * als * hyy / (c_ * sqPiRho);
  so[5][7] = 0.25 * als * hzz / (c_ * sqPiRho);

  so[6][1] = 0.0;
  so[6][2] = 0.5 * als * as / cc;
  so[6][3] = 0.5 * alf * af * hyy * sih / cc;
  so[6][4] = 0.5 * alf * af * hzz * sih / cc;
  so[6][5] = 0.5 * als / (Rho * cc);
  so[6][6] = -0.25 * alf * hyy / (c_ * sqPiRho);
  so[6][7] = -0.25 * alf * hzz / (c_ * sqPiRho);

  so[7][1] = 0.0;
  so[7][2] = -0.5 * als * as / cc;
  so[7][3] = -0.5 * alf * af * hyy * sih / cc;
  so[7][4] = -0.5 * alf * af * hzz * sih / cc;
  so[7][5] = 0.5 * als / (Rho * cc);
  so[7][6] = -0.25 * alf * hyy / (c_ * sqPiRho);
  so[7][7] = -0.25 * alf * hzz / (c_ * sqPiRho);

  for (int r = 1; r <= 7; ++r) {
    double s = so[r][1] * du[1];
    for (int q = 2; q <= 7; ++q) s = s + so[r][q] * du[q];
    lu[r] = Ae[r] * s;
  }
  for (int r = 1; r <= 7; ++r) {
    double s = sp[r][1] * lu[1];
    for (int q = 2; q <= 7; ++q) s = s + sp[r][q] * lu[q];
    ra[r] = s;
  }
  ra[5] = ra[1] * kk + Rho * (U * ra[2] + V * ra[3] + W * ra[4]) + ra[5] / hgamma +
          D_1_4PI * (BY * ra[6] + BZ * ra[7]);
  ra[2] = U * ra[1] + Rho * ra[2];
  ra[3] = V * ra[1] + Rho * ra[3];
  ra[4] = W * ra[1] + Rho * ra[4];

  g[0] = 0.5 * (fl[1] + fr[1] + ra[1]);
  g[inorm] = 0.5 * (fl[2] + fr[2] + ra[2]);
  g[itan1] = 0.5 * (fl[3] + fr[3] + ra[3]);
  g[itan2] = 0.5 * (fl[4] + fr[4] + ra[4]);
  g[4] = 0.5 * (fl[5] + fr[5] + ra[5]);
  g[itanB1] = 0.5 * (fl[6] + fr[6] + ra[6]);
  g[itanB2] = 0.5 * (fl[7] + fr[7] + ra[7]);
  g[inormB] = 0.0;
}

/* RUSANOVF (src/RusanovF.ChF:4-197), one face. */
static void rusanov_face(const Ctx* c, int idir, const double* wl, const double* wr, double* g) {
  const double gamma = c->gamma, hgamma = c->hgamma, smallp = c->smallp, smallr = c->smallr;
  const int inorm = 1 + idir, itan1 = 1 + (idir + 1) % 3, itan2 = 1 + (idir + 2) % 3;
  const int inormB = 5 + idir, itanB1 = 5 + (idir + 1) % 3, itanB2 = 5 + (idir + 2) % 3;
  double PGasL = fmax(smallp, wl[4]), RhoL = fmax(smallr, wl[0]);
  double UL = wl[inorm], VL = wl[itan1], WL = wl[itan2];
  double BXL = wl[inormB], BYL = wl[itanB1], BZL = wl[itanB2];
  double PGasR = fmax(smallp, wr[4]), RhoR = fmax(smallr, wr[0]);
  double UR = wr[inorm], VR = wr[itan1], WR = wr[itan2];
  double BXR = wr[inormB], BYR = wr[itanB1], BZR = wr[itanB2];
  double RUL = RhoL * UL, RVL = RhoL * VL, RWL = RhoL * WL;
  double BxBL = D_1_8PI * (BXL * BXL + BYL * BYL + BZL * BZL);
  double RUxUL = 0.5 * (RUL * UL + RVL * VL + RWL * WL);
  double PL = PGasL + BxBL;
  double EL = PGasL / hgamma + RUxUL + BxBL;
  double BXL_4PI = BXL * D_1_4PI;
  double RUR = RhoR * UR, RVR = RhoR * VR, RWR = RhoR * WR;
  double BxBR = D_1_8PI * (BXR * BXR + BYR * BYR + BZR * BZR);
  double RUxUR = 0.5 * (RUR * UR + RVR * VR + RWR * WR);
  double PR = PGasR + BxBR;
  double ER = PGasR / hgamma + RUxUR + BxBR;
  double BXR_4PI = BXR * D_1_4PI;
  double Rho, U, BX2, BxBH, A2;
  if (c->aver == 1) {
    double HL = (EL + PL) / RhoL, HR = (ER + PR) / RhoR;
    double coefRL = 1.0 / (1.0 + sqrt(RhoR / RhoL));
    double coefRR = 1.0 - coefRL;
    Rho = RhoR * coefRL + RhoL * coefRR;
    U = UL * coefRL + UR * coefRR;
    double V = VL * coefRL + VR * coefRR;
    double W = WL * coefRL + WR * coefRR;
    double HAV = HL * coefRL + HR * coefRR;
    double BX = BXR * coefRL + BXL * coefRR;
    double BY = BYR * coefRL + BYL * coefRR;
    double BZ = BZR * coefRL + BZL * coefRR;
    double BXAV = 0.5 * (BXL + BXR);
    BX2 = BXAV * BXAV;
    double BY2 = BY * BY, BZ2 = BZ * BZ;
    double BYZ2 = BY2 + BZ2;
    BxBH = D_1_8PI * (BX2 + BYZ2);
    double kk = 0.5 * (U * U + V * V + W * W);
    double DBX = BXR - BXL, DBY = BYR - BYL, DBZ = BZR - BZL;
    double X = D_1_8PI * (DBX * DBX + DBY * DBY + DBZ * DBZ) * coefRL * coefRL / RhoL;
    A2 = hgamma * (HAV - kk - D_1_4PI * (BX * BXAV + BYZ2) / Rho) + (2.0 - gamma) * X;
  } else {
    Rho = 0.5 * (RhoL + RhoR);
    U = 0.5 * (UL + UR);
    double BX = 0.5 * (BXL + BXR), BY = 0.5 * (BYL + BYR), BZ = 0.5 * (BZL + BZR);
    double PGas = 0.5 * (PGasL + PGasR);
    BX2 = BX * BX;
    double BY2 = BY * BY, BZ2 = BZ * BZ;
    BxBH = D_1_8PI * (BX2 + BY2 + BZ2);
    A2 = gamma * PGas / Rho;
  }
  double bb = D_1_4PI * BX2 / Rho;
  double szb = A2 + (BxBH + BxBH) / Rho;
  double h = sqrt(szb * szb - 4.0 * A2 * bb);
  double aaf = 0.5 * (szb + h);
  double af = sqrt(aaf);
  double eigmax = fabs(U) + af;
  double fl[9], fr[9], du[9];
  fl[1] = RUL;
  fl[2] = UL * RUL - BXL_4PI * BXL + PL;
  fl[3] = UL * RVL - BXL_4PI * BYL;
  fl[4] = UL * RWL - BXL_4PI * BZL;
  fl[5] = UL * (EL + PL) - BXL_4PI * (UL * BXL + VL * BYL + WL * BZL);
  fl[6] = 0.0;
  fl[7] = UL * BYL - BXL * VL;
  fl[8] = UL * BZL - BXL * WL;
  fr[1] = RUR;
  fr[2] = UR * RUR - BXR_4PI * BXR + PR;
  fr[3] = UR * RVR - BXR_4PI * BYR;
  fr[4] = UR * RWR - BXR_4PI * BZR;
  fr[5] = UR * (ER + PR) - BXR_4PI * (UR * BXR + VR * BYR + WR * BZR);
  fr[6] = 0.0;
  fr[7] = UR * BYR - BXR * VR;
  fr[8] = UR * BZR - BXR * WR;
  du[1] = RhoL - RhoR;
  du[2] = RUL - RUR;
  du[3] = RVL - RVR;
  du[4] = RWL - RWR;
  du[5] = EL - ER;
  du[6] = BXL - BXR;
  du[7] = BYL - BYR;
  du[8] = BZL - BZR;
  g[0] = 0.5 * (fl[1] + fr[1] + eigmax * du[1]);
  g[inorm] = 0.5 * (fl[2] + fr[2] + eigmax * du[2]);
  g[itan1] = 0.5 * (fl[3] + fr[3] + eigmax * du[3]);
  g[itan2] = 0.5 * (fl[4] + fr[4] + eigmax * du[4]);
  g[4] = 0.5 * (fl[5] + fr[5] + eigmax * du[5]);
  g[inormB] = 0.5 * (fl[6] + fr[6] + eigmax * du[6]);
  g[itanB1] = 0.5 * (fl[7] + fr[7] + eigmax * du[7]);
  g[itanB2] = 0.5 * (fl[8] + fr[8] + eigmax * du[8]);
}

/* DEDNER2X2F (src/DednerF.ChF:89-170): (Bn, psi) flux with speed Ch. */
static void dedner_face(const Ctx* c, int idir, const double* wl, const double* wr, double* g) {
  const int inormB = 5 + idir, iPsi = 8;
  double dCh = c->dCh, dCh2 = dCh * dCh;
  double sp11 = 1.0, sp12 = 1.0, sp21 = -dCh, sp22 = dCh;
  double so11 = 0.5, so12 = -0.5 / dCh, so21 = 0.5, so22 = 0.5 / dCh;
  double BXL = wl[inormB], PsiL = wl[iPsi], BXR = wr[inormB], PsiR = wr[iPsi];
  double Aeigen1 = dCh, Aeigen2 = dCh;
  double fl1 = PsiL, fl2 = dCh2 * BXL, fr1 = PsiR, fr2 = dCh2 * BXR;
  double du1 = BXL - BXR, du2 = PsiL - PsiR;
  double lu1 = Aeigen1 * (so11 * du1 + so12 * du2);
  double lu2 = Aeigen2 * (so21 * du1 + so22 * du2);
  double ra1 = sp11 * lu1 + sp12 * lu2;
  double ra2 = sp21 * lu1 + sp22 * lu2;
  g[inormB] = 0.5 * (fl1 + fr1 + ra1);
  g[iPsi] = 0.5 * (fl2 + fr2 + ra2);
}

/* VANLEERF (src/VanLeerRSF.ChF:4-130): van Leer flux-vector splitting of one
   Euler fluid whose density sits at index irho. */
static void vanleer_face(const Ctx* c, int idir, int irho, const double* wl, const double* wr,
                         double* g) {
  const double gamma = c->gamma, hgamma = c->hgamma, smallp = c->smallp, smallr = c->smallr;
  const int iPres = irho + 4;
  const int inorm = irho + 1 + idir, itan1 = irho + 1 + (idir + 1) % 3,
            itan2 = irho + 1 + (idir + 2) % 3;
  double fl1, fl2, fl3, fl4, fl5, fr1, fr2, fr3, fr4, fr5;
  double PGasL = fmax(smallp, wl[iPres]), RhoL = fmax(smallr, wl[irho]);
  double UL = wl[inorm], VL = wl[itan1], WL = wl[itan2];
  double RUL = RhoL * UL, RVL = RhoL * VL, RWL = RhoL * WL;
  double RUxUL = 0.5 * (RUL * UL + RVL * VL + RWL * WL);
  double EL = PGasL / hgamma + RUxUL;
  double AL2 = gamma * PGasL / RhoL;
  double AL = sqrt(AL2);
  if (UL <= -AL) {
    fr1 = fr2 = fr3 = fr4 = fr5 = 0.0;
  } else if (UL >= AL) {
    fr1 = RhoL * UL;
    fr2 = fr1 * UL + PGasL;
    fr3 = fr1 * VL;
    fr4 = fr1 * WL;
    fr5 = UL * (EL + PGasL);
  } else {
    double UA = (-UL + (AL + AL)) / gamma;
    double H = (EL + PGasL) / RhoL;
    double HU = UL + AL;
    fr1 = 0.25 * RhoL * HU * HU / AL;
    fr2 = fr1 * (UL + UA);
    fr3 = fr1 * (VL);
    fr4 = fr1 * (WL);
    fr5 = fr1 * (H);
  }
  double PGasR = fmax(smallp, wr[iPres]), RhoR = fmax(smallr, wr[irho]);
  double UR = wr[inorm], VR = wr[itan1], WR = wr[itan2];
  double RUR = RhoR * UR, RVR = RhoR * VR, RWR = RhoR * WR;
  double RUxUR = 0.5 * (RUR * UR + RVR * VR + RWR * WR);
  double ER = PGasR / hgamma + RUxUR;
  double AR2 = gamma * PGasR / RhoR;
  double AR = sqrt(AR2);
  if (UR >= AR) {
    fl1 = fl2 = fl3 = fl4 = fl5 = 0.0;
  } else if (UR <= -AR) {
    fl1 = RhoR * UR;
    fl2 = fl1 * UR + PGasR;
    fl3 = fl1 * VR;
    fl4 = fl1 * WR;
    fl5 = UR * (ER + PGasR);
  } else {
    double UA = (-UR - (AR + AR)) / gamma;
    double H = (ER + PGasR) / RhoR;
    double HU = UR - AR;
    fl1 = -0.25 * RhoR * HU * HU / AR;
    fl2 = fl1 * (UR + UA);
    fl3 = fl1 * (VR);
    fl4 = fl1 * (WR);
    fl5 = fl1 * (H);
  }
  g[irho] = fl1 + fr1;
  g[inorm] = fl2 + fr2;
  g[itan1] = fl3 + fr3;
  g[itan2] = fl4 + fr4;
  g[iPres] = fl5 + fr5;
}

/* PatchMHDMF::fluxesRP (srcIdeal/PatchMHDMF.cpp:408-440) on one face. */
/* VFROE_FLUXES (src/VFRoeF.ChF:327-658) with arithmetic averaging, the only
   form RiemannSolver::make builds (flux 5, src/RiemannSolver.cpp:69-74): the
   middle state of the linearised Riemann problem (each wave strength times
   sign(1/2, eigenvalue)) and the exact MHD flux of that state. */
static void vfroe_face(const Ctx* c, int idir, const double* wl, const double* wr, double* g) {
  const double gamma = c->gamma, hgamma = c->hgamma, smallp = c->smallp, smallr = c->smallr;
  const int inorm = 1 + idir, itan1 = 1 + (idir + 1) % 3, itan2 = 1 + (idir + 2) % 3;
  const int inormB = 5 + idir, itanB1 = 5 + (idir + 1) % 3, itanB2 = 5 + (idir + 2) % 3;
  double PGasL = fmax(smallp, wl[4]), RhoL = fmax(smallr, wl[0]);
  double UL = wl[inorm], VL = wl[itan1], WL = wl[itan2];
  double BXL = wl[inormB], BYL = wl[itanB1], BZL = wl[itanB2];
  double PGasR = fmax(smallp, wr[4]), RhoR = fmax(smallr, wr[0]);
  double UR = wr[inorm], VR = wr[itan1], WR = wr[itan2];
  double BXR = wr[inormB], BYR = wr[itanB1], BZR = wr[itanB2];
  /* average state */
  double Rho = 0.5 * (RhoL + RhoR);
  double U = 0.5 * (UL + UR);
  double BX = 0.5 * (BXL + BXR), BY = 0.5 * (BYL + BYR), BZ = 0.5 * (BZL + BZR);
  double PGas = 0.5 * (PGasL + PGasR);
  double BX2 = BX * BX, BY2 = BY * BY, BZ2 = BZ * BZ;
  double BYZ2 = BY2 + BZ2;
  double BxBH = D_1_8PI * (BX2 + BYZ2);
  double cc = gamma * PGas / Rho;
  double bb = D_1_4PI * BX2 / Rho;
  double szb = cc + (BxBH + BxBH) / Rho;
  double h = sqrt(szb * szb - 4.0 * cc * bb);
  double aaf = 0.5 * (szb + h);
  double aas = cc * bb / aaf;
  double cs = sqrt(cc), af = sqrt(aaf), as = sqrt(aas);
  double eig[9];
  eig[1] = U;
  eig[2] = U;
  eig[3] = U + sqrt(bb);
  eig[4] = U - sqrt(bb);
  eig[5] = U + af;
  eig[6] = U - af;
  eig[7] = U + as;
  eig[8] = U - as;
  /* alphas */
  double alphaF, alphaS;
  double dfs = aaf - aas;
  if (dfs < 1.0e-12) {
    alphaF = 1.0;
    alphaS = 0.0;
  } else if ((cc - aas) <= 0.0) {
    alphaF = 0.0;
    alphaS = 1.0;
  } else if ((aaf - cc) <= 0.0) {
    alphaF = 1.0;
    alphaS = 0.0;
  } else {
    alphaF = sqrt((cc - aas) / dfs);
    alphaS = sqrt((aaf - cc) / dfs);
  }
  double betaY, betaZ;
  if (BYZ2 < c->smallB * c->smallB) {
    betaY = D_SQRT_2;
    betaZ = D_SQRT_2;
  } else {
    double hyz = sqrt(BYZ2);
    betaY = BY / hyz;
    betaZ = BZ / hyz;
  }
  double siBX = copysign(1.0, BX);
  double betaYX = betaY, betaZX = betaZ;
  if (BX < 0.0) {
    betaYX = -betaY;
    betaZX = -betaZ;
  }
  double dP = PGasR - PGasL, dRho = RhoR - RhoL, dUn = UR - UL, dUt1 = VR - VL, dUt2 = WR - WL;
  double dBt1 = BYR - BYL, dBt2 = BZR - BZL;
  double a[9];
  a[1] = dRho - dP / cc;
  a[2] = BXR - BXL;
  double h1 = D_SQRT_2 * (betaY * dUt2 - betaZ * dUt1);
  double h2 = siBX * (betaZ * dBt1 - betaY * dBt2) / (2.0 * sqrt(2.0 * D_PI * Rho));
  a[3] = h1 + h2;
  a[4] = h1 - h2;
  h1 = dP / (2.0 * Rho * cc);
  h2 = dUn / (2.0 * cc);
  double h3 = (betaY * dBt1 + betaZ * dBt2) / (4.0 * cs * sqrt(D_PI * Rho));
  double h4 = siBX * (betaY * dUt1 + betaZ * dUt2) / (2.0 * cc);
  a[5] = alphaF * (h1 + af * h2) + alphaS * (h3 - as * h4);
  a[6] = alphaF * (h1 - af * h2) + alphaS * (h3 + as * h4);
  a[7] = alphaS * (h1 + as * h2) - alphaF * (h3 - af * h4);
  a[8] = alphaS * (h1 - as * h2) - alphaF * (h3 + af * h4);
  /* middle state */
  for (int q = 1; q <= 8; ++q) a[q] = (eig[q] == 0.0) ? 0.0 : a[q] * copysign(0.5, eig[q]);
  a[3] = D_SQRT_2 * a[3];
  a[4] = D_SQRT_2 * a[4];
  double alph3p4 = a[3] + a[4], alph3m4 = a[3] - a[4];
  double alph5p6 = a[5] + a[6], alph5m6 = a[5] - a[6];
  double alph7p8 = a[7] + a[8], alph7m8 = a[7] - a[8];
  double DN = 2.0 * sqrt(D_PI * Rho);
  double HRho = Rho * (alphaF * alph5p6 + alphaS * alph7p8);
  double HU = alphaS * as * alph5m6 - alphaF * af * alph7m8;
  double HB = cs * (alphaS * alph5p6 - alphaF * alph7p8);
  double RhoM = 0.5 * (RhoR + RhoL) - (a[1] + HRho);
  double UM = 0.5 * (UR + UL) - (alphaF * af * alph5m6 + alphaS * as * alph7m8);
  double VM = 0.5 * (VR + VL) + (betaZ * alph3p4 + betaYX * HU);
  double WM = 0.5 * (WR + WL) - (betaY * alph3p4 - betaZX * HU);
  double PGasM = 0.5 * (PGasR + PGasL) - cc * HRho;
  double BXM = 0.5 * (BXR + BXL);
  double BYM = 0.5 * (BYR + BYL) - DN * (betaZX * alph3m4 + betaY * HB);
  double BZM = 0.5 * (BZR + BZL) - DN * (-betaYX * alph3m4 + betaZ * HB);
  double BxBM = D_1_8PI * (BXM * BXM + BYM * BYM + BZM * BZM);
  double kk = 0.5 * (UM * UM + VM * VM + WM * WM);
  double HUM = BXM * UM + BYM * VM + BZM * WM;
  double E = PGasM / hgamma + RhoM * kk;
  double P = PGasM + BxBM;
  E = E + BxBM;
  g[0] = RhoM * UM;
  g[inorm] = RhoM * UM * UM + P - D_1_4PI * BXM * BXM;
  g[itan1] = RhoM * UM * VM - D_1_4PI * BXM * BYM;
  g[itan2] = RhoM * UM * WM - D_1_4PI * BXM * BZM;
  g[4] = UM * (E + P) - D_1_4PI * BXM * HUM;
  g[inormB] = 0.0;
  g[itanB1] = UM * BYM - VM * BXM;
  g[itanB2] = UM * BZM - WM * BXM;
}

static void face_flux(const Ctx* c, int dir, const double* wl, const double* wr, double* g) {
  if (c->rs == RS_ROE8)
    roe8_face(c, dir, wl, wr, g);
  else if (c->rs == RS_ROE7)
    roe7_face(c, dir, wl, wr, g);
  else if (c->rs == RS_VFROE)
    vfroe_face(c, dir, wl, wr, g);
  else
    rusanov_face(c, dir, wl, wr, g);
  if (c->glm) dedner_face(c, dir, wl, wr, g);
  for (int f = 1; f < c->nf; ++f) vanleer_face(c, dir, c->irhon + (f - 1) * 5, wl, wr, g);
}


/* ------------------------------------------------------------------------ */
/* heliosphere boundary fluxes                                               */
/* ------------------------------------------------------------------------ */
/* States below are in the frame of a face: rho, vn, vt1, vt2, p, Bn, Bt1, Bt2
   (tangential directions (d+1)%3, (d+2)%3); fluxes in the same order
   (mass, normal and tangential momentum, energy, Bn, Bt1, Bt2). */

/* ROE8WAVEF (src/Roe8WaveF.ChF:604-1144) is the body of RIEMANNF without the
   input floors; its callers floor rho and p first, so RIEMANNF on the same
   states in a frame whose normal is x gives it exactly. */
static void roe8_local(const Ctx* c, const double* L, const double* R, double* F) {
  roe8_face(c, 0, L, R, F);
}

/* BFLUX (swlism/HeliosphericF.ChF:1363-1560) and, with exitR, BFLUXR
   (:1562-1768; its position arguments only feed a radial speed it does not
   use).  in: the domain side, out: the ghost side, normal pointing out. */
static void bflux(const Ctx* c, int exitR, const double* in, const double* out, double* F,
                  double* BnValue) {
  const double gamma = c->gamma, hgamma = c->hgamma, d_4PI = 4.0 * D_PI;
  double U = in[1], V = in[2], W = in[3], R = in[0], BX = in[5], BY = in[6], BZ = in[7];
  double PG = in[4];
  double BB = BX * BX + BY * BY + BZ * BZ;
  double P = PG + D_1_8PI * BB;
  double KE = 0.5 * (in[1] * in[1] + in[2] * in[2] + in[3] * in[3]);
  double E = PG / hgamma + in[0] * KE + D_1_8PI * BB;
  double SZ = sqrt(gamma * PG / R);
  double B2 = BB;
  double SP = 0.5 * sqrt(d_4PI * R);
  double EM = SZ * SZ + B2 / (d_4PI * R) + SZ * fabs(BX) / SP;
  double EMM = SZ * SZ + B2 / (d_4PI * R) - SZ * fabs(BX) / SP;
  double CF = 0.5 * (sqrt(EM) + sqrt(EMM));
  double CS = 0.5 * (sqrt(EM) - sqrt(EMM));
  if (U >= CF) {
    *BnValue = BX;
    F[0] = R * U;
    F[1] = R * U * U + P - D_1_4PI * BX * BX;
    F[2] = R * U * V - D_1_4PI * BX * BY;
    F[3] = R * U * W - D_1_4PI * BX * BZ;
    F[4] = U * (E + P) - D_1_4PI * BX * (U * BX + V * BY + W * BZ);
    F[5] = 0.0;
    F[6] = U * BY - V * BX;
    F[7] = U * BZ - W * BX;
    return;
  }
  double U1 = out[1], V1 = out[2], W1 = out[3], R1 = out[0], BX1 = out[5], BY1 = out[6];
  double BZ1 = out[7], PG1 = out[4];
  double BB1 = BX1 * BX1 + BY1 * BY1 + BZ1 * BZ1;
  double P1 = PG1 + D_1_8PI * BB1;
  double KE1 = 0.5 * (out[1] * out[1] + out[2] * out[2] + out[3] * out[3]);
  double E1 = PG1 / hgamma + out[0] * KE1 + D_1_8PI * BB1;
  if (U < -CF) {
    *BnValue = BX1;
    F[0] = R1 * U1;
    F[1] = R1 * U1 * U1 + P1 - D_1_4PI * BX1 * BX1;
    F[2] = R1 * U1 * V1 - D_1_4PI * BX1 * BY1;
    F[3] = R1 * U1 * W1 - D_1_4PI * BX1 * BZ1;
    F[4] = U1 * (E1 + P1) - D_1_4PI * BX1 * (U1 * BX1 + V1 * BY1 + W1 * BZ1);
    F[5] = 0.0;
    F[6] = U1 * BY1 - V1 * BX1;
    F[7] = U1 * BZ1 - W1 * BX1;
    return;
  }
  double SZ1 = sqrt(gamma * PG1 / R1);
  double SP1 = 0.5 * sqrt(d_4PI * R1);
  double EM1 = SZ1 * SZ1 + BB1 / (d_4PI * R1) + SZ1 * fabs(BX1) / SP1;
  double EMM1 = SZ1 * SZ1 + BB1 / (d_4PI * R1) - SZ1 * fabs(BX1) / SP1;
  double CF1 = 0.5 * (sqrt(EM1) + sqrt(EMM1));
  int middle = exitR ? ((U < CF) && (U >= 0.0)) : ((U < CF) && (U >= 0.0) && (U1 > CF1));
  if (middle) {
    double SCM = SZ * SZ - CS * CS;
    double SCP = SZ * SZ + CS * CS;
    double DEM = sqrt(EM * EMM);
    double THE = -0.5 * CF * (BX * BX) / (R * d_4PI * DEM);
    THE = THE + (BZ * BZ + BY * BY) * CF * SCP * 0.5 / (R * DEM * d_4PI * SCM);
    THE = THE + 0.5 * CF * hgamma * (SZ * SZ) / DEM;
    THE = THE - SZ * fabs(BX) * CS * (gamma - 2.0) * 0.25 / (SP * DEM);
    double hyz = BY * BY + BZ * BZ, hy2, hz2;
    if (hyz < 1.0e-10) {
      hy2 = 0.5;
      hz2 = 0.5;
    } else {
      hy2 = BY * BY / hyz;
      hz2 = BZ * BZ / hyz;
    }
    double U16, R16, DRho, HRho, SZ16, BY16, BZ16;
    if (exitR) {
      double BE = 2.0 * d_4PI * (CF * CF - SZ * SZ);
      R16 = fmax(R + R * (U - CF) / (THE + CF), 1.0e-14);
      DRho = R16 - R;
      HRho = DRho / R;
      U16 = U - HRho * CF;
      SZ16 = SZ * (1.0 + 0.5 * hgamma * HRho);
      BZ16 = BZ * BZ + BE * hz2 * DRho;
      BY16 = BY * BY + BE * hy2 * DRho;
    } else {
      U16 = (U * THE + CF * CF) / (THE + CF);
      HRho = (U - CF) / (THE + CF);
      DRho = R * HRho;
      R16 = R + DRho;
      SZ16 = SZ * (1.0 + 0.5 * hgamma * HRho);
      double BE = 2.0 * d_4PI * (CF * CF - SZ * SZ) * DRho;
      BZ16 = BZ * BZ + BE * hz2;
      BY16 = BY * BY + BE * hy2;
    }
    if (BZ16 <= 0.0) {
      BZ16 = 0.0;
    } else {
      BZ16 = sqrt(BZ16);
      if (BZ < 0.0) BZ16 = -BZ16;
    }
    if (BY16 <= 0.0) {
      BY16 = 0.0;
    } else {
      BY16 = sqrt(BY16);
      if (BY < 0.0) BY16 = -BY16;
    }
    double BX16 = BX;
    double ALF = D_1_4PI * BX / (R * CF);
    double W16 = W + ALF * (BZ16 - BZ);
    double V16 = V + ALF * (BY16 - BY);
    double PG16 = SZ16 * SZ16 * R16 / gamma;
    double BB16 = D_1_4PI * (BX16 * BX16 + BY16 * BY16 + BZ16 * BZ16);
    double P16 = PG16 + 0.5 * BB16;
    double E16 = PG16 / hgamma + 0.5 * (R16 * (U16 * U16 + V16 * V16 + W16 * W16) + BB16);
    double BXq = D_1_4PI * BX16;
    *BnValue = BX16;
    F[0] = R16 * U16;
    F[1] = R16 * U16 * U16 + P16 - BXq * BX16;
    F[2] = R16 * U16 * V16 - BXq * BY16;
    F[3] = R16 * U16 * W16 - BXq * BZ16;
    F[4] = U16 * (E16 + P16) - BXq * (U16 * BX16 + V16 * BY16 + W16 * BZ16);
    F[5] = 0.0;
    F[6] = U16 * BY16 - V16 * BX16;
    F[7] = U16 * BZ16 - W16 * BX16;
    return;
  }
  if (exitR && U >= 0.0) {
    double o2[8] = {in[0], in[1], in[2], in[3], out[4], out[5], out[6], out[7]};
    *BnValue = BX;
    roe8_local(c, in, o2, F);
  } else {
    *BnValue = 0.5 * (BX + BX1);
    roe8_local(c, in, out, F);
  }
}

/* One neutral population's outflow-only flux from the domain-side state
   (HELIOBC, the formula of the fluid 2/3 branches and of fluid 1 on the
   low-x side). */
static void neutral_outflow(const Ctx* c, const double* s, double vn, double* F) {
  double rho = s[0], vt1 = s[2], vt2 = s[3], p = s[4];
  double ke = rho * (vn * vn + vt1 * vt1 + vt2 * vt2);
  double e = p / c->hgamma + 0.5 * ke;
  F[0] = rho * vn;
  F[1] = rho * vn * vn + p;
  F[2] = rho * vn * vt1;
  F[3] = rho * vn * vt2;
  F[4] = vn * (e + p);
}

/* HELIOBC (swlism/HeliosphericF.ChF:221-910) on one face of the domain
   boundary in direction d; side 0: low face (wl is the ghost side), 1: high
   face (wr is the ghost side).  Overwrites the plasma fluxes 0..7, the
   neutral fluxes and Bn (the GLM psi flux stays). */
static void helio_bc_face(const Ctx* c, int d, int side, const double* wl, const double* wr,
                          double* g, double* bn) {
  const int t1 = (d + 1) % 3, t2 = (d + 2) % 3;
  const int iv[3] = {1 + d, 1 + t1, 1 + t2}, ib[3] = {5 + d, 5 + t1, 5 + t2};
  const double smallr = c->smallr, smallp = c->smallp;
  double F[8], Bv;
  /* local states: inner (domain side) and outer (ghost side); low faces are
     mirrored so that the normal points out of the domain */
  const double* Win = side ? wl : wr;
  const double* Wout = side ? wr : wl;
  const double sg = side ? 1.0 : -1.0;
  if (d == 0 && side == 1) {
    /* inflow: the exact flux of the far-field state */
    const double* b = c->p->bc_plasma;
    double density = b[0], velx = b[1], vely = b[2], velz = b[3], pressure = b[4];
    double Bx = b[5], By = b[6], Bz = b[7];
    double bm = D_1_8PI * (Bx * Bx + By * By + Bz * Bz);
    double ke = density * (velx * velx + vely * vely + velz * velz);
    double bu = Bx * velx + By * vely + Bz * velz;
    double Pt = pressure + bm;
    double e = pressure / c->hgamma + 0.5 * ke + bm;
    g[0] = density * velx;
    g[1] = density * velx * velx - D_1_4PI * Bx * Bx + Pt;
    g[2] = density * velx * vely - D_1_4PI * Bx * By;
    g[3] = density * velx * velz - D_1_4PI * Bx * Bz;
    g[4] = velx * (e + Pt) - D_1_4PI * Bx * bu;
    g[5] = 0.0;
    g[6] = velx * By - vely * Bx;
    g[7] = velx * Bz - velz * Bx;
    *bn = Bx;
  } else {
    double L[8], Rt[8];
    L[0] = Win[0];
    Rt[0] = Wout[0];
    L[4] = Win[4];
    Rt[4] = Wout[4];
    for (int a = 0; a < 3; ++a) {
      L[1 + a] = sg * Win[iv[a]];
      Rt[1 + a] = sg * Wout[iv[a]];
      L[5 + a] = sg * Win[ib[a]];
      Rt[5 + a] = sg * Wout[ib[a]];
    }
    Rt[0] = fmax(smallr, Rt[0]);
    Rt[4] = fmax(smallp, Rt[4]);
    L[0] = fmax(smallr, L[0]);
    L[4] = fmax(smallp, L[4]);
    bflux(c, d == 0, L, Rt, F, &Bv);
    g[0] = sg * F[0];
    g[iv[0]] = F[1];
    g[iv[1]] = F[2];
    g[iv[2]] = F[3];
    g[4] = sg * F[4];
    g[ib[0]] = F[5];
    g[ib[1]] = F[6];
    g[ib[2]] = F[7];
    *bn = sg * Bv;
  }
  /* neutral populations */
  for (int f = 1; f < c->nf; ++f) {
    const int s0 = c->irhon + (f - 1) * 5;
    const int nv[3] = {s0 + 1 + d, s0 + 1 + t1, s0 + 1 + t2};
    double Fn[5];
    if (f == 2 || f == 3) {
      double fd = (f == 2) ? NETF2_DENS : NETF3_DENS, fp = (f == 2) ? NETF2_PRES : NETF3_PRES;
      double st[5] = {fmax(fd, Win[s0]), Win[nv[0]], Win[nv[1]], Win[nv[2]], fmax(fp, Win[s0 + 4])};
      double vn = side ? fmax(0.0, st[1]) : fmin(0.0, st[1]);
      neutral_outflow(c, st, vn, Fn);
      g[s0] = Fn[0];
      g[nv[0]] = Fn[1];
      g[nv[1]] = Fn[2];
      g[nv[2]] = Fn[3];
      g[s0 + 4] = Fn[4];
      continue;
    }
    /* fluids 1 and 4 */
    if (side == 0 && d == 0) {
      double st[5] = {fmax(smallr, Win[s0]), Win[nv[0]], Win[nv[1]], Win[nv[2]],
                      fmax(smallp, Win[s0 + 4])};
      double vn = fmin(-1.0e-6, st[1]);
      neutral_outflow(c, st, vn, Fn);
      g[s0] = Fn[0];
      g[nv[0]] = Fn[1];
      g[nv[1]] = Fn[2];
      g[nv[2]] = Fn[3];
      g[s0 + 4] = Fn[4];
      continue;
    }
    double Ln[5], Rn[5];
    Ln[0] = fmax(smallr, Win[s0]);
    Ln[4] = fmax(smallp, Win[s0 + 4]);
    Rn[0] = fmax(smallr, Wout[s0]);
    Rn[4] = fmax(smallp, Wout[s0 + 4]);
    for (int a = 0; a < 3; ++a) {
      Ln[1 + a] = sg * Win[nv[a]];
      Rn[1 + a] = sg * Wout[nv[a]];
    }
    if (Ln[1] > 0.0) {
      Rn[1] = Ln[1];
      Rn[2] = Ln[2];
      Rn[3] = Ln[3];
      if (f == 1) Rn[0] = Ln[0];
    }
    /* VANLEERRS (src/VanLeerRSF.ChF:132-236) = VANLEERF without its floors,
       which the floors above make no-ops */
    double gl[5];
    vanleer_face(c, 0, 0, Ln, Rn, gl);
    g[s0] = sg * gl[0];
    g[nv[0]] = gl[1];
    g[nv[1]] = gl[2];
    g[nv[2]] = gl[3];
    g[s0 + 4] = sg * gl[4];
  }
}

/* ------------------------------------------------------------------------ */
/* sources                                                                   */
/* ------------------------------------------------------------------------ */

/* DEFINE_REGIONS_2F (swlism/SWLISMF.ChF:654-742), Cartesian branch. */
/* DEFINE_REGIONS_TRACER_4F (swlism/SWLISMF.ChF:839-1016), Cartesian: the
   sign of the region tracer W[nc-1] separates the solar wind (< 0) from the
   interstellar medium.  The thresholds are the routine's literals (its "3mG"
   set).  Its last test, x > 650 -> 1, reads x, which the routine assigns only
   in the solar-wind branch (so it holds the x of the last solar-wind cell
   visited); here it is the cell's own x.  The two agree on every domain
   whose cells all lie at x <= 650 from the sun. */
static int region_tracer_cell(const Ctx* c, int i, int j, int k, const double* W) {
  const mf_params* p = c->p;
  const double rho_thr = 1.2, vel_thr = 0.8, vel_ang_thr = 0.95, temp_thr = 9000;
  double dx = p->dx;
  double LIMSUN = 0.6 * p->sun_v;
  double coeff = p->region_t_coeff;
  double sunR2 = p->sun_r * p->sun_r;
  double regtr = W[c->nc - 1];
  double x = (i + 0.5) * dx - p->sun_center[0];
  double ux = W[1], uy = W[2], uz = W[3];
  int reg;
  if (regtr < 0.0) {
    double y = (j + 0.5) * dx - p->sun_center[1];
    double z = 0.0, r2, invr, ur;
    if (c->sd == 3) {
      z = (k + 0.5) * dx - p->sun_center[2];
      r2 = x * x + y * y + z * z;
      invr = 1.0 / sqrt(r2);
      ur = ux * (x * invr) + uy * (y * invr) + uz * (z * invr);
    } else {
      r2 = x * x + y * y;
      invr = 1.0 / sqrt(r2);
      ur = ux * (x * invr) + uy * (y * invr);
    }
    if (fabs(ur) >= LIMSUN) {
      double TEMP = coeff * W[4] / W[0];
      if ((TEMP >= 1.0e6) && (r2 > sunR2))
        reg = 2;
      else
        reg = 3;
    } else {
      reg = 2;
    }
    if (c->sd == 3 && ((z < p->region_zbot) || (z > p->region_ztop))) reg = 4;
  } else {
    reg = 1;
    double vel = (c->sd == 3) ? (ux * ux + uy * uy + uz * uz) : (ux * ux + uy * uy);
    vel = sqrt(vel);
    double ang = (ux * p->lism_u[0] + uy * p->lism_u[1] + uz * p->lism_u[2]) / vel;
    double rho = W[0], pr = W[4];
    double TEMP = coeff * pr / rho;
    if (rho > rho_thr) reg = 4;
    if (vel < vel_thr) reg = 4;
    if (ang < vel_ang_thr) reg = 4;
    if (TEMP > temp_thr) reg = 4;
    if (x > 650) reg = 1;
  }
  return reg;
}

/* DEFINE_REGIONS_2F (swlism/SWLISMF.ChF:654-742), Cartesian; the region
   tracer variant above when mf_params.region_tracer is set
   (HeliosphericProblem::defineRegions, swlism/HeliosphericProblem.cpp:
   2538-2575). */
static int region_cell(const Ctx* c, int i, int j, int k, const double* W) {
  const mf_params* p = c->p;
  if (p->region_tracer) return region_tracer_cell(c, i, j, k, W);
  double dx = p->dx;
  double LIMSUN = 0.6 * p->sun_v;
  double coeff = p->region_t_coeff;
  double sunR2 = p->sun_r * p->sun_r;
  double x = (i + 0.5) * dx - p->sun_center[0];
  double y = (j + 0.5) * dx - p->sun_center[1];
  double z = 0.0, r2, invr, ur;
  if (c->sd == 3) {
    z = (k + 0.5) * dx - p->sun_center[2];
    r2 = x * x + y * y + z * z;
    invr = 1.0 / sqrt(r2);
    ur = W[1] * (x * invr) + W[2] * (y * invr) + W[3] * (z * invr);
  } else {
    r2 = x * x + y * y;
    invr = 1.0 / sqrt(r2);
    ur = W[1] * (x * invr) + W[2] * (y * invr);
  }
  double TEMP = coeff * W[4] / W[0];
  int reg;
  if (fabs(ur) >= LIMSUN) {
    if ((TEMP >= 1.0e6) && (r2 > sunR2))
      reg = 2;
    else
      reg = 3;
    if (c->sd == 3 && ((z < p->region_zbot) || (z > p->region_ztop))) reg = 1;
  } else {
    if (TEMP >= p->region_tmlim) {
      reg = 2;
      if (c->sd == 3 && ((z < p->region_zbot) || (z > p->region_ztop))) reg = 1;
    } else {
      reg = 1;
    }
  }
  return reg;
}

/* Neutral fluid that receives the newly created neutrals in region REG:
   CHARGE_EXCHANGE_2F/3F/4F/MF (swlism/ChargeExchange2F.ChF:294-432,
   434-671, 673-993, 995-1149). 0 = none. */
static int ce_recipient(int nN, int reg) {
  if (nN == 1) return (reg == 1 || reg == 4) ? 1 : 0;
  if (nN == 2) return (reg == 1) ? 1 : (reg == 2) ? 2 : 0;
  if (nN == 3) return (reg == 1 || reg == 4) ? 1 : (reg == 2) ? 2 : (reg == 3) ? 3 : 0;
  return (reg >= 1 && reg <= nN) ? reg : 0;
}

/* Charge-exchange source of one cell (Pauls & Zank rates), S = -dt*H.  The
   cross-section is parametric: sigma(v) = scale*(a - b ln(v*scaleVel))^2,
   optionally damped by (1-exp(-c/(v*scaleVel)))^pow (the reference's Lindsay &
   Stebbings form is a=13.493, b=0.531, c=2.946e9, pow=4.5).  S[0] and the
   magnetic (and psi) entries are zero. */
static void charge_exchange_cell(const Ctx* c, const double* W, int reg, double dt, double* S) {
  const mf_params* p = c->p;
  const int nN = c->nf - 1;
  double rho = W[0], ux = W[1], uy = W[2], uz = W[3], pp = W[4];
  double U2 = ux * ux + uy * uy + uz * uz;
  double VVTP = pp / rho;
  double h2 = 0, h3 = 0, h4 = 0, h5 = 0, PPLUX = 0, PPLUY = 0, PPLUZ = 0, ENPLU = 0;
  double DENPLU[MF_MAX_FLUIDS], PMIX[MF_MAX_FLUIDS], PMIY[MF_MAX_FLUIDS], PMIZ[MF_MAX_FLUIDS],
      ENMI[MF_MAX_FLUIDS];
  for (int f = 1; f <= nN; ++f) {
    int s = c->irhon + (f - 1) * 5;
    double rhoN = W[s], uxN = W[s + 1], uyN = W[s + 2], uzN = W[s + 3], pN = W[s + 4];
    double UH2 = uxN * uxN + uyN * uyN + uzN * uzN;
    double DU2 = (ux - uxN) * (ux - uxN) + (uy - uyN) * (uy - uyN) + (uz - uzN) * (uz - uzN);
    double VPHH = (ux - uxN) * uxN + (uy - uyN) * uyN + (uz - uzN) * uzN;
    double VPHP = (ux - uxN) * ux + (uy - uyN) * uy + (uz - uzN) * uz;
    double VVTH = 2.0 * pN / rhoN;
    double UD = sqrt(4.0 * (VVTP + VVTH) / D_PI + DU2);
    double UPM = sqrt(16.0 * VVTP / D_PI + 2.25 * D_PI * VVTH + 4.0 * DU2);
    double UHM = sqrt(2.25 * D_PI * VVTP + 16.0 * VVTH / D_PI + 4.0 * DU2);
    double UPE = sqrt((4.0 * VVTP + 64.0 * VVTH / 9.0) / D_PI + DU2);
    double UHE = sqrt((64.0 * VVTP / 9.0 + 4.0 * VVTH) / D_PI + DU2);
    double UDS = p->ce_scale_vel * UD;
    double t = p->ce_sigma_a - p->ce_sigma_b * log(UDS);
    double SIGMAL = t * t;
    if (p->ce_damp_c > 0.0) SIGMAL = SIGMAL * pow(1.0 - exp(-p->ce_damp_c / UDS), p->ce_damp_pow);
    SIGMAL = p->ce_sigma_scale * SIGMAL;
    double ARR = SIGMAL * rhoN * rho;
    double VVTHU = VVTH / UPM;
    h2 = h2 + ARR * (ux - uxN) * (UD + VVTHU + VVTP / UHM);
    h3 = h3 + ARR * (uy - uyN) * (UD + VVTHU + VVTP / UHM);
    h4 = h4 + ARR * (uz - uzN) * (UD + VVTHU + VVTP / UHM);
    h5 = h5 + 0.5 * ARR *
                  (1.5 * (UHE * VVTP - UPE * VVTH) + UD * (U2 - UH2) +
                   2.0 * (VVTHU * VPHH + VVTP * VPHP / UHM));
    DENPLU[f] = -ARR * UD;
    PPLUX = PPLUX - ARR * (ux * UD - (uxN - ux) * VVTP / UHM);
    PPLUY = PPLUY - ARR * (uy * UD - (uyN - uy) * VVTP / UHM);
    PPLUZ = PPLUZ - ARR * (uz * UD - (uzN - uz) * VVTP / UHM);
    ENPLU = ENPLU - ARR * (0.5 * U2 * UD + VVTP * (VPHP / UHM + 0.75 * UHE));
    PMIX[f] = ARR * (uxN * UD + (uxN - ux) * VVTHU);
    PMIY[f] = ARR * (uyN * UD + (uyN - uy) * VVTHU);
    PMIZ[f] = ARR * (uzN * UD + (uzN - uz) * VVTHU);
    ENMI[f] = ARR * (0.5 * UH2 * UD - VPHH * VVTHU + 0.75 * VVTH * UPE);
  }
  for (int q = 0; q < c->nc; ++q) S[q] = 0.0;
  S[1] = -dt * h2;
  S[2] = -dt * h3;
  S[3] = -dt * h4;
  S[4] = -dt * h5;
  int rk = ce_recipient(nN, reg);
  for (int f = 1; f <= nN; ++f) {
    double H1, H2, H3, H4, H5;
    if (f == rk) {
      if (nN <= 3) {
        /* 2F/3F/4F: sum of the other populations in index order */
        int first = 1;
        H1 = 0.0;
        for (int q = 1; q <= nN; ++q) {
          if (q == f) continue;
          if (first) {
            H1 = DENPLU[q];
            first = 0;
          } else {
            H1 = H1 + DENPLU[q];
          }
        }
      } else {
        /* MF: sum(DENPLU) - DENPLU(iFluid) */
        double sum = DENPLU[1];
        for (int q = 2; q <= nN; ++q) sum = sum + DENPLU[q];
        H1 = sum - DENPLU[f];
      }
      H2 = PPLUX + PMIX[f];
      H3 = PPLUY + PMIY[f];
      H4 = PPLUZ + PMIZ[f];
      H5 = ENPLU + ENMI[f];
    } else {
      H1 = -DENPLU[f];
      H2 = PMIX[f];
      H3 = PMIY[f];
      H4 = PMIZ[f];
      H5 = ENMI[f];
    }
    int s = c->irhon + (f - 1) * 5;
    S[s] = -dt * H1;
    S[s + 1] = -dt * H2;
    S[s + 2] = -dt * H3;
    S[s + 3] = -dt * H4;
    S[s + 4] = -dt * H5;
  }
}

/* HELIOREINIT_DEFAULT (swlism/HeliosphericPlasmaBCF.ChF:1435-1566): the
   plasma inside r <= Rinit is reset to the radial wind at time t
   (HeliosphericProblem::postprocessing passes the stage's time plus its dt,
   swlism/HeliosphericProblem.cpp:2399-2405).  With sunBmonopolar != 1 the
   field is bipolar: it keeps its sign where the colatitude theta is below
   the current sheet's thetaS and flips elsewhere, and the current-sheet
   surface iHCS is set to +1 / -1 (:1537-1564). */
static void reinit_cell(const Ctx* c, int i, int j, int k, double t, double* U) {
  const mf_params* p = c->p;
  double dx = p->dx;
  double x = (i + 0.5) * dx - p->sun_center[0];
  double y = (j + 0.5) * dx - p->sun_center[1];
  double z = 0.0;
  if (c->sd == 3) z = (k + 0.5) * dx - p->sun_center[2];
  double r2 = (c->sd == 3) ? (x * x + y * y + z * z) : (x * x + y * y);
  double sunR2 = p->reinit_r0 * p->reinit_r0;
  if (!(r2 <= sunR2)) return;
  double r = sqrt(r2);
  double rr = r / p->sun_int_bc_radius;
  double xy = sqrt(x * x + y * y);
  double cosT = z / r;
  double sinT = sqrt(1.0 - cosT * cosT);
  double cosF = x / xy;
  double sinF = y / xy;
  double rho = p->sun_rho / (rr * rr);
  double ux = p->sun_v * sinT * cosF;
  double uy = p->sun_v * sinT * sinF;
  double uz = p->sun_v * cosT;
  double pr = p->sun_p / pow(rr, 2.0 * c->gamma);
  double br = p->dir_br * p->sun_b / (rr * rr);
  double bp = -p->sun_beta * br * r * sinT;
  double bx = br * sinT * cosF - bp * sinF;
  double by = br * sinT * sinF + bp * cosF;
  double bz = br * cosT;
  double b = bx * bx + by * by + bz * bz;
  double e0 = pr / c->hgamma + 0.5 * (rho * p->sun_v * p->sun_v + D_1_4PI * b);
  if (!c->monopolar) {
    double theta = acos(cosT);
    double cosBr = cos(p->sun_beta * (r - p->sun_v * t));
    double sinBr = sin(p->sun_beta * (r - p->sun_v * t));
    double sinB = sinF * cosBr + cosF * sinBr;
    double cosB = cosF * cosBr - sinF * sinBr;
    double thetaS =
        c->sin_tilt * sinB / sqrt((c->cos_tilt * cosB) * (c->cos_tilt * cosB) + sinB * sinB);
    thetaS = asin(thetaS) + D_PI_2;
    if (theta < thetaS) {
      /* the field as computed */
    } else {
      bx = -bx;
      by = -by;
      bz = -bz;
    }
    if (c->ihcs >= 0) U[c->ihcs] = (theta < thetaS) ? 1.0 : -1.0;
  }
  U[0] = rho;
  U[1] = rho * ux;
  U[2] = rho * uy;
  U[3] = rho * uz;
  U[4] = e0;
  U[5] = bx;
  U[6] = by;
  U[7] = bz;
}

/* POSTPROCESSING (srcIdeal/PatchIdealMHDF.ChF:1019-1070) and
   POSTPROCESSING_MF (srcIdeal/PatchMHDMFF.ChF:301-511). */
static void positivity_cell(const Ctx* c, double* U) {
  const double hgamma = c->hgamma, smallR = c->smallr, smallP = c->smallp;
  if (c->nf == 1) {
    double Rho = U[0];
    int iWas = 0;
    if (Rho < smallR) {
      Rho = smallR;
      iWas = 1;
    }
    double invRho = 1.0 / Rho;
    double Ux = U[1] * invRho, Uy = U[2] * invRho, Uz = U[3] * invRho;
    double E = U[4];
    double Bx = U[5], By = U[6], Bz = U[7];
    double BxB = D_1_8PI * (Bx * Bx + By * By + Bz * Bz);
    double UxU = 0.5 * (Ux * Ux + Uy * Uy + Uz * Uz);
    double P = hgamma * (E - BxB - Rho * UxU);
    if (P < smallP) {
      P = smallP;
      iWas = 1;
    }
    if (iWas == 1) {
      U[0] = Rho;
      U[4] = P / hgamma + Rho * UxU + BxB;
    }
    return;
  }
  {
    double Rho = U[0];
    double invRho = 1.0 / Rho;
    double Ux = U[1] * invRho, Uy = U[2] * invRho, Uz = U[3] * invRho;
    double E = U[4];
    double Bx = U[5], By = U[6], Bz = U[7];
    double BxB = D_1_8PI * (Bx * Bx + By * By + Bz * Bz);
    double UxU = 0.5 * (Ux * Ux + Uy * Uy + Uz * Uz);
    double P = hgamma * (E - BxB - Rho * UxU);
    int iWas = 0;
    if (Rho < smallR) {
      Rho = smallR;
      iWas = 1;
    }
    if (P < smallP) {
      P = smallP;
      iWas = 1;
    }
    if (iWas == 1) {
      U[0] = Rho;
      U[1] = Rho * Ux;
      U[2] = Rho * Uy;
      U[3] = Rho * Uz;
      U[4] = P / hgamma + Rho * UxU + BxB;
    }
  }
  for (int f = 1; f < c->nf; ++f) {
    double fd, fp;
    if (f == 1) {
      fd = smallR;
      fp = smallP;
    } else if (f == 3) {
      fd = NETF3_DENS;
      fp = NETF3_PRES;
    } else {
      fd = NETF2_DENS;
      fp = NETF2_PRES;
    }
    int s = c->irhon + (f - 1) * 5;
    double Rho = U[s];
    double invRho = 1.0 / Rho;
    double Ux = U[s + 1] * invRho, Uy = U[s + 2] * invRho, Uz = U[s + 3] * invRho;
    double E = U[s + 4];
    double UxU = 0.5 * (Ux * Ux + Uy * Uy + Uz * Uz);
    double P = hgamma * (E - Rho * UxU);
    int iWas = 0;
    if (Rho < fd) {
      Rho = fd;
      iWas = 1;
    }
    if (P < fp) {
      P = fp;
      iWas = 1;
    }
    if (iWas == 1) {
      U[s] = Rho;
      U[s + 1] = Rho * Ux;
      U[s + 2] = Rho * Uy;
      U[s + 3] = Rho * Uz;
      U[s + 4] = P / hgamma + Rho * UxU;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* physical boundary: primitive ghost cells outside the domain               */
/* ------------------------------------------------------------------------ */

/* Far-field ghost fill after HELIOGS (swlism/HeliosphericF.ChF:978-1140): the
   plasma and neutral fluid 1 take the far-field state, the other neutral
   fluids copy the nearest cell inside the domain along the boundary normal.
   Applied per direction in order 0,1,2 over the part of W's box outside the
   domain in that direction (HeliosphericProblem::fillGhostCells,
   swlism/HeliosphericProblem.cpp:1663-1760). */
/* HELIOGS (swlism/HeliosphericF.ChF:978-1140) on the primitive ghosts outside
   the domain.  The region tracer holds +1 there (:996-1000).  Other tracking
   surfaces are not set by HELIOGS (the reference leaves those ghosts of W
   unassigned); here they copy U's ghost value. */
static void fill_ghost_cells(const Ctx* c, const Fab* U, Fab* W) {
  const mf_params* p = c->p;
  if (p->bc_kind != MF_BC_FARFIELD) return;
  for (int d = 0; d < c->sd; ++d) {
    if (p->periodic[d]) continue;
    for (int side = 0; side < 2; ++side) {
      mf_box bb = W->b;
      int edge;
      if (side == 0) {
        if (bb.lo[d] >= p->domain_lo[d]) continue;
        bb.hi[d] = p->domain_lo[d] - 1;
        edge = p->domain_lo[d];
      } else {
        if (bb.hi[d] <= p->domain_hi[d]) continue;
        bb.lo[d] = p->domain_hi[d] + 1;
        edge = p->domain_hi[d];
      }
      FOR_BOX(bb, i, j, k) {
        for (int q = c->ils; q < c->nc; ++q) AT(W, i, j, k, q) = AT(U, i, j, k, q);
        if (p->region_tracer) AT(W, i, j, k, c->nc - 1) = 1.0;
        for (int q = 0; q < 8; ++q) AT(W, i, j, k, q) = p->bc_plasma[q];
        if (c->glm) AT(W, i, j, k, 8) = 0.0;
        if (c->nf > 1)
          for (int q = 0; q < 5; ++q) AT(W, i, j, k, c->irhon + q) = p->bc_neutral1[q];
        for (int f = 2; f < c->nf; ++f) {
          int ii = i, jj = j, kk = k;
          if (d == 0) ii = edge;
          if (d == 1) jj = edge;
          if (d == 2) kk = edge;
          int s = c->irhon + (f - 1) * 5;
          for (int q = 0; q < 5; ++q) AT(W, i, j, k, s + q) = AT(W, ii, jj, kk, s + q);
        }
      }
    }
  }
}

/* ------------------------------------------------------------------------ */
/* tracking surfaces (level sets)                                            */
/* ------------------------------------------------------------------------ */

/* LEVELSETFLUX (src/LevelSetF.ChF:37-105) of one face for every surface:
   the left face state (high face of the low cell) where
   sqrt(rho_L) u_L + sqrt(rho_R) u_R > 0 with the plasma density and normal
   velocity (lsIndexField = WVELX, src/PhysProblem.cpp:327-330), else the
   right one.  Called after fluxBC (src/PatchMHDAM.cpp:644-648). */
static void level_set_flux(const Ctx* c, int d, const double* wl, const double* wr, double* g) {
  double Uavg = sqrt(wl[0]) * wl[1 + d] + sqrt(wr[0]) * wr[1 + d];
  for (int q = c->ils; q < c->nc; ++q) g[q] = (Uavg > 0.0) ? wl[q] : wr[q];
}

/* UPDATELEVELSET (src/LevelSetF.ChF:200-234), Cartesian (dx constant, metric
   coefficient 1): phi -= dt/dx * u_d * (F(i+e_d) - F(i)), u_d the cell's
   velocity of the primitive state W. */
static void level_set_update(const Ctx* c, Fab* U, const Fab* W, const Fab* Fl, int d, double dt,
                             mf_box box) {
  int o[3] = {0, 0, 0};
  o[d] = 1;
  const double du = c->p->dx * 1.0;
  for (int q = c->ils; q < c->nc; ++q)
    FOR_BOX(box, i, j, k) {
      double vel = AT(W, i, j, k, 1 + d);
      AT(U, i, j, k, q) = AT(U, i, j, k, q) - dt / du * vel *
                                                  (AT(Fl, i + o[0], j + o[1], k + o[2], q) -
                                                   AT(Fl, i, j, k, q));
    }
}

/* POSTPROCESSING_LS (src/LevelSetF.ChF:426-465) from PatchMHDMF::
   postprocessing (srcIdeal/PatchMHDMF.cpp:1414-1424): Umin = min of the
   stage-start values of the cell and its 2*SpaceDim neighbours, lowered to
   -|max|.  The routine assigns min(LS, Umax) and then max(LS, Umin) from the
   same LS, so only the floor remains. */
static void level_set_postprocess(const Ctx* c, Fab* U, const Fab* Uold, mf_box box) {
  for (int q = c->ils; q < c->nc; ++q)
    FOR_BOX(box, i, j, k) {
      double Umax = AT(Uold, i, j, k, q), Umin = AT(Uold, i, j, k, q);
      for (int ii = -1; ii <= 1; ii += 2) {
        Umax = fmax(Umax, AT(Uold, i + ii, j, k, q));
        Umin = fmin(Umin, AT(Uold, i + ii, j, k, q));
        Umax = fmax(Umax, AT(Uold, i, j + ii, k, q));
        Umin = fmin(Umin, AT(Uold, i, j + ii, k, q));
        if (c->sd == 3) {
          Umax = fmax(Umax, AT(Uold, i, j, k + ii, q));
          Umin = fmin(Umin, AT(Uold, i, j, k + ii, q));
        }
      }
      double abmax = fabs(Umax);
      double abmin = fabs(Umin);
      Umax = fmax(Umax, abmin);
      Umin = fmin(Umin, -abmax);
      double LS = AT(U, i, j, k, q);
      AT(U, i, j, k, q) = fmin(LS, Umax);
      AT(U, i, j, k, q) = fmax(LS, Umin);
    }
}

/* ------------------------------------------------------------------------ */
/* constrained transport                                                     */
/* ------------------------------------------------------------------------ */

/* EdgeBox (src/EdgeBox.cpp:105-131): in 3D, E[d] on surroundingNodes(box)
   .enclosedCells(d) (cell-centred along d, nodal across); in 2D one nodal
   array that E[0], E[1] and E[2] all address (operator[], :63-73). */
typedef struct {
  Fab e[3];
  int n;
} Edges;

static void edges_alloc(Edges* E, mf_box box, int sd) {
  mf_box nb = box;
  for (int d = 0; d < sd; ++d) nb.hi[d] += 1;
  if (sd == 3) {
    E->n = 3;
    for (int d = 0; d < 3; ++d) {
      mf_box b = nb;
      b.hi[d] -= 1;
      E->e[d] = fab_alloc(b, 1);
    }
  } else {
    E->n = 1;
    E->e[0] = fab_alloc(nb, 1);
    E->e[1] = E->e[2] = E->e[0];
  }
}

static void edges_free(Edges* E) {
  for (int d = 0; d < E->n; ++d) fab_free(&E->e[d]);
}

/* dst = src on the edges both hold (EdgeBox::copy on the intersection) */
static void edges_copy(Edges* dst, const Edges* src) {
  for (int d = 0; d < dst->n; ++d) {
    mf_box b = dst->e[d].b;
    for (int q = 0; q < 3; ++q) {
      if (src->e[d].b.lo[q] > b.lo[q]) b.lo[q] = src->e[d].b.lo[q];
      if (src->e[d].b.hi[q] < b.hi[q]) b.hi[q] = src->e[d].b.hi[q];
    }
    FOR_BOX(b, i, j, k) AT(&dst->e[d], i, j, k, 0) = AT(&src->e[d], i, j, k, 0);
  }
}

/* electricFieldBS (srcIdeal/DivCleaningF.ChF:75-310): the edge field as the
   mean of the tangential magnetic-field fluxes of the faces around the edge
   that lie in the flux boxes of box (the faces of box).  2D: EZ from the
   x-flux of By and the y-flux of Bx with weights 1/4, 1/3, 1/2 as the
   literal H4, H3, H2; 3D: the sum over the present faces divided by their
   count, EX from the z-flux of By and the y-flux of Bz, EY from the z-flux of
   Bx and the x-flux of Bz, EZ from the y-flux of Bx and the x-flux of By. */
static void electric_field_bs(const Ctx* c, const Fab* Fl, mf_box box, Edges* E) {
  const double H2 = 0.5, H3 = 0.333333333333333333333333333333333333, H4 = 0.25;
  const int lo0 = box.lo[0], hi0 = box.hi[0], lo1 = box.lo[1], hi1 = box.hi[1];
  if (c->sd == 2) {
    const Fab *F = &Fl[0], *G = &Fl[1];
    Fab* EZ = &E->e[0];
    FOR_BOX(EZ->b, i, j, k) {
      double s = 0.0;
      int n = 0;
      if (i > lo0) {
        s = AT(G, i - 1, j, k, 5);
        n = 1;
      }
      if (i <= hi0) {
        s = n ? s + AT(G, i, j, k, 5) : AT(G, i, j, k, 5);
        n += 1;
      }
      if (j > lo1) {
        s = s - AT(F, i, j - 1, k, 6);
        n += 1;
      }
      if (j <= hi1) {
        s = s - AT(F, i, j, k, 6);
        n += 1;
      }
      const double h = (n == 4) ? H4 : (n == 3) ? H3 : H2;
      AT(EZ, i, j, k, 0) = h * s;
    }
    return;
  }
  const int lo2 = box.lo[2], hi2 = box.hi[2];
  const Fab *F = &Fl[0], *G = &Fl[1], *H = &Fl[2];
  FOR_BOX(E->e[0].b, i, j, k) {
    double EE = 0.0;
    int iE = 0;
    if (j > lo1) { EE = EE + AT(H, i, j - 1, k, 6); iE = iE + 1; }
    if (j <= hi1) { EE = EE + AT(H, i, j, k, 6); iE = iE + 1; }
    if (k > lo2) { EE = EE - AT(G, i, j, k - 1, 7); iE = iE + 1; }
    if (k <= hi2) { EE = EE - AT(G, i, j, k, 7); iE = iE + 1; }
    AT(&E->e[0], i, j, k, 0) = EE / iE;
  }
  FOR_BOX(E->e[1].b, i, j, k) {
    double EE = 0.0;
    int iE = 0;
    if (i > lo0) { EE = EE - AT(H, i - 1, j, k, 5); iE = iE + 1; }
    if (i <= hi0) { EE = EE - AT(H, i, j, k, 5); iE = iE + 1; }
    if (k > lo2) { EE = EE + AT(F, i, j, k - 1, 7); iE = iE + 1; }
    if (k <= hi2) { EE = EE + AT(F, i, j, k, 7); iE = iE + 1; }
    AT(&E->e[1], i, j, k, 0) = EE / iE;
  }
  FOR_BOX(E->e[2].b, i, j, k) {
    double EE = 0.0;
    int iE = 0;
    if (i > lo0) { EE = EE + AT(G, i - 1, j, k, 5); iE = iE + 1; }
    if (i <= hi0) { EE = EE + AT(G, i, j, k, 5); iE = iE + 1; }
    if (j > lo1) { EE = EE - AT(F, i, j - 1, k, 6); iE = iE + 1; }
    if (j <= hi1) { EE = EE - AT(F, i, j, k, 6); iE = iE + 1; }
    AT(&E->e[2], i, j, k, 0) = EE / iE;
  }
}

/* electricFieldGS0 / electricFieldGS1 in 2D (srcIdeal/DivCleaningF.ChF:
   335-408, 596-697; the result is stored through EX, which in 2D is the one
   nodal array): the face average corrected by the difference between the
   face fluxes and the cell-centred field EQ = u_y B_x - u_x B_y of the
   cells around the node (W: velocity at 1..3, field at 5..7).  GS1 takes
   the cell on the upwind side of each face by the sign of its mass flux. */
static void electric_field_gs(const Ctx* c, const Fab* W, const Fab* Fl, mf_box box, Edges* E,
                              int upwind) {
  const int lo0 = box.lo[0], hi0 = box.hi[0], lo1 = box.lo[1], hi1 = box.hi[1];
  const Fab *F = &Fl[0], *G = &Fl[1];
  (void)c;
  Fab* EX = &E->e[0];
  FOR_BOX(EX->b, i, j, k) {
    double EE = 0.0, EQ, DEDD;
    int iE = 0;
    double D1_00 = 0.0, D2_00 = 0.0, D1_10 = 0.0, D2_10 = 0.0;
    double D1_01 = 0.0, D2_01 = 0.0, D1_11 = 0.0, D2_11 = 0.0;
    int i00 = 0, i10 = 0, i01 = 0, i11 = 0;
#define EQAT(ii, jj) \
  (AT(W, ii, jj, k, 2) * AT(W, ii, jj, k, 5) - AT(W, ii, jj, k, 1) * AT(W, ii, jj, k, 6))
    if ((lo0 < i) && (lo1 < j)) {
      EQ = EQAT(i - 1, j - 1);
      D1_00 = -AT(F, i, j - 1, k, 6) - EQ;
      D2_00 = AT(G, i - 1, j, k, 5) - EQ;
      i00 = 1;
    }
    if ((hi0 >= i) && (lo1 < j)) {
      EQ = EQAT(i, j - 1);
      D1_10 = EQ + AT(F, i, j - 1, k, 6);
      D2_10 = AT(G, i, j, k, 5) - EQ;
      i10 = 1;
    }
    if ((lo0 < i) && (hi1 >= j)) {
      EQ = EQAT(i - 1, j);
      D1_01 = -AT(F, i, j, k, 6) - EQ;
      D2_01 = EQ - AT(G, i - 1, j, k, 5);
      i01 = 1;
    }
    if ((hi0 >= i) && (hi1 >= j)) {
      EQ = EQAT(i, j);
      D1_11 = EQ + AT(F, i, j, k, 6);
      D2_11 = EQ - AT(G, i, j, k, 5);
      i11 = 1;
    }
#undef EQAT
    if (lo0 < i) {
      if (upwind) {
        int iMN = i00, iPL = i01;
        const double m = AT(G, i - 1, j, k, 0);
        if (iMN * m > 0.0) iPL = 0;
        else if (iPL * m < 0.0) iMN = 0;
        DEDD = (iPL * D1_01 + iMN * D1_00) / (iPL + iMN);
      } else {
        DEDD = (D1_01 + D1_00) / (i01 + i00);
      }
      EE = EE + AT(G, i - 1, j, k, 5) + DEDD;
      iE = iE + 1;
    }
    if (hi0 >= i) {
      if (upwind) {
        int iMN = i10, iPL = i11;
        const double m = AT(G, i, j, k, 0);
        if (iMN * m > 0.0) iPL = 0;
        else if (iPL * m < 0.0) iMN = 0;
        DEDD = (iMN * D1_10 + iPL * D1_11) / (iMN + iPL);
      } else {
        DEDD = (D1_10 + D1_11) / (i10 + i11);
      }
      EE = EE + AT(G, i, j, k, 5) - DEDD;
      iE = iE + 1;
    }
    if (lo1 < j) {
      if (upwind) {
        int iMN = i00, iPL = i10;
        const double m = AT(F, i, j - 1, k, 0);
        if (iMN * m > 0.0) iPL = 0;
        else if (iPL * m < 0.0) iMN = 0;
        DEDD = (iMN * D2_00 + iPL * D2_10) / (iMN + iPL);
      } else {
        DEDD = (D2_00 + D2_10) / (i00 + i10);
      }
      EE = EE - AT(F, i, j - 1, k, 6) + DEDD;
      iE = iE + 1;
    }
    if (hi1 >= j) {
      if (upwind) {
        int iMN = i01, iPL = i11;
        const double m = AT(F, i, j, k, 0);
        if (iMN * m > 0.0) iPL = 0;
        else if (iPL * m < 0.0) iMN = 0;
        DEDD = (iMN * D2_01 + iPL * D2_11) / (iMN + iPL);
      } else {
        DEDD = (D2_01 + D2_11) / (i01 + i11);
      }
      EE = EE - AT(F, i, j, k, 6) - DEDD;
      iE = iE + 1;
    }
    AT(EX, i, j, k, 0) = EE / iE;
  }
}

/* PatchMHDMF::calculateElectricField (srcIdeal/PatchMHDMF.cpp:1487-1560) */
static void electric_field(const Ctx* c, const Fab* W, const Fab* Fl, mf_box box, Edges* E) {
  if (c->ct == 1)
    electric_field_bs(c, Fl, box, E);
  else
    electric_field_gs(c, W, Fl, box, E, c->ct == 3);
}

/* recalculateB (srcIdeal/DivCleaningF.ChF:4-72) from PatchMHDMF::
   recalculateMagneticField (srcIdeal/PatchMHDMF.cpp:1461-1484): the cell
   field from the old one and the circulation of the edge field around the
   cell, HX = dt/(2 dx); the energy keeps its non-magnetic part.  Bold: any
   array with the old field at components 5..7 (U or W). */
static void recalc_b(const Ctx* c, Fab* U, const Fab* Bold, const Edges* E, double dt,
                     mf_box box) {
  const double HX = 0.5 * dt / c->p->dx;
  const Fab *EX = &E->e[0], *EY = &E->e[1], *EZ = &E->e[2];
  FOR_BOX(box, i, j, k) {
    double bx = AT(U, i, j, k, 5), by = AT(U, i, j, k, 6), bz = AT(U, i, j, k, 7);
    double b = D_1_8PI * (bx * bx + by * by + bz * bz);
    double e = AT(U, i, j, k, 4) - b;
    const int kk = (c->sd == 3) ? 1 : 0;
    bx = AT(Bold, i, j, k, 5) - HX * (AT(EZ, i + 1, j + 1, k, 0) + AT(EZ, i, j + 1, k, 0) -
                                      AT(EZ, i + 1, j, k, 0) - AT(EZ, i, j, k, 0));
    by = AT(Bold, i, j, k, 6) + HX * (AT(EZ, i + 1, j + 1, k, 0) + AT(EZ, i + 1, j, k, 0) -
                                      AT(EZ, i, j + 1, k, 0) - AT(EZ, i, j, k, 0));
    if (kk) {
      bx = bx + HX * (AT(EY, i + 1, j, k + 1, 0) + AT(EY, i, j, k + 1, 0) -
                      AT(EY, i + 1, j, k, 0) - AT(EY, i, j, k, 0));
      by = by - HX * (AT(EX, i, j + 1, k + 1, 0) + AT(EX, i, j, k + 1, 0) -
                      AT(EX, i, j + 1, k, 0) - AT(EX, i, j, k, 0));
      bz = AT(Bold, i, j, k, 7) -
           HX * (AT(EY, i + 1, j, k + 1, 0) + AT(EY, i + 1, j, k, 0) - AT(EY, i, j, k + 1, 0) -
                 AT(EY, i, j, k, 0) -
                 (AT(EX, i, j + 1, k + 1, 0) + AT(EX, i, j + 1, k, 0) - AT(EX, i, j, k + 1, 0) -
                  AT(EX, i, j, k, 0)));
    }
    b = D_1_8PI * (bx * bx + by * by + bz * bz);
    AT(U, i, j, k, 4) = e + b;
    AT(U, i, j, k, 5) = bx;
    AT(U, i, j, k, 6) = by;
    AT(U, i, j, k, 7) = bz;
  }
}

/* ------------------------------------------------------------------------ */
/* EulerStep                                                                 */
/* ------------------------------------------------------------------------ */

/* PatchMHDAM::EulerStep (src/PatchMHDAM.cpp:495-709) for PatchMHDMF. */
static int euler_step(const Ctx* c, double time, Fab* U, Fab* F /* [sd] or NULL */, Fab* divBout,
                      double dt, mf_box a_box, Edges* Eout /* nullable */) {
  const mf_params* p = c->p;
  const int sd = c->sd, nc = c->nc, np = c->nprim;

  mf_box UBox = U->b;
  /* With a far-field boundary the primitive ghosts outside the domain come
     from the boundary state; otherwise the caller filled U's ghosts. */
  mf_box WBoxB = (p->bc_kind == MF_BC_FARFIELD) ? box_and_domain(UBox, p) : UBox;
  Fab Uold = fab_alloc(UBox, nc);
  memcpy(Uold.p, U->p, sizeof(double) * (size_t)(Uold.csz * nc));
  Fab W = fab_alloc(UBox, np);
  double u[MF_MAX_COMP], w[MF_MAX_COMP];

  /* stateToPrim on UBox & domain, then fillGhostCells */
  FOR_BOX(WBoxB, i, j, k) {
    for (int q = 0; q < nc; ++q) u[q] = AT(U, i, j, k, q);
    cons_to_prim_cell(c, u, w);
    for (int q = 0; q < np; ++q) AT(&W, i, j, k, q) = w[q];
  }
  fill_ghost_cells(c, U, &W);

  mf_box valueBox = box_and_domain(a_box, p);
  mf_box slopeBox = box_grow(valueBox, 1, sd);

  /* reconstruction: WMinus = value on the low face, WPlus on the high face */
  Fab Wm[3], Wp[3];
  for (int d = 0; d < sd; ++d) {
    Wm[d] = fab_alloc(slopeBox, np);
    Wp[d] = fab_alloc(slopeBox, np);
    int o[3] = {0, 0, 0};
    o[d] = 1;
    FOR_BOX(slopeBox, i, j, k) {
      if (p->char_reconstruction) {
        double a[MF_MAX_COMP], b[MF_MAX_COMP], e[MF_MAX_COMP], lo[MF_MAX_COMP], hi[MF_MAX_COMP];
        for (int v = 0; v < np; ++v) {
          a[v] = AT(&W, i - o[0], j - o[1], k - o[2], v);
          b[v] = AT(&W, i, j, k, v);
          e[v] = AT(&W, i + o[0], j + o[1], k + o[2], v);
        }
        char_face_values(c, d, a, b, e, lo, hi);
        for (int v = 0; v < np; ++v) {
          AT(&Wm[d], i, j, k, v) = lo[v];
          AT(&Wp[d], i, j, k, v) = hi[v];
        }
        continue;
      }
      for (int v = 0; v < np; ++v) {
        double lo, hi;
        face_values(limiter_of(c, v), AT(&W, i - o[0], j - o[1], k - o[2], v), AT(&W, i, j, k, v),
                    AT(&W, i + o[0], j + o[1], k + o[2], v), &lo, &hi);
        AT(&Wm[d], i, j, k, v) = lo;
        AT(&Wp[d], i, j, k, v) = hi;
      }
    }
    if (p->check_positivity) {
      /* CHECKPOSITIVITY on rho and p, REDUCEORDER on every variable
         (src/Reconstruction.cpp:209-234) */
      FOR_BOX(slopeBox, i, j, k) {
        int neg = 0;
        if (AT(&Wm[d], i, j, k, 0) <= 0.0) neg = 1;
        if (AT(&Wp[d], i, j, k, 0) <= 0.0) neg = 1;
        if (AT(&Wm[d], i, j, k, 4) <= 0.0) neg = 1;
        if (AT(&Wp[d], i, j, k, 4) <= 0.0) neg = 1;
        if (neg)
          for (int v = 0; v < np; ++v) {
            AT(&Wm[d], i, j, k, v) = AT(&W, i, j, k, v);
            AT(&Wp[d], i, j, k, v) = AT(&W, i, j, k, v);
          }
      }
    }
  }

  /* fluxes on fluxBox = surroundingNodes(valueBox): interior faces by the
     Riemann solvers, domain-boundary faces (fluxBC) by the same solvers on
     the ghost-filled states; Bn = average of the two face states, one-sided
     on non-periodic domain faces (PatchMHDMF::computeBn :509-620). */
  Fab Fl[3], Bn[3];
  for (int d = 0; d < sd; ++d) {
    mf_box fb = box_nodes(valueBox, d);
    Fl[d] = fab_alloc(fb, nc);
    Bn[d] = fab_alloc(fb, 1);
    int o[3] = {0, 0, 0};
    o[d] = 1;
    double wl[MF_MAX_COMP], wr[MF_MAX_COMP], g[MF_MAX_COMP];
    FOR_BOX(fb, i, j, k) {
      for (int v = 0; v < np; ++v) {
        wl[v] = AT(&Wp[d], i - o[0], j - o[1], k - o[2], v);
        wr[v] = AT(&Wm[d], i, j, k, v);
      }
      for (int q = 0; q < nc; ++q) g[q] = NAN;
      face_flux(c, d, wl, wr, g);
      for (int q = 0; q < nc; ++q) AT(&Fl[d], i, j, k, q) = g[q];
      int f = (d == 0) ? i : (d == 1) ? j : k;
      double bn;
      if (p->divb_method == 2) {
        bn = 0.5 * (AT(&W, i - o[0], j - o[1], k - o[2], 5 + d) + AT(&W, i, j, k, 5 + d));
      } else {
        bn = 0.5 * (wl[5 + d] + wr[5 + d]);
        if (!p->periodic[d]) {
          if (f == p->domain_lo[d]) bn = wr[5 + d];
          if (f == p->domain_hi[d] + 1) bn = wl[5 + d];
        }
      }
      if (p->divb_method == 0) bn = 0.0;
      /* HeliosphericProblem::fluxBC (swlism/HeliosphericProblem.cpp:1994-2188)
         after the Riemann fluxes and computeBn (src/PatchMHDAM.cpp:608-623) */
      if (p->helio_bc && p->bc_kind == MF_BC_FARFIELD && !p->periodic[d] &&
          (f == p->domain_lo[d] || f == p->domain_hi[d] + 1)) {
        helio_bc_face(c, d, f == p->domain_lo[d] ? 0 : 1, wl, wr, g, &bn);
        for (int q = 0; q < nc; ++q) AT(&Fl[d], i, j, k, q) = g[q];
      }
      AT(&Bn[d], i, j, k, 0) = bn;
      if (c->nls) {
        level_set_flux(c, d, wl, wr, g);
        for (int q = c->ils; q < nc; ++q) AT(&Fl[d], i, j, k, q) = g[q];
      }
    }
  }

  /* finalUpdate (src/PatchMHDAM.cpp:475-493): UPDATECONS (src/PatchMHDAMF.ChF:
     542-587) on the fluid components, then UPDATELEVELSET */
  double invvol = 1.0 / p->dx;
  for (int d = 0; d < sd; ++d) {
    int o[3] = {0, 0, 0};
    o[d] = 1;
    for (int q = 0; q < c->ils; ++q) {
      FOR_BOX(valueBox, i, j, k) {
        AT(U, i, j, k, q) = AT(U, i, j, k, q) - dt * invvol *
                                                    (AT(&Fl[d], i + o[0], j + o[1], k + o[2], q) -
                                                     AT(&Fl[d], i, j, k, q));
      }
    }
    level_set_update(c, U, &W, &Fl[d], d, dt, valueBox);
  }

  /* addExplicitSources (srcIdeal/PatchMHDMF.cpp:1149-1389) */
  double psicoef = 0.0;
  if (c->glm) psicoef = exp(-dt * c->dCh * c->dCh / (c->dCp * c->dCp));
  double dtbydx = dt / p->dx;
  double S[MF_MAX_COMP];
  FOR_BOX(valueBox, i, j, k) {
    double divB = 0.0;
    for (int d = 0; d < sd; ++d) {
      int o[3] = {0, 0, 0};
      o[d] = 1;
      divB = divB + AT(&Bn[d], i + o[0], j + o[1], k + o[2], 0) - AT(&Bn[d], i, j, k, 0);
    }
    for (int q = 0; q < np; ++q) w[q] = AT(&W, i, j, k, q);
    if (p->use_8wave) {
      /* SOURCE8WAVES (srcIdeal/PatchIdealMHDF.ChF:681-722) + ADDSOURCES */
      double dB = -divB * dtbydx;
      double Ux = w[1], Uy = w[2], Uz = w[3];
      double Bx = D_1_4PI * w[5], By = D_1_4PI * w[6], Bz = D_1_4PI * w[7];
      S[1] = dB * Bx;
      S[2] = dB * By;
      S[3] = dB * Bz;
      S[4] = dB * (Bx * Ux + By * Uy + Bz * Uz);
      S[5] = dB * Ux;
      S[6] = dB * Uy;
      S[7] = dB * Uz;
      for (int q = 1; q <= 7; ++q) AT(U, i, j, k, q) = AT(U, i, j, k, q) + S[q];
      if (divBout && box_in(&divBout->b, i, j, k)) AT(divBout, i, j, k, 0) = divB;
    }
    if (c->glm) AT(U, i, j, k, 8) = psicoef * AT(U, i, j, k, 8); /* PSIPARABOLIC */
    if (p->charge_exchange && c->nf >= 2) {
      /* HeliosphericProblem::explicitSource (swlism/HeliosphericProblem.cpp:1394-1539) */
      int reg = region_cell(c, i, j, k, w);
      charge_exchange_cell(c, w, reg, dt, S);
      int iEND = c->irhon + (c->nf - 2) * 5 + 4;
      for (int q = 1; q <= iEND; ++q) AT(U, i, j, k, q) = AT(U, i, j, k, q) + S[q];
    }
  }

  /* constrained transport: the edge field of the stage's fluxes and the cell
     field from Uold (src/PatchMHDAM.cpp:684-698) */
  if (c->ct) {
    Edges E;
    edges_alloc(&E, valueBox, sd);
    electric_field(c, &W, Fl, valueBox, &E);
    recalc_b(c, U, &Uold, &E, dt, valueBox);
    if (Eout) edges_copy(Eout, &E);
    edges_free(&E);
  }

  /* problem postprocessing, then positivity (src/PatchMHDAM.cpp:705-707) */
  FOR_BOX(valueBox, i, j, k) {
    for (int q = 0; q < nc; ++q) u[q] = AT(U, i, j, k, q);
    if (p->reinit_sphere) reinit_cell(c, i, j, k, time + dt, u);
    positivity_cell(c, u);
    for (int q = 0; q < nc; ++q) AT(U, i, j, k, q) = u[q];
  }
  if (c->nls) level_set_postprocess(c, U, &Uold, valueBox);

  if (F) {
    for (int d = 0; d < sd; ++d) {
      mf_box fb = box_nodes(valueBox, d);
      if (!box_contains(&F[d].b, &fb)) continue;
      for (int q = 0; q < nc; ++q) FOR_BOX(fb, i, j, k) AT(&F[d], i, j, k, q) = AT(&Fl[d], i, j, k, q);
    }
  }

  for (int d = 0; d < sd; ++d) {
    fab_free(&Wm[d]);
    fab_free(&Wp[d]);
    fab_free(&Fl[d]);
    fab_free(&Bn[d]);
  }
  fab_free(&W);
  fab_free(&Uold);
  return MF_OK;
}


/* ------------------------------------------------------------------------ */
/* Hancock                                                                   */
/* ------------------------------------------------------------------------ */

/* Reconstruction::faceValues + checkPositivity on slopeBox (as EulerStep):
   Wm = value on the low face of each cell, Wp on the high face. */
static void reconstruct_faces(const Ctx* c, const Fab* W, mf_box slopeBox, Fab* Wm, Fab* Wp) {
  const mf_params* p = c->p;
  const int np = c->nprim;
  for (int d = 0; d < c->sd; ++d) {
    Wm[d] = fab_alloc(slopeBox, np);
    Wp[d] = fab_alloc(slopeBox, np);
    int o[3] = {0, 0, 0};
    o[d] = 1;
    FOR_BOX(slopeBox, i, j, k) {
      if (p->char_reconstruction) {
        double a[MF_MAX_COMP], b[MF_MAX_COMP], e[MF_MAX_COMP], lo[MF_MAX_COMP], hi[MF_MAX_COMP];
        for (int v = 0; v < np; ++v) {
          a[v] = AT(W, i - o[0], j - o[1], k - o[2], v);
          b[v] = AT(W, i, j, k, v);
          e[v] = AT(W, i + o[0], j + o[1], k + o[2], v);
        }
        char_face_values(c, d, a, b, e, lo, hi);
        for (int v = 0; v < np; ++v) {
          AT(&Wm[d], i, j, k, v) = lo[v];
          AT(&Wp[d], i, j, k, v) = hi[v];
        }
        continue;
      }
      for (int v = 0; v < np; ++v) {
        double lo, hi;
        face_values(limiter_of(c, v), AT(W, i - o[0], j - o[1], k - o[2], v), AT(W, i, j, k, v),
                    AT(W, i + o[0], j + o[1], k + o[2], v), &lo, &hi);
        AT(&Wm[d], i, j, k, v) = lo;
        AT(&Wp[d], i, j, k, v) = hi;
      }
    }
    if (p->check_positivity) {
      FOR_BOX(slopeBox, i, j, k) {
        int neg = 0;
        if (AT(&Wm[d], i, j, k, 0) <= 0.0) neg = 1;
        if (AT(&Wp[d], i, j, k, 0) <= 0.0) neg = 1;
        if (AT(&Wm[d], i, j, k, 4) <= 0.0) neg = 1;
        if (AT(&Wp[d], i, j, k, 4) <= 0.0) neg = 1;
        if (neg)
          for (int v = 0; v < np; ++v) {
            AT(&Wm[d], i, j, k, v) = AT(W, i, j, k, v);
            AT(&Wp[d], i, j, k, v) = AT(W, i, j, k, v);
          }
      }
    }
  }
}

/* PatchMHDMF::computeBn (srcIdeal/PatchMHDMF.cpp:509-620) on the faces fb of
   direction d: method 1 = average of the two face states (one-sided on
   non-periodic domain faces), method 2 = central average of W. */
static void compute_bn(const Ctx* c, const Fab* W, const Fab* Wm, const Fab* Wp, int d, mf_box fb,
                       Fab* Bn) {
  const mf_params* p = c->p;
  int o[3] = {0, 0, 0};
  o[d] = 1;
  FOR_BOX(fb, i, j, k) {
    double wl = AT(Wp, i - o[0], j - o[1], k - o[2], 5 + d);
    double wr = AT(Wm, i, j, k, 5 + d);
    int f = (d == 0) ? i : (d == 1) ? j : k;
    double bn;
    if (p->divb_method == 2) {
      bn = 0.5 * (AT(W, i - o[0], j - o[1], k - o[2], 5 + d) + AT(W, i, j, k, 5 + d));
    } else {
      bn = 0.5 * (wl + wr);
      if (!p->periodic[d]) {
        if (f == p->domain_lo[d]) bn = wr;
        if (f == p->domain_hi[d] + 1) bn = wl;
      }
    }
    if (p->divb_method == 0) bn = 0.0;
    AT(Bn, i, j, k, 0) = bn;
  }
}

/* FLUXESHANCOCK (srcIdeal/PatchIdealMHDF.ChF:235-297) for the plasma and
   FLUXESHANCOCK_E (srcIdeal/PatchEulerF.ChF:417-468) for each neutral
   fluid: the physical flux in direction d of one primitive state.  The psi
   flux is not set by the reference (FArrayBox::resize leaves it
   uninitialised); here it is zero. */
static void hancock_point_flux(const Ctx* c, int d, const double* w, double* F) {
  const int in = 1 + d, it1 = 1 + (d + 1) % 3, it2 = 1 + (d + 2) % 3;
  const int inB = 5 + d, itB1 = 5 + (d + 1) % 3, itB2 = 5 + (d + 2) % 3;
  double rho = w[0] > c->smallr ? w[0] : c->smallr;
  double u = w[in], v = w[it1], ww = w[it2];
  double pr = w[4] > c->smallp ? w[4] : c->smallp;
  double bx = w[inB], by = w[itB1], bz = w[itB2];
  double b = D_1_8PI * (bx * bx + by * by + bz * bz);
  double ke = 0.5 * (u * u + v * v + ww * ww);
  double bu = bx * u + by * v + bz * ww;
  double e = pr * c->invhgamma + rho * ke;
  pr = pr + b;
  e = e + b;
  F[0] = rho * u;
  F[in] = rho * u * u + pr - D_1_4PI * bx * bx;
  F[it1] = rho * u * v - D_1_4PI * bx * by;
  F[it2] = rho * u * ww - D_1_4PI * bx * bz;
  F[4] = u * (e + pr) - D_1_4PI * bx * bu;
  F[inB] = 0.0;
  F[itB1] = u * by - v * bx;
  F[itB2] = u * bz - ww * bx;
  if (c->glm) F[8] = 0.0;
  for (int f = 1; f < c->nf; ++f) {
    const int s = c->irhon + (f - 1) * 5;
    double r = w[s] > c->smallr ? w[s] : c->smallr;
    double un = w[s + 1 + d], vn = w[s + 1 + (d + 1) % 3], wn = w[s + 1 + (d + 2) % 3];
    double pn = w[s + 4] > c->smallp ? w[s + 4] : c->smallp;
    double k2 = 0.5 * (un * un + vn * vn + wn * wn);
    double en = pn * c->invhgamma + r * k2;
    F[s] = r * un;
    F[s + 1 + d] = r * un * un + pn;
    F[s + 1 + (d + 1) % 3] = r * un * vn;
    F[s + 1 + (d + 2) % 3] = r * un * wn;
    F[s + 4] = un * (en + pn);
  }
  /* FLUXESHANCOCK_LS (src/LevelSetF.ChF:9-35): surface times the plasma
     normal velocity */
  for (int q = c->ils; q < c->nc; ++q) F[q] = w[q] * w[in];
}

/* addExplicitSources for PatchMHDMF (srcIdeal/PatchMHDMF.cpp:1149-1389) on
   box with the primitive state W and face Bn: 8-wave, PSIPARABOLIC, charge
   exchange (regions from W). */
static void explicit_sources(const Ctx* c, Fab* U, const Fab* W, Fab* Bn, double dt, mf_box box,
                             Fab* divBout) {
  const mf_params* p = c->p;
  const int sd = c->sd, np = c->nprim;
  double psicoef = 0.0;
  if (c->glm) psicoef = exp(-dt * c->dCh * c->dCh / (c->dCp * c->dCp));
  double dtbydx = dt / p->dx;
  double S[MF_MAX_COMP], w[MF_MAX_COMP];
  FOR_BOX(box, i, j, k) {
    double divB = 0.0;
    for (int d = 0; d < sd; ++d) {
      int o[3] = {0, 0, 0};
      o[d] = 1;
      divB = divB + AT(&Bn[d], i + o[0], j + o[1], k + o[2], 0) - AT(&Bn[d], i, j, k, 0);
    }
    for (int q = 0; q < np; ++q) w[q] = AT(W, i, j, k, q);
    if (p->use_8wave) {
      double dB = -divB * dtbydx;
      double Ux = w[1], Uy = w[2], Uz = w[3];
      double Bx = D_1_4PI * w[5], By = D_1_4PI * w[6], Bz = D_1_4PI * w[7];
      S[1] = dB * Bx;
      S[2] = dB * By;
      S[3] = dB * Bz;
      S[4] = dB * (Bx * Ux + By * Uy + Bz * Uz);
      S[5] = dB * Ux;
      S[6] = dB * Uy;
      S[7] = dB * Uz;
      for (int q = 1; q <= 7; ++q) AT(U, i, j, k, q) = AT(U, i, j, k, q) + S[q];
      if (divBout && box_in(&divBout->b, i, j, k)) AT(divBout, i, j, k, 0) = divB;
    }
    if (c->glm) AT(U, i, j, k, 8) = psicoef * AT(U, i, j, k, 8);
    if (p->charge_exchange && c->nf >= 2) {
      int reg = region_cell(c, i, j, k, w);
      charge_exchange_cell(c, w, reg, dt, S);
      int iEND = c->irhon + (c->nf - 2) * 5 + 4;
      for (int q = 1; q <= iEND; ++q) AT(U, i, j, k, q) = AT(U, i, j, k, q) + S[q];
    }
  }
}

static void prim_fab(const Ctx* c, const Fab* U, mf_box WBoxB, Fab* W) {
  double u[MF_MAX_COMP], w[MF_MAX_COMP];
  FOR_BOX(WBoxB, i, j, k) {
    for (int q = 0; q < c->nc; ++q) u[q] = AT(U, i, j, k, q);
    cons_to_prim_cell(c, u, w);
    for (int q = 0; q < c->nprim; ++q) AT(W, i, j, k, q) = w[q];
  }
  fill_ghost_cells(c, U, W);
}

/* updateState, TA_Hancock (src/PatchMHDAM.cpp:1287-1301): predictorHancock
   (:836-1000) with dt/2 on box.grow(1), then correctorHancock (:1002-1189)
   with dt on box. */
static int hancock_step(const Ctx* c, double time, Fab* U, Fab* F, Fab* divBout, double dt,
                        mf_box a_box, Edges* Eout) {
  const mf_params* p = c->p;
  const int sd = c->sd, nc = c->nc, np = c->nprim;

  mf_box UBox = U->b;
  mf_box WBoxB = (p->bc_kind == MF_BC_FARFIELD) ? box_and_domain(UBox, p) : UBox;
  const double dtp = 0.5 * dt;

  /* ---- predictor ---- */
  Fab W = fab_alloc(UBox, np);
  prim_fab(c, U, WBoxB, &W);
  mf_box valueBox = box_and_domain(box_grow(a_box, 1, sd), p);
  mf_box slopeBox = box_grow(valueBox, 1, sd);
  Fab Wm[3], Wp[3], Bn[3];
  reconstruct_faces(c, &W, slopeBox, Wm, Wp);
  for (int d = 0; d < sd; ++d) {
    Bn[d] = fab_alloc(box_nodes(valueBox, d), 1);
    compute_bn(c, &W, &Wm[d], &Wp[d], d, box_nodes(valueBox, d), &Bn[d]);
  }
  Fab Up = fab_alloc(UBox, nc);
  memcpy(Up.p, U->p, sizeof(double) * (size_t)(Up.csz * nc));
  /* updateHancock -> UPDATECONSHANCOCK (src/PatchMHDAMF.ChF:589-638), one
     direction after another, every conserved component */
  double invvol = 1.0 / p->dx;
  double wm[MF_MAX_COMP], wp[MF_MAX_COMP], fm[MF_MAX_COMP], fp[MF_MAX_COMP];
  for (int d = 0; d < sd; ++d) {
    FOR_BOX(valueBox, i, j, k) {
      for (int v = 0; v < np; ++v) {
        wm[v] = AT(&Wm[d], i, j, k, v);
        wp[v] = AT(&Wp[d], i, j, k, v);
      }
      hancock_point_flux(c, d, wm, fm);
      hancock_point_flux(c, d, wp, fp);
      /* UPDATELEVELSETHANCOCK (src/LevelSetF.ChF:354-388), Cartesian */
      double vel = AT(&W, i, j, k, 1 + d);
      for (int q = c->ils; q < nc; ++q)
        AT(&Up, i, j, k, q) = AT(&Up, i, j, k, q) - dtp / (p->dx * 1.0) * vel * (fp[q] - fm[q]);
      for (int q = 0; q < c->ils; ++q)
        AT(&Up, i, j, k, q) = AT(&Up, i, j, k, q) - dtp * invvol * (fp[q] - fm[q]);
    }
  }
  explicit_sources(c, &Up, &W, Bn, dtp, valueBox, NULL);
  /* predicted primitive state, then UPDATEVALUESONFACES (:640-661) */
  Fab Wpr = fab_alloc(UBox, np);
  prim_fab(c, &Up, WBoxB, &Wpr);
  for (int d = 0; d < sd; ++d) {
    FOR_BOX(slopeBox, i, j, k) {
      for (int v = 0; v < np; ++v) {
        double aux = AT(&Wpr, i, j, k, v) - AT(&W, i, j, k, v);
        AT(&Wm[d], i, j, k, v) = AT(&Wm[d], i, j, k, v) + aux;
        AT(&Wp[d], i, j, k, v) = AT(&Wp[d], i, j, k, v) + aux;
      }
    }
    compute_bn(c, &W, &Wm[d], &Wp[d], d, box_nodes(valueBox, d), &Bn[d]);
  }

  /* ---- corrector ---- */
  mf_box vb2 = box_and_domain(a_box, p);
  Fab Fl[3];
  double wl[MF_MAX_COMP], wr[MF_MAX_COMP], g[MF_MAX_COMP];
  for (int d = 0; d < sd; ++d) {
    mf_box fb = box_nodes(vb2, d);
    Fl[d] = fab_alloc(fb, nc);
    int o[3] = {0, 0, 0};
    o[d] = 1;
    FOR_BOX(fb, i, j, k) {
      for (int v = 0; v < np; ++v) {
        wl[v] = AT(&Wp[d], i - o[0], j - o[1], k - o[2], v);
        wr[v] = AT(&Wm[d], i, j, k, v);
      }
      for (int q = 0; q < nc; ++q) g[q] = NAN;
      face_flux(c, d, wl, wr, g);
      /* fluxBC of correctorHancock (src/PatchMHDAM.cpp:1105-1106): also
         replaces the predictor's Bn of the boundary faces */
      int f = (d == 0) ? i : (d == 1) ? j : k;
      if (p->helio_bc && p->bc_kind == MF_BC_FARFIELD && !p->periodic[d] &&
          (f == p->domain_lo[d] || f == p->domain_hi[d] + 1)) {
        double bnv = AT(&Bn[d], i, j, k, 0);
        helio_bc_face(c, d, f == p->domain_lo[d] ? 0 : 1, wl, wr, g, &bnv);
        AT(&Bn[d], i, j, k, 0) = bnv;
      }
      if (c->nls) level_set_flux(c, d, wl, wr, g);
      for (int q = 0; q < nc; ++q) AT(&Fl[d], i, j, k, q) = g[q];
    }
  }
  /* the corrector's Uold: the state before the step (src/PatchMHDAM.cpp:
     1043-1044; the predictor advanced a copy) */
  Fab Uold = fab_alloc(UBox, nc);
  memcpy(Uold.p, U->p, sizeof(double) * (size_t)(Uold.csz * nc));
  /* finalUpdate with the full dt: UPDATECONS, then UPDATELEVELSET with the
     velocity of W(t) (correctorHancock receives the predictor's WOld) */
  for (int d = 0; d < sd; ++d) {
    int o[3] = {0, 0, 0};
    o[d] = 1;
    for (int q = 0; q < c->ils; ++q) {
      FOR_BOX(vb2, i, j, k) {
        AT(U, i, j, k, q) = AT(U, i, j, k, q) - dt * invvol *
                                                    (AT(&Fl[d], i + o[0], j + o[1], k + o[2], q) -
                                                     AT(&Fl[d], i, j, k, q));
      }
    }
    level_set_update(c, U, &W, &Fl[d], d, dt, vb2);
  }
  explicit_sources(c, U, &Wpr, Bn, dt, vb2, divBout);
  /* constrained transport with W(t+dt/2) (src/PatchMHDAM.cpp:1150-1160) */
  if (c->ct) {
    Edges E;
    edges_alloc(&E, vb2, sd);
    electric_field(c, &Wpr, Fl, vb2, &E);
    recalc_b(c, U, &Uold, &E, dt, vb2);
    if (Eout) edges_copy(Eout, &E);
    edges_free(&E);
  }
  double u[MF_MAX_COMP];
  FOR_BOX(vb2, i, j, k) {
    for (int q = 0; q < nc; ++q) u[q] = AT(U, i, j, k, q);
    if (p->reinit_sphere) reinit_cell(c, i, j, k, time + dt, u);
    positivity_cell(c, u);
    for (int q = 0; q < nc; ++q) AT(U, i, j, k, q) = u[q];
  }
  if (c->nls) level_set_postprocess(c, U, &Uold, vb2);
  fab_free(&Uold);
  if (F) {
    for (int d = 0; d < sd; ++d) {
      mf_box fb = box_nodes(vb2, d);
      if (!box_contains(&F[d].b, &fb)) continue;
      for (int q = 0; q < nc; ++q) FOR_BOX(fb, i, j, k) AT(&F[d], i, j, k, q) = AT(&Fl[d], i, j, k, q);
    }
  }
  for (int d = 0; d < sd; ++d) {
    fab_free(&Wm[d]);
    fab_free(&Wp[d]);
    fab_free(&Bn[d]);
    fab_free(&Fl[d]);
  }
  fab_free(&W);
  fab_free(&Wpr);
  fab_free(&Up);
  return MF_OK;
}

/* ------------------------------------------------------------------------ */
/* dt                                                                        */
/* ------------------------------------------------------------------------ */

/* MAXWAVESPEED (srcIdeal/PatchIdealMHDF.ChF:5-63) + MAXWAVESPEED_E
   (srcIdeal/PatchEulerF.ChF:5-50) of one cell. */
static double max_wave_speed_cell(const Ctx* c, const double* cons) {
  const double gamma = c->gamma, hgamma = c->hgamma;
  double cmax = 0.0;
  {
    double rho = cons[0];
    double invrho = 1.0 / rho;
    double ru = cons[1], rv = cons[2], rw = cons[3];
    double u = ru * invrho, v = rv * invrho, w = rw * invrho;
    double ke = ru * u + rv * v + rw * w;
    double bx = cons[5], by = cons[6], bz = cons[7];
    double b = D_1_4PI * (bx * bx + by * by + bz * bz);
    double p = hgamma * (cons[4] - 0.5 * (ke + b));
    p = fmax(p, c->smallp);
    double a2 = gamma * p * invrho;
    double as2 = 0.5 * (a2 + invrho * b);
    double as4 = as2 * as2;
    double bn2 = D_1_4PI * bx * bx * invrho;
    double cf2 = as2 + sqrt(as4 - a2 * bn2);
    double umax = fabs(u) + sqrt(cf2);
    bn2 = D_1_4PI * by * by * invrho;
    cf2 = as2 + sqrt(as4 - a2 * bn2);
    umax = fmax(fabs(v) + sqrt(cf2), umax);
    bn2 = D_1_4PI * bz * bz * invrho;
    cf2 = as2 + sqrt(as4 - a2 * bn2);
    umax = fmax(fabs(w) + sqrt(cf2), umax);
    cmax = fmax(umax, cmax);
  }
  for (int f = 1; f < c->nf; ++f) {
    int s = c->irhon + (f - 1) * 5;
    double rho = cons[s];
    rho = fmax(rho, c->smallr);
    double invrho = 1.0 / rho;
    double ru = cons[s + 1], rv = cons[s + 2], rw = cons[s + 3];
    double u = ru * invrho, v = rv * invrho, w = rw * invrho;
    double ke = ru * u + rv * v + rw * w;
    double p = hgamma * (cons[s + 4] - 0.5 * ke);
    p = fmax(p, c->smallp);
    double a = sqrt(gamma * p * invrho);
    double umax = fmax(fmax(fabs(u), fabs(v)), fabs(w)) + a;
    cmax = fmax(umax, cmax);
  }
  return cmax;
}

/* PatchMHDMF::computeDt + PhysProblem::computeDt (src/PhysProblem.cpp:298-319):
   dt = dx / cmax, first minimum in box order (FArrayBox::minIndex). */
static void compute_dt_fab(const Ctx* c, const Fab* U, mf_box box, double* dt, int cell[3]) {
  double u[MF_MAX_COMP];
  int first = 1;
  double best = 0.0;
  FOR_BOX(box, i, j, k) {
    for (int q = 0; q < c->nc; ++q) u[q] = AT(U, i, j, k, q);
    double cm = max_wave_speed_cell(c, u);
    double v = c->p->dx / cm;
    if (first || v < best) {
      best = v;
      cell[0] = i;
      cell[1] = j;
      cell[2] = k;
      first = 0;
    }
  }
  *dt = best;
}

/* ------------------------------------------------------------------------ */
/* updateState                                                               */
/* ------------------------------------------------------------------------ */

static int check_fab(const Ctx* c, const mf_fab* U, const mf_box* valid) {
  if (!U || !U->data || !valid) return MF_ERR_BAD_ARG;
  if (U->ncomp != c->nc) return MF_ERR_BAD_ARG;
  mf_box need = box_grow(*valid, num_ghost(c->p), c->sd);
  if (!box_contains(&U->box, &need)) return MF_ERR_BAD_ARG;
  return MF_OK;
}

/* Edges view of caller fabs on the edges of box (E[0..2] in 3D, E[0] in 2D) */
static int edges_wrap(const Ctx* c, mf_fab* Ef, mf_box box, Edges* E) {
  Edges want;
  edges_alloc(&want, box, c->sd);
  int ok = 1;
  E->n = want.n;
  for (int d = 0; d < want.n; ++d) {
    if (!Ef[d].data || !box_contains(&Ef[d].box, &want.e[d].b)) ok = 0;
    E->e[d] = fab_wrap(Ef[d].data, Ef[d].box, 1);
  }
  if (c->sd == 2) E->e[1] = E->e[2] = E->e[0];
  edges_free(&want);
  return ok ? MF_OK : MF_ERR_BAD_ARG;
}

int mf_oracle_patch_update(const mf_params* p, double time, mf_fab* Uf, const mf_box* valid,
                           double dt, mf_fab* Fout, mf_fab* divBf, double* new_dt,
                           int min_cell[3]) {
  return mf_oracle_patch_update_e(p, time, Uf, valid, dt, Fout, divBf, NULL, new_dt, min_cell);
}

int mf_oracle_patch_update_e(const mf_params* p, double time, mf_fab* Uf, const mf_box* valid,
                             double dt, mf_fab* Fout, mf_fab* divBf, mf_fab* Ef, double* new_dt,
                             int min_cell[3]) {
  Ctx c;
  int st = ctx_init(&c, p);
  if (st) return st;
  st = check_fab(&c, Uf, valid);
  if (st) return st;
  Edges Eo, *pE = NULL;
  if (Ef && c.ct) {
    st = edges_wrap(&c, Ef, *valid, &Eo);
    if (st) return st;
    pE = &Eo;
  }
  Fab U = fab_wrap(Uf->data, Uf->box, Uf->ncomp);
  Fab divB, *pdivB = NULL;
  if (divBf && divBf->data) {
    divB = fab_wrap(divBf->data, divBf->box, 1);
    pdivB = &divB;
  }
  Fab F[3], *pF = NULL;
  if (Fout) {
    for (int d = 0; d < c.sd; ++d) F[d] = fab_wrap(Fout[d].data, Fout[d].box, Fout[d].ncomp);
    pF = F;
  }
  long n = U.csz * c.nc;
  if (p->time_approximation == MF_TA_RK2) {
    /* src/PatchMHDAM.cpp:1239-1286 */
    Fab Uold = fab_alloc(U.b, c.nc);
    Fab Upred = fab_alloc(U.b, c.nc);
    memcpy(Uold.p, U.p, sizeof(double) * (size_t)n);
    memcpy(Upred.p, U.p, sizeof(double) * (size_t)n);
    Fab Fp[3];
    mf_box bp = box_grow(*valid, 2, c.sd);
    mf_box vbp = box_and_domain(bp, p);
    for (int d = 0; d < c.sd; ++d) Fp[d] = fab_alloc(box_nodes(vbp, d), c.nc);
    Edges Ep; /* EPredictor on the box of the caller's E */
    if (pE) edges_alloc(&Ep, *valid, c.sd);
    euler_step(&c, time, &Upred, pF ? Fp : NULL, pdivB, dt, bp, pE ? &Ep : NULL);
    memcpy(U.p, Upred.p, sizeof(double) * (size_t)n);
    euler_step(&c, time, &U, pF, pdivB, 0.5 * dt, *valid, pE);
    if (pE) { /* a_E += EPredictor; a_E *= 0.5 */
      for (int d = 0; d < pE->n; ++d) FOR_BOX(Ep.e[d].b, i, j, k) {
          AT(&pE->e[d], i, j, k, 0) = AT(&pE->e[d], i, j, k, 0) + AT(&Ep.e[d], i, j, k, 0);
          AT(&pE->e[d], i, j, k, 0) = AT(&pE->e[d], i, j, k, 0) * 0.5;
        }
      edges_free(&Ep);
    }
    if (pF) {
      mf_box vb = box_and_domain(*valid, p);
      for (int d = 0; d < c.sd; ++d) {
        mf_box fb = box_nodes(vb, d);
        for (int q = 0; q < c.nc; ++q) FOR_BOX(fb, i, j, k) {
            AT(&F[d], i, j, k, q) = AT(&F[d], i, j, k, q) + AT(&Fp[d], i, j, k, q);
            AT(&F[d], i, j, k, q) = AT(&F[d], i, j, k, q) * 0.5;
          }
      }
    }
    /* AVERAGESTATE (src/PatchMHDAMF.ChF:289-316) */
    for (int q = 0; q < c.nc; ++q) FOR_BOX((*valid), i, j, k) {
        AT(&U, i, j, k, q) =
            AT(&U, i, j, k, q) + 0.5 * (AT(&Uold, i, j, k, q) - AT(&Upred, i, j, k, q));
      }
    for (int d = 0; d < c.sd; ++d) fab_free(&Fp[d]);
    fab_free(&Uold);
    fab_free(&Upred);
  } else if (p->time_approximation == MF_TA_HANCOCK) {
    hancock_step(&c, time, &U, pF, pdivB, dt, *valid, pE);
  } else {
    euler_step(&c, time, &U, pF, pdivB, dt, *valid, pE);
  }
  double ndt;
  int cell[3] = {0, 0, 0};
  compute_dt_fab(&c, &U, *valid, &ndt, cell);
  if (new_dt) *new_dt = ndt;
  if (min_cell) {
    min_cell[0] = cell[0];
    min_cell[1] = cell[1];
    min_cell[2] = cell[2];
  }
  return MF_OK;
}

int mf_oracle_recalculate_b(const mf_params* p, mf_fab* Uf, const mf_fab* Uoldf, mf_fab* Ef,
                            double dt, const mf_box* box) {
  Ctx c;
  int st = ctx_init(&c, p);
  if (st) return st;
  if (!c.ct) return MF_ERR_BAD_ARG;
  if (!Uf || !Uoldf || !Ef || !box || !box_contains(&Uf->box, box) ||
      !box_contains(&Uoldf->box, box))
    return MF_ERR_BAD_ARG;
  Edges E;
  st = edges_wrap(&c, Ef, *box, &E);
  if (st) return st;
  Fab U = fab_wrap(Uf->data, Uf->box, Uf->ncomp);
  Fab Uo = fab_wrap(Uoldf->data, Uoldf->box, Uoldf->ncomp);
  recalc_b(&c, &U, &Uo, &E, dt, *box);
  return MF_OK;
}

int mf_oracle_compute_dt(const mf_params* p, const mf_fab* Uf, const mf_box* box, double* dt,
                         int min_cell[3]) {
  Ctx c;
  int st = ctx_init(&c, p);
  if (st) return st;
  if (!Uf || !box || !box_contains(&Uf->box, box)) return MF_ERR_BAD_ARG;
  Fab U = fab_wrap(Uf->data, Uf->box, Uf->ncomp);
  int cell[3] = {0, 0, 0};
  compute_dt_fab(&c, &U, *box, dt, cell);
  if (min_cell) memcpy(min_cell, cell, sizeof(cell));
  return MF_OK;
}

/* ------------------------------------------------------------------------ */
/* level                                                                     */
/* ------------------------------------------------------------------------ */

int mf_oracle_level_exchange(const mf_params* p, int npatch, mf_fab* Uf, const mf_box* valid) {
  int sd = p->space_dim;
  int L[3] = {0, 0, 0};
  for (int d = 0; d < sd; ++d) L[d] = p->domain_hi[d] - p->domain_lo[d] + 1;
  int rng[3][2];
  for (int d = 0; d < 3; ++d) {
    int r = (d < sd && p->periodic[d]) ? 1 : 0;
    rng[d][0] = -r;
    rng[d][1] = r;
  }
  for (int dp = 0; dp < npatch; ++dp) {
    Fab D = fab_wrap(Uf[dp].data, Uf[dp].box, Uf[dp].ncomp);
    for (int sp_ = 0; sp_ < npatch; ++sp_) {
      Fab S = fab_wrap(Uf[sp_].data, Uf[sp_].box, Uf[sp_].ncomp);
      for (int a = rng[0][0]; a <= rng[0][1]; ++a)
        for (int b = rng[1][0]; b <= rng[1][1]; ++b)
          for (int e = rng[2][0]; e <= rng[2][1]; ++e) {
            if (sp_ == dp && a == 0 && b == 0 && e == 0) continue;
            int sh[3] = {a * L[0], b * L[1], e * L[2]};
            mf_box r;
            int empty = 0;
            for (int d = 0; d < 3; ++d) {
              r.lo[d] = valid[sp_].lo[d] + sh[d];
              r.hi[d] = valid[sp_].hi[d] + sh[d];
              if (r.lo[d] < D.b.lo[d]) r.lo[d] = D.b.lo[d];
              if (r.hi[d] > D.b.hi[d]) r.hi[d] = D.b.hi[d];
              if (r.lo[d] > r.hi[d]) empty = 1;
            }
            if (empty) continue;
            for (int q = 0; q < D.nc; ++q) FOR_BOX(r, i, j, k) {
                if (box_in(&valid[dp], i, j, k)) continue;
                AT(&D, i, j, k, q) = AT(&S, i - sh[0], j - sh[1], k - sh[2], q);
              }
          }
    }
  }
  return MF_OK;
}

/* HeliosphericProblem::postTimeStep -> NEUTRALS_SUNBC (swlism/SWLISMF.ChF:
   1555-1598) on the strips of HeliosphericProblem::define
   (swlism/HeliosphericProblem.cpp:476-527): the cells of the sphere of radius
   sunR downstream of the sun take neutral fluid 1 (and 4) from the cell
   mirrored across the sun's x plane, y and z momenta reversed. */
static int neutral_sun_bc(const mf_params* p, int npatch, mf_fab* Uf, const mf_box* valid) {
  if (!p->neutral_sun_bc || p->n_fluids < 2 || p->space_dim != 3) return MF_OK;
  int sun[3];
  for (int d = 0; d < 3; ++d) {
    sun[d] = (int)floor(p->sun_center[d] / p->dx + 0.5);
    if (fabs(sun[d] * p->dx - p->sun_center[d]) >= 1e-6) return MF_ERR_UNSUPPORTED;
  }
  const int iR0 = 1 + (int)floor(p->reinit_r0 / p->dx + 0.5);
  const double sunR2 = p->sun_r * p->sun_r;
  const int irhon = 8 + (p->divb_cleaning == 5 ? 1 : 0);
  const double sg[5] = {1.0, 1.0, -1.0, -1.0, 1.0};
  for (int a = 0; a < iR0; ++a)
    for (int k = sun[2] - iR0 - 1; k <= sun[2] + iR0; ++k)
      for (int j = sun[1] - iR0 - 1; j <= sun[1] + iR0; ++j) {
        const int i = sun[0] + a;
        double x = (i + 0.5) * p->dx - p->sun_center[0];
        double y = (j + 0.5) * p->dx - p->sun_center[1];
        double z = (k + 0.5) * p->dx - p->sun_center[2];
        double r2 = x * x + y * y + z * z;
        if (!(r2 <= sunR2)) continue;
        const int iRefl = sun[0] - (i - sun[0] + 1);
        int bt = -1, bf = -1;
        for (int b = 0; b < npatch; ++b) {
          if (box_in(&valid[b], i, j, k)) bt = b;
          if (box_in(&valid[b], iRefl, j, k)) bf = b;
        }
        if (bt < 0 || bf < 0) continue;
        Fab T = fab_wrap(Uf[bt].data, Uf[bt].box, Uf[bt].ncomp);
        Fab S = fab_wrap(Uf[bf].data, Uf[bf].box, Uf[bf].ncomp);
        for (int f = 1; f < p->n_fluids; f += 3)
          for (int m = 0; m < 5; ++m) {
            const int q = irhon + (f - 1) * 5 + m;
            AT(&T, i, j, k, q) = sg[m] * AT(&S, iRefl, j, k, q);
          }
      }
  return MF_OK;
}

/* per-patch state of constrained transport across a level step: the
   level's UOld (AMRLevelIdealMHD::preTimeStep, srcIdeal/AMRLevelIdealMHD.cpp:
   673-681) and the edge field each updateState returns */
typedef struct {
  int on;
  Fab* uold;
  mf_fab (*ef)[3];
  Edges* e;
} CtLevel;

static int ct_level_init(CtLevel* L, const mf_params* p, int npatch, const mf_box* valid) {
  Ctx c;
  memset(L, 0, sizeof(*L));
  int st = ctx_init(&c, p);
  if (st) return st;
  if (!c.ct) return MF_OK;
  L->on = 1;
  L->uold = (Fab*)calloc((size_t)npatch, sizeof(Fab));
  L->ef = (mf_fab(*)[3])calloc((size_t)npatch, sizeof(mf_fab[3]));
  L->e = (Edges*)calloc((size_t)npatch, sizeof(Edges));
  for (int ip = 0; ip < npatch; ++ip) {
    edges_alloc(&L->e[ip], valid[ip], c.sd);
    for (int d = 0; d < 3; ++d) {
      const Fab* f = &L->e[ip].e[d < L->e[ip].n ? d : 0];
      L->ef[ip][d].data = f->p;
      L->ef[ip][d].box = f->b;
      L->ef[ip][d].ncomp = 1;
    }
  }
  return MF_OK;
}

static void ct_level_free(CtLevel* L, int npatch) {
  for (int ip = 0; ip < npatch; ++ip) {
    edges_free(&L->e[ip]);
    fab_free(&L->uold[ip]);
  }
  free(L->uold);
  free(L->ef);
  free(L->e);
  memset(L, 0, sizeof(*L));
}

int mf_oracle_level_step(const mf_params* p, double time, int npatch, mf_fab* Uf,
                         const mf_box* valid, double dt, int nthreads, double* new_dt,
                         int* min_patch, int min_cell[3]) {
  int st = mf_oracle_level_exchange(p, npatch, Uf, valid);
  if (st) return st;
  CtLevel ct;
  st = ct_level_init(&ct, p, npatch, valid);
  if (st) return st;
  double* dts = (double*)malloc(sizeof(double) * (size_t)npatch);
  int* cells = (int*)malloc(sizeof(int) * 3 * (size_t)npatch);
  int* sts = (int*)malloc(sizeof(int) * (size_t)npatch);
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#else
  (void)nthreads;
#endif
  for (int ip = 0; ip < npatch; ++ip) {
    mf_fab* Ep = NULL;
    if (ct.on) {
      ct.uold[ip] = fab_alloc(Uf[ip].box, Uf[ip].ncomp);
      memcpy(ct.uold[ip].p, Uf[ip].data, sizeof(double) * (size_t)(ct.uold[ip].csz * Uf[ip].ncomp));
      Ep = ct.ef[ip];
    }
    sts[ip] = mf_oracle_patch_update_e(p, time, &Uf[ip], &valid[ip], dt, NULL, NULL, Ep, &dts[ip],
                                       &cells[3 * ip]);
  }
  int best = -1;
  if (st == MF_OK) st = neutral_sun_bc(p, npatch, Uf, valid);
  /* AMRLevelIdealMHD::postTimeStep with constrained transport on a single
     level (srcIdeal/AMRLevelIdealMHD.cpp:1649-1688): every patch's field
     again from the level's UOld and the patch's step-averaged edge field */
  if (ct.on) {
    for (int ip = 0; ip < npatch; ++ip) {
      if (st == MF_OK && sts[ip] == MF_OK) {
        mf_fab uo = {ct.uold[ip].p, Uf[ip].box, Uf[ip].ncomp};
        int r = mf_oracle_recalculate_b(p, &Uf[ip], &uo, ct.ef[ip], dt, &valid[ip]);
        if (r) st = r;
      }
    }
    ct_level_free(&ct, npatch);
  }
  for (int ip = 0; ip < npatch; ++ip) {
    if (sts[ip]) st = sts[ip];
    if (best < 0 || dts[ip] < dts[best]) best = ip;
  }
  if (best >= 0) {
    if (new_dt) *new_dt = dts[best];
    if (min_patch) *min_patch = best;
    if (min_cell) memcpy(min_cell, &cells[3 * best], sizeof(int) * 3);
  }
  free(dts);
  free(cells);
  free(sts);
  return st;
}

/* ------------------------------------------------------------------------ */
/* single-point entry points for known-answer tests                          */
/* ------------------------------------------------------------------------ */

int mf_oracle_face_values(int lim, double wm1, double wp, double wp1, double* lo, double* hi) {
  if (!lo || !hi) return MF_ERR_BAD_ARG;
  face_values(lim, wm1, wp, wp1, lo, hi);
  return MF_OK;
}

int mf_oracle_face_slopes(int lim, double* sleft, double* sright) {
  if (!sleft || !sright) return MF_ERR_BAD_ARG;
  face_slopes(lim, sleft, sright);
  return MF_OK;
}

int mf_oracle_face_flux(const mf_params* p, int dir, const double* wl, const double* wr,
                        double* f) {
  Ctx c;
  int st = ctx_init(&c, p);
  if (st) return st;
  face_flux(&c, dir, wl, wr, f);
  return MF_OK;
}

int mf_oracle_helio_bc_face(const mf_params* p, int dir, int side, const double* wl,
                            const double* wr, double* f, double* bn) {
  Ctx c;
  int st = ctx_init(&c, p);
  if (st) return st;
  if (dir < 0 || dir >= c.sd || side < 0 || side > 1 || c.sd != 3) return MF_ERR_BAD_ARG;
  face_flux(&c, dir, wl, wr, f);
  helio_bc_face(&c, dir, side, wl, wr, f, bn);
  return MF_OK;
}

int mf_oracle_cons_to_prim(const mf_params* p, const double* u, double* w) {
  Ctx c;
  int st = ctx_init(&c, p);
  if (st) return st;
  cons_to_prim_cell(&c, u, w);
  return MF_OK;
}

int mf_oracle_charge_exchange(const mf_params* p, const double* w, int reg, double dt,
                              double* s) {
  Ctx c;
  int st = ctx_init(&c, p);
  if (st) return st;
  if (c.nf < 2) return MF_ERR_BAD_ARG;
  charge_exchange_cell(&c, w, reg, dt, s);
  return MF_OK;
}

int mf_oracle_region(const mf_params* p, int i, int j, int k, const double* w) {
  Ctx c;
  if (ctx_init(&c, p)) return -1;
  return region_cell(&c, i, j, k, w);
}

/* ORSZAGINIT (problems/OrszagF.ChF:27-79). */
int mf_oracle_init_orszag(const mf_params* p, mf_fab* Uf, const mf_box* box) {
  Ctx c;
  int st = ctx_init(&c, p);
  if (st) return st;
  Fab U = fab_wrap(Uf->data, Uf->box, Uf->ncomp);
  double gamma = p->gamma, hgamma = gamma - 1.0, dx = p->dx;
  double p0 = D_1_4PI * gamma;
  double r0 = p0 * gamma;
  FOR_BOX((*box), i, j, k) {
    double x = (i + 0.5) * dx;
    double y = (j + 0.5) * dx;
    double Ux = -sin(D_2PI * y);
    double Uy = sin(D_2PI * x);
    double Bx = -sin(D_2PI * y);
    double By = sin((D_2PI + D_2PI) * x);
    double b = D_1_4PI * (Bx * Bx + By * By);
    double ke = Ux * Ux + Uy * Uy;
    double e0 = p0 / hgamma + 0.5 * (r0 * ke + b);
    AT(&U, i, j, k, 0) = r0;
    AT(&U, i, j, k, 1) = r0 * Ux;
    AT(&U, i, j, k, 2) = r0 * Uy;
    AT(&U, i, j, k, 3) = 0.0;
    AT(&U, i, j, k, 4) = e0;
    AT(&U, i, j, k, 5) = Bx;
    AT(&U, i, j, k, 6) = By;
    AT(&U, i, j, k, 7) = 0.0;
    if (c.glm) AT(&U, i, j, k, 8) = 0.0;
  }
  return MF_OK;
}

/* The synthetic heliosphere's initial state: the uniform inflow given as
   primitive states (wp: plasma rho, u, v, w, p, bx, by, bz; wn: rho, u, v, w,
   p of each neutral fluid) through PRIMTOCONS_MF (srcIdeal/PatchMHDMFF.ChF:
   82-149), psi = 0, the tracking surfaces (the region tracer -1 inside the
   sphere r <= Rinit and +1 outside, as HELIOINIT sets it,
   swlism/HeliosphericF.ChF:1228-1231,1302-1304; the current-sheet surface of
   a bipolar field +1, as HeliosphericProblem's component reset sets it,
   swlism/HeliosphericProblem.cpp:2387-2393; any other surface the signed
   distance r - Rinit), then the inner sphere reset at time 0
   (HELIOREINIT_DEFAULT). */
int mf_oracle_init_helio(const mf_params* p, const double* wp, const double* wn, mf_fab* Uf,
                         const mf_box* box) {
  Ctx c;
  int st = ctx_init(&c, p);
  if (st) return st;
  if (!wp || !Uf || !Uf->data || !box || !box_contains(&Uf->box, box)) return MF_ERR_BAD_ARG;
  if (Uf->ncomp != c.nc || (c.nf > 1 && !wn)) return MF_ERR_BAD_ARG;
  Fab U = fab_wrap(Uf->data, Uf->box, Uf->ncomp);
  const double invhgamma = 1.0 / c.hgamma;
  double u[MF_MAX_COMP];
  FOR_BOX((*box), i, j, k) {
    double rho = fmax(wp[0], c.smallr);
    double uu = wp[1], vv = wp[2], ww = wp[3], pr = wp[4];
    double bx = wp[5], by = wp[6], bz = wp[7];
    double b = D_1_4PI * (bx * bx + by * by + bz * bz);
    double ke = uu * uu + vv * vv + ww * ww;
    u[0] = rho;
    u[1] = rho * uu;
    u[2] = rho * vv;
    u[3] = rho * ww;
    u[4] = pr * invhgamma + 0.5 * (rho * ke + b);
    u[5] = bx;
    u[6] = by;
    u[7] = bz;
    if (c.glm) u[8] = 0.0;
    for (int f = 1; f < c.nf; ++f) {
      const double* w = wn + 5 * (f - 1);
      int s = c.irhon + 5 * (f - 1);
      double r = fmax(w[0], c.smallr);
      double k2 = w[1] * w[1] + w[2] * w[2] + w[3] * w[3];
      u[s] = r;
      u[s + 1] = r * w[1];
      u[s + 2] = r * w[2];
      u[s + 3] = r * w[3];
      u[s + 4] = w[4] * invhgamma + 0.5 * r * k2;
    }
    if (c.nls) {
      double x = (i + 0.5) * p->dx - p->sun_center[0];
      double y = (j + 0.5) * p->dx - p->sun_center[1];
      double z = (c.sd == 3) ? (k + 0.5) * p->dx - p->sun_center[2] : 0.0;
      double r2 = x * x + y * y + z * z;
      for (int q = c.ils; q < c.nc; ++q) u[q] = sqrt(r2) - p->reinit_r0;
      if (p->region_tracer) u[c.nc - 1] = (r2 <= p->reinit_r0 * p->reinit_r0) ? -1.0 : 1.0;
      if (p->reinit_sphere && c.ihcs >= 0) u[c.ihcs] = 1.0;
    }
    if (p->reinit_sphere) reinit_cell(&c, i, j, k, 0.0, u);
    for (int q = 0; q < c.nc; ++q) AT(&U, i, j, k, q) = u[q];
  }
  return MF_OK;
}

int mf_oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* coarse-fine coupling of a subcycled hierarchy                             */
/* ------------------------------------------------------------------------ */
/* Boxes below are in the index space of their level; a level refined by r
   has cell iv above coarse cell floor(iv / r).  Coarse data outside the
   domain in a periodic direction is the periodic image of valid data. */

static int imod_(int a, int n) {
  int m = a % n;
  return m < 0 ? m + n : m;
}

static int floordiv_(int a, int r) { return (a >= 0) ? a / r : -((-a + r - 1) / r); }

static mf_box box_coarsen(mf_box b, int r, int sd) {
  for (int d = 0; d < sd; ++d) {
    b.lo[d] = floordiv_(b.lo[d], r);
    b.hi[d] = floordiv_(b.hi[d], r);
  }
  return b;
}

/* Periodic image inside the domain; 0 outside the domain in a non-periodic
   direction. */
static int wrap_cell(const mf_params* p, int iv[3]) {
  for (int d = 0; d < p->space_dim; ++d) {
    int lo = p->domain_lo[d], n = p->domain_hi[d] - lo + 1;
    if (p->periodic[d])
      iv[d] = lo + imod_(iv[d] - lo, n);
    else if (iv[d] < lo || iv[d] > p->domain_hi[d])
      return 0;
  }
  return 1;
}

/* Index of the box holding the periodic image of cell c, -1 if none. */
static int find_box_wrapped(const mf_params* p, int n, const mf_box* b, const int c[3]) {
  int w[3] = {c[0], c[1], c[2]};
  if (!wrap_cell(p, w)) return -1;
  for (int q = 0; q < n; ++q)
    if (box_in(&b[q], w[0], w[1], w[2])) return q;
  return -1;
}

/* Is the image of coarse cell c under a coarsened fine box? */
static int covered_by_fine(const mf_params* pc, int r, int nf, const mf_box* vf, const int c[3]) {
  int w[3] = {c[0], c[1], c[2]};
  if (!wrap_cell(pc, w)) return 0;
  for (int q = 0; q < nf; ++q) {
    mf_box cb = box_coarsen(vf[q], r, pc->space_dim);
    if (box_in(&cb, w[0], w[1], w[2])) return 1;
  }
  return 0;
}

/* interp_divB_0 (srcIdeal/FineInterpMHDAMF.ChF:449-555): correct the limited
   slopes d(Bx)/dx, d(By)/dy, d(Bz)/dz of one coarse cell towards a
   divergence-free linear profile. */
static void interp_divb0(int sd, double* sx, double* sy, double* sz) {
  const double eps_divB = 1.0e-8;
  double DBXDX = *sx, DBYDY = *sy, DBZDZ = (sd == 3) ? *sz : 0.0;
  double fact = (sd == 3) ? -1.0 / (1.0 + 1.0 + 1.0) : -1.0 / (1.0 + 1.0);
  double divB = (sd == 3) ? DBXDX + DBYDY + DBZDZ : DBXDX + DBYDY;
  double del = fact * divB;
  double adel = fabs(del);
  if (!(adel > eps_divB)) return;
  double delX = minmod(-DBXDX, del), delY = minmod(-DBYDY, del);
  double delZ = (sd == 3) ? minmod(-DBZDZ, del) : 0.0;
  double del2 = (sd == 3) ? delX + delY + delZ : delX + delY;
  if (fabs(del2) < fabs(divB)) {
    if (sd == 2) {
      delX = minmod(DBXDX, -DBYDY);
      delY = -delX;
      delX = delX - DBXDX;
      delY = delY - DBYDY;
    } else if (fabs(delX) < adel) {
      del = -0.5 * (delX + divB);
      delY = minmod(-DBYDY, del);
      delZ = minmod(-DBZDZ, del);
      del2 = delX + delY + delZ;
      if (fabs(del2) < fabs(divB)) {
        if (fabs(delY) < adel)
          delZ = -(divB + delX + delY);
        else
          delY = -(divB + delX + delZ);
      }
    } else if (fabs(delY) < adel) {
      del = -0.5 * (delY + divB);
      delX = minmod(-DBXDX, del);
      delZ = minmod(-DBZDZ, del);
      del2 = delX + delY + delZ;
      if (fabs(del2) < fabs(divB)) {
        if (fabs(delX) < adel)
          delZ = -(divB + delX + delY);
        else
          delX = -(divB + delY + delZ);
      }
    } else {
      del = -0.5 * (delZ + divB);
      adel = fabs(del);
      delX = minmod(-DBXDX, del);
      delY = minmod(-DBYDY, del);
      del2 = delX + delY + delZ;
      if (fabs(del2) < fabs(divB)) {
        if (fabs(delX) < adel)
          delY = -(divB + delX + delZ);
        else
          delX = -(divB + delY + delZ);
      }
    }
  }
  *sx = *sx + delX;
  *sy = *sy + delY;
  if (sd == 3) *sz = *sz + delZ;
}

/* PiecewiseLinearFillPatchMHDAM::define + fillInterp
   (srcIdeal/PiecewiseLinearFillPatchMHDAM.cpp:120-380, 382-900): fill the ghost
   cells of every fine patch that lie over coarse cells no coarsened fine box
   covers, from the coarse data interpolated in time (alpha between the old
   and new coarse states) and linearly in space with limited slopes
   (INTERPLIMIT_V, srcIdeal/FineInterpMHDAMF.ChF:235-386). */
static int cf_fill(const mf_params* pc, const mf_params* pf, int r, int ncp, mf_fab* Uold,
                   mf_fab* Unew, const mf_box* vc, int nfp, mf_fab* Uf, const mf_box* vf,
                   double alpha, int ng) {
  const int sd = pc->space_dim, nc = Unew[0].ncomp;
  const int csr = (ng + r - 1) / r, cgr = csr + 1;
  const double dxc = pc->dx, dxf = pf->dx;
  const int divb = (pc->divb_cleaning != 0);
  const int iBX = 5;
  double volc = (sd == 3) ? dxc * dxc * dxc : dxc * dxc;
  double volf = (sd == 3) ? dxf * dxf * dxf : dxf * dxf;
  double refScale = 1.0;
  for (int d = 0; d < sd; ++d) refScale *= r;
  const double coeff = volc / (volf * refScale);
  for (int f = 0; f < nfp; ++f) {
    mf_box cfb = box_coarsen(vf[f], r, sd);
    mf_box wb = box_grow(cfb, cgr, sd);
    Fab Wk = fab_alloc(wb, nc), Sl[3];
    for (long q = 0; q < Wk.csz * nc; ++q) Wk.p[q] = -666.666;
    for (int d = 0; d < 3; ++d) {
      Sl[d] = fab_alloc(wb, nc);
      for (long q = 0; q < Sl[d].csz * nc; ++q) Sl[d].p[q] = -666.666;
    }
    /* timeInterp: coarse valid data (and periodic images) into the work box */
    FOR_BOX(wb, i, j, k) {
      int c[3] = {i, j, k};
      int b = find_box_wrapped(pc, ncp, vc, c);
      if (b < 0) continue;
      int w[3] = {i, j, k};
      wrap_cell(pc, w);
      Fab O = fab_wrap(Uold[b].data, Uold[b].box, nc), N = fab_wrap(Unew[b].data, Unew[b].box, nc);
      for (int q = 0; q < nc; ++q) {
        double vn = AT(&N, w[0], w[1], w[2], q), vo = AT(&O, w[0], w[1], w[2], q);
        double v;
        if (alpha == 1.0)
          v = vn;
        else if (alpha == 0.0)
          v = vo;
        else
          v = vn * alpha + vo * (1.0 - alpha);
        AT(&Wk, i, j, k, q) = v;
      }
    }
    /* coarse cells to interpolate from */
    mf_box ib = box_and_domain(box_coarsen(box_grow(vf[f], ng, sd), r, sd), pc);
    Fab In = fab_alloc(ib, 1);
    FOR_BOX(ib, i, j, k) {
      int c[3] = {i, j, k};
      AT(&In, i, j, k, 0) = covered_by_fine(pc, r, nfp, vf, c) ? 0.0 : 1.0;
    }
    /* slopes: centred where both neighbours are coarse valid cells, one-sided
       otherwise (computeSlopes, :585-760; the high-sided difference wins where
       both neighbours are missing) */
    for (int d = 0; d < sd; ++d) {
      int e[3] = {0, 0, 0};
      e[d] = 1;
      const double c1c = 0.5 / dxc, c1s = 1.0 / dxc;
      FOR_BOX(ib, i, j, k) {
        if (AT(&In, i, j, k, 0) == 0.0) continue;
        int cp[3] = {i + e[0], j + e[1], k + e[2]}, cm[3] = {i - e[0], j - e[1], k - e[2]};
        int hasp = find_box_wrapped(pc, ncp, vc, cp) >= 0;
        int hasm = find_box_wrapped(pc, ncp, vc, cm) >= 0;
        for (int q = 0; q < nc; ++q) {
          double s;
          double v0 = AT(&Wk, i, j, k, q);
          double vp = AT(&Wk, cp[0], cp[1], cp[2], q), vm = AT(&Wk, cm[0], cm[1], cm[2], q);
          if (!hasm)
            s = c1s * (vp - v0);
          else if (!hasp)
            s = c1s * (v0 - vm);
          else
            s = c1c * (vp - vm);
          AT(&Sl[d], i, j, k, q) = s;
        }
      }
    }
    /* limiting (INTERPLIMIT_V) away from non-periodic domain edges, then the
       divergence correction of the B slopes */
    FOR_BOX(ib, i, j, k) {
      if (AT(&In, i, j, k, 0) == 0.0) continue;
      int c[3] = {i, j, k}, edge = 0;
      for (int d = 0; d < sd; ++d)
        if (!pc->periodic[d] && (c[d] == pc->domain_lo[d] || c[d] == pc->domain_hi[d])) edge = 1;
      if (edge) continue;
      for (int q = 0; q < nc; ++q) {
        double s0 = AT(&Wk, i, j, k, q);
        double smax = s0, smin = s0;
        for (int kk = (sd == 3 ? -1 : 0); kk <= (sd == 3 ? 1 : 0); ++kk)
          for (int jj = -1; jj <= 1; ++jj)
            for (int ii = -1; ii <= 1; ++ii) {
              if (!box_in(&wb, i + ii, j + jj, k + kk)) continue;
              double v = AT(&Wk, i + ii, j + jj, k + kk, q);
              smax = fmax(smax, v);
              smin = fmin(smin, v);
            }
        double dsum = (sd == 3) ? 0.5 * (fabs(AT(&Sl[0], i, j, k, q) * dxc) +
                                         fabs(AT(&Sl[1], i, j, k, q) * dxc) +
                                         fabs(AT(&Sl[2], i, j, k, q) * dxc))
                                : 0.5 * (fabs(AT(&Sl[0], i, j, k, q) * dxc) +
                                         fabs(AT(&Sl[1], i, j, k, q) * dxc));
        double eta = fmin(smax - s0, s0 - smin);
        if (eta <= 1.0e-9 * fabs(smax))
          eta = 0.0;
        else if (dsum > eta)
          eta = eta / dsum;
        else
          eta = 1.0;
        for (int d = 0; d < sd; ++d) AT(&Sl[d], i, j, k, q) = eta * AT(&Sl[d], i, j, k, q);
      }
      if (divb)
        interp_divb0(sd, &AT(&Sl[0], i, j, k, iBX), &AT(&Sl[1], i, j, k, iBX + 1),
                     sd == 3 ? &AT(&Sl[2], i, j, k, iBX + 2) : NULL);
    }
    /* fine cells: constant part, then the linear term of each direction */
    mf_box fb = box_and_domain(box_grow(vf[f], ng, sd), pf);
    Fab U = fab_wrap(Uf[f].data, Uf[f].box, nc);
    FOR_BOX(fb, i, j, k) {
      int c[3] = {floordiv_(i, r), floordiv_(j, r), sd == 3 ? floordiv_(k, r) : k};
      if (!box_in(&ib, c[0], c[1], c[2]) || AT(&In, c[0], c[1], c[2], 0) == 0.0) continue;
      for (int q = 0; q < nc; ++q) AT(&U, i, j, k, q) = AT(&Wk, c[0], c[1], c[2], q);
    }
    for (int d = 0; d < sd; ++d) FOR_BOX(fb, i, j, k) {
        int iv[3] = {i, j, k};
        int c[3] = {floordiv_(i, r), floordiv_(j, r), sd == 3 ? floordiv_(k, r) : k};
        if (!box_in(&ib, c[0], c[1], c[2]) || AT(&In, c[0], c[1], c[2], 0) == 0.0) continue;
        double icoef = dxf * (iv[d] + 0.5) - dxc * (c[d] + 0.5);
        for (int q = 0; q < nc; ++q) {
          double slope = coeff * icoef * AT(&Sl[d], c[0], c[1], c[2], q);
          AT(&U, i, j, k, q) = AT(&U, i, j, k, q) + slope;
        }
      }
    fab_free(&In);
    fab_free(&Wk);
    for (int d = 0; d < 3; ++d) fab_free(&Sl[d]);
  }
  return MF_OK;
}

/* One face of a flux register (LevelFluxRegister between a coarse level and
   the next finer one): the coarse cell outside the fine region next to a
   fine patch's side, its coarse patch, and where the fine faces lie. */
typedef struct {
  int pc, cell[3]; /* coarse patch and the (wrapped) coarse cell */
  int d, side;     /* direction; side 0: cell below the fine region, 1: above */
  int fp, fnode;   /* fine patch, node index of the fine faces along d */
  int tlo[3];      /* fine cell index of the first fine face (other directions) */
} RegFace;

typedef struct {
  int n;
  RegFace* f;
  double* reg; /* n * nc */
} Register;

static int reg_build(const mf_params* pc, int r, int ncp, const mf_box* vc, int nfp,
                     const mf_box* vf, int nc, Register* R) {
  const int sd = pc->space_dim;
  int cap = 64;
  R->n = 0;
  R->f = (RegFace*)malloc(sizeof(RegFace) * (size_t)cap);
  R->reg = NULL;
  for (int f = 0; f < nfp; ++f) {
    mf_box cb = box_coarsen(vf[f], r, sd);
    for (int d = 0; d < sd; ++d)
      for (int side = 0; side < 2; ++side) {
        mf_box sb = cb;
        sb.lo[d] = sb.hi[d] = side ? cb.hi[d] + 1 : cb.lo[d] - 1;
        FOR_BOX(sb, i, j, k) {
          int c[3] = {i, j, k};
          int w[3] = {i, j, k};
          if (!wrap_cell(pc, w)) continue; /* physical boundary */
          if (covered_by_fine(pc, r, nfp, vf, c)) continue;
          int b = find_box_wrapped(pc, ncp, vc, c);
          if (b < 0) return MF_ERR_BAD_ARG; /* fine level not nested */
          if (R->n == cap) {
            cap *= 2;
            R->f = (RegFace*)realloc(R->f, sizeof(RegFace) * (size_t)cap);
          }
          RegFace* F = &R->f[R->n++];
          F->pc = b;
          memcpy(F->cell, w, sizeof(w));
          F->d = d;
          F->side = side;
          F->fp = f;
          F->fnode = side ? vf[f].hi[d] + 1 : vf[f].lo[d];
          for (int e = 0; e < 3; ++e) F->tlo[e] = (e < sd) ? c[e] * r : c[e];
        }
      }
  }
  R->reg = (double*)calloc((size_t)(R->n > 0 ? R->n : 1) * (size_t)nc, sizeof(double));
  return MF_OK;
}

/* incrementCoarse: the register of each face starts as -dt * coarse flux
   (updateState's flux: for RK2 the average of both stages). */
static void reg_set_coarse(Register* R, int nc, Fab* const* Fc /* [patch][d] */, double dt) {
  for (int n = 0; n < R->n; ++n) {
    const RegFace* F = &R->f[n];
    int node[3] = {F->cell[0], F->cell[1], F->cell[2]};
    if (F->side == 0) node[F->d] += 1; /* the cell's high face */
    for (int q = 0; q < nc; ++q) {
      double v = 0.0;
      v = v + (-dt) * AT(&Fc[F->pc][F->d], node[0], node[1], node[2], q);
      R->reg[(long)n * nc + q] = v;
    }
  }
}

/* incrementFine: add dt/r^(D-1) times every fine flux on the coarse face,
   the first transverse direction fastest. */
static void reg_add_fine(Register* R, int nc, int sd, int r, Fab* const* Ff, double dt) {
  double denom = 1.0;
  for (int e = 0; e < sd - 1; ++e) denom *= r;
  const double s = dt / denom;
  for (int n = 0; n < R->n; ++n) {
    const RegFace* F = &R->f[n];
    int t[2] = {0, 0}, nt = 0;
    for (int e = 0; e < sd; ++e)
      if (e != F->d) t[nt++] = e;
    const int n1 = (nt > 1) ? r : 1;
    for (int b = 0; b < n1; ++b)
      for (int a = 0; a < r; ++a) {
        int node[3] = {F->tlo[0], F->tlo[1], F->tlo[2]};
        node[F->d] = F->fnode;
        node[t[0]] += a;
        if (nt > 1) node[t[1]] += b;
        for (int q = 0; q < nc; ++q)
          R->reg[(long)n * nc + q] =
              R->reg[(long)n * nc + q] + s * AT(&Ff[F->fp][F->d], node[0], node[1], node[2], q);
      }
  }
}

/* reflux (scale -1 with the inverse cell size): per direction, the cells
   below the fine region first, then those above. */
static void reg_reflux(const Register* R, const mf_params* pc, int nc, mf_fab* Uc) {
  const double invdx = 1.0 / pc->dx;
  for (int d = 0; d < pc->space_dim; ++d)
    for (int side = 0; side < 2; ++side)
      for (int n = 0; n < R->n; ++n) {
        const RegFace* F = &R->f[n];
        if (F->d != d || F->side != side) continue;
        Fab U = fab_wrap(Uc[F->pc].data, Uc[F->pc].box, nc);
        for (int q = 0; q < nc; ++q) {
          double rg = R->reg[(long)n * nc + q];
          double* u = &AT(&U, F->cell[0], F->cell[1], F->cell[2], q);
          *u = side ? *u + invdx * rg : *u - invdx * rg;
        }
      }
}

/* CoarseAverageExt::averageToCoarse with AVERAGEWITHVOLUMES
   (src/CoarseAverageExt.cpp:117-192, src/CoarseAverageExtF.ChF:10-50). */
static int average_down(const mf_params* pc, const mf_params* pf, int r, int ncp, mf_fab* Uc,
                        const mf_box* vc, int nfp, mf_fab* Uf, const mf_box* vf) {
  const int sd = pc->space_dim, nc = Uc[0].ncomp;
  const double dxf = pf->dx;
  const double vol = (sd == 3) ? dxf * dxf * dxf : dxf * dxf;
  for (int f = 0; f < nfp; ++f) {
    mf_box cb = box_coarsen(vf[f], r, sd);
    Fab Fi = fab_wrap(Uf[f].data, Uf[f].box, nc);
    FOR_BOX(cb, i, j, k) {
      int c[3] = {i, j, k};
      int b = find_box_wrapped(pc, ncp, vc, c);
      if (b < 0) return MF_ERR_BAD_ARG;
      Fab C = fab_wrap(Uc[b].data, Uc[b].box, nc);
      const int rk = (sd == 3) ? r : 1;
      for (int q = 0; q < nc; ++q) {
        double sum = 0.0, volc = 0.0;
        for (int kk = 0; kk < rk; ++kk)
          for (int jj = 0; jj < r; ++jj)
            for (int ii = 0; ii < r; ++ii) {
              int fi = i * r + ii, fj = j * r + jj, fk = (sd == 3) ? k * r + kk : k;
              sum = sum + vol * AT(&Fi, fi, fj, fk, q);
              volc = volc + vol;
            }
        AT(&C, i, j, k, q) = sum / volc;
      }
    }
  }
  return MF_OK;
}

typedef struct {
  const mf_oracle_level* lev;
  int nlev;
  const int* ratio;
  int nthreads;
  mf_params* p;  /* per-level copies (GLM speeds updated during the step) */
  double* t;     /* level times */
  double* dt;    /* level steps */
  double* ndt;   /* per level: last new dt */
  mf_fab** old;  /* UOld per level (levels with a finer level) */
  Fab** F;       /* per level: npatch * 3 face-flux fabs */
  Register* reg; /* per pair (l, l+1) */
  int ng;
} Hier;

/* AMRLevelIdealMHD::advance of level l: UOld, preTimeStep's ghost
   interpolation (srcIdeal/AMRLevelIdealMHD.cpp:669-752), exchange, the
   patch updates with the register increments (:1248-1308), the level time
   and the GLM speeds of the base level (:1528-1548). */
static int hier_advance(Hier* H, int l) {
  const mf_oracle_level* L = &H->lev[l];
  const int nc = L->U[0].ncomp, sd = H->p[l].space_dim;
  int st = MF_OK;
  if (l + 1 < H->nlev)
    for (int b = 0; b < L->npatch; ++b) {
      Fab f = fab_wrap(L->U[b].data, L->U[b].box, nc);
      memcpy(H->old[l][b].data, L->U[b].data, sizeof(double) * (size_t)(f.csz * nc));
    }
  if (l > 0) {
    const int r = H->ratio[l - 1];
    double tNew = H->t[l - 1], tOld = tNew - H->dt[l - 1];
    double alpha = (H->t[l] - tOld) / (tNew - tOld);
    double eps = 0.04 * H->dt[l] / r;
    if (fabs(alpha) < eps) alpha = 0.0;
    if (fabs(1.0 - alpha) < eps) alpha = 1.0;
    if (alpha < 0.0 || alpha > 1.0) return MF_ERR_BAD_ARG;
    const mf_oracle_level* C = &H->lev[l - 1];
    st = cf_fill(&H->p[l - 1], &H->p[l], r, C->npatch, H->old[l - 1], C->U, C->valid,
                 L->npatch, L->U, L->valid, alpha, H->ng);
    if (st) return st;
  }
  st = mf_oracle_level_exchange(&H->p[l], L->npatch, L->U, L->valid);
  if (st) return st;
  double* dts = (double*)malloc(sizeof(double) * (size_t)L->npatch);
  int* sts = (int*)malloc(sizeof(int) * (size_t)L->npatch);
#ifdef _OPENMP
  int nth = H->nthreads > 0 ? H->nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(nth)
#endif
  for (int b = 0; b < L->npatch; ++b) {
    mf_fab Fo[3];
    for (int d = 0; d < 3; ++d) {
      Fo[d].data = H->F[l][3 * b + d].p;
      Fo[d].box = H->F[l][3 * b + d].b;
      Fo[d].ncomp = nc;
    }
    int cell[3];
    sts[b] = mf_oracle_patch_update(&H->p[l], H->t[l], &L->U[b], &L->valid[b], H->dt[l], Fo,
                                    NULL, &dts[b], cell);
  }
  double nd = 0.0;
  for (int b = 0; b < L->npatch; ++b) {
    if (sts[b]) st = sts[b];
    if (b == 0 || dts[b] < nd) nd = dts[b];
  }
  free(dts);
  free(sts);
  if (st) return st;
  st = neutral_sun_bc(&H->p[l], L->npatch, L->U, L->valid);
  if (st) return st;
  H->ndt[l] = nd;
  Fab** Fl = (Fab**)malloc(sizeof(Fab*) * (size_t)L->npatch);
  for (int b = 0; b < L->npatch; ++b) Fl[b] = &H->F[l][3 * b];
  const int ncons = nc - H->p[l].num_tracking_surfaces;
  if (l + 1 < H->nlev) reg_set_coarse(&H->reg[l], ncons, Fl, H->dt[l]);
  if (l > 0) reg_add_fine(&H->reg[l - 1], ncons, sd, H->ratio[l - 1], Fl, H->dt[l]);
  free(Fl);
  H->t[l] = H->t[l] + H->dt[l];
  if (l == 0 && H->p[0].divb_cleaning == 5 && H->p[0].factor_ch > 0.0) {
    double dx = H->p[0].dx;
    double Ch = H->p[0].factor_ch * dx / nd;
    double Cp = sqrt(Ch * dx / H->p[0].factor_cp);
    for (int q = 0; q < H->nlev; ++q) {
      H->p[q].dedner_ch = Ch;
      H->p[q].dedner_cp = Cp;
    }
  }
  return MF_OK;
}

/* AMR_MHDAM::timeStep (srcIdeal/AMR_MHDAM.cpp:1707-1880): advance, then the
   finer level ratio times, then postTimeStep (reflux, average down;
   srcIdeal/AMRLevelIdealMHD.cpp:1633-1646). */
static int hier_time_step(Hier* H, int l) {
  int st = hier_advance(H, l);
  if (st) return st;
  if (l + 1 < H->nlev) {
    for (int k = 0; k < H->ratio[l]; ++k) {
      st = hier_time_step(H, l + 1);
      if (st) return st;
    }
    const mf_oracle_level *C = &H->lev[l], *Fn = &H->lev[l + 1];
    reg_reflux(&H->reg[l], &H->p[l], C->U[0].ncomp - H->p[l].num_tracking_surfaces, C->U);
    st = average_down(&H->p[l], &H->p[l + 1], H->ratio[l], C->npatch, C->U, C->valid,
                      Fn->npatch, Fn->U, Fn->valid);
  }
  return st;
}

int mf_oracle_hier_step(int nlev, const mf_oracle_level* lev, const int* ratio, double* time,
                        double dt0, int nthreads, double* new_dt, double* dedner) {
  /* constrained transport across levels (edge registers, averageToCoarse of
     the accumulated edge field) is not restated */
  for (int l = 0; l < nlev; ++l)
    if (lev[l].p->divb_cleaning >= 1 && lev[l].p->divb_cleaning <= 3) return MF_ERR_UNSUPPORTED;
  if (nlev < 1 || !lev || (nlev > 1 && !ratio) || !time || !(dt0 > 0.0)) return MF_ERR_BAD_ARG;
  Hier H;
  memset(&H, 0, sizeof(H));
  H.lev = lev;
  H.nlev = nlev;
  H.ratio = ratio;
  H.nthreads = nthreads;
  H.p = (mf_params*)malloc(sizeof(mf_params) * (size_t)nlev);
  H.t = (double*)malloc(sizeof(double) * (size_t)nlev);
  H.dt = (double*)malloc(sizeof(double) * (size_t)nlev);
  H.ndt = (double*)malloc(sizeof(double) * (size_t)nlev);
  H.old = (mf_fab**)calloc((size_t)nlev, sizeof(mf_fab*));
  H.F = (Fab**)calloc((size_t)nlev, sizeof(Fab*));
  H.reg = (Register*)calloc((size_t)nlev, sizeof(Register));
  int st = MF_OK;
  for (int l = 0; l < nlev; ++l) {
    H.p[l] = *lev[l].p;
    H.t[l] = time[l];
    H.dt[l] = (l == 0) ? dt0 : H.dt[l - 1] / ratio[l - 1];
  }
  H.ng = num_ghost(lev[0].p);
  for (int l = 0; l < nlev && st == MF_OK; ++l) {
    const mf_oracle_level* L = &lev[l];
    const int nc = L->U[0].ncomp, sd = L->p->space_dim;
    H.F[l] = (Fab*)malloc(sizeof(Fab) * 3 * (size_t)L->npatch);
    for (int b = 0; b < L->npatch; ++b)
      for (int d = 0; d < 3; ++d)
        H.F[l][3 * b + d] = fab_alloc(box_nodes(L->valid[b], d < sd ? d : 0), nc);
    if (l + 1 < nlev) {
      H.old[l] = (mf_fab*)malloc(sizeof(mf_fab) * (size_t)L->npatch);
      for (int b = 0; b < L->npatch; ++b) {
        Fab f = fab_wrap(L->U[b].data, L->U[b].box, nc);
        H.old[l][b] = L->U[b];
        H.old[l][b].data = (double*)malloc(sizeof(double) * (size_t)(f.csz * nc));
      }
      /* the registers hold the fluid components (consInterval,
         srcIdeal/AMRLevelIdealMHD.cpp:1282-1305), not the tracking surfaces */
      st = reg_build(L->p, ratio[l], L->npatch, L->valid, lev[l + 1].npatch, lev[l + 1].valid,
                     nc - L->p->num_tracking_surfaces, &H.reg[l]);
    }
  }
  if (st == MF_OK) st = hier_time_step(&H, 0);
  if (st == MF_OK) {
    double m = 1.0, best = 0.0;
    for (int l = 0; l < nlev; ++l) {
      if (l > 0) m *= ratio[l - 1];
      double v = H.ndt[l] * m;
      if (l == 0 || v < best) best = v;
    }
    if (new_dt) *new_dt = best;
    for (int l = 0; l < nlev; ++l) time[l] = H.t[l];
    if (dedner) {
      dedner[0] = H.p[0].dedner_ch;
      dedner[1] = H.p[0].dedner_cp;
    }
  }
  for (int l = 0; l < nlev; ++l) {
    const mf_oracle_level* L = &lev[l];
    if (H.F[l]) {
      for (int q = 0; q < 3 * L->npatch; ++q) fab_free(&H.F[l][q]);
      free(H.F[l]);
    }
    if (H.old[l]) {
      for (int b = 0; b < L->npatch; ++b) free(H.old[l][b].data);
      free(H.old[l]);
    }
    free(H.reg[l].f);
    free(H.reg[l].reg);
  }
  free(H.p);
  free(H.t);
  free(H.dt);
  free(H.ndt);
  free(H.old);
  free(H.F);
  free(H.reg);
  return st;
}

int mf_oracle_cf_fill(const mf_params* pc, const mf_params* pf, int ratio, int ncoarse,
                      mf_fab* Uc_old, mf_fab* Uc_new, const mf_box* vc, int nfine, mf_fab* Uf,
                      const mf_box* vf, double alpha) {
  if (!pc || !pf || ratio < 2 || ncoarse < 1 || nfine < 1) return MF_ERR_BAD_ARG;
  return cf_fill(pc, pf, ratio, ncoarse, Uc_old, Uc_new, vc, nfine, Uf, vf, alpha,
                 num_ghost(pf));
}

int mf_oracle_average_down(const mf_params* pc, const mf_params* pf, int ratio, int ncoarse,
                           mf_fab* Uc, const mf_box* vc, int nfine, mf_fab* Uf,
                           const mf_box* vf) {
  if (!pc || !pf || ratio < 2 || ncoarse < 1 || nfine < 1) return MF_ERR_BAD_ARG;
  return average_down(pc, pf, ratio, ncoarse, Uc, vc, nfine, Uf, vf);
}
