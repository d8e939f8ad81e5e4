// mf_device.cuh - device-side physics of the multi-fluid MHD patch update.
//
// Every routine restates one reference kernel (paths inside MHDAM-3.2.4).  The
// arithmetic keeps the reference's evaluation order for each non-zero term; the
// Roe solvers skip the structurally zero entries of their 8x8 eigenmatrices,
// which changes no result (x + 0*y == x for finite y).
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/mf_patch.h"

namespace mf {

constexpr double kInv4Pi = 0.079577471545947667884441881686257181;   // d_1_4PI
constexpr double kInv8Pi = 0.039788735772973833942220940843128591;   // d_1_8PI
constexpr double kSqrtHalf = 0.707106781186547524400844362104849039; // d_SQRT_2
constexpr double kPi = 3.14159265358979323846264338327950288;
constexpr double k2Pi = 6.28318530717958647692528676655900576;
// srcIdeal/EosCommon.fh:31-37
constexpr double kNet2Dens = 1.0e-6, kNet2Pres = 1.0e-8;
constexpr double kNet3Dens = 1.0e-7, kNet3Pres = 1.0e-9;

enum RsKind : int { kRoe8 = 0, kRoe7 = 1, kRusanov = 2, kVFRoe = 3 };

// Parameters as the kernels see them (mf_params + derived constants).
struct DevParams {
  int sd, nf, glm, nc, irhon;
  int rs, aver;
  int use8, divb_method, check_pos, ce, reinit, bc_kind;
  int char_rec, check_tvd;
  int helio_bc;  // HELIOBC fluxes on the faces of the domain boundary
  // tracking surfaces: components [ils, nc) after the fluids (ils = number of
  // fluid components), limiter lim_ls; reg_tracer: the last one is the
  // region tracer, lism_u the interstellar flow direction
  int ils, nls, lim_ls, reg_tracer;
  int ct;  // constrained transport: 0 off, 1 Balsara-Spicer, 2 / 3 Gardiner-Stone (2D)
  int ce32;  // mixed precision with FP32 charge-exchange rates (MF_PREC_MIXED_CE32)
  // inner-sphere field: 1 monopolar, 0 bipolar; ihcs: component of the
  // current-sheet surface set by the bipolar reset (-1: none)
  int monopolar, ihcs;
  int lim[8];
  int periodic[3], dlo[3], dhi[3];
  double gamma, hgamma, invhgamma, invgamma, smallr, smallp, del2, smallB, dx, invdx;
  double factor_ch, factor_cp;
  double ce_scale_vel, ce_sigma_scale, ce_a, ce_b, ce_damp_c, ce_damp_pow;
  double sun_c[3], sun_r, sun_v, t_coeff, tmlim, zbot, ztop;
  double r0, rint, sun_rho, sun_p, sun_b, sun_beta, dir_br;
  double sin_tilt, cos_tilt;  // sin / cos of the current-sheet tilt (radians)
  double max_growth;          // assignDt growth cap of chained time steps (<= 0: none)
  double bc_plasma[8], bc_n1[5];
  double lism_u[3];
};

// Values that change from step to step; kept in device memory so that a
// captured CUDA graph reads the current ones.
struct StepState {
  double dt;        // time step of the step being taken
  double time;      // start time of the step being taken (advanced by dt after it)
  double ch, cp;    // GLM speeds
  double cfl;       // dt of the next async step = cfl * dt_min
  double dt_min;    // result: minimum of dx/cmax
  int min_desc;     // result: patch index of the minimum
  int min_idx;      // result: Fortran-order index inside the valid box
  unsigned flags;   // error bits (kFlag*)
  int pad;
};

// Problem time of a stage's post-processing: HeliosphericProblem::postprocessing
// is called with the step's start time and the stage's dt and works at their
// sum (swlism/HeliosphericProblem.cpp:2399-2405).
__device__ __forceinline__ double stage_time(const StepState& ss, double dt_stage) {
  return ss.time + dt_stage;
}

// Values that differ between the runs of one batch (independent simulations,
// or AMR levels, stepped in shared launches): grid spacing, domain extent in
// cells, far-field state, and where the run's items sit in the launch.
struct RunParams {
  double dx, invdx;
  int dlo[3], dhi[3];
  double bc_plasma[8], bc_n1[5];
  int d0, nd;    // first desc of the run and number of descs
  int v0, v1;    // flattened valueBox-cell range [v0, v1); v0 is a multiple of kRunAlign
  int pad;
};

// Alignment of every run's valueBox-cell range in a flattened launch: no
// block of the update or dt kernel (<= 256 threads) holds cells of two runs,
// so block partials of the dt reduction belong to one run.
constexpr int kRunAlign = 256;

constexpr unsigned kFlagNonFinite = 1u;
constexpr unsigned kFlagBadDt = 2u;

// A patch as seen by one stage.
struct StageDesc {
  long long u_off;        // offset (doubles) of the fab in U / W / Uold buffers
  long long f_off[3];     // offset (elements) of the face-flux fab of each direction
  long long bn_off[3];    // offset (elements) of the Bn fab of each direction
  int flo[3], fn[3];      // fab box lo and extents (U, W)
  int vlo[3], vn[3];      // valueBox lo and extents
  int wlo[3], wn[3];      // box on which W is computed
  // first index of this patch's items in a flattened launch over a batch:
  // [kRegW] cells of the W box, [kRegF + d] faces in direction d,
  // [kRegV] cells of the valueBox, [kRegS] cells of the slope box.
  // Ascending over the batch.
  int g0[6];              // [kRegS]: cells of the slope box (Hancock)
  int run;                // index of the run (RunParams / StepState) of this patch
  // Hancock: the predictor's slope box (valueBox.grow(1)) and the offsets
  // (doubles) of the patch's face-value arrays (low then high face value of
  // every primitive component per cell of the slope box), per direction.
  int slo[3], sn[3];
  long long fv_off[3];
};

// Plasma state and current-sheet surface value of the inner-sphere reset.
// The parameters of the inner-sphere reset, copied out of DevParams so that
// the out-of-line reset takes them by value (a kernel parameter passed by
// reference to a function that is not inlined would be copied into every
// thread's local memory).
struct ReinitIn {
  double rint, sun_rho, sun_v, sun_p, gamma, hgamma, dir_br, sun_b, sun_beta;
  double sin_tilt, cos_tilt;
  int monopolar;
};

__device__ __host__ __forceinline__ ReinitIn reinit_in(const DevParams& P) {
  ReinitIn r;
  r.rint = P.rint;
  r.sun_rho = P.sun_rho;
  r.sun_v = P.sun_v;
  r.sun_p = P.sun_p;
  r.gamma = P.gamma;
  r.hgamma = P.hgamma;
  r.dir_br = P.dir_br;
  r.sun_b = P.sun_b;
  r.sun_beta = P.sun_beta;
  r.sin_tilt = P.sin_tilt;
  r.cos_tilt = P.cos_tilt;
  r.monopolar = P.monopolar;
  return r;
}

// sin and cos of a phase through sincospi(phase / pi) on the device (exact
// argument reduction, no out-of-line slow path); sin / cos on the host.
__device__ __host__ __forceinline__ void reinit_sincos(double ph, double& sn, double& cs) {
#ifdef __CUDA_ARCH__
  sincospi(ph / kPi, &sn, &cs);
#else
  sn = std::sin(ph);
  cs = std::cos(ph);
#endif
}

struct ReinitState {
  double u[8];
  double hcs;
};

// Per-block partial of the dt reduction.
struct DtPartial {
  double dt;
  int desc;
  int idx;
};

// ---------------------------------------------------------------------------
// small helpers
// ---------------------------------------------------------------------------
template <typename R> __device__ __forceinline__ R rmax(R a, R b) { return fmax(a, b); }
template <typename R> __device__ __forceinline__ R rmin(R a, R b) { return fmin(a, b); }
template <typename R> __device__ __forceinline__ R rabs(R a) { return fabs(a); }
template <typename R> __device__ __forceinline__ R sqrt_r(R a) { return sqrt(a); }

// ---------------------------------------------------------------------------
// VFRoe MHD flux: VFROE_FLUXES (src/VFRoeF.ChF:327-658) with arithmetic
// averaging, the form RiemannSolver::make builds for flux 5
// (src/RiemannSolver.cpp:69-74).  The middle state of the linearised Riemann
// problem (each wave strength times sign(1/2, eigenvalue)) and the exact MHD
// flux of that state, in the Fortran's order of operations.  wl/wr: rho, u,
// v, w, p, bx, by, bz in the global frame; g: fluxes in the same order.  One
// template for every precision mode: the translation unit's contraction
// flags decide whether products fuse.
// ---------------------------------------------------------------------------
template <typename R, int DIR>
__device__ __forceinline__ void vfroe_mhd(const DevParams& P, const R* wl, const R* wr, R* g) {
  constexpr int in = 1 + DIR, it1 = 1 + (DIR + 1) % 3, it2 = 1 + (DIR + 2) % 3;
  constexpr int inB = 5 + DIR, it1B = 5 + (DIR + 1) % 3, it2B = 5 + (DIR + 2) % 3;
  const R gamma = R(P.gamma), hgamma = R(P.hgamma);
  const R i4pi = R(kInv4Pi), i8pi = R(kInv8Pi), sq2 = R(kSqrtHalf), pi = R(kPi);
  const R PGasL = rmax<R>(R(P.smallp), wl[4]), RhoL = rmax<R>(R(P.smallr), wl[0]);
  const R UL = wl[in], VL = wl[it1], WL = wl[it2], BXL = wl[inB], BYL = wl[it1B], BZL = wl[it2B];
  const R PGasR = rmax<R>(R(P.smallp), wr[4]), RhoR = rmax<R>(R(P.smallr), wr[0]);
  const R UR = wr[in], VR = wr[it1], WR = wr[it2], BXR = wr[inB], BYR = wr[it1B], BZR = wr[it2B];
  // average state
  const R Rho = R(0.5) * (RhoL + RhoR);
  const R U = R(0.5) * (UL + UR);
  const R BX = R(0.5) * (BXL + BXR), BY = R(0.5) * (BYL + BYR), BZ = R(0.5) * (BZL + BZR);
  const R PGas = R(0.5) * (PGasL + PGasR);
  const R BX2 = BX * BX, BY2 = BY * BY, BZ2 = BZ * BZ;
  const R BYZ2 = BY2 + BZ2;
  const R BxBH = i8pi * (BX2 + BYZ2);
  const R cc = gamma * PGas / Rho;
  const R bb = i4pi * BX2 / Rho;
  const R szb = cc + (BxBH + BxBH) / Rho;
  const R h = sqrt_r<R>(szb * szb - R(4) * cc * bb);
  const R aaf = R(0.5) * (szb + h);
  const R aas = cc * bb / aaf;
  const R b = sqrt_r<R>(bb), c = sqrt_r<R>(cc), af = sqrt_r<R>(aaf), as = sqrt_r<R>(aas);
  const R eig[9] = {R(0), U, U, U + b, U - b, U + af, U - af, U + as, U - as};
  // alphas
  R alphaF, alphaS;
  const R dfs = aaf - aas;
  if (dfs < R(1.0e-12)) {
    alphaF = R(1);
    alphaS = R(0);
  } else if ((cc - aas) <= R(0)) {
    alphaF = R(0);
    alphaS = R(1);
  } else if ((aaf - cc) <= R(0)) {
    alphaF = R(1);
    alphaS = R(0);
  } else {
    alphaF = sqrt_r<R>((cc - aas) / dfs);
    alphaS = sqrt_r<R>((aaf - cc) / dfs);
  }
  R betaY, betaZ;
  if (BYZ2 < R(P.smallB) * R(P.smallB)) {
    betaY = sq2;
    betaZ = sq2;
  } else {
    const R hyz = sqrt_r<R>(BYZ2);
    betaY = BY / hyz;
    betaZ = BZ / hyz;
  }
  const R siBX = copysign(R(1), BX);
  R betaYX = betaY, betaZX = betaZ;
  if (BX < R(0)) {
    betaYX = -betaY;
    betaZX = -betaZ;
  }
  const R dP = PGasR - PGasL, dRho = RhoR - RhoL, dUn = UR - UL, dUt1 = VR - VL, dUt2 = WR - WL;
  const R dBt1 = BYR - BYL, dBt2 = BZR - BZL;
  R a[9];
  a[0] = R(0);
  a[1] = dRho - dP / cc;
  a[2] = BXR - BXL;
  R h1 = sq2 * (betaY * dUt2 - betaZ * dUt1);
  R h2 = siBX * (betaZ * dBt1 - betaY * dBt2) / (R(2) * sqrt_r<R>(R(2) * pi * Rho));
  a[3] = h1 + h2;
  a[4] = h1 - h2;
  h1 = dP / (R(2) * Rho * cc);
  h2 = dUn / (R(2) * cc);
  const R h3 = (betaY * dBt1 + betaZ * dBt2) / (R(4) * c * sqrt_r<R>(pi * Rho));
  const R h4 = siBX * (betaY * dUt1 + betaZ * dUt2) / (R(2) * cc);
  a[5] = alphaF * (h1 + af * h2) + alphaS * (h3 - as * h4);
  a[6] = alphaF * (h1 - af * h2) + alphaS * (h3 + as * h4);
  a[7] = alphaS * (h1 + as * h2) - alphaF * (h3 - af * h4);
  a[8] = alphaS * (h1 - as * h2) - alphaF * (h3 + af * h4);
  // middle state
#pragma unroll
  for (int q = 1; q <= 8; ++q) a[q] = (eig[q] == R(0)) ? R(0) : a[q] * copysign(R(0.5), eig[q]);
  a[3] = sq2 * a[3];
  a[4] = sq2 * a[4];
  const R a34p = a[3] + a[4], a34m = a[3] - a[4];
  const R a56p = a[5] + a[6], a56m = a[5] - a[6];
  const R a78p = a[7] + a[8], a78m = a[7] - a[8];
  const R DN = R(2) * sqrt_r<R>(pi * Rho);
  const R HRho = Rho * (alphaF * a56p + alphaS * a78p);
  const R HU = alphaS * as * a56m - alphaF * af * a78m;
  const R HB = c * (alphaS * a56p - alphaF * a78p);
  const R RhoM = R(0.5) * (RhoR + RhoL) - (a[1] + HRho);
  const R UM = R(0.5) * (UR + UL) - (alphaF * af * a56m + alphaS * as * a78m);
  const R VM = R(0.5) * (VR + VL) + (betaZ * a34p + betaYX * HU);
  const R WM = R(0.5) * (WR + WL) - (betaY * a34p - betaZX * HU);
  const R PGasM = R(0.5) * (PGasR + PGasL) - cc * HRho;
  const R BXM = R(0.5) * (BXR + BXL);
  const R BYM = R(0.5) * (BYR + BYL) - DN * (betaZX * a34m + betaY * HB);
  const R BZM = R(0.5) * (BZR + BZL) - DN * (-betaYX * a34m + betaZ * HB);
  const R BxBM = i8pi * (BXM * BXM + BYM * BYM + BZM * BZM);
  const R kk = R(0.5) * (UM * UM + VM * VM + WM * WM);
  const R HUM = BXM * UM + BYM * VM + BZM * WM;
  R E = PGasM / hgamma + RhoM * kk;
  const R Pt = PGasM + BxBM;
  E = E + BxBM;
  g[0] = RhoM * UM;
  g[in] = RhoM * UM * UM + Pt - i4pi * BXM * BXM;
  g[it1] = RhoM * UM * VM - i4pi * BXM * BYM;
  g[it2] = RhoM * UM * WM - i4pi * BXM * BZM;
  g[4] = UM * (E + Pt) - i4pi * BXM * HUM;
  g[inB] = R(0);
  g[it1B] = UM * BYM - VM * BXM;
  g[it2B] = UM * BZM - WM * BXM;
}

// ---------------------------------------------------------------------------
// conserved -> primitive: CONSTOPRIM (srcIdeal/PatchIdealMHDF.ChF:143-189),
// CONSTOPRIM_MF (srcIdeal/PatchMHDMFF.ChF:5-80), psi copy (EqSysMHDMF.cpp:198-201)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cons_to_prim_plasma(const DevParams& P, const double* u,
                                                    double* w) {
  double rho = (P.nf == 1) ? u[0] : fmax(u[0], P.smallr);
  double ru = u[1], rv = u[2], rw = u[3];
  double invrho = 1.0 / rho;
  double uu = ru * invrho, vv = rv * invrho, ww = rw * invrho;
  double ke = ru * uu + rv * vv + rw * ww;
  double bx = u[5], by = u[6], bz = u[7];
  double b = kInv4Pi * (bx * bx + by * by + bz * bz);
  double p = P.hgamma * (u[4] - 0.5 * (ke + b));
  p = fmax(p, P.smallp);
  w[0] = rho; w[1] = uu; w[2] = vv; w[3] = ww; w[4] = p;
  w[5] = bx; w[6] = by; w[7] = bz;
}

__device__ __forceinline__ void cons_to_prim_euler(const DevParams& P, const double* u,
                                                   double* w) {
  double rho = fmax(u[0], P.smallr);
  double ru = u[1], rv = u[2], rw = u[3];
  double invrho = 1.0 / rho;
  double uu = ru * invrho, vv = rv * invrho, ww = rw * invrho;
  double ke = ru * uu + rv * vv + rw * ww;
  double p = P.hgamma * (u[4] - 0.5 * ke);
  p = fmax(p, P.smallp);
  w[0] = rho; w[1] = uu; w[2] = vv; w[3] = ww; w[4] = p;
}

// ---------------------------------------------------------------------------
// limited face values (src/reconstructionF.ChF, every limiter of
// limiter1D::make, src/limiter1D.cpp:21-63): returns the value on the low
// face (lo) and on the high face (hi) of the centre cell
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R minmod_(R A, R B) {  // reconstructionF.ChF:5-13
  R signA = copysign(R(1), A);
  return signA * rmax<R>(R(0), rmin<R>(rabs<R>(A), signA * B));
}

template <typename R>
__device__ __forceinline__ void face_values(int lim, R wm1, R wp, R wp1, R& lo, R& hi) {
  R dWR = wp1 - wp;
  R dWL = wp - wm1;
  R slope;
  switch (lim) {
    case MF_LIM_CD:  // CDFACEVALUES :1056-1079
      lo = R(0.5) * (wp + wp1);
      hi = R(0.5) * (wp + wm1);
      return;
    case MF_LIM_SUPERBEE: {  // :258-301
      if (dWL * dWR <= R(0)) { lo = wp; hi = wp; return; }
      R AR = rabs<R>(dWR), AL = rabs<R>(dWL);
      if (AL <= R(0.5) * AR) slope = dWL;
      else if (AL <= AR) slope = R(0.5) * dWR;
      else if (AL <= AR + AR) slope = R(0.5) * dWL;
      else slope = dWR;
      break;
    }
    case MF_LIM_VANALBADA: {  // :550-589
      const R dSave = R(1.0e-6), dSaveS = dSave + dSave;
      if (dWL * dWR <= R(0)) { lo = wp; hi = wp; return; }
      slope = R(0.5) * (dWR * dWL + dSave) * (dWR + dWL) / (dWR * dWR + dWL * dWL + dSaveS);
      break;
    }
    case MF_LIM_MC: {  // :622-661
      if (dWL * dWR <= R(0)) { lo = wp; hi = wp; return; }
      R AR = rabs<R>(dWR), AL = rabs<R>(dWL);
      if (R(3) * AL <= AR) slope = dWL;
      else if (AL <= R(3) * AR) slope = R(0.25) * (dWR + dWL);
      else slope = dWR;
      break;
    }
    case MF_LIM_HARMONIC: {  // :492-524
      if (dWL * dWR <= R(0)) { lo = wp; hi = wp; return; }
      slope = dWR / (R(1) + dWR / dWL);
      break;
    }
    case MF_LIM_HYPERBEE: {  // :430-464
      if (dWL * dWR <= R(0)) { lo = wp; hi = wp; return; }
      const R A = R(1) + sqrt_r<R>(dWR / dWL);
      slope = dWR / (A * A);
      slope = slope + slope;
      break;
    }
    case MF_LIM_KOREN: {  // :883-918
      const R dSave = R(1.0e-10);
      if (dWL * dWR <= R(0)) { lo = wp; hi = wp; return; }
      const R H = dWL * dWR / (R(2) * (dWL * dWL + dWR * dWR + dSave) - dWL * dWR);
      lo = wp - (dWL + R(0.5) * dWR) * H;
      hi = wp + (dWR + R(0.5) * dWL) * H;
      return;
    }
    case MF_LIM_VENKATAKRISHNAN: {  // :950-988
      const R dSave = R(1.0e-10), dSave2 = R(1.0e-10 * 1.0e-10);
      if (dWL * dWR <= R(0)) { lo = wp; hi = wp; return; }
      const R H = (dWR + dWL) / (R(6) * (dWR * dWR + dWL * dWL + dSave2));
      lo = wp - (dWR + R(2) * dWL) * (dWL + dSave) * H;
      hi = wp + (dWL + R(2) * dWR) * (dWR + dSave) * H;
      return;
    }
    case MF_LIM_WENO3: {  // :1096-1136
      const R dSave = R(1.0e-6);
      const R BR = dWR * dWR + dSave, AR = R(1) / (BR * BR);
      const R BL = dWL * dWL + dSave, AL = R(1) / (BL * BL);
      R H = AR / (AR + R(2) * AL);
      lo = wp - R(0.5) * (dWL + H * (dWR - dWL));
      H = AL / (AL + R(2) * AR);
      hi = wp + R(0.5) * (dWR - H * (dWR - dWL));
      return;
    }
    case MF_LIM_WENO3YC: {  // :1169-1212
      const R dSave = R(1.0e-6);
      const R BR = dWR * dWR + dSave, BL = dWL * dWL + dSave;
      R D2P = dWR - dWL;
      D2P = D2P * D2P;
      const R AL = R(1) + D2P / BL, AR = R(1) + D2P / BR;
      R H = AR / (AR + R(2) * AL);
      lo = wp - R(0.5) * (dWL + H * (dWR - dWL));
      H = AL / (AL + R(2) * AR);
      hi = wp + R(0.5) * (dWR - H * (dWR - dWL));
      return;
    }
    case MF_LIM_VANLEER: {  // :794-841
      const R dSLim = R(1.0 / 3.0);
      const R BT = (R(3) - dSLim) / (R(1) - dSLim);
      const R SL1 = R(0.25) * (R(1) - dSLim);
      const R SL2 = R(0.25) * (R(1) + dSLim);
      if (dWL * dWR <= R(0)) { lo = wp; hi = wp; return; }
      R SL = rmin<R>(rabs<R>(dWR), rabs<R>(BT * dWL));
      R SR = rmin<R>(rabs<R>(dWL), rabs<R>(BT * dWR));
      R sl = SL1 * SL + SL2 * SR;
      R sr = SL1 * SR + SL2 * SL;
      if (dWR < R(0)) { sl = -sl; sr = -sr; }
      lo = wp - sl;
      hi = wp + sr;
      return;
    }
    default:  // MINMODFACEVALUES :126-155
      slope = R(0.5) * minmod_<R>(dWR, dWL);
      break;
  }
  lo = wp - slope;
  hi = wp + slope;
}

}  // namespace mf

namespace mf {

// ---------------------------------------------------------------------------
// characteristic reconstruction (Reconstruction::faceValues with
// isCharactistic(), src/Reconstruction.cpp:178-203)
// ---------------------------------------------------------------------------
template <typename R>
__device__ __forceinline__ R minmod3_(R A, R B, R C) {  // reconstructionF.ChF:15-22
  R signA = copysign(R(1), A);
  return signA * rmax<R>(R(0), rmin<R>(rabs<R>(A), rmin<R>(signA * B, signA * C)));
}

// *FACESLOPES of one variable (reconstructionF.ChF: MINMOD :157-178,
// SUPERBEE :356-392, HYPERBEE :466-490, HARMONIC :526-550, VANALBADA
// :591-622, MC :664-697, VANLEER :843-880, KOREN :920-948, VENKATAKRISHNAN
// :990-1021, CD :1081-1096, WENO3 :1138-1167, WENO3YC :1214-1246):
// Sleft/Sright in = left/right differences, out = limited slopes.
template <typename R>
__device__ __forceinline__ void face_slopes(int lim, R& Sleft, R& Sright) {
  const R dSR = Sright, dSL = Sleft;
  R SLOPE = R(0);
  switch (lim) {
    case MF_LIM_CD:
      Sleft = R(0.5) * Sleft;
      Sright = R(0.5) * Sright;
      return;
    case MF_LIM_SUPERBEE:
      if (dSL * dSR > R(0)) {
        const R AR = rabs<R>(dSR), AL = rabs<R>(dSL);
        if (AL <= R(0.5) * AR) SLOPE = dSL;
        else if (AL <= AR) SLOPE = R(0.5) * dSR;
        else if (AL <= AR + AR) SLOPE = R(0.5) * dSL;
        else SLOPE = dSR;
      }
      break;
    case MF_LIM_HARMONIC:
      if (dSL * dSR > R(0)) SLOPE = dSR * dSL / (dSL + dSR);
      break;
    case MF_LIM_VANALBADA: {
      const R dSave = R(1.0e-6), dSaveS = dSave + dSave;
      if (dSL * dSR > R(0))
        SLOPE = R(0.5) * (dSR * dSL + dSave) * (dSR + dSL) / (dSR * dSR + dSL * dSL + dSaveS);
      break;
    }
    case MF_LIM_MC:
      if (dSL * dSR > R(0)) {
        const R AR = rabs<R>(dSR), AL = rabs<R>(dSL);
        if (R(3) * AL <= AR) SLOPE = dSL;
        else if (AL <= R(3) * AR) SLOPE = R(0.25) * (dSR + dSL);
        else SLOPE = dSR;
      }
      break;
    case MF_LIM_HYPERBEE:  // :466-490
      if (dSL * dSR > R(0)) {
        const R A = R(1) + sqrt_r<R>(dSR / dSL);
        SLOPE = dSR / (A * A);
        SLOPE = SLOPE + SLOPE;
      }
      break;
    case MF_LIM_KOREN: {  // :920-948
      const R dSave = R(1.0e-10);
      R SLOPL = R(0), SLOPR = R(0);
      if (dSL * dSR > R(0)) {
        const R H = dSL * dSR / (R(2) * (dSL * dSL + dSR * dSR + dSave) - dSL * dSR);
        SLOPL = (dSL + R(0.5) * dSR) * H;
        SLOPR = (dSR + R(0.5) * dSL) * H;
      }
      Sleft = SLOPL;
      Sright = SLOPR;
      return;
    }
    case MF_LIM_VENKATAKRISHNAN: {  // :990-1021
      const R dSave = R(1.0e-10), dSave2 = R(1.0e-10 * 1.0e-10);
      R SLOPL = R(0), SLOPR = R(0);
      if (dSL * dSR > R(0)) {
        const R H = (dSR + dSL) / (R(6) * (dSR * dSR + dSL * dSL + dSave2));
        SLOPL = (dSR + R(2) * dSL) * (dSL + dSave) * H;
        SLOPR = (dSL + R(2) * dSR) * (dSR + dSave) * H;
      }
      Sleft = SLOPL;
      Sright = SLOPR;
      return;
    }
    case MF_LIM_WENO3: {  // :1138-1167
      const R dSave = R(1.0e-6);
      const R BR = dSR * dSR + dSave, AR = R(1) / (BR * BR);
      const R BL = dSL * dSL + dSave, AL = R(1) / (BL * BL);
      R H = AR / (AR + R(2) * AL);
      Sleft = R(0.5) * (dSL + H * (dSR - dSL));
      H = AL / (AL + R(2) * AR);
      Sright = R(0.5) * (dSR - H * (dSR - dSL));
      return;
    }
    case MF_LIM_WENO3YC: {  // :1214-1246
      const R dSave = R(1.0e-6);
      const R BR = dSR * dSR + dSave, BL = dSL * dSL + dSave;
      R D2P = dSR - dSL;
      D2P = D2P * D2P;
      const R AL = R(1) + D2P / BL, AR = R(1) + D2P / BR;
      R H = AR / (AR + R(2) * AL);
      Sleft = R(0.5) * (dSL + H * (dSR - dSL));
      H = AL / (AL + R(2) * AR);
      Sright = R(0.5) * (dSR - H * (dSR - dSL));
      return;
    }
    case MF_LIM_VANLEER: {
      const R dSLim = R(1.0 / 3.0);
      const R BT = (R(3) - dSLim) / (R(1) - dSLim);
      const R SL1 = R(0.25) * (R(1) - dSLim);
      const R SL2 = R(0.25) * (R(1) + dSLim);
      R SLOPL = R(0), SLOPR = R(0);
      if (dSL * dSR > R(0)) {
        const R SL = rmin<R>(rabs<R>(dSR), rabs<R>(BT * dSL));
        const R SR = rmin<R>(rabs<R>(dSL), rabs<R>(BT * dSR));
        SLOPL = SL1 * SL + SL2 * SR;
        SLOPR = SL1 * SR + SL2 * SL;
        if (dSR < R(0)) {
          SLOPL = -SLOPL;
          SLOPR = -SLOPR;
        }
      }
      Sleft = SLOPL;
      Sright = SLOPR;
      return;
    }
    default:
      SLOPE = R(0.5) * minmod_<R>(dSR, dSL);
      break;
  }
  Sleft = SLOPE;
  Sright = SLOPE;
}

// Face values of a tracking surface from the cell values a, b, c (b the
// cell): the *FACEVALUES form with limiter_LS, or with characteristic
// reconstruction INITIALSLOPES + *FACESLOPES (the surfaces are not projected;
// src/Reconstruction.cpp:178-203).
template <typename R>
__device__ __forceinline__ void ls_face_values(const DevParams& P, R a, R b, R c, R& lo, R& hi) {
  if (P.char_rec) {
    R SL = b - a, SR = c - b;
    face_slopes<R>(P.lim_ls, SL, SR);
    lo = b - SL;
    hi = b + SR;
  } else {
    face_values<R>(P.lim_ls, a, b, c, lo, hi);
  }
}

// Wave speeds and mixing coefficients at a cell state, as CHARANALYSISF
// (srcIdeal/PatchIdealMHDF.ChF:1167-1328, dfs cut-off 1e-12) and
// CHARSYNTHESISF (:1330-1500, cut-off 1e-8) compute them.
struct CharState {
  double Rho, cc, c, as, af, alphaF, alphaS, betaY, betaZ, BX;
};

template <int D>
__device__ __forceinline__ void char_state(const DevParams& P, const double* w, double dfs_cut,
                                           CharState& s) {
  constexpr int inB = 5 + D, itB1 = 5 + (D + 1) % 3, itB2 = 5 + (D + 2) % 3;
  const double PGas = fmax(P.smallp, w[4]);
  const double Rho = fmax(P.smallr, w[0]);
  const double BX = w[inB], BY = w[itB1], BZ = w[itB2];
  const double cc = P.gamma * PGas / Rho;
  const double cs = sqrt(cc);
  const double BX2 = BX * BX, BY2 = BY * BY, BZ2 = BZ * BZ;
  const double BYZ2 = BY2 + BZ2;
  const double BxBH = kInv8Pi * (BX2 + BYZ2);
  const double bb = kInv4Pi * BX2 / Rho;
  const double b = sqrt(bb);
  double betaY, betaZ, aaf, aas, af, as;
  if (BYZ2 < P.smallB * P.smallB) {
    betaY = kSqrtHalf;
    betaZ = kSqrtHalf;
    if (bb > cc) { aaf = bb; aas = cc; af = b; as = cs; }
    else { aaf = cc; aas = bb; af = cs; as = b; }
  } else {
    const double hyz = sqrt(BYZ2);
    betaY = BY / hyz;
    betaZ = BZ / hyz;
    const double szb = cc + (BxBH + BxBH) / Rho;
    const double h = sqrt(szb * szb - 4.0 * cc * bb);
    aas = 0.5 * (szb - h);
    as = sqrt(aas);
    aaf = 0.5 * (szb + h);
    af = sqrt(aaf);
  }
  const double dfs = aaf - aas;
  double alphaF, alphaS;
  if (dfs < dfs_cut) { alphaF = 1.0; alphaS = 0.0; }
  else if ((cc - aas) <= 0.0) { alphaF = 0.0; alphaS = 1.0; }
  else if ((aaf - cc) <= 0.0) { alphaF = 1.0; alphaS = 0.0; }
  else {
    alphaF = sqrt((cc - aas) / dfs);
    alphaS = sqrt((aaf - cc) / dfs);
  }
  s.Rho = Rho; s.cc = cc; s.c = cs; s.as = as; s.af = af;
  s.alphaF = alphaF; s.alphaS = alphaS; s.betaY = betaY; s.betaZ = betaZ; s.BX = BX;
}

// CHARANALYSISF on one slope vector (plasma primitives), in place.
template <int D>
__device__ __forceinline__ void char_analysis(const CharState& s, double* dW) {
  constexpr int in = 1 + D, it1 = 1 + (D + 1) % 3, it2 = 1 + (D + 2) % 3;
  constexpr int inB = 5 + D, itB1 = 5 + (D + 1) % 3, itB2 = 5 + (D + 2) % 3;
  const double siBX = copysign(1.0, s.BX);
  const double dP = dW[4], dRho = dW[0], dUn = dW[in], dUt1 = dW[it1], dUt2 = dW[it2];
  const double dBn = dW[inB], dBt1 = dW[itB1], dBt2 = dW[itB2];
  const double Rho = s.Rho, cc = s.cc, betaY = s.betaY, betaZ = s.betaZ;
  dW[0] = dRho - dP / cc;
  dW[1] = dBn;
  double h1 = kSqrtHalf * (betaY * dUt2 - betaZ * dUt1);
  double h2 = siBX * (betaZ * dBt1 - betaY * dBt2) / (2.0 * sqrt(2.0 * kPi * Rho));
  dW[2] = h1 + h2;
  dW[3] = h1 - h2;
  h1 = dP / (2.0 * Rho * cc);
  h2 = dUn / (2.0 * cc);
  const double h3 = (betaY * dBt1 + betaZ * dBt2) / (4.0 * s.c * sqrt(kPi * Rho));
  const double h4 = siBX * (betaY * dUt1 + betaZ * dUt2) / (2.0 * cc);
  const double aF = s.alphaF, aS = s.alphaS, af = s.af, as = s.as;
  dW[4] = aF * (h1 + af * h2) + aS * (h3 - as * h4);
  dW[5] = aF * (h1 - af * h2) + aS * (h3 + as * h4);
  dW[6] = aS * (h1 + as * h2) - aF * (h3 - af * h4);
  dW[7] = aS * (h1 - as * h2) - aF * (h3 + af * h4);
}

// CHARSYNTHESISF on one vector of wave amplitudes, in place.
template <int D>
__device__ __forceinline__ void char_synthesis(const CharState& s, double* dW) {
  constexpr int in = 1 + D, it1 = 1 + (D + 1) % 3, it2 = 1 + (D + 2) % 3;
  constexpr int inB = 5 + D, itB1 = 5 + (D + 1) % 3, itB2 = 5 + (D + 2) % 3;
  const double betaY = s.betaY, betaZ = s.betaZ;
  const double betaYX = (s.BX < 0.0) ? -betaY : betaY;
  const double betaZX = (s.BX < 0.0) ? -betaZ : betaZ;
  const double alpha1 = dW[0], alpha2 = dW[1];
  const double alpha3 = kSqrtHalf * dW[2], alpha4 = kSqrtHalf * dW[3];
  const double alpha5 = dW[4], alpha6 = dW[5], alpha7 = dW[6], alpha8 = dW[7];
  const double alph3p4 = alpha3 + alpha4, alph3m4 = alpha3 - alpha4;
  const double alph5p6 = alpha5 + alpha6, alph5m6 = alpha5 - alpha6;
  const double alph7p8 = alpha7 + alpha8, alph7m8 = alpha7 - alpha8;
  const double aF = s.alphaF, aS = s.alphaS, af = s.af, as = s.as;
  const double DN = 2.0 * sqrt(kPi * s.Rho);
  const double HRho = s.Rho * (aF * alph5p6 + aS * alph7p8);
  const double HU = aS * as * alph5m6 - aF * af * alph7m8;
  const double HB = s.c * (aS * alph5p6 - aF * alph7p8);
  dW[0] = alpha1 + HRho;
  dW[in] = aF * af * alph5m6 + aS * as * alph7m8;
  dW[it1] = -betaZ * alph3p4 - betaYX * HU;
  dW[it2] = betaY * alph3p4 - betaZX * HU;
  dW[4] = s.cc * HRho;
  dW[inB] = alpha2;
  dW[itB1] = DN * (betaZX * alph3m4 + betaY * HB);
  dW[itB2] = DN * (-betaYX * alph3m4 + betaZ * HB);
}

// Characteristic face values of the 8 plasma variables of one cell from the
// cells c-1, c, c+1 (FP64): lo = value on the low face, hi on the high face.
template <int D>
__device__ __forceinline__ void char_face_values(const DevParams& P, const double* wm1,
                                                 const double* w0, const double* wp1,
                                                 double* lo, double* hi) {
  double SL[8], SR[8];
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    SL[v] = w0[v] - wm1[v];
    SR[v] = wp1[v] - w0[v];
  }
  CharState s;
  char_state<D>(P, w0, 1.0e-12, s);
  char_analysis<D>(s, SL);
  char_analysis<D>(s, SR);
#pragma unroll
  for (int v = 0; v < 8; ++v) face_slopes<double>(P.lim[v], SL[v], SR[v]);
  char_state<D>(P, w0, 1.0e-8, s);
  char_synthesis<D>(s, SL);
  char_synthesis<D>(s, SR);
#pragma unroll
  for (int v = 0; v < 8; ++v) {
    lo[v] = w0[v] - SL[v];
    hi[v] = w0[v] + SR[v];
  }
  if (P.check_tvd) {  // CHECKTVD (reconstructionF.ChF:1248-1279)
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      if (P.check_tvd == 1 || v == 0 || v == 4) {
        const double WP = w0[v];
        const double dWR = wp1[v] - WP, dWL = WP - wm1[v];
        const double dSL = WP - lo[v], dSR = hi[v] - WP;
        lo[v] = WP - minmod3_<double>(dWL, dWR, dSL);
        hi[v] = WP + minmod3_<double>(dWL, dWR, dSR);
      }
    }
  }
}

}  // namespace mf
