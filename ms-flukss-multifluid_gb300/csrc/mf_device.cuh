// mf_device.cuh - device-side physics of the multi-fluid MHD patch update.
//
// Every routine restates one reference kernel (paths inside MHDAM-3.2.4).  The
// arithmetic keeps the reference's evaluation order for each non-zero term; the
// Roe solvers skip the structurally zero entries of their 8x8 eigenmatrices,
// which changes no result (x + 0*y == x for finite y).
#pragma once

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

enum RsKind : int { kRoe8 = 0, kRoe7 = 1, kRusanov = 2 };

// Parameters as the kernels see them (mf_params + derived constants).
struct DevParams {
  int sd, nf, glm, nc, irhon;
  int rs, aver;
  int use8, divb_method, check_pos, ce, reinit, bc_kind;
  int lim[8];
  int periodic[3], dlo[3], dhi[3];
  double gamma, hgamma, invhgamma, smallr, smallp, del2, smallB, dx, invdx;
  double factor_ch, factor_cp;
  double ce_scale_vel, ce_sigma_scale, ce_a, ce_b, ce_damp_c, ce_damp_pow;
  double sun_c[3], sun_r, sun_v, t_coeff, tmlim, zbot, ztop;
  double r0, rint, sun_rho, sun_p, sun_b, sun_beta, dir_br;
  double bc_plasma[8], bc_n1[5];
};

// Values that change from step to step; kept in device memory so that a
// captured CUDA graph reads the current ones.
struct StepState {
  double dt;        // time step of the step being taken
  double ch, cp;    // GLM speeds
  double cfl;       // dt of the next async step = cfl * dt_min
  double dt_min;    // result: minimum of dx/cmax
  int min_desc;     // result: patch index of the minimum
  int min_idx;      // result: Fortran-order index inside the valid box
  unsigned flags;   // error bits (kFlag*)
  int pad;
};

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
template <typename R> __device__ __forceinline__ R rsqrt_(R a) { return sqrt(a); }

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
// limited face values (src/reconstructionF.ChF): returns the value on the
// low face (lo) and on the high face (hi) of the centre cell
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

// ---------------------------------------------------------------------------
// Roe 8-wave / 7-wave MHD flux: RIEMANNF (src/Roe8WaveF.ChF:5-601) and
// RIEMANN7F (src/Roe7WaveF.ChF:5-558).  wl/wr: rho,u,v,w,p,bx,by,bz in the
// global frame; g: fluxes in the same order.  SEVEN drops the normal-B wave
// (RIEMANN7F), whose normal-B flux is zero.
// ---------------------------------------------------------------------------
template <typename R, int DIR, bool SEVEN>
__device__ __forceinline__ void roe_mhd(const DevParams& P, const R* wl, const R* wr, R* g) {
  constexpr int in = 1 + DIR, it1 = 1 + (DIR + 1) % 3, it2 = 1 + (DIR + 2) % 3;
  constexpr int inB = 5 + DIR, it1B = 5 + (DIR + 1) % 3, it2B = 5 + (DIR + 2) % 3;
  const R gamma = R(P.gamma), hgamma = R(P.hgamma);
  const R smallp = R(P.smallp), smallr = R(P.smallr);
  const R i4pi = R(kInv4Pi), i8pi = R(kInv8Pi), sq2 = R(kSqrtHalf);

  R PGasL = rmax<R>(smallp, wl[4]), RhoL = rmax<R>(smallr, wl[0]);
  R UL = wl[in], VL = wl[it1], WL = wl[it2];
  R BXL = wl[inB], BYL = wl[it1B], BZL = wl[it2B];
  R PGasR = rmax<R>(smallp, wr[4]), RhoR = rmax<R>(smallr, wr[0]);
  R UR = wr[in], VR = wr[it1], WR = wr[it2];
  R BXR = wr[inB], BYR = wr[it1B], BZR = wr[it2B];

  R RUL = RhoL * UL, RVL = RhoL * VL, RWL = RhoL * WL;
  R BxBL = i8pi * (BXL * BXL + BYL * BYL + BZL * BZL);
  R RUxUL = R(0.5) * (RUL * UL + RVL * VL + RWL * WL);
  R PL = PGasL + BxBL;
  R EL = PGasL / hgamma + RUxUL + BxBL;
  R AL2 = gamma * PGasL / RhoL;

  R RUR = RhoR * UR, RVR = RhoR * VR, RWR = RhoR * WR;
  R BxBR = i8pi * (BXR * BXR + BYR * BYR + BZR * BZR);
  R RUxUR = R(0.5) * (RUR * UR + RVR * VR + RWR * WR);
  R PR = PGasR + BxBR;
  R ER = PGasR / hgamma + RUxUR + BxBR;
  R AR2 = gamma * PGasR / RhoR;

  R ccmi, ccma;
  if (AL2 > AR2) { ccmi = AR2; ccma = AL2; } else { ccmi = AL2; ccma = AR2; }

  R Rho, U, V, W, BX, BY, BZ, BX2, BYZ2, BxBH, kk, cc;
  if (P.aver == 1) {
    R HL = (EL + PL) / RhoL, HR = (ER + PR) / RhoR;
    R coefRL = R(1) / (R(1) + rsqrt_<R>(RhoR / RhoL));
    R coefRR = R(1) - coefRL;
    Rho = RhoR * coefRL + RhoL * coefRR;
    U = UL * coefRL + UR * coefRR;
    V = VL * coefRL + VR * coefRR;
    W = WL * coefRL + WR * coefRR;
    R HAV = HL * coefRL + HR * coefRR;
    BX = BXR * coefRL + BXL * coefRR;
    BY = BYR * coefRL + BYL * coefRR;
    BZ = BZR * coefRL + BZL * coefRR;
    R BXAV = R(0.5) * (BXL + BXR);
    BX2 = BXAV * BXAV;
    R BY2 = BY * BY, BZ2 = BZ * BZ;
    BYZ2 = BY2 + BZ2;
    BxBH = i8pi * (BX2 + BYZ2);
    kk = R(0.5) * (U * U + V * V + W * W);
    R DBX = BXR - BXL, DBY = BYR - BYL, DBZ = BZR - BZL;
    R X = i8pi * (DBX * DBX + DBY * DBY + DBZ * DBZ) * coefRL * coefRL / RhoL;
    cc = hgamma * (HAV - kk - i4pi * (BX * BXAV + BYZ2) / Rho) + (R(2) - gamma) * X;
  } else {
    Rho = R(0.5) * (RhoL + RhoR);
    U = R(0.5) * (UL + UR);
    V = R(0.5) * (VL + VR);
    W = R(0.5) * (WL + WR);
    BX = R(0.5) * (BXL + BXR);
    BY = R(0.5) * (BYL + BYR);
    BZ = R(0.5) * (BZL + BZR);
    R Pav = R(0.5) * (PL + PR);
    BX2 = BX * BX;
    R BY2 = BY * BY, BZ2 = BZ * BZ;
    BYZ2 = BY2 + BZ2;
    BxBH = i8pi * (BX2 + BYZ2);
    kk = R(0.5) * (U * U + V * V + W * W);
    R PGas = Pav - BxBH;
    cc = gamma * PGas / Rho;
  }

  R bb = i4pi * BX2 / Rho;
  R b = rsqrt_<R>(bb);
  if (cc < ccmi) cc = ccmi;
  if (cc > ccma) cc = ccma;
  R c = rsqrt_<R>(cc);

  R hyy, hzz, aaf, aas, af, as;
  const R smallB = R(P.smallB);
  if (BYZ2 < smallB * smallB) {
    hyy = sq2;
    hzz = sq2;
    if (bb > cc) { aaf = bb; aas = cc; af = b; as = c; }
    else { aaf = cc; aas = bb; af = c; as = b; }
  } else {
    R hyz = rsqrt_<R>(BYZ2);
    hyy = BY / hyz;
    hzz = BZ / hyz;
    R szb = cc + (BxBH + BxBH) / Rho;
    R h = rsqrt_<R>(szb * szb - R(4) * cc * bb);
    aas = R(0.5) * (szb - h);
    if (aas <= R(0)) { aas = R(0); as = R(0); }
    else if (aas >= cc) { aas = cc; as = c; }
    else { as = rsqrt_<R>(aas); }
    aaf = R(0.5) * (szb + h);
    if (aaf <= cc) { aaf = cc; af = c; }
    else { af = rsqrt_<R>(aaf); }
  }

  // entropy-fixed speeds (Roe8 numbering: 1 entropy, 2 div-B, 3/4 Alfven,
  // 5/6 fast, 7/8 slow)
  const R eigmax = rabs<R>(U) + rabs<R>(V) + rabs<R>(W) + af;
  const R del = R(P.del2) * eigmax;
  const R dell2 = del * del;
  auto fix = [&](R e) -> R {
    R z = rabs<R>(e);
    return (z >= del) ? z : R(0.5) * (z * z + dell2) / del;
  };
  R A1 = fix(U);
  R A2 = fix(U);
  R A3 = fix(U + b), A4 = fix(U - b);
  R A5 = fix(U + af), A6 = fix(U - af);
  R A7 = fix(U + as), A8 = fix(U - as);

  R alf, als;
  R dfs = aaf - aas;
  if (dfs < R(1.0e-8)) { alf = R(1); als = R(0); }
  else if ((cc - aas) <= R(0)) { alf = R(0); als = R(1); }
  else if ((aaf - cc) <= R(0)) { alf = R(1); als = R(0); }
  else { alf = rsqrt_<R>((cc - aas) / dfs); als = rsqrt_<R>((aaf - cc) / dfs); }

  R sih = R(-1);
  if (BX >= R(0)) sih = R(1);

  R fl1 = RUL;
  R fl2 = UL * RUL - BXL * BXL * i4pi + PL;
  R fl3 = UL * RVL - BXL * BYL * i4pi;
  R fl4 = UL * RWL - BXL * BZL * i4pi;
  R fl5 = UL * (EL + PL) - BXL * (UL * BXL + VL * BYL + WL * BZL) * i4pi;
  R fl7 = UL * BYL - BXL * VL;
  R fl8 = UL * BZL - BXL * WL;
  R fr1 = RUR;
  R fr2 = UR * RUR - BXR * BXR * i4pi + PR;
  R fr3 = UR * RVR - BXR * BYR * i4pi;
  R fr4 = UR * RWR - BXR * BZR * i4pi;
  R fr5 = UR * (ER + PR) - BXR * (UR * BXR + VR * BYR + WR * BZR) * i4pi;
  R fr7 = UR * BYR - BXR * VR;
  R fr8 = UR * BZR - BXR * WR;

  R du1 = RhoL - RhoR;
  R du2 = RUL - RUR;
  R du3 = RVL - RVR;
  R du4 = RWL - RWR;
  R du5 = EL - ER;
  R du6 = BXL - BXR;
  R du7 = BYL - BYR;
  R du8 = BZL - BZR;
  if (SEVEN)
    du5 = -hgamma * (-kk * du1 + U * du2 + V * du3 + W * du4 - du5 + (BY * du7 + BZ * du8) * i4pi);
  else
    du5 = -hgamma *
          (-kk * du1 + U * du2 + V * du3 + W * du4 - du5 + (BX * du6 + BY * du7 + BZ * du8) * i4pi);
  du2 = (-U * du1 + du2) / Rho;
  du3 = (-V * du1 + du3) / Rho;
  du4 = (-W * du1 + du4) / Rho;

  const R sqPiRho = rsqrt_<R>(R(kPi) * Rho);
  const R sq2PiRho = rsqrt_<R>(R(k2Pi) * Rho);

  // left eigenvectors (non-zero entries only)
  R so15 = -R(1) / cc;
  R so33 = -hzz * sq2, so34 = hyy * sq2;
  R so37 = R(0.5) * hzz * sih / sq2PiRho, so38 = -R(0.5) * hyy * sih / sq2PiRho;
  R so47 = -R(0.5) * hzz * sih / sq2PiRho, so48 = R(0.5) * hyy * sih / sq2PiRho;
  R so52 = R(0.5) * alf * af / cc;
  R so53 = -R(0.5) * als * as * hyy * sih / cc;
  R so54 = -R(0.5) * als * as * hzz * sih / cc;
  R so55 = R(0.5) * alf / (cc * Rho);
  R so57 = R(0.25) * als * hyy / (c * sqPiRho);
  R so58 = R(0.25) * als * hzz / (c * sqPiRho);
  R so62 = -R(0.5) * alf * af / cc;
  R so63 = R(0.5) * als * as * hyy * sih / cc;
  R so64 = R(0.5) * als * as * hzz * sih / cc;
  R so72 = R(0.5) * als * as / cc;
  R so73 = R(0.5) * alf * af * hyy * sih / cc;
  R so74 = R(0.5) * alf * af * hzz * sih / cc;
  R so75 = R(0.5) * als / (Rho * cc);
  R so77 = -R(0.25) * alf * hyy / (c * sqPiRho);
  R so78 = -R(0.25) * alf * hzz / (c * sqPiRho);
  R so82 = -R(0.5) * als * as / cc;
  R so83 = -R(0.5) * alf * af * hyy * sih / cc;
  R so84 = -R(0.5) * alf * af * hzz * sih / cc;

  R lu1 = A1 * (du1 + so15 * du5);
  R lu2 = A2 * du6;
  R lu3 = A3 * (so33 * du3 + so34 * du4 + so37 * du7 + so38 * du8);
  R lu4 = A4 * (so33 * du3 + so34 * du4 + so47 * du7 + so48 * du8);
  R lu5 = A5 * (so52 * du2 + so53 * du3 + so54 * du4 + so55 * du5 + so57 * du7 + so58 * du8);
  R lu6 = A6 * (so62 * du2 + so63 * du3 + so64 * du4 + so55 * du5 + so57 * du7 + so58 * du8);
  R lu7 = A7 * (so72 * du2 + so73 * du3 + so74 * du4 + so75 * du5 + so77 * du7 + so78 * du8);
  R lu8 = A8 * (so82 * du2 + so83 * du3 + so84 * du4 + so75 * du5 + so77 * du7 + so78 * du8);

  // right eigenvectors (non-zero entries only)
  R sp15 = Rho * alf, sp17 = Rho * als;
  R sp25 = alf * af, sp26 = -alf * af, sp27 = als * as, sp28 = -als * as;
  R sp33 = -hzz * sq2;
  R sp35 = -als * as * hyy * sih, sp36 = als * as * hyy * sih;
  R sp37 = alf * af * hyy * sih, sp38 = -alf * af * hyy * sih;
  R sp43 = hyy * sq2;
  R sp45 = -als * as * hzz * sih, sp46 = als * as * hzz * sih;
  R sp47 = alf * af * hzz * sih, sp48 = -alf * af * hzz * sih;
  R sp55 = alf * Rho * cc, sp57 = als * Rho * cc;
  R sp73 = hzz * sq2PiRho * sih, sp74 = -hzz * sq2PiRho * sih;
  R sp75 = R(2) * als * sqPiRho * c * hyy;
  R sp77 = -R(2) * alf * sqPiRho * c * hyy;
  R sp83 = -hyy * sq2PiRho * sih, sp84 = hyy * sq2PiRho * sih;
  R sp85 = R(2) * als * sqPiRho * c * hzz;
  R sp87 = -R(2) * alf * sqPiRho * c * hzz;

  R ra1 = lu1 + sp15 * lu5 + sp15 * lu6 + sp17 * lu7 + sp17 * lu8;
  R ra2 = sp25 * lu5 + sp26 * lu6 + sp27 * lu7 + sp28 * lu8;
  R ra3 = sp33 * lu3 + sp33 * lu4 + sp35 * lu5 + sp36 * lu6 + sp37 * lu7 + sp38 * lu8;
  R ra4 = sp43 * lu3 + sp43 * lu4 + sp45 * lu5 + sp46 * lu6 + sp47 * lu7 + sp48 * lu8;
  R ra5 = sp55 * lu5 + sp55 * lu6 + sp57 * lu7 + sp57 * lu8;
  R ra6 = lu2;
  R ra7 = sp73 * lu3 + sp74 * lu4 + sp75 * lu5 + sp75 * lu6 + sp77 * lu7 + sp77 * lu8;
  R ra8 = sp83 * lu3 + sp84 * lu4 + sp85 * lu5 + sp85 * lu6 + sp87 * lu7 + sp87 * lu8;

  if (SEVEN)
    ra5 = ra1 * kk + Rho * (U * ra2 + V * ra3 + W * ra4) + ra5 / hgamma + i4pi * (BY * ra7 + BZ * ra8);
  else
    ra5 = ra1 * kk + Rho * (U * ra2 + V * ra3 + W * ra4) + ra5 / hgamma +
          i4pi * (BX * ra6 + BY * ra7 + BZ * ra8);
  ra2 = U * ra1 + Rho * ra2;
  ra3 = V * ra1 + Rho * ra3;
  ra4 = W * ra1 + Rho * ra4;

  g[0] = R(0.5) * (fl1 + fr1 + ra1);
  g[in] = R(0.5) * (fl2 + fr2 + ra2);
  g[it1] = R(0.5) * (fl3 + fr3 + ra3);
  g[it2] = R(0.5) * (fl4 + fr4 + ra4);
  g[4] = R(0.5) * (fl5 + fr5 + ra5);
  g[inB] = SEVEN ? R(0) : R(0.5) * (R(0) + R(0) + ra6);
  g[it1B] = R(0.5) * (fl7 + fr7 + ra7);
  g[it2B] = R(0.5) * (fl8 + fr8 + ra8);
}

// RUSANOVF (src/RusanovF.ChF:4-197)
template <typename R, int DIR>
__device__ __forceinline__ void rusanov_mhd(const DevParams& P, const R* wl, const R* wr, R* g) {
  constexpr int in = 1 + DIR, it1 = 1 + (DIR + 1) % 3, it2 = 1 + (DIR + 2) % 3;
  constexpr int inB = 5 + DIR, it1B = 5 + (DIR + 1) % 3, it2B = 5 + (DIR + 2) % 3;
  const R gamma = R(P.gamma), hgamma = R(P.hgamma);
  const R i4pi = R(kInv4Pi), i8pi = R(kInv8Pi);
  R PGasL = rmax<R>(R(P.smallp), wl[4]), RhoL = rmax<R>(R(P.smallr), wl[0]);
  R UL = wl[in], VL = wl[it1], WL = wl[it2], BXL = wl[inB], BYL = wl[it1B], BZL = wl[it2B];
  R PGasR = rmax<R>(R(P.smallp), wr[4]), RhoR = rmax<R>(R(P.smallr), wr[0]);
  R UR = wr[in], VR = wr[it1], WR = wr[it2], BXR = wr[inB], BYR = wr[it1B], BZR = wr[it2B];
  R RUL = RhoL * UL, RVL = RhoL * VL, RWL = RhoL * WL;
  R BxBL = i8pi * (BXL * BXL + BYL * BYL + BZL * BZL);
  R RUxUL = R(0.5) * (RUL * UL + RVL * VL + RWL * WL);
  R PL = PGasL + BxBL;
  R EL = PGasL / hgamma + RUxUL + BxBL;
  R BXL_4PI = BXL * i4pi;
  R RUR = RhoR * UR, RVR = RhoR * VR, RWR = RhoR * WR;
  R BxBR = i8pi * (BXR * BXR + BYR * BYR + BZR * BZR);
  R RUxUR = R(0.5) * (RUR * UR + RVR * VR + RWR * WR);
  R PR = PGasR + BxBR;
  R ER = PGasR / hgamma + RUxUR + BxBR;
  R BXR_4PI = BXR * i4pi;
  R Rho, U, BX2, BxBH, A2;
  if (P.aver == 1) {
    R HL = (EL + PL) / RhoL, HR = (ER + PR) / RhoR;
    R coefRL = R(1) / (R(1) + rsqrt_<R>(RhoR / RhoL));
    R coefRR = R(1) - coefRL;
    Rho = RhoR * coefRL + RhoL * coefRR;
    U = UL * coefRL + UR * coefRR;
    R V = VL * coefRL + VR * coefRR;
    R W = WL * coefRL + WR * coefRR;
    R HAV = HL * coefRL + HR * coefRR;
    R BX = BXR * coefRL + BXL * coefRR;
    R BY = BYR * coefRL + BYL * coefRR;
    R BZ = BZR * coefRL + BZL * coefRR;
    R BXAV = R(0.5) * (BXL + BXR);
    BX2 = BXAV * BXAV;
    R BY2 = BY * BY, BZ2 = BZ * BZ;
    R BYZ2 = BY2 + BZ2;
    BxBH = i8pi * (BX2 + BYZ2);
    R kk = R(0.5) * (U * U + V * V + W * W);
    R DBX = BXR - BXL, DBY = BYR - BYL, DBZ = BZR - BZL;
    R X = i8pi * (DBX * DBX + DBY * DBY + DBZ * DBZ) * coefRL * coefRL / RhoL;
    A2 = hgamma * (HAV - kk - i4pi * (BX * BXAV + BYZ2) / Rho) + (R(2) - gamma) * X;
  } else {
    Rho = R(0.5) * (RhoL + RhoR);
    U = R(0.5) * (UL + UR);
    R BX = R(0.5) * (BXL + BXR), BY = R(0.5) * (BYL + BYR), BZ = R(0.5) * (BZL + BZR);
    R PGas = R(0.5) * (PGasL + PGasR);
    BX2 = BX * BX;
    R BY2 = BY * BY, BZ2 = BZ * BZ;
    BxBH = i8pi * (BX2 + BY2 + BZ2);
    A2 = gamma * PGas / Rho;
  }
  R bb = i4pi * BX2 / Rho;
  R szb = A2 + (BxBH + BxBH) / Rho;
  R h = rsqrt_<R>(szb * szb - R(4) * A2 * bb);
  R aaf = R(0.5) * (szb + h);
  R af = rsqrt_<R>(aaf);
  R em = rabs<R>(U) + af;
  g[0] = R(0.5) * (RUL + RUR + em * (RhoL - RhoR));
  g[in] = R(0.5) * ((UL * RUL - BXL_4PI * BXL + PL) + (UR * RUR - BXR_4PI * BXR + PR) + em * (RUL - RUR));
  g[it1] = R(0.5) * ((UL * RVL - BXL_4PI * BYL) + (UR * RVR - BXR_4PI * BYR) + em * (RVL - RVR));
  g[it2] = R(0.5) * ((UL * RWL - BXL_4PI * BZL) + (UR * RWR - BXR_4PI * BZR) + em * (RWL - RWR));
  g[4] = R(0.5) * ((UL * (EL + PL) - BXL_4PI * (UL * BXL + VL * BYL + WL * BZL)) +
                   (UR * (ER + PR) - BXR_4PI * (UR * BXR + VR * BYR + WR * BZR)) + em * (EL - ER));
  g[inB] = R(0.5) * (R(0) + R(0) + em * (BXL - BXR));
  g[it1B] = R(0.5) * ((UL * BYL - BXL * VL) + (UR * BYR - BXR * VR) + em * (BYL - BYR));
  g[it2B] = R(0.5) * ((UL * BZL - BXL * WL) + (UR * BZR - BXR * WR) + em * (BZL - BZR));
}

// DEDNER2X2F (src/DednerF.ChF:89-170): returns the Bn and psi fluxes.
template <typename R>
__device__ __forceinline__ void dedner_2x2(R ch, R bxl, R psil, R bxr, R psir, R& fbn, R& fpsi) {
  R ch2 = ch * ch;
  R so12 = -R(0.5) / ch, so22 = R(0.5) / ch;
  R du1 = bxl - bxr, du2 = psil - psir;
  R lu1 = ch * (R(0.5) * du1 + so12 * du2);
  R lu2 = ch * (R(0.5) * du1 + so22 * du2);
  R ra1 = lu1 + lu2;
  R ra2 = -ch * lu1 + ch * lu2;
  fbn = R(0.5) * (psil + psir + ra1);
  fpsi = R(0.5) * (ch2 * bxl + ch2 * bxr + ra2);
}

// VANLEERF (src/VanLeerRSF.ChF:4-130): wl/wr = rho,u,v,w,p of one Euler fluid.
template <typename R, int DIR>
__device__ __forceinline__ void vanleer_euler(const DevParams& P, const R* wl, const R* wr, R* g) {
  constexpr int in = 1 + DIR, it1 = 1 + (DIR + 1) % 3, it2 = 1 + (DIR + 2) % 3;
  const R gamma = R(P.gamma), hgamma = R(P.hgamma);
  R fl1, fl2, fl3, fl4, fl5, fr1, fr2, fr3, fr4, fr5;
  R PGasL = rmax<R>(R(P.smallp), wl[4]), RhoL = rmax<R>(R(P.smallr), wl[0]);
  R UL = wl[in], VL = wl[it1], WL = wl[it2];
  R RUL = RhoL * UL, RVL = RhoL * VL, RWL = RhoL * WL;
  R RUxUL = R(0.5) * (RUL * UL + RVL * VL + RWL * WL);
  R EL = PGasL / hgamma + RUxUL;
  R AL = rsqrt_<R>(gamma * PGasL / RhoL);
  if (UL <= -AL) {
    fr1 = fr2 = fr3 = fr4 = fr5 = R(0);
  } else if (UL >= AL) {
    fr1 = RhoL * UL;
    fr2 = fr1 * UL + PGasL;
    fr3 = fr1 * VL;
    fr4 = fr1 * WL;
    fr5 = UL * (EL + PGasL);
  } else {
    R UA = (-UL + (AL + AL)) / gamma;
    R H = (EL + PGasL) / RhoL;
    R HU = UL + AL;
    fr1 = R(0.25) * RhoL * HU * HU / AL;
    fr2 = fr1 * (UL + UA);
    fr3 = fr1 * VL;
    fr4 = fr1 * WL;
    fr5 = fr1 * H;
  }
  R PGasR = rmax<R>(R(P.smallp), wr[4]), RhoR = rmax<R>(R(P.smallr), wr[0]);
  R UR = wr[in], VR = wr[it1], WR = wr[it2];
  R RUR = RhoR * UR, RVR = RhoR * VR, RWR = RhoR * WR;
  R RUxUR = R(0.5) * (RUR * UR + RVR * VR + RWR * WR);
  R ER = PGasR / hgamma + RUxUR;
  R AR = rsqrt_<R>(gamma * PGasR / RhoR);
  if (UR >= AR) {
    fl1 = fl2 = fl3 = fl4 = fl5 = R(0);
  } else if (UR <= -AR) {
    fl1 = RhoR * UR;
    fl2 = fl1 * UR + PGasR;
    fl3 = fl1 * VR;
    fl4 = fl1 * WR;
    fl5 = UR * (ER + PGasR);
  } else {
    R UA = (-UR - (AR + AR)) / gamma;
    R H = (ER + PGasR) / RhoR;
    R HU = UR - AR;
    fl1 = -R(0.25) * RhoR * HU * HU / AR;
    fl2 = fl1 * (UR + UA);
    fl3 = fl1 * VR;
    fl4 = fl1 * WR;
    fl5 = fl1 * H;
  }
  g[0] = fl1 + fr1;
  g[in] = fl2 + fr2;
  g[it1] = fl3 + fr3;
  g[it2] = fl4 + fr4;
  g[4] = fl5 + fr5;
}

// ---------------------------------------------------------------------------
// cell sources (always FP64)
// ---------------------------------------------------------------------------

// DEFINE_REGIONS_2F (swlism/SWLISMF.ChF:654-742), Cartesian branch.
__device__ __forceinline__ int region_cell(const DevParams& P, int i, int j, int k,
                                           const double* w) {
  double x = (i + 0.5) * P.dx - P.sun_c[0];
  double y = (j + 0.5) * P.dx - P.sun_c[1];
  double z = 0.0, r2, invr, ur;
  if (P.sd == 3) {
    z = (k + 0.5) * P.dx - P.sun_c[2];
    r2 = x * x + y * y + z * z;
    invr = 1.0 / sqrt(r2);
    ur = w[1] * (x * invr) + w[2] * (y * invr) + w[3] * (z * invr);
  } else {
    r2 = x * x + y * y;
    invr = 1.0 / sqrt(r2);
    ur = w[1] * (x * invr) + w[2] * (y * invr);
  }
  double TEMP = P.t_coeff * w[4] / w[0];
  int reg;
  bool zout = (P.sd == 3) && ((z < P.zbot) || (z > P.ztop));
  if (fabs(ur) >= 0.6 * P.sun_v) {
    reg = ((TEMP >= 1.0e6) && (r2 > P.sun_r * P.sun_r)) ? 2 : 3;
    if (zout) reg = 1;
  } else {
    if (TEMP >= P.tmlim) {
      reg = 2;
      if (zout) reg = 1;
    } else {
      reg = 1;
    }
  }
  return reg;
}

// Recipient of newly created neutrals: CHARGE_EXCHANGE_2F/3F/4F/MF
// (swlism/ChargeExchange2F.ChF:294-1149).
__device__ __forceinline__ int ce_recipient(int nN, int reg) {
  if (nN == 1) return (reg == 1 || reg == 4) ? 1 : 0;
  if (nN == 2) return (reg == 1) ? 1 : (reg == 2) ? 2 : 0;
  if (nN == 3) return (reg == 1 || reg == 4) ? 1 : (reg == 2) ? 2 : (reg == 3) ? 3 : 0;
  return (reg >= 1 && reg <= nN) ? reg : 0;
}

// Pauls & Zank charge-exchange rates of one cell; adds S = -dt*H to u
// (HeliosphericProblem::explicitSource, swlism/HeliosphericProblem.cpp:1394-1539).
template <int IRHON>
__device__ __forceinline__ void charge_exchange_add(const DevParams& P, const double* w, int reg,
                                                    double dt, double* u) {
  const int nN = P.nf - 1;
  double rho = w[0], ux = w[1], uy = w[2], uz = w[3], pp = w[4];
  double U2 = ux * ux + uy * uy + uz * uz;
  double VVTP = pp / rho;
  double h2 = 0, h3 = 0, h4 = 0, h5 = 0, PPLUX = 0, PPLUY = 0, PPLUZ = 0, ENPLU = 0;
  double DENPLU[MF_MAX_FLUIDS], PMIX[MF_MAX_FLUIDS], PMIY[MF_MAX_FLUIDS], PMIZ[MF_MAX_FLUIDS],
      ENMI[MF_MAX_FLUIDS];
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f) {
    if (f > nN) break;
    const double* wn = w + IRHON + (f - 1) * 5;
    double rhoN = wn[0], uxN = wn[1], uyN = wn[2], uzN = wn[3], pN = wn[4];
    double UH2 = uxN * uxN + uyN * uyN + uzN * uzN;
    double DU2 = (ux - uxN) * (ux - uxN) + (uy - uyN) * (uy - uyN) + (uz - uzN) * (uz - uzN);
    double VPHH = (ux - uxN) * uxN + (uy - uyN) * uyN + (uz - uzN) * uzN;
    double VPHP = (ux - uxN) * ux + (uy - uyN) * uy + (uz - uzN) * uz;
    double VVTH = 2.0 * pN / rhoN;
    double UD = sqrt(4.0 * (VVTP + VVTH) / kPi + DU2);
    double UPM = sqrt(16.0 * VVTP / kPi + 2.25 * kPi * VVTH + 4.0 * DU2);
    double UHM = sqrt(2.25 * kPi * VVTP + 16.0 * VVTH / kPi + 4.0 * DU2);
    double UPE = sqrt((4.0 * VVTP + 64.0 * VVTH / 9.0) / kPi + DU2);
    double UHE = sqrt((64.0 * VVTP / 9.0 + 4.0 * VVTH) / kPi + DU2);
    double UDS = P.ce_scale_vel * UD;
    double t = P.ce_a - P.ce_b * log(UDS);
    double SIG = t * t;
    if (P.ce_damp_c > 0.0) SIG = SIG * pow(1.0 - exp(-P.ce_damp_c / UDS), P.ce_damp_pow);
    SIG = P.ce_sigma_scale * SIG;
    double ARR = SIG * rhoN * rho;
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
  u[1] = u[1] + (-dt * h2);
  u[2] = u[2] + (-dt * h3);
  u[3] = u[3] + (-dt * h4);
  u[4] = u[4] + (-dt * h5);
  // S of the magnetic field (and of psi) is zero: u + 0 == u
  const int rk = ce_recipient(nN, reg);
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f) {
    if (f > nN) break;
    double H1, H2, H3, H4, H5;
    if (f == rk) {
      if (nN <= 3) {
        bool first = true;
        H1 = 0.0;
#pragma unroll
        for (int q = 1; q < MF_MAX_FLUIDS; ++q) {
          if (q > nN) break;
          if (q == f) continue;
          H1 = first ? DENPLU[q] : H1 + DENPLU[q];
          first = false;
        }
      } else {
        double sum = DENPLU[1];
#pragma unroll
        for (int q = 2; q < MF_MAX_FLUIDS; ++q)
          if (q <= nN) sum = sum + DENPLU[q];
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
    double* un = u + IRHON + (f - 1) * 5;
    un[0] = un[0] + (-dt * H1);
    un[1] = un[1] + (-dt * H2);
    un[2] = un[2] + (-dt * H3);
    un[3] = un[3] + (-dt * H4);
    un[4] = un[4] + (-dt * H5);
  }
}

// HELIOREINIT_DEFAULT (swlism/HeliosphericPlasmaBCF.ChF:1435-1555), monopolar field.
__device__ __host__ inline void reinit_cell(const DevParams& P, int i, int j, int k, double* u) {
  double x = (i + 0.5) * P.dx - P.sun_c[0];
  double y = (j + 0.5) * P.dx - P.sun_c[1];
  double z = 0.0;
  if (P.sd == 3) z = (k + 0.5) * P.dx - P.sun_c[2];
  double r2 = (P.sd == 3) ? (x * x + y * y + z * z) : (x * x + y * y);
  if (!(r2 <= P.r0 * P.r0)) return;
  double r = sqrt(r2);
  double rr = r / P.rint;
  double xy = sqrt(x * x + y * y);
  double cosT = z / r;
  double sinT = sqrt(1.0 - cosT * cosT);
  double cosF = x / xy;
  double sinF = y / xy;
  double rho = P.sun_rho / (rr * rr);
  double ux = P.sun_v * sinT * cosF;
  double uy = P.sun_v * sinT * sinF;
  double uz = P.sun_v * cosT;
  double pr = P.sun_p / pow(rr, 2.0 * P.gamma);
  double br = P.dir_br * P.sun_b / (rr * rr);
  double bp = -P.sun_beta * br * r * sinT;
  double bx = br * sinT * cosF - bp * sinF;
  double by = br * sinT * sinF + bp * cosF;
  double bz = br * cosT;
  double b = bx * bx + by * by + bz * bz;
  double e0 = pr / P.hgamma + 0.5 * (rho * P.sun_v * P.sun_v + kInv4Pi * b);
  u[0] = rho;
  u[1] = rho * ux;
  u[2] = rho * uy;
  u[3] = rho * uz;
  u[4] = e0;
  u[5] = bx;
  u[6] = by;
  u[7] = bz;
}

// POSTPROCESSING (srcIdeal/PatchIdealMHDF.ChF:1019-1070) and POSTPROCESSING_MF
// (srcIdeal/PatchMHDMFF.ChF:301-511).
template <int IRHON>
__device__ __forceinline__ void positivity_cell(const DevParams& P, double* u) {
  const double hg = P.hgamma, smallR = P.smallr, smallP = P.smallp;
  if (P.nf == 1) {
    double Rho = u[0];
    bool was = false;
    if (Rho < smallR) { Rho = smallR; was = true; }
    double invRho = 1.0 / Rho;
    double Ux = u[1] * invRho, Uy = u[2] * invRho, Uz = u[3] * invRho;
    double BxB = kInv8Pi * (u[5] * u[5] + u[6] * u[6] + u[7] * u[7]);
    double UxU = 0.5 * (Ux * Ux + Uy * Uy + Uz * Uz);
    double Pr = hg * (u[4] - BxB - Rho * UxU);
    if (Pr < smallP) { Pr = smallP; was = true; }
    if (was) {
      u[0] = Rho;
      u[4] = Pr / hg + Rho * UxU + BxB;
    }
    return;
  }
  {
    double Rho = u[0];
    double invRho = 1.0 / Rho;
    double Ux = u[1] * invRho, Uy = u[2] * invRho, Uz = u[3] * invRho;
    double BxB = kInv8Pi * (u[5] * u[5] + u[6] * u[6] + u[7] * u[7]);
    double UxU = 0.5 * (Ux * Ux + Uy * Uy + Uz * Uz);
    double Pr = hg * (u[4] - BxB - Rho * UxU);
    bool was = false;
    if (Rho < smallR) { Rho = smallR; was = true; }
    if (Pr < smallP) { Pr = smallP; was = true; }
    if (was) {
      u[0] = Rho;
      u[1] = Rho * Ux;
      u[2] = Rho * Uy;
      u[3] = Rho * Uz;
      u[4] = Pr / hg + Rho * UxU + BxB;
    }
  }
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f) {
    if (f >= P.nf) break;
    double fd = (f == 1) ? smallR : (f == 3) ? kNet3Dens : kNet2Dens;
    double fp = (f == 1) ? smallP : (f == 3) ? kNet3Pres : kNet2Pres;
    double* un = u + IRHON + (f - 1) * 5;
    double Rho = un[0];
    double invRho = 1.0 / Rho;
    double Ux = un[1] * invRho, Uy = un[2] * invRho, Uz = un[3] * invRho;
    double UxU = 0.5 * (Ux * Ux + Uy * Uy + Uz * Uz);
    double Pr = hg * (un[4] - Rho * UxU);
    bool was = false;
    if (Rho < fd) { Rho = fd; was = true; }
    if (Pr < fp) { Pr = fp; was = true; }
    if (was) {
      un[0] = Rho;
      un[1] = Rho * Ux;
      un[2] = Rho * Uy;
      un[3] = Rho * Uz;
      un[4] = Pr / hg + Rho * UxU;
    }
  }
}

// MAXWAVESPEED (srcIdeal/PatchIdealMHDF.ChF:5-63) + MAXWAVESPEED_E
// (srcIdeal/PatchEulerF.ChF:5-50) of one cell.
template <int IRHON>
__device__ __forceinline__ double max_wave_speed(const DevParams& P, const double* u) {
  double cmax = 0.0;
  {
    double rho = u[0];
    double invrho = 1.0 / rho;
    double ru = u[1], rv = u[2], rw = u[3];
    double uu = ru * invrho, vv = rv * invrho, ww = rw * invrho;
    double ke = ru * uu + rv * vv + rw * ww;
    double bx = u[5], by = u[6], bz = u[7];
    double b = kInv4Pi * (bx * bx + by * by + bz * bz);
    double p = P.hgamma * (u[4] - 0.5 * (ke + b));
    p = fmax(p, P.smallp);
    double a2 = P.gamma * p * invrho;
    double as2 = 0.5 * (a2 + invrho * b);
    double as4 = as2 * as2;
    double bn2 = kInv4Pi * bx * bx * invrho;
    double umax = fabs(uu) + sqrt(as2 + sqrt(as4 - a2 * bn2));
    bn2 = kInv4Pi * by * by * invrho;
    umax = fmax(fabs(vv) + sqrt(as2 + sqrt(as4 - a2 * bn2)), umax);
    bn2 = kInv4Pi * bz * bz * invrho;
    umax = fmax(fabs(ww) + sqrt(as2 + sqrt(as4 - a2 * bn2)), umax);
    cmax = fmax(umax, cmax);
  }
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f) {
    if (f >= P.nf) break;
    const double* un = u + IRHON + (f - 1) * 5;
    double rho = fmax(un[0], P.smallr);
    double invrho = 1.0 / rho;
    double ru = un[1], rv = un[2], rw = un[3];
    double uu = ru * invrho, vv = rv * invrho, ww = rw * invrho;
    double ke = ru * uu + rv * vv + rw * ww;
    double p = P.hgamma * (un[4] - 0.5 * ke);
    p = fmax(p, P.smallp);
    double a = sqrt(P.gamma * p * invrho);
    double umax = fmax(fmax(fabs(uu), fabs(vv)), fabs(ww)) + a;
    cmax = fmax(umax, cmax);
  }
  return cmax;
}

}  // namespace mf
