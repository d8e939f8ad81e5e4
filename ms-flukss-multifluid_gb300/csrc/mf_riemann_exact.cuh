// mf_riemann_exact.cuh - face fluxes of the FP64 parity path: Roe 8/7-wave
// MHD, Rusanov MHD, Dedner (GLM) 2x2 and van Leer splitting, each written in
// the reference's evaluation order (every division and product as in the
// Fortran; structurally zero eigenmatrix entries skipped, which is exact).
// Compiled without multiply-add contraction, so each operation rounds as in
// the CPU restatement.
#pragma once

#include "mf_device.cuh"

namespace mf {
namespace exact {

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
    R coefRL = R(1) / (R(1) + sqrt_r<R>(RhoR / RhoL));
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
  R b = sqrt_r<R>(bb);
  if (cc < ccmi) cc = ccmi;
  if (cc > ccma) cc = ccma;
  R c = sqrt_r<R>(cc);

  R hyy, hzz, aaf, aas, af, as;
  const R smallB = R(P.smallB);
  if (BYZ2 < smallB * smallB) {
    hyy = sq2;
    hzz = sq2;
    if (bb > cc) { aaf = bb; aas = cc; af = b; as = c; }
    else { aaf = cc; aas = bb; af = c; as = b; }
  } else {
    R hyz = sqrt_r<R>(BYZ2);
    hyy = BY / hyz;
    hzz = BZ / hyz;
    R szb = cc + (BxBH + BxBH) / Rho;
    R h = sqrt_r<R>(szb * szb - R(4) * cc * bb);
    aas = R(0.5) * (szb - h);
    if (aas <= R(0)) { aas = R(0); as = R(0); }
    else if (aas >= cc) { aas = cc; as = c; }
    else { as = sqrt_r<R>(aas); }
    aaf = R(0.5) * (szb + h);
    if (aaf <= cc) { aaf = cc; af = c; }
    else { af = sqrt_r<R>(aaf); }
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
  else { alf = sqrt_r<R>((cc - aas) / dfs); als = sqrt_r<R>((aaf - cc) / dfs); }

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

  const R sqPiRho = sqrt_r<R>(R(kPi) * Rho);
  const R sq2PiRho = sqrt_r<R>(R(k2Pi) * Rho);

  // left eigenvectors (non-zero entries only)
  R so15 = -R(1) / cc;
  R so33 = -hzz * sq2, so34 = hyy * sq2;
  R so37 = R(0.5) * hzz * sih / sq2PiRho, so38 = -R(0.5) * hyy * sih / sq2PiRho;
  // (-a)/b == -(a/b) exactly: the mirrored coefficients are negations
  R so47 = -so37, so48 = -so38;
  R so52 = R(0.5) * alf * af / cc;
  R so53 = -R(0.5) * als * as * hyy * sih / cc;
  R so54 = -R(0.5) * als * as * hzz * sih / cc;
  R so55 = R(0.5) * alf / (cc * Rho);
  R so57 = R(0.25) * als * hyy / (c * sqPiRho);
  R so58 = R(0.25) * als * hzz / (c * sqPiRho);
  R so62 = -so52;
  R so63 = -so53;
  R so64 = -so54;
  R so72 = R(0.5) * als * as / cc;
  R so73 = R(0.5) * alf * af * hyy * sih / cc;
  R so74 = R(0.5) * alf * af * hzz * sih / cc;
  R so75 = R(0.5) * als / (Rho * cc);
  R so77 = -R(0.25) * alf * hyy / (c * sqPiRho);
  R so78 = -R(0.25) * alf * hzz / (c * sqPiRho);
  R so82 = -so72;
  R so83 = -so73;
  R so84 = -so74;

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
    R coefRL = R(1) / (R(1) + sqrt_r<R>(RhoR / RhoL));
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
  R h = sqrt_r<R>(szb * szb - R(4) * A2 * bb);
  R aaf = R(0.5) * (szb + h);
  R af = sqrt_r<R>(aaf);
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
  R AL = sqrt_r<R>(gamma * PGasL / RhoL);
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
  R AR = sqrt_r<R>(gamma * PGasR / RhoR);
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


}  // namespace exact
}  // namespace mf
