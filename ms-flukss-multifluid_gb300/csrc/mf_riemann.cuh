// mf_riemann.cuh - face fluxes: Roe 8/7-wave MHD, Rusanov MHD, Dedner (GLM)
// 2x2 system and van Leer flux-vector splitting of the neutral fluids.
//
// Each routine computes the same fluxes as the cited reference kernel.  The
// FP64 budget of GB300 makes every FP64 instruction count, so repeated
// divisions by one denominator become one reciprocal and multiplications,
// square roots that are also needed as reciprocals come from rsqrt, and the
// structurally zero entries of the 8x8 eigenmatrices are skipped.  These
// change results only at the rounding level (continuous functions of their
// inputs); the limiter and region decisions upstream stay bit-exact.
#pragma once

#include "mf_device.cuh"

namespace mf {
namespace fast {

template <typename R> __device__ __forceinline__ R rrsqrt(R a);
template <> __device__ __forceinline__ double rrsqrt<double>(double a) { return rsqrt(a); }
template <> __device__ __forceinline__ float rrsqrt<float>(float a) { return rsqrtf(a); }

// RIEMANNF (src/Roe8WaveF.ChF:5-601) and RIEMANN7F (src/Roe7WaveF.ChF:5-558).
// wl/wr: rho,u,v,w,p,bx,by,bz in the global frame; g: fluxes in that order.
// SEVEN drops the normal-B wave (RIEMANN7F), whose normal-B flux is zero.
template <typename R, int DIR, bool SEVEN>
__device__ __forceinline__ void roe_mhd(const DevParams& P, const R* wl, const R* wr, R* g) {
  constexpr int in = 1 + DIR, it1 = 1 + (DIR + 1) % 3, it2 = 1 + (DIR + 2) % 3;
  constexpr int inB = 5 + DIR, it1B = 5 + (DIR + 1) % 3, it2B = 5 + (DIR + 2) % 3;
  const R gamma = R(P.gamma), hgamma = R(P.hgamma), ihg = R(P.invhgamma);
  const R smallp = R(P.smallp), smallr = R(P.smallr);
  const R i4pi = R(kInv4Pi), i8pi = R(kInv8Pi), sq2 = R(kSqrtHalf);

  const R PGasL = rmax<R>(smallp, wl[4]), RhoL = rmax<R>(smallr, wl[0]);
  const R UL = wl[in], VL = wl[it1], WL = wl[it2];
  const R BXL = wl[inB], BYL = wl[it1B], BZL = wl[it2B];
  const R PGasR = rmax<R>(smallp, wr[4]), RhoR = rmax<R>(smallr, wr[0]);
  const R UR = wr[in], VR = wr[it1], WR = wr[it2];
  const R BXR = wr[inB], BYR = wr[it1B], BZR = wr[it2B];
  const R iRhoL = R(1) / RhoL, iRhoR = R(1) / RhoR;

  const R RUL = RhoL * UL, RVL = RhoL * VL, RWL = RhoL * WL;
  const R BxBL = i8pi * (BXL * BXL + BYL * BYL + BZL * BZL);
  const R PL = PGasL + BxBL;
  const R EL = PGasL * ihg + R(0.5) * (RUL * UL + RVL * VL + RWL * WL) + BxBL;
  const R AL2 = gamma * PGasL * iRhoL;
  const R RUR = RhoR * UR, RVR = RhoR * VR, RWR = RhoR * WR;
  const R BxBR = i8pi * (BXR * BXR + BYR * BYR + BZR * BZR);
  const R PR = PGasR + BxBR;
  const R ER = PGasR * ihg + R(0.5) * (RUR * UR + RVR * VR + RWR * WR) + BxBR;
  const R AR2 = gamma * PGasR * iRhoR;
  const R ccmi = (AL2 > AR2) ? AR2 : AL2;
  const R ccma = (AL2 > AR2) ? AL2 : AR2;

  R Rho, U, V, W, BX, BY, BZ, BX2, BYZ2, BxBH, kk, cc, iRho;
  if (P.aver == 1) {
    const R HL = (EL + PL) * iRhoL, HR = (ER + PR) * iRhoR;
    const R coefRL = R(1) / (R(1) + sqrt(RhoR * iRhoL));
    const R coefRR = R(1) - coefRL;
    Rho = RhoR * coefRL + RhoL * coefRR;
    iRho = R(1) / Rho;
    U = UL * coefRL + UR * coefRR;
    V = VL * coefRL + VR * coefRR;
    W = WL * coefRL + WR * coefRR;
    const R HAV = HL * coefRL + HR * coefRR;
    BX = BXR * coefRL + BXL * coefRR;
    BY = BYR * coefRL + BYL * coefRR;
    BZ = BZR * coefRL + BZL * coefRR;
    const R BXAV = R(0.5) * (BXL + BXR);
    BX2 = BXAV * BXAV;
    BYZ2 = BY * BY + BZ * BZ;
    BxBH = i8pi * (BX2 + BYZ2);
    kk = R(0.5) * (U * U + V * V + W * W);
    const R DBX = BXR - BXL, DBY = BYR - BYL, DBZ = BZR - BZL;
    const R X = i8pi * (DBX * DBX + DBY * DBY + DBZ * DBZ) * coefRL * coefRL * iRhoL;
    cc = hgamma * (HAV - kk - i4pi * (BX * BXAV + BYZ2) * iRho) + (R(2) - gamma) * X;
  } else {
    Rho = R(0.5) * (RhoL + RhoR);
    iRho = R(1) / Rho;
    U = R(0.5) * (UL + UR);
    V = R(0.5) * (VL + VR);
    W = R(0.5) * (WL + WR);
    BX = R(0.5) * (BXL + BXR);
    BY = R(0.5) * (BYL + BYR);
    BZ = R(0.5) * (BZL + BZR);
    BX2 = BX * BX;
    BYZ2 = BY * BY + BZ * BZ;
    BxBH = i8pi * (BX2 + BYZ2);
    kk = R(0.5) * (U * U + V * V + W * W);
    cc = gamma * (R(0.5) * (PL + PR) - BxBH) * iRho;
  }

  const R bb = i4pi * BX2 * iRho;
  const R b = sqrt(bb);
  if (cc < ccmi) cc = ccmi;
  if (cc > ccma) cc = ccma;
  const R ic = rrsqrt<R>(cc);
  const R c = cc * ic;
  const R icc = ic * ic;

  R hyy, hzz, aaf, aas, af, as;
  const R smallB = R(P.smallB);
  if (BYZ2 < smallB * smallB) {
    hyy = sq2;
    hzz = sq2;
    if (bb > cc) { aaf = bb; aas = cc; af = b; as = c; }
    else { aaf = cc; aas = bb; af = c; as = b; }
  } else {
    const R ihyz = rrsqrt<R>(BYZ2);
    hyy = BY * ihyz;
    hzz = BZ * ihyz;
    const R szb = cc + (BxBH + BxBH) * iRho;
    // szb^2 - 4 cc bb >= 0 exactly; rounding (FP32 above all) can make it
    // slightly negative where cc ~ bb and the transverse field is weak
    const R h = sqrt(rmax<R>(R(0), szb * szb - R(4) * cc * bb));
    aas = R(0.5) * (szb - h);
    if (aas <= R(0)) { aas = R(0); as = R(0); }
    else if (aas >= cc) { aas = cc; as = c; }
    else { as = sqrt(aas); }
    aaf = R(0.5) * (szb + h);
    if (aaf <= cc) { aaf = cc; af = c; }
    else { af = sqrt(aaf); }
  }

  // entropy-fixed speeds (1 entropy, 2 div-B, 3/4 Alfven, 5/6 fast, 7/8 slow)
  const R eigmax = rabs<R>(U) + rabs<R>(V) + rabs<R>(W) + af;
  const R del = R(P.del2) * eigmax;
  const R dell2 = del * del;
  const R hdel = R(0.5) / del;
  auto fix = [&](R e) -> R {
    const R z = rabs<R>(e);
    return (z >= del) ? z : (z * z + dell2) * hdel;
  };
  const R A1 = fix(U);
  const R A3 = fix(U + b), A4 = fix(U - b);
  const R A5 = fix(U + af), A6 = fix(U - af);
  const R A7 = fix(U + as), A8 = fix(U - as);

  R alf, als;
  const R dfs = aaf - aas;
  // Near the triple point (aaf ~ cc ~ aas) cc - aas and aaf - cc are
  // differences of nearly equal numbers.  The reference's absolute 1e-8
  // cut-off suits FP64 rounding; in FP32 dfs can sit far above it and still be
  // rounding noise, so the fast path also treats dfs below a few FP32 ulps of
  // aaf as degenerate, and renormalises so that alf^2 + als^2 = 1 (the
  // condition under which the left and right eigenvectors stay inverse).
  const R dfs_tol = (sizeof(R) == 4) ? rmax<R>(R(1.0e-8), R(4.0e-6) * aaf) : R(1.0e-8);
  if (dfs < dfs_tol) { alf = R(1); als = R(0); }
  else if ((cc - aas) <= R(0)) { alf = R(0); als = R(1); }
  else if ((aaf - cc) <= R(0)) { alf = R(1); als = R(0); }
  else {
    const R a2f = cc - aas, a2s = aaf - cc;
    const R inorm = rrsqrt<R>(a2f + a2s);
    alf = sqrt(a2f) * inorm;
    als = sqrt(a2s) * inorm;
  }
  const R sih = (BX >= R(0)) ? R(1) : R(-1);

  const R fl1 = RUL;
  const R fl2 = UL * RUL - BXL * BXL * i4pi + PL;
  const R fl3 = UL * RVL - BXL * BYL * i4pi;
  const R fl4 = UL * RWL - BXL * BZL * i4pi;
  const R fl5 = UL * (EL + PL) - BXL * (UL * BXL + VL * BYL + WL * BZL) * i4pi;
  const R fl7 = UL * BYL - BXL * VL;
  const R fl8 = UL * BZL - BXL * WL;
  const R fr1 = RUR;
  const R fr2 = UR * RUR - BXR * BXR * i4pi + PR;
  const R fr3 = UR * RVR - BXR * BYR * i4pi;
  const R fr4 = UR * RWR - BXR * BZR * i4pi;
  const R fr5 = UR * (ER + PR) - BXR * (UR * BXR + VR * BYR + WR * BZR) * i4pi;
  const R fr7 = UR * BYR - BXR * VR;
  const R fr8 = UR * BZR - BXR * WR;

  const R du1 = RhoL - RhoR;
  const R du6 = BXL - BXR;
  const R du7 = BYL - BYR;
  const R du8 = BZL - BZR;
  const R bdot = SEVEN ? (BY * du7 + BZ * du8) : (BX * du6 + BY * du7 + BZ * du8);
  const R du5 = -hgamma * (-kk * du1 + U * (RUL - RUR) + V * (RVL - RVR) + W * (RWL - RWR) -
                           (EL - ER) + bdot * i4pi);
  const R du2 = (-U * du1 + (RUL - RUR)) * iRho;
  const R du3 = (-V * du1 + (RVL - RVR)) * iRho;
  const R du4 = (-W * du1 + (RWL - RWR)) * iRho;

  const R sqPiRho = sqrt(R(kPi) * Rho);
  const R isq2 = R(kSqrtHalf) / sqPiRho;  // 1 / sqrt(2 pi rho)
  const R icsq = ic / sqPiRho;            // 1 / (c sqrt(pi rho))
  const R sq2PiRho = sqPiRho * R(1.41421356237309504880);

  const R aff = alf * af, ass = als * as;
  const R hys = hyy * sih, hzs = hzz * sih;
  // left eigenvectors (non-zero entries)
  const R so15 = -icc;
  const R so33 = -hzz * sq2, so34 = hyy * sq2;
  const R so37 = R(0.5) * hzs * isq2, so38 = -R(0.5) * hys * isq2;
  const R so52 = R(0.5) * aff * icc;
  const R so53 = -R(0.5) * ass * hys * icc;
  const R so54 = -R(0.5) * ass * hzs * icc;
  const R so55 = R(0.5) * alf * icc * iRho;
  const R so57 = R(0.25) * als * hyy * icsq;
  const R so58 = R(0.25) * als * hzz * icsq;
  const R so72 = R(0.5) * ass * icc;
  const R so73 = R(0.5) * aff * hys * icc;
  const R so74 = R(0.5) * aff * hzs * icc;
  const R so75 = R(0.5) * als * icc * iRho;
  const R so77 = -R(0.25) * alf * hyy * icsq;
  const R so78 = -R(0.25) * alf * hzz * icsq;

  const R t34 = so33 * du3 + so34 * du4;
  const R t78 = so37 * du7 + so38 * du8;
  const R lu1 = A1 * (du1 + so15 * du5);
  const R lu3 = A3 * (t34 + t78);
  const R lu4 = A4 * (t34 - t78);
  const R f5 = so52 * du2 + so53 * du3 + so54 * du4;
  const R g5 = so55 * du5 + so57 * du7 + so58 * du8;
  const R lu5 = A5 * (f5 + g5);
  const R lu6 = A6 * (g5 - f5);
  const R f7 = so72 * du2 + so73 * du3 + so74 * du4;
  const R g7 = so75 * du5 + so77 * du7 + so78 * du8;
  const R lu7 = A7 * (f7 + g7);
  const R lu8 = A8 * (g7 - f7);

  // right eigenvectors (non-zero entries)
  const R l56 = lu5 + lu6, d56 = lu5 - lu6;
  const R l78 = lu7 + lu8, d78 = lu7 - lu8;
  const R l34 = lu3 + lu4;
  R ra1 = lu1 + Rho * (alf * l56 + als * l78);
  R ra2 = aff * d56 + ass * d78;
  R ra3 = -hzz * sq2 * l34 - ass * hys * d56 + aff * hys * d78;
  R ra4 = hyy * sq2 * l34 - ass * hzs * d56 + aff * hzs * d78;
  R ra5 = Rho * cc * (alf * l56 + als * l78);
  const R two_sqc = R(2) * sqPiRho * c;
  const R ra7 = hzs * sq2PiRho * (lu3 - lu4) + two_sqc * hyy * (als * l56 - alf * l78);
  const R ra8 = -hys * sq2PiRho * (lu3 - lu4) + two_sqc * hzz * (als * l56 - alf * l78);

  if (SEVEN)
    ra5 = ra1 * kk + Rho * (U * ra2 + V * ra3 + W * ra4) + ra5 * ihg + i4pi * (BY * ra7 + BZ * ra8);
  else
    ra5 = ra1 * kk + Rho * (U * ra2 + V * ra3 + W * ra4) + ra5 * ihg +
          i4pi * (BX * (fix(U) * du6) + BY * ra7 + BZ * ra8);
  ra2 = U * ra1 + Rho * ra2;
  ra3 = V * ra1 + Rho * ra3;
  ra4 = W * ra1 + Rho * ra4;

  g[0] = R(0.5) * (fl1 + fr1 + ra1);
  g[in] = R(0.5) * (fl2 + fr2 + ra2);
  g[it1] = R(0.5) * (fl3 + fr3 + ra3);
  g[it2] = R(0.5) * (fl4 + fr4 + ra4);
  g[4] = R(0.5) * (fl5 + fr5 + ra5);
  g[inB] = SEVEN ? R(0) : R(0.5) * (fix(U) * du6);
  g[it1B] = R(0.5) * (fl7 + fr7 + ra7);
  g[it2B] = R(0.5) * (fl8 + fr8 + ra8);
}

// RUSANOVF (src/RusanovF.ChF:4-197)
template <typename R, int DIR>
__device__ __forceinline__ void rusanov_mhd(const DevParams& P, const R* wl, const R* wr, R* g) {
  constexpr int in = 1 + DIR, it1 = 1 + (DIR + 1) % 3, it2 = 1 + (DIR + 2) % 3;
  constexpr int inB = 5 + DIR, it1B = 5 + (DIR + 1) % 3, it2B = 5 + (DIR + 2) % 3;
  const R gamma = R(P.gamma), hgamma = R(P.hgamma), ihg = R(P.invhgamma);
  const R i4pi = R(kInv4Pi), i8pi = R(kInv8Pi);
  const R PGasL = rmax<R>(R(P.smallp), wl[4]), RhoL = rmax<R>(R(P.smallr), wl[0]);
  const R UL = wl[in], VL = wl[it1], WL = wl[it2];
  const R BXL = wl[inB], BYL = wl[it1B], BZL = wl[it2B];
  const R PGasR = rmax<R>(R(P.smallp), wr[4]), RhoR = rmax<R>(R(P.smallr), wr[0]);
  const R UR = wr[in], VR = wr[it1], WR = wr[it2];
  const R BXR = wr[inB], BYR = wr[it1B], BZR = wr[it2B];
  const R RUL = RhoL * UL, RVL = RhoL * VL, RWL = RhoL * WL;
  const R BxBL = i8pi * (BXL * BXL + BYL * BYL + BZL * BZL);
  const R PL = PGasL + BxBL;
  const R EL = PGasL * ihg + R(0.5) * (RUL * UL + RVL * VL + RWL * WL) + BxBL;
  const R BXL_4PI = BXL * i4pi;
  const R RUR = RhoR * UR, RVR = RhoR * VR, RWR = RhoR * WR;
  const R BxBR = i8pi * (BXR * BXR + BYR * BYR + BZR * BZR);
  const R PR = PGasR + BxBR;
  const R ER = PGasR * ihg + R(0.5) * (RUR * UR + RVR * VR + RWR * WR) + BxBR;
  const R BXR_4PI = BXR * i4pi;
  R Rho, U, BX2, BxBH, A2, iRho;
  if (P.aver == 1) {
    const R iRhoL = R(1) / RhoL, iRhoR = R(1) / RhoR;
    const R HL = (EL + PL) * iRhoL, HR = (ER + PR) * iRhoR;
    const R coefRL = R(1) / (R(1) + sqrt(RhoR * iRhoL));
    const R coefRR = R(1) - coefRL;
    Rho = RhoR * coefRL + RhoL * coefRR;
    iRho = R(1) / Rho;
    U = UL * coefRL + UR * coefRR;
    const R V = VL * coefRL + VR * coefRR;
    const R W = WL * coefRL + WR * coefRR;
    const R HAV = HL * coefRL + HR * coefRR;
    const R BX = BXR * coefRL + BXL * coefRR;
    const R BY = BYR * coefRL + BYL * coefRR;
    const R BZ = BZR * coefRL + BZL * coefRR;
    const R BXAV = R(0.5) * (BXL + BXR);
    BX2 = BXAV * BXAV;
    const R BYZ2 = BY * BY + BZ * BZ;
    BxBH = i8pi * (BX2 + BYZ2);
    const R kk = R(0.5) * (U * U + V * V + W * W);
    const R DBX = BXR - BXL, DBY = BYR - BYL, DBZ = BZR - BZL;
    const R X = i8pi * (DBX * DBX + DBY * DBY + DBZ * DBZ) * coefRL * coefRL * iRhoL;
    A2 = hgamma * (HAV - kk - i4pi * (BX * BXAV + BYZ2) * iRho) + (R(2) - gamma) * X;
  } else {
    Rho = R(0.5) * (RhoL + RhoR);
    iRho = R(1) / Rho;
    U = R(0.5) * (UL + UR);
    const R BX = R(0.5) * (BXL + BXR), BY = R(0.5) * (BYL + BYR), BZ = R(0.5) * (BZL + BZR);
    BX2 = BX * BX;
    BxBH = i8pi * (BX2 + BY * BY + BZ * BZ);
    A2 = gamma * R(0.5) * (PGasL + PGasR) * iRho;
  }
  const R bb = i4pi * BX2 * iRho;
  const R szb = A2 + (BxBH + BxBH) * iRho;
  const R h = sqrt(rmax<R>(R(0), szb * szb - R(4) * A2 * bb));
  const R em = rabs<R>(U) + sqrt(R(0.5) * (szb + h));
  g[0] = R(0.5) * (RUL + RUR + em * (RhoL - RhoR));
  g[in] = R(0.5) * ((UL * RUL - BXL_4PI * BXL + PL) + (UR * RUR - BXR_4PI * BXR + PR) + em * (RUL - RUR));
  g[it1] = R(0.5) * ((UL * RVL - BXL_4PI * BYL) + (UR * RVR - BXR_4PI * BYR) + em * (RVL - RVR));
  g[it2] = R(0.5) * ((UL * RWL - BXL_4PI * BZL) + (UR * RWR - BXR_4PI * BZR) + em * (RWL - RWR));
  g[4] = R(0.5) * ((UL * (EL + PL) - BXL_4PI * (UL * BXL + VL * BYL + WL * BZL)) +
                   (UR * (ER + PR) - BXR_4PI * (UR * BXR + VR * BYR + WR * BZR)) + em * (EL - ER));
  g[inB] = R(0.5) * (em * (BXL - BXR));
  g[it1B] = R(0.5) * ((UL * BYL - BXL * VL) + (UR * BYR - BXR * VR) + em * (BYL - BYR));
  g[it2B] = R(0.5) * ((UL * BZL - BXL * WL) + (UR * BZR - BXR * WR) + em * (BZL - BZR));
}

// DEDNER2X2F (src/DednerF.ChF:89-170): Bn and psi fluxes with speed ch.
template <typename R>
__device__ __forceinline__ void dedner_2x2(R ch, R bxl, R psil, R bxr, R psir, R& fbn, R& fpsi) {
  // ra1 = ch*(bxl-bxr), ra2 = ch*(psil-psir) after the eigen-projection
  fbn = R(0.5) * (psil + psir + ch * (bxl - bxr));
  fpsi = R(0.5) * (ch * ch * (bxl + bxr) + ch * (psil - psir));
}

// VANLEERF (src/VanLeerRSF.ChF:4-130): wl/wr = rho,u,v,w,p of one Euler fluid.
template <typename R, int DIR>
__device__ __forceinline__ void vanleer_euler(const DevParams& P, const R* wl, const R* wr, R* g) {
  constexpr int in = 1 + DIR, it1 = 1 + (DIR + 1) % 3, it2 = 1 + (DIR + 2) % 3;
  const R gamma = R(P.gamma), ihg = R(P.invhgamma), igam = R(P.invgamma);
  R fl1, fl2, fl3, fl4, fl5, fr1, fr2, fr3, fr4, fr5;
  {
    const R PGas = rmax<R>(R(P.smallp), wl[4]), Rho = rmax<R>(R(P.smallr), wl[0]);
    const R Uu = wl[in], Vv = wl[it1], Ww = wl[it2];
    const R iRho = R(1) / Rho;
    const R E = PGas * ihg + R(0.5) * Rho * (Uu * Uu + Vv * Vv + Ww * Ww);
    const R a2 = gamma * PGas * iRho;
    const R ia = rrsqrt<R>(a2);
    const R A = a2 * ia;
    if (Uu <= -A) {
      fr1 = fr2 = fr3 = fr4 = fr5 = R(0);
    } else if (Uu >= A) {
      fr1 = Rho * Uu;
      fr2 = fr1 * Uu + PGas;
      fr3 = fr1 * Vv;
      fr4 = fr1 * Ww;
      fr5 = Uu * (E + PGas);
    } else {
      const R HU = Uu + A;
      fr1 = R(0.25) * Rho * HU * HU * ia;
      fr2 = fr1 * (Uu + (-Uu + (A + A)) * igam);
      fr3 = fr1 * Vv;
      fr4 = fr1 * Ww;
      fr5 = fr1 * ((E + PGas) * iRho);
    }
  }
  {
    const R PGas = rmax<R>(R(P.smallp), wr[4]), Rho = rmax<R>(R(P.smallr), wr[0]);
    const R Uu = wr[in], Vv = wr[it1], Ww = wr[it2];
    const R iRho = R(1) / Rho;
    const R E = PGas * ihg + R(0.5) * Rho * (Uu * Uu + Vv * Vv + Ww * Ww);
    const R a2 = gamma * PGas * iRho;
    const R ia = rrsqrt<R>(a2);
    const R A = a2 * ia;
    if (Uu >= A) {
      fl1 = fl2 = fl3 = fl4 = fl5 = R(0);
    } else if (Uu <= -A) {
      fl1 = Rho * Uu;
      fl2 = fl1 * Uu + PGas;
      fl3 = fl1 * Vv;
      fl4 = fl1 * Ww;
      fl5 = Uu * (E + PGas);
    } else {
      const R HU = Uu - A;
      fl1 = -R(0.25) * Rho * HU * HU * ia;
      fl2 = fl1 * (Uu + (-Uu - (A + A)) * igam);
      fl3 = fl1 * Vv;
      fl4 = fl1 * Ww;
      fl5 = fl1 * ((E + PGas) * iRho);
    }
  }
  g[0] = fl1 + fr1;
  g[in] = fl2 + fr2;
  g[it1] = fl3 + fr3;
  g[it2] = fl4 + fr4;
  g[4] = fl5 + fr5;
}

}  // namespace fast
}  // namespace mf
