// mf_sources.cuh - cell sources and cell-wise post-processing (always FP64):
// region classification, charge exchange, inner-sphere reset, positivity and
// the CFL wave speed.
//
// The region and sphere tests are thresholds on the primitive state; they use
// intrinsics that never fuse into multiply-adds so that each cell lands on the
// same side of every threshold as in the CPU restatement.
#pragma once

#include "mf_device.cuh"

namespace mf {
namespace fast {

constexpr double kInvPi = 0.318309886183790671537767526745028724;

// DEFINE_REGIONS_TRACER_4F (swlism/SWLISMF.ChF:839-1016), Cartesian: regtr
// is the region tracer of the cell (negative: solar wind).  The thresholds
// are the routine's literals.  Its x > 650 test reads the x of the last
// solar-wind cell the routine visited (x is assigned in that branch only);
// here the cell's own x, the same on every domain within x <= 650.
__device__ __forceinline__ int region_tracer_cell(const DevParams& P, double dx, int i, int j,
                                                  int k, const double* w, double regtr) {
  const double x = __dadd_rn(__dmul_rn(i + 0.5, dx), -P.sun_c[0]);
  const double ux = w[1], uy = w[2], uz = w[3];
  int reg;
  if (regtr < 0.0) {
    const double y = __dadd_rn(__dmul_rn(j + 0.5, dx), -P.sun_c[1]);
    double z = 0.0, r2, invr, ur;
    if (P.sd == 3) {
      z = __dadd_rn(__dmul_rn(k + 0.5, dx), -P.sun_c[2]);
      r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
      invr = __ddiv_rn(1.0, __dsqrt_rn(r2));
      ur = __dadd_rn(__dadd_rn(__dmul_rn(ux, __dmul_rn(x, invr)), __dmul_rn(uy, __dmul_rn(y, invr))),
                     __dmul_rn(uz, __dmul_rn(z, invr)));
    } else {
      r2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
      invr = __ddiv_rn(1.0, __dsqrt_rn(r2));
      ur = __dadd_rn(__dmul_rn(ux, __dmul_rn(x, invr)), __dmul_rn(uy, __dmul_rn(y, invr)));
    }
    if (fabs(ur) >= __dmul_rn(0.6, P.sun_v)) {
      const double TEMP = __ddiv_rn(__dmul_rn(P.t_coeff, w[4]), w[0]);
      reg = ((TEMP >= 1.0e6) && (r2 > __dmul_rn(P.sun_r, P.sun_r))) ? 2 : 3;
    } else {
      reg = 2;
    }
    if (P.sd == 3 && ((z < P.zbot) || (z > P.ztop))) reg = 4;
  } else {
    reg = 1;
    double vel = __dadd_rn(__dmul_rn(ux, ux), __dmul_rn(uy, uy));
    if (P.sd == 3) vel = __dadd_rn(vel, __dmul_rn(uz, uz));
    vel = __dsqrt_rn(vel);
    const double ang = __ddiv_rn(
        __dadd_rn(__dadd_rn(__dmul_rn(ux, P.lism_u[0]), __dmul_rn(uy, P.lism_u[1])),
                  __dmul_rn(uz, P.lism_u[2])),
        vel);
    const double TEMP = __ddiv_rn(__dmul_rn(P.t_coeff, w[4]), w[0]);
    if (w[0] > 1.2) reg = 4;
    if (vel < 0.8) reg = 4;
    if (ang < 0.95) reg = 4;
    if (TEMP > 9000.0) reg = 4;
    if (x > 650.0) reg = 1;
  }
  return reg;
}

// DEFINE_REGIONS_2F (swlism/SWLISMF.ChF:654-742), Cartesian branch, or the
// tracer variant above (HeliosphericProblem::defineRegions,
// swlism/HeliosphericProblem.cpp:2538-2575).
__device__ __forceinline__ int region_cell(const DevParams& P, double dx, int i, int j, int k,
                                           const double* w, double regtr) {
  if (P.reg_tracer) return region_tracer_cell(P, dx, i, j, k, w, regtr);
  const double x = __dadd_rn(__dmul_rn(i + 0.5, dx), -P.sun_c[0]);
  const double y = __dadd_rn(__dmul_rn(j + 0.5, dx), -P.sun_c[1]);
  double z = 0.0, r2, invr, ur;
  if (P.sd == 3) {
    z = __dadd_rn(__dmul_rn(k + 0.5, dx), -P.sun_c[2]);
    r2 = __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
    invr = __ddiv_rn(1.0, __dsqrt_rn(r2));
    ur = __dadd_rn(__dadd_rn(__dmul_rn(w[1], __dmul_rn(x, invr)), __dmul_rn(w[2], __dmul_rn(y, invr))),
                   __dmul_rn(w[3], __dmul_rn(z, invr)));
  } else {
    r2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
    invr = __ddiv_rn(1.0, __dsqrt_rn(r2));
    ur = __dadd_rn(__dmul_rn(w[1], __dmul_rn(x, invr)), __dmul_rn(w[2], __dmul_rn(y, invr)));
  }
  const double TEMP = __ddiv_rn(__dmul_rn(P.t_coeff, w[4]), w[0]);
  const double LIMSUN = __dmul_rn(0.6, P.sun_v);
  const double sunR2 = __dmul_rn(P.sun_r, P.sun_r);
  const bool zout = (P.sd == 3) && ((z < P.zbot) || (z > P.ztop));
  int reg;
  if (fabs(ur) >= LIMSUN) {
    reg = ((TEMP >= 1.0e6) && (r2 > sunR2)) ? 2 : 3;
    if (zout) reg = 1;
  } else if (TEMP >= P.tmlim) {
    reg = zout ? 1 : 2;
  } else {
    reg = 1;
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
// (HeliosphericProblem::explicitSource, swlism/HeliosphericProblem.cpp:1394-1539,
// CHARGE_EXCHANGE_4F swlism/ChargeExchange2F.ChF:673-993 and _MF :995-1149).
template <int IRHON>
__device__ __forceinline__ void charge_exchange_add(const DevParams& P, const double* w, int reg,
                                                    double dt, double* u) {
  const int nN = P.nf - 1;
  const double rho = w[0], ux = w[1], uy = w[2], uz = w[3];
  const double U2 = ux * ux + uy * uy + uz * uz;
  const double VVTP = w[4] / rho;
  double h2 = 0, h3 = 0, h4 = 0, h5 = 0, PPLUX = 0, PPLUY = 0, PPLUZ = 0, ENPLU = 0;
  double DENPLU[MF_MAX_FLUIDS], PMIX[MF_MAX_FLUIDS], PMIY[MF_MAX_FLUIDS], PMIZ[MF_MAX_FLUIDS],
      ENMI[MF_MAX_FLUIDS];
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f) {
    if (f > nN) break;
    const double* wn = w + IRHON + (f - 1) * 5;
    const double rhoN = wn[0], uxN = wn[1], uyN = wn[2], uzN = wn[3];
    const double dx_ = ux - uxN, dy_ = uy - uyN, dz_ = uz - uzN;
    const double UH2 = uxN * uxN + uyN * uyN + uzN * uzN;
    const double DU2 = dx_ * dx_ + dy_ * dy_ + dz_ * dz_;
    const double VPHH = dx_ * uxN + dy_ * uyN + dz_ * uzN;
    const double VPHP = dx_ * ux + dy_ * uy + dz_ * uz;
    const double VVTH = 2.0 * wn[4] / rhoN;
    // thermal + relative speeds; every argument is > 0, so sqrt(a) = a*rsqrt(a)
    const double aUD = (4.0 * kInvPi) * (VVTP + VVTH) + DU2;
    const double UD = aUD * rsqrt(aUD);
    const double iUPM = rsqrt((16.0 * kInvPi) * VVTP + (2.25 * kPi) * VVTH + 4.0 * DU2);
    const double iUHM = rsqrt((2.25 * kPi) * VVTP + (16.0 * kInvPi) * VVTH + 4.0 * DU2);
    const double aPE = kInvPi * (4.0 * VVTP + (64.0 / 9.0) * VVTH) + DU2;
    const double UPE = aPE * rsqrt(aPE);
    const double aHE = kInvPi * ((64.0 / 9.0) * VVTP + 4.0 * VVTH) + DU2;
    const double UHE = aHE * rsqrt(aHE);
    const double UDS = P.ce_scale_vel * UD;
    const double t = P.ce_a - P.ce_b * log(UDS);
    double SIG = t * t;
    if (P.ce_damp_c > 0.0) SIG = SIG * pow(1.0 - exp(-P.ce_damp_c / UDS), P.ce_damp_pow);
    const double ARR = P.ce_sigma_scale * SIG * rhoN * rho;
    const double VVTHU = VVTH * iUPM;
    const double VP_UHM = VVTP * iUHM;
    const double hv = ARR * (UD + VVTHU + VP_UHM);
    h2 = h2 + hv * dx_;
    h3 = h3 + hv * dy_;
    h4 = h4 + hv * dz_;
    h5 = h5 + 0.5 * ARR *
                  (1.5 * (UHE * VVTP - UPE * VVTH) + UD * (U2 - UH2) +
                   2.0 * (VVTHU * VPHH + VPHP * VP_UHM));
    DENPLU[f] = -ARR * UD;
    PPLUX = PPLUX - ARR * (ux * UD + dx_ * VP_UHM);
    PPLUY = PPLUY - ARR * (uy * UD + dy_ * VP_UHM);
    PPLUZ = PPLUZ - ARR * (uz * UD + dz_ * VP_UHM);
    ENPLU = ENPLU - ARR * (0.5 * U2 * UD + VPHP * VP_UHM + 0.75 * VVTP * UHE);
    PMIX[f] = ARR * (uxN * UD - dx_ * VVTHU);
    PMIY[f] = ARR * (uyN * UD - dy_ * VVTHU);
    PMIZ[f] = ARR * (uzN * UD - dz_ * VVTHU);
    ENMI[f] = ARR * (0.5 * UH2 * UD - VPHH * VVTHU + 0.75 * VVTH * UPE);
  }
  u[1] = u[1] - dt * h2;
  u[2] = u[2] - dt * h3;
  u[3] = u[3] - dt * h4;
  u[4] = u[4] - dt * h5;
  // S of the magnetic field (and of psi) is zero
  const int rk = ce_recipient(nN, reg);
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f) {
    if (f > nN) break;
    double H1, H2, H3, H4, H5;
    if (f == rk) {
      if (nN <= 3) {
        H1 = 0.0;
#pragma unroll
        for (int q = 1; q < MF_MAX_FLUIDS; ++q)
          if (q <= nN && q != f) H1 = H1 + DENPLU[q];
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
    un[0] = un[0] - dt * H1;
    un[1] = un[1] - dt * H2;
    un[2] = un[2] - dt * H3;
    un[3] = un[3] - dt * H4;
    un[4] = un[4] - dt * H5;
  }
}

// HELIOREINIT_DEFAULT (swlism/HeliosphericPlasmaBCF.ChF:1435-1555) with a
// monopolar field: the plasma in r <= Rinit becomes the radial wind.  The
// membership test uses non-fused arithmetic (host and device agree exactly).
__device__ __host__ inline void reinit_cell(const DevParams& P, double dx, int i, int j, int k,
                                            double* u) {
#ifdef __CUDA_ARCH__
  const double x = __dadd_rn(__dmul_rn(i + 0.5, dx), -P.sun_c[0]);
  const double y = __dadd_rn(__dmul_rn(j + 0.5, dx), -P.sun_c[1]);
  const double z = (P.sd == 3) ? __dadd_rn(__dmul_rn(k + 0.5, dx), -P.sun_c[2]) : 0.0;
  const double r2 = (P.sd == 3)
                        ? __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z))
                        : __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
  if (!(r2 <= __dmul_rn(P.r0, P.r0))) return;
#else
  const double x = (i + 0.5) * dx - P.sun_c[0];
  const double y = (j + 0.5) * dx - P.sun_c[1];
  const double z = (P.sd == 3) ? (k + 0.5) * dx - P.sun_c[2] : 0.0;
  const double r2 = (P.sd == 3) ? (x * x + y * y + z * z) : (x * x + y * y);
  if (!(r2 <= P.r0 * P.r0)) return;
#endif
  const double r = sqrt(r2);
  const double rr = r / P.rint;
  const double xy = sqrt(x * x + y * y);
  const double cosT = z / r;
  const double sinT = sqrt(fmax(0.0, 1.0 - cosT * cosT));
  const double cosF = x / xy;
  const double sinF = y / xy;
  const double rho = P.sun_rho / (rr * rr);
  const double ux = P.sun_v * sinT * cosF;
  const double uy = P.sun_v * sinT * sinF;
  const double uz = P.sun_v * cosT;
  const double pr = P.sun_p / pow(rr, 2.0 * P.gamma);
  const double br = P.dir_br * P.sun_b / (rr * rr);
  const double bp = -P.sun_beta * br * r * sinT;
  const double bx = br * sinT * cosF - bp * sinF;
  const double by = br * sinT * sinF + bp * cosF;
  const double bz = br * cosT;
  const double b = bx * bx + by * by + bz * bz;
  const double e0 = pr / P.hgamma + 0.5 * (rho * P.sun_v * P.sun_v + kInv4Pi * b);
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
  const double hg = P.hgamma, ihg = P.invhgamma, smallR = P.smallr, smallP = P.smallp;
  if (P.nf == 1) {
    double Rho = u[0];
    bool was = false;
    if (Rho < smallR) { Rho = smallR; was = true; }
    const double invRho = 1.0 / Rho;
    const double Ux = u[1] * invRho, Uy = u[2] * invRho, Uz = u[3] * invRho;
    const double BxB = kInv8Pi * (u[5] * u[5] + u[6] * u[6] + u[7] * u[7]);
    const double UxU = 0.5 * (Ux * Ux + Uy * Uy + Uz * Uz);
    double Pr = hg * (u[4] - BxB - Rho * UxU);
    if (Pr < smallP) { Pr = smallP; was = true; }
    if (was) {
      u[0] = Rho;
      u[4] = Pr * ihg + Rho * UxU + BxB;
    }
    return;
  }
  {
    const double Rho0 = u[0];
    const double invRho = 1.0 / Rho0;
    const double Ux = u[1] * invRho, Uy = u[2] * invRho, Uz = u[3] * invRho;
    const double BxB = kInv8Pi * (u[5] * u[5] + u[6] * u[6] + u[7] * u[7]);
    const double UxU = 0.5 * (Ux * Ux + Uy * Uy + Uz * Uz);
    double Pr = hg * (u[4] - BxB - Rho0 * UxU);
    double Rho = Rho0;
    bool was = false;
    if (Rho < smallR) { Rho = smallR; was = true; }
    if (Pr < smallP) { Pr = smallP; was = true; }
    if (was) {
      u[0] = Rho;
      u[1] = Rho * Ux;
      u[2] = Rho * Uy;
      u[3] = Rho * Uz;
      u[4] = Pr * ihg + Rho * UxU + BxB;
    }
  }
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f) {
    if (f >= P.nf) break;
    const double fd = (f == 1) ? smallR : (f == 3) ? kNet3Dens : kNet2Dens;
    const double fp = (f == 1) ? smallP : (f == 3) ? kNet3Pres : kNet2Pres;
    double* un = u + IRHON + (f - 1) * 5;
    const double Rho0 = un[0];
    const double invRho = 1.0 / Rho0;
    const double Ux = un[1] * invRho, Uy = un[2] * invRho, Uz = un[3] * invRho;
    const double UxU = 0.5 * (Ux * Ux + Uy * Uy + Uz * Uz);
    double Pr = hg * (un[4] - Rho0 * UxU);
    double Rho = Rho0;
    bool was = false;
    if (Rho < fd) { Rho = fd; was = true; }
    if (Pr < fp) { Pr = fp; was = true; }
    if (was) {
      un[0] = Rho;
      un[1] = Rho * Ux;
      un[2] = Rho * Uy;
      un[3] = Rho * Uz;
      un[4] = Pr * ihg + Rho * UxU;
    }
  }
}

// MAXWAVESPEED (srcIdeal/PatchIdealMHDF.ChF:5-63) + MAXWAVESPEED_E
// (srcIdeal/PatchEulerF.ChF:5-50) of one cell.
template <int IRHON>
__device__ __forceinline__ double max_wave_speed(const DevParams& P, const double* u) {
  double cmax = 0.0;
  {
    const double invrho = 1.0 / u[0];
    const double uu = u[1] * invrho, vv = u[2] * invrho, ww = u[3] * invrho;
    const double ke = u[1] * uu + u[2] * vv + u[3] * ww;
    const double bx = u[5], by = u[6], bz = u[7];
    const double b = kInv4Pi * (bx * bx + by * by + bz * bz);
    double p = P.hgamma * (u[4] - 0.5 * (ke + b));
    p = fmax(p, P.smallp);
    const double a2 = P.gamma * p * invrho;
    const double as2 = 0.5 * (a2 + invrho * b);
    const double as4 = as2 * as2;
    const double k4 = kInv4Pi * invrho * a2;
    // as4 - k4 b^2 >= 0 exactly; contracted rounding can push it below 0
    double umax = fabs(uu) + sqrt(as2 + sqrt(fmax(0.0, as4 - k4 * bx * bx)));
    umax = fmax(fabs(vv) + sqrt(as2 + sqrt(fmax(0.0, as4 - k4 * by * by))), umax);
    umax = fmax(fabs(ww) + sqrt(as2 + sqrt(fmax(0.0, as4 - k4 * bz * bz))), umax);
    cmax = fmax(umax, cmax);
  }
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f) {
    if (f >= P.nf) break;
    const double* un = u + IRHON + (f - 1) * 5;
    const double rho = fmax(un[0], P.smallr);
    const double invrho = 1.0 / rho;
    const double uu = un[1] * invrho, vv = un[2] * invrho, ww = un[3] * invrho;
    const double ke = un[1] * uu + un[2] * vv + un[3] * ww;
    double p = P.hgamma * (un[4] - 0.5 * ke);
    p = fmax(p, P.smallp);
    const double a = sqrt(P.gamma * p * invrho);
    const double umax = fmax(fmax(fabs(uu), fabs(vv)), fabs(ww)) + a;
    cmax = fmax(umax, cmax);
  }
  return cmax;
}

}  // namespace fast
}  // namespace mf
