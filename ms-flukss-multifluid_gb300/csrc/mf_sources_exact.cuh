// mf_sources_exact.cuh - cell sources and post-processing of the FP64 parity
// path (region classification, charge exchange, inner-sphere reset,
// positivity, CFL wave speed) in the reference's evaluation order.  Compiled
// without multiply-add contraction.
#pragma once

#include "mf_device.cuh"

namespace mf {
namespace exact {

// ---------------------------------------------------------------------------
// DEFINE_REGIONS_TRACER_4F (swlism/SWLISMF.ChF:839-1016), Cartesian: regtr
// is the region tracer of the cell (negative: solar wind).  The thresholds
// are the routine's literals.  Its x > 650 test reads the x of the last
// solar-wind cell the routine visited (x is assigned in that branch only);
// here the cell's own x, the same on every domain within x <= 650.
__device__ __forceinline__ int region_tracer_cell(const DevParams& P, double dx, int i, int j,
                                                  int k, const double* w, double regtr) {
  const double x = (i + 0.5) * dx - P.sun_c[0];
  const double ux = w[1], uy = w[2], uz = w[3];
  int reg;
  if (regtr < 0.0) {
    const double y = (j + 0.5) * dx - P.sun_c[1];
    double z = 0.0, r2, invr, ur;
    if (P.sd == 3) {
      z = (k + 0.5) * dx - P.sun_c[2];
      r2 = x * x + y * y + z * z;
      invr = 1.0 / sqrt(r2);
      ur = ux * (x * invr) + uy * (y * invr) + uz * (z * invr);
    } else {
      r2 = x * x + y * y;
      invr = 1.0 / sqrt(r2);
      ur = ux * (x * invr) + uy * (y * invr);
    }
    if (fabs(ur) >= 0.6 * P.sun_v) {
      const double TEMP = P.t_coeff * w[4] / w[0];
      reg = ((TEMP >= 1.0e6) && (r2 > P.sun_r * P.sun_r)) ? 2 : 3;
    } else {
      reg = 2;
    }
    if (P.sd == 3 && ((z < P.zbot) || (z > P.ztop))) reg = 4;
  } else {
    reg = 1;
    double vel = (P.sd == 3) ? (ux * ux + uy * uy + uz * uz) : (ux * ux + uy * uy);
    vel = sqrt(vel);
    const double ang = (ux * P.lism_u[0] + uy * P.lism_u[1] + uz * P.lism_u[2]) / vel;
    const double TEMP = P.t_coeff * w[4] / w[0];
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
  double x = (i + 0.5) * dx - P.sun_c[0];
  double y = (j + 0.5) * dx - P.sun_c[1];
  double z = 0.0, r2, invr, ur;
  if (P.sd == 3) {
    z = (k + 0.5) * dx - P.sun_c[2];
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
// T names the arithmetic type for interface symmetry with the fast physics;
// the parity physics is FP64 only.
// NN > 0: the number of neutral populations fixed at compile time (the same
// operations in the same order; the loops run a known count, so the
// populations' independent chains can be scheduled together); 0: P.nf - 1.
template <int IRHON, typename T = double, typename WA = const double*, int NN = 0>
__device__ __forceinline__ void charge_exchange_add(const DevParams& P, const WA& w, int reg,
                                                    double dt, double* u) {
  static_assert(sizeof(T) == sizeof(double), "FP64 physics");
  const int nN = NN > 0 ? NN : P.nf - 1;
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

// HELIOREINIT_DEFAULT (swlism/HeliosphericPlasmaBCF.ChF:1435-1566) at time t
// (the stage's start time plus its dt), in the routine's order of
// operations; sunBmonopolar != 1: the bipolar field (sign by theta < thetaS)
// and the current-sheet surface iHCS (:1537-1564).
// The wind state of a cell inside the sphere.  Inlined: a call out of line
// would cost the whole calling kernel local-memory traffic.
static __device__ __host__ __forceinline__ void reinit_state(const ReinitIn P, double x,
                                                          double y, double z, double r2,
                                                          double t, ReinitState& o) {
  o.hcs = 0.0;
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
  if (!P.monopolar) {
    double theta = acos(cosT);
    // cos / sin of the spiral phase sunBeta (r - sunV t), through the phase
    // in units of pi (an exact argument reduction: no slow path for large
    // phases); the phase only places the current sheet
    double sinBr, cosBr;
    reinit_sincos(P.sun_beta * (r - P.sun_v * t), sinBr, cosBr);
    double sinB = sinF * cosBr + cosF * sinBr;
    double cosB = cosF * cosBr - sinF * sinBr;
    double thetaS = P.sin_tilt * sinB / sqrt((P.cos_tilt * cosB) * (P.cos_tilt * cosB) + sinB * sinB);
    thetaS = asin(thetaS) + 0.5 * kPi;
    if (!(theta < thetaS)) {
      bx = -bx;
      by = -by;
      bz = -bz;
    }
    o.hcs = (theta < thetaS) ? 1.0 : -1.0;
  }
  o.u[0] = rho;
  o.u[1] = rho * ux;
  o.u[2] = rho * uy;
  o.u[3] = rho * uz;
  o.u[4] = e0;
  o.u[5] = bx;
  o.u[6] = by;
  o.u[7] = bz;
}

// The reset of one cell: the membership test, then the wind state.
__device__ __host__ __forceinline__ void reinit_cell(const DevParams& P, double dx, int i, int j, int k,
                                            double t, double* u) {
  double x = (i + 0.5) * dx - P.sun_c[0];
  double y = (j + 0.5) * dx - P.sun_c[1];
  double z = 0.0;
  if (P.sd == 3) z = (k + 0.5) * dx - P.sun_c[2];
  double r2 = (P.sd == 3) ? (x * x + y * y + z * z) : (x * x + y * y);
  if (!(r2 <= P.r0 * P.r0)) return;
  ReinitState o;
  reinit_state(reinit_in(P), x, y, z, r2, t, o);
#pragma unroll
  for (int q = 0; q < 8; ++q) u[q] = o.u[q];
  if (!P.monopolar) {
    // a select per component keeps u in registers (ihcs is -1 or a surface
    // component; conditional stores would be merged into one indexed store,
    // which puts u in local memory)
#pragma unroll
    for (int q = 8; q < MF_MAX_COMP; ++q) u[q] = (q == P.ihcs) ? o.hcs : u[q];
  }
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
template <int IRHON, typename T = double>
__device__ __forceinline__ double max_wave_speed(const DevParams& P, const double* u) {
  static_assert(sizeof(T) == sizeof(double), "FP64 physics");
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

}  // namespace exact
}  // namespace mf
