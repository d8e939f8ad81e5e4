// mf_sources.cuh - cell sources and cell-wise post-processing (always FP64):
// region classification, charge exchange, inner-sphere reset, positivity and
// the CFL wave speed.
//
// The region and sphere tests are thresholds on the primitive state; they use
// intrinsics that never fuse into multiply-adds so that each cell lands on the
// same side of every threshold as in the CPU restatement.
#pragma once

#include "mf_device.cuh"
#include "mf_fp64.cuh"

namespace mf {
namespace fast {

constexpr double kInvPi = 0.318309886183790671537767526745028724;

// DEFINE_REGIONS_TRACER_4F (swlism/SWLISMF.ChF:839-1016), Cartesian: regtr
// is the region tracer of the cell (negative: solar wind).  The thresholds
// are the routine's literals.  Its x > 650 test reads the x of the last
// solar-wind cell the routine visited (x is assigned in that branch only);
// here the cell's own x, the same on every domain within x <= 650.
template <typename WA>
__device__ __forceinline__ int region_tracer_cell(const DevParams& P, double dx, int i, int j,
                                                  int k, const WA& w, double regtr) {
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
template <typename WA>
__device__ __forceinline__ int region_cell(const DevParams& P, double dx, int i, int j, int k,
                                           const WA& w, double regtr) {
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

// Arithmetic type of the charge-exchange rates: FP64, or FP32 in the opt-in
// MF_PREC_MIXED_CE32 mode (the rates scale a source that is a small fraction
// of the state per step).  The FP64 forms take the reciprocal and logarithm
// of mf_fp64.cuh (within a few units of 2^-53 of the library's).  The state
// update itself is FP64 either way.
__device__ __forceinline__ double ce_rsqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ float ce_rsqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double ce_log(double x) { return fp64::log64(x); }
__device__ __forceinline__ float ce_log(float x) { return logf(x); }
__device__ __forceinline__ double ce_rcp(double x) { return fp64::rcp64(x); }
__device__ __forceinline__ float ce_rcp(float x) { return 1.0f / x; }
__device__ __forceinline__ double ce_exp(double x) { return exp(x); }
__device__ __forceinline__ float ce_exp(float x) { return expf(x); }
__device__ __forceinline__ double ce_pow(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float ce_pow(float x, float y) { return powf(x, y); }
// conversions between the FP64 state and the rates' type T (identities for
// T = double).  The conversion instructions: their integer forms
// (fp64::d2f / f2d) made the FP32-rate update 10% slower (more registers
// and branches in a kernel bounded at 128 registers), measured.
template <typename T>
__device__ __forceinline__ T to_t(double x) {
  return static_cast<T>(x);
}
__device__ __forceinline__ double to_d(float x) { return static_cast<double>(x); }
__device__ __forceinline__ double to_d(double x) { return x; }

// Pauls & Zank charge-exchange rates of one cell; adds S = -dt*H to u
// (HeliosphericProblem::explicitSource, swlism/HeliosphericProblem.cpp:1394-1539,
// CHARGE_EXCHANGE_4F swlism/ChargeExchange2F.ChF:673-993 and _MF :995-1149).
// T is the arithmetic type of the rates (double, or float in the opt-in
// FP32-rate mode).  The plasma's thermal-speed terms that every neutral
// population shares are formed once per cell.
// w: the stage-start primitive state (an array, or a column view that
// loads each component where it is used).
// NN > 0: the number of neutral populations fixed at compile time (the
// loops run a known count, so the populations' independent chains can be
// scheduled together); 0: P.nf - 1 at run time.
template <int IRHON, typename T = double, typename WA = const double*, int NN = 0>
__device__ __forceinline__ void charge_exchange_add(const DevParams& P, const WA& w, int reg,
                                                    double dt, double* u) {
  const int nN = NN > 0 ? NN : P.nf - 1;
  constexpr T c4p = T(4.0 * kInvPi), c16p = T(16.0 * kInvPi), c94pi = T(2.25 * kPi);
  constexpr T c4ip = T(4.0 * kInvPi), c649ip = T(64.0 / 9.0 * kInvPi);
  const T rho = to_t<T>(w[0]), ux = to_t<T>(w[1]), uy = to_t<T>(w[2]), uz = to_t<T>(w[3]);
  const T U2 = ux * ux + uy * uy + uz * uz, hU2 = T(0.5) * U2;
  const T VVTP = to_t<T>(w[4]) * ce_rcp(rho);
  // plasma thermal-speed terms of the five speed arguments
  const T aUDp = c4p * VVTP, aUPMp = c16p * VVTP, aUHMp = c94pi * VVTP;
  const T aPEp = c4ip * VVTP, aHEp = c649ip * VVTP, q75VP = T(0.75) * VVTP;
  const T scale_vel = to_t<T>(P.ce_scale_vel), ce_a = to_t<T>(P.ce_a), ce_b = to_t<T>(P.ce_b);
  const T damp_c = to_t<T>(P.ce_damp_c), damp_pow = to_t<T>(P.ce_damp_pow);
  const T srho = to_t<T>(P.ce_sigma_scale) * rho;
  // Each population's own loss / gain is applied inside the loop; the
  // recipient of the newly created neutrals (region-dependent) then also
  // receives the plasma's totals.  The products ARR*UD, ARR*VVTHU and
  // ARR*VP_UHM that several terms share are formed once, and the plasma's
  // terms that carry a cell factor (ux, U2/2, 3 VVTP/4) are summed without it
  // and scaled after the loop: the reference's H, summed in another order.
  // G: the sum of ARR (VPHP VP_UHM + 3 VVTP UHE / 4), which both the energy
  // source and the recipient's energy gain hold; H5: the rest of h5.
  T h2 = 0, h3 = 0, h4 = 0, DSUM = 0, S1x = 0, S1y = 0, S1z = 0, G = 0, H5 = 0;
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f) {
    if (f > nN) break;
    const int o = IRHON + (f - 1) * 5;
    const T rhoN = to_t<T>(w[o]), uxN = to_t<T>(w[o + 1]), uyN = to_t<T>(w[o + 2]), uzN = to_t<T>(w[o + 3]);
    const T dx_ = ux - uxN, dy_ = uy - uyN, dz_ = uz - uzN;
    const T UH2 = uxN * uxN + uyN * uyN + uzN * uzN;
    const T DU2 = dx_ * dx_ + dy_ * dy_ + dz_ * dz_, DU2x4 = T(4) * DU2;
    const T VPHH = dx_ * uxN + dy_ * uyN + dz_ * uzN;
    const T VPHP = dx_ * ux + dy_ * uy + dz_ * uz;
    const T VVTH = T(2) * (to_t<T>(w[o + 4]) * ce_rcp(rhoN));
    // thermal + relative speeds; every argument is > 0, so sqrt(a) = a*rsqrt(a)
    const T aUD = (aUDp + c4p * VVTH) + DU2;
    const T UD = aUD * ce_rsqrt(aUD);
    const T iUPM = ce_rsqrt((aUPMp + c94pi * VVTH) + DU2x4);
    const T iUHM = ce_rsqrt((aUHMp + c16p * VVTH) + DU2x4);
    const T aPE = (aPEp + c649ip * VVTH) + DU2;
    const T UPE = aPE * ce_rsqrt(aPE);
    const T aHE = (aHEp + c4ip * VVTH) + DU2;
    const T UHE = aHE * ce_rsqrt(aHE);
    const T UDS = scale_vel * UD;
    const T t = ce_a - ce_b * ce_log(UDS);
    T SIG = t * t;
    if (damp_c > T(0)) SIG = SIG * ce_pow(T(1) - ce_exp(-damp_c / UDS), damp_pow);
    const T ARR = SIG * (rhoN * srho);
    const T aU = ARR * UD;                  // -DENPLU
    const T aT = ARR * (VVTH * iUPM);       // ARR*VVTHU
    const T aV = ARR * (VVTP * iUHM);       // ARR*VP_UHM
    const T Y = (ARR * UPE) * VVTH;
    const T hv = aU + aT + aV;
    h2 = h2 + hv * dx_;
    h3 = h3 + hv * dy_;
    h4 = h4 + hv * dz_;
    S1x = S1x + aV * dx_;
    S1y = S1y + aV * dy_;
    S1z = S1z + aV * dz_;
    DSUM = DSUM - aU;
    G = G + aV * VPHP + q75VP * (ARR * UHE);
    H5 = H5 + aT * VPHH + aU * (hU2 - T(0.5) * UH2) - T(0.75) * Y;
    double* un = u + IRHON + (f - 1) * 5;
    un[0] = un[0] - dt * to_d(aU);
    un[1] = un[1] - dt * to_d(uxN * aU - dx_ * aT);
    un[2] = un[2] - dt * to_d(uyN * aU - dy_ * aT);
    un[3] = un[3] - dt * to_d(uzN * aU - dz_ * aT);
    un[4] = un[4] - dt * to_d((T(0.5) * UH2) * aU - VPHH * aT + T(0.75) * Y);
  }
  const T h5 = G + H5;
  const T PPLUX = ux * DSUM - S1x, PPLUY = uy * DSUM - S1y, PPLUZ = uz * DSUM - S1z;
  const T ENPLU = hU2 * DSUM - G;
  u[1] = u[1] - dt * to_d(h2);
  u[2] = u[2] - dt * to_d(h3);
  u[3] = u[3] - dt * to_d(h4);
  u[4] = u[4] - dt * to_d(h5);
  // S of the magnetic field (and of psi) is zero; the recipient gets the
  // other populations' lost density (DSUM less its own, already applied)
  const int rk = ce_recipient(nN, reg);
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f) {
    if (f > nN) break;
    const bool rec = (f == rk);
    double* un = u + IRHON + (f - 1) * 5;
    un[0] = rec ? un[0] - dt * to_d(DSUM) : un[0];
    un[1] = rec ? un[1] - dt * to_d(PPLUX) : un[1];
    un[2] = rec ? un[2] - dt * to_d(PPLUY) : un[2];
    un[3] = rec ? un[3] - dt * to_d(PPLUZ) : un[3];
    un[4] = rec ? un[4] - dt * to_d(ENPLU) : un[4];
  }
}

// HELIOREINIT_DEFAULT (swlism/HeliosphericPlasmaBCF.ChF:1435-1566): the
// plasma in r <= Rinit becomes the radial wind at time t (the stage's start
// time plus its dt); bipolar field: B flips where the colatitude is not
// below the current sheet's, and the current-sheet surface takes +1 / -1.
// The wind state of a cell inside the sphere.  Inlined: a call out of line
// would cost the whole calling kernel local-memory traffic.
static __device__ __host__ __forceinline__ void reinit_state(const ReinitIn P, double x,
                                                          double y, double z, double r2,
                                                          double t, ReinitState& o) {
  o.hcs = 0.0;
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
  double bx = br * sinT * cosF - bp * sinF;
  double by = br * sinT * sinF + bp * cosF;
  double bz = br * cosT;
  const double b = bx * bx + by * by + bz * bz;
  const double e0 = pr / P.hgamma + 0.5 * (rho * P.sun_v * P.sun_v + kInv4Pi * b);
  if (!P.monopolar) {
    const double theta = acos(cosT);
    double sinBr, cosBr;
    reinit_sincos(P.sun_beta * (r - P.sun_v * t), sinBr, cosBr);
    const double sinB = sinF * cosBr + cosF * sinBr;
    const double cosB = cosF * cosBr - sinF * sinBr;
    const double ct = P.cos_tilt * cosB;
    const double thetaS = asin(P.sin_tilt * sinB / sqrt(ct * ct + sinB * sinB)) + 0.5 * kPi;
    const bool keep = theta < thetaS;
    if (!keep) {
      bx = -bx;
      by = -by;
      bz = -bz;
    }
    o.hcs = keep ? 1.0 : -1.0;
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

// The reset of one cell: the membership test in non-fused arithmetic (host
// and device agree exactly), then the wind state.
__device__ __host__ __forceinline__ void reinit_cell(const DevParams& P, double dx, int i, int j, int k,
                                            double t, double* u) {
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
  const double hg = P.hgamma, ihg = P.invhgamma, smallR = P.smallr, smallP = P.smallp;
  if (P.nf == 1) {
    double Rho = u[0];
    bool was = false;
    if (Rho < smallR) { Rho = smallR; was = true; }
    const double invRho = fp64::rcp64(Rho);
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
    const double invRho = fp64::rcp64(Rho0);
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
    const double invRho = fp64::rcp64(Rho0);
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
// (srcIdeal/PatchEulerF.ChF:5-50) of one cell.  The pressure is recovered
// from the total energy in FP64 (E minus kinetic minus magnetic cancels in
// cold, low-beta flow); the speeds are formed in T (FP64, or FP32 in the
// mixed precision modes, whose time step then carries FP32 rounding).
__device__ __forceinline__ double ws_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float ws_sqrt(float x) { return sqrtf(x); }

template <int IRHON, typename T = double>
__device__ __forceinline__ double max_wave_speed(const DevParams& P, const double* u) {
  const T i4pi = T(kInv4Pi), gam = to_t<T>(P.gamma);
  T cmax = 0;
  {
    const double rinv = fp64::rcp64(u[0]);
    const double m1 = u[1], m2 = u[2], m3 = u[3], bx = u[5], by = u[6], bz = u[7];
    const double ke = (m1 * m1 + m2 * m2 + m3 * m3) * rinv;
    const double bb = kInv4Pi * (bx * bx + by * by + bz * bz);
    const double p = fmax(P.hgamma * (u[4] - 0.5 * (ke + bb)), P.smallp);
    const T invrho = to_t<T>(rinv), b = to_t<T>(bb);
    const T uu = to_t<T>(m1) * invrho, vv = to_t<T>(m2) * invrho, ww = to_t<T>(m3) * invrho;
    const T bxt = to_t<T>(bx), byt = to_t<T>(by), bzt = to_t<T>(bz);
    const T a2 = gam * to_t<T>(p) * invrho;
    const T as2 = T(0.5) * (a2 + invrho * b);
    const T as4 = as2 * as2;
    const T k4 = i4pi * invrho * a2;
    // as4 - k4 b^2 >= 0 exactly; contracted rounding can push it below 0
    T umax = fabs(uu) + ws_sqrt(as2 + ws_sqrt(fmax(T(0), as4 - k4 * bxt * bxt)));
    umax = fmax(fabs(vv) + ws_sqrt(as2 + ws_sqrt(fmax(T(0), as4 - k4 * byt * byt))), umax);
    umax = fmax(fabs(ww) + ws_sqrt(as2 + ws_sqrt(fmax(T(0), as4 - k4 * bzt * bzt))), umax);
    cmax = fmax(umax, cmax);
  }
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f) {
    if (f >= P.nf) break;
    const double* un = u + IRHON + (f - 1) * 5;
    const double rinv = fp64::rcp64(fmax(un[0], P.smallr));
    const double m1 = un[1], m2 = un[2], m3 = un[3];
    const double ke = (m1 * m1 + m2 * m2 + m3 * m3) * rinv;
    const double p = fmax(P.hgamma * (un[4] - 0.5 * ke), P.smallp);
    const T invrho = to_t<T>(rinv);
    const T uu = to_t<T>(m1) * invrho, vv = to_t<T>(m2) * invrho, ww = to_t<T>(m3) * invrho;
    const T a = ws_sqrt(gam * to_t<T>(p) * invrho);
    const T umax = fmax(fmax(fabs(uu), fabs(vv)), fabs(ww)) + a;
    cmax = fmax(umax, cmax);
  }
  return to_d(cmax);
}

}  // namespace fast
}  // namespace mf
