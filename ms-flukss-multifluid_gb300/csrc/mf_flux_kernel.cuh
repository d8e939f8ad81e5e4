// mf_flux_kernel.cuh - the face-flux kernel.  Included by mf_flux.cu (fast
// physics, contraction allowed) and mf_flux_exact.cu (parity physics, no
// contraction); MF_PHYS names the physics namespace of the including unit.
#pragma once

#include "mf_kernels.cuh"

namespace mf {
namespace {
using namespace MF_PHYS;

// Plasma flux of one face with the configured solver.  Mixed-precision
// guard: the Roe eigenvectors carry factors 1/c and 1/c^2 of the gas sound
// speed, so where c^2 is far below the magnetic speed^2 (cold, magnetically
// dominated plasma, e.g. a cell at the pressure floor) the FP32 products in
// R |Lambda| L dU lose every digit and the flux can be off by orders of
// magnitude.  There (c^2 < 1e-3 b^2 on either side) the FP32 path takes the
// Rusanov flux of the same states instead; FP64 keeps the Roe flux.  The
// same holds for VFRoe, whose wave strengths carry 1/c^2 too.
template <typename R, int DIR>
__device__ __forceinline__ void plasma_flux(const DevParams& P, const R* wl, const R* wr, R* g) {
  bool cold = false;
  if (sizeof(R) == 4 && P.rs != kRusanov) {
    const R rl = rmax<R>(R(P.smallr), wl[0]), rr = rmax<R>(R(P.smallr), wr[0]);
    const R pl = rmax<R>(R(P.smallp), wl[4]), pr = rmax<R>(R(P.smallp), wr[4]);
    const R a2 = R(P.gamma) * rmin<R>(pl / rl, pr / rr);
    const R bl = (wl[5] * wl[5] + wl[6] * wl[6] + wl[7] * wl[7]) / rl;
    const R br = (wr[5] * wr[5] + wr[6] * wr[6] + wr[7] * wr[7]) / rr;
    cold = a2 < R(1.0e-3) * R(kInv4Pi) * rmax<R>(bl, br);
  }
  if (cold || P.rs == kRusanov)
    rusanov_mhd<R, DIR>(P, wl, wr, g);
  else if (P.rs == kVFRoe)
    vfroe_mhd<R, DIR>(P, wl, wr, g);
  else if (P.rs == kRoe8)
    roe_mhd<R, DIR, false>(P, wl, wr, g);
  else
    roe_mhd<R, DIR, true>(P, wl, wr, g);
}


// ---------------------------------------------------------------------------
// Heliosphere boundary fluxes: HELIOBC (swlism/HeliosphericF.ChF:221-910)
// as HeliosphericProblem::fluxBC applies it after the Riemann fluxes
// (swlism/HeliosphericProblem.cpp:1994-2188), in FP64 in every precision
// mode (the faces of the domain boundary are a few percent of all faces).
// Face-frame states: rho, vn, vt1, vt2, p, Bn, Bt1, Bt2; fluxes in the same
// order.  ROE8WAVEF is RIEMANNF's body without the input floors (the states
// are floored before), so the unit's Roe 8-wave flux in a frame whose
// normal is x gives it; VANLEERRS likewise is VANLEERF without its floors.
// ---------------------------------------------------------------------------
// BFLUX (:1363-1560) and, with exitR, BFLUXR (:1562-1768); in: domain side,
// out: ghost side, normal pointing out of the domain.
__device__ void hbc_bflux(const DevParams& P, bool exitR, const double* in, const double* out,
                          double* F, double& BnValue) {
  const double gamma = P.gamma, hgamma = P.hgamma, d_4PI = 4.0 * kPi;
  const double U = in[1], V = in[2], W = in[3], R = in[0], BX = in[5], BY = in[6], BZ = in[7];
  const double PG = in[4];
  const double BB = BX * BX + BY * BY + BZ * BZ;
  const double Pt = PG + kInv8Pi * BB;
  const double KE = 0.5 * (in[1] * in[1] + in[2] * in[2] + in[3] * in[3]);
  const double E = PG / hgamma + in[0] * KE + kInv8Pi * BB;
  const double SZ = sqrt(gamma * PG / R);
  const double SP = 0.5 * sqrt(d_4PI * R);
  const double EM = SZ * SZ + BB / (d_4PI * R) + SZ * fabs(BX) / SP;
  const double EMM = SZ * SZ + BB / (d_4PI * R) - SZ * fabs(BX) / SP;
  const double CF = 0.5 * (sqrt(EM) + sqrt(EMM));
  const double CS = 0.5 * (sqrt(EM) - sqrt(EMM));
  if (U >= CF) {
    BnValue = BX;
    F[0] = R * U;
    F[1] = R * U * U + Pt - kInv4Pi * BX * BX;
    F[2] = R * U * V - kInv4Pi * BX * BY;
    F[3] = R * U * W - kInv4Pi * BX * BZ;
    F[4] = U * (E + Pt) - kInv4Pi * BX * (U * BX + V * BY + W * BZ);
    F[5] = 0.0;
    F[6] = U * BY - V * BX;
    F[7] = U * BZ - W * BX;
    return;
  }
  const double U1 = out[1], V1 = out[2], W1 = out[3], R1 = out[0], BX1 = out[5], BY1 = out[6];
  const double BZ1 = out[7], PG1 = out[4];
  const double BB1 = BX1 * BX1 + BY1 * BY1 + BZ1 * BZ1;
  const double P1 = PG1 + kInv8Pi * BB1;
  const double KE1 = 0.5 * (out[1] * out[1] + out[2] * out[2] + out[3] * out[3]);
  const double E1 = PG1 / hgamma + out[0] * KE1 + kInv8Pi * BB1;
  if (U < -CF) {
    BnValue = BX1;
    F[0] = R1 * U1;
    F[1] = R1 * U1 * U1 + P1 - kInv4Pi * BX1 * BX1;
    F[2] = R1 * U1 * V1 - kInv4Pi * BX1 * BY1;
    F[3] = R1 * U1 * W1 - kInv4Pi * BX1 * BZ1;
    F[4] = U1 * (E1 + P1) - kInv4Pi * BX1 * (U1 * BX1 + V1 * BY1 + W1 * BZ1);
    F[5] = 0.0;
    F[6] = U1 * BY1 - V1 * BX1;
    F[7] = U1 * BZ1 - W1 * BX1;
    return;
  }
  const double SZ1 = sqrt(gamma * PG1 / R1);
  const double SP1 = 0.5 * sqrt(d_4PI * R1);
  const double EM1 = SZ1 * SZ1 + BB1 / (d_4PI * R1) + SZ1 * fabs(BX1) / SP1;
  const double EMM1 = SZ1 * SZ1 + BB1 / (d_4PI * R1) - SZ1 * fabs(BX1) / SP1;
  const double CF1 = 0.5 * (sqrt(EM1) + sqrt(EMM1));
  const bool middle = exitR ? ((U < CF) && (U >= 0.0)) : ((U < CF) && (U >= 0.0) && (U1 > CF1));
  if (middle) {
    const double SCM = SZ * SZ - CS * CS;
    const double SCP = SZ * SZ + CS * CS;
    const double DEM = sqrt(EM * EMM);
    double THE = -0.5 * CF * (BX * BX) / (R * d_4PI * DEM);
    THE = THE + (BZ * BZ + BY * BY) * CF * SCP * 0.5 / (R * DEM * d_4PI * SCM);
    THE = THE + 0.5 * CF * hgamma * (SZ * SZ) / DEM;
    THE = THE - SZ * fabs(BX) * CS * (gamma - 2.0) * 0.25 / (SP * DEM);
    const double hyz = BY * BY + BZ * BZ;
    double hy2, hz2;
    if (hyz < 1.0e-10) {
      hy2 = 0.5;
      hz2 = 0.5;
    } else {
      hy2 = BY * BY / hyz;
      hz2 = BZ * BZ / hyz;
    }
    double U16, R16, DRho, HRho, SZ16, BY16, BZ16;
    if (exitR) {
      const double BE = 2.0 * d_4PI * (CF * CF - SZ * SZ);
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
      const double BE = 2.0 * d_4PI * (CF * CF - SZ * SZ) * DRho;
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
    const double BX16 = BX;
    const double ALF = kInv4Pi * BX / (R * CF);
    const double W16 = W + ALF * (BZ16 - BZ);
    const double V16 = V + ALF * (BY16 - BY);
    const double PG16 = SZ16 * SZ16 * R16 / gamma;
    const double BB16 = kInv4Pi * (BX16 * BX16 + BY16 * BY16 + BZ16 * BZ16);
    const double P16 = PG16 + 0.5 * BB16;
    const double E16 = PG16 / hgamma + 0.5 * (R16 * (U16 * U16 + V16 * V16 + W16 * W16) + BB16);
    const double BXq = kInv4Pi * BX16;
    BnValue = BX16;
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
    const double o2[8] = {in[0], in[1], in[2], in[3], out[4], out[5], out[6], out[7]};
    BnValue = BX;
    roe_mhd<double, 0, false>(P, in, o2, F);
  } else {
    BnValue = 0.5 * (BX + BX1);
    roe_mhd<double, 0, false>(P, in, out, F);
  }
}

// plasma fluxes 0..7 and Bn of a face on the domain boundary (side 0: low
// face, wl is the ghost side; 1: high face, wr is the ghost side)
template <int DIR>
__device__ void helio_plasma(const DevParams& P, const RunParams& RP, int side, const double* wl,
                             const double* wr, double* g, double& bn) {
  constexpr int t1 = (DIR + 1) % 3, t2 = (DIR + 2) % 3;
  const int iv[3] = {1 + DIR, 1 + t1, 1 + t2}, ib[3] = {5 + DIR, 5 + t1, 5 + t2};
  if (DIR == 0 && side == 1) {  // inflow: the exact flux of the far-field state
    const double* b = RP.bc_plasma;
    const double density = b[0], velx = b[1], vely = b[2], velz = b[3], pressure = b[4];
    const double Bx = b[5], By = b[6], Bz = b[7];
    const double bm = kInv8Pi * (Bx * Bx + By * By + Bz * Bz);
    const double ke = density * (velx * velx + vely * vely + velz * velz);
    const double bu = Bx * velx + By * vely + Bz * velz;
    const double Pt = pressure + bm;
    const double e = pressure / P.hgamma + 0.5 * ke + bm;
    g[0] = density * velx;
    g[1] = density * velx * velx - kInv4Pi * Bx * Bx + Pt;
    g[2] = density * velx * vely - kInv4Pi * Bx * By;
    g[3] = density * velx * velz - kInv4Pi * Bx * Bz;
    g[4] = velx * (e + Pt) - kInv4Pi * Bx * bu;
    g[5] = 0.0;
    g[6] = velx * By - vely * Bx;
    g[7] = velx * Bz - velz * Bx;
    bn = Bx;
    return;
  }
  // element-wise selects at fixed indices keep both face states in registers
  // (a pointer chosen at run time between two arrays would put them in local memory)
  const bool hi = side != 0;
  const double sg = hi ? 1.0 : -1.0;
  double L[8], Rt[8], F[8], Bv;
  L[0] = hi ? wl[0] : wr[0];
  Rt[0] = hi ? wr[0] : wl[0];
  L[4] = hi ? wl[4] : wr[4];
  Rt[4] = hi ? wr[4] : wl[4];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    L[1 + a] = sg * (hi ? wl[iv[a]] : wr[iv[a]]);
    Rt[1 + a] = sg * (hi ? wr[iv[a]] : wl[iv[a]]);
    L[5 + a] = sg * (hi ? wl[ib[a]] : wr[ib[a]]);
    Rt[5 + a] = sg * (hi ? wr[ib[a]] : wl[ib[a]]);
  }
  Rt[0] = fmax(P.smallr, Rt[0]);
  Rt[4] = fmax(P.smallp, Rt[4]);
  L[0] = fmax(P.smallr, L[0]);
  L[4] = fmax(P.smallp, L[4]);
  hbc_bflux(P, DIR == 0, L, Rt, F, Bv);
  g[0] = sg * F[0];
  g[iv[0]] = F[1];
  g[iv[1]] = F[2];
  g[iv[2]] = F[3];
  g[4] = sg * F[4];
  g[ib[0]] = F[5];
  g[ib[1]] = F[6];
  g[ib[2]] = F[7];
  bn = sg * Bv;
}

// one neutral population (fl = 1, 2, 3, 4) of a face on the domain boundary;
// nl / nr: rho, u, v, w, p of the two face states (global frame)
template <int DIR>
__device__ void helio_neutral(const DevParams& P, int side, int fl, const double* nl,
                              const double* nr, double* gn) {
  constexpr int t1 = (DIR + 1) % 3, t2 = (DIR + 2) % 3;
  const int nv[3] = {1 + DIR, 1 + t1, 1 + t2};
  const bool hi = side != 0;
  double Win[5], Wout[5];
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    Win[c] = hi ? nl[c] : nr[c];
    Wout[c] = hi ? nr[c] : nl[c];
  }
  auto outflow = [&](const double* st, double vn) {
    const double rho = st[0], vt1 = st[2], vt2 = st[3], p = st[4];
    const double ke = rho * (vn * vn + vt1 * vt1 + vt2 * vt2);
    const double e = p / P.hgamma + 0.5 * ke;
    gn[0] = rho * vn;
    gn[nv[0]] = rho * vn * vn + p;
    gn[nv[1]] = rho * vn * vt1;
    gn[nv[2]] = rho * vn * vt2;
    gn[4] = vn * (e + p);
  };
  if (fl == 2 || fl == 3) {
    const double fd = (fl == 2) ? kNet2Dens : kNet3Dens, fp = (fl == 2) ? kNet2Pres : kNet3Pres;
    const double st[5] = {fmax(fd, Win[0]), Win[nv[0]], Win[nv[1]], Win[nv[2]], fmax(fp, Win[4])};
    outflow(st, side ? fmax(0.0, st[1]) : fmin(0.0, st[1]));
    return;
  }
  if (side == 0 && DIR == 0) {
    const double st[5] = {fmax(P.smallr, Win[0]), Win[nv[0]], Win[nv[1]], Win[nv[2]],
                          fmax(P.smallp, Win[4])};
    outflow(st, fmin(-1.0e-6, st[1]));
    return;
  }
  const double sg = side ? 1.0 : -1.0;
  double Ln[5], Rn[5], gl[5];
  Ln[0] = fmax(P.smallr, Win[0]);
  Ln[4] = fmax(P.smallp, Win[4]);
  Rn[0] = fmax(P.smallr, Wout[0]);
  Rn[4] = fmax(P.smallp, Wout[4]);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    Ln[1 + a] = sg * Win[nv[a]];
    Rn[1 + a] = sg * Wout[nv[a]];
  }
  if (Ln[1] > 0.0) {
    Rn[1] = Ln[1];
    Rn[2] = Ln[2];
    Rn[3] = Ln[3];
    if (fl == 1) Rn[0] = Ln[0];
  }
  vanleer_euler<double, 0>(P, Ln, Rn, gl);
  gn[0] = sg * gl[0];
  gn[nv[0]] = gl[1];
  gn[nv[1]] = gl[2];
  gn[nv[2]] = gl[3];
  gn[4] = sg * gl[4];
}

// side of the domain boundary a face lies on (-1: interior or periodic)
template <int DIR>
__device__ __forceinline__ int helio_side(const DevParams& P, const RunParams& RP, int i, int j,
                                          int k) {
  if (!P.helio_bc || P.periodic[DIR]) return -1;
  const int f = (DIR == 0) ? i : (DIR == 1) ? j : k;
  return (f == RP.dlo[DIR]) ? 0 : (f == RP.dhi[DIR] + 1) ? 1 : -1;
}

// The fluxes of face gi of the batch's flat face index of direction DIR
// (gi >= total: none).  WF: read the limiter inputs from Wf, the FP32 copy of
// W the prim kernel wrote (R = float), instead of converting W value by
// value here.
template <typename R, int DIR, int WF>
__device__ __forceinline__ void flux_face(const DevParams& P, const double* __restrict__ W,
                                          const float* __restrict__ Wf, R* __restrict__ F,
                                          R* __restrict__ Bn,
                                          const StageDesc* __restrict__ descs, int ndesc,
                                          int gi, int total,
                                          const RunParams* __restrict__ runs,
                                          const StepState* __restrict__ states) {
  if (gi >= total) return;
  const StageDesc& D = descs[find_desc(descs, ndesc, kRegF + DIR, gi)];
  const int lin = gi - D.g0[kRegF + DIR];
  const RunParams& RP = runs[D.run];
  int fnb[3] = {D.vn[0], D.vn[1], D.vn[2]};
  fnb[DIR] += 1;
  int i, j, k;
  decode(lin, D.vlo, fnb, i, j, k);
  const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
  const long long st = (DIR == 0) ? 1 : (DIR == 1) ? (long long)D.fn[0]
                                                   : (long long)D.fn[0] * D.fn[1];
  // cell on the high side of face (i,j,k) has the same index
  const double* __restrict__ w0 = W + D.u_off + loc(D.flo, D.fn, i, j, k);
  const float* __restrict__ f0 = WF ? Wf + D.u_off + loc(D.flo, D.fn, i, j, k) : nullptr;
  // component v of the cell o cells along DIR from the face's high-side cell
  auto ld = [&](int v, long long o) -> R {
    if (WF) return R(f0[v * cs + o * st]);
    return R(w0[v * cs + o * st]);
  };
  const long long fcs = (long long)fnb[0] * fnb[1] * fnb[2];
  const long long fo = loc(D.vlo, fnb, i, j, k);
  R* __restrict__ Fo = F + D.f_off[DIR] + fo;

  // positivity check of rho and p face values (CHECKPOSITIVITY / REDUCEORDER,
  // src/reconstructionF.ChF:1023-1054): first order for the whole cell
  bool negL = false, negR = false;
  R wl[9], wr[9];
  if (P.char_rec) {
    // characteristic limiting of the plasma variables (FP64 in every mode:
    // the projections carry 1/c^2), then the same positivity fallback
    double a8[8], b8[8], c8[8], d8[8], lo8[8], hiL[8], loR[8], hi8[8];
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      const double* wv = w0 + v * cs;
      a8[v] = wv[-2 * st];
      b8[v] = wv[-st];
      c8[v] = wv[0];
      d8[v] = wv[st];
    }
    char_face_values<DIR>(P, a8, b8, c8, lo8, hiL);
    if (P.check_pos) negL = lo8[0] <= 0.0 || hiL[0] <= 0.0 || lo8[4] <= 0.0 || hiL[4] <= 0.0;
    char_face_values<DIR>(P, b8, c8, d8, loR, hi8);
    if (P.check_pos) negR = loR[0] <= 0.0 || hi8[0] <= 0.0 || loR[4] <= 0.0 || hi8[4] <= 0.0;
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      wl[v] = R(negL ? b8[v] : hiL[v]);
      wr[v] = R(negR ? c8[v] : loR[v]);
    }
  } else if (P.check_pos) {
#pragma unroll
    for (int t = 0; t < 2; ++t) {
      const int v = t ? 4 : 0;
      R a = ld(v, -2), b = ld(v, -1), c = ld(v, 0), d = ld(v, 1);
      R lo, hi;
      face_values<R>(P.lim[v], a, b, c, lo, hi);
      if (lo <= R(0) || hi <= R(0)) negL = true;
      face_values<R>(P.lim[v], b, c, d, lo, hi);
      if (lo <= R(0) || hi <= R(0)) negR = true;
    }
  }

  // plasma (+ psi) face states: left = high-face value of the low cell,
  // right = low-face value of the high cell (Roe8WavesRS::fluxes,
  // src/Roe8WavesRS.cpp:38-78)
#pragma unroll
  for (int v = 0; v < 9; ++v) {
    if (v < 8 && P.char_rec) continue;
    if (v < 8 || P.glm) {
      const int lim = (v < 8) ? P.lim[v] : (int)MF_LIM_MINMOD;
      R a = ld(v, -2), b = ld(v, -1), c = ld(v, 0), d = ld(v, 1);
      R lo, hi;
      face_values<R>(lim, a, b, c, lo, hi);
      wl[v] = negL ? b : hi;
      face_values<R>(lim, b, c, d, lo, hi);
      wr[v] = negR ? c : lo;
    } else {
      wl[v] = R(0);
      wr[v] = R(0);
    }
  }
  R g[9];
  plasma_flux<R, DIR>(P, wl, wr, g);
  if (P.glm) {
    R fbn, fpsi;
    dedner_2x2<R>(R(states[D.run].ch), wl[5 + DIR], wl[8], wr[5 + DIR], wr[8], fbn, fpsi);
    g[5 + DIR] = fbn;
    g[8] = fpsi;
  }

  // face-normal B (PatchMHDMF::computeBn, srcIdeal/PatchMHDMF.cpp:509-620)
  R bn = R(0);
  if (P.divb_method == 1) {
    bn = R(0.5) * (wl[5 + DIR] + wr[5 + DIR]);
    if (!P.periodic[DIR]) {
      const int f = (DIR == 0) ? i : (DIR == 1) ? j : k;
      if (f == RP.dlo[DIR]) bn = wr[5 + DIR];
      if (f == RP.dhi[DIR] + 1) bn = wl[5 + DIR];
    }
  } else if (P.divb_method == 2) {
    const double* wv = w0 + (5 + DIR) * cs;
    bn = R(0.5 * (wv[-st] + wv[0]));
  }
  // HELIOBC on the domain boundary (after the Riemann fluxes and Bn)
  const int hside = helio_side<DIR>(P, RP, i, j, k);
  if (hside >= 0) {
    double dl[8], dr[8], dg[8], dbn = double(bn);
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      dl[v] = double(wl[v]);
      dr[v] = double(wr[v]);
    }
    helio_plasma<DIR>(P, RP, hside, dl, dr, dg, dbn);
#pragma unroll
    for (int v = 0; v < 8; ++v) g[v] = R(dg[v]);
    bn = R(dbn);
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) Fo[q * fcs] = g[q];
  if (P.glm) Fo[8 * fcs] = g[8];
  Bn[D.bn_off[DIR] + fo] = bn;

  // neutral fluids: minmod face states, van Leer splitting (VANLEERF)
  for (int fl = 1; fl < P.nf; ++fl) {
    const int s = P.irhon + (fl - 1) * 5;
    R nl[5], nr[5], gn[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      R a = ld(s + m, -2), b = ld(s + m, -1), c = ld(s + m, 0), d = ld(s + m, 1);
      R lo, hi;
      face_values<R>(MF_LIM_MINMOD, a, b, c, lo, hi);
      nl[m] = negL ? b : hi;
      face_values<R>(MF_LIM_MINMOD, b, c, d, lo, hi);
      nr[m] = negR ? c : lo;
    }
    if (hside >= 0) {
      double dl[5], dr[5], dg[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        dl[m] = double(nl[m]);
        dr[m] = double(nr[m]);
      }
      helio_neutral<DIR>(P, hside, fl, dl, dr, dg);
#pragma unroll
      for (int m = 0; m < 5; ++m) gn[m] = R(dg[m]);
    } else {
      vanleer_euler<R, DIR>(P, nl, nr, gn);
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) Fo[(s + m) * fcs] = gn[m];
  }

  // tracking surfaces: LEVELSETFLUX (src/LevelSetF.ChF:37-105) after the
  // boundary fluxes (src/PatchMHDAM.cpp:644-648): the upwind face value by the
  // sign of sqrt(rho_L) u_L + sqrt(rho_R) u_R of the plasma face states
  if (P.nls) {
    const R uavg = sqrt(wl[0]) * wl[1 + DIR] + sqrt(wr[0]) * wr[1 + DIR];
    for (int q = P.ils; q < P.nc; ++q) {
      const R a = ld(q, -2), b = ld(q, -1), c = ld(q, 0), d = ld(q, 1);
      R lo, hi;
      ls_face_values<R>(P, a, b, c, lo, hi);
      const R l = negL ? b : hi;
      ls_face_values<R>(P, b, c, d, lo, hi);
      const R r = negR ? c : lo;
      Fo[q * fcs] = (uavg > R(0)) ? l : r;
    }
  }
}

template <typename R, int DIR, int WF>
__global__ void __launch_bounds__(kMaxBlock, WF ? 2 : 1)
    k_flux(const __grid_constant__ DevParams P, const double* __restrict__ W, const float* __restrict__ Wf,
           R* __restrict__ F, R* __restrict__ Bn, const StageDesc* __restrict__ descs, int ndesc,
           int first, int total, const RunParams* __restrict__ runs,
           const StepState* __restrict__ states) {
  // faces [first, total) of the batch's flat face index (first > 0: a chunk
  // of the batch's patches)
  flux_face<R, DIR, WF>(P, W, Wf, F, Bn, descs, ndesc, first + blockIdx.x * blockDim.x + threadIdx.x,
                        total, runs, states);
}

// Fluxes of face (i,j,k) (normal DIR) from given face states: the plasma
// solver, the GLM (Bn, psi) system, Bn (PatchMHDMF::computeBn), HELIOBC on
// the domain boundary, the neutral van Leer fluxes and LEVELSETFLUX.  fs(side,
// v): component v of the left (side 0: the high-face value of the low cell)
// or the right (side 1: the low-face value of the high cell) state.  Written
// to F / Bn at the face's offsets; W: the cell-centred primitive state (Bn of
// divb_method 2).
template <typename R, int DIR, typename FS>
__device__ __forceinline__ void riemann_face(const DevParams& P, const RunParams& RP,
                                             const StageDesc& D, int i, int j, int k,
                                             const double* __restrict__ W, R* __restrict__ F,
                                             R* __restrict__ Bn, const StepState* states,
                                             const FS& fs) {
  int fnb[3] = {D.vn[0], D.vn[1], D.vn[2]};
  fnb[DIR] += 1;
  const long long fcs = (long long)fnb[0] * fnb[1] * fnb[2];
  R* __restrict__ Fo = F + D.f_off[DIR] + loc(D.vlo, fnb, i, j, k);
  R wl[9], wr[9];
#pragma unroll
  for (int v = 0; v < 9; ++v) {
    const bool on = (v < 8) || P.glm;
    wl[v] = on ? R(fs(0, v)) : R(0);
    wr[v] = on ? R(fs(1, v)) : R(0);
  }
  R g[9];
  plasma_flux<R, DIR>(P, wl, wr, g);
  if (P.glm) {
    R fbn, fpsi;
    dedner_2x2<R>(R(states[D.run].ch), wl[5 + DIR], wl[8], wr[5 + DIR], wr[8], fbn, fpsi);
    g[5 + DIR] = fbn;
    g[8] = fpsi;
  }
  R bn = R(0);
  if (P.divb_method == 1) {
    bn = R(0.5) * (wl[5 + DIR] + wr[5 + DIR]);
    if (!P.periodic[DIR]) {
      const int f = (DIR == 0) ? i : (DIR == 1) ? j : k;
      if (f == RP.dlo[DIR]) bn = wr[5 + DIR];
      if (f == RP.dhi[DIR] + 1) bn = wl[5 + DIR];
    }
  } else if (P.divb_method == 2) {
    const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
    const long long st = (DIR == 0) ? 1 : (DIR == 1) ? (long long)D.fn[0]
                                                     : (long long)D.fn[0] * D.fn[1];
    const double* wv = W + D.u_off + loc(D.flo, D.fn, i, j, k) + (5 + DIR) * cs;
    bn = R(0.5 * (wv[-st] + wv[0]));
  }
  // HELIOBC on the domain boundary (after the Riemann fluxes and Bn)
  const int hside = helio_side<DIR>(P, RP, i, j, k);
  if (hside >= 0) {
    double dl[8], dr[8], dg[8], dbn = double(bn);
#pragma unroll
    for (int v = 0; v < 8; ++v) {
      dl[v] = double(wl[v]);
      dr[v] = double(wr[v]);
    }
    helio_plasma<DIR>(P, RP, hside, dl, dr, dg, dbn);
#pragma unroll
    for (int v = 0; v < 8; ++v) g[v] = R(dg[v]);
    bn = R(dbn);
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) Fo[q * fcs] = g[q];
  if (P.glm) Fo[8 * fcs] = g[8];
  Bn[D.bn_off[DIR] + loc(D.vlo, fnb, i, j, k)] = bn;
  for (int fl = 1; fl < P.nf; ++fl) {
    const int s0 = P.irhon + (fl - 1) * 5;
    R nl[5], nr[5], gn[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      nl[m] = R(fs(0, s0 + m));
      nr[m] = R(fs(1, s0 + m));
    }
    if (hside >= 0) {
      double dl[5], dr[5], dg[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        dl[m] = double(nl[m]);
        dr[m] = double(nr[m]);
      }
      helio_neutral<DIR>(P, hside, fl, dl, dr, dg);
#pragma unroll
      for (int m = 0; m < 5; ++m) gn[m] = R(dg[m]);
    } else {
      vanleer_euler<R, DIR>(P, nl, nr, gn);
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) Fo[(s0 + m) * fcs] = gn[m];
  }
  // tracking surfaces: LEVELSETFLUX (src/LevelSetF.ChF:37-105), the upwind
  // face value by the sign of sqrt(rho_L) u_L + sqrt(rho_R) u_R
  if (P.nls) {
    const R uavg = sqrt(wl[0]) * wl[1 + DIR] + sqrt(wr[0]) * wr[1 + DIR];
    for (int q = P.ils; q < P.nc; ++q) {
      const R l = R(fs(0, q)), r = R(fs(1, q));
      Fo[q * fcs] = (uavg > R(0)) ? l : r;
    }
  }
}

// Corrector fluxes of the Hancock step (correctorHancock, src/PatchMHDAM.cpp:
// 1002-1189): the Riemann problem of each face of the valueBox between the
// high-face value of the low cell and the low-face value of the high cell,
// both shifted by W(t+dt/2) - W(t); Bn from the same states (recomputed
// after the shift in predictorHancock, :981-985); fluxBC of correctorHancock
// (:1105-1106) and LEVELSETFLUX of the shifted face values (:1111-1115).
// Face values: fv[(side*nc + v)*cells(slope) + cell], side 0 = low face,
// 1 = high face.
template <typename R, int DIR>
__global__ void __launch_bounds__(kMaxBlock)
    k_hflux(const __grid_constant__ DevParams P, const double* __restrict__ W, const double* __restrict__ FV,
            R* __restrict__ F, R* __restrict__ Bn, const StageDesc* __restrict__ descs, int ndesc,
            int total, const RunParams* __restrict__ runs, const StepState* __restrict__ states) {
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
  if (gi >= total) return;
  const StageDesc& D = descs[find_desc(descs, ndesc, kRegF + DIR, gi)];
  const int lin = gi - D.g0[kRegF + DIR];
  const RunParams& RP = runs[D.run];
  int fnb[3] = {D.vn[0], D.vn[1], D.vn[2]};
  fnb[DIR] += 1;
  int i, j, k;
  decode(lin, D.vlo, fnb, i, j, k);
  const long long scs = (long long)D.sn[0] * D.sn[1] * D.sn[2];
  const double* __restrict__ fv = FV + D.fv_off[DIR];
  const long long cr = loc(D.slo, D.sn, i, j, k);
  const long long cl = cr - ((DIR == 0) ? 1 : (DIR == 1) ? (long long)D.sn[0]
                                                         : (long long)D.sn[0] * D.sn[1]);
  const int nc = P.nc;
  riemann_face<R, DIR>(P, RP, D, i, j, k, W, F, Bn, states, [&](int side, int v) -> double {
    return side ? fv[v * scs + cr] : fv[(nc + v) * scs + cl];
  });
}

// Face fluxes of one direction by lines (FP64 paths): a block takes whole
// lines of faces along DIR of one patch (LineWork); it first computes the
// limited face values of every cell of its lines once (the cells from one
// below to one above the valueBox along DIR, with the positivity fallback
// and characteristic limiting as k_flux applies them) into shared memory,
// then the Riemann fluxes of the lines' faces from them.  k_flux evaluates
// the limiters of both cells beside each face, i.e. twice per cell; the
// results are the same values (the same face_values calls on the same
// inputs).  Shared memory: sv[(2 v + side) ncell + c], side 0 = low face,
// c = the thread index of the cell in phase 1 (x-fastest order).
template <typename R, int DIR>
__global__ void __launch_bounds__(kLineThreads, 2)
    k_lflux(const __grid_constant__ DevParams P, const double* __restrict__ W, R* __restrict__ F,
            R* __restrict__ Bn, const StageDesc* __restrict__ descs,
            const LineWork* __restrict__ work, const RunParams* __restrict__ runs,
            const StepState* __restrict__ states) {
  extern __shared__ double sv[];
  const LineWork Wk = work[blockIdx.x];
  const StageDesc& D = descs[Wk.desc];
  const RunParams& RP = runs[D.run];
  constexpr int T1 = (DIR == 0) ? 1 : 0, T2 = (DIR == 2) ? 1 : 2;  // transverse dims
  const int nd = D.vn[DIR], nt1 = D.vn[T1];
  const int nl = Wk.nlines, ncl = nd + 2, ncell = nl * ncl;
  const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
  const long long st = (DIR == 0) ? 1 : (DIR == 1) ? (long long)D.fn[0]
                                                   : (long long)D.fn[0] * D.fn[1];
  const int nc = P.nc;
  // phase 1: DIR 0 takes a line's cells consecutively, DIR 1 and 2 the lines
  // (consecutive x) consecutively, so that loads follow the x-fastest layout
  for (int t = threadIdx.x; t < ncell; t += blockDim.x) {
    int line, pos;
    if (DIR == 0) {
      line = t / ncl;
      pos = t - line * ncl;
    } else {
      pos = t / nl;
      line = t - pos * nl;
    }
    const int L = Wk.line0 + line;
    int x[3];
    x[DIR] = D.vlo[DIR] - 1 + pos;
    x[T1] = D.vlo[T1] + L % nt1;
    x[T2] = D.vlo[T2] + L / nt1;
    const double* __restrict__ w0 = W + D.u_off + loc(D.flo, D.fn, x[0], x[1], x[2]);
    bool neg = false;
    double clo[8], chi[8];
    if (P.char_rec) {
      double a8[8], b8[8], c8[8];
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        const double* wv = w0 + v * cs;
        a8[v] = wv[-st];
        b8[v] = wv[0];
        c8[v] = wv[st];
      }
      char_face_values<DIR>(P, a8, b8, c8, clo, chi);
      if (P.check_pos) neg = clo[0] <= 0.0 || chi[0] <= 0.0 || clo[4] <= 0.0 || chi[4] <= 0.0;
    } else if (P.check_pos) {
#pragma unroll
      for (int q = 0; q < 2; ++q) {
        const int v = q ? 4 : 0;
        const double* wv = w0 + v * cs;
        R lo, hi;
        face_values<R>(P.lim[v], R(wv[-st]), R(wv[0]), R(wv[st]), lo, hi);
        if (lo <= R(0) || hi <= R(0)) neg = true;
      }
    }
    for (int v = 0; v < nc; ++v) {
      const double* wv = w0 + v * cs;
      R lo, hi;
      if (neg) {
        lo = R(wv[0]);
        hi = lo;
      } else if (P.char_rec && v < 8) {
        lo = R(clo[v]);
        hi = R(chi[v]);
      } else if (v >= P.ils) {
        ls_face_values<R>(P, R(wv[-st]), R(wv[0]), R(wv[st]), lo, hi);
      } else {
        const int lim = (v < 8) ? P.lim[v] : (int)MF_LIM_MINMOD;
        face_values<R>(lim, R(wv[-st]), R(wv[0]), R(wv[st]), lo, hi);
      }
      sv[(2 * v) * ncell + t] = double(lo);
      sv[(2 * v + 1) * ncell + t] = double(hi);
    }
  }
  __syncthreads();
  // phase 2: the faces of the lines, x-fastest as in phase 1
  const int nfl = nd + 1, nface = nl * nfl;
  for (int t = threadIdx.x; t < nface; t += blockDim.x) {
    int line, f, cl, cr;
    if (DIR == 0) {
      line = t / nfl;
      f = t - line * nfl;
      cl = line * ncl + f;
      cr = cl + 1;
    } else {
      f = t / nl;
      line = t - f * nl;
      cl = f * nl + line;
      cr = cl + nl;
    }
    const int L = Wk.line0 + line;
    int x[3];
    x[DIR] = D.vlo[DIR] + f;
    x[T1] = D.vlo[T1] + L % nt1;
    x[T2] = D.vlo[T2] + L / nt1;
    riemann_face<R, DIR>(P, RP, D, x[0], x[1], x[2], W, F, Bn, states,
                         [&](int side, int v) -> double {
                           return side ? sv[(2 * v) * ncell + cr] : sv[(2 * v + 1) * ncell + cl];
                         });
  }
}

// Launch the line kernel for direction dir on a batch's line work list.
template <typename R>
cudaError_t launch_lflux_t(const DevParams& P, int dir, const double* w, void* f, void* bn,
                           const Batch& b, const LinePlan& lp, const StepState* state,
                           cudaStream_t s) {
  const int n = lp.n[dir];
  if (n <= 0) return cudaSuccess;
  const size_t smem = line_smem_bytes(P.nc, lp.maxcells[dir]);
  R* F = (R*)f;
  R* Bn = (R*)bn;
  if (dir == 0)
    k_lflux<R, 0><<<n, kLineThreads, smem, s>>>(P, w, F, Bn, b.desc, lp.w[0], b.runs, state);
  if (dir == 1)
    k_lflux<R, 1><<<n, kLineThreads, smem, s>>>(P, w, F, Bn, b.desc, lp.w[1], b.runs, state);
  if (dir == 2)
    k_lflux<R, 2><<<n, kLineThreads, smem, s>>>(P, w, F, Bn, b.desc, lp.w[2], b.runs, state);
  return cudaGetLastError();
}

// Allow the line kernels' shared memory (once per device, outside any capture).
template <typename R>
cudaError_t lflux_allow_t() {
  const int most = (int)line_smem_bytes(MF_MAX_COMP, kLineMaxCells);
  cudaError_t e = cudaFuncSetAttribute(k_lflux<R, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_lflux<R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_lflux<R, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
  return e;
}

template <typename R>
cudaError_t launch_hflux_t(const DevParams& P, int dir, const double* w, const double* fv,
                           void* f, void* bn, const Batch& b, const StepState* state,
                           cudaStream_t s) {
  const int tot = b.tot_f[dir];
  if (tot <= 0) return cudaSuccess;
  const int nt = b.nt[1];
  const unsigned g = flat_blocks(tot, nt);
  R* F = (R*)f;
  R* Bn = (R*)bn;
  if (dir == 0) k_hflux<R, 0><<<g, nt, 0, s>>>(P, w, fv, F, Bn, b.desc, b.ndesc, tot, b.runs, state);
  if (dir == 1) k_hflux<R, 1><<<g, nt, 0, s>>>(P, w, fv, F, Bn, b.desc, b.ndesc, tot, b.runs, state);
  if (dir == 2) k_hflux<R, 2><<<g, nt, 0, s>>>(P, w, fv, F, Bn, b.desc, b.ndesc, tot, b.runs, state);
  return cudaGetLastError();
}

// Fluxes of given face states (no reconstruction): the plasma solver, the
// GLM (Bn, psi) system with speed ch and the neutral van Leer fluxes of
// k_flux, one face per thread.  wl / wr / f: n faces x nc primitive values
// (fluxes out as FP64).
template <typename R, int DIR>
__global__ void __launch_bounds__(128)
    k_face_flux(const __grid_constant__ DevParams P, const double* __restrict__ wl, const double* __restrict__ wr,
                double* __restrict__ f, int n, double ch) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const long long o = (long long)t * P.nc;
  R L[9], Rt[9], g[9];
#pragma unroll
  for (int v = 0; v < 9; ++v) {
    const bool on = (v < 8) || P.glm;
    L[v] = on ? R(wl[o + v]) : R(0);
    Rt[v] = on ? R(wr[o + v]) : R(0);
  }
  plasma_flux<R, DIR>(P, L, Rt, g);
  if (P.glm) {
    R fbn, fpsi;
    dedner_2x2<R>(R(ch), L[5 + DIR], L[8], Rt[5 + DIR], Rt[8], fbn, fpsi);
    g[5 + DIR] = fbn;
    g[8] = fpsi;
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) f[o + q] = (double)g[q];
  if (P.glm) f[o + 8] = (double)g[8];
  for (int fl = 1; fl < P.nf; ++fl) {
    const int s0 = P.irhon + (fl - 1) * 5;
    R nl[5], nr[5], gn[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      nl[m] = R(wl[o + s0 + m]);
      nr[m] = R(wr[o + s0 + m]);
    }
    vanleer_euler<R, DIR>(P, nl, nr, gn);
#pragma unroll
    for (int m = 0; m < 5; ++m) f[o + s0 + m] = (double)gn[m];
  }
}

template <typename R>
cudaError_t launch_face_flux_t(const DevParams& P, int dir, const double* wl, const double* wr,
                               double* f, int n, double ch, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const unsigned g = (unsigned)((n + 127) / 128);
  if (dir == 0) k_face_flux<R, 0><<<g, 128, 0, s>>>(P, wl, wr, f, n, ch);
  if (dir == 1) k_face_flux<R, 1><<<g, 128, 0, s>>>(P, wl, wr, f, n, ch);
  if (dir == 2) k_face_flux<R, 2><<<g, 128, 0, s>>>(P, wl, wr, f, n, ch);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// update + sources + positivity (+ RK2 average, + dt)
}  // namespace
}  // namespace mf
