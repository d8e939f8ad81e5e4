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

template <typename R, int DIR>
__global__ void __launch_bounds__(kMaxBlock)
    k_flux(const DevParams P, const double* __restrict__ W, R* __restrict__ F,
           R* __restrict__ Bn, const StageDesc* __restrict__ descs, int ndesc, int total,
           const RunParams* __restrict__ runs, const StepState* __restrict__ states) {
  const int gi = blockIdx.x * blockDim.x + threadIdx.x;
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
      const double* wv = w0 + v * cs;
      R a = R(wv[-2 * st]), b = R(wv[-st]), c = R(wv[0]), d = R(wv[st]);
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
      const double* wv = w0 + v * cs;
      R a = R(wv[-2 * st]), b = R(wv[-st]), c = R(wv[0]), d = R(wv[st]);
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
#pragma unroll
  for (int q = 0; q < 8; ++q) Fo[q * fcs] = g[q];
  if (P.glm) Fo[8 * fcs] = g[8];

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
  Bn[D.bn_off[DIR] + fo] = bn;

  // neutral fluids: minmod face states, van Leer splitting (VANLEERF)
  for (int fl = 1; fl < P.nf; ++fl) {
    const int s = P.irhon + (fl - 1) * 5;
    R nl[5], nr[5], gn[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const double* wv = w0 + (s + m) * cs;
      R a = R(wv[-2 * st]), b = R(wv[-st]), c = R(wv[0]), d = R(wv[st]);
      R lo, hi;
      face_values<R>(MF_LIM_MINMOD, a, b, c, lo, hi);
      nl[m] = negL ? b : hi;
      face_values<R>(MF_LIM_MINMOD, b, c, d, lo, hi);
      nr[m] = negR ? c : lo;
    }
    vanleer_euler<R, DIR>(P, nl, nr, gn);
#pragma unroll
    for (int m = 0; m < 5; ++m) Fo[(s + m) * fcs] = gn[m];
  }
}

// Corrector fluxes of the Hancock step (correctorHancock, src/PatchMHDAM.cpp:
// 1002-1189): the Riemann problem of each face of the valueBox between the
// high-face value of the low cell and the low-face value of the high cell,
// both shifted by W(t+dt/2) - W(t); Bn from the same states (recomputed
// after the shift in predictorHancock, :981-985).  Face values: fv[(side*nc
// + v)*cells(slope) + cell], side 0 = low face, 1 = high face.
template <typename R, int DIR>
__global__ void __launch_bounds__(kMaxBlock)
    k_hflux(const DevParams P, const double* __restrict__ W, const double* __restrict__ FV,
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
  const long long fcs = (long long)fnb[0] * fnb[1] * fnb[2];
  R* __restrict__ Fo = F + D.f_off[DIR] + loc(D.vlo, fnb, i, j, k);
  R wl[9], wr[9];
#pragma unroll
  for (int v = 0; v < 9; ++v) {
    const bool on = (v < 8) || P.glm;
    wl[v] = on ? R(fv[(nc + v) * scs + cl]) : R(0);
    wr[v] = on ? R(fv[v * scs + cr]) : R(0);
  }
  R g[9];
  plasma_flux<R, DIR>(P, wl, wr, g);
  if (P.glm) {
    R fbn, fpsi;
    dedner_2x2<R>(R(states[D.run].ch), wl[5 + DIR], wl[8], wr[5 + DIR], wr[8], fbn, fpsi);
    g[5 + DIR] = fbn;
    g[8] = fpsi;
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) Fo[q * fcs] = g[q];
  if (P.glm) Fo[8 * fcs] = g[8];
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
  Bn[D.bn_off[DIR] + loc(D.vlo, fnb, i, j, k)] = bn;
  for (int fl = 1; fl < P.nf; ++fl) {
    const int s0 = P.irhon + (fl - 1) * 5;
    R nl[5], nr[5], gn[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      nl[m] = R(fv[(nc + s0 + m) * scs + cl]);
      nr[m] = R(fv[(s0 + m) * scs + cr]);
    }
    vanleer_euler<R, DIR>(P, nl, nr, gn);
#pragma unroll
    for (int m = 0; m < 5; ++m) Fo[(s0 + m) * fcs] = gn[m];
  }
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
    k_face_flux(const DevParams P, const double* __restrict__ wl, const double* __restrict__ wr,
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
