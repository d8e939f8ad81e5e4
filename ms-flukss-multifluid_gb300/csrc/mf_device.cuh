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
  double gamma, hgamma, invhgamma, invgamma, smallr, smallp, del2, smallB, dx, invdx;
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

}  // namespace mf
