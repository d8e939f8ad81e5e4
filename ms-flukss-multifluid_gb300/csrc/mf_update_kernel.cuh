// mf_update_kernel.cuh - the update kernel (flux divergence, sources,
// positivity, RK2 averaging, per-cell dt).  Included by mf_update.cu (fast
// physics) and mf_update_exact.cu (parity physics); MF_PHYS names the physics
// namespace of the including unit.
#pragma once

#include <type_traits>

#include "mf_fp64.cuh"
#include "mf_kernels.cuh"

namespace mf {
namespace {
using namespace MF_PHYS;

// Difference of the fluxes on the two faces of a cell.  FP64 fluxes: in
// FP64.  FP32 fluxes (mixed precision): in FP32, whose rounding is below the
// FP32 error the fluxes already carry, converted exactly with integer
// instructions (fp64::f2d); the accumulation into the state stays FP64.
__device__ __forceinline__ double flux_diff(double hi, double lo) { return hi - lo; }
__device__ __forceinline__ double flux_diff(float hi, float lo) { return fp64::f2d(hi - lo); }

// Floor of POSTPROCESSING_LS (src/LevelSetF.ChF:426-465) for surface q of
// the cell at x (offset base): the minimum of the stage-start values of the
// cell and its 2*SpaceDim neighbours, lowered to -|maximum|.  Stage-start
// values: the primitive copy wls inside the domain, the state uin on
// far-field ghosts (where the primitive ghost holds boundary values; no stage
// writes there, so uin is the stage-start state even for in-place stages).
__device__ __forceinline__ double ls_floor(const DevParams& P, const RunParams& RP,
                                           const double* __restrict__ wls,
                                           const double* __restrict__ uin, const int* fn,
                                           long long base, long long cs, const int* x, int q) {
  auto old_at = [&](int d, int o) {
    const long long st = (d == 0) ? 1 : (d == 1) ? (long long)fn[0] : (long long)fn[0] * fn[1];
    const long long idx = base + o * st + q * cs;
    const int y = x[d] + o;
    const bool ghost = P.bc_kind == MF_BC_FARFIELD && !P.periodic[d] &&
                       (y < RP.dlo[d] || y > RP.dhi[d]);
    return ghost ? uin[idx] : wls[idx];
  };
  const double c = wls[base + q * cs];
  double Umax = c, Umin = c;
#pragma unroll
  for (int o = -1; o <= 1; o += 2) {
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (d < P.sd) {
        const double v = old_at(d, o);
        Umax = fmax(Umax, v);
        Umin = fmin(Umin, v);
      }
    }
  }
  const double abmax = fabs(Umax);
  return fmin(Umin, -abmax);
}

__device__ __forceinline__ bool dt_less(double a, int ia, double b, int ib) {
  return (a < b) || (a == b && ia < ib);
}

// Block minimum of (dt, flattened index) into partials[slot]: warp
// shuffles, then one thread over the warps.  The flattened index orders cells
// by (patch, Fortran-order index), so the minimum is the reference's
// lexicographic one; it is turned back into (patch, index) once per block.
__device__ __forceinline__ void block_dt_min(double dtc, int myidx,
                                             const StageDesc* __restrict__ descs, int ndesc,
                                             DtPartial* __restrict__ partials, int slot) {
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    double od = __shfl_down_sync(0xffffffffu, dtc, off);
    int oi = __shfl_down_sync(0xffffffffu, myidx, off);
    if (dt_less(od, oi, dtc, myidx)) {
      dtc = od;
      myidx = oi;
    }
  }
  __shared__ double sdt[kMaxBlock / 32];
  __shared__ int sidx[kMaxBlock / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sdt[wid] = dtc;
    sidx[wid] = myidx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double bd = sdt[0];
    int bi = sidx[0];
    const int nw = blockDim.x >> 5;
    for (int q = 1; q < nw; ++q)
      if (dt_less(sdt[q], sidx[q], bd, bi)) {
        bd = sdt[q];
        bi = sidx[q];
      }
    DtPartial pr;
    pr.dt = bd;
    pr.desc = INT_MAX;
    pr.idx = INT_MAX;
    if (bi != INT_MAX) {
      const int di = find_desc(descs, ndesc, kRegV, bi);
      pr.desc = di;
      pr.idx = bi - descs[di].g0[kRegV];
    }
    partials[slot] = pr;
  }
}

// GLM damping factor exp(-dt Ch^2 / Cp^2) of PSIPARABOLIC (src/DednerF.ChF:
// 65-87) for the run of the calling warp: one evaluation per warp instead of
// one per cell (the same expression on the same values), by the first lane
// with a cell, broadcast by shuffle.  A warp never holds cells of two runs
// (each run's cells start on a multiple of kRunAlign); every lane calls.
__device__ __forceinline__ double warp_psi_damping(const StageDesc* Dp,
                                                   const StepState* __restrict__ states,
                                                   double dt_scale) {
  const unsigned m = __ballot_sync(0xffffffffu, Dp != nullptr);
  if (!m) return 1.0;
  const int src = __ffs(m) - 1;
  double v = 1.0;
  if ((int)(threadIdx.x & 31) == src) {
    const StepState& S = states[Dp->run];
    const double dt = S.dt * dt_scale;
    v = exp(-dt * S.ch * S.ch / (S.cp * S.cp));
  }
  return __shfl_sync(0xffffffffu, v, src);
}

// The stage-start primitive state of a cell as the update tail reads it:
// all components in registers, or a column of the W array read where used.
struct WArray {
  double v[MF_MAX_COMP];
};
struct WColumn {
  const double* __restrict__ p;
  long long cs;
  __device__ __forceinline__ double operator[](int q) const { return __ldg(p + q * cs); }
};
__device__ __forceinline__ const double* w_arg(const WArray& w) { return w.v; }
__device__ __forceinline__ const WColumn& w_arg(const WColumn& w) { return w; }

// The update of one cell after its flux divergence: u holds the stage-start
// state minus dt/dx times the flux differences (UPDATECONS); divB is the
// cell's face-normal B divergence (8-wave source).  Sources with the
// stage-start primitive state, the GLM damping psi_damp, charge exchange,
// problem post-processing and positivity, the tracking surfaces' floor, RK2
// averaging, the store, and the cell's dt (into dtc / myidx = g).
// CE: arithmetic type of the charge-exchange rates (double, or float in the
// MF_PREC_MIXED_CE32 form); R: type of the face fluxes (the wave speeds'
// type).
template <typename R, int GLM, int FLAGS, typename CE>
__device__ __forceinline__ void update_tail(const DevParams& P, const StageBuffers& B,
                                            const StageDesc& D, const RunParams& RP,
                                            StepState* __restrict__ ss, int i, int j, int k,
                                            long long base, long long cs, double dt,
                                            double psi_damp, double divB, double* u, int g,
                                            double& dtc, int& myidx) {
  constexpr int IRHON = 8 + GLM;
  const double* __restrict__ wst = B.wls ? B.wls : B.w;
  // addExplicitSources (srcIdeal/PatchMHDMF.cpp:1149-1389) with the
  // stage-start primitive state
  // FP64 fluxes: the primitive state in registers.  FP32 fluxes (mixed
  // precision, 2 blocks per SM): a column view that loads each component
  // where it is used, which keeps the register count within the bound.
  typename std::conditional<sizeof(R) == 4, WColumn, WArray>::type ws;
  if constexpr (sizeof(R) == 4) {
    ws.p = B.w + base;
    ws.cs = cs;
  } else if (P.use8 || (P.ce && P.nf >= 2)) {
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.ils) ws.v[q] = B.w[base + q * cs];
  }
  const auto& w = w_arg(ws);
  if (P.use8) {
    // SOURCE8WAVES (srcIdeal/PatchIdealMHDF.ChF:681-722) + ADDSOURCES
    const double dtbydx = dt / RP.dx;
    const double dB = -divB * dtbydx;
    const double Ux = w[1], Uy = w[2], Uz = w[3];
    const double Bx = kInv4Pi * w[5], By = kInv4Pi * w[6], Bz = kInv4Pi * w[7];
    u[1] = u[1] + dB * Bx;
    u[2] = u[2] + dB * By;
    u[3] = u[3] + dB * Bz;
    u[4] = u[4] + dB * (Bx * Ux + By * Uy + Bz * Uz);
    u[5] = u[5] + dB * Ux;
    u[6] = u[6] + dB * Uy;
    u[7] = u[7] + dB * Uz;
  }
  if (GLM) u[8] = psi_damp * u[8];  // PSIPARABOLIC (src/DednerF.ChF:65-87)
  if (P.ce && P.nf >= 2) {
    const double regtr = P.reg_tracer ? B.w[base + (P.nc - 1) * cs] : 0.0;
    const int reg = region_cell(P, RP.dx, i, j, k, w, regtr);
    // three neutral populations (the multi-fluid model's usual 4 fluids)
    // with a compile-time count, others with the run-time one
    if (P.nf == 4)
      charge_exchange_add<IRHON, CE, typename std::decay<decltype(w)>::type, 3>(P, w, reg, dt, u);
    else
      charge_exchange_add<IRHON, CE>(P, w, reg, dt, u);
  }
  // problem post-processing and positivity (src/PatchMHDAM.cpp:705-707); with
  // constrained transport they follow the recalculation of B (k_recalc_b)
  if (!P.ct) {
    if (P.reinit) reinit_cell(P, RP.dx, i, j, k, stage_time(*ss, dt), u);
    positivity_cell<IRHON>(P, u);
  }
  if (P.nls) {  // POSTPROCESSING_LS (srcIdeal/PatchMHDMF.cpp:1414-1424)
    const int x[3] = {i, j, k};
    const double f0 = ls_floor(P, RP, wst, B.uin, D.fn, base, cs, x, P.ils);
    const double f1 = (P.nls > 1) ? ls_floor(P, RP, wst, B.uin, D.fn, base, cs, x, P.ils + 1)
                                  : 0.0;
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q >= P.ils && q < P.nc) u[q] = fmax(u[q], (q == P.ils) ? f0 : f1);
  }

  if (FLAGS & kStageAverage) {  // AVERAGESTATE (src/PatchMHDAMF.ChF:289-316), every state
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.nc) u[q] = u[q] + 0.5 * (B.uold[base + q * cs] - B.uin[base + q * cs]);
  }
  bool finite = true;
#pragma unroll
  for (int q = 0; q < MF_MAX_COMP; ++q)
    if (q < P.nc) {
      // exponent field not all ones: an integer test, off the FP64 pipe
      finite = finite && ((__double2hiint(u[q]) & 0x7ff00000) != 0x7ff00000);
      B.uout[base + q * cs] = u[q];
    }
  if (!finite) atomicOr(&ss->flags, kFlagNonFinite);
  if (FLAGS & kStageDt) {
    dtc = RP.dx / max_wave_speed<IRHON, R>(P, u);
    myidx = g;
    if (B.divb && P.use8) B.divb[loc(B.divb_lo, B.divb_n, i, j, k)] = divB;
  }
}

// The update of cell g of the batch's flat cell index (g >= total: no cell)
// by every thread of a block; the block's dt minimum goes to partials[slot].
template <typename R, int GLM, int FLAGS, typename CE>
__device__ __forceinline__ void update_cells(const DevParams& P, const StageBuffers& B,
                                             const StageDesc* __restrict__ descs, int ndesc,
                                             int g, int total, const RunParams* __restrict__ runs,
                                             StepState* __restrict__ states,
                                             const double dt_scale,
                                             DtPartial* __restrict__ partials, int slot) {
  double dtc = DBL_MAX;
  int myidx = INT_MAX;
  const StageDesc* Dp = nullptr;
  int lin = 0;
  if (g < total) {
    Dp = &descs[find_desc(descs, ndesc, kRegV, g)];
    lin = g - Dp->g0[kRegV];
    if (lin >= Dp->vn[0] * Dp->vn[1] * Dp->vn[2]) Dp = nullptr;  // run-alignment gap
  }
  const double psi_damp = GLM ? warp_psi_damping(Dp, states, dt_scale) : 1.0;
  if (Dp) {
    const StageDesc& D = *Dp;
    const RunParams& RP = runs[D.run];
    StepState* __restrict__ ss = states + D.run;
    int i, j, k;
    decode(lin, D.vlo, D.vn, i, j, k);
    const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
    const long long base = D.u_off + loc(D.flo, D.fn, i, j, k);
    const double dt = ss->dt * dt_scale;
    const double* __restrict__ wst = B.wls ? B.wls : B.w;
    double u[MF_MAX_COMP];
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.nc) u[q] = B.uin[base + q * cs];

    // UPDATECONS (src/PatchMHDAMF.ChF:542-587), one direction after another.
    // FP32 fluxes (mixed precision): the differences of the directions are
    // summed in FP32 and enter the FP64 state once per component, so that
    // each component costs one conversion instead of one per direction.
    const double dtinv = dt * RP.invdx;
    float fsum[sizeof(R) == 4 ? MF_MAX_COMP : 1];
    if constexpr (sizeof(R) == 4) {
#pragma unroll
      for (int q = 0; q < MF_MAX_COMP; ++q) fsum[q] = 0.0f;
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (d < P.sd) {
        int fnb[3] = {D.vn[0], D.vn[1], D.vn[2]};
        fnb[d] += 1;
        const long long fcs = (long long)fnb[0] * fnb[1] * fnb[2];
        const long long sf = (d == 0) ? 1 : (d == 1) ? (long long)fnb[0]
                                                     : (long long)fnb[0] * fnb[1];
        const R* __restrict__ Fd = (const R*)B.f[d] + D.f_off[d] + loc(D.vlo, fnb, i, j, k);
        if constexpr (sizeof(R) == 4) {
#pragma unroll
          for (int q = 0; q < MF_MAX_COMP; ++q)
            if (q < P.ils) fsum[q] = fsum[q] + (Fd[q * fcs + sf] - Fd[q * fcs]);
        } else {
#pragma unroll
          for (int q = 0; q < MF_MAX_COMP; ++q)
            if (q < P.ils)
              u[q] = u[q] - dtinv * flux_diff(Fd[q * fcs + sf], Fd[q * fcs]);
        }
        // UPDATELEVELSET (src/LevelSetF.ChF:200-234): the tracking surfaces,
        // non-conservative with the stage-start cell velocity
        if (P.nls) {
          const double vel = wst[base + (1 + d) * cs];
          const double cf = dt / RP.dx * vel;
#pragma unroll
          for (int q = 0; q < MF_MAX_COMP; ++q)
            if (q >= P.ils && q < P.nc)
              u[q] = u[q] - cf * flux_diff(Fd[q * fcs + sf], Fd[q * fcs]);
        }
      }
    }
    if constexpr (sizeof(R) == 4) {
#pragma unroll
      for (int q = 0; q < MF_MAX_COMP; ++q)
        if (q < P.ils) u[q] = u[q] - dtinv * fp64::f2d(fsum[q]);
    }
    double divB = 0.0;
    if (P.use8) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if (d < P.sd) {
          int fnb[3] = {D.vn[0], D.vn[1], D.vn[2]};
          fnb[d] += 1;
          const long long sf = (d == 0) ? 1 : (d == 1) ? (long long)fnb[0]
                                                       : (long long)fnb[0] * fnb[1];
          const R* __restrict__ Bd = (const R*)B.bn[d] + D.bn_off[d] + loc(D.vlo, fnb, i, j, k);
          if constexpr (sizeof(R) == 4)
            divB = divB + fp64::f2d(Bd[sf] - Bd[0]);  // COMPUTEDIVB, FP32 difference
          else
            divB = divB + (double)Bd[sf] - (double)Bd[0];  // COMPUTEDIVB
        }
      }
    }
    update_tail<R, GLM, FLAGS, CE>(P, B, D, RP, ss, i, j, k, base, cs, dt, psi_damp, divB, u, g,
                                   dtc, myidx);
  }
  if (FLAGS & kStageDt) block_dt_min(dtc, myidx, descs, ndesc, partials, slot);
}

template <typename R, int GLM, int FLAGS, typename CE = double>
__global__ void __launch_bounds__(kMaxBlock, sizeof(R) == 4 ? 2 : 1)
    k_update(const __grid_constant__ DevParams P, const __grid_constant__ StageBuffers B, const StageDesc* __restrict__ descs,
             int ndesc, int first, int total, const RunParams* __restrict__ runs,
             StepState* __restrict__ states, const double dt_scale,
             DtPartial* __restrict__ partials) {
  // cells [first, total) of the batch's flat cell index; first is a multiple
  // of the block size, so block b writes the dt partial first/blockDim + b of
  // the launch over the whole batch
  update_cells<R, GLM, FLAGS, CE>(P, B, descs, ndesc, first + blockIdx.x * blockDim.x + threadIdx.x,
                                  total, runs, states, dt_scale, partials,
                                  first / (int)blockDim.x + (int)blockIdx.x);
}

}  // namespace
}  // namespace mf
