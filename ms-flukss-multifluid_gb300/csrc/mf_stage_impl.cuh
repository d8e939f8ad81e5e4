// mf_stage_impl.cuh - the stage kernels of the GB300 patch integrator.
//
// One explicit stage of PatchMHDAM::EulerStep (src/PatchMHDAM.cpp:495-709) is
// three kernels over every patch of a batch (blockIdx.y = patch):
//   k_prim    conserved -> primitive on valueBox.grow(2) (+ far-field ghosts)
//   k_flux<D> limited face states and the Riemann fluxes of every face of
//             valueBox in direction D (plasma, GLM, each neutral fluid) + Bn
//   k_update  flux divergence, 8-wave / GLM / charge-exchange sources, the
//             inner-sphere reset, positivity, RK2 averaging and the per-cell dt
// Threads map to consecutive x cells/faces, so every load and store of the
// component-major FArrayBox data is coalesced.
//
// This file is included by two translation units: mf_stage_fp64.cu (FP64
// reconstruction and fluxes, compiled without multiply-add contraction so that
// every operation rounds as in the CPU restatement) and mf_stage_mixed.cu
// (FP32 reconstruction and fluxes, contraction allowed).  MF_STAGE_REAL selects
// the flux precision; MF_STAGE_COMMON marks the unit that also defines the
// precision-independent kernels.
#pragma once

#include "mf_kernels.cuh"

#include <cfloat>
#include <climits>

namespace mf {
namespace {

constexpr int kBlock = 128;

__device__ __forceinline__ long long loc(const int* lo, const int* n, int i, int j, int k) {
  return (long long)(i - lo[0]) +
         (long long)n[0] * ((long long)(j - lo[1]) + (long long)n[1] * (long long)(k - lo[2]));
}

__device__ __forceinline__ void decode(int lin, const int* lo, const int* n, int& i, int& j,
                                       int& k) {
  i = lo[0] + lin % n[0];
  int t = lin / n[0];
  j = lo[1] + t % n[1];
  k = lo[2] + t / n[1];
}

// ---------------------------------------------------------------------------
// primitive variables
// ---------------------------------------------------------------------------
template <int GLM>
__global__ void __launch_bounds__(kBlock)
    k_prim(const DevParams P, const double* __restrict__ U, double* __restrict__ W,
           const StageDesc* __restrict__ descs) {
  constexpr int IRHON = 8 + GLM;
  const StageDesc& D = descs[blockIdx.y];
  const int n = D.wn[0] * D.wn[1] * D.wn[2];
  const int lin = blockIdx.x * blockDim.x + threadIdx.x;
  if (lin >= n) return;
  int i, j, k;
  decode(lin, D.wlo, D.wn, i, j, k);
  const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
  const long long base = D.u_off + loc(D.flo, D.fn, i, j, k);
  int od = -1;
  if (P.bc_kind == MF_BC_FARFIELD) {
    const int x[3] = {i, j, k};
    for (int d = 0; d < P.sd; ++d)
      if (!P.periodic[d] && (x[d] < P.dlo[d] || x[d] > P.dhi[d])) od = d;
  }
  double w[MF_MAX_COMP];
  if (od < 0) {
    double u[MF_MAX_COMP];
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.nc) u[q] = U[base + q * cs];
    cons_to_prim_plasma(P, u, w);
    if (GLM) w[8] = u[8];
#pragma unroll
    for (int f = 1; f < MF_MAX_FLUIDS; ++f)
      if (f < P.nf) cons_to_prim_euler(P, u + IRHON + (f - 1) * 5, w + IRHON + (f - 1) * 5);
  } else {
    // far-field ghost (HELIOGS, swlism/HeliosphericF.ChF:978-1140): plasma and
    // neutral fluid 1 from the boundary state, the other neutral fluids copy the
    // primitive state of the nearest domain cell along the boundary normal.
#pragma unroll
    for (int q = 0; q < 8; ++q) w[q] = P.bc_plasma[q];
    if (GLM) w[8] = 0.0;
    if (P.nf > 1) {
#pragma unroll
      for (int q = 0; q < 5; ++q) w[IRHON + q] = P.bc_n1[q];
    }
    int x[3] = {i, j, k};
    x[od] = (x[od] < P.dlo[od]) ? P.dlo[od] : P.dhi[od];
    const long long eb = D.u_off + loc(D.flo, D.fn, x[0], x[1], x[2]);
#pragma unroll
    for (int f = 2; f < MF_MAX_FLUIDS; ++f) {
      if (f < P.nf) {
        double u5[5];
#pragma unroll
        for (int q = 0; q < 5; ++q) u5[q] = U[eb + (IRHON + (f - 1) * 5 + q) * cs];
        cons_to_prim_euler(P, u5, w + IRHON + (f - 1) * 5);
      }
    }
  }
#pragma unroll
  for (int q = 0; q < MF_MAX_COMP; ++q)
    if (q < P.nc) W[base + q * cs] = w[q];
}

// ---------------------------------------------------------------------------
// face fluxes in direction DIR
// ---------------------------------------------------------------------------
template <typename R, int DIR>
__global__ void __launch_bounds__(kBlock)
    k_flux(const DevParams P, const double* __restrict__ W, R* __restrict__ F,
           R* __restrict__ Bn, const StageDesc* __restrict__ descs,
           const StepState* __restrict__ ss) {
  const StageDesc& D = descs[blockIdx.y];
  int fnb[3] = {D.vn[0], D.vn[1], D.vn[2]};
  fnb[DIR] += 1;
  const int n = fnb[0] * fnb[1] * fnb[2];
  const int lin = blockIdx.x * blockDim.x + threadIdx.x;
  if (lin >= n) return;
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
  if (P.check_pos) {
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
  R wl[9], wr[9];
#pragma unroll
  for (int v = 0; v < 9; ++v) {
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
  if (P.rs == kRoe8)
    roe_mhd<R, DIR, false>(P, wl, wr, g);
  else if (P.rs == kRoe7)
    roe_mhd<R, DIR, true>(P, wl, wr, g);
  else
    rusanov_mhd<R, DIR>(P, wl, wr, g);
  if (P.glm) {
    R fbn, fpsi;
    dedner_2x2<R>(R(ss->ch), wl[5 + DIR], wl[8], wr[5 + DIR], wr[8], fbn, fpsi);
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
      if (f == P.dlo[DIR]) bn = wr[5 + DIR];
      if (f == P.dhi[DIR] + 1) bn = wl[5 + DIR];
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

// ---------------------------------------------------------------------------
// update + sources + positivity (+ RK2 average, + dt)
// ---------------------------------------------------------------------------
__device__ __forceinline__ bool dt_less(double a, int ia, double b, int ib) {
  return (a < b) || (a == b && ia < ib);
}

template <typename R, int GLM, int FLAGS>
__global__ void __launch_bounds__(kBlock)
    k_update(const DevParams P, const StageBuffers B, const StageDesc* __restrict__ descs,
             StepState* __restrict__ ss, const double dt_scale, DtPartial* __restrict__ partials) {
  constexpr int IRHON = 8 + GLM;
  const StageDesc& D = descs[blockIdx.y];
  const int n = D.vn[0] * D.vn[1] * D.vn[2];
  const int lin = blockIdx.x * blockDim.x + threadIdx.x;
  double dtc = DBL_MAX;
  int myidx = INT_MAX;
  if (lin < n) {
    int i, j, k;
    decode(lin, D.vlo, D.vn, i, j, k);
    const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
    const long long base = D.u_off + loc(D.flo, D.fn, i, j, k);
    const double dt = ss->dt * dt_scale;
    double u[MF_MAX_COMP];
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.nc) u[q] = B.uin[base + q * cs];

    // UPDATECONS (src/PatchMHDAMF.ChF:542-587), one direction after another
    const double dtinv = dt * P.invdx;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      if (d < P.sd) {
        int fnb[3] = {D.vn[0], D.vn[1], D.vn[2]};
        fnb[d] += 1;
        const long long fcs = (long long)fnb[0] * fnb[1] * fnb[2];
        const long long sf = (d == 0) ? 1 : (d == 1) ? (long long)fnb[0]
                                                     : (long long)fnb[0] * fnb[1];
        const R* __restrict__ Fd = (const R*)B.f[d] + D.f_off[d] + loc(D.vlo, fnb, i, j, k);
#pragma unroll
        for (int q = 0; q < MF_MAX_COMP; ++q)
          if (q < P.nc)
            u[q] = u[q] - dtinv * ((double)Fd[q * fcs + sf] - (double)Fd[q * fcs]);
      }
    }

    // addExplicitSources (srcIdeal/PatchMHDMF.cpp:1149-1389) with the
    // stage-start primitive state
    double w[MF_MAX_COMP];
    const bool need_w = P.use8 || (P.ce && P.nf >= 2);
    if (need_w) {
#pragma unroll
      for (int q = 0; q < MF_MAX_COMP; ++q)
        if (q < P.nc) w[q] = B.w[base + q * cs];
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
          divB = divB + (double)Bd[sf] - (double)Bd[0];  // COMPUTEDIVB
        }
      }
      // SOURCE8WAVES (srcIdeal/PatchIdealMHDF.ChF:681-722) + ADDSOURCES
      const double dtbydx = dt / P.dx;
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
    if (GLM) {  // PSIPARABOLIC (src/DednerF.ChF:65-87)
      const double ch = ss->ch, cp = ss->cp;
      u[8] = exp(-dt * ch * ch / (cp * cp)) * u[8];
    }
    if (P.ce && P.nf >= 2) {
      const int reg = region_cell(P, i, j, k, w);
      charge_exchange_add<IRHON>(P, w, reg, dt, u);
    }
    if (P.reinit) reinit_cell(P, i, j, k, u);
    positivity_cell<IRHON>(P, u);

    if (FLAGS & kStageAverage) {  // AVERAGESTATE (src/PatchMHDAMF.ChF:289-316)
#pragma unroll
      for (int q = 0; q < MF_MAX_COMP; ++q)
        if (q < P.nc) u[q] = u[q] + 0.5 * (B.uold[base + q * cs] - B.uin[base + q * cs]);
    }
    bool finite = true;
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.nc) {
        finite = finite && isfinite(u[q]);
        B.uout[base + q * cs] = u[q];
      }
    if (!finite) atomicOr(&ss->flags, kFlagNonFinite);
    if (FLAGS & kStageDt) {
      dtc = P.dx / max_wave_speed<IRHON>(P, u);
      myidx = lin;
      if (B.divb && P.use8) B.divb[loc(B.divb_lo, B.divb_n, i, j, k)] = divB;
    }
  }
  if (FLAGS & kStageDt) {
    // block minimum of (dt, index): warp shuffles, then one warp
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      double od = __shfl_down_sync(0xffffffffu, dtc, off);
      int oi = __shfl_down_sync(0xffffffffu, myidx, off);
      if (dt_less(od, oi, dtc, myidx)) {
        dtc = od;
        myidx = oi;
      }
    }
    __shared__ double sdt[kBlock / 32];
    __shared__ int sidx[kBlock / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
      sdt[wid] = dtc;
      sidx[wid] = myidx;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double bd = sdt[0];
      int bi = sidx[0];
      for (int q = 1; q < kBlock / 32; ++q)
        if (dt_less(sdt[q], sidx[q], bd, bi)) {
          bd = sdt[q];
          bi = sidx[q];
        }
      DtPartial pr;
      pr.dt = bd;
      pr.desc = blockIdx.y;
      pr.idx = bi;
      partials[(long long)blockIdx.y * gridDim.x + blockIdx.x] = pr;
    }
  }
}

// PatchMHDMF::computeDt on its own: dx / max wave speed over the valueBox
template <int GLM>
__global__ void __launch_bounds__(kBlock)
    k_dt(const DevParams P, const double* __restrict__ U, const StageDesc* __restrict__ descs,
         DtPartial* __restrict__ partials) {
  constexpr int IRHON = 8 + GLM;
  const StageDesc& D = descs[blockIdx.y];
  const int n = D.vn[0] * D.vn[1] * D.vn[2];
  const int lin = blockIdx.x * blockDim.x + threadIdx.x;
  double dtc = DBL_MAX;
  int myidx = INT_MAX;
  if (lin < n) {
    int i, j, k;
    decode(lin, D.vlo, D.vn, i, j, k);
    const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
    const long long base = D.u_off + loc(D.flo, D.fn, i, j, k);
    double u[MF_MAX_COMP];
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.nc) u[q] = U[base + q * cs];
    dtc = P.dx / max_wave_speed<IRHON>(P, u);
    myidx = lin;
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    double od = __shfl_down_sync(0xffffffffu, dtc, off);
    int oi = __shfl_down_sync(0xffffffffu, myidx, off);
    if (dt_less(od, oi, dtc, myidx)) {
      dtc = od;
      myidx = oi;
    }
  }
  __shared__ double sdt[kBlock / 32];
  __shared__ int sidx[kBlock / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    sdt[wid] = dtc;
    sidx[wid] = myidx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double bd = sdt[0];
    int bi = sidx[0];
    for (int q = 1; q < kBlock / 32; ++q)
      if (dt_less(sdt[q], sidx[q], bd, bi)) {
        bd = sdt[q];
        bi = sidx[q];
      }
    DtPartial pr;
    pr.dt = bd;
    pr.desc = blockIdx.y;
    pr.idx = bi;
    partials[(long long)blockIdx.y * gridDim.x + blockIdx.x] = pr;
  }
}

__device__ __forceinline__ bool part_less(const DtPartial& a, const DtPartial& b) {
  if (a.dt < b.dt) return true;
  if (a.dt > b.dt) return false;
  if (a.desc != b.desc) return a.desc < b.desc;
  return a.idx < b.idx;
}

__global__ void __launch_bounds__(256)
    k_finalize(const DevParams P, const DtPartial* __restrict__ parts, int np,
               StepState* __restrict__ ss, int advance) {
  DtPartial best;
  best.dt = DBL_MAX;
  best.desc = INT_MAX;
  best.idx = INT_MAX;
  for (int q = threadIdx.x; q < np; q += blockDim.x) {
    DtPartial c = parts[q];
    if (part_less(c, best)) best = c;
  }
  __shared__ DtPartial sb[256];
  sb[threadIdx.x] = best;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s && part_less(sb[threadIdx.x + s], sb[threadIdx.x]))
      sb[threadIdx.x] = sb[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    best = sb[0];
    ss->dt_min = best.dt;
    ss->min_desc = best.desc;
    ss->min_idx = best.idx;
    if (!(best.dt > 0.0) || best.dt >= DBL_MAX) atomicOr(&ss->flags, kFlagBadDt);
    if (advance) {
      // AMRLevelIdealMHD::advance (srcIdeal/AMRLevelIdealMHD.cpp:1531-1548, 1588)
      const double dtn = best.dt;
      ss->dt = ss->cfl * dtn;
      if (P.glm && P.factor_ch > 0.0) {
        const double ch = P.factor_ch * P.dx / dtn;
        ss->ch = ch;
        ss->cp = sqrt(ch * P.dx / P.factor_cp);
      }
    }
  }
}

__global__ void __launch_bounds__(256)
    k_exchange(double* __restrict__ U, const CopyReg* __restrict__ regs, int nc) {
  const CopyReg R = regs[blockIdx.x];
  const int n = R.ext[0] * R.ext[1] * R.ext[2];
  const long long scs = (long long)R.sfn[0] * R.sfn[1] * R.sfn[2];
  const long long dcs = (long long)R.dfn[0] * R.dfn[1] * R.dfn[2];
  const long long tot = (long long)n * nc;
  for (long long t = threadIdx.x; t < tot; t += blockDim.x) {
    const int q = (int)(t / n);
    const int c = (int)(t - (long long)q * n);
    const int a = c % R.ext[0];
    const int r = c / R.ext[0];
    const int b = r % R.ext[1];
    const int e = r / R.ext[1];
    const long long so = R.src_off + q * scs + (R.s0[0] + a) +
                         (long long)R.sfn[0] * ((R.s0[1] + b) + (long long)R.sfn[1] * (R.s0[2] + e));
    const long long dof = R.dst_off + q * dcs + (R.d0[0] + a) +
                          (long long)R.dfn[0] * ((R.d0[1] + b) + (long long)R.dfn[1] * (R.d0[2] + e));
    U[dof] = U[so];
  }
}

template <typename R>
__global__ void k_flux_out(int nc, const R* __restrict__ f2, int l20, int l21, int l22, int n20,
                           int n21, int n22, const R* __restrict__ f1, int l10, int l11, int l12,
                           int n10, int n11, int n12, double* __restrict__ out, int lo0, int lo1,
                           int lo2, int on0, int on1, int on2) {
  const long long n = (long long)on0 * on1 * on2;
  const long long cs2 = (long long)n20 * n21 * n22, cs1 = (long long)n10 * n11 * n12;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n * nc;
       t += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(t / n);
    const long long c = t - (long long)q * n;
    const int a = (int)(c % on0);
    const long long r = c / on0;
    const int b = (int)(r % on1);
    const int e = (int)(r / on1);
    const int i = lo0 + a, j = lo1 + b, k = lo2 + e;
    const long long i2 = q * cs2 + (i - l20) + (long long)n20 * ((j - l21) + (long long)n21 * (k - l22));
    double v = (double)f2[i2];
    if (f1) {
      const long long i1 =
          q * cs1 + (i - l10) + (long long)n10 * ((j - l11) + (long long)n11 * (k - l12));
      v = v + (double)f1[i1];
      v = v * 0.5;
    }
    out[t] = v;
  }
}

template <typename R>
cudaError_t stage_impl(const DevParams& P, const StageBuffers& B, const StageDesc* d_desc,
                       int ndesc, long long max_w, const long long max_f[3], long long max_v,
                       int flags, double dt_scale, StepState* state, DtPartial* partials,
                       int* nblocks_v, cudaStream_t s) {
  const dim3 gw((unsigned)((max_w + kBlock - 1) / kBlock), (unsigned)ndesc);
  if (P.glm)
    k_prim<1><<<gw, kBlock, 0, s>>>(P, B.uin, B.w, d_desc);
  else
    k_prim<0><<<gw, kBlock, 0, s>>>(P, B.uin, B.w, d_desc);
  for (int d = 0; d < P.sd; ++d) {
    const dim3 gf((unsigned)((max_f[d] + kBlock - 1) / kBlock), (unsigned)ndesc);
    R* F = (R*)B.f[d];
    R* Bn = (R*)B.bn[d];
    if (d == 0) k_flux<R, 0><<<gf, kBlock, 0, s>>>(P, B.w, F, Bn, d_desc, state);
    if (d == 1) k_flux<R, 1><<<gf, kBlock, 0, s>>>(P, B.w, F, Bn, d_desc, state);
    if (d == 2) k_flux<R, 2><<<gf, kBlock, 0, s>>>(P, B.w, F, Bn, d_desc, state);
  }
  const dim3 gv((unsigned)((max_v + kBlock - 1) / kBlock), (unsigned)ndesc);
  if (nblocks_v) *nblocks_v = (int)(gv.x * gv.y);
#define MF_UPD(G, FL) k_update<R, G, FL><<<gv, kBlock, 0, s>>>(P, B, d_desc, state, dt_scale, partials)
  if (P.glm) {
    if (flags == 0) MF_UPD(1, 0);
    else if (flags == kStageDt) MF_UPD(1, kStageDt);
    else MF_UPD(1, kStageAverage | kStageDt);
  } else {
    if (flags == 0) MF_UPD(0, 0);
    else if (flags == kStageDt) MF_UPD(0, kStageDt);
    else MF_UPD(0, kStageAverage | kStageDt);
  }
#undef MF_UPD
  return cudaGetLastError();
}

}  // namespace

#ifdef MF_STAGE_COMMON
cudaError_t launch_stage_fp64(const DevParams& P, const StageBuffers& B, const StageDesc* d_desc,
                              int ndesc, long long max_w, const long long max_f[3],
                              long long max_v, int flags, double dt_scale, StepState* state,
                              DtPartial* partials, int* nblocks_v, cudaStream_t s) {
  return stage_impl<double>(P, B, d_desc, ndesc, max_w, max_f, max_v, flags, dt_scale, state,
                            partials, nblocks_v, s);
}
#else
cudaError_t launch_stage_mixed(const DevParams& P, const StageBuffers& B,
                               const StageDesc* d_desc, int ndesc, long long max_w,
                               const long long max_f[3], long long max_v, int flags,
                               double dt_scale, StepState* state, DtPartial* partials,
                               int* nblocks_v, cudaStream_t s) {
  return stage_impl<float>(P, B, d_desc, ndesc, max_w, max_f, max_v, flags, dt_scale, state,
                           partials, nblocks_v, s);
}
#endif

#ifdef MF_STAGE_COMMON
cudaError_t launch_dt(const DevParams& P, const double* u, const StageDesc* d_desc, int ndesc,
                      long long max_v, DtPartial* partials, int* nblocks, cudaStream_t s) {
  const dim3 gv((unsigned)((max_v + kBlock - 1) / kBlock), (unsigned)ndesc);
  if (nblocks) *nblocks = (int)(gv.x * gv.y);
  if (P.glm)
    k_dt<1><<<gv, kBlock, 0, s>>>(P, u, d_desc, partials);
  else
    k_dt<0><<<gv, kBlock, 0, s>>>(P, u, d_desc, partials);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const DevParams& P, const DtPartial* partials, int npart,
                            StepState* state, int advance, cudaStream_t s) {
  k_finalize<<<1, 256, 0, s>>>(P, partials, npart, state, advance);
  return cudaGetLastError();
}

cudaError_t launch_exchange(double* u, const CopyReg* regs, int nreg, int nc, cudaStream_t s) {
  if (nreg <= 0) return cudaSuccess;
  k_exchange<<<nreg, 256, 0, s>>>(u, regs, nc);
  return cudaGetLastError();
}

cudaError_t launch_flux_out(int mixed, int sd, int nc, const void* const f2[3],
                            const int f2lo[3][3], const int f2n[3][3], const void* const f1[3],
                            const int f1lo[3][3], const int f1n[3][3], double* const fout[3],
                            const int olo[3][3], const int on[3][3], cudaStream_t s) {
  for (int d = 0; d < sd; ++d) {
    long long n = (long long)on[d][0] * on[d][1] * on[d][2] * nc;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    if (blocks < 1) blocks = 1;
    if (mixed)
      k_flux_out<float><<<blocks, 256, 0, s>>>(
          nc, (const float*)f2[d], f2lo[d][0], f2lo[d][1], f2lo[d][2], f2n[d][0], f2n[d][1],
          f2n[d][2], (const float*)f1[d], f1lo[d][0], f1lo[d][1], f1lo[d][2], f1n[d][0],
          f1n[d][1], f1n[d][2], fout[d], olo[d][0], olo[d][1], olo[d][2], on[d][0], on[d][1],
          on[d][2]);
    else
      k_flux_out<double><<<blocks, 256, 0, s>>>(
          nc, (const double*)f2[d], f2lo[d][0], f2lo[d][1], f2lo[d][2], f2n[d][0], f2n[d][1],
          f2n[d][2], (const double*)f1[d], f1lo[d][0], f1lo[d][1], f1lo[d][2], f1n[d][0],
          f1n[d][1], f1n[d][2], fout[d], olo[d][0], olo[d][1], olo[d][2], on[d][0], on[d][1],
          on[d][2]);
  }
  return cudaGetLastError();
}

#endif  // MF_STAGE_COMMON

}  // namespace mf
