// mf_hancock_exact.cu - the Hancock time step (PatchMHDAM::updateState with
// TA_Hancock, src/PatchMHDAM.cpp:1287-1301): predictorHancock (:836-1000)
// with dt/2 on box.grow(1), then correctorHancock (:1002-1189) with dt.
//
//   k_prim     primitive state on the predictor's W box (valueBox.grow(2))
//   k_hfaces   limited face values of every cell of the slope box
//              (Reconstruction::faceValues + checkPositivity)
//   k_hpredict per cell of the predictor valueBox: point fluxes of the face
//              values (FLUXESHANCOCK / _E), UPDATECONSHANCOCK with dt/2,
//              sources with W(t) and Bn of the face values, W(t+dt/2)
//   k_hshift   face values += W(t+dt/2) - W(t) (UPDATEVALUESONFACES)
//   k_hflux    corrector Riemann fluxes of the shifted face values (flux units)
//   k_update   UPDATECONS with dt, sources with W(t+dt/2), reset, positivity, dt
//
// The predictor always runs in FP64 with the reference's rounding (this unit
// is built with -fmad=false); the corrector fluxes and update follow the
// context's precision mode.
#include "mf_kernels.cuh"

#define MF_PHYS exact
#include "mf_sources_exact.cuh"

namespace mf {
namespace {
using namespace exact;

__device__ __forceinline__ long long dstride(const int* n, int d) {
  return (d == 0) ? 1 : (d == 1) ? (long long)n[0] : (long long)n[0] * n[1];
}

__global__ void __launch_bounds__(kMaxBlock)
    k_hfaces(const __grid_constant__ DevParams P, const double* __restrict__ W, HancockBuffers H,
             const StageDesc* __restrict__ descs, int ndesc, int total) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const StageDesc& D = descs[find_desc(descs, ndesc, kRegS, g)];
  const int lin = g - D.g0[kRegS];
  int i, j, k;
  decode(lin, D.slo, D.sn, i, j, k);
  const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
  const long long scs = (long long)D.sn[0] * D.sn[1] * D.sn[2];
  const double* __restrict__ w0 = W + D.u_off + loc(D.flo, D.fn, i, j, k);
  const int nc = P.nc;
  for (int d = 0; d < P.sd; ++d) {
    const long long st = dstride(D.fn, d);
    double* __restrict__ fv = H.fv[d] + D.fv_off[d] + lin;
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
      if (d == 0) char_face_values<0>(P, a8, b8, c8, clo, chi);
      else if (d == 1) char_face_values<1>(P, a8, b8, c8, clo, chi);
      else char_face_values<2>(P, a8, b8, c8, clo, chi);
      if (P.check_pos) neg = clo[0] <= 0.0 || chi[0] <= 0.0 || clo[4] <= 0.0 || chi[4] <= 0.0;
    } else if (P.check_pos) {
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        const int v = t ? 4 : 0;
        const double* wv = w0 + v * cs;
        double lo, hi;
        face_values<double>(P.lim[v], wv[-st], wv[0], wv[st], lo, hi);
        if (lo <= 0.0 || hi <= 0.0) neg = true;
      }
    }
    for (int v = 0; v < nc; ++v) {
      const double* wv = w0 + v * cs;
      double lo, hi;
      if (neg) {
        lo = wv[0];
        hi = wv[0];
      } else if (P.char_rec && v < 8) {
        lo = clo[v];
        hi = chi[v];
      } else if (v >= P.ils) {
        ls_face_values<double>(P, wv[-st], wv[0], wv[st], lo, hi);
      } else {
        const int lim = (v < 8) ? P.lim[v] : (int)MF_LIM_MINMOD;
        face_values<double>(lim, wv[-st], wv[0], wv[st], lo, hi);
      }
      fv[v * scs] = lo;
      fv[(nc + v) * scs] = hi;
    }
  }
}

// FLUXESHANCOCK (srcIdeal/PatchIdealMHDF.ChF:235-297) + FLUXESHANCOCK_E
// (srcIdeal/PatchEulerF.ChF:417-468): physical flux in direction D of one
// primitive state.  The psi flux is unset in the reference; zero here.
template <int D, int IRHON>
__device__ __forceinline__ void point_flux(const DevParams& P, const double* w, double* F) {
  constexpr int in = 1 + D, it1 = 1 + (D + 1) % 3, it2 = 1 + (D + 2) % 3;
  constexpr int inB = 5 + D, itB1 = 5 + (D + 1) % 3, itB2 = 5 + (D + 2) % 3;
  const double rho = fmax(P.smallr, w[0]);
  const double u = w[in], v = w[it1], ww = w[it2];
  double pr = fmax(P.smallp, w[4]);
  const double bx = w[inB], by = w[itB1], bz = w[itB2];
  const double b = kInv8Pi * (bx * bx + by * by + bz * bz);
  const double ke = 0.5 * (u * u + v * v + ww * ww);
  const double bu = bx * u + by * v + bz * ww;
  double e = pr * P.invhgamma + rho * ke;
  pr = pr + b;
  e = e + b;
  F[0] = rho * u;
  F[in] = rho * u * u + pr - kInv4Pi * bx * bx;
  F[it1] = rho * u * v - kInv4Pi * bx * by;
  F[it2] = rho * u * ww - kInv4Pi * bx * bz;
  F[4] = u * (e + pr) - kInv4Pi * bx * bu;
  F[inB] = 0.0;
  F[itB1] = u * by - v * bx;
  F[itB2] = u * bz - ww * bx;
  if (IRHON == 9) F[8] = 0.0;
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f) {
    if (f < P.nf) {
      const int s = IRHON + (f - 1) * 5;
      const double r = fmax(P.smallr, w[s]);
      const double un = w[s + 1 + D], vn = w[s + 1 + (D + 1) % 3], wn = w[s + 1 + (D + 2) % 3];
      const double pn = fmax(P.smallp, w[s + 4]);
      const double k2 = 0.5 * (un * un + vn * vn + wn * wn);
      const double en = pn * P.invhgamma + r * k2;
      F[s] = r * un;
      F[s + 1 + D] = r * un * un + pn;
      F[s + 1 + (D + 1) % 3] = r * un * vn;
      F[s + 1 + (D + 2) % 3] = r * un * wn;
      F[s + 4] = un * (en + pn);
    }
  }
  // FLUXESHANCOCK_LS (src/LevelSetF.ChF:9-35): surface times the plasma
  // normal velocity
#pragma unroll
  for (int q = 0; q < MF_MAX_COMP; ++q)
    if (q >= P.ils && q < P.nc) F[q] = w[q] * w[in];
}

// Bn of one face (PatchMHDMF::computeBn, srcIdeal/PatchMHDMF.cpp:509-620)
// from the face values of the two cells (method 1) or the cell states
// (method 2); f = face index in direction d.
__device__ __forceinline__ double face_bn(const DevParams& P, const RunParams& RP, int d, int f,
                                          double wl, double wr, double cl, double cr) {
  if (P.divb_method == 0) return 0.0;
  if (P.divb_method == 2) return 0.5 * (cl + cr);
  double bn = 0.5 * (wl + wr);
  if (!P.periodic[d]) {
    if (f == RP.dlo[d]) bn = wr;
    if (f == RP.dhi[d] + 1) bn = wl;
  }
  return bn;
}

// One direction of the predictor update of a cell: the point fluxes of its
// two face values, the flux difference with dt/2, and the two face Bn.
template <int D, int IRHON>
__device__ __forceinline__ void hpredict_dir(const DevParams& P, const RunParams& RP,
                                             const StageDesc& Dc, const HancockBuffers& H,
                                             const double* __restrict__ W, long long base,
                                             long long cs, long long scs, long long c,
                                             const int* x, int nc, double dtinv, double dtp,
                                             double* u, double& divB) {
  const double* __restrict__ fv = H.fv[D] + Dc.fv_off[D];
  double wm[MF_MAX_COMP], wp[MF_MAX_COMP], fm[MF_MAX_COMP], fp[MF_MAX_COMP];
#pragma unroll
  for (int v = 0; v < MF_MAX_COMP; ++v)
    if (v < nc) {
      wm[v] = fv[v * scs + c];
      wp[v] = fv[(nc + v) * scs + c];
    }
  point_flux<D, IRHON>(P, wm, fm);
  point_flux<D, IRHON>(P, wp, fp);
#pragma unroll
  for (int q = 0; q < MF_MAX_COMP; ++q)
    if (q < P.ils) u[q] = u[q] - dtinv * (fp[q] - fm[q]);
  if (P.nls) {  // UPDATELEVELSETHANCOCK (src/LevelSetF.ChF:354-388), W(t) velocity
    const double cf = dtp / RP.dx * W[base + (1 + D) * cs];
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q >= P.ils && q < nc) u[q] = u[q] - cf * (fp[q] - fm[q]);
  }
  const long long ss = dstride(Dc.sn, D);
  const long long fs = dstride(Dc.fn, D);
  const double* wbn = W + base + (5 + D) * cs;
  const double bn_lo = face_bn(P, RP, D, x[D], fv[(nc + 5 + D) * scs + c - ss],
                               fv[(5 + D) * scs + c], wbn[-fs], wbn[0]);
  const double bn_hi = face_bn(P, RP, D, x[D] + 1, fv[(nc + 5 + D) * scs + c],
                               fv[(5 + D) * scs + c + ss], wbn[0], wbn[fs]);
  divB = divB + bn_hi - bn_lo;
}

template <int GLM>
__global__ void __launch_bounds__(kMaxBlock)
    k_hpredict(const __grid_constant__ DevParams P, const double* __restrict__ U, const double* __restrict__ W,
               HancockBuffers H, const StageDesc* __restrict__ descs, int ndesc, int total,
               const RunParams* __restrict__ runs, const StepState* __restrict__ states) {
  constexpr int IRHON = 8 + GLM;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const StageDesc& D = descs[find_desc(descs, ndesc, kRegV, g)];
  const int lin = g - D.g0[kRegV];
  const RunParams& RP = runs[D.run];
  const StepState& SS = states[D.run];
  int i, j, k;
  decode(lin, D.vlo, D.vn, i, j, k);
  const int x[3] = {i, j, k};
  const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
  const long long base = D.u_off + loc(D.flo, D.fn, i, j, k);
  const long long scs = (long long)D.sn[0] * D.sn[1] * D.sn[2];
  const long long c = loc(D.slo, D.sn, i, j, k);
  const int nc = P.nc;
  const double dtp = 0.5 * SS.dt;
  double u[MF_MAX_COMP];
#pragma unroll
  for (int q = 0; q < MF_MAX_COMP; ++q)
    if (q < nc) u[q] = U[base + q * cs];
  // updateHancock -> UPDATECONSHANCOCK (src/PatchMHDAMF.ChF:589-638), one
  // direction after another; divB from Bn of the face values (COMPUTEDIVB)
  const double dtinv = dtp * RP.invdx;
  double divB = 0.0;
  hpredict_dir<0, IRHON>(P, RP, D, H, W, base, cs, scs, c, x, nc, dtinv, dtp, u, divB);
  if (P.sd > 1)
    hpredict_dir<1, IRHON>(P, RP, D, H, W, base, cs, scs, c, x, nc, dtinv, dtp, u, divB);
  if (P.sd > 2)
    hpredict_dir<2, IRHON>(P, RP, D, H, W, base, cs, scs, c, x, nc, dtinv, dtp, u, divB);
  // addExplicitSources with W(t) and dt/2 (srcIdeal/PatchMHDMF.cpp:1149-1389)
  double w[MF_MAX_COMP];
#pragma unroll
  for (int q = 0; q < MF_MAX_COMP; ++q)
    if (q < nc) w[q] = W[base + q * cs];
  if (P.use8) {
    const double dB = -divB * (dtp / RP.dx);
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
  if (GLM) u[8] = exp(-dtp * SS.ch * SS.ch / (SS.cp * SS.cp)) * u[8];
  if (P.ce && P.nf >= 2) {
    const double regtr = P.reg_tracer ? W[base + (nc - 1) * cs] : 0.0;
    const int reg = region_cell(P, RP.dx, i, j, k, w, regtr);
    charge_exchange_add<IRHON>(P, w, reg, dtp, u);
  }
  // W(t + dt/2) (stateToPrim of the predicted state)
  double wo[MF_MAX_COMP];
  cons_to_prim_plasma(P, u, wo);
  if (GLM) wo[8] = u[8];
#pragma unroll
  for (int f = 1; f < MF_MAX_FLUIDS; ++f)
    if (f < P.nf) cons_to_prim_euler(P, u + IRHON + (f - 1) * 5, wo + IRHON + (f - 1) * 5);
#pragma unroll
  for (int q = 0; q < MF_MAX_COMP; ++q)
    if (q >= P.ils && q < nc) wo[q] = u[q];
#pragma unroll
  for (int q = 0; q < MF_MAX_COMP; ++q)
    if (q < nc) H.w2[base + q * cs] = wo[q];
}

__global__ void __launch_bounds__(kMaxBlock)
    k_hshift(const __grid_constant__ DevParams P, const double* __restrict__ W, HancockBuffers H,
             const StageDesc* __restrict__ descs, int ndesc, int total,
             const RunParams* __restrict__ runs) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const StageDesc& D = descs[find_desc(descs, ndesc, kRegS, g)];
  const int lin = g - D.g0[kRegS];
  const RunParams& RP = runs[D.run];
  int x[3];
  decode(lin, D.slo, D.sn, x[0], x[1], x[2]);
  const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
  const long long scs = (long long)D.sn[0] * D.sn[1] * D.sn[2];
  const int nc = P.nc;
  auto in_v = [&](const int* y) {
    for (int d = 0; d < 3; ++d)
      if (y[d] < D.vlo[d] || y[d] >= D.vlo[d] + D.vn[d]) return false;
    return true;
  };
  // W(t+dt/2) - W(t): predicted cells; far-field ghosts of neutral fluids
  // 2.. copy the nearest domain cell (HELIOGS); every other cell 0
  double delta[MF_MAX_COMP];
#pragma unroll
  for (int q = 0; q < MF_MAX_COMP; ++q) delta[q] = 0.0;
  if (in_v(x)) {
    const long long b = D.u_off + loc(D.flo, D.fn, x[0], x[1], x[2]);
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < nc) delta[q] = H.w2[b + q * cs] - W[b + q * cs];
  } else if (P.bc_kind == MF_BC_FARFIELD && P.nf > 2) {
    int od = -1;
    for (int d = 0; d < P.sd; ++d)
      if (!P.periodic[d] && (x[d] < RP.dlo[d] || x[d] > RP.dhi[d])) od = d;
    if (od >= 0) {
      int y[3] = {x[0], x[1], x[2]};
      y[od] = (y[od] < RP.dlo[od]) ? RP.dlo[od] : RP.dhi[od];
      if (in_v(y)) {
        const long long b = D.u_off + loc(D.flo, D.fn, y[0], y[1], y[2]);
#pragma unroll
        for (int q = 0; q < MF_MAX_COMP; ++q)
          if (q >= P.irhon + 5 && q < nc) delta[q] = H.w2[b + q * cs] - W[b + q * cs];
      }
    }
  }
  for (int d = 0; d < P.sd; ++d) {
    double* __restrict__ fv = H.fv[d] + D.fv_off[d] + lin;
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < nc) {
        fv[q * scs] = fv[q * scs] + delta[q];
        fv[(nc + q) * scs] = fv[(nc + q) * scs] + delta[q];
      }
  }
}

}  // namespace

cudaError_t launch_hancock(const DevParams& P, int precision, const StageBuffers& B,
                           const HancockBuffers& H, const Batch& a, const Batch& c,
                           StepState* state, DtPartial* partials, int* nblocks_v,
                           cudaStream_t s, int corrector_flags) {
  int ne = 0;
  auto mark = [&]() {
    if (B.ev) cudaEventRecord(B.ev[ne++], s);
  };
  cudaError_t e = launch_prim(P, B.uin, B.w, a, s);
  if (e != cudaSuccess) return e;
  mark();
  const int nt = a.nt[0];
  if (a.tot_s > 0)
    k_hfaces<<<flat_blocks(a.tot_s, nt), nt, 0, s>>>(P, B.w, H, a.desc, a.ndesc, a.tot_s);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  mark();
  const int nt2 = a.nt[2];
  if (a.tot_v > 0) {
    if (P.glm)
      k_hpredict<1><<<flat_blocks(a.tot_v, nt2), nt2, 0, s>>>(P, B.uin, B.w, H, a.desc, a.ndesc,
                                                              a.tot_v, a.runs, state);
    else
      k_hpredict<0><<<flat_blocks(a.tot_v, nt2), nt2, 0, s>>>(P, B.uin, B.w, H, a.desc, a.ndesc,
                                                              a.tot_v, a.runs, state);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  mark();
  if (a.tot_s > 0)
    k_hshift<<<flat_blocks(a.tot_s, nt), nt, 0, s>>>(P, B.w, H, a.desc, a.ndesc, a.tot_s, a.runs);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  mark();
  for (int d = 0; d < P.sd; ++d) {
    if (precision == MF_PREC_MIXED)
      e = launch_hflux_fast<float>(P, d, B.w, H.fv[d], B.f[d], B.bn[d], c, state, s);
    else if (precision == MF_PREC_FP64_FAST)
      e = launch_hflux_fast<double>(P, d, B.w, H.fv[d], B.f[d], B.bn[d], c, state, s);
    else
      e = launch_hflux_exact(P, d, B.w, H.fv[d], B.f[d], B.bn[d], c, state, s);
    if (e != cudaSuccess) return e;
    mark();
  }
  StageBuffers B2 = B;
  B2.w = H.w2;
  B2.wls = B.w;
  const int fl = corrector_flags;
  if (precision == MF_PREC_MIXED)
    e = launch_update_fast<float>(P, B2, c, fl, 1.0, state, partials, nblocks_v, s);
  else if (precision == MF_PREC_FP64_FAST)
    e = launch_update_fast<double>(P, B2, c, fl, 1.0, state, partials, nblocks_v, s);
  else
    e = launch_update_exact(P, B2, c, fl, 1.0, state, partials, nblocks_v, s);
  if (e != cudaSuccess) return e;
  mark();
  return cudaSuccess;
}

}  // namespace mf
