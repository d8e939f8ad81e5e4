// mf_prim_exact.cu - conserved -> primitive variables on valueBox.grow(2), and
// the neutral pass-through at the sun after a level step.
//
// Built with -fmad=false: the primitive state feeds the limiter sign tests
// and the region thresholds, so it is rounded exactly as in the CPU
// restatement of the reference (EqSysMHDMF::stateToPrim).  The FP32 copy of
// W (mixed precision) is rounded to nearest by fp64::d2f, which gives the
// conversion instruction's bits with integer instructions (the kernel is
// bound by the FP64 pipe, where the conversion instruction issues).
#include "mf_internal.h"
#include "mf_fp64.cuh"
#include "mf_kernels.cuh"

namespace mf {
namespace {
template <int GLM>
__global__ void __launch_bounds__(kMaxBlock)
    k_prim(const __grid_constant__ DevParams P, const double* __restrict__ U, double* __restrict__ W,
           float* __restrict__ Wf, const StageDesc* __restrict__ descs, int ndesc, int total,
           const RunParams* __restrict__ runs) {
  constexpr int IRHON = 8 + GLM;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const StageDesc& D = descs[find_desc(descs, ndesc, kRegW, g)];
  const int lin = g - D.g0[kRegW];
  const RunParams& R = runs[D.run];
  int i, j, k;
  decode(lin, D.wlo, D.wn, i, j, k);
  const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
  const long long base = D.u_off + loc(D.flo, D.fn, i, j, k);
  int od = -1;
  if (P.bc_kind == MF_BC_FARFIELD) {
    const int x[3] = {i, j, k};
    for (int d = 0; d < P.sd; ++d)
      if (!P.periodic[d] && (x[d] < R.dlo[d] || x[d] > R.dhi[d])) od = d;
  }
  double w[MF_MAX_COMP];
  if (od < 0) {
    double u[MF_MAX_COMP];
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.ils) u[q] = U[base + q * cs];
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
    for (int q = 0; q < 8; ++q) w[q] = R.bc_plasma[q];
    if (GLM) w[8] = 0.0;
    if (P.nf > 1) {
#pragma unroll
      for (int q = 0; q < 5; ++q) w[IRHON + q] = R.bc_n1[q];
    }
    int x[3] = {i, j, k};
    x[od] = (x[od] < R.dlo[od]) ? R.dlo[od] : R.dhi[od];
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
    if (q < P.ils) W[base + q * cs] = w[q];
  // tracking surfaces: copied (EqSysMHDMF::stateToPrim, srcIdeal/EqSysMHDMF.cpp:
  // 207-210); on far-field ghosts the region tracer holds +1 (HELIOGS
  // :996-1000) and the other surfaces, which HELIOGS leaves unassigned, keep
  // U's ghost value
  for (int q = P.ils; q < P.nc; ++q)
    W[base + q * cs] = (od >= 0 && P.reg_tracer && q == P.nc - 1) ? 1.0 : U[base + q * cs];
  if (Wf) {  // the FP32 copy the mixed-precision flux kernels read
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.ils) Wf[base + q * cs] = fp64::d2f(w[q]);
    for (int q = P.ils; q < P.nc; ++q) Wf[base + q * cs] = fp64::d2f(W[base + q * cs]);
  }
}

// Far-field ghosts of the primitive state, exactly as k_prim's far-field
// branch fills them (HELIOGS, swlism/HeliosphericF.ChF:978-1140), for the
// levels whose valid-cell primitives and ghost copies come first: plasma and
// neutral fluid 1 from the boundary state, the other neutral fluids from the
// primitive state of the nearest cell along the boundary normal.  That cell,
// when it lies in the domain, is a valid cell of the patch or a ghost cell
// filled by the copy before this launch (its FP64 state when that copy ran,
// else the FP32 copy, the only one read downstream); outside the domain (a
// corner) its conserved state never changes and is converted here.
template <int GLM>
__global__ void __launch_bounds__(256)
    k_farfield(const __grid_constant__ DevParams P, const double* __restrict__ U, double* __restrict__ W,
               float* __restrict__ Wf, const FarReg* __restrict__ regs,
               const RunParams* __restrict__ runs, int have_w) {
  constexpr int IRHON = 8 + GLM;
  const FarReg F = regs[blockIdx.x];
  const RunParams& R = runs[F.run];
  const int n = F.ext[0] * F.ext[1] * F.ext[2];
  const long long cs = (long long)F.fn[0] * F.fn[1] * F.fn[2];
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    int i, j, k;
    decode(t, F.lo, F.ext, i, j, k);
    const long long base = F.off + loc(F.flo, F.fn, i, j, k);
    int x[3] = {i, j, k};
    int od = -1;
    for (int d = 0; d < P.sd; ++d)
      if (!P.periodic[d] && (x[d] < R.dlo[d] || x[d] > R.dhi[d])) od = d;
    if (od < 0) continue;  // (the regions hold far-field cells only)
    double w[MF_MAX_COMP];
    float wf[MF_MAX_COMP];
#pragma unroll
    for (int q = 0; q < 8; ++q) w[q] = R.bc_plasma[q];
    if (GLM) w[8] = 0.0;
    if (P.nf > 1) {
#pragma unroll
      for (int q = 0; q < 5; ++q) w[IRHON + q] = R.bc_n1[q];
    }
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q) wf[q] = fp64::d2f(w[q]);
    x[od] = (x[od] < R.dlo[od]) ? R.dlo[od] : R.dhi[od];
    bool inside = true;
    for (int d = 0; d < P.sd; ++d)
      if (!P.periodic[d] && (x[d] < R.dlo[d] || x[d] > R.dhi[d])) inside = false;
    const long long eb = F.off + loc(F.flo, F.fn, x[0], x[1], x[2]);
#pragma unroll
    for (int f = 2; f < MF_MAX_FLUIDS; ++f) {
      if (f < P.nf) {
        const int s0 = IRHON + (f - 1) * 5;
        if (!inside) {
          double u5[5];
#pragma unroll
          for (int q = 0; q < 5; ++q) u5[q] = U[eb + (s0 + q) * cs];
          cons_to_prim_euler(P, u5, w + s0);
#pragma unroll
          for (int q = 0; q < 5; ++q) wf[s0 + q] = fp64::d2f(w[s0 + q]);
        } else if (have_w) {
#pragma unroll
          for (int q = 0; q < 5; ++q) {
            w[s0 + q] = W[eb + (s0 + q) * cs];
            wf[s0 + q] = fp64::d2f(w[s0 + q]);
          }
        } else {
#pragma unroll
          for (int q = 0; q < 5; ++q) {
            wf[s0 + q] = Wf[eb + (s0 + q) * cs];
            w[s0 + q] = (double)wf[s0 + q];
          }
        }
      }
    }
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.ils) {
        W[base + q * cs] = w[q];
        if (Wf) Wf[base + q * cs] = wf[q];
      }
    for (int q = P.ils; q < P.nc; ++q) {
      const double v = (P.reg_tracer && q == P.nc - 1) ? 1.0 : U[base + q * cs];
      W[base + q * cs] = v;
      if (Wf) Wf[base + q * cs] = fp64::d2f(v);
    }
  }
}

// ---------------------------------------------------------------------------
// face fluxes in direction DIR
}  // namespace

cudaError_t launch_farfield(const DevParams& P, const double* u, double* w, float* wf,
                            const FarReg* far, int nfar, const RunParams* runs, int have_w,
                            cudaStream_t s) {
  if (nfar <= 0) return cudaSuccess;
  if (P.glm)
    k_farfield<1><<<nfar, 256, 0, s>>>(P, u, w, wf, far, runs, have_w);
  else
    k_farfield<0><<<nfar, 256, 0, s>>>(P, u, w, wf, far, runs, have_w);
  return cudaGetLastError();
}

cudaError_t launch_prim(const DevParams& P, const double* uin, double* w, const Batch& b,
                        cudaStream_t s, float* wf) {
  if (b.tot_w <= 0) return cudaSuccess;
  const int nt = b.nt[0];
  const unsigned gw = flat_blocks(b.tot_w, nt);
  if (P.glm)
    k_prim<1><<<gw, nt, 0, s>>>(P, uin, w, wf, b.desc, b.ndesc, b.tot_w, b.runs);
  else
    k_prim<0><<<gw, nt, 0, s>>>(P, uin, w, wf, b.desc, b.ndesc, b.tot_w, b.runs);
  return cudaGetLastError();
}

}  // namespace mf

namespace mf {
namespace {
// NEUTRALS_SUNBC (swlism/SWLISMF.ChF:1555-1598): neutral fluid 1 (and 4)
// from the mirror cell, y and z momenta reversed.
__global__ void k_sun_copy(double* __restrict__ U, const SunPair* __restrict__ pairs, int n,
                           int irhon, int nf) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const SunPair sp = pairs[t];
  const double sg[5] = {1.0, 1.0, -1.0, -1.0, 1.0};
  for (int f = 1; f < nf; f += 3) {  // fluids 1 and 4
    const int s0 = irhon + (f - 1) * 5;
#pragma unroll
    for (int m = 0; m < 5; ++m)
      U[sp.to + (long long)(s0 + m) * sp.cs_to] =
          sg[m] * U[sp.from + (long long)(s0 + m) * sp.cs_from];
  }
}
}  // namespace

cudaError_t launch_sun_copy(double* U, const SunPair* pairs, int n, int irhon, int nf,
                            cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_sun_copy<<<(n + 127) / 128, 128, 0, s>>>(U, pairs, n, irhon, nf);
  return cudaGetLastError();
}
}  // namespace mf
