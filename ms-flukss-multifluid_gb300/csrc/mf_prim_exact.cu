// mf_prim_exact.cu - conserved -> primitive variables on valueBox.grow(2), and
// the neutral pass-through at the sun after a level step.
//
// Built with -fmad=false: the primitive state feeds the limiter sign tests
// and the region thresholds, so it is rounded exactly as in the CPU
// restatement of the reference (EqSysMHDMF::stateToPrim).
#include "mf_internal.h"
#include "mf_kernels.cuh"

namespace mf {
namespace {
template <int GLM>
__global__ void __launch_bounds__(kMaxBlock)
    k_prim(const DevParams P, const double* __restrict__ U, double* __restrict__ W,
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
      if (q < P.ils) Wf[base + q * cs] = (float)w[q];
    for (int q = P.ils; q < P.nc; ++q) Wf[base + q * cs] = (float)W[base + q * cs];
  }
}

// ---------------------------------------------------------------------------
// face fluxes in direction DIR
}  // namespace

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
