// mf_prim_exact.cu - conserved -> primitive variables on valueBox.grow(2).
//
// Built with -fmad=false: the primitive state feeds the limiter sign tests
// and the region thresholds, so it is rounded exactly as in the CPU
// restatement of the reference (EqSysMHDMF::stateToPrim).
#include "mf_kernels.cuh"

namespace mf {
namespace {
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
}  // namespace

cudaError_t launch_prim(const DevParams& P, const double* uin, double* w, const StageDesc* d_desc,
                        int ndesc, long long max_w, cudaStream_t s) {
  const dim3 gw((unsigned)((max_w + kBlock - 1) / kBlock), (unsigned)ndesc);
  if (P.glm)
    k_prim<1><<<gw, kBlock, 0, s>>>(P, uin, w, d_desc);
  else
    k_prim<0><<<gw, kBlock, 0, s>>>(P, uin, w, d_desc);
  return cudaGetLastError();
}

}  // namespace mf
