// mf_fu.cu - the overlapped form of a mixed-precision stage's flux and update
// launches.  The stage's patches are cut into chunks; launch k computes the
// FP32 face fluxes of chunk k and the update of chunk k - 1, in one grid
// whose blocks alternate between the two (even blocks: fluxes, odd blocks:
// update, then the rest of the larger part), so that every SM holds blocks
// of both: the update is bound by the FP64 pipe and leaves most issue slots
// to the flux blocks, which use the FP32, integer and load pipes.  Launches
// follow each other on one stream, so chunk k's fluxes are complete before
// its update starts in launch k + 1; no block waits on another.
#define MF_PHYS fast
#include "mf_riemann.cuh"
#include "mf_flux_kernel.cuh"
#include "mf_sources.cuh"
#include "mf_update_kernel.cuh"

namespace mf {
namespace {

struct FUJob {
  int f0[3], f1[3], nfb[3];  // faces [f0, f1) per direction and their blocks
  int v0, v1, nub;           // cells [v0, v1) to update and their blocks
};

template <int GLM, int FLAGS, typename CE>
__global__ void __launch_bounds__(kMaxBlock, 2)
    k_flux_update(const __grid_constant__ DevParams P, const __grid_constant__ StageBuffers B,
                  const StageDesc* __restrict__ descs, int ndesc,
                  const RunParams* __restrict__ runs, StepState* __restrict__ states,
                  const double dt_scale, DtPartial* __restrict__ partials,
                  const __grid_constant__ FUJob J) {
  const int nf = J.nfb[0] + J.nfb[1] + J.nfb[2], nu = J.nub;
  const int m = min(nf, nu);
  const int b = blockIdx.x;
  int fb = -1, ub = -1;
  if (b < 2 * m) {
    if (b & 1)
      ub = b >> 1;
    else
      fb = b >> 1;
  } else if (nf > nu) {
    fb = b - m;
  } else {
    ub = b - m;
  }
  const int t = threadIdx.x, bd = blockDim.x;
  if (fb >= 0) {  // a block of face fluxes (the role is the same for the whole block)
    if (fb < J.nfb[0]) {
      flux_face<float, 0, 1>(P, B.w, B.wf, (float*)B.f[0], (float*)B.bn[0], descs, ndesc,
                             J.f0[0] + fb * bd + t, J.f1[0], runs, states);
    } else if (fb < J.nfb[0] + J.nfb[1]) {
      flux_face<float, 1, 1>(P, B.w, B.wf, (float*)B.f[1], (float*)B.bn[1], descs, ndesc,
                             J.f0[1] + (fb - J.nfb[0]) * bd + t, J.f1[1], runs, states);
    } else {
      flux_face<float, 2, 1>(P, B.w, B.wf, (float*)B.f[2], (float*)B.bn[2], descs, ndesc,
                             J.f0[2] + (fb - J.nfb[0] - J.nfb[1]) * bd + t, J.f1[2], runs,
                             states);
    }
  } else {  // a block of cell updates; its dt partial is the unchunked launch's
    update_cells<float, GLM, FLAGS, CE>(P, B, descs, ndesc, J.v0 + ub * bd + t, J.v1, runs,
                                        states, dt_scale, partials, J.v0 / bd + ub);
  }
}

template <int GLM, int FLAGS>
cudaError_t fu_launch(const DevParams& P, const StageBuffers& B, const Batch& b,
                      StepState* state, double dt_scale, DtPartial* partials, const FUJob& J,
                      int nt, cudaStream_t s) {
  const unsigned grid = (unsigned)(J.nfb[0] + J.nfb[1] + J.nfb[2] + J.nub);
  if (grid == 0) return cudaSuccess;
  if (P.ce32)
    k_flux_update<GLM, FLAGS, float><<<grid, nt, 0, s>>>(P, B, b.desc, b.ndesc, b.runs, state,
                                                         dt_scale, partials, J);
  else
    k_flux_update<GLM, FLAGS, double><<<grid, nt, 0, s>>>(P, B, b.desc, b.ndesc, b.runs, state,
                                                          dt_scale, partials, J);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_flux_update_overlap(const DevParams& P, const StageBuffers& B,
                                       const Batch& b, int flags, double dt_scale,
                                       StepState* state, DtPartial* partials, int* nblocks_v,
                                       cudaStream_t s) {
  const OverlapPlan& O = *B.overlap;
  // one block size for both parts: the update's (a divisor of 256, so every
  // chunk's first cell starts a block of the unchunked launch)
  const int nt = b.nt[2];
  if (nblocks_v) *nblocks_v = (int)flat_blocks(b.tot_v, nt);
  cudaError_t e = cudaSuccess;
  for (int k = 0; k <= O.n && e == cudaSuccess; ++k) {
    FUJob J;
    std::memset(&J, 0, sizeof(J));
    if (k < O.n) {
      const Chunk& C = O.c[k];
      for (int d = 0; d < P.sd; ++d) {
        J.f0[d] = C.f0[d];
        J.f1[d] = C.f1[d];
        J.nfb[d] = (int)flat_blocks(C.f1[d] - C.f0[d], nt);
      }
    }
    if (k >= 1) {
      const Chunk& C = O.c[k - 1];
      if (C.v0 % nt != 0) return cudaErrorInvalidValue;
      J.v0 = C.v0;
      J.v1 = C.v1;
      J.nub = (int)flat_blocks(C.v1 - C.v0, nt);
    }
    if (P.glm) {
      if (flags == 0) e = fu_launch<1, 0>(P, B, b, state, dt_scale, partials, J, nt, s);
      else if (flags == kStageDt) e = fu_launch<1, kStageDt>(P, B, b, state, dt_scale, partials, J, nt, s);
      else e = fu_launch<1, kStageAverage | kStageDt>(P, B, b, state, dt_scale, partials, J, nt, s);
    } else {
      if (flags == 0) e = fu_launch<0, 0>(P, B, b, state, dt_scale, partials, J, nt, s);
      else if (flags == kStageDt) e = fu_launch<0, kStageDt>(P, B, b, state, dt_scale, partials, J, nt, s);
      else e = fu_launch<0, kStageAverage | kStageDt>(P, B, b, state, dt_scale, partials, J, nt, s);
    }
    if (e == cudaSuccess && B.ev) e = cudaEventRecord(B.ev[k], s);  // profiling
  }
  return e;
}

}  // namespace mf
