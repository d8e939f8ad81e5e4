// mf_flux_exact.cu - face-flux kernel of the FP64 parity path: the reference's
// evaluation order, built with -fmad=false.
#define MF_PHYS exact
#include "mf_riemann_exact.cuh"
#include "mf_flux_kernel.cuh"

namespace mf {

cudaError_t launch_flux_exact(const DevParams& P, int dir, const double* w, void* f, void* bn,
                              const StageDesc* d_desc, int ndesc, long long max_f,
                              const StepState* state, cudaStream_t s) {
  const dim3 gf((unsigned)((max_f + kBlock - 1) / kBlock), (unsigned)ndesc);
  double* F = (double*)f;
  double* Bn = (double*)bn;
  if (dir == 0) k_flux<double, 0><<<gf, kBlock, 0, s>>>(P, w, F, Bn, d_desc, state);
  if (dir == 1) k_flux<double, 1><<<gf, kBlock, 0, s>>>(P, w, F, Bn, d_desc, state);
  if (dir == 2) k_flux<double, 2><<<gf, kBlock, 0, s>>>(P, w, F, Bn, d_desc, state);
  return cudaGetLastError();
}

}  // namespace mf
