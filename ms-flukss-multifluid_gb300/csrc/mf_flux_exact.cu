// mf_flux_exact.cu - face-flux kernel of the FP64 parity path: the reference's
// evaluation order, built with -fmad=false.
#define MF_PHYS exact
#include "mf_riemann_exact.cuh"
#include "mf_flux_kernel.cuh"

namespace mf {

cudaError_t launch_flux_exact(const DevParams& P, int dir, const double* w, void* f, void* bn,
                              const Batch& b, const StepState* state, cudaStream_t s) {
  const int tot = b.tot_f[dir];
  if (tot <= 0) return cudaSuccess;
  const int nt = b.nt[1];
  const unsigned gf = flat_blocks(tot, nt);
  double* F = (double*)f;
  double* Bn = (double*)bn;
  if (dir == 0)
    k_flux<double, 0, 0><<<gf, nt, 0, s>>>(P, w, nullptr, F, Bn, b.desc, b.ndesc, 0, tot, b.runs,
                                            state);
  if (dir == 1)
    k_flux<double, 1, 0><<<gf, nt, 0, s>>>(P, w, nullptr, F, Bn, b.desc, b.ndesc, 0, tot, b.runs,
                                            state);
  if (dir == 2)
    k_flux<double, 2, 0><<<gf, nt, 0, s>>>(P, w, nullptr, F, Bn, b.desc, b.ndesc, 0, tot, b.runs,
                                            state);
  return cudaGetLastError();
}

cudaError_t launch_flux_lines_exact(const DevParams& P, int dir, const double* w, void* f,
                                    void* bn, const Batch& b, const LinePlan& lp,
                                    const StepState* state, cudaStream_t s) {
  return launch_lflux_t<double>(P, dir, w, f, bn, b, lp, state, s);
}

cudaError_t lines_prepare_exact() { return lflux_allow_t<double>(); }

cudaError_t launch_face_flux_exact(const DevParams& P, int dir, const double* wl,
                                   const double* wr, double* f, int n, double ch,
                                   cudaStream_t s) {
  return launch_face_flux_t<double>(P, dir, wl, wr, f, n, ch, s);
}

cudaError_t launch_hflux_exact(const DevParams& P, int dir, const double* w, const double* fv,
                               void* f, void* bn, const Batch& b, const StepState* state,
                               cudaStream_t s) {
  return launch_hflux_t<double>(P, dir, w, fv, f, bn, b, state, s);
}

}  // namespace mf
