// mf_flux.cu - face-flux kernel with the fast physics (contraction allowed,
// reciprocals reused): FP32 for the mixed-precision path, FP64 for the fast
// FP64 path.
#include <algorithm>

#define MF_PHYS fast
#include "mf_riemann.cuh"
#include "mf_flux_kernel.cuh"

namespace mf {

template <typename R, int WF>
static void flux_dirs(const DevParams& P, int dir, const double* w, const float* wf, R* F,
                      R* Bn, const Batch& b, const StepState* state, unsigned gf, int nt,
                      int first, int end, cudaStream_t s) {
  if (dir == 0)
    k_flux<R, 0, WF><<<gf, nt, 0, s>>>(P, w, wf, F, Bn, b.desc, b.ndesc, first, end, b.runs,
                                       state);
  if (dir == 1)
    k_flux<R, 1, WF><<<gf, nt, 0, s>>>(P, w, wf, F, Bn, b.desc, b.ndesc, first, end, b.runs,
                                       state);
  if (dir == 2)
    k_flux<R, 2, WF><<<gf, nt, 0, s>>>(P, w, wf, F, Bn, b.desc, b.ndesc, first, end, b.runs,
                                       state);
}

template <typename R>
cudaError_t launch_flux_fast(const DevParams& P, int dir, const double* w, void* f, void* bn,
                             const Batch& b, const StepState* state, cudaStream_t s,
                             const float* wf, int first, int end) {
  if (end < 0) end = b.tot_f[dir];
  if (end - first <= 0) return cudaSuccess;
  const int nt = b.nt[1];
  const unsigned gf = flat_blocks(end - first, nt);
  R* F = (R*)f;
  R* Bn = (R*)bn;
  if constexpr (sizeof(R) == 4) {
    if (wf) {
      flux_dirs<R, 1>(P, dir, w, wf, F, Bn, b, state, gf, nt, first, end, s);
      return cudaGetLastError();
    }
  }
  flux_dirs<R, 0>(P, dir, w, nullptr, F, Bn, b, state, gf, nt, first, end, s);
  return cudaGetLastError();
}

cudaError_t launch_flux_lines_fast(const DevParams& P, int dir, const double* w, void* f,
                                   void* bn, const Batch& b, const LinePlan& lp,
                                   const StepState* state, cudaStream_t s) {
  return launch_lflux_t<double>(P, dir, w, f, bn, b, lp, state, s);
}

cudaError_t lines_prepare_exact();

cudaError_t lines_prepare() {
  static bool done[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
  e = lflux_allow_t<double>();
  if (e == cudaSuccess) e = lines_prepare_exact();
  if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
  return e;
}

bool make_lines(const StageDesc* hd, int n, int sd, std::vector<LineWork> out[3],
                int maxcells[3]) {
  for (int d = 0; d < 3; ++d) {
    out[d].clear();
    maxcells[d] = 0;
  }
  for (int d = 0; d < sd; ++d) {
    const int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
    for (int i = 0; i < n; ++i) {
      const StageDesc& D = hd[i];
      const int nd = D.vn[d];
      const int lines = D.vn[t1] * D.vn[t2];
      if (nd <= 0 || lines <= 0) continue;
      if (nd + 2 > kLineMaxCells) return false;
      const int per = std::max(1, kLineThreads / (nd + 1));
      for (int l0 = 0; l0 < lines; l0 += per) {
        LineWork Wk;
        Wk.desc = i;
        Wk.line0 = l0;
        Wk.nlines = std::min(per, lines - l0);
        maxcells[d] = std::max(maxcells[d], Wk.nlines * (nd + 2));
        out[d].push_back(Wk);
      }
    }
  }
  return true;
}

template <typename R>
cudaError_t launch_face_flux_fast(const DevParams& P, int dir, const double* wl,
                                  const double* wr, double* f, int n, double ch, cudaStream_t s) {
  return launch_face_flux_t<R>(P, dir, wl, wr, f, n, ch, s);
}

template <typename R>
cudaError_t launch_hflux_fast(const DevParams& P, int dir, const double* w, const double* fv,
                              void* f, void* bn, const Batch& b, const StepState* state,
                              cudaStream_t s) {
  return launch_hflux_t<R>(P, dir, w, fv, f, bn, b, state, s);
}

template cudaError_t launch_hflux_fast<double>(const DevParams&, int, const double*,
                                               const double*, void*, void*, const Batch&,
                                               const StepState*, cudaStream_t);
template cudaError_t launch_hflux_fast<float>(const DevParams&, int, const double*,
                                              const double*, void*, void*, const Batch&,
                                              const StepState*, cudaStream_t);

template cudaError_t launch_face_flux_fast<double>(const DevParams&, int, const double*,
                                                   const double*, double*, int, double,
                                                   cudaStream_t);
template cudaError_t launch_face_flux_fast<float>(const DevParams&, int, const double*,
                                                  const double*, double*, int, double,
                                                  cudaStream_t);

template cudaError_t launch_flux_fast<double>(const DevParams&, int, const double*, void*, void*,
                                              const Batch&, const StepState*, cudaStream_t,
                                              const float*, int, int);
template cudaError_t launch_flux_fast<float>(const DevParams&, int, const double*, void*, void*,
                                             const Batch&, const StepState*, cudaStream_t,
                                             const float*, int, int);

}  // namespace mf
