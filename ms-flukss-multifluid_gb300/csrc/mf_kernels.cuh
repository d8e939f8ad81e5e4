// mf_kernels.cuh - launch interface of the stage kernels.
//
// One explicit stage of PatchMHDAM::EulerStep (src/PatchMHDAM.cpp:495-709) is
// three kinds of kernel over every patch of a batch (blockIdx.y = patch):
//   k_prim    (mf_prim_exact.cu) conserved -> primitive on valueBox.grow(2)
//   k_flux<D> (mf_flux.cu)       face states + Riemann fluxes in direction D
//   k_update  (mf_update.cu)     flux divergence, sources, positivity, RK2
//                                averaging and the per-cell dt
#pragma once

#include <cfloat>
#include <climits>

#include "mf_device.cuh"

namespace mf {

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

// One block copies one box of cells (all components) from a source fab to a
// destination fab inside the same buffer: a ghost region of LevelData::exchange.
struct CopyReg {
  long long src_off, dst_off;  // fab offsets (doubles)
  int sfn[3], dfn[3];          // fab extents
  int s0[3], d0[3];            // region start, fab-local coordinates
  int ext[3];                  // region extents
};

struct StageBuffers {
  const double* uin;   // state the stage starts from
  double* uout;        // state the stage writes (valueBox cells only)
  const double* uold;  // state before the time step (RK2 averaging)
  double* w;           // primitive scratch, same layout as uin
  void* f[3];          // face fluxes (double or float), per direction
  void* bn[3];         // face-normal B (double or float), per direction
  double* divb;        // optional divB output (single patch: fab on the valid box)
  int divb_lo[3], divb_n[3];
  cudaEvent_t* ev;     // optional: an event recorded after each launch (profiling)
};

enum StageFlags : int { kStageAverage = 1, kStageDt = 2 };

cudaError_t launch_prim(const DevParams& P, const double* uin, double* w, const StageDesc* d_desc,
                        int ndesc, long long max_w, cudaStream_t s);

// FP64 parity path (reference evaluation order, no contraction)
cudaError_t launch_flux_exact(const DevParams& P, int dir, const double* w, void* f, void* bn,
                              const StageDesc* d_desc, int ndesc, long long max_f,
                              const StepState* state, cudaStream_t s);
cudaError_t launch_update_exact(const DevParams& P, const StageBuffers& B,
                                const StageDesc* d_desc, int ndesc, long long max_v, int flags,
                                double dt_scale, StepState* state, DtPartial* partials,
                                int* nblocks_v, cudaStream_t s);
// fast physics: R = float (mixed precision) or double (fast FP64)
template <typename R>
cudaError_t launch_flux_fast(const DevParams& P, int dir, const double* w, void* f, void* bn,
                             const StageDesc* d_desc, int ndesc, long long max_f,
                             const StepState* state, cudaStream_t s);
template <typename R>
cudaError_t launch_update_fast(const DevParams& P, const StageBuffers& B, const StageDesc* d_desc,
                               int ndesc, long long max_v, int flags, double dt_scale,
                               StepState* state, DtPartial* partials, int* nblocks_v,
                               cudaStream_t s);

// Bytes of one face-flux value for a precision mode (MF_PREC_*).
inline size_t flux_bytes(int precision) { return precision == MF_PREC_MIXED ? 4 : 8; }

// Enqueue one stage (prim, fluxes in every direction, update) for ndesc
// patches.  max_w / max_f[d] / max_v: largest region sizes over the descs.
// precision: MF_PREC_FP64 (parity), MF_PREC_FP64_FAST or MF_PREC_MIXED.
cudaError_t launch_stage(const DevParams& P, int precision, const StageBuffers& B,
                         const StageDesc* d_desc, int ndesc, long long max_w,
                         const long long max_f[3], long long max_v, int flags,
                         double dt_scale, StepState* state, DtPartial* partials,
                         int* nblocks_v, cudaStream_t s);

// dx / max wave speed over each desc's valueBox into per-block partials.
cudaError_t launch_dt(const DevParams& P, const double* u, const StageDesc* d_desc, int ndesc,
                      long long max_v, DtPartial* partials, int* nblocks, cudaStream_t s);

// Reduce the dt partials of the last stage; advance = 1 also writes the next
// dt (cfl * minimum) and the GLM speeds into *state.
cudaError_t launch_finalize(const DevParams& P, const DtPartial* partials, int npart,
                            StepState* state, int advance, cudaStream_t s);

cudaError_t launch_exchange(double* u, const CopyReg* regs, int nreg, int nc, cudaStream_t s);

// Fout[d] = average of the two stages' face fluxes (or the single stage's)
// on the faces of the valid box.
cudaError_t launch_flux_out(int mixed, int sd, int nc, const void* const f2[3],
                            const int f2lo[3][3], const int f2n[3][3], const void* const f1[3],
                            const int f1lo[3][3], const int f1n[3][3], double* const fout[3],
                            const int olo[3][3], const int on[3][3], cudaStream_t s);

// Number of kernel launches enqueued by launch_stage for sd dimensions.
inline int stage_launches(int sd) { return 2 + sd; }

}  // namespace mf
