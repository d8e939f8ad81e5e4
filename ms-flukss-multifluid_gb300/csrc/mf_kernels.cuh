// mf_kernels.cuh - launch interface of the stage kernels (see mf_kernels.cu).
#pragma once

#include "mf_device.cuh"

namespace mf {

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
};

enum StageFlags : int { kStageAverage = 1, kStageDt = 2 };

// Enqueue one stage (prim, fluxes in every direction, update) for ndesc
// patches.  max_w / max_f[d] / max_v: largest region sizes over the descs.
cudaError_t launch_stage_fp64(const DevParams& P, const StageBuffers& B, const StageDesc* d_desc,
                              int ndesc, long long max_w, const long long max_f[3],
                              long long max_v, int flags, double dt_scale, StepState* state,
                              DtPartial* partials, int* nblocks_v, cudaStream_t s);
cudaError_t launch_stage_mixed(const DevParams& P, const StageBuffers& B,
                               const StageDesc* d_desc, int ndesc, long long max_w,
                               const long long max_f[3], long long max_v, int flags,
                               double dt_scale, StepState* state, DtPartial* partials,
                               int* nblocks_v, cudaStream_t s);

inline cudaError_t launch_stage(const DevParams& P, int mixed, const StageBuffers& B,
                                const StageDesc* d_desc, int ndesc, long long max_w,
                                const long long max_f[3], long long max_v, int flags,
                                double dt_scale, StepState* state, DtPartial* partials,
                                int* nblocks_v, cudaStream_t s) {
  if (mixed)
    return launch_stage_mixed(P, B, d_desc, ndesc, max_w, max_f, max_v, flags, dt_scale, state,
                              partials, nblocks_v, s);
  return launch_stage_fp64(P, B, d_desc, ndesc, max_w, max_f, max_v, flags, dt_scale, state,
                           partials, nblocks_v, s);
}

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
