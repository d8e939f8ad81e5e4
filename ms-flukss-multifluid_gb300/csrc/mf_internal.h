// mf_internal.h - declarations shared by the library's translation units
// (not part of the public C ABI).
#pragma once

#include <vector>

#include "mf_kernels.cuh"

namespace mf {

struct CtxView {
  const mf_params* p;
  const DevParams* dp;
  int ng, nc;
  double timeout;  // bounded host waits (seconds)
  double time;     // current time (PatchMHDAM::setCurrentTime)
};

// Parameters, device parameters, ghost width and component count of a context.
CtxView ctx_view(const mf_ctx* c);

// Bounded host wait for the work enqueued on s (MF_ERR_TIMEOUT after
// timeout_s seconds), and the status of a step state's error flags.
mf_status host_wait(cudaStream_t s, double timeout_s);
mf_status status_of_flags(unsigned flags);

// Host-side plan of a level of patches: fab layout (offsets in doubles from
// the level's base, every fab 256-byte aligned), the descs of both stages
// (run 0; face offsets in elements from the face arrays' bases), the face
// array sizes, and the ghost-exchange regions (LevelData::exchange: all ng
// layers before a step, 2 layers of the predictor between the RK2 stages).
// A cell that takes neutral fluid 1 (and 4) from its mirror across the
// sun's x plane (NEUTRALS_SUNBC): offsets of component 0 and component strides.
struct SunPair {
  long long to, from;
  int cs_to, cs_from;
};
cudaError_t launch_sun_copy(double* U, const SunPair* pairs, int n, int irhon, int nf,
                            cudaStream_t s);

struct LevelPlan {
  int np = 0;
  std::vector<mf_box> valid, fab;
  std::vector<long long> off;
  long long total = 0, cells = 0;
  std::vector<StageDesc> d1, d2;
  long long fsize[3] = {0, 0, 0}, bsize[3] = {0, 0, 0};
  long long fvsize = 0;  // Hancock face values per direction (doubles)
  std::vector<CopyReg> full, two;
  std::vector<SunPair> sun;  // neutral pass-through at the sun (level steps)
  // lean: every ghost cell of each patch's primitive box (valid.grow(2)) is a
  // sibling's valid cell (or its periodic image) or lies outside the domain,
  // and stage 1 runs on the valid box; the primitive state is then computed
  // on the valid cells (dp: descs whose W box is the valid box), copied into
  // the ghosts (two) and completed by the far-field fill (far).
  bool lean = false;
  std::vector<StageDesc> dp;
  std::vector<FarReg> far;
};

// MF_ERR_BAD_ARG for empty, overlapping or out-of-domain boxes, boxes with
// extent in unused dimensions, or a physical side without the far-field BC.
mf_status build_level_plan(const mf_params& p, int ng, int nc, int npatch, const mf_box* valid,
                           LevelPlan& out);

// A face of a level's face-flux arrays, for the flux registers of a
// hierarchy: offset (elements) of component 0 and the component stride in
// the layout of the RK2 stage-1 batch [0] and of the final stage [1].
struct FaceRef {
  long long off[2];
  int cs[2];
  int dir, pad;
};
// Faces whose fluxes a level step copies out (out[q * n + i], FP64): the
// flux of updateState's result, i.e. the average of both RK2 stages, the
// corrector flux of Hancock, the single stage of first order.
struct FaceGather {
  const FaceRef* refs;
  int n;
  double* out;
};
// mode 0: out = stage-1 flux; 1: out = (out + final flux) / 2; 2: out = final flux
cudaError_t launch_face_gather(int mixed, const void* const f[3], const FaceGather& g, int mode,
                               int nc, cudaStream_t s);

// What the coarse-fine coupling needs of a level.
struct LevelView {
  mf_ctx* ctx;
  const mf_params* p;
  int np, nc, ng;
  const std::vector<mf_box>* valid;
  const std::vector<mf_box>* fab;
  const std::vector<long long>* off;
  const std::vector<StageDesc>* d1;  // RK2 stage-1 descs (face offsets)
  const std::vector<StageDesc>* d2;  // final-stage descs
  double* U;
  cudaStream_t s;
};
LevelView level_view(mf_level* L);
// Replace the face gathers a level step runs (drops the cached step graphs).
void level_set_gathers(mf_level* L, const std::vector<FaceGather>& g);
// Start time of the level's next synchronous step (host mirror only; the
// synchronous step uploads it with the step's dt).
void level_set_time_host(mf_level* L, double time);

}  // namespace mf
