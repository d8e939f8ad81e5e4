// mf_kernels.cuh - launch interface of the stage kernels.
//
// One explicit stage of PatchMHDAM::EulerStep (src/PatchMHDAM.cpp:495-709) is
// three kinds of kernel over every patch of a batch:
//   k_prim    (mf_prim_exact.cu) conserved -> primitive on valueBox.grow(2)
//   k_flux<D> (mf_flux.cu)       face states + Riemann fluxes in direction D
//   k_update  (mf_update.cu)     flux divergence, sources, positivity, RK2
//                                averaging and the per-cell dt
// A launch is flat over the concatenated items (cells or faces) of all
// patches of the batch, so patches of uneven sizes share blocks and no lane
// idles on padding; each thread finds its patch by a binary search over the
// ascending start offsets StageDesc::g0.
#pragma once

#include <cfloat>
#include <climits>
#include <cstring>
#include <vector>

#include "mf_device.cuh"

namespace mf {

constexpr int kBlock = 128;

enum RegionKind : int { kRegW = 0, kRegF = 1, kRegV = 4, kRegS = 5 };

// Patch whose items contain flattened index g (0 <= g < launch total): the
// largest d with descs[d].g0[kind] <= g.  Patches with no items share their
// start with the next one and are skipped by taking the largest such d.
__device__ __forceinline__ int find_desc(const StageDesc* __restrict__ descs, int ndesc, int kind,
                                         int g) {
  int lo = 0, hi = ndesc - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&descs[mid].g0[kind]) <= g)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

// A flattened launch over a batch of patches: the device descs, the total
// item counts of each region kind, and the threads per block of the prim,
// flux and update/dt kernels (multiples of 32, at most kMaxBlock).
struct Batch {
  const StageDesc* desc;
  int ndesc;
  int tot_w, tot_f[3], tot_v, tot_s;
  int nt[3];
  const RunParams* runs;  // device array, nruns entries (StageDesc::run indexes it)
  int nruns;
};

constexpr int kMaxBlock = 256;

// Fill the g0 offsets of n host descs and the totals of a Batch.  The descs
// of one run are consecutive and runs ascend (StageDesc::run); each run's
// valueBox cells start on a multiple of kRunAlign, and hruns (nruns host
// entries, nullable for a single run) receive their desc and cell ranges.
// Returns false when a total does not fit a 32-bit index.
inline bool batch_offsets(StageDesc* hd, int n, int sd, Batch& b, RunParams* hruns = nullptr,
                          int nruns = 1) {
  long long t[6] = {0, 0, 0, 0, 0, 0};
  int cur = -1;
  for (int i = 0; i < n; ++i) {
    StageDesc& D = hd[i];
    if (D.run != cur) {
      if (D.run < cur || D.run >= nruns) return false;
      if (hruns && cur >= 0) hruns[cur].v1 = (int)t[kRegV];
      t[kRegV] = (t[kRegV] + kRunAlign - 1) / kRunAlign * kRunAlign;
      for (int r = cur + 1; r <= D.run && hruns; ++r) {
        hruns[r].d0 = i;
        hruns[r].nd = 0;
        hruns[r].v0 = hruns[r].v1 = (int)t[kRegV];
      }
      cur = D.run;
    }
    if (hruns) hruns[cur].nd += 1;
    long long cnt[6];
    cnt[kRegW] = (long long)D.wn[0] * D.wn[1] * D.wn[2];
    cnt[kRegS] = (long long)D.sn[0] * D.sn[1] * D.sn[2];
    for (int d = 0; d < 3; ++d) {
      long long f = 0;
      if (d < sd) {
        long long e[3] = {D.vn[0], D.vn[1], D.vn[2]};
        e[d] += 1;
        f = e[0] * e[1] * e[2];
      }
      cnt[kRegF + d] = f;
    }
    cnt[kRegV] = (long long)D.vn[0] * D.vn[1] * D.vn[2];
    for (int k = 0; k < 6; ++k) {
      if (t[k] > INT_MAX - 4096) return false;
      D.g0[k] = (int)t[k];
      t[k] += cnt[k];
    }
  }
  for (int k = 0; k < 6; ++k)
    if (t[k] > INT_MAX - 4096) return false;
  if (hruns && cur >= 0) hruns[cur].v1 = (int)t[kRegV];
  for (int r = cur + 1; r < nruns && hruns; ++r) {
    hruns[r].d0 = n;
    hruns[r].nd = 0;
    hruns[r].v0 = hruns[r].v1 = (int)t[kRegV];
  }
  b.ndesc = n;
  b.tot_w = (int)t[kRegW];
  for (int d = 0; d < 3; ++d) b.tot_f[d] = (int)t[kRegF + d];
  b.tot_v = (int)t[kRegV];
  b.tot_s = (int)t[kRegS];
  b.nruns = nruns;
  return true;
}

// The per-run values of a single run with parameters P.
inline RunParams run_params_of(const DevParams& P) {
  RunParams r;
  std::memset(&r, 0, sizeof(r));
  r.dx = P.dx;
  r.invdx = P.invdx;
  for (int d = 0; d < 3; ++d) {
    r.dlo[d] = P.dlo[d];
    r.dhi[d] = P.dhi[d];
  }
  for (int q = 0; q < 8; ++q) r.bc_plasma[q] = P.bc_plasma[q];
  for (int q = 0; q < 5; ++q) r.bc_n1[q] = P.bc_n1[q];
  return r;
}

inline void batch_default_threads(Batch& b) { b.nt[0] = b.nt[1] = b.nt[2] = kBlock; }

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

// A box of far-field ghost cells of a patch's primitive-state box (cells
// outside a non-periodic domain side): filled after the primitive variables
// of the valid cells and the ghost exchange, as the primitive kernel fills
// them (HELIOGS) when it runs over the whole box.
struct FarReg {
  long long off;  // fab offset (doubles) in U / W / Wf
  int fn[3];      // fab extents
  int flo[3];     // fab lo (index space)
  int lo[3];      // region lo (index space)
  int ext[3];     // region extents
  int run;        // run of the patch (RunParams)
  int pad;
};

// Primitive variables on the valid cells only (levels whose primitive-box
// ghosts are all sibling cells or outside the domain): the ghosts come from a
// copy of the siblings' primitive state and the far-field fill, which gives
// the same values as computing them from exchanged conserved ghosts.
struct LeanPrim {
  const Batch* prim;         // descs with the W box = the valid box
  const CopyReg* regs;       // sibling copies into the 2 ghost layers
  int nregs;
  const FarReg* far;         // far-field ghost boxes
  int nfar;
  int exchange_w;            // copy the FP64 W (else only the FP32 copy)
};

struct FusedTile;
// The tiles of one stage's batch for the fused flux + update kernel.
struct FusedPlan {
  const FusedTile* tiles;  // device work list
  int ntiles;
  int tile[3];             // tile shape (cells)
};

struct OverlapPlan;

// Face fluxes by lines (FP64 paths): each block takes whole lines of faces
// along one direction of one patch and shares the cells' face values.
constexpr int kLineThreads = 128;
constexpr int kLineMaxCells = 256;  // cells of one block's lines (2 beyond each line's faces)
struct LineWork {
  int desc;    // desc index in the batch
  int line0;   // first line: index over the transverse cells, the lower dimension fastest
  int nlines;  // lines of the block
};
struct LinePlan {
  const LineWork* w[3];  // device work lists per direction
  int n[3];              // blocks per direction
  int maxcells[3];       // most cells of one block per direction
};
inline size_t line_smem_bytes(int nc, int cells) {
  return sizeof(double) * 2 * (size_t)nc * (size_t)cells;
}
// Work lists of a batch's descs (host) per direction: lines of up to
// kLineThreads faces per block; false when a patch is too long along a
// direction for one block's shared memory (kLineMaxCells).
bool make_lines(const StageDesc* hd, int n, int sd, std::vector<LineWork> out[3],
                int maxcells[3]);

struct StageBuffers {
  const double* uin;   // state the stage starts from
  double* uout;        // state the stage writes (valueBox cells only)
  const double* uold;  // state before the time step (RK2 averaging)
  double* w;           // primitive scratch, same layout as uin
  // primitive state at the stage start when it is not w (the Hancock
  // corrector: w holds W(t+dt/2), wls W(t)): the velocity of the tracking
  // surfaces' update and their stage-start values (Uold); null = w
  const double* wls;
  // mixed precision: an FP32 copy of w (same layout) that the FP32 flux
  // kernels read, written by the prim kernel; null = convert w in the flux kernel
  float* wf;
  void* f[3];          // face fluxes (double or float), per direction
  void* bn[3];         // face-normal B (double or float), per direction
  double* divb;        // optional divB output (single patch: fab on the valid box)
  int divb_lo[3], divb_n[3];
  cudaEvent_t* ev;     // optional: an event recorded after each launch (profiling)
  const LeanPrim* lean;  // optional: primitive state on valid cells + ghost copies
  const FusedPlan* fused;  // optional (mixed precision): fluxes + update in one kernel
  const OverlapPlan* overlap;  // optional (mixed precision): chunked, overlapped flux + update
  const LinePlan* lines;       // optional (FP64 paths): face fluxes by lines
};

enum StageFlags : int { kStageAverage = 1, kStageDt = 2 };

// The flux and update launches of a mixed-precision stage cut into chunks of
// consecutive patches: launch k computes the FP32 fluxes of chunk k and the
// FP64-bound update of chunk k - 1 in one grid of alternating blocks, so the
// two share the SMs (mf_fu.cu).  A chunk's cells start on a multiple of 256.
struct Chunk {
  int v0, v1;        // cells [v0, v1) of the batch's flat cell index
  int f0[3], f1[3];  // faces [f0, f1) per direction
};
struct OverlapPlan {
  const Chunk* c;  // host array
  int n;           // chunks (>= 2): n + 1 launches per stage
};
// Chunks of a batch (host descs hd, n of them): about equal cell counts,
// each starting at a patch whose first cell is a multiple of 256; fewer than
// nchunks where the patches do not allow more.
std::vector<Chunk> make_chunks(const StageDesc* hd, int n, const Batch& b, int nchunks);
// the flux and update launches of a mixed-precision stage in B.overlap's chunks (mf_fu.cu)
cudaError_t launch_flux_update_overlap(const DevParams& P, const StageBuffers& B,
                                       const Batch& b, int flags, double dt_scale,
                                       StepState* state, DtPartial* partials, int* nblocks_v,
                                       cudaStream_t s);

// wf (nullable): also the FP32 copy of w (round to nearest, as the FP32 flux
// kernels would convert each value)
cudaError_t launch_prim(const DevParams& P, const double* uin, double* w, const Batch& b,
                        cudaStream_t s, float* wf = nullptr);

// FP64 parity path (reference evaluation order, no contraction)
cudaError_t launch_flux_exact(const DevParams& P, int dir, const double* w, void* f, void* bn,
                              const Batch& b, const StepState* state, cudaStream_t s);
cudaError_t launch_update_exact(const DevParams& P, const StageBuffers& B, const Batch& b,
                                int flags, double dt_scale, StepState* state,
                                DtPartial* partials, int* nblocks_v, cudaStream_t s);
// fast physics: R = float (mixed precision) or double (fast FP64)
// wf (R = float only, nullable): the FP32 copy of w the prim kernel wrote
// face fluxes by lines (k_lflux), FP64 paths; *_prepare once per device
// before the first launch (outside any capture)
cudaError_t launch_flux_lines_exact(const DevParams& P, int dir, const double* w, void* f,
                                    void* bn, const Batch& b, const LinePlan& lp,
                                    const StepState* state, cudaStream_t s);
cudaError_t launch_flux_lines_fast(const DevParams& P, int dir, const double* w, void* f,
                                   void* bn, const Batch& b, const LinePlan& lp,
                                   const StepState* state, cudaStream_t s);
cudaError_t lines_prepare();
// [first, end): a range of the batch's flat face / cell index (end < 0: to
// the batch's total); an update range starts on a multiple of the block size
template <typename R>
cudaError_t launch_flux_fast(const DevParams& P, int dir, const double* w, void* f, void* bn,
                             const Batch& b, const StepState* state, cudaStream_t s,
                             const float* wf = nullptr, int first = 0, int end = -1);
template <typename R>
cudaError_t launch_update_fast(const DevParams& P, const StageBuffers& B, const Batch& b,
                               int flags, double dt_scale, StepState* state,
                               DtPartial* partials, int* nblocks_v, cudaStream_t s,
                               int first = 0, int end = -1);

// Riemann fluxes of n given face-state pairs (primitive, nc values each) in
// the exact or the fast physics (R = float: mixed precision).
cudaError_t launch_face_flux_exact(const DevParams& P, int dir, const double* wl,
                                   const double* wr, double* f, int n, double ch, cudaStream_t s);
template <typename R>
cudaError_t launch_face_flux_fast(const DevParams& P, int dir, const double* wl,
                                  const double* wr, double* f, int n, double ch, cudaStream_t s);

// Bytes of one face-flux value for a precision mode (MF_PREC_*).
inline size_t flux_bytes(int precision) { return precision == MF_PREC_MIXED ? 4 : 8; }

// Blocks of a flattened launch of n items with nt threads per block.
inline unsigned flat_blocks(long long n, int nt) {
  return (unsigned)(n > 0 ? (n + nt - 1) / nt : 1);
}

// Number of dt partials (blocks of the update or dt kernel) for b.
inline int dt_partials(const Batch& b) { return (int)flat_blocks(b.tot_v, b.nt[2]); }

// Enqueue one stage (prim, fluxes in every direction, update) for the
// patches of b.  precision: MF_PREC_FP64 (parity), MF_PREC_FP64_FAST or
// MF_PREC_MIXED.
cudaError_t launch_stage(const DevParams& P, int precision, const StageBuffers& B,
                         const Batch& b, int flags, double dt_scale, StepState* state,
                         DtPartial* partials, int* nblocks_v, cudaStream_t s);

// dx / max wave speed over each desc's valueBox into per-block partials.
cudaError_t launch_dt(const DevParams& P, const double* u, const Batch& b, DtPartial* partials,
                      int* nblocks, cudaStream_t s);

// Reduce the dt partials of the last stage per run (one block per run, over
// the run's blocks of a launch with nt threads per block; nparts > 0: a
// single run whose partials are [0, nparts), e.g. one per fused tile);
// advance = 1 also writes each run's next dt (cfl * minimum) and GLM speeds
// into state[run].
cudaError_t launch_finalize(const DevParams& P, const DtPartial* partials, const Batch& b,
                            int nt, StepState* state, int advance, cudaStream_t s,
                            int nparts = 0);

cudaError_t launch_exchange(double* u, const CopyReg* regs, int nreg, int nc, cudaStream_t s);
cudaError_t launch_exchange_f(float* u, const CopyReg* regs, int nreg, int nc, cudaStream_t s);
// Far-field ghosts of the primitive state (HELIOGS, as the primitive kernel
// fills them) on the boxes far (W and, when set, its FP32 copy wf).
cudaError_t launch_farfield(const DevParams& P, const double* u, double* w, float* wf,
                            const FarReg* far, int nfar, const RunParams* runs, int have_w,
                            cudaStream_t s);
// Kernel launches of the primitive part of a stage (1 without lean).
inline int prim_launches(const LeanPrim* lp, int mixed) {
  if (!lp) return 1;
  int n = 1;
  if (lp->nregs) n += (lp->exchange_w ? 1 : 0) + (mixed ? 1 : 0);
  if (lp->nfar) n += 1;
  return n;
}

// The valid cells of the descs of b (valueBox = valid box, one run) between
// the fab layout u and the packed layout (nc x the desc's first valid cell,
// component-major): to_fab = 1 scatters packed into u, 0 gathers.
cudaError_t launch_pack(double* u, double* packed, const Batch& b, int nc, int to_fab,
                        cudaStream_t s);

// Fout[d] = average of the two stages' face fluxes (or the single stage's)
// on the faces of the valid box.
cudaError_t launch_flux_out(int mixed, int sd, int nc, const void* const f2[3],
                            const int f2lo[3][3], const int f2n[3][3], const void* const f1[3],
                            const int f1lo[3][3], const int f1n[3][3], double* const fout[3],
                            const int olo[3][3], const int on[3][3], cudaStream_t s);

// Constrained transport (mf_ct_exact.cu).  Internal edge field: 3 components
// laid out like U on each patch's fab, at 3 x the patch's cell offset.
// efield: the edge field of the stage's fluxes f on the nodes of each
// valueBox (W: stage-start primitive state, for the 2D Gardiner-Stone
// methods); with e1 / eavg set also eavg = (e + e1) / 2 there.
cudaError_t launch_efield(const DevParams& P, int mixed, const void* const f[3],
                          const double* w, double* e, const double* e1, double* eavg,
                          const Batch& b, cudaStream_t s);
// recalculateB on each valueBox from bold (components 5..7, laid out like U)
// and the edge field e with time step state[run].dt * dt_scale.  stage = 1:
// a stage's recalculation, then the inner-sphere reset and the positivity fix
// (which the update kernel leaves to it under constrained transport) and,
// with u0 / u1 set, AVERAGESTATE u += (u0 - u1) / 2; stage = 0: the level's
// recalculation after the step alone.
cudaError_t launch_recalc_b(const DevParams& P, double* u, const double* bold, const double* e,
                            const double* u0, const double* u1, const StepState* state,
                            double dt_scale, int stage, const Batch& b, cudaStream_t s);

// recalculateMagneticField on caller fabs: U (in place) from Uold's field and
// the EdgeBox fabs E (3 in 3D, 1 nodal in 2D) on box.
cudaError_t launch_recalc_ext(int sd, double dx, mf_fab* U, const mf_fab* Uold, const mf_fab* E,
                              double dt, const mf_box& box, cudaStream_t s);
// The internal edge field of a single-patch call on the fab box `fab` into
// the caller's EdgeBox fabs, on the edges of the valid box.
cudaError_t launch_edges_out(int sd, const double* e, const mf_box& fab, const mf_box& valid,
                             mf_fab* out, cudaStream_t s);

// Number of kernel launches enqueued by launch_stage for sd dimensions
// (plus prim_launches - 1 with a lean primitive part).
inline int stage_launches(int sd) { return 2 + sd; }

// Fused flux + update stage kernel of the mixed-precision level step
// (mf_fused.cu): one block per tile of a desc's valueBox.
struct FusedTile {
  int desc;   // desc index in the batch
  int lo[3];  // first cell (index space)
  int n[3];   // extents (at most the tile shape)
};
// the options the fused kernel covers, and the tile shapes it accepts
bool fused_supported(const DevParams& P, int precision, int time_approximation);
bool fused_tile_ok(const DevParams& P, const int tile[3]);
size_t fused_smem_bytes(const DevParams& P, const int tile[3]);
// once per device before the first launch (sets the kernels' shared-memory limit)
cudaError_t fused_prepare();
// fluxes + update of the tiles; the dt partials are per tile (one per block)
cudaError_t launch_fused(const DevParams& P, const StageBuffers& B, const Batch& b,
                         const FusedTile* tiles, int ntiles, const int tile[3], int flags,
                         double dt_scale, StepState* state, DtPartial* partials, cudaStream_t s);

// Hancock step (predictorHancock + correctorHancock) of the patches of a
// (predictor descs: valueBox = box.grow(1) & domain, W box, slope box, face
// values) and c (corrector descs: valueBox = box & domain, with the same
// slope boxes and face-value offsets).  fv[d]: face values per direction;
// w2: the predicted primitive state W(t + dt/2), laid out like W.
struct HancockBuffers {
  double* fv[3];
  double* w2;
};
// corrector_flags: the flags of the corrector's update (kStageDt, or 0 when
// the dt follows later, as with constrained transport).
cudaError_t launch_hancock(const DevParams& P, int precision, const StageBuffers& B,
                           const HancockBuffers& H, const Batch& a, const Batch& c,
                           StepState* state, DtPartial* partials, int* nblocks_v,
                           cudaStream_t s, int corrector_flags = kStageDt);
inline int hancock_launches(int sd) { return 5 + sd; }

// Corrector fluxes of the Hancock step from the shifted face values.
cudaError_t launch_hflux_exact(const DevParams& P, int dir, const double* w, const double* fv,
                               void* f, void* bn, const Batch& b, const StepState* state,
                               cudaStream_t s);
template <typename R>
cudaError_t launch_hflux_fast(const DevParams& P, int dir, const double* w, const double* fv,
                              void* f, void* bn, const Batch& b, const StepState* state,
                              cudaStream_t s);

}  // namespace mf
