// mf_server.cu - independent runs stepped together in shared launches.
//
// A serving loop keeps many independent simulations (runs) resident on the
// GPU and advances all of them in the same kernel launches.  Every run is a
// level of patches covering its own domain; the runs share the physics of
// one context (equations, solvers, limiters, sources) and differ in grid
// size, grid spacing and far-field state (RunParams).  A step of the server is
// the level step of mf_capi.cu (ghost exchange, two RK2 stages, dt reduction)
// over the concatenated patches of every admitted run: each StageDesc names
// its run, each run keeps its own StepState (dt, GLM speeds, results), and the
// dt reduction is segmented by run, so a run's numbers do not depend on which
// other runs share its launches.
//
// Memory: one device arena per kind of array (state, predictor and
// primitive state share cell offsets; face fluxes and face-normal B have
// their own), sized once from an HBM budget.  A run is admitted when its
// footprint fits (first-fit over the free ranges); its ranges are returned
// when it retires.  The batch (descs, run table, exchange regions) is rebuilt
// and the step graph re-captured when the set of runs changes.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "mf_internal.h"
#include "mf_kernels.cuh"

using mf::CopyReg;
using mf::DtPartial;
using mf::RunParams;
using mf::StageBuffers;
using mf::StageDesc;
using mf::StepState;

namespace {

#define SV_CUDA(x)                                                 \
  do {                                                             \
    cudaError_t e_ = (x);                                          \
    if (e_ != cudaSuccess)                                         \
      return e_ == cudaErrorMemoryAllocation ? MF_ERR_OOM : MF_ERR_CUDA; \
  } while (0)

struct DevMem {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, n > 0 ? n : 16);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
};

struct HostMem {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t n) {
    if (n <= bytes && p) return cudaSuccess;
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMallocHost(&p, n > 0 ? n : 16);
    if (e == cudaSuccess) bytes = n;
    return e;
  }
  void release() {
    if (p) cudaFreeHost(p);
    p = nullptr;
    bytes = 0;
  }
};

// First-fit allocator over [0, cap) (units of one element of the arena),
// free ranges keyed by offset and merged on release.
struct Arena {
  long long cap = 0;
  std::map<long long, long long> free_;
  void init(long long c) {
    cap = c;
    free_.clear();
    if (c > 0) free_[0] = c;
  }
  bool alloc(long long n, long long* off) {
    n = (n + 63) / 64 * 64;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        *off = it->first;
        const long long rest = it->second - n, at = it->first + n;
        free_.erase(it);
        if (rest > 0) free_[at] = rest;
        return true;
      }
    }
    return false;
  }
  void release(long long off, long long n) {
    n = (n + 63) / 64 * 64;
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
};

long long cells_of(const mf_box& b) {
  long long n = 1;
  for (int d = 0; d < 3; ++d) n *= (long long)(b.hi[d] - b.lo[d] + 1);
  return n;
}

struct Run {
  bool used = false;
  mf_run_spec spec;
  mf::LevelPlan plan;
  long long coff = 0, foff = 0, boff = 0;  // arena offsets
  long long csize = 0, fsize = 0, bsize = 0;
  long long steps = 0;
  bool fresh = false;   // admitted since the last step: needs its first dt
  double dt_min = 0.0;
  unsigned flags = 0;
  RunParams rp;
};

}  // namespace

struct mf_server {
  mf_ctx* ctx = nullptr;
  mf::CtxView cv;
  int sd = 0, nc = 0, ng = 0;
  size_t rs = 8;
  DevMem U, U1, W, Wf, F[3], Bn[3];
  Arena ac, af, ab;
  std::vector<Run> runs;
  // the batch of the admitted runs
  bool dirty = true;
  int nslots = 0;  // runs in the launch: highest admitted slot + 1
  mf::Batch b1, b2;
  DevMem desc, runtab, exfull, extwo, partials, states, tstates, sun;
  int nfull = 0, ntwo = 0, nsun = 0;
  HostMem hstates, staging;
  cudaStream_t s = nullptr;
  cudaGraphExec_t graph = nullptr;
};

namespace {

mf_params run_params(const mf_server* S, const mf_run_spec& sp) {
  mf_params p = *S->cv.p;
  p.dx = sp.dx;
  for (int d = 0; d < 3; ++d) {
    p.domain_lo[d] = 0;
    p.domain_hi[d] = (d < S->sd) ? sp.n[d] - 1 : 0;
  }
  for (int q = 0; q < 8; ++q) p.bc_plasma[q] = sp.bc_plasma[q];
  for (int q = 0; q < 5; ++q) p.bc_neutral1[q] = sp.bc_neutral1[q];
  return p;
}

bool spec_ok(const mf_server* S, const mf_run_spec* sp) {
  if (!sp || sp->patch <= 0 || !(sp->dx > 0.0) || !(sp->cfl > 0.0) || !std::isfinite(sp->dx))
    return false;
  for (int d = 0; d < 3; ++d) {
    if (d < S->sd && (sp->n[d] <= 0 || sp->n[d] > (1 << 20))) return false;
    if (d >= S->sd && sp->n[d] != 1) return false;
  }
  return true;
}

mf_status plan_run(const mf_server* S, const mf_run_spec& sp, mf::LevelPlan& plan) {
  std::vector<mf_box> boxes;
  const int sd = S->sd, P = sp.patch;
  const int nz = (sd == 3) ? sp.n[2] : 1;
  for (int k = 0; k < nz; k += (sd == 3 ? P : 1))
    for (int j = 0; j < sp.n[1]; j += P)
      for (int i = 0; i < sp.n[0]; i += P) {
        mf_box b;
        b.lo[0] = i;
        b.hi[0] = std::min(i + P, sp.n[0]) - 1;
        b.lo[1] = j;
        b.hi[1] = std::min(j + P, sp.n[1]) - 1;
        b.lo[2] = (sd == 3) ? k : 0;
        b.hi[2] = (sd == 3) ? std::min(k + P, nz) - 1 : 0;
        boxes.push_back(b);
      }
  const mf_params p = run_params(S, sp);
  return mf::build_level_plan(p, S->ng, S->nc, (int)boxes.size(), boxes.data(), plan);
}

long long fmax3(const long long* a) { return std::max(a[0], std::max(a[1], a[2])); }

// Concatenate the admitted runs into the launch batch and capture the step.
mf_status rebuild(mf_server* S) {
  if (S->graph) {
    cudaGraphExecDestroy(S->graph);
    S->graph = nullptr;
  }
  int hi = -1;
  for (int r = 0; r < (int)S->runs.size(); ++r)
    if (S->runs[r].used) hi = r;
  S->nslots = hi + 1;
  std::vector<StageDesc> d1, d2;
  std::vector<CopyReg> full, two;
  std::vector<mf::SunPair> sun;
  for (int r = 0; r <= hi; ++r) {
    const Run& R = S->runs[r];
    if (!R.used) continue;
    for (int pass = 0; pass < 2; ++pass) {
      const std::vector<StageDesc>& src = pass ? R.plan.d2 : R.plan.d1;
      std::vector<StageDesc>& dst = pass ? d2 : d1;
      for (StageDesc D : src) {
        D.u_off += R.coff;
        for (int d = 0; d < 3; ++d) {
          D.f_off[d] += R.foff;
          D.bn_off[d] += R.boff;
        }
        D.run = r;
        dst.push_back(D);
      }
    }
    for (int pass = 0; pass < 2; ++pass) {
      const std::vector<CopyReg>& src = pass ? R.plan.two : R.plan.full;
      std::vector<CopyReg>& dst = pass ? two : full;
      for (CopyReg C : src) {
        C.src_off += R.coff;
        C.dst_off += R.coff;
        dst.push_back(C);
      }
    }
    for (mf::SunPair sp : R.plan.sun) {
      sp.to += R.coff;
      sp.from += R.coff;
      sun.push_back(sp);
    }
  }
  std::memset(&S->b1, 0, sizeof(S->b1));
  std::memset(&S->b2, 0, sizeof(S->b2));
  S->dirty = false;
  if (S->nslots == 0) return MF_OK;
  std::vector<RunParams> rt(S->nslots);
  for (int r = 0; r < S->nslots; ++r) {
    rt[r] = S->runs[r].used ? S->runs[r].rp : RunParams();
    if (!S->runs[r].used) std::memset(&rt[r], 0, sizeof(RunParams));
  }
  const int n = (int)d1.size();
  if (!mf::batch_offsets(d1.data(), n, S->sd, S->b1, nullptr, S->nslots) ||
      !mf::batch_offsets(d2.data(), n, S->sd, S->b2, rt.data(), S->nslots))
    return MF_ERR_UNSUPPORTED;
  // unused slots: an empty cell range, dx of 1 (their finalize block only
  // flags their own, unused step state)
  for (int r = 0; r < S->nslots; ++r)
    if (!S->runs[r].used) {
      rt[r].dx = rt[r].invdx = 1.0;
    }
  mf::batch_default_threads(S->b1);
  mf::batch_default_threads(S->b2);
  const size_t dbytes = sizeof(StageDesc) * (size_t)n;
  SV_CUDA(S->desc.ensure(2 * dbytes));
  SV_CUDA(cudaMemcpy(S->desc.p, d1.data(), dbytes, cudaMemcpyHostToDevice));
  SV_CUDA(cudaMemcpy((char*)S->desc.p + dbytes, d2.data(), dbytes, cudaMemcpyHostToDevice));
  SV_CUDA(S->runtab.ensure(sizeof(RunParams) * rt.size()));
  SV_CUDA(cudaMemcpy(S->runtab.p, rt.data(), sizeof(RunParams) * rt.size(),
                     cudaMemcpyHostToDevice));
  S->b1.desc = (const StageDesc*)S->desc.p;
  S->b2.desc = (const StageDesc*)((char*)S->desc.p + dbytes);
  S->b1.runs = S->b2.runs = (const RunParams*)S->runtab.p;
  S->nfull = (int)full.size();
  S->ntwo = (int)two.size();
  SV_CUDA(S->exfull.ensure(sizeof(CopyReg) * std::max<size_t>(1, full.size())));
  if (!full.empty())
    SV_CUDA(cudaMemcpy(S->exfull.p, full.data(), sizeof(CopyReg) * full.size(),
                       cudaMemcpyHostToDevice));
  SV_CUDA(S->extwo.ensure(sizeof(CopyReg) * std::max<size_t>(1, two.size())));
  if (!two.empty())
    SV_CUDA(cudaMemcpy(S->extwo.p, two.data(), sizeof(CopyReg) * two.size(),
                       cudaMemcpyHostToDevice));
  S->nsun = (int)sun.size();
  SV_CUDA(S->sun.ensure(sizeof(mf::SunPair) * std::max<size_t>(1, sun.size())));
  if (!sun.empty())
    SV_CUDA(cudaMemcpy(S->sun.p, sun.data(), sizeof(mf::SunPair) * sun.size(),
                       cudaMemcpyHostToDevice));
  SV_CUDA(S->partials.ensure(sizeof(DtPartial) * (mf::dt_partials(S->b2) + 1)));
  return MF_OK;
}

// Device bytes per fab value of the cell arrays: U, U1, W (FP64), plus the
// FP32 copy of W in mixed precision.
long long cell_bytes(const mf_server* S) {
  return (S->cv.p->precision == MF_PREC_MIXED) ? 28 : 24;
}

// The step of every admitted run (the level step of mf_capi.cu with the
// batch of runs): exchange, RK2 stage 1, exchange of the predictor, stage 2
// with averaging and dt, per-run dt reduction and next dt / GLM speeds.
mf_status enqueue_step(mf_server* S) {
  const mf_params& p = *S->cv.p;
  const mf::DevParams& P = *S->cv.dp;
  StepState* ds = (StepState*)S->states.p;
  DtPartial* parts = (DtPartial*)S->partials.p;
  StageBuffers B;
  std::memset(&B, 0, sizeof(B));
  B.w = (double*)S->W.p;
  B.wf = (p.precision == MF_PREC_MIXED) ? (float*)S->Wf.p : nullptr;
  for (int d = 0; d < 3; ++d) {
    B.f[d] = S->F[d].p;
    B.bn[d] = S->Bn[d].p;
  }
  int nb = 0;
  SV_CUDA(mf::launch_exchange((double*)S->U.p, (const CopyReg*)S->exfull.p, S->nfull, S->nc,
                              S->s));
  if (p.time_approximation == MF_TA_RK2) {
    B.uin = (const double*)S->U.p;
    B.uout = (double*)S->U1.p;
    SV_CUDA(mf::launch_stage(P, p.precision, B, S->b1, 0, 1.0, ds, parts, &nb, S->s));
    SV_CUDA(mf::launch_exchange((double*)S->U1.p, (const CopyReg*)S->extwo.p, S->ntwo, S->nc,
                                S->s));
    B.uin = (const double*)S->U1.p;
    B.uout = (double*)S->U.p;
    B.uold = (const double*)S->U.p;
    SV_CUDA(mf::launch_stage(P, p.precision, B, S->b2, mf::kStageAverage | mf::kStageDt, 0.5, ds,
                             parts, &nb, S->s));
  } else {
    B.uin = (const double*)S->U.p;
    B.uout = (double*)S->U.p;
    SV_CUDA(mf::launch_stage(P, p.precision, B, S->b2, mf::kStageDt, 1.0, ds, parts, &nb, S->s));
  }
  SV_CUDA(mf::launch_finalize(P, parts, S->b2, S->b2.nt[2], ds, 1, S->s));
  // neutral pass-through at the sun of every run (NEUTRALS_SUNBC)
  SV_CUDA(mf::launch_sun_copy((double*)S->U.p, (const mf::SunPair*)S->sun.p, S->nsun, P.irhon,
                              P.nf, S->s));
  return MF_OK;
}

mf_status capture(mf_server* S) {
  cudaGraph_t g = nullptr;
  SV_CUDA(cudaStreamBeginCapture(S->s, cudaStreamCaptureModeThreadLocal));
  mf_status st = enqueue_step(S);
  cudaError_t e = cudaStreamEndCapture(S->s, &g);
  if (st != MF_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return MF_ERR_CUDA;
  e = cudaGraphInstantiate(&S->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    S->graph = nullptr;
    return MF_ERR_CUDA;
  }
  return MF_OK;
}

mf_status join(cudaStream_t from, cudaStream_t to) {
  if (from == to) return MF_OK;
  cudaEvent_t ev;
  SV_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ev, from);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(to, ev, 0);
  cudaEventDestroy(ev);
  return e == cudaSuccess ? MF_OK : MF_ERR_CUDA;
}

// Host copy of a run's state <-> the run's fabs (valid cells; ghosts zero).
void pack(const mf_server* S, const Run& R, const double* host, double* fabs) {
  const int nc = S->nc;
  const long long nx = R.spec.n[0], ny = R.spec.n[1], nz = (S->sd == 3) ? R.spec.n[2] : 1;
  std::memset(fabs, 0, sizeof(double) * R.plan.total);
  for (int i = 0; i < R.plan.np; ++i) {
    const mf_box& v = R.plan.valid[i];
    const mf_box& f = R.plan.fab[i];
    const long long fx = f.hi[0] - f.lo[0] + 1, fy = f.hi[1] - f.lo[1] + 1;
    const long long fcs = cells_of(f);
    double* base = fabs + R.plan.off[i];
    for (int q = 0; q < nc; ++q)
      for (int k = v.lo[2]; k <= v.hi[2]; ++k)
        for (int j = v.lo[1]; j <= v.hi[1]; ++j) {
          const double* src = host + q * nx * ny * nz + (k * ny + j) * nx + v.lo[0];
          double* dst = base + q * fcs + ((k - f.lo[2]) * fy + (j - f.lo[1])) * fx +
                        (v.lo[0] - f.lo[0]);
          std::memcpy(dst, src, sizeof(double) * (v.hi[0] - v.lo[0] + 1));
        }
  }
}

void unpack(const mf_server* S, const Run& R, const double* fabs, double* host) {
  const int nc = S->nc;
  const long long nx = R.spec.n[0], ny = R.spec.n[1], nz = (S->sd == 3) ? R.spec.n[2] : 1;
  for (int i = 0; i < R.plan.np; ++i) {
    const mf_box& v = R.plan.valid[i];
    const mf_box& f = R.plan.fab[i];
    const long long fx = f.hi[0] - f.lo[0] + 1, fy = f.hi[1] - f.lo[1] + 1;
    const long long fcs = cells_of(f);
    const double* base = fabs + R.plan.off[i];
    for (int q = 0; q < nc; ++q)
      for (int k = v.lo[2]; k <= v.hi[2]; ++k)
        for (int j = v.lo[1]; j <= v.hi[1]; ++j) {
          double* dst = host + q * nx * ny * nz + (k * ny + j) * nx + v.lo[0];
          const double* src = base + q * fcs + ((k - f.lo[2]) * fy + (j - f.lo[1])) * fx +
                              (v.lo[0] - f.lo[0]);
          std::memcpy(dst, src, sizeof(double) * (v.hi[0] - v.lo[0] + 1));
        }
  }
}

void release_run(mf_server* S, Run& R) {
  S->ac.release(R.coff, R.csize);
  S->af.release(R.foff, R.fsize);
  S->ab.release(R.boff, R.bsize);
  R = Run();
  S->dirty = true;
}

}  // namespace

extern "C" {

mf_status mf_server_create(mf_ctx* physics, double hbm_budget_bytes, int max_runs,
                           mf_server** out) {
  if (!physics || !out || max_runs <= 0 || max_runs > 4096 || !(hbm_budget_bytes > 0.0))
    return MF_ERR_BAD_ARG;
  *out = nullptr;
  if (mf::ctx_view(physics).p->time_approximation == MF_TA_HANCOCK) return MF_ERR_UNSUPPORTED;
  if (mf::ctx_view(physics).dp->ct) return MF_ERR_UNSUPPORTED;  // constrained transport
  mf_server* S = new (std::nothrow) mf_server();
  if (!S) return MF_ERR_OOM;
  S->ctx = physics;
  S->cv = mf::ctx_view(physics);
  S->sd = S->cv.p->space_dim;
  S->nc = S->cv.nc;
  S->ng = S->cv.ng;
  S->rs = mf::flux_bytes(S->cv.p->precision);
  S->runs.resize(max_runs);
  // split of the budget: cells (U, U1, W: 24 bytes per double of a fab, and
  // 4 more for the FP32 copy of W in mixed precision), face fluxes (3
  // directions) and face-normal B (3 directions) with room for 0.75 face
  // values per fab value
  const double per = (double)cell_bytes(S) + 3.0 * 0.75 * S->rs * (1.0 + 1.0 / S->nc);
  const long long capC = (long long)(hbm_budget_bytes / per) / 64 * 64;
  const long long capF = (long long)(0.75 * capC) / 64 * 64;
  const long long capB = (long long)(0.75 * capC / S->nc) / 64 * 64 + 64 * max_runs;
  mf_status st = MF_OK;
  cudaError_t e = cudaSuccess;
  do {
    if ((e = S->U.ensure(sizeof(double) * capC)) != cudaSuccess) break;
    if ((e = S->U1.ensure(sizeof(double) * capC)) != cudaSuccess) break;
    if ((e = S->W.ensure(sizeof(double) * capC)) != cudaSuccess) break;
    if (S->cv.p->precision == MF_PREC_MIXED &&
        (e = S->Wf.ensure(sizeof(float) * capC)) != cudaSuccess)
      break;
    for (int d = 0; d < S->sd && e == cudaSuccess; ++d) {
      e = S->F[d].ensure(S->rs * capF);
      if (e == cudaSuccess) e = S->Bn[d].ensure(S->rs * capB);
    }
    if (e != cudaSuccess) break;
    if ((e = S->states.ensure(sizeof(StepState) * max_runs)) != cudaSuccess) break;
    if ((e = S->tstates.ensure(sizeof(StepState) * max_runs)) != cudaSuccess) break;
    if ((e = cudaMemset(S->states.p, 0, sizeof(StepState) * max_runs)) != cudaSuccess) break;
    if ((e = S->hstates.ensure(sizeof(StepState) * max_runs)) != cudaSuccess) break;
    if ((e = cudaStreamCreateWithFlags(&S->s, cudaStreamNonBlocking)) != cudaSuccess) break;
  } while (0);
  if (e != cudaSuccess) st = (e == cudaErrorMemoryAllocation) ? MF_ERR_OOM : MF_ERR_CUDA;
  if (st != MF_OK) {
    mf_server_destroy(S);
    return st;
  }
  S->ac.init(capC);
  S->af.init(capF);
  S->ab.init(capB);
  *out = S;
  return MF_OK;
}

void mf_server_destroy(mf_server* S) {
  if (!S) return;
  if (S->s) cudaStreamSynchronize(S->s);
  if (S->graph) cudaGraphExecDestroy(S->graph);
  if (S->s) cudaStreamDestroy(S->s);
  S->U.release();
  S->U1.release();
  S->W.release();
  S->Wf.release();
  for (int d = 0; d < 3; ++d) {
    S->F[d].release();
    S->Bn[d].release();
  }
  S->desc.release();
  S->runtab.release();
  S->sun.release();
  S->exfull.release();
  S->extwo.release();
  S->partials.release();
  S->states.release();
  S->tstates.release();
  S->hstates.release();
  S->staging.release();
  delete S;
}

long long mf_server_run_bytes(const mf_server* S, const mf_run_spec* spec) {
  if (!S || !spec_ok(S, spec)) return -1;
  mf::LevelPlan plan;
  if (plan_run(S, *spec, plan) != MF_OK) return -1;
  return (long long)(cell_bytes(S) * plan.total +
                     3 * S->rs * (fmax3(plan.fsize) + fmax3(plan.bsize)));
}

mf_status mf_server_admit(mf_server* S, const mf_run_spec* spec, const double* state, int* run) {
  if (!S || !state || !run || !spec_ok(S, spec)) return MF_ERR_BAD_ARG;
  *run = -1;
  int slot = -1;
  for (int r = 0; r < (int)S->runs.size(); ++r)
    if (!S->runs[r].used) {
      slot = r;
      break;
    }
  if (slot < 0) return MF_ERR_NO_ROOM;
  Run R;
  R.spec = *spec;
  mf_status st = plan_run(S, *spec, R.plan);
  if (st != MF_OK) return st;
  R.csize = R.plan.total;
  R.fsize = std::max<long long>(64, fmax3(R.plan.fsize));
  R.bsize = std::max<long long>(64, fmax3(R.plan.bsize));
  if (!S->ac.alloc(R.csize, &R.coff)) return MF_ERR_NO_ROOM;
  if (!S->af.alloc(R.fsize, &R.foff)) {
    S->ac.release(R.coff, R.csize);
    return MF_ERR_NO_ROOM;
  }
  if (!S->ab.alloc(R.bsize, &R.boff)) {
    S->ac.release(R.coff, R.csize);
    S->af.release(R.foff, R.fsize);
    return MF_ERR_NO_ROOM;
  }
  std::memset(&R.rp, 0, sizeof(R.rp));
  R.rp.dx = spec->dx;
  R.rp.invdx = 1.0 / spec->dx;
  for (int d = 0; d < 3; ++d) {
    R.rp.dlo[d] = 0;
    R.rp.dhi[d] = (d < S->sd) ? spec->n[d] - 1 : 0;
  }
  for (int q = 0; q < 8; ++q) R.rp.bc_plasma[q] = spec->bc_plasma[q];
  for (int q = 0; q < 5; ++q) R.rp.bc_n1[q] = spec->bc_neutral1[q];
  R.used = true;
  R.fresh = true;
  // state into the arena, the run's step state seeded
  cudaError_t e = S->staging.ensure(sizeof(double) * R.plan.total);
  if (e == cudaSuccess) {
    pack(S, R, state, (double*)S->staging.p);
    e = cudaMemcpyAsync((double*)S->U.p + R.coff, S->staging.p, sizeof(double) * R.plan.total,
                        cudaMemcpyHostToDevice, S->s);
  }
  StepState hs;
  std::memset(&hs, 0, sizeof(hs));
  hs.ch = S->cv.p->dedner_ch;
  hs.cp = S->cv.p->dedner_cp;
  hs.cfl = spec->cfl;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync((StepState*)S->states.p + slot, &hs, sizeof(hs), cudaMemcpyHostToDevice,
                        S->s);
  if (e == cudaSuccess) st = mf::host_wait(S->s, S->cv.timeout);  // staging is reused
  else st = MF_ERR_CUDA;
  S->runs[slot] = R;
  if (st != MF_OK) {
    release_run(S, S->runs[slot]);
    return st;
  }
  S->dirty = true;
  *run = slot;
  return MF_OK;
}

mf_status mf_server_step(mf_server* S, void* stream) {
  if (!S) return MF_ERR_BAD_ARG;
  cudaStream_t us = (cudaStream_t)stream;
  mf_status st = join(us, S->s);
  if (st != MF_OK) return st;
  bool fresh = false;
  for (const Run& R : S->runs) fresh = fresh || (R.used && R.fresh);
  if (S->dirty) {
    st = rebuild(S);
    if (st != MF_OK) return st;
  }
  if (S->nslots == 0) return join(S->s, us);
  if (fresh) {
    // first dt and GLM speeds of the new runs (dx / max wave speed of the
    // admitted state), reduced into a copy of the step states; only the new
    // runs' entries are taken, so the runs already stepping keep the values
    // their last step left
    const size_t sb = sizeof(StepState) * S->nslots;
    SV_CUDA(cudaMemcpyAsync(S->tstates.p, S->states.p, sb, cudaMemcpyDeviceToDevice, S->s));
    int nb = 0;
    SV_CUDA(mf::launch_dt(*S->cv.dp, (const double*)S->U.p, S->b2,
                          (DtPartial*)S->partials.p, &nb, S->s));
    SV_CUDA(mf::launch_finalize(*S->cv.dp, (const DtPartial*)S->partials.p, S->b2,
                                S->b2.nt[2], (StepState*)S->tstates.p, 1, S->s));
    for (int r = 0; r < S->nslots; ++r) {
      Run& R = S->runs[r];
      if (!R.used || !R.fresh) continue;
      SV_CUDA(cudaMemcpyAsync((StepState*)S->states.p + r, (const StepState*)S->tstates.p + r,
                              sizeof(StepState), cudaMemcpyDeviceToDevice, S->s));
      R.fresh = false;
    }
  }
  if (!S->graph) {
    st = capture(S);
    if (st != MF_OK) return st;
  }
  SV_CUDA(cudaGraphLaunch(S->graph, S->s));
  for (Run& R : S->runs)
    if (R.used) R.steps += 1;
  return join(S->s, us);
}

mf_status mf_server_sync(mf_server* S, void* stream) {
  if (!S) return MF_ERR_BAD_ARG;
  mf_status st = join((cudaStream_t)stream, S->s);
  if (st != MF_OK) return st;
  const int n = std::max(1, S->nslots);
  SV_CUDA(cudaMemcpyAsync(S->hstates.p, S->states.p, sizeof(StepState) * n,
                          cudaMemcpyDeviceToHost, S->s));
  st = mf::host_wait(S->s, S->cv.timeout);
  if (st != MF_OK) return st;
  const StepState* hs = (const StepState*)S->hstates.p;
  for (int r = 0; r < S->nslots; ++r) {
    Run& R = S->runs[r];
    if (!R.used || R.steps == 0) continue;
    R.dt_min = hs[r].dt_min;
    R.flags = hs[r].flags;
  }
  return MF_OK;
}

mf_status mf_server_run_info(const mf_server* S, int run, long long* steps, double* dt_min,
                             mf_status* run_status) {
  if (!S || run < 0 || run >= (int)S->runs.size() || !S->runs[run].used) return MF_ERR_BAD_ARG;
  const Run& R = S->runs[run];
  if (steps) *steps = R.steps;
  if (dt_min) *dt_min = R.dt_min;
  if (run_status) *run_status = mf::status_of_flags(R.flags);
  return MF_OK;
}

mf_status mf_server_retire(mf_server* S, int run, double* state, void* stream) {
  if (!S || run < 0 || run >= (int)S->runs.size() || !S->runs[run].used) return MF_ERR_BAD_ARG;
  Run& R = S->runs[run];
  mf_status st = join((cudaStream_t)stream, S->s);
  if (st != MF_OK) return st;
  if (state) {
    SV_CUDA(S->staging.ensure(sizeof(double) * R.plan.total));
    SV_CUDA(cudaMemcpyAsync(S->staging.p, (const double*)S->U.p + R.coff,
                            sizeof(double) * R.plan.total, cudaMemcpyDeviceToHost, S->s));
    st = mf::host_wait(S->s, S->cv.timeout);
    if (st != MF_OK) return st;
    unpack(S, R, (const double*)S->staging.p, state);
  } else {
    st = mf::host_wait(S->s, S->cv.timeout);
    if (st != MF_OK) return st;
  }
  release_run(S, R);
  return MF_OK;
}

mf_status mf_server_set_priority(mf_server* S, int priority) {
  if (!S) return MF_ERR_BAD_ARG;
  int least = 0, greatest = 0;
  SV_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
  // greatest is the numerically lowest value (highest priority)
  const int pr = std::min(least, std::max(greatest, priority));
  mf_status st = mf::host_wait(S->s, S->cv.timeout);
  if (st != MF_OK) return st;
  cudaStream_t ns = nullptr;
  SV_CUDA(cudaStreamCreateWithPriority(&ns, cudaStreamNonBlocking, pr));
  cudaStreamDestroy(S->s);
  S->s = ns;
  return MF_OK;
}

int mf_server_active(const mf_server* S) {
  if (!S) return -1;
  int n = 0;
  for (const Run& R : S->runs) n += R.used ? 1 : 0;
  return n;
}

long long mf_server_free_bytes(const mf_server* S) {
  if (!S) return -1;
  long long c = 0;
  for (const auto& kv : S->ac.free_) c = std::max(c, kv.second);
  return cell_bytes(S) * c;
}

}  // extern "C"
