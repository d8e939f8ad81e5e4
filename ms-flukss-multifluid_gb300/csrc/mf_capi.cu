// mf_capi.cu - C ABI of the GB300 patch integrator (include/mf_patch.h).
//
// mf_patch_update follows PatchMHDAM::updateState (src/PatchMHDAM.cpp:1192-1317)
// on one device fab: RK2 stage 1 on box.grow(2), stage 2 on box, AVERAGESTATE,
// computeDt.  mf_level_* keep every patch of a level resident in one device
// allocation and replace the redundant stage-1 ghost computation by a
// device-side exchange of the stage-1 state between the two stages; both give
// the same results because every stage-1 ghost value equals the value its
// owner patch computes for that cell (with constrained transport it does not:
// there every patch runs stage 1 on box.grow(2) and no exchange follows).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <thread>
#include <unordered_map>
#include <array>
#include <vector>

#include "mf_internal.h"
#include "mf_kernels.cuh"
#include "mf_sources_exact.cuh"

using mf::CopyReg;
using mf::DevParams;
using mf::DtPartial;
using mf::StageBuffers;
using mf::RunParams;
using mf::StageDesc;
using mf::StepState;

namespace {

struct DevBuf {
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

struct PinnedBuf {
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

int space_dim_ok(int sd) { return sd == 2 || sd == 3; }

long long box_cells(const mf_box& b) {
  long long n = 1;
  for (int d = 0; d < 3; ++d) n *= (long long)(b.hi[d] - b.lo[d] + 1);
  return n;
}

bool box_empty(const mf_box& b) {
  for (int d = 0; d < 3; ++d)
    if (b.hi[d] < b.lo[d]) return true;
  return false;
}

mf_box box_grow(mf_box b, int n, int sd) {
  for (int d = 0; d < sd; ++d) {
    b.lo[d] -= n;
    b.hi[d] += n;
  }
  return b;
}

mf_box box_isect(const mf_box& a, const mf_box& b) {
  mf_box r;
  for (int d = 0; d < 3; ++d) {
    r.lo[d] = std::max(a.lo[d], b.lo[d]);
    r.hi[d] = std::min(a.hi[d], b.hi[d]);
  }
  return r;
}

mf_box box_nodes(mf_box b, int d) {
  b.hi[d] += 1;
  return b;
}

bool box_contains(const mf_box& outer, const mf_box& inner) {
  for (int d = 0; d < 3; ++d)
    if (inner.lo[d] < outer.lo[d] || inner.hi[d] > outer.hi[d]) return false;
  return true;
}

// Box & ProblemDomain: only the non-periodic directions are clipped.
mf_box box_and_domain(mf_box b, const mf_params& p) {
  for (int d = 0; d < p.space_dim; ++d) {
    if (p.periodic[d]) continue;
    b.lo[d] = std::max(b.lo[d], p.domain_lo[d]);
    b.hi[d] = std::min(b.hi[d], p.domain_hi[d]);
  }
  return b;
}

void ext3(const mf_box& b, int n[3]) {
  for (int d = 0; d < 3; ++d) n[d] = b.hi[d] - b.lo[d] + 1;
}

// fluid components (EqSysMHDMF::consInterval) and the tracking surfaces after
// them (lvlsStateInterval, srcIdeal/EqSysMHDMF.cpp:11-48)
int num_fluid_cons(const mf_params& p) {
  return 8 + (p.divb_cleaning == 5 ? 1 : 0) + (p.n_fluids - 1) * 5;
}

int num_cons(const mf_params& p) { return num_fluid_cons(p) + p.num_tracking_surfaces; }

int num_ghost_of(const mf_params& p) {
  if (p.time_approximation == MF_TA_RK2) return 4;
  if (p.time_approximation == MF_TA_HANCOCK) return 3;
  return 2;
}

mf_status validate_params(const mf_params& p) {
  if (!space_dim_ok(p.space_dim)) return MF_ERR_BAD_ARG;
  if (p.n_fluids < 1 || p.n_fluids > MF_MAX_FLUIDS) return MF_ERR_BAD_ARG;
  if (!(p.gamma > 1.0) || !(p.dx > 0.0)) return MF_ERR_BAD_ARG;
  if (p.time_approximation != MF_TA_RK2 && p.time_approximation != MF_TA_FIRST_ORDER &&
      p.time_approximation != MF_TA_HANCOCK)
    return MF_ERR_UNSUPPORTED;
  if (p.precision != MF_PREC_FP64 && p.precision != MF_PREC_MIXED &&
      p.precision != MF_PREC_FP64_FAST && p.precision != MF_PREC_MIXED_CE32)
    return MF_ERR_BAD_ARG;
  if (!std::isfinite(p.max_dt_growth) || !std::isfinite(p.sun_tilt)) return MF_ERR_BAD_ARG;
  if (!(p.divb_cleaning == 0 || (p.divb_cleaning >= 1 && p.divb_cleaning <= 3) ||
        p.divb_cleaning == 5))
    return MF_ERR_UNSUPPORTED;
  // electricFieldGS0/GS1 in 3D store the z-edge field through EX
  // (srcIdeal/DivCleaningF.ChF:478-566, 700-852): nothing defined to match
  if (p.divb_cleaning >= 2 && p.divb_cleaning <= 3 && p.space_dim == 3) return MF_ERR_UNSUPPORTED;
  if (p.check_tvd < 0 || p.check_tvd > 2) return MF_ERR_BAD_ARG;
  if (p.helio_bc && (p.bc_kind != MF_BC_FARFIELD || p.space_dim != 3)) return MF_ERR_UNSUPPORTED;
  if (p.neutral_sun_bc && (p.space_dim != 3 || p.n_fluids < 2)) return MF_ERR_UNSUPPORTED;
  if (p.num_tracking_surfaces < 0) return MF_ERR_BAD_ARG;
  if (p.num_tracking_surfaces > 2 || num_cons(p) > MF_MAX_COMP) return MF_ERR_UNSUPPORTED;
  if (p.region_tracer && p.num_tracking_surfaces < 1) return MF_ERR_BAD_ARG;
  // limiter1D::eLimiters (src/limiter1D.H:17-28): every value 0..11
  if (p.num_tracking_surfaces > 0 && (p.limiter_ls < MF_LIM_CD || p.limiter_ls > MF_LIM_WENO3YC))
    return MF_ERR_UNSUPPORTED;
  if (p.divb_cleaning == 5) {
    // main/MHDAM.cpp:1042-1046
    if (p.use_8wave) return MF_ERR_UNSUPPORTED;
    if (!(p.flux == 1 || p.flux == 3)) return MF_ERR_UNSUPPORTED;
  }
  for (int v = 0; v < 8; ++v)
    if (p.limiter[v] < MF_LIM_CD || p.limiter[v] > MF_LIM_WENO3YC) return MF_ERR_UNSUPPORTED;
  if (p.divb_method < 0 || p.divb_method > 2) return MF_ERR_BAD_ARG;
  for (int d = 0; d < p.space_dim; ++d)
    if (p.domain_hi[d] < p.domain_lo[d]) return MF_ERR_BAD_ARG;
  for (int d = p.space_dim; d < 3; ++d)
    if (p.domain_lo[d] != 0 || p.domain_hi[d] != 0) return MF_ERR_BAD_ARG;
  return MF_OK;
}

DevParams make_dev(const mf_params& p) {
  DevParams P;
  std::memset(&P, 0, sizeof(P));
  P.sd = p.space_dim;
  P.nf = p.n_fluids;
  P.glm = (p.divb_cleaning == 5) ? 1 : 0;
  P.nc = num_cons(p);
  P.ils = num_fluid_cons(p);
  P.nls = p.num_tracking_surfaces;
  P.lim_ls = p.limiter_ls;
  P.reg_tracer = (p.region_tracer && P.nls > 0) ? 1 : 0;
  P.ct = (p.divb_cleaning >= 1 && p.divb_cleaning <= 3) ? p.divb_cleaning : 0;
  P.ce32 = (p.precision == MF_PREC_MIXED_CE32) ? 1 : 0;
  // HeliosphericProblem: every sunBmonopolar but 1 is bipolar
  // (swlism/HeliosphericProblem.cpp:156); the current-sheet surface is the
  // first tracking surface, the first of two with the region tracer (:616-631)
  P.monopolar = (p.sun_b_monopolar == 1) ? 1 : 0;
  P.ihcs = -1;
  if (!P.monopolar && p.num_tracking_surfaces > (p.region_tracer ? 1 : 0)) P.ihcs = P.ils;
  for (int d = 0; d < 3; ++d) P.lism_u[d] = p.lism_u[d];
  P.irhon = 8 + P.glm;
  // RiemannSolver::make (src/RiemannSolver.cpp:13-112)
  if (P.glm) {
    P.rs = mf::kRoe7;
    P.aver = (p.flux == 3);
  } else {
    switch (p.flux) {
      case 2: P.rs = mf::kRusanov; P.aver = 0; break;
      case 3: P.rs = mf::kRoe8; P.aver = 1; break;
      case 4: P.rs = mf::kRusanov; P.aver = 1; break;
      case 5: P.rs = mf::kVFRoe; P.aver = 0; break;
      case 11: P.rs = mf::kRoe7; P.aver = 0; break;
      case 13: P.rs = mf::kRoe7; P.aver = 1; break;
      default: P.rs = mf::kRoe8; P.aver = 0; break;
    }
  }
  P.use8 = p.use_8wave ? 1 : 0;
  P.divb_method = p.divb_method;
  P.check_pos = p.check_positivity ? 1 : 0;
  P.char_rec = p.char_reconstruction ? 1 : 0;
  P.check_tvd = p.check_tvd;
  P.helio_bc = (p.helio_bc && p.bc_kind == MF_BC_FARFIELD && p.space_dim == 3) ? 1 : 0;
  P.ce = (p.charge_exchange && p.n_fluids >= 2) ? 1 : 0;
  P.reinit = p.reinit_sphere ? 1 : 0;
  P.bc_kind = p.bc_kind;
  for (int v = 0; v < 8; ++v) P.lim[v] = p.limiter[v];
  for (int d = 0; d < 3; ++d) {
    P.periodic[d] = (d < p.space_dim) ? (p.periodic[d] ? 1 : 0) : 1;
    P.dlo[d] = p.domain_lo[d];
    P.dhi[d] = p.domain_hi[d];
  }
  P.gamma = p.gamma;
  P.hgamma = p.gamma - 1.0;
  P.invhgamma = 1.0 / P.hgamma;
  P.invgamma = 1.0 / p.gamma;
  P.smallr = p.smallr;
  P.smallp = p.smallp;
  P.del2 = p.entropy_fix;
  P.smallB = p.small_b;
  P.dx = p.dx;
  P.invdx = 1.0 / p.dx;
  P.factor_ch = p.factor_ch;
  P.factor_cp = p.factor_cp;
  P.ce_scale_vel = p.ce_scale_vel;
  P.ce_sigma_scale = p.ce_sigma_scale;
  P.ce_a = p.ce_sigma_a;
  P.ce_b = p.ce_sigma_b;
  P.ce_damp_c = p.ce_damp_c;
  P.ce_damp_pow = p.ce_damp_pow;
  for (int d = 0; d < 3; ++d) P.sun_c[d] = p.sun_center[d];
  P.sun_r = p.sun_r;
  P.sun_v = p.sun_v;
  P.t_coeff = p.region_t_coeff;
  P.tmlim = p.region_tmlim;
  P.zbot = p.region_zbot;
  P.ztop = p.region_ztop;
  P.r0 = p.reinit_r0;
  P.rint = p.sun_int_bc_radius;
  P.sun_rho = p.sun_rho;
  P.sun_p = p.sun_p;
  P.sun_b = p.sun_b;
  P.sun_beta = p.sun_beta;
  P.dir_br = p.dir_br;
  // SETHELIOS: sunTILT = ausunTILT * d_PI_180 (swlism/HeliosphericF.ChF:66)
  const double tilt = p.sun_tilt * (mf::kPi / 180.0);
  P.sin_tilt = std::sin(tilt);
  P.cos_tilt = std::cos(tilt);
  P.max_growth = p.max_dt_growth;
  for (int q = 0; q < 8; ++q) P.bc_plasma[q] = p.bc_plasma[q];
  for (int q = 0; q < 5; ++q) P.bc_n1[q] = p.bc_neutral1[q];
  return P;
}

double default_timeout() {
  const char* e = std::getenv("MF_WAIT_TIMEOUT_S");
  if (e) {
    double v = std::atof(e);
    if (v > 0) return v;
  }
  return 600.0;
}

// Bounded host wait: polls an event recorded on s; gives up after timeout_s.
mf_status wait_stream(cudaStream_t s, double timeout_s) {
  cudaEvent_t ev;
  if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) return MF_ERR_CUDA;
  if (cudaEventRecord(ev, s) != cudaSuccess) {
    cudaEventDestroy(ev);
    return MF_ERR_CUDA;
  }
  auto t0 = std::chrono::steady_clock::now();
  mf_status st = MF_OK;
  for (;;) {
    cudaError_t e = cudaEventQuery(ev);
    if (e == cudaSuccess) break;
    if (e != cudaErrorNotReady) {
      st = MF_ERR_CUDA;
      break;
    }
    double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (el >= timeout_s) {
      st = MF_ERR_TIMEOUT;
      break;
    }
    std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
  cudaEventDestroy(ev);
  return st;
}

mf_status flags_status(unsigned flags) {
  if (flags & mf::kFlagNonFinite) return MF_ERR_NONFINITE;
  if (flags & mf::kFlagBadDt) return MF_ERR_NEG_STATE;
  return MF_OK;
}

#define MF_CHECK_CUDA(x)                 \
  do {                                   \
    cudaError_t e_ = (x);                \
    if (e_ != cudaSuccess) {             \
      if (e_ == cudaErrorMemoryAllocation) return MF_ERR_OOM; \
      return MF_ERR_CUDA;                \
    }                                    \
  } while (0)

}  // namespace

struct mf_ctx {
  mf_params p;
  DevParams dp;
  int ng = 0, nc = 0;
  double time = 0.0;
  double timeout = 600.0;
  DevBuf pred, w, f1[3], bn1[3], f2[3], bn2[3], desc, partials, state;
  DevBuf fv[3], w2;  // Hancock face values and predicted primitive state
  DevBuf ct_u0, ct_e1, ct_e2, ct_eo;  // constrained transport: U(t), stage edge fields, average
  DevBuf wf;                          // mixed precision: FP32 copy of w for the flux kernels
  PinnedBuf hdesc, hstate;
};

struct mf_level {
  mf_ctx* ctx = nullptr;
  int np = 0;
  std::vector<mf_box> valid, fab;
  std::vector<long long> off;
  long long total = 0;
  long long cells = 0;
  DevBuf U, U1, W, F[3], Bn[3], desc, exfull, extwo, partials, state, state2;
  DevBuf FV[3];  // Hancock face values (U1 holds W(t+dt/2))
  int nfull = 0, ntwo = 0;
  // b1: RK2 stage 1 (valid boxes grown on uncovered sides); b2: the stage
  // on the valid boxes (RK2 stage 2, first order).  Descs at desc.p: b1's
  // np entries, then b2's.
  mf::Batch b1, b2;
  int nparts = 0;
  PinnedBuf hstate;
  cudaStream_t s = nullptr;
  cudaGraphExec_t gsync = nullptr, gasync = nullptr;
  int launches = 0, base_launches = 0;
  std::vector<StageDesc> hd1, hd2;         // host copies of the stage descs
  std::vector<mf::FaceGather> gathers;     // flux-register faces of a hierarchy
  DevBuf sun;                              // NEUTRALS_SUNBC cell pairs
  int nsun = 0;
  DevBuf ct_u0, ct_e1, ct_e2, ct_eo;       // constrained transport: UOld, edge fields
  DevBuf packed;                           // staging of the valid-cell transfers
  DevBuf Wf;                               // mixed precision: FP32 copy of W
  std::vector<long long> voff;             // packed offset of each patch (doubles)
  double time = 0.0;                       // start time of the next step (host mirror)
  // lean primitive part (LevelPlan::lean): prim batch over the valid boxes,
  // far-field ghost boxes
  bool lean = false;
  mf::Batch bp;
  DevBuf far;
  mf::LeanPrim lp;
  // fused flux + update kernel (mixed precision): tile work lists of both
  // stages' batches (fp1 for b1, fp2 for b2), used while no flux-register
  // gathers are attached
  bool fused = false;
  int fused_saving = 0;  // launches the fused kernel saves per step
  DevBuf tiles;
  mf::FusedPlan fp1, fp2;
  // chunked, overlapped flux + update launches of the split mixed-precision
  // stages (mf_level_set_overlap): a chunk plan per stage batch
  int nchunks = 1;
  std::vector<mf::Chunk> ch1, ch2;
  mf::OverlapPlan op1{}, op2{};
  // face fluxes by lines (FP64 paths, mf_level_set_flux_form): the work lists
  // of both stage batches, built on first use
  int flux_form = MF_FLUX_FACES;
  DevBuf lines;
  mf::LinePlan lp1{}, lp2{};
};

// Kernel launches of one step: the plain count, plus the flux-register
// gathers, less the flux launches the fused kernel replaces, and with the
// chunked overlap n + 1 flux-and-update launches per stage instead of sd + 1.
static void count_launches(mf_level* L) {
  const mf_params& p = L->ctx->p;
  const int per = (p.time_approximation == MF_TA_RK2) ? 2 : 1;
  const int sd = p.space_dim;
  const bool fused = L->fused && L->gathers.empty();
  const bool overlap = L->nchunks > 1 && !L->fused && L->gathers.empty() && !L->ctx->dp.ct;
  L->fused_saving = L->fused ? per * sd : 0;
  L->launches = L->base_launches + per * (int)L->gathers.size() - (fused ? per * sd : 0) +
                (overlap ? per * (L->nchunks - sd) : 0);
}

// Work list of the fused kernel: each desc's valueBox cut into tiles of the
// given shape (the last tile of a row may be shorter).
static std::vector<mf::FusedTile> make_tiles(const std::vector<StageDesc>& hd, int sd,
                                             const int tile[3]) {
  std::vector<mf::FusedTile> out;
  for (int i = 0; i < (int)hd.size(); ++i) {
    const StageDesc& D = hd[i];
    const int t[3] = {tile[0], tile[1], sd == 3 ? tile[2] : 1};
    for (int z = 0; z < D.vn[2]; z += t[2])
      for (int y = 0; y < D.vn[1]; y += t[1])
        for (int x = 0; x < D.vn[0]; x += t[0]) {
          mf::FusedTile T;
          T.desc = i;
          const int o[3] = {x, y, z};
          for (int d = 0; d < 3; ++d) {
            T.lo[d] = D.vlo[d] + o[d];
            T.n[d] = std::min(t[d], D.vn[d] - o[d]);
          }
          out.push_back(T);
        }
  }
  return out;
}

// (Re)build the fused work lists for a tile shape; *ok false when the shape
// does not fit (threads, shared memory).
static cudaError_t level_set_tiles(mf_level* L, const int tile[3], bool* ok) {
  const mf_params& p = L->ctx->p;
  const int sd = p.space_dim;
  *ok = false;
  if (!mf::fused_tile_ok(L->ctx->dp, tile)) return cudaSuccess;
  cudaError_t e = mf::fused_prepare();
  if (e != cudaSuccess) return e;
  std::vector<mf::FusedTile> t1 = make_tiles(L->hd1, sd, tile);
  std::vector<mf::FusedTile> t2 = make_tiles(L->hd2, sd, tile);
  std::vector<mf::FusedTile> all(t1);
  all.insert(all.end(), t2.begin(), t2.end());
  e = L->tiles.ensure(sizeof(mf::FusedTile) * std::max<size_t>(1, all.size()));
  if (e != cudaSuccess) return e;
  e = cudaMemcpy(L->tiles.p, all.data(), sizeof(mf::FusedTile) * all.size(),
                 cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return e;
  const int most = (int)std::max(t1.size(), t2.size());
  e = L->partials.ensure(sizeof(DtPartial) * (std::max(L->nparts, most) + 1));
  if (e != cudaSuccess) return e;
  for (int q = 0; q < 2; ++q) {
    mf::FusedPlan& fp = q ? L->fp2 : L->fp1;
    fp.tiles = (const mf::FusedTile*)L->tiles.p + (q ? t1.size() : 0);
    fp.ntiles = (int)(q ? t2.size() : t1.size());
    for (int d = 0; d < 3; ++d) fp.tile[d] = (d < sd) ? tile[d] : 1;
  }
  *ok = true;
  return cudaSuccess;
}

extern "C" {

void mf_params_default(mf_params* p, int space_dim, int n_fluids) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->space_dim = space_dim;
  p->n_fluids = n_fluids;
  p->time_approximation = MF_TA_FIRST_ORDER;
  p->flux = 1;
  p->divb_cleaning = 0;
  p->use_8wave = 1;
  p->divb_method = 1;
  for (int v = 0; v < 8; ++v) p->limiter[v] = MF_LIM_MINMOD;
  p->check_positivity = 0;
  p->precision = MF_PREC_FP64;
  p->gamma = 5.0 / 3.0;
  p->smallr = 1.0e-12;
  p->smallp = 1.0e-12;
  p->entropy_fix = 0.3;
  p->small_b = 1.0e-9;
  p->dx = 1.0 / 64.0;
  p->dedner_ch = 1.0;
  p->dedner_cp = 1.0;
  p->factor_ch = 0.0;
  p->factor_cp = 1.0;
  p->ce_scale_vel = 1.0;
  p->ce_sigma_scale = 1.0;
  p->ce_sigma_a = 2.1;
  p->ce_sigma_b = 0.092;
  p->ce_damp_c = 0.0;
  p->ce_damp_pow = 4.5;
  p->region_zbot = -1.0e300;
  p->region_ztop = 1.0e300;
  p->region_tmlim = 1.0e300;
  p->sun_int_bc_radius = 1.0;
  p->dir_br = 1.0;
  for (int d = 0; d < 3; ++d) {
    p->domain_lo[d] = 0;
    p->domain_hi[d] = (d < space_dim) ? 63 : 0;
    p->periodic[d] = 1;
  }
  p->bc_kind = MF_BC_NONE;
  p->num_tracking_surfaces = 0;
  p->limiter_ls = MF_LIM_MINMOD;
  p->region_tracer = 0;
  p->lism_u[0] = -1.0;
  p->max_dt_growth = 1.1;   // srcIdeal/AMR_MHDAM.cpp:94
  p->sun_b_monopolar = 0;   // swlism/HeliosphericProblem.cpp:106,156
  p->sun_tilt = 0.0;        // :102
}

int mf_params_num_cons(const mf_params* p) { return p ? num_cons(*p) : 0; }

const char* mf_status_string(mf_status s) {
  switch (s) {
    case MF_OK: return "ok";
    case MF_ERR_BAD_ARG: return "bad argument";
    case MF_ERR_OOM: return "out of memory";
    case MF_ERR_NONFINITE: return "non-finite state";
    case MF_ERR_NEG_STATE: return "non-positive state or time step";
    case MF_ERR_TIMEOUT: return "device wait timed out";
    case MF_ERR_CUDA: return "CUDA error";
    case MF_ERR_UNSUPPORTED: return "unsupported option";
    case MF_ERR_SCRATCH_LIMIT: return "patch exceeds the static scratch of the no-allocation update";
    case MF_ERR_NO_ROOM: return "no free run slot or arena space";
  }
  return "unknown status";
}

mf_status mf_create(const mf_params* p, mf_ctx** out) {
  if (!p || !out) return MF_ERR_BAD_ARG;
  *out = nullptr;
  mf_status st = validate_params(*p);
  if (st != MF_OK) return st;
  mf_ctx* c = new (std::nothrow) mf_ctx();
  if (!c) return MF_ERR_OOM;
  c->p = *p;
  c->dp = make_dev(*p);
  // the FP32-rate form runs every mixed-precision path; only the update's
  // charge-exchange rates differ (DevParams::ce32)
  if (c->p.precision == MF_PREC_MIXED_CE32) c->p.precision = MF_PREC_MIXED;
  c->ng = num_ghost_of(*p);
  c->nc = num_cons(*p);
  c->timeout = default_timeout();
  *out = c;
  return MF_OK;
}

void mf_destroy(mf_ctx* c) {
  if (!c) return;
  c->pred.release();
  c->w.release();
  for (int d = 0; d < 3; ++d) {
    c->f1[d].release();
    c->bn1[d].release();
    c->f2[d].release();
    c->bn2[d].release();
    c->fv[d].release();
  }
  c->w2.release();
  c->desc.release();
  c->partials.release();
  c->state.release();
  c->hdesc.release();
  c->hstate.release();
  delete c;
}

int mf_num_ghost(const mf_ctx* c) { return c ? c->ng : -1; }
int mf_num_cons(const mf_ctx* c) { return c ? c->nc : -1; }

mf_status mf_set_current_time(mf_ctx* c, double t) {
  if (!c) return MF_ERR_BAD_ARG;
  c->time = t;
  return MF_OK;
}

mf_status mf_set_dedner(mf_ctx* c, double ch, double cp) {
  if (!c || !(ch > 0.0) || !(cp > 0.0)) return MF_ERR_BAD_ARG;
  c->p.dedner_ch = ch;
  c->p.dedner_cp = cp;
  return MF_OK;
}

mf_status mf_set_wait_timeout(mf_ctx* c, double seconds) {
  if (!c || !(seconds >= 0.0)) return MF_ERR_BAD_ARG;
  c->timeout = seconds;
  return MF_OK;
}

static mf_status check_fab(const mf_ctx* c, const mf_fab* U, const mf_box* valid) {
  if (!U || !U->data || !valid) return MF_ERR_BAD_ARG;
  if (U->ncomp != c->nc) return MF_ERR_BAD_ARG;
  for (int d = c->p.space_dim; d < 3; ++d)
    if (valid->lo[d] != 0 || valid->hi[d] != 0 || U->box.lo[d] != 0 || U->box.hi[d] != 0)
      return MF_ERR_BAD_ARG;
  if (box_empty(*valid)) return MF_ERR_BAD_ARG;
  // the patch lies inside the problem domain in every non-periodic direction
  for (int d = 0; d < c->p.space_dim; ++d)
    if (!c->p.periodic[d] &&
        (valid->lo[d] < c->p.domain_lo[d] || valid->hi[d] > c->p.domain_hi[d]))
      return MF_ERR_BAD_ARG;
  mf_box need = box_grow(*valid, c->ng, c->p.space_dim);
  if (!box_contains(U->box, need)) return MF_ERR_BAD_ARG;
  if (box_cells(U->box) * c->nc >= (1LL << 31)) return MF_ERR_BAD_ARG;
  return MF_OK;
}

static void fill_desc(StageDesc& D, const mf_box& fab, const mf_box& vbox, const mf_box& wbox) {
  std::memset(&D, 0, sizeof(D));
  for (int d = 0; d < 3; ++d) {
    D.flo[d] = fab.lo[d];
    D.fn[d] = fab.hi[d] - fab.lo[d] + 1;
    D.vlo[d] = vbox.lo[d];
    D.vn[d] = vbox.hi[d] - vbox.lo[d] + 1;
    D.wlo[d] = wbox.lo[d];
    D.wn[d] = wbox.hi[d] - wbox.lo[d] + 1;
  }
}

// Hancock slope box of a desc and its face-value offsets (fv_off: doubles
// from the start of each direction's face-value array; null = 0).
static void set_slope(StageDesc& D, const mf_box& sb, const long long* fv_off) {
  for (int d = 0; d < 3; ++d) {
    D.slo[d] = sb.lo[d];
    D.sn[d] = sb.hi[d] - sb.lo[d] + 1;
    D.fv_off[d] = fv_off ? fv_off[d] : 0;
  }
}

// A batch of one patch: g0 = 0 in the host desc, device desc at dd.  The
// fab-size check of check_fab keeps every count inside a 32-bit index.
static mf::Batch single_batch(StageDesc& hd, const StageDesc* dd, int sd, const RunParams* runs) {
  mf::Batch b;
  std::memset(&b, 0, sizeof(b));
  mf::batch_offsets(&hd, 1, sd, b);
  b.desc = dd;
  b.runs = runs;
  b.nruns = 1;
  mf::batch_default_threads(b);
  return b;
}

// Descriptor block of a single-patch call (host copy and device copy): the
// descs of the two stages and the run's parameters, uploaded together.
struct SingleBlock {
  StageDesc d[2];
  RunParams r;
};

static void single_run(const mf_ctx* c, const mf::Batch& last, RunParams& r) {
  r = mf::run_params_of(c->dp);
  r.d0 = 0;
  r.nd = 1;
  r.v0 = 0;
  r.v1 = last.tot_v;
}

// Edge fabs of an EdgeBox on box (3 in 3D, 1 nodal in 2D) that contain it.
static bool edges_ok(const mf_fab* E, const mf_box& box, int sd) {
  const int nd = (sd == 3) ? 3 : 1;
  for (int d = 0; d < nd; ++d) {
    mf_box b = box;
    for (int e = 0; e < sd; ++e) b.hi[e] += (sd == 3 && e == d) ? 0 : 1;
    if (!E[d].data || E[d].ncomp != 1 || !box_contains(E[d].box, b)) return false;
  }
  return true;
}

static mf_status patch_update_impl(mf_ctx* c, mf_fab* U, const mf_box* valid, double dt,
                                   mf_fab* F, mf_fab* divB, mf_fab* E, double* new_dt,
                                   int min_cell[3], void* stream);

mf_status mf_patch_update(mf_ctx* c, mf_fab* U, const mf_box* valid, double dt, mf_fab* F,
                          mf_fab* divB, double* new_dt, int min_cell[3], void* stream) {
  return patch_update_impl(c, U, valid, dt, F, divB, nullptr, new_dt, min_cell, stream);
}

mf_status mf_patch_update_e(mf_ctx* c, mf_fab* U, const mf_box* valid, double dt, mf_fab* F,
                            mf_fab* divB, mf_fab* E, double* new_dt, int min_cell[3],
                            void* stream) {
  return patch_update_impl(c, U, valid, dt, F, divB, E, new_dt, min_cell, stream);
}

mf_status mf_recalculate_magnetic_field(mf_ctx* c, mf_fab* U, const mf_fab* Uold,
                                        const mf_fab* E, double dt, const mf_box* box,
                                        void* stream) {
  if (!c || !U || !U->data || !Uold || !Uold->data || !E || !box) return MF_ERR_BAD_ARG;
  if (!c->dp.ct) return MF_ERR_BAD_ARG;
  const int sd = c->p.space_dim;
  if (U->ncomp != c->nc || Uold->ncomp < 8 || !box_contains(U->box, *box) ||
      !box_contains(Uold->box, *box) || !edges_ok(E, *box, sd) || !std::isfinite(dt))
    return MF_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  MF_CHECK_CUDA(mf::launch_recalc_ext(sd, c->p.dx, U, Uold, E, dt, *box, s));
  return wait_stream(s, c->timeout);
}

static mf_status patch_update_impl(mf_ctx* c, mf_fab* U, const mf_box* valid, double dt,
                                   mf_fab* F, mf_fab* divB, mf_fab* E, double* new_dt,
                                   int min_cell[3], void* stream) {
  if (!c) return MF_ERR_BAD_ARG;
  mf_status st = check_fab(c, U, valid);
  if (st != MF_OK) return st;
  if (!(dt > 0.0) || !std::isfinite(dt)) return MF_ERR_BAD_ARG;
  const mf_params& p = c->p;
  const int sd = p.space_dim, nc = c->nc;
  const int mixed = (p.precision == MF_PREC_MIXED);
  const size_t rs = mixed ? sizeof(float) : sizeof(double);
  const bool rk2 = (p.time_approximation == MF_TA_RK2);
  const bool hk = (p.time_approximation == MF_TA_HANCOCK);
  cudaStream_t s = (cudaStream_t)stream;
  const long long fabn = box_cells(U->box);

  // stage-1 box: RK2 predictor on box.grow(2), Hancock predictor on box.grow(1)
  mf_box v2 = box_and_domain(*valid, p);
  mf_box v1 = rk2 ? box_and_domain(box_grow(*valid, 2, sd), p)
                  : hk ? box_and_domain(box_grow(*valid, 1, sd), p) : v2;
  mf_box w1 = box_isect(box_grow(v1, 2, sd), U->box);
  mf_box w2 = box_isect(box_grow(v2, 2, sd), U->box);
  if (divB && divB->data && !box_contains(divB->box, v2)) return MF_ERR_BAD_ARG;
  if (F) {
    for (int d = 0; d < sd; ++d)
      if (!F[d].data || F[d].ncomp != nc || !box_contains(F[d].box, box_nodes(v2, d)))
        return MF_ERR_BAD_ARG;
  }
  const bool ct = c->dp.ct != 0;
  if (E && ct && !edges_ok(E, *valid, sd)) return MF_ERR_BAD_ARG;

  MF_CHECK_CUDA(c->w.ensure(sizeof(double) * fabn * nc));
  if (mixed) MF_CHECK_CUDA(c->wf.ensure(sizeof(float) * fabn * nc));
  if (ct) {
    MF_CHECK_CUDA(c->ct_e1.ensure(sizeof(double) * fabn * 3));
    MF_CHECK_CUDA(c->ct_e2.ensure(sizeof(double) * fabn * 3));
    if (rk2) {
      MF_CHECK_CUDA(c->ct_u0.ensure(sizeof(double) * fabn * nc));
      MF_CHECK_CUDA(c->ct_eo.ensure(sizeof(double) * fabn * 3));
    }
  }
  if (rk2) MF_CHECK_CUDA(c->pred.ensure(sizeof(double) * fabn * nc));
  const mf_box s1 = box_grow(v1, 1, sd);  // Hancock slope box
  if (hk) {
    MF_CHECK_CUDA(c->w2.ensure(sizeof(double) * fabn * nc));
    for (int d = 0; d < sd; ++d)
      MF_CHECK_CUDA(c->fv[d].ensure(sizeof(double) * box_cells(s1) * 2 * nc));
  }
  for (int d = 0; d < sd; ++d) {
    MF_CHECK_CUDA(c->f1[d].ensure(rs * box_cells(box_nodes(v1, d)) * nc));
    MF_CHECK_CUDA(c->bn1[d].ensure(rs * box_cells(box_nodes(v1, d))));
    if (rk2) {
      MF_CHECK_CUDA(c->f2[d].ensure(rs * box_cells(box_nodes(v2, d)) * nc));
      MF_CHECK_CUDA(c->bn2[d].ensure(rs * box_cells(box_nodes(v2, d))));
    }
  }
  MF_CHECK_CUDA(c->desc.ensure(sizeof(SingleBlock)));
  MF_CHECK_CUDA(c->hdesc.ensure(sizeof(SingleBlock)));
  MF_CHECK_CUDA(c->state.ensure(sizeof(StepState)));
  MF_CHECK_CUDA(c->hstate.ensure(sizeof(StepState)));
  const long long vmax = box_cells(v2);
  const long long nparts = (vmax + 127) / 128 + 1;
  MF_CHECK_CUDA(c->partials.ensure(sizeof(DtPartial) * nparts));

  SingleBlock* hb = (SingleBlock*)c->hdesc.p;
  SingleBlock* db = (SingleBlock*)c->desc.p;
  StageDesc* hd = hb->d;
  fill_desc(hd[0], U->box, v1, w1);
  fill_desc(hd[1], U->box, v2, w2);
  if (hk)
    for (int e = 0; e < 2; ++e) set_slope(hd[e], s1, nullptr);
  StageDesc* dd = db->d;
  mf::Batch b1 = single_batch(hd[0], dd, sd, &db->r);
  mf::Batch b2 = single_batch(hd[1], dd + 1, sd, &db->r);
  single_run(c, b2, hb->r);
  StepState* hs = (StepState*)c->hstate.p;
  std::memset(hs, 0, sizeof(*hs));
  hs->dt = dt;
  hs->time = c->time;
  hs->ch = p.dedner_ch;
  hs->cp = p.dedner_cp;
  hs->cfl = 0.0;
  StepState* ds = (StepState*)c->state.p;
  MF_CHECK_CUDA(cudaMemcpyAsync(db, hb, sizeof(SingleBlock), cudaMemcpyHostToDevice, s));
  MF_CHECK_CUDA(cudaMemcpyAsync(ds, hs, sizeof(StepState), cudaMemcpyHostToDevice, s));

  int nb = 0;
  DtPartial* parts = (DtPartial*)c->partials.p;
  StageBuffers B;
  std::memset(&B, 0, sizeof(B));
  B.w = (double*)c->w.p;
  B.wf = mixed ? (float*)c->wf.p : nullptr;
  // constrained transport (src/PatchMHDAM.cpp:684-698, 1150-1160): after each
  // stage's update, the edge field of its fluxes and B from the stage-start
  // field; the dt then follows the last recalculation
  double* e1 = (double*)c->ct_e1.p;
  double* e2 = (double*)c->ct_e2.p;
  if (rk2) {
    MF_CHECK_CUDA(cudaMemcpyAsync(c->pred.p, U->data, sizeof(double) * fabn * nc,
                                  cudaMemcpyDeviceToDevice, s));
    if (ct)
      MF_CHECK_CUDA(cudaMemcpyAsync(c->ct_u0.p, U->data, sizeof(double) * fabn * nc,
                                    cudaMemcpyDeviceToDevice, s));
    B.uin = U->data;
    B.uout = (double*)c->pred.p;
    for (int d = 0; d < 3; ++d) {
      B.f[d] = c->f1[d].p;
      B.bn[d] = c->bn1[d].p;
    }
    MF_CHECK_CUDA(mf::launch_stage(c->dp, p.precision, B, b1, 0, 1.0, ds, parts, &nb, s));
    if (ct) {
      MF_CHECK_CUDA(mf::launch_efield(c->dp, mixed, B.f, B.w, e1, nullptr, nullptr, b1, s));
      MF_CHECK_CUDA(
          mf::launch_recalc_b(c->dp, B.uout, B.w, e1, nullptr, nullptr, ds, 1.0, 1, b1, s));
    }
    B.uin = (double*)c->pred.p;
    B.uout = U->data;
    B.uold = U->data;
    for (int d = 0; d < 3; ++d) {
      B.f[d] = c->f2[d].p;
      B.bn[d] = c->bn2[d].p;
    }
    if (divB && divB->data) {
      B.divb = divB->data;
      for (int d = 0; d < 3; ++d) {
        B.divb_lo[d] = divB->box.lo[d];
        B.divb_n[d] = divB->box.hi[d] - divB->box.lo[d] + 1;
      }
    }
    MF_CHECK_CUDA(mf::launch_stage(c->dp, p.precision, B, b2,
                                   ct ? 0 : (mf::kStageAverage | mf::kStageDt), 0.5, ds, parts,
                                   &nb, s));
    if (ct) {
      MF_CHECK_CUDA(mf::launch_efield(c->dp, mixed, B.f, B.w, e2, e1, (double*)c->ct_eo.p, b2,
                                      s));
      MF_CHECK_CUDA(mf::launch_recalc_b(c->dp, U->data, B.w, e2, (const double*)c->ct_u0.p,
                                        (const double*)c->pred.p, ds, 0.5, 1, b2, s));
      MF_CHECK_CUDA(mf::launch_dt(c->dp, U->data, b2, parts, &nb, s));
    }
  } else if (hk) {
    B.uin = U->data;
    B.uout = U->data;
    for (int d = 0; d < 3; ++d) {
      B.f[d] = c->f1[d].p;
      B.bn[d] = c->bn1[d].p;
    }
    if (divB && divB->data) {
      B.divb = divB->data;
      for (int d = 0; d < 3; ++d) {
        B.divb_lo[d] = divB->box.lo[d];
        B.divb_n[d] = divB->box.hi[d] - divB->box.lo[d] + 1;
      }
    }
    mf::HancockBuffers H;
    for (int d = 0; d < 3; ++d) H.fv[d] = (double*)c->fv[d].p;
    H.w2 = (double*)c->w2.p;
    MF_CHECK_CUDA(mf::launch_hancock(c->dp, p.precision, B, H, b1, b2, ds, parts, &nb, s,
                                     ct ? 0 : mf::kStageDt));
    if (ct) {  // the corrector's field: W(t+dt/2) for the edges, B from W(t)
      MF_CHECK_CUDA(mf::launch_efield(c->dp, mixed, B.f, H.w2, e2, nullptr, nullptr, b2, s));
      MF_CHECK_CUDA(
          mf::launch_recalc_b(c->dp, U->data, B.w, e2, nullptr, nullptr, ds, 1.0, 1, b2, s));
      MF_CHECK_CUDA(mf::launch_dt(c->dp, U->data, b2, parts, &nb, s));
    }
  } else {
    B.uin = U->data;
    B.uout = U->data;
    for (int d = 0; d < 3; ++d) {
      B.f[d] = c->f1[d].p;
      B.bn[d] = c->bn1[d].p;
    }
    if (divB && divB->data) {
      B.divb = divB->data;
      for (int d = 0; d < 3; ++d) {
        B.divb_lo[d] = divB->box.lo[d];
        B.divb_n[d] = divB->box.hi[d] - divB->box.lo[d] + 1;
      }
    }
    MF_CHECK_CUDA(mf::launch_stage(c->dp, p.precision, B, b2, ct ? 0 : mf::kStageDt, 1.0, ds,
                                   parts, &nb, s));
    if (ct) {
      MF_CHECK_CUDA(mf::launch_efield(c->dp, mixed, B.f, B.w, e2, nullptr, nullptr, b2, s));
      MF_CHECK_CUDA(
          mf::launch_recalc_b(c->dp, U->data, B.w, e2, nullptr, nullptr, ds, 1.0, 1, b2, s));
      MF_CHECK_CUDA(mf::launch_dt(c->dp, U->data, b2, parts, &nb, s));
    }
  }
  MF_CHECK_CUDA(mf::launch_finalize(c->dp, parts, b2, b2.nt[2], ds, 0, s));
  if (ct && E)  // updateState's E: the step average (RK2) or the one stage's field
    MF_CHECK_CUDA(
        mf::launch_edges_out(sd, rk2 ? (const double*)c->ct_eo.p : e2, U->box, *valid, E, s));
  if (F) {
    const void* f2p[3] = {nullptr, nullptr, nullptr};
    const void* f1p[3] = {nullptr, nullptr, nullptr};
    double* fo[3] = {nullptr, nullptr, nullptr};
    int f2lo[3][3], f2n[3][3], f1lo[3][3], f1n[3][3], olo[3][3], on[3][3];
    std::memset(f2lo, 0, sizeof(f2lo));
    std::memset(f2n, 0, sizeof(f2n));
    std::memset(f1lo, 0, sizeof(f1lo));
    std::memset(f1n, 0, sizeof(f1n));
    std::memset(olo, 0, sizeof(olo));
    std::memset(on, 0, sizeof(on));
    for (int d = 0; d < sd; ++d) {
      mf_box b2 = box_nodes(v2, d), b1 = box_nodes(v1, d);
      f2p[d] = rk2 ? c->f2[d].p : c->f1[d].p;
      f1p[d] = rk2 ? c->f1[d].p : nullptr;
      fo[d] = F[d].data;
      for (int e = 0; e < 3; ++e) {
        f2lo[d][e] = b2.lo[e];
        f2n[d][e] = b2.hi[e] - b2.lo[e] + 1;
        f1lo[d][e] = b1.lo[e];
        f1n[d][e] = b1.hi[e] - b1.lo[e] + 1;
        olo[d][e] = b2.lo[e];
        on[d][e] = b2.hi[e] - b2.lo[e] + 1;
      }
      // the output fab may be larger than the faces of the valid box
      if (!(F[d].box.lo[0] == b2.lo[0] && F[d].box.lo[1] == b2.lo[1] &&
            F[d].box.lo[2] == b2.lo[2] && F[d].box.hi[0] == b2.hi[0] &&
            F[d].box.hi[1] == b2.hi[1] && F[d].box.hi[2] == b2.hi[2]))
        return MF_ERR_BAD_ARG;
    }
    MF_CHECK_CUDA(mf::launch_flux_out(mixed, sd, nc, f2p, f2lo, f2n, f1p, f1lo, f1n, fo, olo, on,
                                      s));
  }
  MF_CHECK_CUDA(cudaMemcpyAsync(hs, ds, sizeof(StepState), cudaMemcpyDeviceToHost, s));
  st = wait_stream(s, c->timeout);
  if (st != MF_OK) return st;
  if (new_dt) *new_dt = hs->dt_min;
  if (min_cell) {
    int n[3];
    ext3(*valid, n);
    int idx = hs->min_idx;
    if (idx < 0 || idx == 0x7fffffff) idx = 0;
    min_cell[0] = valid->lo[0] + idx % n[0];
    min_cell[1] = valid->lo[1] + (idx / n[0]) % n[1];
    min_cell[2] = valid->lo[2] + idx / (n[0] * n[1]);
  }
  return flags_status(hs->flags);
}

mf_status mf_face_fluxes(mf_ctx* c, int dir, int n, const double* wl, const double* wr,
                         double* f, void* stream) {
  if (!c || n < 0 || !wl || !wr || !f || dir < 0 || dir >= c->p.space_dim) return MF_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const double ch = c->p.dedner_ch;
  if (c->p.precision == MF_PREC_MIXED)
    MF_CHECK_CUDA(mf::launch_face_flux_fast<float>(c->dp, dir, wl, wr, f, n, ch, s));
  else if (c->p.precision == MF_PREC_FP64_FAST)
    MF_CHECK_CUDA(mf::launch_face_flux_fast<double>(c->dp, dir, wl, wr, f, n, ch, s));
  else
    MF_CHECK_CUDA(mf::launch_face_flux_exact(c->dp, dir, wl, wr, f, n, ch, s));
  return wait_stream(s, c->timeout);
}

mf_status mf_compute_dt(mf_ctx* c, const mf_fab* U, const mf_box* box, double* dt,
                        int min_cell[3], void* stream) {
  if (!c || !U || !U->data || !box || box_empty(*box) || !box_contains(U->box, *box))
    return MF_ERR_BAD_ARG;
  if (U->ncomp != c->nc) return MF_ERR_BAD_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  const long long nv = box_cells(*box);
  if (nv >= (1LL << 31) - 1024) return MF_ERR_BAD_ARG;
  MF_CHECK_CUDA(c->desc.ensure(sizeof(SingleBlock)));
  MF_CHECK_CUDA(c->hdesc.ensure(sizeof(SingleBlock)));
  MF_CHECK_CUDA(c->state.ensure(sizeof(StepState)));
  MF_CHECK_CUDA(c->hstate.ensure(sizeof(StepState)));
  MF_CHECK_CUDA(c->partials.ensure(sizeof(DtPartial) * ((nv + 127) / 128 + 1)));
  SingleBlock* hb = (SingleBlock*)c->hdesc.p;
  SingleBlock* db = (SingleBlock*)c->desc.p;
  StageDesc* hd = hb->d;
  fill_desc(hd[0], U->box, *box, *box);
  mf::Batch b = single_batch(hd[0], db->d, c->p.space_dim, &db->r);
  single_run(c, b, hb->r);
  StepState* hs = (StepState*)c->hstate.p;
  std::memset(hs, 0, sizeof(*hs));
  StepState* ds = (StepState*)c->state.p;
  DtPartial* parts = (DtPartial*)c->partials.p;
  MF_CHECK_CUDA(cudaMemcpyAsync(db, hb, sizeof(SingleBlock), cudaMemcpyHostToDevice, s));
  MF_CHECK_CUDA(cudaMemcpyAsync(ds, hs, sizeof(StepState), cudaMemcpyHostToDevice, s));
  int nb = 0;
  MF_CHECK_CUDA(mf::launch_dt(c->dp, U->data, b, parts, &nb, s));
  MF_CHECK_CUDA(mf::launch_finalize(c->dp, parts, b, b.nt[2], ds, 0, s));
  MF_CHECK_CUDA(cudaMemcpyAsync(hs, ds, sizeof(StepState), cudaMemcpyDeviceToHost, s));
  mf_status st = wait_stream(s, c->timeout);
  if (st != MF_OK) return st;
  if (dt) *dt = hs->dt_min;
  if (min_cell) {
    int n[3];
    ext3(*box, n);
    int idx = hs->min_idx;
    if (idx < 0 || idx == 0x7fffffff) idx = 0;
    min_cell[0] = box->lo[0] + idx % n[0];
    min_cell[1] = box->lo[1] + (idx / n[0]) % n[1];
    min_cell[2] = box->lo[2] + idx / (n[0] * n[1]);
  }
  return flags_status(hs->flags);
}

// ---------------------------------------------------------------------------
// level
// ---------------------------------------------------------------------------

}  // extern "C"

// Uniform bucket grid over the valid boxes of a level, so that finding the
// patches that meet a box costs the buckets it spans instead of a pass over
// every patch (a level can hold thousands of patches).
struct PatchIndex {
  int nb[3] = {1, 1, 1}, bs[3] = {1, 1, 1}, lo[3] = {0, 0, 0};
  std::vector<std::vector<int>> bucket;
  std::vector<int> stamp;
  int tick = 0;

  void build(const std::vector<mf_box>& v, const mf_params& p) {
    const int sd = p.space_dim;
    for (int d = 0; d < 3; ++d) {
      lo[d] = (d < sd) ? p.domain_lo[d] : 0;
      bs[d] = 1;
      nb[d] = 1;
    }
    for (const mf_box& b : v)
      for (int d = 0; d < sd; ++d) bs[d] = std::max(bs[d], b.hi[d] - b.lo[d] + 1);
    for (int d = 0; d < sd; ++d)
      nb[d] = std::max(1, (p.domain_hi[d] - p.domain_lo[d] + bs[d]) / bs[d]);
    bucket.assign((size_t)nb[0] * nb[1] * nb[2], std::vector<int>());
    stamp.assign(v.size(), 0);
    for (int i = 0; i < (int)v.size(); ++i) {
      int b0[3], b1[3];
      if (!range(v[i], b0, b1)) continue;
      for (int z = b0[2]; z <= b1[2]; ++z)
        for (int y = b0[1]; y <= b1[1]; ++y)
          for (int x = b0[0]; x <= b1[0]; ++x)
            bucket[((size_t)z * nb[1] + y) * nb[0] + x].push_back(i);
    }
  }
  bool range(const mf_box& q, int b0[3], int b1[3]) const {
    for (int d = 0; d < 3; ++d) {
      b0[d] = std::max(0, floordiv(q.lo[d] - lo[d], bs[d]));
      b1[d] = std::min(nb[d] - 1, floordiv(q.hi[d] - lo[d], bs[d]));
      if (b0[d] > b1[d]) return false;
    }
    return true;
  }
  static int floordiv(int a, int b) { return (a >= 0) ? a / b : -((-a + b - 1) / b); }
  // f(i) once for every patch i whose buckets meet q (a superset of the
  // patches whose valid box meets q).
  template <class Fn>
  void query(const mf_box& q, Fn&& f) {
    int b0[3], b1[3];
    if (!range(q, b0, b1)) return;
    ++tick;
    for (int z = b0[2]; z <= b1[2]; ++z)
      for (int y = b0[1]; y <= b1[1]; ++y)
        for (int x = b0[0]; x <= b1[0]; ++x)
          for (int i : bucket[((size_t)z * nb[1] + y) * nb[0] + x])
            if (stamp[i] != tick) {
              stamp[i] = tick;
              f(i);
            }
  }
};

// Periodic image shifts (in cells) of a level's domain: 3^np vectors, np the
// number of periodic directions; the zero shift first.
static std::vector<std::array<int, 3>> periodic_shifts(const mf_params& p) {
  const int sd = p.space_dim;
  int Lp[3] = {0, 0, 0}, rng[3] = {0, 0, 0};
  for (int d = 0; d < sd; ++d) {
    Lp[d] = p.domain_hi[d] - p.domain_lo[d] + 1;
    rng[d] = p.periodic[d] ? 1 : 0;
  }
  std::vector<std::array<int, 3>> out;
  out.push_back({0, 0, 0});
  for (int a = -rng[0]; a <= rng[0]; ++a)
    for (int b = -rng[1]; b <= rng[1]; ++b)
      for (int e = -rng[2]; e <= rng[2]; ++e)
        if (a || b || e) out.push_back({a * Lp[0], b * Lp[1], e * Lp[2]});
  return out;
}

static mf_box box_shift(mf_box b, const std::array<int, 3>& sh) {
  for (int d = 0; d < 3; ++d) {
    b.lo[d] += sh[d];
    b.hi[d] += sh[d];
  }
  return b;
}

// Copy regions of LevelData::exchange: the cells of valid.grow(depth) of each
// patch that lie in another patch's valid box or in a periodic image of one.
static void add_regions(const mf::LevelPlan& L, const mf_params& p, PatchIndex& ix, int depth,
                        std::vector<CopyReg>& out) {
  const int sd = p.space_dim;
  const auto shifts = periodic_shifts(p);
  for (int dp = 0; dp < L.np; ++dp) {
    const mf_box dst = box_grow(L.valid[dp], depth, sd);
    int dfn[3];
    ext3(L.fab[dp], dfn);
    for (size_t k = 0; k < shifts.size(); ++k) {
      const auto& sh = shifts[k];
      const std::array<int, 3> msh = {-sh[0], -sh[1], -sh[2]};
      ix.query(box_shift(dst, msh), [&](int sp) {
        if (sp == dp && k == 0) return;
        const mf_box r = box_isect(box_shift(L.valid[sp], sh), dst);
        if (box_empty(r)) return;
        int sfn[3];
        ext3(L.fab[sp], sfn);
        CopyReg R;
        R.src_off = L.off[sp];
        R.dst_off = L.off[dp];
        for (int d = 0; d < 3; ++d) {
          R.sfn[d] = sfn[d];
          R.dfn[d] = dfn[d];
          R.s0[d] = r.lo[d] - sh[d] - L.fab[sp].lo[d];
          R.d0[d] = r.lo[d] - L.fab[dp].lo[d];
          R.ext[d] = r.hi[d] - r.lo[d] + 1;
        }
        out.push_back(R);
      });
    }
  }
}

// valueBox of RK2 stage 1 for patch i.  Stage 2 needs the predictor on the
// two ghost layers next to each face of the valid box (the face-normal
// stencil of the fluxes on the valid faces).  Where sibling patches (or their
// periodic images) cover such a slab, the exchange between the stages copies
// it; where they do not (a coarse-fine edge of a level that does not cover
// the domain), stage 1 computes it, as the reference does by running stage 1
// on box.grow(2) (src/PatchMHDAM.cpp:1238-1246).  Cells outside a
// non-periodic domain side are never computed (ProblemDomain clipping).
static bool ct_on(const mf_params& p) { return p.divb_cleaning >= 1 && p.divb_cleaning <= 3; }

static mf_box stage1_box(const mf::LevelPlan& L, const mf_params& p, PatchIndex& ix, int i) {
  const int sd = p.space_dim;
  const mf_box& v = L.valid[i];
  // Constrained transport: a stage's edge field is one-sided on its valueBox
  // boundary, so a stage-1 ghost value depends on the patch that computes it;
  // every patch runs stage 1 on box.grow(2), as the reference does, and no
  // exchange follows.
  if (ct_on(p)) return box_and_domain(box_grow(v, 2, sd), p);
  const auto shifts = periodic_shifts(p);
  mf_box g = v;
  for (int d = 0; d < sd; ++d)
    for (int side = 0; side < 2; ++side) {
      mf_box slab = v;
      if (side == 0) {
        slab.lo[d] = v.lo[d] - 2;
        slab.hi[d] = v.lo[d] - 1;
      } else {
        slab.lo[d] = v.hi[d] + 1;
        slab.hi[d] = v.hi[d] + 2;
      }
      slab = box_and_domain(slab, p);
      if (box_empty(slab)) continue;
      long long covered = 0;
      for (const auto& sh : shifts) {
        const std::array<int, 3> msh = {-sh[0], -sh[1], -sh[2]};
        ix.query(box_shift(slab, msh), [&](int j) {
          const mf_box r = box_isect(box_shift(L.valid[j], sh), slab);
          if (!box_empty(r)) covered += box_cells(r);
        });
      }
      if (covered < box_cells(slab)) {
        if (side == 0)
          g.lo[d] -= 2;
        else
          g.hi[d] += 2;
      }
    }
  return box_and_domain(g, p);
}

namespace mf {

mf_status build_level_plan(const mf_params& p, int ng, int nc, int npatch, const mf_box* valid,
                           LevelPlan& L) {
  if (!valid || npatch <= 0) return MF_ERR_BAD_ARG;
  const int sd = p.space_dim;
  for (int d = 0; d < sd; ++d)
    if (!p.periodic[d] && p.bc_kind != MF_BC_FARFIELD) return MF_ERR_UNSUPPORTED;
  L = LevelPlan();
  L.np = npatch;
  L.valid.assign(valid, valid + npatch);
  L.fab.resize(npatch);
  L.off.resize(npatch);
  mf_box dom;
  for (int d = 0; d < 3; ++d) {
    dom.lo[d] = p.domain_lo[d];
    dom.hi[d] = p.domain_hi[d];
  }
  long long off = 0;
  for (int i = 0; i < npatch; ++i) {
    const mf_box& v = valid[i];
    bool bad = box_empty(v) || !box_contains(dom, v);
    for (int d = sd; d < 3; ++d)
      if (v.lo[d] != 0 || v.hi[d] != 0) bad = true;
    if (bad) return MF_ERR_BAD_ARG;
    L.fab[i] = box_grow(v, ng, sd);
    L.off[i] = off;
    off += ((box_cells(L.fab[i]) * nc + 31) / 32) * 32;  // 256-byte aligned fabs
    L.cells += box_cells(v);
  }
  L.total = off;
  PatchIndex ix;
  ix.build(L.valid, p);
  // valid boxes must not overlap
  for (int i = 0; i < npatch; ++i) {
    bool overlap = false;
    ix.query(valid[i], [&](int j) {
      if (j != i && !box_empty(box_isect(valid[i], valid[j]))) overlap = true;
    });
    if (overlap) return MF_ERR_BAD_ARG;
  }
  const bool rk2 = (p.time_approximation == MF_TA_RK2);
  const bool hk = (p.time_approximation == MF_TA_HANCOCK);
  // descs of both stages; face fluxes and Bn of one stage at a time, each
  // patch's face fab 64-element aligned.  Hancock: stage 0 is the predictor
  // on valid.grow(1) & domain (as predictorHancock), stage 1 the corrector.
  L.d1.resize(npatch);
  L.d2.resize(npatch);
  long long fvo = 0;
  for (int stg = 0; stg < 2; ++stg) {
    long long foff[3] = {0, 0, 0}, boff[3] = {0, 0, 0};
    for (int i = 0; i < npatch; ++i) {
      StageDesc& D = (stg == 0) ? L.d1[i] : L.d2[i];
      const mf_box vb = (stg == 0 && rk2)  ? stage1_box(L, p, ix, i)
                        : (stg == 0 && hk) ? box_and_domain(box_grow(valid[i], 1, sd), p)
                                           : valid[i];
      fill_desc(D, L.fab[i], vb, box_isect(box_grow(vb, 2, sd), L.fab[i]));
      if (hk) {
        if (stg == 0) {
          const mf_box sb = box_grow(vb, 1, sd);
          const long long o3[3] = {fvo, fvo, fvo};
          set_slope(D, sb, o3);
          fvo += ((box_cells(sb) * 2 * nc + 31) / 32) * 32;
        } else {
          const StageDesc& A = L.d1[i];
          for (int d = 0; d < 3; ++d) {
            D.slo[d] = A.slo[d];
            D.sn[d] = A.sn[d];
            D.fv_off[d] = A.fv_off[d];
          }
        }
      }
      D.u_off = L.off[i];
      for (int d = 0; d < sd; ++d) {
        const long long nf = box_cells(box_nodes(vb, d));
        D.f_off[d] = foff[d];
        D.bn_off[d] = boff[d];
        foff[d] += ((nf * nc + 63) / 64) * 64;
        boff[d] += ((nf + 63) / 64) * 64;
      }
    }
    for (int d = 0; d < 3; ++d) {
      L.fsize[d] = std::max(L.fsize[d], foff[d]);
      L.bsize[d] = std::max(L.bsize[d], boff[d]);
    }
  }
  L.fvsize = fvo;
  add_regions(L, p, ix, ng, L.full);
  const bool lean_scheme = (rk2 || p.time_approximation == MF_TA_FIRST_ORDER) && !ct_on(p);
  if (lean_scheme) add_regions(L, p, ix, 2, L.two);
  if (lean_scheme) {
    // the lean primitive part: stage 1 on the valid boxes, and the sibling
    // copies cover every in-domain ghost cell of each valid.grow(2)
    std::vector<long long> cov(npatch, 0);
    std::unordered_map<long long, int> by_off;
    for (int i = 0; i < npatch; ++i) by_off[L.off[i]] = i;
    for (const CopyReg& R : L.two) cov[by_off[R.dst_off]] += (long long)R.ext[0] * R.ext[1] * R.ext[2];
    bool lean = true;
    for (int i = 0; i < npatch && lean; ++i) {
      const StageDesc& A = L.d1[i];
      for (int d = 0; d < 3; ++d)
        if (A.vlo[d] != valid[i].lo[d] || A.vn[d] != valid[i].hi[d] - valid[i].lo[d] + 1)
          lean = false;
      const mf_box wb = box_and_domain(box_grow(valid[i], 2, sd), p);
      if (cov[i] != box_cells(wb) - box_cells(valid[i])) lean = false;
    }
    L.lean = lean;
    if (lean) {
      L.dp = L.d2;
      for (int i = 0; i < npatch; ++i) {
        StageDesc& D = L.dp[i];
        for (int d = 0; d < 3; ++d) {
          D.wlo[d] = valid[i].lo[d];
          D.wn[d] = valid[i].hi[d] - valid[i].lo[d] + 1;
        }
        // far-field ghosts of valid.grow(2): slabs peeled off the box one
        // non-periodic direction at a time
        mf_box rest = box_grow(valid[i], 2, sd);
        for (int d = 0; d < sd; ++d) {
          if (p.periodic[d]) continue;
          for (int side = 0; side < 2; ++side) {
            mf_box slab = rest;
            if (side == 0)
              slab.hi[d] = std::min(rest.hi[d], p.domain_lo[d] - 1);
            else
              slab.lo[d] = std::max(rest.lo[d], p.domain_hi[d] + 1);
            if (box_empty(slab)) continue;
            FarReg R;
            std::memset(&R, 0, sizeof(R));
            R.off = L.off[i];
            ext3(L.fab[i], R.fn);
            for (int e = 0; e < 3; ++e) {
              R.flo[e] = L.fab[i].lo[e];
              R.lo[e] = slab.lo[e];
              R.ext[e] = slab.hi[e] - slab.lo[e] + 1;
            }
            R.run = 0;
            L.far.push_back(R);
          }
          rest.lo[d] = std::max(rest.lo[d], p.domain_lo[d]);
          rest.hi[d] = std::min(rest.hi[d], p.domain_hi[d]);
        }
      }
    }
    if (!rk2 && !lean) L.two.clear();
  }
  if (p.neutral_sun_bc && p.n_fluids > 1 && sd == 3) {
    // HeliosphericProblem::define (swlism/HeliosphericProblem.cpp:476-527):
    // the sun on a grid node, strips of iR0 planes on either side of it
    int sun[3];
    for (int d = 0; d < 3; ++d) {
      sun[d] = (int)std::floor(p.sun_center[d] / p.dx + 0.5);
      if (std::fabs(sun[d] * p.dx - p.sun_center[d]) >= 1e-6) return MF_ERR_UNSUPPORTED;
    }
    const int iR0 = 1 + (int)std::floor(p.reinit_r0 / p.dx + 0.5);
    const double sunR2 = p.sun_r * p.sun_r;
    auto cell_of = [&](const int c[3], long long& off, int& cs) -> bool {
      mf_box q;
      for (int d = 0; d < 3; ++d) q.lo[d] = q.hi[d] = c[d];
      int found = -1;
      ix.query(q, [&](int b) {
        const mf_box& v = L.valid[b];
        if (c[0] >= v.lo[0] && c[0] <= v.hi[0] && c[1] >= v.lo[1] && c[1] <= v.hi[1] &&
            c[2] >= v.lo[2] && c[2] <= v.hi[2])
          found = b;
      });
      if (found < 0) return false;
      const mf_box& f = L.fab[found];
      const int n[3] = {f.hi[0] - f.lo[0] + 1, f.hi[1] - f.lo[1] + 1, f.hi[2] - f.lo[2] + 1};
      off = L.off[found] + (c[0] - f.lo[0]) +
            (long long)n[0] * ((c[1] - f.lo[1]) + (long long)n[1] * (c[2] - f.lo[2]));
      cs = n[0] * n[1] * n[2];
      return true;
    };
    for (int a = 0; a < iR0; ++a)
      for (int k = sun[2] - iR0 - 1; k <= sun[2] + iR0; ++k)
        for (int j = sun[1] - iR0 - 1; j <= sun[1] + iR0; ++j) {
          const int i = sun[0] + a;
          // NEUTRALS_SUNBC (swlism/SWLISMF.ChF:1555-1598)
          const double x = (i + 0.5) * p.dx - p.sun_center[0];
          const double y = (j + 0.5) * p.dx - p.sun_center[1];
          const double z = (k + 0.5) * p.dx - p.sun_center[2];
          const double r2 = x * x + y * y + z * z;
          if (!(r2 <= sunR2)) continue;
          const int to[3] = {i, j, k}, from[3] = {sun[0] - (i - sun[0] + 1), j, k};
          SunPair sp;
          if (cell_of(to, sp.to, sp.cs_to) && cell_of(from, sp.from, sp.cs_from))
            L.sun.push_back(sp);
        }
  }
  return MF_OK;
}

}  // namespace mf

extern "C" {

// ev (nullable): events recorded after every launch, in launch order, with
// kinds[] receiving 0 exchange, 1 prim, 2 flux, 3 update, 4 finalize.
static mf_status enqueue_level_step(mf_level* L, int advance, cudaEvent_t* ev = nullptr,
                                    int* kinds = nullptr, int* nev = nullptr) {
  mf_ctx* c = L->ctx;
  const mf_params& p = c->p;
  cudaStream_t s = L->s;
  StepState* ds = (StepState*)L->state.p;
  DtPartial* parts = (DtPartial*)L->partials.p;
  StageBuffers B;
  std::memset(&B, 0, sizeof(B));
  B.w = (double*)L->W.p;
  B.wf = (p.precision == MF_PREC_MIXED) ? (float*)L->Wf.p : nullptr;
  for (int d = 0; d < 3; ++d) {
    B.f[d] = L->F[d].p;
    B.bn[d] = L->Bn[d].p;
  }
  int nb = 0;
  const int nc = c->nc;
  const int sd = p.space_dim;
  int ne = 0;
  auto mark = [&](int kind) {
    if (!ev) return;
    cudaEventRecord(ev[ne], s);
    kinds[ne] = kind;
    ++ne;
  };
  const int mixed = (p.precision == MF_PREC_MIXED);
  // lean levels: the primitive part of each stage computes the valid cells
  // and copies the ghosts; the conserved state is not exchanged (no kernel
  // of the step reads its ghost cells then)
  const mf::LeanPrim* lean = L->lean ? &L->lp : nullptr;
  B.lean = lean;
  const int np0 = mf::prim_launches(lean, mixed);
  // the fused flux + update kernel, unless flux registers need the face fluxes
  const bool fused = L->fused && L->gathers.empty();
  // chunked flux / update overlap of the split mixed-precision stages
  const bool overlap = L->nchunks > 1 && !L->fused && L->gathers.empty() && !c->dp.ct;
  const bool lines = L->flux_form == MF_FLUX_LINES;
  auto stage_marks = [&](int n0) {
    if (!ev) return;
    kinds[n0] = 1;
    for (int q = 1; q < np0; ++q) kinds[n0 + q] = 0;
    if (fused) {
      kinds[n0 + np0] = 8;
      ne = n0 + np0 + 1;
      return;
    }
    if (overlap) {  // chunks + 1 launches of fluxes and updates
      for (int q = 0; q <= L->nchunks; ++q) kinds[n0 + np0 + q] = 9;
      ne = n0 + np0 + L->nchunks + 1;
      return;
    }
    for (int d = 0; d < sd; ++d) kinds[n0 + np0 + d] = 2;
    kinds[n0 + np0 + sd] = 3;
    ne = n0 + np0 + 1 + sd;
  };
  if (!lean) {
    MF_CHECK_CUDA(
        mf::launch_exchange((double*)L->U.p, (const CopyReg*)L->exfull.p, L->nfull, nc, s));
    if (L->nfull) mark(0);
  }
  // constrained transport (src/PatchMHDAM.cpp:684-698, 1150-1160): the level's
  // UOld (AMRLevelIdealMHD::preTimeStep), per stage the edge field of the
  // stage's fluxes and B from the stage-start field, the dt after the last
  // recalculation, and after the step B from UOld and the step's edge field
  // (AMRLevelIdealMHD::postTimeStep, srcIdeal/AMRLevelIdealMHD.cpp:1649-1688)
  const bool ct = c->dp.ct != 0;
  double* e1 = (double*)L->ct_e1.p;
  double* e2 = (double*)L->ct_e2.p;
  double* u0 = (double*)L->ct_u0.p;
  if (ct)
    MF_CHECK_CUDA(cudaMemcpyAsync(u0, L->U.p, sizeof(double) * L->total,
                                  cudaMemcpyDeviceToDevice, s));
  auto ct_stage = [&](const mf::Batch& b, const double* wedge, double* e, const double* ep,
                      double* eavg, double* u, const double* a0, const double* a1,
                      double scale) -> mf_status {
    MF_CHECK_CUDA(mf::launch_efield(c->dp, mixed, B.f, wedge, e, ep, eavg, b, s));
    mark(7);
    MF_CHECK_CUDA(mf::launch_recalc_b(c->dp, u, B.w, e, a0, a1, ds, scale, 1, b, s));
    mark(7);
    return MF_OK;
  };
  auto ct_dt = [&]() -> mf_status {
    MF_CHECK_CUDA(mf::launch_dt(c->dp, (const double*)L->U.p, L->b2, parts, &nb, s));
    mark(3);
    return MF_OK;
  };
  const void* fl[3] = {L->F[0].p, L->F[1].p, L->F[2].p};
  auto gather = [&](int mode) -> mf_status {
    for (const mf::FaceGather& g : L->gathers) {
      // fluid components only: the registers skip the tracking surfaces
      MF_CHECK_CUDA(mf::launch_face_gather(mixed, fl, g, mode, L->ctx->dp.ils, s));
      mark(5);
    }
    return MF_OK;
  };
  mf_status gst = MF_OK;
  if (p.time_approximation == MF_TA_RK2) {
    B.uin = (const double*)L->U.p;
    B.uout = (double*)L->U1.p;
    B.ev = ev ? ev + ne : nullptr;
    B.fused = fused ? &L->fp1 : nullptr;
    B.overlap = overlap ? &L->op1 : nullptr;
    B.lines = lines ? &L->lp1 : nullptr;
    MF_CHECK_CUDA(mf::launch_stage(c->dp, p.precision, B, L->b1, 0, 1.0, ds, parts, &nb, s));
    stage_marks(ne);
    if (ct && (gst = ct_stage(L->b1, B.w, e1, nullptr, nullptr, (double*)L->U1.p, nullptr,
                              nullptr, 1.0)) != MF_OK)
      return gst;
    if ((gst = gather(0)) != MF_OK) return gst;
    if (!lean) {
      MF_CHECK_CUDA(
          mf::launch_exchange((double*)L->U1.p, (const CopyReg*)L->extwo.p, L->ntwo, nc, s));
      if (L->ntwo) mark(0);
    }
    B.uin = (const double*)L->U1.p;
    B.uout = (double*)L->U.p;
    B.uold = (const double*)L->U.p;
    B.ev = ev ? ev + ne : nullptr;
    B.fused = fused ? &L->fp2 : nullptr;
    B.overlap = overlap ? &L->op2 : nullptr;
    B.lines = lines ? &L->lp2 : nullptr;
    MF_CHECK_CUDA(mf::launch_stage(c->dp, p.precision, B, L->b2,
                                   ct ? 0 : (mf::kStageAverage | mf::kStageDt), 0.5, ds, parts,
                                   &nb, s));
    stage_marks(ne);
    if (ct) {
      if ((gst = ct_stage(L->b2, B.w, e2, e1, (double*)L->ct_eo.p, (double*)L->U.p, u0,
                          (const double*)L->U1.p, 0.5)) != MF_OK)
        return gst;
      if ((gst = ct_dt()) != MF_OK) return gst;
    }
    if ((gst = gather(1)) != MF_OK) return gst;
  } else if (p.time_approximation == MF_TA_HANCOCK) {
    B.uin = (const double*)L->U.p;
    B.uout = (double*)L->U.p;
    B.ev = ev ? ev + ne : nullptr;
    mf::HancockBuffers H;
    for (int d = 0; d < 3; ++d) H.fv[d] = (double*)L->FV[d].p;
    H.w2 = (double*)L->U1.p;
    MF_CHECK_CUDA(mf::launch_hancock(c->dp, p.precision, B, H, L->b1, L->b2, ds, parts, &nb, s,
                                     ct ? 0 : mf::kStageDt));
    if (ev) {  // prim, faces, predictor, shift, fluxes, update
      const int k0[4] = {1, 1, 3, 1};
      for (int q = 0; q < 4; ++q) kinds[ne + q] = k0[q];
      for (int d = 0; d < sd; ++d) kinds[ne + 4 + d] = 2;
      kinds[ne + 4 + sd] = 3;
      ne += mf::hancock_launches(sd);
    }
    if (ct) {  // the corrector's edges from W(t+dt/2), B from W(t)
      if ((gst = ct_stage(L->b2, H.w2, e2, nullptr, nullptr, (double*)L->U.p, nullptr, nullptr,
                          1.0)) != MF_OK)
        return gst;
      if ((gst = ct_dt()) != MF_OK) return gst;
    }
    if ((gst = gather(2)) != MF_OK) return gst;
  } else {
    B.uin = (const double*)L->U.p;
    B.uout = (double*)L->U.p;
    B.ev = ev ? ev + ne : nullptr;
    B.fused = fused ? &L->fp2 : nullptr;
    B.overlap = overlap ? &L->op2 : nullptr;
    B.lines = lines ? &L->lp2 : nullptr;
    MF_CHECK_CUDA(mf::launch_stage(c->dp, p.precision, B, L->b2, ct ? 0 : mf::kStageDt, 1.0, ds,
                                   parts, &nb, s));
    stage_marks(ne);
    if (ct) {
      if ((gst = ct_stage(L->b2, B.w, e2, nullptr, nullptr, (double*)L->U.p, nullptr, nullptr,
                          1.0)) != MF_OK)
        return gst;
      if ((gst = ct_dt()) != MF_OK) return gst;
    }
    if ((gst = gather(2)) != MF_OK) return gst;
  }
  MF_CHECK_CUDA(mf::launch_finalize(c->dp, parts, L->b2, L->b2.nt[2], ds, advance, s,
                                    fused ? L->fp2.ntiles : 0));
  mark(4);
  // HeliosphericProblem::postTimeStep (swlism/HeliosphericProblem.cpp:2472-2535),
  // after the step and its dt (AMRLevelIdealMHD::advance)
  if (L->nsun) {
    MF_CHECK_CUDA(mf::launch_sun_copy((double*)L->U.p, (const mf::SunPair*)L->sun.p, L->nsun,
                                      c->dp.irhon, c->dp.nf, s));
    mark(6);
  }
  if (ct) {  // the level's recalculation with the step's dt (scale 1)
    const double* eo = (p.time_approximation == MF_TA_RK2) ? (const double*)L->ct_eo.p : e2;
    MF_CHECK_CUDA(mf::launch_recalc_b(c->dp, (double*)L->U.p, u0, eo, nullptr, nullptr, ds, 1.0,
                                      0, L->b2, s));
    mark(7);
  }
  if (nev) *nev = ne;
  return MF_OK;
}

static mf_status level_graph(mf_level* L, int advance, cudaGraphExec_t* out) {
  if (*out) return MF_OK;
  cudaGraph_t g = nullptr;
  MF_CHECK_CUDA(cudaStreamBeginCapture(L->s, cudaStreamCaptureModeThreadLocal));
  mf_status st = enqueue_level_step(L, advance);
  cudaError_t e = cudaStreamEndCapture(L->s, &g);
  if (st != MF_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return MF_ERR_CUDA;
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    *out = nullptr;
    return MF_ERR_CUDA;
  }
  return MF_OK;
}

// The user stream (if any) and the level's own stream are ordered with events.
static mf_status join_streams(cudaStream_t from, cudaStream_t to) {
  if (from == to) return MF_OK;
  cudaEvent_t ev;
  MF_CHECK_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ev, from);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(to, ev, 0);
  cudaEventDestroy(ev);
  return e == cudaSuccess ? MF_OK : MF_ERR_CUDA;
}

mf_status mf_level_create(mf_ctx* c, int npatch, const mf_box* valid, mf_level** out) {
  if (!c || !valid || !out || npatch <= 0) return MF_ERR_BAD_ARG;
  *out = nullptr;
  const mf_params& p = c->p;
  const int sd = p.space_dim, nc = c->nc;
  mf::LevelPlan plan;
  mf_status pst = mf::build_level_plan(p, c->ng, nc, npatch, valid, plan);
  if (pst != MF_OK) return pst;
  mf_level* L = new (std::nothrow) mf_level();
  if (!L) return MF_ERR_OOM;
  L->ctx = c;
  L->time = c->time;
  L->np = npatch;
  L->valid = plan.valid;
  L->fab = plan.fab;
  L->off = plan.off;
  L->total = plan.total;
  L->cells = plan.cells;
  L->hd1 = plan.d1;
  L->hd2 = plan.d2;
  const int mixed = (p.precision == MF_PREC_MIXED);
  const size_t rs = mixed ? sizeof(float) : sizeof(double);
  std::vector<StageDesc> hd(plan.d1);
  hd.insert(hd.end(), plan.d2.begin(), plan.d2.end());
  L->lean = plan.lean;
  if (L->lean) hd.insert(hd.end(), plan.dp.begin(), plan.dp.end());
  const long long* fsize = plan.fsize;
  const long long* bsize = plan.bsize;
  std::memset(&L->b1, 0, sizeof(L->b1));
  std::memset(&L->b2, 0, sizeof(L->b2));
  std::memset(&L->bp, 0, sizeof(L->bp));
  std::memset(&L->lp, 0, sizeof(L->lp));
  RunParams hrun = mf::run_params_of(c->dp);
  if (!mf::batch_offsets(hd.data(), npatch, sd, L->b1) ||
      !mf::batch_offsets(hd.data() + npatch, npatch, sd, L->b2, &hrun, 1) ||
      (L->lean && !mf::batch_offsets(hd.data() + 2 * npatch, npatch, sd, L->bp))) {
    delete L;
    return MF_ERR_UNSUPPORTED;  // more than 2^31 cells or faces in one launch
  }
  // the host copies with their flat offsets (the overlap's chunk plans read them)
  L->hd1.assign(hd.begin(), hd.begin() + npatch);
  L->hd2.assign(hd.begin() + npatch, hd.begin() + 2 * npatch);
  mf::batch_default_threads(L->b1);
  mf::batch_default_threads(L->b2);
  mf::batch_default_threads(L->bp);
  const std::vector<CopyReg>& full = plan.full;
  const std::vector<CopyReg>& two = plan.two;
  L->nfull = (int)full.size();
  L->ntwo = (int)two.size();
  L->nparts = mf::dt_partials(L->b2);
  mf_status st = MF_OK;
  auto fail = [&](cudaError_t e) {
    st = (e == cudaErrorMemoryAllocation) ? MF_ERR_OOM : MF_ERR_CUDA;
  };
  cudaError_t e = cudaSuccess;
  do {
    if ((e = L->U.ensure(sizeof(double) * L->total)) != cudaSuccess) break;
    if ((e = cudaMemset(L->U.p, 0, sizeof(double) * L->total)) != cudaSuccess) break;
    if (p.time_approximation == MF_TA_RK2 || p.time_approximation == MF_TA_HANCOCK) {
      if ((e = L->U1.ensure(sizeof(double) * L->total)) != cudaSuccess) break;
      if ((e = cudaMemset(L->U1.p, 0, sizeof(double) * L->total)) != cudaSuccess) break;
    }
    if (p.time_approximation == MF_TA_HANCOCK)
      for (int d = 0; d < sd && e == cudaSuccess; ++d)
        e = L->FV[d].ensure(sizeof(double) * std::max<long long>(plan.fvsize, 1));
    if (e != cudaSuccess) break;
    if ((e = L->W.ensure(sizeof(double) * L->total)) != cudaSuccess) break;
    if (mixed && (e = L->Wf.ensure(sizeof(float) * L->total)) != cudaSuccess) break;
    for (int d = 0; d < sd && e == cudaSuccess; ++d) {
      e = L->F[d].ensure(rs * fsize[d]);
      if (e == cudaSuccess) e = L->Bn[d].ensure(rs * bsize[d]);
    }
    if (e != cudaSuccess) break;
    // descs of both stages, then the level's run parameters
    const size_t dbytes = sizeof(StageDesc) * hd.size();
    if ((e = L->desc.ensure(dbytes + sizeof(RunParams))) != cudaSuccess) break;
    if ((e = cudaMemcpy(L->desc.p, hd.data(), dbytes, cudaMemcpyHostToDevice)) != cudaSuccess)
      break;
    RunParams* druns = (RunParams*)((char*)L->desc.p + dbytes);
    if ((e = cudaMemcpy(druns, &hrun, sizeof(RunParams), cudaMemcpyHostToDevice)) != cudaSuccess)
      break;
    L->b1.desc = (const StageDesc*)L->desc.p;
    L->b2.desc = (const StageDesc*)L->desc.p + npatch;
    L->bp.desc = (const StageDesc*)L->desc.p + 2 * npatch;
    L->b1.runs = L->b2.runs = L->bp.runs = druns;
    if (L->lean) {
      if ((e = L->far.ensure(sizeof(mf::FarReg) * std::max<size_t>(1, plan.far.size()))) !=
          cudaSuccess)
        break;
      if (!plan.far.empty() &&
          (e = cudaMemcpy(L->far.p, plan.far.data(), sizeof(mf::FarReg) * plan.far.size(),
                          cudaMemcpyHostToDevice)) != cudaSuccess)
        break;
    }
    if ((e = L->exfull.ensure(sizeof(CopyReg) * std::max<size_t>(1, full.size()))) != cudaSuccess)
      break;
    if (!full.empty() &&
        (e = cudaMemcpy(L->exfull.p, full.data(), sizeof(CopyReg) * full.size(),
                        cudaMemcpyHostToDevice)) != cudaSuccess)
      break;
    if ((e = L->extwo.ensure(sizeof(CopyReg) * std::max<size_t>(1, two.size()))) != cudaSuccess)
      break;
    if (!two.empty() && (e = cudaMemcpy(L->extwo.p, two.data(), sizeof(CopyReg) * two.size(),
                                        cudaMemcpyHostToDevice)) != cudaSuccess)
      break;
    L->nsun = (int)plan.sun.size();
    if ((e = L->sun.ensure(sizeof(mf::SunPair) * std::max<size_t>(1, plan.sun.size()))) !=
        cudaSuccess)
      break;
    if (!plan.sun.empty() &&
        (e = cudaMemcpy(L->sun.p, plan.sun.data(), sizeof(mf::SunPair) * plan.sun.size(),
                        cudaMemcpyHostToDevice)) != cudaSuccess)
      break;
    if (c->dp.ct) {  // UOld of the level and three edge fields (3 per cell of U)
      const size_t eb = sizeof(double) * 3 * (size_t)(L->total / c->nc + 1);
      if ((e = L->ct_u0.ensure(sizeof(double) * L->total)) != cudaSuccess) break;
      if ((e = L->ct_e1.ensure(eb)) != cudaSuccess) break;
      if ((e = L->ct_e2.ensure(eb)) != cudaSuccess) break;
      if ((e = L->ct_eo.ensure(eb)) != cudaSuccess) break;
    }
    if ((e = L->partials.ensure(sizeof(DtPartial) * (L->nparts + 1))) != cudaSuccess) break;
    if ((e = L->state.ensure(sizeof(StepState))) != cudaSuccess) break;
    if ((e = L->state2.ensure(sizeof(StepState))) != cudaSuccess) break;
    if ((e = L->hstate.ensure(sizeof(StepState))) != cudaSuccess) break;
    std::memset(L->hstate.p, 0, sizeof(StepState));
    if ((e = cudaMemcpy(L->state.p, L->hstate.p, sizeof(StepState), cudaMemcpyHostToDevice)) !=
        cudaSuccess)
      break;
    if ((e = cudaStreamCreateWithFlags(&L->s, cudaStreamNonBlocking)) != cudaSuccess) break;
  } while (0);
  if (e != cudaSuccess) fail(e);
  if (st != MF_OK) {
    mf_level_destroy(L);
    return st;
  }
  if (L->lean) {
    L->lp.prim = &L->bp;
    L->lp.regs = (const CopyReg*)L->extwo.p;
    L->lp.nregs = L->ntwo;
    L->lp.far = (const mf::FarReg*)L->far.p;
    L->lp.nfar = (int)plan.far.size();
    // the FP64 primitive ghosts are read by the FP64 flux kernels, the
    // characteristic projections, central Bn and the tracking surfaces'
    // floor; the FP32 flux kernels read only the FP32 copy
    L->lp.exchange_w = (!mixed || p.char_reconstruction || p.divb_method == 2 ||
                        p.num_tracking_surfaces > 0)
                           ? 1
                           : 0;
  }
  // the split flux and update kernels until mf_level_set_schedule or the
  // autotuner picks the fused kernel
  L->fused = false;
  const int per_stage = mf::stage_launches(sd);
  L->launches = (p.time_approximation == MF_TA_RK2) ? (2 * per_stage + 2 + 1)
                : (p.time_approximation == MF_TA_HANCOCK) ? (mf::hancock_launches(sd) + 1 + 1)
                                                          : (per_stage + 1 + 1);
  if (L->nfull == 0) L->launches -= 1;
  if (p.time_approximation == MF_TA_RK2 && L->ntwo == 0) L->launches -= 1;
  if (L->lean) {  // no exchange of U; the primitive part of every stage instead
    const int stages = (p.time_approximation == MF_TA_RK2) ? 2 : 1;
    if (L->nfull) L->launches -= 1;
    if (p.time_approximation == MF_TA_RK2 && L->ntwo) L->launches -= 1;
    L->launches += stages * (mf::prim_launches(&L->lp, mixed) - 1);
  }
  // one fused kernel instead of the fluxes and the update (while no gathers)
  L->fused_saving = L->fused ? ((p.time_approximation == MF_TA_RK2) ? 2 : 1) * sd : 0;
  if (L->nsun) L->launches += 1;
  // constrained transport: edge field + recalculation per stage, the dt after
  // them, and the level's recalculation
  if (c->dp.ct) L->launches += (p.time_approximation == MF_TA_RK2) ? 6 : 4;
  L->base_launches = L->launches;
  L->launches -= L->fused_saving;
  *out = L;
  return MF_OK;
}

void mf_level_destroy(mf_level* L) {
  if (!L) return;
  if (L->gsync) cudaGraphExecDestroy(L->gsync);
  if (L->gasync) cudaGraphExecDestroy(L->gasync);
  if (L->s) cudaStreamDestroy(L->s);
  L->lines.release();
  L->U.release();
  L->U1.release();
  L->W.release();
  for (int d = 0; d < 3; ++d) {
    L->F[d].release();
    L->Bn[d].release();
    L->FV[d].release();
  }
  L->desc.release();
  L->exfull.release();
  L->extwo.release();
  L->partials.release();
  L->state.release();
  L->state2.release();
  L->sun.release();
  L->hstate.release();
  L->ct_u0.release();
  L->ct_e1.release();
  L->ct_e2.release();
  L->ct_eo.release();
  L->packed.release();
  L->Wf.release();
  L->far.release();
  L->tiles.release();
  delete L;
}

long long mf_level_num_doubles(const mf_level* L) { return L ? L->total : -1; }
long long mf_level_num_cells(const mf_level* L) { return L ? L->cells : -1; }

long long mf_level_patch_offset(const mf_level* L, int p) {
  if (!L || p < 0 || p >= L->np) return -1;
  return L->off[p];
}

// Packed valid-cell offsets: nc x the patch's first cell in the order of the
// stage descs (patch order, valid boxes back to back), as k_pack indexes them.
static void level_voff(mf_level* L) {
  if ((int)L->voff.size() == L->np + 1) return;
  L->voff.assign(L->np + 1, 0);
  for (int i = 0; i < L->np; ++i)
    L->voff[i + 1] = L->voff[i] + box_cells(L->valid[i]) * L->ctx->nc;
}

long long mf_level_valid_doubles(const mf_level* L) {
  if (!L) return -1;
  level_voff(const_cast<mf_level*>(L));
  return L->voff[L->np];
}

long long mf_level_valid_offset(const mf_level* L, int p) {
  if (!L || p < 0 || p >= L->np) return -1;
  level_voff(const_cast<mf_level*>(L));
  return L->voff[p];
}

static mf_status level_pack(mf_level* L, double* host, int to_fab, void* stream) {
  level_voff(L);
  const long long n = L->voff[L->np];
  MF_CHECK_CUDA(L->packed.ensure(sizeof(double) * (size_t)std::max<long long>(n, 1)));
  cudaStream_t us = (cudaStream_t)stream;
  mf_status st = join_streams(us, L->s);
  if (st != MF_OK) return st;
  double* dp = (double*)L->packed.p;
  if (to_fab) {
    MF_CHECK_CUDA(cudaMemcpyAsync(dp, host, sizeof(double) * n, cudaMemcpyHostToDevice, L->s));
    MF_CHECK_CUDA(mf::launch_pack((double*)L->U.p, dp, L->b2, L->ctx->nc, 1, L->s));
  } else {
    MF_CHECK_CUDA(mf::launch_pack((double*)L->U.p, dp, L->b2, L->ctx->nc, 0, L->s));
    MF_CHECK_CUDA(cudaMemcpyAsync(host, dp, sizeof(double) * n, cudaMemcpyDeviceToHost, L->s));
  }
  st = join_streams(L->s, us);
  if (st != MF_OK) return st;
  return wait_stream(L->s, L->ctx->timeout);
}

mf_status mf_level_upload_valid(mf_level* L, const double* host, void* stream) {
  if (!L || !host) return MF_ERR_BAD_ARG;
  return level_pack(L, const_cast<double*>(host), 1, stream);
}

mf_status mf_level_download_valid(mf_level* L, double* host, void* stream) {
  if (!L || !host) return MF_ERR_BAD_ARG;
  return level_pack(L, host, 0, stream);
}

mf_status mf_level_patch_fab(const mf_level* L, int p, mf_fab* out) {
  if (!L || !out || p < 0 || p >= L->np) return MF_ERR_BAD_ARG;
  out->data = (double*)L->U.p + L->off[p];
  out->box = L->fab[p];
  out->ncomp = L->ctx->nc;
  return MF_OK;
}

mf_status mf_level_upload(mf_level* L, const double* host, void* stream) {
  if (!L || !host) return MF_ERR_BAD_ARG;
  cudaStream_t us = (cudaStream_t)stream;
  mf_status st = join_streams(us, L->s);
  if (st != MF_OK) return st;
  MF_CHECK_CUDA(
      cudaMemcpyAsync(L->U.p, host, sizeof(double) * L->total, cudaMemcpyHostToDevice, L->s));
  st = join_streams(L->s, us);
  if (st != MF_OK) return st;
  return wait_stream(L->s, L->ctx->timeout);
}

mf_status mf_level_download(const mf_level* L, double* host, void* stream) {
  if (!L || !host) return MF_ERR_BAD_ARG;
  cudaStream_t us = (cudaStream_t)stream;
  mf_status st = join_streams(us, L->s);
  if (st != MF_OK) return st;
  MF_CHECK_CUDA(
      cudaMemcpyAsync(host, L->U.p, sizeof(double) * L->total, cudaMemcpyDeviceToHost, L->s));
  return wait_stream(L->s, L->ctx->timeout);
}

mf_status mf_level_exchange(mf_level* L, void* stream) {
  if (!L) return MF_ERR_BAD_ARG;
  cudaStream_t us = (cudaStream_t)stream;
  mf_status st = join_streams(us, L->s);
  if (st != MF_OK) return st;
  MF_CHECK_CUDA(mf::launch_exchange((double*)L->U.p, (const CopyReg*)L->exfull.p, L->nfull,
                                    L->ctx->nc, L->s));
  st = join_streams(L->s, us);
  if (st != MF_OK) return st;
  return wait_stream(L->s, L->ctx->timeout);
}

static void decode_result(const mf_level* L, const StepState* hs, double* new_dt, int* min_patch,
                          int min_cell[3]) {
  if (new_dt) *new_dt = hs->dt_min;
  int pi = hs->min_desc;
  if (pi < 0 || pi >= L->np) pi = 0;
  if (min_patch) *min_patch = pi;
  if (min_cell) {
    int n[3];
    ext3(L->valid[pi], n);
    int idx = hs->min_idx;
    if (idx < 0 || idx == 0x7fffffff) idx = 0;
    min_cell[0] = L->valid[pi].lo[0] + idx % n[0];
    min_cell[1] = L->valid[pi].lo[1] + (idx / n[0]) % n[1];
    min_cell[2] = L->valid[pi].lo[2] + idx / (n[0] * n[1]);
  }
}

mf_status mf_level_step(mf_level* L, double dt, double* new_dt, int* min_patch, int min_cell[3],
                        void* stream) {
  if (!L || !(dt > 0.0) || !std::isfinite(dt)) return MF_ERR_BAD_ARG;
  mf_ctx* c = L->ctx;
  mf_status st = level_graph(L, 0, &L->gsync);
  if (st != MF_OK) return st;
  cudaStream_t us = (cudaStream_t)stream;
  st = join_streams(us, L->s);
  if (st != MF_OK) return st;
  StepState* hs = (StepState*)L->hstate.p;
  std::memset(hs, 0, sizeof(*hs));
  hs->dt = dt;
  hs->time = L->time;
  hs->ch = c->p.dedner_ch;
  hs->cp = c->p.dedner_cp;
  MF_CHECK_CUDA(cudaMemcpyAsync(L->state.p, hs, sizeof(StepState), cudaMemcpyHostToDevice, L->s));
  MF_CHECK_CUDA(cudaGraphLaunch(L->gsync, L->s));
  MF_CHECK_CUDA(cudaMemcpyAsync(hs, L->state.p, sizeof(StepState), cudaMemcpyDeviceToHost, L->s));
  st = join_streams(L->s, us);
  if (st != MF_OK) return st;
  st = wait_stream(L->s, c->timeout);
  if (st != MF_OK) return st;
  L->time = hs->time;
  decode_result(L, hs, new_dt, min_patch, min_cell);
  return flags_status(hs->flags);
}

mf_status mf_level_compute_dt(mf_level* L, double* dt, int* min_patch, int min_cell[3],
                              void* stream) {
  if (!L) return MF_ERR_BAD_ARG;
  mf_ctx* c = L->ctx;
  cudaStream_t us = (cudaStream_t)stream;
  mf_status st = join_streams(us, L->s);
  if (st != MF_OK) return st;
  StepState* hs = (StepState*)L->hstate.p;
  std::memset(hs, 0, sizeof(*hs));
  MF_CHECK_CUDA(cudaMemcpyAsync(L->state2.p, hs, sizeof(StepState), cudaMemcpyHostToDevice, L->s));
  int nb = 0;
  MF_CHECK_CUDA(
      mf::launch_dt(c->dp, (const double*)L->U.p, L->b2, (DtPartial*)L->partials.p, &nb, L->s));
  MF_CHECK_CUDA(mf::launch_finalize(c->dp, (const DtPartial*)L->partials.p, L->b2,
                                    L->b2.nt[2], (StepState*)L->state2.p, 0, L->s));
  MF_CHECK_CUDA(
      cudaMemcpyAsync(hs, L->state2.p, sizeof(StepState), cudaMemcpyDeviceToHost, L->s));
  st = wait_stream(L->s, c->timeout);
  if (st != MF_OK) return st;
  decode_result(L, hs, dt, min_patch, min_cell);
  return flags_status(hs->flags);
}

mf_status mf_level_seed_dt(mf_level* L, double dt, double cfl, void* stream) {
  if (!L || !(dt > 0.0) || !(cfl > 0.0)) return MF_ERR_BAD_ARG;
  mf_ctx* c = L->ctx;
  cudaStream_t us = (cudaStream_t)stream;
  mf_status st = join_streams(us, L->s);
  if (st != MF_OK) return st;
  StepState* hs = (StepState*)L->hstate.p;
  std::memset(hs, 0, sizeof(*hs));
  hs->dt = dt;
  hs->time = L->time;
  hs->cfl = cfl;
  hs->ch = c->p.dedner_ch;
  hs->cp = c->p.dedner_cp;
  MF_CHECK_CUDA(cudaMemcpyAsync(L->state.p, hs, sizeof(StepState), cudaMemcpyHostToDevice, L->s));
  return wait_stream(L->s, c->timeout);
}

mf_status mf_level_step_async(mf_level* L, void* stream) {
  if (!L) return MF_ERR_BAD_ARG;
  mf_status st = level_graph(L, 1, &L->gasync);
  if (st != MF_OK) return st;
  cudaStream_t us = (cudaStream_t)stream;
  st = join_streams(us, L->s);
  if (st != MF_OK) return st;
  MF_CHECK_CUDA(cudaGraphLaunch(L->gasync, L->s));
  return join_streams(L->s, us);
}

mf_status mf_level_result(mf_level* L, double* new_dt, int* min_patch, int min_cell[3],
                          void* stream) {
  if (!L) return MF_ERR_BAD_ARG;
  cudaStream_t us = (cudaStream_t)stream;
  mf_status st = join_streams(us, L->s);
  if (st != MF_OK) return st;
  StepState* hs = (StepState*)L->hstate.p;
  MF_CHECK_CUDA(cudaMemcpyAsync(hs, L->state.p, sizeof(StepState), cudaMemcpyDeviceToHost, L->s));
  st = wait_stream(L->s, L->ctx->timeout);
  if (st != MF_OK) return st;
  L->time = hs->time;
  decode_result(L, hs, new_dt, min_patch, min_cell);
  return flags_status(hs->flags);
}

mf_status mf_level_set_time(mf_level* L, double time) {
  if (!L || !std::isfinite(time)) return MF_ERR_BAD_ARG;
  L->time = time;
  // the device copy, which the async steps read and advance
  StepState* hs = (StepState*)L->hstate.p;
  hs->time = time;
  MF_CHECK_CUDA(cudaMemcpyAsync((char*)L->state.p + offsetof(StepState, time), &hs->time,
                                sizeof(double), cudaMemcpyHostToDevice, L->s));
  return wait_stream(L->s, L->ctx->timeout);
}

mf_status mf_level_time(mf_level* L, double* time) {
  if (!L || !time) return MF_ERR_BAD_ARG;
  StepState* hs = (StepState*)L->hstate.p;
  MF_CHECK_CUDA(cudaMemcpyAsync(&hs->time, (const char*)L->state.p + offsetof(StepState, time),
                                sizeof(double), cudaMemcpyDeviceToHost, L->s));
  mf_status st = wait_stream(L->s, L->ctx->timeout);
  if (st != MF_OK) return st;
  L->time = hs->time;
  *time = hs->time;
  return MF_OK;
}

int mf_level_launches_per_step(const mf_level* L) { return L ? L->launches : -1; }

// Make the level step with the fused kernel (its work lists already built)
// or the split kernels; the captured graphs are rebuilt on next use.
static void apply_schedule(mf_level* L, bool fused) {
  L->fused = fused;
  count_launches(L);
  if (L->gsync) cudaGraphExecDestroy(L->gsync);
  if (L->gasync) cudaGraphExecDestroy(L->gasync);
  L->gsync = L->gasync = nullptr;
}

mf_status mf_level_set_schedule(mf_level* L, const int tile[3]) {
  if (!L || !tile) return MF_ERR_BAD_ARG;
  const mf_params& p = L->ctx->p;
  const int sd = p.space_dim;
  bool fused = false;
  if (tile[0] != 0) {
    if (!mf::fused_supported(L->ctx->dp, p.precision, p.time_approximation))
      return MF_ERR_UNSUPPORTED;
    const int t[3] = {tile[0], tile[1], sd == 3 ? tile[2] : 1};
    if (!mf::fused_tile_ok(L->ctx->dp, t)) return MF_ERR_BAD_ARG;
    mf_status st = wait_stream(L->s, L->ctx->timeout);  // the old lists may be in use
    if (st != MF_OK) return st;
    bool ok = false;
    MF_CHECK_CUDA(level_set_tiles(L, t, &ok));
    if (!ok) return MF_ERR_BAD_ARG;
    fused = true;
  }
  apply_schedule(L, fused);
  return MF_OK;
}

// Cut the split flux and update launches of each stage into chunks of
// consecutive patches whose fluxes and updates overlap (MF_PREC_MIXED and
// MF_PREC_MIXED_CE32, RK2 or first order, no constrained transport); 1 = one
// launch each.
static mf_status level_set_chunks(mf_level* L, int chunks) {
  const mf_params& p = L->ctx->p;
  if (chunks < 1 || chunks > MF_MAX_OVERLAP_CHUNKS) return MF_ERR_BAD_ARG;
  if (chunks > 1 && (p.precision != MF_PREC_MIXED ||
                     (p.time_approximation != MF_TA_RK2 &&
                      p.time_approximation != MF_TA_FIRST_ORDER) ||
                     L->ctx->dp.ct))
    return MF_ERR_UNSUPPORTED;
  mf_status st = wait_stream(L->s, L->ctx->timeout);  // the old plans may be in use
  if (st != MF_OK) return st;
  int n = 1;
  if (chunks > 1) {
    L->ch1 = mf::make_chunks(L->hd1.data(), (int)L->hd1.size(), L->b1, chunks);
    L->ch2 = mf::make_chunks(L->hd2.data(), (int)L->hd2.size(), L->b2, chunks);
    n = (int)std::min(L->ch1.size(), L->ch2.size());
    if (L->ch1.size() != L->ch2.size()) {  // keep the two stages alike
      L->ch1 = mf::make_chunks(L->hd1.data(), (int)L->hd1.size(), L->b1, n);
      L->ch2 = mf::make_chunks(L->hd2.data(), (int)L->hd2.size(), L->b2, n);
      n = (int)std::min(L->ch1.size(), L->ch2.size());
    }
  }
  L->nchunks = std::max(1, n);
  L->op1 = {L->ch1.data(), (int)L->ch1.size()};
  L->op2 = {L->ch2.data(), (int)L->ch2.size()};
  count_launches(L);
  if (L->gsync) cudaGraphExecDestroy(L->gsync);
  if (L->gasync) cudaGraphExecDestroy(L->gasync);
  L->gsync = L->gasync = nullptr;
  return MF_OK;
}

// Face fluxes of the FP64 paths per face (k_flux) or by lines (k_lflux);
// the line work lists of both stage batches are built on first use.
static mf_status level_set_flux_form(mf_level* L, int form) {
  const mf_params& p = L->ctx->p;
  if (form != MF_FLUX_FACES && form != MF_FLUX_LINES) return MF_ERR_BAD_ARG;
  if (form == MF_FLUX_LINES &&
      (p.precision == MF_PREC_MIXED || p.time_approximation == MF_TA_HANCOCK))
    return MF_ERR_UNSUPPORTED;
  mf_status st = wait_stream(L->s, L->ctx->timeout);  // the old lists may be in use
  if (st != MF_OK) return st;
  if (form == MF_FLUX_LINES && L->lp1.w[0] == nullptr) {
    const int sd = p.space_dim;
    std::vector<mf::LineWork> w1[3], w2[3];
    int m1[3], m2[3];
    if (!mf::make_lines(L->hd1.data(), (int)L->hd1.size(), sd, w1, m1) ||
        !mf::make_lines(L->hd2.data(), (int)L->hd2.size(), sd, w2, m2))
      return MF_ERR_UNSUPPORTED;  // a patch too long along a direction
    std::vector<mf::LineWork> all;
    size_t o1[3], o2[3];
    for (int d = 0; d < 3; ++d) {
      o1[d] = all.size();
      all.insert(all.end(), w1[d].begin(), w1[d].end());
    }
    for (int d = 0; d < 3; ++d) {
      o2[d] = all.size();
      all.insert(all.end(), w2[d].begin(), w2[d].end());
    }
    MF_CHECK_CUDA(mf::lines_prepare());
    MF_CHECK_CUDA(L->lines.ensure(sizeof(mf::LineWork) * std::max<size_t>(1, all.size())));
    MF_CHECK_CUDA(cudaMemcpy(L->lines.p, all.data(), sizeof(mf::LineWork) * all.size(),
                             cudaMemcpyHostToDevice));
    const mf::LineWork* base = (const mf::LineWork*)L->lines.p;
    for (int d = 0; d < 3; ++d) {
      L->lp1.w[d] = base + o1[d];
      L->lp1.n[d] = (int)w1[d].size();
      L->lp1.maxcells[d] = m1[d];
      L->lp2.w[d] = base + o2[d];
      L->lp2.n[d] = (int)w2[d].size();
      L->lp2.maxcells[d] = m2[d];
    }
  }
  L->flux_form = form;
  if (L->gsync) cudaGraphExecDestroy(L->gsync);
  if (L->gasync) cudaGraphExecDestroy(L->gasync);
  L->gsync = L->gasync = nullptr;
  return MF_OK;
}

mf_status mf_level_set_flux_form(mf_level* L, int form) {
  if (!L) return MF_ERR_BAD_ARG;
  return level_set_flux_form(L, form);
}

mf_status mf_level_flux_form(const mf_level* L, int* form) {
  if (!L || !form) return MF_ERR_BAD_ARG;
  *form = L->flux_form;
  return MF_OK;
}

mf_status mf_level_set_overlap(mf_level* L, int chunks) {
  if (!L) return MF_ERR_BAD_ARG;
  return level_set_chunks(L, chunks);
}

mf_status mf_level_overlap(const mf_level* L, int* chunks) {
  if (!L || !chunks) return MF_ERR_BAD_ARG;
  *chunks = L->nchunks;
  return MF_OK;
}

mf_status mf_level_schedule(const mf_level* L, int tile[3]) {
  if (!L || !tile) return MF_ERR_BAD_ARG;
  for (int d = 0; d < 3; ++d) tile[d] = L->fused ? L->fp1.tile[d] : 0;
  return MF_OK;
}

mf_status mf_level_profile_step(mf_level* L, double dt, float* ms, int* kinds, int* nlaunch,
                                int max_launch) {
  if (!L || !ms || !kinds || !nlaunch || !(dt > 0.0)) return MF_ERR_BAD_ARG;
  if (max_launch < L->launches) return MF_ERR_BAD_ARG;
  mf_ctx* c = L->ctx;
  std::vector<cudaEvent_t> ev(L->launches + 1);
  for (auto& e : ev) MF_CHECK_CUDA(cudaEventCreate(&e));
  StepState* hs = (StepState*)L->hstate.p;
  std::memset(hs, 0, sizeof(*hs));
  hs->dt = dt;
  hs->time = L->time;
  hs->ch = c->p.dedner_ch;
  hs->cp = c->p.dedner_cp;
  mf_status st = MF_OK;
  int ne = 0;
  do {
    if (cudaMemcpyAsync(L->state.p, hs, sizeof(StepState), cudaMemcpyHostToDevice, L->s) !=
        cudaSuccess) {
      st = MF_ERR_CUDA;
      break;
    }
    cudaEventRecord(ev[0], L->s);
    st = enqueue_level_step(L, 0, ev.data() + 1, kinds, &ne);
    if (st != MF_OK) break;
    st = wait_stream(L->s, c->timeout);
    if (st != MF_OK) break;
    L->time += dt;
    for (int q = 0; q < ne; ++q) {
      float t = 0.f;
      cudaEventElapsedTime(&t, ev[q], ev[q + 1]);
      ms[q] = t;
    }
    *nlaunch = ne;
  } while (0);
  for (auto& e : ev) cudaEventDestroy(e);
  return st;
}

// Time `reps` launches of one kernel kind of stage 1 (0 prim, 1 fluxes of
// every direction, 2 update without averaging, 3 the fused flux + update
// kernel on the work list in fp1, 4 the fluxes and update in the level's
// overlap chunks) with the level's current threads.
// Stage 1 reads U and writes only W, F, Bn and U1, so the level's state is
// left as it was; the step state used is a private copy with dt = 0.
static mf_status time_kind(mf_level* L, int kind, int reps, cudaEvent_t e0, cudaEvent_t e1,
                           float* ms) {
  mf_ctx* c = L->ctx;
  const mf_params& p = c->p;
  StageBuffers B;
  std::memset(&B, 0, sizeof(B));
  B.uin = (const double*)L->U.p;
  B.uout = (double*)(p.time_approximation == MF_TA_RK2 ? L->U1.p : L->W.p);
  B.w = (double*)L->W.p;
  B.wf = (p.precision == MF_PREC_MIXED) ? (float*)L->Wf.p : nullptr;
  for (int d = 0; d < 3; ++d) {
    B.f[d] = L->F[d].p;
    B.bn[d] = L->Bn[d].p;
  }
  StepState* ds = (StepState*)L->state2.p;
  DtPartial* parts = (DtPartial*)L->partials.p;
  const mf::Batch& b = (p.time_approximation == MF_TA_RK2) ? L->b1 : L->b2;
  const int sd = p.space_dim;
  MF_CHECK_CUDA(cudaEventRecord(e0, L->s));
  for (int r = 0; r < reps; ++r) {
    cudaError_t e = cudaSuccess;
    if (kind == 0) {
      e = mf::launch_prim(c->dp, B.uin, B.w, L->lean ? L->bp : b, L->s, B.wf);
    } else if (kind == 1) {
      const mf::LinePlan& lp = (p.time_approximation == MF_TA_RK2) ? L->lp1 : L->lp2;
      const bool lines = L->flux_form == MF_FLUX_LINES;
      for (int d = 0; d < sd && e == cudaSuccess; ++d) {
        if (p.precision == MF_PREC_MIXED)
          e = mf::launch_flux_fast<float>(c->dp, d, B.w, B.f[d], B.bn[d], b, ds, L->s, B.wf);
        else if (p.precision == MF_PREC_FP64_FAST)
          e = lines ? mf::launch_flux_lines_fast(c->dp, d, B.w, B.f[d], B.bn[d], b, lp, ds, L->s)
                    : mf::launch_flux_fast<double>(c->dp, d, B.w, B.f[d], B.bn[d], b, ds, L->s);
        else
          e = lines ? mf::launch_flux_lines_exact(c->dp, d, B.w, B.f[d], B.bn[d], b, lp, ds, L->s)
                    : mf::launch_flux_exact(c->dp, d, B.w, B.f[d], B.bn[d], b, ds, L->s);
      }
    } else if (kind == 4) {  // fluxes + update of stage 1 in the level's chunks, overlapped
      StageBuffers Bo = B;
      Bo.overlap = (p.time_approximation == MF_TA_RK2) ? &L->op1 : &L->op2;
      int nb = 0;
      e = mf::launch_flux_update_overlap(c->dp, Bo, b, 0, 1.0, ds, parts, &nb, L->s);
    } else if (kind == 3) {  // the fused kernel on stage 1's work list
      e = mf::launch_fused(c->dp, B, b, L->fp1.tiles, L->fp1.ntiles, L->fp1.tile, 0, 1.0, ds,
                           parts, L->s);
    } else {
      int nb = 0;
      if (p.precision == MF_PREC_MIXED)
        e = mf::launch_update_fast<float>(c->dp, B, b, 0, 1.0, ds, parts, &nb, L->s);
      else if (p.precision == MF_PREC_FP64_FAST)
        e = mf::launch_update_fast<double>(c->dp, B, b, 0, 1.0, ds, parts, &nb, L->s);
      else
        e = mf::launch_update_exact(c->dp, B, b, 0, 1.0, ds, parts, &nb, L->s);
    }
    MF_CHECK_CUDA(e);
  }
  MF_CHECK_CUDA(cudaEventRecord(e1, L->s));
  mf_status st = wait_stream(L->s, c->timeout);
  if (st != MF_OK) return st;
  MF_CHECK_CUDA(cudaEventElapsedTime(ms, e0, e1));
  return MF_OK;
}

mf_status mf_level_autotune(mf_level* L, int reps, int threads[3]) {
  if (!L || reps <= 0 || reps > 1000) return MF_ERR_BAD_ARG;
  mf_ctx* c = L->ctx;
  StepState* hs = (StepState*)L->hstate.p;
  std::memset(hs, 0, sizeof(*hs));
  hs->ch = c->p.dedner_ch;
  hs->cp = c->p.dedner_cp;
  MF_CHECK_CUDA(cudaMemcpyAsync(L->state2.p, hs, sizeof(StepState), cudaMemcpyHostToDevice, L->s));
  // dt partials of the tried launches: the largest count (fewest threads)
  const int most = (int)mf::flat_blocks(std::max(L->b1.tot_v, L->b2.tot_v), 64);
  MF_CHECK_CUDA(L->partials.ensure(sizeof(DtPartial) * (most + 1)));
  cudaEvent_t e0, e1;
  MF_CHECK_CUDA(cudaEventCreate(&e0));
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return MF_ERR_CUDA;
  }
  static const int cand[3] = {64, 128, 256};
  mf_status st = MF_OK;
  for (int kind = 0; kind < 3 && st == MF_OK; ++kind) {
    float best = 0.f;
    int bnt = L->b1.nt[kind];
    for (int q = 0; q < 3 && st == MF_OK; ++q) {
      L->b1.nt[kind] = L->b2.nt[kind] = L->bp.nt[kind] = cand[q];
      float ms = 0.f;
      st = time_kind(L, kind, 1, e0, e1, &ms);  // warm-up
      if (st == MF_OK) st = time_kind(L, kind, reps, e0, e1, &ms);
      if (st == MF_OK && (q == 0 || ms < best)) {
        best = ms;
        bnt = cand[q];
      }
    }
    L->b1.nt[kind] = L->b2.nt[kind] = L->bp.nt[kind] = bnt;
  }
  // schedule, by the time of stage 1's fluxes + update: the split kernels,
  // unchunked or in 2, 4, 8 overlapped chunks (mixed precision), against the
  // fused kernel at each tile shape that fits the options.  A level feeding
  // flux registers keeps the split, unchunked kernels, which store the fluxes.
  const mf_params& p = c->p;
  const int sd = p.space_dim;
  // FP64 paths: the face fluxes per face against by lines
  if (st == MF_OK && p.precision != MF_PREC_MIXED && p.time_approximation != MF_TA_HANCOCK) {
    float tfa = 0.f, tli = 0.f;
    st = level_set_flux_form(L, MF_FLUX_FACES);
    if (st == MF_OK) st = time_kind(L, 1, reps, e0, e1, &tfa);
    int form = MF_FLUX_FACES;
    if (st == MF_OK && level_set_flux_form(L, MF_FLUX_LINES) == MF_OK) {
      st = time_kind(L, 1, 1, e0, e1, &tli);  // warm-up
      if (st == MF_OK) st = time_kind(L, 1, reps, e0, e1, &tli);
      if (st == MF_OK && tli < tfa) form = MF_FLUX_LINES;
    }
    if (st == MF_OK) st = level_set_flux_form(L, form);
  }
  if (st == MF_OK && L->gathers.empty()) {
    float tf = 0.f, tu = 0.f;
    if (p.precision == MF_PREC_MIXED) st = level_set_chunks(L, 1);
    if (st == MF_OK) st = time_kind(L, 1, reps, e0, e1, &tf);
    if (st == MF_OK) st = time_kind(L, 2, reps, e0, e1, &tu);
    float best = tf + tu;
    int bk = 1;
    if (p.precision == MF_PREC_MIXED && !c->dp.ct &&
        (p.time_approximation == MF_TA_RK2 || p.time_approximation == MF_TA_FIRST_ORDER)) {
      static const int ck[3] = {2, 4, 8};
      for (int q = 0; q < 3 && st == MF_OK; ++q) {
        st = level_set_chunks(L, ck[q]);
        if (st != MF_OK || L->nchunks < 2) continue;
        float ms = 0.f;
        st = time_kind(L, 4, 1, e0, e1, &ms);  // warm-up
        if (st == MF_OK) st = time_kind(L, 4, reps, e0, e1, &ms);
        if (st == MF_OK && ms < best) {
          best = ms;
          bk = L->nchunks;
        }
      }
    }
    int bt[3] = {0, 0, 0};
    if (st == MF_OK && mf::fused_supported(c->dp, p.precision, p.time_approximation)) {
      static const int c3[][3] = {{8, 8, 4}, {8, 4, 4}, {16, 8, 2}, {8, 8, 2}, {4, 4, 4}};
      static const int c2[][3] = {{16, 16, 1}, {32, 8, 1}, {16, 8, 1}, {8, 8, 1}};
      const int ncand = (sd == 3) ? 5 : 4;
      for (int q = 0; q < ncand && st == MF_OK; ++q) {
        const int* t = (sd == 3) ? c3[q] : c2[q];
        bool ok = false;
        if (level_set_tiles(L, t, &ok) != cudaSuccess) {
          st = MF_ERR_CUDA;
          break;
        }
        if (!ok) continue;
        float ms = 0.f;
        st = time_kind(L, 3, 1, e0, e1, &ms);  // warm-up
        if (st == MF_OK) st = time_kind(L, 3, reps, e0, e1, &ms);
        if (st == MF_OK && ms < best) {
          best = ms;
          for (int d = 0; d < 3; ++d) bt[d] = t[d];
        }
      }
    }
    bool fused = false;
    if (st == MF_OK && bt[0] != 0) {
      bool ok = false;
      if (level_set_tiles(L, bt, &ok) != cudaSuccess) st = MF_ERR_CUDA;
      fused = ok;
    }
    if (p.precision == MF_PREC_MIXED && st == MF_OK) st = level_set_chunks(L, fused ? 1 : bk);
    apply_schedule(L, st == MF_OK && fused);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != MF_OK) {
    mf::batch_default_threads(L->b1);
    mf::batch_default_threads(L->b2);
    mf::batch_default_threads(L->bp);
  }
  L->nparts = mf::dt_partials(L->b2);
  if ((size_t)(L->nparts + 1) * sizeof(DtPartial) > L->partials.bytes) return MF_ERR_CUDA;
  // graphs captured with the old launch shapes are rebuilt on next use
  if (L->gsync) cudaGraphExecDestroy(L->gsync);
  if (L->gasync) cudaGraphExecDestroy(L->gasync);
  L->gsync = L->gasync = nullptr;
  if (threads)
    for (int k = 0; k < 3; ++k) threads[k] = L->b2.nt[k];
  return st;
}

// ---------------------------------------------------------------------------
// problem set-up on host fabs
// ---------------------------------------------------------------------------

static inline long long hidx(const mf_fab* U, int i, int j, int k, int q) {
  int n[3];
  ext3(U->box, n);
  return (long long)(i - U->box.lo[0]) +
         (long long)n[0] * ((long long)(j - U->box.lo[1]) +
                            (long long)n[1] * ((long long)(k - U->box.lo[2]) + (long long)n[2] * q));
}

mf_status mf_init_orszag_host(const mf_params* p, mf_fab* U, const mf_box* box) {
  // ORSZAGINIT (problems/OrszagF.ChF:27-79)
  if (!p || !U || !U->data || !box || !box_contains(U->box, *box)) return MF_ERR_BAD_ARG;
  if (U->ncomp != num_cons(*p)) return MF_ERR_BAD_ARG;
  const double gamma = p->gamma, hgamma = gamma - 1.0, dx = p->dx;
  const double p0 = mf::kInv4Pi * gamma;
  const double r0 = p0 * gamma;
  const int glm = (p->divb_cleaning == 5);
  for (int k = box->lo[2]; k <= box->hi[2]; ++k)
    for (int j = box->lo[1]; j <= box->hi[1]; ++j)
      for (int i = box->lo[0]; i <= box->hi[0]; ++i) {
        double x = (i + 0.5) * dx, y = (j + 0.5) * dx;
        double Ux = -std::sin(mf::k2Pi * y);
        double Uy = std::sin(mf::k2Pi * x);
        double Bx = -std::sin(mf::k2Pi * y);
        double By = std::sin((mf::k2Pi + mf::k2Pi) * x);
        double b = mf::kInv4Pi * (Bx * Bx + By * By);
        double ke = Ux * Ux + Uy * Uy;
        double e0 = p0 / hgamma + 0.5 * (r0 * ke + b);
        double* d = U->data;
        d[hidx(U, i, j, k, 0)] = r0;
        d[hidx(U, i, j, k, 1)] = r0 * Ux;
        d[hidx(U, i, j, k, 2)] = r0 * Uy;
        d[hidx(U, i, j, k, 3)] = 0.0;
        d[hidx(U, i, j, k, 4)] = e0;
        d[hidx(U, i, j, k, 5)] = Bx;
        d[hidx(U, i, j, k, 6)] = By;
        d[hidx(U, i, j, k, 7)] = 0.0;
        if (glm) d[hidx(U, i, j, k, 8)] = 0.0;
        for (int q = 8 + glm; q < U->ncomp; ++q) d[hidx(U, i, j, k, q)] = 0.0;
      }
  return MF_OK;
}

mf_status mf_init_helio_host(const mf_params* p, const double* wp, const double* wn, mf_fab* U,
                             const mf_box* box) {
  // uniform inflow from primitive states (PRIMTOCONS_MF, srcIdeal/PatchMHDMFF.ChF:82-149)
  // plus the inner solar-wind sphere (HELIOREINIT_DEFAULT)
  if (!p || !wp || !U || !U->data || !box || !box_contains(U->box, *box)) return MF_ERR_BAD_ARG;
  if (U->ncomp != num_cons(*p)) return MF_ERR_BAD_ARG;
  if (p->n_fluids > 1 && !wn) return MF_ERR_BAD_ARG;
  const DevParams P = make_dev(*p);
  const double hg = p->gamma - 1.0, invhg = 1.0 / hg;
  const int glm = P.glm, irhon = 8 + glm;
  double u[MF_MAX_COMP];
  for (int k = box->lo[2]; k <= box->hi[2]; ++k)
    for (int j = box->lo[1]; j <= box->hi[1]; ++j)
      for (int i = box->lo[0]; i <= box->hi[0]; ++i) {
        double rho = std::max(wp[0], p->smallr);
        double uu = wp[1], vv = wp[2], ww = wp[3], pr = wp[4];
        double bx = wp[5], by = wp[6], bz = wp[7];
        double b = mf::kInv4Pi * (bx * bx + by * by + bz * bz);
        double ke = uu * uu + vv * vv + ww * ww;
        u[0] = rho;
        u[1] = rho * uu;
        u[2] = rho * vv;
        u[3] = rho * ww;
        u[4] = pr * invhg + 0.5 * (rho * ke + b);
        u[5] = bx;
        u[6] = by;
        u[7] = bz;
        if (glm) u[8] = 0.0;
        for (int f = 1; f < p->n_fluids; ++f) {
          const double* w = wn + 5 * (f - 1);
          int s = irhon + 5 * (f - 1);
          double r = std::max(w[0], p->smallr);
          double ke2 = w[1] * w[1] + w[2] * w[2] + w[3] * w[3];
          u[s] = r;
          u[s + 1] = r * w[1];
          u[s + 2] = r * w[2];
          u[s + 3] = r * w[3];
          u[s + 4] = w[4] * invhg + 0.5 * r * ke2;
        }
        // tracking surfaces: the region tracer -1 in the wind sphere, +1
        // outside (HELIOINIT, swlism/HeliosphericF.ChF:1228-1231,1302-1304);
        // the current-sheet surface of a bipolar field +1 (the component
        // reset of swlism/HeliosphericProblem.cpp:2387-2393; the sphere's
        // reset below sets +1 / -1 inside); any other surface r - R0, a
        // level set of the sphere
        if (P.nls) {
          const double x = (i + 0.5) * P.dx - P.sun_c[0], y = (j + 0.5) * P.dx - P.sun_c[1];
          const double z = (P.sd == 3) ? (k + 0.5) * P.dx - P.sun_c[2] : 0.0;
          const double r2 = x * x + y * y + z * z;
          for (int q = P.ils; q < P.nc; ++q) u[q] = std::sqrt(r2) - P.r0;
          if (P.reg_tracer) u[P.nc - 1] = (r2 <= P.r0 * P.r0) ? -1.0 : 1.0;
          if (P.reinit && P.ihcs >= 0) u[P.ihcs] = 1.0;
        }
        if (p->reinit_sphere) mf::exact::reinit_cell(P, P.dx, i, j, k, 0.0, u);
        for (int q = 0; q < U->ncomp; ++q) U->data[hidx(U, i, j, k, q)] = u[q];
      }
  return MF_OK;
}

}  // extern "C"

// Read-only view of a context for the other translation units of the library.
namespace mf {
CtxView ctx_view(const mf_ctx* c) {
  CtxView v;
  v.p = &c->p;
  v.dp = &c->dp;
  v.ng = c->ng;
  v.nc = c->nc;
  v.timeout = c->timeout;
  v.time = c->time;
  return v;
}

mf_status host_wait(cudaStream_t s, double timeout_s) { return wait_stream(s, timeout_s); }

LevelView level_view(mf_level* L) {
  LevelView v;
  v.ctx = L->ctx;
  v.p = &L->ctx->p;
  v.np = L->np;
  v.nc = L->ctx->nc;
  v.ng = L->ctx->ng;
  v.valid = &L->valid;
  v.fab = &L->fab;
  v.off = &L->off;
  v.d1 = &L->hd1;
  v.d2 = &L->hd2;
  v.U = (double*)L->U.p;
  v.s = L->s;
  return v;
}

void level_set_gathers(mf_level* L, const std::vector<FaceGather>& g) {
  L->gathers = g;
  if (L->gsync) cudaGraphExecDestroy(L->gsync);
  if (L->gasync) cudaGraphExecDestroy(L->gasync);
  L->gsync = L->gasync = nullptr;
  // the fused kernel keeps no face fluxes to gather: with gathers the level
  // steps through the split flux and update kernels, unchunked
  count_launches(L);
}

mf_status status_of_flags(unsigned flags) { return flags_status(flags); }
void level_set_time_host(mf_level* L, double time) { L->time = time; }
}  // namespace mf
