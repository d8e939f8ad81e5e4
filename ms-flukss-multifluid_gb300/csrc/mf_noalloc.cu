// mf_noalloc.cu - a patch update that allocates nothing.
//
// Some callers cannot call cudaMalloc when they advance a patch: processes
// whose device memory is handed in full to a pool allocator that must not be
// bypassed (the host application owns every byte of HBM), and real-time or
// serving loops that forbid any allocation after start-up (an allocation can
// synchronise the device and stalls the loop for an unbounded time).
// mf_patch_update_noalloc serves them: it runs the same kernels as
// mf_patch_update, with every scratch buffer (RK2 predictor, primitive
// state, face fluxes, face-normal B, stage descriptors, step state, dt
// partials) carved from one file-scope device array of
// MF_NOALLOC_SCRATCH_BYTES.  The caller still passes the state, the optional
// flux and divB outputs and the stream.
//
// The array is loaded with the library's device code, so every GPU that loads
// the library holds it until the process exits.  Its device address is looked
// up once per device, at the first call on that device with the device
// current (cudaGetSymbolAddress); that first call should come before any
// stream capture, and the device must not be reset (cudaDeviceReset) while
// the library is in use, since the address is kept.  All calls share the
// array and it keeps the last call's contents; the step state (error flags
// included) is rewritten at the start of every call, and everything else is
// fully written before it is read.  Calls that overlap on the GPU (same
// device, different streams or threads) race on the array and must be
// serialised by the caller.
#include <cmath>
#include <cstring>
#include <mutex>

#include "mf_internal.h"
#include "mf_kernels.cuh"

static __device__ __align__(256) unsigned char g_noalloc_scratch[MF_NOALLOC_SCRATCH_BYTES];

namespace {

using mf::DtPartial;
using mf::StageBuffers;
using mf::StageDesc;
using mf::StepState;

constexpr int kMaxDevices = 64;
void* g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

// Device address of the scratch array on the current device.  The array's
// name is a host-side stand-in, not a device address; the address comes from
// cudaGetSymbolAddress, queried once per device with that device current.
mf_status scratch_base(void** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess) return MF_ERR_CUDA;
  if (dev < 0 || dev >= kMaxDevices) return MF_ERR_UNSUPPORTED;
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return MF_ERR_CUDA;
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return MF_OK;
}

long long cells(const mf_box& b) {
  long long n = 1;
  for (int d = 0; d < 3; ++d) n *= (long long)(b.hi[d] - b.lo[d] + 1);
  return n;
}

mf_box grow(mf_box b, int n, int sd) {
  for (int d = 0; d < sd; ++d) {
    b.lo[d] -= n;
    b.hi[d] += n;
  }
  return b;
}

mf_box isect(const mf_box& a, const mf_box& b) {
  mf_box r;
  for (int d = 0; d < 3; ++d) {
    r.lo[d] = a.lo[d] > b.lo[d] ? a.lo[d] : b.lo[d];
    r.hi[d] = a.hi[d] < b.hi[d] ? a.hi[d] : b.hi[d];
  }
  return r;
}

mf_box nodes(mf_box b, int d) {
  b.hi[d] += 1;
  return b;
}

bool contains(const mf_box& o, const mf_box& i) {
  for (int d = 0; d < 3; ++d)
    if (i.lo[d] < o.lo[d] || i.hi[d] > o.hi[d]) return false;
  return true;
}

bool empty(const mf_box& b) {
  for (int d = 0; d < 3; ++d)
    if (b.hi[d] < b.lo[d]) return true;
  return false;
}

mf_box and_domain(mf_box b, const mf_params& p) {
  for (int d = 0; d < p.space_dim; ++d) {
    if (p.periodic[d]) continue;
    if (b.lo[d] < p.domain_lo[d]) b.lo[d] = p.domain_lo[d];
    if (b.hi[d] > p.domain_hi[d]) b.hi[d] = p.domain_hi[d];
  }
  return b;
}

void fill(StageDesc& D, const mf_box& fab, const mf_box& v, const mf_box& w) {
  std::memset(&D, 0, sizeof(D));
  for (int d = 0; d < 3; ++d) {
    D.flo[d] = fab.lo[d];
    D.fn[d] = fab.hi[d] - fab.lo[d] + 1;
    D.vlo[d] = v.lo[d];
    D.vn[d] = v.hi[d] - v.lo[d] + 1;
    D.wlo[d] = w.lo[d];
    D.wn[d] = w.hi[d] - w.lo[d] + 1;
  }
}

size_t up256(size_t n) { return (n + 255) & ~size_t(255); }

#define NA_CUDA(x)                                                         \
  do {                                                                     \
    if ((x) != cudaSuccess) return MF_ERR_CUDA;                            \
  } while (0)

}  // namespace

extern "C" mf_status mf_patch_update_noalloc(mf_ctx* ctx, mf_fab* U, const mf_box* valid,
                                             double dt, mf_fab* F, mf_fab* divB, double* new_dt,
                                             int min_cell[3], void* stream) {
  if (!ctx || !U || !U->data || !valid) return MF_ERR_BAD_ARG;
  const mf::CtxView cv = mf::ctx_view(ctx);
  const mf_params& p = *cv.p;
  const int sd = p.space_dim, nc = cv.nc, ng = cv.ng;
  if (U->ncomp != nc || empty(*valid)) return MF_ERR_BAD_ARG;
  if (!(dt > 0.0) || !std::isfinite(dt)) return MF_ERR_BAD_ARG;
  for (int d = sd; d < 3; ++d)
    if (valid->lo[d] != 0 || valid->hi[d] != 0 || U->box.lo[d] != 0 || U->box.hi[d] != 0)
      return MF_ERR_BAD_ARG;
  for (int d = 0; d < sd; ++d)
    if (!p.periodic[d] && (valid->lo[d] < p.domain_lo[d] || valid->hi[d] > p.domain_hi[d]))
      return MF_ERR_BAD_ARG;
  if (!contains(U->box, grow(*valid, ng, sd))) return MF_ERR_BAD_ARG;

  if (p.time_approximation == MF_TA_HANCOCK) return MF_ERR_UNSUPPORTED;
  if (p.divb_cleaning >= 1 && p.divb_cleaning <= 3) return MF_ERR_UNSUPPORTED;  // CT
  const bool rk2 = (p.time_approximation == MF_TA_RK2);
  const int mixed = (p.precision == MF_PREC_MIXED);
  const size_t rs = mf::flux_bytes(p.precision);
  const long long fabn = cells(U->box);
  const mf_box v2 = and_domain(*valid, p);
  const mf_box v1 = rk2 ? and_domain(grow(*valid, 2, sd), p) : v2;
  const mf_box w1 = isect(grow(v1, 2, sd), U->box);
  const mf_box w2 = isect(grow(v2, 2, sd), U->box);
  if (divB && divB->data && !contains(divB->box, v2)) return MF_ERR_BAD_ARG;
  if (F) {
    for (int d = 0; d < sd; ++d) {
      const mf_box b2 = nodes(v2, d);
      if (!F[d].data || F[d].ncomp != nc) return MF_ERR_BAD_ARG;
      for (int e = 0; e < 3; ++e)
        if (F[d].box.lo[e] != b2.lo[e] || F[d].box.hi[e] != b2.hi[e]) return MF_ERR_BAD_ARG;
    }
  }

  // layout of the scratch array
  size_t off = 0;
  const size_t o_pred = off;
  if (rk2) off += up256(sizeof(double) * fabn * nc);
  const size_t o_w = off;
  off += up256(sizeof(double) * fabn * nc);
  size_t o_f1[3] = {0, 0, 0}, o_b1[3] = {0, 0, 0}, o_f2[3] = {0, 0, 0}, o_b2[3] = {0, 0, 0};
  long long nf1[3] = {0, 0, 0}, nf2[3] = {0, 0, 0};
  for (int d = 0; d < sd; ++d) {
    nf1[d] = cells(nodes(v1, d));
    nf2[d] = cells(nodes(v2, d));
    o_f1[d] = off;
    off += up256(rs * nf1[d] * nc);
    o_b1[d] = off;
    off += up256(rs * nf1[d]);
    if (rk2) {
      o_f2[d] = off;
      off += up256(rs * nf2[d] * nc);
      o_b2[d] = off;
      off += up256(rs * nf2[d]);
    }
  }
  const size_t o_desc = off;  // two stage descs, then the run's parameters
  off += up256(sizeof(StageDesc) * 2 + sizeof(mf::RunParams));
  const size_t o_state = off;
  off += up256(sizeof(StepState));
  const long long nparts = (cells(v2) + mf::kBlock - 1) / mf::kBlock + 1;
  const size_t o_parts = off;
  off += up256(sizeof(DtPartial) * nparts);
  if (off > (size_t)MF_NOALLOC_SCRATCH_BYTES) return MF_ERR_SCRATCH_LIMIT;

  void* basev = nullptr;
  mf_status st = scratch_base(&basev);
  if (st != MF_OK) return st;
  unsigned char* base = (unsigned char*)basev;
  cudaStream_t s = (cudaStream_t)stream;

  // descriptors and step state travel from host stack memory: a copy from
  // pageable memory returns once the data has been taken
  struct {
    StageDesc d[2];
    mf::RunParams r;
  } hblk;
  StageDesc* hd = hblk.d;
  fill(hd[0], U->box, v1, w1);
  fill(hd[1], U->box, v2, w2);
  StepState hs;
  std::memset(&hs, 0, sizeof(hs));
  hs.dt = dt;
  hs.time = cv.time;
  hs.ch = p.dedner_ch;
  hs.cp = p.dedner_cp;
  StageDesc* dd = (StageDesc*)(base + o_desc);
  mf::Batch b1, b2;
  std::memset(&b1, 0, sizeof(b1));
  std::memset(&b2, 0, sizeof(b2));
  mf::batch_offsets(&hd[0], 1, sd, b1);  // the fab-size check keeps counts < 2^31
  mf::batch_offsets(&hd[1], 1, sd, b2);
  b1.desc = dd;
  b2.desc = dd + 1;
  mf::batch_default_threads(b1);
  mf::batch_default_threads(b2);
  mf::RunParams* druns = (mf::RunParams*)(base + o_desc + sizeof(StageDesc) * 2);
  b1.runs = b2.runs = druns;
  b1.nruns = b2.nruns = 1;
  hblk.r = mf::run_params_of(*cv.dp);
  hblk.r.d0 = 0;
  hblk.r.nd = 1;
  hblk.r.v0 = 0;
  hblk.r.v1 = b2.tot_v;
  StepState* ds = (StepState*)(base + o_state);
  DtPartial* parts = (DtPartial*)(base + o_parts);
  NA_CUDA(cudaMemcpyAsync(dd, &hblk, sizeof(hblk), cudaMemcpyHostToDevice, s));
  NA_CUDA(cudaMemcpyAsync(ds, &hs, sizeof(hs), cudaMemcpyHostToDevice, s));

  StageBuffers B;
  std::memset(&B, 0, sizeof(B));
  B.w = (double*)(base + o_w);
  int nb = 0;
  if (divB && divB->data) {
    for (int d = 0; d < 3; ++d) {
      B.divb_lo[d] = divB->box.lo[d];
      B.divb_n[d] = divB->box.hi[d] - divB->box.lo[d] + 1;
    }
  }
  if (rk2) {
    double* pred = (double*)(base + o_pred);
    NA_CUDA(cudaMemcpyAsync(pred, U->data, sizeof(double) * fabn * nc, cudaMemcpyDeviceToDevice,
                            s));
    B.uin = U->data;
    B.uout = pred;
    for (int d = 0; d < 3; ++d) {
      B.f[d] = d < sd ? (void*)(base + o_f1[d]) : nullptr;
      B.bn[d] = d < sd ? (void*)(base + o_b1[d]) : nullptr;
    }
    NA_CUDA(mf::launch_stage(*cv.dp, p.precision, B, b1, 0, 1.0, ds, parts, &nb, s));
    B.uin = pred;
    B.uout = U->data;
    B.uold = U->data;
    for (int d = 0; d < 3; ++d) {
      B.f[d] = d < sd ? (void*)(base + o_f2[d]) : nullptr;
      B.bn[d] = d < sd ? (void*)(base + o_b2[d]) : nullptr;
    }
    B.divb = (divB && divB->data) ? divB->data : nullptr;
    NA_CUDA(mf::launch_stage(*cv.dp, p.precision, B, b2, mf::kStageAverage | mf::kStageDt, 0.5,
                             ds, parts, &nb, s));
  } else {
    B.uin = U->data;
    B.uout = U->data;
    for (int d = 0; d < 3; ++d) {
      B.f[d] = d < sd ? (void*)(base + o_f1[d]) : nullptr;
      B.bn[d] = d < sd ? (void*)(base + o_b1[d]) : nullptr;
    }
    B.divb = (divB && divB->data) ? divB->data : nullptr;
    NA_CUDA(mf::launch_stage(*cv.dp, p.precision, B, b2, mf::kStageDt, 1.0, ds, parts, &nb, s));
  }
  NA_CUDA(mf::launch_finalize(*cv.dp, parts, b2, b2.nt[2], ds, 0, s));
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
      const mf_box b2 = nodes(v2, d), b1 = nodes(v1, d);
      f2p[d] = rk2 ? (const void*)(base + o_f2[d]) : (const void*)(base + o_f1[d]);
      f1p[d] = rk2 ? (const void*)(base + o_f1[d]) : nullptr;
      fo[d] = F[d].data;
      for (int e = 0; e < 3; ++e) {
        f2lo[d][e] = b2.lo[e];
        f2n[d][e] = b2.hi[e] - b2.lo[e] + 1;
        f1lo[d][e] = b1.lo[e];
        f1n[d][e] = b1.hi[e] - b1.lo[e] + 1;
        olo[d][e] = b2.lo[e];
        on[d][e] = b2.hi[e] - b2.lo[e] + 1;
      }
    }
    NA_CUDA(mf::launch_flux_out(mixed, sd, nc, f2p, f2lo, f2n, f1p, f1lo, f1n, fo, olo, on, s));
  }
  // bounded wait for the step (MF_ERR_TIMEOUT after the context's wait
  // limit, as every host wait of the library), then the step state: a copy
  // into pageable memory returns once the data has arrived
  st = mf::host_wait(s, cv.timeout);
  if (st != MF_OK) return st;
  NA_CUDA(cudaMemcpyAsync(&hs, ds, sizeof(hs), cudaMemcpyDeviceToHost, s));
  if (new_dt) *new_dt = hs.dt_min;
  if (min_cell) {
    const int n0 = valid->hi[0] - valid->lo[0] + 1, n1 = valid->hi[1] - valid->lo[1] + 1;
    int idx = hs.min_idx;
    if (idx < 0 || idx == 0x7fffffff) idx = 0;
    min_cell[0] = valid->lo[0] + idx % n0;
    min_cell[1] = valid->lo[1] + (idx / n0) % n1;
    min_cell[2] = valid->lo[2] + idx / (n0 * n1);
  }
  if (hs.flags & mf::kFlagNonFinite) return MF_ERR_NONFINITE;
  if (hs.flags & mf::kFlagBadDt) return MF_ERR_NEG_STATE;
  return MF_OK;
}
