// mf_amr_exact.cu - coarse-fine coupling of a subcycled hierarchy of levels
// and the hierarchy time step (C ABI: mf_hier_*).
//
// For levels of patches resident on the device this restates:
//  * PiecewiseLinearFillPatchMHDAM::fillInterp
//    (srcIdeal/PiecewiseLinearFillPatchMHDAM.cpp:120-900; INTERPLIMIT_V and
//    interp_divB_0, srcIdeal/FineInterpMHDAMF.ChF:235-555): the fine ghost
//    cells over coarse cells that no coarsened fine box covers get the coarse
//    state interpolated in time (between the coarse state before and after
//    the coarse step) and linearly in space with limited slopes;
//  * LevelFluxRegister incrementCoarse / incrementFine / reflux as used by
//    AMRLevelIdealMHD::step and postTimeStep
//    (srcIdeal/AMRLevelIdealMHD.cpp:1276-1308, 1633-1642);
//  * CoarseAverageExt::averageToCoarse (src/CoarseAverageExt.cpp:117-192,
//    src/CoarseAverageExtF.ChF:10-50);
//  * AMR_MHDAM::timeStep (srcIdeal/AMR_MHDAM.cpp:1707-1880) with
//    AMRLevelIdealMHD::advance / preTimeStep / postTimeStep.
//
// Once per pair of levels the host turns the box geometry into flat lists
// over the levels' flat device arrays (interpolation sites and targets,
// register faces, reflux cells, averaged cells); every operation is then one
// flat kernel over its list.  The flux registers are fed by face gathers that
// run inside the level steps.  Compiled without fused multiply-adds: each
// value rounds as in the CPU restatement.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <unordered_map>
#include <vector>

#include "mf_internal.h"

namespace mf {
namespace {

constexpr int kThreads = 256;

// ---------------------------------------------------------------------------
// device lists
// ---------------------------------------------------------------------------
struct NbCell {      // a coarse cell read by the interpolation
  long long off;     // offset of component 0 in the coarse level's U
  int cs, pad;       // component stride (cells of its fab)
};
struct CfSite {      // a coarse cell fine ghosts are interpolated from
  int nb[27];        // NbCell slots of the 3^D neighbourhood, centre at 13
  int type[3];       // slope per direction: 0 centred, 1 low-sided, 2 high-sided
  int limit;         // limited (not on a non-periodic domain edge)
};
struct CfTarget {    // a fine ghost cell
  long long off;
  int cs, site;
  int iv[3], pad;    // fine cell index (unwrapped)
};
struct RefluxCell {  // a coarse cell next to the fine region
  long long off;
  int cs, first, count, pad;
};
struct RefluxTerm {  // a register face acting on it (ordered by direction, side)
  int reg, sign;
};
struct AvgCell {     // a coarse cell under a fine patch
  long long coff, foff;
  int ccs, fcs, sy, sz;
};
struct CfConsts {
  double alpha, c1c, c1s, dxc, dxf, coeff;
  int nc, sd, r, divb, nsites, nnb;
};

__device__ __forceinline__ int floordiv_d(int a, int r) {
  return (a >= 0) ? a / r : -((-a + r - 1) / r);
}

// minmod (src/reconstructionF.ChF:4-14)
__device__ __forceinline__ double minmod_d(double A, double B) {
  const double signA = copysign(1.0, A);
  return signA * fmax(0.0, fmin(fabs(A), signA * B));
}

// interp_divB_0 (srcIdeal/FineInterpMHDAMF.ChF:449-555): correct the limited
// slopes d(Bx)/dx, d(By)/dy, d(Bz)/dz of one coarse cell towards a
// divergence-free linear profile.
__device__ void divb_correct(int sd, double& sx, double& sy, double& sz) {
  const double eps_divB = 1.0e-8;
  const double DBXDX = sx, DBYDY = sy, DBZDZ = (sd == 3) ? sz : 0.0;
  const double fact = (sd == 3) ? -1.0 / (1.0 + 1.0 + 1.0) : -1.0 / (1.0 + 1.0);
  const double divB = (sd == 3) ? DBXDX + DBYDY + DBZDZ : DBXDX + DBYDY;
  double del = fact * divB;
  double adel = fabs(del);
  if (!(adel > eps_divB)) return;
  double delX = minmod_d(-DBXDX, del), delY = minmod_d(-DBYDY, del);
  double delZ = (sd == 3) ? minmod_d(-DBZDZ, del) : 0.0;
  double del2 = (sd == 3) ? delX + delY + delZ : delX + delY;
  if (fabs(del2) < fabs(divB)) {
    if (sd == 2) {
      delX = minmod_d(DBXDX, -DBYDY);
      delY = -delX;
      delX = delX - DBXDX;
      delY = delY - DBYDY;
    } else if (fabs(delX) < adel) {
      del = -0.5 * (delX + divB);
      delY = minmod_d(-DBYDY, del);
      delZ = minmod_d(-DBZDZ, del);
      del2 = delX + delY + delZ;
      if (fabs(del2) < fabs(divB)) {
        if (fabs(delY) < adel)
          delZ = -(divB + delX + delY);
        else
          delY = -(divB + delX + delZ);
      }
    } else if (fabs(delY) < adel) {
      del = -0.5 * (delY + divB);
      delX = minmod_d(-DBXDX, del);
      delZ = minmod_d(-DBZDZ, del);
      del2 = delX + delY + delZ;
      if (fabs(del2) < fabs(divB)) {
        if (fabs(delX) < adel)
          delZ = -(divB + delX + delY);
        else
          delX = -(divB + delY + delZ);
      }
    } else {
      del = -0.5 * (delZ + divB);
      adel = fabs(del);
      delX = minmod_d(-DBXDX, del);
      delY = minmod_d(-DBYDY, del);
      del2 = delX + delY + delZ;
      if (fabs(del2) < fabs(divB)) {
        if (fabs(delX) < adel)
          delY = -(divB + delX + delZ);
        else
          delX = -(divB + delY + delZ);
      }
    }
  }
  sx = sx + delX;
  sy = sy + delY;
  if (sd == 3) sz = sz + delZ;
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
// the coarse values the interpolation reads, before the coarse step
__global__ void k_cf_snapshot(const double* __restrict__ U, const NbCell* __restrict__ nb, int nnb,
                              int nc, double* __restrict__ old) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nnb * nc) return;
  const int n = (int)(t % nnb), q = (int)(t / nnb);
  old[t] = U[nb[n].off + (long long)q * nb[n].cs];
}

// One coarse site per thread: the time-interpolated value and the limited
// slopes of every component (sv[(q * 4 + k) * nsites + site], k = 0 value,
// 1..3 slopes).
__global__ void k_cf_sites(const double* __restrict__ U, const NbCell* __restrict__ nb,
                           const double* __restrict__ old, const CfSite* __restrict__ sites,
                           const CfConsts K, double* __restrict__ sv) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= K.nsites) return;
  const CfSite& S = sites[s];
  const int ns = K.nsites;
  const double om = 1.0 - K.alpha;
  for (int q = 0; q < K.nc; ++q) {
    auto val = [&](int slot) -> double {
      const NbCell& c = nb[slot];
      const double vn = U[c.off + (long long)q * c.cs];
      const double vo = old[(long long)q * K.nnb + slot];
      if (K.alpha == 1.0) return vn;
      if (K.alpha == 0.0) return vo;
      return vn * K.alpha + vo * om;
    };
    const double v0 = val(S.nb[13]);
    double sl[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < K.sd; ++d) {
      const int st = (d == 0) ? 1 : (d == 1) ? 3 : 9;
      if (S.type[d] == 0)
        sl[d] = K.c1c * (val(S.nb[13 + st]) - val(S.nb[13 - st]));
      else if (S.type[d] == 1)
        sl[d] = K.c1s * (v0 - val(S.nb[13 - st]));
      else
        sl[d] = K.c1s * (val(S.nb[13 + st]) - v0);
    }
    if (S.limit) {
      double smax = v0, smin = v0;
      const int a0 = (K.sd == 3) ? 0 : 9, a1 = (K.sd == 3) ? 27 : 18;
      for (int a = a0; a < a1; ++a) {
        const double v = val(S.nb[a]);
        smax = fmax(smax, v);
        smin = fmin(smin, v);
      }
      const double dsum = (K.sd == 3) ? 0.5 * (fabs(sl[0] * K.dxc) + fabs(sl[1] * K.dxc) +
                                                fabs(sl[2] * K.dxc))
                                       : 0.5 * (fabs(sl[0] * K.dxc) + fabs(sl[1] * K.dxc));
      double eta = fmin(smax - v0, v0 - smin);
      if (eta <= 1.0e-9 * fabs(smax))
        eta = 0.0;
      else if (dsum > eta)
        eta = eta / dsum;
      else
        eta = 1.0;
      for (int d = 0; d < K.sd; ++d) sl[d] = eta * sl[d];
    }
    sv[(long long)(q * 4) * ns + s] = v0;
    for (int d = 0; d < 3; ++d) sv[(long long)(q * 4 + 1 + d) * ns + s] = sl[d];
  }
  if (K.divb && S.limit) {
    const int iBX = 5;
    double* px = sv + (long long)(iBX * 4 + 1) * ns + s;
    double* py = sv + (long long)((iBX + 1) * 4 + 2) * ns + s;
    double* pz = sv + (long long)((iBX + 2) * 4 + 3) * ns + s;
    double x = *px, y = *py, z = (K.sd == 3) ? *pz : 0.0;
    divb_correct(K.sd, x, y, z);
    *px = x;
    *py = y;
    if (K.sd == 3) *pz = z;
  }
}

// the fine ghost cells: constant part, then the linear term of each direction
__global__ void k_cf_fill(const CfTarget* __restrict__ tg, int nt, const double* __restrict__ sv,
                          const CfConsts K, double* __restrict__ Uf) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nt * K.nc) return;
  const int i = (int)(t % nt), q = (int)(t / nt);
  const CfTarget& T = tg[i];
  const int ns = K.nsites;
  double v = sv[(long long)(q * 4) * ns + T.site];
  for (int d = 0; d < K.sd; ++d) {
    const int c = floordiv_d(T.iv[d], K.r);
    const double icoef = K.dxf * (T.iv[d] + 0.5) - K.dxc * (c + 0.5);
    v = v + K.coeff * icoef * sv[(long long)(q * 4 + 1 + d) * ns + T.site];
  }
  Uf[T.off + (long long)q * T.cs] = v;
}

template <typename R>
__global__ void k_face_gather(const R* __restrict__ F0, const R* __restrict__ F1,
                              const R* __restrict__ F2, const FaceRef* __restrict__ refs, int n,
                              int nc, int mode, double* __restrict__ out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * nc) return;
  const int i = (int)(t % n), q = (int)(t / n);
  const FaceRef& f = refs[i];
  const R* F = (f.dir == 0) ? F0 : (f.dir == 1) ? F1 : F2;
  const int slot = (mode == 0) ? 0 : 1;
  const double v = (double)F[f.off[slot] + (long long)q * f.cs[slot]];
  if (mode == 1)
    out[t] = (out[t] + v) * 0.5;  // updateState's RK2 flux: (F1 + F2) * 0.5
  else
    out[t] = v;
}

// incrementCoarse: register = -dt * coarse flux
__global__ void k_reg_coarse(double* __restrict__ reg, const double* __restrict__ rf,
                             long long n, double mdt) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  reg[t] = 0.0 + mdt * rf[t];
}

// incrementFine: register += dt / r^(D-1) * each fine flux on the face,
// the first transverse direction fastest
__global__ void k_reg_fine(double* __restrict__ reg, const double* __restrict__ rf, int n, int S,
                           int nc, double s) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * nc) return;
  const int i = (int)(t % n), q = (int)(t / n);
  double r = reg[t];
  const double* f = rf + (long long)q * n * S + (long long)i * S;
  for (int k = 0; k < S; ++k) r = r + s * f[k];
  reg[t] = r;
}

// reflux with scale -1 and the inverse cell size: U -= reg/dx below the fine
// region, U += reg/dx above it
__global__ void k_reflux(double* __restrict__ U, const RefluxCell* __restrict__ cells, int ncell,
                         const RefluxTerm* __restrict__ terms, const double* __restrict__ reg,
                         int nreg, int nc, double invdx) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)ncell * nc) return;
  const int i = (int)(t % ncell), q = (int)(t / ncell);
  const RefluxCell& c = cells[i];
  double* u = U + c.off + (long long)q * c.cs;
  double v = *u;
  for (int k = c.first; k < c.first + c.count; ++k) {
    const double rg = reg[(long long)q * nreg + terms[k].reg];
    v = (terms[k].sign > 0) ? v + invdx * rg : v - invdx * rg;
  }
  *u = v;
}

// AVERAGEWITHVOLUMES: volume-weighted mean of the r^D fine cells
__global__ void k_average(const double* __restrict__ Uf, double* __restrict__ Uc,
                          const AvgCell* __restrict__ cells, int n, int nc, int r, int sd,
                          double vol) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)n * nc) return;
  const int i = (int)(t % n), q = (int)(t / n);
  const AvgCell& a = cells[i];
  const double* f = Uf + a.foff + (long long)q * a.fcs;
  double sum = 0.0, volc = 0.0;
  const int rk = (sd == 3) ? r : 1;
  for (int kk = 0; kk < rk; ++kk)
    for (int jj = 0; jj < r; ++jj)
      for (int ii = 0; ii < r; ++ii) {
        sum = sum + vol * f[ii + (long long)jj * a.sy + (long long)kk * a.sz];
        volc = volc + vol;
      }
  Uc[a.coff + (long long)q * a.ccs] = sum / volc;
}

inline unsigned blocks(long long n, int t = kThreads) { return (unsigned)((n + t - 1) / t); }

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct DBuf {
  void* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  cudaError_t put(const void* src, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (bytes > n) {
      if (p) cudaFree(p);
      p = nullptr;
      n = 0;
      cudaError_t e = cudaMalloc(&p, bytes);
      if (e != cudaSuccess) return e;
      n = bytes;
    }
    return src ? cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice) : cudaMemset(p, 0, bytes);
  }
  template <typename T>
  cudaError_t put(const std::vector<T>& v) {
    return v.empty() ? put(nullptr, 16) : put(v.data(), sizeof(T) * v.size());
  }
  ~DBuf() {
    if (p) cudaFree(p);
  }
};

inline int imod(int a, int n) {
  int m = a % n;
  return m < 0 ? m + n : m;
}
inline int floordiv(int a, int r) { return (a >= 0) ? a / r : -((-a + r - 1) / r); }

inline long long loc3(const int lo[3], const int n[3], const int c[3]) {
  return (c[0] - lo[0]) + (long long)n[0] * ((c[1] - lo[1]) + (long long)n[1] * (c[2] - lo[2]));
}

inline bool in_box(const mf_box& b, const int c[3]) {
  return c[0] >= b.lo[0] && c[0] <= b.hi[0] && c[1] >= b.lo[1] && c[1] <= b.hi[1] &&
         c[2] >= b.lo[2] && c[2] <= b.hi[2];
}

// Cells of a level's domain, periodic images folded in.
struct DomainMap {
  int sd = 3, lo[3] = {0, 0, 0}, n[3] = {1, 1, 1}, per[3] = {0, 0, 0};
  long long size = 0;
  void init(const mf_params& p) {
    sd = p.space_dim;
    size = 1;
    for (int d = 0; d < 3; ++d) {
      lo[d] = (d < sd) ? p.domain_lo[d] : 0;
      n[d] = (d < sd) ? p.domain_hi[d] - p.domain_lo[d] + 1 : 1;
      per[d] = (d < sd) ? p.periodic[d] : 1;
      size *= n[d];
    }
  }
  // linear index of the periodic image of c (w: its indices); -1 outside a
  // non-periodic side
  long long wrap(const int c[3], int w[3]) const {
    for (int d = 0; d < 3; ++d) {
      if (d >= sd) {
        if (c[d] != 0) return -1;
        w[d] = 0;
        continue;
      }
      if (per[d])
        w[d] = lo[d] + imod(c[d] - lo[d], n[d]);
      else if (c[d] < lo[d] || c[d] >= lo[d] + n[d])
        return -1;
      else
        w[d] = c[d];
    }
    return (w[0] - lo[0]) + (long long)n[0] * ((w[1] - lo[1]) + (long long)n[1] * (w[2] - lo[2]));
  }
};

mf_box coarsen_box(mf_box b, int r, int sd) {
  for (int d = 0; d < sd; ++d) {
    b.lo[d] = floordiv(b.lo[d], r);
    b.hi[d] = floordiv(b.hi[d], r);
  }
  return b;
}

mf_box grow_box(mf_box b, int g, int sd) {
  for (int d = 0; d < sd; ++d) {
    b.lo[d] -= g;
    b.hi[d] += g;
  }
  return b;
}

mf_box clip_domain(mf_box b, const mf_params& p) {
  for (int d = 0; d < p.space_dim; ++d) {
    if (p.periodic[d]) continue;
    b.lo[d] = std::max(b.lo[d], p.domain_lo[d]);
    b.hi[d] = std::min(b.hi[d], p.domain_hi[d]);
  }
  return b;
}

// A face (node index along dir) of patch b in both stage layouts.
bool face_ref(const LevelView& v, int b, int dir, const int node[3], int rk2, FaceRef& out) {
  out.dir = dir;
  out.pad = 0;
  for (int slot = 0; slot < 2; ++slot) {
    const std::vector<StageDesc>& ds = (slot == 0 && rk2) ? *v.d1 : *v.d2;
    const StageDesc& D = ds[b];
    int fnb[3] = {D.vn[0], D.vn[1], D.vn[2]};
    fnb[dir] += 1;
    for (int e = 0; e < 3; ++e)
      if (node[e] < D.vlo[e] || node[e] >= D.vlo[e] + fnb[e]) return false;
    out.off[slot] = D.f_off[dir] + loc3(D.vlo, fnb, node);
    out.cs[slot] = fnb[0] * fnb[1] * fnb[2];
  }
  return true;
}

}  // namespace
}  // namespace mf

using namespace mf;

// Coupling of a level with the next finer one.
struct mf_cf {
  mf_level *lc = nullptr, *lf = nullptr;
  LevelView vc, vf;
  int r = 2, nc = 0, sd = 3, divb = 0;
  int ncons = 0;  // fluid components: the flux registers skip the tracking surfaces
  int nnb = 0, nsites = 0, ntg = 0, nreg = 0, nsub = 1, nrc = 0, navg = 0;
  double c1c = 0, c1s = 0, dxc = 0, dxf = 0, coeff = 0, invdx = 0, vol = 0;
  DBuf nb, sites, tg, old, sv;     // interpolation
  DBuf cref, fref, rfc, rff, reg;  // flux register
  DBuf rcell, rterm;               // reflux
  DBuf avg;                        // average down
  FaceGather gc, gf;               // gathers run by the level steps
};

struct mf_hier {
  std::vector<mf_level*> lv;
  std::vector<int> ratio;
  std::vector<mf_cf*> cf;
  std::vector<double> t, dt, ndt;
  cudaStream_t s = nullptr;
  int launches = 0;
  double last_dt0 = 0.0, last_new_dt = 0.0;  // the last mf_hier_step (assignDt inputs)
};

static mf_status cuda_status(cudaError_t e) {
  return e == cudaSuccess ? MF_OK : (e == cudaErrorMemoryAllocation ? MF_ERR_OOM : MF_ERR_CUDA);
}
#define MF_CUDA(x)                                 \
  do {                                             \
    cudaError_t e_ = (x);                          \
    if (e_ != cudaSuccess) return cuda_status(e_); \
  } while (0)

// Geometry of one pair of levels into the flat lists.  MF_ERR_BAD_ARG when
// the fine level is not properly nested (a coarse cell the interpolation,
// the registers or the averaging needs is not a coarse valid cell) or a fine
// box is not aligned to the refinement ratio.
static mf_status build_cf(mf_cf* C) {
  const LevelView &vc = C->vc, &vf = C->vf;
  const mf_params &pc = *vc.p, &pf = *vf.p;
  const int sd = pc.space_dim, r = C->r, ng = vf.ng;
  if (pf.space_dim != sd || vf.nc != vc.nc || r < 2) return MF_ERR_BAD_ARG;
  for (int d = 0; d < sd; ++d) {
    if (pf.domain_lo[d] != pc.domain_lo[d] * r ||
        pf.domain_hi[d] - pf.domain_lo[d] + 1 != (pc.domain_hi[d] - pc.domain_lo[d] + 1) * r ||
        pf.periodic[d] != pc.periodic[d])
      return MF_ERR_BAD_ARG;
  }
  const int nc = vc.nc;
  const int rk2c = (pc.time_approximation == MF_TA_RK2);
  const int rk2f = (pf.time_approximation == MF_TA_RK2);
  DomainMap dm;
  dm.init(pc);
  if (dm.size > (1LL << 28)) return MF_ERR_UNSUPPORTED;
  std::vector<int> cpatch(dm.size, -1);
  std::vector<unsigned char> cfine(dm.size, 0);
  int w[3];
  for (int b = 0; b < vc.np; ++b) {
    const mf_box& B = (*vc.valid)[b];
    for (int k = B.lo[2]; k <= B.hi[2]; ++k)
      for (int j = B.lo[1]; j <= B.hi[1]; ++j)
        for (int i = B.lo[0]; i <= B.hi[0]; ++i) {
          int c[3] = {i, j, k};
          long long l = dm.wrap(c, w);
          if (l < 0) return MF_ERR_BAD_ARG;
          cpatch[l] = b;
        }
  }
  for (int f = 0; f < vf.np; ++f) {
    const mf_box& B = (*vf.valid)[f];
    for (int d = 0; d < sd; ++d)
      if (imod(B.lo[d], r) != 0 || imod(B.hi[d] + 1, r) != 0) return MF_ERR_BAD_ARG;
    mf_box cb = coarsen_box(B, r, sd);
    for (int k = cb.lo[2]; k <= cb.hi[2]; ++k)
      for (int j = cb.lo[1]; j <= cb.hi[1]; ++j)
        for (int i = cb.lo[0]; i <= cb.hi[0]; ++i) {
          int c[3] = {i, j, k};
          long long l = dm.wrap(c, w);
          if (l < 0) return MF_ERR_BAD_ARG;
          cfine[l] = 1;
        }
  }
  auto coarse_loc = [&](long long lin, const int wc[3], long long& off, int& cs) -> bool {
    const int b = cpatch[lin];
    if (b < 0) return false;
    const mf_box& fb = (*vc.fab)[b];
    int n[3] = {fb.hi[0] - fb.lo[0] + 1, fb.hi[1] - fb.lo[1] + 1, fb.hi[2] - fb.lo[2] + 1};
    off = (*vc.off)[b] + loc3(fb.lo, n, wc);
    cs = n[0] * n[1] * n[2];
    return true;
  };

  // --- interpolation sites and targets
  std::vector<NbCell> nbs;
  std::vector<CfSite> sites;
  std::vector<CfTarget> tgs;
  std::unordered_map<long long, int> nbmap, sitemap;
  auto nb_slot = [&](long long lin, const int wc[3]) -> int {
    auto it = nbmap.find(lin);
    if (it != nbmap.end()) return it->second;
    NbCell c;
    c.pad = 0;
    if (!coarse_loc(lin, wc, c.off, c.cs)) return -1;
    const int id = (int)nbs.size();
    nbs.push_back(c);
    nbmap.emplace(lin, id);
    return id;
  };
  mf_status bad = MF_OK;
  auto site_of = [&](long long lin, const int wc[3]) -> int {
    auto it = sitemap.find(lin);
    if (it != sitemap.end()) return it->second;
    CfSite S;
    for (int a = 0; a < 27; ++a) S.nb[a] = -1;
    S.limit = 1;
    for (int d = 0; d < sd; ++d)
      if (!pc.periodic[d] && (wc[d] == pc.domain_lo[d] || wc[d] == pc.domain_hi[d])) S.limit = 0;
    const int kr = (sd == 3) ? 1 : 0;
    for (int kk = -kr; kk <= kr; ++kk)
      for (int jj = -1; jj <= 1; ++jj)
        for (int ii = -1; ii <= 1; ++ii) {
          int c[3] = {wc[0] + ii, wc[1] + jj, wc[2] + kk}, cw[3];
          long long l = dm.wrap(c, cw);
          S.nb[(kk + 1) * 9 + (jj + 1) * 3 + (ii + 1)] = (l >= 0) ? nb_slot(l, cw) : -1;
        }
    if (S.nb[13] < 0) bad = MF_ERR_BAD_ARG;
    for (int d = 0; d < 3; ++d) {
      S.type[d] = 0;
      if (d >= sd) continue;
      const int st = (d == 0) ? 1 : (d == 1) ? 3 : 9;
      const bool hp = S.nb[13 + st] >= 0, hm = S.nb[13 - st] >= 0;
      if (!hp && !hm) bad = MF_ERR_BAD_ARG;
      S.type[d] = !hm ? 2 : !hp ? 1 : 0;
    }
    if (S.limit) {
      const int a0 = (sd == 3) ? 0 : 9, a1 = (sd == 3) ? 27 : 18;
      for (int a = a0; a < a1; ++a)
        if (S.nb[a] < 0) bad = MF_ERR_BAD_ARG;
    }
    const int id = (int)sites.size();
    sites.push_back(S);
    sitemap.emplace(lin, id);
    return id;
  };
  for (int f = 0; f < vf.np; ++f) {
    const mf_box& V = (*vf.valid)[f];
    const mf_box& FB = (*vf.fab)[f];
    int fn[3] = {FB.hi[0] - FB.lo[0] + 1, FB.hi[1] - FB.lo[1] + 1, FB.hi[2] - FB.lo[2] + 1};
    mf_box gb = clip_domain(grow_box(V, ng, sd), pf);
    for (int k = gb.lo[2]; k <= gb.hi[2]; ++k)
      for (int j = gb.lo[1]; j <= gb.hi[1]; ++j)
        for (int i = gb.lo[0]; i <= gb.hi[0]; ++i) {
          int iv[3] = {i, j, k};
          if (in_box(V, iv)) continue;
          int c[3] = {floordiv(i, r), floordiv(j, r), sd == 3 ? floordiv(k, r) : k}, cw[3];
          long long l = dm.wrap(c, cw);
          if (l < 0 || cfine[l]) continue;
          const int sidx = site_of(l, cw);
          if (bad != MF_OK) return bad;
          CfTarget T;
          T.off = (*vf.off)[f] + loc3(FB.lo, fn, iv);
          T.cs = fn[0] * fn[1] * fn[2];
          T.site = sidx;
          T.iv[0] = i;
          T.iv[1] = j;
          T.iv[2] = k;
          T.pad = 0;
          tgs.push_back(T);
        }
  }

  // --- flux-register faces (coarse cells next to a fine patch, not covered
  // by the fine level, inside the domain) and the reflux cells
  std::vector<FaceRef> cref, fref;
  struct RT {
    long long lin;
    int d, side, reg;
    long long off;
    int cs;
  };
  std::vector<RT> rts;
  const int S = (sd == 3) ? r * r : r;
  for (int f = 0; f < vf.np; ++f) {
    const mf_box& V = (*vf.valid)[f];
    mf_box cb = coarsen_box(V, r, sd);
    for (int d = 0; d < sd; ++d)
      for (int side = 0; side < 2; ++side) {
        mf_box sb = cb;
        sb.lo[d] = sb.hi[d] = side ? cb.hi[d] + 1 : cb.lo[d] - 1;
        for (int k = sb.lo[2]; k <= sb.hi[2]; ++k)
          for (int j = sb.lo[1]; j <= sb.hi[1]; ++j)
            for (int i = sb.lo[0]; i <= sb.hi[0]; ++i) {
              int c[3] = {i, j, k}, cw[3];
              long long l = dm.wrap(c, cw);
              if (l < 0 || cfine[l]) continue;
              const int b = cpatch[l];
              if (b < 0) return MF_ERR_BAD_ARG;
              int node[3] = {cw[0], cw[1], cw[2]};
              if (side == 0) node[d] += 1;
              FaceRef fr;
              if (!face_ref(vc, b, d, node, rk2c, fr)) return MF_ERR_BAD_ARG;
              const int ridx = (int)cref.size();
              cref.push_back(fr);
              int t[2] = {0, 0}, nt = 0;
              for (int e = 0; e < sd; ++e)
                if (e != d) t[nt++] = e;
              const int n1 = (nt > 1) ? r : 1;
              for (int bb = 0; bb < n1; ++bb)
                for (int aa = 0; aa < r; ++aa) {
                  int fnode[3] = {c[0] * r, c[1] * r, sd == 3 ? c[2] * r : c[2]};
                  fnode[d] = side ? V.hi[d] + 1 : V.lo[d];
                  fnode[t[0]] += aa;
                  if (nt > 1) fnode[t[1]] += bb;
                  FaceRef ff;
                  if (!face_ref(vf, f, d, fnode, rk2f, ff)) return MF_ERR_BAD_ARG;
                  fref.push_back(ff);
                }
              RT rt;
              rt.lin = l;
              rt.d = d;
              rt.side = side;
              rt.reg = ridx;
              if (!coarse_loc(l, cw, rt.off, rt.cs)) return MF_ERR_BAD_ARG;
              rts.push_back(rt);
            }
      }
  }
  std::sort(rts.begin(), rts.end(), [](const RT& a, const RT& b) {
    if (a.lin != b.lin) return a.lin < b.lin;
    if (a.d != b.d) return a.d < b.d;
    return a.side < b.side;
  });
  std::vector<RefluxCell> rcs;
  std::vector<RefluxTerm> rterms;
  for (size_t q = 0; q < rts.size(); ++q) {
    if (q == 0 || rts[q].lin != rts[q - 1].lin) {
      RefluxCell c;
      c.off = rts[q].off;
      c.cs = rts[q].cs;
      c.first = (int)rterms.size();
      c.count = 0;
      c.pad = 0;
      rcs.push_back(c);
    }
    RefluxTerm t;
    t.reg = rts[q].reg;
    t.sign = rts[q].side ? 1 : -1;
    rterms.push_back(t);
    rcs.back().count += 1;
  }

  // --- averaged coarse cells
  std::vector<AvgCell> avgs;
  for (int f = 0; f < vf.np; ++f) {
    const mf_box& V = (*vf.valid)[f];
    const mf_box& FB = (*vf.fab)[f];
    int fn[3] = {FB.hi[0] - FB.lo[0] + 1, FB.hi[1] - FB.lo[1] + 1, FB.hi[2] - FB.lo[2] + 1};
    mf_box cb = coarsen_box(V, r, sd);
    for (int k = cb.lo[2]; k <= cb.hi[2]; ++k)
      for (int j = cb.lo[1]; j <= cb.hi[1]; ++j)
        for (int i = cb.lo[0]; i <= cb.hi[0]; ++i) {
          int c[3] = {i, j, k}, cw[3];
          long long l = dm.wrap(c, cw);
          AvgCell a;
          if (l < 0 || !coarse_loc(l, cw, a.coff, a.ccs)) return MF_ERR_BAD_ARG;
          int f0[3] = {i * r, j * r, sd == 3 ? k * r : k};
          a.foff = (*vf.off)[f] + loc3(FB.lo, fn, f0);
          a.fcs = fn[0] * fn[1] * fn[2];
          a.sy = fn[0];
          a.sz = fn[0] * fn[1];
          avgs.push_back(a);
        }
  }

  if (nbs.size() > (size_t)INT32_MAX / 32 || tgs.size() > (size_t)INT32_MAX / 32 ||
      fref.size() > (size_t)INT32_MAX / 32 || avgs.size() > (size_t)INT32_MAX / 32)
    return MF_ERR_UNSUPPORTED;
  C->nc = nc;
  // incrementCoarse / incrementFine over consInterval only
  // (srcIdeal/AMRLevelIdealMHD.cpp:1282-1305)
  C->ncons = nc - pc.num_tracking_surfaces;
  C->sd = sd;
  C->divb = (pc.divb_cleaning != 0);
  C->nnb = (int)nbs.size();
  C->nsites = (int)sites.size();
  C->ntg = (int)tgs.size();
  C->nreg = (int)cref.size();
  C->nsub = S;
  C->nrc = (int)rcs.size();
  C->navg = (int)avgs.size();
  C->dxc = pc.dx;
  C->dxf = pf.dx;
  C->c1c = 0.5 / pc.dx;
  C->c1s = 1.0 / pc.dx;
  const double volc = (sd == 3) ? pc.dx * pc.dx * pc.dx : pc.dx * pc.dx;
  const double volf = (sd == 3) ? pf.dx * pf.dx * pf.dx : pf.dx * pf.dx;
  double refScale = 1.0;
  for (int d = 0; d < sd; ++d) refScale *= r;
  C->coeff = volc / (volf * refScale);
  C->invdx = 1.0 / pc.dx;
  C->vol = volf;
  MF_CUDA(C->nb.put(nbs));
  MF_CUDA(C->sites.put(sites));
  MF_CUDA(C->tg.put(tgs));
  MF_CUDA(C->old.put(nullptr, sizeof(double) * (size_t)C->nnb * nc));
  MF_CUDA(C->sv.put(nullptr, sizeof(double) * (size_t)C->nsites * nc * 4));
  MF_CUDA(C->cref.put(cref));
  MF_CUDA(C->fref.put(fref));
  MF_CUDA(C->rfc.put(nullptr, sizeof(double) * (size_t)C->nreg * nc));
  MF_CUDA(C->rff.put(nullptr, sizeof(double) * (size_t)C->nreg * S * nc));
  MF_CUDA(C->reg.put(nullptr, sizeof(double) * (size_t)C->nreg * nc));
  MF_CUDA(C->rcell.put(rcs));
  MF_CUDA(C->rterm.put(rterms));
  MF_CUDA(C->avg.put(avgs));
  C->gc.refs = (const FaceRef*)C->cref.p;
  C->gc.n = C->nreg;
  C->gc.out = (double*)C->rfc.p;
  C->gf.refs = (const FaceRef*)C->fref.p;
  C->gf.n = C->nreg * S;
  C->gf.out = (double*)C->rff.p;
  return MF_OK;
}

static CfConsts cf_consts(const mf_cf* C, double alpha) {
  CfConsts K;
  K.alpha = alpha;
  K.c1c = C->c1c;
  K.c1s = C->c1s;
  K.dxc = C->dxc;
  K.dxf = C->dxf;
  K.coeff = C->coeff;
  K.nc = C->nc;
  K.sd = C->sd;
  K.r = C->r;
  K.divb = C->divb;
  K.nsites = C->nsites;
  K.nnb = C->nnb;
  return K;
}

static mf_status cf_snapshot(mf_cf* C, cudaStream_t s) {
  const long long n = (long long)C->nnb * C->nc;
  if (n > 0)
    k_cf_snapshot<<<blocks(n), kThreads, 0, s>>>(C->vc.U, (const NbCell*)C->nb.p, C->nnb, C->nc,
                                                  (double*)C->old.p);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

static mf_status cf_interp(mf_cf* C, double alpha, cudaStream_t s) {
  const CfConsts K = cf_consts(C, alpha);
  if (C->nsites > 0)
    k_cf_sites<<<blocks(C->nsites, 128), 128, 0, s>>>(
        C->vc.U, (const NbCell*)C->nb.p, (const double*)C->old.p, (const CfSite*)C->sites.p, K,
        (double*)C->sv.p);
  MF_CUDA(cudaGetLastError());
  const long long n = (long long)C->ntg * C->nc;
  if (n > 0)
    k_cf_fill<<<blocks(n), kThreads, 0, s>>>((const CfTarget*)C->tg.p, C->ntg,
                                              (const double*)C->sv.p, K, C->vf.U);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

static mf_status cf_reg_coarse(mf_cf* C, double dt, cudaStream_t s) {
  const long long n = (long long)C->nreg * C->ncons;
  if (n > 0)
    k_reg_coarse<<<blocks(n), kThreads, 0, s>>>((double*)C->reg.p, (const double*)C->rfc.p, n,
                                                 -dt);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

static mf_status cf_reg_fine(mf_cf* C, double dt, cudaStream_t s) {
  double denom = 1.0;
  for (int e = 0; e < C->sd - 1; ++e) denom *= C->r;
  const long long n = (long long)C->nreg * C->ncons;
  if (n > 0)
    k_reg_fine<<<blocks(n), kThreads, 0, s>>>((double*)C->reg.p, (const double*)C->rff.p,
                                               C->nreg, C->nsub, C->ncons, dt / denom);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

static mf_status cf_average(mf_cf* C, cudaStream_t s) {
  const long long m = (long long)C->navg * C->nc;
  if (m > 0)
    k_average<<<blocks(m), kThreads, 0, s>>>(C->vf.U, C->vc.U, (const AvgCell*)C->avg.p, C->navg,
                                              C->nc, C->r, C->sd, C->vol);
  MF_CUDA(cudaGetLastError());
  return MF_OK;
}

static mf_status cf_reflux_average(mf_cf* C, cudaStream_t s) {
  const long long n = (long long)C->nrc * C->ncons;
  if (n > 0)
    k_reflux<<<blocks(n), kThreads, 0, s>>>(C->vc.U, (const RefluxCell*)C->rcell.p, C->nrc,
                                             (const RefluxTerm*)C->rterm.p,
                                             (const double*)C->reg.p, C->nreg, C->ncons,
                                             C->invdx);
  MF_CUDA(cudaGetLastError());
  return cf_average(C, s);
}

namespace mf {
cudaError_t launch_face_gather(int mixed, const void* const f[3], const FaceGather& g, int mode,
                               int nc, cudaStream_t s) {
  const long long n = (long long)g.n * nc;
  if (n <= 0) return cudaSuccess;
  if (mixed)
    k_face_gather<float><<<blocks(n), kThreads, 0, s>>>(
        (const float*)f[0], (const float*)f[1], (const float*)f[2], g.refs, g.n, nc, mode, g.out);
  else
    k_face_gather<double><<<blocks(n), kThreads, 0, s>>>((const double*)f[0],
                                                        (const double*)f[1],
                                                        (const double*)f[2], g.refs, g.n, nc,
                                                        mode, g.out);
  return cudaGetLastError();
}
}  // namespace mf

static void attach_gathers(mf_hier* h) {
  const int n = (int)h->lv.size();
  for (int l = 0; l < n; ++l) {
    std::vector<FaceGather> g;
    if (l + 1 < n) g.push_back(h->cf[l]->gc);
    if (l > 0) g.push_back(h->cf[l - 1]->gf);
    level_set_gathers(h->lv[l], g);
  }
}

static mf_status join_into(cudaStream_t from, cudaStream_t to) {
  if (!from || from == to) return MF_OK;
  cudaEvent_t ev;
  MF_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  cudaError_t e = cudaEventRecord(ev, from);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(to, ev, 0);
  cudaEventDestroy(ev);
  MF_CUDA(e);
  return MF_OK;
}

static mf_status hier_wait(mf_hier* h) {
  const CtxView v = ctx_view(level_view(h->lv[0]).ctx);
  return host_wait(h->s, v.timeout);
}

// AMRLevelIdealMHD::advance of level l: preTimeStep's ghost interpolation
// (srcIdeal/AMRLevelIdealMHD.cpp:669-752), the level step with its register
// increments (:1248-1308) and the GLM speeds of the base level (:1528-1548).
static mf_status hier_advance(mf_hier* h, int l) {
  const int n = (int)h->lv.size();
  mf_status st;
  if (l + 1 < n && (st = cf_snapshot(h->cf[l], h->s)) != MF_OK) return st;
  if (l > 0) {
    const int r = h->ratio[l - 1];
    const double tNew = h->t[l - 1], tOld = tNew - h->dt[l - 1];
    double alpha = (h->t[l] - tOld) / (tNew - tOld);
    const double eps = 0.04 * h->dt[l] / r;
    if (std::fabs(alpha) < eps) alpha = 0.0;
    if (std::fabs(1.0 - alpha) < eps) alpha = 1.0;
    if (alpha < 0.0 || alpha > 1.0) return MF_ERR_BAD_ARG;
    if ((st = cf_interp(h->cf[l - 1], alpha, h->s)) != MF_OK) return st;
  }
  double nd = 0.0;
  int mp = 0, cell[3];
  level_set_time_host(h->lv[l], h->t[l]);
  st = mf_level_step(h->lv[l], h->dt[l], &nd, &mp, cell, h->s);
  if (st != MF_OK) return st;
  h->ndt[l] = nd;
  if (l + 1 < n && (st = cf_reg_coarse(h->cf[l], h->dt[l], h->s)) != MF_OK) return st;
  if (l > 0 && (st = cf_reg_fine(h->cf[l - 1], h->dt[l], h->s)) != MF_OK) return st;
  h->t[l] = h->t[l] + h->dt[l];
  const mf_params& p0 = *level_view(h->lv[0]).p;
  if (l == 0 && p0.divb_cleaning == 5 && p0.factor_ch > 0.0) {
    const double dx = p0.dx;
    const double Ch = p0.factor_ch * dx / nd;
    const double Cp = std::sqrt(Ch * dx / p0.factor_cp);
    for (int q = 0; q < n; ++q) mf_set_dedner(level_view(h->lv[q]).ctx, Ch, Cp);
  }
  return MF_OK;
}

// AMR_MHDAM::timeStep: advance, the finer level ratio times, postTimeStep
// (reflux, average down; srcIdeal/AMRLevelIdealMHD.cpp:1633-1646).
static mf_status hier_time_step(mf_hier* h, int l) {
  mf_status st = hier_advance(h, l);
  if (st != MF_OK) return st;
  if (l + 1 < (int)h->lv.size()) {
    for (int k = 0; k < h->ratio[l]; ++k)
      if ((st = hier_time_step(h, l + 1)) != MF_OK) return st;
    if ((st = cf_reflux_average(h->cf[l], h->s)) != MF_OK) return st;
  }
  return MF_OK;
}

extern "C" {

mf_status mf_hier_create(int nlevels, mf_level* const* levels, const int* ratios, mf_hier** out) {
  if (!out || nlevels < 1 || !levels || (nlevels > 1 && !ratios)) return MF_ERR_BAD_ARG;
  *out = nullptr;
  for (int l = 0; l < nlevels; ++l)
    if (!levels[l]) return MF_ERR_BAD_ARG;
  for (int l = 0; l < nlevels; ++l)
    for (int m = l + 1; m < nlevels; ++m)
      if (levels[l] == levels[m] || level_view(levels[l]).ctx == level_view(levels[m]).ctx)
        return MF_ERR_BAD_ARG;  // one context (dx, domain, GLM speeds) per level
  // constrained transport across levels (the accumulated edge field averaged
  // onto the coarser level, srcIdeal/AMRLevelIdealMHD.cpp:1649-1688) is not built
  for (int l = 0; l < nlevels && nlevels > 1; ++l) {
    const int dc = level_view(levels[l]).p->divb_cleaning;
    if (dc >= 1 && dc <= 3) return MF_ERR_UNSUPPORTED;
  }
  mf_hier* h = new (std::nothrow) mf_hier();
  if (!h) return MF_ERR_OOM;
  h->lv.assign(levels, levels + nlevels);
  if (nlevels > 1) h->ratio.assign(ratios, ratios + nlevels - 1);
  h->t.assign(nlevels, 0.0);
  h->dt.assign(nlevels, 0.0);
  h->ndt.assign(nlevels, 0.0);
  mf_status st = MF_OK;
  for (int l = 0; l + 1 < nlevels && st == MF_OK; ++l) {
    mf_cf* C = new (std::nothrow) mf_cf();
    if (!C) {
      st = MF_ERR_OOM;
      break;
    }
    h->cf.push_back(C);
    C->lc = levels[l];
    C->lf = levels[l + 1];
    C->vc = level_view(C->lc);
    C->vf = level_view(C->lf);
    C->r = h->ratio[l];
    const mf_params &pc = *C->vc.p, &pf = *C->vf.p;
    if (pc.time_approximation != pf.time_approximation || pc.precision != pf.precision)
      st = MF_ERR_BAD_ARG;
    else
      st = build_cf(C);
  }
  if (st == MF_OK && cudaStreamCreateWithFlags(&h->s, cudaStreamNonBlocking) != cudaSuccess)
    st = MF_ERR_CUDA;
  if (st != MF_OK) {
    for (mf_cf* C : h->cf) delete C;
    delete h;
    return st;
  }
  attach_gathers(h);
  // launches per coarse step: level steps (with their gathers) + coupling
  int mult = 1;
  for (int l = 0; l < nlevels; ++l) {
    if (l > 0) mult *= h->ratio[l - 1];
    int per = mf_level_launches_per_step(levels[l]);
    if (l + 1 < nlevels) per += 2;  // snapshot, register set
    if (l > 0) per += 3;            // sites, fill, register add
    h->launches += mult * per;
    if (l + 1 < nlevels) h->launches += mult * 2;  // reflux, average
  }
  *out = h;
  return MF_OK;
}

void mf_hier_destroy(mf_hier* h) {
  if (!h) return;
  if (h->s) cudaStreamSynchronize(h->s);
  for (mf_level* L : h->lv) level_set_gathers(L, std::vector<FaceGather>());
  for (mf_cf* C : h->cf) delete C;
  if (h->s) cudaStreamDestroy(h->s);
  delete h;
}

mf_status mf_hier_set_time(mf_hier* h, double time) {
  if (!h || !std::isfinite(time)) return MF_ERR_BAD_ARG;
  for (double& t : h->t) t = time;
  return MF_OK;
}

mf_status mf_hier_times(const mf_hier* h, double* times) {
  if (!h || !times) return MF_ERR_BAD_ARG;
  for (size_t l = 0; l < h->t.size(); ++l) times[l] = h->t[l];
  return MF_OK;
}

int mf_hier_launches_per_step(const mf_hier* h) { return h ? h->launches : -1; }

mf_status mf_hier_info(const mf_hier* h, int pair, long long counts[6]) {
  if (!h || !counts || pair < 0 || pair >= (int)h->cf.size()) return MF_ERR_BAD_ARG;
  const mf_cf* C = h->cf[pair];
  counts[0] = C->nsites;
  counts[1] = C->ntg;
  counts[2] = C->nreg;
  counts[3] = C->nrc;
  counts[4] = C->navg;
  counts[5] = C->nnb;
  return MF_OK;
}

mf_status mf_hier_snapshot(mf_hier* h, int level, void* stream) {
  if (!h || level < 0 || level >= (int)h->cf.size()) return MF_ERR_BAD_ARG;
  mf_status st = join_into((cudaStream_t)stream, h->s);
  if (st == MF_OK) st = cf_snapshot(h->cf[level], h->s);
  return st != MF_OK ? st : hier_wait(h);
}

mf_status mf_hier_fill_ghosts(mf_hier* h, int level, double alpha, void* stream) {
  if (!h || level < 1 || level >= (int)h->lv.size() || !(alpha >= 0.0 && alpha <= 1.0))
    return MF_ERR_BAD_ARG;
  mf_status st = join_into((cudaStream_t)stream, h->s);
  if (st == MF_OK) st = cf_interp(h->cf[level - 1], alpha, h->s);
  return st != MF_OK ? st : hier_wait(h);
}

mf_status mf_hier_average_down(mf_hier* h, int level, void* stream) {
  if (!h || level < 0 || level >= (int)h->cf.size()) return MF_ERR_BAD_ARG;
  mf_status st = join_into((cudaStream_t)stream, h->s);
  if (st == MF_OK) st = cf_average(h->cf[level], h->s);
  return st != MF_OK ? st : hier_wait(h);
}

mf_status mf_hier_step(mf_hier* h, double dt0, double* new_dt, void* stream) {
  if (!h || !(dt0 > 0.0) || !std::isfinite(dt0)) return MF_ERR_BAD_ARG;
  const int n = (int)h->lv.size();
  mf_status st = join_into((cudaStream_t)stream, h->s);
  if (st != MF_OK) return st;
  for (int l = 0; l < n; ++l) h->dt[l] = (l == 0) ? dt0 : h->dt[l - 1] / h->ratio[l - 1];
  st = hier_time_step(h, 0);
  if (st != MF_OK) return st;
  st = hier_wait(h);
  if (st != MF_OK) return st;
  double m = 1.0, best = 0.0;
  for (int l = 0; l < n; ++l) {
    if (l > 0) m *= h->ratio[l - 1];
    const double v = h->ndt[l] * m;
    if (l == 0 || v < best) best = v;
  }
  if (new_dt) *new_dt = best;
  h->last_dt0 = dt0;
  h->last_new_dt = best;
  return MF_OK;
}

mf_status mf_hier_assign_dt(const mf_hier* h, double cfl, double* dt0) {
  if (!h || !dt0 || !(cfl > 0.0) || !(h->last_dt0 > 0.0)) return MF_ERR_BAD_ARG;
  // AMR_MHDAM::assignDt with subcycling (srcIdeal/AMR_MHDAM.cpp:1586-1626):
  // the minimum over the levels of cfl * dt_new[l] * refinement, i.e. cfl
  // times mf_hier_step's new_dt, then at most max_dt_growth times the
  // current dt of every level times its refinement, which is dt0 for all
  const double g = level_view(h->lv[0]).p->max_dt_growth;
  double d = cfl * h->last_new_dt;
  if (g > 0.0) d = std::min(d, h->last_dt0 * g);
  *dt0 = d;
  return MF_OK;
}

}  // extern "C"
