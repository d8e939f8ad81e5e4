// mf_update_exact.cu - update kernel of the FP64 parity path, the stand-alone
// dt kernel, the level dt finalisation, the device ghost exchange and the
// face-flux output of the single-patch call.  Built with -fmad=false.
#include <cfloat>
#include <climits>

#define MF_PHYS exact
#include "mf_sources_exact.cuh"
#include "mf_update_kernel.cuh"

namespace mf {
namespace {
using namespace MF_PHYS;

template <int GLM>
__global__ void __launch_bounds__(kMaxBlock)
    k_dt(const __grid_constant__ DevParams P, const double* __restrict__ U, const StageDesc* __restrict__ descs,
         int ndesc, int total, const RunParams* __restrict__ runs,
         DtPartial* __restrict__ partials) {
  constexpr int IRHON = 8 + GLM;
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  double dtc = DBL_MAX;
  int myidx = INT_MAX;
  const StageDesc* Dp = nullptr;
  int lin = 0;
  if (g < total) {
    Dp = &descs[find_desc(descs, ndesc, kRegV, g)];
    lin = g - Dp->g0[kRegV];
    if (lin >= Dp->vn[0] * Dp->vn[1] * Dp->vn[2]) Dp = nullptr;  // run-alignment gap
  }
  if (Dp) {
    const StageDesc& D = *Dp;
    int i, j, k;
    decode(lin, D.vlo, D.vn, i, j, k);
    const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
    const long long base = D.u_off + loc(D.flo, D.fn, i, j, k);
    double u[MF_MAX_COMP];
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.nc) u[q] = U[base + q * cs];
    dtc = runs[D.run].dx / max_wave_speed<IRHON>(P, u);
    myidx = g;
  }
  block_dt_min(dtc, myidx, descs, ndesc, partials, blockIdx.x);
}

__device__ __forceinline__ bool part_less(const DtPartial& a, const DtPartial& b) {
  if (a.dt < b.dt) return true;
  if (a.dt > b.dt) return false;
  if (a.desc != b.desc) return a.desc < b.desc;
  return a.idx < b.idx;
}

// One block per run: the minimum over the run's block partials, the run's
// time after the step, then (advance) its next dt and GLM speeds
// (AMRLevelIdealMHD::advance, srcIdeal/AMRLevelIdealMHD.cpp:1531-1548, 1588).
__global__ void __launch_bounds__(256)
    k_finalize(const __grid_constant__ DevParams P, const DtPartial* __restrict__ parts,
               const RunParams* __restrict__ runs, int nt, StepState* __restrict__ states,
               int advance, int nparts) {
  const RunParams& R = runs[blockIdx.x];
  StepState* __restrict__ ss = states + blockIdx.x;
  const int p0 = (nparts > 0) ? 0 : R.v0 / nt;
  const int p1 = (nparts > 0) ? nparts : (R.v1 + nt - 1) / nt;
  DtPartial best;
  best.dt = DBL_MAX;
  best.desc = INT_MAX;
  best.idx = INT_MAX;
  for (int q = p0 + threadIdx.x; q < p1; q += blockDim.x) {
    DtPartial c = parts[q];
    if (part_less(c, best)) best = c;
  }
  __shared__ DtPartial sb[256];
  sb[threadIdx.x] = best;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s && part_less(sb[threadIdx.x + s], sb[threadIdx.x]))
      sb[threadIdx.x] = sb[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    best = sb[0];
    ss->dt_min = best.dt;
    ss->min_desc = (best.desc == INT_MAX) ? INT_MAX : best.desc - R.d0;
    ss->min_idx = best.idx;
    if (!(best.dt > 0.0) || best.dt >= DBL_MAX) atomicOr(&ss->flags, kFlagBadDt);
    // the level's time after the step (AMRLevelIdealMHD::advance, :1587)
    const double dt_step = ss->dt;
    ss->time = ss->time + dt_step;
    if (advance) {
      const double dtn = best.dt;
      // AMR_MHDAM::assignDt (srcIdeal/AMR_MHDAM.cpp:1675-1681): the next dt is
      // cfl * dt_min, grown at most by max_dt_growth over the step's dt (a
      // run's first dt, reduced before it has taken a step, is not capped)
      double next = ss->cfl * dtn;
      if (P.max_growth > 0.0 && dt_step > 0.0) next = fmin(next, dt_step * P.max_growth);
      ss->dt = next;
      if (P.glm && P.factor_ch > 0.0) {
        const double ch = P.factor_ch * R.dx / dtn;
        ss->ch = ch;
        ss->cp = sqrt(ch * R.dx / P.factor_cp);
      }
    }
  }
}

// 16-byte vector of V elements of T
template <typename T, int V>
struct Vec;
template <> struct Vec<float, 4> { using type = float4; };
template <> struct Vec<double, 2> { using type = double2; };
template <typename T> struct Vec<T, 1> { using type = T; };

// The copy of one region's components in vectors of V elements along x (V
// divides the region's x extent, and every row starts on a multiple of V).
// Flat over the (component, vector) items so that small regions still occupy
// the block; 32-bit index arithmetic (a region is part of one patch's ghost
// layers: 2^31 elements would take a patch whose fab alone exceeds HBM); four
// loads in flight per thread before their stores.
template <typename T, int V>
__device__ __forceinline__ void copy_region(T* __restrict__ U, const CopyReg& R, int nc,
                                            long long scs, long long dcs) {
  using VT = typename Vec<T, V>::type;
  const int rowv = R.ext[0] / V;
  const int n = rowv * R.ext[1] * R.ext[2];
  const int tot = n * nc;
  const int step = blockDim.x;
  for (int t0 = threadIdx.x; t0 < tot; t0 += 4 * step) {
    VT v[4];
    long long dof[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int t = t0 + j * step;
      if (t < tot) {
        const int q = t / n;
        const int c = t - q * n;
        const int a = c % rowv;
        const int r = c / rowv;
        const int b = r % R.ext[1];
        const int e = r / R.ext[1];
        const long long so = R.src_off + q * scs + (R.s0[0] + a * V) +
                             (long long)R.sfn[0] * ((R.s0[1] + b) + (long long)R.sfn[1] * (R.s0[2] + e));
        dof[j] = R.dst_off + q * dcs + (R.d0[0] + a * V) +
                 (long long)R.dfn[0] * ((R.d0[1] + b) + (long long)R.dfn[1] * (R.d0[2] + e));
        v[j] = __ldg(reinterpret_cast<const VT*>(U + so));
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (t0 + j * step < tot) *reinterpret_cast<VT*>(U + dof[j]) = v[j];
  }
}

// One block per copy region.  Sources are valid cells and destinations ghost
// cells, never the same, so the sources are read through the read-only path.
// Rows are copied in 16-byte vectors where the region's x extent, its rows'
// starts and the fabs' strides are multiples of the vector (the fabs start on
// 256-byte boundaries), else element by element.
template <typename T>
__global__ void __launch_bounds__(256)
    k_exchange(T* __restrict__ U, const CopyReg* __restrict__ regs, int nc) {
  constexpr int V = 16 / sizeof(T);
  const CopyReg R = regs[blockIdx.x];
  const long long scs = (long long)R.sfn[0] * R.sfn[1] * R.sfn[2];
  const long long dcs = (long long)R.dfn[0] * R.dfn[1] * R.dfn[2];
  const bool vec = R.ext[0] % V == 0 && (R.src_off + R.s0[0]) % V == 0 &&
                   (R.dst_off + R.d0[0]) % V == 0 && R.sfn[0] % V == 0 && R.dfn[0] % V == 0 &&
                   scs % V == 0 && dcs % V == 0;
  if (vec)
    copy_region<T, V>(U, R, nc, scs, dcs);
  else
    copy_region<T, 1>(U, R, nc, scs, dcs);
}

template <typename R>
__global__ void k_flux_out(int nc, const R* __restrict__ f2, int l20, int l21, int l22, int n20,
                           int n21, int n22, const R* __restrict__ f1, int l10, int l11, int l12,
                           int n10, int n11, int n12, double* __restrict__ out, int lo0, int lo1,
                           int lo2, int on0, int on1, int on2) {
  const long long n = (long long)on0 * on1 * on2;
  const long long cs2 = (long long)n20 * n21 * n22, cs1 = (long long)n10 * n11 * n12;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n * nc;
       t += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(t / n);
    const long long c = t - (long long)q * n;
    const int a = (int)(c % on0);
    const long long r = c / on0;
    const int b = (int)(r % on1);
    const int e = (int)(r / on1);
    const int i = lo0 + a, j = lo1 + b, k = lo2 + e;
    const long long i2 = q * cs2 + (i - l20) + (long long)n20 * ((j - l21) + (long long)n21 * (k - l22));
    double v = (double)f2[i2];
    if (f1) {
      const long long i1 =
          q * cs1 + (i - l10) + (long long)n10 * ((j - l11) + (long long)n11 * (k - l12));
      v = v + (double)f1[i1];
      v = v * 0.5;
    }
    out[t] = v;
  }
}

}  // namespace

cudaError_t launch_update_exact(const DevParams& P, const StageBuffers& B, const Batch& b,
                                int flags, double dt_scale, StepState* state,
                                DtPartial* partials, int* nblocks_v, cudaStream_t s) {
  const int nt = b.nt[2];
  const unsigned gv = flat_blocks(b.tot_v, nt);
  if (nblocks_v) *nblocks_v = (int)gv;
#define MF_UPD(G, FL)                                                                         \
  k_update<double, G, FL><<<gv, nt, 0, s>>>(P, B, b.desc, b.ndesc, 0, b.tot_v, b.runs, state, \
                                            dt_scale, partials)
  if (P.glm) {
    if (flags == 0) MF_UPD(1, 0);
    else if (flags == kStageDt) MF_UPD(1, kStageDt);
    else MF_UPD(1, kStageAverage | kStageDt);
  } else {
    if (flags == 0) MF_UPD(0, 0);
    else if (flags == kStageDt) MF_UPD(0, kStageDt);
    else MF_UPD(0, kStageAverage | kStageDt);
  }
#undef MF_UPD
  return cudaGetLastError();
}

cudaError_t launch_dt(const DevParams& P, const double* u, const Batch& b, DtPartial* partials,
                      int* nblocks, cudaStream_t s) {
  const int nt = b.nt[2];
  const unsigned gv = flat_blocks(b.tot_v, nt);
  if (nblocks) *nblocks = (int)gv;
  if (P.glm)
    k_dt<1><<<gv, nt, 0, s>>>(P, u, b.desc, b.ndesc, b.tot_v, b.runs, partials);
  else
    k_dt<0><<<gv, nt, 0, s>>>(P, u, b.desc, b.ndesc, b.tot_v, b.runs, partials);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const DevParams& P, const DtPartial* partials, const Batch& b,
                            int nt, StepState* state, int advance, cudaStream_t s, int nparts) {
  if (b.nruns <= 0) return cudaSuccess;
  k_finalize<<<nparts > 0 ? 1 : b.nruns, 256, 0, s>>>(P, partials, b.runs, nt, state, advance,
                                                     nparts);
  return cudaGetLastError();
}

cudaError_t launch_exchange(double* u, const CopyReg* regs, int nreg, int nc, cudaStream_t s) {
  if (nreg <= 0) return cudaSuccess;
  k_exchange<double><<<nreg, 256, 0, s>>>(u, regs, nc);
  return cudaGetLastError();
}

cudaError_t launch_exchange_f(float* u, const CopyReg* regs, int nreg, int nc, cudaStream_t s) {
  if (nreg <= 0) return cudaSuccess;
  k_exchange<float><<<nreg, 256, 0, s>>>(u, regs, nc);
  return cudaGetLastError();
}

cudaError_t launch_flux_out(int mixed, int sd, int nc, const void* const f2[3],
                            const int f2lo[3][3], const int f2n[3][3], const void* const f1[3],
                            const int f1lo[3][3], const int f1n[3][3], double* const fout[3],
                            const int olo[3][3], const int on[3][3], cudaStream_t s) {
  for (int d = 0; d < sd; ++d) {
    long long n = (long long)on[d][0] * on[d][1] * on[d][2] * nc;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 4096) blocks = 4096;
    if (blocks < 1) blocks = 1;
    if (mixed)
      k_flux_out<float><<<blocks, 256, 0, s>>>(
          nc, (const float*)f2[d], f2lo[d][0], f2lo[d][1], f2lo[d][2], f2n[d][0], f2n[d][1],
          f2n[d][2], (const float*)f1[d], f1lo[d][0], f1lo[d][1], f1lo[d][2], f1n[d][0],
          f1n[d][1], f1n[d][2], fout[d], olo[d][0], olo[d][1], olo[d][2], on[d][0], on[d][1],
          on[d][2]);
    else
      k_flux_out<double><<<blocks, 256, 0, s>>>(
          nc, (const double*)f2[d], f2lo[d][0], f2lo[d][1], f2lo[d][2], f2n[d][0], f2n[d][1],
          f2n[d][2], (const double*)f1[d], f1lo[d][0], f1lo[d][1], f1lo[d][2], f1n[d][0],
          f1n[d][1], f1n[d][2], fout[d], olo[d][0], olo[d][1], olo[d][2], on[d][0], on[d][1],
          on[d][2]);
  }
  return cudaGetLastError();
}


}  // namespace mf
