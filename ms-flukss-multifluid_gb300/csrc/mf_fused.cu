// mf_fused.cu - one kernel per stage for the mixed-precision level step: the
// face fluxes of every direction and the update of a tile of cells, without
// face-flux arrays in HBM.
//
// A block takes one tile of a patch's valueBox (a work list of (patch, tile)
// items built with the level).  Per fluid group (the plasma with psi, then
// each neutral fluid) it stages the FP32 primitive state of the tile and a
// two-cell halo in shared memory, computes the fluxes of every face of the
// tile, all directions in one pass, into shared memory (one thread per face:
// the limited face states, the Riemann solver, Bn, the heliosphere boundary
// fluxes), and adds each cell's flux differences to its FP32 accumulators in
// the order the split kernels use (x, then y, then z).  The update of the
// cell then runs the update kernel's own code (sources with the FP64
// stage-start state, charge exchange, positivity, RK2 averaging, the dt
// partial of the block).  The primitive state and its FP32 copy come from the
// stage's primitive part, so no grid barrier is needed: ghosts are filled
// before the stage, and the halo of a tile is read, not recomputed.
//
// Supported: RK2 and first order, no constrained transport, no
// characteristic reconstruction, no tracking surfaces, Bn methods 0 and 1, no
// flux-register gathers (the level uses the split kernels otherwise).
#define MF_PHYS fast
#include "mf_riemann.cuh"
#include "mf_flux_kernel.cuh"
#include "mf_sources.cuh"
#include "mf_update_kernel.cuh"

namespace mf {
namespace {

constexpr int kFusedThreads = 256;
// largest fluid group: plasma (8) + psi
constexpr int kGroupMax = 9;
// shared memory of one block at most (two blocks per SM)
constexpr size_t kFusedSmemMax = 112 * 1024;

struct FusedShape {
  int t[3];   // tile extents (cells)
  int h[3];   // halo box extents (tile + 4 in each used direction)
  int nh;     // halo box cells
  int nfmax;  // faces of all directions of a full tile (shared-memory stride)
};

// Face grids of a tile of extents n per direction, and the offsets of each
// direction in the tile's face list (x faces, then y, then z).
struct TileFaces {
  int fn[3][3];
  int off[4];
};

__device__ __forceinline__ TileFaces tile_faces(const FusedTile& T, int sd) {
  TileFaces F;
  F.off[0] = 0;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
#pragma unroll
    for (int e = 0; e < 3; ++e) F.fn[d][e] = T.n[e] + (e == d ? 1 : 0);
    F.off[d + 1] = F.off[d] + ((d < sd) ? F.fn[d][0] * F.fn[d][1] * F.fn[d][2] : 0);
  }
  return F;
}

__device__ __forceinline__ int hidx(const FusedShape& S, int a, int b, int c) {
  return a + S.h[0] * (b + S.h[1] * c);
}

template <int DIR>
__device__ __forceinline__ int hstride(const FusedShape& S) {
  return DIR == 0 ? 1 : DIR == 1 ? S.h[0] : S.h[0] * S.h[1];
}

// The fluxes of one group on one face in direction DIR: face fd of the
// direction's face grid fn ((n[DIR]+1) along DIR) lies on the low side of the
// tile-local cell (fi, fj, fk); stencil cells -2..+1 along DIR.  The results
// go to slot f of the tile's face list.  The same steps as the split flux
// kernel (k_flux) on the FP32 copy of W.
template <int DIR, int GLM>
__device__ __forceinline__ void face_group(const DevParams& P, const RunParams& RP,
                                           const StepState& SS, const FusedShape& S,
                                           const FusedTile& T, int grp, const int* fn, int fd,
                                           int f, const float* __restrict__ sw,
                                           float* __restrict__ sf,
                                           unsigned char* __restrict__ sneg) {
  const int st = hstride<DIR>(S);
  const int off3 = (P.sd == 3) ? 2 : 0;
  const int fi = fd % fn[0], fj = (fd / fn[0]) % fn[1], fk = fd / (fn[0] * fn[1]);
  const int hc = hidx(S, fi + 2, fj + 2, fk + off3);
  const int i = T.lo[0] + fi, j = T.lo[1] + fj, k = T.lo[2] + fk;
  auto ld = [&](int v, int o) -> float { return sw[v * S.nh + hc + o * st]; };
  const int hside = helio_side<DIR>(P, RP, i, j, k);
  if (grp == 0) {
    // CHECKPOSITIVITY / REDUCEORDER (src/reconstructionF.ChF:1023-1054)
    bool negL = false, negR = false;
    if (P.check_pos) {
#pragma unroll
      for (int t = 0; t < 2; ++t) {
        const int v = t ? 4 : 0;
        const float a = ld(v, -2), b = ld(v, -1), c = ld(v, 0), d = ld(v, 1);
        float lo, hi;
        face_values<float>(P.lim[v], a, b, c, lo, hi);
        if (lo <= 0.0f || hi <= 0.0f) negL = true;
        face_values<float>(P.lim[v], b, c, d, lo, hi);
        if (lo <= 0.0f || hi <= 0.0f) negR = true;
      }
      sneg[f] = (unsigned char)((negL ? 1 : 0) | (negR ? 2 : 0));
    }
    // plasma (+ psi) face states: left = high-face value of the low cell,
    // right = low-face value of the high cell
    float wl[9], wr[9];
#pragma unroll
    for (int v = 0; v < 9; ++v) {
      if (v < 8 || GLM) {
        const int lim = (v < 8) ? P.lim[v] : (int)MF_LIM_MINMOD;
        const float a = ld(v, -2), b = ld(v, -1), c = ld(v, 0), d = ld(v, 1);
        float lo, hi;
        face_values<float>(lim, a, b, c, lo, hi);
        wl[v] = negL ? b : hi;
        face_values<float>(lim, b, c, d, lo, hi);
        wr[v] = negR ? c : lo;
      } else {
        wl[v] = 0.0f;
        wr[v] = 0.0f;
      }
    }
    float g[9];
    plasma_flux<float, DIR>(P, wl, wr, g);
    if (GLM) {
      float fbn, fpsi;
      dedner_2x2<float>(float(SS.ch), wl[5 + DIR], wl[8], wr[5 + DIR], wr[8], fbn, fpsi);
      g[5 + DIR] = fbn;
      g[8] = fpsi;
    }
    // face-normal B (PatchMHDMF::computeBn, srcIdeal/PatchMHDMF.cpp:509-620)
    float bn = 0.0f;
    if (P.divb_method == 1) {
      bn = 0.5f * (wl[5 + DIR] + wr[5 + DIR]);
      if (!P.periodic[DIR]) {
        const int fx = (DIR == 0) ? i : (DIR == 1) ? j : k;
        if (fx == RP.dlo[DIR]) bn = wr[5 + DIR];
        if (fx == RP.dhi[DIR] + 1) bn = wl[5 + DIR];
      }
    }
    if (hside >= 0) {  // HELIOBC on the domain boundary
      double dl[8], dr[8], dg[8], dbn = double(bn);
#pragma unroll
      for (int v = 0; v < 8; ++v) {
        dl[v] = double(wl[v]);
        dr[v] = double(wr[v]);
      }
      helio_plasma<DIR>(P, RP, hside, dl, dr, dg, dbn);
#pragma unroll
      for (int v = 0; v < 8; ++v) g[v] = float(dg[v]);
      bn = float(dbn);
    }
#pragma unroll
    for (int q = 0; q < 8; ++q) sf[q * S.nfmax + f] = g[q];
    if (GLM) sf[8 * S.nfmax + f] = g[8];
    sf[kGroupMax * S.nfmax + f] = bn;
  } else {
    // neutral fluid grp: minmod face states, van Leer splitting (VANLEERF)
    const unsigned char ng = P.check_pos ? sneg[f] : 0;
    const bool negL = ng & 1, negR = ng & 2;
    float nl[5], nr[5], gn[5];
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      const float a = ld(m, -2), b = ld(m, -1), c = ld(m, 0), d = ld(m, 1);
      float lo, hi;
      face_values<float>(MF_LIM_MINMOD, a, b, c, lo, hi);
      nl[m] = negL ? b : hi;
      face_values<float>(MF_LIM_MINMOD, b, c, d, lo, hi);
      nr[m] = negR ? c : lo;
    }
    if (hside >= 0) {
      double dl[5], dr[5], dg[5];
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        dl[m] = double(nl[m]);
        dr[m] = double(nr[m]);
      }
      helio_neutral<DIR>(P, hside, grp, dl, dr, dg);
#pragma unroll
      for (int m = 0; m < 5; ++m) gn[m] = float(dg[m]);
    } else {
      vanleer_euler<float, DIR>(P, nl, nr, gn);
    }
#pragma unroll
    for (int m = 0; m < 5; ++m) sf[m * S.nfmax + f] = gn[m];
  }
}

// The fluxes of one group on every face of the tile (all directions in one
// pass over the tile's face list).
template <int GLM>
__device__ __forceinline__ void group_faces(const DevParams& P, const RunParams& RP,
                                            const StepState& SS, const FusedShape& S,
                                            const FusedTile& T, const TileFaces& TF, int grp,
                                            const float* __restrict__ sw,
                                            float* __restrict__ sf,
                                            unsigned char* __restrict__ sneg) {
  const int nf = (P.sd == 3) ? TF.off[3] : TF.off[2];  // (static indices)
  for (int f = threadIdx.x; f < nf; f += blockDim.x) {
    if (f < TF.off[1])
      face_group<0, GLM>(P, RP, SS, S, T, grp, TF.fn[0], f, f, sw, sf, sneg);
    else if (f < TF.off[2])
      face_group<1, GLM>(P, RP, SS, S, T, grp, TF.fn[1], f - TF.off[1], f, sw, sf, sneg);
    else
      face_group<2, GLM>(P, RP, SS, S, T, grp, TF.fn[2], f - TF.off[2], f, sw, sf, sneg);
  }
}

// Each cell of the tile adds its flux differences to its accumulators, one
// direction after another (FP32, as the split update sums them) and, for the
// plasma group, its Bn differences to divB (FP64, as COMPUTEDIVB).
__device__ __forceinline__ void group_accumulate(const DevParams& P, const FusedShape& S,
                                                 const FusedTile& T, const TileFaces& TF,
                                                 int q0, int ncg, const float* __restrict__ sf,
                                                 float* __restrict__ acc, int ncell, bool plasma,
                                                 double& divB) {
  const int t = threadIdx.x;
  if (t >= ncell) return;
  const int ci = t % T.n[0], cj = (t / T.n[0]) % T.n[1], ck = t / (T.n[0] * T.n[1]);
  int flo[3], fs[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int* fn = TF.fn[d];
    flo[d] = TF.off[d] + ci + fn[0] * (cj + fn[1] * ck);
    fs[d] = (d == 0) ? 1 : (d == 1) ? fn[0] : fn[0] * fn[1];
  }
  for (int q = 0; q < ncg; ++q) {
    float a = acc[(q0 + q) * kFusedThreads + t];
    const float* sq = sf + q * S.nfmax;
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (d < P.sd) a = a + (sq[flo[d] + fs[d]] - sq[flo[d]]);
    acc[(q0 + q) * kFusedThreads + t] = a;
  }
  if (plasma && P.use8) {
    const float* bn = sf + kGroupMax * S.nfmax;
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (d < P.sd) divB = divB + fp64::f2d(bn[flo[d] + fs[d]] - bn[flo[d]]);
  }
}

template <int GLM, int FLAGS, typename CE>
__global__ void __launch_bounds__(kFusedThreads, 2)
    k_fused(const __grid_constant__ DevParams P, const __grid_constant__ StageBuffers B, const StageDesc* __restrict__ descs,
            int ndesc, const FusedTile* __restrict__ tiles, const FusedShape S,
            const RunParams* __restrict__ runs, StepState* __restrict__ states,
            const double dt_scale, DtPartial* __restrict__ partials) {
  extern __shared__ float smem[];
  const FusedTile T = tiles[blockIdx.x];
  const StageDesc& D = descs[T.desc];
  const RunParams& RP = runs[D.run];
  StepState* __restrict__ ss = states + D.run;
  const int ncell = T.n[0] * T.n[1] * T.n[2];
  const TileFaces TF = tile_faces(T, P.sd);
  float* sw = smem;                                                     // [kGroupMax][nh]
  float* sf = sw + kGroupMax * S.nh;                                    // [kGroupMax+1][nfmax]
  float* acc = sf + (kGroupMax + 1) * S.nfmax;                          // [ils][kFusedThreads]
  unsigned char* sneg = (unsigned char*)(acc + P.ils * kFusedThreads);  // [nfmax]
  const int t = threadIdx.x;
  for (int q = 0; q < P.ils; ++q) acc[q * kFusedThreads + t] = 0.0f;

  const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
  const float* __restrict__ Wf = B.wf;
  const int z0 = (P.sd == 3) ? 2 : 0;
  double divB = 0.0;
  for (int grp = 0; grp < P.nf; ++grp) {  // plasma, then each neutral fluid
    const int q0 = (grp == 0) ? 0 : P.irhon + (grp - 1) * 5;
    const int ncg = (grp == 0) ? 8 + GLM : 5;
    // stage the group's FP32 primitive state on the tile's halo box (the
    // tile grown by 2 cells, inside the stage's primitive box)
    __syncthreads();
    const int lh0 = T.n[0] + 4, lh1 = T.n[1] + 4, lh2 = (P.sd == 3) ? T.n[2] + 4 : 1;
    const int nlh = lh0 * lh1 * lh2;
    for (int e = t; e < ncg * nlh; e += blockDim.x) {
      const int v = e / nlh, h = e - v * nlh;
      const int a = h % lh0, b = (h / lh0) % lh1, c = h / (lh0 * lh1);
      const long long gi = D.u_off + (q0 + v) * cs +
                           loc(D.flo, D.fn, T.lo[0] - 2 + a, T.lo[1] - 2 + b, T.lo[2] - z0 + c);
      sw[v * S.nh + hidx(S, a, b, c)] = Wf[gi];
    }
    __syncthreads();
    group_faces<GLM>(P, RP, *ss, S, T, TF, grp, sw, sf, sneg);
    __syncthreads();
    group_accumulate(P, S, T, TF, q0, ncg, sf, acc, ncell, grp == 0, divB);
  }

  // the update of the thread's cell
  double dtc = DBL_MAX;
  int myidx = INT_MAX;
  const StageDesc* Dp = (t < ncell) ? &D : nullptr;
  const double psi_damp = GLM ? warp_psi_damping(Dp, states, dt_scale) : 1.0;
  if (t < ncell) {
    const int ci = t % T.n[0], cj = (t / T.n[0]) % T.n[1], ck = t / (T.n[0] * T.n[1]);
    const int i = T.lo[0] + ci, j = T.lo[1] + cj, k = T.lo[2] + ck;
    const long long base = D.u_off + loc(D.flo, D.fn, i, j, k);
    const double dt = ss->dt * dt_scale;
    const int lin = (int)loc(D.vlo, D.vn, i, j, k);
    double u[MF_MAX_COMP];
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.nc) u[q] = B.uin[base + q * cs];
    // UPDATECONS with the FP32 sums of the directions' differences
    const double dtinv = dt * RP.invdx;
#pragma unroll
    for (int q = 0; q < MF_MAX_COMP; ++q)
      if (q < P.ils) u[q] = u[q] - dtinv * fp64::f2d(acc[q * kFusedThreads + t]);
    update_tail<float, GLM, FLAGS, CE>(P, B, D, RP, ss, i, j, k, base, cs, dt, psi_damp, divB, u,
                                       D.g0[kRegV] + lin, dtc, myidx);
  }
  if (FLAGS & kStageDt) block_dt_min(dtc, myidx, descs, ndesc, partials, blockIdx.x);
}

FusedShape fused_shape(const int tile[3], int sd) {
  FusedShape S;
  for (int d = 0; d < 3; ++d) {
    S.t[d] = (d < sd) ? tile[d] : 1;
    S.h[d] = (d < sd) ? tile[d] + 4 : 1;
  }
  S.nh = S.h[0] * S.h[1] * S.h[2];
  S.nfmax = 0;
  for (int d = 0; d < sd; ++d) {
    int n[3] = {S.t[0], S.t[1], S.t[2]};
    n[d] += 1;
    S.nfmax += n[0] * n[1] * n[2];
  }
  S.nfmax = (S.nfmax + 3) & ~3;
  return S;
}

template <int GLM, int FLAGS, typename CE>
cudaError_t fused_launch(const DevParams& P, const StageBuffers& B, const Batch& b,
                         const FusedTile* tiles, int ntiles, const FusedShape& S, size_t smem,
                         double dt_scale, StepState* state, DtPartial* partials, cudaStream_t s) {
  k_fused<GLM, FLAGS, CE><<<ntiles, kFusedThreads, smem, s>>>(P, B, b.desc, b.ndesc, tiles, S,
                                                              b.runs, state, dt_scale, partials);
  return cudaGetLastError();
}

template <int GLM, int FLAGS, typename CE>
cudaError_t fused_allow() {
  return cudaFuncSetAttribute(k_fused<GLM, FLAGS, CE>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kFusedSmemMax);
}

}  // namespace

// Allow every instantiation kFusedSmemMax of dynamic shared memory on the
// current device (once per device, outside any stream capture).
cudaError_t fused_prepare() {
  static bool done[64] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
  const cudaError_t r[] = {
      fused_allow<0, 0, double>(), fused_allow<0, kStageDt, double>(),
      fused_allow<0, kStageAverage | kStageDt, double>(), fused_allow<1, 0, double>(),
      fused_allow<1, kStageDt, double>(), fused_allow<1, kStageAverage | kStageDt, double>(),
      fused_allow<0, 0, float>(), fused_allow<0, kStageDt, float>(),
      fused_allow<0, kStageAverage | kStageDt, float>(), fused_allow<1, 0, float>(),
      fused_allow<1, kStageDt, float>(), fused_allow<1, kStageAverage | kStageDt, float>()};
  for (cudaError_t x : r)
    if (x != cudaSuccess) return x;
  if (dev >= 0 && dev < 64) done[dev] = true;
  return cudaSuccess;
}

size_t fused_smem_bytes(const DevParams& P, const int tile[3]) {
  const FusedShape S = fused_shape(tile, P.sd);
  return sizeof(float) * ((size_t)kGroupMax * S.nh + (size_t)(kGroupMax + 1) * S.nfmax +
                          (size_t)P.ils * kFusedThreads) +
         (size_t)S.nfmax;
}

bool fused_supported(const DevParams& P, int precision, int time_approximation) {
  return precision == MF_PREC_MIXED &&
         (time_approximation == MF_TA_RK2 || time_approximation == MF_TA_FIRST_ORDER) &&
         !P.ct && !P.char_rec && P.nls == 0 && P.divb_method != 2;
}

bool fused_tile_ok(const DevParams& P, const int tile[3]) {
  int cells = 1;
  for (int d = 0; d < P.sd; ++d) {
    if (tile[d] < 1) return false;
    cells *= tile[d];
  }
  return cells <= kFusedThreads && fused_smem_bytes(P, tile) <= kFusedSmemMax;
}

cudaError_t launch_fused(const DevParams& P, const StageBuffers& B, const Batch& b,
                         const FusedTile* tiles, int ntiles, const int tile[3], int flags,
                         double dt_scale, StepState* state, DtPartial* partials, cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  const FusedShape S = fused_shape(tile, P.sd);
  const size_t smem = fused_smem_bytes(P, tile);
#define MF_FUSED(G, FL, CE) \
  return fused_launch<G, FL, CE>(P, B, b, tiles, ntiles, S, smem, dt_scale, state, partials, s)
#define MF_FUSED_CE(G, FL)              \
  do {                                  \
    if (P.ce32) MF_FUSED(G, FL, float); \
    MF_FUSED(G, FL, double);            \
  } while (0)
  if (P.glm) {
    if (flags == 0) MF_FUSED_CE(1, 0);
    if (flags == kStageDt) MF_FUSED_CE(1, kStageDt);
    MF_FUSED_CE(1, kStageAverage | kStageDt);
  } else {
    if (flags == 0) MF_FUSED_CE(0, 0);
    if (flags == kStageDt) MF_FUSED_CE(0, kStageDt);
    MF_FUSED_CE(0, kStageAverage | kStageDt);
  }
#undef MF_FUSED_CE
#undef MF_FUSED
}

}  // namespace mf
