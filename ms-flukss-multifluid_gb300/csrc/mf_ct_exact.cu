// mf_ct_exact.cu - constrained transport (mf_params.divb_cleaning 1-3,
// eDivergenceCleaning DC_CT_BS / DC_CT_GS0 / DC_CT_GS1, src/PatchMHDAM.H:43-50):
//
//   k_efield      the edge field of a stage's face fluxes
//                 (PatchMHDMF::calculateElectricField, srcIdeal/PatchMHDMF.cpp:
//                 1487-1560 -> electricFieldBS / electricFieldGS0 / GS1,
//                 srcIdeal/DivCleaningF.ChF:75-854), and for the second RK2
//                 stage the step average (E + E_predictor) / 2 of updateState
//                 (src/PatchMHDAM.cpp:1266-1275)
//   k_recalc_b    the cell field from an old field and the edge field
//                 (recalculateB, srcIdeal/DivCleaningF.ChF:4-72), with the
//                 AVERAGESTATE of the second RK2 stage fused after it
//   k_recalc_ext  the same on caller fabs (recalculateMagneticField)
//   k_edges_out   the step's edge field into the caller's EdgeBox fabs
//
// Built with -fmad=false: every sum and product rounds as in the CPU
// restatement of the reference.
//
// Internal edge-field storage: three components laid out like U on each
// patch's fab (the patch's cell offset in U times 3); the edge whose node
// indices are (i,j,k) - cell-centred along its own direction - is stored at
// cell (i,j,k).  Every edge a stage touches lies inside the fab: the
// valueBox of each stage keeps at least one cell to the fab's high side.
// In 2D the single nodal field (EdgeBox keeps one array there, src/EdgeBox.cpp:
// 5-12, 63-73) is component 0.
#include "mf_internal.h"
#include "mf_kernels.cuh"
#include "mf_sources_exact.cuh"

namespace mf {
namespace {

__device__ __forceinline__ long long ct_stride(const int* n, int d) {
  return (d == 0) ? 1 : (d == 1) ? (long long)n[0] : (long long)n[0] * n[1];
}

// Face flux component q of direction d at face index x (the face box is the
// valueBox made nodal along d).
template <typename R>
struct FaceView {
  const R* f[3];
  int vlo[3], fn[3][3];
  long long fcs[3];
  __device__ __forceinline__ double operator()(int d, int q, int i, int j, int k) const {
    const int* n = fn[d];
    const long long o = (long long)(i - vlo[0]) + (long long)n[0] * ((j - vlo[1]) + (long long)n[1] * (k - vlo[2]));
    return (double)f[d][q * fcs[d] + o];
  }
};

// electricFieldBS (DivCleaningF.ChF:75-310) at node (i,j,k).  2D: the
// literal weights H4, H3, H2 times the sum of the present terms in the
// routine's order; 3D: the sum over the present faces divided by their count.
template <typename R>
__device__ void edge_bs(int sd, const FaceView<R>& F, const int* lo, const int* hi, int i, int j,
                        int k, double* out, bool* has) {
  const double H2 = 0.5, H3 = 0.333333333333333333333333333333333333, H4 = 0.25;
  if (sd == 2) {
    double s = 0.0;
    int n = 0;
    if (i > lo[0]) {
      s = F(1, 5, i - 1, j, k);
      n = 1;
    }
    if (i <= hi[0]) {
      s = n ? s + F(1, 5, i, j, k) : F(1, 5, i, j, k);
      n += 1;
    }
    if (j > lo[1]) {
      s = s - F(0, 6, i, j - 1, k);
      n += 1;
    }
    if (j <= hi[1]) {
      s = s - F(0, 6, i, j, k);
      n += 1;
    }
    out[0] = ((n == 4) ? H4 : (n == 3) ? H3 : H2) * s;
    has[0] = true;
    return;
  }
  if (i <= hi[0]) {  // EX: z-flux of By, y-flux of Bz
    double EE = 0.0;
    int iE = 0;
    if (j > lo[1]) { EE = EE + F(2, 6, i, j - 1, k); iE = iE + 1; }
    if (j <= hi[1]) { EE = EE + F(2, 6, i, j, k); iE = iE + 1; }
    if (k > lo[2]) { EE = EE - F(1, 7, i, j, k - 1); iE = iE + 1; }
    if (k <= hi[2]) { EE = EE - F(1, 7, i, j, k); iE = iE + 1; }
    out[0] = EE / iE;
    has[0] = true;
  }
  if (j <= hi[1]) {  // EY: z-flux of Bx, x-flux of Bz
    double EE = 0.0;
    int iE = 0;
    if (i > lo[0]) { EE = EE - F(2, 5, i - 1, j, k); iE = iE + 1; }
    if (i <= hi[0]) { EE = EE - F(2, 5, i, j, k); iE = iE + 1; }
    if (k > lo[2]) { EE = EE + F(0, 7, i, j, k - 1); iE = iE + 1; }
    if (k <= hi[2]) { EE = EE + F(0, 7, i, j, k); iE = iE + 1; }
    out[1] = EE / iE;
    has[1] = true;
  }
  if (k <= hi[2]) {  // EZ: y-flux of Bx, x-flux of By
    double EE = 0.0;
    int iE = 0;
    if (i > lo[0]) { EE = EE + F(1, 5, i - 1, j, k); iE = iE + 1; }
    if (i <= hi[0]) { EE = EE + F(1, 5, i, j, k); iE = iE + 1; }
    if (j > lo[1]) { EE = EE - F(0, 6, i, j - 1, k); iE = iE + 1; }
    if (j <= hi[1]) { EE = EE - F(0, 6, i, j, k); iE = iE + 1; }
    out[2] = EE / iE;
    has[2] = true;
  }
}

// electricFieldGS0 / GS1 in 2D (DivCleaningF.ChF:335-408, 596-697): the face
// average corrected by the face fluxes minus the cell-centred field
// EQ = u_y B_x - u_x B_y of the cells around the node; GS1 keeps the cell on
// the upwind side of each face by the sign of its mass flux.  w(c, ii, jj):
// primitive component c of cell (ii, jj).
template <typename R, typename WAt>
__device__ double edge_gs2(const FaceView<R>& F, const WAt& w, const int* lo, const int* hi,
                           int i, int j, int k, bool upwind) {
  double EE = 0.0, EQ, DEDD;
  int iE = 0;
  double D1_00 = 0.0, D2_00 = 0.0, D1_10 = 0.0, D2_10 = 0.0;
  double D1_01 = 0.0, D2_01 = 0.0, D1_11 = 0.0, D2_11 = 0.0;
  int i00 = 0, i10 = 0, i01 = 0, i11 = 0;
  auto eq = [&](int ii, int jj) { return w(2, ii, jj) * w(5, ii, jj) - w(1, ii, jj) * w(6, ii, jj); };
  if ((lo[0] < i) && (lo[1] < j)) {
    EQ = eq(i - 1, j - 1);
    D1_00 = -F(0, 6, i, j - 1, k) - EQ;
    D2_00 = F(1, 5, i - 1, j, k) - EQ;
    i00 = 1;
  }
  if ((hi[0] >= i) && (lo[1] < j)) {
    EQ = eq(i, j - 1);
    D1_10 = EQ + F(0, 6, i, j - 1, k);
    D2_10 = F(1, 5, i, j, k) - EQ;
    i10 = 1;
  }
  if ((lo[0] < i) && (hi[1] >= j)) {
    EQ = eq(i - 1, j);
    D1_01 = -F(0, 6, i, j, k) - EQ;
    D2_01 = EQ - F(1, 5, i - 1, j, k);
    i01 = 1;
  }
  if ((hi[0] >= i) && (hi[1] >= j)) {
    EQ = eq(i, j);
    D1_11 = EQ + F(0, 6, i, j, k);
    D2_11 = EQ - F(1, 5, i, j, k);
    i11 = 1;
  }
  // the upwind choice of GS1 between the two cells beside a face
  auto pick = [&](int& iMN, int& iPL, double m) {
    if (iMN * m > 0.0)
      iPL = 0;
    else if (iPL * m < 0.0)
      iMN = 0;
  };
  if (lo[0] < i) {
    if (upwind) {
      int iMN = i00, iPL = i01;
      pick(iMN, iPL, F(1, 0, i - 1, j, k));
      DEDD = (iPL * D1_01 + iMN * D1_00) / (iPL + iMN);
    } else {
      DEDD = (D1_01 + D1_00) / (i01 + i00);
    }
    EE = EE + F(1, 5, i - 1, j, k) + DEDD;
    iE = iE + 1;
  }
  if (hi[0] >= i) {
    if (upwind) {
      int iMN = i10, iPL = i11;
      pick(iMN, iPL, F(1, 0, i, j, k));
      DEDD = (iMN * D1_10 + iPL * D1_11) / (iMN + iPL);
    } else {
      DEDD = (D1_10 + D1_11) / (i10 + i11);
    }
    EE = EE + F(1, 5, i, j, k) - DEDD;
    iE = iE + 1;
  }
  if (lo[1] < j) {
    if (upwind) {
      int iMN = i00, iPL = i10;
      pick(iMN, iPL, F(0, 0, i, j - 1, k));
      DEDD = (iMN * D2_00 + iPL * D2_10) / (iMN + iPL);
    } else {
      DEDD = (D2_00 + D2_10) / (i00 + i10);
    }
    EE = EE - F(0, 6, i, j - 1, k) + DEDD;
    iE = iE + 1;
  }
  if (hi[1] >= j) {
    if (upwind) {
      int iMN = i01, iPL = i11;
      pick(iMN, iPL, F(0, 0, i, j, k));
      DEDD = (iMN * D2_01 + iPL * D2_11) / (iMN + iPL);
    } else {
      DEDD = (D2_01 + D2_11) / (i01 + i11);
    }
    EE = EE - F(0, 6, i, j, k) - DEDD;
    iE = iE + 1;
  }
  return EE / iE;
}

// One thread per cell of each desc's W box; the threads on the nodes of the
// valueBox compute the edges there.  E1 / Eavg (nullable): the first RK2
// stage's field and the step average written on the same edges.
template <typename R>
__global__ void __launch_bounds__(kMaxBlock)
    k_efield(const __grid_constant__ DevParams P, const void* f0, const void* f1, const void* f2,
             const double* __restrict__ W, double* __restrict__ E, const double* __restrict__ E1,
             double* __restrict__ Eavg, const StageDesc* __restrict__ descs, int ndesc,
             int total) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const StageDesc& D = descs[find_desc(descs, ndesc, kRegW, g)];
  const int lin = g - D.g0[kRegW];
  int x[3];
  decode(lin, D.wlo, D.wn, x[0], x[1], x[2]);
  int lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = D.vlo[d];
    hi[d] = D.vlo[d] + D.vn[d] - 1;
    const int top = (d < P.sd) ? hi[d] + 1 : hi[d];
    if (x[d] < lo[d] || x[d] > top) return;
  }
  FaceView<R> F;
  const void* fp[3] = {f0, f1, f2};
  for (int d = 0; d < 3; ++d) {
    F.vlo[d] = D.vlo[d];
    for (int e = 0; e < 3; ++e) F.fn[d][e] = D.vn[e] + ((e == d && d < P.sd) ? 1 : 0);
    F.fcs[d] = (long long)F.fn[d][0] * F.fn[d][1] * F.fn[d][2];
    F.f[d] = (d < P.sd) ? (const R*)fp[d] + D.f_off[d] : nullptr;
  }
  const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
  const long long cell0 = D.u_off / P.nc;  // the patch's cell offset in U
  const long long e = cell0 * 3 + loc(D.flo, D.fn, x[0], x[1], x[2]);
  double out[3] = {0.0, 0.0, 0.0};
  bool has[3] = {false, false, false};
  if (P.ct == 1 || P.sd == 3) {
    edge_bs<R>(P.sd, F, lo, hi, x[0], x[1], x[2], out, has);
  } else {
    const long long wb = D.u_off;
    auto w = [&](int c, int ii, int jj) {
      return W[wb + loc(D.flo, D.fn, ii, jj, x[2]) + c * cs];
    };
    out[0] = edge_gs2<R>(F, w, lo, hi, x[0], x[1], x[2], P.ct == 3);
    has[0] = true;
  }
  for (int d = 0; d < 3; ++d)
    if (has[d]) {
      E[e + d * cs] = out[d];
      if (Eavg) {  // a_E += EPredictor; a_E *= 0.5
        double a = out[d] + E1[e + d * cs];
        Eavg[e + d * cs] = a * 0.5;
      }
    }
}

// recalculateB (DivCleaningF.ChF:4-72) of one cell: ub / bo / eat give U,
// the old field (components 5..7) and the edge field at offsets from the
// cell; HX = dt / (2 dx).  Writes B and the energy with its magnetic part
// replaced.
template <typename UAt, typename BAt, typename EAt>
__device__ __forceinline__ void recalc_cell(int sd, double HX, const UAt& u, const BAt& bo,
                                            const EAt& E) {
  double bx = u(5), by = u(6), bz = u(7);
  double b = kInv8Pi * (bx * bx + by * by + bz * bz);
  const double e = u(4) - b;
  bx = bo(5) - HX * (E(2, 1, 1, 0) + E(2, 0, 1, 0) - E(2, 1, 0, 0) - E(2, 0, 0, 0));
  by = bo(6) + HX * (E(2, 1, 1, 0) + E(2, 1, 0, 0) - E(2, 0, 1, 0) - E(2, 0, 0, 0));
  if (sd == 3) {
    bx = bx + HX * (E(1, 1, 0, 1) + E(1, 0, 0, 1) - E(1, 1, 0, 0) - E(1, 0, 0, 0));
    by = by - HX * (E(0, 0, 1, 1) + E(0, 0, 0, 1) - E(0, 0, 1, 0) - E(0, 0, 0, 0));
    bz = bo(7) - HX * (E(1, 1, 0, 1) + E(1, 1, 0, 0) - E(1, 0, 0, 1) - E(1, 0, 0, 0) -
                       (E(0, 0, 1, 1) + E(0, 0, 1, 0) - E(0, 0, 0, 1) - E(0, 0, 0, 0)));
  }
  b = kInv8Pi * (bx * bx + by * by + bz * bz);
  u.set(4, e + b);
  u.set(5, bx);
  u.set(6, by);
  u.set(7, bz);
}

// Per cell of each desc's valueBox: recalculateB from Bold (components 5..7
// laid out like U: the stage-start primitive state or the level's UOld) and
// the internal edge field.  POST: a stage's recalculation, followed as in
// EulerStep / correctorHancock (src/PatchMHDAM.cpp:684-707, 1150-1166) by the
// inner-sphere reset and the positivity fix, and with U0 / U1 set by the
// AVERAGESTATE of the second RK2 stage, U += (U0 - U1) / 2 over every
// component.  Without POST: the level's recalculation alone
// (AMRLevelIdealMHD::postTimeStep).  Constrained transport excludes GLM, so
// the neutral fluids start at component 8.
template <int POST>
__global__ void __launch_bounds__(kMaxBlock)
    k_recalc_b(const __grid_constant__ DevParams P, double* __restrict__ U, const double* __restrict__ Bold,
               const double* __restrict__ E, const double* __restrict__ U0,
               const double* __restrict__ U1, const StepState* __restrict__ states,
               double dt_scale, const StageDesc* __restrict__ descs, int ndesc, int total,
               const RunParams* __restrict__ runs) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const StageDesc& D = descs[find_desc(descs, ndesc, kRegV, g)];
  const int lin = g - D.g0[kRegV];
  if (lin >= D.vn[0] * D.vn[1] * D.vn[2]) return;  // run-alignment gap
  int i, j, k;
  decode(lin, D.vlo, D.vn, i, j, k);
  const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
  const long long c = loc(D.flo, D.fn, i, j, k);
  const long long base = D.u_off + c;
  const long long eb = D.u_off / P.nc * 3 + c;
  const long long sy = ct_stride(D.fn, 1), sz = ct_stride(D.fn, 2);
  const RunParams& RP = runs[D.run];
  const double dt = states[D.run].dt * dt_scale;
  const double HX = 0.5 * dt / RP.dx;
  double u[MF_MAX_COMP];
#pragma unroll
  for (int q = 0; q < MF_MAX_COMP; ++q)
    if (q < P.nc) u[q] = U[base + q * cs];
  struct {
    double* p;
    __device__ double operator()(int q) const { return p[q]; }
    __device__ void set(int q, double v) const { p[q] = v; }
  } ua{u};
  auto bo = [&](int q) { return Bold[base + q * cs]; };
  const int sd = P.sd;
  auto ea = [&](int d, int di, int dj, int dk) {
    return E[eb + (sd == 3 ? d : 0) * cs + di + dj * sy + dk * sz];
  };
  recalc_cell(P.sd, HX, ua, bo, ea);
  if (POST) {
    if (P.reinit) exact::reinit_cell(P, RP.dx, i, j, k, states[D.run].time + dt, u);
    exact::positivity_cell<8>(P, u);
    if (U0) {
#pragma unroll
      for (int q = 0; q < MF_MAX_COMP; ++q)
        if (q < P.nc) u[q] = u[q] + 0.5 * (U0[base + q * cs] - U1[base + q * cs]);
    }
  }
#pragma unroll
  for (int q = 0; q < MF_MAX_COMP; ++q)
    if (q < P.nc) U[base + q * cs] = u[q];
}

// A fab given by pointer, box lo and extents.
struct FabView {
  double* p;
  int lo[3], n[3];
  __device__ __forceinline__ long long at(int i, int j, int k) const {
    return (long long)(i - lo[0]) + (long long)n[0] * ((j - lo[1]) + (long long)n[1] * (k - lo[2]));
  }
  __host__ __device__ __forceinline__ long long cs() const {
    return (long long)n[0] * n[1] * n[2];
  }
};

__global__ void __launch_bounds__(128)
    k_recalc_ext(int sd, FabView U, FabView Uo, FabView e0, FabView e1, FabView e2, double HX,
                 int blo0, int blo1, int blo2, int bn0, int bn1, int bn2) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)bn0 * bn1 * bn2) return;
  const int i = blo0 + (int)(t % bn0), j = blo1 + (int)((t / bn0) % bn1),
            k = blo2 + (int)(t / ((long long)bn0 * bn1));
  const long long cu = U.at(i, j, k), co = Uo.at(i, j, k);
  struct {
    double* p;
    long long cs;
    __device__ double operator()(int q) const { return p[q * cs]; }
    __device__ void set(int q, double v) const { p[q * cs] = v; }
  } u{U.p + cu, U.cs()};
  auto bo = [&](int q) { return Uo.p[co + q * Uo.cs()]; };
  const FabView* ev[3] = {&e0, &e1, &e2};
  auto ea = [&](int d, int di, int dj, int dk) {
    const FabView& f = *ev[d];
    return f.p[f.at(i + di, j + dj, k + dk)];
  };
  recalc_cell(sd, HX, u, bo, ea);
}

// The internal edge field of a single-patch call (fab box flo / fn, cell
// offset 0) into the caller's EdgeBox fab of direction d, on the edges of
// the valid box (elo / en: that edge box, inside both the fab and `out`).
__global__ void __launch_bounds__(128)
    k_edges_out(const double* __restrict__ E, int d, int flo0, int flo1, int flo2, int fn0,
                int fn1, int fn2, int elo0, int elo1, int elo2, int en0, int en1, int en2,
                FabView out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)en0 * en1 * en2) return;
  const int i = elo0 + (int)(t % en0);
  const int j = elo1 + (int)((t / en0) % en1);
  const int k = elo2 + (int)(t / ((long long)en0 * en1));
  const long long cs = (long long)fn0 * fn1 * fn2;
  const long long c = (long long)(i - flo0) + (long long)fn0 * ((j - flo1) + (long long)fn1 * (k - flo2));
  out.p[out.at(i, j, k)] = E[d * cs + c];
}

}  // namespace

cudaError_t launch_efield(const DevParams& P, int mixed, const void* const f[3],
                          const double* w, double* e, const double* e1, double* eavg,
                          const Batch& b, cudaStream_t s) {
  if (b.tot_w <= 0) return cudaSuccess;
  const int nt = b.nt[0];
  const unsigned g = flat_blocks(b.tot_w, nt);
  if (mixed)
    k_efield<float><<<g, nt, 0, s>>>(P, f[0], f[1], f[2], w, e, e1, eavg, b.desc, b.ndesc,
                                     b.tot_w);
  else
    k_efield<double><<<g, nt, 0, s>>>(P, f[0], f[1], f[2], w, e, e1, eavg, b.desc, b.ndesc,
                                      b.tot_w);
  return cudaGetLastError();
}

cudaError_t launch_recalc_b(const DevParams& P, double* u, const double* bold, const double* e,
                            const double* u0, const double* u1, const StepState* state,
                            double dt_scale, int stage, const Batch& b, cudaStream_t s) {
  if (b.tot_v <= 0) return cudaSuccess;
  const int nt = b.nt[2];
  const unsigned g = flat_blocks(b.tot_v, nt);
  if (stage)
    k_recalc_b<1><<<g, nt, 0, s>>>(P, u, bold, e, u0, u1, state, dt_scale, b.desc, b.ndesc,
                                   b.tot_v, b.runs);
  else
    k_recalc_b<0><<<g, nt, 0, s>>>(P, u, bold, e, u0, u1, state, dt_scale, b.desc, b.ndesc,
                                   b.tot_v, b.runs);
  return cudaGetLastError();
}

static FabView fab_view(double* p, const mf_box& bx) {
  FabView v;
  v.p = p;
  for (int d = 0; d < 3; ++d) {
    v.lo[d] = bx.lo[d];
    v.n[d] = bx.hi[d] - bx.lo[d] + 1;
  }
  return v;
}

cudaError_t launch_recalc_ext(int sd, double dx, mf_fab* U, const mf_fab* Uold, const mf_fab* E,
                              double dt, const mf_box& box, cudaStream_t s) {
  const long long n = (long long)(box.hi[0] - box.lo[0] + 1) * (box.hi[1] - box.lo[1] + 1) *
                      (box.hi[2] - box.lo[2] + 1);
  if (n <= 0) return cudaSuccess;
  FabView ev[3];
  for (int d = 0; d < 3; ++d) {
    const mf_fab& f = E[(sd == 3) ? d : 0];
    ev[d] = fab_view(f.data, f.box);
  }
  const double HX = 0.5 * dt / dx;
  k_recalc_ext<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(
      sd, fab_view(U->data, U->box), fab_view(Uold->data, Uold->box), ev[0], ev[1], ev[2], HX,
      box.lo[0], box.lo[1], box.lo[2], box.hi[0] - box.lo[0] + 1, box.hi[1] - box.lo[1] + 1,
      box.hi[2] - box.lo[2] + 1);
  return cudaGetLastError();
}

cudaError_t launch_edges_out(int sd, const double* e, const mf_box& fab, const mf_box& valid,
                             mf_fab* out, cudaStream_t s) {
  const int nd = (sd == 3) ? 3 : 1;
  for (int d = 0; d < nd; ++d) {
    int elo[3], en[3];
    for (int q = 0; q < 3; ++q) {
      elo[q] = valid.lo[q];
      en[q] = valid.hi[q] - valid.lo[q] + 1 + ((q < sd && !(sd == 3 && q == d)) ? 1 : 0);
    }
    const long long n = (long long)en[0] * en[1] * en[2];
    if (n <= 0) continue;
    k_edges_out<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(
        e, d, fab.lo[0], fab.lo[1], fab.lo[2], fab.hi[0] - fab.lo[0] + 1,
        fab.hi[1] - fab.lo[1] + 1, fab.hi[2] - fab.lo[2] + 1, elo[0], elo[1], elo[2], en[0],
        en[1], en[2], fab_view(out[d].data, out[d].box));
  }
  return cudaGetLastError();
}

}  // namespace mf
