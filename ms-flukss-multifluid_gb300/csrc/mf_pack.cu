// mf_pack.cu - the valid cells of a level between its fab layout and a packed
// layout without ghosts (patch p's valid box at nc x its first valid cell,
// component-major, x fastest), for host transfers of the valid state only.
// One thread per valid cell over the stage descs of the level (valueBox =
// valid box, consecutive patches, no alignment gaps within the one run).
#include "mf_kernels.cuh"

namespace mf {
namespace {

template <int TO_FAB>
__global__ void __launch_bounds__(kMaxBlock)
    k_pack(double* __restrict__ U, double* __restrict__ packed, const StageDesc* __restrict__ descs,
           int ndesc, int total, int nc) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= total) return;
  const StageDesc& D = descs[find_desc(descs, ndesc, kRegV, g)];
  const int lin = g - D.g0[kRegV];
  const long long cells = (long long)D.vn[0] * D.vn[1] * D.vn[2];
  if (lin >= cells) return;
  int i, j, k;
  decode(lin, D.vlo, D.vn, i, j, k);
  const long long cs = (long long)D.fn[0] * D.fn[1] * D.fn[2];
  const long long f = D.u_off + loc(D.flo, D.fn, i, j, k);
  const long long p = (long long)nc * D.g0[kRegV] + lin;
  for (int q = 0; q < nc; ++q) {
    if (TO_FAB)
      U[f + q * cs] = packed[p + q * cells];
    else
      packed[p + q * cells] = U[f + q * cs];
  }
}

}  // namespace

cudaError_t launch_pack(double* u, double* packed, const Batch& b, int nc, int to_fab,
                        cudaStream_t s) {
  if (b.tot_v <= 0) return cudaSuccess;
  const int nt = b.nt[2];
  if (to_fab)
    k_pack<1><<<flat_blocks(b.tot_v, nt), nt, 0, s>>>(u, packed, b.desc, b.ndesc, b.tot_v, nc);
  else
    k_pack<0><<<flat_blocks(b.tot_v, nt), nt, 0, s>>>(u, packed, b.desc, b.ndesc, b.tot_v, nc);
  return cudaGetLastError();
}

}  // namespace mf
