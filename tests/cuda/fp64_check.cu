// Accuracy of the FP64 reciprocal and logarithm of mf_fp64.cuh against the
// CUDA library's 1/x and log: prints the largest differences (in ulps of the
// library's 1/x; in units of 2^-53 max(1, |log x|) for log) over
// log-uniform inputs in [2^-1000, 2^1000] and around 1, and whether the
// special inputs (0, negative, subnormal, inf, NaN) give the library's result.
#include <cstdio>
#include <cstdint>
#include <cmath>
#include <cuda_runtime.h>

#include "mf_fp64.cuh"

__device__ double input(uint32_t i, int j) {
  uint64_t h = (uint64_t)i * 0x9E3779B97F4A7C15ull + (uint64_t)j * 0xD1B54A32D192ED03ull;
  h ^= h >> 29;
  h *= 0xBF58476D1CE4E5B9ull;
  h ^= h >> 32;
  const double u = (double)(h >> 11) * (1.0 / 9007199254740992.0);  // [0,1)
  if (j == 0) return exp2(-1000.0 + 2000.0 * u);
  if (j == 1) return 0.5 + u;          // around 1
  return 1.0 + (u - 0.5) * 1e-6;       // very close to 1
}

__device__ void amax(unsigned long long* a, double v) {
  atomicMax(a, (unsigned long long)(v * 1024.0));
}

__global__ void k_check(int n, unsigned long long* worst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double ulp = 1.1102230246251565e-16;  // 2^-53
  for (int j = 0; j < 3; ++j) {
    const double x = input(i, j);
    const double r = mf::fp64::rcp64(x), rl = 1.0 / x;
    int e;
    frexp(rl, &e);  // rl = f 2^e, f in [0.5, 1): one ulp is 2^(e-53)
    amax(&worst[0], fabs(r - rl) / ldexp(1.0, e - 53));
    const double l = mf::fp64::log64(x), ll = log(x);
    amax(&worst[1], fabs(l - ll) / (fmax(1.0, fabs(ll)) * ulp));
  }
}

// f2d against the conversion instruction, bit for bit, on every exponent
// (subnormals, zeros, inf and NaN included) with hashed fractions and signs
__global__ void k_f2d(int n, unsigned* mismatches) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t h = (uint32_t)i * 2654435761u;
  h ^= h >> 16;
  h *= 2246822519u;
  h ^= h >> 13;
  const unsigned bits = (h & 0x807fffffu) | ((unsigned)(i & 0xff) << 23);
  const float f = __uint_as_float(bits);
  const double a = mf::fp64::f2d(f), b = (double)f;
  const bool same = (__double_as_longlong(a) == __double_as_longlong(b)) || (isnan(a) && isnan(b));
  if (!same) atomicAdd(mismatches, 1u);
}

// d2f against the conversion instruction, bit for bit: doubles over the
// whole exponent range with hashed fractions, and fractions whose 29 dropped
// bits are exactly half, just below and just above half (rounding ties)
__global__ void k_d2f(int n, unsigned* mismatches) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t h = (uint64_t)i * 0x9E3779B97F4A7C15ull;
  h ^= h >> 31;
  h *= 0xBF58476D1CE4E5B9ull;
  h ^= h >> 29;
  const uint64_t expo = (uint64_t)((i >> 2) % 2048) << 52;
  uint64_t frac = h & 0x000fffffffffffffull;
  const int tie = i & 3;  // 0: hashed; 1: exactly half; 2: half - 1; 3: half + 1
  if (tie) frac = (frac & ~0x1fffffffull) | (0x10000000ull + (tie == 2 ? -1ll : tie == 3 ? 1 : 0));
  const uint64_t bits = (h & 0x8000000000000000ull) | expo | frac;
  const double x = __longlong_as_double((long long)bits);
  const float a = mf::fp64::d2f(x), b = (float)x;
  const bool same = (__float_as_uint(a) == __float_as_uint(b)) || (isnan(a) && isnan(b));
  if (!same) atomicAdd(mismatches, 1u);
}

__global__ void k_special(int* bad) {
  const double xs[8] = {0.0, -0.0, -1.0, 4.9406564584124654e-324, 1e-310, INFINITY, -INFINITY, NAN};
  int b = 0;
  for (int q = 0; q < 8; ++q) {
    const double x = xs[q];
    const double r = mf::fp64::rcp64(x), rl = 1.0 / x;
    const double l = mf::fp64::log64(x), ll = log(x);
    if (!((r == rl) || (isnan(r) && isnan(rl)))) b |= 1 << q;
    if (!((l == ll) || (isnan(l) && isnan(ll)))) b |= 1 << (q + 8);
  }
  *bad = b;
}

int main() {
  const int n = 1 << 22;
  unsigned long long* w;
  int* bad;
  if (cudaMalloc(&w, 2 * sizeof(unsigned long long)) != cudaSuccess) return 2;
  if (cudaMalloc(&bad, sizeof(int)) != cudaSuccess) return 2;
  cudaMemset(w, 0, 2 * sizeof(unsigned long long));
  k_check<<<(n + 255) / 256, 256>>>(n, w);
  k_special<<<1, 1>>>(bad);
  unsigned* mm;
  if (cudaMalloc(&mm, sizeof(unsigned)) != cudaSuccess) return 2;
  cudaMemset(mm, 0, sizeof(unsigned));
  k_f2d<<<(n + 255) / 256, 256>>>(n, mm);
  unsigned hm = 1;
  cudaMemcpy(&hm, mm, sizeof(unsigned), cudaMemcpyDeviceToHost);
  cudaMemset(mm, 0, sizeof(unsigned));
  k_d2f<<<(n + 255) / 256, 256>>>(n, mm);
  unsigned hd = 1;
  cudaMemcpy(&hd, mm, sizeof(unsigned), cudaMemcpyDeviceToHost);
  unsigned long long hw[2];
  int hb = -1;
  cudaMemcpy(hw, w, sizeof(hw), cudaMemcpyDeviceToHost);
  cudaMemcpy(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaDeviceSynchronize();
  printf("rcp64_ulp %.4f\nlog64_ulp %.4f\nspecial_mismatch %d\nf2d_mismatch %u\nd2f_mismatch %u\n"
         "status %s\n",
         hw[0] / 1024.0, hw[1] / 1024.0, hb, hm, hd, cudaGetErrorString(e));
  return e == cudaSuccess ? 0 : 1;
}
