// mf_fp64.cuh - FP64 reciprocal and logarithm with fewer FP64-pipe
// instructions than the correctly rounded library forms, for the paths that
// do not reproduce the reference's rounding (MF_PREC_FP64_FAST and the FP64
// charge-exchange rates of MF_PREC_MIXED).  GB300 issues FP64 arithmetic at a
// small fraction of its FP32 rate, so on those paths every FP64 instruction
// counts against the step time.
//
// rcp64: the hardware's approximate FP64 reciprocal (rcp.approx.ftz.f64,
// relative error about 2^-20) refined by one third-order Newton-Raphson step
// y <- y (1 + e + e^2), e = 1 - x y, whose truncation error is e^3 (< 2^-58):
// 3 FP64 instructions, within one ulp of the correctly rounded 1/x.
//
// f2d: the exact FP32 -> FP64 conversion done with integer instructions;
// d2f: the rounded FP64 -> FP32 conversion likewise (normal results).
//
// log64: Tang's table-driven method (P. T. P. Tang, "Table-driven
// implementation of the logarithm function in IEEE floating-point
// arithmetic", ACM TOMS 16(4), 1990): x = 2^k m with m in [1, 2), a table
// entry c_j (j = the leading seven bits of m's fraction, c_j the midpoint of
// its interval) holds rc_j = 1/c_j rounded and L_j = -log(rc_j); then
// r = m rc_j - 1 in one fused multiply-add, |r| <= 2^-8, and
// log x = k log 2 + L_j + log1p(r) with log1p(r) from its Taylor series to
// r^6 (truncation below 2^-58).  10 FP64 instructions, absolute error a few
// units of 2^-53 max(1, |log x|).  The table is built at compile time from
// the series log z = 2 atanh((z - 1) / (z + 1)).
#pragma once

#include <cuda_runtime.h>

namespace mf {
namespace fp64 {

struct LogTable {
  double2 e[128];  // {rc_j, L_j}
};

constexpr double series_log(double z) {
  const double s = (z - 1.0) / (z + 1.0), s2 = s * s;
  double term = s, sum = 0.0;
  for (int n = 0; n < 40; ++n) {
    sum += term / (2 * n + 1);
    term *= s2;
  }
  return 2.0 * sum;
}

constexpr LogTable make_log_table() {
  LogTable t{};
  for (int j = 0; j < 128; ++j) {
    const double c = 1.0 + (j + 0.5) / 128.0;
    const double rc = 1.0 / c;
    t.e[j].x = rc;
    t.e[j].y = -series_log(rc);
  }
  return t;
}

static __device__ constexpr LogTable kLogTable = make_log_table();

constexpr double kLn2 = 0.693147180559945309417232121458176568;

__device__ __forceinline__ double rcp_seed(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  return y;
}

// 1/x for |x| in [2^-1021, 2^1020); outside that (zero, subnormal, huge,
// inf, NaN) the library's division, which the seed would not cover.
__device__ __forceinline__ double rcp64(double x) {
  const unsigned ahi = static_cast<unsigned>(__double2hiint(x)) & 0x7fffffffu;
  if (ahi < 0x00200000u || ahi >= 0x7fb00000u) return 1.0 / x;
  const double y = rcp_seed(x);
  const double e = fma(-x, y, 1.0);
  return fma(y, fma(e, e, e), y);
}

// log(x) for normal positive x; other x (zero, negative, subnormal, inf,
// NaN) take the library's log.
__device__ __forceinline__ double log64(double x) {
  const int hi = __double2hiint(x);
  if (hi < 0x00100000 || hi >= 0x7ff00000) return log(x);
  const int lo = __double2loint(x);
  const int k = (hi >> 20) - 1023;
  const double m = __hiloint2double((hi & 0x000fffff) | 0x3ff00000, lo);
  const double2 t = __ldg(&kLogTable.e[(hi >> 13) & 127]);
  const double r = fma(m, t.x, -1.0);
  // k as a double: 2^52 + 2^31 + k assembled in the bits, minus 2^52 + 2^31
  const double kd =
      __hiloint2double(0x43300000, static_cast<int>(static_cast<unsigned>(k) ^ 0x80000000u)) -
      4503601774854144.0;
  double p = fma(r, -1.0 / 6.0, 1.0 / 5.0);
  p = fma(p, r, -1.0 / 4.0);
  p = fma(p, r, 1.0 / 3.0);
  p = fma(p, r, -0.5);
  const double l1p = fma(p, r * r, r);
  return fma(kd, kLn2, t.y) + l1p;
}

// Exact FP32 -> FP64 conversion in integer arithmetic (the same value as
// the conversion instruction, which issues on the FP64 pipe): sign and
// fraction move into place, the exponent is rebiased by 1023 - 127; a
// subnormal input is normalised by its leading-zero count; zero stays a
// signed zero and inf / NaN keep their fraction.
__device__ __forceinline__ double f2d(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned sign = b & 0x80000000u;
  const unsigned e = (b >> 23) & 0xffu;
  unsigned m = b & 0x007fffffu;
  unsigned ed;
  if (e == 0xffu) {
    ed = 0x7ffu;
  } else if (e != 0u) {
    ed = e + 896u;
  } else if (m == 0u) {
    ed = 0u;
  } else {  // subnormal: m * 2^-149, shift the leading one to bit 23
    const int sh = __clz(m) - 8;
    m = (m << sh) & 0x007fffffu;
    ed = 897u - static_cast<unsigned>(sh);
  }
  return __hiloint2double(static_cast<int>(sign | (ed << 20) | (m >> 3)),
                          static_cast<int>(m << 29));
}

// FP64 -> FP32 conversion, round to nearest even, in integer arithmetic (the
// conversion instruction's result, bit for bit) for results in the normal
// FP32 range: the 52-bit fraction keeps its leading 23 bits, the 29 dropped
// bits decide the rounding (above half, or exactly half with an odd last
// bit), and a carry out of the fraction moves into the exponent (up to inf).
// Zero stays a signed zero; results below the normal range, inf and NaN
// take the conversion instruction.
__device__ __forceinline__ float d2f(double x) {
  const unsigned hi = static_cast<unsigned>(__double2hiint(x));
  const unsigned lo = static_cast<unsigned>(__double2loint(x));
  const unsigned sign = hi & 0x80000000u;
  const unsigned e = (hi >> 20) & 0x7ffu;
  if (e - 897u < 254u) {  // FP32 exponent e - 896 in [1, 254]
    const unsigned m = ((hi & 0x000fffffu) << 3) | (lo >> 29);
    const unsigned rem = lo & 0x1fffffffu;
    unsigned bits = ((e - 896u) << 23) | m;
    bits += (rem > 0x10000000u || (rem == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return __uint_as_float(sign | bits);
  }
  if ((hi & 0x7fffffffu) == 0u && lo == 0u) return __uint_as_float(sign);
  return static_cast<float>(x);
}

}  // namespace fp64
}  // namespace mf
