// xg_fast_rcp.cuh — the FP64 reciprocal of the FMA load build.
//
// Newton–Raphson on f(x) = 1/x − b: from the hardware's approximate
// reciprocal (PTX rcp.approx.ftz.f64), each step x ← x + x·(1 − b·x) squares
// the relative error, so two steps take a seed good to ~20 bits past double
// precision, leaving the rounding of the last step (within ~1 ulp of 1/b).
// Four fused multiply-adds and no branch on the fast path, against the longer
// correctly rounded sequence of `1.0 / b`.  Outside [2^-1000, 2^1000] (zero,
// subnormal, huge, infinite, NaN; the approximation flushes subnormals) it
// returns the IEEE quotient, tested on the exponent bits with integer
// instructions so the FP64 pipe does not pay for the test.  Held to
// `1.0 / b` within 2 ulp by tests/test_gpu_load.py (xg_probe_reciprocal).
#pragma once

namespace xg {

__device__ __forceinline__ double fast_rcp(double b) {
  const unsigned e = (unsigned(__double2hiint(b)) >> 20) & 0x7ffu;
  if (e - 23u > 2000u) return 1.0 / b;  // biased exponent outside [23, 2023]
  double x;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(x) : "d"(b));
  double t = fma(-b, x, 1.0);
  x = fma(x, t, x);
  t = fma(-b, x, 1.0);
  return fma(x, t, x);
}

}  // namespace xg
