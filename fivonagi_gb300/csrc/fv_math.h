// fv_math.h -- the transcendental functions of the apps' hooks, evaluated
// identically on the host (init hooks, parameter set-up) and the device
// (boundary hooks).
//
// Why: the reference's FP32 state is rounded through (u1 + 1) - 1 by the
// diffusion step every step (apps/na/source.h:40, 84), so a last-bit
// difference in a single ghost value (e.g. a device sinf against a host
// sinf) grows into a ~1e-4 relative difference after a few hundred steps,
// as large as the whole FP32-vs-FP64 error. A host libm and CUDA's device
// library differ in the last bit for some arguments; these functions do
// not, because both sides execute the same IEEE double operations (no FMA
// contraction: device code uses the __d*_rn intrinsics, host code is built
// with -ffp-contract=off) and round once to float.
//
// Method (textbook, e.g. Muller, "Elementary Functions", ch. 6 and 11):
//  * sin/cos: Cody-Waite reduction x = k*pi/2 + r with pi/2 split into
//    three doubles (32 + 32 + 53 bits, so k*PIO2_1 and k*PIO2_2 are exact
//    for |k| < 2^21), then Taylor polynomials of sin and cos on
//    |r| <= pi/4 through r^17 / r^16 (truncation < 1e-17).
//  * exp: x = k*ln2 + r with ln2 split 40 + 53 bits, Taylor through r^13 on
//    |r| <= ln2/2 (truncation < 1e-17), scaled by 2^k.
//  * tanh: e = expm1(2|x|) (Taylor through u^14 for u < 0.35, else
//    exp(u) - 1), tanh = e / (e + 2), sign restored; |x| > 10 gives +-1.
// The double results are accurate to a few 1e-16, so the float results are
// the correctly rounded values except in rare near-halfway cases; the
// tests check them against the host libm to within 1 ulp.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define FVM_HD __host__ __device__ __forceinline__
#else
#define FVM_HD inline
#endif

namespace fvm {

FVM_HD double mul(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
FVM_HD double add(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}
FVM_HD double sub(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
FVM_HD double div(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}

constexpr double PIO2_1 = 1.5707963267341256;       // pi/2, top 32 bits
constexpr double PIO2_2 = 6.077100506303966e-11;    // next 32 bits
constexpr double PIO2_3 = 2.0222662487959506e-21;   // remainder
constexpr double TWO_OVER_PI = 0.6366197723675814;
constexpr double LN2_HI = 0.6931471805592082;       // ln 2, top 40 bits
constexpr double LN2_LO = 7.371002565167799e-13;
constexpr double INV_LN2 = 1.4426950408889634;

// sin(r), cos(r) on |r| <= pi/4: Taylor coefficients (-1)^k/(2k+1)!, (-1)^k/(2k)!
FVM_HD double sin_poly(double r) {
  const double z = mul(r, r);
  double p = 2.8114572543455206e-15;
  p = add(mul(p, z), -7.647163731819816e-13);
  p = add(mul(p, z), 1.6059043836821613e-10);
  p = add(mul(p, z), -2.505210838544172e-08);
  p = add(mul(p, z), 2.7557319223985893e-06);
  p = add(mul(p, z), -0.0001984126984126984);
  p = add(mul(p, z), 0.008333333333333333);
  p = add(mul(p, z), -0.16666666666666666);
  return add(r, mul(mul(r, z), p));
}
FVM_HD double cos_poly(double r) {
  const double z = mul(r, r);
  double p = 4.779477332387385e-14;
  p = add(mul(p, z), -1.1470745597729725e-11);
  p = add(mul(p, z), 2.08767569878681e-09);
  p = add(mul(p, z), -2.755731922398589e-07);
  p = add(mul(p, z), 2.48015873015873e-05);
  p = add(mul(p, z), -0.001388888888888889);
  p = add(mul(p, z), 0.041666666666666664);
  p = add(mul(p, z), -0.5);
  return add(1.0, mul(z, p));
}

// x = k*pi/2 + r; returns r and the quadrant k mod 4
FVM_HD double reduce_pio2(double x, int &q) {
  const double k = rint(mul(x, TWO_OVER_PI));
  double r = sub(x, mul(k, PIO2_1));
  r = sub(r, mul(k, PIO2_2));
  r = sub(r, mul(k, PIO2_3));
  const long long ki = (long long)k;
  q = (int)(ki & 3);
  return r;
}

FVM_HD double sin_d(double x) {
  if (x == 0.0) return x;  // keeps the sign of zero
  int q;
  const double r = reduce_pio2(x, q);
  switch (q) {
    case 0: return sin_poly(r);
    case 1: return cos_poly(r);
    case 2: return -sin_poly(r);
    default: return -cos_poly(r);
  }
}

FVM_HD double cos_d(double x) {
  int q;
  const double r = reduce_pio2(x, q);
  switch (q) {
    case 0: return cos_poly(r);
    case 1: return -sin_poly(r);
    case 2: return -cos_poly(r);
    default: return sin_poly(r);
  }
}

// exp on |x| <= 700
FVM_HD double exp_d(double x) {
  if (x > 709.0) return INFINITY;
  if (x < -745.0) return 0.0;
  const double k = rint(mul(x, INV_LN2));
  double r = sub(x, mul(k, LN2_HI));
  r = sub(r, mul(k, LN2_LO));
  double p = 1.6059043836821613e-10;  // 1/13!
  p = add(mul(p, r), 2.08767569878681e-09);
  p = add(mul(p, r), 2.505210838544172e-08);
  p = add(mul(p, r), 2.755731922398589e-07);
  p = add(mul(p, r), 2.7557319223985893e-06);
  p = add(mul(p, r), 2.48015873015873e-05);
  p = add(mul(p, r), 0.0001984126984126984);
  p = add(mul(p, r), 0.001388888888888889);
  p = add(mul(p, r), 0.008333333333333333);
  p = add(mul(p, r), 0.041666666666666664);
  p = add(mul(p, r), 0.16666666666666666);
  p = add(mul(p, r), 0.5);
  p = add(mul(p, r), 1.0);
  p = add(mul(p, r), 1.0);
  return ldexp(p, (int)k);
}

FVM_HD double expm1_d(double u) {
  if (u < 0.35 && u > -0.35) {
    double p = 1.1470745597729725e-11;  // 1/14!
    p = add(mul(p, u), 1.6059043836821613e-10);
    p = add(mul(p, u), 2.08767569878681e-09);
    p = add(mul(p, u), 2.505210838544172e-08);
    p = add(mul(p, u), 2.755731922398589e-07);
    p = add(mul(p, u), 2.7557319223985893e-06);
    p = add(mul(p, u), 2.48015873015873e-05);
    p = add(mul(p, u), 0.0001984126984126984);
    p = add(mul(p, u), 0.001388888888888889);
    p = add(mul(p, u), 0.008333333333333333);
    p = add(mul(p, u), 0.041666666666666664);
    p = add(mul(p, u), 0.16666666666666666);
    p = add(mul(p, u), 0.5);
    p = add(mul(p, u), 1.0);
    return mul(p, u);
  }
  return sub(exp_d(u), 1.0);
}

FVM_HD double tanh_d(double x) {
  const double t = fabs(x);
  if (t > 10.0) return x > 0 ? 1.0 : -1.0;
  const double e = expm1_d(add(t, t));
  const double r = div(e, add(e, 2.0));
  return copysign(r, x);
}

FVM_HD float sinf_(float x) { return (float)sin_d((double)x); }
FVM_HD float cosf_(float x) { return (float)cos_d((double)x); }
FVM_HD float expf_(float x) { return (float)exp_d((double)x); }
FVM_HD float tanhf_(float x) { return (float)tanh_d((double)x); }

}  // namespace fvm
