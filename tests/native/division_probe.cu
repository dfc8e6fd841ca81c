// Checks the step kernel's FMA division (fvgb::DivFma, fv_device.cuh)
// against the GPU's IEEE-754 division.
//
//  1. Exhaustive: for every float b with 2^-126 <= |b| <= 2^24 the refined
//     reciprocal fvgb::refined_recip(b) equals the IEEE quotient 1/b
//     (condition (1) of the Markstein argument in fv_device.cuh).
//  2. Sampled div(): quotients over operand classes that straddle every
//     bound of the safety check (dividends near 2^-100 and 2^39, divisors
//     near 2^-85 and 2^24, powers of two with any dividend, zeros,
//     subnormals, all-ones significands, solver-like magnitudes, divisors
//     from zero through the subnormals to 2^-124). Every
//     quotient the policy does not flag as unsafe must equal the IEEE
//     quotient bit for bit (NaN matching NaN).
//  3. Sampled DivExact::div() over the same classes, and DivExact::ratio()
//     over the limiter's: every quotient it does not flag (it flags only
//     operands out of range, NaN and infinity) must equal the IEEE quotient.
//     The same for DivNormal::div(), which also flags subnormal quotients.
//  4. Sampled ratio(): the limiter's quotient of a product-like dividend
//     and a positive sum-of-squares divisor. Unflagged results equal the
//     IEEE quotient (DivNormal's as a value: a zero may have either sign),
//     or, for DivFma where that exceeds 2^59 in magnitude, have its sign and
//     more than 2^59 in magnitude.
//
// Prints one line per check: "<name> <count> <flagged> <mismatches>" and
// exits 0 when no check found a mismatch.
#include <cstdint>
#include <cstdio>

#include "fv_device.cuh"

namespace {

__device__ __forceinline__ uint64_t mix(uint64_t x) {
  x += 0x9e3779b97f4a7c15ull;
  x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
  x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
  return x ^ (x >> 31);
}

// a float with random sign and significand and exponent in [emin, emax]
// (emax <= 127); exponents below -126 give subnormals (the significand
// shifted right) and below -149 zeros
__device__ float rnd(uint64_t h, int emin, int emax) {
  const uint32_t m = h & 0x7fffffu;
  const int e = emin + (int)((h >> 23) % (uint64_t)(emax - emin + 1));
  const uint32_t sign = (uint32_t)((h >> 40) & 1) << 31;
  if (e >= -126) return __uint_as_float(sign | (uint32_t)(e + 127) << 23 | m);
  const int sh = -126 - e;
  return __uint_as_float(sign | (sh > 23 ? 0u : ((0x800000u | m) >> sh)));
}

__global__ void recip_all(unsigned e_lo, unsigned e_hi, unsigned long long *bad) {
  const unsigned long long n = (unsigned long long)(e_hi - e_lo + 1) << 24;
  unsigned long long local = 0;
  for (unsigned long long k = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; k < n;
       k += (unsigned long long)gridDim.x * blockDim.x) {
    const unsigned m = (unsigned)(k & 0x7fffff), s = (unsigned)((k >> 23) & 1);
    const unsigned e = e_lo + (unsigned)(k >> 24);
    const float b = __uint_as_float(s << 31 | e << 23 | m);
    const float y = fvgb::refined_recip(b);
    local += (__float_as_uint(y) != __float_as_uint(1.0f / b)) ? 1 : 0;
  }
  if (local) atomicAdd(bad, local);
}

__device__ void operands(int mode, uint64_t h1, uint64_t h2, float &a, float &b) {
  switch (mode) {
    case 0: a = rnd(h1, -40, 40); b = rnd(h2, -40, 24); break;                  // general
    case 1: a = rnd(h1, -104, -96); b = rnd(h2, -3, 3); break;                  // dividends near 2^-100
    case 2: a = rnd(h1, -130, -110); b = rnd(h2, -15, 15); break;               // tiny dividends
    case 3: a = rnd(h1, 35, 44); b = rnd(h2, -90, -80); break;                  // dividends near 2^39, large quotients
    case 4: a = rnd(h1, -60, 39); b = rnd(h2, -90, -80); break;                 // divisors near 2^-85
    case 5: a = rnd(h1, -60, 60); b = rnd(h2, 20, 28); break;                   // divisors near 2^24
    case 6: a = __uint_as_float((uint32_t)(h1 & 0x807fffffu)); b = rnd(h2, -20, 20); break;  // subnormal a
    case 7: a = (h1 & 1) ? 0.0f : -0.0f; b = rnd(h2, -140, 127); break;         // zero dividends
    case 8: {                                                                  // all-ones-ish significands
      a = rnd(h1, -90, 90);
      const uint32_t mb = (uint32_t)(h2 & 0xffu) | 0x7fff00u;
      b = __uint_as_float((uint32_t)(h2 >> 63) << 31 | (uint32_t)(127 + (int)((h2 >> 30) % 40) - 20) << 23 | mb);
      break;
    }
    case 9: a = rnd(h1, -30, -1); b = 1.0f + rnd(h2, -24, -4); break;           // solver-like: v / rho
    case 10: { b = rnd(h2, -10, 10); a = b * rnd(h1, -10, 10); break; }        // exact-ish quotients
    case 11: {                                                                 // powers of two, any dividend
      a = __uint_as_float((uint32_t)h1);
      b = __uint_as_float((uint32_t)(h2 >> 63) << 31 | (uint32_t)(127 + (int)((h2 >> 8) % 130) - 100) << 23);
      break;
    }
    case 12: { a = __uint_as_float((uint32_t)h1 & 0x807fffffu); b = ((h2 & 1) ? -1.0f : 1.0f) * ((h2 & 2) ? 2.0f : 1.0f); break; }  // tails: subnormal / +-1, +-2
    case 14: a = rnd(h1, -149, -40); b = rnd(h2, -152, -125); break;           // zero, subnormal and 2^-126 divisors
    default: a = __uint_as_float((uint32_t)h1); b = __uint_as_float((uint32_t)h2); break;  // any bits
  }
}

__global__ void div_sample(int mode, uint64_t seed, long long n, unsigned long long *flagged,
                           unsigned long long *bad, float *example) {
  unsigned long long fl = 0, bd = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    float a, b;
    operands(mode, mix(seed + 2 * (uint64_t)k), mix(seed + 2 * (uint64_t)k + 1), a, b);
    fvgb::DivFma d;
    const float q = d.div(a, b);
    if (d.unsafe()) {
      ++fl;
      continue;
    }
    const float ref = a / b;
    if (__float_as_uint(q) != __float_as_uint(ref) && !(q != q && ref != ref)) {
      ++bd;
      example[0] = a;
      example[1] = b;
      example[2] = q;
    }
  }
  if (fl) atomicAdd(flagged, fl);
  if (bd) atomicAdd(bad, bd);
}

__global__ void exact_sample(int mode, uint64_t seed, long long n, unsigned long long *flagged,
                             unsigned long long *bad, float *example) {
  unsigned long long fl = 0, bd = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    float a, b;
    operands(mode, mix(seed + 2 * (uint64_t)k), mix(seed + 2 * (uint64_t)k + 1), a, b);
    fvgb::DivExact d;
    const float q = d.div(a, b);
    if (d.unsafe()) {
      ++fl;
      continue;
    }
    const float ref = a / b;
    if (__float_as_uint(q) != __float_as_uint(ref) && !(q != q && ref != ref)) {
      ++bd;
      example[0] = a;
      example[1] = b;
      example[2] = q;
    }
  }
  if (fl) atomicAdd(flagged, fl);
  if (bd) atomicAdd(bad, bd);
}

// DivNormal (the exact-division step kernel's policy for quotients that are
// normal in practice): every quotient it does not flag equals IEEE division
__global__ void normal_sample(int mode, uint64_t seed, long long n, unsigned long long *flagged,
                              unsigned long long *bad, float *example) {
  unsigned long long fl = 0, bd = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    float a, b;
    operands(mode, mix(seed + 2 * (uint64_t)k), mix(seed + 2 * (uint64_t)k + 1), a, b);
    fvgb::DivNormal d;
    const float q = d.div(a, b);
    if (d.unsafe()) {
      ++fl;
      continue;
    }
    const float ref = a / b;
    if (__float_as_uint(q) != __float_as_uint(ref) && !(q != q && ref != ref)) {
      ++bd;
      example[0] = a;
      example[1] = b;
      example[2] = q;
    }
  }
  if (fl) atomicAdd(flagged, fl);
  if (bd) atomicAdd(bad, bd);
}

// the limiter's operands: a = sum of products of wave components, b = sum
// of their squares (> 0); exponents anywhere from subnormal to large
__global__ void ratio_sample(int mode, uint64_t seed, long long n, unsigned long long *flagged,
                             unsigned long long *bad, float *example) {
  unsigned long long fl = 0, bd = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
       k += (long long)gridDim.x * blockDim.x) {
    const uint64_t h1 = mix(seed + 2 * (uint64_t)k), h2 = mix(seed + 2 * (uint64_t)k + 1);
    float a, b;
    if (mode == 0) {
      a = rnd(h1, -149, 10);
      b = fabsf(rnd(h2, -149, 10));
    } else if (mode == 1) {
      a = rnd(h1, -70, -50);
      b = fabsf(rnd(h2, -70, -50));
    } else {
      const float w = rnd(h2, -80, 0), v = rnd(h1, -80, 0);
      a = w * v;
      b = w * w;
    }
    if (b == 0.0f) b = 1.0f;  // the limiter divides by 1 for a zero wave
    const float ref = a / b;
    fvgb::DivExact x;
    const float qx = x.ratio(a, b);
    if (!x.unsafe() && __float_as_uint(qx) != __float_as_uint(ref) && !(qx != qx && ref != ref)) {
      ++bd;
      example[0] = a;
      example[1] = b;
      example[2] = qx;
    }
    // DivNormal's ratio leaves a zero quotient's sign out (the limiter
    // gives +0 for either): equal to IEEE as a value, bit for bit otherwise
    fvgb::DivNormal nr;
    const float qn = nr.ratio(a, b);
    if (!nr.unsafe() && !(qn == ref) && !(qn != qn && ref != ref)) {
      ++bd;
      example[0] = a;
      example[1] = b;
      example[2] = qn;
    }
    fvgb::DivFma d;
    const float q = d.ratio(a, b);
    if (d.unsafe()) {
      ++fl;
      continue;
    }
    const float big = 5.764607523034235e17f;  // 2^59
    const bool same = __float_as_uint(q) == __float_as_uint(ref);
    const bool saturated = fabsf(q) > big && fabsf(ref) > big && ((q > 0.0f) == (ref > 0.0f));
    if (!same && !saturated) {
      ++bd;
      example[0] = a;
      example[1] = b;
      example[2] = q;
    }
  }
  if (fl) atomicAdd(flagged, fl);
  if (bd) atomicAdd(bad, bd);
}

}  // namespace

int main(int argc, char **argv) {
  const long long per_mode = argc > 1 ? atoll(argv[1]) : 400000000LL;
  unsigned long long *cnt;
  float *ex;
  if (cudaMalloc(&cnt, 2 * sizeof(unsigned long long)) != cudaSuccess || cudaMalloc(&ex, 4 * sizeof(float)) != cudaSuccess) {
    std::printf("cuda allocation failed\n");
    return 2;
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  const int grid = (sms > 0 ? sms : 152) * 8;
  int rc = 0;
  // 1. every divisor of magnitude 2^-126 .. 2^24
  cudaMemset(cnt, 0, 2 * sizeof(unsigned long long));
  recip_all<<<grid, 256>>>(127 - 126, 127 + 24, cnt);
  unsigned long long h[2] = {0, 0};
  cudaMemcpy(h, cnt, sizeof(h), cudaMemcpyDeviceToHost);
  std::printf("recip_all %llu 0 %llu\n", (unsigned long long)(151ull << 24), h[0]);
  if (h[0]) rc = 1;
  // 2. sampled quotients
  constexpr int kModes = 15;
  const char *names[kModes] = {"general", "dividend_2^-100", "tiny_dividend", "dividend_2^39",
                               "divisor_2^-85", "divisor_2^24", "subnormal_dividend", "zero_dividend",
                               "ones_significand", "solver_like", "exact_quotients", "pow2_divisor",
                               "tail_divisors", "everything", "divisor_below_2^-124"};
  for (int mode = 0; mode < kModes; ++mode) {
    cudaMemset(cnt, 0, 2 * sizeof(unsigned long long));
    div_sample<<<grid, 256>>>(mode, 0x5eed0000ull + 7919ull * mode, per_mode, cnt, cnt + 1, ex);
    float e[4] = {0, 0, 0, 0};
    cudaMemcpy(h, cnt, sizeof(h), cudaMemcpyDeviceToHost);
    cudaMemcpy(e, ex, 3 * sizeof(float), cudaMemcpyDeviceToHost);
    std::printf("%s %lld %llu %llu", names[mode], per_mode, h[0], h[1]);
    if (h[1]) std::printf("  a=%a b=%a got=%a", e[0], e[1], e[2]);
    std::printf("\n");
    if (h[1]) rc = 1;
  }
  // 3. the fix-up pass's exact division
  for (int mode = 0; mode < kModes; ++mode) {
    cudaMemset(cnt, 0, 2 * sizeof(unsigned long long));
    exact_sample<<<grid, 256>>>(mode, 0x4b1d0000ull + 7919ull * mode, per_mode / 4, cnt, cnt + 1, ex);
    float e[4] = {0, 0, 0, 0};
    cudaMemcpy(h, cnt, sizeof(h), cudaMemcpyDeviceToHost);
    cudaMemcpy(e, ex, 3 * sizeof(float), cudaMemcpyDeviceToHost);
    std::printf("xdiv_%s %lld %llu %llu", names[mode], per_mode / 4, h[0], h[1]);
    if (h[1]) std::printf("  a=%a b=%a got=%a", e[0], e[1], e[2]);
    std::printf("\n");
    if (h[1]) rc = 1;
  }
  // 3b. the exact-division step kernel's normal-quotient division
  for (int mode = 0; mode < kModes; ++mode) {
    cudaMemset(cnt, 0, 2 * sizeof(unsigned long long));
    normal_sample<<<grid, 256>>>(mode, 0x90a10000ull + 7919ull * mode, per_mode / 4, cnt, cnt + 1, ex);
    float e[4] = {0, 0, 0, 0};
    cudaMemcpy(h, cnt, sizeof(h), cudaMemcpyDeviceToHost);
    cudaMemcpy(e, ex, 3 * sizeof(float), cudaMemcpyDeviceToHost);
    std::printf("ndiv_%s %lld %llu %llu", names[mode], per_mode / 4, h[0], h[1]);
    if (h[1]) std::printf("  a=%a b=%a got=%a", e[0], e[1], e[2]);
    std::printf("\n");
    if (h[1]) rc = 1;
  }
  // 4. the limiter's ratio
  const char *rnames[3] = {"ratio_wide", "ratio_mid", "ratio_waves"};
  for (int mode = 0; mode < 3; ++mode) {
    cudaMemset(cnt, 0, 2 * sizeof(unsigned long long));
    ratio_sample<<<grid, 256>>>(mode, 0x7a7e0000ull + 104729ull * mode, per_mode, cnt, cnt + 1, ex);
    float e[4] = {0, 0, 0, 0};
    cudaMemcpy(h, cnt, sizeof(h), cudaMemcpyDeviceToHost);
    cudaMemcpy(e, ex, 3 * sizeof(float), cudaMemcpyDeviceToHost);
    std::printf("%s %lld %llu %llu", rnames[mode], per_mode, h[0], h[1]);
    if (h[1]) std::printf("  a=%a b=%a got=%a", e[0], e[1], e[2]);
    std::printf("\n");
    if (h[1]) rc = 1;
  }
  const cudaError_t err = cudaDeviceSynchronize();
  if (err != cudaSuccess) {
    std::printf("cuda error: %s\n", cudaGetErrorString(err));
    return 2;
  }
  return rc;
}
