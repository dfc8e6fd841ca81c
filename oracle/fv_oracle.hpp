// fv_oracle.hpp -- CPU restatement of FiVoNAGI's time-step hot path.
//
// TEST INFRASTRUCTURE ONLY. This is the oracle that the CUDA path is checked
// against: tests/, __graft_entry__.smoke() and bench.py's CPU baseline use
// it, nothing in the fivonagi_gb300 package does.
//
// It restates, operation by operation and in the reference's evaluation
// order, the per-step arithmetic of
//   apps/na/fv.h        (Riemann solve, first-order update, MC limiter,
//                        second-order correction, per-cell CFL),
//   apps/na/source.h    (fractional velocity diffusion),
//   common/filter.h     (identity: the kernel returns at :14),
//   common/main.cu      (step order :310-635, CFL reduction :179-212 with
//                        its even-offset stopping point :503-519, dt and T
//                        updates :214-238),
//   apps/*/boundary.h, apps/*/init.h (plugins),
// structured as whole-grid phases over scratch arrays, as the reference's
// kernels are. Built with -ffp-contract=off so that every a*b+c rounds
// twice, as the reference's kernels do under nvcc --fmad=false.
//
// Parity pin: tests/test_oracle_golden.py checks this restatement bit for
// bit against fixtures produced by a host build of the reference's own
// headers (oracle/ref_shim.cpp, recipe oracle/Makefile).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../include/fivonagi.h"
#include "../fivonagi_gb300/csrc/fv_math.h"
#include "fv_dual.hpp"

namespace fvo {

// The apps' transcendental functions. libm mode calls the host libm, as the
// reference's hooks do when built for the host (oracle/ref_shim.cpp), and
// is the mode pinned to the reference. fvm mode evaluates them with
// fv_math.h, the portable functions the library uses on both host and
// device, so that the restatement and the CUDA path can be compared bit for
// bit; the two modes differ only in those function values.
template <class R> struct Fn;
template <> struct Fn<float> {
  static float sin(float x, bool m) { return m ? fvm::sinf_(x) : std::sin(x); }
  static float cos(float x, bool m) { return m ? fvm::cosf_(x) : std::cos(x); }
  static float exp(float x, bool m) { return m ? fvm::expf_(x) : std::exp(x); }
  static float tanh(float x, bool m) { return m ? fvm::tanhf_(x) : std::tanh(x); }
};
template <> struct Fn<double> {
  static double sin(double x, bool m) { return m ? fvm::sin_d(x) : std::sin(x); }
  static double cos(double x, bool m) { return m ? fvm::cos_d(x) : std::cos(x); }
  static double exp(double x, bool m) { return m ? fvm::exp_d(x) : std::exp(x); }
  static double tanh(double x, bool m) { return m ? fvm::tanh_d(x) : std::tanh(x); }
};

// The tangent-linear model's dual numbers: values as the plain type's,
// derivatives by the chain rule (fv_dual.hpp).
template <class V, int K> struct Fn<Dual<V, K>> {
  using D = Dual<V, K>;
  static D sin(const D &x, bool m) { return dchain(Fn<V>::sin(x.v, m), std::cos(double(x.v)), x); }
  static D cos(const D &x, bool m) { return dchain(Fn<V>::cos(x.v, m), -std::sin(double(x.v)), x); }
  static D exp(const D &x, bool m) {
    const V e = Fn<V>::exp(x.v, m);
    return dchain(e, std::exp(double(x.v)), x);
  }
  static D tanh(const D &x, bool m) {
    const double t = std::tanh(double(x.v));
    return dchain(Fn<V>::tanh(x.v, m), 1.0 - t * t, x);
  }
};

// sqrt and fabs of the working type (the plain types' own, or the duals')
template <class R> static inline R osqrt(R x) { return std::sqrt(x); }
template <class R> static inline R ofabs(R x) { return std::fabs(x); }
template <class V, int K> static inline Dual<V, K> osqrt(Dual<V, K> x) { return dsqrt(x); }
template <class V, int K> static inline Dual<V, K> ofabs(Dual<V, K> x) { return dfabs(x); }

// getmax / getmin exactly as common/main.cu:63-69: the second argument wins
// ties and NaN comparisons.
template <class R> static inline R getmax(R x, R y) { return (x > y) ? x : y; }
template <class R> static inline R getmin(R x, R y) { return (x < y) ? x : y; }

template <class R> struct Consts;
template <> struct Consts<float> {
  static float pi() { return 3.1415926f; }  // common/numbers.h:13-14 (PRECISION 1)
};
template <> struct Consts<double> {
  static double pi() { return 3.141592653589793; }  // common/numbers.h:15-16
};
template <class V, int K> struct Consts<Dual<V, K>> {
  static Dual<V, K> pi() { return Dual<V, K>::of(Consts<V>::pi()); }
};

// The Riemann solution at one interface, in the sweep's local frame:
// component 1 = rho-1, component 2 = normal momentum, component 3 =
// transverse momentum. W13 = W23 = 0 always (apps/na/fv.h:137-138).
template <class R> struct Wave {
  R s1, s2, s3;
  R w11, w21, w31, w12, w22, w32, w33;
  R amdq1, amdq2, amdq3, apdq1, apdq2, apdq3;
};

// One interface between cell b (index k-1) and cell a (index k).
// rho = u1 + 1 (the `+ Num1` on every read, apps/na/fv.h:62-63).
// Follows apps/na/fv.h:91-180 (x) and :279-368 (y), which are the same
// formula with the normal and transverse roles exchanged.
// Returns false on tmp3 < 0 (simError 2, fv.h:102, 290).
template <class R>
static inline bool riemann(R rho_a, R un_a, R ut_a, R rho_b, R un_b, R ut_b,
                           R beta, R dtx, R &cfl, Wave<R> &w) {
  const R n0 = R(0), n1 = R(1), n2 = R(2);
  R Z1 = (rho_a + rho_b) / n2;
  R Zn = (un_a / rho_a + un_b / rho_b) / n2;
  R Zt = (ut_a / rho_a + ut_b / rho_b) / n2;
  R tmp1 = Zn / Z1;
  R tmp2 = (Zn * Zn) / Z1;
  R tmp3 = tmp1 * tmp1 - n2 * tmp2 + n1 + n2 * (beta - n1) * (Z1 - n1);
  if (tmp3 < n0) return false;
  R L1 = tmp1 + osqrt(tmp3);
  R L2 = tmp1 - osqrt(tmp3);
  R L3 = tmp1;
  R A1 = (L1 * Zt - n2 * Zn * Zt) / (L1 * Z1 - Zt);
  R A2 = (L2 * Zt - n2 * Zn * Zt) / (L2 * Z1 - Zt);
  R a1 = (un_a - un_b - (rho_a - rho_b) * L2) / (L1 - L2);
  R a2 = rho_a - rho_b - a1;
  R a3 = (((L1 * A2 - L2 * A1) * (rho_a - rho_b)) + ((A1 - A2) * (un_a - un_b))) /
             (L2 - L1) +
         ut_a - ut_b;
  w.s1 = L1; w.s2 = L2; w.s3 = L3;
  w.w11 = a1; w.w21 = a1 * L1; w.w31 = a1 * A1;
  w.w12 = a2; w.w22 = a2 * L2; w.w32 = a2 * A2;
  w.w33 = a3;
  w.amdq1 = n0; w.amdq2 = n0; w.amdq3 = n0;
  w.apdq1 = n0; w.apdq2 = n0; w.apdq3 = n0;
  if (L1 < n0) {
    w.amdq1 += L1 * a1; w.amdq2 += L1 * (a1 * L1); w.amdq3 += L1 * (a1 * A1);
    cfl = getmax(cfl, -L1 * dtx);
  } else if (L1 > n0) {
    w.apdq1 += L1 * a1; w.apdq2 += L1 * (a1 * L1); w.apdq3 += L1 * (a1 * A1);
    cfl = getmax(cfl, L1 * dtx);
  }
  if (L2 < n0) {
    w.amdq1 += L2 * a2; w.amdq2 += L2 * (a2 * L2); w.amdq3 += L2 * (a2 * A2);
    cfl = getmax(cfl, -L2 * dtx);
  } else if (L2 > n0) {
    w.apdq1 += L2 * a2; w.apdq2 += L2 * (a2 * L2); w.apdq3 += L2 * (a2 * A2);
    cfl = getmax(cfl, L2 * dtx);
  }
  if (L3 < n0) {
    w.amdq3 += L3 * a3;
    cfl = getmax(cfl, -L3 * dtx);
  } else if (L3 > n0) {
    w.apdq3 += L3 * a3;
    cfl = getmax(cfl, L3 * dtx);
  }
  return true;
}

// MC limiter for one wave, philim.f-style, apps/na/fv.h:587-605.
template <class R>
static inline R mc_limit(R wnorm2, R dotl, R dotr, R s) {
  const R n0 = R(0), n1 = R(1), n2 = R(2);
  R wl;
  if (wnorm2 != n0) {
    R r = (s > n0) ? dotl / wnorm2 : dotr / wnorm2;
    R r2 = n2 * r;
    R c = (n1 + r) / n2;
    wl = getmin(c, n2);
    wl = getmin(wl, r2);
    wl = getmax(wl, n0);
  } else {
    wl = n1;
  }
  return wl;
}

// Second-order correction flux at interface k from the waves at k-1, k,
// k+1: calcLimiters_x/_y (apps/na/fv.h:579-711, 800-921), the result that
// the reference stores into the amdq arrays.
template <class R>
static inline void correction(const Wave<R> &wm, const Wave<R> &w0,
                              const Wave<R> &wp, R dtx, R f[3]) {
  const R n0 = R(0), n1 = R(1);
  const R z = n0;  // W13 = W23 = 0
  R wnorm2, dotr, dotl;
  wnorm2 = w0.w11 * w0.w11 + w0.w21 * w0.w21 + w0.w31 * w0.w31;
  dotr = w0.w11 * wp.w11 + w0.w21 * wp.w21 + w0.w31 * wp.w31;
  dotl = w0.w11 * wm.w11 + w0.w21 * wm.w21 + w0.w31 * wm.w31;
  R l1 = mc_limit(wnorm2, dotl, dotr, w0.s1);
  wnorm2 = w0.w12 * w0.w12 + w0.w22 * w0.w22 + w0.w32 * w0.w32;
  dotr = w0.w12 * wp.w12 + w0.w22 * wp.w22 + w0.w32 * wp.w32;
  dotl = w0.w12 * wm.w12 + w0.w22 * wm.w22 + w0.w32 * wm.w32;
  R l2 = mc_limit(wnorm2, dotl, dotr, w0.s2);
  wnorm2 = z * z + z * z + w0.w33 * w0.w33;
  dotr = z * z + z * z + w0.w33 * wp.w33;
  dotl = z * z + z * z + w0.w33 * wm.w33;
  R l3 = mc_limit(wnorm2, dotl, dotr, w0.s3);
  R a1 = ofabs(w0.s1), a2 = ofabs(w0.s2), a3 = ofabs(w0.s3);
  R c1 = a1 * (n1 - a1 * dtx) * w0.w11 * l1 + a2 * (n1 - a2 * dtx) * w0.w12 * l2 +
         a3 * (n1 - a3 * dtx) * z * l3;
  R c2 = a1 * (n1 - a1 * dtx) * w0.w21 * l1 + a2 * (n1 - a2 * dtx) * w0.w22 * l2 +
         a3 * (n1 - a3 * dtx) * z * l3;
  R c3 = a1 * (n1 - a1 * dtx) * w0.w31 * l1 + a2 * (n1 - a2 * dtx) * w0.w32 * l2 +
         a3 * (n1 - a3 * dtx) * w0.w33 * l3;
  const R half = R(0.5);
  f[0] = half * c1;
  f[1] = half * c2;
  f[2] = half * c3;
}

// Per-app parameters in working precision, derived from fv_params the way
// each app's parameters.h derives them.
template <class R> struct AppConsts {
  int app;
  R ampl, frec, ispw, ispa, ispf;          // hifu
  R isprhoa, ispc, isptheta, mdt;          // taylor
  R angle;                                 // plane wave
  R aperture, center, ramp;                // focused beam
  int nelem = 0, arr_j0 = 0, arr_elem = 1;  // phased array
  std::vector<R> amp, phase;
};

template <class R> class Sim {
 public:
  fv_params p{};
  bool fvm_mode = false;  // see Fn<R>
  int nx = 0, ny = 0;
  R dx{}, dy{}, beta{}, diffdelta{}, cflmax{}, cflwhish{};
  AppConsts<R> ac{};
  // time-stepping scalars, device-side in the reference
  R dt{}, T{};
  int32_t n = 0, mdx = 0, mdy = 0;
  int status = 0;
  R last_cfl{};
  R last_dt{};  // dt of the last attempt
  int64_t accepted = 0, rejected = 0;
  int rejected_last = 0;  // the reference's device simError == 1 after a rejection
  // state (the A/B pair holds the same values between steps)
  std::vector<R> u[3];
  // scratch
  std::vector<R> s0[3], s1a[3], s1[3], s2a[3], s2[3], s3[3], cfl;
  std::vector<Wave<R>> wv;  // waves of one sweep, indexed by cell offset
  std::vector<R> fadd[3];

  explicit Sim(const fv_params &pp, bool fvm_math = false);
  size_t size() const { return size_t(nx) * size_t(ny); }
  size_t off(int i, int j) const { return size_t(i) + size_t(j) * size_t(nx); }
  bool interior(int i, int j) const {
    return i >= 2 && i <= nx - 3 && j >= 2 && j <= ny - 3;
  }

  void init_state();
  void reset_scalars() {
    dt = R(p.dtini);
    T = -R(p.tide);
    n = 0; mdx = 0; mdy = 0;
    status = 0; rejected_last = 0;
  }
  // Phases of one attempted step. Each reads `in` and writes `out`.
  void boundary(std::vector<R> const *in, std::vector<R> *out);
  bool sweep(int dir, std::vector<R> const *in, std::vector<R> *mid,
             std::vector<R> *out);
  void source(std::vector<R> const *in, std::vector<R> *out);
  R reduce_cfl() const;
  // One attempted step; returns 0 accepted, 1 rejected, 2 negative eigenvalue.
  int attempt(int stop_stage = -1);
  int run(int64_t nsteps);
};

}  // namespace fvo
