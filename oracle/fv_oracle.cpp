// fv_oracle.cpp -- CPU restatement of FiVoNAGI's time-step hot path, and
// its C API (liboracle.so, loaded by tests/ and bench.py through ctypes).
//
// TEST INFRASTRUCTURE ONLY: the oracle the CUDA path is checked against.
// See fv_oracle.hpp for what is restated from where.
#include "fv_oracle.hpp"

#include <algorithm>
#include <cstdio>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace fvo {

template <class R>
Sim<R>::Sim(const fv_params &pp, bool fvm_math) : p(pp), fvm_mode(fvm_math) {
  nx = p.nx;
  ny = p.ny;
  // dx = XMAX/(NX-1), dy = YMAX/(NY-1) in working precision
  // (common/main.cu:790-791).
  dx = R(p.xmax) / R(nx - 1);
  dy = R(p.ymax) / R(ny - 1);
  beta = R(p.beta);
  diffdelta = R(p.diffdelta);
  cflmax = R(p.cflmax);
  cflwhish = R(p.cflwhish);
  ac.app = p.app;
  ac.ampl = R(p.ampl);
  ac.frec = R(p.frec);
  // ISPW = Num2*PI*FREC (apps/hifu-beam/parameters.h:89)
  ac.ispw = R(2) * Consts<R>::pi() * ac.frec;
  ac.ispa = R(p.isp_a);
  ac.ispf = R(p.isp_f);
  ac.isprhoa = R(p.isp_rhoa);
  ac.ispc = R(p.isp_c);
  ac.isptheta = R(p.angle);
  ac.mdt = R(p.mdt);
  ac.angle = R(p.angle);
  ac.aperture = R(p.aperture * 0.5);  // half aperture, cells
  ac.center = R(p.center);
  ac.ramp = R(p.frec / p.ramp_periods);
  if (p.app == FV_APP_PHASED_ARRAY) {
    // element k drives rows [arr_j0 + k*arr_elem, arr_j0 + (k+1)*arr_elem)
    ac.nelem = p.array_elems;
    ac.arr_elem = int(p.aperture / p.array_elems);
    ac.arr_j0 = int(std::lround(p.center - 0.5 * p.aperture));
    ac.amp.assign(size_t(ac.nelem), R(p.ampl));
    ac.phase.assign(size_t(ac.nelem), R(0));
  }
  for (int f = 0; f < 3; ++f) {
    u[f].assign(size(), R(0));
    s0[f].assign(size(), R(0));
    s1a[f].assign(size(), R(0));
    s1[f].assign(size(), R(0));
    s2a[f].assign(size(), R(0));
    s2[f].assign(size(), R(0));
    s3[f].assign(size(), R(0));
    fadd[f].assign(size(), R(0));
  }
  cfl.assign(size(), R(0));
  wv.assign(size(), Wave<R>{});
  reset_scalars();
}

// ---------------------------------------------------------------- init hooks

template <class R> void Sim<R>::init_state() {
  const int app = p.app;
  for (int j = 0; j < ny; ++j) {
    for (int i = 0; i < nx; ++i) {
      size_t o = off(i, j);
      R v1 = R(0), v2 = R(0), v3 = R(0);
      if (app == FV_APP_TAYLOR_ANGLE_XY) {
        // apps/taylor-angle-xy/init.h:19-27
        const R th = ac.isptheta;
        const bool m = fvm_mode;
        R rhop = ac.isprhoa *
                 Fn<R>::tanh(ac.ispc * (R(i) * dx * Fn<R>::cos(th, m) +
                                        (R(j - ny / 2) * dy + ac.mdt * Fn<R>::sin(th, m)) *
                                            Fn<R>::sin(th, m) +
                                        R(p.tide)),
                             m);
        v1 = rhop;
        v2 = rhop * Fn<R>::cos(th, m);
        v3 = rhop * Fn<R>::sin(th, m);
      } else if (app == FV_APP_PLANE_WAVE) {
        // u1 = A sin(2 pi FREC (x cos a + y sin a)), u2,u3 = u1 (cos a, sin a):
        // the taylor init form (init.h:25-27) with a sinusoidal profile,
        // evaluated in double and rounded once.
        const double ddx = p.xmax / double(nx - 1), ddy = p.ymax / double(ny - 1);
        const bool m = fvm_mode;
        const double ca = Fn<double>::cos(p.angle, m), sa = Fn<double>::sin(p.angle, m);
        const double ph = 2.0 * 3.141592653589793 * p.frec *
                          (double(i) * ddx * ca + double(j) * ddy * sa);
        const double a = p.ampl * Fn<double>::sin(ph, m);
        v1 = R(a);
        v2 = R(a * ca);
        v3 = R(a * sa);
      }
      // hifu-beam (apps/hifu-beam/init.h:16-25) and the focused beam: zeros
      u[0][o] = v1;
      u[1][o] = v2;
      u[2][o] = v3;
    }
  }
  reset_scalars();
}

// ------------------------------------------------------------ boundary hooks

// packet() of apps/hifu-beam/boundary.h:10-17. opT is evaluated in double
// (the literals 2.0 and 8.0 are double) and rounded to R on assignment.
template <class R>
static inline R hifu_packet(const AppConsts<R> &ac, R T, R phi, bool m) {
  R opT = R(2.0 * double(ac.frec) * double(T + phi) / 8.0);
  R res = ac.ampl * Fn<R>::sin(ac.ispw * (T + phi), m);
  res = res * Fn<R>::exp(-opT * opT * opT * opT * opT * opT * opT * opT * opT * opT, m);
  return res;
}

template <class R>
void Sim<R>::boundary(std::vector<R> const *in, std::vector<R> *out) {
  const int app = p.app;
  const R zero = R(0), one = R(1);
#pragma omp parallel for schedule(static)
  for (int j = 0; j < ny; ++j) {
    for (int i = 0; i < nx; ++i) {
      const size_t o = off(i, j);
      R v1 = in[0][o], v2 = in[1][o], v3 = in[2][o];
      const bool ghost = (i <= 1 || i >= nx - 2 || j <= 1 || j >= ny - 2);
      if (ghost) {
        const bool corner = (i <= 1 || i >= nx - 2) && (j <= 1 || j >= ny - 2);
        auto take = [&](int ii, int jj) {
          size_t s = off(ii, jj);
          v1 = in[0][s]; v2 = in[1][s]; v3 = in[2][s];
        };
        if (app == FV_APP_TAYLOR_ANGLE_XY) {
          // apps/taylor-angle-xy/boundary.h:38-55: every ghost cell, corners
          // included, is the analytic profile.
          const R th = ac.isptheta;
          const bool m = fvm_mode;
          R rhop = ac.isprhoa *
                   Fn<R>::tanh(ac.ispc * (R(i + mdx) * dx * Fn<R>::cos(th, m) +
                                          (R(j + mdy - ny / 2) * dy + ac.mdt * Fn<R>::sin(th, m)) *
                                              Fn<R>::sin(th, m) -
                                          T),
                               m);
          v1 = rhop;
          v2 = rhop * Fn<R>::cos(th, m);
          v3 = rhop * Fn<R>::sin(th, m);
        } else if (corner) {
          // apps/hifu-beam/boundary.h:125-133 (and the same convention for
          // the plane-wave and focused-beam apps)
          v1 = zero; v2 = zero; v3 = zero;
        } else if (i >= nx - 2) {
          take(nx - 3, j);  // zero-order extrapolation (hifu :49-61)
        } else if (j >= ny - 2) {
          if (app == FV_APP_PLANE_WAVE) {
            take(i, 2 * (ny - 3) - j);  // no-flux wall, mirror about ny-3
            v3 = -v3;
          } else {
            take(i, ny - 3);  // hifu :63-75
          }
        } else if (i <= 1) {
          if (app == FV_APP_HIFU_BEAM) {
            // hifu :77-107
            int width = static_cast<int>(double(ac.ispa / dy));
            int jprime = j - 2;
            if (std::abs(jprime) < width && jprime >= 0 && mdx == 0) {
              R jprime2 = static_cast<R>(jprime * jprime);
              R nudenom = osqrt(jprime2 + ac.ispf * ac.ispf);
              R nux = ac.ispf / nudenom;
              R nuy = -static_cast<R>(jprime) / nudenom;
              R phi = (dx * jprime2) / (R(2) * ac.ispf);
              R pack = hifu_packet(ac, T, phi, fvm_mode);
              v1 = pack;
              v2 = nux * pack * (pack + one);
              v3 = nuy * pack * (pack + one);
            } else {
              take(2, j);
            }
          } else if (app == FV_APP_PHASED_ARRAY) {
            // phased array: the focused beam's packet at normal incidence,
            // with each element's own amplitude and phase
            const int jr = j - ac.arr_j0;
            if (jr >= 0 && jr < ac.nelem * ac.arr_elem && mdx == 0) {
              const int e = jr / ac.arr_elem;
              R ramp = getmin(getmax(T * ac.ramp, zero), one);
              R pack = ac.amp[e] * ramp * Fn<R>::sin(ac.ispw * T + ac.phase[e], fvm_mode);
              v1 = pack;
              v2 = pack * (pack + one);
              v3 = zero;
            } else {
              take(2, j);
            }
          } else if (app == FV_APP_FOCUSED_BEAM) {
            R jp = R(j) - ac.center;
            if (ofabs(jp) < ac.aperture && mdx == 0) {
              R jp2 = jp * jp;
              R nudenom = osqrt(jp2 + ac.ispf * ac.ispf);
              R nux = ac.ispf / nudenom;
              R nuy = -jp / nudenom;
              R phi = (dx * jp2) / (R(2) * ac.ispf);
              R t = T + phi;
              R ramp = getmin(getmax(t * ac.ramp, zero), one);
              R pack = ac.ampl * ramp * Fn<R>::sin(ac.ispw * t, fvm_mode);
              v1 = pack;
              v2 = nux * pack * (pack + one);
              v3 = nuy * pack * (pack + one);
            } else {
              take(2, j);
            }
          } else {
            take(2, j);  // plane wave: zero-order extrapolation
          }
        } else {  // j <= 1
          if (app == FV_APP_FOCUSED_BEAM || app == FV_APP_PHASED_ARRAY) {
            take(i, 2);  // open lateral side, common/boundary.h:41-53
          } else {
            take(i, 4 - j);  // reflecting, hifu :110-122
            v3 = -v3;
          }
        }
      }
      out[0][o] = v1;
      out[1][o] = v2;
      out[2][o] = v3;
    }
  }
}

// -------------------------------------------------------------------- sweeps

// One dimensional-splitting sweep: waves at every interface, first-order
// update (step_x/_y, apps/na/fv.h:384-499), MC-limited correction
// (calcLimiters_x/_y :502-930) and its update (writeLimiters_x/_y
// :933-1054). dir 1 = y (runs first, CFL starts at 0), dir 0 = x (CFL
// starts from the y value of the same cell, fv.h:57).
template <class R>
bool Sim<R>::sweep(int dir, std::vector<R> const *in, std::vector<R> *mid,
                   std::vector<R> *out) {
  const R dd = dir ? dy : dx;
  const R dtx = dt / dd;
  const int un = dir ? 2 : 1;  // normal momentum component
  const int ut = dir ? 1 : 2;  // transverse momentum component
  bool ok = true;
#pragma omp parallel for schedule(static) reduction(&& : ok)
  for (int j = 0; j < ny; ++j) {
    for (int i = 0; i < nx; ++i) {
      const size_t o = off(i, j);
      const int k = dir ? j : i;
      if (k == 0) {
        cfl[o] = R(0);
        continue;
      }
      const size_t b = dir ? off(i, j - 1) : off(i - 1, j);
      R c = dir ? R(0) : cfl[o];
      R rho_a = in[0][o] + R(1), rho_b = in[0][b] + R(1);
      if (!riemann(rho_a, in[un][o], in[ut][o], rho_b, in[un][b], in[ut][b], beta,
                   dtx, c, wv[o]))
        ok = false;
      cfl[o] = c;
    }
  }
  if (!ok) return false;
  const size_t stride = dir ? size_t(nx) : 1;
  // first-order update: u - dt/d (apdq(c) + amdq(c+1))
#pragma omp parallel for schedule(static)
  for (int j = 0; j < ny; ++j) {
    for (int i = 0; i < nx; ++i) {
      const size_t o = off(i, j);
      if (interior(i, j)) {
        const Wave<R> &wa = wv[o], &wb = wv[o + stride];
        mid[0][o] = in[0][o] - dtx * (wa.apdq1 + wb.amdq1);
        mid[un][o] = in[un][o] - dtx * (wa.apdq2 + wb.amdq2);
        mid[ut][o] = in[ut][o] - dtx * (wa.apdq3 + wb.amdq3);
      } else {
        mid[0][o] = in[0][o];
        mid[1][o] = in[1][o];
        mid[2][o] = in[2][o];
      }
    }
  }
  // correction fluxes at the interfaces the interior update consumes
#pragma omp parallel for schedule(static)
  for (int j = 1; j < ny - 1; ++j) {
    for (int i = 1; i < nx - 1; ++i) {
      const size_t o = off(i, j);
      const int k = dir ? j : i;
      if (k < 2) continue;  // fadd at k = 1 reads a wave the sweep never wrote
      R f[3];
      correction(wv[o - stride], wv[o], wv[o + stride], dtx, f);
      fadd[0][o] = f[0];
      fadd[1][o] = f[1];
      fadd[2][o] = f[2];
    }
  }
  // correction update: u - dt/d (fadd(c+1) - fadd(c))
#pragma omp parallel for schedule(static)
  for (int j = 0; j < ny; ++j) {
    for (int i = 0; i < nx; ++i) {
      const size_t o = off(i, j);
      if (interior(i, j)) {
        out[0][o] = mid[0][o] - dtx * (fadd[0][o + stride] - fadd[0][o]);
        out[un][o] = mid[un][o] - dtx * (fadd[1][o + stride] - fadd[1][o]);
        out[ut][o] = mid[ut][o] - dtx * (fadd[2][o + stride] - fadd[2][o]);
      } else {
        out[0][o] = mid[0][o];
        out[1][o] = mid[1][o];
        out[2][o] = mid[2][o];
      }
    }
  }
  return true;
}

// Fractional velocity diffusion, apps/na/source.h:9-117. u1 passes through
// as (u1 + 1) - 1, the reference's own rounding (source.h:40, 84).
template <class R>
void Sim<R>::source(std::vector<R> const *in, std::vector<R> *out) {
  const R n1 = R(1), n2 = R(2);
  const R ddtx2 = diffdelta * dt / (dx * dx);
  const R ddty2 = diffdelta * dt / (dy * dy);
#pragma omp parallel for schedule(static)
  for (int j = 0; j < ny; ++j) {
    for (int i = 0; i < nx; ++i) {
      const size_t o = off(i, j);
      if (!interior(i, j)) {
        out[0][o] = in[0][o];
        out[1][o] = in[1][o];
        out[2][o] = in[2][o];
        continue;
      }
      const size_t oim = o - 1, oip = o + 1, ojm = o - nx, ojp = o + nx;
      const R r0 = in[0][o] + n1, rim = in[0][oim] + n1, rjm = in[0][ojm] + n1,
              rip = in[0][oip] + n1, rjp = in[0][ojp] + n1;
      out[0][o] = r0 - n1;
      for (int f = 1; f <= 2; ++f) {
        const std::vector<R> &q = in[f];
        out[f][o] = q[o] +
                    ddtx2 * (q[oim] / rim - n2 * (q[o] / r0) + q[oip] / rip) +
                    ddty2 * (q[ojm] / rjm - n2 * (q[o] / r0) + q[ojp] / rjp);
      }
    }
  }
}

// The reference halves `cfl` pairwise and stops at two elements
// (common/main.cu:503-519), so cfl[0] is the maximum over even flat
// offsets. With max being order-independent on non-NaN values, a scan over
// the same set gives the same value.
template <class R> R Sim<R>::reduce_cfl() const {
  R m = R(0);
  const size_t step = p.cfl_even_only ? 2 : 1;
  for (size_t o = 0; o < size(); o += step) m = getmax(m, cfl[o]);
  return m;
}

template <class R> int Sim<R>::attempt(int stop_stage) {
  last_dt = dt;
  boundary(u, s0);
  if (stop_stage == FV_STAGE_BOUNDARY) return 0;
  if (!sweep(1, s0, s1a, s1)) { status = FV_NEGATIVE_EIGENVALUE; return 2; }
  if (stop_stage == FV_STAGE_SWEEP_Y) return 0;
  if (!sweep(0, s1, s2a, s2)) { status = FV_NEGATIVE_EIGENVALUE; return 2; }
  if (stop_stage == FV_STAGE_SWEEP_X) return 0;
  const R c = reduce_cfl();
  last_cfl = c;
  if (stop_stage == FV_STAGE_SOURCE) {
    source(s2, s3);
    return 0;
  }
  int sim_error = 0;
  if (c < cflmax) {  // reduceCFL2, common/main.cu:200-212
    source(s2, s3);
    T = T + dt;  // update_T, main.cu:232-238
    n = n + 1;
    if (p.moving_domain && T >= ac.mdt) {
      // moveDomain + updateMDXY, common/main.cu:109-177
      const int mdi = static_cast<int>(double((T - ac.mdt) * R(p.mdvx) / dx)) - mdx;
      const int mdj = static_cast<int>(double((T - ac.mdt) * R(p.mdvy) / dy)) - mdy;
      for (int j = 0; j < ny; ++j)
        for (int i = 0; i < nx; ++i) {
          int ir = i + mdi, jr = j + mdj;
          if (!(ir <= nx - 1 && jr <= ny - 1)) { ir = i; jr = j; }
          ir = std::max(ir, 0);
          jr = std::max(jr, 0);
          for (int f = 0; f < 3; ++f) u[f][off(i, j)] = s3[f][off(ir, jr)];
        }
      mdx += mdi;
      mdy += mdj;
    } else {
      for (int f = 0; f < 3; ++f) u[f].swap(s3[f]);
    }
    accepted++;
  } else {
    sim_error = 1;  // rejected: the state is kept and the step retried
    rejected++;
  }
  // update_dt, common/main.cu:214-230; `0.9` is a double literal
  R new_dt = dt * cflwhish / c;
  if (sim_error == 1 && double(new_dt) > double(dt) * 0.9)
    dt = R(double(dt) * 0.9);
  else
    dt = new_dt;
  return sim_error;
}

template <class R> int Sim<R>::run(int64_t nsteps) {
  int64_t done = 0;
  int consecutive = 0;
  const int max_retries = p.max_retries > 0 ? p.max_retries : 64;
  while (done < nsteps) {
    int r = attempt();
    if (r == 2) return FV_NEGATIVE_EIGENVALUE;
    if (r == 1) {
      if (++consecutive >= max_retries) { status = FV_DT_TOO_LARGE; return status; }
      continue;
    }
    consecutive = 0;
    ++done;
  }
  return FV_OK;
}

template class Sim<float>;
template class Sim<double>;

// The tangent-linear model: the same step on dual numbers (fv_dual.hpp),
// with up to kTlmDirs derivative directions.
constexpr int kTlmDirs = 16;
template class Sim<Dual<float, kTlmDirs>>;
template class Sim<Dual<double, kTlmDirs>>;

// The working type of tlm_loss: duals with K directions, or the plain type
// for K = 0 (the loss alone).
template <class V, int K> struct TlmType { using type = Dual<V, K>; };
template <class V> struct TlmType<V, 0> { using type = V; };
template <class V, int K> static inline void seed(Dual<V, K> &x, int r) { x.d[r] = 1.0; }
template <class V> static inline void seed(V &, int) {}
template <class V, int K> static inline double deriv(const Dual<V, K> &x, int r) { return x.d[r]; }
template <class V> static inline double deriv(const V &, int) { return 0.0; }
template <class V, int K> static inline double value(const Dual<V, K> &x) { return double(x.v); }
template <class V> static inline double value(const V &x) { return double(x); }

// Loss and its derivatives along the seeded directions: the phased array's
// weights (amplitudes [0, nelem), phases [nelem, 2 nelem)) are the inputs;
// the dt schedule is held fixed (dts[n], Ts[n]: dt and T of accepted step
// n), as the library's adjoint holds it; loss = mean of u1^2 over the
// window [i0, i0+ni) x [j0, j0+nj) and accepted steps first..last.
template <class V, int K = kTlmDirs>
static int tlm_loss(const fv_params *p, bool fvm, const double *amp, const double *phase, int nelem, int ndir,
                    const int *dir_param, int64_t nsteps, const double *dts, const double *Ts, const int *win,
                    double *loss, double *grad) {
  using D = typename TlmType<V, K>::type;
  if (ndir < 0 || ndir > K || p->app != FV_APP_PHASED_ARRAY || nelem != p->array_elems) return FV_BAD_ARG;
  fv_params q = *p;
  q.cflmax = 1e30;  // the schedule is given: every attempt is accepted
  Sim<D> s(q, fvm);
  for (int k = 0; k < nelem; ++k) {
    s.ac.amp[k] = D(amp[k]);
    s.ac.phase[k] = D(phase[k]);
  }
  for (int r = 0; r < ndir; ++r) {
    const int idx = dir_param[r];
    if (idx < 0 || idx >= 2 * nelem) return FV_BAD_ARG;
    if (idx < nelem) seed(s.ac.amp[idx], r);
    else seed(s.ac.phase[idx - nelem], r);
  }
  s.init_state();
  const int i0 = win[0], j0 = win[1], ni = win[2], nj = win[3], first = win[4], last = win[5];
  double acc = 0.0, accd[kTlmDirs + 1] = {};
  for (int64_t n = 0; n < nsteps; ++n) {
    s.dt = D(dts[n]);
    s.T = D(Ts[n]);
    s.n = int32_t(n);
    const int r = s.attempt();
    if (r != 0) return r == 2 ? FV_NEGATIVE_EIGENVALUE : FV_DT_TOO_LARGE;
    if (n + 1 >= first && n + 1 <= last) {
      for (int j = j0; j < j0 + nj; ++j)
        for (int i = i0; i < i0 + ni; ++i) {
          const D &u1 = s.u[0][s.off(i, j)];
          const double v = value(u1);
          acc += v * v;
          for (int k = 0; k < ndir; ++k) accd[k] += 2.0 * v * deriv(u1, k);
        }
    }
  }
  const double cnt = double(last - first + 1) * double(ni) * double(nj);
  *loss = acc / cnt;
  for (int k = 0; k < ndir; ++k) grad[k] = accd[k] / cnt;
  return FV_OK;
}

}  // namespace fvo

// --------------------------------------------------------------------- C API

namespace {
struct Handle {
  int prec;
  fvo::Sim<float> *f = nullptr;
  fvo::Sim<double> *d = nullptr;
};

template <class R>
void copy_out(const fvo::Sim<R> &s, const std::vector<R> *src, void *a, void *b, void *c) {
  void *dst[3] = {a, b, c};
  for (int f = 0; f < 3; ++f)
    if (dst[f]) std::memcpy(dst[f], src[f].data(), s.size() * sizeof(R));
}

template <class R> void stats_of(const fvo::Sim<R> &s, fv_run_stats *st) {
  if (!st) return;
  st->accepted = s.accepted;
  st->rejected = s.rejected;
  st->dt = double(s.dt);
  st->T = double(s.T);
  st->cfl = double(s.last_cfl);
  st->n = s.n;
  st->status = s.status;
  st->mdx = s.mdx;
  st->mdy = s.mdy;
}
}  // namespace

#define FVO_DISPATCH(h, BODY)                                              \
  do {                                                                     \
    if (!(h)) return FV_BAD_ARG;                                           \
    if ((h)->prec == 4) { auto &s = *(h)->f; BODY; }                       \
    else { auto &s = *(h)->d; BODY; }                                      \
  } while (0)

extern "C" {

// flags bit 0: evaluate the apps' transcendental functions with fv_math.h
// (see Fn<R>) instead of the host libm.
void *fvo_create(const fv_params *p, int prec, int flags) {
  if (!p || (prec != 4 && prec != 8) || p->nx < 8 || p->ny < 8) return nullptr;
  Handle *h = new Handle();
  h->prec = prec;
  const bool m = (flags & 1) != 0;
  if (prec == 4) h->f = new fvo::Sim<float>(*p, m);
  else h->d = new fvo::Sim<double>(*p, m);
  return h;
}

void fvo_destroy(void *hv) {
  Handle *h = static_cast<Handle *>(hv);
  if (!h) return;
  delete h->f;
  delete h->d;
  delete h;
}

int fvo_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

int fvo_init_state(void *hv) {
  Handle *h = static_cast<Handle *>(hv);
  FVO_DISPATCH(h, { s.init_state(); s.accepted = 0; s.rejected = 0; });
  return FV_OK;
}

int fvo_set_state(void *hv, const void *u1, const void *u2, const void *u3) {
  Handle *h = static_cast<Handle *>(hv);
  const void *src[3] = {u1, u2, u3};
  FVO_DISPATCH(h, {
    for (int f = 0; f < 3; ++f)
      std::memcpy(s.u[f].data(), src[f], s.size() * sizeof(s.u[f][0]));
    s.reset_scalars();
    s.accepted = 0;
    s.rejected = 0;
  });
  return FV_OK;
}

int fvo_get_state(void *hv, void *u1, void *u2, void *u3) {
  Handle *h = static_cast<Handle *>(hv);
  FVO_DISPATCH(h, { copy_out(s, s.u, u1, u2, u3); });
  return FV_OK;
}

int fvo_set_scalars(void *hv, double dt, double T, int n) {
  Handle *h = static_cast<Handle *>(hv);
  FVO_DISPATCH(h, {
    s.dt = decltype(s.dt)(dt);
    s.T = decltype(s.T)(T);
    s.n = n;
  });
  return FV_OK;
}

// Phased-array element weights (amplitudes, phases), given in double.
int fvo_set_weights(void *hv, const double *amp, const double *phase, int nelem) {
  Handle *h = static_cast<Handle *>(hv);
  int rc = 0;
  FVO_DISPATCH(h, {
    if (nelem != s.ac.nelem) {
      rc = 1;
    } else {
      for (int k = 0; k < nelem; ++k) {
        s.ac.amp[k] = decltype(s.dt)(amp[k]);
        s.ac.phase[k] = decltype(s.dt)(phase[k]);
      }
    }
  });
  return rc;
}

int fvo_get_stats(void *hv, fv_run_stats *st) {
  Handle *h = static_cast<Handle *>(hv);
  FVO_DISPATCH(h, { stats_of(s, st); });
  return FV_OK;
}

int fvo_run(void *hv, int64_t nsteps, fv_run_stats *st) {
  Handle *h = static_cast<Handle *>(hv);
  int rc = 0;
  FVO_DISPATCH(h, {
    s.accepted = 0;
    s.rejected = 0;
    rc = s.run(nsteps);
    stats_of(s, st);
  });
  return rc;
}

// One attempted step stopped after `stage`; the stage's grid is copied out
// and the state and scalars are left as they were.
int fvo_debug_step(void *hv, int stage, void *u1, void *u2, void *u3) {
  Handle *h = static_cast<Handle *>(hv);
  int rc = 0;
  FVO_DISPATCH(h, {
    auto saved_dt = s.dt; auto saved_T = s.T; auto saved_n = s.n;
    auto acc = s.accepted; auto rej = s.rejected;
    auto st = s.status; auto mx = s.mdx; auto my = s.mdy;
    rc = s.attempt(stage);
    const std::vector<decltype(s.dt)> *src =
        stage == FV_STAGE_BOUNDARY ? s.s0 : stage == FV_STAGE_SWEEP_Y ? s.s1
        : stage == FV_STAGE_SWEEP_X ? s.s2 : s.s3;
    copy_out(s, src, u1, u2, u3);
    s.dt = saved_dt; s.T = saved_T; s.n = saved_n;
    s.accepted = acc; s.rejected = rej; s.status = st; s.mdx = mx; s.mdy = my;
  });
  return rc == 2 ? FV_NEGATIVE_EIGENVALUE : FV_OK;
}

// fv_math.h (fn 0 sin, 1 cos, 2 exp, 3 tanh) evaluated on the host over n
// floats, for checking those functions against the host libm.
void fvo_fvm_eval(int fn, const float *x, float *y, int64_t n) {
  for (int64_t k = 0; k < n; ++k) {
    switch (fn) {
      case 0: y[k] = fvm::sinf_(x[k]); break;
      case 1: y[k] = fvm::cosf_(x[k]); break;
      case 2: y[k] = fvm::expf_(x[k]); break;
      default: y[k] = fvm::tanhf_(x[k]); break;
    }
  }
}

// The loss alone on a fixed schedule (tlm_loss's loss without derivatives),
// in FP32 (prec 4) or FP64 (prec 8): the central differences' evaluations.
int fvo_schedule_loss(const fv_params *p, int prec, int flags, const double *amp, const double *phase, int nelem,
                      int64_t nsteps, const double *dts, const double *Ts, const int *win, double *loss) {
  if (!p || !amp || !phase || !dts || !Ts || !win || !loss) return FV_BAD_ARG;
  const bool m = (flags & 1) != 0;
  const int dummy = 0;
  double g = 0.0;
  if (prec == 4)
    return fvo::tlm_loss<float, 0>(p, m, amp, phase, nelem, 0, &dummy, nsteps, dts, Ts, win, loss, &g);
  if (prec == 8)
    return fvo::tlm_loss<double, 0>(p, m, amp, phase, nelem, 0, &dummy, nsteps, dts, Ts, win, loss, &g);
  return FV_BAD_ARG;
}

// The tangent-linear gradient (tlm_loss above) in FP32 values (prec 4:
// along the FP32 oracle's trajectory, which the CUDA path reproduces bit for
// bit) or FP64 values (prec 8); derivatives are double either way. win:
// i0, j0, ni, nj, first, last.
int fvo_tlm_loss(const fv_params *p, int prec, int flags, const double *amp, const double *phase, int nelem,
                 int ndir, const int *dir_param, int64_t nsteps, const double *dts, const double *Ts,
                 const int *win, double *loss, double *grad) {
  if (!p || !amp || !phase || !dir_param || !dts || !Ts || !win || !loss || !grad) return FV_BAD_ARG;
  const bool m = (flags & 1) != 0;
  if (prec == 4)
    return fvo::tlm_loss<float>(p, m, amp, phase, nelem, ndir, dir_param, nsteps, dts, Ts, win, loss, grad);
  if (prec == 8)
    return fvo::tlm_loss<double>(p, m, amp, phase, nelem, ndir, dir_param, nsteps, dts, Ts, win, loss, grad);
  return FV_BAD_ARG;
}

// dt of the attempt that fvo_run accepted last (the schedule of a run).
double fvo_last_dt(void *hv) {
  Handle *h = static_cast<Handle *>(hv);
  if (!h) return -1.0;
  return h->prec == 4 ? double(h->f->last_dt) : h->d->last_dt;
}

// The CFL of the step that fvo_debug_step or fvo_run attempted last.
double fvo_last_cfl(void *hv) {
  Handle *h = static_cast<Handle *>(hv);
  if (!h) return -1.0;
  return h->prec == 4 ? double(h->f->last_cfl) : h->d->last_cfl;
}

}  // extern "C"
