// ref_shim.cpp -- host build of the reference's own hot-path headers.
//
// TEST INFRASTRUCTURE ONLY. Compiled by oracle/Makefile straight from the
// reference source tree (REF_ROOT), once per (app, precision), into
// oracle/_ref/libfvref.so. Its outputs pin the oracle restatement
// (fv_oracle.cpp) and generate tests/golden/ fixtures.
//
// The reference's CUDA no longer builds (texture references and
// cudaBindTexture2D are gone from CUDA 12+, and its driver needs GL/GLUT),
// so this file stands in for everything around the numerics:
//   * CUDA keywords compile away, and threadIdx/blockIdx/blockDim/gridDim
//     are host globals set so that offset = i + j*NX (blockDim.x = NX);
//   * each texture fetch wrapper tex*_read(int*, int*) reads a bound host
//     array with clamp addressing, the texture's default
//     (common/data_definitions.h:94-133, 149-364, 648-760);
//   * the __constant__ scratch pointers s1_ptr..apdq3_ptr are host pointers
//     (data_definitions.h:387-406);
//   * parameters.h constants are run-time globals with the same names;
//   * getmax/getmin are the two-line helpers of common/main.cu:63-69;
//   * run_steps() restates the step loop of common/main.cu:310-635, kernel
//     by kernel, including the pairwise CFL reduction (main.cu:503-519).
// The headers apps/na/fv.h, apps/na/source.h, common/filter.h,
// common/numbers.h and the app's boundary.h/init.h are included unmodified.
//
// One deliberate difference: on a rejected step (CFL >= CFLMAX) the
// reference restores only buffer A and never clears the device simError
// (main.cu:620-634), so its loop rejects forever. Here both buffers are
// restored and simError is cleared: a clean retry.
//
// Build-time macros: ROOT (reference tree, also on the include path),
// FVREF_APP_BOUNDARY / FVREF_APP_INIT (quoted paths of the app's hook
// headers), FVREF_SYM (entry-point name), PRECISION (1 float, 2 double).
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../include/fivonagi.h"

using namespace std;

#if PRECISION == 1
#define DATATYPEV float
#define DATATYPET float
#elif PRECISION == 2
#define DATATYPEV double
#define DATATYPET double
#else
#error PRECISION must be 1 or 2
#endif

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define INC_DEBUG_TOOLS_H 1
#define GPUGD_VARSFD bool none
#define GPUGD_VARSFC none
// The reference's own include-path macros (apps/hifu-beam/driver.cu:14-23),
// needed because its app headers include ROOT_PATH(/common/debug_tools.h).
#define EXPAND1(x) x
#define EXPAND2(x) #x
#define CONCAT_STR(x, y) EXPAND1(x)y
#define QUOTE(x) EXPAND2(x)
#define ROOT_PATH(FILE) QUOTE(CONCAT_STR(EXPAND1(ROOT), EXPAND1(FILE)))

namespace {

struct dim3h { int x, y, z; };
dim3h threadIdx, blockIdx, blockDim, gridDim;
const bool none = true;

// parameters.h names, set per call from fv_params
int NX, NY;
DATATYPEV BETA, DIFFDELTA, CFLMAX, CFLWHISH, MDVX, MDVY, MDT, TIDE;
DATATYPEV AMPL, FREC, ISPW, ISPa, ISPF;             // hifu-beam
DATATYPEV ISPRHOA, ISPC, ISPTHETA;                  // taylor-angle-xy
double PW_AMPL, PW_FREC, PW_ANGLE, PW_XMAX, PW_YMAX;  // plane wave
DATATYPEV FB_CENTER, FB_HALFAP, FB_RAMP;            // focused beam

template <typename TTT> inline TTT getmax(TTT x, TTT y) { return (x > y) ? x : y; }
template <typename TTT> inline TTT getmin(TTT x, TTT y) { return (x < y) ? x : y; }

#define FVREF_TEX(name)                                             \
  DATATYPEV *name##_bound = nullptr;                                \
  inline DATATYPEV name##_read(int *i, int *j) {                    \
    int ii = *i < 0 ? 0 : (*i > NX - 1 ? NX - 1 : *i);              \
    int jj = *j < 0 ? 0 : (*j > NY - 1 ? NY - 1 : *j);              \
    return name##_bound[ii + jj * NX];                              \
  }
FVREF_TEX(texAu1) FVREF_TEX(texAu2) FVREF_TEX(texAu3)
FVREF_TEX(texBu1) FVREF_TEX(texBu2) FVREF_TEX(texBu3)
FVREF_TEX(texCu1) FVREF_TEX(texCu2) FVREF_TEX(texCu3)
FVREF_TEX(texs1) FVREF_TEX(texs2) FVREF_TEX(texs3)
FVREF_TEX(texW11) FVREF_TEX(texW21) FVREF_TEX(texW31)
FVREF_TEX(texW12) FVREF_TEX(texW22) FVREF_TEX(texW32)
FVREF_TEX(texW13) FVREF_TEX(texW23) FVREF_TEX(texW33)
FVREF_TEX(texamdq1) FVREF_TEX(texapdq1) FVREF_TEX(texamdq2)
FVREF_TEX(texapdq2) FVREF_TEX(texamdq3) FVREF_TEX(texapdq3)

DATATYPEV *s1_ptr, *s2_ptr, *s3_ptr;
DATATYPEV *W11_ptr, *W21_ptr, *W31_ptr, *W12_ptr, *W22_ptr, *W32_ptr;
DATATYPEV *W13_ptr, *W23_ptr, *W33_ptr;
DATATYPEV *amdq1_ptr, *apdq1_ptr, *amdq2_ptr, *apdq2_ptr, *amdq3_ptr, *apdq3_ptr;

#include "common/numbers.h"
#include "common/filter.h"
#include "apps/na/source.h"
#include "apps/na/fv.h"
#include FVREF_APP_BOUNDARY
#include FVREF_APP_INIT

// A "launch" runs the kernel body once per cell of the NX x NY grid.
template <class F> void launch(F &&body) {
  blockDim = {NX, NY, 1};
  gridDim = {1, 1, 1};
  blockIdx = {0, 0, 0};
  for (int j = 0; j < NY; ++j)
    for (int i = 0; i < NX; ++i) {
      threadIdx = {i, j, 0};
      body();
    }
}

struct Buffers {
  size_t n;
  std::vector<DATATYPEV> A[3], B[3], C[3], s[3], W[9], amdq[3], apdq[3], cfl;
  explicit Buffers(size_t nn) : n(nn) {
    for (auto *v : {A, B, C, s, amdq, apdq})
      for (int f = 0; f < 3; ++f) v[f].assign(n, DATATYPEV(0));
    for (auto &w : W) w.assign(n, DATATYPEV(0));
    cfl.assign(n, DATATYPEV(0));
    texAu1_bound = A[0].data(); texAu2_bound = A[1].data(); texAu3_bound = A[2].data();
    texBu1_bound = B[0].data(); texBu2_bound = B[1].data(); texBu3_bound = B[2].data();
    texCu1_bound = C[0].data(); texCu2_bound = C[1].data(); texCu3_bound = C[2].data();
    texs1_bound = s1_ptr = s[0].data();
    texs2_bound = s2_ptr = s[1].data();
    texs3_bound = s3_ptr = s[2].data();
    DATATYPEV **wp[9] = {&W11_ptr, &W21_ptr, &W31_ptr, &W12_ptr, &W22_ptr,
                         &W32_ptr, &W13_ptr, &W23_ptr, &W33_ptr};
    DATATYPEV **wt[9] = {&texW11_bound, &texW21_bound, &texW31_bound,
                         &texW12_bound, &texW22_bound, &texW32_bound,
                         &texW13_bound, &texW23_bound, &texW33_bound};
    for (int k = 0; k < 9; ++k) *wp[k] = *wt[k] = W[k].data();
    texamdq1_bound = amdq1_ptr = amdq[0].data();
    texamdq2_bound = amdq2_ptr = amdq[1].data();
    texamdq3_bound = amdq3_ptr = amdq[2].data();
    texapdq1_bound = apdq1_ptr = apdq[0].data();
    texapdq2_bound = apdq2_ptr = apdq[1].data();
    texapdq3_bound = apdq3_ptr = apdq[2].data();
  }
};

void set_params(const fv_params *p) {
  NX = p->nx;
  NY = p->ny;
  BETA = DATATYPEV(p->beta);
  DIFFDELTA = DATATYPEV(p->diffdelta);
  CFLMAX = DATATYPEV(p->cflmax);
  CFLWHISH = DATATYPEV(p->cflwhish);
  MDVX = DATATYPEV(p->mdvx);
  MDVY = DATATYPEV(p->mdvy);
  MDT = DATATYPEV(p->mdt);
  TIDE = DATATYPEV(p->tide);
  AMPL = DATATYPEV(p->ampl);
  FREC = DATATYPEV(p->frec);
  ISPW = Num2 * PI * FREC;  // apps/hifu-beam/parameters.h:89
  ISPa = DATATYPEV(p->isp_a);
  ISPF = DATATYPEV(p->isp_f);
  ISPRHOA = DATATYPEV(p->isp_rhoa);
  ISPC = DATATYPEV(p->isp_c);
  ISPTHETA = DATATYPEV(p->angle);
  PW_AMPL = p->ampl;
  PW_FREC = p->frec;
  PW_ANGLE = p->angle;
  PW_XMAX = p->xmax;
  PW_YMAX = p->ymax;
  FB_CENTER = DATATYPEV(p->center);
  FB_HALFAP = DATATYPEV(p->aperture * 0.5);
  FB_RAMP = DATATYPEV(p->frec / p->ramp_periods);
}

struct Scalars {
  DATATYPEV dt, T, dx, dy;
  int n, MDX, MDY, simError;
};

void copy3(std::vector<DATATYPEV> *dst, std::vector<DATATYPEV> const *src) {
  for (int f = 0; f < 3; ++f) dst[f] = src[f];
}

// One attempted step of common/main.cu:310-635. Returns 0 accepted, 1
// rejected, 2 negative eigenvalue; stop_stage >= 0 stops after that stage
// and leaves the stage's grid in `stage_out`.
int attempt(Buffers &b, Scalars &sc, bool &uOut, const fv_params *p,
            int stop_stage, std::vector<DATATYPEV> *stage_out) {
  std::vector<DATATYPEV> *R = uOut ? b.A : b.B;
  std::vector<DATATYPEV> *Wt = uOut ? b.B : b.A;
  DATATYPEV *dt = &sc.dt, *dx = &sc.dx, *dy = &sc.dy, *T = &sc.T;
  int *MDX = &sc.MDX, *MDY = &sc.MDY, *simError = &sc.simError;
  DATATYPEV *cfl = b.cfl.data();
  DATATYPEV *C[3] = {b.C[0].data(), b.C[1].data(), b.C[2].data()};
  DATATYPEV *Rp[3] = {R[0].data(), R[1].data(), R[2].data()};
  DATATYPEV *Wp[3] = {Wt[0].data(), Wt[1].data(), Wt[2].data()};

  // texCpy(C <- !uOut buffer), main.cu:334-336
  launch([&] {
    int i = threadIdx.x, j = threadIdx.y, o = i + j * NX;
    bool dstOut = !uOut;
    C[0][o] = dstOut ? texAu1_read(&i, &j) : texBu1_read(&i, &j);
    C[1][o] = dstOut ? texAu2_read(&i, &j) : texBu2_read(&i, &j);
    C[2][o] = dstOut ? texAu3_read(&i, &j) : texBu3_read(&i, &j);
  });
  launch([&] { boundary(MDX, MDY, Rp[0], Rp[1], Rp[2], dx, dy, dt, T, none, !uOut); });
  if (stop_stage == FV_STAGE_BOUNDARY) { copy3(stage_out, R); return 0; }
  // y sweep, main.cu:353-419
  launch([&] { getWavesSpeedsCFL_y(cfl, dy, dt, simError, none, uOut); });
  if (*simError == 2) return 2;
  launch([&] { step_y(Wp[0], Wp[1], Wp[2], dy, dt, none, uOut); });
  launch([&] { calcLimiters_y(none, dy, dt); });
  launch([&] { writeLimiters_y(Rp[0], Rp[1], Rp[2], dy, dt, none, !uOut); });
  if (stop_stage == FV_STAGE_SWEEP_Y) { copy3(stage_out, R); return 0; }
  // x sweep, main.cu:430-496
  launch([&] { getWavesSpeedsCFL_x(cfl, dx, dt, simError, none, uOut); });
  if (*simError == 2) return 2;
  launch([&] { step_x(Wp[0], Wp[1], Wp[2], dx, dt, none, uOut); });
  launch([&] { calcLimiters_x(none, dx, dt); });
  launch([&] { writeLimiters_x(Rp[0], Rp[1], Rp[2], dx, dt, none, !uOut); });
  if (stop_stage == FV_STAGE_SWEEP_X) { copy3(stage_out, R); return 0; }
  // reduceCFL: pairwise halving to two elements, main.cu:503-519
  int sizered = NX * NY;
  auto reduce = [&](int sz) {
    for (int i = 0; i < sz; ++i)
      if (i >= 0 && i <= NX * NY - 1) cfl[i] = getmax(cfl[i], cfl[i + sz]);
  };
  while (sizered > 32) { sizered = sizered / 2; reduce(sizered); }
  while (sizered > 2) { sizered = sizered / 2; reduce(sizered); }
  // reduceCFL2, main.cu:200-212
  if (!(cfl[0] < CFLMAX)) *simError = 1;
  if (stop_stage == FV_STAGE_SOURCE) {
    launch([&] { source(Wp[0], Wp[1], Wp[2], dx, dy, dt, MDX, MDY, none, uOut); });
    copy3(stage_out, Wt);
    return 0;
  }
  int result;
  if (*simError == 0) {
    launch([&] { source(Wp[0], Wp[1], Wp[2], dx, dy, dt, MDX, MDY, none, uOut); });
    *T = (*T) + (*dt);  // update_T, main.cu:232-238
    sc.n = sc.n + 1;
    // moveDomain (A <- shifted B), main.cu:109-164, 575-580
    int MDi = 0, MDj = 0;
    if (p->moving_domain && (*T) >= MDT) {
      MDi = static_cast<int>(((*T) - MDT) * MDVX / (*dx)) - (*MDX);
      MDj = static_cast<int>(((*T) - MDT) * MDVY / (*dy)) - (*MDY);
    }
    launch([&] {
      int i = threadIdx.x, j = threadIdx.y, o = i + j * NX;
      int ir = i + MDi, jr = j + MDj;
      if (!(ir <= NX - 1 && jr <= NY - 1)) { ir = i; jr = j; }
      bool dstOut = !uOut;
      Rp[0][o] = dstOut ? texAu1_read(&ir, &jr) : texBu1_read(&ir, &jr);
      Rp[1][o] = dstOut ? texAu2_read(&ir, &jr) : texBu2_read(&ir, &jr);
      Rp[2][o] = dstOut ? texAu3_read(&ir, &jr) : texBu3_read(&ir, &jr);
    });
    *MDX += MDi;  // updateMDXY, main.cu:166-177
    *MDY += MDj;
    // texCpy(W <- uOut buffer), main.cu:592-593
    launch([&] {
      int i = threadIdx.x, j = threadIdx.y, o = i + j * NX;
      Wp[0][o] = uOut ? texAu1_read(&i, &j) : texBu1_read(&i, &j);
      Wp[1][o] = uOut ? texAu2_read(&i, &j) : texBu2_read(&i, &j);
      Wp[2][o] = uOut ? texAu3_read(&i, &j) : texBu3_read(&i, &j);
    });
    uOut = !uOut;
    result = 0;
  } else {
    // restore (R <- C), main.cu:93-107, 620-623; and W <- C (clean retry)
    copy3(R, b.C);
    copy3(Wt, b.C);
    result = 1;
  }
  // update_dt, main.cu:214-230
  DATATYPEV cflStep = cfl[0];
  DATATYPEV new_dt = (*dt) * CFLWHISH / cflStep;
  if (*simError == 1 && new_dt > (*dt) * 0.9) *dt = (*dt) * 0.9;
  else *dt = new_dt;
  *simError = 0;
  return result;
}

}  // namespace

// op: 0 = init hook into u; 1 = run nsteps accepted steps from u and the
// scalars (dt, T, n, MDX, MDY in `scal`), result back into u and scal;
// 10 + stage = one attempt stopped after `stage`, stage grid into u.
// Returns an fv_status; st (optional) gets accepted/rejected counts.
extern "C" int FVREF_SYM(const fv_params *p, int op, int64_t nsteps,
                         DATATYPEV *u1, DATATYPEV *u2, DATATYPEV *u3,
                         double *scal, fv_run_stats *st) {
  set_params(p);
  const size_t n = size_t(NX) * size_t(NY);
  Scalars sc{};
  sc.dx = DATATYPEV(p->xmax) / DATATYPEV(NX - 1);  // main.cu:790-791
  sc.dy = DATATYPEV(p->ymax) / DATATYPEV(NY - 1);
  if (op == 0) {
    DATATYPEV dtv = DATATYPEV(p->dtini);
    init(u1, u2, u3, &sc.dx, &sc.dy, &dtv, none);
    return FV_OK;
  }
  Buffers b(n);
  DATATYPEV *u[3] = {u1, u2, u3};
  for (int f = 0; f < 3; ++f) {
    std::memcpy(b.A[f].data(), u[f], n * sizeof(DATATYPEV));
    std::memcpy(b.B[f].data(), u[f], n * sizeof(DATATYPEV));
  }
  sc.dt = DATATYPEV(scal[0]);
  sc.T = DATATYPEV(scal[1]);
  sc.n = int(scal[2]);
  sc.MDX = int(scal[3]);
  sc.MDY = int(scal[4]);
  sc.simError = 0;
  bool uOut = true;
  int rc = FV_OK;
  int64_t acc = 0, rej = 0;
  if (op >= 10) {
    std::vector<DATATYPEV> out[3];
    int r = attempt(b, sc, uOut, p, op - 10, out);
    if (r == 2) return FV_NEGATIVE_EIGENVALUE;
    for (int f = 0; f < 3; ++f) std::memcpy(u[f], out[f].data(), n * sizeof(DATATYPEV));
    return FV_OK;
  }
  int consecutive = 0;
  const int max_retries = p->max_retries > 0 ? p->max_retries : 64;
  while (acc < nsteps) {
    int r = attempt(b, sc, uOut, p, -1, nullptr);
    if (r == 2) { rc = FV_NEGATIVE_EIGENVALUE; break; }
    if (r == 1) {
      ++rej;
      if (++consecutive >= max_retries) { rc = FV_DT_TOO_LARGE; break; }
      continue;
    }
    consecutive = 0;
    ++acc;
  }
  std::vector<DATATYPEV> *cur = uOut ? b.A : b.B;
  for (int f = 0; f < 3; ++f) std::memcpy(u[f], cur[f].data(), n * sizeof(DATATYPEV));
  scal[0] = double(sc.dt);
  scal[1] = double(sc.T);
  scal[2] = double(sc.n);
  scal[3] = double(sc.MDX);
  scal[4] = double(sc.MDY);
  if (st) {
    st->accepted = acc;
    st->rejected = rej;
    st->dt = scal[0];
    st->T = scal[1];
    st->n = sc.n;
    st->status = rc;
    st->mdx = sc.MDX;
    st->mdy = sc.MDY;
  }
  return rc;
}
