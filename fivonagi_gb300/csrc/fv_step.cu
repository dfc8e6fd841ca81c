// fv_step.cu -- the fused time-step kernel for sm_103a.
//
// An attempt runs the reference's loop body (common/main.cu:310-635):
//   boundary (app hook)  ->  y sweep  ->  x sweep  ->  CFL max  ->
//   [accepted] diffusion, T += dt, n += 1  ->  dt update,
// as four launches: the ghost-frame pre-pass (the app hook's values of the
// ghost cells), the step kernel, the fix-up kernel and a one-CTA finalize
// kernel. The reference runs it as ~34 kernel launches that pass 19 scratch
// grids through global memory (~750 B per cell-update) and 7 blocking
// device-to-host copies. Here every intermediate lives in registers:
//
//  * Each warp streams a window of 32 consecutive columns up the grid, one
//    row per iteration. Lanes 3..28 produce output; the three lanes on each
//    side are the x-halo the limiter and diffusion need.
//  * y sweep: a lane keeps the last rows of its own column (state, waves,
//    first-order sums, correction fluxes) in registers, so each y interface
//    is solved once per window and each cell is updated two rows behind the
//    row being loaded.
//  * x sweep: once a row of y-updated cells is ready, neighbouring columns
//    are neighbouring lanes; the Riemann inputs, waves, dot products,
//    fluctuations and correction fluxes move between lanes with warp
//    shuffles.
//  * diffusion (source): runs two rows behind the x sweep, on registers.
//  * CFL: each lane keeps a running maximum over its output cells; warp
//    shuffles and a CTA reduction give one value per CTA, and the finalize
//    kernel reduces those, accepts or rejects the step, and updates dt, T,
//    n and the current-buffer index in device memory. A rejected step
//    leaves the input buffer current, so the retry starts from the pre-step
//    state.
//
// Work distribution: every warp streams an equal share of the launch's
// cost, in (window, row) order, windows being the 26-column output spans.
// A row of a window with ghost columns costs 1.5 rows of an interior one,
// and each window start costs 6 rows (the warp that enters it runs the
// loop's warm-up and drain again); a share may span two windows.
//
// Division (fv_device.cuh): by default the step kernel divides exactly
// (kStageExactDiv): DivExact for the quotients that can be subnormal, and
// DivNormal, which flags a subnormal result, for the others. Stage -1
// divides with Markstein's FMA sequence (DivFma) instead, which equals IEEE
// division unless an operand is tiny, huge or not finite. Either way, a
// warp that meets a flagged division in an iteration marks the rows that
// iteration can influence (chunks of kFixRows rows of its window) and
// leaves their CFL and negative-eigenvalue checks out; the fix-up kernel
// then recomputes the marked chunks from the same input with DivExact (IEEE
// division wherever even that flags), overwriting their output, before the
// finalize kernel decides the attempt. Marked chunks are rare (none in
// practice with exact division), and the step kernel's arithmetic has no
// branches: its only branches are uniform over a warp (interior-row loads,
// the store of an attempt without a window shift, the rare marks).
// The same flag carries the subsonic solve's assumption (L1 > 0 > L2 at
// every interface; DivPair in fv_device.cuh): the step kernel skips the
// speed-sign tests and the negative-eigenvalue check, and the fix-up
// kernel's general solve redoes any rows where the assumption fails.
//
// This file is compiled twice: FV_VARIANT_EXACT with --fmad=false (the
// oracle's evaluation, bit for bit) and the fast variant with FMA
// contraction.
#include <cuda_runtime.h>

#include <type_traits>

#include "fv_device.cuh"

#ifndef FV_VARIANT_EXACT
#define FV_VARIANT_EXACT 0
#endif

namespace fvgb {
#if FV_VARIANT_EXACT
namespace exact_ns {
#else
namespace fast_ns {
#endif

constexpr int kWarps = 4;
constexpr int kThreads = kWarps * kLanes;
constexpr int kStripCols = kWarps * kWarpCols;  // 104 output columns per strip

__device__ __forceinline__ float shup(float v) { return __shfl_up_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ float shdn(float v) { return __shfl_down_sync(0xffffffffu, v, 1); }

struct Cell3 {
  float u1, u2, u3;
};

// Results of the y chain of one iteration (interface r, flux r-1).
struct YOut {
  float vx, vy;  // velocities of row r
  WaveN w;       // waves at interface r
  Fluct f;
  float cy;      // CFL of interface r
  bool ok;       // no negative eigenvalue
  Dots dr;       // dots of interfaces r-1, r
  float fa1, fa2, fa3;  // correction flux at interface r-1
};

// Results of the x chain of one iteration (row r-3).
struct XOut {
  Cell3 s2;        // state after the x sweep
  float vx2, vy2;  // its velocities
  float cx;        // CFL of the cell (y and x interfaces)
  bool ok;
};

__device__ __forceinline__ void store3(float *const *out, int o, const Cell3 &v) {
  out[0][o] = v.u1;
  out[1][o] = v.u2;
  out[2][o] = v.u3;
}

// Marks chunks of one warp window for the fix-up kernel (layout in
// fv_internal.h). Called warp-uniformly; lane 0 does the atomics. The
// layout is read from the launch's parameters when a mark happens, so the
// row loop holds only `last` in a register.
struct StepMarker {
  const StepArgs &a;
  int last;  // last chunk this warp marked in this strip segment
  // rows lo..hi (inclusive) of the window of the warp at column xw
  __device__ __forceinline__ void mark(int xw, int lo, int hi) {
    const int c0 = max(lo / kFixRows, last + 1), c1 = hi / kFixRows;
    if ((threadIdx.x & 31) == 0) {
      const unsigned cpw = (unsigned)fix_chunks_per_window(a.p.ny);
      const unsigned words = (unsigned)fix_bitmap_words((long long)a.nstrips * (kStripCols / kWarpCols), a.p.ny);
      uint32_t *fix = a.fix;
      for (int c = c0; c <= c1; ++c) {
        const unsigned id = (unsigned)(xw / kWarpCols) * cpw + (unsigned)c;
        const unsigned bit = 1u << (id & 31u);
        if (!(atomicOr(fix + 4 + (id >> 5), bit) & bit)) fix[4 + words + atomicAdd(fix, 1u)] = id;
      }
    }
    last = max(last, c1);
  }
};

// For division policies that never flag.
struct NoMarker {
  __device__ __forceinline__ void mark(int, int, int) {}
};

// Records that some iteration was flagged (the fix-up pass redoes the
// window with IEEE division then).
struct FlagMarker {
  bool flagged = false;
  __device__ __forceinline__ void mark(int, int, int) { flagged = true; }
};

// Stream one warp's 32 columns over output rows [y0, y1) of a strip.
//
// Iteration r loads row r and runs three chains that do not depend on each
// other within the iteration, so their instructions interleave:
//   Y: y interface r, correction flux at r-1, y update of row r-2 (S1);
//   X: x sweep of row r-3 (S1 of the previous iteration -> S2) and the CFL
//      of its cells;
//   D: diffusion of row r-5 from S2 of rows r-6, r-5, r-4 (source).
// Warm-up and drain iterations run only the chains whose results the
// window needs (three phases, below); results on rows outside the window
// are discarded (stores and checks are predicated).
// EDGE: the warp's columns include ghost columns.
// STAGE < 0: full step into `out`; STAGE 0..3: that stage's grid into `out`;
// kStageRecord: the full step into out[0..2] and the stage grids B, S1, S2
// into out[3..11].
// DP: division policy. With DivFma, an iteration whose divisions may differ
// from IEEE division marks the output rows it can influence (mk), and the
// CFL and negative-eigenvalue checks that depend on it are left to the
// fix-up kernel:
//   a division of the y chain of iteration f (row f's velocities, the
//   interface f solve, the limiter at f-1) feeds the waves at interfaces f
//   and f+1, hence the correction fluxes at f-1 .. f+2, the y-updated rows
//   f-2 .. f+2, and after diffusion rows f-3 .. f+3; the x chain of
//   iteration f (row f-3) feeds diffusion rows f-4 .. f-2. So iteration f
//   marks rows f-4 .. f+3. The CFL of row r-3, taken in iteration r,
//   depends on y chains r-5 .. r-1 and the x chain r; the y solve's
//   eigenvalue check at interface r on y chains r-1 and r.
// PRE: rows loaded ahead of the one in use (the fix-up's short items load
// all their rows at once).
template <int STAGE, bool EDGE, class DP, int PRE, class MK>
__device__ __forceinline__ void stream_strip(const DevParams &p, const float *const *in,
                                             const float *const *frame,
                                             float *const *out, int xw, int y0, int y1,
                                             float dt, float T, int mdx, int mdy, int shx,
                                             int shy, float &cmax, bool &neg, MK &mk) {
  const int lane = threadIdx.x & (kLanes - 1);
  const int nx = p.nx, ny = p.ny;
  const int i = xw - kHalo + lane;
  // A window without ghost columns has all its 32 columns in [2, nx-3]
  // (stream_window's test), so those column tests are constant there.
  const bool col_ok = EDGE ? ((i >= 0) && (i < nx)) : true;
  const bool out_lane = col_ok && lane >= kHalo && lane < kLanes - kHalo;
  const bool col_int = EDGE ? ((i >= 2) && (i <= nx - 3)) : true;
  const float dtx = dt / p.dx;
  const float dty = dt / p.dy;
  const float ddtx2 = p.diffdelta * dt / (p.dx * p.dx);
  const float ddty2 = p.diffdelta * dt / (p.dy * p.dy);
  const float two_bm1 = 2.0f * (p.beta - 1.0f);
  const int ci = col_ok ? i : 0;
  const bool even_only = p.cfl_even_only != 0;
  const float *const i0 = in[0], *const i1 = in[1], *const i2 = in[2];
  const float *const f0 = frame[0], *const f1 = frame[1], *const f2 = frame[2];

  // ---- carried state (names give the row relative to the loaded row r)
  Cell3 s0_m2{0.f, 0.f, 0.f}, s0_m1{0.f, 0.f, 0.f};  // boundary-applied state
  float vx_m1 = 0.f, vy_m1 = 0.f;
  WaveN w_m1{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // y waves, interface r-1
  Dots dl_m1{0.f, 0.f, 0.f};                     // dots of interfaces r-2, r-1
  float ap1 = 0.f, ap2 = 0.f, ap3 = 0.f;         // apdq, interface r-1
  float fo1 = 0.f, fo2 = 0.f, fo3 = 0.f;         // first-order sum of cell r-2
  float fa1 = 0.f, fa2 = 0.f, fa3 = 0.f;         // correction flux, interface r-2
  float cy_m1 = 0.f, cy_m2 = 0.f, cy_m3 = 0.f;   // y CFL of rows r-1..r-3
  Cell3 s1_m3{0.f, 0.f, 0.f};                    // S1 of row r-3 (X input)
  Cell3 s2_m4{0.f, 0.f, 0.f}, s2_m5{0.f, 0.f, 0.f};  // S2 of rows r-4, r-5
  float vx2_m4 = 0.f, vy2_m4 = 0.f, vx2_m5 = 0.f, vy2_m5 = 0.f, vx2_m6 = 0.f, vy2_m6 = 0.f;

  // Row r of the state after the boundary hook: ghost cells come from the
  // ghost frame. Warps without ghost columns only meet ghost rows, which
  // are the same for the whole warp.
  auto load_raw = [&](int r, Cell3 &v) {
    if constexpr (!EDGE) {
      // interior rows of an interior window (a branch uniform over the
      // warp): plain loads
      if (r >= 2 && r < ny - 2) {
        const int o = i + r * nx;
        v.u1 = __ldg(i0 + o);
        v.u2 = __ldg(i1 + o);
        v.u3 = __ldg(i2 + o);
        return;
      }
    }
    if (col_ok && r >= 0 && r < ny) {
      const bool gh = EDGE ? is_ghost(p, i, r) : (r <= 1 || r >= ny - 2);
      const int o = gh ? frame_index(ci, r, nx, ny) : ci + r * nx;
      v.u1 = __ldg((gh ? f0 : i0) + o);
      v.u2 = __ldg((gh ? f1 : i1) + o);
      v.u3 = __ldg((gh ? f2 : i2) + o);
    } else {
      v = Cell3{0.f, 0.f, 0.f};
    }
  };
  static_assert(PRE >= 1, "at least the row in use");
  Cell3 pf[PRE];  // prefetched raw rows r .. r+PRE-1
#pragma unroll
  for (int k = 0; k < PRE; ++k) load_raw(y0 - 3 + k, pf[k]);

  unsigned yhist = 0u;
  // One iteration at loaded row r with the chains it needs. Y's results
  // are used for r in [y0-3, y1+2], X's for [y0+2, y1+3], D's for
  // [y0+5, y1+4]. The loop below runs three compile-time phases: Y alone
  // for r <= y0+1, all three chains up to y1+2, X and D for the last two
  // (the other chains' results there lie outside the window, and their
  // stores and checks are predicated on the window's rows). Each phase's
  // body stays free of branches, so its chains interleave; three copies
  // of the body keep the instruction footprint small.
  auto iterate = [&](int r, auto run_y, auto run_x, auto run_d) {
    constexpr bool RY = decltype(run_y)::value;
    constexpr bool RX = decltype(run_x)::value;
    constexpr bool RD = decltype(run_d)::value;
    Cell3 u{0.f, 0.f, 0.f};
    if constexpr (RY) {
      u = pf[0];
#pragma unroll
      for (int k = 0; k + 1 < PRE; ++k) pf[k] = pf[k + 1];
      if (r + PRE <= y1 + 2) load_raw(r + PRE, pf[PRE - 1]);
    }

    // ======== Y chain: interface r, flux r-1, update of row r-2
    // ======== X chain: row r-3; normal = u2, transverse = u3
    YOut yo;
    XOut xo;
    auto y_chain = [&](auto &dp) {
      const float rho = u.u1 + 1.0f;
      const auto rr = dp.s.recip(rho);
      yo.vx = dp.s.div_r(u.u2, rr);
      yo.vy = dp.x.div_r(u.u3, rr);
      yo.cy = 0.0f;
      // normal = u3: the normal velocity's quotients are the others (DivPair)
      yo.ok = riemann<true, DP::kSubsonic>(rho, u.u3, u.u2, yo.vy, yo.vx, s0_m1.u1 + 1.0f, s0_m1.u3, s0_m1.u2, vy_m1,
                            vx_m1, two_bm1, dty, yo.cy, yo.w, yo.f, dp.s, dp.x);
      yo.dr = wave_dots<DP::kSubsonic>(w_m1, yo.w);
      correction<DP::kSubsonic>(w_m1, dl_m1, yo.dr, dty, yo.fa1, yo.fa2, yo.fa3, dp.s);
    };
    auto x_chain = [&](auto &dp) {
      const float rho1 = s1_m3.u1 + 1.0f;
      const auto rr = dp.s.recip(rho1);
      const float vn1 = dp.s.div_r(s1_m3.u2, rr);
      const float vt1 = dp.x.div_r(s1_m3.u3, rr);
      const float rho1m = shup(rho1), u2m = shup(s1_m3.u2), u3m = shup(s1_m3.u3);
      const float vn1m = shup(vn1), vt1m = shup(vt1);
      WaveN wx;
      Fluct fx;
      xo.cx = cy_m3;  // the x kernel starts from the cell's y value (fv.h:57)
      // transverse = u3: the transverse velocity's quotients are the others
      xo.ok = riemann<false, DP::kSubsonic>(rho1, s1_m3.u2, s1_m3.u3, vn1, vt1, rho1m, u2m, u3m, vn1m, vt1m, two_bm1,
                             dtx, xo.cx, wx, fx, dp.s, dp.x);
      WaveN wn;
      wn.w11 = shdn(wx.w11); wn.w21 = shdn(wx.w21); wn.w31 = shdn(wx.w31);
      wn.w12 = shdn(wx.w12); wn.w22 = shdn(wx.w22); wn.w32 = shdn(wx.w32);
      wn.w33 = shdn(wx.w33);
      const Dots drx = wave_dots<DP::kSubsonic>(wx, wn);
      Dots dlx;
      dlx.d1 = shup(drx.d1); dlx.d2 = shup(drx.d2); dlx.d3 = shup(drx.d3);
      float fx1, fx2, fx3;
      correction<DP::kSubsonic>(wx, dlx, drx, dtx, fx1, fx2, fx3, dp.s);
      const float amn1 = shdn(fx.am1), amn2 = shdn(fx.am2), amn3 = shdn(fx.am3);
      const float fxn1 = shdn(fx1), fxn2 = shdn(fx2), fxn3 = shdn(fx3);
      const bool in_x = col_int && r - 3 >= 2 && r - 3 <= ny - 3;
      const float m1 = s1_m3.u1 - dtx * (fx.ap1 + amn1);
      const float m2 = s1_m3.u2 - dtx * (fx.ap2 + amn2);
      const float m3 = s1_m3.u3 - dtx * (fx.ap3 + amn3);
      xo.s2.u1 = in_x ? m1 - dtx * (fxn1 - fx1) : s1_m3.u1;
      xo.s2.u2 = in_x ? m2 - dtx * (fxn2 - fx2) : s1_m3.u2;
      xo.s2.u3 = in_x ? m3 - dtx * (fxn3 - fx3) : s1_m3.u3;
      const float rho2 = xo.s2.u1 + 1.0f;
      const auto rr2 = dp.s.recip(rho2);
      xo.vx2 = dp.s.div_r(xo.s2.u2, rr2);
      xo.vy2 = dp.x.div_r(xo.s2.u3, rr2);
    };
    DP dy, dx;
    if constexpr (RY) y_chain(dy);
    if constexpr (RX) x_chain(dx);
    bool excl_y = false, excl_x = false, flagged = false;
    if constexpr (DP::kFlags) {
      bool yf = false, xf = false;
      if constexpr (RY) yf = __any_sync(0xffffffffu, dy.unsafe());
      if constexpr (RX) xf = __any_sync(0xffffffffu, dx.unsafe());
      yhist = (yhist << 1) | (yf ? 1u : 0u);  // bit k: y chain of iteration r-k
      excl_y = (yhist & 0x3u) != 0u;
      excl_x = xf || (yhist & 0x3eu) != 0u;
      flagged = yf || xf;
    }

    // ---- Y results
    if constexpr (RY) {
      const float cy = (r <= 0) ? 0.0f : yo.cy;  // cfl = 0 on j == 0 (apps/na/fv.h:212-215)
      // (the subsonic solve flags tmp3 < 0 too, so the fix-up pass makes
      // this check there)
      if constexpr (!DP::kSubsonic) neg = neg || (!yo.ok && !excl_y && out_lane && r >= y0 && r < y1 && r >= 1);
      const float fn1 = ap1 + yo.f.am1, fn2 = ap2 + yo.f.am2, fn3 = ap3 + yo.f.am3;
      const int cyr = r - 2;  // row of the y update
      Cell3 s1 = s0_m2;
      {
        // local components: 1 -> u1, 2 (normal) -> u3, 3 (transverse) -> u2
        const float m1 = s0_m2.u1 - dty * fo1;
        const float m3 = s0_m2.u3 - dty * fo2;
        const float m2 = s0_m2.u2 - dty * fo3;
        const bool in_y = col_int && cyr >= 2 && cyr <= ny - 3;
        s1.u1 = in_y ? m1 - dty * (yo.fa1 - fa1) : s0_m2.u1;
        s1.u3 = in_y ? m3 - dty * (yo.fa2 - fa2) : s0_m2.u3;
        s1.u2 = in_y ? m2 - dty * (yo.fa3 - fa3) : s0_m2.u2;
      }
      if (STAGE == FV_STAGE_BOUNDARY || STAGE == FV_STAGE_SWEEP_Y) {
        if (out_lane && cyr >= y0 && cyr < y1) store3(out, i + cyr * nx, STAGE == FV_STAGE_BOUNDARY ? s0_m2 : s1);
      }
      if (STAGE == kStageRecord) {
        if (out_lane && cyr >= y0 && cyr < y1) {
          store3(out + 3, i + cyr * nx, s0_m2);
          store3(out + 6, i + cyr * nx, s1);
        }
      }
      // rotate the Y chain's carried values (the X chain of this iteration
      // has already read s1_m3 and cy_m3)
      s0_m2 = s0_m1;
      s0_m1 = u;
      vx_m1 = yo.vx;
      vy_m1 = yo.vy;
      w_m1 = yo.w;
      dl_m1 = yo.dr;
      ap1 = yo.f.ap1; ap2 = yo.f.ap2; ap3 = yo.f.ap3;
      fo1 = fn1; fo2 = fn2; fo3 = fn3;
      fa1 = yo.fa1; fa2 = yo.fa2; fa3 = yo.fa3;
      cy_m3 = cy_m2;
      cy_m2 = cy_m1;
      cy_m1 = cy;
      s1_m3 = s1;
    }

    // ---- X results
    if constexpr (RX) {
      const int cxr = r - 3;
      const bool own_x = out_lane && cxr >= y0 && cxr < y1;
      if constexpr (!DP::kSubsonic) neg = neg || (!xo.ok && !excl_x && own_x && i >= 1);
      {
        // CFL of cell (i, r-3): its y and x interfaces; 0 on i == 0
        const float cell = (i == 0) ? 0.0f : xo.cx;
        const bool counted = own_x && !excl_x && (!even_only || ((i + cxr * nx) & 1) == 0);
        cmax = counted ? nanmax(cmax, cell) : cmax;
      }
      if (STAGE == FV_STAGE_SWEEP_X) {
        if (own_x) store3(out, i + cxr * nx, xo.s2);
      }
      if (STAGE == kStageRecord) {
        if (own_x) store3(out + 9, i + cxr * nx, xo.s2);
      }
    }

    // ======== D chain: diffusion of row r-5 (apps/na/source.h:22-104)
    if constexpr (RD) {
      const int cdr = r - 5;
      const float vxl = shup(vx2_m5), vyl = shup(vy2_m5);
      const float vxr = shdn(vx2_m5), vyr = shdn(vy2_m5);
      if (STAGE < 0 || STAGE == FV_STAGE_SOURCE) {
        const bool in_d = col_int && cdr >= 2 && cdr <= ny - 3;
        Cell3 o3;
        o3.u1 = in_d ? (s2_m5.u1 + 1.0f) - 1.0f : s2_m5.u1;
        o3.u2 = in_d ? s2_m5.u2 + ddtx2 * (vxl - 2.0f * vx2_m5 + vxr) +
                           ddty2 * (vx2_m6 - 2.0f * vx2_m5 + vx2_m4)
                     : s2_m5.u2;
        o3.u3 = in_d ? s2_m5.u3 + ddtx2 * (vyl - 2.0f * vy2_m5 + vyr) +
                           ddty2 * (vy2_m6 - 2.0f * vy2_m5 + vy2_m4)
                     : s2_m5.u3;
        if (out_lane && cdr >= y0 && cdr < y1) {
          if (STAGE < 0 && shx == 0 && shy == 0) {
            store3(out, i + cdr * nx, o3);  // no shift this attempt (uniform)
          } else if (STAGE < 0) {
            // moving window (moveDomain, common/main.cu:109-164): the new
            // cell (i - shx, j - shy) takes this cell's value, and a cell
            // whose source would lie past the far edge keeps its own value
            const int ti = i - shx, tj = cdr - shy;
            if (ti >= 0 && tj >= 0) store3(out, ti + tj * nx, o3);
            if (i + shx > nx - 1 || cdr + shy > ny - 1) store3(out, i + cdr * nx, o3);
          } else {
            store3(out, i + cdr * nx, o3);
          }
        }
      }
    }

    // ======== rotate the X chain's results (read by the D chain above)
    if constexpr (RX) {
      s2_m5 = s2_m4;
      s2_m4 = xo.s2;
      vx2_m6 = vx2_m5; vy2_m6 = vy2_m5;
      vx2_m5 = vx2_m4; vy2_m5 = vy2_m4;
      vx2_m4 = xo.vx2; vy2_m4 = xo.vy2;
    }

    // ======== rare: mark the rows this iteration can influence
    if constexpr (DP::kFlags) {
      if (flagged) {
        const int lo = max(r - 4, y0), hi = min(r + 3, y1 - 1);
        if (lo <= hi) mk.mark(xw, lo, hi);
      }
    }
  };
  const std::true_type on{};
  const std::false_type off{};
  int r = y0 - 3;
  for (; r <= y0 + 1; ++r) iterate(r, on, off, off);  // warm-up: Y only
  for (; r <= y1 + 2; ++r) iterate(r, on, on, on);
  for (; r <= y1 + 4; ++r) iterate(r, off, on, on);  // drain: no Y
}

// Accept or reject an attempt from its CFL, and update dt/T/n/cur/MDX/MDY
// (reduceCFL2, update_T, updateMDXY and update_dt of common/main.cu:166-230).
// One thread; the control block is not read by anyone else until the next
// launch.
__device__ void decide(volatile Ctrl *vc, const DevParams &p, float cfl, bool negative) {
  const float dt = vc->dt;
  vc->last_cfl = cfl;
  if (negative) {
    vc->status = FV_NEGATIVE_EIGENVALUE;
    vc->neg_flag = 0;
    vc->last_accepted = 0;
    return;
  }
  int sim_error = 0;
  if (cfl < p.cflmax) {  // reduceCFL2, common/main.cu:200-212
    const float Tn = vc->T + dt;  // update_T, main.cu:232-238
    vc->T = Tn;
    vc->n = vc->n + 1;
    if (p.moving_domain && Tn >= p.mdt) {  // updateMDXY, main.cu:166-177
      const int mx = vc->mdx, my = vc->mdy;
      vc->mdx = mx + (static_cast<int>((Tn - p.mdt) * p.mdvx / p.dx) - mx);
      vc->mdy = my + (static_cast<int>((Tn - p.mdt) * p.mdvy / p.dy) - my);
    }
    vc->cur = vc->cur ^ 1;
    vc->remaining = vc->remaining - 1;
    vc->accepted = vc->accepted + 1;
    vc->consecutive_rejects = 0;
  } else {
    sim_error = 1;
    vc->rejected = vc->rejected + 1;
    const int cr = vc->consecutive_rejects + 1;
    vc->consecutive_rejects = cr;
    if (cr >= p.max_retries) vc->status = FV_DT_TOO_LARGE;
  }
  vc->sim_error = sim_error;
  vc->last_accepted = sim_error ? 0 : 1;
  // update_dt, main.cu:214-230 (the 0.9 is a double literal)
  const float new_dt = dt * p.cflwhish / cfl;
  if (sim_error == 1 && (double)new_dt > (double)dt * 0.9)
    vc->dt = (float)((double)dt * 0.9);
  else
    vc->dt = new_dt;
}

// Whether an attempt runs: the run has steps left, no error, T < t_stop.
// The control block only changes between launches, so every CTA of a
// launch sees the same answer.
__device__ __forceinline__ bool attempt_active(const Ctrl *ctl) {
  const int status = __ldcg(&ctl->status);
  const long long remaining = __ldcg((const long long *)&ctl->remaining);
  const float T0 = __ldcg(&ctl->T), ts = __ldcg(&ctl->t_stop);
  return status == 0 && remaining > 0 && T0 < ts;
}

// Reduce the partial CFL maxima of the step launch (and of the fix-up
// launch, when it had chunks to do) and decide; one CTA (all its threads).
__device__ void finalize(const StepArgs &a, float *red) {
  Ctrl *ctl = a.ctrl;
  float m = 0.0f;
  const int np = a.nblocks + (__ldcg(a.fix) > 0u ? a.fix_blocks : 0);
  for (int b = threadIdx.x; b < np; b += blockDim.x) m = nanmax(m, __ldcg(a.partials + b));
  for (int off = 16; off > 0; off >>= 1) m = nanmax(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x != 0) return;
  float cfl = 0.0f;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) cfl = nanmax(cfl, red[w]);
  volatile Ctrl *vc = ctl;
  decide(vc, a.p, cfl, vc->neg_flag != 0);
  // the fix-up scratch is zero again for the next attempt (the bitmap was
  // cleared chunk by chunk)
  volatile uint32_t *fx = a.fix;
  fx[0] = 0u;
  fx[1] = 0u;
  __threadfence();
}

// Shift of the moving window this attempt applies if it is accepted:
// updateMDXY with the updated T (common/main.cu:126-137, 166-177); 0 before
// MDT.
__device__ __forceinline__ void window_shift(const DevParams &p, float T, float dt, int mdx, int mdy,
                                             int &shx, int &shy) {
  shx = 0;
  shy = 0;
  if (p.moving_domain) {
    const float Tn = T + dt;
    if (Tn >= p.mdt) {
      shx = static_cast<int>((Tn - p.mdt) * p.mdvx / p.dx) - mdx;
      shy = static_cast<int>((Tn - p.mdt) * p.mdvy / p.dy) - mdy;
    }
  }
}

// One warp's window [y0, y1) at column xw, with the division policy DP and
// PRE rows loaded ahead.
template <int STAGE, class DP, int PRE = 2, class MK>
__device__ __forceinline__ void stream_window(const DevParams &p, const float *const *in,
                                              const float *const *frame, float *const *out,
                                              int xw, int y0, int y1, float dt, float T, int mdx,
                                              int mdy, int shx, int shy, float &cmax, bool &neg,
                                              MK &mk) {
  // ghost columns among the warp's 32 columns?
  const bool edge = (xw - kHalo <= 1) || (xw + kLanes - kHalo - 1 >= p.nx - 2);
  if (edge)
    stream_strip<STAGE, true, DP, PRE>(p, in, frame, out, xw, y0, y1, dt, T, mdx, mdy, shx, shy, cmax, neg, mk);
  else
    stream_strip<STAGE, false, DP, PRE>(p, in, frame, out, xw, y0, y1, dt, T, mdx, mdy, shx, shy, cmax, neg, mk);
}

// The CTA's CFL maximum into partials[slot], and the negative-eigenvalue
// flag into the control block.
template <int W = kWarps>
__device__ __forceinline__ void publish(const StepArgs &a, float cmax, bool neg, int slot, float *red,
                                        int *sh) {
  const int warp = threadIdx.x >> 5;
  for (int off = 16; off > 0; off >>= 1) cmax = nanmax(cmax, __shfl_xor_sync(0xffffffffu, cmax, off));
  if (threadIdx.x == 0) sh[0] = 0;
  __syncthreads();
  if (__any_sync(0xffffffffu, neg) && (threadIdx.x & 31) == 0) sh[0] = 1;
  if ((threadIdx.x & 31) == 0) red[warp] = cmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = red[0];
    for (int w = 1; w < W; ++w) m = nanmax(m, red[w]);
    a.partials[slot] = m;
    if (sh[0]) ((volatile Ctrl *)a.ctrl)->neg_flag = 1;
  }
}

// The step: STAGE < 0 is the full attempt with FMA division, followed by
// the fix-up and finalize launches (kStageRecord also writes the stage
// grids); STAGE 0..3 write that stage's grid to the debug buffers with IEEE
// division. W warps per CTA, built for MINB CTAs per SM (the register
// budget): the CTA shape (StepArgs::shape) only changes how the launch's
// warps are grouped and how many fit on an SM; every warp streams its own
// share either way.
template <int STAGE, int W, int PRE = 2>
__device__ __forceinline__ void step_body(const StepArgs &a) {
  __shared__ float red[W];
  __shared__ int sh[1];
  const Ctrl *ctl = a.ctrl;
  // Uniform early exit: the control block only changes between launches.
  if (STAGE < 0 && !attempt_active(ctl)) return;
  const float dt = __ldcg(&ctl->dt);
  const float T = __ldcg(&ctl->T);
  const int cur = __ldcg(&ctl->cur);
  const int mdx = __ldcg(&ctl->mdx), mdy = __ldcg(&ctl->mdy);
  int shx = 0, shy = 0;
  if (STAGE < 0) window_shift(a.p, T, dt, mdx, mdy, shx, shy);
  const float *in[3] = {a.state[cur][0], a.state[cur][1], a.state[cur][2]};
  float *out[STAGE == kStageRecord ? 12 : 3];
  if constexpr (STAGE == kStageRecord) {
    for (int f = 0; f < 3; ++f) out[f] = a.state[cur ^ 1][f];
    for (int k = 0; k < 9; ++k) out[3 + k] = a.stages[k];
  } else {
    for (int f = 0; f < 3; ++f) out[f] = (STAGE < 0) ? a.state[cur ^ 1][f] : a.dbg[f];
  }
  const float *frame[3] = {a.frame[0], a.frame[1], a.frame[2]};
  // Exact division for kStageExactDiv and for the adjoint's
  // stage-recording replays (DivNormal where quotients are normal in
  // practice, DivExact where they can be subnormal): the fix-up pass then
  // has no work in practice. Whether that beats FMA division with its
  // fix-up pass depends on the grid (see fv_set_division). The replays
  // gain 3% per backward step at 1024x1024.
  using DP = typename std::conditional<(STAGE == kStageRecord || STAGE == kStageExactDiv), PairNormalExact,
                                       typename std::conditional<(STAGE < 0), PairFma, PairIEEE>::type>::type;

  const int warp = threadIdx.x >> 5;
  const int ny = a.p.ny;
  float cmax = 0.0f;
  bool neg = false;
  // Each warp streams the (window, row) pairs of an equal share of the
  // launch's cost (ShareCost).
  const ShareCost sc(a.p.nx, ny);
  const long long C = sc.total();
  const long long G = (long long)a.nblocks * W;
  const long long g = (long long)blockIdx.x * W + warp;
  const long long s0 = sc.pos(g * C / G), s1 = sc.pos((g + 1) * C / G);
  for (long long pos = s0; pos < s1;) {
    const int win = (int)(pos / ny);
    const int y0 = (int)(pos - (long long)win * ny);
    const long long left = s1 - pos;
    const int y1 = (int)((long long)y0 + left < ny ? (long long)y0 + left : ny);
    const int xw = win * kWarpCols;
    if constexpr (STAGE < 0) {
      StepMarker mk{a, -1};
      stream_window<STAGE, DP, PRE>(a.p, in, frame, out, xw, y0, y1, dt, T, mdx, mdy, shx, shy, cmax, neg, mk);
    } else {
      NoMarker mk;
      stream_window<STAGE, DP, PRE>(a.p, in, frame, out, xw, y0, y1, dt, T, mdx, mdy, shx, shy, cmax, neg, mk);
    }
    pos += y1 - y0;
  }
  if (STAGE >= 0) return;
  publish<W>(a, cmax, neg, blockIdx.x, red, sh);
}

// PRE: input rows loaded ahead of the row in use (2 by default; the
// autotuner also times 1 and 3 in shapes 4 and 5).
template <int STAGE, int W = kWarps, int MINB = 4, int PRE = 2>
__global__ void __launch_bounds__(W * kLanes, MINB) step_kernel(StepArgs a) {
  step_body<STAGE, W, PRE>(a);
}

// One-warp CTAs with a register cap (__maxnreg__ cannot join
// __launch_bounds__): MAXREG registers a thread hold 65536 / (32 MAXREG)
// warps per SM.
template <int STAGE, int MAXREG>
__global__ void __maxnreg__(MAXREG) step_kernel_r(StepArgs a) {
  step_body<STAGE, 1>(a);
}

// The exact-division step kernel in the CTA shape `shape` (kStepShapes):
// warps per CTA and the CTAs per SM it is built for.
static void *exact_step_ptr(int shape, int &threads) {
  switch (shape) {
    case 1: threads = 2 * kLanes; return (void *)step_kernel<kStageExactDiv, 2, 8>;
    case 2: threads = kLanes; return (void *)step_kernel_r<kStageExactDiv, 128>;
    case 3: threads = kLanes; return (void *)step_kernel_r<kStageExactDiv, 112>;
    case 4: threads = kThreads; return (void *)step_kernel<kStageExactDiv, kWarps, 4, 1>;
    case 5: threads = kThreads; return (void *)step_kernel<kStageExactDiv, kWarps, 4, 3>;
    default: threads = kThreads; return (void *)step_kernel<kStageExactDiv, kWarps, 4>;
  }
}

static void launch_exact_step(const StepArgs &a, cudaStream_t st) {
  switch (a.shape) {
    case 1: step_kernel<kStageExactDiv, 2, 8><<<a.nblocks, 2 * kLanes, 0, st>>>(a); break;
    case 2: step_kernel_r<kStageExactDiv, 128><<<a.nblocks, kLanes, 0, st>>>(a); break;
    case 3: step_kernel_r<kStageExactDiv, 112><<<a.nblocks, kLanes, 0, st>>>(a); break;
    case 4: step_kernel<kStageExactDiv, kWarps, 4, 1><<<a.nblocks, kThreads, 0, st>>>(a); break;
    case 5: step_kernel<kStageExactDiv, kWarps, 4, 3><<<a.nblocks, kThreads, 0, st>>>(a); break;
    default: step_kernel<kStageExactDiv><<<a.nblocks, kThreads, 0, st>>>(a); break;
  }
}

// Recomputes the chunks the step launch marked, with exact division
// (DivExact), before finalize_kernel decides the attempt. Each chunk is split
// into items of kFixItemRows rows; warp w of the launch takes items w,
// w + W, w + 2W, ... (W warps). The rows of an item are a serial loop
// (plus the pipeline's warm-up and drain) that runs with few other warps on
// its SM, so its latency, not the work, sets the pass's duration: short
// items, no shared cursor, and all of an item's input rows loaded at once
// (kFixPrefetch) keep it small. An item whose operands fall outside
// DivExact's range (never in a physical state) is redone with IEEE
// division.
constexpr int kFixItemRows = 2;
constexpr int kFixPrefetch = kFixItemRows + 6;  // input rows y0-3 .. y1+2 of an item
static_assert(kFixRows % kFixItemRows == 0, "fix-up items must tile a chunk");

// STAGE: -1, or kStageRecord (the chunks' stage rows are rewritten too).
template <int STAGE>
__global__ void __launch_bounds__(kThreads, 2) fixup_kernel(StepArgs a) {
  __shared__ float red[kWarps];
  __shared__ int sh[1];
  // nothing marked (the usual case with exact division): one load and out;
  // the finalize launch then reads the step's partials only
  constexpr unsigned kItems = kFixRows / kFixItemRows;  // items per chunk
  const unsigned n = __ldcg(a.fix) * kItems;
  if (n == 0u) return;
  const Ctrl *ctl = a.ctrl;
  if (!attempt_active(ctl)) return;
  const float dt = __ldcg(&ctl->dt);
  const float T = __ldcg(&ctl->T);
  const int cur = __ldcg(&ctl->cur);
  const int mdx = __ldcg(&ctl->mdx), mdy = __ldcg(&ctl->mdy);
  int shx = 0, shy = 0;
  window_shift(a.p, T, dt, mdx, mdy, shx, shy);
  const float *in[3] = {a.state[cur][0], a.state[cur][1], a.state[cur][2]};
  float *out[STAGE == kStageRecord ? 12 : 3];
  for (int f = 0; f < 3; ++f) out[f] = a.state[cur ^ 1][f];
  if constexpr (STAGE == kStageRecord) {
    for (int k = 0; k < 9; ++k) out[3 + k] = a.stages[k];
  }
  const float *frame[3] = {a.frame[0], a.frame[1], a.frame[2]};
  const int lane = threadIdx.x & 31;
  const int ny = a.p.ny;
  const int cpw = fix_chunks_per_window(ny);
  const long long bitmap_words = fix_bitmap_words((long long)a.nstrips * kWarps, ny);
  const uint32_t *list = a.fix + 4 + bitmap_words;
  float cmax = 0.0f;
  bool neg = false;
  const unsigned nw = gridDim.x * kWarps;
  for (unsigned k = blockIdx.x * kWarps + (threadIdx.x >> 5); k < n; k += nw) {
    const unsigned id = __ldcg(list + k / kItems);
    const int window = (int)(id / (unsigned)cpw), c = (int)(id - (unsigned)window * (unsigned)cpw);
    if (lane == 0 && k % kItems == 0u) atomicAnd(a.fix + 4 + (id >> 5), ~(1u << (id & 31u)));
    const int xw = window * kWarpCols;
    const int y0 = c * kFixRows + (int)(k % kItems) * kFixItemRows;
    if (y0 >= ny) continue;
    const int y1 = min(ny, y0 + kFixItemRows);
    float cm = 0.0f;
    bool ng = false;
    FlagMarker fm;
    stream_window<STAGE, PairExact, kFixPrefetch>(a.p, in, frame, out, xw, y0, y1, dt, T, mdx, mdy, shx, shy, cm,
                                                  ng, fm);
    if (__any_sync(0xffffffffu, fm.flagged)) {
      cm = 0.0f;
      ng = false;
      NoMarker none;
      stream_window<STAGE, PairIEEE>(a.p, in, frame, out, xw, y0, y1, dt, T, mdx, mdy, shx, shy, cm, ng, none);
    }
    cmax = nanmax(cmax, cm);
    neg = neg || ng;
  }
  publish(a, cmax, neg, a.nblocks + blockIdx.x, red, sh);
}

// Decides the attempt after the step and fix-up launches: one CTA, so no
// CTA of the wide launches has to count who finishes last.
constexpr int kFinalizeThreads = 1024;  // one CTA; enough threads that the partials take one or two loads each

__global__ void __launch_bounds__(kFinalizeThreads) finalize_kernel(StepArgs a) {
  __shared__ float red[kFinalizeThreads / 32];
  if (attempt_active(a.ctrl)) finalize(a, red);
  if (a.host_ring && threadIdx.x == 0) {
    // the attempt's control block for the host, without a copy launch
    // (finalize's own writes came from this thread): the block, then the
    // slot's pass number, which the host polls
    volatile Ctrl *vc = a.ctrl;
    const long long q = vc->mirror_seq;
    vc->mirror_seq = q + 1;
    HostSlot *slot = a.host_ring + (q % kHostRing);
    const volatile uint32_t *src = reinterpret_cast<const volatile uint32_t *>(a.ctrl);
    volatile uint32_t *dst = reinterpret_cast<volatile uint32_t *>(&slot->c);
    for (int w = 0; w < int(sizeof(Ctrl) / 4); ++w) dst[w] = src[w];
    __threadfence_system();
    *reinterpret_cast<volatile uint32_t *>(&slot->gen) = uint32_t(q / kHostRing) + 1u;
    __threadfence_system();
  }
}

// The app's boundary hook (boundary(), apps/*/boundary.h) evaluated for
// frame cell k of one simulation: the four ghost rows first, then the left
// and right ghost column pairs.
__device__ __forceinline__ void frame_job(const DevParams &p, const float *const *state,
                                          float *const *frame, int k, float T, int mdx, int mdy) {
  const int nx = p.nx, ny = p.ny;
  const int rows = 4 * nx, cols = 2 * (ny - 4);
  int i, j;
  if (k < rows) {
    const int rr = k / nx;
    i = k - rr * nx;
    j = rr < 2 ? rr : ny - 4 + rr;
  } else if (k < rows + cols) {
    const int q = k - rows;
    j = 2 + (q >> 1);
    i = q & 1;
  } else {
    const int q = k - rows - cols;
    j = 2 + (q >> 1);
    i = nx - 2 + (q & 1);
  }
  const Ghost g{state[0], state[1], state[2], nx};
  float v1, v2, v3;
  ghost_value(p, g, i, j, T, mdx, mdy, v1, v2, v3);
  const int o = frame_index(i, j, nx, ny);
  frame[0][o] = v1;
  frame[1][o] = v2;
  frame[2][o] = v3;
}

__device__ __forceinline__ int frame_jobs(const DevParams &p) { return 4 * p.nx + 4 * (p.ny - 4); }

// Pre-pass of each attempt: the ghost frame of the current state. Skips
// like the step kernel does when the run is idle or stopped.
__global__ void __launch_bounds__(256) ghost_frame_kernel(StepArgs a, int check_ctrl) {
  const Ctrl *ctl = a.ctrl;
  if (check_ctrl && !attempt_active(ctl)) return;
  const float T = __ldcg(&ctl->T);
  const int cur = __ldcg(&ctl->cur);
  const int mdx = __ldcg(&ctl->mdx), mdy = __ldcg(&ctl->mdy);
  const int total = frame_jobs(a.p);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x)
    frame_job(a.p, a.state[cur], a.frame, k, T, mdx, mdy);
}

// ---------------------------------------------------------------- batches

// Ghost frames of every active simulation of a batch; blockIdx.y picks it.
__global__ void __launch_bounds__(256) batch_frame_kernel(BatchArgs b) {
  const BatchInst &I = b.inst[blockIdx.y];
  if (!attempt_active(I.ctrl)) return;
  const float T = __ldcg(&I.ctrl->T);
  const int cur = __ldcg(&I.ctrl->cur);
  const int mdx = __ldcg(&I.ctrl->mdx), mdy = __ldcg(&I.ctrl->mdy);
  const DevParams p = I.p;
  const int total = frame_jobs(p);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total; k += gridDim.x * blockDim.x)
    frame_job(p, I.state[cur], I.frame, k, T, mdx, mdy);
}

// Marks chunks of one warp window of batch instance `inst` (layout of
// BatchArgs::fix): as StepMarker, with the instance's chunk ids offset by
// its fix_base and the instance index stored beside each listed id.
struct BatchMarker {
  const BatchArgs &b;
  int inst;
  int last;
  __device__ __forceinline__ void mark(int xw, int lo, int hi) {
    const int c0 = max(lo / kFixRows, last + 1), c1 = hi / kFixRows;
    if ((threadIdx.x & 31) == 0) {
      const BatchInst &I = b.inst[inst];
      const long long cpw = fix_chunks_per_window(I.p.ny);
      const long long words = (b.fix_chunks + 31) / 32;
      uint32_t *fix = b.fix;
      for (int c = c0; c <= c1; ++c) {
        const unsigned long long id = (unsigned long long)I.fix_base + (unsigned long long)(xw / kWarpCols) * cpw + c;
        const unsigned bit = 1u << (id & 31u);
        if (!(atomicOr(fix + 4 + (id >> 5), bit) & bit)) {
          const unsigned slot = atomicAdd(fix, 1u);
          fix[4 + words + 2 * (long long)slot] = (uint32_t)id;
          fix[4 + words + 2 * (long long)slot + 1] = (uint32_t)inst;
        }
      }
    }
    last = max(last, c1);
  }
};

// One attempted step of every active simulation of a batch (uneven grid
// sizes and parameters) in one launch. CTAs share the batch's concatenated
// (simulation, strip, row) space evenly. A CTA contributes its rows of one
// simulation with an atomic max of their CFL (float bits of non-negative
// values order like unsigned integers, and NaN above all) and the
// negative-eigenvalue flag; rows whose FMA division may differ from IEEE
// division are marked for the batch fix-up launch, whose last CTA decides
// every simulation's attempt. No CTA waits on another. Three CTAs per SM:
// the simulation's buffers and parameters come from global memory, and at
// four the kernel would spill (measured: three is faster).
// STAGE -1: the attempt; kStageRecord: the attempt plus the stage grids of
// BatchInst::stages (the batched adjoint's replays).
template <int STAGE>
__global__ void __launch_bounds__(kThreads, 3) batch_step_kernel(BatchArgs b) {
  // Each warp streams the (simulation, window, row) triples of an equal
  // share of the batch's cost (the simulations' ShareCost totals, end to
  // end) and folds its CFL maximum and negative-eigenvalue flag into each
  // simulation it touched.
  const long long C = b.cost;
  const long long G = (long long)b.nblocks * kWarps;
  const long long g = (long long)blockIdx.x * kWarps + (threadIdx.x >> 5);
  const long long c0 = g * C / G, c1 = (g + 1) * C / G;
  int lo = 0, hi = b.n - 1;  // the simulation holding c0: last with cost_begin <= c0
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (b.inst[mid].cost_begin <= c0) lo = mid; else hi = mid - 1;
  }
  int k = lo;
  long long c = c0;
  while (c < c1 && k < b.n) {
    const BatchInst &I = b.inst[k];
    const long long kb = I.cost_begin, ke = kb + I.cost;
    const long long ce = c1 < ke ? c1 : ke;
    const ShareCost sc(I.p.nx, I.p.ny);
    // this simulation's window-rows [pos, seg_end)
    const long long pos = sc.pos(c - kb), seg_end = sc.pos(ce - kb);
    if (pos < seg_end && attempt_active(I.ctrl)) {
      const DevParams &p = I.p;  // read in place (L1), not copied into registers
      const Ctrl *ctl = I.ctrl;
      const float dt = __ldcg(&ctl->dt);
      const float T = __ldcg(&ctl->T);
      const int cur = __ldcg(&ctl->cur);
      const int mdx = __ldcg(&ctl->mdx), mdy = __ldcg(&ctl->mdy);
      int shx = 0, shy = 0;
      window_shift(p, T, dt, mdx, mdy, shx, shy);
      const float *in[3] = {I.state[cur][0], I.state[cur][1], I.state[cur][2]};
      float *out[STAGE == kStageRecord ? 12 : 3];
      for (int f = 0; f < 3; ++f) out[f] = I.state[cur ^ 1][f];
      if constexpr (STAGE == kStageRecord) {
        for (int k2 = 0; k2 < 9; ++k2) out[3 + k2] = I.stages[k2];
      }
      const float *frame[3] = {I.frame[0], I.frame[1], I.frame[2]};
      float cmax = 0.0f;
      bool neg = false;
      for (long long q = pos; q < seg_end;) {
        const int win = (int)(q / p.ny);
        const int y0 = (int)(q - (long long)win * p.ny);
        const long long left = seg_end - q;
        const int y1 = (int)((long long)y0 + left < p.ny ? (long long)y0 + left : p.ny);
        BatchMarker mk{b, k, -1};
        // exact division (no fix-up work in practice), as the single-grid
        // step kernel's default: measured faster for the batch than FMA
        // division with its fix-up pass
        stream_window<STAGE, PairNormalExact>(p, in, frame, out, win * kWarpCols, y0, y1, dt, T, mdx, mdy, shx, shy,
                                              cmax, neg, mk);
        q += y1 - y0;
      }
      for (int off = 16; off > 0; off >>= 1) cmax = nanmax(cmax, __shfl_xor_sync(0xffffffffu, cmax, off));
      // (with the subsonic solve of PairNormalExact neg stays false: a
      // negative eigenvalue flags its rows, and the batch fix-up pass
      // reports it)
      const bool wneg = __any_sync(0xffffffffu, neg);
      if ((threadIdx.x & 31) == 0) {
        atomicMax(b.cfl_bits + k, __float_as_uint(cmax));
        if (wneg) atomicExch(b.neg + k, 1);
      }
    }
    c = ce;
    ++k;
  }
}

// The batch's fix-up launch: recomputes the marked chunks of every
// simulation in items of kFixItemRows rows with exact division (as
// fixup_kernel) and folds their CFL and eigenvalue checks into the
// simulation's atomics; batch_finalize_kernel then decides.
template <int STAGE>
__global__ void __launch_bounds__(kThreads, 2) batch_fixup_kernel(BatchArgs b) {
  const int lane = threadIdx.x & 31;
  constexpr unsigned kItems = kFixRows / kFixItemRows;
  const long long words = (b.fix_chunks + 31) / 32;
  const uint32_t *list = b.fix + 4 + words;
  const unsigned n = __ldcg(b.fix) * kItems;
  if (n == 0u) return;
  const unsigned nw = gridDim.x * kWarps;
  for (unsigned k = blockIdx.x * kWarps + (threadIdx.x >> 5); k < n; k += nw) {
    const unsigned e = k / kItems;
    const unsigned id = __ldcg(list + 2 * (long long)e);
    const int inst = (int)__ldcg(list + 2 * (long long)e + 1);
    if (lane == 0 && k % kItems == 0u) atomicAnd(b.fix + 4 + (id >> 5), ~(1u << (id & 31u)));
    const BatchInst &I = b.inst[inst];
    const DevParams p = I.p;
    const int cpw = fix_chunks_per_window(p.ny);
    const long long local = (long long)id - I.fix_base;
    const int window = (int)(local / cpw), c = (int)(local - (long long)window * cpw);
    const int xw = window * kWarpCols;
    const int y0 = c * kFixRows + (int)(k % kItems) * kFixItemRows;
    if (y0 >= p.ny) continue;
    const int y1 = min(p.ny, y0 + kFixItemRows);
    const Ctrl *ctl = I.ctrl;
    const float dt = __ldcg(&ctl->dt);
    const float T = __ldcg(&ctl->T);
    const int cur = __ldcg(&ctl->cur);
    const int mdx = __ldcg(&ctl->mdx), mdy = __ldcg(&ctl->mdy);
    int shx = 0, shy = 0;
    window_shift(p, T, dt, mdx, mdy, shx, shy);
    const float *in[3] = {I.state[cur][0], I.state[cur][1], I.state[cur][2]};
    float *out[STAGE == kStageRecord ? 12 : 3];
    for (int f = 0; f < 3; ++f) out[f] = I.state[cur ^ 1][f];
    if constexpr (STAGE == kStageRecord) {
      for (int k2 = 0; k2 < 9; ++k2) out[3 + k2] = I.stages[k2];
    }
    const float *frame[3] = {I.frame[0], I.frame[1], I.frame[2]};
    float cm = 0.0f;
    bool ng = false;
    FlagMarker fm;
    stream_window<STAGE, PairExact, kFixPrefetch>(p, in, frame, out, xw, y0, y1, dt, T, mdx, mdy, shx, shy, cm, ng,
                                                  fm);
    if (__any_sync(0xffffffffu, fm.flagged)) {
      cm = 0.0f;
      ng = false;
      NoMarker none;
      stream_window<STAGE, PairIEEE>(p, in, frame, out, xw, y0, y1, dt, T, mdx, mdy, shx, shy, cm, ng, none);
    }
    for (int off = 16; off > 0; off >>= 1) cm = nanmax(cm, __shfl_xor_sync(0xffffffffu, cm, off));
    const bool wneg = __any_sync(0xffffffffu, ng);
    if (lane == 0) {
      atomicMax(b.cfl_bits + inst, __float_as_uint(cm));
      if (wneg) atomicExch(b.neg + inst, 1);
    }
  }
}

// Decides every active simulation's attempt after the batch step and fix-up
// launches, and clears the per-simulation accumulators; one CTA.
__global__ void __launch_bounds__(256) batch_finalize_kernel(BatchArgs b) {
  for (int k = threadIdx.x; k < b.n; k += blockDim.x) {
    const BatchInst &I = b.inst[k];
    if (!attempt_active(I.ctrl)) continue;
    const float cfl = __uint_as_float(atomicExch(b.cfl_bits + k, 0u));
    const int negative = atomicExch(b.neg + k, 0);
    decide((volatile Ctrl *)I.ctrl, I.p, cfl, negative != 0);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile uint32_t *fx = b.fix;
    fx[0] = 0u;
    fx[1] = 0u;
    __threadfence();
  }
}

static int launch_batch_impl(const BatchArgs &b, void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  dim3 fgrid((b.max_frame + 255) / 256, b.n);
  batch_frame_kernel<<<fgrid, 256, 0, st>>>(b);
  batch_step_kernel<-1><<<b.nblocks, kThreads, 0, st>>>(b);
  batch_fixup_kernel<-1><<<b.fix_blocks, kThreads, 0, st>>>(b);
  batch_finalize_kernel<<<1, 256, 0, st>>>(b);
  return (int)cudaGetLastError();
}

// The replays of the batched adjoint: no decision (the schedule is frozen);
// the caller resets the fix-up header and the accumulators before each one.
static int launch_batch_replay_impl(const BatchArgs &b, void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  dim3 fgrid((b.max_frame + 255) / 256, b.n);
  batch_frame_kernel<<<fgrid, 256, 0, st>>>(b);
  batch_step_kernel<kStageRecord><<<b.nblocks, kThreads, 0, st>>>(b);
  batch_fixup_kernel<kStageRecord><<<b.fix_blocks, kThreads, 0, st>>>(b);
  return (int)cudaGetLastError();
}

static int batch_occupancy() {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, (void *)batch_step_kernel<-1>, kThreads, 0) != cudaSuccess)
    return 1;
  return nb > 0 ? nb : 1;
}

template <int STAGE> static void *kernel_ptr() { return (void *)step_kernel<STAGE>; }

static int launch_impl(const StepArgs &a, int stage, void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  const int ftotal = 4 * a.p.nx + 4 * (a.p.ny - 4);
  if (stage != kLaunchStep && stage != kLaunchFixFinal)
    ghost_frame_kernel<<<(ftotal + 255) / 256, 256, 0, st>>>(a, stage < 0 ? 1 : 0);
  dim3 grid(a.nblocks), block(kThreads);
  switch (stage) {
    case kLaunchFrame: break;
    case kLaunchStep:
      if (a.div_exact)
        launch_exact_step(a, st);
      else
        step_kernel<-1><<<grid, block, 0, st>>>(a);
      break;
    case kLaunchFixFinal:
      fixup_kernel<-1><<<a.fix_blocks, block, 0, st>>>(a);
      finalize_kernel<<<1, kFinalizeThreads, 0, st>>>(a);
      break;
    case -1:
      if (a.div_exact)
        launch_exact_step(a, st);
      else
        step_kernel<-1><<<grid, block, 0, st>>>(a);
      fixup_kernel<-1><<<a.fix_blocks, block, 0, st>>>(a);
      finalize_kernel<<<1, kFinalizeThreads, 0, st>>>(a);
      break;
    case kStageRecord:
    case kStageReplay:
      step_kernel<kStageRecord><<<grid, block, 0, st>>>(a);
      fixup_kernel<kStageRecord><<<a.fix_blocks, block, 0, st>>>(a);
      if (stage == kStageRecord) finalize_kernel<<<1, kFinalizeThreads, 0, st>>>(a);
      break;
    case 0: step_kernel<0><<<grid, block, 0, st>>>(a); break;
    case 1: step_kernel<1><<<grid, block, 0, st>>>(a); break;
    case 2: step_kernel<2><<<grid, block, 0, st>>>(a); break;
    case 3: step_kernel<3><<<grid, block, 0, st>>>(a); break;
    default: return (int)cudaErrorInvalidValue;
  }
  return (int)cudaGetLastError();
}

static int occupancy(int stage) {
  int nb = 0;
  void *k = stage < 0 ? kernel_ptr<-1>() : kernel_ptr<3>();
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, kThreads, 0) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

// CTAs per SM of the exact-division step kernel in CTA shape `shape`.
static int shape_occupancy(int shape, int &warps) {
  int threads = 0, nb = 0;
  void *k = exact_step_ptr(shape, threads);
  warps = threads / kLanes;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, threads, 0) != cudaSuccess) return 1;
  return nb > 0 ? nb : 1;
}

}  // namespace exact_ns / fast_ns

#if FV_VARIANT_EXACT
int launch_batch_exact(const BatchArgs &a, void *stream) { return exact_ns::launch_batch_impl(a, stream); }
int launch_batch_replay_exact(const BatchArgs &a, void *stream) { return exact_ns::launch_batch_replay_impl(a, stream); }
int max_batch_blocks_per_sm_exact() { return exact_ns::batch_occupancy(); }
int launch_step_exact(const StepArgs &a, int warps, int stage, void *stream) {
  return warps == exact_ns::kWarps ? exact_ns::launch_impl(a, stage, stream)
                                   : (int)cudaErrorInvalidValue;
}
int max_blocks_per_sm_exact(int warps, int stage) {
  return warps == exact_ns::kWarps ? exact_ns::occupancy(stage) : 0;
}
int step_shape_blocks_per_sm_exact(int shape, int *warps) { return exact_ns::shape_occupancy(shape, *warps); }
#else
int launch_batch_fast(const BatchArgs &a, void *stream) { return fast_ns::launch_batch_impl(a, stream); }
int launch_batch_replay_fast(const BatchArgs &a, void *stream) { return fast_ns::launch_batch_replay_impl(a, stream); }
int max_batch_blocks_per_sm_fast() { return fast_ns::batch_occupancy(); }
int launch_step_fast(const StepArgs &a, int warps, int stage, void *stream) {
  return warps == fast_ns::kWarps ? fast_ns::launch_impl(a, stage, stream)
                                  : (int)cudaErrorInvalidValue;
}
int max_blocks_per_sm_fast(int warps, int stage) {
  return warps == fast_ns::kWarps ? fast_ns::occupancy(stage) : 0;
}
int step_shape_blocks_per_sm_fast(int shape, int *warps) { return fast_ns::shape_occupancy(shape, *warps); }
#endif

}  // namespace fvgb
