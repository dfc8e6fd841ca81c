// fv_step.cu -- the fused time-step kernel for sm_103a.
//
// One launch performs one attempted step of the reference's loop body
// (common/main.cu:310-635):
//   boundary (app hook)  ->  y sweep  ->  x sweep  ->  CFL max  ->
//   [accepted] diffusion, T += dt, n += 1  ->  dt update.
// The reference runs this as ~34 kernel launches that pass 19 scratch
// grids through global memory (~750 B per cell-update) and 7 blocking
// device-to-host copies. Here every intermediate lives in registers:
//
//  * Each warp owns a strip of 32 consecutive columns and streams up the
//    grid one row per iteration. Lanes 3..28 produce output; the three
//    lanes on each side are the x-halo the limiter and diffusion need.
//  * y sweep: a lane keeps the last rows of its own column (state, waves,
//    first-order sums, correction fluxes) in registers, so each y interface
//    is solved once per strip and each cell is updated two rows behind the
//    row being loaded.
//  * x sweep: once a row of y-updated cells is ready, neighbouring columns
//    are neighbouring lanes; the Riemann inputs, waves, dot products,
//    fluctuations and correction fluxes move between lanes with warp
//    shuffles.
//  * diffusion (source): runs one row behind the x sweep, on registers.
//  * CFL: each lane keeps a running maximum over its output cells; warp
//    shuffles and a CTA reduction produce one value per CTA, and the last
//    CTA to finish (atomic counter) reduces those, accepts or rejects the
//    step, and updates dt, T, n and the current-buffer index in device
//    memory. A rejected step leaves the input buffer current, so the retry
//    starts from the pre-step state.
//
// Work distribution: CTAs are persistent over a balanced share of the
// (column strip, row) space, so every CTA streams the same number of rows;
// a share may span two strips.
//
// This file is compiled twice: FV_VARIANT_EXACT with --fmad=false (the
// oracle's evaluation, bit for bit) and the fast variant with FMA
// contraction.
#include <cuda_runtime.h>

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

__device__ __forceinline__ void store3(float *const *out, int o, const Cell3 &v) {
  out[0][o] = v.u1;
  out[1][o] = v.u2;
  out[2][o] = v.u3;
}

// Stream one warp's 32 columns over output rows [y0, y1) of a strip.
//
// Iteration r loads row r and runs three chains that do not depend on each
// other within the iteration, so their instructions interleave:
//   Y: y interface r, correction flux at r-1, y update of row r-2 (S1);
//   X: x sweep of row r-3 (S1 of the previous iteration -> S2) and the CFL
//      of its cells;
//   D: diffusion of row r-5 from S2 of rows r-6, r-5, r-4 (source).
// Warm-up and drain iterations compute on rows outside [y0-1, y1] and
// discard the results (stores and flags are predicated), which keeps the
// loop body free of branches.
// EDGE: the warp's columns or rows include ghost cells, whose boundary-hook
// values replace the loaded ones.
// STAGE < 0: full step into `out`; STAGE 0..3: that stage's grid into `out`.
template <int STAGE, bool EDGE>
__device__ __forceinline__ void stream_strip(const DevParams &p, const float *const *in,
                                             float *const *out, int xw, int y0, int y1,
                                             float dt, float T, int mdx, int mdy, float &cmax,
                                             bool &neg) {
  const int lane = threadIdx.x & (kLanes - 1);
  const int nx = p.nx, ny = p.ny;
  const int i = xw - kHalo + lane;
  const bool col_ok = (i >= 0) && (i < nx);
  const bool out_lane = col_ok && lane >= kHalo && lane < kLanes - kHalo;
  const bool col_int = (i >= 2) && (i <= nx - 3);
  const float dtx = dt / p.dx;
  const float dty = dt / p.dy;
  const float ddtx2 = p.diffdelta * dt / (p.dx * p.dx);
  const float ddty2 = p.diffdelta * dt / (p.dy * p.dy);
  const float two_bm1 = 2.0f * (p.beta - 1.0f);
  const Ghost g{in[0], in[1], in[2], nx};
  const int ci = col_ok ? i : 0;
  const bool even_only = p.cfl_even_only != 0;

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

  auto load_raw = [&](int r, Cell3 &v) {
    if (col_ok && r >= 0 && r < ny) {
      const int o = ci + r * nx;
      v.u1 = __ldg(in[0] + o);
      v.u2 = __ldg(in[1] + o);
      v.u3 = __ldg(in[2] + o);
    } else {
      v = Cell3{0.f, 0.f, 0.f};
    }
  };
  Cell3 pf0, pf1;  // prefetched raw rows r, r+1
  load_raw(y0 - 3, pf0);
  load_raw(y0 - 2, pf1);

  const int r_end = y1 + 4;
  for (int r = y0 - 3; r <= r_end; ++r) {
    Cell3 u = pf0;
    pf0 = pf1;
    if (r + 2 <= y1 + 2) load_raw(r + 2, pf1);
    if (EDGE) {
      if (col_ok && r >= 0 && r < ny && is_ghost(p, i, r)) ghost_value(p, g, i, r, T, mdx, mdy, u.u1, u.u2, u.u3);
    }

    // ======== Y chain: interface r, flux r-1, update of row r-2
    const float rho = u.u1 + 1.0f;
    const float vx = u.u2 / rho;
    const float vy = u.u3 / rho;
    WaveN w;
    Fluct f;
    float cy = 0.0f;
    const bool oky = riemann(rho, u.u3, u.u2, vy, vx, s0_m1.u1 + 1.0f, s0_m1.u3, s0_m1.u2, vy_m1,
                             vx_m1, two_bm1, dty, cy, w, f);
    cy = (r <= 0) ? 0.0f : cy;  // cfl = 0 on j == 0 (apps/na/fv.h:212-215)
    neg = neg || (!oky && out_lane && r >= y0 && r < y1 && r >= 1);
    const float fn1 = ap1 + f.am1, fn2 = ap2 + f.am2, fn3 = ap3 + f.am3;
    const Dots dr = wave_dots(w_m1, w);
    float fan1, fan2, fan3;
    correction(w_m1, dl_m1, dr, dty, fan1, fan2, fan3);
    const int cyr = r - 2;  // row of the y update
    Cell3 s1 = s0_m2;
    {
      // local components: 1 -> u1, 2 (normal) -> u3, 3 (transverse) -> u2
      const float m1 = s0_m2.u1 - dty * fo1;
      const float m3 = s0_m2.u3 - dty * fo2;
      const float m2 = s0_m2.u2 - dty * fo3;
      const bool in_y = col_int && cyr >= 2 && cyr <= ny - 3;
      s1.u1 = in_y ? m1 - dty * (fan1 - fa1) : s0_m2.u1;
      s1.u3 = in_y ? m3 - dty * (fan2 - fa2) : s0_m2.u3;
      s1.u2 = in_y ? m2 - dty * (fan3 - fa3) : s0_m2.u2;
    }
    if (STAGE == FV_STAGE_BOUNDARY || STAGE == FV_STAGE_SWEEP_Y) {
      if (out_lane && cyr >= y0 && cyr < y1) store3(out, i + cyr * nx, STAGE == FV_STAGE_BOUNDARY ? s0_m2 : s1);
    }

    // ======== X chain: row r-3; normal = u2, transverse = u3
    const int cxr = r - 3;
    const float rho1 = s1_m3.u1 + 1.0f;
    const float vn1 = s1_m3.u2 / rho1;
    const float vt1 = s1_m3.u3 / rho1;
    const float rho1m = shup(rho1), u2m = shup(s1_m3.u2), u3m = shup(s1_m3.u3);
    const float vn1m = shup(vn1), vt1m = shup(vt1);
    WaveN wx;
    Fluct fx;
    float cx = cy_m3;  // the x kernel starts from the cell's y value (fv.h:57)
    const bool okx = riemann(rho1, s1_m3.u2, s1_m3.u3, vn1, vt1, rho1m, u2m, u3m, vn1m, vt1m,
                             two_bm1, dtx, cx, wx, fx);
    const bool own_x = out_lane && cxr >= y0 && cxr < y1;
    neg = neg || (!okx && own_x && i >= 1);
    WaveN wn;
    wn.w11 = shdn(wx.w11); wn.w21 = shdn(wx.w21); wn.w31 = shdn(wx.w31);
    wn.w12 = shdn(wx.w12); wn.w22 = shdn(wx.w22); wn.w32 = shdn(wx.w32);
    wn.w33 = shdn(wx.w33);
    const Dots drx = wave_dots(wx, wn);
    Dots dlx;
    dlx.d1 = shup(drx.d1); dlx.d2 = shup(drx.d2); dlx.d3 = shup(drx.d3);
    float fx1, fx2, fx3;
    correction(wx, dlx, drx, dtx, fx1, fx2, fx3);
    const float amn1 = shdn(fx.am1), amn2 = shdn(fx.am2), amn3 = shdn(fx.am3);
    const float fxn1 = shdn(fx1), fxn2 = shdn(fx2), fxn3 = shdn(fx3);
    Cell3 s2;
    {
      const bool in_x = col_int && cxr >= 2 && cxr <= ny - 3;
      const float m1 = s1_m3.u1 - dtx * (fx.ap1 + amn1);
      const float m2 = s1_m3.u2 - dtx * (fx.ap2 + amn2);
      const float m3 = s1_m3.u3 - dtx * (fx.ap3 + amn3);
      s2.u1 = in_x ? m1 - dtx * (fxn1 - fx1) : s1_m3.u1;
      s2.u2 = in_x ? m2 - dtx * (fxn2 - fx2) : s1_m3.u2;
      s2.u3 = in_x ? m3 - dtx * (fxn3 - fx3) : s1_m3.u3;
    }
    const float rho2 = s2.u1 + 1.0f;
    const float vx2 = s2.u2 / rho2;
    const float vy2 = s2.u3 / rho2;
    {
      // CFL of cell (i, r-3): its y and x interfaces; 0 on i == 0
      const float cell = (i == 0) ? 0.0f : cx;
      const bool counted = own_x && (!even_only || ((i + cxr * nx) & 1) == 0);
      cmax = counted ? nanmax(cmax, cell) : cmax;
    }
    if (STAGE == FV_STAGE_SWEEP_X) {
      if (own_x) store3(out, i + cxr * nx, s2);
    }

    // ======== D chain: diffusion of row r-5 (apps/na/source.h:22-104)
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
      if (out_lane && cdr >= y0 && cdr < y1) store3(out, i + cdr * nx, o3);
    }

    // ======== rotate
    s0_m2 = s0_m1;
    s0_m1 = u;
    vx_m1 = vx;
    vy_m1 = vy;
    w_m1 = w;
    dl_m1 = dr;
    ap1 = f.ap1; ap2 = f.ap2; ap3 = f.ap3;
    fo1 = fn1; fo2 = fn2; fo3 = fn3;
    fa1 = fan1; fa2 = fan2; fa3 = fan3;
    cy_m3 = cy_m2;
    cy_m2 = cy_m1;
    cy_m1 = cy;
    s1_m3 = s1;
    s2_m5 = s2_m4;
    s2_m4 = s2;
    vx2_m6 = vx2_m5; vy2_m6 = vy2_m5;
    vx2_m5 = vx2_m4; vy2_m5 = vy2_m4;
    vx2_m4 = vx2; vy2_m4 = vy2;
  }
}

// Reduce the partial CFL maxima, accept or reject, update dt/T/n/cur.
// Runs on the last CTA of the launch (all its threads).
__device__ void finalize(const StepArgs &a, float *red) {
  Ctrl *ctl = a.ctrl;
  float m = 0.0f;
  for (int b = threadIdx.x; b < a.nblocks; b += blockDim.x) m = nanmax(m, __ldcg(a.partials + b));
  for (int off = 16; off > 0; off >>= 1) m = nanmax(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x != 0) return;
  float cfl = 0.0f;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) cfl = nanmax(cfl, red[w]);
  volatile Ctrl *vc = ctl;
  const float dt = vc->dt;
  vc->last_cfl = cfl;
  if (vc->neg_flag) {
    vc->status = FV_NEGATIVE_EIGENVALUE;
    vc->neg_flag = 0;
    vc->blocks_done = 0;
    return;
  }
  int sim_error = 0;
  if (cfl < a.p.cflmax) {  // reduceCFL2, common/main.cu:200-212
    vc->T = vc->T + dt;    // update_T, main.cu:232-238
    vc->n = vc->n + 1;
    vc->cur = vc->cur ^ 1;
    vc->remaining = vc->remaining - 1;
    vc->accepted = vc->accepted + 1;
    vc->consecutive_rejects = 0;
  } else {
    sim_error = 1;
    vc->rejected = vc->rejected + 1;
    const int cr = vc->consecutive_rejects + 1;
    vc->consecutive_rejects = cr;
    if (cr >= a.p.max_retries) vc->status = FV_DT_TOO_LARGE;
  }
  vc->sim_error = sim_error;
  // update_dt, main.cu:214-230 (the 0.9 is a double literal)
  const float new_dt = dt * a.p.cflwhish / cfl;
  if (sim_error == 1 && (double)new_dt > (double)dt * 0.9)
    vc->dt = (float)((double)dt * 0.9);
  else
    vc->dt = new_dt;
  __threadfence();
  vc->blocks_done = 0;
}

template <int STAGE>
__global__ void __launch_bounds__(kThreads, 4) step_kernel(StepArgs a) {
  __shared__ float red[kWarps];
  __shared__ int neg_any;
  __shared__ int is_last;
  const Ctrl *ctl = a.ctrl;
  // Uniform early exit: the control block only changes between launches.
  if (STAGE < 0) {
    const int status = __ldcg(&ctl->status);
    const long long remaining = __ldcg((const long long *)&ctl->remaining);
    const float T0 = __ldcg(&ctl->T), ts = __ldcg(&ctl->t_stop);
    if (status != 0 || remaining <= 0 || !(T0 < ts)) return;
  }
  if (threadIdx.x == 0) neg_any = 0;
  __syncthreads();
  const float dt = __ldcg(&ctl->dt);
  const float T = __ldcg(&ctl->T);
  const int cur = __ldcg(&ctl->cur);
  const int mdx = __ldcg(&ctl->mdx), mdy = __ldcg(&ctl->mdy);
  const float *in[3] = {a.state[cur][0], a.state[cur][1], a.state[cur][2]};
  float *out[3];
  for (int f = 0; f < 3; ++f) out[f] = (STAGE < 0) ? a.state[cur ^ 1][f] : a.dbg[f];

  const int warp = threadIdx.x >> 5;
  const int ny = a.p.ny;
  float cmax = 0.0f;
  bool neg = false;
  const long long W = a.work;
  const long long b = blockIdx.x;
  const long long s0 = b * W / a.nblocks, s1 = (b + 1) * W / a.nblocks;
  for (long long pos = s0; pos < s1;) {
    const int strip = (int)(pos / ny);
    const int y0 = (int)(pos - (long long)strip * ny);
    const long long left = s1 - pos;
    const int y1 = (int)((long long)y0 + left < ny ? (long long)y0 + left : ny);
    const int xw = strip * kStripCols + warp * kWarpCols;
    if (xw < a.p.nx) {
      // ghost cells among the loaded rows [y0-3, y1+2] or the warp's columns?
      const bool edge = (y0 - 3 <= 1) || (y1 + 2 >= ny - 2) || (xw - kHalo <= 1) ||
                        (xw + kLanes - kHalo - 1 >= a.p.nx - 2);
      if (edge)
        stream_strip<STAGE, true>(a.p, in, out, xw, y0, y1, dt, T, mdx, mdy, cmax, neg);
      else
        stream_strip<STAGE, false>(a.p, in, out, xw, y0, y1, dt, T, mdx, mdy, cmax, neg);
    }
    pos += y1 - y0;
  }
  if (STAGE >= 0) return;

  // CTA maximum of the CFL, and the negative-eigenvalue flag
  for (int off = 16; off > 0; off >>= 1) cmax = nanmax(cmax, __shfl_xor_sync(0xffffffffu, cmax, off));
  if (__any_sync(0xffffffffu, neg) && (threadIdx.x & 31) == 0) neg_any = 1;
  if ((threadIdx.x & 31) == 0) red[warp] = cmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = red[0];
    for (int w = 1; w < kWarps; ++w) m = nanmax(m, red[w]);
    a.partials[blockIdx.x] = m;
    if (neg_any) ((volatile Ctrl *)a.ctrl)->neg_flag = 1;
    __threadfence();
    const unsigned prev = atomicAdd(&a.ctrl->blocks_done, 1u);
    is_last = (prev == (unsigned)(a.nblocks - 1));
  }
  __syncthreads();
  if (is_last) {
    __threadfence();
    finalize(a, red);
  }
}

template <int STAGE> static void *kernel_ptr() { return (void *)step_kernel<STAGE>; }

static int launch_impl(const StepArgs &a, int stage, void *stream) {
  cudaStream_t st = (cudaStream_t)stream;
  dim3 grid(a.nblocks), block(kThreads);
  switch (stage) {
    case -1: step_kernel<-1><<<grid, block, 0, st>>>(a); break;
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

}  // namespace exact_ns / fast_ns

#if FV_VARIANT_EXACT
int launch_step_exact(const StepArgs &a, int warps, int stage, void *stream) {
  return warps == exact_ns::kWarps ? exact_ns::launch_impl(a, stage, stream)
                                   : (int)cudaErrorInvalidValue;
}
int max_blocks_per_sm_exact(int warps, int stage) {
  return warps == exact_ns::kWarps ? exact_ns::occupancy(stage) : 0;
}
#else
int launch_step_fast(const StepArgs &a, int warps, int stage, void *stream) {
  return warps == fast_ns::kWarps ? fast_ns::launch_impl(a, stage, stream)
                                  : (int)cudaErrorInvalidValue;
}
int max_blocks_per_sm_fast(int warps, int stage) {
  return warps == fast_ns::kWarps ? fast_ns::occupancy(stage) : 0;
}
#endif

}  // namespace fvgb
