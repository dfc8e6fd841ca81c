// fv_internal.h -- types shared by the step kernels and the C-ABI host code.
#pragma once

#include <cstdint>

#include "../../include/fivonagi.h"

namespace fvgb {

// Output columns per warp: each warp's 32 lanes cover 32 consecutive
// columns, of which the middle 26 are written; the three columns on each
// side are the halo the x sweep (limiter + diffusion) needs.
constexpr int kLanes = 32;
constexpr int kHalo = 3;
constexpr int kWarpCols = kLanes - 2 * kHalo;  // 26

// Parameters the step kernel reads, already rounded to FP32 the way the
// reference's `static const DATATYPEV` definitions round them.
struct DevParams {
  int32_t app;
  int32_t nx, ny;
  int32_t cfl_even_only;
  int32_t hifu_width;     // static_cast<int>(ISPa/dy), apps/hifu-beam/boundary.h:78
  int32_t max_retries;
  float dx, dy;
  float beta, diffdelta, cflmax, cflwhish;
  float ampl, frec, ispw;  // ISPW = Num2*PI*FREC
  float ispa, ispf;
  float isprhoa, ispc, mdt;
  float cos_th, sin_th;    // cos/sin(ISPTHETA), evaluated once on the host
  float center, halfap, ramp;
};

// Device-resident time-stepping state of one simulation. The reference
// keeps dt, T, n, MDX, MDY and simError in device memory too
// (common/data_definitions.h:73-83) but copies them to the host every
// step; here only the last block of each step kernel touches them.
struct Ctrl {
  float dt;               // dt of the next attempt
  float T;                // simulation time
  float last_cfl;         // CFL of the last attempt
  float t_stop;           // attempts are no-ops once T >= t_stop
  int32_t n;              // accepted steps since the state was set
  int32_t cur;            // state buffer holding the current state (0/1)
  int32_t status;         // sticky fv_status of the device run
  int32_t neg_flag;       // set by any block that met tmp3 < 0 this attempt
  int32_t sim_error;      // 1 after a rejected attempt (update_dt's branch)
  int32_t consecutive_rejects;
  int32_t mdx, mdy;
  int64_t remaining;      // accepted steps still to take; 0 = idle
  int64_t accepted;       // counters since the last fv_run/fv_sync reset
  int64_t rejected;
  uint32_t blocks_done;   // last-block-done counter of the current attempt
  uint32_t pad;
};

struct StepArgs {
  DevParams p;
  float *state[2][3];     // two full state buffers (u1, u2, u3 each)
  Ctrl *ctrl;
  float *partials;        // one CFL maximum per CTA
  float *dbg[3];          // debug-stage output (stage kernels only)
  int32_t nstrips;        // column strips of width kWarpCols * warps
  int32_t nblocks;        // CTAs of the launch
  int64_t work;           // nstrips * ny: strip-rows to share among the CTAs
};

// Launch configuration picked for a grid size.
struct LaunchCfg {
  int warps;              // warps per CTA
  int blocks;             // CTAs per launch
};

// Launchers, one translation unit per arithmetic variant:
// exact = no FMA contraction (bit-identical to the oracle), fast = FMA.
int launch_step_exact(const StepArgs &a, int warps, int stage, void *stream);
int launch_step_fast(const StepArgs &a, int warps, int stage, void *stream);
int max_blocks_per_sm_exact(int warps, int stage);
int max_blocks_per_sm_fast(int warps, int stage);

}  // namespace fvgb
