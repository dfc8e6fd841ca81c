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

#ifdef __CUDACC__
#define FV_HD __host__ __device__ __forceinline__
#else
#define FV_HD inline
#endif

// A grid's work in cost order, by which the step kernels give every warp
// an equal share of (window, row) pairs: window w costs kShareStart (the
// loop's warm-up and drain, run again by the warp that enters it) plus ny
// rows of kShareRow, or of kShareEdgeRow when it has ghost columns (w == 0
// and w >= w_hi1). Measured on the focused beam, 4096x2048, against equal
// rows per warp: 4.1% shorter attempts; edge rows weighted 1.25 or 1.75,
// or starts of 2 rows, were slower.
constexpr long long kShareRow = 16;
constexpr long long kShareEdgeRow = 24;
constexpr long long kShareStart = 6 * kShareRow;

struct ShareCost {
  long long ny, windows, w_hi1;  // w_hi1: first ghost-column window past 0
  FV_HD ShareCost(long long nx, long long ny_) : ny(ny_) {
    windows = (nx + kWarpCols - 1) / kWarpCols;
    // window w has ghost columns when its 32 columns reach column 1 or
    // column nx-2 (the step kernel's edge test): w == 0, or 26w + 28 >= nx - 2
    const long long reach = nx - 2 - (kLanes - kHalo - 1);  // 26w >= reach
    const long long w_hi = reach > 0 ? (reach + kWarpCols - 1) / kWarpCols : 0;
    w_hi1 = w_hi > 1 ? w_hi : 1;
  }
  // cost of windows [0, w)
  FV_HD long long prefix(long long w) const {
    const long long edges = (w > 0 ? 1 : 0) + (w > w_hi1 ? w - w_hi1 : 0);
    return w * (kShareStart + ny * kShareRow) + ny * (kShareEdgeRow - kShareRow) * edges;
  }
  FV_HD long long total() const { return prefix(windows); }
  // (window * ny + row) of the first row at or after cost c; monotone in c,
  // so consecutive cost ranges give consecutive row ranges
  FV_HD long long pos(long long c) const {
    if (c >= total()) return windows * ny;
    long long w = c / (kShareStart + ny * kShareRow);  // >= the window of c
    if (w >= windows) w = windows - 1;
    while (w > 0 && prefix(w) > c) --w;                // at most the edge windows' extra cost
    while (w + 1 < windows && prefix(w + 1) <= c) ++w;
    const long long o = c - prefix(w) - kShareStart;
    const long long u = (w == 0 || w >= w_hi1) ? kShareEdgeRow : kShareRow;
    const long long r = o <= 0 ? 0 : (o + u - 1) / u;
    return w * ny + (r < ny ? r : ny);
  }
};


// Parameters the step kernel reads, already rounded to FP32 the way the
// reference's `static const DATATYPEV` definitions round them.
struct DevParams {
  int32_t app;
  int32_t nx, ny;
  int32_t cfl_even_only;
  int32_t hifu_width;     // static_cast<int>(ISPa/dy), apps/hifu-beam/boundary.h:78
  int32_t max_retries;
  int32_t moving_domain;
  float mdvx, mdvy;       // MDVX, MDVY (mdt below)
  float dx, dy;
  float beta, diffdelta, cflmax, cflwhish;
  float ampl, frec, ispw;  // ISPW = Num2*PI*FREC
  float ispa, ispf;
  float isprhoa, ispc, mdt;
  float cos_th, sin_th;    // cos/sin(ISPTHETA), evaluated once on the host
  float center, halfap, ramp;
  // phased array: elements of arr_elem rows from row arr_j0; weights holds
  // the amplitudes [0, nelem) then the phases [nelem, 2 nelem) (device)
  int32_t nelem, arr_j0, arr_elem, pad1;
  const float *weights;
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
  uint32_t blocks_done;   // unused (zero)
  int32_t last_accepted;  // the last decided attempt was accepted (1) or rejected (0)
  int64_t mirror_seq;     // attempts whose control block went to the host ring
};

// One slot of the host ring that finalize_kernel writes when StepArgs'
// host_ring is set: the attempt's control block, then its pass over the
// ring (the host waits until `gen` reaches the pass it expects).
constexpr int kHostRing = 64;
struct HostSlot {
  Ctrl c;
  uint32_t gen;
  uint32_t pad;
};
static_assert(sizeof(Ctrl) % 4 == 0, "the finalize launch copies the control block in words");

// Ghost frame: the boundary hook's values of the ghost cells (the two
// outermost rows and columns), written by a small pre-pass each attempt and
// read by the step kernel in place of the state's own ghost cells. Layout:
// rows j = 0, 1, ny-2, ny-1 (corners included) as four rows of nx, then the
// left and right column pairs as [j][2] blocks of ny each.
FV_HD int frame_cells(int nx, int ny) { return 4 * nx + 4 * ny; }
FV_HD int frame_index(int i, int j, int nx, int ny) {
  if (j <= 1) return j * nx + i;
  if (j >= ny - 2) return (j - ny + 4) * nx + i;
  if (i <= 1) return 4 * nx + 2 * j + i;
  return 4 * nx + 2 * ny + 2 * j + (i - nx + 2);
}

// Fix-up bookkeeping of the step kernel. The step kernel divides with
// FMA-based division and marks the rows whose results may differ from IEEE
// division; a second kernel recomputes those rows with exact division. Rows
// are marked in chunks of kFixRows rows of one warp window (the 26 output
// columns of one warp of a strip). Layout of the uint32 scratch:
//   [0] number of listed chunks   [1], [2], [3] unused
//   bitmap of marked chunks (one bit per chunk), then the list of marked
//   chunk ids (window * chunks_per_window + chunk), one per marked chunk.
constexpr int kFixRows = 8;

// A full attempt (DivFma step, fix-up, finalize) that also writes the
// boundary-applied state, the state after the y sweep and the state after
// the x sweep (StepArgs::stages), exact in every row: the fix-up pass
// rewrites the stage rows of the chunks it recomputes. The adjoint's
// segment replay records its linearisation points this way.
constexpr int kStageRecord = -2;
// The parts of an attempt (stage -1), for launching one at a time with
// events between them (fv_time_attempts): the ghost-frame pre-pass, the
// step kernel, and the fix-up and finalize launches.
constexpr int kLaunchFrame = -3, kLaunchStep = -4, kLaunchFixFinal = -5;
// A full attempt whose step kernel divides exactly (DivExact) instead of
// with FMA division: the fix-up pass then meets only operands out of
// range. Chosen by StepArgs::div_exact.
constexpr int kStageExactDiv = -6;
// kStageRecord without the finalize launch: the adjoint's replays follow a
// frozen schedule, so there is nothing to decide. Their caller resets the
// fix-up scratch's header before each one and checks the eigenvalue flag.
constexpr int kStageReplay = -7;
FV_HD int fix_chunks_per_window(int ny) {
  return (ny + kFixRows - 1) / kFixRows;
}
FV_HD long long fix_bitmap_words(long long windows, int ny) {
  return (windows * fix_chunks_per_window(ny) + 31) / 32;
}
// uint32 words of the whole fix-up scratch for `windows` warp windows
FV_HD long long fix_scratch_words(long long windows, int ny) {
  return 4 + fix_bitmap_words(windows, ny) + windows * fix_chunks_per_window(ny);
}

struct StepArgs {
  DevParams p;
  float *state[2][3];     // two full state buffers (u1, u2, u3 each)
  float *frame[3];        // ghost frame (see frame_index)
  Ctrl *ctrl;
  float *partials;        // one CFL maximum per CTA of the step launch, then
                          // one per CTA of the fix-up launch
  float *dbg[3];          // debug-stage output (stage kernels 0..3 only)
  float *stages[9];       // kStageRecord output: boundary-applied state, y-swept, x-swept
  uint32_t *fix;          // fix-up scratch, zero between attempts (see above)
  int32_t nstrips;        // column strips of width kWarpCols * warps
  int32_t nblocks;        // CTAs of the launch
  int64_t work;           // nstrips * ny: strip-rows (sizes the default launch)
  int32_t fix_blocks;     // CTAs of the fix-up launch
  int32_t div_exact;      // attempts (-1, kLaunchStep) run the step kernel with exact
                          // division (kStageExactDiv) instead of FMA division
  int32_t shape;          // CTA shape of the exact-division step kernel (kStepShapes)
  HostSlot *host_ring;    // or nullptr: the finalize launch also copies the control
                          // block, decided or not, to slot mirror_seq % kHostRing
                          // of this ring (mapped pinned host memory)
};

// CTA shapes of the exact-division step kernel: {warps per CTA, CTAs per
// SM it is built for, rows loaded ahead}. 0: 4 x 4 (16 warps per SM), 1:
// 2 x 8, 2: 1 x 16, 3: 1 x 18 (18 warps per SM, at most 112 registers a
// thread), all loading 2 rows ahead; 4 and 5: 4 x 4 loading 1 and 3 rows
// ahead. The FMA-division and stage-recording kernels run shape 0.
constexpr int kStepShapes = 6;

// One simulation of a batch: its parameters, buffers and control block,
// and where its window-rows start in the batch's concatenated work.
struct BatchInst {
  DevParams p;
  float *state[2][3];
  float *frame[3];
  Ctrl *ctrl;
  int64_t work_begin;     // first window-row of this instance in the batch
  int64_t work;           // windows * ny (windows of kWarpCols output columns)
  int64_t cost_begin;     // first cost unit of this instance in the batch
  int64_t cost;           // ShareCost(nx, ny).total()
  int64_t fix_base;       // first chunk id of this instance in the fix-up scratch
  float *stages[9];       // the record launches' stage grids (batched adjoint replays)
};

// The batch's fix-up scratch has the layout of a single simulation's
// (fv_internal.h's fix_* helpers) over the concatenated chunk ids of all
// instances, except that each list entry is a pair (chunk id, instance).
struct BatchArgs {
  const BatchInst *inst;  // device array of n instances
  uint32_t *cfl_bits;     // per instance: running max CFL as float bits (non-negative)
  int32_t *neg;           // per instance: a Riemann solve met tmp3 < 0
  uint32_t *fix;          // fix-up scratch, zero between attempts
  int32_t n;
  int32_t nblocks;
  int64_t work;           // total window-rows
  int64_t cost;           // total cost units (ShareCost)
  int64_t fix_chunks;     // total chunks over all instances
  int32_t max_frame;      // largest frame pre-pass work of an instance
  int32_t fix_blocks;     // CTAs of the fix-up launch
};

// Launchers, one translation unit per arithmetic variant:
// exact = no FMA contraction (bit-identical to the oracle), fast = FMA.
int launch_step_exact(const StepArgs &a, int warps, int stage, void *stream);
int launch_step_fast(const StepArgs &a, int warps, int stage, void *stream);
int max_blocks_per_sm_exact(int warps, int stage);
int max_blocks_per_sm_fast(int warps, int stage);
// CTAs per SM of the exact-division step kernel in a CTA shape, and its warps per CTA
int step_shape_blocks_per_sm_exact(int shape, int *warps);
int step_shape_blocks_per_sm_fast(int shape, int *warps);
int launch_batch_exact(const BatchArgs &a, void *stream);
int launch_batch_fast(const BatchArgs &a, void *stream);
// Stage-recording attempts of every instance without the finalize launch
// (the batched adjoint's replays on frozen schedules: ghost frame, step
// with the stage grids of BatchInst::stages, fix-up).
int launch_batch_replay_exact(const BatchArgs &a, void *stream);
int launch_batch_replay_fast(const BatchArgs &a, void *stream);
int max_batch_blocks_per_sm_exact();
int max_batch_blocks_per_sm_fast();

// Shared by the C-ABI translation units (fv_api.cu).
DevParams dev_params_of(const fv_params &p);
fv_status validate_params(const fv_params *p);
long long default_blocks(int max_resident, long long work, int cta_warps);  // CTAs of a step launch
int default_div_exact(const fv_params &p);                     // step kernel's division
void init_state_host(const fv_params &p, float *u1, float *u2, float *u3);
void set_last_error(const char *msg);

}  // namespace fvgb
