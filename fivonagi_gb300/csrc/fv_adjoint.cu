// fv_adjoint.cu -- discrete adjoint of the time step, for the phased array's
// element weights.
//
// The reference has no adjoint. This is the reverse mode of this library's
// own forward step, differentiated at the forward's own states (recorded
// during the segment replays) with the dt schedule of a base forward run
// held fixed:
//
//   u_n = S(u_{n-1}; weights, dt_{n-1}, T_{n-1}),   S = D o X o Y o B
//
// B the boundary hook (ghost cells), Y and X the dimensionally split sweeps
// (apps/na/fv.h), D the diffusion (apps/na/source.h). The loss is the mean
// of u1^2 over a window of cells and a range of accepted steps.
//
// Forward: the ordinary attempt launches (ghost frame, step, fix-up,
// finalize), with
// three one-thread kernels around each attempt that record the dt and T of
// accepted steps, copy a checkpoint every C accepted steps and add the
// step's window sum to the loss -- all device-side, no host round trip per
// step. Backward: segment by segment from the last checkpoint, replay the
// segment's steps from its checkpoint (frozen dt) into a buffer of C
// states; each replayed attempt also records its stage grids B, Y, X (the
// step kernel writes them as it goes, kStageRecord), the linearisation
// points of the reverse step. Then walk the segment backwards. A reverse
// step runs grid-wide reverse kernels: diffusion, x sweep, y sweep (three
// kernels each: waves, interface adjoints, per-cell gather), boundary
// (ghost cells back to the cells they copy, and the source cells to the
// weights).
// Memory: 3 (N / C) + 12 C + ~40 grids; C = ceil(sqrt(N)) by default.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <new>
#include <vector>

#include "fv_adjoint.cuh"
#include "fv_internal.h"

using namespace fvgb;

namespace {

constexpr int kBX = 32, kBY = 8;  // 2-D launch shape of the grid kernels
constexpr int kWarpsPerStep = 4;  // the step kernel's warps per CTA

struct G3 {
  float *f[3];
};
struct CG3 {
  const float *f[3];
};
struct WaveStore {
  float *w[10];  // s1 s2 s3 w11 w21 w31 w12 w22 w32 w33, per interface (at its 'a' cell)
};
struct AdjStore {
  float *g[6];  // ga (the interface's 'a' cell) then gb (its 'b' cell), local frame
};

// Records of the forward run, written by one-thread kernels.
struct AdjRec {
  float dt0, T0;  // scalars before the attempt
  int n0;         // accepted steps before the attempt
  int accepted;   // the attempt was accepted
};

fv_status afail(fv_status s, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  set_last_error(buf);
  return s;
}

#define FVA_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess) return afail(FV_CUDA_ERROR, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

__device__ __forceinline__ bool interior(const DevParams &p, int i, int j) {
  return i >= 2 && i <= p.nx - 3 && j >= 2 && j <= p.ny - 3;
}

// ------------------------------------------------------------ forward records

__global__ void adj_pre_kernel(const Ctrl *c, AdjRec *r) {
  r->dt0 = c->dt;
  r->T0 = c->T;
  r->n0 = c->n;
  r->accepted = 0;
}

__global__ void adj_post_kernel(const Ctrl *c, AdjRec *r, float *sched_dt, float *sched_T, int nsteps) {
  if (c->n == r->n0 + 1 && r->n0 < nsteps) {
    r->accepted = 1;
    sched_dt[r->n0] = r->dt0;
    sched_T[r->n0] = r->T0;
  }
}

// After an accepted attempt: the checkpoint every `every` steps.
__global__ void adj_checkpoint_kernel(const Ctrl *c, const AdjRec *r, G3 s0, G3 s1, float *ckpt,
                                      size_t stride, size_t ncell, int every) {
  if (!r->accepted) return;
  const int n = c->n;
  if (n % every != 0) return;
  const G3 &src = c->cur ? s1 : s0;
  float *dst = ckpt + size_t(n / every) * 3 * stride;
  for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < ncell; k += size_t(gridDim.x) * blockDim.x) {
    dst[k] = src.f[0][k];
    dst[stride + k] = src.f[1][k];
    dst[2 * stride + k] = src.f[2][k];
  }
}

// Window sum of u1^2 of the current state after an accepted attempt whose
// step lies in [first, last]; `rec` may be null (replays: every attempt is
// accepted).
__global__ void adj_loss_kernel(const Ctrl *c, const AdjRec *r, G3 s0, G3 s1, int nx, int i0, int j0,
                                int ni, int nj, long long first, long long last, double *acc) {
  if (r && !r->accepted) return;
  const long long n = c->n;
  if (n < first || n > last) return;
  const float *u1 = (c->cur ? s1 : s0).f[0];
  double sum = 0.0;
  for (int k = threadIdx.x; k < ni * nj; k += blockDim.x) {
    const int i = i0 + k % ni, j = j0 + k / ni;
    const double v = u1[i + size_t(j) * nx];
    sum += v * v;
  }
  __shared__ double red[256];
  red[threadIdx.x] = sum;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) atomicAdd(acc, red[0]);
}

// Scalars of step n of the frozen schedule (0-based: the step from u_n).
__global__ void adj_sched_kernel(Ctrl *c, const float *sched_dt, const float *sched_T, int n, int cur) {
  c->dt = sched_dt[n];
  c->T = sched_T[n];
  c->n = n;
  if (cur >= 0) c->cur = cur;
  c->status = 0;
  c->neg_flag = 0;
  c->sim_error = 0;
  c->consecutive_rejects = 0;
  c->mdx = 0;
  c->mdy = 0;
  c->remaining = 1;
  c->t_stop = __int_as_float(0x7f800000);
  c->blocks_done = 0;
}

__global__ void adj_ctrl_reset_kernel(Ctrl *c, float dt, float T, long long remaining) {
  c->dt = dt;
  c->T = T;
  c->last_cfl = 0.0f;
  c->t_stop = __int_as_float(0x7f800000);
  c->n = 0;
  c->cur = 0;
  c->status = 0;
  c->neg_flag = 0;
  c->sim_error = 0;
  c->consecutive_rejects = 0;
  c->mdx = 0;
  c->mdy = 0;
  c->remaining = remaining;
  c->accepted = 0;
  c->rejected = 0;
  c->blocks_done = 0;
}

// ------------------------------------------------------------ reverse kernels

// Diffusion (source, apps/na/source.h:22-104): o1 = (u1 + 1) - 1,
// o2 = u2 + ddtx2 (vx(i-1) - 2 vx + vx(i+1)) + ddty2 (vx(j-1) - 2 vx + vx(j+1)),
// o3 likewise with vy, on interior cells; identity elsewhere.
__global__ void adj_diffusion_kernel(DevParams p, float dt, CG3 s2, CG3 lo, G3 li) {
  const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
  const int nx = p.nx, ny = p.ny;
  if (i >= nx || j >= ny) return;
  const size_t o = size_t(i) + size_t(j) * nx;
  const float ddtx2 = p.diffdelta * dt / (p.dx * p.dx);
  const float ddty2 = p.diffdelta * dt / (p.dy * p.dy);
  float gvx = 0.f, gvy = 0.f;
  if (interior(p, i, j)) {
    gvx -= 2.0f * (ddtx2 + ddty2) * lo.f[1][o];
    gvy -= 2.0f * (ddtx2 + ddty2) * lo.f[2][o];
  }
  const int ni[4] = {i - 1, i + 1, i, i};
  const int nj[4] = {j, j, j - 1, j + 1};
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (!interior(p, ni[k], nj[k])) continue;
    const size_t q = size_t(ni[k]) + size_t(nj[k]) * nx;
    const float c = k < 2 ? ddtx2 : ddty2;
    gvx += c * lo.f[1][q];
    gvy += c * lo.f[2][q];
  }
  const float rho = s2.f[0][o] + 1.0f;
  const float vx = fdiv(s2.f[1][o], rho), vy = fdiv(s2.f[2][o], rho);
  li.f[0][o] = lo.f[0][o] - fdiv(gvx * vx + gvy * vy, rho);
  li.f[1][o] = lo.f[1][o] + fdiv(gvx, rho);
  li.f[2][o] = lo.f[2][o] + fdiv(gvy, rho);
}

// Local frame of a sweep: component 1 = u1; x sweep (dir 0): normal = u2,
// transverse = u3; y sweep (dir 1): normal = u3, transverse = u2
// (apps/na/fv.h:489-493).
__device__ __forceinline__ void local3(const CG3 &g, int dir, size_t o, float &q1, float &qn, float &qt) {
  q1 = g.f[0][o];
  qn = g.f[dir == 0 ? 1 : 2][o];
  qt = g.f[dir == 0 ? 2 : 1][o];
}

__device__ __forceinline__ WaveN load_wave(const WaveStore &ws, size_t o) {
  WaveN w;
  w.s1 = ws.w[0][o]; w.s2 = ws.w[1][o]; w.s3 = ws.w[2][o];
  w.w11 = ws.w[3][o]; w.w21 = ws.w[4][o]; w.w31 = ws.w[5][o];
  w.w12 = ws.w[6][o]; w.w22 = ws.w[7][o]; w.w32 = ws.w[8][o];
  w.w33 = ws.w[9][o];
  return w;
}

// Waves and speeds at every interface of a sweep (the interface between a
// cell and its predecessor along the sweep; none for the first cell).
__global__ void adj_waves_kernel(DevParams p, int dir, float dt, CG3 s, WaveStore ws) {
  const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
  const int nx = p.nx, ny = p.ny;
  if (i >= nx || j >= ny) return;
  const size_t o = size_t(i) + size_t(j) * nx;
  const int k = dir == 0 ? i : j;
  WaveN w{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (k >= 1) {
    const size_t b = dir == 0 ? o - 1 : o - size_t(nx);
    float q1a, qna, qta, q1b, qnb, qtb;
    local3(s, dir, o, q1a, qna, qta);
    local3(s, dir, b, q1b, qnb, qtb);
    const float ra = q1a + 1.0f, rb = q1b + 1.0f;
    const float dtx = dt / (dir == 0 ? p.dx : p.dy);
    float cfl = 0.0f;
    Fluct f;
    DivFast fast;
    riemann(ra, qna, qta, fdiv(qna, ra), fdiv(qta, ra), rb, qnb, qtb, fdiv(qnb, rb), fdiv(qtb, rb),
            2.0f * (p.beta - 1.0f), dtx, cfl, w, f, fast);
  }
  ws.w[0][o] = w.s1; ws.w[1][o] = w.s2; ws.w[2][o] = w.s3;
  ws.w[3][o] = w.w11; ws.w[4][o] = w.w21; ws.w[5][o] = w.w31;
  ws.w[6][o] = w.w12; ws.w[7][o] = w.w22; ws.w[8][o] = w.w32;
  ws.w[9][o] = w.w33;
}

// Adjoints of the two cells of each interface. The sweep updates interior
// cell R as u_R - dtx (apdq_R + amdq_{R+1}) - dtx (F_{R+1} - F_R), F_k the
// limited correction flux at interface k (step_x/_y, writeLimiters_x/_y,
// apps/na/fv.h:384-499, 933-1054). With mu the output adjoint on interior
// cells (0 elsewhere): d apdq_k = -dtx mu_k, d amdq_k = -dtx mu_{k-1},
// d F_k = dtx (mu_k - mu_{k-1}). The waves at k feed the corrections at
// k-1, k, k+1, whose reverses are gathered here; then the Riemann solve's
// reverse gives the two cells' adjoints.
__global__ void adj_interface_kernel(DevParams p, int dir, float dt, CG3 s, CG3 lo, WaveStore ws,
                                     AdjStore as) {
  const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
  const int nx = p.nx, ny = p.ny;
  if (i >= nx || j >= ny) return;
  const size_t o = size_t(i) + size_t(j) * nx;
  const int k = dir == 0 ? i : j;
  const int n = dir == 0 ? nx : ny;
  const long long step = dir == 0 ? 1 : nx;
  Adj3 ga{0.f, 0.f, 0.f}, gb{0.f, 0.f, 0.f};
  if (k >= 1) {
    const float dtx = dt / (dir == 0 ? p.dx : p.dy);
    auto mu = [&](int kk) {
      Adj3 m{0.f, 0.f, 0.f};
      const int ii = dir == 0 ? kk : i, jj = dir == 0 ? j : kk;
      if (kk >= 0 && kk < n && interior(p, ii, jj)) {
        local3(lo, dir, size_t(ii) + size_t(jj) * nx, m.q1, m.qn, m.qt);
      }
      return m;
    };
    auto wave = [&](int kk) {
      if (kk < 1 || kk > n - 1) return WaveN{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
      return load_wave(ws, size_t((long long)o + (long long)(kk - k) * step));
    };
    const Adj3 mm2 = mu(k - 2), mm1 = mu(k - 1), m0 = mu(k), mp1 = mu(k + 1);
    const WaveN wm2 = wave(k - 2), wm1 = wave(k - 1), w0 = wave(k), wp1 = wave(k + 1), wp2 = wave(k + 2);
    WaveAdj gw, dm, dz, dp;
    zero(gw); zero(dm); zero(dz); zero(dp);
    // correction at k-1 (waves k-2, k-1, k): its right-neighbour part
    if (k - 1 >= 1)
      correction_adj(wm2, wm1, w0, dtx, dtx * (mm1.q1 - mm2.q1), dtx * (mm1.qn - mm2.qn),
                     dtx * (mm1.qt - mm2.qt), dm, dz, gw);
    // correction at k (waves k-1, k, k+1): its own part
    correction_adj(wm1, w0, wp1, dtx, dtx * (m0.q1 - mm1.q1), dtx * (m0.qn - mm1.qn), dtx * (m0.qt - mm1.qt),
                   dm, gw, dp);
    // correction at k+1 (waves k, k+1, k+2): its left-neighbour part
    if (k + 1 <= n - 1)
      correction_adj(w0, wp1, wp2, dtx, dtx * (mp1.q1 - m0.q1), dtx * (mp1.qn - m0.qn),
                     dtx * (mp1.qt - m0.qt), gw, dz, dp);
    FluctAdj gf;
    gf.am1 = -dtx * mm1.q1; gf.am2 = -dtx * mm1.qn; gf.am3 = -dtx * mm1.qt;
    gf.ap1 = -dtx * m0.q1; gf.ap2 = -dtx * m0.qn; gf.ap3 = -dtx * m0.qt;
    float q1a, qna, qta, q1b, qnb, qtb;
    local3(s, dir, o, q1a, qna, qta);
    local3(s, dir, size_t((long long)o - step), q1b, qnb, qtb);
    riemann_adj(q1a, qna, qta, q1b, qnb, qtb, 2.0f * (p.beta - 1.0f), gw, gf, ga, gb);
  }
  as.g[0][o] = ga.q1; as.g[1][o] = ga.qn; as.g[2][o] = ga.qt;
  as.g[3][o] = gb.q1; as.g[4][o] = gb.qn; as.g[5][o] = gb.qt;
}

// Input adjoint of a sweep: the output adjoint (the update's identity part)
// plus the cell's share of its two interfaces.
__global__ void adj_combine_kernel(DevParams p, int dir, CG3 lo, AdjStore as, G3 li) {
  const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
  const int nx = p.nx, ny = p.ny;
  if (i >= nx || j >= ny) return;
  const size_t o = size_t(i) + size_t(j) * nx;
  const int k = dir == 0 ? i : j;
  const int n = dir == 0 ? nx : ny;
  float a1 = 0.f, an = 0.f, at = 0.f;
  if (k >= 1) {
    a1 += as.g[0][o]; an += as.g[1][o]; at += as.g[2][o];
  }
  if (k + 1 <= n - 1) {
    const size_t q = dir == 0 ? o + 1 : o + size_t(nx);
    a1 += as.g[3][q]; an += as.g[4][q]; at += as.g[5][q];
  }
  li.f[0][o] = lo.f[0][o] + a1;
  li.f[dir == 0 ? 1 : 2][o] = lo.f[dir == 0 ? 1 : 2][o] + an;
  li.f[dir == 0 ? 2 : 1][o] = lo.f[dir == 0 ? 2 : 1][o] + at;
}

__device__ __forceinline__ bool array_row(const DevParams &p, int j) {
  const int jr = j - p.arr_j0;
  return jr >= 0 && jr < p.nelem * p.arr_elem;
}

// Boundary hook of the phased array (fv_device.cuh ghost_value): interior
// cells pass through; ghost cells are copies of the nearest interior cell
// (right column pair, top and bottom row pairs, left pair outside the
// array), zeros (corners) or the source (left pair on the array's rows).
// The copies' adjoints return to the cells they copy.
__global__ void adj_boundary_kernel(DevParams p, CG3 lb, G3 lp) {
  const int i = blockIdx.x * kBX + threadIdx.x, j = blockIdx.y * kBY + threadIdx.y;
  const int nx = p.nx, ny = p.ny;
  if (i >= nx || j >= ny) return;
  const size_t o = size_t(i) + size_t(j) * nx;
  float a[3] = {0.f, 0.f, 0.f};
  if (interior(p, i, j)) {
    auto add = [&](int ii, int jj) {
      const size_t q = size_t(ii) + size_t(jj) * nx;
      a[0] += lb.f[0][q]; a[1] += lb.f[1][q]; a[2] += lb.f[2][q];
    };
    add(i, j);
    if (i == nx - 3) { add(nx - 2, j); add(nx - 1, j); }
    if (j == ny - 3) { add(i, ny - 2); add(i, ny - 1); }
    if (j == 2) { add(i, 0); add(i, 1); }
    if (i == 2 && !array_row(p, j)) { add(0, j); add(1, j); }
  }
  lp.f[0][o] = a[0];
  lp.f[1][o] = a[1];
  lp.f[2][o] = a[2];
}

// Weight gradients of one step from the adjoints of the source ghost cells:
// u1 = pack, u2 = pack (pack + 1), pack = amp ramp(T) sin(ISPW T + phase).
// One warp per element: the lanes load the element's ghost cells at once
// (a strided loop when an element spans more than 16 rows), a warp
// reduction in FP64 sums them, and lane 0 updates the element's sums.
__global__ void adj_weights_kernel(DevParams p, float T, CG3 lb, double *g_amp, double *g_ph) {
  const int e = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (e >= p.nelem) return;  // warp-uniform
  const float amp = p.weights[e], ph = p.weights[p.nelem + e];
  const float ramp = gmin(gmax(T * p.ramp, 0.0f), 1.0f);
  const float arg = p.ispw * T + ph;
  const float sn = fvm::sinf_(arg);
  const float pack = amp * ramp * sn;
  double sum = 0.0;
  for (int k = lane; k < 2 * p.arr_elem; k += 32) {
    const int j = p.arr_j0 + e * p.arr_elem + (k >> 1), i = k & 1;
    if (j < 2 || j > p.ny - 3) continue;  // corners are zero, not the source
    const size_t q = size_t(i) + size_t(j) * p.nx;
    sum += (double)lb.f[0][q] + (double)lb.f[1][q] * (2.0 * pack + 1.0);
  }
  for (int off = 16; off > 0; off >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, off);
  if (lane == 0) {
    const float cs = fvm::cosf_(arg);
    g_amp[e] += sum * (double)ramp * (double)sn;
    g_ph[e] += sum * (double)amp * (double)ramp * (double)cs;
  }
}

// Loss gradient of the state after accepted step n: 2 u1 coef on the window.
__global__ void adj_loss_grad_kernel(const float *u1, float *l1, int nx, int i0, int j0, int ni, int nj,
                                     float coef) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= ni * nj) return;
  const size_t o = size_t(i0 + k % ni) + size_t(j0 + k / ni) * nx;
  l1[o] += 2.0f * u1[o] * coef;
}

}  // namespace

// ------------------------------------------------------------------ handle

struct fv_adjoint {
  fv_params params{};
  DevParams dp{}, dp_replay{};  // replay: CFLMAX infinite (the schedule is fixed)
  fv_loss_window win{};
  long long nsteps = 0;
  int every = 1;                // checkpoint interval C
  int nckpt = 0;                // checkpoints 0, C, 2C, ... <= nsteps
  int sms = 0, max_resident = 0;
  size_t ncell = 0, stride = 0;
  cudaStream_t stream = nullptr, own_stream = nullptr;
  // device memory: one allocation of grids, plus small arrays
  float *mem = nullptr;
  float *state[2][3] = {};      // forward state pair
  float *ckpt = nullptr;        // nckpt states
  float *seg = nullptr;         // C + 1 states of the segment being reversed
  float *stg = nullptr;         // C stage triples (B, S1, S2) of the segment's steps
  float *lam[2][3] = {};        // adjoint ping-pong
  float *tmp[2][3] = {};        // sweep adjoints
  float *waves[10] = {};
  float *gab[6] = {};
  float *frame = nullptr;
  float *weights = nullptr;     // amplitudes then phases
  Ctrl *ctrl = nullptr;
  AdjRec *rec = nullptr;
  float *partials = nullptr;
  uint32_t *fix = nullptr;
  size_t fix_words = 0;
  int nblocks = 0, fix_blocks = 0, nstrips = 0;
  float *sched = nullptr;       // dt[nsteps] then T[nsteps]
  double *acc = nullptr;        // loss sum, then gradient sums (2 nelem)
  std::vector<float> h_dt, h_T;
  bool have_schedule = false;  // a recorded dt schedule (replays need it)
  bool have_forward = false;   // checkpoints of the recorded run (the backward needs them)
  int final_cur = 0;           // state[final_cur] holds the last forward's final state
                               // (the backward's replays reuse the control block)
  int exact = 1;
};

namespace {

StepArgs step_args(const fv_adjoint *a, const DevParams &dp, float *const in[3], float *const out[3]) {
  StepArgs s{};
  s.p = dp;
  for (int f = 0; f < 3; ++f) {
    s.state[0][f] = in[f];
    s.state[1][f] = out[f];
    s.frame[f] = a->frame + size_t(f) * size_t(frame_cells(a->params.nx, a->params.ny));
  }
  s.ctrl = a->ctrl;
  s.partials = a->partials;
  s.fix = a->fix;
  s.nstrips = a->nstrips;
  s.nblocks = a->nblocks;
  s.work = (long long)a->nstrips * a->params.ny;
  s.fix_blocks = a->fix_blocks;
  return s;
}

int launch(const fv_adjoint *a, const StepArgs &s, int stage) {
  return a->exact ? launch_step_exact(s, kWarpsPerStep, stage, a->stream)
                  : launch_step_fast(s, kWarpsPerStep, stage, a->stream);
}

G3 g3(float *const f[3]) { return G3{{f[0], f[1], f[2]}}; }
CG3 cg3(float *const f[3]) { return CG3{{f[0], f[1], f[2]}}; }

float *slot(float *base, size_t stride, long long k, int f) { return base + (size_t(k) * 3 + f) * stride; }
// grid f of stage st (0 = B, 1 = S1, 2 = S2) of the segment's k-th step
float *stage_grid(const fv_adjoint *a, long long k, int st, int f) {
  return a->stg + ((size_t(k) * 3 + st) * 3 + f) * a->stride;
}

fv_status set_weights(fv_adjoint *a, const float *amp, const float *phase) {
  const int n = a->dp.nelem;
  FVA_CUDA(cudaMemcpyAsync(a->weights, amp, sizeof(float) * n, cudaMemcpyHostToDevice, a->stream));
  FVA_CUDA(cudaMemcpyAsync(a->weights + n, phase, sizeof(float) * n, cudaMemcpyHostToDevice, a->stream));
  return FV_OK;
}

// Runs the forward from the initial state (zero) with the adaptive dt
// (record = true: records the schedule and checkpoints) or with the
// recorded schedule (record = false); returns the loss.
fv_status run_forward(fv_adjoint *a, bool record, double *loss) {
  const fv_params &P = a->params;
  const size_t bytes = 3 * a->stride * sizeof(float);
  for (int b = 0; b < 2; ++b) FVA_CUDA(cudaMemsetAsync(a->state[b][0], 0, bytes, a->stream));
  FVA_CUDA(cudaMemsetAsync(a->acc, 0, sizeof(double), a->stream));
  FVA_CUDA(cudaMemsetAsync(a->fix, 0, a->fix_words * sizeof(uint32_t), a->stream));
  G3 s0 = g3(a->state[0]), s1 = g3(a->state[1]);
  const fv_loss_window &w = a->win;
  if (record) {
    // checkpoint 0: the initial state
    FVA_CUDA(cudaMemsetAsync(a->ckpt, 0, bytes, a->stream));
    adj_ctrl_reset_kernel<<<1, 1, 0, a->stream>>>(a->ctrl, float(P.dtini), -float(P.tide), a->nsteps);
    const StepArgs s = step_args(a, a->dp, a->state[0], a->state[1]);
    const int cgrid = std::max(1, a->sms * 4);
    long long todo = a->nsteps;
    for (int round = 0; round < 64 && todo > 0; ++round) {
      for (long long k = 0; k < todo; ++k) {
        adj_pre_kernel<<<1, 1, 0, a->stream>>>(a->ctrl, a->rec);
        int rc = launch(a, s, -1);
        if (rc != 0) return afail(FV_CUDA_ERROR, "step launch: %s", cudaGetErrorString((cudaError_t)rc));
        adj_post_kernel<<<1, 1, 0, a->stream>>>(a->ctrl, a->rec, a->sched, a->sched + a->nsteps, int(a->nsteps));
        adj_checkpoint_kernel<<<cgrid, 256, 0, a->stream>>>(a->ctrl, a->rec, s0, s1, a->ckpt, a->stride, a->ncell,
                                                             a->every);
        adj_loss_kernel<<<1, 256, 0, a->stream>>>(a->ctrl, a->rec, s0, s1, P.nx, w.i0, w.j0, w.ni, w.nj,
                                                   w.step_first, w.step_last, a->acc);
      }
      FVA_CUDA(cudaGetLastError());
      Ctrl c;
      FVA_CUDA(cudaMemcpyAsync(&c, a->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, a->stream));
      FVA_CUDA(cudaStreamSynchronize(a->stream));
      if (c.status) return afail((fv_status)c.status, "forward run stopped with status %d", c.status);
      todo = c.remaining;  // rejected attempts are made up
    }
    if (todo > 0) return afail(FV_DT_TOO_LARGE, "forward run did not finish");
    a->h_dt.resize(a->nsteps);
    a->h_T.resize(a->nsteps);
    FVA_CUDA(cudaMemcpy(a->h_dt.data(), a->sched, sizeof(float) * a->nsteps, cudaMemcpyDeviceToHost));
    FVA_CUDA(cudaMemcpy(a->h_T.data(), a->sched + a->nsteps, sizeof(float) * a->nsteps, cudaMemcpyDeviceToHost));
  } else {
    adj_ctrl_reset_kernel<<<1, 1, 0, a->stream>>>(a->ctrl, float(P.dtini), -float(P.tide), 0);
    const StepArgs s = step_args(a, a->dp_replay, a->state[0], a->state[1]);
    for (long long n = 0; n < a->nsteps; ++n) {
      adj_sched_kernel<<<1, 1, 0, a->stream>>>(a->ctrl, a->sched, a->sched + a->nsteps, int(n), -1);
      int rc = launch(a, s, -1);
      if (rc != 0) return afail(FV_CUDA_ERROR, "step launch: %s", cudaGetErrorString((cudaError_t)rc));
      adj_loss_kernel<<<1, 256, 0, a->stream>>>(a->ctrl, nullptr, s0, s1, P.nx, w.i0, w.j0, w.ni, w.nj,
                                                 w.step_first, w.step_last, a->acc);
    }
    FVA_CUDA(cudaGetLastError());
    Ctrl c;
    FVA_CUDA(cudaMemcpyAsync(&c, a->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, a->stream));
    FVA_CUDA(cudaStreamSynchronize(a->stream));
    if (c.status) return afail((fv_status)c.status, "replay stopped with status %d", c.status);
  }
  {
    Ctrl c;
    FVA_CUDA(cudaMemcpyAsync(&c, a->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, a->stream));
    FVA_CUDA(cudaStreamSynchronize(a->stream));
    a->final_cur = c.cur & 1;
  }
  double sum = 0.0;
  FVA_CUDA(cudaMemcpy(&sum, a->acc, sizeof(double), cudaMemcpyDeviceToHost));
  const double K = double(w.step_last - w.step_first + 1), W = double(w.ni) * double(w.nj);
  if (loss) *loss = sum / (K * W);
  return FV_OK;
}

}  // namespace

extern "C" {

fv_status fv_adjoint_create(const fv_params *p, const fv_loss_window *w, int64_t nsteps,
                            int32_t checkpoint_every, fv_adjoint **out) {
  if (!p || !w || !out) return afail(FV_BAD_ARG, "NULL argument");
  *out = nullptr;
  fv_status s = validate_params(p);
  if (s != FV_OK) return s;
  if (p->app != FV_APP_PHASED_ARRAY) return afail(FV_BAD_ARG, "the adjoint is for the phased array app");
  if (p->moving_domain) return afail(FV_BAD_ARG, "the adjoint needs moving_domain = 0");
  if (nsteps < 1 || nsteps > (1LL << 24)) return afail(FV_BAD_ARG, "nsteps must be 1..2^24");
  if (w->ni < 1 || w->nj < 1 || w->i0 < 0 || w->j0 < 0 || w->i0 + w->ni > p->nx || w->j0 + w->nj > p->ny)
    return afail(FV_BAD_ARG, "loss window outside the grid");
  if (w->step_first < 1 || w->step_last < w->step_first || w->step_last > nsteps)
    return afail(FV_BAD_ARG, "loss steps must satisfy 1 <= first <= last <= nsteps");
  int dev = 0;
  FVA_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  FVA_CUDA(cudaGetDeviceProperties(&prop, dev));
  if (prop.major != 10 || prop.minor != 3) return afail(FV_NO_DEVICE, "device is not sm_103");

  fv_adjoint *a = new (std::nothrow) fv_adjoint();
  if (!a) return afail(FV_CUDA_ERROR, "out of host memory");
  auto cleanup = [&](fv_status st) {
    fv_adjoint_destroy(a);
    return st;
  };
  a->params = *p;
  a->win = *w;
  a->nsteps = nsteps;
  a->exact = p->exact ? 1 : 0;
  a->every = checkpoint_every > 0 ? checkpoint_every
                                  : std::max(1, int(std::ceil(std::sqrt(double(nsteps)))));
  a->nckpt = int(nsteps / a->every) + 1;
  a->ncell = size_t(p->nx) * size_t(p->ny);
  a->stride = (a->ncell + 63) & ~size_t(63);
  a->sms = prop.multiProcessorCount;
  a->dp = dev_params_of(*p);
  a->dp_replay = a->dp;
  a->dp_replay.cflmax = __builtin_huge_valf();
  // grids: state 2x3, checkpoints, segment (C + 1 states), C stage
  // triples 3x3, lam 2x3, tmp 2x3, waves 10, gab 6
  const size_t nstates = 2 + size_t(a->nckpt) + size_t(a->every + 1) + 3 * size_t(a->every) + 2 + 2;
  const size_t ngrids = nstates * 3 + 10 + 6;
  cudaError_t e = cudaMalloc(&a->mem, ngrids * a->stride * sizeof(float));
  if (e != cudaSuccess)
    return cleanup(afail(FV_CUDA_ERROR, "cudaMalloc adjoint grids (%zu MB): %s", ngrids * a->stride * 4 >> 20,
                         cudaGetErrorString(e)));
  float *cur = a->mem;
  auto take = [&](size_t nst) {
    float *r = cur;
    cur += nst * 3 * a->stride;
    return r;
  };
  for (int b = 0; b < 2; ++b) {
    float *base = take(1);
    for (int f = 0; f < 3; ++f) a->state[b][f] = base + f * a->stride;
  }
  a->ckpt = take(a->nckpt);
  a->seg = take(a->every + 1);
  a->stg = take(3 * size_t(a->every));
  for (int k = 0; k < 2; ++k) {
    float *base = take(1);
    for (int f = 0; f < 3; ++f) a->lam[k][f] = base + f * a->stride;
  }
  for (int k = 0; k < 2; ++k) {
    float *base = take(1);
    for (int f = 0; f < 3; ++f) a->tmp[k][f] = base + f * a->stride;
  }
  for (int k = 0; k < 10; ++k) a->waves[k] = cur + k * a->stride;
  cur += 10 * a->stride;
  for (int k = 0; k < 6; ++k) a->gab[k] = cur + k * a->stride;

  const int strip_c = kWarpsPerStep * kWarpCols;
  a->nstrips = (p->nx + strip_c - 1) / strip_c;
  const long long work = (long long)a->nstrips * p->ny;
  const int per_sm = a->exact ? max_blocks_per_sm_exact(kWarpsPerStep, -1) : max_blocks_per_sm_fast(kWarpsPerStep, -1);
  a->max_resident = per_sm * a->sms;
  a->nblocks = int(std::max(1LL, std::min((long long)a->max_resident, work / 32)));  // one wave
  a->fix_blocks = 4 * a->sms;
  a->fix_words = size_t(fix_scratch_words((long long)a->nstrips * kWarpsPerStep, p->ny));
  e = cudaMalloc(&a->frame, 3 * size_t(frame_cells(p->nx, p->ny)) * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&a->weights, 2 * size_t(p->array_elems) * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&a->ctrl, sizeof(Ctrl));
  if (e == cudaSuccess) e = cudaMalloc(&a->rec, sizeof(AdjRec));
  if (e == cudaSuccess) e = cudaMalloc(&a->partials, size_t(a->nblocks + a->fix_blocks) * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&a->fix, a->fix_words * sizeof(uint32_t));
  if (e == cudaSuccess) e = cudaMalloc(&a->sched, 2 * size_t(nsteps) * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&a->acc, (1 + 2 * size_t(p->array_elems)) * sizeof(double));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&a->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cleanup(afail(FV_CUDA_ERROR, "adjoint allocation: %s", cudaGetErrorString(e)));
  a->stream = a->own_stream;
  a->dp.weights = a->weights;
  a->dp_replay.weights = a->weights;
  std::vector<float> w0(2 * size_t(p->array_elems), 0.0f);
  for (int k = 0; k < p->array_elems; ++k) w0[k] = float(p->ampl);
  e = cudaMemcpy(a->weights, w0.data(), w0.size() * sizeof(float), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cleanup(afail(FV_CUDA_ERROR, "weights: %s", cudaGetErrorString(e)));
  *out = a;
  return FV_OK;
}

fv_status fv_adjoint_destroy(fv_adjoint *a) {
  if (!a) return FV_OK;
  if (a->stream) cudaStreamSynchronize(a->stream);
  if (a->mem) cudaFree(a->mem);
  if (a->frame) cudaFree(a->frame);
  if (a->weights) cudaFree(a->weights);
  if (a->ctrl) cudaFree(a->ctrl);
  if (a->rec) cudaFree(a->rec);
  if (a->partials) cudaFree(a->partials);
  if (a->fix) cudaFree(a->fix);
  if (a->sched) cudaFree(a->sched);
  if (a->acc) cudaFree(a->acc);
  if (a->own_stream) cudaStreamDestroy(a->own_stream);
  delete a;
  return FV_OK;
}

fv_status fv_adjoint_set_stream(fv_adjoint *a, void *cuda_stream) {
  if (!a) return afail(FV_BAD_ARG, "NULL argument");
  FVA_CUDA(cudaStreamSynchronize(a->stream));
  a->stream = cuda_stream ? (cudaStream_t)cuda_stream : a->own_stream;
  return FV_OK;
}

fv_status fv_adjoint_forward(fv_adjoint *a, const float *amp, const float *phase, double *loss) {
  if (!a || !amp || !phase) return afail(FV_BAD_ARG, "NULL argument");
  fv_status s = set_weights(a, amp, phase);
  if (s != FV_OK) return s;
  a->have_forward = false;
  a->have_schedule = false;
  s = run_forward(a, true, loss);
  if (s != FV_OK) return s;
  a->have_forward = true;
  a->have_schedule = true;
  return FV_OK;
}

fv_status fv_adjoint_replay(fv_adjoint *a, const float *amp, const float *phase, double *loss) {
  if (!a || !amp || !phase) return afail(FV_BAD_ARG, "NULL argument");
  if (!a->have_schedule) return afail(FV_BAD_ARG, "no forward run: its dt schedule is replayed");
  fv_status s = set_weights(a, amp, phase);
  if (s != FV_OK) return s;
  // the replay overwrites the weights and the state the backward pass
  // would differentiate: a backward needs a new fv_adjoint_forward
  a->have_forward = false;
  return run_forward(a, false, loss);
}

fv_status fv_adjoint_schedule(fv_adjoint *a, double *dt, double *T) {
  if (!a || !dt || !T) return afail(FV_BAD_ARG, "NULL argument");
  if (a->h_dt.size() != size_t(a->nsteps)) return afail(FV_BAD_ARG, "no forward run");
  for (long long k = 0; k < a->nsteps; ++k) {
    dt[k] = a->h_dt[k];
    T[k] = a->h_T[k];
  }
  return FV_OK;
}

fv_status fv_adjoint_get_state(fv_adjoint *a, float *u1, float *u2, float *u3) {
  if (!a || !u1 || !u2 || !u3) return afail(FV_BAD_ARG, "NULL argument");
  FVA_CUDA(cudaStreamSynchronize(a->stream));
  float *dst[3] = {u1, u2, u3};
  for (int f = 0; f < 3; ++f)
    FVA_CUDA(cudaMemcpy(dst[f], a->state[a->final_cur][f], a->ncell * sizeof(float), cudaMemcpyDeviceToHost));
  return FV_OK;
}

fv_status fv_adjoint_backward(fv_adjoint *a, double *grad_amp, double *grad_phase) {
  if (!a || !grad_amp || !grad_phase) return afail(FV_BAD_ARG, "NULL argument");
  if (!a->have_forward) return afail(FV_BAD_ARG, "no forward run (fv_adjoint_forward) to differentiate");
  const fv_params &P = a->params;
  const int nx = P.nx, ny = P.ny, nelem = P.array_elems;
  const fv_loss_window &w = a->win;
  const float coef = float(1.0 / (double(w.step_last - w.step_first + 1) * double(w.ni) * double(w.nj)));
  const dim3 blk(kBX, kBY), grd((nx + kBX - 1) / kBX, (ny + kBY - 1) / kBY);
  const int wthreads = w.ni * w.nj, wblocks = (wthreads + 255) / 256;
  double *g_amp = a->acc + 1, *g_ph = a->acc + 1 + nelem;
  FVA_CUDA(cudaMemsetAsync(g_amp, 0, 2 * size_t(nelem) * sizeof(double), a->stream));
  const size_t bytes = 3 * a->stride * sizeof(float);
  // lambda_N: the loss gradient of the final state
  int lc = 0;  // lam[lc] holds lambda_n
  FVA_CUDA(cudaMemsetAsync(a->lam[lc][0], 0, bytes, a->stream));
  if (a->nsteps >= w.step_first && a->nsteps <= w.step_last)
    adj_loss_grad_kernel<<<wblocks, 256, 0, a->stream>>>(a->state[a->final_cur][0], a->lam[lc][0], nx, w.i0,
                                                          w.j0, w.ni, w.nj, coef);
  WaveStore ws;
  for (int k = 0; k < 10; ++k) ws.w[k] = a->waves[k];
  AdjStore as;
  for (int k = 0; k < 6; ++k) as.g[k] = a->gab[k];
  const long long C = a->every;
  for (long long seg0 = ((a->nsteps - 1) / C) * C; seg0 >= 0; seg0 -= C) {
    const long long seg1 = std::min(seg0 + C, a->nsteps);  // steps seg0+1 .. seg1
    // the segment's states u_seg0 .. u_seg1 and the stage grids of steps
    // seg0+1 .. seg1: checkpoint, then replay with stage recording
    FVA_CUDA(cudaMemcpyAsync(slot(a->seg, a->stride, 0, 0), slot(a->ckpt, a->stride, seg0 / C, 0), bytes,
                             cudaMemcpyDeviceToDevice, a->stream));
    for (long long n = seg0 + 1; n <= seg1; ++n) {
      float *in[3], *out[3];
      for (int f = 0; f < 3; ++f) {
        in[f] = slot(a->seg, a->stride, n - 1 - seg0, f);
        out[f] = slot(a->seg, a->stride, n - seg0, f);
      }
      adj_sched_kernel<<<1, 1, 0, a->stream>>>(a->ctrl, a->sched, a->sched + a->nsteps, int(n - 1), 0);
      StepArgs s = step_args(a, a->dp_replay, in, out);
      for (int st = 0; st < 3; ++st)
        for (int f = 0; f < 3; ++f) s.stages[3 * st + f] = stage_grid(a, n - 1 - seg0, st, f);
      const int rc = launch(a, s, kStageRecord);
      if (rc != 0) return afail(FV_CUDA_ERROR, "replay launch: %s", cudaGetErrorString((cudaError_t)rc));
    }
    for (long long n = seg1; n > seg0; --n) {
      // reverse of step n, whose input is u_{n-1}
      float *in[3];
      for (int f = 0; f < 3; ++f) in[f] = slot(a->seg, a->stride, n - 1 - seg0, f);
      const float dt = a->h_dt[n - 1], T = a->h_T[n - 1];
      // the recorded boundary-applied, y-swept and x-swept states
      float *stage[3][3];
      for (int st = 0; st < 3; ++st)
        for (int f = 0; f < 3; ++f) stage[st][f] = stage_grid(a, n - 1 - seg0, st, f);
      float *const *lo = a->lam[lc];
      float *const *li = a->lam[lc ^ 1];
      // diffusion: lam_n -> tmp0 (adjoint of S2)
      adj_diffusion_kernel<<<grd, blk, 0, a->stream>>>(a->dp, dt, cg3(stage[2]), cg3(lo), g3(a->tmp[0]));
      // x sweep on S1: tmp0 -> tmp1 (adjoint of S1)
      adj_waves_kernel<<<grd, blk, 0, a->stream>>>(a->dp, 0, dt, cg3(stage[1]), ws);
      adj_interface_kernel<<<grd, blk, 0, a->stream>>>(a->dp, 0, dt, cg3(stage[1]), cg3(a->tmp[0]), ws, as);
      adj_combine_kernel<<<grd, blk, 0, a->stream>>>(a->dp, 0, cg3(a->tmp[0]), as, g3(a->tmp[1]));
      // y sweep on B: tmp1 -> tmp0 (adjoint of B)
      adj_waves_kernel<<<grd, blk, 0, a->stream>>>(a->dp, 1, dt, cg3(stage[0]), ws);
      adj_interface_kernel<<<grd, blk, 0, a->stream>>>(a->dp, 1, dt, cg3(stage[0]), cg3(a->tmp[1]), ws, as);
      adj_combine_kernel<<<grd, blk, 0, a->stream>>>(a->dp, 1, cg3(a->tmp[1]), as, g3(a->tmp[0]));
      // boundary: weights, then lam_{n-1}
      adj_weights_kernel<<<(nelem + 3) / 4, 128, 0, a->stream>>>(a->dp, T, cg3(a->tmp[0]), g_amp, g_ph);
      adj_boundary_kernel<<<grd, blk, 0, a->stream>>>(a->dp, cg3(a->tmp[0]), g3(li));
      if (n - 1 >= w.step_first && n - 1 <= w.step_last)
        adj_loss_grad_kernel<<<wblocks, 256, 0, a->stream>>>(in[0], li[0], nx, w.i0, w.j0, w.ni, w.nj, coef);
      lc ^= 1;
    }
    FVA_CUDA(cudaGetLastError());
  }
  FVA_CUDA(cudaStreamSynchronize(a->stream));
  FVA_CUDA(cudaMemcpy(grad_amp, g_amp, sizeof(double) * nelem, cudaMemcpyDeviceToHost));
  FVA_CUDA(cudaMemcpy(grad_phase, g_ph, sizeof(double) * nelem, cudaMemcpyDeviceToHost));
  return FV_OK;
}

}  // extern "C"
