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
// finalize), each followed by one record launch that keeps the dt and T of
// accepted steps, copies a checkpoint every C accepted steps and adds the
// step's window sum to the loss -- all device-side, no host round trip per
// step. Backward: segment by segment from the last checkpoint, replay the
// segment's steps from its checkpoint (frozen dt) into a buffer of C
// states; each replayed attempt also records its stage grids B, Y, X (the
// step kernel writes them as it goes, kStageRecord), the linearisation
// points of the reverse step. Then walk the segment backwards. A reverse
// step runs the reverse kernels: one fused kernel per sweep (waves,
// limiter reverse, solve reverse and the per-cell gather, with the sweep's
// neighbours in registers and warp shuffles; the x sweep's kernel also
// reverses the diffusion); boundary (ghost cells
// back to the cells they copy, and the source cells to the weights).
// Memory: 3 (N / C) + 12 C + ~21 grids; C = ceil(sqrt(N)) by default.
#include <cuda_runtime.h>

#include <algorithm>
#include <type_traits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
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

// Issues one backward segment's launches (`issue`, returning a status)
// captured as a CUDA graph on `st` and launches the graph: the first
// capture is instantiated into `exec`, later ones update it in place (every
// full segment has the same launches with other arguments), with a new
// instantiation when the shape differs (the short segment at the end of the
// run). A stream that cannot be captured (the legacy default stream) gets
// the launches directly.
template <class F>
fv_status run_captured(cudaStream_t st, cudaGraphExec_t &exec, F &&issue) {
  if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    return issue();
  }
  const fv_status s = issue();
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(st, &g);
  if (s != FV_OK || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return s != FV_OK ? s : afail(FV_CUDA_ERROR, "segment capture: %s", cudaGetErrorString(e));
  }
  if (exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(exec, g, &info) != cudaSuccess) {
      cudaGetLastError();  // a different shape: instantiate anew
      cudaGraphExecDestroy(exec);
      exec = nullptr;
    }
  }
  if (!exec) e = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return afail(FV_CUDA_ERROR, "segment graph: %s", cudaGetErrorString(e));
  e = cudaGraphLaunch(exec, st);
  if (e != cudaSuccess) return afail(FV_CUDA_ERROR, "segment graph launch: %s", cudaGetErrorString(e));
  return FV_OK;
}

// The recorded forward's attempts in graphs of kRecordGraphAttempts (even:
// the record launch alternates between two slots by attempt parity), each
// captured once per handle (the launches' arguments do not change).
constexpr int kRecordGraphAttempts = 32;
// Issues n attempts (`attempt(k)` for k = first .. first + n - 1), the even-
// aligned whole chunks of them through the cached graph `g` (captured on
// first use; a stream that cannot be captured gets the launches directly).
template <class F>
fv_status run_attempts(cudaStream_t st, cudaGraphExec_t &g, long long first, long long n, F &&attempt) {
  long long k = first, end = first + n;
  if (n >= kRecordGraphAttempts + 1 || (n >= kRecordGraphAttempts && (first & 1) == 0)) {
    if (k & 1) {
      const fv_status s = attempt(k++);
      if (s != FV_OK) return s;
    }
    if (!g && cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      fv_status s = FV_OK;
      for (long long j = 0; j < kRecordGraphAttempts && s == FV_OK; ++j) s = attempt(j);
      cudaGraph_t cg = nullptr;
      const cudaError_t e = cudaStreamEndCapture(st, &cg);
      if (s == FV_OK && e == cudaSuccess && cudaGraphInstantiate(&g, cg, 0) != cudaSuccess) g = nullptr;
      if (cg) cudaGraphDestroy(cg);
      if (s != FV_OK) return s;
      if (e != cudaSuccess || !g) return afail(FV_CUDA_ERROR, "forward graph: %s", cudaGetErrorString(cudaGetLastError()));
    }
    cudaGetLastError();
    if (g) {
      for (; end - k >= kRecordGraphAttempts; k += kRecordGraphAttempts) {
        const cudaError_t e = cudaGraphLaunch(g, st);
        if (e != cudaSuccess) return afail(FV_CUDA_ERROR, "forward graph launch: %s", cudaGetErrorString(e));
      }
    }
  }
  for (; k < end; ++k) {
    const fv_status s = attempt(k);
    if (s != FV_OK) return s;
  }
  return FV_OK;
}

// A side stream and two events: launches between fork() and join() run on
// the side stream, concurrently with what the main stream does meanwhile
// (inside a capture they become a parallel branch of the graph).
struct Fork {
  cudaStream_t side = nullptr;
  cudaEvent_t go = nullptr, done = nullptr;
  cudaError_t init() {
    if (side) return cudaSuccess;
    cudaError_t e = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&go, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&done, cudaEventDisableTiming);
    return e;
  }
  cudaError_t fork(cudaStream_t main) {
    cudaError_t e = cudaEventRecord(go, main);
    return e == cudaSuccess ? cudaStreamWaitEvent(side, go, 0) : e;
  }
  cudaError_t join(cudaStream_t main) {
    cudaError_t e = cudaEventRecord(done, side);
    return e == cudaSuccess ? cudaStreamWaitEvent(main, done, 0) : e;
  }
  void release() {
    if (go) cudaEventDestroy(go);
    if (done) cudaEventDestroy(done);
    if (side) cudaStreamDestroy(side);
    side = nullptr;
    go = done = nullptr;
  }
};

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

// Window sum of u1^2 of the current state after a replayed attempt (every
// replayed attempt is accepted) whose step lies in [first, last].
__global__ void adj_loss_kernel(const Ctrl *c, G3 s0, G3 s1, int nx, int i0, int j0, int ni, int nj,
                                long long first, long long last, double *acc) {
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

// After attempt k of the recorded forward, whose scalars before the attempt
// are in rec[parity] (parity = k & 1): whether it was accepted (n advanced
// by one); then its dt and T into the schedule, the checkpoint every
// `every` steps (all blocks) and the window sum of u1^2 (block 0), and the
// scalars before attempt k+1 into rec[parity ^ 1]. One launch per attempt
// instead of a snapshot, a record, a checkpoint and a loss launch; the two
// slots keep block 0's write of the next snapshot from racing with the
// other blocks' read of this one.
__device__ __forceinline__ void record_body(const Ctrl *c, AdjRec *rec, int parity, float *sched_dt,
                                            float *sched_T, int nsteps, const G3 &s0, const G3 &s1, float *ckpt,
                                            size_t stride, size_t ncell, int every, int nx, int i0, int j0, int ni,
                                            int nj, long long first, long long last, double *acc) {
  const AdjRec r = rec[parity];
  const int n = c->n;
  const bool accepted = (n == r.n0 + 1) && r.n0 < nsteps;
  const G3 &src = c->cur ? s1 : s0;
  if (blockIdx.x == 0) {
    if (threadIdx.x == 0) {
      if (accepted) {
        sched_dt[r.n0] = r.dt0;
        sched_T[r.n0] = r.T0;
      }
      AdjRec &next = rec[parity ^ 1];
      next.dt0 = c->dt;
      next.T0 = c->T;
      next.n0 = n;
      next.accepted = 0;
    }
    if (accepted && n >= first && n <= last) {
      double sum = 0.0;
      for (int k = threadIdx.x; k < ni * nj; k += blockDim.x) {
        const int i = i0 + k % ni, j = j0 + k / ni;
        const double v = src.f[0][i + size_t(j) * nx];
        sum += v * v;
      }
      __shared__ double red[256];
      red[threadIdx.x] = sum;
      __syncthreads();
      for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
        __syncthreads();
      }
      if (threadIdx.x == 0) atomicAdd(acc, red[0]);
    }
  }
  if (accepted && n % every == 0) {
    float *dst = ckpt + size_t(n / every) * 3 * stride;
    for (size_t k = blockIdx.x * size_t(blockDim.x) + threadIdx.x; k < ncell; k += size_t(gridDim.x) * blockDim.x) {
      dst[k] = src.f[0][k];
      dst[stride + k] = src.f[1][k];
      dst[2 * stride + k] = src.f[2][k];
    }
  }
}


// Scalars of step n of the frozen schedule (0-based: the step from u_n).
// With `fix` (the backward's replays, which run without the finalize
// launch): also a zero fix-up header, and a negative eigenvalue met by the
// previous replay counted in `rejected` before the flag is cleared.
__global__ void adj_sched_kernel(Ctrl *c, const float *sched_dt, const float *sched_T, int n, int cur,
                                 uint32_t *fix = nullptr) {
  if (fix) {
    fix[0] = 0u;
    fix[1] = 0u;
    if (c->neg_flag) c->rejected += 1;
  }
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

// Local frame of a sweep: component 1 = u1; x sweep: normal = u2,
// transverse = u3; y sweep: normal = u3, transverse = u2
// (apps/na/fv.h:489-493).
__device__ __forceinline__ Adj3 load_local(const CG3 &g, bool xsweep, size_t o) {
  return Adj3{g.f[0][o], g.f[xsweep ? 1 : 2][o], g.f[xsweep ? 2 : 1][o]};
}
__device__ __forceinline__ void store_local(const G3 &g, bool xsweep, size_t o, const Adj3 &v) {
  g.f[0][o] = v.q1;
  g.f[xsweep ? 1 : 2][o] = v.qn;
  g.f[xsweep ? 2 : 1][o] = v.qt;
}

__device__ __forceinline__ float shup(float v) { return __shfl_up_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ float shdn(float v) { return __shfl_down_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ Adj3 shup(const Adj3 &v) { return Adj3{shup(v.q1), shup(v.qn), shup(v.qt)}; }
__device__ __forceinline__ Adj3 shdn(const Adj3 &v) { return Adj3{shdn(v.q1), shdn(v.qn), shdn(v.qt)}; }
__device__ __forceinline__ WaveN shup(const WaveN &w) {
  return WaveN{shup(w.s1), shup(w.s2), shup(w.s3), shup(w.w11), shup(w.w21),
               shup(w.w31), shup(w.w12), shup(w.w22), shup(w.w32), shup(w.w33)};
}
__device__ __forceinline__ WaveN shdn(const WaveN &w) {
  return WaveN{shdn(w.s1), shdn(w.s2), shdn(w.s3), shdn(w.w11), shdn(w.w21),
               shdn(w.w31), shdn(w.w12), shdn(w.w22), shdn(w.w32), shdn(w.w33)};
}
__device__ __forceinline__ WaveAdj shup(const WaveAdj &w) {
  return WaveAdj{shup(w.s1), shup(w.s2), shup(w.s3), shup(w.w11), shup(w.w21),
                 shup(w.w31), shup(w.w12), shup(w.w22), shup(w.w32), shup(w.w33)};
}
__device__ __forceinline__ WaveAdj shdn(const WaveAdj &w) {
  return WaveAdj{shdn(w.s1), shdn(w.s2), shdn(w.s3), shdn(w.w11), shdn(w.w21),
                 shdn(w.w31), shdn(w.w12), shdn(w.w22), shdn(w.w32), shdn(w.w33)};
}
__device__ __forceinline__ void add_to(WaveAdj &a, const WaveAdj &b) {
  a.s1 += b.s1; a.s2 += b.s2; a.s3 += b.s3;
  a.w11 += b.w11; a.w21 += b.w21; a.w31 += b.w31;
  a.w12 += b.w12; a.w22 += b.w22; a.w32 += b.w32; a.w33 += b.w33;
}

// Waves and speeds of the solve between cell a and its predecessor b along
// the sweep (zero where the interface does not exist).
__device__ __forceinline__ WaveN sweep_waves(const Adj3 &sa, const Adj3 &sb, float two_bm1, float dtx, bool exists) {
  WaveN w{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (exists) {
    const float ra = sa.q1 + 1.0f, rb = sb.q1 + 1.0f;
    float cfl = 0.0f;
    Fluct f;
    DivFast fast;
    riemann(ra, sa.qn, sa.qt, fdiv(sa.qn, ra), fdiv(sa.qt, ra), rb, sb.qn, sb.qt, fdiv(sb.qn, rb), fdiv(sb.qt, rb),
            two_bm1, dtx, cfl, w, f, fast);
  }
  return w;
}

__device__ __forceinline__ Adj3 masked(const Adj3 &v, bool keep) {
  return keep ? v : Adj3{0.f, 0.f, 0.f};
}

// The reverse of one sweep, whose forward updates interior cell k as
//   u_k - dtx (apdq_k + amdq_{k+1}) - dtx (F_{k+1} - F_k),
// F_k the limited correction flux at interface k (step_x/_y and
// writeLimiters_x/_y, apps/na/fv.h:384-499, 933-1054). With mu the output
// adjoint on interior cells (0 elsewhere): d apdq_k = -dtx mu_k,
// d amdq_k = -dtx mu_{k-1}, d F_k = dtx (mu_k - mu_{k-1}). Per interface k:
// the solve's waves; the limiter's reverse at k, whose adjoints go to the
// waves at k-1, k, k+1; the waves' adjoint at k, gathered from the limiter
// reverses at k-1, k, k+1; the solve's reverse, giving the adjoints of its
// two cells (ga to cell k, gb to cell k-1); and the sweep's input adjoint
// lo_k + ga_k + gb_{k+1}. Interface k exists for 1 <= k <= n-1.
//
// x sweep: lanes along a row, 26 output columns per warp with a 3-column
// halo each side (the columns of the step kernel's windows); neighbours are
// neighbouring lanes. A warp takes (window, row) pairs, consecutive warps
// neighbouring windows of one row.
//
// The x sweep's kernel also reverses the diffusion that follows the sweep
// (source, apps/na/source.h:22-104): o1 = (u1 + 1) - 1, o2 = u2 +
// ddtx2 (vx(i-1) - 2 vx + vx(i+1)) + ddty2 (vx(j-1) - 2 vx + vx(j+1)), o3
// likewise with vy, on interior cells, identity elsewhere; v = u / rho of
// the x-swept state s2. From the output adjoint lam it forms the sweep's
// output adjoint lo at each lane's cell (the neighbours along the row are
// neighbouring lanes), so lo never passes through memory.
__device__ __forceinline__ Adj3 diffusion_reverse(const DevParams &p, float ddtx2, float ddty2, int i, int j,
                                                  bool in, size_t o, const CG3 &s2, const CG3 &lam) {
  const int nx = p.nx, ny = p.ny;
  float l0 = 0.f, l1 = 0.f, l2 = 0.f;  // lam at (i, j), global components
  float d1 = 0.f, d2 = 0.f, u1 = 0.f, u2 = 0.f;  // lam components 2, 3 at (i, j-1), (i, j+1)
  float q0 = 0.f, q1 = 0.f, q2 = 0.f;  // s2 at (i, j)
  if (in) {
    l0 = lam.f[0][o]; l1 = lam.f[1][o]; l2 = lam.f[2][o];
    q0 = s2.f[0][o]; q1 = s2.f[1][o]; q2 = s2.f[2][o];
    if (j - 1 >= 0) { d1 = lam.f[1][o - nx]; d2 = lam.f[2][o - nx]; }
    if (j + 1 < ny) { u1 = lam.f[1][o + nx]; u2 = lam.f[2][o + nx]; }
  }
  const float lm1 = shup(l1), lm2 = shup(l2), lp1 = shdn(l1), lp2 = shdn(l2);
  float gvx = 0.f, gvy = 0.f;
  if (interior(p, i, j)) {
    gvx -= 2.0f * (ddtx2 + ddty2) * l1;
    gvy -= 2.0f * (ddtx2 + ddty2) * l2;
  }
  if (interior(p, i - 1, j)) { gvx += ddtx2 * lm1; gvy += ddtx2 * lm2; }
  if (interior(p, i + 1, j)) { gvx += ddtx2 * lp1; gvy += ddtx2 * lp2; }
  if (interior(p, i, j - 1)) { gvx += ddty2 * d1; gvy += ddty2 * d2; }
  if (interior(p, i, j + 1)) { gvx += ddty2 * u1; gvy += ddty2 * u2; }
  const float rho = q0 + 1.0f;
  const float vx = fdiv(q1, rho), vy = fdiv(q2, rho);
  // local frame of the x sweep: q1 = u1, qn = u2, qt = u3
  return Adj3{l0 - fdiv(gvx * vx + gvy * vy, rho), l1 + fdiv(gvx, rho), l2 + fdiv(gvy, rho)};
}

__device__ __forceinline__ void sweep_x_body(const DevParams &p, float dt, const CG3 &s, const CG3 &s2,
                                             const CG3 &lam, const G3 &li) {
  const int nx = p.nx, ny = p.ny;
  const int lane = threadIdx.x & 31;
  const long long windows = (nx + kWarpCols - 1) / kWarpCols;
  const long long total = windows * ny;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  const float dtx = dt / p.dx;
  const float two_bm1 = 2.0f * (p.beta - 1.0f);
  const float ddtx2 = p.diffdelta * dt / (p.dx * p.dx);
  const float ddty2 = p.diffdelta * dt / (p.dy * p.dy);
  for (long long t = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < total; t += nw) {
    const int win = (int)(t % windows), j = (int)(t / windows);
    const int i = win * kWarpCols - kHalo + lane;
    const bool in = i >= 0 && i < nx;
    const size_t o = in ? size_t(i) + size_t(j) * nx : 0;
    const Adj3 sa = in ? load_local(s, true, o) : Adj3{0.f, 0.f, 0.f};
    const Adj3 l = diffusion_reverse(p, ddtx2, ddty2, i, j, in, o, s2, lam);
    const Adj3 mu = masked(l, interior(p, i, j));
    const Adj3 sb = shup(sa), mul = shup(mu);
    const bool exists = i >= 1 && i <= nx - 1;
    const WaveN w = sweep_waves(sa, sb, two_bm1, dtx, exists);
    // the limiter's reverse at interface i
    WaveAdj cm, c0, cp;
    zero(cm); zero(c0); zero(cp);
    {
      const WaveN wl = shup(w), wr = shdn(w);
      if (exists)
        correction_adj(wl, w, wr, dtx, dtx * (mu.q1 - mul.q1), dtx * (mu.qn - mul.qn), dtx * (mu.qt - mul.qt),
                       cm, c0, cp);
    }
    // the waves' adjoint at interface i
    WaveAdj g = shup(cp);
    add_to(g, c0);
    add_to(g, shdn(cm));
    FluctAdj gf;
    gf.am1 = -dtx * mul.q1; gf.am2 = -dtx * mul.qn; gf.am3 = -dtx * mul.qt;
    gf.ap1 = -dtx * mu.q1; gf.ap2 = -dtx * mu.qn; gf.ap3 = -dtx * mu.qt;
    Adj3 ga{0.f, 0.f, 0.f}, gb{0.f, 0.f, 0.f};
    if (exists) riemann_adj(sa.q1, sa.qn, sa.qt, sb.q1, sb.qn, sb.qt, two_bm1, g, gf, ga, gb);
    const Adj3 gbr = shdn(gb);
    if (in && lane >= kHalo && lane < kLanes - kHalo) {
      float a1 = 0.f, an = 0.f, at = 0.f;
      if (i >= 1) { a1 += ga.q1; an += ga.qn; at += ga.qt; }
      if (i + 1 <= nx - 1) { a1 += gbr.q1; an += gbr.qn; at += gbr.qt; }
      store_local(li, true, o, Adj3{l.q1 + a1, l.qn + an, l.qt + at});
    }
  }
}

// y sweep: each lane streams one column down a segment of rows [j0, j1),
// carrying the last three rows' states and adjoints, two interfaces' waves
// and the limiter reverses' pending parts in registers. Iteration j loads
// row j, solves interface j, reverses the limiter at j-1 and the solve at
// j-2, and writes the input adjoint of row j-3.
__device__ __forceinline__ void sweep_y_body(const DevParams &p, float dt, const CG3 &s, const CG3 &lo,
                                             const G3 &li, int seg) {
  const int nx = p.nx, ny = p.ny;
  const int lane = threadIdx.x & 31;
  const long long strips = (nx + 31) / 32, nseg = (ny + seg - 1) / seg;
  const long long total = strips * nseg;
  const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
  const float dty = dt / p.dy;
  const float two_bm1 = 2.0f * (p.beta - 1.0f);
  for (long long t = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); t < total; t += nw) {
    const int i = (int)(t % strips) * 32 + lane;
    const int j0 = (int)(t / strips) * seg, j1 = min(ny, j0 + seg);
    const bool col = i < nx;
    auto load = [&](int r, Adj3 &sv, Adj3 &lv) {
      if (col && r >= 0 && r < ny) {
        const size_t o = size_t(i) + size_t(r) * nx;
        sv = load_local(s, false, o);
        lv = load_local(lo, false, o);
      } else {
        sv = Adj3{0.f, 0.f, 0.f};
        lv = Adj3{0.f, 0.f, 0.f};
      }
    };
    Adj3 s1, l1;  // row j-1
    load(j0 - 3, s1, l1);
    Adj3 s2{0.f, 0.f, 0.f}, s3{0.f, 0.f, 0.f}, l2{0.f, 0.f, 0.f}, l3{0.f, 0.f, 0.f};  // rows j-2, j-3
    WaveN w1{0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, w2 = w1;  // interfaces j-1, j-2
    WaveAdj cp1, cp2, c0p;  // cp of the limiter reverses at j-2 and j-3, c0 of the one at j-2
    zero(cp1); zero(cp2); zero(c0p);
    Adj3 gap{0.f, 0.f, 0.f};  // ga of the solve at j-3
    // Iteration j: the waves at interface j (always needed), the limiter's
    // reverse at j-1 (needed from j = j0 on: the limiters at j0-1 .. j1+1
    // feed the solves' reverses at j0 .. j1) and the solve's reverse at j-2
    // (needed from j = j0+2 on). Three compile-time phases keep the loop
    // body free of branches.
    auto iterate = [&](int j, auto do_limiter, auto do_solve) {
      constexpr bool kLimiter = decltype(do_limiter)::value;
      constexpr bool kSolve = decltype(do_solve)::value;
      Adj3 s0, l0;
      load(j, s0, l0);
      const WaveN w0 = sweep_waves(s0, s1, two_bm1, dty, j >= 1 && j <= ny - 1);
      WaveAdj cm, c0, cp;
      zero(cm); zero(c0); zero(cp);
      if constexpr (kLimiter) {
        // the limiter's reverse at interface j-1 (waves j-2, j-1, j)
        const Adj3 mu1 = masked(l1, interior(p, i, j - 1)), mu2 = masked(l2, interior(p, i, j - 2));
        if (j - 1 >= 1 && j - 1 <= ny - 1)
          correction_adj(w2, w1, w0, dty, dty * (mu1.q1 - mu2.q1), dty * (mu1.qn - mu2.qn),
                         dty * (mu1.qt - mu2.qt), cm, c0, cp);
      }
      Adj3 ga{0.f, 0.f, 0.f}, gb{0.f, 0.f, 0.f};
      if constexpr (kSolve) {
        // the waves' adjoint at interface j-2 and the solve's reverse there
        const Adj3 mu2 = masked(l2, interior(p, i, j - 2)), mu3 = masked(l3, interior(p, i, j - 3));
        WaveAdj g = cp2;
        add_to(g, c0p);
        add_to(g, cm);
        FluctAdj gf;
        gf.am1 = -dty * mu3.q1; gf.am2 = -dty * mu3.qn; gf.am3 = -dty * mu3.qt;
        gf.ap1 = -dty * mu2.q1; gf.ap2 = -dty * mu2.qn; gf.ap3 = -dty * mu2.qt;
        if (j - 2 >= 1 && j - 2 <= ny - 1)
          riemann_adj(s2.q1, s2.qn, s2.qt, s3.q1, s3.qn, s3.qt, two_bm1, g, gf, ga, gb);
        // row j-3: lo + ga (solve at j-3) + gb (solve at j-2)
        const int r3 = j - 3;
        if (col && r3 >= j0 && r3 < j1) {
          float a1 = 0.f, an = 0.f, at = 0.f;
          if (r3 >= 1) { a1 += gap.q1; an += gap.qn; at += gap.qt; }
          if (r3 + 1 <= ny - 1) { a1 += gb.q1; an += gb.qn; at += gb.qt; }
          store_local(li, false, size_t(i) + size_t(r3) * nx, Adj3{l3.q1 + a1, l3.qn + an, l3.qt + at});
        }
      }
      s3 = s2; s2 = s1; s1 = s0;
      l3 = l2; l2 = l1; l1 = l0;
      w2 = w1; w1 = w0;
      cp2 = cp1; cp1 = cp; c0p = c0;
      gap = ga;
    };
    const std::true_type on{};
    const std::false_type off{};
    int j = j0 - 2;
    for (; j <= j0 - 1; ++j) iterate(j, off, off);
    for (; j <= j0 + 1; ++j) iterate(j, on, off);
    for (; j <= j1 + 2; ++j) iterate(j, on, on);
  }
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
// `loss`: the loss gradient of the state u1 after the step's input (a
// window of the design's loss, or none) added to the output's u1 adjoint.
struct LossTerm {
  const float *u1;  // nullptr: the step is outside the loss steps
  int i0, j0, ni, nj;
  float coef;
};
__device__ __forceinline__ void boundary_body(const DevParams &p, const CG3 &lb, const G3 &lp, const LossTerm &loss) {
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
  if (loss.u1 && i >= loss.i0 && i < loss.i0 + loss.ni && j >= loss.j0 && j < loss.j0 + loss.nj)
    a[0] += 2.0f * loss.u1[o] * loss.coef;
  lp.f[0][o] = a[0];
  lp.f[1][o] = a[1];
  lp.f[2][o] = a[2];
}

// Weight gradients of one step from the adjoints of the source ghost cells:
// u1 = pack, u2 = pack (pack + 1), pack = amp ramp(T) sin(ISPW T + phase).
// One warp per element: the lanes load the element's ghost cells at once
// (a strided loop when an element spans more than 16 rows), a warp
// reduction in FP64 sums them, and lane 0 updates the element's sums.
__device__ __forceinline__ void weights_body(const DevParams &p, const float *weights, float T, const CG3 &lb,
                                             double *g_amp, double *g_ph, int e, int lane) {
  if (e >= p.nelem) return;  // warp-uniform
  const float amp = weights[e], ph = weights[p.nelem + e];
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


}  // namespace

// ========================================================= batched adjoint
//
// fv_adjoint_batch: D designs of one grid and one set of physical
// parameters (each with its own element weights, loss window and adaptive
// dt schedule) run as one launch sequence: every attempt of the recorded
// forward is one batched attempt (the batch kernels of fv_step.cu over the
// D designs) plus one record launch over all designs; every replayed step
// of the backward is one stage-recording batched attempt; every reverse
// step is one launch per reverse kernel over all designs (blockIdx.y or
// blockIdx.z picks the design). The reverse kernels below take their
// design's buffers from a descriptor array; fv_adjoint launches the same
// kernels with a one-design array, so the two give the same gradients bit
// for bit (the reverse kernels are built with FMA contraction, whose
// choices could differ between two kernels that inline the same body).

namespace {

// Where one design's buffers live (device copy in fv_adjoint_batch::ddesc).
struct AdjDesign {
  float *weights;             // amplitudes then phases
  float *sched_dt, *sched_T;  // nsteps each
  float *state[2][3];
  float *ckpt, *seg, *stg;    // bases of nckpt, C + 1 and 3 C states (3 grids each)
  float *lam[2][3], *tmp[2][3];
  double *acc;                // loss sum, then gradient sums (2 nelem)
  Ctrl *ctrl;
  AdjRec *rec;                // two slots, by attempt parity
  int i0, j0, ni, nj;
  long long first, last;
  float loss_coef;            // 1 / (loss steps x window cells), rounded once
};

// Up to kDesignsPerLaunch designs' descriptors by value, as a kernel
// parameter: parameter space cannot alias the kernels' stores, so the
// compiler re-reads the buffers' addresses from it where a descriptor in
// global memory would hold them in registers through the sweeps' loops.
constexpr int kDesignsPerLaunch = 16;
struct AdjDesignSet {
  AdjDesign d[kDesignsPerLaunch];
};

__device__ __forceinline__ CG3 cstate(const float *base, size_t stride, long long k) {
  return CG3{{base + (size_t(k) * 3 + 0) * stride, base + (size_t(k) * 3 + 1) * stride,
              base + (size_t(k) * 3 + 2) * stride}};
}
// stage grid triple st (0 = B, 1 = S1, 2 = S2) of the segment's k-th step
__device__ __forceinline__ CG3 cstage(const float *stg, size_t stride, long long k, int st) {
  return cstate(stg, stride, k * 3 + st);
}
__device__ __forceinline__ CG3 cg(const float *const f[3]) { return CG3{{f[0], f[1], f[2]}}; }
__device__ __forceinline__ G3 gg(float *const f[3]) { return G3{{f[0], f[1], f[2]}}; }

// Every design back to rest: control block (dt = DTINI, T = -TIDE,
// `remaining` steps), the record slot before attempt 0, the loss sum.
__global__ void adjb_reset_kernel(const AdjDesign *D, int nd, float dt, float T, long long remaining) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nd) return;
  Ctrl *c = D[d].ctrl;
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
  c->last_accepted = 0;
  AdjRec &r = D[d].rec[0];
  r.dt0 = dt;
  r.T0 = T;
  r.n0 = 0;
  r.accepted = 0;
  D[d].acc[0] = 0.0;
}

// The record launch of a batched forward attempt (record_body per design).
__global__ void adjb_record_kernel(const __grid_constant__ AdjDesignSet D, int parity, int nsteps, size_t stride,
                                   size_t ncell, int every, int nx) {
  const AdjDesign &a = D.d[blockIdx.y];
  record_body(a.ctrl, a.rec, parity, a.sched_dt, a.sched_T, nsteps, gg(a.state[0]), gg(a.state[1]), a.ckpt, stride,
              ncell, every, nx, a.i0, a.j0, a.ni, a.nj, a.first, a.last, a.acc);
}

// Before the replay of step n (0-based: the step from u_n, segment slot
// `slot`): every design's control block from its frozen schedule, its
// instance's input, output and stage grids in the segment buffers, a
// negative eigenvalue met by the previous replay counted in `rejected`,
// and the batch's fix-up header and CFL accumulator reset.
__global__ void adjb_sched_kernel(const AdjDesign *D, BatchInst *inst, int nd, int n, int slot, size_t stride,
                                  uint32_t *fix, int32_t *neg, uint32_t *cfl_bits) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d == 0) {
    fix[0] = 0u;
    fix[1] = 0u;
  }
  if (d >= nd) return;
  const AdjDesign &a = D[d];
  Ctrl *c = a.ctrl;
  if (neg[d]) c->rejected += 1;
  neg[d] = 0;
  cfl_bits[d] = 0u;
  c->dt = a.sched_dt[n];
  c->T = a.sched_T[n];
  c->n = n;
  c->cur = 0;
  c->status = 0;
  c->neg_flag = 0;
  c->sim_error = 0;
  c->consecutive_rejects = 0;
  c->mdx = 0;
  c->mdy = 0;
  c->remaining = 1;
  c->t_stop = __int_as_float(0x7f800000);
  BatchInst &I = inst[d];
  for (int f = 0; f < 3; ++f) {
    I.state[0][f] = a.seg + (size_t(slot) * 3 + f) * stride;
    I.state[1][f] = a.seg + (size_t(slot + 1) * 3 + f) * stride;
    for (int st = 0; st < 3; ++st) I.stages[3 * st + f] = a.stg + ((size_t(slot) * 3 + st) * 3 + f) * stride;
  }
}

// Every design's instance back on its forward state pair.
__global__ void adjb_forward_inst_kernel(const AdjDesign *D, BatchInst *inst, int nd) {
  const int d = blockIdx.x * blockDim.x + threadIdx.x;
  if (d >= nd) return;
  for (int b = 0; b < 2; ++b)
    for (int f = 0; f < 3; ++f) inst[d].state[b][f] = D[d].state[b][f];
}

// Reverse step n (input u_{n-1}, segment slot `slot`): diffusion and x sweep,
// lam[lc] -> tmp[1].
__global__ void __launch_bounds__(128) adjb_sweep_x_kernel(DevParams p, const __grid_constant__ AdjDesignSet D,
                                                           int n, int slot, int lc, size_t stride) {
  const AdjDesign &a = D.d[blockIdx.y];
  sweep_x_body(p, a.sched_dt[n - 1], cstage(a.stg, stride, slot, 1), cstage(a.stg, stride, slot, 2), cg(a.lam[lc]),
               gg(a.tmp[1]));
}

// y sweep: tmp[1] -> tmp[0].
__global__ void __launch_bounds__(128) adjb_sweep_y_kernel(DevParams p, const __grid_constant__ AdjDesignSet D,
                                                           int n, int slot, int seg, size_t stride) {
  const AdjDesign &a = D.d[blockIdx.y];
  sweep_y_body(p, a.sched_dt[n - 1], cstage(a.stg, stride, slot, 0), cg(a.tmp[1]), gg(a.tmp[0]), seg);
}

// Weight gradients of reverse step n from tmp[0] (a warp per element).
__global__ void __launch_bounds__(128) adjb_weights_kernel(DevParams p, const __grid_constant__ AdjDesignSet D, int n) {
  const AdjDesign &a = D.d[blockIdx.y];
  weights_body(p, a.weights, a.sched_T[n - 1], cg(a.tmp[0]), a.acc + 1, a.acc + 1 + p.nelem,
               (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), (int)(threadIdx.x & 31));
}

// The boundary reverse of step n (input u_{n-1}, segment slot `slot`):
// tmp[0] -> lam[lc ^ 1], with the loss gradient of u_{n-1} added where the
// step is among the loss steps.
__global__ void adjb_boundary_kernel(DevParams p, const __grid_constant__ AdjDesignSet D, int n, int slot, int lc,
                                     size_t stride) {
  const AdjDesign &a = D.d[blockIdx.z];
  const long long m = n - 1;  // the loss of the state after accepted step m
  LossTerm loss{nullptr, a.i0, a.j0, a.ni, a.nj, 0.0f};
  if (m >= a.first && m <= a.last) {
    loss.u1 = a.seg + size_t(slot) * 3 * stride;
    loss.coef = a.loss_coef;
  }
  boundary_body(p, cg(a.tmp[0]), gg(a.lam[lc ^ 1]), loss);
}

// The loss gradient of the state after accepted step m (segment slot
// `slot`, or the final forward state when slot < 0) into lam[lc], for the
// designs whose loss steps include m.
__global__ void adjb_loss_grad_kernel(const __grid_constant__ AdjDesignSet D, int m, int slot, int lc, int final_cur,
                                      int nx, size_t stride) {
  const AdjDesign &a = D.d[blockIdx.y];
  if (m < a.first || m > a.last) return;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.ni * a.nj) return;
  const float coef = a.loss_coef;
  const float *u1 = slot < 0 ? a.state[final_cur][0] : a.seg + size_t(slot) * 3 * stride;
  const size_t o = size_t(a.i0 + k % a.ni) + size_t(a.j0 + k / a.ni) * nx;
  a.lam[lc][0][o] += 2.0f * u1[o] * coef;
}

}  // namespace

// ------------------------------------------------------------------ handle

// The loss's weight of one window cell and step (the device kernels read
// it from the descriptor: an FP64 division per thread is slow on this GPU).
static float loss_coef(const fv_loss_window &w) {
  return float(1.0 / (double(w.step_last - w.step_first + 1) * double(w.ni) * double(w.nj)));
}

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
  cudaGraphExec_t seg_graph = nullptr;  // the backward's segment graph
  cudaGraphExec_t rec_graph = nullptr;  // the recorded forward's attempts
  Fork fork;                            // the weights' branch of a reverse step
  // device memory: one allocation of grids, plus small arrays
  float *mem = nullptr;
  float *state[2][3] = {};      // forward state pair
  float *ckpt = nullptr;        // nckpt states
  float *seg = nullptr;         // C + 1 states of the segment being reversed
  float *stg = nullptr;         // C stage triples (B, S1, S2) of the segment's steps
  float *lam[2][3] = {};        // adjoint ping-pong
  float *tmp[2][3] = {};        // sweep adjoints
  float *frame = nullptr;
  float *weights = nullptr;     // amplitudes then phases
  Ctrl *ctrl = nullptr;
  AdjRec *rec = nullptr;
  float *partials = nullptr;
  uint32_t *fix = nullptr;
  size_t fix_words = 0;
  int nblocks = 0, fix_blocks = 0, nstrips = 0;
  int sweep_x_blocks = 0, sweep_y_blocks = 0, sweep_y_seg = 0;  // launch shapes of the reverse sweeps
  float *sched = nullptr;       // dt[nsteps] then T[nsteps]
  double *acc = nullptr;        // loss sum, then gradient sums (2 nelem)
  std::vector<float> h_dt, h_T;
  bool have_schedule = false;  // a recorded dt schedule (replays need it)
  bool have_forward = false;   // checkpoints of the recorded run (the backward needs them)
  int final_cur = 0;           // state[final_cur] holds the last forward's final state
                               // (the backward's replays reuse the control block)
  int exact = 1;
  AdjDesignSet desc{};         // this design's buffers for the reverse kernels (entry 0)
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
  s.div_exact = 1;  // exact division in the step kernel, as fv_create's default
  return s;
}

int launch(const fv_adjoint *a, const StepArgs &s, int stage) {
  return a->exact ? launch_step_exact(s, kWarpsPerStep, stage, a->stream)
                  : launch_step_fast(s, kWarpsPerStep, stage, a->stream);
}

G3 g3(float *const f[3]) { return G3{{f[0], f[1], f[2]}}; }

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
    long long attempt = 0;
    adj_pre_kernel<<<1, 1, 0, a->stream>>>(a->ctrl, a->rec);  // the scalars before attempt 0
    auto one = [&](long long k) -> fv_status {
      const int rc = launch(a, s, -1);
      if (rc != 0) return afail(FV_CUDA_ERROR, "step launch: %s", cudaGetErrorString((cudaError_t)rc));
      adjb_record_kernel<<<dim3(cgrid, 1), 256, 0, a->stream>>>(a->desc, int(k & 1), int(a->nsteps), a->stride,
                                                                a->ncell, a->every, P.nx);
      return FV_OK;
    };
    for (int round = 0; round < 64 && todo > 0; ++round) {
      const fv_status rs = run_attempts(a->stream, a->rec_graph, attempt, todo, one);
      if (rs != FV_OK) return rs;
      attempt += todo;
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
      adj_loss_kernel<<<1, 256, 0, a->stream>>>(a->ctrl, s0, s1, P.nx, w.i0, w.j0, w.ni, w.nj,
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
  // triples 3x3, lam 2x3, tmp 2x3
  const size_t nstates = 2 + size_t(a->nckpt) + size_t(a->every + 1) + 3 * size_t(a->every) + 2 + 2;
  const size_t ngrids = nstates * 3;
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

  const int strip_c = kWarpsPerStep * kWarpCols;
  a->nstrips = (p->nx + strip_c - 1) / strip_c;
  const long long work = (long long)a->nstrips * p->ny;
  const int per_sm = a->exact ? max_blocks_per_sm_exact(kWarpsPerStep, -1) : max_blocks_per_sm_fast(kWarpsPerStep, -1);
  a->max_resident = per_sm * a->sms;
  a->nblocks = int(std::max(1LL, std::min((long long)a->max_resident, work / 32)));  // one wave
  a->fix_blocks = 4 * a->sms;
  // reverse sweeps: grid-stride warps, as many CTAs as are resident at once
  {
    int ox = 0, oy = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ox, adjb_sweep_x_kernel, 128, 0) != cudaSuccess || ox < 1) ox = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&oy, adjb_sweep_y_kernel, 128, 0) != cudaSuccess || oy < 1) oy = 1;
    const long long xwarps = (long long)((p->nx + kWarpCols - 1) / kWarpCols) * p->ny;
    a->sweep_x_blocks = int(std::max(1LL, std::min((long long)ox * a->sms, (xwarps + 3) / 4)));
    // y sweep: enough row segments to fill the resident warps, at least 16 rows each
    const long long strips = (p->nx + 31) / 32, ywarps = 4LL * oy * a->sms;
    const long long nseg = std::max(1LL, std::min((long long)(p->ny + 15) / 16, ywarps / strips));
    a->sweep_y_seg = int((p->ny + nseg - 1) / nseg);
    const long long ytotal = strips * ((p->ny + a->sweep_y_seg - 1) / a->sweep_y_seg);
    a->sweep_y_blocks = int(std::max(1LL, std::min((long long)oy * a->sms, (ytotal + 3) / 4)));
  }
  a->fix_words = size_t(fix_scratch_words((long long)a->nstrips * kWarpsPerStep, p->ny));
  e = cudaMalloc(&a->frame, 3 * size_t(frame_cells(p->nx, p->ny)) * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&a->weights, 2 * size_t(p->array_elems) * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&a->ctrl, sizeof(Ctrl));
  if (e == cudaSuccess) e = cudaMalloc(&a->rec, 2 * sizeof(AdjRec));  // two slots, by attempt parity
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
  {
    // this design's buffers, as the reverse kernels read them
    AdjDesign d{};
    d.weights = a->weights;
    d.sched_dt = a->sched;
    d.sched_T = a->sched + nsteps;
    for (int b = 0; b < 2; ++b)
      for (int f = 0; f < 3; ++f) {
        d.state[b][f] = a->state[b][f];
        d.lam[b][f] = a->lam[b][f];
        d.tmp[b][f] = a->tmp[b][f];
      }
    d.ckpt = a->ckpt;
    d.seg = a->seg;
    d.stg = a->stg;
    d.acc = a->acc;
    d.ctrl = a->ctrl;
    d.rec = a->rec;
    d.i0 = w->i0;
    d.j0 = w->j0;
    d.ni = w->ni;
    d.nj = w->nj;
    d.first = w->step_first;
    d.last = w->step_last;
    d.loss_coef = loss_coef(*w);
    a->desc.d[0] = d;
  }
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
  if (a->seg_graph) cudaGraphExecDestroy(a->seg_graph);
  if (a->rec_graph) cudaGraphExecDestroy(a->rec_graph);
  a->fork.release();
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
  FVA_CUDA(a->fork.init());
  const fv_params &P = a->params;
  const int nx = P.nx, ny = P.ny, nelem = P.array_elems;
  const fv_loss_window &w = a->win;
  const dim3 blk(kBX, kBY), grd((nx + kBX - 1) / kBX, (ny + kBY - 1) / kBY);
  const int wthreads = w.ni * w.nj, wblocks = (wthreads + 255) / 256;
  double *g_amp = a->acc + 1, *g_ph = a->acc + 1 + nelem;
  FVA_CUDA(cudaMemsetAsync(g_amp, 0, 2 * size_t(nelem) * sizeof(double), a->stream));
  // the replays count the negative eigenvalues they meet here (none, unless
  // a replay differs from the recorded forward)
  FVA_CUDA(cudaMemsetAsync(&a->ctrl->rejected, 0, sizeof(a->ctrl->rejected), a->stream));
  FVA_CUDA(cudaMemsetAsync(&a->ctrl->neg_flag, 0, sizeof(a->ctrl->neg_flag), a->stream));
  const size_t bytes = 3 * a->stride * sizeof(float);
  // lambda_N: the loss gradient of the final state
  int lc = 0;  // lam[lc] holds lambda_n
  FVA_CUDA(cudaMemsetAsync(a->lam[lc][0], 0, bytes, a->stream));
  adjb_loss_grad_kernel<<<dim3(wblocks, 1), 256, 0, a->stream>>>(a->desc, int(a->nsteps), -1, lc, a->final_cur, nx,
                                                                  a->stride);
  const long long C = a->every;
  for (long long seg0 = ((a->nsteps - 1) / C) * C; seg0 >= 0; seg0 -= C) {
    const long long seg1 = std::min(seg0 + C, a->nsteps);  // steps seg0+1 .. seg1
    const fv_status rs = run_captured(a->stream, a->seg_graph, [&]() -> fv_status {
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
        adj_sched_kernel<<<1, 1, 0, a->stream>>>(a->ctrl, a->sched, a->sched + a->nsteps, int(n - 1), 0, a->fix);
        StepArgs s = step_args(a, a->dp_replay, in, out);
        for (int st = 0; st < 3; ++st)
          for (int f = 0; f < 3; ++f) s.stages[3 * st + f] = stage_grid(a, n - 1 - seg0, st, f);
        const int rc = launch(a, s, kStageReplay);
        if (rc != 0) return afail(FV_CUDA_ERROR, "replay launch: %s", cudaGetErrorString((cudaError_t)rc));
      }
      for (long long n = seg1; n > seg0; --n) {
        // reverse of step n, whose input is u_{n-1} (segment slot n-1-seg0;
        // its recorded boundary-applied, y-swept and x-swept states are the
        // slot's stage grids)
        const int slot = int(n - 1 - seg0);
        // diffusion (on S2) and x sweep (on S1): lam[lc] -> tmp1 (adjoint of S1)
        adjb_sweep_x_kernel<<<dim3(a->sweep_x_blocks, 1), 128, 0, a->stream>>>(a->dp, a->desc, int(n), slot, lc,
                                                                               a->stride);
        // y sweep on B: tmp1 -> tmp0 (adjoint of B)
        adjb_sweep_y_kernel<<<dim3(a->sweep_y_blocks, 1), 128, 0, a->stream>>>(a->dp, a->desc, int(n), slot,
                                                                               a->sweep_y_seg, a->stride);
        // the weights' gradient (side branch) beside the boundary with the
        // loss gradient of u_{n-1}: lam[lc ^ 1] = lam_{n-1}; both read tmp0,
        // which the next y sweep overwrites after the join
        FVA_CUDA(a->fork.fork(a->stream));
        adjb_weights_kernel<<<dim3((nelem + 3) / 4, 1), 128, 0, a->fork.side>>>(a->dp, a->desc, int(n));
        adjb_boundary_kernel<<<dim3(grd.x, grd.y, 1), blk, 0, a->stream>>>(a->dp, a->desc, int(n), slot, lc,
                                                                            a->stride);
        FVA_CUDA(a->fork.join(a->stream));
        lc ^= 1;
      }
      FVA_CUDA(cudaGetLastError());
      return FV_OK;
    });
    if (rs != FV_OK) return rs;
  }
  FVA_CUDA(cudaStreamSynchronize(a->stream));
  {
    Ctrl c;
    FVA_CUDA(cudaMemcpy(&c, a->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost));
    if (c.rejected != 0 || c.neg_flag != 0)
      return afail(FV_NEGATIVE_EIGENVALUE, "a replay of the recorded forward met a negative eigenvalue");
  }
  FVA_CUDA(cudaMemcpy(grad_amp, g_amp, sizeof(double) * nelem, cudaMemcpyDeviceToHost));
  FVA_CUDA(cudaMemcpy(grad_phase, g_ph, sizeof(double) * nelem, cudaMemcpyDeviceToHost));
  return FV_OK;
}

}  // extern "C"

struct fv_adjoint_batch {
  fv_params params{};
  DevParams dp{};
  int nd = 0;                   // designs
  long long nsteps = 0;
  int every = 1, nckpt = 0;
  int sms = 0;
  size_t ncell = 0, stride = 0;
  int exact = 1;
  cudaStream_t stream = nullptr, own_stream = nullptr;
  cudaGraphExec_t seg_graph = nullptr;  // the backward's segment graph
  cudaGraphExec_t rec_graph = nullptr;  // the recorded forward's attempts
  Fork fork;                            // the weights' branch of a reverse step
  std::vector<fv_loss_window> win;
  std::vector<float *> mem;     // per design: all grids
  std::vector<AdjDesign> hdesc;
  AdjDesign *ddesc = nullptr;   // device copy (the control-block kernels)
  std::vector<AdjDesignSet> sets;  // by value, kDesignsPerLaunch designs a launch (the reverse kernels)
  float *small = nullptr;       // weights, schedules of every design
  double *acc = nullptr;        // per design: 1 + 2 nelem
  Ctrl *ctrl = nullptr;         // per design
  AdjRec *rec = nullptr;        // per design: 2 slots
  // the batch kernels' arguments over the D designs
  std::vector<BatchInst> hinst;
  BatchInst *inst = nullptr;
  uint32_t *cfl_bits = nullptr;
  int32_t *neg = nullptr;
  uint32_t *fix = nullptr;
  size_t fix_words = 0;
  float *frame = nullptr;
  BatchArgs args{};
  int sweep_x_blocks = 0, sweep_y_blocks = 0, sweep_y_seg = 0;
  std::vector<int> final_cur;
  bool have_forward = false;
  std::vector<std::vector<float>> h_dt, h_T;
};

namespace {

// designs in group g of the batch's descriptor sets
int group_size(const fv_adjoint_batch *b, size_t g) {
  return std::min(kDesignsPerLaunch, b->nd - int(g) * kDesignsPerLaunch);
}

int launch_b(const fv_adjoint_batch *b, bool replay) {
  if (replay) return b->exact ? launch_batch_replay_exact(b->args, b->stream) : launch_batch_replay_fast(b->args, b->stream);
  return b->exact ? launch_batch_exact(b->args, b->stream) : launch_batch_fast(b->args, b->stream);
}

}  // namespace

extern "C" {

fv_status fv_adjoint_batch_create(const fv_params *p, int32_t ndesigns, const fv_loss_window *windows,
                                  int64_t nsteps, int32_t checkpoint_every, fv_adjoint_batch **out) {
  if (!p || !windows || !out || ndesigns < 1 || ndesigns > 1024) return afail(FV_BAD_ARG, "bad argument");
  *out = nullptr;
  fv_status s = validate_params(p);
  if (s != FV_OK) return s;
  if (p->app != FV_APP_PHASED_ARRAY) return afail(FV_BAD_ARG, "the adjoint is for the phased array app");
  if (p->moving_domain) return afail(FV_BAD_ARG, "the adjoint needs moving_domain = 0");
  if (nsteps < 1 || nsteps > (1LL << 24)) return afail(FV_BAD_ARG, "nsteps must be 1..2^24");
  for (int d = 0; d < ndesigns; ++d) {
    const fv_loss_window &w = windows[d];
    if (w.ni < 1 || w.nj < 1 || w.i0 < 0 || w.j0 < 0 || w.i0 + w.ni > p->nx || w.j0 + w.nj > p->ny)
      return afail(FV_BAD_ARG, "loss window %d outside the grid", d);
    if (w.step_first < 1 || w.step_last < w.step_first || w.step_last > nsteps)
      return afail(FV_BAD_ARG, "loss steps of window %d must satisfy 1 <= first <= last <= nsteps", d);
  }
  int dev = 0;
  FVA_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  FVA_CUDA(cudaGetDeviceProperties(&prop, dev));
  if (prop.major != 10 || prop.minor != 3) return afail(FV_NO_DEVICE, "device is not sm_103");
  fv_adjoint_batch *b = new (std::nothrow) fv_adjoint_batch();
  if (!b) return afail(FV_CUDA_ERROR, "out of host memory");
  auto cleanup = [&](fv_status st) {
    fv_adjoint_batch_destroy(b);
    return st;
  };
  b->params = *p;
  b->nd = ndesigns;
  b->nsteps = nsteps;
  b->exact = p->exact ? 1 : 0;
  b->every = checkpoint_every > 0 ? checkpoint_every : std::max(1, int(std::ceil(std::sqrt(double(nsteps)))));
  b->nckpt = int(nsteps / b->every) + 1;
  b->ncell = size_t(p->nx) * size_t(p->ny);
  b->stride = (b->ncell + 63) & ~size_t(63);
  b->sms = prop.multiProcessorCount;
  b->dp = dev_params_of(*p);
  b->win.assign(windows, windows + ndesigns);
  b->final_cur.assign(ndesigns, 0);
  b->h_dt.resize(ndesigns);
  b->h_T.resize(ndesigns);
  const int nelem = p->array_elems;
  const size_t nstates = 2 + size_t(b->nckpt) + size_t(b->every + 1) + 3 * size_t(b->every) + 2 + 2;
  const size_t fcells = size_t(frame_cells(p->nx, p->ny));
  const size_t fstride = (fcells + 63) & ~size_t(63);
  cudaError_t e = cudaSuccess;
  b->mem.assign(ndesigns, nullptr);
  for (int d = 0; d < ndesigns && e == cudaSuccess; ++d) e = cudaMalloc(&b->mem[d], nstates * 3 * b->stride * sizeof(float));
  if (e != cudaSuccess)
    return cleanup(afail(FV_CUDA_ERROR, "cudaMalloc adjoint grids (%d designs of %zu MB): %s", ndesigns,
                         nstates * 3 * b->stride * 4 >> 20, cudaGetErrorString(e)));
  const size_t small_per = 2 * size_t(nelem) + 2 * size_t(nsteps);
  e = cudaMalloc(&b->small, small_per * ndesigns * sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&b->acc, (1 + 2 * size_t(nelem)) * ndesigns * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&b->ctrl, sizeof(Ctrl) * ndesigns);
  if (e == cudaSuccess) e = cudaMalloc(&b->rec, 2 * sizeof(AdjRec) * ndesigns);
  if (e == cudaSuccess) e = cudaMalloc(&b->ddesc, sizeof(AdjDesign) * ndesigns);
  if (e == cudaSuccess) e = cudaMalloc(&b->inst, sizeof(BatchInst) * ndesigns);
  if (e == cudaSuccess) e = cudaMalloc(&b->cfl_bits, sizeof(uint32_t) * ndesigns);
  if (e == cudaSuccess) e = cudaMalloc(&b->neg, sizeof(int32_t) * ndesigns);
  if (e == cudaSuccess) e = cudaMalloc(&b->frame, 3 * fstride * ndesigns * sizeof(float));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cleanup(afail(FV_CUDA_ERROR, "adjoint batch allocation: %s", cudaGetErrorString(e)));
  b->stream = b->own_stream;

  // per design: its grids (as fv_adjoint lays them out), weights, schedule
  b->hdesc.resize(ndesigns);
  b->hinst.resize(ndesigns);
  const int windows_x = (p->nx + kWarpCols - 1) / kWarpCols;
  long long work = 0, cost = 0, fix_chunks = 0;
  for (int d = 0; d < ndesigns; ++d) {
    AdjDesign &a = b->hdesc[d];
    float *cur = b->mem[d];
    auto take = [&](size_t nst) {
      float *r = cur;
      cur += nst * 3 * b->stride;
      return r;
    };
    for (int k = 0; k < 2; ++k) {
      float *base = take(1);
      for (int f = 0; f < 3; ++f) a.state[k][f] = base + f * b->stride;
    }
    a.ckpt = take(b->nckpt);
    a.seg = take(b->every + 1);
    a.stg = take(3 * size_t(b->every));
    for (int k = 0; k < 2; ++k) {
      float *base = take(1);
      for (int f = 0; f < 3; ++f) a.lam[k][f] = base + f * b->stride;
    }
    for (int k = 0; k < 2; ++k) {
      float *base = take(1);
      for (int f = 0; f < 3; ++f) a.tmp[k][f] = base + f * b->stride;
    }
    float *sm = b->small + small_per * d;
    a.weights = sm;
    a.sched_dt = sm + 2 * nelem;
    a.sched_T = sm + 2 * nelem + nsteps;
    a.acc = b->acc + (1 + 2 * size_t(nelem)) * d;
    a.ctrl = b->ctrl + d;
    a.rec = b->rec + 2 * d;
    const fv_loss_window &w = windows[d];
    a.i0 = w.i0;
    a.j0 = w.j0;
    a.ni = w.ni;
    a.nj = w.nj;
    a.first = w.step_first;
    a.last = w.step_last;
    a.loss_coef = loss_coef(w);

    BatchInst &I = b->hinst[d];
    std::memset(&I, 0, sizeof(I));
    I.p = b->dp;
    I.p.weights = a.weights;
    for (int k = 0; k < 2; ++k)
      for (int f = 0; f < 3; ++f) I.state[k][f] = a.state[k][f];
    for (int f = 0; f < 3; ++f) I.frame[f] = b->frame + (3 * size_t(d) + f) * fstride;
    I.ctrl = a.ctrl;
    I.work_begin = work;
    I.work = (long long)windows_x * p->ny;
    work += I.work;
    I.cost_begin = cost;
    I.cost = ShareCost(p->nx, p->ny).total();
    cost += I.cost;
    I.fix_base = fix_chunks;
    fix_chunks += (long long)windows_x * fix_chunks_per_window(p->ny);
  }
  if (fix_chunks >= (1LL << 32)) return cleanup(afail(FV_BAD_ARG, "batch above 2^32 fix-up chunks"));
  b->fix_words = size_t(4 + (fix_chunks + 31) / 32 + 2 * fix_chunks);
  e = cudaMalloc(&b->fix, b->fix_words * sizeof(uint32_t));
  if (e != cudaSuccess) return cleanup(afail(FV_CUDA_ERROR, "cudaMalloc fix-up scratch: %s", cudaGetErrorString(e)));
  FVA_CUDA(cudaMemcpyAsync(b->ddesc, b->hdesc.data(), sizeof(AdjDesign) * ndesigns, cudaMemcpyHostToDevice, b->stream));
  for (int g0 = 0; g0 < ndesigns; g0 += kDesignsPerLaunch) {
    AdjDesignSet set{};
    for (int k = 0; k < kDesignsPerLaunch && g0 + k < ndesigns; ++k) set.d[k] = b->hdesc[g0 + k];
    b->sets.push_back(set);
  }
  FVA_CUDA(cudaMemcpyAsync(b->inst, b->hinst.data(), sizeof(BatchInst) * ndesigns, cudaMemcpyHostToDevice, b->stream));
  FVA_CUDA(cudaMemsetAsync(b->fix, 0, b->fix_words * sizeof(uint32_t), b->stream));
  FVA_CUDA(cudaMemsetAsync(b->cfl_bits, 0, sizeof(uint32_t) * ndesigns, b->stream));
  FVA_CUDA(cudaMemsetAsync(b->neg, 0, sizeof(int32_t) * ndesigns, b->stream));
  FVA_CUDA(cudaMemsetAsync(b->frame, 0, 3 * fstride * ndesigns * sizeof(float), b->stream));
  {
    // every design starts with every element at amplitude AMPL and phase 0
    std::vector<float> w0(2 * size_t(nelem), 0.0f);
    for (int k = 0; k < nelem; ++k) w0[k] = float(p->ampl);
    for (int d = 0; d < ndesigns; ++d)
      FVA_CUDA(cudaMemcpyAsync(b->hdesc[d].weights, w0.data(), w0.size() * sizeof(float), cudaMemcpyHostToDevice,
                               b->stream));
    FVA_CUDA(cudaStreamSynchronize(b->stream));  // w0 is a host temporary
  }
  const int per_sm = b->exact ? max_batch_blocks_per_sm_exact() : max_batch_blocks_per_sm_fast();
  const long long resident = (long long)per_sm * b->sms;
  BatchArgs &A = b->args;
  A.inst = b->inst;
  A.cfl_bits = b->cfl_bits;
  A.neg = b->neg;
  A.fix = b->fix;
  A.n = ndesigns;
  A.work = work;
  A.cost = cost;
  A.fix_chunks = fix_chunks;
  A.max_frame = 4 * p->nx + 4 * (p->ny - 4);
  A.fix_blocks = 4 * b->sms;
  // eight waves of resident CTAs (fv_batch's default), at least 128 rows a CTA
  A.nblocks = int(std::max(1LL, std::min(8 * resident, work / 128)));
  {
    int ox = 0, oy = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ox, adjb_sweep_x_kernel, 128, 0) != cudaSuccess || ox < 1) ox = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&oy, adjb_sweep_y_kernel, 128, 0) != cudaSuccess || oy < 1) oy = 1;
    // the y sweep's row segments as for one design; the CTAs of both sweeps
    // are spread over the designs (gridDim.y)
    const long long xwarps = (long long)windows_x * p->ny;
    const long long per_launch = std::min(ndesigns, kDesignsPerLaunch);
    b->sweep_x_blocks = int(std::max(1LL, std::min(std::max(1LL, (long long)ox * b->sms / per_launch), (xwarps + 3) / 4)));
    const long long strips = (p->nx + 31) / 32, ywarps = 4LL * oy * b->sms;
    const long long nseg = std::max(1LL, std::min((long long)(p->ny + 15) / 16, ywarps / strips));
    b->sweep_y_seg = int((p->ny + nseg - 1) / nseg);
    const long long ytotal = strips * ((p->ny + b->sweep_y_seg - 1) / b->sweep_y_seg);
    b->sweep_y_blocks = int(std::max(1LL, std::min(std::max(1LL, (long long)oy * b->sms / per_launch), (ytotal + 3) / 4)));
  }
  e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return cleanup(afail(FV_CUDA_ERROR, "adjoint batch set-up: %s", cudaGetErrorString(e)));
  *out = b;
  return FV_OK;
}

fv_status fv_adjoint_batch_destroy(fv_adjoint_batch *b) {
  if (!b) return FV_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (float *m : b->mem)
    if (m) cudaFree(m);
  if (b->small) cudaFree(b->small);
  if (b->acc) cudaFree(b->acc);
  if (b->ctrl) cudaFree(b->ctrl);
  if (b->rec) cudaFree(b->rec);
  if (b->ddesc) cudaFree(b->ddesc);
  if (b->inst) cudaFree(b->inst);
  if (b->cfl_bits) cudaFree(b->cfl_bits);
  if (b->neg) cudaFree(b->neg);
  if (b->fix) cudaFree(b->fix);
  if (b->frame) cudaFree(b->frame);
  if (b->seg_graph) cudaGraphExecDestroy(b->seg_graph);
  if (b->rec_graph) cudaGraphExecDestroy(b->rec_graph);
  b->fork.release();
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
  return FV_OK;
}

fv_status fv_adjoint_batch_set_stream(fv_adjoint_batch *b, void *cuda_stream) {
  if (!b) return afail(FV_BAD_ARG, "NULL argument");
  FVA_CUDA(cudaStreamSynchronize(b->stream));
  b->stream = cuda_stream ? (cudaStream_t)cuda_stream : b->own_stream;
  return FV_OK;
}

fv_status fv_adjoint_batch_forward(fv_adjoint_batch *b, const float *amp, const float *phase, double *loss) {
  if (!b || !amp || !phase) return afail(FV_BAD_ARG, "NULL argument");
  const fv_params &P = b->params;
  const int nelem = P.array_elems, nd = b->nd;
  b->have_forward = false;
  const size_t bytes = 3 * b->stride * sizeof(float);
  for (int d = 0; d < nd; ++d) {
    const AdjDesign &a = b->hdesc[d];
    FVA_CUDA(cudaMemcpyAsync(a.weights, amp + size_t(d) * nelem, sizeof(float) * nelem, cudaMemcpyHostToDevice,
                             b->stream));
    FVA_CUDA(cudaMemcpyAsync(a.weights + nelem, phase + size_t(d) * nelem, sizeof(float) * nelem,
                             cudaMemcpyHostToDevice, b->stream));
    for (int k = 0; k < 2; ++k) FVA_CUDA(cudaMemsetAsync(a.state[k][0], 0, bytes, b->stream));
    FVA_CUDA(cudaMemsetAsync(a.ckpt, 0, bytes, b->stream));  // checkpoint 0: the initial state
  }
  FVA_CUDA(cudaMemsetAsync(b->fix, 0, b->fix_words * sizeof(uint32_t), b->stream));
  FVA_CUDA(cudaMemsetAsync(b->cfl_bits, 0, sizeof(uint32_t) * nd, b->stream));
  FVA_CUDA(cudaMemsetAsync(b->neg, 0, sizeof(int32_t) * nd, b->stream));
  const int tb = 128, tg = (nd + tb - 1) / tb;
  adjb_forward_inst_kernel<<<tg, tb, 0, b->stream>>>(b->ddesc, b->inst, nd);
  adjb_reset_kernel<<<tg, tb, 0, b->stream>>>(b->ddesc, nd, float(P.dtini), -float(P.tide), b->nsteps);
  FVA_CUDA(cudaGetLastError());
  const int rx = std::max(1, b->sms * 4 / nd);
  std::vector<Ctrl> hc(nd);
  long long todo = b->nsteps, attempt = 0;
  auto one = [&](long long k) -> fv_status {
    const int rc = launch_b(b, false);
    if (rc != 0) return afail(FV_CUDA_ERROR, "batch step launch: %s", cudaGetErrorString((cudaError_t)rc));
    for (size_t g = 0; g < b->sets.size(); ++g)
      adjb_record_kernel<<<dim3(rx, group_size(b, g)), 256, 0, b->stream>>>(b->sets[g], int(k & 1), int(b->nsteps),
                                                                           b->stride, b->ncell, b->every, P.nx);
    return FV_OK;
  };
  for (int round = 0; round < 64 && todo > 0; ++round) {
    const fv_status rs = run_attempts(b->stream, b->rec_graph, attempt, todo, one);
    if (rs != FV_OK) return rs;
    attempt += todo;
    FVA_CUDA(cudaGetLastError());
    FVA_CUDA(cudaMemcpyAsync(hc.data(), b->ctrl, sizeof(Ctrl) * nd, cudaMemcpyDeviceToHost, b->stream));
    FVA_CUDA(cudaStreamSynchronize(b->stream));
    todo = 0;
    for (int d = 0; d < nd; ++d) {
      if (hc[d].status) return afail((fv_status)hc[d].status, "design %d's forward stopped with status %d", d, hc[d].status);
      todo = std::max<long long>(todo, hc[d].remaining);  // rejected attempts are made up
    }
  }
  if (todo > 0) return afail(FV_DT_TOO_LARGE, "forward run did not finish");
  for (int d = 0; d < nd; ++d) {
    const AdjDesign &a = b->hdesc[d];
    b->final_cur[d] = hc[d].cur & 1;
    b->h_dt[d].resize(b->nsteps);
    b->h_T[d].resize(b->nsteps);
    FVA_CUDA(cudaMemcpy(b->h_dt[d].data(), a.sched_dt, sizeof(float) * b->nsteps, cudaMemcpyDeviceToHost));
    FVA_CUDA(cudaMemcpy(b->h_T[d].data(), a.sched_T, sizeof(float) * b->nsteps, cudaMemcpyDeviceToHost));
    double sum = 0.0;
    FVA_CUDA(cudaMemcpy(&sum, a.acc, sizeof(double), cudaMemcpyDeviceToHost));
    const fv_loss_window &w = b->win[d];
    if (loss) loss[d] = sum / (double(w.step_last - w.step_first + 1) * double(w.ni) * double(w.nj));
  }
  b->have_forward = true;
  return FV_OK;
}

fv_status fv_adjoint_batch_backward(fv_adjoint_batch *b, double *grad_amp, double *grad_phase) {
  if (!b || !grad_amp || !grad_phase) return afail(FV_BAD_ARG, "NULL argument");
  if (!b->have_forward) return afail(FV_BAD_ARG, "no forward run (fv_adjoint_batch_forward) to differentiate");
  FVA_CUDA(b->fork.init());
  const fv_params &P = b->params;
  const int nx = P.nx, ny = P.ny, nelem = P.array_elems, nd = b->nd;
  const size_t bytes = 3 * b->stride * sizeof(float);
  const int tb = 128, tg = (nd + tb - 1) / tb;
  int wmax = 1;
  for (int d = 0; d < nd; ++d) wmax = std::max(wmax, b->win[d].ni * b->win[d].nj);
  const int lx = (wmax + 255) / 256;
  const dim3 bblk(kBX, kBY);
  const int bgx = (nx + kBX - 1) / kBX, bgy = (ny + kBY - 1) / kBY;
  for (int d = 0; d < nd; ++d) {
    const AdjDesign &a = b->hdesc[d];
    FVA_CUDA(cudaMemsetAsync(a.acc + 1, 0, 2 * size_t(nelem) * sizeof(double), b->stream));
    FVA_CUDA(cudaMemsetAsync(&a.ctrl->rejected, 0, sizeof(a.ctrl->rejected), b->stream));
  }
  FVA_CUDA(cudaMemsetAsync(b->neg, 0, sizeof(int32_t) * nd, b->stream));
  // every design takes the same number of accepted steps, so every final
  // state is in the same buffer of its pair
  for (int d = 0; d < nd; ++d)
    if (b->final_cur[d] != b->final_cur[0]) return afail(FV_CUDA_ERROR, "designs end in different buffers");
  // lambda_N: the loss gradient of the final state
  int lc = 0;
  for (int d = 0; d < nd; ++d) FVA_CUDA(cudaMemsetAsync(b->hdesc[d].lam[lc][0], 0, bytes, b->stream));
  for (size_t g = 0; g < b->sets.size(); ++g)
    adjb_loss_grad_kernel<<<dim3(lx, group_size(b, g)), 256, 0, b->stream>>>(b->sets[g], int(b->nsteps), -1, lc,
                                                                             b->final_cur[0], nx, b->stride);
  const long long C = b->every;
  for (long long seg0 = ((b->nsteps - 1) / C) * C; seg0 >= 0; seg0 -= C) {
    const long long seg1 = std::min(seg0 + C, b->nsteps);  // steps seg0+1 .. seg1
    const fv_status rs = run_captured(b->stream, b->seg_graph, [&]() -> fv_status {
      for (int d = 0; d < nd; ++d) {
        const AdjDesign &a = b->hdesc[d];
        FVA_CUDA(cudaMemcpyAsync(a.seg, a.ckpt + size_t(seg0 / C) * 3 * b->stride, bytes, cudaMemcpyDeviceToDevice,
                                 b->stream));
      }
      for (long long n = seg0 + 1; n <= seg1; ++n) {
        adjb_sched_kernel<<<tg, tb, 0, b->stream>>>(b->ddesc, b->inst, nd, int(n - 1), int(n - 1 - seg0), b->stride,
                                                    b->fix, b->neg, b->cfl_bits);
        const int rc = launch_b(b, true);
        if (rc != 0) return afail(FV_CUDA_ERROR, "replay launch: %s", cudaGetErrorString((cudaError_t)rc));
      }
      for (long long n = seg1; n > seg0; --n) {
        const int slot = int(n - 1 - seg0);
        for (size_t g = 0; g < b->sets.size(); ++g) {
          const AdjDesignSet &S = b->sets[g];
          const int gn = group_size(b, g);
          adjb_sweep_x_kernel<<<dim3(b->sweep_x_blocks, gn), 128, 0, b->stream>>>(b->dp, S, int(n), slot, lc,
                                                                                  b->stride);
          adjb_sweep_y_kernel<<<dim3(b->sweep_y_blocks, gn), 128, 0, b->stream>>>(b->dp, S, int(n), slot,
                                                                                  b->sweep_y_seg, b->stride);
          FVA_CUDA(b->fork.fork(b->stream));
          adjb_weights_kernel<<<dim3((nelem + 3) / 4, gn), 128, 0, b->fork.side>>>(b->dp, S, int(n));
          adjb_boundary_kernel<<<dim3(bgx, bgy, gn), bblk, 0, b->stream>>>(b->dp, S, int(n), slot, lc, b->stride);
          FVA_CUDA(b->fork.join(b->stream));
        }
        lc ^= 1;
      }
      FVA_CUDA(cudaGetLastError());
      return FV_OK;
    });
    if (rs != FV_OK) return rs;
  }
  // a negative eigenvalue met by the last replay
  adjb_sched_kernel<<<tg, tb, 0, b->stream>>>(b->ddesc, b->inst, nd, 0, 0, b->stride, b->fix, b->neg, b->cfl_bits);
  FVA_CUDA(cudaStreamSynchronize(b->stream));
  std::vector<Ctrl> hc(nd);
  FVA_CUDA(cudaMemcpy(hc.data(), b->ctrl, sizeof(Ctrl) * nd, cudaMemcpyDeviceToHost));
  for (int d = 0; d < nd; ++d) {
    if (hc[d].rejected != 0)
      return afail(FV_NEGATIVE_EIGENVALUE, "a replay of design %d's recorded forward met a negative eigenvalue", d);
    const AdjDesign &a = b->hdesc[d];
    FVA_CUDA(cudaMemcpy(grad_amp + size_t(d) * nelem, a.acc + 1, sizeof(double) * nelem, cudaMemcpyDeviceToHost));
    FVA_CUDA(cudaMemcpy(grad_phase + size_t(d) * nelem, a.acc + 1 + nelem, sizeof(double) * nelem,
                        cudaMemcpyDeviceToHost));
  }
  // (the replays wrote only the segment buffers: the checkpoints and the
  // final state stay, so a second backward gives the same gradients)
  return FV_OK;
}

fv_status fv_adjoint_batch_schedule(fv_adjoint_batch *b, int32_t design, double *dt, double *T) {
  if (!b || !dt || !T || design < 0 || design >= b->nd) return afail(FV_BAD_ARG, "bad argument");
  if (b->h_dt[design].size() != size_t(b->nsteps)) return afail(FV_BAD_ARG, "no forward run");
  for (long long k = 0; k < b->nsteps; ++k) {
    dt[k] = b->h_dt[design][k];
    T[k] = b->h_T[design][k];
  }
  return FV_OK;
}

}  // extern "C"
