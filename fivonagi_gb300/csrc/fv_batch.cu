// fv_batch.cu -- many independent simulations stepped by one launch.
//
// The reference runs one simulation per process, and its sweep scripts
// recompile and rerun it for every parameter point (apps/*/run.sh). A batch
// holds n simulations of uneven grid sizes and parameters (each with its own
// app hooks, dt, T, CFL and rejections). Every launch pair -- the ghost-frame
// pre-pass and batch_step_kernel -- attempts one step of each simulation that
// still has steps to take, and bulk runs replay a captured CUDA graph of such
// pairs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <vector>

#include "fv_internal.h"

using namespace fvgb;

namespace {

// Eight waves of resident CTAs, but at least 32 rows per warp. The
// simulations of a batch cost different amounts per row (grid sizes, ghost
// columns, fix-up marks), and later waves even out what the even split of
// rows leaves uneven: measured on 64 simulations of sides 256..2048, 8
// waves take 4.33 ms per attempt, 4 waves 4.56 ms and one wave 5.24 ms.
long long default_batch_blocks(int max_resident, long long work) {
  return std::max(1LL, std::min(8LL * max_resident, work / 128));
}

constexpr int kBatchGraphAttempts = 16;

fv_status bfail(fv_status s, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  set_last_error(buf);
  return s;
}

#define FVB_CUDA(call)                                                                    \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return bfail(FV_CUDA_ERROR, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                   __FILE__, __LINE__);                                                   \
  } while (0)

__global__ void batch_ctrl_begin_kernel(Ctrl *c, int n, long long remaining) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  c[k].remaining = remaining;
  c[k].t_stop = __int_as_float(0x7f800000);
  c[k].accepted = 0;
  c[k].rejected = 0;
  c[k].consecutive_rejects = 0;
}

}  // namespace

struct fv_batch {
  int n = 0;
  bool exact = true;
  std::vector<fv_params> params;
  std::vector<BatchInst> host_inst;
  std::vector<size_t> ncell;
  BatchInst *inst = nullptr;
  Ctrl *ctrl = nullptr;
  Ctrl *ctrl_host = nullptr;
  uint32_t *cfl_bits = nullptr;
  int32_t *neg = nullptr;
  uint32_t *fix = nullptr;  // fix-up scratch of the batch launches
  float *mem = nullptr;  // all state buffers and frames
  cudaStream_t own_stream = nullptr, stream = nullptr;
  cudaGraphExec_t graph = nullptr;
  BatchArgs args{};
  int max_resident = 0;
};

namespace {

fv_status read_batch_ctrl(fv_batch *b) {
  FVB_CUDA(cudaMemcpyAsync(b->ctrl_host, b->ctrl, sizeof(Ctrl) * b->n, cudaMemcpyDeviceToHost, b->stream));
  FVB_CUDA(cudaStreamSynchronize(b->stream));
  return FV_OK;
}

int launch_batch(fv_batch *b) {
  return b->exact ? launch_batch_exact(b->args, b->stream) : launch_batch_fast(b->args, b->stream);
}

fv_status enqueue_batch(fv_batch *b, long long n) {
  if (n >= kBatchGraphAttempts) {
    if (!b->graph) {
      cudaGraph_t g = nullptr;
      FVB_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      int rc = 0;
      for (int k = 0; k < kBatchGraphAttempts && rc == 0; ++k) rc = launch_batch(b);
      cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
      if (rc != 0) return bfail(FV_CUDA_ERROR, "batch launch during capture: %s", cudaGetErrorString((cudaError_t)rc));
      if (ec != cudaSuccess) return bfail(FV_CUDA_ERROR, "batch graph capture: %s", cudaGetErrorString(ec));
      ec = cudaGraphInstantiate(&b->graph, g, 0);
      cudaGraphDestroy(g);
      if (ec != cudaSuccess) {
        b->graph = nullptr;
        return bfail(FV_CUDA_ERROR, "batch graph instantiate: %s", cudaGetErrorString(ec));
      }
    }
    while (n >= kBatchGraphAttempts) {
      FVB_CUDA(cudaGraphLaunch(b->graph, b->stream));
      n -= kBatchGraphAttempts;
    }
  }
  for (long long k = 0; k < n; ++k) {
    int rc = launch_batch(b);
    if (rc != 0) return bfail(FV_CUDA_ERROR, "batch launch: %s", cudaGetErrorString((cudaError_t)rc));
  }
  return FV_OK;
}

// Every simulation back to dt = DTINI, T = -TIDE, n = 0, current buffer 0.
fv_status reset_all(fv_batch *b) {
  for (int k = 0; k < b->n; ++k) {
    Ctrl c;
    std::memset(&c, 0, sizeof(c));
    c.dt = float(b->params[k].dtini);
    c.T = -float(b->params[k].tide);
    c.t_stop = std::numeric_limits<float>::infinity();
    b->ctrl_host[k] = c;
  }
  FVB_CUDA(cudaMemcpyAsync(b->ctrl, b->ctrl_host, sizeof(Ctrl) * b->n, cudaMemcpyHostToDevice, b->stream));
  FVB_CUDA(cudaStreamSynchronize(b->stream));
  return FV_OK;
}

}  // namespace

extern "C" {

fv_status fv_batch_create(int32_t n, const fv_params *params, fv_batch **out) {
  if (!out || !params || n <= 0) return bfail(FV_BAD_ARG, "bad argument");
  *out = nullptr;
  bool exact = params[0].exact != 0;
  for (int k = 0; k < n; ++k) {
    if (params[k].app == FV_APP_PHASED_ARRAY)
      return bfail(FV_BAD_ARG, "the phased array is not supported in batches");
    fv_status s = validate_params(&params[k]);
    if (s != FV_OK) return s;
    if ((params[k].exact != 0) != exact) return bfail(FV_BAD_ARG, "all simulations of a batch share `exact`");
  }
  int ndev = 0, dev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return bfail(FV_NO_DEVICE, "no CUDA device");
  FVB_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  FVB_CUDA(cudaGetDeviceProperties(&prop, dev));
  if (prop.major != 10 || prop.minor != 3) return bfail(FV_NO_DEVICE, "device is not sm_103");

  fv_batch *b = new (std::nothrow) fv_batch();
  if (!b) return bfail(FV_CUDA_ERROR, "out of host memory");
  b->n = n;
  b->exact = exact;
  b->params.assign(params, params + n);
  auto cleanup = [&](fv_status st) {
    fv_batch_destroy(b);
    return st;
  };
  // one allocation: per simulation two state buffers and a frame
  size_t total = 0;
  std::vector<size_t> off_state(n), off_frame(n), stride(n);
  for (int k = 0; k < n; ++k) {
    const size_t nc = size_t(params[k].nx) * size_t(params[k].ny);
    b->ncell.push_back(nc);
    stride[k] = (nc + 63) & ~size_t(63);
    off_state[k] = total;
    total += 6 * stride[k];
    off_frame[k] = total;
    total += 3 * ((size_t(frame_cells(params[k].nx, params[k].ny)) + 63) & ~size_t(63));
  }
  cudaError_t e = cudaMalloc(&b->mem, total * sizeof(float));
  if (e != cudaSuccess) return cleanup(bfail(FV_CUDA_ERROR, "cudaMalloc batch state (%zu MB): %s",
                                             total * 4 >> 20, cudaGetErrorString(e)));
  e = cudaMalloc(&b->ctrl, sizeof(Ctrl) * n);
  if (e == cudaSuccess) e = cudaMallocHost(&b->ctrl_host, sizeof(Ctrl) * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->inst, sizeof(BatchInst) * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->cfl_bits, sizeof(uint32_t) * n);
  if (e == cudaSuccess) e = cudaMalloc(&b->neg, sizeof(int32_t) * n);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cleanup(bfail(FV_CUDA_ERROR, "batch allocation: %s", cudaGetErrorString(e)));
  b->stream = b->own_stream;

  long long work = 0, cost = 0, fix_chunks = 0;
  int max_frame = 0;
  b->host_inst.resize(n);
  for (int k = 0; k < n; ++k) {
    BatchInst &I = b->host_inst[k];
    I.p = dev_params_of(params[k]);
    for (int buf = 0; buf < 2; ++buf)
      for (int f = 0; f < 3; ++f) I.state[buf][f] = b->mem + off_state[k] + (size_t(buf) * 3 + f) * stride[k];
    const size_t fc = (size_t(frame_cells(params[k].nx, params[k].ny)) + 63) & ~size_t(63);
    for (int f = 0; f < 3; ++f) I.frame[f] = b->mem + off_frame[k] + size_t(f) * fc;
    I.ctrl = b->ctrl + k;
    const int windows = (params[k].nx + kWarpCols - 1) / kWarpCols;
    I.work_begin = work;
    I.work = (long long)windows * params[k].ny;
    work += I.work;
    I.cost_begin = cost;
    I.cost = ShareCost(params[k].nx, params[k].ny).total();
    cost += I.cost;
    I.fix_base = fix_chunks;
    fix_chunks += (long long)windows * fix_chunks_per_window(params[k].ny);
    max_frame = std::max(max_frame, 4 * params[k].nx + 4 * (params[k].ny - 4));
  }
  if (fix_chunks >= (1LL << 32)) return cleanup(bfail(FV_BAD_ARG, "batch above 2^32 fix-up chunks"));
  const size_t fix_words = size_t(4 + (fix_chunks + 31) / 32 + 2 * fix_chunks);
  e = cudaMalloc(&b->fix, fix_words * sizeof(uint32_t));
  if (e != cudaSuccess) return cleanup(bfail(FV_CUDA_ERROR, "cudaMalloc batch fix-up scratch: %s", cudaGetErrorString(e)));
  FVB_CUDA(cudaMemsetAsync(b->fix, 0, fix_words * sizeof(uint32_t), b->stream));
  FVB_CUDA(cudaMemcpyAsync(b->inst, b->host_inst.data(), sizeof(BatchInst) * n, cudaMemcpyHostToDevice, b->stream));
  FVB_CUDA(cudaMemsetAsync(b->cfl_bits, 0, sizeof(uint32_t) * n, b->stream));
  FVB_CUDA(cudaMemsetAsync(b->neg, 0, sizeof(int32_t) * n, b->stream));
  FVB_CUDA(cudaMemsetAsync(b->mem, 0, total * sizeof(float), b->stream));
  const int per_sm = exact ? max_batch_blocks_per_sm_exact() : max_batch_blocks_per_sm_fast();
  b->max_resident = per_sm * prop.multiProcessorCount;
  BatchArgs &a = b->args;
  a.inst = b->inst;
  a.cfl_bits = b->cfl_bits;
  a.neg = b->neg;
  a.fix = b->fix;
  a.n = n;
  a.work = work;
  a.cost = cost;
  a.fix_chunks = fix_chunks;
  a.max_frame = max_frame;
  // the fix-up launch: four CTAs per SM (its occupancy) take the marked chunks
  a.fix_blocks = 4 * prop.multiProcessorCount;
  a.nblocks = int(default_batch_blocks(b->max_resident, work));
  fv_status s = reset_all(b);
  if (s != FV_OK) return cleanup(s);
  *out = b;
  return FV_OK;
}

fv_status fv_batch_destroy(fv_batch *b) {
  if (!b) return FV_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->mem) cudaFree(b->mem);
  if (b->ctrl) cudaFree(b->ctrl);
  if (b->ctrl_host) cudaFreeHost(b->ctrl_host);
  if (b->inst) cudaFree(b->inst);
  if (b->cfl_bits) cudaFree(b->cfl_bits);
  if (b->neg) cudaFree(b->neg);
  if (b->fix) cudaFree(b->fix);
  if (b->own_stream) cudaStreamDestroy(b->own_stream);
  delete b;
  return FV_OK;
}

fv_status fv_batch_set_stream(fv_batch *b, void *cuda_stream) {
  if (!b) return bfail(FV_BAD_ARG, "batch is NULL");
  FVB_CUDA(cudaStreamSynchronize(b->stream));
  b->stream = cuda_stream ? (cudaStream_t)cuda_stream : b->own_stream;
  return FV_OK;
}

fv_status fv_batch_init_state(fv_batch *b) {
  if (!b) return bfail(FV_BAD_ARG, "batch is NULL");
  for (int k = 0; k < b->n; ++k) {
    std::vector<float> u(3 * b->ncell[k]);
    init_state_host(b->params[k], u.data(), u.data() + b->ncell[k], u.data() + 2 * b->ncell[k]);
    for (int f = 0; f < 3; ++f)
      FVB_CUDA(cudaMemcpyAsync(b->host_inst[k].state[0][f], u.data() + f * b->ncell[k],
                               b->ncell[k] * sizeof(float), cudaMemcpyHostToDevice, b->stream));
    FVB_CUDA(cudaStreamSynchronize(b->stream));
  }
  return reset_all(b);
}

fv_status fv_batch_set_state(fv_batch *b, int32_t k, const float *u1, const float *u2,
                             const float *u3, int32_t on_device) {
  if (!b || k < 0 || k >= b->n || !u1 || !u2 || !u3) return bfail(FV_BAD_ARG, "bad argument");
  // the other simulations keep their state; this one restarts from dtini/-tide
  FVB_CUDA(cudaStreamSynchronize(b->stream));
  fv_status s = read_batch_ctrl(b);
  if (s != FV_OK) return s;
  const int cur = b->ctrl_host[k].cur;
  const float *src[3] = {u1, u2, u3};
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  for (int f = 0; f < 3; ++f)
    FVB_CUDA(cudaMemcpyAsync(b->host_inst[k].state[cur][f], src[f], b->ncell[k] * sizeof(float), kind, b->stream));
  Ctrl c = b->ctrl_host[k];
  c.dt = float(b->params[k].dtini);
  c.T = -float(b->params[k].tide);
  c.n = 0;
  c.status = 0;
  c.neg_flag = 0;
  c.sim_error = 0;
  c.consecutive_rejects = 0;
  c.mdx = c.mdy = 0;
  c.remaining = 0;
  c.accepted = c.rejected = 0;
  c.blocks_done = 0;
  b->ctrl_host[k] = c;
  FVB_CUDA(cudaMemcpyAsync(b->ctrl + k, &b->ctrl_host[k], sizeof(Ctrl), cudaMemcpyHostToDevice, b->stream));
  FVB_CUDA(cudaStreamSynchronize(b->stream));
  return FV_OK;
}

fv_status fv_batch_get_state(fv_batch *b, int32_t k, float *u1, float *u2, float *u3, int32_t on_device) {
  if (!b || k < 0 || k >= b->n || !u1 || !u2 || !u3) return bfail(FV_BAD_ARG, "bad argument");
  fv_status s = read_batch_ctrl(b);
  if (s != FV_OK) return s;
  const int cur = b->ctrl_host[k].cur;
  float *dst[3] = {u1, u2, u3};
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  for (int f = 0; f < 3; ++f)
    FVB_CUDA(cudaMemcpyAsync(dst[f], b->host_inst[k].state[cur][f], b->ncell[k] * sizeof(float), kind, b->stream));
  FVB_CUDA(cudaStreamSynchronize(b->stream));
  return FV_OK;
}

fv_status fv_batch_run(fv_batch *b, int64_t nsteps, fv_run_stats *out) {
  if (!b || nsteps < 0) return bfail(FV_BAD_ARG, "bad argument");
  batch_ctrl_begin_kernel<<<(b->n + 127) / 128, 128, 0, b->stream>>>(b->ctrl, b->n, (long long)nsteps);
  FVB_CUDA(cudaGetLastError());
  long long todo = nsteps;
  for (;;) {
    fv_status s = enqueue_batch(b, todo);
    if (s != FV_OK) return s;
    s = read_batch_ctrl(b);
    if (s != FV_OK) return s;
    long long most = 0;
    for (int k = 0; k < b->n; ++k)
      if (b->ctrl_host[k].status == 0) most = std::max<long long>(most, b->ctrl_host[k].remaining);
    if (most <= 0) break;
    todo = most;  // rejected attempts are made up
  }
  int worst = 0;
  for (int k = 0; k < b->n; ++k) {
    const Ctrl &c = b->ctrl_host[k];
    if (out) {
      out[k].accepted = c.accepted;
      out[k].rejected = c.rejected;
      out[k].dt = c.dt;
      out[k].T = c.T;
      out[k].cfl = c.last_cfl;
      out[k].n = c.n;
      out[k].status = c.status;
      out[k].mdx = c.mdx;
      out[k].mdy = c.mdy;
    }
    if (c.status && !worst) worst = c.status;
  }
  if (worst) return bfail((fv_status)worst, "a simulation of the batch stopped with status %d", worst);
  return FV_OK;
}

fv_status fv_batch_launch_attempts(fv_batch *b, int64_t nattempts) {
  if (!b || nattempts < 0) return bfail(FV_BAD_ARG, "bad argument");
  batch_ctrl_begin_kernel<<<(b->n + 127) / 128, 128, 0, b->stream>>>(b->ctrl, b->n, (long long)nattempts);
  FVB_CUDA(cudaGetLastError());
  return enqueue_batch(b, nattempts);
}

fv_status fv_batch_time_run(fv_batch *b, int64_t nattempts, float *ms) {
  if (!b || nattempts < 1 || !ms) return bfail(FV_BAD_ARG, "bad argument");
  cudaEvent_t ev[2] = {};
  for (int k = 0; k < 2; ++k) {
    const cudaError_t e = cudaEventCreate(&ev[k]);
    if (e != cudaSuccess) {
      if (k) cudaEventDestroy(ev[0]);
      return bfail(FV_CUDA_ERROR, "cudaEventCreate: %s", cudaGetErrorString(e));
    }
  }
  cudaError_t e = cudaEventRecord(ev[0], b->stream);
  fv_status s = FV_OK;
  if (e == cudaSuccess) s = fv_batch_launch_attempts(b, nattempts);
  if (e == cudaSuccess && s == FV_OK) e = cudaEventRecord(ev[1], b->stream);
  if (e == cudaSuccess && s == FV_OK) e = cudaEventSynchronize(ev[1]);
  float t = 0.0f;
  if (e == cudaSuccess && s == FV_OK) e = cudaEventElapsedTime(&t, ev[0], ev[1]);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (s != FV_OK) return s;
  if (e != cudaSuccess) return bfail(FV_CUDA_ERROR, "timing events: %s", cudaGetErrorString(e));
  *ms = t;
  return FV_OK;
}

fv_status fv_batch_sync(fv_batch *b, fv_run_stats *out) {
  if (!b) return bfail(FV_BAD_ARG, "batch is NULL");
  fv_status s = read_batch_ctrl(b);
  if (s != FV_OK) return s;
  for (int k = 0; k < b->n && out; ++k) {
    const Ctrl &c = b->ctrl_host[k];
    out[k].accepted = c.accepted;
    out[k].rejected = c.rejected;
    out[k].dt = c.dt;
    out[k].T = c.T;
    out[k].cfl = c.last_cfl;
    out[k].n = c.n;
    out[k].status = c.status;
    out[k].mdx = c.mdx;
    out[k].mdy = c.mdy;
  }
  return FV_OK;
}

fv_status fv_batch_set_launch(fv_batch *b, int32_t blocks) {
  if (!b || blocks < 0) return bfail(FV_BAD_ARG, "bad argument");
  FVB_CUDA(cudaStreamSynchronize(b->stream));
  b->args.nblocks = blocks == 0 ? int(default_batch_blocks(b->max_resident, b->args.work)) : blocks;
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  return FV_OK;
}

fv_status fv_batch_get_launch(fv_batch *b, int32_t *blocks, int32_t *max_resident) {
  if (!b) return bfail(FV_BAD_ARG, "batch is NULL");
  if (blocks) *blocks = b->args.nblocks;
  if (max_resident) *max_resident = b->max_resident;
  return FV_OK;
}

}  // extern "C"
