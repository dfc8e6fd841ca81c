// fv_noalloc.cu -- one step attempt without any device allocation.
//
// Some callers of this library cannot let it call cudaMalloc: programs that
// hand all device memory to one allocator of their own (a framework's
// caching allocator, or a fixed arena sized at start-up) would see a
// library allocation bypass their accounting, or fail outright once the
// arena holds the whole device. fv_step_noalloc serves them: the caller
// passes the input and output state buffers, and the step kernel's scratch
// (control block, per-CTA CFL maxima, ghost frame, fix-up scratch) lives in one file-scope
// __device__ array of fixed size instead of fv_create's allocations.
//
// The array is FV_NOALLOC_SCRATCH_BYTES per device; every GPU that loads the
// library holds it until the process exits. All calls on a device share it,
// so calls that overlap on the GPU (two streams, or a call issued before
// the previous one finished) race on it and must be serialised by the
// caller. The first call on each device looks up the array's device address
// (cudaGetSymbolAddress), so make that first call before any stream capture.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>

#include "fv_internal.h"

using namespace fvgb;

namespace {

constexpr int kNoallocMaxCtas = FV_NOALLOC_MAX_CTAS;
constexpr int kNoallocMaxFixCtas = 1024;                          // CTAs of the fix-up launch
constexpr int kNoallocMaxFrame = 4 * FV_NOALLOC_MAX_PERIMETER;  // frame_cells(nx, ny) <= this
constexpr size_t kCtrlBytes = 256;                               // Ctrl, padded
constexpr size_t kPartialBytes = size_t(kNoallocMaxCtas + kNoallocMaxFixCtas) * sizeof(float);
constexpr size_t kFrameBytes = 3 * size_t(kNoallocMaxFrame) * sizeof(float);
// fix_scratch_words() of every grid with nx + ny <= 16384 is at most
// 336633 words (nx = 8120, ny = 8264); the host checks each call's need.
constexpr size_t kFixBytes = 337920 * sizeof(uint32_t);
static_assert(sizeof(Ctrl) <= kCtrlBytes, "control block does not fit its slot");
static_assert(kCtrlBytes + kPartialBytes + kFrameBytes + kFixBytes <= FV_NOALLOC_SCRATCH_BYTES,
              "scratch layout exceeds FV_NOALLOC_SCRATCH_BYTES");

// The scratch itself: a host-side stand-in in host code, a real array on
// every device. Host code must use the address from cudaGetSymbolAddress.
__device__ __align__(256) unsigned char g_noalloc_scratch[FV_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char *g_scratch_addr[kMaxDevices] = {};
int g_max_resident[kMaxDevices][2] = {};  // [device][exact variant]
int g_sms[kMaxDevices] = {};

// Errors go to the library's per-thread message (fv_last_error_string).
fv_status nafail(fv_status s, const char *msg, cudaError_t e = cudaSuccess) {
  char buf[256];
  if (e != cudaSuccess)
    snprintf(buf, sizeof(buf), "fv_step_noalloc: %s: %s", msg, cudaGetErrorString(e));
  else
    snprintf(buf, sizeof(buf), "fv_step_noalloc: %s", msg);
  set_last_error(buf);
  return s;
}

// Writes every control-block field the step kernel reads or counts with,
// and zeroes the fix-up counters and bitmap, so the previous call's
// contents never leak into this one.
__global__ void noalloc_begin_kernel(Ctrl *c, uint32_t *fix, int fix_zero_words, float dt, float T,
                                     int mdx, int mdy) {
  for (int k = threadIdx.x; k < fix_zero_words; k += blockDim.x) fix[k] = 0u;
  if (threadIdx.x != 0) return;
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
  c->mdx = mdx;
  c->mdy = mdy;
  c->remaining = 1;
  c->accepted = 0;
  c->rejected = 0;
  c->blocks_done = 0u;
}

}  // namespace

extern "C" fv_status fv_step_noalloc(const fv_params *p, const float *in_u1, const float *in_u2,
                                     const float *in_u3, float *out_u1, float *out_u2,
                                     float *out_u3, double dt, double T, int32_t mdx,
                                     int32_t mdy, void *cuda_stream, fv_step_result *res) {
  if (!p || !in_u1 || !in_u2 || !in_u3 || !out_u1 || !out_u2 || !out_u3 || !res)
    return nafail(FV_BAD_ARG, "NULL argument");
  // the checks fv_create makes, then this entry point's own limits
  const fv_status vs = validate_params(p);
  if (vs != FV_OK) return vs;
  if (p->app == FV_APP_PHASED_ARRAY)
    return nafail(FV_BAD_ARG, "the phased array needs fv_create's weights");
  if ((long long)p->nx + (long long)p->ny > FV_NOALLOC_MAX_PERIMETER)
    return nafail(FV_BAD_ARG, "nx + ny above FV_NOALLOC_MAX_PERIMETER (the ghost frame's room in the scratch array)");
  if (!(dt > 0)) return nafail(FV_BAD_ARG, "dt must be positive");
  // the step kernel streams its input while it writes its output: the two
  // states must be distinct buffers
  const float *ins[3] = {in_u1, in_u2, in_u3};
  const float *outs[3] = {out_u1, out_u2, out_u3};
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      if (ins[a] == outs[b]) return nafail(FV_BAD_ARG, "an output buffer is also an input buffer");

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return nafail(FV_NO_DEVICE, "cudaGetDevice", e);
  if (dev < 0 || dev >= kMaxDevices) return nafail(FV_NO_DEVICE, "device index out of range");
  const int variant = p->exact ? 1 : 0;
  unsigned char *base = nullptr;
  int max_resident = 0, sms = 0;
  {
    // Set-up, once per device, with that device current.
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
      cudaDeviceProp prop;
      e = cudaGetDeviceProperties(&prop, dev);
      if (e != cudaSuccess) return nafail(FV_NO_DEVICE, "cudaGetDeviceProperties", e);
      if (prop.major != 10 || prop.minor != 3) return nafail(FV_NO_DEVICE, "not an sm_103 device");
      void *ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess || !ptr) return nafail(FV_CUDA_ERROR, "cudaGetSymbolAddress(scratch)", e);
      // resident CTAs of each arithmetic variant's step kernel
      g_max_resident[dev][0] = max_blocks_per_sm_fast(4, -1) * prop.multiProcessorCount;
      g_max_resident[dev][1] = max_blocks_per_sm_exact(4, -1) * prop.multiProcessorCount;
      g_sms[dev] = prop.multiProcessorCount;
      g_scratch_addr[dev] = static_cast<unsigned char *>(ptr);
    }
    base = g_scratch_addr[dev];
    max_resident = g_max_resident[dev][variant];
    sms = g_sms[dev];
  }

  StepArgs a{};
  a.p = dev_params_of(*p);
  const int strip_cols = 4 * kWarpCols;
  const int nstrips = (p->nx + strip_cols - 1) / strip_cols;
  const long long work = (long long)nstrips * p->ny;
  // fv_create's launch shape and division
  long long blocks = default_blocks(max_resident, work, 4);
  if (blocks > kNoallocMaxCtas) blocks = kNoallocMaxCtas;
  const long long windows = (long long)nstrips * 4;
  if (size_t(fix_scratch_words(windows, p->ny)) * sizeof(uint32_t) > kFixBytes)
    return nafail(FV_BAD_ARG, "grid needs more fix-up scratch than the scratch array holds");
  Ctrl *ctrl = reinterpret_cast<Ctrl *>(base);
  float *partials = reinterpret_cast<float *>(base + kCtrlBytes);
  float *frame = reinterpret_cast<float *>(base + kCtrlBytes + kPartialBytes);
  uint32_t *fix = reinterpret_cast<uint32_t *>(base + kCtrlBytes + kPartialBytes + kFrameBytes);
  const size_t fcells = size_t(frame_cells(p->nx, p->ny));
  a.state[0][0] = const_cast<float *>(in_u1);
  a.state[0][1] = const_cast<float *>(in_u2);
  a.state[0][2] = const_cast<float *>(in_u3);
  a.state[1][0] = out_u1;
  a.state[1][1] = out_u2;
  a.state[1][2] = out_u3;
  for (int f = 0; f < 3; ++f) a.frame[f] = frame + size_t(f) * fcells;
  a.ctrl = ctrl;
  a.partials = partials;
  a.fix = fix;
  a.nstrips = nstrips;
  a.nblocks = int(blocks);
  a.work = work;
  a.fix_blocks = std::min(kNoallocMaxFixCtas, std::max(1, 4 * sms));
  a.div_exact = default_div_exact(*p);

  cudaStream_t st = (cudaStream_t)cuda_stream;
  const int fix_zero_words = int(4 + fix_bitmap_words(windows, p->ny));
  noalloc_begin_kernel<<<1, 256, 0, st>>>(ctrl, fix, fix_zero_words, float(dt), float(T), mdx, mdy);
  e = cudaGetLastError();
  if (e != cudaSuccess) return nafail(FV_CUDA_ERROR, "control-block launch", e);
  const int rc = p->exact ? launch_step_exact(a, 4, -1, st) : launch_step_fast(a, 4, -1, st);
  if (rc != 0) return nafail(FV_CUDA_ERROR, "step launch", (cudaError_t)rc);
  Ctrl c;
  e = cudaMemcpyAsync(&c, ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return nafail(FV_CUDA_ERROR, "reading the control block", e);
  res->accepted = c.accepted > 0 ? 1 : 0;
  res->status = c.status;
  res->cfl = c.last_cfl;
  res->dt_next = c.dt;
  res->T = c.T;
  res->mdx = c.mdx;
  res->mdy = c.mdy;
  if (c.status == FV_NEGATIVE_EIGENVALUE) return nafail(FV_NEGATIVE_EIGENVALUE, "negative eigenvalue (tmp3 < 0)");
  return FV_OK;
}
