// fv_api.cu -- the C ABI of include/fivonagi.h.
//
// Owns the device state of a simulation (two state buffers, the control
// block, per-CTA CFL partials), runs the apps' initial-value hooks on the
// host as the reference does, and drives the fused step kernel: bulk
// attempts are replayed from a captured CUDA graph, the host synchronises
// once per call, and every error comes back as an fv_status.
#include <cuda_runtime.h>
#include <cufft.h>
#include <dlfcn.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "fv_internal.h"
#include "fv_math.h"

using namespace fvgb;

namespace {

thread_local std::string g_last_error;

fv_status fail(fv_status s, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return s;
}

#define FV_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess)                                                              \
      return fail(FV_CUDA_ERROR, "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                  __FILE__, __LINE__);                                                  \
  } while (0)

// Graph of this many attempts, replayed for bulk runs.
constexpr int kGraphAttempts = 32;
constexpr int kMinRowsPerBlock = 32;

__global__ void ctrl_begin_kernel(Ctrl *c, long long remaining, float t_stop) {
  c->remaining = remaining;
  c->t_stop = t_stop;
  c->accepted = 0;
  c->rejected = 0;
  c->consecutive_rejects = 0;
  c->mirror_seq = 0;
}

__global__ void ctrl_reset_kernel(Ctrl *c, float dt, float T, int n) {
  c->dt = dt;
  c->T = T;
  c->n = n;
  c->cur = 0;
  c->status = 0;
  c->neg_flag = 0;
  c->sim_error = 0;
  c->consecutive_rejects = 0;
  c->mdx = 0;
  c->mdy = 0;
  c->remaining = 0;
  c->accepted = 0;
  c->rejected = 0;
  c->blocks_done = 0;
  c->last_cfl = 0.0f;
  c->t_stop = __int_as_float(0x7f800000);
}

__global__ void ctrl_scalars_kernel(Ctrl *c, float dt, float T, int n) {
  c->dt = dt;
  c->T = T;
  c->n = n;
}

// On-device data collection (the reference's dataCollect, apps/hifu-beam/
// data_collect.h:6-107): after each accepted step with T > 0, the step's T
// and CFL, u1 at the probe cells, and the running u1 maximum along a lab
// row. One CTA; the control block says whether the attempt was accepted
// and which step it was, so attempts after the run ended collect nothing.
struct CollectDev {
  int nprobes;
  int pi[8], pj[8];
  int env_row, env_len, capacity;
  float halfwidth, eta;
  float *T, *cfl, *probes, *env;
  int *count;  // [0] steps in the series, [1] step number n of the last collected step
};

__global__ void collect_kernel(Ctrl *c, const float *u1a, const float *u1b, int nx, int ny, CollectDev d) {
  __shared__ int go, k;
  if (threadIdx.x == 0) {
    const int n = c->n;
    go = (c->status == 0 && c->last_accepted && n != d.count[1] && c->T > 0.0f) ? 1 : 0;
    if (go) {
      k = d.count[0];
      if (k >= d.capacity) {
        c->status = FV_COLLECT_OVERFLOW;  // simError 4 (data_collect.h:94)
        go = 0;
      } else {
        d.count[0] = k + 1;
        d.count[1] = n;
      }
    }
  }
  __syncthreads();
  if (!go) return;
  const float *u1 = c->cur ? u1b : u1a;
  const int mdx = c->mdx, mdy = c->mdy;
  const float T = c->T;
  if (threadIdx.x == 0) {
    d.T[k] = T;
    d.cfl[k] = c->last_cfl;
  }
  if ((int)threadIdx.x < d.nprobes) {
    const int p = threadIdx.x;
    const int i = d.pi[p] - mdx, j = d.pj[p] - mdy;
    d.probes[size_t(k) * 8 + p] = (i >= 0 && i < nx && j >= 0 && j < ny) ? u1[i + size_t(j) * nx] : 0.0f;
  }
  const int j = d.env_row - mdy;
  if (d.env_row >= 0 && j >= 0 && j < ny) {
    for (int i = threadIdx.x; i < nx; i += blockDim.x) {
      const int lab = i + mdx;
      if (lab >= d.env_len) continue;
      // the central peak only (data_collect.h:99-102)
      if (d.halfwidth > 0.0f && fabsf((float)lab / d.eta - T) > d.halfwidth) continue;
      const float v = u1[i + size_t(j) * nx];
      d.env[lab] = (v > d.env[lab]) ? v : d.env[lab];  // getmax, common/main.cu:63
    }
  }
}

// Spectral low-pass (the filter hook the reference leaves commented out,
// common/filter.h:16-39, main.cu:672-708): zero the coefficients of the
// half spectrum (NY rows of NX/2+1, row j holding wavenumber ky = j or
// j - NY) whose wavenumber radius exceeds `radius`, and scale the rest by
// 1/(NX NY) so that the inverse transform returns the field itself.
__global__ void lowpass_kernel(cufftComplex *spec, int nx, int ny, float radius) {
  const int kxn = nx / 2 + 1;
  const long long total = (long long)kxn * ny;
  const float scale = 1.0f / ((float)nx * (float)ny);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < total; k += (long long)gridDim.x * blockDim.x) {
    const int kx = (int)(k % kxn);
    const int row = (int)(k / kxn);
    const int ky = row <= ny / 2 ? row : row - ny;
    const float r2 = (float)kx * (float)kx + (float)ky * (float)ky;
    cufftComplex c = spec[k];
    const bool keep = r2 <= radius * radius;
    c.x = keep ? c.x * scale : 0.0f;
    c.y = keep ? c.y * scale : 0.0f;
    spec[k] = c;
  }
}

// Headless display (the reference's draw + colour map, apps/hifu-beam/
// draw_float_cut.h:8-106, rendered to a GL bitmap there): a map of u1 over
// a window of the grid, sampled every `zoom` cells, scaled to [0, 1] as
// u1 / (2 PLOTSCALE AMPL) + 0.5 with the reference's guide lines, and under
// it a 128-pixel plot of u1 along row jcut; then a hue/lightness colour map
// to RGBA8.
struct RenderArgs {
  const float *u1;
  int nx, ny, mdx;
  int i0, j0, width, height, zoom, jcut, overlays;
  float scale;        // 1 / (PLOTSCALE * AMPL)
  int focal_i;        // ISPF (lab column), -1: none
  int aperture_j;     // ISPa * ETA, -1: none
  uint8_t *rgba;
};

// HLS to RGB, one channel (Foley, van Dam, Feiner, Hughes, "Computer
// Graphics: Principles and Practice", 2nd ed., sec. 13.3.5).
__device__ __forceinline__ uint8_t hls_channel(float n1, float n2, int hue) {
  hue = ((hue % 360) + 360) % 360;
  float v;
  if (hue < 60) v = n1 + (n2 - n1) * (float)hue / 60.0f;
  else if (hue < 180) v = n2;
  else if (hue < 240) v = n1 + (n2 - n1) * (float)(240 - hue) / 60.0f;
  else v = n1;
  return (uint8_t)(255.0f * v);
}

__global__ void render_kernel(RenderArgs r) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  const int rows = r.height + (r.jcut >= 0 ? 128 : 0);
  if (x >= r.width || y >= rows) return;
  auto at = [&](int i, int j) {
    i = min(max(i, 0), r.nx - 1);  // clamp addressing, as the texture reads
    j = min(max(j, 0), r.ny - 1);
    return r.u1[i + size_t(j) * r.nx];
  };
  const int iread = x * r.zoom + r.i0;
  float l;
  if (y < r.height) {
    const int jread = y * r.zoom + r.j0;
    l = fminf(fmaxf(at(iread, jread) * r.scale * 0.5f + 0.5f, 0.0f), 1.0f);
    if (r.overlays) {
      if (r.jcut >= 0 && abs(jread - r.jcut) <= r.zoom - 1) l = (iread % 40 < 20) ? 1.0f : 0.0f;
      if (r.focal_i >= 0 && abs(iread - (r.focal_i - r.mdx)) <= r.zoom - 1) l = (jread % 40 < 20) ? 1.0f : 0.0f;
      if (abs(x - r.width / 2) <= 1) l = 0.7f;
      if (r.aperture_j >= 0 && abs(jread - r.aperture_j) <= 1) l = 0.7f;
    }
  } else {
    // the cut plot: the curve, the zero line and the +-AMPL*PLOTSCALE lines
    const float d = at(iread, r.jcut) * r.scale * 0.25f;
    const int yy = y - r.height;
    if (fabsf((float)yy - 64.0f - d * 128.0f) < 1.0f) l = 1.0f;
    else if (yy == 64) l = 0.5f;
    else if (yy == 96 || yy == 32) l = 0.25f;
    else l = 0.0f;
  }
  // lightness l, saturation 1, hue (180 + 360 l) mod 360
  const int hue = (180 + (int)(360.0f * l)) % 360;
  const float m2 = l <= 0.5f ? l * 2.0f : 1.0f;
  const float m1 = 2.0f * l - m2;
  uint8_t *px = r.rgba + 4 * (size_t(y) * r.width + x);
  px[0] = hls_channel(m1, m2, hue + 120);
  px[1] = hls_channel(m1, m2, hue);
  px[2] = hls_channel(m1, m2, hue - 120);
  px[3] = 255;
}

// cuFFT, opened on first use so that the library itself does not depend on
// it.
struct CufftApi {
  bool tried = false, ok = false;
  cufftResult (*plan2d)(cufftHandle *, int, int, cufftType) = nullptr;
  cufftResult (*set_stream)(cufftHandle, cudaStream_t) = nullptr;
  cufftResult (*exec_r2c)(cufftHandle, cufftReal *, cufftComplex *) = nullptr;
  cufftResult (*exec_c2r)(cufftHandle, cufftComplex *, cufftReal *) = nullptr;
  cufftResult (*destroy)(cufftHandle) = nullptr;
};

CufftApi &cufft_api() {
  static CufftApi api;
  static std::mutex m;
  std::lock_guard<std::mutex> lock(m);
  if (api.tried) return api;
  api.tried = true;
  void *lib = dlopen("libcufft.so.12", RTLD_NOW | RTLD_LOCAL);
  if (!lib) lib = dlopen("libcufft.so", RTLD_NOW | RTLD_LOCAL);
  if (!lib) return api;
  api.plan2d = reinterpret_cast<decltype(api.plan2d)>(dlsym(lib, "cufftPlan2d"));
  api.set_stream = reinterpret_cast<decltype(api.set_stream)>(dlsym(lib, "cufftSetStream"));
  api.exec_r2c = reinterpret_cast<decltype(api.exec_r2c)>(dlsym(lib, "cufftExecR2C"));
  api.exec_c2r = reinterpret_cast<decltype(api.exec_c2r)>(dlsym(lib, "cufftExecC2R"));
  api.destroy = reinterpret_cast<decltype(api.destroy)>(dlsym(lib, "cufftDestroy"));
  api.ok = api.plan2d && api.set_stream && api.exec_r2c && api.exec_c2r && api.destroy;
  return api;
}

}  // namespace

namespace fvgb {
void set_last_error(const char *msg) { g_last_error = msg; }
}  // namespace fvgb

struct fv_handle {
  fv_params params{};
  DevParams dp{};
  int device = 0;
  size_t ncell = 0;
  float *state_mem = nullptr;   // 2 buffers x 3 fields
  size_t field_stride = 0;      // floats between fields (256-byte aligned)
  float *dbg_mem = nullptr;
  float *frame_mem = nullptr;   // ghost frame, 3 fields
  Ctrl *ctrl = nullptr;
  Ctrl *ctrl_host = nullptr;    // pinned mirror for reads
  float *partials = nullptr;
  uint32_t *fix = nullptr;      // fix-up scratch of the step launches
  float *weights = nullptr;     // phased array: amplitudes then phases (device)
  bool collect = false;         // data collection on
  CollectDev coll{};            // its device buffers and spec
  float *coll_mem = nullptr;
  float *snap_mem = nullptr;    // fv_snapshot: one state (3 fields)
  Ctrl *snap_ctrl = nullptr;    // fv_snapshot: the control block
  int snap_cur = -1;            // buffer the snapshot was taken from; -1: none
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph = nullptr;   // kGraphAttempts attempts
  cudaGraphExec_t graph1 = nullptr;  // fv_run(h, 1): control-block set-up and one attempt
  // fv_steps_async / fv_step_wait: attempts in flight; each one's finalize
  // launch writes its control block to the next slot of a host ring
  HostSlot *ring_host = nullptr, *ring_dev = nullptr;  // kHostRing slots, host and device views
  cudaGraphExec_t ring_graph = nullptr;   // kGraphAttempts attempts writing the ring
  cudaGraphExec_t ring_graph1 = nullptr;  // one attempt writing the ring
  long long ring_enq = 0, ring_got = 0;   // attempts of this run of them enqueued, collected
  long long ring_acc = 0, ring_rej = 0;   // counters of the last collected attempt
  StepArgs args{};
  int warps = 4;
  bool exact = true;
  int max_resident = 0;       // CTAs of the current step launch that fit on the device at once
  int partials_cap = 0;       // capacity of `partials`
  int sms = 0;
  int fma_resident = 0;                  // resident CTAs of the FMA-division step kernel
  int shape_resident[kStepShapes] = {};  // ... of the exact-division kernel in each CTA shape
  int shape_warps[kStepShapes] = {};     // warps per CTA of each shape
};

namespace {

int launch(fv_handle *h, int stage, const StepArgs &a) {
  return h->exact ? launch_step_exact(a, h->warps, stage, h->stream)
                  : launch_step_fast(a, h->warps, stage, h->stream);
}

// warps per CTA of the attempts' step launch
int step_cta_warps(const fv_handle *h) { return h->args.div_exact ? h->shape_warps[h->args.shape] : 4; }

// One attempt of the run: the step's launches, then the collector if on.
int launch_attempt(fv_handle *h) {
  int rc = launch(h, -1, h->args);
  if (rc == 0 && h->collect) {
    collect_kernel<<<1, 1024, 0, h->stream>>>(h->ctrl, h->args.state[0][0], h->args.state[1][0], h->params.nx,
                                              h->params.ny, h->coll);
    rc = (int)cudaGetLastError();
  }
  return rc;
}

fv_status validate(const fv_params *p) {
  if (!p) return fail(FV_BAD_ARG, "params is NULL");
  if (p->app < FV_APP_HIFU_BEAM || p->app > FV_APP_PHASED_ARRAY)
    return fail(FV_BAD_ARG, "unknown app %d", p->app);
  if (p->nx < 8 || p->ny < 8) return fail(FV_BAD_ARG, "grid %dx%d below 8x8", p->nx, p->ny);
  if ((long long)p->nx * (long long)p->ny > (1LL << 30))
    return fail(FV_BAD_ARG, "grid %dx%d above 2^30 cells", p->nx, p->ny);
  if (!(p->xmax > 0) || !(p->ymax > 0)) return fail(FV_BAD_ARG, "xmax/ymax must be positive");
  if (!(p->cflmax > 0) || !(p->cflwhish > 0) || !(p->dtini > 0))
    return fail(FV_BAD_ARG, "cflmax, cflwhish and dtini must be positive");
  if (p->moving_domain && (p->mdvx < 0 || p->mdvy < 0))
    return fail(FV_BAD_ARG, "moving_domain needs mdvx, mdvy >= 0");
  if ((p->app == FV_APP_FOCUSED_BEAM || p->app == FV_APP_PHASED_ARRAY) && !(p->ramp_periods > 0))
    return fail(FV_BAD_ARG, "focused beam and phased array need ramp_periods > 0");
  if (p->app == FV_APP_PHASED_ARRAY) {
    if (p->array_elems < 1 || p->array_elems > 4096) return fail(FV_BAD_ARG, "array_elems must be 1..4096");
    const double w = p->aperture / p->array_elems;
    if (!(w >= 1) || w != std::floor(w)) return fail(FV_BAD_ARG, "aperture must be a multiple of array_elems cells");
  }
  return FV_OK;
}

DevParams make_dev_params(const fv_params &p) {
  DevParams d{};
  d.app = p.app;
  d.nx = p.nx;
  d.ny = p.ny;
  d.cfl_even_only = p.cfl_even_only ? 1 : 0;
  d.max_retries = p.max_retries > 0 ? p.max_retries : 64;
  d.moving_domain = p.moving_domain ? 1 : 0;
  d.mdvx = float(p.mdvx);
  d.mdvy = float(p.mdvy);
  // FP32 rounding of each parameter, as `static const DATATYPEV` does
  d.dx = float(p.xmax) / float(p.nx - 1);
  d.dy = float(p.ymax) / float(p.ny - 1);
  d.beta = float(p.beta);
  d.diffdelta = float(p.diffdelta);
  d.cflmax = float(p.cflmax);
  d.cflwhish = float(p.cflwhish);
  d.ampl = float(p.ampl);
  d.frec = float(p.frec);
  d.ispw = 2.0f * 3.1415926f * d.frec;  // Num2*PI*FREC, common/numbers.h:14
  d.ispa = float(p.isp_a);
  d.ispf = float(p.isp_f);
  d.hifu_width = static_cast<int>(d.ispa / d.dy);
  d.isprhoa = float(p.isp_rhoa);
  d.ispc = float(p.isp_c);
  d.mdt = float(p.mdt);
  const float th = float(p.angle);
  d.cos_th = fvm::cosf_(th);
  d.sin_th = fvm::sinf_(th);
  d.center = float(p.center);
  d.halfap = float(p.aperture * 0.5);
  d.ramp = p.ramp_periods > 0 ? float(p.frec / p.ramp_periods) : 0.0f;
  if (p.app == FV_APP_PHASED_ARRAY) {
    d.nelem = p.array_elems;
    d.arr_elem = int(p.aperture / p.array_elems);
    d.arr_j0 = int(std::lround(p.center - 0.5 * p.aperture));
  }
  return d;
}

// Host initial-value hooks (the reference's init<TTT> runs on the host too).
void init_host(const fv_params &p, const DevParams &d, float *u1, float *u2, float *u3) {
  const int nx = p.nx, ny = p.ny;
  for (int j = 0; j < ny; ++j)
    for (int i = 0; i < nx; ++i) {
      const size_t o = size_t(i) + size_t(j) * size_t(nx);
      float v1 = 0.f, v2 = 0.f, v3 = 0.f;
      if (p.app == FV_APP_TAYLOR_ANGLE_XY) {
        // apps/taylor-angle-xy/init.h:19-27
        const float th = float(p.angle);
        const float c = fvm::cosf_(th), sn = fvm::sinf_(th);
        const float rhop =
            d.isprhoa * fvm::tanhf_(d.ispc * (float(i) * d.dx * c +
                                              (float(j - ny / 2) * d.dy + d.mdt * sn) * sn +
                                              float(p.tide)));
        v1 = rhop;
        v2 = rhop * c;
        v3 = rhop * sn;
      } else if (p.app == FV_APP_PLANE_WAVE) {
        // sinusoidal plane wave in the taylor init form, in double
        const double ddx = p.xmax / double(nx - 1), ddy = p.ymax / double(ny - 1);
        const double ca = fvm::cos_d(p.angle), sa = fvm::sin_d(p.angle);
        const double ph = 2.0 * 3.141592653589793 * p.frec * (double(i) * ddx * ca + double(j) * ddy * sa);
        const double a = p.ampl * fvm::sin_d(ph);
        v1 = float(a);
        v2 = float(a * ca);
        v3 = float(a * sa);
      }
      u1[o] = v1;
      u2[o] = v2;
      u3[o] = v3;
    }
}

}  // namespace

namespace fvgb {
DevParams dev_params_of(const fv_params &p) { return make_dev_params(p); }
fv_status validate_params(const fv_params *p) { return validate(p); }
void init_state_host(const fv_params &p, float *u1, float *u2, float *u3) {
  init_host(p, make_dev_params(p), u1, u2, u3);
}

// One wave of resident CTAs, but no fewer than kMinRowsPerBlock rows per
// warp (small grids). Every warp of the step kernel streams the same number
// of rows, so all CTAs of a wave finish together; a second wave would add
// the warm-up rows of shorter segments, and a partial one (for instance 640
// CTAs for 608 slots) nearly doubles the time.
long long default_blocks(int max_resident, long long work, int cta_warps) {
  // work counts rows of 4-window strips: kMinRowsPerBlock rows per warp
  const long long most = work * 4 / ((long long)std::max(cta_warps, 1) * kMinRowsPerBlock);
  return std::max(1LL, std::min((long long)max_resident, most));
}

// Exact division in the step kernel by default. With the normal-quotient
// division where quotients are normal in practice (DivPair), it is faster
// than FMA division with its fix-up pass at every size measured: per
// attempt 0.056 against 0.061 ms at 512x512, 0.096 against 0.109 ms at
// 1024x1024, 0.144 against 0.165 ms at 2048x1024, 0.447 against 0.498 ms
// at 4096x2048.
int default_div_exact(const fv_params &) { return 1; }
}  // namespace fvgb

namespace {

float *field_ptr(fv_handle *h, int buf, int f) {
  return h->state_mem + (size_t(buf) * 3 + size_t(f)) * h->field_stride;
}

fv_status read_ctrl(fv_handle *h) {
  FV_CUDA(cudaMemcpyAsync(h->ctrl_host, h->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream));
  FV_CUDA(cudaStreamSynchronize(h->stream));
  return FV_OK;
}

void fill_stats(const fv_handle *h, fv_run_stats *st) {
  if (!st) return;
  const Ctrl &c = *h->ctrl_host;
  st->accepted = c.accepted;
  st->rejected = c.rejected;
  st->dt = c.dt;
  st->T = c.T;
  st->cfl = c.last_cfl;
  st->n = c.n;
  st->status = c.status;
  st->mdx = c.mdx;
  st->mdy = c.mdy;
}

// The captured graphs hold the launch shape, division and collector of
// when they were captured: changing any of them drops them.
void drop_graphs(fv_handle *h) {
  // attempts enqueued by fv_steps_async may still run from these graphs
  if (h->ring_enq != h->ring_got && h->stream) cudaStreamSynchronize(h->stream);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  if (h->graph1) cudaGraphExecDestroy(h->graph1);
  h->graph = nullptr;
  h->graph1 = nullptr;
  if (h->ring_graph) cudaGraphExecDestroy(h->ring_graph);
  if (h->ring_graph1) cudaGraphExecDestroy(h->ring_graph1);
  h->ring_graph = nullptr;
  h->ring_graph1 = nullptr;
}

// The graphs of attempts whose finalize launches write the host ring: n
// attempts (kGraphAttempts or 1) into `g`.
fv_status ensure_ring_graph(fv_handle *h, int n, cudaGraphExec_t &gx) {
  if (gx) return FV_OK;
  StepArgs a = h->args;
  a.host_ring = h->ring_dev;
  cudaGraph_t g = nullptr;
  FV_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int rc = 0;
  for (int k = 0; k < n && rc == 0; ++k) {
    rc = launch(h, -1, a);
    if (rc == 0 && h->collect) {
      collect_kernel<<<1, 1024, 0, h->stream>>>(h->ctrl, h->args.state[0][0], h->args.state[1][0], h->params.nx,
                                                h->params.ny, h->coll);
      rc = (int)cudaGetLastError();
    }
  }
  cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
  if (rc != 0) return fail(FV_CUDA_ERROR, "step launch during capture: %s", cudaGetErrorString((cudaError_t)rc));
  if (ec != cudaSuccess) return fail(FV_CUDA_ERROR, "graph capture: %s", cudaGetErrorString(ec));
  ec = cudaGraphInstantiate(&gx, g, 0);
  cudaGraphDestroy(g);
  if (ec != cudaSuccess) {
    gx = nullptr;
    return fail(FV_CUDA_ERROR, "graph instantiate: %s", cudaGetErrorString(ec));
  }
  return FV_OK;
}

// Attempts launched by fv_steps_async not yet collected by fv_step_wait:
// the other runs would reset the counters those attempts report from.
fv_status check_idle(const fv_handle *h) {
  if (h->ring_enq != h->ring_got)
    return fail(FV_BAD_ARG, "%lld attempts in flight: collect them with fv_step_wait first",
                h->ring_enq - h->ring_got);
  return FV_OK;
}

fv_status ensure_graph1(fv_handle *h) {
  if (h->graph1) return FV_OK;
  cudaGraph_t g = nullptr;
  FV_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  ctrl_begin_kernel<<<1, 1, 0, h->stream>>>(h->ctrl, 1LL, std::numeric_limits<float>::infinity());
  int rc = (int)cudaGetLastError();
  if (rc == 0) rc = launch_attempt(h);
  // and the control block back to the host, for the step's stats
  if (rc == 0)
    rc = (int)cudaMemcpyAsync(h->ctrl_host, h->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream);
  cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
  if (rc != 0) return fail(FV_CUDA_ERROR, "step launch during capture: %s", cudaGetErrorString((cudaError_t)rc));
  if (ec != cudaSuccess) return fail(FV_CUDA_ERROR, "graph capture: %s", cudaGetErrorString(ec));
  ec = cudaGraphInstantiate(&h->graph1, g, 0);
  cudaGraphDestroy(g);
  if (ec != cudaSuccess) {
    h->graph1 = nullptr;
    return fail(FV_CUDA_ERROR, "graph instantiate: %s", cudaGetErrorString(ec));
  }
  return FV_OK;
}

fv_status ensure_graph(fv_handle *h) {
  if (h->graph) return FV_OK;
  cudaGraph_t g = nullptr;
  FV_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int rc = 0;
  for (int k = 0; k < kGraphAttempts && rc == 0; ++k) rc = launch_attempt(h);
  cudaError_t ec = cudaStreamEndCapture(h->stream, &g);
  if (rc != 0) return fail(FV_CUDA_ERROR, "step launch during capture: %s", cudaGetErrorString((cudaError_t)rc));
  if (ec != cudaSuccess) return fail(FV_CUDA_ERROR, "graph capture: %s", cudaGetErrorString(ec));
  ec = cudaGraphInstantiate(&h->graph, g, 0);
  cudaGraphDestroy(g);
  if (ec != cudaSuccess) {
    h->graph = nullptr;
    return fail(FV_CUDA_ERROR, "graph instantiate: %s", cudaGetErrorString(ec));
  }
  return FV_OK;
}

// Enqueue n attempts: whole graphs, then single launches.
fv_status enqueue_attempts(fv_handle *h, long long n) {
  if (n >= kGraphAttempts) {
    fv_status s = ensure_graph(h);
    if (s != FV_OK) return s;
    while (n >= kGraphAttempts) {
      FV_CUDA(cudaGraphLaunch(h->graph, h->stream));
      n -= kGraphAttempts;
    }
  }
  for (long long k = 0; k < n; ++k) {
    int rc = launch_attempt(h);
    if (rc != 0) return fail(FV_CUDA_ERROR, "step launch: %s", cudaGetErrorString((cudaError_t)rc));
  }
  return FV_OK;
}

fv_status reset_ctrl(fv_handle *h) {
  const DevParams &d = h->dp;
  ctrl_reset_kernel<<<1, 1, 0, h->stream>>>(h->ctrl, float(h->params.dtini),
                                            -float(h->params.tide), 0);
  (void)d;
  FV_CUDA(cudaGetLastError());
  return FV_OK;
}

}  // namespace

extern "C" {

const char *fv_version(void) { return "fivonagi-gb300 1 (sm_103a)"; }

const char *fv_last_error_string(void) { return g_last_error.c_str(); }

fv_status fv_default_params(int32_t app, fv_params *out) {
  if (!out) return fail(FV_BAD_ARG, "out is NULL");
  fv_params p;
  std::memset(&p, 0, sizeof(p));
  p.app = app;
  p.cfl_even_only = 1;
  p.exact = 1;
  p.max_retries = 64;
  p.cflmax = 1.0;
  p.cflwhish = double(float(90 / 100.0));  // CFLWHISH = CFLW/100.0 with CFLW = 90
  p.dtini = double(0.005f);
  switch (app) {
    case FV_APP_HIFU_BEAM: {
      // apps/hifu-beam/parameters.h:12-104 with ETAC=1, CFLW=90, ISPAM=30;
      // each value is the FP32 result of the reference's own expression.
      const int NX = 512, NY = 1024;
      const float XMAX = 12.5f * 2.0f, YMAX = 12.5f * 4.0f, FREC = 1.0f;
      const float PI = 3.1415926f;
      const float ISPW = 2.0f * PI * FREC;
      const float ISPlambda = 2.0f * PI / ISPW;
      const float ISPa = 30 * ISPlambda;
      const float ISPF = float(50.0 * ISPlambda / (XMAX / (NX - 1)));
      const float TIDE = float(std::floor(2 + 4 / FREC +
                                          (ISPa * ISPa * (XMAX / (NX - 1))) /
                                              (2.0 * ISPF * (YMAX / (NY - 1)) * (YMAX / (NY - 1)))));
      p.nx = NX;
      p.ny = NY;
      p.xmax = XMAX;
      p.ymax = YMAX;
      p.beta = double(4.8f);
      p.diffdelta = double(0.0002974f);
      p.ampl = double(0.0004217f);
      p.frec = FREC;
      p.isp_a = ISPa;
      p.isp_f = ISPF;
      p.tide = TIDE;
      p.mdvx = 1.0;
      p.mdvy = 0.0;
      p.mdt = double(XMAX * 0.5f);
      p.moving_domain = 1;
      break;
    }
    case FV_APP_TAYLOR_ANGLE_XY: {
      // apps/taylor-angle-xy/parameters.h:12-109 with ETAC=1, CFLW=90,
      // ANGLE=0, SIN=0, COS=1
      const float XMAX = 12.5f, YMAX = 12.5f, BETA = 1.0f, DIFFDELTA = 0.0000001f;
      const int COS = 1, SIN = 0;
      const float MDT = float(XMAX * 0.5 / COS);
      p.nx = 64;
      p.ny = 64;
      p.xmax = XMAX;
      p.ymax = YMAX;
      p.beta = BETA;
      p.diffdelta = DIFFDELTA;
      p.frec = 1.0;
      p.mdvx = COS;
      p.mdvy = SIN;
      p.mdt = MDT;
      p.tide = float(std::ceil(4 + (YMAX * 0.5 - MDT * SIN) * SIN));
      p.isp_rhoa = double(-DIFFDELTA / BETA);
      p.isp_c = double(2.1972245773362196f);
      p.angle = 0.0;
      p.ampl = -p.isp_rhoa;
      p.moving_domain = 1;
      break;
    }
    case FV_APP_PLANE_WAVE: {
      // 512 x 512, 16 cells per wavelength, 30 degrees, Mach 1e-3
      p.nx = 512;
      p.ny = 512;
      p.xmax = 511.0 / 16.0;
      p.ymax = 511.0 / 16.0;
      p.beta = 3.5;
      p.diffdelta = 1e-4;
      p.ampl = 1e-3;
      p.frec = 1.0;
      p.angle = 3.141592653589793 / 6.0;
      p.tide = 0.0;
      break;
    }
    case FV_APP_FOCUSED_BEAM: {
      // 4096 (axial) x 2048 (lateral), 24 cells per wavelength, aperture
      // 1024 cells centred on j = 1024, focus 3000 cells, Mach 5e-3
      // reached over 5 periods
      p.nx = 4096;
      p.ny = 2048;
      p.xmax = 4095.0 / 24.0;
      p.ymax = 2047.0 / 24.0;
      p.beta = 3.5;
      p.diffdelta = 5e-5;
      p.ampl = 5e-3;
      p.frec = 1.0;
      p.isp_f = 3000.0;
      p.aperture = 1024.0;
      p.center = 1024.0;
      p.ramp_periods = 5.0;
      p.tide = 0.0;
      break;
    }
    case FV_APP_PHASED_ARRAY: {
      // 1024 x 1024, 24 cells per wavelength, 128 elements of 8 cells on
      // the left edge centred on j = 512, Mach 2e-3 per element reached
      // over 5 periods
      p.nx = 1024;
      p.ny = 1024;
      p.xmax = 1023.0 / 24.0;
      p.ymax = 1023.0 / 24.0;
      p.beta = 3.5;
      p.diffdelta = 5e-5;
      p.ampl = 2e-3;
      p.frec = 1.0;
      p.array_elems = 128;
      p.aperture = 1024.0;
      p.center = 512.0;
      p.ramp_periods = 5.0;
      p.tide = 0.0;
      break;
    }
    default:
      return fail(FV_BAD_ARG, "unknown app %d", app);
  }
  *out = p;
  return FV_OK;
}

fv_status fv_create(const fv_params *p, fv_handle **out) {
  if (!out) return fail(FV_BAD_ARG, "out is NULL");
  *out = nullptr;
  fv_status s = validate(p);
  if (s != FV_OK) return s;
  int dev = 0, ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(FV_NO_DEVICE, "no CUDA device");
  FV_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  FV_CUDA(cudaGetDeviceProperties(&prop, dev));
  if (prop.major != 10 || prop.minor != 3)
    return fail(FV_NO_DEVICE, "device %d is sm_%d%d; this library is built for sm_103a", dev,
                prop.major, prop.minor);

  fv_handle *h = new (std::nothrow) fv_handle();
  if (!h) return fail(FV_CUDA_ERROR, "out of host memory");
  h->params = *p;
  h->dp = make_dev_params(*p);
  if (p->app == FV_APP_PHASED_ARRAY) {
    // every element starts at amplitude AMPL and phase 0
    std::vector<float> w(2 * size_t(p->array_elems), 0.0f);
    for (int k = 0; k < p->array_elems; ++k) w[k] = float(p->ampl);
    cudaError_t ew = cudaMalloc(&h->weights, w.size() * sizeof(float));
    if (ew == cudaSuccess) ew = cudaMemcpy(h->weights, w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (ew != cudaSuccess) {
      fv_destroy(h);
      return fail(FV_CUDA_ERROR, "phased-array weights: %s", cudaGetErrorString(ew));
    }
    h->dp.weights = h->weights;
  }
  h->device = dev;
  h->exact = p->exact != 0;
  h->ncell = size_t(p->nx) * size_t(p->ny);
  h->field_stride = (h->ncell + 63) & ~size_t(63);
  auto cleanup = [&](fv_status st) {
    fv_destroy(h);
    return st;
  };
  cudaError_t e = cudaMalloc(&h->state_mem, 6 * h->field_stride * sizeof(float));
  if (e != cudaSuccess) return cleanup(fail(FV_CUDA_ERROR, "cudaMalloc state: %s", cudaGetErrorString(e)));
  const size_t fcells = size_t(frame_cells(p->nx, p->ny));
  e = cudaMalloc(&h->frame_mem, 3 * fcells * sizeof(float));
  if (e != cudaSuccess) return cleanup(fail(FV_CUDA_ERROR, "cudaMalloc frame: %s", cudaGetErrorString(e)));
  e = cudaMalloc(&h->ctrl, sizeof(Ctrl));
  if (e != cudaSuccess) return cleanup(fail(FV_CUDA_ERROR, "cudaMalloc ctrl: %s", cudaGetErrorString(e)));
  e = cudaMallocHost(&h->ctrl_host, sizeof(Ctrl));
  if (e != cudaSuccess) return cleanup(fail(FV_CUDA_ERROR, "cudaMallocHost: %s", cudaGetErrorString(e)));
  e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cleanup(fail(FV_CUDA_ERROR, "stream: %s", cudaGetErrorString(e)));
  h->stream = h->own_stream;

  // launch shape: persistent CTAs whose warps each stream a balanced share of
  // the (window, row) space
  const int strip_cols = h->warps * kWarpCols;
  const int nstrips = (p->nx + strip_cols - 1) / strip_cols;
  const long long work = (long long)nstrips * p->ny;
  h->sms = prop.multiProcessorCount;
  const int per_sm = h->exact ? max_blocks_per_sm_exact(h->warps, -1) : max_blocks_per_sm_fast(h->warps, -1);
  h->fma_resident = per_sm * prop.multiProcessorCount;
  int most_resident = h->fma_resident;
  for (int k = 0; k < kStepShapes; ++k) {
    int w = 4;
    const int nb = h->exact ? step_shape_blocks_per_sm_exact(k, &w) : step_shape_blocks_per_sm_fast(k, &w);
    h->shape_resident[k] = nb * prop.multiProcessorCount;
    h->shape_warps[k] = w;
    most_resident = std::max(most_resident, h->shape_resident[k]);
  }
  h->max_resident = default_div_exact(*p) ? h->shape_resident[0] : h->fma_resident;
  long long blocks = default_blocks(h->max_resident, work, 4);
  h->partials_cap = std::max(most_resident, 1) * 8;
  // the fix-up launch: four CTAs per SM (two waves at its occupancy of two);
  // warp w takes marked items w, w + W, ..., so warps past the last item exit
  // at once
  const int fix_blocks = 4 * prop.multiProcessorCount;
  e = cudaMalloc(&h->partials, size_t(h->partials_cap + fix_blocks) * sizeof(float));
  if (e != cudaSuccess) return cleanup(fail(FV_CUDA_ERROR, "cudaMalloc partials: %s", cudaGetErrorString(e)));
  const size_t fix_words = size_t(fix_scratch_words((long long)nstrips * h->warps, p->ny));
  e = cudaMalloc(&h->fix, fix_words * sizeof(uint32_t));
  if (e != cudaSuccess) return cleanup(fail(FV_CUDA_ERROR, "cudaMalloc fix-up scratch: %s", cudaGetErrorString(e)));

  StepArgs &a = h->args;
  a.p = h->dp;
  for (int b = 0; b < 2; ++b)
    for (int f = 0; f < 3; ++f) a.state[b][f] = field_ptr(h, b, f);
  for (int f = 0; f < 3; ++f) a.frame[f] = h->frame_mem + size_t(f) * fcells;
  a.ctrl = h->ctrl;
  a.partials = h->partials;
  a.fix = h->fix;
  a.nstrips = nstrips;
  a.nblocks = int(blocks);
  a.work = work;
  a.fix_blocks = fix_blocks;
  a.div_exact = default_div_exact(*p);
  FV_CUDA(cudaMemsetAsync(h->state_mem, 0, 6 * h->field_stride * sizeof(float), h->stream));
  FV_CUDA(cudaMemsetAsync(h->fix, 0, fix_words * sizeof(uint32_t), h->stream));
  s = reset_ctrl(h);
  if (s != FV_OK) return cleanup(s);
  e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return cleanup(fail(FV_CUDA_ERROR, "create sync: %s", cudaGetErrorString(e)));
  *out = h;
  return FV_OK;
}

fv_status fv_destroy(fv_handle *h) {
  if (!h) return FV_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graphs(h);
  if (h->state_mem) cudaFree(h->state_mem);
  if (h->dbg_mem) cudaFree(h->dbg_mem);
  if (h->frame_mem) cudaFree(h->frame_mem);
  if (h->ctrl) cudaFree(h->ctrl);
  if (h->ctrl_host) cudaFreeHost(h->ctrl_host);
  if (h->partials) cudaFree(h->partials);
  if (h->fix) cudaFree(h->fix);
  if (h->weights) cudaFree(h->weights);
  if (h->coll_mem) cudaFree(h->coll_mem);
  if (h->snap_mem) cudaFree(h->snap_mem);
  if (h->snap_ctrl) cudaFree(h->snap_ctrl);
  if (h->ring_host) cudaFreeHost(h->ring_host);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
  return FV_OK;
}

fv_status fv_set_stream(fv_handle *h, void *cuda_stream) {
  if (!h) return fail(FV_BAD_ARG, "handle is NULL");
  FV_CUDA(cudaStreamSynchronize(h->stream));
  h->stream = cuda_stream ? (cudaStream_t)cuda_stream : h->own_stream;
  return FV_OK;
}

fv_status fv_init_state(fv_handle *h) {
  if (!h) return fail(FV_BAD_ARG, "handle is NULL");
  std::vector<float> u(3 * h->ncell);
  init_host(h->params, h->dp, u.data(), u.data() + h->ncell, u.data() + 2 * h->ncell);
  return fv_set_state(h, u.data(), u.data() + h->ncell, u.data() + 2 * h->ncell, 0);
}

fv_status fv_set_state(fv_handle *h, const float *u1, const float *u2, const float *u3,
                       int32_t on_device) {
  if (!h || !u1 || !u2 || !u3) return fail(FV_BAD_ARG, "NULL argument");
  const float *src[3] = {u1, u2, u3};
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  for (int f = 0; f < 3; ++f)
    FV_CUDA(cudaMemcpyAsync(field_ptr(h, 0, f), src[f], h->ncell * sizeof(float), kind, h->stream));
  fv_status s = reset_ctrl(h);
  if (s != FV_OK) return s;
  if (h->collect) {
    const int none[2] = {0, -1};
    FV_CUDA(cudaMemcpyAsync(h->coll.count, none, sizeof(none), cudaMemcpyHostToDevice, h->stream));
    FV_CUDA(cudaMemsetAsync(h->coll.env, 0, size_t(h->coll.env_len) * sizeof(float), h->stream));
  }
  FV_CUDA(cudaStreamSynchronize(h->stream));
  return FV_OK;
}

fv_status fv_filter_u1(fv_handle *h, double radius, float *out, int32_t on_device) {
  if (!h || !out) return fail(FV_BAD_ARG, "NULL argument");
  if (!(radius >= 0)) return fail(FV_BAD_ARG, "radius must be >= 0");
  CufftApi &api = cufft_api();
  if (!api.ok) return fail(FV_CUDA_ERROR, "cuFFT (libcufft.so.12) could not be loaded");
  fv_status s = read_ctrl(h);
  if (s != FV_OK) return s;
  const int nx = h->params.nx, ny = h->params.ny;
  const size_t ncomplex = size_t(nx / 2 + 1) * size_t(ny);
  // the half spectrum, then the filtered field in a buffer of its own (an
  // in-place inverse would write rows padded to 2 (NX/2 + 1) floats)
  void *buf = nullptr;
  FV_CUDA(cudaMalloc(&buf, ncomplex * sizeof(cufftComplex) + h->ncell * sizeof(float)));
  cufftReal *field = reinterpret_cast<cufftReal *>(static_cast<cufftComplex *>(buf) + ncomplex);
  cufftHandle fwd = 0, inv = 0;
  auto done = [&](fv_status st) {
    if (fwd) api.destroy(fwd);
    if (inv) api.destroy(inv);
    cudaFree(buf);
    return st;
  };
  // rows of NX floats, i fastest: the plan's dimensions are (NY, NX)
  if (api.plan2d(&fwd, ny, nx, CUFFT_R2C) != CUFFT_SUCCESS || api.plan2d(&inv, ny, nx, CUFFT_C2R) != CUFFT_SUCCESS)
    return done(fail(FV_CUDA_ERROR, "cufftPlan2d failed"));
  api.set_stream(fwd, h->stream);
  api.set_stream(inv, h->stream);
  cufftComplex *spec = static_cast<cufftComplex *>(buf);
  if (api.exec_r2c(fwd, field_ptr(h, h->ctrl_host->cur, 0), spec) != CUFFT_SUCCESS)
    return done(fail(FV_CUDA_ERROR, "cufftExecR2C failed"));
  lowpass_kernel<<<4 * 152, 256, 0, h->stream>>>(spec, nx, ny, float(radius));
  if (api.exec_c2r(inv, spec, field) != CUFFT_SUCCESS)
    return done(fail(FV_CUDA_ERROR, "cufftExecC2R failed"));
  cudaError_t e = cudaMemcpyAsync(out, field, h->ncell * sizeof(float),
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) return done(fail(FV_CUDA_ERROR, "filter: %s", cudaGetErrorString(e)));
  return done(FV_OK);
}

fv_status fv_render(fv_handle *h, const fv_render_spec *spec, uint8_t *rgba, int32_t on_device) {
  if (!h || !spec || !rgba) return fail(FV_BAD_ARG, "NULL argument");
  if (spec->width < 1 || spec->height < 1 || spec->zoom < 1 || spec->width > 16384 || spec->height > 16384)
    return fail(FV_BAD_ARG, "render size must be 1..16384 pixels and zoom >= 1");
  if (!(spec->plot_scale > 0)) return fail(FV_BAD_ARG, "plot_scale must be positive");
  fv_status s = read_ctrl(h);
  if (s != FV_OK) return s;
  const Ctrl &c = *h->ctrl_host;
  RenderArgs r{};
  r.u1 = field_ptr(h, c.cur, 0);
  r.nx = h->params.nx;
  r.ny = h->params.ny;
  r.mdx = c.mdx;
  r.i0 = spec->i0;
  r.j0 = spec->j0;
  r.width = spec->width;
  r.height = spec->height;
  r.zoom = spec->zoom;
  r.jcut = spec->jcut;
  r.overlays = spec->overlays;
  r.scale = float(1.0 / (spec->plot_scale * h->params.ampl));
  r.focal_i = h->params.app == FV_APP_HIFU_BEAM ? int(h->dp.ispf) : -1;
  r.aperture_j = h->params.app == FV_APP_HIFU_BEAM ? int(h->dp.ispa * (float(h->params.nx) / float(h->params.xmax))) : -1;
  const int rows = spec->height + (spec->jcut >= 0 ? 128 : 0);
  const size_t bytes = size_t(spec->width) * size_t(rows) * 4;
  uint8_t *dev = rgba;
  if (!on_device) FV_CUDA(cudaMalloc(&dev, bytes));
  r.rgba = dev;
  const dim3 blk(32, 8), grd((spec->width + 31) / 32, (rows + 7) / 8);
  render_kernel<<<grd, blk, 0, h->stream>>>(r);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && !on_device) e = cudaMemcpyAsync(rgba, dev, bytes, cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (!on_device) cudaFree(dev);
  if (e != cudaSuccess) return fail(FV_CUDA_ERROR, "render: %s", cudaGetErrorString(e));
  return FV_OK;
}

fv_status fv_collect_enable(fv_handle *h, const fv_collect_spec *spec) {
  if (!h) return fail(FV_BAD_ARG, "handle is NULL");
  FV_CUDA(cudaStreamSynchronize(h->stream));
  drop_graphs(h);
  if (h->coll_mem) cudaFree(h->coll_mem);
  h->coll_mem = nullptr;
  h->collect = false;
  h->coll = CollectDev{};
  if (!spec) return FV_OK;
  if (spec->nprobes < 0 || spec->nprobes > 8) return fail(FV_BAD_ARG, "nprobes must be 0..8");
  if (spec->capacity < 1 || spec->capacity > (1 << 24)) return fail(FV_BAD_ARG, "capacity must be 1..2^24");
  if (spec->envelope_row >= 0 && (spec->envelope_len < 1 || spec->envelope_len > (1 << 26)))
    return fail(FV_BAD_ARG, "envelope_len must be 1..2^26");
  CollectDev d{};
  d.nprobes = spec->nprobes;
  for (int p = 0; p < 8; ++p) {
    d.pi[p] = spec->probe_i[p];
    d.pj[p] = spec->probe_j[p];
  }
  d.env_row = spec->envelope_row;
  d.env_len = spec->envelope_row >= 0 ? spec->envelope_len : 0;
  d.capacity = spec->capacity;
  d.halfwidth = float(spec->envelope_halfwidth);
  d.eta = float(h->params.nx) / float(h->params.xmax);  // ETA = NX/XMAX (hifu parameters.h:30)
  const size_t cap = size_t(d.capacity);
  const size_t floats = cap * 2 + cap * 8 + size_t(d.env_len) + 2;
  FV_CUDA(cudaMalloc(&h->coll_mem, floats * sizeof(float)));
  d.T = h->coll_mem;
  d.cfl = d.T + cap;
  d.probes = d.cfl + cap;
  d.env = d.probes + cap * 8;
  d.count = reinterpret_cast<int *>(d.env + d.env_len);
  FV_CUDA(cudaMemsetAsync(h->coll_mem, 0, floats * sizeof(float), h->stream));
  const int none[2] = {0, -1};
  FV_CUDA(cudaMemcpyAsync(d.count, none, sizeof(none), cudaMemcpyHostToDevice, h->stream));
  FV_CUDA(cudaStreamSynchronize(h->stream));
  h->coll = d;
  h->collect = true;
  return FV_OK;
}

fv_status fv_collect_read(fv_handle *h, int32_t *nsteps, float *T, float *cfl, float *probes,
                          float *envelope) {
  if (!h) return fail(FV_BAD_ARG, "handle is NULL");
  if (!h->collect) return fail(FV_BAD_ARG, "collection is off (fv_collect_enable)");
  const CollectDev &d = h->coll;
  int count[2] = {0, -1};
  FV_CUDA(cudaMemcpyAsync(count, d.count, sizeof(count), cudaMemcpyDeviceToHost, h->stream));
  FV_CUDA(cudaStreamSynchronize(h->stream));
  const size_t k = size_t(count[0]);
  if (nsteps) *nsteps = count[0];
  if (T && k) FV_CUDA(cudaMemcpy(T, d.T, k * sizeof(float), cudaMemcpyDeviceToHost));
  if (cfl && k) FV_CUDA(cudaMemcpy(cfl, d.cfl, k * sizeof(float), cudaMemcpyDeviceToHost));
  if (probes && k) FV_CUDA(cudaMemcpy(probes, d.probes, k * 8 * sizeof(float), cudaMemcpyDeviceToHost));
  if (envelope && d.env_len)
    FV_CUDA(cudaMemcpy(envelope, d.env, size_t(d.env_len) * sizeof(float), cudaMemcpyDeviceToHost));
  // empty the series for the next frame; the last collected step stays
  FV_CUDA(cudaMemsetAsync(d.count, 0, sizeof(int), h->stream));
  FV_CUDA(cudaStreamSynchronize(h->stream));
  return FV_OK;
}

fv_status fv_get_state(fv_handle *h, float *u1, float *u2, float *u3, int32_t on_device) {
  if (!h || !u1 || !u2 || !u3) return fail(FV_BAD_ARG, "NULL argument");
  fv_status s = read_ctrl(h);
  if (s != FV_OK) return s;
  const int cur = h->ctrl_host->cur;
  float *dst[3] = {u1, u2, u3};
  const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  for (int f = 0; f < 3; ++f)
    FV_CUDA(cudaMemcpyAsync(dst[f], field_ptr(h, cur, f), h->ncell * sizeof(float), kind, h->stream));
  FV_CUDA(cudaStreamSynchronize(h->stream));
  return FV_OK;
}

fv_status fv_set_scalars(fv_handle *h, double dt, double T, int32_t n) {
  if (!h) return fail(FV_BAD_ARG, "handle is NULL");
  ctrl_scalars_kernel<<<1, 1, 0, h->stream>>>(h->ctrl, float(dt), float(T), n);
  FV_CUDA(cudaGetLastError());
  FV_CUDA(cudaStreamSynchronize(h->stream));
  return FV_OK;
}

// The reference keeps a copy of the pre-step state (texCpy, common/
// main.cu:72-91) and copies it back after a rejected step (restore,
// :93-107). The step kernel never overwrites its input, so retries need no
// copy here; fv_snapshot/fv_restore offer the same save-and-return to
// callers, with the time-stepping scalars.
fv_status fv_set_array_weights(fv_handle *h, const float *amp, const float *phase, int32_t nelem) {
  if (!h || !amp || !phase) return fail(FV_BAD_ARG, "NULL argument");
  if (!h->weights) return fail(FV_BAD_ARG, "not a phased-array simulation");
  if (nelem != h->dp.nelem) return fail(FV_BAD_ARG, "nelem %d, the array has %d elements", nelem, h->dp.nelem);
  FV_CUDA(cudaStreamSynchronize(h->stream));
  FV_CUDA(cudaMemcpy(h->weights, amp, size_t(nelem) * sizeof(float), cudaMemcpyHostToDevice));
  FV_CUDA(cudaMemcpy(h->weights + nelem, phase, size_t(nelem) * sizeof(float), cudaMemcpyHostToDevice));
  return FV_OK;
}

fv_status fv_snapshot(fv_handle *h) {
  if (!h) return fail(FV_BAD_ARG, "handle is NULL");
  if (!h->snap_mem) FV_CUDA(cudaMalloc(&h->snap_mem, 3 * h->field_stride * sizeof(float)));
  if (!h->snap_ctrl) FV_CUDA(cudaMalloc(&h->snap_ctrl, sizeof(Ctrl)));
  fv_status s = read_ctrl(h);
  if (s != FV_OK) return s;
  const int cur = h->ctrl_host->cur;
  FV_CUDA(cudaMemcpyAsync(h->snap_mem, field_ptr(h, cur, 0), 3 * h->field_stride * sizeof(float),
                          cudaMemcpyDeviceToDevice, h->stream));
  FV_CUDA(cudaMemcpyAsync(h->snap_ctrl, h->ctrl, sizeof(Ctrl), cudaMemcpyDeviceToDevice, h->stream));
  FV_CUDA(cudaStreamSynchronize(h->stream));
  h->snap_cur = cur;
  return FV_OK;
}

fv_status fv_restore(fv_handle *h) {
  if (!h) return fail(FV_BAD_ARG, "handle is NULL");
  if (h->snap_cur < 0) return fail(FV_BAD_ARG, "no snapshot taken");
  FV_CUDA(cudaMemcpyAsync(field_ptr(h, h->snap_cur, 0), h->snap_mem, 3 * h->field_stride * sizeof(float),
                          cudaMemcpyDeviceToDevice, h->stream));
  FV_CUDA(cudaMemcpyAsync(h->ctrl, h->snap_ctrl, sizeof(Ctrl), cudaMemcpyDeviceToDevice, h->stream));
  FV_CUDA(cudaStreamSynchronize(h->stream));
  return FV_OK;
}

fv_status fv_get_stats(fv_handle *h, fv_run_stats *out) {
  if (!h || !out) return fail(FV_BAD_ARG, "NULL argument");
  fv_status s = read_ctrl(h);
  if (s != FV_OK) return s;
  fill_stats(h, out);
  return FV_OK;
}

fv_status fv_launch_attempts(fv_handle *h, int64_t nattempts) {
  if (!h || nattempts < 0) return fail(FV_BAD_ARG, "bad argument");
  if (fv_status busy = check_idle(h)) return busy;
  ctrl_begin_kernel<<<1, 1, 0, h->stream>>>(h->ctrl, (long long)nattempts,
                                            std::numeric_limits<float>::infinity());
  FV_CUDA(cudaGetLastError());
  return enqueue_attempts(h, nattempts);
}

fv_status fv_time_attempts(fv_handle *h, int32_t nattempts, float *step_kernel_ms, float *attempt_ms) {
  if (!h || nattempts < 1 || !step_kernel_ms || !attempt_ms) return fail(FV_BAD_ARG, "bad argument");
  if (fv_status busy = check_idle(h)) return busy;
  ctrl_begin_kernel<<<1, 1, 0, h->stream>>>(h->ctrl, (long long)nattempts,
                                            std::numeric_limits<float>::infinity());
  FV_CUDA(cudaGetLastError());
  cudaEvent_t ev[4] = {};
  for (int k = 0; k < 4; ++k) {
    const cudaError_t e = cudaEventCreate(&ev[k]);
    if (e != cudaSuccess) {
      for (int j = 0; j < k; ++j) cudaEventDestroy(ev[j]);
      return fail(FV_CUDA_ERROR, "cudaEventCreate: %s", cudaGetErrorString(e));
    }
  }
  double step_sum = 0.0, att_sum = 0.0;
  int rc = 0;
  cudaError_t ec = cudaSuccess;
  const int parts[3] = {kLaunchFrame, kLaunchStep, kLaunchFixFinal};
  for (int n = 0; n < nattempts && rc == 0 && ec == cudaSuccess; ++n) {
    ec = cudaEventRecord(ev[0], h->stream);
    for (int k = 0; k < 3 && rc == 0 && ec == cudaSuccess; ++k) {
      rc = launch(h, parts[k], h->args);
      if (rc == 0 && k == 2 && h->collect) {  // the attempt's collector, as in launch_attempt
        collect_kernel<<<1, 1024, 0, h->stream>>>(h->ctrl, h->args.state[0][0], h->args.state[1][0],
                                                  h->params.nx, h->params.ny, h->coll);
        rc = (int)cudaGetLastError();
      }
      if (rc == 0) ec = cudaEventRecord(ev[k + 1], h->stream);
    }
    if (rc == 0 && ec == cudaSuccess) ec = cudaEventSynchronize(ev[3]);
    float ms_step = 0.f, ms_all = 0.f;
    if (rc == 0 && ec == cudaSuccess) ec = cudaEventElapsedTime(&ms_step, ev[1], ev[2]);
    if (rc == 0 && ec == cudaSuccess) ec = cudaEventElapsedTime(&ms_all, ev[0], ev[3]);
    step_sum += ms_step;
    att_sum += ms_all;
  }
  for (int k = 0; k < 4; ++k) cudaEventDestroy(ev[k]);
  if (rc != 0) return fail(FV_CUDA_ERROR, "step launch: %s", cudaGetErrorString((cudaError_t)rc));
  if (ec != cudaSuccess) return fail(FV_CUDA_ERROR, "timing events: %s", cudaGetErrorString(ec));
  *step_kernel_ms = float(step_sum / nattempts);
  *attempt_ms = float(att_sum / nattempts);
  return FV_OK;
}

fv_status fv_time_run(fv_handle *h, int64_t nattempts, float *ms) {
  if (!h || nattempts < 1 || !ms) return fail(FV_BAD_ARG, "bad argument");
  if (fv_status busy = check_idle(h)) return busy;
  cudaEvent_t ev[2] = {};
  for (int k = 0; k < 2; ++k) {
    const cudaError_t e = cudaEventCreate(&ev[k]);
    if (e != cudaSuccess) {
      if (k) cudaEventDestroy(ev[0]);
      return fail(FV_CUDA_ERROR, "cudaEventCreate: %s", cudaGetErrorString(e));
    }
  }
  cudaError_t e = cudaEventRecord(ev[0], h->stream);
  fv_status s = FV_OK;
  if (e == cudaSuccess) s = fv_launch_attempts(h, nattempts);
  if (e == cudaSuccess && s == FV_OK) e = cudaEventRecord(ev[1], h->stream);
  if (e == cudaSuccess && s == FV_OK) e = cudaEventSynchronize(ev[1]);
  float t = 0.0f;
  if (e == cudaSuccess && s == FV_OK) e = cudaEventElapsedTime(&t, ev[0], ev[1]);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (s != FV_OK) return s;
  if (e != cudaSuccess) return fail(FV_CUDA_ERROR, "timing events: %s", cudaGetErrorString(e));
  *ms = t;
  return FV_OK;
}

fv_status fv_device_name(char *name, int32_t len) {
  if (!name || len < 1) return fail(FV_BAD_ARG, "bad argument");
  int dev = 0;
  FV_CUDA(cudaGetDevice(&dev));
  cudaDeviceProp prop;
  FV_CUDA(cudaGetDeviceProperties(&prop, dev));
  snprintf(name, size_t(len), "%s", prop.name);
  return FV_OK;
}

fv_status fv_sync(fv_handle *h, fv_run_stats *out) {
  if (!h) return fail(FV_BAD_ARG, "handle is NULL");
  fv_status s = read_ctrl(h);
  if (s != FV_OK) return s;
  fill_stats(h, out);
  return h->ctrl_host->status ? (fv_status)h->ctrl_host->status : FV_OK;
}

fv_status fv_steps_async(fv_handle *h, int32_t nattempts) {
  if (!h || nattempts < 1) return fail(FV_BAD_ARG, "bad argument");
  if (h->ring_enq - h->ring_got + nattempts > kHostRing)
    return fail(FV_BAD_ARG, "more than %d attempts in flight: collect some with fv_step_wait", kHostRing);
  if (!h->ring_host) {
    FV_CUDA(cudaHostAlloc(&h->ring_host, kHostRing * sizeof(HostSlot), cudaHostAllocMapped));
    FV_CUDA(cudaHostGetDevicePointer(&h->ring_dev, h->ring_host, 0));
  }
  fv_status s = ensure_ring_graph(h, kGraphAttempts, h->ring_graph);
  if (s == FV_OK) s = ensure_ring_graph(h, 1, h->ring_graph1);
  if (s != FV_OK) return s;
  if (h->ring_enq == h->ring_got) {
    // a new run of enqueued attempts (every earlier one collected, so no
    // ring write is pending): no step budget or stop time, counters and the
    // ring's sequence from zero
    std::memset(h->ring_host, 0, kHostRing * sizeof(HostSlot));
    h->ring_enq = h->ring_got = 0;
    h->ring_acc = h->ring_rej = 0;
    ctrl_begin_kernel<<<1, 1, 0, h->stream>>>(h->ctrl, std::numeric_limits<long long>::max(),
                                              std::numeric_limits<float>::infinity());
    FV_CUDA(cudaGetLastError());
  }
  for (int k = 0; k < nattempts;) {
    const bool whole = nattempts - k >= kGraphAttempts;
    FV_CUDA(cudaGraphLaunch(whole ? h->ring_graph : h->ring_graph1, h->stream));
    k += whole ? kGraphAttempts : 1;
  }
  h->ring_enq += nattempts;
  return FV_OK;
}

fv_status fv_step_wait(fv_handle *h, fv_run_stats *out) {
  if (!h) return fail(FV_BAD_ARG, "handle is NULL");
  if (h->ring_got == h->ring_enq) return fail(FV_BAD_ARG, "no attempt in flight (fv_steps_async)");
  const long long i = h->ring_got;
  const HostSlot &slot = h->ring_host[i % kHostRing];
  const uint32_t pass = uint32_t(i / kHostRing) + 1u;
  const volatile uint32_t *gen = &slot.gen;
  // the device writes the block, then the pass; a wait that outlives the
  // stream's work (an error, or the attempts done without the write) ends
  for (unsigned spin = 1; *gen != pass; ++spin) {
    if ((spin & 1023u) == 0u) {
      const cudaError_t e = cudaStreamQuery(h->stream);
      if (e == cudaSuccess && *gen != pass) return fail(FV_CUDA_ERROR, "attempt done without its control block");
      if (e != cudaSuccess && e != cudaErrorNotReady) return fail(FV_CUDA_ERROR, "%s", cudaGetErrorString(e));
      std::this_thread::yield();
    }
  }
  std::atomic_thread_fence(std::memory_order_acquire);
  ++h->ring_got;
  std::memcpy(h->ctrl_host, (const void *)&slot.c, sizeof(Ctrl));
  fill_stats(h, out);
  const Ctrl &c = *h->ctrl_host;
  if (out) {
    out->accepted = c.accepted - h->ring_acc;
    out->rejected = c.rejected - h->ring_rej;
  }
  h->ring_acc = c.accepted;
  h->ring_rej = c.rejected;
  const int st = c.status;
  if (st == FV_NEGATIVE_EIGENVALUE) return fail(FV_NEGATIVE_EIGENVALUE, "negative eigenvalue (tmp3 < 0)");
  if (st == FV_DT_TOO_LARGE) return fail(FV_DT_TOO_LARGE, "dt too large after %d retries", h->dp.max_retries);
  return st ? (fv_status)st : FV_OK;
}

fv_status fv_run(fv_handle *h, int64_t nsteps, fv_run_stats *out) {
  if (!h || nsteps < 0) return fail(FV_BAD_ARG, "bad argument");
  if (fv_status busy = check_idle(h)) return busy;
  long long todo = nsteps;
  bool have_ctrl = false;  // ctrl_host holds the control block after the launches
  if (nsteps == 1) {
    // one step, the call of a caller that reads every step's stats: the
    // control-block set-up, the attempt and the copy of the control block
    // to the host as one graph launch
    fv_status s = ensure_graph1(h);
    if (s != FV_OK) return s;
    FV_CUDA(cudaGraphLaunch(h->graph1, h->stream));
    FV_CUDA(cudaStreamSynchronize(h->stream));
    todo = 0;
    have_ctrl = true;
  } else {
    ctrl_begin_kernel<<<1, 1, 0, h->stream>>>(h->ctrl, (long long)nsteps,
                                              std::numeric_limits<float>::infinity());
    FV_CUDA(cudaGetLastError());
  }
  for (;;) {
    fv_status s = todo > 0 ? enqueue_attempts(h, todo) : FV_OK;
    if (s != FV_OK) return s;
    if (!have_ctrl) s = read_ctrl(h);
    have_ctrl = false;
    if (s != FV_OK) return s;
    const Ctrl &c = *h->ctrl_host;
    if (c.status != 0 || c.remaining <= 0) break;
    todo = c.remaining;  // rejected attempts are made up
  }
  fill_stats(h, out);
  const int st = h->ctrl_host->status;
  if (st == FV_NEGATIVE_EIGENVALUE) return fail(FV_NEGATIVE_EIGENVALUE, "negative eigenvalue (tmp3 < 0)");
  if (st == FV_DT_TOO_LARGE) return fail(FV_DT_TOO_LARGE, "dt too large after %d retries", h->dp.max_retries);
  return st ? (fv_status)st : FV_OK;
}

fv_status fv_run_until(fv_handle *h, double t_stop, fv_run_stats *out) {
  if (!h) return fail(FV_BAD_ARG, "handle is NULL");
  if (fv_status busy = check_idle(h)) return busy;
  ctrl_begin_kernel<<<1, 1, 0, h->stream>>>(h->ctrl, std::numeric_limits<long long>::max(),
                                            float(t_stop));
  FV_CUDA(cudaGetLastError());
  fv_status s = read_ctrl(h);
  if (s != FV_OK) return s;
  while (h->ctrl_host->status == 0 && h->ctrl_host->T < float(t_stop)) {
    const double dt = std::max(double(h->ctrl_host->dt), 1e-30);
    long long est = (long long)std::ceil((double(t_stop) - h->ctrl_host->T) / dt) + 1;
    est = std::min<long long>(std::max<long long>(est, 1), 1 << 16);
    s = enqueue_attempts(h, est);
    if (s != FV_OK) return s;
    s = read_ctrl(h);
    if (s != FV_OK) return s;
  }
  fill_stats(h, out);
  const int st = h->ctrl_host->status;
  if (st) return fail((fv_status)st, "device run stopped with status %d", st);
  return FV_OK;
}

fv_status fv_set_launch(fv_handle *h, int32_t blocks) {
  if (!h || blocks < 0) return fail(FV_BAD_ARG, "bad argument");
  const long long b = blocks == 0 ? default_blocks(h->max_resident, h->args.work, step_cta_warps(h)) : blocks;
  if (b > h->partials_cap) return fail(FV_BAD_ARG, "blocks %lld above %d", b, h->partials_cap);
  FV_CUDA(cudaStreamSynchronize(h->stream));
  h->args.nblocks = int(b);
  drop_graphs(h);
  return FV_OK;
}

fv_status fv_get_launch(fv_handle *h, int32_t *blocks, int32_t *max_resident) {
  if (!h) return fail(FV_BAD_ARG, "handle is NULL");
  if (blocks) *blocks = h->args.nblocks;
  if (max_resident) *max_resident = h->max_resident;
  return FV_OK;
}

fv_status fv_set_division(fv_handle *h, int32_t mode) {
  if (!h || mode < FV_DIVISION_DEFAULT || mode > FV_DIVISION_EXACT) return fail(FV_BAD_ARG, "bad argument");
  FV_CUDA(cudaStreamSynchronize(h->stream));
  h->args.div_exact = mode == FV_DIVISION_DEFAULT ? default_div_exact(h->params) : (mode == FV_DIVISION_EXACT);
  h->max_resident = h->args.div_exact ? h->shape_resident[h->args.shape] : h->fma_resident;
  drop_graphs(h);
  return FV_OK;
}

fv_status fv_set_cta_shape(fv_handle *h, int32_t shape) {
  if (!h || shape < 0 || shape >= kStepShapes) return fail(FV_BAD_ARG, "bad argument");
  FV_CUDA(cudaStreamSynchronize(h->stream));
  h->args.shape = shape;
  h->max_resident = h->args.div_exact ? h->shape_resident[shape] : h->fma_resident;
  h->args.nblocks = int(default_blocks(h->max_resident, h->args.work, step_cta_warps(h)));
  drop_graphs(h);
  return FV_OK;
}

fv_status fv_get_cta_shape(fv_handle *h, int32_t *shape, int32_t *warps_per_cta) {
  if (!h) return fail(FV_BAD_ARG, "handle is NULL");
  if (shape) *shape = h->args.shape;
  if (warps_per_cta) *warps_per_cta = step_cta_warps(h);
  return FV_OK;
}

fv_status fv_get_division(fv_handle *h, int32_t *mode) {
  if (!h || !mode) return fail(FV_BAD_ARG, "NULL argument");
  *mode = h->args.div_exact ? FV_DIVISION_EXACT : FV_DIVISION_FMA;
  return FV_OK;
}

fv_status fv_debug_step(fv_handle *h, int32_t stage, float *u1, float *u2, float *u3) {
  if (!h || !u1 || !u2 || !u3) return fail(FV_BAD_ARG, "NULL argument");
  if (fv_status busy = check_idle(h)) return busy;
  if (stage < FV_STAGE_BOUNDARY || stage > FV_STAGE_SOURCE) return fail(FV_BAD_ARG, "bad stage %d", stage);
  if (!h->dbg_mem) FV_CUDA(cudaMalloc(&h->dbg_mem, 3 * h->field_stride * sizeof(float)));
  StepArgs a = h->args;
  for (int f = 0; f < 3; ++f) a.dbg[f] = h->dbg_mem + size_t(f) * h->field_stride;
  FV_CUDA(cudaMemsetAsync(h->dbg_mem, 0, 3 * h->field_stride * sizeof(float), h->stream));
  int rc = launch(h, stage, a);
  if (rc != 0) return fail(FV_CUDA_ERROR, "stage launch: %s", cudaGetErrorString((cudaError_t)rc));
  float *dst[3] = {u1, u2, u3};
  for (int f = 0; f < 3; ++f)
    FV_CUDA(cudaMemcpyAsync(dst[f], a.dbg[f], h->ncell * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
  FV_CUDA(cudaStreamSynchronize(h->stream));
  return FV_OK;
}

}  // extern "C"
