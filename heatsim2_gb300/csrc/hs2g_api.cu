// C ABI of the hs2g library (declared in include/hs2g.h).  Host-side runtime: owns device buffers, compiles a
// problem into step coefficients and queues timesteps on a stream.
#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "hs2g_internal.cuh"

using hs2g::Coeffs;
using hs2g::Dims;

// A host-buffer step (hs2g_step without HS2G_DEVICE) uploads T in kCopyChunks slabs of planes of shrinking
// size, starting the x sweep of each slab's planes (on a stream of its own: an x CTA is latency-bound for the
// whole length of its lines, so slabs must not wait for one another) as soon as the slab and the plane after
// it have arrived, and downloads T' in kCopyChunks blocks of rows, each as soon as the z sweep has finished
// its columns.  The host link (~0.2 TB/s each way on GB300) is then busy while the sweeps run.
constexpr int kCopyChunks = 4;
constexpr double kSlabEnd[kCopyChunks] = {0.55, 0.80, 0.93, 1.0};  // upload slab c ends at this fraction of nz
// x-lines per CTA of each slab's x sweep: a small launch lasts as long as one CTA's chunk loop, so the later,
// smaller slabs take smaller CTAs and finish sooner after their upload (64x512x512 composite panel: 1.77 ms
// per host-buffer step against 1.85 ms with 32 lines throughout; 16 for every slab 1.80, 8 for the last two
// 1.83)
constexpr int kSlabLines[kCopyChunks] = {32, 32, 16, 8};
constexpr int64_t kPipelineMinVoxels = int64_t(1) << 20;

struct hs2g_handle {
  int device = 0;
  Dims d{0, 0, 0};
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  // compiled problem (device)
  double* Gz = nullptr;
  double* Gy = nullptr;
  double* Gx = nullptr;
  double* M = nullptr;
  uint8_t* compute = nullptr;
  uint8_t* vclass = nullptr;
  double* coef_block = nullptr;
  int64_t xb_len = 0;
  Coeffs c{};
  // per-step scratch (device)
  double* W0 = nullptr;
  double* W1 = nullptr;
  // staging for host-pointer calls (device), allocated on first use
  double* Tin_dev = nullptr;
  double* Tout_dev = nullptr;
  double* qdense_dev = nullptr;
  double* hist_dev = nullptr;
  int64_t hist_len = 0;
  // per-voxel source shapes (hs2g_source_zdecay / hs2g_source_point): the multiplier field, which classes
  // have one, the device copies of their z coordinates / joules / cell volumes, and the rank-scan scratch
  double* qshape = nullptr;
  bool shaped[HS2G_MAX_CLASSES] = {};
  double* shape_zgrid[HS2G_MAX_CLASSES] = {};
  double* shape_joules[HS2G_MAX_CLASSES] = {};
  int64_t shape_joules_len[HS2G_MAX_CLASSES] = {};
  double* shape_volumes = nullptr;
  int64_t* shape_tiles = nullptr;
  unsigned long long* err_dev = nullptr;
  int* status_dev = nullptr;
  bool bulk_y = false, bulk_z = false, z_discard = true;
  bool graph_pdl = true;  // the captured step graphs launch their sweeps with programmatic dependent launch
  bool per_row = false;  // compiled from per-row conductances (hs2g_create_rows): no shared face arrays
  hs2g::TensorMapCache* tmaps = nullptr;
  int64_t bytes = 0;
  // host-buffer steps overlap their copies with the sweeps: a copy stream, one stream per upload slab for
  // its x sweep, and per-chunk events
  cudaStream_t copy_stream = nullptr;
  cudaStream_t x_stream[kCopyChunks] = {};
  cudaEvent_t ev_in[kCopyChunks] = {}, ev_x[kCopyChunks] = {}, ev_out[kCopyChunks] = {}, ev_begin = nullptr;
  // device source schedule (hs2g_set_schedule): the descriptor the x sweep of a step with a source reads, the
  // rows and their flags on the device, the flags mirrored on the host (which steps have a source), and the
  // clock (the schedule row of the next scheduled step)
  hs2g::DevSchedule* sched_dev = nullptr;
  double* sched_q = nullptr;
  uint8_t* sched_active = nullptr;
  int64_t sched_cap = 0, sched_n = 0;
  std::vector<uint8_t> sched_flags;
  int64_t clock = 0;
  // captured in-place step graphs of hs2g_run, keyed by what they bake in; captured on a stream of their own
  // (capture is not allowed on the legacy default stream the caller may have chosen) and launched on `stream`
  struct StepGraph {
    double* T;
    double* hist;
    int layer;
    double dz2;
    bool source;  // one step whose x sweep reads its row of the schedule; else `steps` steps without a source
    int steps;
    cudaGraphExec_t exec;
  };
  std::vector<StepGraph> graphs;
  cudaStream_t cap_stream = nullptr;
};

namespace {

thread_local std::string g_last_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(HS2G_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

#define HS2G_CUDA(call, what)                          \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

// Restores the caller's current device on scope exit, so that calls into the library leave torch's (or any
// other runtime user's) device selection unchanged.
struct DeviceGuard {
  int prev = -1;
  bool ok = false;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    ok = (prev == dev) || (cudaSetDevice(dev) == cudaSuccess);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

template <typename T>
int dalloc(hs2g_handle* h, T** p, int64_t count, const char* what) {
  const size_t bytes = (size_t)(count > 0 ? count : 1) * sizeof(T);
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(HS2G_ERR_NOMEM, "cudaMalloc of %zu bytes for %s failed: %s", bytes, what, cudaGetErrorString(e));
  }
  h->bytes += (int64_t)bytes;
  return HS2G_OK;
}

template <typename T>
void dfree(hs2g_handle* h, T*& p, int64_t count) {
  if (p) {
    cudaFree(p);
    h->bytes -= (int64_t)(count > 0 ? count : 1) * (int64_t)sizeof(T);
  }
  p = nullptr;
}

const char* axis_name(int axis) { return axis == 0 ? "z" : axis == 1 ? "y" : axis == 2 ? "x" : "voxel"; }

int check_kernel_error(hs2g_handle* h) {
  unsigned long long v = 0;
  HS2G_CUDA(cudaMemcpyAsync(&v, h->err_dev, sizeof(v), cudaMemcpyDeviceToHost, h->stream), "read error word");
  HS2G_CUDA(cudaStreamSynchronize(h->stream), "compile");
  if (!v) return HS2G_OK;
  const int code = -(int)(v >> 56);
  const int axis = (int)((v >> 54) & 3);
  const int64_t idx = (int64_t)(v & ((1ull << 54) - 1));
  const Dims& d = h->d;
  int64_t fz = d.nz, fy = d.ny, fx = d.nx;
  if (axis == 0) fz += 1;
  if (axis == 1) fy += 1;
  if (axis == 2) fx += 1;
  const int64_t i = idx % fx, j = (idx / fx) % fy, k = idx / (fx * fy);
  const char* what = "invalid problem";
  switch (code) {
    case HS2G_ERR_EXTERIOR:
      what = "a computed voxel has a non-insulating face on the exterior of the grid (the reference would read "
             "outside the domain); set exterior faces to an insulating class";
      break;
    case HS2G_ERR_KTYPE:
      what = "a boundary class uses the conductivity in a form the material does not have (scalar boundary "
             "class with a matrix k, or an indexed one with a scalar k)";
      break;
    case HS2G_ERR_UNALIGNED:
      what = "a face flux couples temperatures across axes: anisotropy not aligned with the grid axes "
             "(unaligned_anisotropic) is not supported";
      break;
    case HS2G_ERR_FORM:
      what = "a face flux is not a conservative two-point difference inside a Crank-Nicolson group()";
      break;
    case HS2G_ERR_CAPACITY:
      what = "a computed voxel has rho*c/dt <= 0 or not finite";
      break;
    case HS2G_ERR_ARG:
      what = "a class index is out of range of the materials / boundaries tuple, or a value is not finite";
      break;
  }
  return fail(code, "%s (at %s index [%lld,%lld,%lld])", what, axis_name(axis), (long long)k, (long long)j,
              (long long)i);
}

// Row pitch of the y sweep's arrays: nx rounded up to an even count, so that TMA tile rows start on 16-byte
// boundaries whatever nx is (HS2G_ROW_PITCH=<multiple> pads further, for tests of the padded layout).
int64_t y_pitch(int64_t nx) {
  int64_t m = 2;
  if (const char* e = getenv("HS2G_ROW_PITCH")) {
    const long long v = atoll(e);
    if (v >= 2 && v % 2 == 0 && v <= 1024) m = v;
  }
  return (nx + m - 1) / m * m;
}

int alloc_common(hs2g_handle* h, bool faces = true) {
  const int64_t n = h->d.nvox();
  h->c.px = y_pitch(h->d.nx);
  const int64_t np = h->d.nz * h->d.ny * h->c.px;  // voxels of the padded y-sweep arrays
  int rc;
  if (faces && (rc = dalloc(h, &h->Gz, (h->d.nz + 1) * h->d.nxy(), "Gz"))) return rc;
  if (faces && (rc = dalloc(h, &h->Gy, h->d.nz * (h->d.ny + 1) * h->d.nx, "Gy"))) return rc;
  if (faces && (rc = dalloc(h, &h->Gx, h->d.nz * h->d.ny * (h->d.nx + 1), "Gx"))) return rc;
  if ((rc = dalloc(h, &h->M, n, "capacity"))) return rc;
  if ((rc = dalloc(h, &h->compute, n, "compute mask"))) return rc;
  if ((rc = dalloc(h, &h->vclass, n, "source classes"))) return rc;
  if ((rc = dalloc(h, &h->W0, np, "stage buffer 0"))) return rc;
  if ((rc = dalloc(h, &h->W1, np, "stage buffer 1"))) return rc;
  if ((rc = dalloc(h, &h->coef_block, np * hs2g::kNumCoeffArrays, "step coefficients"))) return rc;
  h->c.nchunks = (h->d.nx + 31) / 32;
  h->xb_len = h->d.nz * h->d.ny * h->c.nchunks * hs2g::kXBlockCoeffs * 32;
  if ((rc = dalloc(h, &h->c.xb, h->xb_len, "x stencil coefficients"))) return rc;
  HS2G_CUDA(cudaMemsetAsync(h->c.xb, 0, sizeof(double) * h->xb_len, h->stream), "clear x coefficients");
  if ((rc = dalloc(h, &h->err_dev, 1, "error word"))) return rc;
  if ((rc = dalloc(h, &h->status_dev, 1, "status word"))) return rc;
  double** slots[hs2g::kNumCoeffArrays] = {&h->c.a0, &h->c.b0, &h->c.a1, &h->c.b1, &h->c.a2, &h->c.b2};
  for (int s = 0; s < hs2g::kNumCoeffArrays; ++s) *slots[s] = h->coef_block + (int64_t)s * np;
  HS2G_CUDA(cudaMemsetAsync(h->err_dev, 0, sizeof(unsigned long long), h->stream), "clear error word");
  HS2G_CUDA(cudaMemsetAsync(h->status_dev, 0, sizeof(int), h->stream), "clear status word");
  // tensor-tile line sweeps need 16-byte aligned coefficient arrays (an even voxel count) and even row pitches
  HS2G_CUDA(hs2g::lines_bulk_prepare(), "configure line-sweep kernels");
  // Kernel variants (defaults are the fastest measured on GB300; the others stay selectable for comparison
  // and testing): HS2G_LINE_SWEEP=plain the plain-load y sweep, HS2G_Z_SWEEP=tma the TMA tensor-tile z sweep,
  // HS2G_Z_DISCARD=0 the plain z sweep leaving its forward values to L2's own eviction, HS2G_PDL=0 the step
  // graphs' sweeps launched without programmatic dependent launch (0.5702 against 0.5689 ms per step at
  // 65x512x512).
  const char* ymode = getenv("HS2G_LINE_SWEEP");
  const char* zmode = getenv("HS2G_Z_SWEEP");
  const char* zdiscard = getenv("HS2G_Z_DISCARD");
  const char* pdl = getenv("HS2G_PDL");
  h->z_discard = !(zdiscard && strcmp(zdiscard, "0") == 0);
  h->graph_pdl = !(pdl && strcmp(pdl, "0") == 0);
  h->bulk_y = !(ymode && strcmp(ymode, "plain") == 0) && hs2g::lines_bulk_supported(h->d, 1, h->c.px);
  h->bulk_z = (zmode && strcmp(zmode, "tma") == 0) && h->c.px == h->d.nx && (n % 2 == 0) &&
              hs2g::lines_bulk_supported(h->d, 2, h->d.nx);

  h->tmaps = hs2g::tensor_map_cache_create();
  return HS2G_OK;
}

// Step arguments common to every call; T pointers and the source table are filled in by the caller.
hs2g::StepArgs make_args(const hs2g_handle* h, const double* T_in, const double* T_out) {
  hs2g::StepArgs a{};
  a.d = h->d;
  a.W0 = h->W0;
  a.W1 = h->W1;
  a.vclass = h->vclass;
  a.status = h->status_dev;
  const bool aligned = ((reinterpret_cast<uintptr_t>(T_in) | reinterpret_cast<uintptr_t>(T_out)) & 15u) == 0;
  a.bulk_y = h->bulk_y;
  a.bulk_z = h->bulk_z && aligned;
  a.z_discard = h->z_discard;
  a.tmaps = h->tmaps;
  return a;
}

// After a synchronisation: report a bounded device wait that ran out (and clear the word).
int check_status(hs2g_handle* h) {
  int v = 0;
  HS2G_CUDA(cudaMemcpy(&v, h->status_dev, sizeof(int), cudaMemcpyDeviceToHost), "read status word");
  if (v == 0) return HS2G_OK;
  cudaMemset(h->status_dev, 0, sizeof(int));
  return fail(v, "a device wait in a sweep kernel ran out of time (error %d)", v);
}

int new_handle(int device, const Dims& d, hs2g_handle** out) {
  if (d.nz < 1 || d.ny < 1 || d.nx < 1) return fail(HS2G_ERR_ARG, "grid shape must be positive");
  if (d.nvox() > ((int64_t)1 << 40)) return fail(HS2G_ERR_ARG, "grid too large");
  hs2g_handle* h = new hs2g_handle();
  h->device = device;
  h->d = d;
  cudaError_t e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete h;
    return cuda_fail(e, "cudaStreamCreate");
  }
  h->stream = h->own_stream;
  *out = h;
  return HS2G_OK;
}

int factor(hs2g_handle* h) {
  const int64_t n = h->d.nvox();
  double *s2 = nullptr, *sigma = nullptr;
  int rc;
  if ((rc = dalloc(h, &s2, n, "factor scratch"))) return rc;
  if ((rc = dalloc(h, &sigma, n, "factor scratch"))) {
    dfree(h, s2, n);
    return rc;
  }
  cudaError_t e = hs2g::launch_factor(h->d, h->Gz, h->Gy, h->Gx, h->M, h->compute, s2, sigma, h->c, h->stream);
  cudaError_t e2 = cudaStreamSynchronize(h->stream);
  dfree(h, s2, n);
  dfree(h, sigma, n);
  if (e != cudaSuccess) return cuda_fail(e, "factor kernels");
  if (e2 != cudaSuccess) return cuda_fail(e2, "factor kernels");
  return HS2G_OK;
}

int ensure_staging(hs2g_handle* h) {
  const int64_t n = h->d.nvox();
  int rc;
  if (!h->Tin_dev && (rc = dalloc(h, &h->Tin_dev, n, "input staging"))) return rc;
  if (!h->Tout_dev && (rc = dalloc(h, &h->Tout_dev, n, "output staging"))) return rc;
  return HS2G_OK;
}

int ensure_copy_pipeline(hs2g_handle* h) {
  if (h->copy_stream) return HS2G_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking);
  for (int c = 0; c < kCopyChunks && e == cudaSuccess; ++c) {
    e = cudaStreamCreateWithFlags(&h->x_stream[c], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_in[c], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_x[c], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_out[c], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&h->ev_begin, cudaEventDisableTiming);
  if (e != cudaSuccess) return cuda_fail(e, "copy pipeline");
  return HS2G_OK;
}

// One step from host T_in to host T_out with the copies overlapped (see kCopyChunks).  Slab c of the upload
// holds planes [k_c, k_{c+1}); once it is in, the x sweep can run on x-lines of planes up to k_{c+1} - 2 (an
// x-line reads the planes above and below it).  The z sweep runs in blocks of rows j, each block's columns
// complete after its launch, and a 2-D copy takes those rows of every plane back to the host.
int step_host_pipelined(hs2g_handle* h, hs2g::StepArgs& a, const hs2g::QTable& q, const double* T_in,
                        double* T_out) {
  const Dims& d = h->d;
  cudaStream_t s = h->stream, cs = h->copy_stream;
  const int nout = (int)std::min<int64_t>(kCopyChunks, d.ny / 4);
  const size_t plane = sizeof(double) * (size_t)d.nxy();
  // the copy and x streams start after everything queued on the step stream so far (e.g. source uploads)
  HS2G_CUDA(cudaEventRecord(h->ev_begin, s), "pipeline begin");
  HS2G_CUDA(cudaStreamWaitEvent(cs, h->ev_begin, 0), "pipeline begin");
  int64_t k0 = 0, done = 0;  // planes [0, k0) are queued for upload; x-lines [0, done) for the x sweep
  for (int c = 0; c < kCopyChunks; ++c) {
    const int64_t k1 = c + 1 == kCopyChunks ? d.nz : std::min<int64_t>(d.nz, std::max<int64_t>(
                                                          k0 + 2, (int64_t)(kSlabEnd[c] * (double)d.nz)));
    if (k1 > k0) {
      HS2G_CUDA(cudaMemcpyAsync(h->Tin_dev + k0 * d.nxy(), T_in + k0 * d.nxy(), plane * (size_t)(k1 - k0),
                                cudaMemcpyHostToDevice, cs), "upload T");
    }
    HS2G_CUDA(cudaEventRecord(h->ev_in[c], cs), "upload T");
    cudaStream_t xs = h->x_stream[c];
    HS2G_CUDA(cudaStreamWaitEvent(xs, h->ev_begin, 0), "upload T");
    HS2G_CUDA(cudaStreamWaitEvent(xs, h->ev_in[c], 0), "upload T");
    const int64_t upto = (k1 == d.nz ? d.nz : k1 - 1) * d.ny;
    cudaError_t e = hs2g::launch_x_range(a, h->c, q, done, upto, kSlabLines[c], xs);
    if (e != cudaSuccess) return cuda_fail(e, "x sweep");
    HS2G_CUDA(cudaEventRecord(h->ev_x[c], xs), "x sweep");
    HS2G_CUDA(cudaStreamWaitEvent(s, h->ev_x[c], 0), "x sweep");
    done = upto;
    k0 = k1;
  }
  cudaError_t e = hs2g::launch_y(a, h->c, s);
  if (e != cudaSuccess) return cuda_fail(e, "y sweep");
  for (int c = 0; c < nout; ++c) {
    const int64_t j0 = d.ny * c / nout, j1 = d.ny * (c + 1) / nout;
    e = hs2g::launch_z_range(a, h->c, j0 * d.nx, j1 * d.nx, s);
    if (e != cudaSuccess) return cuda_fail(e, "z sweep");
    HS2G_CUDA(cudaEventRecord(h->ev_out[c], s), "download T");
    HS2G_CUDA(cudaStreamWaitEvent(cs, h->ev_out[c], 0), "download T");
    HS2G_CUDA(cudaMemcpy2DAsync(T_out + j0 * d.nx, plane, h->Tout_dev + j0 * d.nx, plane,
                                sizeof(double) * (size_t)((j1 - j0) * d.nx), (size_t)d.nz, cudaMemcpyDeviceToHost,
                                cs),
              "download T");
  }
  HS2G_CUDA(cudaStreamSynchronize(cs), "step");
  HS2G_CUDA(cudaStreamSynchronize(s), "step");
  return check_status(h);
}

// The shape field applies to a step whose table gives a shaped class a non-zero value.
const double* active_shape(const hs2g_handle* h, const double* qtab) {
  if (!h->qshape || !qtab) return nullptr;
  for (int c = 0; c < HS2G_MAX_CLASSES; ++c)
    if (h->shaped[c] && qtab[c] != 0.0) return h->qshape;
  return nullptr;
}

// A new source-class map invalidates every shape: reset the field to 1 and forget which classes had one.
int reset_shapes(hs2g_handle* h) {
  for (int c = 0; c < HS2G_MAX_CLASSES; ++c) h->shaped[c] = false;
  if (h->qshape) HS2G_CUDA(hs2g::launch_fill(h->qshape, h->d.nvox(), 1.0, h->stream), "reset source shapes");
  return HS2G_OK;
}

int ensure_shape(hs2g_handle* h) {
  if (h->qshape) return HS2G_OK;
  int rc = dalloc(h, &h->qshape, h->d.nvox(), "source shape");
  if (rc) return rc;
  HS2G_CUDA(hs2g::launch_fill(h->qshape, h->d.nvox(), 1.0, h->stream), "initialise source shape");
  return HS2G_OK;
}

// The device copy of a per-voxel input of a shaped class: the caller's pointer (HS2G_DEVICE), the copy kept
// from the previous call (HS2G_REUSE), or a fresh upload into the handle's buffer.
int shape_input(hs2g_handle* h, double** buf, int64_t* buf_len, int64_t len, const double* src, int flags,
                const char* what, const double** out) {
  if (flags & HS2G_DEVICE) {
    *out = src;
    return HS2G_OK;
  }
  if (flags & HS2G_REUSE) {
    if (!*buf || *buf_len != len) return fail(HS2G_ERR_STATE, "%s: nothing to reuse (no earlier upload of %lld values)", what, (long long)len);
    *out = *buf;
    return HS2G_OK;
  }
  if (*buf && *buf_len != len) {
    dfree(h, *buf, *buf_len);
    *buf_len = 0;
  }
  if (!*buf) {
    int rc = dalloc(h, buf, len, what);
    if (rc) return rc;
    *buf_len = len;
  }
  HS2G_CUDA(cudaMemcpyAsync(*buf, src, sizeof(double) * len, cudaMemcpyHostToDevice, h->stream), what);
  *out = *buf;
  return HS2G_OK;
}

}  // namespace

int hs2g::set_last_error(int code, const char* message) { return fail(code, "%s", message); }

extern "C" {

int hs2g_abi_version(void) { return HS2G_ABI_VERSION; }

const char* hs2g_last_error(void) { return g_last_error.c_str(); }

void hs2g_destroy(hs2g_handle* h) {
  if (!h) return;
  DeviceGuard g(h->device);
  cudaStreamSynchronize(h->stream);
  if (h->own_stream) cudaStreamSynchronize(h->own_stream);
  const int64_t n = h->d.nvox();
  dfree(h, h->status_dev, 1);
  hs2g::tensor_map_cache_destroy(h->tmaps);
  h->tmaps = nullptr;
  dfree(h, h->Gz, 0);
  dfree(h, h->Gy, 0);
  dfree(h, h->Gx, 0);
  dfree(h, h->M, n);
  dfree(h, h->compute, n);
  dfree(h, h->vclass, n);
  const int64_t np = h->d.nz * h->d.ny * h->c.px;
  dfree(h, h->coef_block, np * hs2g::kNumCoeffArrays);
  dfree(h, h->c.xb, h->xb_len);
  dfree(h, h->W0, np);
  dfree(h, h->W1, np);
  dfree(h, h->Tin_dev, n);
  dfree(h, h->Tout_dev, n);
  dfree(h, h->qdense_dev, n);
  dfree(h, h->hist_dev, h->hist_len);
  dfree(h, h->qshape, n);
  for (int c = 0; c < HS2G_MAX_CLASSES; ++c) {
    dfree(h, h->shape_zgrid[c], n);
    dfree(h, h->shape_joules[c], h->shape_joules_len[c]);
  }
  dfree(h, h->shape_volumes, n);
  dfree(h, h->shape_tiles, hs2g::point_shape_tiles(n));
  dfree(h, h->err_dev, 1);
  if (h->copy_stream) {
    cudaStreamSynchronize(h->copy_stream);
    cudaStreamDestroy(h->copy_stream);
  }
  for (int c = 0; c < kCopyChunks; ++c) {
    if (h->x_stream[c]) cudaStreamDestroy(h->x_stream[c]);
    if (h->ev_in[c]) cudaEventDestroy(h->ev_in[c]);
    if (h->ev_x[c]) cudaEventDestroy(h->ev_x[c]);
    if (h->ev_out[c]) cudaEventDestroy(h->ev_out[c]);
  }
  if (h->ev_begin) cudaEventDestroy(h->ev_begin);
  for (auto& g : h->graphs) cudaGraphExecDestroy(g.exec);
  if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
  dfree(h, h->sched_dev, 1);
  dfree(h, h->sched_q, h->sched_cap * HS2G_MAX_CLASSES);
  dfree(h, h->sched_active, h->sched_cap);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
}

int hs2g_create_classes(const hs2g_class_problem* p, int device, hs2g_handle** out) {
  if (!p || !out) return fail(HS2G_ERR_ARG, "null argument");
  *out = nullptr;
  if (!p->materials || !p->forms || !p->material || !p->boundary_z || !p->boundary_y || !p->boundary_x)
    return fail(HS2G_ERR_ARG, "null array in problem");
  if (p->nmat < 1 || p->nmat > HS2G_MAX_CLASSES || p->nbnd < 1 || p->nbnd > HS2G_MAX_CLASSES)
    return fail(HS2G_ERR_ARG, "material / boundary class count must be in 1..256");
  for (int b = 0; b < p->nbnd * 3; ++b)
    if (p->forms[b].nzero < 0 || p->forms[b].nzero > HS2G_MAX_ZERO_FORMS)
      return fail(HS2G_ERR_ARG, "boundary form %d has %d zero forms", b / 3, p->forms[b].nzero);
  DeviceGuard g(device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", device);
  hs2g_handle* h = nullptr;
  int rc = new_handle(device, Dims{p->nz, p->ny, p->nx}, &h);
  if (rc) return rc;
  const Dims& d = h->d;
  const int64_t n = d.nvox();
  uint8_t *mat = nullptr, *bz = nullptr, *by = nullptr, *bx = nullptr;
  hs2g_material* mats = nullptr;
  hs2g_face_form* forms = nullptr;
  auto cleanup_tmp = [&]() {
    dfree(h, mat, n);
    dfree(h, bz, 0);
    dfree(h, by, 0);
    dfree(h, bx, 0);
    dfree(h, mats, p->nmat);
    dfree(h, forms, p->nbnd * 3);
  };
  const int64_t nfz = (d.nz + 1) * d.nxy(), nfy = d.nz * (d.ny + 1) * d.nx, nfx = d.nz * d.ny * (d.nx + 1);
  if ((rc = alloc_common(h)) || (rc = dalloc(h, &mat, n, "material classes")) ||
      (rc = dalloc(h, &bz, nfz, "z boundary classes")) || (rc = dalloc(h, &by, nfy, "y boundary classes")) ||
      (rc = dalloc(h, &bx, nfx, "x boundary classes")) || (rc = dalloc(h, &mats, p->nmat, "material table")) ||
      (rc = dalloc(h, &forms, p->nbnd * 3, "boundary forms"))) {
    std::string msg = g_last_error;
    cleanup_tmp();
    hs2g_destroy(h);
    g_last_error = msg;
    return rc;
  }
  cudaStream_t s = h->stream;
  cudaError_t e = cudaSuccess;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
  };
  up(mat, p->material, (size_t)n);
  up(bz, p->boundary_z, (size_t)nfz);
  up(by, p->boundary_y, (size_t)nfy);
  up(bx, p->boundary_x, (size_t)nfx);
  up(mats, p->materials, sizeof(hs2g_material) * p->nmat);
  up(forms, p->forms, sizeof(hs2g_face_form) * p->nbnd * 3);
  if (p->volumetric)
    up(h->vclass, p->volumetric, (size_t)n);
  else if (e == cudaSuccess)
    e = cudaMemsetAsync(h->vclass, 0, (size_t)n, s);
  if (e == cudaSuccess) e = hs2g::launch_faces(d, 0, mat, bz, mats, p->nmat, forms, p->nbnd, h->Gz, h->err_dev, s);
  if (e == cudaSuccess) e = hs2g::launch_faces(d, 1, mat, by, mats, p->nmat, forms, p->nbnd, h->Gy, h->err_dev, s);
  if (e == cudaSuccess) e = hs2g::launch_faces(d, 2, mat, bx, mats, p->nmat, forms, p->nbnd, h->Gx, h->err_dev, s);
  if (e == cudaSuccess)
    e = hs2g::launch_capacity_from_classes(d, mat, mats, p->nmat, h->M, h->compute, h->err_dev, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cleanup_tmp();
  if (e != cudaSuccess) {
    rc = cuda_fail(e, "compile kernels");
  } else {
    rc = check_kernel_error(h);
  }
  if (!rc) rc = factor(h);
  if (rc) {
    std::string msg = g_last_error;
    hs2g_destroy(h);
    g_last_error = msg;
    return rc;
  }
  *out = h;
  return HS2G_OK;
}

int hs2g_create_dense(const hs2g_dense_problem* p, int device, hs2g_handle** out) {
  if (!p || !out) return fail(HS2G_ERR_ARG, "null argument");
  *out = nullptr;
  if (!p->Gz || !p->Gy || !p->Gx || !p->capacity) return fail(HS2G_ERR_ARG, "null array in problem");
  DeviceGuard g(device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", device);
  hs2g_handle* h = nullptr;
  int rc = new_handle(device, Dims{p->nz, p->ny, p->nx}, &h);
  if (rc) return rc;
  const Dims& d = h->d;
  const int64_t n = d.nvox();
  if ((rc = alloc_common(h))) {
    std::string msg = g_last_error;
    hs2g_destroy(h);
    g_last_error = msg;
    return rc;
  }
  cudaStream_t s = h->stream;
  cudaError_t e = cudaSuccess;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
  };
  up(h->Gz, p->Gz, sizeof(double) * (d.nz + 1) * d.nxy());
  up(h->Gy, p->Gy, sizeof(double) * d.nz * (d.ny + 1) * d.nx);
  up(h->Gx, p->Gx, sizeof(double) * d.nz * d.ny * (d.nx + 1));
  up(h->M, p->capacity, sizeof(double) * n);
  std::vector<uint8_t> comp((size_t)n, 1);
  if (p->fixed)
    for (int64_t v = 0; v < n; ++v) comp[(size_t)v] = p->fixed[v] ? 0 : 1;
  up(h->compute, comp.data(), (size_t)n);
  if (p->volumetric)
    up(h->vclass, p->volumetric, (size_t)n);
  else if (e == cudaSuccess)
    e = cudaMemsetAsync(h->vclass, 0, (size_t)n, s);
  if (e == cudaSuccess) e = hs2g::launch_validate_dense(d, h->Gz, h->Gy, h->Gx, h->M, h->compute, h->err_dev, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  rc = (e != cudaSuccess) ? cuda_fail(e, "dense compile") : check_kernel_error(h);
  if (!rc) rc = factor(h);
  if (rc) {
    std::string msg = g_last_error;
    hs2g_destroy(h);
    g_last_error = msg;
    return rc;
  }
  *out = h;
  return HS2G_OK;
}

int hs2g_create_rows(const hs2g_rows_problem* p, int device, hs2g_handle** out) {
  if (!p || !out) return fail(HS2G_ERR_ARG, "null argument");
  *out = nullptr;
  const double* src[6] = {p->zlo, p->zhi, p->ylo, p->yhi, p->xlo, p->xhi};
  for (const double* a : src)
    if (!a) return fail(HS2G_ERR_ARG, "null array in problem");
  if (!p->capacity) return fail(HS2G_ERR_ARG, "null array in problem");
  DeviceGuard g(device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", device);
  hs2g_handle* h = nullptr;
  int rc = new_handle(device, Dims{p->nz, p->ny, p->nx}, &h);
  if (rc) return rc;
  const Dims& d = h->d;
  const int64_t n = d.nvox();
  double* rows = nullptr;  // the six per-row arrays live on the device only while the problem is compiled
  auto bail = [&](int code) {
    std::string msg = g_last_error;
    if (rows) dfree(h, rows, 6 * n);
    hs2g_destroy(h);
    g_last_error = msg;
    return code;
  };
  h->per_row = true;
  if ((rc = alloc_common(h, false))) return bail(rc);
  if ((rc = dalloc(h, &rows, 6 * n, "per-row conductances"))) return bail(rc);
  cudaStream_t s = h->stream;
  cudaError_t e = cudaSuccess;
  auto up = [&](void* dst, const void* from, size_t bytes) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(dst, from, bytes, cudaMemcpyHostToDevice, s);
  };
  const double* dev_rows[6];
  for (int r = 0; r < 6; ++r) {
    dev_rows[r] = rows + (int64_t)r * n;
    up(rows + (int64_t)r * n, src[r], sizeof(double) * n);
  }
  up(h->M, p->capacity, sizeof(double) * n);
  std::vector<uint8_t> comp((size_t)n, 1);
  if (p->fixed)
    for (int64_t v = 0; v < n; ++v) comp[(size_t)v] = p->fixed[v] ? 0 : 1;
  up(h->compute, comp.data(), (size_t)n);
  if (p->volumetric)
    up(h->vclass, p->volumetric, (size_t)n);
  else if (e == cudaSuccess)
    e = cudaMemsetAsync(h->vclass, 0, (size_t)n, s);
  if (e == cudaSuccess) e = hs2g::launch_validate_rows(d, dev_rows, h->M, h->compute, h->err_dev, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  rc = (e != cudaSuccess) ? cuda_fail(e, "per-row compile") : check_kernel_error(h);
  if (rc) return bail(rc);
  double *s2 = nullptr, *sigma = nullptr;
  if ((rc = dalloc(h, &s2, n, "factor scratch"))) return bail(rc);
  if ((rc = dalloc(h, &sigma, n, "factor scratch"))) {
    dfree(h, s2, n);
    return bail(rc);
  }
  e = hs2g::launch_factor_rows(d, dev_rows, h->M, h->compute, s2, sigma, h->c, s);
  cudaError_t e2 = cudaStreamSynchronize(s);
  dfree(h, s2, n);
  dfree(h, sigma, n);
  dfree(h, rows, 6 * n);
  rows = nullptr;
  if (e != cudaSuccess) return bail(cuda_fail(e, "factor kernels"));
  if (e2 != cudaSuccess) return bail(cuda_fail(e2, "factor kernels"));
  *out = h;
  return HS2G_OK;
}

int hs2g_selftest_wait(int device, int64_t limit_ns, int arrive, int* status) {
  if (!status || limit_ns <= 0 || limit_ns > 10000000000ll)
    return fail(HS2G_ERR_ARG, "hs2g_selftest_wait: limit must be in (0, 10 s]");
  DeviceGuard g(device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", device);
  int* st = nullptr;
  cudaError_t e = cudaMalloc(&st, sizeof(int));
  if (e != cudaSuccess) return cuda_fail(e, "hs2g_selftest_wait");
  e = hs2g::wait_selftest((uint64_t)limit_ns, arrive, st, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(status, st, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(st);
  return e == cudaSuccess ? HS2G_OK : cuda_fail(e, "hs2g_selftest_wait");
}

int hs2g_set_stream(hs2g_handle* h, void* stream) {
  if (!h) return fail(HS2G_ERR_ARG, "null handle");
  h->stream = (cudaStream_t)stream;
  return HS2G_OK;
}

int hs2g_shape(const hs2g_handle* h, int64_t shape[3]) {
  if (!h || !shape) return fail(HS2G_ERR_ARG, "null argument");
  shape[0] = h->d.nz;
  shape[1] = h->d.ny;
  shape[2] = h->d.nx;
  return HS2G_OK;
}

int64_t hs2g_device_bytes(const hs2g_handle* h) { return h ? h->bytes : 0; }

int hs2g_source_table(int nsrc, const int32_t* kind, const double* params, double t, double dt, double volume,
                      double* qtab) {
  if (nsrc < 0 || nsrc > HS2G_MAX_CLASSES || !qtab || (nsrc > 0 && (!kind || !params)))
    return fail(HS2G_ERR_ARG, "bad source table arguments");
  int active = 0;
  for (int c = 0; c < HS2G_MAX_CLASSES; ++c) qtab[c] = 0.0;
  for (int c = 0; c < nsrc; ++c) {
    const double* a = params + 4 * c;
    double q = 0.0;
    switch (kind[c]) {
      case HS2G_NO_SOURCE:
        break;
      case HS2G_IMPULSE_SOURCE:  // exact time match, energy / dt (alternatingdirection_c_pyx.pyx:296-300)
        if (t == a[0]) q = a[1] / dt;
        break;
      case HS2G_STEPPED_SOURCE:  // inclusive window (pyx:301-306)
        if (t >= a[0] && t <= a[1]) q = a[2];
        break;
      case HS2G_IMPULSE_POINT_SOURCE_JOULES:  // joules per element / (volume * dt) (pyx:307-319)
        if (t == a[0]) q = a[1] / (volume * dt);
        break;
      case HS2G_SHAPED_IMPULSE:  // per-voxel value from the handle's source shape, at t == t0 exactly
        if (t == a[0]) q = 1.0;
        break;
      default:
        return fail(HS2G_ERR_ARG, "source class %d has kind %d, which is not evaluated per class", c, kind[c]);
    }
    qtab[c] = q;
    if (q != 0.0) ++active;
  }
  return active;
}

int hs2g_step(hs2g_handle* h, const double* T_in, double* T_out, const double* qtab, const double* qdense,
              const uint8_t* volumetric, int flags) {
  if (!h || !T_in || !T_out) return fail(HS2G_ERR_ARG, "null argument");
  DeviceGuard g(h->device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", h->device);
  const Dims& d = h->d;
  const int64_t n = d.nvox();
  const bool dev = (flags & HS2G_DEVICE) != 0;
  cudaStream_t s = h->stream;
  if (volumetric) {
    HS2G_CUDA(cudaMemcpyAsync(h->vclass, volumetric, (size_t)n, cudaMemcpyHostToDevice, s), "upload classes");
    int rc = reset_shapes(h);
    if (rc) return rc;
  }
  const double* Tin_d = T_in;
  double* Tout_d = T_out;
  if (!dev) {
    int rc = ensure_staging(h);
    if (rc) return rc;
    Tin_d = h->Tin_dev;
    Tout_d = h->Tout_dev;
  }
  hs2g::StepArgs a = make_args(h, Tin_d, Tout_d);
  hs2g::QTable q;
  a.has_qtab = false;
  if (qtab) {
    for (int c = 0; c < HS2G_MAX_CLASSES; ++c) {
      q.q[c] = qtab[c];
      if (qtab[c] != 0.0) a.has_qtab = true;
    }
  } else {
    memset(&q, 0, sizeof(q));
  }
  a.qshape = active_shape(h, qtab);
  if (qdense) {
    if (dev) {
      a.qdense = qdense;
    } else {
      int rc;
      if (!h->qdense_dev && (rc = dalloc(h, &h->qdense_dev, n, "source staging"))) return rc;
      HS2G_CUDA(cudaMemcpyAsync(h->qdense_dev, qdense, sizeof(double) * n, cudaMemcpyHostToDevice, s),
                "upload source field");
      a.qdense = h->qdense_dev;
    }
  }
  a.T_in = Tin_d;
  a.T_out = Tout_d;
  if (!dev && !a.bulk_z && n >= kPipelineMinVoxels && d.nz >= 8 && d.ny >= 8) {
    int rc = ensure_copy_pipeline(h);
    if (rc) return rc;
    return step_host_pipelined(h, a, q, T_in, T_out);
  }
  if (!dev)
    HS2G_CUDA(cudaMemcpyAsync(h->Tin_dev, T_in, sizeof(double) * n, cudaMemcpyHostToDevice, s), "upload T");
  cudaError_t e = hs2g::launch_step(a, h->c, q, s);
  if (e != cudaSuccess) return cuda_fail(e, "step kernels");
  if (!dev) {
    HS2G_CUDA(cudaMemcpyAsync(T_out, h->Tout_dev, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "download T");
    HS2G_CUDA(cudaStreamSynchronize(s), "step");
    return check_status(h);
  } else if (flags & HS2G_SYNC) {
    HS2G_CUDA(cudaStreamSynchronize(s), "step");
    return check_status(h);
  }
  return HS2G_OK;
}

namespace {
int ensure_schedule(hs2g_handle* h) {
  if (h->sched_dev) return HS2G_OK;
  int rc = dalloc(h, &h->sched_dev, 1, "source schedule");
  if (rc) return rc;
  HS2G_CUDA(cudaMemsetAsync(h->sched_dev, 0, sizeof(hs2g::DevSchedule), h->stream), "clear source schedule");
  return HS2G_OK;
}

// Queue the schedule descriptor's rows, flags, row count and shape field on the handle's stream.  The
// descriptor names the shape field only while some class has a shape: a voxel's class value is multiplied by
// its shape value, which is 1 for every voxel of a class without one, so the product is exact for those classes.
int write_schedule_header(hs2g_handle* h) {
  bool any_shape = false;
  for (int c = 0; c < HS2G_MAX_CLASSES && h->qshape; ++c) any_shape |= h->shaped[c];
  const hs2g::DevSchedule hdr{h->sched_q, h->sched_active, any_shape ? h->qshape : nullptr, h->sched_n, 0, 0, 0};
  // a pageable source is staged before the call returns, so the local descriptor may go out of scope
  HS2G_CUDA(cudaMemcpyAsync(h->sched_dev, &hdr, offsetof(hs2g::DevSchedule, step), cudaMemcpyHostToDevice,
                            h->stream),
            "write source schedule");
  return HS2G_OK;
}

// Replace the schedule's rows by qtabs[nsteps][HS2G_MAX_CLASSES] (host, or device when device_ptr) and set the
// clock to 0.  Work already queued on the handle's stream reads the old rows before they are overwritten.  The
// flags (row has a non-zero value) are kept on both sides: the host picks each step's graph from them.  Host
// rows are flagged on the host; device rows on the device, and read back (the call then waits for the stream).
int set_schedule_rows(hs2g_handle* h, int64_t nsteps, const double* qtabs, bool device_ptr) {
  int rc = ensure_schedule(h);
  if (rc) return rc;
  if (nsteps > h->sched_cap) {
    HS2G_CUDA(cudaStreamSynchronize(h->stream), "source schedule");  // queued steps may read the old rows
    dfree(h, h->sched_q, h->sched_cap * HS2G_MAX_CLASSES);
    dfree(h, h->sched_active, h->sched_cap);
    h->sched_cap = h->sched_n = 0;
    if ((rc = dalloc(h, &h->sched_q, nsteps * HS2G_MAX_CLASSES, "source schedule rows"))) return rc;
    if ((rc = dalloc(h, &h->sched_active, nsteps, "source schedule flags"))) return rc;
    h->sched_cap = nsteps;
  }
  h->sched_flags.assign((size_t)nsteps, 0);
  if (nsteps > 0) {
    HS2G_CUDA(cudaMemcpyAsync(h->sched_q, qtabs, sizeof(double) * HS2G_MAX_CLASSES * (size_t)nsteps,
                              device_ptr ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->stream),
              "upload source schedule");
    if (device_ptr) {
      HS2G_CUDA(hs2g::launch_schedule_flags(h->sched_q, nsteps, h->sched_active, h->stream), "schedule flags");
      HS2G_CUDA(cudaMemcpyAsync(h->sched_flags.data(), h->sched_active, (size_t)nsteps, cudaMemcpyDeviceToHost,
                                h->stream),
                "read schedule flags");
      HS2G_CUDA(cudaStreamSynchronize(h->stream), "source schedule");
    } else {
      for (int64_t r = 0; r < nsteps; ++r)
        for (int c = 0; c < HS2G_MAX_CLASSES && !h->sched_flags[(size_t)r]; ++c)
          h->sched_flags[(size_t)r] = qtabs[r * HS2G_MAX_CLASSES + c] != 0.0;
      // pageable source: staged before the call returns, so the flags may change on the host afterwards
      HS2G_CUDA(cudaMemcpyAsync(h->sched_active, h->sched_flags.data(), (size_t)nsteps, cudaMemcpyHostToDevice,
                                h->stream),
                "upload schedule flags");
    }
  }
  h->sched_n = nsteps;
  h->clock = 0;
  return write_schedule_header(h);
}

// One step src -> dst queued on s: with `source`, the x sweep whose class table is the schedule's row at the
// device clock (set by the caller), else the x sweep without a source; then y, z and the history row.
cudaError_t queue_step(hs2g_handle* h, const double* src, double* dst, double* hist, int layer, double dz2,
                       bool source, cudaStream_t s, bool pdl = false, bool pdl_x = false) {
  hs2g::StepArgs a = make_args(h, src, dst);
  a.T_in = src;
  a.T_out = dst;
  a.pdl = pdl;
  a.pdl_x = pdl_x;
  cudaError_t e;
  if (source) {
    e = hs2g::launch_step_row(a, h->c, h->sched_dev, s);
  } else {
    hs2g::QTable q;
    memset(&q, 0, sizeof(q));
    a.has_qtab = false;
    e = hs2g::launch_step(a, h->c, q, s);
  }
  if (e == cudaSuccess && hist) e = hs2g::launch_history_row(h->d, dst, layer, dz2, hist, h->sched_dev, s, pdl);
  return e;
}

// The captured in-place steps on T (T_in == T_out == T): one step with a source, or `steps` without; from the
// handle's cache or captured now.
constexpr size_t kMaxStepGraphs = 8;
int step_graph(hs2g_handle* h, double* T, double* hist, int layer, double dz2, bool source, int steps,
               cudaGraphExec_t* out) {
  for (const auto& g : h->graphs)
    if (g.T == T && g.hist == hist && g.layer == layer && g.dz2 == dz2 && g.source == source && g.steps == steps) {
      *out = g.exec;
      return HS2G_OK;
    }
  if (!h->cap_stream)
    HS2G_CUDA(cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking), "capture stream");
  HS2G_CUDA(cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal), "begin step capture");
  cudaError_t e = cudaSuccess;
  for (int k = 0; k < steps && e == cudaSuccess; ++k)
    e = queue_step(h, T, T, hist, layer, dz2, source, h->cap_stream, h->graph_pdl, h->graph_pdl && k > 0);
  cudaGraph_t g = nullptr;
  const cudaError_t e_end = cudaStreamEndCapture(h->cap_stream, &g);
  if (e == cudaSuccess) e = e_end;
  cudaGraphExec_t exec = nullptr;
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_fail(e, "capture of the step graph");
  }
  if (h->graphs.size() >= kMaxStepGraphs) {  // a graph still executing is released when it completes
    cudaGraphExecDestroy(h->graphs.front().exec);
    h->graphs.erase(h->graphs.begin());
  }
  h->graphs.push_back({T, hist, layer, dz2, source, steps, exec});
  *out = exec;
  return HS2G_OK;
}

// Steps without a source are replayed kStepsPerGraph at a time: the boundary between two graph launches costs
// about 3 us more than one between kernels of a graph (0.5777 against 0.5810 ms per step at 65x512x512; 16
// steps per graph measured the same as 4).
constexpr int kStepsPerGraph = 4;

// hs2g_run and hs2g_run_surface: after every step, history receives layer record_layer of T, or (surface_dz > 0)
// the insulating z = 0 surface temperature estimated from layers 0 and 1.  The first step of a call with
// T_in != T_out is queued directly; the others are replays of captured in-place step graphs.  A scheduled
// step whose row has a source writes the clock to the descriptor and replays the one-step source graph; runs
// of steps without one replay the plain graphs.
int run_steps(hs2g_handle* h, int nsteps, const double* T_in, double* T_out, const double* qtabs, int record_layer,
              double surface_dz, double* history, int flags) {
  DeviceGuard g(h->device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", h->device);
  const Dims& d = h->d;
  const int64_t n = d.nvox();
  const bool dev = (flags & HS2G_DEVICE) != 0;
  cudaStream_t s = h->stream;
  int rc = ensure_schedule(h);
  if (rc) return rc;
  bool scheduled = (flags & HS2G_SCHEDULED) != 0;
  if (qtabs) {
    if ((rc = set_schedule_rows(h, nsteps, qtabs, false))) return rc;
    scheduled = true;
  } else if ((rc = write_schedule_header(h))) {  // the shape field may have changed since the schedule was set
    return rc;
  }
  const double* src = T_in;
  double* dst = T_out;
  if (!dev) {
    if ((rc = ensure_staging(h))) return rc;
    HS2G_CUDA(cudaMemcpyAsync(h->Tin_dev, T_in, sizeof(double) * n, cudaMemcpyHostToDevice, s), "upload T");
    src = h->Tin_dev;
    dst = h->Tout_dev;
  }
  double* hist = nullptr;
  if (history) {
    if (dev) {
      hist = history;
    } else {
      const int64_t need = (int64_t)nsteps * d.nxy();
      if (need > h->hist_len) {
        dfree(h, h->hist_dev, h->hist_len);
        h->hist_len = 0;
        if ((rc = dalloc(h, &h->hist_dev, need, "surface history"))) return rc;
        h->hist_len = need;
      }
      hist = h->hist_dev;
    }
    // the history row and the count of the history kernel's finished CTAs start at 0
    HS2G_CUDA(cudaMemsetAsync(&h->sched_dev->row, 0, sizeof(int64_t) + sizeof(unsigned int), s),
              "reset history row");
  }
  const int layer = hist && surface_dz <= 0.0 ? record_layer : 0;
  const double dz2 = hist && surface_dz > 0.0 ? hs2g::surface_dz2(surface_dz) : 0.0;
  // whether scheduled step `i` of this call has a source, and queueing one such step (its row set first)
  auto has_source = [&](int i) {
    const int64_t st = h->clock + i;
    return scheduled && st < h->sched_n && h->sched_flags[(size_t)st] != 0;
  };
  auto set_row = [&](int i) {
    const int64_t st = h->clock + i;
    return cudaMemcpyAsync(&h->sched_dev->step, &st, sizeof(st), cudaMemcpyHostToDevice, s);
  };
  int done = 0;
  if (nsteps > 0 && src != dst) {
    const bool source = has_source(0);
    cudaError_t e = source ? set_row(0) : cudaSuccess;
    if (e == cudaSuccess) e = queue_step(h, src, dst, hist, layer, dz2, source, s);
    if (e != cudaSuccess) return cuda_fail(e, "step kernels");
    done = 1;
  }
  while (done < nsteps) {
    cudaGraphExec_t graph = nullptr;
    if (has_source(done)) {
      HS2G_CUDA(set_row(done), "set schedule row");
      if ((rc = step_graph(h, dst, hist, layer, dz2, true, 1, &graph))) return rc;
      HS2G_CUDA(cudaGraphLaunch(graph, s), "step graph");
      ++done;
      continue;
    }
    int idle = 1;  // steps without a source from here on
    while (done + idle < nsteps && !has_source(done + idle)) ++idle;
    if (idle >= kStepsPerGraph) {
      if ((rc = step_graph(h, dst, hist, layer, dz2, false, kStepsPerGraph, &graph))) return rc;
      for (; idle >= kStepsPerGraph; idle -= kStepsPerGraph, done += kStepsPerGraph)
        HS2G_CUDA(cudaGraphLaunch(graph, s), "step graph");
    }
    if (idle > 0) {
      if ((rc = step_graph(h, dst, hist, layer, dz2, false, 1, &graph))) return rc;
      for (; idle > 0; --idle, ++done) HS2G_CUDA(cudaGraphLaunch(graph, s), "step graph");
    }
  }
  if (scheduled) h->clock += nsteps;
  if (nsteps == 0 && src != dst) {
    HS2G_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, s), "copy T");
  }
  if (!dev) {
    HS2G_CUDA(cudaMemcpyAsync(T_out, h->Tout_dev, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "download T");
    if (history)
      HS2G_CUDA(cudaMemcpyAsync(history, h->hist_dev, sizeof(double) * nsteps * d.nxy(), cudaMemcpyDeviceToHost, s),
                "download history");
    HS2G_CUDA(cudaStreamSynchronize(s), "run");
    return check_status(h);
  } else if (flags & HS2G_SYNC) {
    HS2G_CUDA(cudaStreamSynchronize(s), "run");
    return check_status(h);
  }
  return HS2G_OK;
}
}  // namespace

int hs2g_set_schedule(hs2g_handle* h, int64_t nsteps, const double* qtabs, int flags) {
  if (!h || nsteps < 0 || (nsteps > 0 && !qtabs)) return fail(HS2G_ERR_ARG, "hs2g_set_schedule: bad argument");
  DeviceGuard g(h->device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", h->device);
  int rc = set_schedule_rows(h, nsteps, qtabs, (flags & HS2G_DEVICE) != 0);
  if (rc) return rc;
  if (flags & HS2G_SYNC) HS2G_CUDA(cudaStreamSynchronize(h->stream), "hs2g_set_schedule");
  return HS2G_OK;
}

int hs2g_set_clock(hs2g_handle* h, int64_t step) {
  if (!h || step < 0) return fail(HS2G_ERR_ARG, "hs2g_set_clock: bad argument");
  h->clock = step;
  return HS2G_OK;
}

int hs2g_get_clock(hs2g_handle* h, int64_t* step) {
  if (!h || !step) return fail(HS2G_ERR_ARG, "hs2g_get_clock: bad argument");
  *step = h->clock;
  return HS2G_OK;
}

int hs2g_run(hs2g_handle* h, int nsteps, const double* T_in, double* T_out, const double* qtabs,
             int record_layer, double* history, int flags) {
  if (!h || !T_in || !T_out || nsteps < 0) return fail(HS2G_ERR_ARG, "bad argument");
  if (history && (record_layer < 0 || record_layer >= h->d.nz))
    return fail(HS2G_ERR_ARG, "record_layer %d outside 0..%lld", record_layer, (long long)h->d.nz - 1);
  return run_steps(h, nsteps, T_in, T_out, qtabs, record_layer, 0.0, history, flags);
}

int hs2g_run_surface(hs2g_handle* h, int nsteps, const double* T_in, double* T_out, const double* qtabs, double dz,
                     double* history, int flags) {
  if (!h || !T_in || !T_out || !history || nsteps < 0) return fail(HS2G_ERR_ARG, "bad argument");
  if (!(dz > 0.0) || !std::isfinite(dz)) return fail(HS2G_ERR_ARG, "dz must be positive and finite");
  if (h->d.nz < 2) return fail(HS2G_ERR_ARG, "the surface estimate needs nz >= 2");
  return run_steps(h, nsteps, T_in, T_out, qtabs, 0, dz, history, flags);
}

int hs2g_surface_temperature(int device, int64_t nz, int64_t ny, int64_t nx, const double* T, double dz,
                             double* out, void* stream, int flags) {
  if (!T || !out || nz < 2 || ny < 1 || nx < 1 || ny > (int64_t(1) << 40) / nx)
    return fail(HS2G_ERR_ARG, "bad argument (the surface estimate needs nz >= 2)");
  if (!(dz > 0.0) || !std::isfinite(dz)) return fail(HS2G_ERR_ARG, "dz must be positive and finite");
  DeviceGuard g(device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", device);
  cudaStream_t s = (cudaStream_t)stream;
  const int64_t nxy = ny * nx;
  if (flags & HS2G_DEVICE) {
    HS2G_CUDA(hs2g::launch_surface_estimate(nxy, T, dz, out, s), "surface estimate");
    if (flags & HS2G_SYNC) HS2G_CUDA(cudaStreamSynchronize(s), "surface estimate");
    return HS2G_OK;
  }
  // host pointers: layers 0 and 1 up, the estimate down (temporary device buffers)
  double* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, sizeof(double) * 3 * nxy);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? HS2G_ERR_NOMEM : HS2G_ERR_CUDA, "surface estimate: %s",
                cudaGetErrorString(e));
  }
  e = cudaMemcpyAsync(buf, T, sizeof(double) * 2 * nxy, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = hs2g::launch_surface_estimate(nxy, buf, dz, buf + 2 * nxy, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(out, buf + 2 * nxy, sizeof(double) * nxy, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(buf);
  if (e != cudaSuccess) return fail(HS2G_ERR_CUDA, "surface estimate: %s", cudaGetErrorString(e));
  return HS2G_OK;
}

int hs2g_run_timed(hs2g_handle* h, int nsteps, const double* T_in, double* T_out, const double* qtabs, int flags,
                   double* kernel_ms) {
  if (!h || !T_in || !T_out || nsteps < 0 || !kernel_ms) return fail(HS2G_ERR_ARG, "bad argument");
  if (!(flags & HS2G_DEVICE)) return fail(HS2G_ERR_ARG, "hs2g_run_timed takes device pointers");
  DeviceGuard g(h->device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", h->device);
  cudaStream_t s = h->stream;
  std::vector<cudaEvent_t> ev((size_t)nsteps * 4);
  for (auto& e : ev) HS2G_CUDA(cudaEventCreate(&e), "cudaEventCreate");
  hs2g::StepArgs a = make_args(h, T_in, T_out);
  hs2g::QTable q;
  memset(&q, 0, sizeof(q));
  const double* src = T_in;
  int rc = HS2G_OK;
  for (int st = 0; st < nsteps && rc == HS2G_OK; ++st) {
    a.has_qtab = false;
    a.qshape = nullptr;
    if (qtabs) {
      const double* qt = qtabs + (int64_t)st * HS2G_MAX_CLASSES;
      for (int c = 0; c < HS2G_MAX_CLASSES; ++c) {
        q.q[c] = qt[c];
        if (qt[c] != 0.0) a.has_qtab = true;
      }
      a.qshape = active_shape(h, qt);
    }
    a.T_in = src;
    a.T_out = T_out;
    cudaError_t e = hs2g::launch_step_events(a, h->c, q, s, &ev[(size_t)st * 4]);
    if (e != cudaSuccess) rc = cuda_fail(e, "step kernels");
    src = T_out;
  }
  if (rc == HS2G_OK) {
    cudaError_t e = cudaStreamSynchronize(s);
    rc = (e != cudaSuccess) ? cuda_fail(e, "run") : check_status(h);
  }
  kernel_ms[0] = kernel_ms[1] = kernel_ms[2] = kernel_ms[3] = 0.0;
  for (int st = 0; st < nsteps && rc == HS2G_OK; ++st)
    for (int k = 0; k < 3; ++k) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ev[(size_t)st * 4 + k], ev[(size_t)st * 4 + k + 1]);
      kernel_ms[k] += ms;
    }
  if (rc == HS2G_OK && nsteps > 0) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev[0], ev[(size_t)(nsteps - 1) * 4 + 3]);
    kernel_ms[3] = ms;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return rc;
}

int hs2g_fp64_fma_rate(int device, double* fma_per_s) {
  if (!fma_per_s) return fail(HS2G_ERR_ARG, "null argument");
  DeviceGuard g(device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", device);
  cudaError_t e = hs2g::fp64_fma_rate(fma_per_s);
  if (e != cudaSuccess) return cuda_fail(e, "fp64 probe");
  return HS2G_OK;
}

int hs2g_get_faces(hs2g_handle* h, double* Gz, double* Gy, double* Gx, double* capacity, uint8_t* fixed) {
  if (!h) return fail(HS2G_ERR_ARG, "null handle");
  if (h->per_row && (Gz || Gy || Gx))
    return fail(HS2G_ERR_STATE, "a per-row problem has no shared face conductances");
  DeviceGuard g(h->device);
  const Dims& d = h->d;
  const int64_t n = d.nvox();
  cudaStream_t s = h->stream;
  if (Gz) HS2G_CUDA(cudaMemcpyAsync(Gz, h->Gz, sizeof(double) * (d.nz + 1) * d.nxy(), cudaMemcpyDeviceToHost, s), "Gz");
  if (Gy)
    HS2G_CUDA(cudaMemcpyAsync(Gy, h->Gy, sizeof(double) * d.nz * (d.ny + 1) * d.nx, cudaMemcpyDeviceToHost, s), "Gy");
  if (Gx)
    HS2G_CUDA(cudaMemcpyAsync(Gx, h->Gx, sizeof(double) * d.nz * d.ny * (d.nx + 1), cudaMemcpyDeviceToHost, s), "Gx");
  if (capacity) HS2G_CUDA(cudaMemcpyAsync(capacity, h->M, sizeof(double) * n, cudaMemcpyDeviceToHost, s), "M");
  std::vector<uint8_t> comp;
  if (fixed) {
    comp.resize((size_t)n);
    HS2G_CUDA(cudaMemcpyAsync(comp.data(), h->compute, (size_t)n, cudaMemcpyDeviceToHost, s), "mask");
  }
  HS2G_CUDA(cudaStreamSynchronize(s), "get faces");
  if (fixed)
    for (int64_t v = 0; v < n; ++v) fixed[v] = comp[(size_t)v] ? 0 : 1;
  return HS2G_OK;
}

int hs2g_set_source_classes(hs2g_handle* h, const uint8_t* volumetric, int flags) {
  if (!h || !volumetric) return fail(HS2G_ERR_ARG, "null argument");
  DeviceGuard g(h->device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", h->device);
  const cudaMemcpyKind kind = (flags & HS2G_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  HS2G_CUDA(cudaMemcpyAsync(h->vclass, volumetric, (size_t)h->d.nvox(), kind, h->stream), "upload classes");
  int rc = reset_shapes(h);
  if (rc) return rc;
  if (flags & HS2G_SYNC) HS2G_CUDA(cudaStreamSynchronize(h->stream), "upload classes");
  return HS2G_OK;
}

int hs2g_source_zdecay(hs2g_handle* h, int cls, const double* zgrid, double direction, double offset, double ddz,
                       double joules_per_m2, double length, double dt, int flags) {
  if (!h || (!zgrid && !(flags & HS2G_REUSE))) return fail(HS2G_ERR_ARG, "null argument");
  if (cls < 0 || cls >= HS2G_MAX_CLASSES) return fail(HS2G_ERR_ARG, "source class %d outside 0..255", cls);
  if (!(direction == 1.0 || direction == -1.0))
    return fail(HS2G_ERR_ARG, "the decay direction must be +z or -z (direction +1 or -1)");
  if (!(length > 0.0) || !(ddz > 0.0) || !(dt > 0.0) || !std::isfinite(offset) || !std::isfinite(joules_per_m2))
    return fail(HS2G_ERR_ARG, "z-decaying impulse: length, ddz and dt must be positive, offset and J finite");
  DeviceGuard g(h->device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", h->device);
  const int64_t n = h->d.nvox();
  int rc = ensure_shape(h);
  if (rc) return rc;
  int64_t len = h->shape_zgrid[cls] ? n : 0;
  const double* z = nullptr;
  if ((rc = shape_input(h, &h->shape_zgrid[cls], &len, n, zgrid, flags, "z coordinates", &z))) return rc;
  HS2G_CUDA(hs2g::launch_zdecay_shape(n, h->vclass, cls, z, direction, offset, ddz, joules_per_m2, length, dt,
                                      h->qshape, h->stream),
            "z-decaying source shape");
  h->shaped[cls] = true;
  if (flags & HS2G_SYNC) HS2G_CUDA(cudaStreamSynchronize(h->stream), "z-decaying source shape");
  return HS2G_OK;
}

int hs2g_source_point(hs2g_handle* h, int cls, const double* joules, int64_t count, const double* volumes,
                      double volume, double dt, int flags) {
  if (!h || (!joules && !(flags & HS2G_REUSE)) || count < 1) return fail(HS2G_ERR_ARG, "bad argument");
  if (cls < 0 || cls >= HS2G_MAX_CLASSES) return fail(HS2G_ERR_ARG, "source class %d outside 0..255", cls);
  if (!(dt > 0.0) || (!volumes && !(volume > 0.0)))
    return fail(HS2G_ERR_ARG, "point source: dt and the cell volume must be positive");
  DeviceGuard g(h->device);
  if (!g.ok) return fail(HS2G_ERR_CUDA, "cannot select device %d", h->device);
  const int64_t n = h->d.nvox();
  int rc = ensure_shape(h);
  if (rc) return rc;
  if (!h->shape_tiles && (rc = dalloc(h, &h->shape_tiles, hs2g::point_shape_tiles(n), "rank scan"))) return rc;
  const double* J = nullptr;
  if ((rc = shape_input(h, &h->shape_joules[cls], &h->shape_joules_len[cls], count, joules, flags, "joules", &J)))
    return rc;
  const double* V = nullptr;
  if (volumes) {
    // the per-cell volumes follow the same DEVICE / REUSE rule as the joules
    int64_t vlen = h->shape_volumes ? n : 0;
    if ((rc = shape_input(h, &h->shape_volumes, &vlen, n, volumes, flags, "cell volumes", &V))) return rc;
  }
  HS2G_CUDA(hs2g::launch_point_shape(n, h->vclass, cls, h->shape_tiles, J, count, V, volume, dt, h->qshape,
                                     h->stream),
            "point source shape");
  h->shaped[cls] = true;
  if (flags & HS2G_SYNC) HS2G_CUDA(cudaStreamSynchronize(h->stream), "point source shape");
  return HS2G_OK;
}

}  // extern "C"
