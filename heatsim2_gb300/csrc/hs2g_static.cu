// hs2g_step_static: one ADI timestep that allocates no memory.
//
// For callers that cannot call cudaMalloc: a plugin inside a host application that owns every device
// allocation and forbids its plugins from allocating (a fixed device-memory budget, or a pool allocator that
// must not be bypassed), or code running where allocation is not allowed.  Such a caller cannot create an
// hs2g handle (hs2g_create_* allocates the compiled coefficients and the stage buffers), so this entry point
// takes the problem itself -- per-face conductances, per-voxel capacities, the fixed-temperature mask and the
// source field, all in caller-owned device memory -- and factorises every line on the fly.
//
// Its intermediate fields live in one file-scope __device__ array (kStaticVoxels voxels x 3 doubles, 24 MiB),
// which every GPU that loads the library holds until the process exits.  Every call shares that array and it
// keeps the last call's contents; nothing in it has to start at zero, because each call writes every element
// it later reads.  Calls that overlap on the GPU (on different streams, or from different host threads)
// race on the array and must be serialised by the caller.
//
// The array's host-side name is only a stand-in for it; its device address is taken with
// cudaGetSymbolAddress on the first call made with a device current, and again after that device's context
// changed (a cudaDeviceReset reloads the module at a new address).  Make that first call before any stream
// capture.
//
// The call validates what the kernels read: every computed voxel's capacity must be positive and finite.
// The kernels record the first bad voxel in a device status word next to the array, and the call waits for
// them (it synchronises `stream`) to return HS2G_ERR_CAPACITY; the output is then not a valid step.
//
// Arithmetic: the Douglas delta form of the step, (M - Lx/2) dT0 = L T + Q, (M - Ly/2) dT1 = M dT0,
// (M - Lz/2) dT2 = M dT1, T' = T + dT2, each line solved by the Thomas algorithm in the reference's
// normalisation (tridiag.pyx:25-41, :58-67) with the pivots formed as the line is swept.  One thread per line.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdio>
#include <mutex>

#include "hs2g_internal.cuh"

namespace {

constexpr int64_t kStaticVoxels = HS2G_STATIC_MAX_VOXELS;
constexpr int kMaxDevices = 64;

// dT0 / dT2 forward values, dT1, and the current sweep's normalised super-diagonal u = hi / pivot
__device__ __align__(256) double g_static_scratch[3 * kStaticVoxels];
// first invalid voxel seen by the kernels of the current call (hs2g::record_error encoding), 0 when none
__device__ unsigned long long g_static_status;

struct StaticView {
  double* w0;
  double* w1;
  double* u;
};

struct Problem {
  hs2g::Dims d;
  const double* Gz;
  const double* Gy;
  const double* Gx;
  const double* M;
  const uint8_t* fixed;
  const double* Q;
};

__device__ __forceinline__ bool computed(const Problem& P, int64_t p) { return !P.fixed || P.fixed[p] == 0; }

// Stage 0: R0 = sum over faces of G (T_nbr - T) + Q along all three axes; solve (M - Lx/2) dT0 = R0 on x-lines.
__global__ void static_x_kernel(Problem P, const double* __restrict__ T, StaticView s) {
  const hs2g::Dims& d = P.d;
  const int64_t L = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (L >= d.nz * d.ny) return;
  const int64_t k = L / d.ny, j = L - k * d.ny;
  const int64_t nxy = d.nxy();
  double u_prev = 0.0, z = 0.0;
  for (int64_t i = 0; i < d.nx; ++i) {
    const int64_t p = L * d.nx + i;
    double dd = 1.0, lo = 0.0, hi = 0.0, r = 0.0;
    if (computed(P, p)) {
      if (!(P.M[p] > 0.0 && P.M[p] < INFINITY)) hs2g::record_error(&g_static_status, HS2G_ERR_CAPACITY, 3, p);
      const int64_t fx = L * (d.nx + 1) + i, fy = (k * (d.ny + 1) + j) * d.nx + i;
      const double t = T[p];
      const double gxl = i > 0 ? P.Gx[fx] : 0.0, gxh = i + 1 < d.nx ? P.Gx[fx + 1] : 0.0;
      const double gyl = j > 0 ? P.Gy[fy] : 0.0, gyh = j + 1 < d.ny ? P.Gy[fy + d.nx] : 0.0;
      const double gzl = k > 0 ? P.Gz[p] : 0.0, gzh = k + 1 < d.nz ? P.Gz[p + nxy] : 0.0;
      if (gxl != 0.0) r += gxl * (T[p - 1] - t);
      if (gxh != 0.0) r += gxh * (T[p + 1] - t);
      if (gyl != 0.0) r += gyl * (T[p - d.nx] - t);
      if (gyh != 0.0) r += gyh * (T[p + d.nx] - t);
      if (gzl != 0.0) r += gzl * (T[p - nxy] - t);
      if (gzh != 0.0) r += gzh * (T[p + nxy] - t);
      if (P.Q) r += P.Q[p];
      dd = P.M[p] + 0.5 * (gxl + gxh);
      lo = -(0.5 * gxl);
      hi = -(0.5 * gxh);
    }
    const double piv = dd - u_prev * lo;
    z = (r - lo * z) / piv;
    u_prev = hi / piv;
    s.w0[p] = z;
    s.u[p] = u_prev;
  }
  double x = 0.0;
  for (int64_t i = d.nx - 1; i >= 0; --i) {
    const int64_t p = L * d.nx + i;
    x = s.w0[p] - s.u[p] * x;
    s.w0[p] = x;
  }
}

// Stage 1: (M - Ly/2) dT1 = M dT0 on y-lines.
__global__ void static_y_kernel(Problem P, StaticView s) {
  const hs2g::Dims& d = P.d;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= d.nz * d.nx) return;
  const int64_t k = t / d.nx, i = t - k * d.nx;
  double u_prev = 0.0, z = 0.0;
  for (int64_t j = 0; j < d.ny; ++j) {
    const int64_t p = (k * d.ny + j) * d.nx + i;
    double dd = 1.0, lo = 0.0, hi = 0.0, r = 0.0;
    if (computed(P, p)) {
      const int64_t fy = (k * (d.ny + 1) + j) * d.nx + i;
      const double gyl = j > 0 ? P.Gy[fy] : 0.0, gyh = j + 1 < d.ny ? P.Gy[fy + d.nx] : 0.0;
      r = P.M[p] * s.w0[p];
      dd = P.M[p] + 0.5 * (gyl + gyh);
      lo = -(0.5 * gyl);
      hi = -(0.5 * gyh);
    }
    const double piv = dd - u_prev * lo;
    z = (r - lo * z) / piv;
    u_prev = hi / piv;
    s.w1[p] = z;
    s.u[p] = u_prev;
  }
  double x = 0.0;
  for (int64_t j = d.ny - 1; j >= 0; --j) {
    const int64_t p = (k * d.ny + j) * d.nx + i;
    x = s.w1[p] - s.u[p] * x;
    s.w1[p] = x;
  }
}

// Stage 2: (M - Lz/2) dT2 = M dT1 on z-lines; T_out = T_in + dT2.
__global__ void static_z_kernel(Problem P, const double* T_in, double* T_out, StaticView s) {
  const hs2g::Dims& d = P.d;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nxy = d.nxy();
  if (t >= nxy) return;
  double u_prev = 0.0, z = 0.0;
  for (int64_t k = 0; k < d.nz; ++k) {
    const int64_t p = k * nxy + t;
    double dd = 1.0, lo = 0.0, hi = 0.0, r = 0.0;
    if (computed(P, p)) {
      const double gzl = k > 0 ? P.Gz[p] : 0.0, gzh = k + 1 < d.nz ? P.Gz[p + nxy] : 0.0;
      r = P.M[p] * s.w1[p];
      dd = P.M[p] + 0.5 * (gzl + gzh);
      lo = -(0.5 * gzl);
      hi = -(0.5 * gzh);
    }
    const double piv = dd - u_prev * lo;
    z = (r - lo * z) / piv;
    u_prev = hi / piv;
    s.w0[p] = z;
    s.u[p] = u_prev;
  }
  double x = 0.0;
  for (int64_t k = d.nz - 1; k >= 0; --k) {
    const int64_t p = k * nxy + t;
    x = s.w0[p] - s.u[p] * x;
    T_out[p] = T_in[p] + x;
  }
}

std::mutex g_static_mutex;

// The scratch array's and the status word's device addresses, per device, with the context they were taken in.
struct StaticAddress {
  CUcontext ctx = nullptr;
  double* scratch = nullptr;
  unsigned long long* status = nullptr;
};
StaticAddress g_static_addr[kMaxDevices];

PFN_cuCtxGetCurrent_v4000 ctx_get_current_fn() {
  static PFN_cuCtxGetCurrent_v4000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuCtxGetCurrent_v4000>(p);
  });
  return fn;
}

// Set-up: device addresses of the scratch array and the status word on the current device, taken with
// cudaGetSymbolAddress the first time and whenever the device's current context is no longer the one they were
// taken in.
cudaError_t static_addresses(StaticAddress* out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  PFN_cuCtxGetCurrent_v4000 get_ctx = ctx_get_current_fn();
  CUcontext ctx = nullptr;
  if (!get_ctx || get_ctx(&ctx) != CUDA_SUCCESS) return cudaErrorInitializationError;
  std::lock_guard<std::mutex> lock(g_static_mutex);
  StaticAddress& a = g_static_addr[dev];
  if (!ctx || !a.scratch || a.ctx != ctx) {
    // (with no context current yet, the first runtime call below creates the device's primary context)
    void* scratch = nullptr;
    void* status = nullptr;
    e = cudaGetSymbolAddress(&scratch, g_static_scratch);
    if (e != cudaSuccess) return e;
    e = cudaGetSymbolAddress(&status, g_static_status);
    if (e != cudaSuccess) return e;
    if (!ctx && (get_ctx(&ctx) != CUDA_SUCCESS || !ctx)) return cudaErrorInitializationError;
    a.ctx = ctx;
    a.scratch = static_cast<double*>(scratch);
    a.status = static_cast<unsigned long long*>(status);
  }
  *out = a;
  return cudaSuccess;
}

}  // namespace

extern "C" int hs2g_step_static(int64_t nz, int64_t ny, int64_t nx, const double* Gz, const double* Gy,
                                const double* Gx, const double* capacity, const uint8_t* fixed, const double* Q,
                                const double* T_in, double* T_out, void* stream) {
  if (nz < 1 || ny < 1 || nx < 1 || !Gz || !Gy || !Gx || !capacity || !T_in || !T_out)
    return hs2g::set_last_error(HS2G_ERR_ARG, "hs2g_step_static: null array or non-positive grid dimension");
  if (nz > kStaticVoxels || ny > kStaticVoxels || nx > kStaticVoxels || nz * ny > kStaticVoxels ||
      nz * ny * nx > kStaticVoxels)
    return hs2g::set_last_error(HS2G_ERR_ARG,
                                "hs2g_step_static: grid larger than HS2G_STATIC_MAX_VOXELS (1048576) voxels; "
                                "use hs2g_create_dense + hs2g_step");
  char msg[256];
  StaticAddress a;
  cudaError_t e = static_addresses(&a);
  if (e != cudaSuccess) {
    snprintf(msg, sizeof(msg), "hs2g_step_static: cannot take the scratch array's device address: %s",
             cudaGetErrorString(e));
    return hs2g::set_last_error(HS2G_ERR_CUDA, msg);
  }
  StaticView s{a.scratch, a.scratch + kStaticVoxels, a.scratch + 2 * kStaticVoxels};
  Problem P{hs2g::Dims{nz, ny, nx}, Gz, Gy, Gx, capacity, fixed, Q};
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int th = 128;
  // a launch error below must be this call's: drop a non-sticky error the caller left pending (a sticky error
  // of an earlier failure in the context is reported by the launches themselves)
  cudaGetLastError();
  e = cudaMemsetAsync(a.status, 0, sizeof(unsigned long long), st);
  if (e == cudaSuccess) {
    static_x_kernel<<<(unsigned)((nz * ny + th - 1) / th), th, 0, st>>>(P, T_in, s);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    static_y_kernel<<<(unsigned)((nz * nx + th - 1) / th), th, 0, st>>>(P, s);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    static_z_kernel<<<(unsigned)((ny * nx + th - 1) / th), th, 0, st>>>(P, T_in, T_out, s);
    e = cudaGetLastError();
  }
  unsigned long long status = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&status, a.status, sizeof(status), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    snprintf(msg, sizeof(msg), "hs2g_step_static: %s (%s)", cudaGetErrorName(e), cudaGetErrorString(e));
    return hs2g::set_last_error(HS2G_ERR_CUDA, msg);
  }
  if (status) {
    const int64_t p = (int64_t)(status & ((1ull << 54) - 1));
    snprintf(msg, sizeof(msg),
             "hs2g_step_static: computed voxel [%lld,%lld,%lld] has rho*c/dt <= 0 or not finite; the output is "
             "not a valid step",
             (long long)(p / (ny * nx)), (long long)((p / nx) % ny), (long long)(p % nx));
    return hs2g::set_last_error(HS2G_ERR_CAPACITY, msg);
  }
  return HS2G_OK;
}
