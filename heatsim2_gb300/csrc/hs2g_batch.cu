// Batched timestep: many independent problems of uneven size advanced together.
//
// All instances live in one concatenated device state (instance b's fields start at voxel offset off[b], each
// (nz_b, ny_b, nx_b) C-ordered).  The three sweeps are persistent kernels that walk flattened work lists --
// x: (instance, 32 x-lines), y: (instance, 128 y-lines), z: (instance, 128 z-lines) -- ordered longest lines
// first so the static round-robin over the persistent grid balances uneven instances.  One timestep (three
// sweeps + a step-counter increment) is captured once in a CUDA graph and replayed; the per-step source
// tables are uploaded once and selected on the device by the step counter, so the graph never changes.
//
// The arithmetic per line is that of the single-problem kernels (hs2g_sweep.cu, scaled delta-form Douglas
// ADI), templated on the storage type: double (results equal to the single-problem path bit for bit) or float
// (coefficients compiled in double, rounded once; its error against double is measured by the caller).
// Block sizes and persistent grid sizes per axis are chosen by hs2g_batch_autotune (timed on the batch).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hs2g_internal.cuh"

namespace hs2g {
namespace {

struct Inst {
  Dims d;
  int64_t off;      // voxel offset in the concatenated fields
  int64_t xb_off;   // element offset of the instance's stencil blocks
  int64_t nchunks;  // 32-column chunks per x-line
};

struct XWork {
  int32_t inst;
  int32_t pad;
  int64_t L0;  // first x-line of the block
};
struct LWork {
  int32_t inst;
  int32_t pad;
  int64_t g0;  // first line of the block (y: k*nx + i, z: j*nx + i)
};

template <typename R>
struct BatchView {
  const Inst* inst;
  R* T;
  R* W0;
  R* W1;
  const R* xb;
  const R* a0;
  const R* b0;
  const R* a1;
  const R* b1;
  const R* a2;
  const R* b2;
  const uint8_t* vclass;
  const R* qtabs;          // [nsched][ninst][nclass]
  const uint8_t* active;   // [nsched][ninst] any source active
  const int* step;         // device step counter
  int nsched, ninst, nclass;
  const XWork* xw;
  int64_t nx_work;
  const LWork* yw;
  int64_t ny_work;
  const LWork* zw;
  int64_t nz_work;
};

constexpr int kMaxBatchClasses = HS2G_MAX_CLASSES;

// IX: index type of the voxel, line and stencil-block arithmetic within an instance (int32_t when every
// instance and its stencil blocks have fewer than 2^31 elements)
template <typename R, bool HAS_Q, typename IX = int64_t>
__device__ __forceinline__ R batch_stencil(const Inst& I, const R* __restrict__ T, const R* __restrict__ xb,
                                           const uint8_t* __restrict__ vclass, const R* sq, IX L, int ch,
                                           int lane) {
  const Dims& d = I.d;
  const IX nx = (IX)d.nx, ny = (IX)d.ny, nz = (IX)d.nz;
  const IX i = (IX)ch * 32 + lane;
  const IX k = L / ny, j = L - k * ny;
  const IX p = L * nx + i;
  const IX nxy = nx * ny;
  const R* __restrict__ w = xb + I.xb_off + ((L * (IX)I.nchunks + ch) * kXBlockCoeffs) * 32 + lane;
  const R* Ti = T + I.off;
  const R t = Ti[p];
  const R txl = i > 0 ? Ti[p - 1] : t;
  const R txh = i + 1 < nx ? Ti[p + 1] : t;
  const R tyl = j > 0 ? Ti[p - nx] : t;
  const R tyh = j + 1 < ny ? Ti[p + nx] : t;
  const R tzl = k > 0 ? Ti[p - nxy] : t;
  const R tzh = k + 1 < nz ? Ti[p + nxy] : t;
  R r = w[kWc * 32] * t;
  r = fma(w[kWxl * 32], txl, r);
  r = fma(w[kWxh * 32], txh, r);
  r = fma(w[kWyl * 32], tyl, r);
  r = fma(w[kWyh * 32], tyh, r);
  r = fma(w[kWzl * 32], tzl, r);
  r = fma(w[kWzh * 32], tzh, r);
  if (HAS_Q) r = fma(w[kWq * 32], sq[vclass[I.off + p]], r);
  return r;
}

// One block of 32 x-lines of one instance (CTA of 128 threads), same structure as sweep_x_kernel.
template <typename R, bool HAS_Q, typename IX = int64_t>
__device__ void batch_x_block(const BatchView<R>& v, const Inst& I, int64_t L0_, const R* sq, R (*sr)[33],
                              R (*sa)[33]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const Dims& d = I.d;
  const IX nx = (IX)d.nx, L0 = (IX)L0_;
  const IX nlines = (IX)(d.nz * d.ny);
  const int nchunks = (int)I.nchunks;
  R* W0 = v.W0 + I.off;
  const R* a0 = v.a0 + I.off;
  const R* b0 = v.b0 + I.off;
  R carry = 0;
  for (int ch = 0; ch < nchunks; ++ch) {
    const IX i = (IX)ch * 32 + lane;
#pragma unroll
    for (int ll = 0; ll < 8; ++ll) {
      const int l = warp * 8 + ll;
      const IX L = L0 + l;
      R r = 0, a = 0;
      if (L < nlines && i < nx) {
        r = batch_stencil<R, HAS_Q, IX>(I, v.T, v.xb, v.vclass, sq, L, ch, lane);
        a = a0[L * nx + i];
      }
      sr[l][lane] = r;
      sa[l][lane] = a;
    }
    __syncthreads();
    if (warp == 0) {
      const int cw = (int)min((int64_t)32, d.nx - (int64_t)ch * 32);
      R z = carry;
      if (cw == 32) {  // full chunks unrolled: the shared loads of later rows issue ahead of the chain
#pragma unroll 4
        for (int cc = 0; cc < 32; ++cc) {
          z = fma(-sa[lane][cc], z, sr[lane][cc]);
          sr[lane][cc] = z;
        }
      } else {
        for (int cc = 0; cc < cw; ++cc) {
          z = fma(-sa[lane][cc], z, sr[lane][cc]);
          sr[lane][cc] = z;
        }
      }
      carry = z;
    }
    __syncthreads();
#pragma unroll
    for (int ll = 0; ll < 8; ++ll) {
      const int l = warp * 8 + ll;
      const IX L = L0 + l;
      if (L < nlines && i < nx) W0[L * nx + i] = sr[l][lane];
    }
    __syncthreads();
  }
  carry = 0;
  for (int ch = nchunks - 1; ch >= 0; --ch) {
    const IX i = (IX)ch * 32 + lane;
#pragma unroll
    for (int ll = 0; ll < 8; ++ll) {
      const int l = warp * 8 + ll;
      const IX L = L0 + l;
      R z = 0, b = 0;
      if (L < nlines && i < nx) {
        z = W0[L * nx + i];
        b = b0[L * nx + i];
      }
      sr[l][lane] = z;
      sa[l][lane] = b;
    }
    __syncthreads();
    if (warp == 0) {
      const int cw = (int)min((int64_t)32, d.nx - (int64_t)ch * 32);
      R x = carry;
      if (cw == 32) {
#pragma unroll 4
        for (int cc = 31; cc >= 0; --cc) {
          x = fma(-sa[lane][cc], x, sr[lane][cc]);
          sr[lane][cc] = x;
        }
      } else {
        for (int cc = cw - 1; cc >= 0; --cc) {
          x = fma(-sa[lane][cc], x, sr[lane][cc]);
          sr[lane][cc] = x;
        }
      }
      carry = x;
    }
    __syncthreads();
#pragma unroll
    for (int ll = 0; ll < 8; ++ll) {
      const int l = warp * 8 + ll;
      const IX L = L0 + l;
      if (L < nlines && i < nx) W0[L * nx + i] = sr[l][lane];
    }
    __syncthreads();
  }
}

// 72 registers (7 CTAs of 128 threads per SM): more loads in flight per thread than at 64 registers, which
// left the kernel load-latency bound (2.25e10 against 2.47e10 voxel-steps/s on the 256-instance batch).
// IX = int32_t (every batch whose instances have fewer than 2^31 voxels and stencil-block elements): 32-bit
// line, voxel and block arithmetic within an instance, 9.55 against 10.65 ms per FP64 step of that batch (the
// same for the y and z sweeps changed nothing there).
template <typename R, typename IX = int64_t>
__global__ void __launch_bounds__(128, 7) batch_x_kernel(BatchView<R> v) {
  __shared__ R sr[32][33];
  __shared__ R sa[32][33];
  __shared__ R sq[kMaxBatchClasses];
  const int step = *v.step;
  const bool sched = step < v.nsched;
  for (int64_t w = blockIdx.x; w < v.nx_work; w += gridDim.x) {
    const XWork item = v.xw[w];
    const Inst I = v.inst[item.inst];
    const bool has_q = sched && v.active[(int64_t)step * v.ninst + item.inst];
    if (has_q) {
      const R* q = v.qtabs + ((int64_t)step * v.ninst + item.inst) * v.nclass;
      for (int c = threadIdx.x; c < kMaxBatchClasses; c += blockDim.x) sq[c] = c < v.nclass ? q[c] : R(0);
      __syncthreads();
      batch_x_block<R, true, IX>(v, I, item.L0, sq, sr, sa);
    } else {
      batch_x_block<R, false, IX>(v, I, item.L0, sq, sr, sa);
    }
  }
}

// y lines (thread per line): W1 = s2*dT1 from W0 = sigma*dT0
template <typename R>
__global__ void batch_y_kernel(BatchView<R> v) {
  for (int64_t w = blockIdx.x; w < v.ny_work; w += gridDim.x) {
    const LWork item = v.yw[w];
    const Inst I = v.inst[item.inst];
    const Dims& d = I.d;
    const int64_t g = item.g0 + threadIdx.x;
    if (g >= d.nz * d.nx) continue;
    const int64_t k = g / d.nx, i = g - k * d.nx;
    const R* W0 = v.W0 + I.off;
    const R* a1 = v.a1 + I.off;
    const R* b1 = v.b1 + I.off;
    R* W1 = v.W1 + I.off;
    int64_t p = k * d.nxy() + i;
    R z = 0;
#pragma unroll 4
    for (int64_t j = 0; j < d.ny; ++j, p += d.nx) {
      z = fma(-a1[p], z, W0[p]);
      W1[p] = z;
    }
    R x = 0;
#pragma unroll 4
    for (int64_t j = d.ny - 1; j >= 0; --j) {
      p -= d.nx;
      x = fma(-b1[p], x, W1[p]);
      W1[p] = x;
    }
  }
}

// z lines (thread per line): T += dT2 from W1 = s2*dT1, W0 as scratch
template <typename R>
__global__ void batch_z_kernel(BatchView<R> v) {
  for (int64_t w = blockIdx.x; w < v.nz_work; w += gridDim.x) {
    const LWork item = v.zw[w];
    const Inst I = v.inst[item.inst];
    const Dims& d = I.d;
    const int64_t nxy = d.nxy();
    const int64_t g = item.g0 + threadIdx.x;
    if (g >= nxy) continue;
    const R* W1 = v.W1 + I.off;
    const R* a2 = v.a2 + I.off;
    const R* b2 = v.b2 + I.off;
    R* Z = v.W0 + I.off;
    R* T = v.T + I.off;
    int64_t p = g;
    R z = 0;
#pragma unroll 4
    for (int64_t k = 0; k < d.nz; ++k, p += nxy) {
      z = fma(-a2[p], z, W1[p]);
      Z[p] = z;
    }
    R x = 0;
#pragma unroll 4
    for (int64_t k = d.nz - 1; k >= 0; --k) {
      p -= nxy;
      x = fma(-b2[p], x, Z[p]);
      T[p] = T[p] + x;
    }
  }
}

__global__ void batch_advance_kernel(int* step) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *step += 1;
}

template <typename R>
__global__ void convert_kernel(const double* __restrict__ src, R* __restrict__ dst, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    dst[e] = (R)src[e];
}
template <typename R>
__global__ void widen_kernel(const R* __restrict__ src, double* __restrict__ dst, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    dst[e] = (double)src[e];
}

struct Tuning {
  int x_grid;
  int y_block, y_grid;
  int z_block, z_grid;
};

}  // namespace

// ---------------------------------------------------------------------------------------------------------
// Batch object
// ---------------------------------------------------------------------------------------------------------
struct Batch {
  int device = 0;
  int precision = 64;
  int ninst = 0;
  cudaStream_t stream = nullptr;
  std::vector<Inst> inst;
  std::vector<int64_t> offsets;  // [ninst+1] voxel offsets
  int64_t nvox = 0, xb_len = 0;
  Inst* inst_dev = nullptr;
  void* T = nullptr;  // R*
  void* W0 = nullptr;
  void* W1 = nullptr;
  void* coef = nullptr;  // 6 arrays of nvox R
  void* xb = nullptr;
  uint8_t* vclass = nullptr;
  void* qtabs = nullptr;
  uint8_t* active = nullptr;
  int nsched = 0, nclass = 1;
  int* step = nullptr;
  XWork* xw = nullptr;
  LWork* yw = nullptr;
  LWork* zw = nullptr;
  int64_t nxw = 0, nyw = 0, nzw = 0;
  Tuning tune{0, 128, 0, 128, 0};
  bool ix32 = false;  // every instance's voxels and stencil blocks below 2^31 elements: 32-bit x-sweep indices
  cudaGraphExec_t graph = nullptr;
  int64_t bytes = 0;
  size_t elem() const { return precision == 64 ? 8 : 4; }
};

namespace {

template <typename R>
BatchView<R> view(const Batch& b) {
  BatchView<R> v{};
  v.inst = b.inst_dev;
  v.T = (R*)b.T;
  v.W0 = (R*)b.W0;
  v.W1 = (R*)b.W1;
  R* c = (R*)b.coef;
  v.a0 = c;
  v.b0 = c + b.nvox;
  v.a1 = c + 2 * b.nvox;
  v.b1 = c + 3 * b.nvox;
  v.a2 = c + 4 * b.nvox;
  v.b2 = c + 5 * b.nvox;
  v.xb = (const R*)b.xb;
  v.vclass = b.vclass;
  v.qtabs = (const R*)b.qtabs;
  v.active = b.active;
  v.step = b.step;
  v.nsched = b.nsched;
  v.ninst = b.ninst;
  v.nclass = b.nclass;
  v.xw = b.xw;
  v.nx_work = b.nxw;
  v.yw = b.yw;
  v.ny_work = b.nyw;
  v.zw = b.zw;
  v.nz_work = b.nzw;
  return v;
}

template <typename R>
cudaError_t launch_axis(const Batch& b, int axis, const Tuning& t, cudaStream_t s) {
  BatchView<R> v = view<R>(b);
  if (axis == 0) {
    if (b.ix32)
      batch_x_kernel<R, int32_t><<<(unsigned)std::max(1, t.x_grid), 128, 0, s>>>(v);
    else
      batch_x_kernel<R><<<(unsigned)std::max(1, t.x_grid), 128, 0, s>>>(v);
  } else if (axis == 1) {
    batch_y_kernel<R><<<(unsigned)std::max(1, t.y_grid), t.y_block, 0, s>>>(v);
  } else if (axis == 2) {
    batch_z_kernel<R><<<(unsigned)std::max(1, t.z_grid), t.z_block, 0, s>>>(v);
  } else {
    batch_advance_kernel<<<1, 32, 0, s>>>(b.step);
  }
  return cudaGetLastError();
}

cudaError_t launch_axis_any(const Batch& b, int axis, const Tuning& t, cudaStream_t s) {
  return b.precision == 64 ? launch_axis<double>(b, axis, t, s) : launch_axis<float>(b, axis, t, s);
}

cudaError_t launch_step_batch(const Batch& b, cudaStream_t s) {
  cudaError_t e = cudaSuccess;
  for (int axis = 0; axis < 4 && e == cudaSuccess; ++axis) e = launch_axis_any(b, axis, b.tune, s);
  return e;
}

}  // namespace

// Work lists: blocks of 32 x-lines / block_y y-lines / block_z z-lines per instance, longest lines first.
void batch_build_work(Batch& b, int block_y, int block_z, std::vector<XWork>& xw, std::vector<LWork>& yw,
                      std::vector<LWork>& zw) {
  xw.clear();
  yw.clear();
  zw.clear();
  std::vector<int> order(b.ninst);
  for (int i = 0; i < b.ninst; ++i) order[i] = i;
  auto by = [&](auto len) {
    std::vector<int> o = order;
    std::stable_sort(o.begin(), o.end(), [&](int p, int q) { return len(b.inst[p].d) > len(b.inst[q].d); });
    return o;
  };
  for (int ib : by([](const Dims& d) { return d.nx; })) {
    const Dims& d = b.inst[ib].d;
    for (int64_t L0 = 0; L0 < d.nz * d.ny; L0 += 32) xw.push_back(XWork{ib, 0, L0});
  }
  for (int ib : by([](const Dims& d) { return d.ny; })) {
    const Dims& d = b.inst[ib].d;
    for (int64_t g0 = 0; g0 < d.nz * d.nx; g0 += block_y) yw.push_back(LWork{ib, 0, g0});
  }
  for (int ib : by([](const Dims& d) { return d.nz; })) {
    const Dims& d = b.inst[ib].d;
    for (int64_t g0 = 0; g0 < d.nxy(); g0 += block_z) zw.push_back(LWork{ib, 0, g0});
  }
}

cudaError_t batch_upload_work(Batch& b, int block_y, int block_z) {
  std::vector<XWork> xw;
  std::vector<LWork> yw, zw;
  batch_build_work(b, block_y, block_z, xw, yw, zw);
  if (b.xw) cudaFree(b.xw);
  if (b.yw) cudaFree(b.yw);
  if (b.zw) cudaFree(b.zw);
  b.xw = nullptr;
  b.yw = b.zw = nullptr;
  cudaError_t e = cudaMalloc(&b.xw, sizeof(XWork) * std::max<size_t>(1, xw.size()));
  if (e == cudaSuccess) e = cudaMalloc(&b.yw, sizeof(LWork) * std::max<size_t>(1, yw.size()));
  if (e == cudaSuccess) e = cudaMalloc(&b.zw, sizeof(LWork) * std::max<size_t>(1, zw.size()));
  if (e == cudaSuccess) e = cudaMemcpy(b.xw, xw.data(), sizeof(XWork) * xw.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b.yw, yw.data(), sizeof(LWork) * yw.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b.zw, zw.data(), sizeof(LWork) * zw.size(), cudaMemcpyHostToDevice);
  b.nxw = (int64_t)xw.size();
  b.nyw = (int64_t)yw.size();
  b.nzw = (int64_t)zw.size();
  return e;
}

cudaError_t batch_convert(const double* src, void* dst, int64_t n, int precision, cudaStream_t s) {
  if (precision == 64) return cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
  convert_kernel<float><<<1024, 256, 0, s>>>(src, (float*)dst, n);
  return cudaGetLastError();
}

cudaError_t batch_widen(const void* src, double* dst, int64_t n, int precision, cudaStream_t s) {
  if (precision == 64) return cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
  widen_kernel<float><<<1024, 256, 0, s>>>((const float*)src, dst, n);
  return cudaGetLastError();
}

cudaError_t batch_step(Batch& b, cudaStream_t s) { return launch_step_batch(b, s); }

cudaError_t batch_time_axis(Batch& b, int axis, const Tuning& t, int reps, float* ms) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaError_t e = launch_axis_any(b, axis, t, b.stream);  // warm-up
  cudaEventRecord(e0, b.stream);
  for (int r = 0; r < reps && e == cudaSuccess; ++r) e = launch_axis_any(b, axis, t, b.stream);
  cudaEventRecord(e1, b.stream);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  float v = 0.f;
  cudaEventElapsedTime(&v, e0, e1);
  *ms = v / reps;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return e;
}

// Candidate launch shapes per axis, timed on the batch itself.  Returns the report in `report`.
cudaError_t batch_autotune(Batch& b, std::string& report) {
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b.device);
  Tuning best = b.tune;
  char line[256];
  cudaError_t e = cudaSuccess;
  // x: persistent grid size (CTAs of 128 threads)
  {
    float bt = 1e30f;
    // per = 0: one CTA per work item, the hardware's block scheduler doing the balancing
    for (int per : {4, 5, 6, 7, 8, 10, 0}) {
      Tuning t = best;
      t.x_grid = (int)std::min<int64_t>(std::min<int64_t>(b.nxw, 1 << 30), per ? (int64_t)sms * per : b.nxw);
      float ms;
      if ((e = batch_time_axis(b, 0, t, 2, &ms)) != cudaSuccess) return e;
      snprintf(line, sizeof line, "x grid %d: %.3f ms\n", t.x_grid, ms);
      report += line;
      if (ms < bt) bt = ms, best.x_grid = t.x_grid;
    }
  }
  // y and z: block size (work list granularity) and persistent grid
  for (int axis = 1; axis <= 2; ++axis) {
    float bt = 1e30f;
    int bb = 128, bg = 0;
    for (int blk : {64, 128, 256}) {
      if ((e = batch_upload_work(b, axis == 1 ? blk : best.y_block, axis == 2 ? blk : best.z_block)) != cudaSuccess)
        return e;
      for (int per : {8, 16, 32}) {
        Tuning t = best;
        const int64_t nwork = axis == 1 ? b.nyw : b.nzw;
        const int grid = (int)std::min<int64_t>(nwork, (int64_t)sms * per * 256 / blk);
        if (axis == 1) t.y_block = blk, t.y_grid = grid;
        else t.z_block = blk, t.z_grid = grid;
        float ms;
        if ((e = batch_time_axis(b, axis, t, 2, &ms)) != cudaSuccess) return e;
        snprintf(line, sizeof line, "%s block %d grid %d: %.3f ms\n", axis == 1 ? "y" : "z", blk, grid, ms);
        report += line;
        if (ms < bt) bt = ms, bb = blk, bg = grid;
      }
    }
    if (axis == 1) best.y_block = bb, best.y_grid = bg;
    else best.z_block = bb, best.z_grid = bg;
    if ((e = batch_upload_work(b, best.y_block, best.z_block)) != cudaSuccess) return e;
  }
  b.tune = best;
  snprintf(line, sizeof line, "chosen: x grid %d, y block %d grid %d, z block %d grid %d\n", best.x_grid,
           best.y_block, best.y_grid, best.z_block, best.z_grid);
  report += line;
  return e;
}

}  // namespace hs2g

// ---------------------------------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------------------------------
struct hs2g_batch {
  hs2g::Batch b;
};

namespace {

using hs2g::Batch;

struct BatchDeviceGuard {
  int prev = -1;
  bool ok = false;
  explicit BatchDeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    ok = (prev == dev) || (cudaSetDevice(dev) == cudaSuccess);
  }
  ~BatchDeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

int bfail(int code, const char* msg) { return hs2g::set_last_error(code, msg); }
int bcuda(cudaError_t e, const char* what) {
  cudaGetLastError();  // a failed allocation leaves its error as the last error: clear it for later checks
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  return hs2g::set_last_error(e == cudaErrorMemoryAllocation ? HS2G_ERR_NOMEM : HS2G_ERR_CUDA, buf);
}

template <typename T>
cudaError_t balloc(Batch& b, T** p, int64_t count) {
  const size_t bytes = sizeof(T) * (size_t)std::max<int64_t>(1, count);
  cudaError_t e = cudaMalloc((void**)p, bytes);
  if (e == cudaSuccess) b.bytes += (int64_t)bytes;
  else *p = nullptr;
  return e;
}

void batch_free(Batch& b) {
  if (b.graph) cudaGraphExecDestroy(b.graph);
  b.graph = nullptr;
  for (void* p : {(void*)b.inst_dev, b.T, b.W0, b.W1, b.coef, b.xb, (void*)b.vclass, b.qtabs, (void*)b.active,
                  (void*)b.step, (void*)b.xw, (void*)b.yw, (void*)b.zw})
    if (p) cudaFree(p);
  if (b.stream) cudaStreamDestroy(b.stream);
}

int64_t xb_elems(const hs2g::Dims& d) { return d.nz * d.ny * ((d.nx + 31) / 32) * hs2g::kXBlockCoeffs * 32; }

// Compile instance `ib` of problem p into the batch (FP64 workspace ws, then into the batch's storage type).
int compile_instance(Batch& b, int ib, const hs2g_class_problem& p, double* ws, unsigned long long* err) {
  const hs2g::Inst& I = b.inst[ib];
  const hs2g::Dims& d = I.d;
  const int64_t n = d.nvox();
  const int64_t nfz = (d.nz + 1) * d.nxy(), nfy = d.nz * (d.ny + 1) * d.nx, nfx = d.nz * d.ny * (d.nx + 1);
  cudaStream_t s = b.stream;
  // workspace layout (doubles): faces z, y, x | M s2 sigma | 6 coefficient arrays | x blocks | bytes:
  // compute mask, material, boundary classes | material table | boundary forms
  double* fz = ws;
  double* fy = fz + nfz;
  double* fx = fy + nfy;
  double* M = fx + nfx;
  double* s2 = M + n;
  double* sg = s2 + n;
  double* c6 = sg + n;
  double* xbw = c6 + 6 * n;
  uint8_t* u8 = reinterpret_cast<uint8_t*>(xbw + xb_elems(d));
  uint8_t* comp = u8;
  uint8_t* mat = comp + n;
  uint8_t* bz = mat + n;
  uint8_t* by = bz + nfz;
  uint8_t* bx = by + nfy;
  hs2g_material* mats = reinterpret_cast<hs2g_material*>((reinterpret_cast<uintptr_t>(bx + nfx) + 255) & ~uintptr_t(255));
  hs2g_face_form* forms = reinterpret_cast<hs2g_face_form*>(
      (reinterpret_cast<uintptr_t>(mats + HS2G_MAX_CLASSES) + 255) & ~uintptr_t(255));
  cudaError_t e = cudaSuccess;
  auto up = [&](void* dst, const void* src, size_t bytes) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s);
  };
  up(mat, p.material, (size_t)n);
  up(bz, p.boundary_z, (size_t)nfz);
  up(by, p.boundary_y, (size_t)nfy);
  up(bx, p.boundary_x, (size_t)nfx);
  up(mats, p.materials, sizeof(hs2g_material) * p.nmat);
  up(forms, p.forms, sizeof(hs2g_face_form) * p.nbnd * 3);
  if (p.volumetric) up(b.vclass + I.off, p.volumetric, (size_t)n);
  else if (e == cudaSuccess) e = cudaMemsetAsync(b.vclass + I.off, 0, (size_t)n, s);
  if (e == cudaSuccess) e = hs2g::launch_faces(d, 0, mat, bz, mats, p.nmat, forms, p.nbnd, fz, err, s);
  if (e == cudaSuccess) e = hs2g::launch_faces(d, 1, mat, by, mats, p.nmat, forms, p.nbnd, fy, err, s);
  if (e == cudaSuccess) e = hs2g::launch_faces(d, 2, mat, bx, mats, p.nmat, forms, p.nbnd, fx, err, s);
  if (e == cudaSuccess) e = hs2g::launch_capacity_from_classes(d, mat, mats, p.nmat, M, comp, err, s);
  if (e != cudaSuccess) return bcuda(e, "batch compile");
  unsigned long long v = 0;
  if ((e = cudaMemcpyAsync(&v, err, sizeof v, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return bcuda(e, "batch compile");
  if (v) {
    char buf[160];
    const int code = -(int)(v >> 56);
    snprintf(buf, sizeof buf, "instance %d: invalid problem (error %d at axis %d index %llu)", ib, code,
             (int)((v >> 54) & 3), (unsigned long long)(v & ((1ull << 54) - 1)));
    return bfail(code, buf);
  }
  hs2g::Coeffs c{};
  c.nchunks = I.nchunks;
  c.px = d.nx;  // the batched sweeps use plain loads on unpadded rows
  const bool f64 = b.precision == 64;
  double* cbase = f64 ? (double*)b.coef : c6;
  const int64_t cstride = f64 ? b.nvox : n;
  const int64_t coff = f64 ? I.off : 0;
  c.a0 = cbase + coff;
  c.b0 = cbase + cstride + coff;
  c.a1 = cbase + 2 * cstride + coff;
  c.b1 = cbase + 3 * cstride + coff;
  c.a2 = cbase + 4 * cstride + coff;
  c.b2 = cbase + 5 * cstride + coff;
  c.xb = f64 ? (double*)b.xb + I.xb_off : xbw;
  if (!f64 && (e = cudaMemsetAsync(xbw, 0, sizeof(double) * xb_elems(d), s)) != cudaSuccess)
    return bcuda(e, "batch compile");
  if ((e = hs2g::launch_factor(d, fz, fy, fx, M, comp, s2, sg, c, s)) != cudaSuccess)
    return bcuda(e, "batch factor");
  if (!f64) {
    for (int a = 0; a < 6 && e == cudaSuccess; ++a)
      e = hs2g::batch_convert(c6 + a * n, (float*)b.coef + a * b.nvox + I.off, n, 32, s);
    if (e == cudaSuccess) e = hs2g::batch_convert(xbw, (float*)b.xb + I.xb_off, xb_elems(d), 32, s);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? HS2G_OK : bcuda(e, "batch factor");
}

int capture(Batch& b) {
  if (b.graph) {
    cudaGraphExecDestroy(b.graph);
    b.graph = nullptr;
  }
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(b.stream, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return bcuda(e, "graph capture");
  cudaError_t le = hs2g::batch_step(b, b.stream);
  e = cudaStreamEndCapture(b.stream, &g);
  if (le != cudaSuccess) return bcuda(le, "graph capture: launch");
  if (e != cudaSuccess) return bcuda(e, "graph capture");
  e = cudaGraphInstantiate(&b.graph, g, 0);
  cudaGraphDestroy(g);
  return e == cudaSuccess ? HS2G_OK : bcuda(e, "graph instantiate");
}

}  // namespace

extern "C" {

int hs2g_batch_create(int n, const hs2g_class_problem* problems, int precision, int device, hs2g_batch** out) {
  if (!out || !problems || n < 1 || n > (1 << 20) || (precision != 64 && precision != 32))
    return bfail(HS2G_ERR_ARG, "hs2g_batch_create: bad argument");
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    const hs2g_class_problem& p = problems[i];
    if (p.nz < 1 || p.ny < 1 || p.nx < 1 || !p.materials || !p.forms || !p.material || !p.boundary_z ||
        !p.boundary_y || !p.boundary_x || p.nmat < 1 || p.nmat > HS2G_MAX_CLASSES || p.nbnd < 1 ||
        p.nbnd > HS2G_MAX_CLASSES)
      return bfail(HS2G_ERR_ARG, "hs2g_batch_create: bad problem");
  }
  BatchDeviceGuard g(device);
  if (!g.ok) return bfail(HS2G_ERR_CUDA, "hs2g_batch_create: cannot select device");
  hs2g_batch* hb = new hs2g_batch();
  Batch& b = hb->b;
  b.device = device;
  b.precision = precision;
  b.ninst = n;
  auto bail = [&](int rc) {
    std::string msg = hs2g_last_error();
    batch_free(b);
    delete hb;
    hs2g::set_last_error(rc, msg.c_str());
    return rc;
  };
  cudaError_t e = cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete hb;
    return bcuda(e, "cudaStreamCreate");
  }
  int64_t off = 0, xoff = 0, ws = 0;
  b.offsets.push_back(0);
  for (int i = 0; i < n; ++i) {
    hs2g::Inst I{};
    I.d = hs2g::Dims{problems[i].nz, problems[i].ny, problems[i].nx};
    I.off = off;
    I.xb_off = xoff;
    I.nchunks = (I.d.nx + 31) / 32;
    b.inst.push_back(I);
    const hs2g::Dims& d = I.d;
    const int64_t nn = d.nvox();
    off += nn + (nn & 1);  // keep every instance 16-byte aligned
    xoff += xb_elems(d);
    b.offsets.push_back(off);
    const int64_t faces = (d.nz + 1) * d.nxy() + d.nz * (d.ny + 1) * d.nx + d.nz * d.ny * (d.nx + 1);
    const int64_t need = faces + 9 * nn + xb_elems(d) + (faces + 3 * nn) / 8 + 2048 +
                         (int64_t)(sizeof(hs2g_material) * HS2G_MAX_CLASSES + sizeof(hs2g_face_form) * 3 *
                                   HS2G_MAX_CLASSES) / 8 + 256;
    ws = std::max(ws, need);
  }
  b.nvox = off;
  b.xb_len = xoff;
  b.ix32 = true;
  for (const hs2g::Inst& I : b.inst)
    b.ix32 = b.ix32 && I.d.nvox() < ((int64_t)1 << 31) && xb_elems(I.d) < ((int64_t)1 << 31);
  const size_t el = b.elem();
  double* wsp = nullptr;
  unsigned long long* err = nullptr;
  if ((e = balloc(b, &b.inst_dev, n)) != cudaSuccess || (e = balloc(b, (char**)&b.T, b.nvox * el)) != cudaSuccess ||
      (e = balloc(b, (char**)&b.W0, b.nvox * el)) != cudaSuccess ||
      (e = balloc(b, (char**)&b.W1, b.nvox * el)) != cudaSuccess ||
      (e = balloc(b, (char**)&b.coef, 6 * b.nvox * el)) != cudaSuccess ||
      (e = balloc(b, (char**)&b.xb, b.xb_len * el)) != cudaSuccess ||
      (e = balloc(b, &b.vclass, b.nvox)) != cudaSuccess || (e = balloc(b, &b.step, 1)) != cudaSuccess ||
      (e = cudaMalloc(&wsp, sizeof(double) * ws)) != cudaSuccess ||
      (e = cudaMalloc(&err, sizeof(unsigned long long))) != cudaSuccess) {
    if (wsp) cudaFree(wsp);
    if (err) cudaFree(err);
    hs2g::set_last_error(HS2G_ERR_NOMEM, "hs2g_batch_create: device allocation failed");
    return bail(HS2G_ERR_NOMEM);
  }
  cudaMemsetAsync(b.xb, 0, b.xb_len * el, b.stream);
  cudaMemsetAsync(b.T, 0, b.nvox * el, b.stream);
  cudaMemsetAsync(b.W0, 0, b.nvox * el, b.stream);
  cudaMemsetAsync(b.W1, 0, b.nvox * el, b.stream);
  cudaMemsetAsync(b.coef, 0, 6 * b.nvox * el, b.stream);
  cudaMemsetAsync(b.vclass, 0, b.nvox, b.stream);
  cudaMemsetAsync(b.step, 0, sizeof(int), b.stream);
  cudaMemcpyAsync(b.inst_dev, b.inst.data(), sizeof(hs2g::Inst) * n, cudaMemcpyHostToDevice, b.stream);
  int rc = HS2G_OK;
  for (int i = 0; i < n && rc == HS2G_OK; ++i) {
    cudaMemsetAsync(err, 0, sizeof(unsigned long long), b.stream);
    rc = compile_instance(b, i, problems[i], wsp, err);
  }
  cudaFree(wsp);
  cudaFree(err);
  if (rc != HS2G_OK) return bail(rc);
  if ((e = hs2g::batch_upload_work(b, 128, 128)) != cudaSuccess) return bail(bcuda(e, "work lists"));
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  b.tune.x_grid = (int)std::min<int64_t>(b.nxw, (int64_t)sms * 7);  // the x kernel's 7 resident CTAs per SM
  b.tune.y_grid = (int)std::min<int64_t>(b.nyw, (int64_t)sms * 16);
  b.tune.z_grid = (int)std::min<int64_t>(b.nzw, (int64_t)sms * 16);
  if ((e = cudaStreamSynchronize(b.stream)) != cudaSuccess) return bail(bcuda(e, "batch create"));
  *out = hb;
  return HS2G_OK;
}

void hs2g_batch_destroy(hs2g_batch* hb) {
  if (!hb) return;
  BatchDeviceGuard g(hb->b.device);
  cudaStreamSynchronize(hb->b.stream);
  batch_free(hb->b);
  delete hb;
}

int hs2g_batch_layout(const hs2g_batch* hb, int64_t* offsets, int64_t* dims) {
  if (!hb) return bfail(HS2G_ERR_ARG, "null batch");
  const Batch& b = hb->b;
  for (int i = 0; i <= b.ninst && offsets; ++i) offsets[i] = b.offsets[i];
  for (int i = 0; i < b.ninst && dims; ++i) {
    dims[3 * i] = b.inst[i].d.nz;
    dims[3 * i + 1] = b.inst[i].d.ny;
    dims[3 * i + 2] = b.inst[i].d.nx;
  }
  return HS2G_OK;
}

int64_t hs2g_batch_device_bytes(const hs2g_batch* hb) { return hb ? hb->b.bytes : 0; }

int hs2g_batch_set_temperature(hs2g_batch* hb, const double* T, int flags) {
  if (!hb || !T) return bfail(HS2G_ERR_ARG, "null argument");
  Batch& b = hb->b;
  BatchDeviceGuard g(b.device);
  const bool dev = flags & HS2G_DEVICE;
  cudaError_t e = cudaSuccess;
  if (b.precision == 64) {
    e = cudaMemcpyAsync(b.T, T, sizeof(double) * b.nvox, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                        b.stream);
  } else {
    const double* src = T;
    double* tmp = nullptr;
    if (!dev) {
      if ((e = cudaMallocAsync(&tmp, sizeof(double) * b.nvox, b.stream)) == cudaSuccess)
        e = cudaMemcpyAsync(tmp, T, sizeof(double) * b.nvox, cudaMemcpyHostToDevice, b.stream);
      src = tmp;
    }
    if (e == cudaSuccess) e = hs2g::batch_convert(src, b.T, b.nvox, 32, b.stream);
    if (tmp) cudaFreeAsync(tmp, b.stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(b.stream);
  return e == cudaSuccess ? HS2G_OK : bcuda(e, "set temperature");
}

int hs2g_batch_get_temperature(hs2g_batch* hb, double* T, int flags) {
  if (!hb || !T) return bfail(HS2G_ERR_ARG, "null argument");
  Batch& b = hb->b;
  BatchDeviceGuard g(b.device);
  const bool dev = flags & HS2G_DEVICE;
  cudaError_t e = cudaSuccess;
  if (b.precision == 64) {
    e = cudaMemcpyAsync(T, b.T, sizeof(double) * b.nvox, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                        b.stream);
  } else {
    double* dst = T;
    double* tmp = nullptr;
    if (!dev) {
      e = cudaMallocAsync(&tmp, sizeof(double) * b.nvox, b.stream);
      dst = tmp;
    }
    if (e == cudaSuccess) e = hs2g::batch_widen(b.T, dst, b.nvox, 32, b.stream);
    if (e == cudaSuccess && tmp) e = cudaMemcpyAsync(T, tmp, sizeof(double) * b.nvox, cudaMemcpyDeviceToHost, b.stream);
    if (tmp) cudaFreeAsync(tmp, b.stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(b.stream);
  return e == cudaSuccess ? HS2G_OK : bcuda(e, "get temperature");
}

int hs2g_batch_set_sources(hs2g_batch* hb, int nsteps, int nclass, const double* qtabs) {
  if (!hb || nsteps < 0 || nclass < 1 || nclass > HS2G_MAX_CLASSES || (nsteps > 0 && !qtabs))
    return bfail(HS2G_ERR_ARG, "hs2g_batch_set_sources: bad argument");
  Batch& b = hb->b;
  BatchDeviceGuard g(b.device);
  cudaStreamSynchronize(b.stream);
  if (b.qtabs) cudaFree(b.qtabs);
  if (b.active) cudaFree(b.active);
  b.qtabs = nullptr;
  b.active = nullptr;
  const int64_t nq = (int64_t)nsteps * b.ninst * nclass;
  std::vector<uint8_t> act((size_t)std::max<int64_t>(1, (int64_t)nsteps * b.ninst), 0);
  for (int64_t s = 0; s < (int64_t)nsteps * b.ninst; ++s)
    for (int c = 0; c < nclass; ++c)
      if (qtabs[s * nclass + c] != 0.0) act[(size_t)s] = 1;
  cudaError_t e = cudaMalloc(&b.qtabs, b.elem() * (size_t)std::max<int64_t>(1, nq));
  if (e == cudaSuccess) e = cudaMalloc(&b.active, act.size());
  if (e == cudaSuccess) e = cudaMemcpy(b.active, act.data(), act.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && nq > 0) {
    if (b.precision == 64) {
      e = cudaMemcpy(b.qtabs, qtabs, sizeof(double) * nq, cudaMemcpyHostToDevice);
    } else {
      std::vector<float> f((size_t)nq);
      for (int64_t i = 0; i < nq; ++i) f[(size_t)i] = (float)qtabs[i];
      e = cudaMemcpy(b.qtabs, f.data(), sizeof(float) * nq, cudaMemcpyHostToDevice);
    }
  }
  if (e == cudaSuccess) e = cudaMemset(b.step, 0, sizeof(int));
  b.nsched = nsteps;
  b.nclass = nclass;
  if (b.graph) {
    cudaGraphExecDestroy(b.graph);
    b.graph = nullptr;
  }
  return e == cudaSuccess ? HS2G_OK : bcuda(e, "set sources");
}

int hs2g_batch_set_clock(hs2g_batch* hb, int step) {
  if (!hb || step < 0) return bfail(HS2G_ERR_ARG, "bad argument");
  BatchDeviceGuard g(hb->b.device);
  cudaError_t e = cudaMemcpyAsync(hb->b.step, &step, sizeof(int), cudaMemcpyHostToDevice, hb->b.stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(hb->b.stream);
  return e == cudaSuccess ? HS2G_OK : bcuda(e, "set clock");
}

int hs2g_batch_run(hs2g_batch* hb, int nsteps, int flags, double* elapsed_ms) {
  if (!hb || nsteps < 0) return bfail(HS2G_ERR_ARG, "bad argument");
  Batch& b = hb->b;
  BatchDeviceGuard g(b.device);
  if (!b.qtabs) {
    int rc = hs2g_batch_set_sources(hb, 0, 1, nullptr);
    if (rc) return rc;
  }
  if (!b.graph) {
    int rc = capture(b);
    if (rc) return rc;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (elapsed_ms) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, b.stream);
  }
  cudaError_t e = cudaSuccess;
  for (int s = 0; s < nsteps && e == cudaSuccess; ++s) e = cudaGraphLaunch(b.graph, b.stream);
  if (elapsed_ms) cudaEventRecord(e1, b.stream);
  if (e == cudaSuccess && (elapsed_ms || (flags & HS2G_SYNC))) e = cudaStreamSynchronize(b.stream);
  if (elapsed_ms) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    *elapsed_ms = ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  return e == cudaSuccess ? HS2G_OK : bcuda(e, "batch run");
}

int hs2g_batch_autotune(hs2g_batch* hb, char* report, int report_len) {
  if (!hb) return bfail(HS2G_ERR_ARG, "null batch");
  Batch& b = hb->b;
  BatchDeviceGuard g(b.device);
  if (!b.qtabs) {
    int rc = hs2g_batch_set_sources(hb, 0, 1, nullptr);
    if (rc) return rc;
  }
  // the z sweep updates T in place: tune on a saved copy and restore it afterwards
  void* save = nullptr;
  const size_t bytes = b.elem() * (size_t)b.nvox;
  cudaError_t e = cudaMalloc(&save, bytes);
  if (e != cudaSuccess) return bcuda(e, "autotune");
  e = cudaMemcpyAsync(save, b.T, bytes, cudaMemcpyDeviceToDevice, b.stream);
  std::string rep;
  if (e == cudaSuccess) e = hs2g::batch_autotune(b, rep);
  cudaError_t e2 = cudaMemcpyAsync(b.T, save, bytes, cudaMemcpyDeviceToDevice, b.stream);
  cudaStreamSynchronize(b.stream);
  cudaFree(save);
  if (b.graph) {
    cudaGraphExecDestroy(b.graph);
    b.graph = nullptr;
  }
  if (report && report_len > 0) {
    strncpy(report, rep.c_str(), (size_t)report_len - 1);
    report[report_len - 1] = 0;
  }
  if (e != cudaSuccess) return bcuda(e, "autotune");
  return e2 == cudaSuccess ? HS2G_OK : bcuda(e2, "autotune restore");
}

}  // extern "C"
