// Per-voxel source shapes evaluated on the device: the two source kinds of the reference that are not uniform
// over their class (alternatingdirection_c_pyx.pyx:307-319 point joules with per-voxel values or per-cell
// volumes, :320-384 the spatially z-decaying impulse).
//
// A handle may hold a shape field S (one double per voxel, 1.0 where no shape was set).  A class whose source
// has a shape gets a per-step table value of 1 on the steps it fires, and the x sweep adds q = table[class] * S
// for every voxel (S = 1 for class-uniform sources, so their values pass unchanged).  The shape of a class is
// written only for that class's voxels, from the device-resident class map and a few scalars (and the z
// coordinates, or the per-voxel joules), so a firing step uploads nothing beyond the step's own input.
#include <cmath>

#include "hs2g_internal.cuh"

namespace hs2g {
namespace {

constexpr int kTile = 1024;  // voxels per tile of the rank scan (one thread each)

__global__ void fill_kernel(double* __restrict__ p, int64_t n, double v) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
    p[e] = v;
}

// Spatially z-decaying impulse (pyx:320-384): the energy per unit area J deposited by a (1/l) exp(-d/l) profile
// into each cell between its z boundaries, d measured along direction (+1 or -1 times z) from offset and
// clipped at 0, divided by the cell thickness and dt.  Cells whose far boundary lies at d <= 0 get nothing.
// The operations follow the reference's order (centre, boundaries, clip, -exp(-b/l) + exp(-a/l), * J,
// / (ddz * dt)); exp is the device's, within an ulp of the host's.
__global__ void zdecay_kernel(int64_t n, const uint8_t* __restrict__ vclass, int cls, const double* __restrict__ zgrid,
                              double direction, double offset, double ddz, double jpm2, double length, double dt,
                              double* __restrict__ shape) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    if (vclass[p] != cls) continue;
    const double centre = zgrid[p] * direction - offset;
    double left = centre - ddz / 2.0;
    const double right = centre + ddz / 2.0;
    if (!(right > 0.0)) {
      shape[p] = 0.0;
      continue;
    }
    if (left < 0.0) left = 0.0;
    const double frac = -exp(-right / length) + exp(-left / length);
    shape[p] = frac * jpm2 / (ddz * dt);
  }
}

// Rank of each class voxel among the class's voxels in C order, in two passes over tiles of kTile voxels:
// per-tile counts, then (after an exclusive scan of the counts) the ranks inside each tile.
__global__ void tile_count_kernel(int64_t n, const uint8_t* __restrict__ vclass, int cls, int64_t* __restrict__ count) {
  const int64_t p = (int64_t)blockIdx.x * kTile + threadIdx.x;
  const int in = p < n && vclass[p] == cls;
  const int c = __syncthreads_count(in);
  if (threadIdx.x == 0) count[blockIdx.x] = c;
}

// exclusive scan of ntile counts in place, one CTA (ntile = voxels / 1024: a few thousand at most in practice)
__global__ void tile_scan_kernel(int64_t ntile, int64_t* __restrict__ v) {
  __shared__ int64_t part[kTile];
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < ntile; base += kTile) {
    const int64_t e = base + threadIdx.x;
    const int64_t x = e < ntile ? v[e] : 0;
    part[threadIdx.x] = x;
    __syncthreads();
    for (int off = 1; off < kTile; off <<= 1) {  // Hillis-Steele inclusive scan
      const int64_t add = threadIdx.x >= off ? part[threadIdx.x - off] : 0;
      __syncthreads();
      part[threadIdx.x] += add;
      __syncthreads();
    }
    if (e < ntile) v[e] = carry + part[threadIdx.x] - x;
    __syncthreads();
    if (threadIdx.x == kTile - 1) carry += part[kTile - 1];
    __syncthreads();
  }
}

// Point-joules impulse (pyx:307-319): J per voxel / (V * dt), V the cell volume (volumes[p] when given, as in
// the curved-surface mode) and J the class's scalar (count == 1) or its value for this voxel, taken in the
// order of the class's voxels in C order (the order of numpy's boolean-mask assignment).
__global__ void point_kernel(int64_t n, const uint8_t* __restrict__ vclass, int cls, const int64_t* __restrict__ tile_off,
                             const double* __restrict__ joules, int64_t count, const double* __restrict__ volumes,
                             double volume, double dt, double* __restrict__ shape) {
  __shared__ int warp_sum[kTile / 32];
  const int64_t p = (int64_t)blockIdx.x * kTile + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool in = p < n && vclass[p] == cls;
  const unsigned ball = __ballot_sync(0xffffffffu, in);
  if (lane == 0) warp_sum[warp] = __popc(ball);
  __syncthreads();
  if (warp == 0) {  // exclusive scan of the 32 warp counts
    const int x = warp_sum[lane];
    int s = x;
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, off);
      if (lane >= off) s += y;
    }
    warp_sum[lane] = s - x;
  }
  __syncthreads();
  if (!in) return;
  const int64_t rank = tile_off[blockIdx.x] + warp_sum[warp] + __popc(ball & ((1u << lane) - 1u));
  if (count != 1 && rank >= count) return;  // more class voxels than values: checked by the host first
  const double J = joules[count == 1 ? 0 : rank];
  const double V = volumes ? volumes[p] : volume;
  shape[p] = J / (V * dt);
}

inline unsigned grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > (1 << 20)) b = 1 << 20;
  return (unsigned)b;
}

}  // namespace

cudaError_t launch_fill(double* p, int64_t n, double v, cudaStream_t s) {
  fill_kernel<<<grid_for(n, 256), 256, 0, s>>>(p, n, v);
  return cudaGetLastError();
}

cudaError_t launch_zdecay_shape(int64_t n, const uint8_t* vclass, int cls, const double* zgrid, double direction,
                                double offset, double ddz, double jpm2, double length, double dt, double* shape,
                                cudaStream_t s) {
  zdecay_kernel<<<grid_for(n, 256), 256, 0, s>>>(n, vclass, cls, zgrid, direction, offset, ddz, jpm2, length, dt,
                                                  shape);
  return cudaGetLastError();
}

int64_t point_shape_tiles(int64_t n) { return (n + kTile - 1) / kTile; }

cudaError_t launch_point_shape(int64_t n, const uint8_t* vclass, int cls, int64_t* tile_scratch, const double* joules,
                               int64_t count, const double* volumes, double volume, double dt, double* shape,
                               cudaStream_t s) {
  const int64_t ntile = point_shape_tiles(n);
  tile_count_kernel<<<(unsigned)ntile, kTile, 0, s>>>(n, vclass, cls, tile_scratch);
  tile_scan_kernel<<<1, kTile, 0, s>>>(ntile, tile_scratch);
  point_kernel<<<(unsigned)ntile, kTile, 0, s>>>(n, vclass, cls, tile_scratch, joules, count, volumes, volume, dt,
                                                 shape);
  return cudaGetLastError();
}

}  // namespace hs2g
