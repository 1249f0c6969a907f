// The per-step sweep kernels: one Douglas ADI timestep in scaled delta form (see hs2g_compile.cu for the
// algebra and hs2g_internal.cuh for the coefficient layout).  Replaces, per timestep, the reference's
// source-field assembly and three permute / CSR mat-vec / tridiagonal-solve stages
// (alternatingdirection_c_pyx.pyx:294-416, tridiag.pyx:46-69).
//
// FP64 is the binding resource on GB300 (about 0.6e12 DFMA/s against ~6.5 TB/s of HBM), so the step is
// arranged for the fewest FP64 operations: 7 stencil FMAs (+1 when a source is active) and 2 recurrence
// FMAs per voxel in the x sweep, 2 FMAs per voxel in the y sweep, 2 FMAs and 1 add per voxel in the z sweep.
//
// Memory layout: every field is (nz, ny, nx) with x fastest; the stage-0 stencil coefficients are
// chunk-blocked (hs2g_internal.cuh).
//   x sweep: a CTA owns 32 consecutive x-lines.  The stencil is evaluated in 32-column chunks with lanes
//            along x (coalesced loads of T and of the line's coefficient block), staged through shared memory,
//            and one warp runs the 32 line recurrences down the transposed chunk (lane = line).  The forward
//            values are kept in the output array W0 and re-read by the back substitution in the same CTA.
//   y sweep: TMA tensor tiles (hs2g_lines.cu), or one thread per y-line with plain loads.
//   z sweep: one thread per z-line (j,i); neighbouring lanes have neighbouring i, so each k step is one
//            coalesced 256-byte access per array per warp (a TMA variant exists, HS2G_Z_SWEEP=tma).
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "hs2g_internal.cuh"

namespace hs2g {
namespace {

constexpr int kXLines = 32;   // x-lines per CTA
constexpr int kXChunk = 32;   // columns per staged chunk
constexpr int kXThreads = 128;
constexpr int kXWarps = kXThreads / 32;
// Register budget of the x sweep: at 72 registers 7 CTAs of 128 threads fit on an SM, so the 1040 CTAs of a
// 65 x 512-line grid run in one wave on 152 SMs with the most loads in flight per thread (332 us at
// 65x512x512; 80 registers: 6 CTAs per SM and a second wave, 530 us; the compiler's own choice of 48
// registers: 415 us; a bound of 7 blocks also gives 72 registers but schedules worse: 347-363 us).  The
// whole-grid kernels set the budget directly (__maxnreg__); the host-buffer step's line-range kernels keep a
// bound of 6 blocks (kXMinBlocks).  Check -Xptxas -v after a change.
constexpr int kXMinBlocks = 6;
constexpr int kLineThreads = 128;

// Stage-0 right-hand side of voxel (L, i) of x-line L = k*ny + j, pre-scaled by the line's pivot:
// wc*T + wxl*T[i-1] + wxh*T[i+1] + wyl*T[j-1] + wyh*T[j+1] + wzl*T[k-1] + wzh*T[k+1] (+ wq*Q).
// Out-of-grid neighbours carry a zero coefficient (exterior faces are insulating): T[p] is read instead.
// Column i = ch*32 + lane of the chunk; the coefficients come from the line's chunk block.
// A sweep's forward values are written and read back by the same thread block within microseconds; with
// every line in flight they add up to more than L2 (136 MB at 65x512x512), so they are stored with an
// evict-last L2 policy where that keeps them on chip.
// IX: the index type of the voxel, line and coefficient-block arithmetic (int32_t when the grid and its stencil
// blocks have fewer than 2^31 elements, which makes the line -> (k, j) division a 32-bit one).
template <bool HAS_Q, typename IX = int64_t>
__device__ __forceinline__ double stencil_x(const Dims& d, const double* __restrict__ T, const Coeffs& c,
                                            const uint8_t* __restrict__ vclass, const double* __restrict__ qdense,
                                            const double* __restrict__ qshape, const double* sq, IX L, int ch,
                                            int lane) {
  const IX nx = (IX)d.nx, ny = (IX)d.ny, nz = (IX)d.nz;
  const IX i = (IX)ch * 32 + lane;
  const IX k = L / ny, j = L - k * ny;
  const IX p = L * nx + i;
  const IX nxy = nx * ny;
  const double* __restrict__ w = c.xb + ((L * (IX)c.nchunks + ch) * kXBlockCoeffs) * 32 + lane;
  const double t = T[p];
  const double txl = i > 0 ? T[p - 1] : t;
  const double txh = i + 1 < nx ? T[p + 1] : t;
  const double tyl = j > 0 ? T[p - nx] : t;
  const double tyh = j + 1 < ny ? T[p + nx] : t;
  const double tzl = k > 0 ? T[p - nxy] : t;
  const double tzh = k + 1 < nz ? T[p + nxy] : t;
  double r = w[kWc * 32] * t;
  r = fma(w[kWxl * 32], txl, r);
  r = fma(w[kWxh * 32], txh, r);
  r = fma(w[kWyl * 32], tyl, r);
  r = fma(w[kWyh * 32], tyh, r);
  r = fma(w[kWzl * 32], tzl, r);
  r = fma(w[kWzh * 32], tzh, r);
  if (HAS_Q) {
    double q = sq[vclass[p]];
    if (qshape) q *= qshape[p];
    if (qdense) q += qdense[p];
    r = fma(w[kWq * 32], q, r);
  }
  return r;
}

// RANGED: the launch covers x-lines [line_begin, line_end) (the overlapped host-buffer step); otherwise all
// nz*ny lines, with the arguments unused -- the two are separate instances so that the whole-grid kernel keeps
// its own register allocation.  LINES x-lines per CTA: 32 for the whole grid; the host-buffer step's later,
// smaller slabs take 16 or 8, whose CTAs finish sooner (a CTA's chunk loop, not the GPU's throughput, sets
// how long a small launch takes).
// PITCH 0: W0 shares T's row pitch nx; 1: one pad column (odd nx: pitch nx + 1, so the W0 index of voxel (L, i)
// is its T index plus L); 2: any other pitch c.px (padding for tests).
template <int PITCH, typename IX = int64_t>
__device__ __forceinline__ IX w0_index(const Dims& d, const Coeffs& c, IX L, IX i) {
  if (PITCH == 0) return L * (IX)d.nx + i;
  if (PITCH == 1) return L * (IX)d.nx + i + L;
  return L * (IX)c.px + i;
}

// The class source values come from the kernel's parameter table qt, or (QROW) from the global row qrow.  The
// kernel owns the shared arrays: sr, sa [LINES][kXChunk + 1] and sq [HS2G_MAX_CLASSES when HAS_Q].
template <bool HAS_Q, bool RANGED, int LINES, int PITCHED, bool QROW = false, typename QT = QTable,
          typename IX = int64_t>
__device__ __forceinline__ void sweep_x_body(const Dims& d, const double* __restrict__ T, const Coeffs& c,
                                             const uint8_t* __restrict__ vclass, const double* __restrict__ qdense,
                                             const double* __restrict__ qshape, const QT& qt,
                                             const double* __restrict__ qrow, double* __restrict__ W0,
                                             int64_t line_begin, int64_t line_end, double (*sr)[kXChunk + 1],
                                             double (*sa)[kXChunk + 1], double* sq) {
  constexpr int kPerWarp = LINES / kXWarps;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if constexpr (HAS_Q) {
    for (int e = threadIdx.x; e < HS2G_MAX_CLASSES; e += kXThreads) {
      if constexpr (QROW)
        sq[e] = qrow[e];
      else
        sq[e] = qt.q[e];
    }
  }
  const IX nx = (IX)d.nx;
  const IX nlines = RANGED ? (IX)line_end : (IX)(d.nz * d.ny);
  const IX L0 = (RANGED ? (IX)line_begin : 0) + (IX)blockIdx.x * LINES;
  const int nchunks = (int)((d.nx + kXChunk - 1) / kXChunk);
  wait_prior_grid();  // T comes from the previous step's z sweep, which used W0 as its scratch
  __syncthreads();

  // forward: z_i = R'_i - a0_i * z_{i-1}
  double carry = 0.0;
  for (int ch = 0; ch < nchunks; ++ch) {
    const IX i = (IX)ch * kXChunk + lane;
#pragma unroll
    for (int ll = 0; ll < kPerWarp; ++ll) {
      const int l = warp * kPerWarp + ll;
      const IX L = L0 + l;
      double r = 0.0, a = 0.0;
      if (L < nlines && i < nx) {
        r = stencil_x<HAS_Q, IX>(d, T, c, vclass, qdense, qshape, sq, L, ch, lane);
        a = c.a0[L * nx + i];
      }
      sr[l][lane] = r;
      sa[l][lane] = a;
    }
    __syncthreads();
    if (warp * 32 + lane < LINES) {  // lane = line of the recurrence
      const int l = warp * 32 + lane;
      const int cw = (int)min((int64_t)kXChunk, d.nx - (int64_t)ch * kXChunk);
      double z = carry;
      if (cw == kXChunk) {  // full chunks unrolled: the shared loads of later rows issue ahead of the chain
#pragma unroll 4
        for (int cc = 0; cc < kXChunk; ++cc) {
          z = fma(-sa[l][cc], z, sr[l][cc]);
          sr[l][cc] = z;
        }
      } else {
        for (int cc = 0; cc < cw; ++cc) {
          z = fma(-sa[l][cc], z, sr[l][cc]);
          sr[l][cc] = z;
        }
      }
      carry = z;
    }
    __syncthreads();
#pragma unroll
    for (int ll = 0; ll < kPerWarp; ++ll) {
      const int l = warp * kPerWarp + ll;
      const IX L = L0 + l;
      if (L < nlines && i < nx) W0[w0_index<PITCHED, IX>(d, c, L, i)] = sr[l][lane];
    }
    __syncthreads();
  }

  // back substitution: W0_i = z_i - b0_i * W0_{i+1}
  carry = 0.0;
  for (int ch = nchunks - 1; ch >= 0; --ch) {
    const IX i = (IX)ch * kXChunk + lane;
#pragma unroll
    for (int ll = 0; ll < kPerWarp; ++ll) {
      const int l = warp * kPerWarp + ll;
      const IX L = L0 + l;
      double z = 0.0, b = 0.0;
      if (L < nlines && i < nx) {
        const IX p = L * nx + i;
        z = W0[w0_index<PITCHED, IX>(d, c, L, i)];
        b = c.b0[p];
      }
      sr[l][lane] = z;
      sa[l][lane] = b;
    }
    __syncthreads();
    if (warp * 32 + lane < LINES) {
      const int l = warp * 32 + lane;
      const int cw = (int)min((int64_t)kXChunk, d.nx - (int64_t)ch * kXChunk);
      double x = carry;
      if (cw == kXChunk) {
#pragma unroll 4
        for (int cc = kXChunk - 1; cc >= 0; --cc) {
          x = fma(-sa[l][cc], x, sr[l][cc]);
          sr[l][cc] = x;
        }
      } else {
        for (int cc = cw - 1; cc >= 0; --cc) {
          x = fma(-sa[l][cc], x, sr[l][cc]);
          sr[l][cc] = x;
        }
      }
      carry = x;
    }
    __syncthreads();
#pragma unroll
    for (int ll = 0; ll < kPerWarp; ++ll) {
      const int l = warp * kPerWarp + ll;
      const IX L = L0 + l;
      if (L < nlines && i < nx) W0[w0_index<PITCHED, IX>(d, c, L, i)] = sr[l][lane];
    }
    __syncthreads();
  }
}

// The x sweep over the whole grid: the register budget is set to 72, which keeps 7 CTAs of 128 threads per SM, so
// the 1040 CTAs of a 65x512-line grid run in one wave (332 us at 65x512x512; under a bound of 6 blocks the
// instance without a source also gets 72 registers and takes 334 us, while the instances with a source term or
// padded W0 rows take 78-80 registers there, 6 CTAs per SM, two waves: 694 us for a source step).  Padded rows
// of an odd nx use the one-column index (349 us at 65x512x511; with a general pitch 362 us).
// The class table is a kernel parameter only in the instances with a source (2 KB that the others would copy at
// every launch for nothing).
template <bool HAS_Q>
using XTable = typename std::conditional<HAS_Q, QTable, int>::type;
template <bool HAS_Q, bool RANGED, int LINES, int PITCH, typename IX = int64_t>
__global__ void __maxnreg__(72) sweep_x_lean_kernel(Dims d, const double* __restrict__ T, Coeffs c,
                                                    const uint8_t* __restrict__ vclass,
                                                    const double* __restrict__ qdense,
                                                    const double* __restrict__ qshape, XTable<HAS_Q> qt,
                                                    double* __restrict__ W0, int64_t line_begin, int64_t line_end) {
  __shared__ double sr[LINES][kXChunk + 1];
  __shared__ double sa[LINES][kXChunk + 1];
  __shared__ double sq[HAS_Q ? HS2G_MAX_CLASSES : 1];
  sweep_x_body<HAS_Q, RANGED, LINES, PITCH, false, XTable<HAS_Q>, IX>(d, T, c, vclass, qdense, qshape, qt, nullptr,
                                                                      W0, line_begin, line_end, sr, sa, sq);
}
// The line ranges of the host-buffer step on unpadded rows keep the 6-block bound (80 registers at 32 lines per
// CTA): measured against the 72-register build there, 9.62e9 against 9.39e9 voxel-steps/s end to end.
template <bool HAS_Q, bool RANGED, int LINES = kXLines>
__global__ void __launch_bounds__(kXThreads, kXMinBlocks) sweep_x_kernel(Dims d, const double* __restrict__ T, Coeffs c,
                                                             const uint8_t* __restrict__ vclass,
                                                             const double* __restrict__ qdense,
                                                             const double* __restrict__ qshape, XTable<HAS_Q> qt,
                                                             double* __restrict__ W0, int64_t line_begin,
                                                             int64_t line_end) {
  __shared__ double sr[LINES][kXChunk + 1];
  __shared__ double sa[LINES][kXChunk + 1];
  __shared__ double sq[HAS_Q ? HS2G_MAX_CLASSES : 1];
  sweep_x_body<HAS_Q, RANGED, LINES, 0>(d, T, c, vclass, qdense, qshape, qt, nullptr, W0, line_begin, line_end, sr,
                                        sa, sq);
}

// The x sweep of a step whose class table is row ds->step of the handle's device schedule (the steps with a
// source in the captured step graphs of hs2g_run): thread 0 reads the row's address once for the CTA; an
// inactive row or one past the schedule's end gives the zero table.  Only the source body is compiled here:
// the steps without a source run sweep_x_lean_kernel, whose code a second body in the same kernel would slow
// (measured 3 us per step at 65x512x512).
__device__ const double kZeroRow[HS2G_MAX_CLASSES] = {};
template <int PITCH>
__global__ void __maxnreg__(72) sweep_x_row_kernel(Dims d, const double* __restrict__ T, Coeffs c,
                                                   const uint8_t* __restrict__ vclass,
                                                   const DevSchedule* __restrict__ ds, double* __restrict__ W0) {
  __shared__ double sr[kXLines][kXChunk + 1];
  __shared__ double sa[kXLines][kXChunk + 1];
  __shared__ double sq[HS2G_MAX_CLASSES];
  __shared__ const double* s_row;
  if (threadIdx.x == 0) {
    const int64_t st = ds->step;
    s_row = st >= 0 && st < ds->n && ds->active[st] ? ds->q + st * HS2G_MAX_CLASSES : kZeroRow;
  }
  __syncthreads();
  const int no_table = 0;  // the table comes from the row
  sweep_x_body<true, false, kXLines, PITCH, true>(d, T, c, vclass, nullptr, ds->shape, no_table, s_row, W0, 0, 0, sr,
                                                  sa, sq);
}

// Whether the whole-grid x sweep may index in 32 bits: every voxel index (with the pad column of an odd nx) and
// every stencil-block element below 2^31.  HS2G_X_INDEX=64 keeps 64-bit indices.
bool x_index32(const Dims& d, const Coeffs& c) {
  static const bool off = [] {
    const char* e = getenv("HS2G_X_INDEX");
    return e && strcmp(e, "64") == 0;
  }();
  const int64_t lim = (int64_t)1 << 31;
  return !off && d.nvox() + d.nz * d.ny < lim && d.nz * d.ny * c.nchunks * kXBlockCoeffs * 32 < lim;
}

// x sweep over all lines (RANGED false) or the lines [line_begin, line_end) of the host-buffer step
template <bool RANGED, int LINES>
void launch_x(const StepArgs& a, const Coeffs& c, const QTable& q, int64_t line_begin, int64_t line_end,
              cudaStream_t s) {
  const Dims& d = a.d;
  const unsigned gx = (unsigned)(((RANGED ? line_end - line_begin : d.nz * d.ny) + LINES - 1) / LINES);
  const bool has_q = a.has_qtab || a.qdense != nullptr;
  const int pitch = c.px == d.nx ? 0 : c.px == d.nx + 1 ? 1 : 2;
#define HS2G_X(KERNEL, TABLE, ...)                                                                             \
  launch_kernel(KERNEL<__VA_ARGS__>, dim3(gx), dim3(kXThreads), 0, s, a.pdl_x, d, a.T_in, c, a.vclass, a.qdense, \
                a.qshape, TABLE, a.W0, line_begin, line_end)
  if constexpr (!RANGED) {
    if (pitch < 2 && x_index32(d, c)) {
      if (pitch == 0) {
        if (has_q)
          HS2G_X(sweep_x_lean_kernel, q, true, false, LINES, 0, int32_t);
        else
          HS2G_X(sweep_x_lean_kernel, 0, false, false, LINES, 0, int32_t);
      } else {
        if (has_q)
          HS2G_X(sweep_x_lean_kernel, q, true, false, LINES, 1, int32_t);
        else
          HS2G_X(sweep_x_lean_kernel, 0, false, false, LINES, 1, int32_t);
      }
      return;
    }
  }
  if (RANGED && pitch == 0) {
    if (has_q)
      HS2G_X(sweep_x_kernel, q, true, RANGED, LINES);
    else
      HS2G_X(sweep_x_kernel, 0, false, RANGED, LINES);
  } else if (pitch == 0) {
    if (has_q)
      HS2G_X(sweep_x_lean_kernel, q, true, RANGED, LINES, 0);
    else
      HS2G_X(sweep_x_lean_kernel, 0, false, RANGED, LINES, 0);
  } else if (pitch == 1) {
    if (has_q)
      HS2G_X(sweep_x_lean_kernel, q, true, RANGED, LINES, 1);
    else
      HS2G_X(sweep_x_lean_kernel, 0, false, RANGED, LINES, 1);
  } else {
    if (has_q)
      HS2G_X(sweep_x_lean_kernel, q, true, RANGED, LINES, 2);
    else
      HS2G_X(sweep_x_lean_kernel, 0, false, RANGED, LINES, 2);
  }
#undef HS2G_X
}

void launch_x_row(const StepArgs& a, const Coeffs& c, const DevSchedule* ds, cudaStream_t s) {
  const Dims& d = a.d;
  const unsigned gx = (unsigned)((d.nz * d.ny + kXLines - 1) / kXLines);
  const int pitch = c.px == d.nx ? 0 : c.px == d.nx + 1 ? 1 : 2;
  if (pitch == 0)
    launch_kernel(sweep_x_row_kernel<0>, dim3(gx), dim3(kXThreads), 0, s, a.pdl_x, d, a.T_in, c, a.vclass, ds, a.W0);
  else if (pitch == 1)
    launch_kernel(sweep_x_row_kernel<1>, dim3(gx), dim3(kXThreads), 0, s, a.pdl_x, d, a.T_in, c, a.vclass, ds, a.W0);
  else
    launch_kernel(sweep_x_row_kernel<2>, dim3(gx), dim3(kXThreads), 0, s, a.pdl_x, d, a.T_in, c, a.vclass, ds, a.W0);
}

// y lines: W1 = s2 * dT1 from W0 = sigma * dT0
__global__ void __launch_bounds__(kLineThreads) sweep_y_kernel(Dims d, const double* __restrict__ W0,
                                                                const double* __restrict__ a1,
                                                                const double* __restrict__ b1,
                                                                double* __restrict__ W1, int64_t px) {
  wait_prior_grid();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= d.nz * d.nx) return;
  const int64_t k = t / d.nx, i = t - k * d.nx;
  int64_t p = k * d.ny * px + i;  // the y-sweep arrays have row pitch px
  double z = 0.0;
#pragma unroll 4
  for (int64_t j = 0; j < d.ny; ++j, p += px) {
    z = fma(-a1[p], z, W0[p]);
    W1[p] = z;
  }
  double x = 0.0;
#pragma unroll 4
  for (int64_t j = d.ny - 1; j >= 0; --j) {
    p -= px;
    x = fma(-b1[p], x, W1[p]);
    W1[p] = x;
  }
}

// z lines: dT2 from W1 = s2 * dT1; T_out = T_in + dT2.  Z is scratch (the x sweep's buffer, free by now).
// T_in may equal T_out: each voxel's T_in is read by the same thread just before its T_out is written.
// DISCARD: the forward values are read once by the back substitution and never again, so once a warp has read
// a group of 4 rows k .. k+3 (k a multiple of 4) it drops their Z lines from L2 (lanes 0 and 16 each own one
// 128-byte line of a row), which saves the write-back of every line still cached; only warps whose 32 columns
// are whole lines of every plane do this (nxy a multiple of 16, warp-aligned columns inside the launch's range),
// and the rows above the top group (nz mod 4 of them) are left as they are.
// 16 CTAs per SM (32 registers): the 2048 CTAs of a 512x512-column grid are resident at once.
template <bool DISCARD>
__global__ void __launch_bounds__(kLineThreads, 16) sweep_z_kernel(Dims d, const double* __restrict__ W1,
                                                                const double* __restrict__ a2,
                                                                const double* __restrict__ b2, const double* T_in,
                                                                double* __restrict__ Z, double* T_out,
                                                                int64_t col_begin, int64_t col_end, int64_t px) {
  // this launch covers the z-lines (columns j*nx + i) [col_begin, col_end); W1 has row pitch px
  const int64_t t = col_begin + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t nxy = d.nxy();
  const int64_t t0 = t - (threadIdx.x & 31);  // the warp's first column
  const bool drop = DISCARD && nxy % 16 == 0 && t0 % 32 == 0 && t0 + 32 <= col_end;  // warp-uniform
  wait_prior_grid();
  if (t >= col_end) return;
  int64_t p = t;
  const int64_t jw = t / d.nx;
  int64_t pw = jw * px + (t - jw * d.nx);
  const int64_t nxyw = d.ny * px;
  const uint64_t keep = l2_evict_last();  // the forward values come back to this thread after its last row
  double z = 0.0;
#pragma unroll 4
  for (int64_t k = 0; k < d.nz; ++k, p += nxy, pw += nxyw) {
    z = fma(-a2[p], z, W1[pw]);
    st_hint(Z + p, z, keep);
  }
  double x = 0.0;
  if (!DISCARD) {
#pragma unroll 4
    for (int64_t k = d.nz - 1; k >= 0; --k) {
      p -= nxy;
      x = fma(-b2[p], x, Z[p]);
      T_out[p] = T_in[p] + x;
    }
    return;
  }
  int64_t k = d.nz - 1;
#pragma unroll 1
  for (; (k & 3) != 3; --k) {  // rows above the last whole group of 4
    p -= nxy;
    x = fma(-b2[p], x, Z[p]);
    T_out[p] = T_in[p] + x;
  }
#pragma unroll 1
  for (; k >= 3; k -= 4) {  // rows k-3 .. k, then their Z lines dropped
    p -= 4 * nxy;
    double z3 = Z[p + 3 * nxy], z2 = Z[p + 2 * nxy], z1 = Z[p + nxy], z0 = Z[p];
    x = fma(-b2[p + 3 * nxy], x, z3);
    T_out[p + 3 * nxy] = T_in[p + 3 * nxy] + x;
    x = fma(-b2[p + 2 * nxy], x, z2);
    T_out[p + 2 * nxy] = T_in[p + 2 * nxy] + x;
    x = fma(-b2[p + nxy], x, z1);
    T_out[p + nxy] = T_in[p + nxy] + x;
    x = fma(-b2[p], x, z0);
    T_out[p] = T_in[p] + x;
    if (!drop) continue;
    __syncwarp();  // every lane of the warp has read its four rows of Z
    if ((threadIdx.x & 15) == 0) {
      l2_discard_line(Z + p);
      l2_discard_line(Z + p + nxy);
      l2_discard_line(Z + p + 2 * nxy);
      l2_discard_line(Z + p + 3 * nxy);
    }
  }
}

__global__ void copy_layer_kernel(Dims d, const double* __restrict__ T, int layer, double* __restrict__ dst) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < d.nxy()) dst[t] = T[(int64_t)layer * d.nxy() + t];
}

// Temperature of the z = 0 surface estimated from layers 0 and 1 as the reference's
// insulating_z_min_surface_temperature(T, dz) does (surface_temperature.py:4-36): the mean of a quadratic with
// zero slope at the surface through the two layer centres, c = T0 - (0.25 a) dz^2 with a = (T1 - T0)/(2 dz^2),
// and the linear extrapolation T0 - (T1 - T0)/2.  Same operations in the same order, each rounding explicit.
__device__ __forceinline__ double surface_value(double t0, double t1, double dz2) {
  const double a = __ddiv_rn(__dsub_rn(t1, t0), __dmul_rn(2.0, dz2));
  const double c = __dsub_rn(t0, __dmul_rn(__dmul_rn(0.25, a), dz2));
  const double lin = __dsub_rn(t0, __ddiv_rn(__dsub_rn(t1, t0), 2.0));
  return __ddiv_rn(__dadd_rn(lin, c), 2.0);
}
__global__ void surface_estimate_kernel(int64_t nxy, const double* __restrict__ T, double dz2,
                                        double* __restrict__ dst) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < nxy) dst[t] = surface_value(T[t], T[nxy + t], dz2);
}

inline unsigned blocks(int64_t n, int per) { return (unsigned)((n + per - 1) / per); }
// History of a step into row ds->row of hist: layer `layer` of T, or (dz2 > 0) the surface estimate; the last
// CTA to finish advances the row (every CTA read it at its start).
__global__ void history_row_kernel(int64_t nxy, const double* __restrict__ T, int layer, double dz2,
                                   double* __restrict__ hist, DevSchedule* ds) {
  __shared__ int64_t s_row;
  wait_prior_grid();
  if (threadIdx.x == 0) s_row = *(volatile int64_t*)&ds->row;
  __syncthreads();
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < nxy)
    hist[s_row * nxy + t] = dz2 > 0.0 ? surface_value(T[t], T[nxy + t], dz2) : T[(int64_t)layer * nxy + t];
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&ds->hist_done, 1u) == gridDim.x - 1) {
      ds->row = s_row + 1;
      ds->hist_done = 0;
      __threadfence();
    }
  }
}

__global__ void schedule_flags_kernel(const double* __restrict__ q, int64_t nrows, uint8_t* __restrict__ active) {
  const int64_t r = blockIdx.x * (int64_t)(blockDim.x / 32) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= nrows) return;
  bool any = false;
  for (int c = lane; c < HS2G_MAX_CLASSES; c += 32) any |= q[r * HS2G_MAX_CLASSES + c] != 0.0;
  any = __any_sync(0xffffffffu, any);
  if (lane == 0) active[r] = any ? 1 : 0;
}


// FP64 issue-rate probe: 8 independent FMA chains per thread, registers only, one store per thread.
__global__ void fp64_probe_kernel(double* out, int iters, double a, double b) {
  double acc[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) acc[k] = (double)(threadIdx.x + k);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = fma(acc[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += acc[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

cudaError_t fp64_fma_rate(double* fma_per_s) {
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const int blocksN = sms * 4, threads = 256, iters = 4096;
  double* out = nullptr;
  e = cudaMalloc(&out, sizeof(double) * blocksN * threads);
  if (e != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0, 0);
    fp64_probe_kernel<<<blocksN, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1, 0);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  *fma_per_s = (double)blocksN * threads * iters * 8 / (best * 1e-3);
  return e;
}

namespace {
// the y and z sweeps of a step, with events before each and after the last when ev is given
cudaError_t launch_yz(const StepArgs& a, const Coeffs& c, cudaStream_t s, cudaEvent_t* ev) {
  const Dims& d = a.d;
  cudaError_t e = cudaSuccess;
  if (a.bulk_y)
    e = launch_lines_bulk(d, 1, a.W0, c.a1, a.W1, c.b1, nullptr, a.W1, a.status, a.tmaps, s, c.px, a.pdl);
  else
    e = launch_kernel(sweep_y_kernel, dim3(blocks(d.nz * d.nx, kLineThreads)), dim3(kLineThreads), 0, s, a.pdl, d,
                      a.W0, c.a1, c.b1, a.W1, c.px);
  if (e != cudaSuccess) return e;
  if (ev) cudaEventRecord(ev[2], s);
  if (a.bulk_z)
    e = launch_lines_bulk(d, 2, a.W1, c.a2, a.W0, c.b2, a.T_in, a.T_out, a.status, a.tmaps, s, d.nx, a.pdl);
  else
    e = launch_z_range(a, c, 0, d.nxy(), s);
  if (e != cudaSuccess) return e;
  if (ev) cudaEventRecord(ev[3], s);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_step_events(const StepArgs& a, const Coeffs& c, const QTable& q, cudaStream_t s,
                               cudaEvent_t ev[4]) {
  if (ev) cudaEventRecord(ev[0], s);
  launch_x<false, kXLines>(a, c, q, 0, 0, s);
  if (ev) cudaEventRecord(ev[1], s);
  return launch_yz(a, c, s, ev);
}

cudaError_t launch_step(const StepArgs& a, const Coeffs& c, const QTable& q, cudaStream_t s) {
  return launch_step_events(a, c, q, s, nullptr);
}

cudaError_t launch_step_row(const StepArgs& a, const Coeffs& c, const DevSchedule* ds, cudaStream_t s) {
  launch_x_row(a, c, ds, s);
  return launch_yz(a, c, s, nullptr);
}

cudaError_t launch_history_row(const Dims& d, const double* T, int layer, double dz2, double* hist, DevSchedule* ds,
                               cudaStream_t s, bool pdl) {
  return launch_kernel(history_row_kernel, dim3(blocks(d.nxy(), 256)), dim3(256), 0, s, pdl, d.nxy(), T, layer, dz2,
                       hist, ds);
}

cudaError_t launch_schedule_flags(const double* q, int64_t nrows, uint8_t* active, cudaStream_t s) {
  if (nrows <= 0) return cudaSuccess;
  schedule_flags_kernel<<<blocks(nrows, 8), 256, 0, s>>>(q, nrows, active);
  return cudaGetLastError();
}

double surface_dz2(double dz) {
  // dz^2 as the reference's dz**2.0 computes it: the C library's pow, which can differ from dz*dz by an ulp (the
  // volatile exponent keeps the compiler from replacing the call by a multiplication)
  volatile double two = 2.0;
  return std::pow(dz, (double)two);
}

template <int LINES>
void launch_x_lines(const StepArgs& a, const Coeffs& c, const QTable& q, int64_t line_begin, int64_t line_end,
                    cudaStream_t s) {
  launch_x<true, LINES>(a, c, q, line_begin, line_end, s);
}

cudaError_t launch_x_range(const StepArgs& a, const Coeffs& c, const QTable& q, int64_t line_begin,
                           int64_t line_end, int lines_per_cta, cudaStream_t s) {
  if (line_end <= line_begin) return cudaSuccess;
  if (lines_per_cta == 8)
    launch_x_lines<8>(a, c, q, line_begin, line_end, s);
  else if (lines_per_cta == 16)
    launch_x_lines<16>(a, c, q, line_begin, line_end, s);
  else
    launch_x_lines<kXLines>(a, c, q, line_begin, line_end, s);
  return cudaGetLastError();
}

cudaError_t launch_y(const StepArgs& a, const Coeffs& c, cudaStream_t s) {
  const Dims& d = a.d;
  if (a.bulk_y)
    return launch_lines_bulk(d, 1, a.W0, c.a1, a.W1, c.b1, nullptr, a.W1, a.status, a.tmaps, s, c.px);
  sweep_y_kernel<<<blocks(d.nz * d.nx, kLineThreads), kLineThreads, 0, s>>>(d, a.W0, c.a1, c.b1, a.W1, c.px);
  return cudaGetLastError();
}

cudaError_t launch_z_range(const StepArgs& a, const Coeffs& c, int64_t col_begin, int64_t col_end, cudaStream_t s) {
  const Dims& d = a.d;
  if (col_end <= col_begin) return cudaSuccess;
  const unsigned grid = blocks(col_end - col_begin, kLineThreads);
  if (a.z_discard)
    return launch_kernel(sweep_z_kernel<true>, dim3(grid), dim3(kLineThreads), 0, s, a.pdl, d, a.W1, c.a2, c.b2,
                         a.T_in, a.W0, a.T_out, col_begin, col_end, c.px);
  return launch_kernel(sweep_z_kernel<false>, dim3(grid), dim3(kLineThreads), 0, s, a.pdl, d, a.W1, c.a2, c.b2, a.T_in,
                       a.W0, a.T_out, col_begin, col_end, c.px);
}

cudaError_t launch_copy_layer(const Dims& d, const double* T, int layer, double* dst, cudaStream_t s) {
  copy_layer_kernel<<<blocks(d.nxy(), 256), 256, 0, s>>>(d, T, layer, dst);
  return cudaGetLastError();
}

cudaError_t launch_surface_estimate(int64_t nxy, const double* T, double dz, double* dst, cudaStream_t s) {
  const double dz2 = surface_dz2(dz);
  surface_estimate_kernel<<<blocks(nxy, 256), 256, 0, s>>>(nxy, T, dz2, dst);
  return cudaGetLastError();
}

}  // namespace hs2g
