// Adjoint of the ADI timestep: gradients of a top-surface misfit with respect to per-voxel conductivity k,
// volumetric heat capacity C = rho*c and source amplitude q, for one problem or a batch of independent
// problems of uneven size advanced together (no counterpart in the reference, which has no derivatives).
//
// Model per instance (every voxel computed, exterior faces insulating, interior faces conducting with the
// arithmetic face mean of boundary_conducting, G_f = (k_lo + k_hi) / (2 d^2)), M = C/dt, source s_n * q at
// step n.  The step is the Douglas delta form of the forward path (hs2g_sweep.cu):
//     r0 = L T + s_n q,  A_x y0 = r0,  A_y y1 = M y0,  A_z y2 = M y1,  T' = T + y2,   A_a = M - L_a / 2.
// Loss per instance J = sum_n sum_{top layer k=0} (T_{n+1} - d_n)^2.
// Discrete adjoint of one step, lambda the adjoint of T' (including the misfit gradient at T'):
//     mu2 = A_z^-T lambda,  mu1 = A_y^-T (M mu2),  mu0 = A_x^-T (M mu1),  lambda_T = lambda + L mu0
//     dJ/dG_f (face q|p on axis a, q the lower voxel) += -(mu0_p - mu0_q)(T_p - T_q)
//                                                       - (mu_a,p - mu_a,q)(y_a,p - y_a,q) / 2
//     dJ/dM_p += mu2 y1 + mu1 y0 - mu0 y0 - mu1 y1 - mu2 y2,     dJ/dq_p += s_n mu0_p
// with (mu_a, y_a) = (mu0, y0), (mu1, y1), (mu2, y2) for a = x, y, z (L is symmetric).  A_a = M - L_a/2 is
// symmetric too, so A_a^-T = A_a^-1: the adjoint's line solves are the forward ones, with the same factors.
//
// Memory: T is checkpointed every `ckpt` steps in the forward pass (ceil(nsteps/ckpt) states); the backward
// pass recomputes a segment from its checkpoint, keeping T_n, y0, y1, y2 of each of its steps (4*ckpt states,
// allocated by the first backward pass), then sweeps the segment backwards.
// Concatenated layout: instance i occupies voxels [off_i, off_i + nz*ny*nx) of every field; each kernel covers
// all instances in one launch (lines or voxels of the whole batch, the instance found by binary search).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "hs2g_internal.cuh"

namespace hs2g {
namespace {

constexpr int kTh = 128;

struct AInst {
  int64_t off;              // first voxel
  int64_t nz, ny, nx;
  double idx2, idy2, idz2;  // 1/d^2 per axis
  int64_t obs_off;          // first observation of the instance (nsteps * ny * nx each)
};

struct AView {
  const AInst* inst;
  const int64_t* vox_off;   // ninst + 1 voxel prefix
  const int64_t* line_off;  // 3 * (ninst + 1) line prefixes, axis-major (x, y, z)
  const int64_t* xg_off;    // ninst + 1 prefix of x-line groups (kXL consecutive x-lines of one instance)
  int ninst;
  int64_t nvox;
};

constexpr int kXL = 32;   // x-lines per CTA of the tiled x kernels
constexpr int kXC = 32;   // columns per chunk
constexpr int kXT = 128;  // threads: 4 warps, 8 lines each when loading and storing a chunk

inline unsigned nblk(int64_t n) { return (unsigned)std::max<int64_t>(1, (n + kTh - 1) / kTh); }

// index of the last prefix entry <= v (prefix[0] = 0; instances are non-empty so the prefix increases)
__device__ __forceinline__ int find_inst(const int64_t* prefix, int n, int64_t v) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(prefix + mid) <= v) lo = mid; else hi = mid - 1;
  }
  return lo;
}

struct Line {
  int64_t base, stride, len;
};

// global line t of axis (0 = x, 1 = y, 2 = z) -> first voxel, stride, length
__device__ __forceinline__ Line line_at(const AView& v, int axis, int64_t t) {
  const int64_t* pre = v.line_off + axis * (v.ninst + 1);
  const int i = find_inst(pre, v.ninst, t);
  const AInst& in = v.inst[i];
  const int64_t l = t - pre[i], nxy = in.ny * in.nx;
  if (axis == 0) return Line{in.off + l * in.nx, 1, in.nx};
  if (axis == 1) return Line{in.off + (l / in.nx) * nxy + l % in.nx, in.nx, in.ny};
  return Line{in.off + l, nxy, in.nz};
}

struct Vox {
  int64_t i, j, k, nx, ny, nz, nxy;
  int inst;
};
// voxel p -> instance and (k, j, i); 32-bit divisions (hs2g_adjoint_create refuses batches of 2^31 voxels)
__device__ __forceinline__ Vox vox_at(const AView& v, int64_t p) {
  const int n = find_inst(v.vox_off, v.ninst, p);
  const AInst& in = v.inst[n];
  const uint32_t l = (uint32_t)(p - in.off), nx = (uint32_t)in.nx, ny = (uint32_t)in.ny;
  const uint32_t row = l / nx, k = row / ny;
  Vox r;
  r.inst = n;
  r.nx = in.nx; r.ny = in.ny; r.nz = in.nz; r.nxy = in.nx * in.ny;
  r.i = l - row * nx; r.j = row - k * ny; r.k = k;
  return r;
}

// per-voxel low-face conductances of each axis from k (zero on the exterior), M = C / dt
__global__ void adj_setup_kernel(AView v, const double* __restrict__ k, const double* __restrict__ C, double inv_dt,
                                 double* __restrict__ gx, double* __restrict__ gy, double* __restrict__ gz,
                                 double* __restrict__ M) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= v.nvox) return;
  const Vox x = vox_at(v, p);
  const AInst& in = v.inst[x.inst];
  const double kp = k[p];
  gx[p] = x.i > 0 ? 0.5 * (k[p - 1] + kp) * in.idx2 : 0.0;
  gy[p] = x.j > 0 ? 0.5 * (k[p - x.nx] + kp) * in.idy2 : 0.0;
  gz[p] = x.k > 0 ? 0.5 * (k[p - x.nxy] + kp) * in.idz2 : 0.0;
  M[p] = C[p] * inv_dt;
}

// A fixed-temperature voxel gets this capacity: its row of every stage matrix is then M times the identity to
// within 1e-290, its increments vanish against T, and the stage matrices stay symmetric (the reference's
// identity rows with couplings from computed neighbours are not), so the adjoint's transposed solves remain
// the forward solves.
constexpr double kFixedCapacity = 1e300;

// The same with face classes and fixed voxels: the conductance of a face of class c on axis a is the class's
// affine form f0 + flo k_lo + fhi k_hi, the k of a fixed side replaced by its computed neighbour's
// (crank_nicolson.pyx:298-338); a face between two fixed voxels conducts nothing.  A class index past the
// table records an error.
__global__ void adj_setup_faces_kernel(AView v, const double* __restrict__ k, const double* __restrict__ C,
                                       double inv_dt, const uint8_t* __restrict__ fcls, int nclass,
                                       const double* __restrict__ forms, const uint8_t* __restrict__ fixed,
                                       double* __restrict__ gx, double* __restrict__ gy, double* __restrict__ gz,
                                       double* __restrict__ M, int* __restrict__ err) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= v.nvox) return;
  const Vox x = vox_at(v, p);
  const bool fp = fixed && fixed[p];
  M[p] = fp ? kFixedCapacity : C[p] * inv_dt;
  double* out[3] = {gz, gy, gx};
  const bool has_low[3] = {x.k > 0, x.j > 0, x.i > 0};
  const int64_t step[3] = {x.nxy, x.nx, 1};
  for (int a = 0; a < 3; ++a) {
    double G = 0.0;
    if (has_low[a]) {
      const int64_t q = p - step[a];
      const bool fq = fixed && fixed[q];
      const int c = fcls[a * v.nvox + p];
      if (c >= nclass) {
        atomicExch(err, 1);
      } else if (!(fp && fq)) {
        const double* f = forms + ((int64_t)(x.inst * nclass + c) * 3 + a) * 3;
        const double klo = fq ? k[p] : k[q], khi = fp ? k[q] : k[p];
        G = fma(f[2], khi, fma(f[1], klo, f[0]));
      }
    }
    out[a][p] = G;
  }
}

// D = the sum of a voxel's six face conductances (the diagonal of -L)
__global__ void adj_diag_kernel(AView v, const double* __restrict__ gx, const double* __restrict__ gy,
                                const double* __restrict__ gz, double* __restrict__ D) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= v.nvox) return;
  const Vox x = vox_at(v, p);
  double d = gx[p] + gy[p] + gz[p];
  if (x.i + 1 < x.nx) d += gx[p + 1];
  if (x.j + 1 < x.ny) d += gy[p + x.nx];
  if (x.k + 1 < x.nz) d += gz[p + x.nxy];
  D[p] = d;
}

// factors of A_a = M - L_a/2 per line, kept in the form the one-FMA-per-row recurrences of the solves use:
// e = lo / piv (lo the sub-diagonal), u = (super-diagonal) / piv, ip = 1 / piv, mip = M / piv (the scale of
// the stages whose right-hand side is M rhs)
__global__ void adj_factor_kernel(AView v, int axis, int64_t nlines, const double* __restrict__ M,
                                  const double* __restrict__ g, double* __restrict__ e, double* __restrict__ u,
                                  double* __restrict__ ip, double* __restrict__ mip) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nlines) return;
  const Line ln = line_at(v, axis, t);
  double u_prev = 0.0;
  for (int64_t r = 0; r < ln.len; ++r) {
    const int64_t p = ln.base + r * ln.stride;
    const double gl = g[p];
    const double gh = r + 1 < ln.len ? g[p + ln.stride] : 0.0;
    const double l = -(0.5 * gl);
    const double piv = M[p] + 0.5 * (gl + gh) - u_prev * l;
    const double uu = -(0.5 * gh) / piv;
    const double inv = 1.0 / piv;
    e[p] = l * inv;
    u[p] = uu;
    ip[p] = inv;
    mip[p] = __dmul_rn(M[p], inv);
    u_prev = uu;
  }
}

// Every line solve below is y = A_a^-1 b with A_a = Lo U (Lo: pivots on the diagonal, lo below; U: unit
// diagonal, u above) in two passes of one dependent FMA per row:
//     z_r = fma(-e_r, z_{r-1}, c_r),  c_r = rhs_r * s_r       (rows ascending)
//     y_r = fma(-u_r, y_{r+1}, z_r)                           (rows descending)
// with b = M rhs and s = mip = M / piv for the stages weighted by M (one multiplication per row instead of
// two), b = rhs and s = ip = 1 / piv otherwise (the residual r0 in the forward x stage, lambda in the first
// adjoint stage).  The rounding of every operation is explicit (no contraction left to the compiler), so the
// register-blocked kernels for many lines and the shared-memory few-line kernels give the same bits.

// The x-line kernels below stage 32 lines x 32 columns of each operand through shared memory: loads and
// stores are row-contiguous (lane = column), the recurrence runs one line per lane of warp 0 (lane = line).
// CTA b covers the x-lines [l0, l0 + nl) of one instance, a contiguous (nl, nx) block of every field.
struct XGroup {
  int64_t off, l0, nl, nx, ny, nz;
};
__device__ __forceinline__ XGroup xgroup(const AView& v, int64_t b) {
  const int i = find_inst(v.xg_off, v.ninst, b);
  const AInst& in = v.inst[i];
  XGroup g;
  g.off = in.off;
  g.nx = in.nx;
  g.ny = in.ny;
  g.nz = in.nz;
  g.l0 = (b - v.xg_off[i]) * kXL;
  g.nl = min((int64_t)kXL, in.nz * in.ny - g.l0);
  return g;
}

// r0 = s q - D T_p + sum over faces of G T_nbr at voxel p = (k, j, i) of an (nz, ny, nx) instance (D = the sum
// of the six G): 8 FP64 operations against 13 for the face-by-face differences; temperatures are offsets
// from their initial mean, so the cancellation in -D T_p + sum G T_nbr stays at the rounding of the increments
__device__ __forceinline__ double residual_at(const double* __restrict__ T, const double* __restrict__ gx,
                                              const double* __restrict__ gy, const double* __restrict__ gz,
                                              const double* __restrict__ D, const double* __restrict__ q, double s,
                                              int64_t p, int64_t i, int64_t j, int64_t k, int64_t nx, int64_t ny,
                                              int64_t nz) {
  const int64_t nxy = nx * ny;
  double r = __fma_rn(-D[p], T[p], __dmul_rn(s, q[p]));
  if (i > 0) r = __fma_rn(gx[p], T[p - 1], r);
  if (i + 1 < nx) r = __fma_rn(gx[p + 1], T[p + 1], r);
  if (j > 0) r = __fma_rn(gy[p], T[p - nx], r);
  if (j + 1 < ny) r = __fma_rn(gy[p + nx], T[p + nx], r);
  if (k > 0) r = __fma_rn(gz[p], T[p - nxy], r);
  if (k + 1 < nz) r = __fma_rn(gz[p + nxy], T[p + nxy], r);
  return r;
}

// x stage: y = A_x^-1 b.  RESID: b = the residual r0 = L T + s q (the forward step's first stage, fused),
// scale = ip; otherwise b = M rhs (the adjoint's last stage, mu0 = A_x^-1 (M mu1)), scale = mip.
template <bool RESID>
__global__ void __launch_bounds__(kXT) adj_xsolve_kernel(AView v, const double* __restrict__ T,
                                                         const double* __restrict__ gx, const double* __restrict__ gy,
                                                         const double* __restrict__ gz, const double* __restrict__ D,
                                                         const double* __restrict__ q, double s,
                                                         const double* __restrict__ rhs, const double* __restrict__ e,
                                                         const double* __restrict__ u,
                                                         const double* __restrict__ scale, double* __restrict__ y) {
  wait_prior_grid();  // the previous kernel on the stream (programmatic dependent launch)
  __shared__ double sc[kXL][kXC + 1], se[kXL][kXC + 1];
  const XGroup g = xgroup(v, blockIdx.x);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int kPer = kXL / (kXT / 32);
  const int nch = (int)((g.nx + kXC - 1) / kXC);
  double carry = 0.0;
  for (int ch = 0; ch < nch; ++ch) {
    const int64_t i = (int64_t)ch * kXC + lane;
    // four lines' loads in flight per warp (64 registers): the 32-instance adjoint batch at 14.3 gradient
    // evaluations/s against 13.9 with two and 13.8 with eight
#pragma unroll 4
    for (int ll = 0; ll < kPer; ++ll) {
      const int l = warp * kPer + ll;
      if (l < g.nl && i < g.nx) {
        const int64_t line = g.l0 + l;
        const int64_t p = g.off + line * g.nx + i;
        const double b =
            RESID ? residual_at(T, gx, gy, gz, D, q, s, p, i, line % g.ny, line / g.ny, g.nx, g.ny, g.nz) : rhs[p];
        sc[l][lane] = __dmul_rn(b, scale[p]);
        se[l][lane] = e[p];
      }
    }
    __syncthreads();
    if (warp == 0 && lane < g.nl) {
      const int cw = (int)min((int64_t)kXC, g.nx - (int64_t)ch * kXC);
      double z = carry;
      for (int cc = 0; cc < cw; ++cc) {
        z = __fma_rn(-se[lane][cc], z, sc[lane][cc]);
        sc[lane][cc] = z;
      }
      carry = z;
    }
    __syncthreads();
    for (int ll = 0; ll < kPer; ++ll) {
      const int l = warp * kPer + ll;
      if (l < g.nl && i < g.nx) y[g.off + (g.l0 + l) * g.nx + i] = sc[l][lane];
    }
    __syncthreads();
  }
  carry = 0.0;
  for (int ch = nch - 1; ch >= 0; --ch) {
    const int64_t i = (int64_t)ch * kXC + lane;
    for (int ll = 0; ll < kPer; ++ll) {
      const int l = warp * kPer + ll;
      if (l < g.nl && i < g.nx) {
        const int64_t p = g.off + (g.l0 + l) * g.nx + i;
        sc[l][lane] = y[p];
        se[l][lane] = u[p];
      }
    }
    __syncthreads();
    if (warp == 0 && lane < g.nl) {
      const int cw = (int)min((int64_t)kXC, g.nx - (int64_t)ch * kXC);
      double x = carry;
      for (int cc = cw - 1; cc >= 0; --cc) {
        x = __fma_rn(-se[lane][cc], x, sc[lane][cc]);
        sc[lane][cc] = x;
      }
      carry = x;
    }
    __syncthreads();
    for (int ll = 0; ll < kPer; ++ll) {
      const int l = warp * kPer + ll;
      if (l < g.nl && i < g.nx) y[g.off + (g.l0 + l) * g.nx + i] = sc[l][lane];
    }
    __syncthreads();
  }
}

// y / z stage: y = A_a^-1 b along each strided line, c_r = rhs_r * scale_r (scale = mip for b = M rhs, ip for
// b = rhs), one thread per line,
// neighbouring threads on neighbouring lines, so every row access is coalesced; T_out = T_in + y when T_out
// is given (T_out may equal T_in).  Rows go in blocks of kRB: the loads of a block are issued together, then
// the recurrence runs through it, so a line pays one memory latency per block instead of one per row.
// Occupancy matters more than rows in flight: with 32-bit offsets, 4-row blocks at 12 CTAs per SM fit in 40
// registers without spilling, and the 32-instance adjoint batch runs 16.8 gradient evaluations/s against
// 14.3 with 8-row blocks at 4 CTAs per SM (128 registers, 64-bit offsets) and 15.3-16.4 for the other
// combinations of 2-8 rows and 8-16 CTAs per SM.
constexpr int kRB = 4;
constexpr int kYMinBlocks = 12;

template <bool ADD_T>
__global__ void __launch_bounds__(128, kYMinBlocks) adj_ysolve_kernel(AView v, int axis, int64_t nlines,
                                                                      const double* rhs,
                                                                      const double* __restrict__ e,
                                                                      const double* __restrict__ u,
                                                                      const double* __restrict__ scale, double* y,
                                                                      const double* T_in, double* T_out) {
  wait_prior_grid();  // the previous kernel on the stream (programmatic dependent launch)
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nlines) return;
  const Line ln = line_at(v, axis, t);
  // voxel offsets in 32 bits (hs2g_adjoint_create refuses batches of 2^31 voxels or more), walked row by row
  const uint32_t stride = (uint32_t)ln.stride;
  const int len = (int)ln.len;
  double z = 0.0;
  uint32_t o = (uint32_t)ln.base;  // row r0
  for (int r0 = 0; r0 < len; r0 += kRB, o += kRB * stride) {
    double c[kRB], ee[kRB];
#pragma unroll
    for (int k = 0; k < kRB; ++k) {
      if (r0 + k < len) {
        const uint32_t p = o + k * stride;
        c[k] = __dmul_rn(rhs[p], scale[p]);
        ee[k] = e[p];
      }
    }
#pragma unroll
    for (int k = 0; k < kRB; ++k) {
      if (r0 + k < len) {
        z = __fma_rn(-ee[k], z, c[k]);
        y[o + k * stride] = z;
      }
    }
  }
  double x = 0.0;
  o = (uint32_t)ln.base + (uint32_t)(len - 1) * stride;  // row r1
  for (int r1 = len - 1; r1 >= 0; r1 -= kRB, o -= kRB * stride) {
    double yy[kRB], uu[kRB], tt[kRB] = {};
#pragma unroll
    for (int k = 0; k < kRB; ++k) {
      if (r1 - k >= 0) {
        const uint32_t p = o - k * stride;
        yy[k] = y[p];
        uu[k] = u[p];
        if (ADD_T) tt[k] = T_in[p];
      }
    }
#pragma unroll
    for (int k = 0; k < kRB; ++k) {
      if (r1 - k >= 0) {
        const uint32_t p = o - k * stride;
        x = __fma_rn(-uu[k], x, yy[k]);
        y[p] = x;
        if (ADD_T) T_out[p] = __dadd_rn(tt[k], x);
      }
    }
  }
}

// Few-line form of adj_ysolve_kernel.  A small problem (4096 y-lines of 128 rows at 32x128x128) leaves each
// SM about one warp, whose line is then a chain of memory round trips, one per block of rows.  Here the rows
// of a CTA's 32 lines stream through a ring of kFS stages of kFR rows with cp.async, and the first pass's
// values of the whole line stay in shared memory for the second pass.  Same operations, same order, same
// rounding as adj_ysolve_kernel.
// What bounds it is the recurrence warp's own instruction stream (about 6 cycles per instruction with
// nothing to interleave), not memory: at 32x128x128 the 128-row y solve took 38 us with one warp issuing both
// the copies and the recurrence, 26 us with the copies left out (a timing probe) and takes 31 us with the
// copies on a second warp (a third warp sharing the copies: unchanged).  Eight ring stages or 16-row stages
// were slower, staging each block's operands in registers changed nothing, and spreading the lines over four
// 8-lane warps doubled the z time.
constexpr int kFS = 4;            // ring stages
constexpr int kFR = 8;            // rows per stage
constexpr int kFewMaxLen = 512;   // longest line the few-line kernels hold (128 KB of line values)

__device__ __forceinline__ void cp_async8(double* dst, const double* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// dynamic shared memory of a few-line launch: the line values, then the ring (room for 4 operands, 3 used)
inline size_t few_smem_bytes(int64_t max_len) {
  return sizeof(double) * 32 * (size_t)(max_len + kFS * kFR * 4);
}

// slot of operand a of row k of block g in the ring (block g in slot g % kFS)
struct FewRing {
  double* ring;
  int lane;
  __device__ __forceinline__ double* at(int g, int k, int a) const {
    return ring + (((g % kFS) * kFR + k) * 4 + a) * 32 + lane;
  }
};

__device__ __forceinline__ void named_bar_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(id), "r"(nthreads) : "memory");
}
__device__ __forceinline__ void named_bar_arrive(int id, int nthreads) {
  asm volatile("bar.arrive %0, %1;\n" ::"r"(id), "r"(nthreads) : "memory");
}

// Two warps per CTA over the same 32 lines (lane = line): warp 1 issues the copies and forms each forward row's
// scaled right-hand side c = rhs * scale once the row has landed, warp 0 runs the recurrence.  A warp issues
// one FP64 instruction per 64 cycles on GB300 (the measured latency of a dependent FMA is the same 64 cycles),
// so the multiplications that do not depend on the recurrence run on the copying warp's sub-partition while the
// recurrence warp issues only its chained FMAs.  Ring slot s is handed over with named barriers, FULL(s) = 1 + s
// from producer to consumer once the slot's copies have landed and its c values are written, EMPTY(s) =
// 1 + kFS + s back once it is consumed.  Both warps count the blocks of the two passes as one sequence
// q = 0 .. 2 nb - 1 (nb = blocks of the CTA's longest line), slot q % kFS, and run the same barrier sequence
// whatever their lines' lengths, so every barrier is met.
constexpr int kFewLag = 2;  // blocks the producer keeps in flight before handing the oldest over

template <bool ADD_T>
__global__ void __launch_bounds__(64) adj_ysolve_few_kernel(AView v, int axis, int64_t nlines, int64_t max_len,
                                                            const double* rhs, const double* __restrict__ e,
                                                            const double* __restrict__ u,
                                                            const double* __restrict__ scale, double* y,
                                                            const double* T_in, double* T_out) {
  wait_prior_grid();  // the previous kernel on the stream (programmatic dependent launch)
  extern __shared__ double few_sm[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t t = blockIdx.x * (int64_t)32 + lane;
  const Line ln = t < nlines ? line_at(v, axis, t) : Line{0, 0, 0};
  double* line = few_sm;  // line[r * 32 + lane]
  const FewRing R{few_sm + 32 * max_len, lane};
  const int len = (int)ln.len;
  const int nb = __reduce_max_sync(0xffffffffu, (len + kFR - 1) / kFR), nq = 2 * nb;
  if (warp == 1) {
    // producer: block q < nb is rows [q kFR, q kFR + kFR) ascending (rhs, e, scale; rhs replaced by c once
    // landed), block q >= nb rows len - 1 - (q - nb) kFR - k descending (u, T_in)
    auto hand_over = [&](int qq) {  // block qq has landed (this thread's copies): form c, then release the slot
      if (qq < nb) {
#pragma unroll
        for (int k = 0; k < kFR; ++k)
          if (qq * kFR + k < len) *R.at(qq, k, 0) = __dmul_rn(*R.at(qq, k, 0), *R.at(qq, k, 2));
      }
      __threadfence_block();
      named_bar_arrive(1 + qq % kFS, 64);
    };
    for (int q = 0; q < nq; ++q) {
      if (q >= kFS) named_bar_sync(1 + kFS + q % kFS, 64);  // the consumer is done with block q - kFS
#pragma unroll
      for (int k = 0; k < kFR; ++k) {
        if (q < nb) {
          const int r = q * kFR + k;
          if (r < len) {
            const int64_t p = ln.base + r * ln.stride;
            cp_async8(R.at(q, k, 0), rhs + p);
            cp_async8(R.at(q, k, 1), e + p);
            cp_async8(R.at(q, k, 2), scale + p);
          }
        } else {
          const int r = len - 1 - ((q - nb) * kFR + k);
          if (r >= 0) {
            const int64_t p = ln.base + r * ln.stride;
            cp_async8(R.at(q, k, 0), u + p);
            if (ADD_T) cp_async8(R.at(q, k, 1), T_in + p);
          }
        }
      }
      cp_async_commit();
      if (q >= kFewLag) {
        cp_async_wait<kFewLag>();  // block q - kFewLag has landed
        hand_over(q - kFewLag);
      }
    }
    cp_async_wait<0>();
    for (int q = nq > kFewLag ? nq - kFewLag : 0; q < nq; ++q) hand_over(q);
    return;
  }
  double z = 0.0, x = 0.0;
  for (int q = 0; q < nq; ++q) {
    named_bar_sync(1 + q % kFS, 64);
    if (q < nb) {
      double ce[kFR], cc[kFR];  // the block's operands in registers before the chain (no wait behind its stores)
#pragma unroll
      for (int k = 0; k < kFR; ++k) {
        ce[k] = *R.at(q, k, 1);
        cc[k] = *R.at(q, k, 0);
      }
#pragma unroll
      for (int k = 0; k < kFR; ++k) {
        const int r = q * kFR + k;
        if (r < len) {
          z = __fma_rn(-ce[k], z, cc[k]);
          line[r * 32 + lane] = z;
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < kFR; ++k) {
        const int r = len - 1 - ((q - nb) * kFR + k);
        if (r >= 0) {
          const int64_t p = ln.base + r * ln.stride;
          x = __fma_rn(-*R.at(q, k, 0), x, line[r * 32 + lane]);
          y[p] = x;
          if (ADD_T) T_out[p] = __dadd_rn(*R.at(q, k, 1), x);
        }
      }
    }
    if (q + kFS < nq) named_bar_arrive(1 + kFS + q % kFS, 64);
  }
}

// Few-line form of adj_xsolve_kernel.  A 32-line group of a small problem is a latency chain in the fused
// kernel (four dependent load rounds per 32-column chunk); here each of four warps streams the chunks of
// kFewLanes of the group's lines through a ring of kXFS tiles with cp.async (lane = column, row-contiguous
// copies), recurs with lane = line while the next two chunks are in flight, keeps the whole lines in shared
// memory between the two passes and stores them once, row-contiguous.  The forward stage's residual r0 comes
// from adj_resid_kernel (one thread per voxel) instead of being fused.  Same operations, same order, same
// rounding as adj_xsolve_kernel.
constexpr int kXFS = 3;              // ring stages (tiles of kXL lines x kXC columns x 3 operands)
constexpr int kFewLanes = 8;         // lines per warp (four warps per group: the copies spread over them)
constexpr int kFewXGroups = 2 * 152; // at most this many 32-line groups
constexpr int kFewMaxNx = 448;       // longest x-line the few-line kernel holds (187 KB of shared memory)

inline size_t few_x_smem_bytes(int64_t max_nx, int nops) {
  return sizeof(double) * ((size_t)kXL * (size_t)(max_nx + 1) + (size_t)kXFS * nops * kXL * (kXC + 1));
}

__global__ void adj_resid_kernel(AView v, const double* __restrict__ T, const double* __restrict__ gx,
                                 const double* __restrict__ gy, const double* __restrict__ gz,
                                 const double* __restrict__ D, const double* __restrict__ q, double s,
                                 double* __restrict__ r0) {
  wait_prior_grid();  // the previous kernel on the stream (programmatic dependent launch)
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= v.nvox) return;
  const Vox x = vox_at(v, p);
  r0[p] = residual_at(T, gx, gy, gz, D, q, s, p, x.i, x.j, x.k, x.nx, x.ny, x.nz);
}

// the group's line buffer and tiles in dynamic shared memory: lines[l * (max_nx + 1) + c], then the ring of
// kXFS slots of nops operand tiles
struct FewX {
  double* lines;
  double* ring;
  int64_t zs;
  int nops;
  __device__ __forceinline__ double* tile(int seq, int a, int l) const {
    return ring + (((seq % kXFS) * nops + a) * kXL + l) * (kXC + 1);
  }
};

// copies columns [ch * kXC, ch * kXC + kXC) of the group's lines [l_begin, l_end) of the given operands (null
// ones skipped) into ring slot seq % kXFS (nothing when ch is outside the line); always commits a group
__device__ __forceinline__ void few_x_issue(const FewX& F, const XGroup& g, int seq, int ch, int lane, int l_begin,
                                            int l_end, const double* a0, const double* a1, const double* a2,
                                            const double* a3) {
  const int64_t c = (int64_t)ch * kXC + lane;
  if (ch >= 0 && c < g.nx) {
    const int64_t row0 = g.off + g.l0 * g.nx + c;
    for (int l = l_begin; l < l_end; ++l) {
      const int64_t p = row0 + (int64_t)l * g.nx;
      cp_async8(F.tile(seq, 0, l) + lane, a0 + p);
      if (a1) cp_async8(F.tile(seq, 1, l) + lane, a1 + p);
      if (a2) cp_async8(F.tile(seq, 2, l) + lane, a2 + p);
      if (a3) cp_async8(F.tile(seq, 3, l) + lane, a3 + p);
    }
  }
  cp_async_commit();
}

// y = A_x^-1 b with c = rhs * scale: scale = mip for b = M rhs (the adjoint's last stage), ip for b = rhs (the
// forward stage's residual r0; rhs may alias y)
__global__ void __launch_bounds__(128) adj_xsolve_few_kernel(AView v, int64_t max_nx, const double* rhs,
                                                             const double* __restrict__ e,
                                                             const double* __restrict__ u,
                                                             const double* __restrict__ scale, double* y) {
  wait_prior_grid();  // the previous kernel on the stream (programmatic dependent launch)
  extern __shared__ double few_sm[];
  const XGroup g = xgroup(v, blockIdx.x);
  // warp w solves the group's lines [lb, le): it copies them with lane = column and recurs with lane = line
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int lb = min(warp * kFewLanes, (int)g.nl), le = min(lb + kFewLanes, (int)g.nl), ln = lb + lane;
  const FewX F{few_sm, few_sm + kXL * (max_nx + 1), max_nx + 1, 3};
  const int nch = (int)((g.nx + kXC - 1) / kXC);
  for (int q = 0; q < kXFS - 1; ++q) few_x_issue(F, g, q, q < nch ? q : -1, lane, lb, le, rhs, e, scale, nullptr);
  double z = 0.0;
  for (int ch = 0; ch < nch; ++ch) {
    __syncwarp();  // every lane is done with the slot refilled here
    const int nxt = ch + kXFS - 1;
    few_x_issue(F, g, nxt, nxt < nch ? nxt : -1, lane, lb, le, rhs, e, scale, nullptr);
    cp_async_wait<kXFS - 1>();
    __syncwarp();  // chunk ch's copies by every lane are visible
    // c = rhs * scale with lane = column, one multiplication per 32 columns, before the recurrence (lane = line,
    // kFewLanes lines per warp) runs its chained FMAs alone
    if ((int64_t)ch * kXC + lane < g.nx)
      for (int l = lb; l < le; ++l) {
        double* tb = F.tile(ch, 0, l) + lane;
        *tb = __dmul_rn(*tb, F.tile(ch, 2, l)[lane]);
      }
    __syncwarp();
    if (ln < le) {
      const int cw = (int)min((int64_t)kXC, g.nx - (int64_t)ch * kXC);
      const double *tc = F.tile(ch, 0, ln), *te = F.tile(ch, 1, ln);
      double* zr = F.lines + ln * F.zs + ch * kXC;
      auto step = [&](int cc) {
        z = __fma_rn(-te[cc], z, tc[cc]);
        zr[cc] = z;
      };
      if (cw == kXC) {
        // eight columns' operands in registers before their part of the chain (the loads do not wait behind the
        // chain's stores to the line buffer)
#pragma unroll
        for (int c0 = 0; c0 < kXC; c0 += 8) {
          double ee[8], c8[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            ee[u] = te[c0 + u];
            c8[u] = tc[c0 + u];
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            z = __fma_rn(-ee[u], z, c8[u]);
            zr[c0 + u] = z;
          }
        }
      } else {
        for (int cc = 0; cc < cw; ++cc) step(cc);
      }
    }
  }
  __syncwarp();
  for (int q = 0; q < kXFS - 1; ++q)
    few_x_issue(F, g, q, nch - 1 - q, lane, lb, le, u, nullptr, nullptr, nullptr);
  double x = 0.0;
  for (int q = 0; q < nch; ++q) {
    __syncwarp();
    few_x_issue(F, g, q + kXFS - 1, nch - kXFS - q, lane, lb, le, u, nullptr, nullptr, nullptr);
    cp_async_wait<kXFS - 1>();
    __syncwarp();
    const int ch = nch - 1 - q;
    if (ln < le) {
      const int cw = (int)min((int64_t)kXC, g.nx - (int64_t)ch * kXC);
      const double* tu = F.tile(q, 0, ln);
      double* zr = F.lines + ln * F.zs + ch * kXC;
      auto step = [&](int cc) {
        x = __fma_rn(-tu[cc], x, zr[cc]);
        zr[cc] = x;
      };
      if (cw == kXC) {
#pragma unroll
        for (int c1 = kXC - 1; c1 >= 0; c1 -= 8) {  // eight columns' operands in registers first
          double u8[8], z8[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            u8[u] = tu[c1 - u];
            z8[u] = zr[c1 - u];
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            x = __fma_rn(-u8[u], x, z8[u]);
            zr[c1 - u] = x;
          }
        }
      } else {
        for (int cc = cw - 1; cc >= 0; --cc) step(cc);
      }
    }
  }
  __syncwarp();
  for (int l = lb; l < le; ++l)
    for (int64_t c = lane; c < g.nx; c += 32) y[g.off + (g.l0 + l) * g.nx + c] = F.lines[l * F.zs + c];
}

// lambda = misfit gradient of the last observation, 2 (T_N - d_{N-1}) on the top layer, 0 below
__global__ void adj_seed_kernel(AView v, const double* __restrict__ T, const double* __restrict__ obs,
                                int64_t obs_step, double* __restrict__ lam) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= v.nvox) return;
  const Vox x = vox_at(v, p);
  const AInst& in = v.inst[x.inst];
  lam[p] = x.k == 0 ? 2.0 * (T[p] - obs[in.obs_off + obs_step * x.nxy + (p - in.off)]) : 0.0;
}

// lambda += L mu0 (+ the misfit gradient of observation obs_step, at T_n, when obs_step >= 0), and the
// gradient accumulation of one step; one thread per voxel, each voxel owning its three low faces
__global__ void adj_update_kernel(AView v, const double* __restrict__ gx, const double* __restrict__ gy,
                                  const double* __restrict__ gz, const double* __restrict__ T,
                                  const double* __restrict__ y0, const double* __restrict__ y1,
                                  const double* __restrict__ y2, const double* __restrict__ mu0,
                                  const double* __restrict__ mu1, const double* __restrict__ mu2, double s,
                                  const double* __restrict__ obs, int64_t obs_step, double* __restrict__ lam,
                                  double* __restrict__ ggx, double* __restrict__ ggy, double* __restrict__ ggz,
                                  double* __restrict__ gM, double* __restrict__ gq) {
  wait_prior_grid();  // the previous kernel on the stream (programmatic dependent launch)
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= v.nvox) return;
  const Vox x = vox_at(v, p);
  const double m0 = mu0[p], Tp = T[p];
  const double m1 = mu1[p], m2 = mu2[p];
  const double a0 = y0[p], a1 = y1[p], a2 = y2[p];
  // each low-face difference of mu0 serves both lambda's update (L mu0) and that face's gradient
  double l = lam[p];
  if (x.i > 0) {
    const int64_t q = p - 1;
    const double d0 = m0 - mu0[q];
    l = fma(-gx[p], d0, l);
    ggx[p] = fma(-d0, fma(0.5, a0 - y0[q], Tp - T[q]), ggx[p]);
  }
  if (x.j > 0) {
    const int64_t q = p - x.nx;
    const double d0 = m0 - mu0[q];
    l = fma(-gy[p], d0, l);
    ggy[p] = fma(-0.5 * (m1 - mu1[q]), a1 - y1[q], fma(-d0, Tp - T[q], ggy[p]));
  }
  if (x.k > 0) {
    const int64_t q = p - x.nxy;
    const double d0 = m0 - mu0[q];
    l = fma(-gz[p], d0, l);
    ggz[p] = fma(-0.5 * (m2 - mu2[q]), a2 - y2[q], fma(-d0, Tp - T[q], ggz[p]));
  }
  if (x.i + 1 < x.nx) l = fma(gx[p + 1], mu0[p + 1] - m0, l);
  if (x.j + 1 < x.ny) l = fma(gy[p + x.nx], mu0[p + x.nx] - m0, l);
  if (x.k + 1 < x.nz) l = fma(gz[p + x.nxy], mu0[p + x.nxy] - m0, l);
  if (obs_step >= 0 && x.k == 0) {
    const AInst& in = v.inst[x.inst];
    l += 2.0 * (Tp - obs[in.obs_off + obs_step * x.nxy + (p - in.off)]);
  }
  lam[p] = l;
  // mu2 y1 + mu1 y0 - mu0 y0 - mu1 y1 - mu2 y2 = mu2 (y1 - y2) + mu1 (y0 - y1) - mu0 y0
  gM[p] = fma(m2, a1 - a2, fma(m1, a0 - a1, fma(-m0, a0, gM[p])));
  gq[p] = fma(s, m0, gq[p]);
}

// s + v as an unevaluated pair: returns the rounded sum, err receives its exact rounding error (Knuth's TwoSum)
__device__ __forceinline__ double two_sum(double s, double v, double& err) {
  const double t = s + v;
  const double bp = t - s;
  err = (s - (t - bp)) + (v - bp);
  return t;
}

// misfit of step `step`, as compensated pairs: block (c, i) sums (T - obs)^2 over its slice of instance i's
// top layer with per-thread Neumaier sums and a TwoSum tree (256 threads, fixed order) and writes
// part[2*((step*ninst + i)*kMisfitBlocks + c)] and the next entry (rounded sum, error); summing the pairs
// exactly on the host leaves the loss with no summation error that would swamp the small loss differences
// finite-difference checks take
constexpr int kMisfitBlocks = 32;
__global__ void adj_misfit_kernel(AView v, const double* __restrict__ T, const double* __restrict__ obs,
                                  int64_t step, double* __restrict__ part) {
  wait_prior_grid();  // the previous kernel on the stream (programmatic dependent launch)
  __shared__ double sh_hi[256], sh_lo[256];
  const AInst& in = v.inst[blockIdx.y];
  const int64_t m = in.ny * in.nx;
  const double* o = obs + in.obs_off + step * m;
  const double* t = T + in.off;
  double hi = 0.0, lo = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < m; e += (int64_t)gridDim.x * blockDim.x) {
    const double r = t[e] - o[e];
    const double sq = r * r;
    double err;
    hi = two_sum(hi, sq, err);
    lo += err + fma(r, r, -sq);  // the square's own rounding error, exactly
  }
  sh_hi[threadIdx.x] = hi;
  sh_lo[threadIdx.x] = lo;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      double err;
      const double s2 = two_sum(sh_hi[threadIdx.x], sh_hi[threadIdx.x + w], err);
      sh_lo[threadIdx.x] += sh_lo[threadIdx.x + w] + err;
      sh_hi[threadIdx.x] = s2;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const int64_t at = 2 * ((step * v.ninst + blockIdx.y) * kMisfitBlocks + blockIdx.x);
    part[at] = sh_hi[0];
    part[at + 1] = sh_lo[0];
  }
}

// chain to the parameters: gk from the face gradients (G = (k_lo + k_hi) / (2 d^2)), gC = gM / dt
__global__ void adj_chain_kernel(AView v, const double* __restrict__ ggx, const double* __restrict__ ggy,
                                 const double* __restrict__ ggz, const double* __restrict__ gM, double inv_dt,
                                 double* __restrict__ gk, double* __restrict__ gC) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= v.nvox) return;
  const Vox x = vox_at(v, p);
  const AInst& in = v.inst[x.inst];
  double fx = 0.0, fy = 0.0, fz = 0.0;
  if (x.i > 0) fx += ggx[p];
  if (x.i + 1 < x.nx) fx += ggx[p + 1];
  if (x.j > 0) fy += ggy[p];
  if (x.j + 1 < x.ny) fy += ggy[p + x.nx];
  if (x.k > 0) fz += ggz[p];
  if (x.k + 1 < x.nz) fz += ggz[p + x.nxy];
  gk[p] = 0.5 * (in.idx2 * fx + in.idy2 * fy + in.idz2 * fz);
  gC[p] = gM[p] * inv_dt;
}

// The chain with face classes: d G_f / d k of each side from the face's affine form (both coefficients to the
// computed side of a face with a fixed neighbour); no gradient for fixed voxels' k, C and q.
__global__ void adj_chain_faces_kernel(AView v, const double* __restrict__ ggx, const double* __restrict__ ggy,
                                       const double* __restrict__ ggz, const double* __restrict__ gM, double inv_dt,
                                       const uint8_t* __restrict__ fcls, int nclass, const double* __restrict__ forms,
                                       const uint8_t* __restrict__ fixed, double* __restrict__ gk,
                                       double* __restrict__ gC, double* __restrict__ gq) {
  const int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (p >= v.nvox) return;
  const Vox x = vox_at(v, p);
  const bool fp = fixed && fixed[p];
  if (fp) {
    gk[p] = 0.0;
    gC[p] = 0.0;
    gq[p] = 0.0;
    return;
  }
  const double* gg[3] = {ggz, ggy, ggx};
  const int64_t coord[3] = {x.k, x.j, x.i}, len[3] = {x.nz, x.ny, x.nx}, step[3] = {x.nxy, x.nx, 1};
  double acc = 0.0;
  for (int a = 0; a < 3; ++a) {
    if (coord[a] > 0) {  // low face: p is its hi side
      const int64_t q = p - step[a];
      const int c = min((int)fcls[a * v.nvox + p], nclass - 1);
      const double* f = forms + ((int64_t)(x.inst * nclass + c) * 3 + a) * 3;
      const bool fq = fixed && fixed[q];
      acc = fma(gg[a][p], fq ? f[1] + f[2] : f[2], acc);
    }
    if (coord[a] + 1 < len[a]) {  // high face (the low face of r): p is its lo side
      const int64_t r = p + step[a];
      const int c = min((int)fcls[a * v.nvox + r], nclass - 1);
      const double* f = forms + ((int64_t)(x.inst * nclass + c) * 3 + a) * 3;
      const bool fr = fixed && fixed[r];
      acc = fma(gg[a][r], fr ? f[1] + f[2] : f[1], acc);
    }
  }
  gk[p] = acc;
  gC[p] = gM[p] * inv_dt;
}

}  // namespace
}  // namespace hs2g

struct hs2g_adjoint {
  int device = 0;
  double dt = 0.0;
  cudaStream_t stream = nullptr;
  bool own_stream = true;
  int ninst = 0;
  int64_t n = 0, nobs_step = 0;  // voxels; top-layer voxels of all instances (observations per step)
  int64_t nlines[3] = {0, 0, 0};
  int64_t max_len[3] = {0, 0, 0};  // longest line of each axis over the instances
  std::vector<hs2g::AInst> host_inst;
  std::vector<int64_t> host_vox_off;
  hs2g::AInst* inst = nullptr;
  int64_t* vox_off = nullptr;
  int64_t* line_off = nullptr;
  int64_t* xg_off = nullptr;
  int64_t nxgroups = 0;
  // parameters and derived fields
  double *k = nullptr, *C = nullptr, *q = nullptr, *M = nullptr, *D = nullptr;
  double* g[3] = {nullptr, nullptr, nullptr};
  // face classes and fixed voxels (hs2g_adjoint_set_faces): without them every interior face conducts with the
  // arithmetic mean of k and every voxel is computed
  uint8_t* fcls = nullptr;   // 3 * n: class of each voxel's low face on z, y, x
  uint8_t* fixed = nullptr;  // n, or null
  double* forms = nullptr;   // [ninst][nclass][3][3]
  int nclass = 0;
  int* err = nullptr;
  // line factors of A_x, A_y, A_z: e = lo / piv, u = super-diagonal / piv, ip = 1 / piv, mip = M / piv
  double *e[3] = {nullptr, nullptr, nullptr}, *u[3] = {nullptr, nullptr, nullptr},
         *ip[3] = {nullptr, nullptr, nullptr}, *mip[3] = {nullptr, nullptr, nullptr};
  // run state
  bool have_params = false;
  int nsteps = 0, ckpt = 1;
  std::vector<double> sched;
  double* obs = nullptr;    // nsteps * nobs_step
  double* ckpts = nullptr;  // ceil(nsteps / ckpt) * n
  double* seg = nullptr;    // ckpt * 4 * n: T, y0, y1, y2 of each step of a segment
  double* seg2 = nullptr;   // a second segment store: the next segment is recomputed while this one is swept
  int stored_seg = -1;      // the segment whose states the last forward pass left in its store (-1: none)
  cudaStream_t rec_stream = nullptr;  // the recompute stream
  cudaEvent_t ev_rec[2] = {nullptr, nullptr}, ev_done[2] = {nullptr, nullptr}, ev_start = nullptr;
  double* T = nullptr;      // forward state
  double *lam = nullptr, *mu[3] = {nullptr, nullptr, nullptr};
  double *gg[3] = {nullptr, nullptr, nullptr}, *gM = nullptr, *gq = nullptr;
  double* parts = nullptr;  // 2 * kMisfitBlocks * nsteps * ninst misfit parts (compensated pairs)
  int64_t obs_cap = 0, ckpt_cap = 0, seg_cap = 0, seg2_cap = 0, parts_cap = 0;
  int64_t fixed_bytes = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
};

namespace {

using hs2g::kTh;
using hs2g::nblk;
using hs2g::launch_kernel;

// The kernels of a step are launched with programmatic dependent launch (each waits for the previous kernel at its
// start; no kernel triggers early): the launch latency at each kernel boundary is hidden.  HS2G_PDL=0 turns it
// off.
bool adj_pdl() {
  static const bool on = [] {
    const char* e = getenv("HS2G_PDL");
    return !(e && strcmp(e, "0") == 0);
  }();
  return on;
}

int afail(int code, const char* m) { return hs2g::set_last_error(code, m); }
int acuda(cudaError_t e, const char* what) {
  cudaGetLastError();  // a failed allocation leaves its error as the last error: clear it for later checks
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
  return hs2g::set_last_error(e == cudaErrorMemoryAllocation ? HS2G_ERR_NOMEM : HS2G_ERR_CUDA, buf);
}

struct AGuard {
  int prev = -1;
  bool ok = false;
  explicit AGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
    ok = (prev == dev) || (cudaSetDevice(dev) == cudaSuccess);
  }
  ~AGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
  }
};

hs2g::AView view(const hs2g_adjoint* a) {
  return hs2g::AView{a->inst, a->vox_off, a->line_off, a->xg_off, a->ninst, a->n};
}

// threads per CTA of the one-thread-per-line kernels: smaller CTAs when there are few lines, so that they
// spread over every SM
int line_threads(int64_t nlines) {
  const int64_t want = 2 * 152;
  return nlines >= 128 * want ? 128 : (nlines >= 64 * want ? 64 : 32);
}
unsigned line_blocks(int64_t nlines) {
  const int th = line_threads(nlines);
  return (unsigned)std::max<int64_t>(1, (nlines + th - 1) / th);
}

cudaError_t grow(double** p, int64_t* cap, int64_t need) {
  if (*p && *cap >= need) return cudaSuccess;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t e = cudaMalloc(p, sizeof(double) * std::max<int64_t>(1, need));
  if (e == cudaSuccess) *cap = need;
  return e;
}

// line solves: the few-line kernels when the lines leave each SM about one warp (y, z) or two groups (x) and
// fit in shared memory, else the register-blocked / fused ones (same bits either way)
bool few_lines(const hs2g_adjoint* a, int axis) {
  return line_threads(a->nlines[axis]) == 32 && a->max_len[axis] <= hs2g::kFewMaxLen;
}
bool few_x(const hs2g_adjoint* a) {
  return a->nxgroups <= hs2g::kFewXGroups && a->max_len[0] <= hs2g::kFewMaxNx;
}
template <bool ADD_T>
void launch_ysolve(const hs2g::AView& v, cudaStream_t st, int axis, int64_t nl, const double* rhs, const double* e,
                   const double* u, const double* scale, double* y, const double* T_in, double* T_out) {
  launch_kernel(hs2g::adj_ysolve_kernel<ADD_T>, dim3(line_blocks(nl)), dim3(line_threads(nl)), 0, st, adj_pdl(), v,
                axis, nl, rhs, e, u, scale, y, T_in, T_out);
}
// y = A_a^-1 (M rhs) on the y or z lines (weighted false: A_a^-1 rhs); T_out = T_in + y when T_out is given
void ysolve(hs2g_adjoint* a, cudaStream_t st, int axis, bool weighted, const double* rhs, double* y,
            const double* T_in, double* T_out) {
  const hs2g::AView v = view(a);
  const int64_t nl = a->nlines[axis];
  const double *e = a->e[axis], *u = a->u[axis], *scale = weighted ? a->mip[axis] : a->ip[axis];
  if (few_lines(a, axis)) {
    const unsigned nbk = line_blocks(nl);
    const size_t sm = hs2g::few_smem_bytes(a->max_len[axis]);
    const int64_t ml = a->max_len[axis];
    if (T_out)
      launch_kernel(hs2g::adj_ysolve_few_kernel<true>, dim3(nbk), dim3(64), sm, st, adj_pdl(), v, axis, nl, ml, rhs,
                    e, u, scale, y, T_in, T_out);
    else
      launch_kernel(hs2g::adj_ysolve_few_kernel<false>, dim3(nbk), dim3(64), sm, st, adj_pdl(), v, axis, nl, ml, rhs,
                    e, u, scale, y, T_in, T_out);
  } else if (T_out) {
    launch_ysolve<true>(v, st, axis, nl, rhs, e, u, scale, y, T_in, T_out);
  } else {
    launch_ysolve<false>(v, st, axis, nl, rhs, e, u, scale, y, T_in, T_out);
  }
}

// one forward step T_in -> T_out on stream st keeping y0, y1, y2 (T_out may alias T_in; NULL skips it)
cudaError_t fwd_step(hs2g_adjoint* a, cudaStream_t st, const double* T_in, double* T_out, double* y0, double* y1,
                     double* y2, double s) {
  const hs2g::AView v = view(a);
  if (few_x(a)) {
    launch_kernel(hs2g::adj_resid_kernel, dim3(nblk(a->n)), dim3(kTh), 0, st, adj_pdl(), v, T_in, a->g[0], a->g[1],
                  a->g[2], a->D, a->q, s, y0);
    launch_kernel(hs2g::adj_xsolve_few_kernel, dim3((unsigned)a->nxgroups), dim3(128),
                  hs2g::few_x_smem_bytes(a->max_len[0], 3), st, adj_pdl(), v, a->max_len[0], y0, a->e[0], a->u[0],
                  a->ip[0], y0);
  } else {
    launch_kernel(hs2g::adj_xsolve_kernel<true>, dim3((unsigned)a->nxgroups), dim3(hs2g::kXT), 0, st, adj_pdl(), v,
                  T_in, a->g[0], a->g[1], a->g[2], a->D, a->q, s, nullptr, a->e[0], a->u[0], a->ip[0], y0);
  }
  ysolve(a, st, 1, true, y0, y1, nullptr, nullptr);
  ysolve(a, st, 2, true, y1, y2, T_in, T_out);
  return cudaGetLastError();
}

// adjoint of one step: lambda (the adjoint of T_{n+1}) -> the adjoint of T_n, gradients accumulated.
// A_a is symmetric, so the transposed solves A_a^-T are the forward line solves.
cudaError_t bwd_step(hs2g_adjoint* a, const double* Tn, const double* y0, const double* y1, const double* y2,
                     double s, int64_t obs_step) {
  const hs2g::AView v = view(a);
  cudaStream_t st = a->stream;
  ysolve(a, st, 2, false, a->lam, a->mu[2], nullptr, nullptr);
  ysolve(a, st, 1, true, a->mu[2], a->mu[1], nullptr, nullptr);
  if (few_x(a))
    launch_kernel(hs2g::adj_xsolve_few_kernel, dim3((unsigned)a->nxgroups), dim3(128),
                  hs2g::few_x_smem_bytes(a->max_len[0], 3), st, adj_pdl(), v, a->max_len[0], a->mu[1], a->e[0],
                  a->u[0], a->mip[0], a->mu[0]);
  else
    launch_kernel(hs2g::adj_xsolve_kernel<false>, dim3((unsigned)a->nxgroups), dim3(hs2g::kXT), 0, st, adj_pdl(), v,
                  nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, 0.0, a->mu[1], a->e[0], a->u[0], a->mip[0],
                  a->mu[0]);
  launch_kernel(hs2g::adj_update_kernel, dim3(nblk(a->n)), dim3(kTh), 0, st, adj_pdl(), v, a->g[0], a->g[1], a->g[2],
                Tn, y0, y1, y2, a->mu[0], a->mu[1], a->mu[2], s, a->obs, obs_step, a->lam, a->gg[0], a->gg[1],
                a->gg[2], a->gM, a->gq);
  return cudaGetLastError();
}

void adj_free(hs2g_adjoint* a) {
  void* ptrs[] = {a->inst, a->vox_off, a->line_off, a->xg_off, a->k, a->C, a->q, a->M, a->D, a->g[0], a->g[1],
                  a->g[2], a->e[0], a->e[1], a->e[2], a->u[0], a->u[1], a->u[2], a->ip[0], a->ip[1], a->ip[2],
                  a->mip[0], a->mip[1], a->mip[2],
                  a->obs, a->ckpts, a->seg, a->seg2, a->T, a->lam, a->mu[0], a->mu[1], a->mu[2], a->gg[0], a->gg[1],
                  a->gg[2], a->gM, a->gq, a->parts, a->fcls, a->fixed, a->forms, a->err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (a->ev0) cudaEventDestroy(a->ev0);
  if (a->ev1) cudaEventDestroy(a->ev1);
  cudaEvent_t evs[] = {a->ev_rec[0], a->ev_rec[1], a->ev_done[0], a->ev_done[1], a->ev_start};
  for (cudaEvent_t ev : evs)
    if (ev) cudaEventDestroy(ev);
  if (a->rec_stream) cudaStreamDestroy(a->rec_stream);
  if (a->stream && a->own_stream) cudaStreamDestroy(a->stream);
}

cudaMemcpyKind in_kind(int flags) { return (flags & HS2G_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice; }
cudaMemcpyKind out_kind(int flags) { return (flags & HS2G_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost; }

void read_elapsed(hs2g_adjoint* a, double* elapsed_ms) {
  if (!elapsed_ms) return;
  float ms = 0.f;
  *elapsed_ms = cudaEventElapsedTime(&ms, a->ev0, a->ev1) == cudaSuccess ? ms : -1.0;
}

}  // namespace

extern "C" {

int hs2g_adjoint_create(int n, const hs2g_adjoint_grid* grids, double dt, int device, hs2g_adjoint** out) {
  if (!out) return afail(HS2G_ERR_ARG, "hs2g_adjoint_create: null output");
  *out = nullptr;
  if (n < 1 || !grids || !(dt > 0) || !std::isfinite(dt))
    return afail(HS2G_ERR_ARG, "hs2g_adjoint_create: bad argument");
  std::vector<hs2g::AInst> inst((size_t)n);
  std::vector<int64_t> vox_off((size_t)n + 1, 0), line_off(3 * ((size_t)n + 1), 0), xg_off((size_t)n + 1, 0);
  int64_t nobs = 0;
  const int64_t limit = int64_t(1) << 40;
  for (int i = 0; i < n; ++i) {
    const hs2g_adjoint_grid& g = grids[i];
    if (g.nz < 1 || g.ny < 1 || g.nx < 1 || !(g.dz > 0) || !(g.dy > 0) || !(g.dx > 0) || !std::isfinite(g.dz) ||
        !std::isfinite(g.dy) || !std::isfinite(g.dx))
      return afail(HS2G_ERR_ARG, "hs2g_adjoint_create: bad grid");
    if (g.ny > limit / g.nx || g.nz > limit / (g.ny * g.nx)) return afail(HS2G_ERR_ARG, "hs2g_adjoint_create: grid too large");
    hs2g::AInst& a = inst[i];
    a.off = vox_off[i];
    a.nz = g.nz;
    a.ny = g.ny;
    a.nx = g.nx;
    a.idx2 = 1.0 / (g.dx * g.dx);
    a.idy2 = 1.0 / (g.dy * g.dy);
    a.idz2 = 1.0 / (g.dz * g.dz);
    a.obs_off = nobs;  // in units of nsteps, scaled when the step count is known
    nobs += g.ny * g.nx;
    vox_off[i + 1] = vox_off[i] + g.nz * g.ny * g.nx;
    if (vox_off[i + 1] > limit) return afail(HS2G_ERR_ARG, "hs2g_adjoint_create: batch too large");
    line_off[0 * (n + 1) + i + 1] = line_off[0 * (n + 1) + i] + g.nz * g.ny;
    line_off[1 * (n + 1) + i + 1] = line_off[1 * (n + 1) + i] + g.nz * g.nx;
    line_off[2 * (n + 1) + i + 1] = line_off[2 * (n + 1) + i] + g.ny * g.nx;
    xg_off[i + 1] = xg_off[i] + (g.nz * g.ny + hs2g::kXL - 1) / hs2g::kXL;
  }
  if (xg_off[n] > 0x7fffffff) return afail(HS2G_ERR_ARG, "hs2g_adjoint_create: batch too large");
  // the line kernels index voxels with 32 bits; 2^31 voxels would need 515 GB for the 30 per-voxel fields
  if (vox_off[n] > 0x7fffffff) return afail(HS2G_ERR_ARG, "hs2g_adjoint_create: batch too large (2^31 voxels)");
  AGuard guard(device);
  if (!guard.ok) return afail(HS2G_ERR_CUDA, "hs2g_adjoint_create: cannot select device");
  hs2g_adjoint* a = new hs2g_adjoint();
  a->device = device;
  a->dt = dt;
  a->ninst = n;
  a->n = vox_off[n];
  a->nobs_step = nobs;
  for (int ax = 0; ax < 3; ++ax) a->nlines[ax] = line_off[ax * (n + 1) + n];
  for (const auto& in : inst) {
    a->max_len[0] = std::max(a->max_len[0], in.nx);
    a->max_len[1] = std::max(a->max_len[1], in.ny);
    a->max_len[2] = std::max(a->max_len[2], in.nz);
  }
  a->nxgroups = xg_off[n];
  a->host_inst = inst;
  a->host_vox_off = vox_off;
  cudaError_t e = cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&a->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&a->ev1);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&a->rec_stream, cudaStreamNonBlocking);
  for (int b = 0; b < 2 && e == cudaSuccess; ++b) {
    e = cudaEventCreateWithFlags(&a->ev_rec[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&a->ev_done[b], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&a->ev_start, cudaEventDisableTiming);
  {
    const void* few_y[] = {(const void*)hs2g::adj_ysolve_few_kernel<true>,
                           (const void*)hs2g::adj_ysolve_few_kernel<false>};
    for (const void* f : few_y)
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)hs2g::few_smem_bytes(hs2g::kFewMaxLen));
  }
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(hs2g::adj_xsolve_few_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)hs2g::few_x_smem_bytes(hs2g::kFewMaxNx, 3));
  if (e == cudaSuccess) e = cudaMalloc(&a->inst, sizeof(hs2g::AInst) * n);
  if (e == cudaSuccess) e = cudaMalloc(&a->vox_off, sizeof(int64_t) * (n + 1));
  if (e == cudaSuccess) e = cudaMalloc(&a->line_off, sizeof(int64_t) * 3 * (n + 1));
  if (e == cudaSuccess) e = cudaMalloc(&a->xg_off, sizeof(int64_t) * (n + 1));
  double** per_voxel[] = {&a->k, &a->C, &a->q, &a->M, &a->D, &a->g[0], &a->g[1], &a->g[2], &a->e[0], &a->e[1],
                          &a->e[2], &a->u[0], &a->u[1], &a->u[2], &a->ip[0], &a->ip[1], &a->ip[2], &a->mip[0],
                          &a->mip[1], &a->mip[2], &a->T,
                          &a->lam, &a->mu[0], &a->mu[1], &a->mu[2], &a->gg[0], &a->gg[1], &a->gg[2], &a->gM,
                          &a->gq};
  const int nfields = (int)(sizeof(per_voxel) / sizeof(per_voxel[0]));
  for (double** p : per_voxel)
    if (e == cudaSuccess) e = cudaMalloc(p, sizeof(double) * a->n);
  if (e == cudaSuccess) e = cudaMemcpy(a->inst, inst.data(), sizeof(hs2g::AInst) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(a->vox_off, vox_off.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(a->line_off, line_off.data(), sizeof(int64_t) * 3 * (n + 1), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(a->xg_off, xg_off.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    const int rc = acuda(e, "hs2g_adjoint_create");
    adj_free(a);
    delete a;
    return rc;
  }
  a->fixed_bytes = (int64_t)nfields * a->n * (int64_t)sizeof(double);
  *out = a;
  return HS2G_OK;
}

void hs2g_adjoint_destroy(hs2g_adjoint* a) {
  if (!a) return;
  AGuard guard(a->device);
  cudaStreamSynchronize(a->stream);
  adj_free(a);
  delete a;
}

int hs2g_adjoint_set_stream(hs2g_adjoint* a, void* stream) {
  if (!a) return afail(HS2G_ERR_ARG, "null handle");
  if (!a->own_stream && a->stream == (cudaStream_t)stream) return HS2G_OK;
  AGuard guard(a->device);
  cudaStreamSynchronize(a->stream);
  if (a->own_stream) cudaStreamDestroy(a->stream);
  a->stream = (cudaStream_t)stream;  // NULL = the legacy default stream
  a->own_stream = false;
  return HS2G_OK;
}

int hs2g_adjoint_layout(const hs2g_adjoint* a, int64_t* offsets) {
  if (!a || !offsets) return afail(HS2G_ERR_ARG, "null argument");
  for (int i = 0; i <= a->ninst; ++i) offsets[i] = a->host_vox_off[i];
  return HS2G_OK;
}

int64_t hs2g_adjoint_device_bytes(const hs2g_adjoint* a) {
  if (!a) return 0;
  return a->fixed_bytes +
         (int64_t)sizeof(double) * (a->obs_cap + a->ckpt_cap + a->seg_cap + a->seg2_cap + a->parts_cap);
}

int hs2g_adjoint_set_parameters(hs2g_adjoint* a, const double* k, const double* C, const double* q, int flags) {
  if (!a || !k || !C || !q) return afail(HS2G_ERR_ARG, "hs2g_adjoint_set_parameters: null argument");
  AGuard guard(a->device);
  cudaStream_t st = a->stream;
  const int64_t n = a->n;
  const cudaMemcpyKind kind = in_kind(flags);
  a->have_params = false;
  a->nsteps = 0;
  a->stored_seg = -1;
  cudaError_t e = cudaMemcpyAsync(a->k, k, sizeof(double) * n, kind, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a->C, C, sizeof(double) * n, kind, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a->q, q, sizeof(double) * n, kind, st);
  if (e != cudaSuccess) return acuda(e, "hs2g_adjoint_set_parameters");
  const hs2g::AView v = view(a);
  if (a->forms) {
    e = cudaMemsetAsync(a->err, 0, sizeof(int), st);
    if (e != cudaSuccess) return acuda(e, "hs2g_adjoint_set_parameters");
    hs2g::adj_setup_faces_kernel<<<nblk(n), kTh, 0, st>>>(v, a->k, a->C, 1.0 / a->dt, a->fcls, a->nclass, a->forms,
                                                          a->fixed, a->g[0], a->g[1], a->g[2], a->M, a->err);
  } else {
    hs2g::adj_setup_kernel<<<nblk(n), kTh, 0, st>>>(v, a->k, a->C, 1.0 / a->dt, a->g[0], a->g[1], a->g[2], a->M);
  }
  hs2g::adj_diag_kernel<<<nblk(n), kTh, 0, st>>>(v, a->g[0], a->g[1], a->g[2], a->D);
  for (int ax = 0; ax < 3; ++ax)
    hs2g::adj_factor_kernel<<<nblk(a->nlines[ax]), kTh, 0, st>>>(v, ax, a->nlines[ax], a->M, a->g[ax], a->e[ax],
                                                                a->u[ax], a->ip[ax], a->mip[ax]);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return acuda(e, "hs2g_adjoint_set_parameters");
  if (a->forms) {
    int bad = 0;
    e = cudaMemcpy(&bad, a->err, sizeof(int), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return acuda(e, "hs2g_adjoint_set_parameters");
    if (bad) return afail(HS2G_ERR_ARG, "hs2g_adjoint_set_parameters: a face class index is past the forms table");
  }
  a->have_params = true;
  return HS2G_OK;
}

int hs2g_adjoint_set_faces(hs2g_adjoint* a, int nclass, const double* forms, const uint8_t* face_z,
                           const uint8_t* face_y, const uint8_t* face_x, const uint8_t* fixed, int flags) {
  if (a && nclass == 0) {  // back to the default: every interior face conducting, every voxel computed
    AGuard guard(a->device);
    cudaStreamSynchronize(a->stream);
    void* ptrs[] = {a->forms, a->fcls, a->fixed};
    for (void* p : ptrs)
      if (p) cudaFree(p);
    a->forms = nullptr;
    a->fcls = a->fixed = nullptr;
    a->nclass = 0;
    a->have_params = false;
    a->nsteps = 0;
    a->stored_seg = -1;
    return HS2G_OK;
  }
  if (!a || nclass < 1 || nclass > HS2G_MAX_CLASSES || !forms || !face_z || !face_y || !face_x)
    return afail(HS2G_ERR_ARG, "hs2g_adjoint_set_faces: bad argument");
  const int64_t nf = (int64_t)a->ninst * nclass * 9;
  for (int64_t t = 0; t < nf; ++t)
    if (!std::isfinite(forms[t])) return afail(HS2G_ERR_ARG, "hs2g_adjoint_set_faces: non-finite face form");
  AGuard guard(a->device);
  cudaStream_t st = a->stream;
  const int64_t n = a->n;
  const cudaMemcpyKind kind = in_kind(flags);
  cudaError_t e = cudaSuccess;
  if (a->forms && a->nclass != nclass) {
    cudaFree(a->forms);
    a->forms = nullptr;
  }
  if (!a->forms) e = cudaMalloc(&a->forms, sizeof(double) * nf);
  if (e == cudaSuccess && !a->fcls) e = cudaMalloc(&a->fcls, 3 * (size_t)n);
  if (e == cudaSuccess && !a->err) e = cudaMalloc(&a->err, sizeof(int));
  if (e == cudaSuccess && fixed && !a->fixed) e = cudaMalloc(&a->fixed, (size_t)n);
  if (e != cudaSuccess) {
    cudaFree(a->forms);
    a->forms = nullptr;
    return acuda(e, "hs2g_adjoint_set_faces: device allocation");
  }
  a->nclass = nclass;
  e = cudaMemcpyAsync(a->forms, forms, sizeof(double) * nf, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a->fcls, face_z, (size_t)n, kind, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a->fcls + n, face_y, (size_t)n, kind, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a->fcls + 2 * n, face_x, (size_t)n, kind, st);
  if (e == cudaSuccess && fixed) e = cudaMemcpyAsync(a->fixed, fixed, (size_t)n, kind, st);
  if (e == cudaSuccess && !fixed && a->fixed) {
    cudaFree(a->fixed);
    a->fixed = nullptr;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return acuda(e, "hs2g_adjoint_set_faces");
  a->have_params = false;  // the faces apply from the next hs2g_adjoint_set_parameters
  a->nsteps = 0;
  a->stored_seg = -1;
  return HS2G_OK;
}

int hs2g_adjoint_forward(hs2g_adjoint* a, int nsteps, const double* schedule, const double* T0, const double* obs,
                         int ckpt, double* loss, double* T_out, int flags, double* elapsed_ms) {
  if (!a || nsteps < 1 || !schedule || !T0 || !obs || ckpt < 1 || !loss)
    return afail(HS2G_ERR_ARG, "hs2g_adjoint_forward: bad argument");
  if (!a->have_params) return afail(HS2G_ERR_STATE, "hs2g_adjoint_forward: parameters not set");
  for (int s = 0; s < nsteps; ++s)
    if (!std::isfinite(schedule[s])) return afail(HS2G_ERR_ARG, "hs2g_adjoint_forward: non-finite schedule");
  AGuard guard(a->device);
  cudaStream_t st = a->stream;
  const int64_t n = a->n;
  ckpt = std::min(ckpt, nsteps);
  const int64_t nck = (nsteps + ckpt - 1) / ckpt;
  a->nsteps = 0;
  cudaError_t e = cudaStreamSynchronize(st);  // buffers may be reallocated below
  if (e == cudaSuccess) e = grow(&a->obs, &a->obs_cap, (int64_t)nsteps * a->nobs_step);
  if (e == cudaSuccess) e = grow(&a->ckpts, &a->ckpt_cap, nck * n);
  if (e == cudaSuccess) e = grow(&a->parts, &a->parts_cap, (int64_t)2 * hs2g::kMisfitBlocks * nsteps * a->ninst);
  if (e != cudaSuccess) return acuda(e, "hs2g_adjoint_forward: device allocation");
  std::vector<hs2g::AInst> inst = a->host_inst;
  for (auto& in : inst) in.obs_off *= nsteps;
  e = cudaMemcpyAsync(a->inst, inst.data(), sizeof(hs2g::AInst) * a->ninst, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a->obs, obs, sizeof(double) * nsteps * a->nobs_step, in_kind(flags), st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(a->T, T0, sizeof(double) * n, in_kind(flags), st);
  if (e == cudaSuccess) e = cudaEventRecord(a->ev0, st);
  a->sched.assign(schedule, schedule + nsteps);
  a->stored_seg = -1;
  // The last segment's states (T, y0, y1, y2 of each step, the layout the recompute writes) go straight into
  // the segment store the backward pass sweeps first, when the stores already exist from an earlier backward
  // pass: that pass then skips its first recompute, the one nothing overlaps.  The same kernels compute the
  // same states, so the gradients do not change.
  const int64_t seg_need = (int64_t)ckpt * 4 * n;
  double* store = nullptr;
  if (a->seg && a->seg_cap >= seg_need && (nck == 1 || (a->seg2 && a->seg2_cap >= seg_need)))
    store = ((nck - 1) & 1) ? a->seg2 : a->seg;
  const int s_store = store ? (int)((nck - 1) * ckpt) : nsteps;
  const hs2g::AView v = view(a);
  for (int s = 0; s < nsteps && e == cudaSuccess; ++s) {
    if (s % ckpt == 0)
      e = cudaMemcpyAsync(a->ckpts + (int64_t)(s / ckpt) * n, a->T, sizeof(double) * n, cudaMemcpyDeviceToDevice,
                          st);
    double* out = a->T;
    if (s < s_store) {
      // the adjoint buffers are free during the forward pass and hold the increments
      if (e == cudaSuccess) e = fwd_step(a, st, a->T, a->T, a->mu[0], a->mu[1], a->mu[2], a->sched[s]);
    } else {
      double* slot = store + (int64_t)(s - s_store) * 4 * n;
      if (s == s_store && e == cudaSuccess)
        e = cudaMemcpyAsync(slot, a->T, sizeof(double) * n, cudaMemcpyDeviceToDevice, st);
      if (s + 1 < nsteps) out = slot + 4 * n;
      if (e == cudaSuccess) e = fwd_step(a, st, slot, out, slot + n, slot + 2 * n, slot + 3 * n, a->sched[s]);
    }
    if (e == cudaSuccess) {
      e = launch_kernel(hs2g::adj_misfit_kernel, dim3(hs2g::kMisfitBlocks, a->ninst), dim3(256), 0, st, adj_pdl(), v,
                        out, a->obs, (int64_t)s, a->parts);
    }
  }
  if (e == cudaSuccess) e = cudaEventRecord(a->ev1, st);
  std::vector<double> parts((size_t)2 * hs2g::kMisfitBlocks * nsteps * a->ninst);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(parts.data(), a->parts, sizeof(double) * parts.size(), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && T_out) e = cudaMemcpyAsync(T_out, a->T, sizeof(double) * n, out_kind(flags), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return acuda(e, "hs2g_adjoint_forward");
  read_elapsed(a, elapsed_ms);
  for (int i = 0; i < a->ninst; ++i) {  // Neumaier sum of the per-step, per-block pairs
    double acc = 0.0, comp = 0.0;
    for (int s = 0; s < nsteps; ++s)
      for (int h = 0; h < 2 * hs2g::kMisfitBlocks; ++h) {
        const double v = parts[2 * ((size_t)s * a->ninst + i) * hs2g::kMisfitBlocks + h];
        const double t = acc + v;
        comp += std::fabs(acc) >= std::fabs(v) ? (acc - t) + v : (v - t) + acc;
        acc = t;
      }
    loss[i] = acc + comp;
  }
  a->nsteps = nsteps;
  a->ckpt = ckpt;
  a->stored_seg = store ? (int)(nck - 1) : -1;
  return HS2G_OK;
}

int hs2g_adjoint_backward(hs2g_adjoint* a, double* gk, double* gC, double* gq, double* gT0, int flags,
                          double* elapsed_ms) {
  if (!a || !gk || !gC || !gq) return afail(HS2G_ERR_ARG, "hs2g_adjoint_backward: null argument");
  if (a->nsteps < 1) return afail(HS2G_ERR_STATE, "hs2g_adjoint_backward: no forward pass to differentiate");
  AGuard guard(a->device);
  cudaStream_t st = a->stream;
  const hs2g::AView v = view(a);
  const int64_t n = a->n;
  const int N = a->nsteps, C = a->ckpt;
  // the segment stores (T, y0, y1, y2 of ckpt steps) exist only while gradients are taken; with two of them
  // the recompute of segment sg-1 (rec_stream) runs while segment sg is swept backwards (the handle's stream)
  cudaError_t e = grow(&a->seg, &a->seg_cap, (int64_t)C * 4 * n);
  if (e != cudaSuccess) return acuda(e, "hs2g_adjoint_backward: device allocation");
  const int nseg = (N + C - 1) / C;
  bool dbl = false;
  if (nseg > 1) {
    dbl = grow(&a->seg2, &a->seg2_cap, (int64_t)C * 4 * n) == cudaSuccess;
    if (!dbl) cudaGetLastError();  // out of memory for the second store: recompute and sweep in turn
  }
  double* bufs[2] = {a->seg, dbl ? a->seg2 : a->seg};
  // the last forward pass may have left the last segment in its store (see hs2g_adjoint_forward)
  const bool stored = a->stored_seg == nseg - 1 && (nseg == 1 || dbl);
  a->stored_seg = -1;
  e = cudaEventRecord(a->ev0, st);
  double* zero_list[] = {a->gg[0], a->gg[1], a->gg[2], a->gM, a->gq};
  for (double* p : zero_list)
    if (e == cudaSuccess) e = cudaMemsetAsync(p, 0, sizeof(double) * n, st);
  if (e == cudaSuccess) {
    hs2g::adj_seed_kernel<<<nblk(n), kTh, 0, st>>>(v, a->T, a->obs, N - 1, a->lam);
    e = cudaGetLastError();
  }
  cudaStream_t rs = dbl ? a->rec_stream : st;
  if (e == cudaSuccess && dbl) e = cudaEventRecord(a->ev_start, st);  // checkpoints and parameters are ready
  if (e == cudaSuccess && dbl) e = cudaStreamWaitEvent(rs, a->ev_start, 0);
  // recompute segment sg into its store: slot j holds T, y0, y1, y2 of step s0 + j (the end state is not kept)
  auto recompute = [&](int sg) -> cudaError_t {
    const int s0 = sg * C, s1 = std::min(N, s0 + C);
    double* buf = bufs[sg & 1];
    cudaError_t r = cudaMemcpyAsync(buf, a->ckpts + (int64_t)sg * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, rs);
    for (int s = s0; s < s1 && r == cudaSuccess; ++s) {
      double* slot = buf + (int64_t)(s - s0) * 4 * n;
      double* next = s + 1 < s1 ? slot + 4 * n : nullptr;
      r = fwd_step(a, rs, slot, next, slot + n, slot + 2 * n, slot + 3 * n, a->sched[s]);
    }
    if (r == cudaSuccess && dbl) r = cudaEventRecord(a->ev_rec[sg & 1], rs);
    return r;
  };
  if (e == cudaSuccess && !stored) e = recompute(nseg - 1);
  for (int sg = nseg - 1; sg >= 0 && e == cudaSuccess; --sg) {
    if (dbl && sg >= 1) {
      // store (sg-1)&1 was last read by the sweep of segment sg+1
      e = cudaStreamWaitEvent(rs, a->ev_done[(sg - 1) & 1], 0);
      if (e == cudaSuccess) e = recompute(sg - 1);
    }
    if (e == cudaSuccess && dbl && !(stored && sg == nseg - 1)) e = cudaStreamWaitEvent(st, a->ev_rec[sg & 1], 0);
    const int s0 = sg * C, s1 = std::min(N, s0 + C);
    const double* buf = bufs[sg & 1];
    for (int s = s1 - 1; s >= s0 && e == cudaSuccess; --s) {
      const double* slot = buf + (int64_t)(s - s0) * 4 * n;
      // T_s (s >= 1) is the state observed after step s - 1
      e = bwd_step(a, slot, slot + n, slot + 2 * n, slot + 3 * n, a->sched[s], s >= 1 ? s - 1 : -1);
    }
    if (e == cudaSuccess && dbl) e = cudaEventRecord(a->ev_done[sg & 1], st);
    if (e == cudaSuccess && !dbl && sg >= 1) e = recompute(sg - 1);
  }
  if (e == cudaSuccess) {
    if (a->forms)
      hs2g::adj_chain_faces_kernel<<<nblk(n), kTh, 0, st>>>(v, a->gg[0], a->gg[1], a->gg[2], a->gM, 1.0 / a->dt,
                                                            a->fcls, a->nclass, a->forms, a->fixed, a->mu[0],
                                                            a->mu[1], a->gq);
    else
      hs2g::adj_chain_kernel<<<nblk(n), kTh, 0, st>>>(v, a->gg[0], a->gg[1], a->gg[2], a->gM, 1.0 / a->dt,
                                                      a->mu[0], a->mu[1]);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaEventRecord(a->ev1, st);
  const cudaMemcpyKind kind = out_kind(flags);
  if (e == cudaSuccess) e = cudaMemcpyAsync(gk, a->mu[0], sizeof(double) * n, kind, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(gC, a->mu[1], sizeof(double) * n, kind, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(gq, a->gq, sizeof(double) * n, kind, st);
  if (e == cudaSuccess && gT0) e = cudaMemcpyAsync(gT0, a->lam, sizeof(double) * n, kind, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return acuda(e, "hs2g_adjoint_backward");
  read_elapsed(a, elapsed_ms);
  return HS2G_OK;
}

}  // extern "C"
