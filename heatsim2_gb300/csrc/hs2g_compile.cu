// Setup-time kernels: the coefficient compiler (class arrays -> per-face conductances) and the per-line
// tridiagonal factorisations that turn conductances (shared per face, or per row in the curved-surface mode)
// and capacities into the step coefficients.
//
// Replaces the reference's Python voxel loop and symbolic assembly (crank_nicolson.pyx:272-491,
// alternatingdirection_c.c:102-199) and its LU factorisation at finalize (tridiag.pyx:9-43,
// alternatingdirection_c_pyx.pyx:279).  All FP64.  One thread per face (compiler) or per grid line (LU).
#include "hs2g_internal.cuh"

namespace hs2g {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ double eval_form(const double* f, const double* klo, const double* khi) {
  double acc = f[0];
#pragma unroll
  for (int e = 0; e < HS2G_K_ENTRIES; ++e) {
    const double cl = f[1 + e];
    const double ch = f[1 + HS2G_K_ENTRIES + e];
    if (cl != 0.0) acc += cl * klo[e];
    if (ch != 0.0) acc += ch * khi[e];
  }
  return acc;
}

// One thread per face of `axis`.  The two voxels that meet at a face are lo (index - 1 along the axis) and hi.
// A face only matters to the compute voxels beside it; the reference evaluates its flux from a compute
// voxel's equation with the neighbour's k replaced by the voxel's own when the neighbour is fixed or outside
// the grid (crank_nicolson.pyx:298-338), so both compute sides see the same k pair and one value per face
// serves both.
__global__ void faces_kernel(Dims d, int axis, const uint8_t* __restrict__ material,
                             const uint8_t* __restrict__ bclass, const hs2g_material* __restrict__ mats, int nmat,
                             const hs2g_face_form* __restrict__ forms, int nbnd, double* __restrict__ G,
                             unsigned long long* err) {
  const int64_t fz = d.nz + (axis == 0), fy = d.ny + (axis == 1), fx = d.nx + (axis == 2);
  const int64_t nfaces = fz * fy * fx;
  for (int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; f < nfaces;
       f += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = f % fx;
    const int64_t j = (f / fx) % fy;
    const int64_t k = f / (fx * fy);
    const int64_t c = axis == 0 ? k : (axis == 1 ? j : i);
    const int64_t n_axis = axis == 0 ? d.nz : (axis == 1 ? d.ny : d.nx);
    const bool lo_in = c > 0, hi_in = c < n_axis;
    // the hi voxel has the face's coordinates, the lo voxel is one step back along the axis
    const int64_t phi = hi_in ? (k * d.ny + j) * d.nx + i : -1;
    const int64_t plo =
        lo_in ? ((k - (axis == 0)) * d.ny + (j - (axis == 1))) * d.nx + (i - (axis == 2)) : -1;
    int mlo = -1, mhi = -1;
    if (lo_in) mlo = material[plo];
    if (hi_in) mhi = material[phi];
    if ((lo_in && mlo >= nmat) || (hi_in && mhi >= nmat)) {
      record_error(err, HS2G_ERR_ARG, axis, f);
      G[f] = 0.0;
      continue;
    }
    const bool lo_c = lo_in && mats[mlo].kind == HS2G_TEMPERATURE_COMPUTE;
    const bool hi_c = hi_in && mats[mhi].kind == HS2G_TEMPERATURE_COMPUTE;
    if (!lo_c && !hi_c) {
      G[f] = 0.0;
      continue;
    }
    const int b = bclass[f];
    if (b >= nbnd) {
      record_error(err, HS2G_ERR_ARG, axis, f);
      G[f] = 0.0;
      continue;
    }
    const double* klo = lo_c ? mats[mlo].k : mats[mhi].k;
    const double* khi = hi_c ? mats[mhi].k : mats[mlo].k;
    const hs2g_face_form& form = forms[b * 3 + axis];
    const double g = eval_form(form.normal, klo, khi);
    if (!(g == g) || isinf(g)) {
      record_error(err, HS2G_ERR_KTYPE, axis, f);
      G[f] = 0.0;
      continue;
    }
    const double tol = 1e-12 * fabs(g);
    for (int z = 0; z < form.nzero; ++z) {
      const double v = eval_form(form.zero[z], klo, khi);
      if (!(fabs(v) <= tol)) record_error(err, form.zero_code[z], axis, f);
    }
    if ((!lo_in || !hi_in) && g != 0.0) record_error(err, HS2G_ERR_EXTERIOR, axis, f);
    G[f] = g;
  }
}

// Per-voxel capacity M = rho*c/dt for computed voxels, 1 for fixed ones (their rows are the identity).
__global__ void capacity_kernel(Dims d, const uint8_t* __restrict__ material, const hs2g_material* __restrict__ mats,
                                int nmat, double* __restrict__ M, uint8_t* __restrict__ compute,
                                unsigned long long* err) {
  const int64_t n = d.nvox();
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int m = material[p];
    if (m >= nmat) {
      record_error(err, HS2G_ERR_ARG, 3, p);
      M[p] = 1.0;
      compute[p] = 0;
      continue;
    }
    const bool c = mats[m].kind == HS2G_TEMPERATURE_COMPUTE;
    const double cap = mats[m].capacity;
    if (c && !(cap > 0.0 && cap < INFINITY)) record_error(err, HS2G_ERR_CAPACITY, 3, p);
    M[p] = c ? cap : 1.0;
    compute[p] = c ? 1 : 0;
  }
}

// Dense problems: capacities arrive per voxel; check them and that computed voxels have no exterior flux.
__global__ void validate_dense_kernel(Dims d, const double* __restrict__ Gz, const double* __restrict__ Gy,
                                      const double* __restrict__ Gx, double* __restrict__ M,
                                      uint8_t* __restrict__ compute, unsigned long long* err) {
  const int64_t n = d.nvox();
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = p % d.nx, j = (p / d.nx) % d.ny, k = p / d.nxy();
    if (!compute[p]) {
      M[p] = 1.0;
      continue;
    }
    const double cap = M[p];
    if (!(cap > 0.0 && cap < INFINITY)) record_error(err, HS2G_ERR_CAPACITY, 3, p);
    const double gzl = Gz[(k * d.ny + j) * d.nx + i], gzh = Gz[((k + 1) * d.ny + j) * d.nx + i];
    const double gyl = Gy[(k * (d.ny + 1) + j) * d.nx + i], gyh = Gy[(k * (d.ny + 1) + j + 1) * d.nx + i];
    const double gxl = Gx[(k * d.ny + j) * (d.nx + 1) + i], gxh = Gx[(k * d.ny + j) * (d.nx + 1) + i + 1];
    if ((k == 0 && gzl != 0.0) || (k == d.nz - 1 && gzh != 0.0)) record_error(err, HS2G_ERR_EXTERIOR, 0, p);
    if ((j == 0 && gyl != 0.0) || (j == d.ny - 1 && gyh != 0.0)) record_error(err, HS2G_ERR_EXTERIOR, 1, p);
    if ((i == 0 && gxl != 0.0) || (i == d.nx - 1 && gxh != 0.0)) record_error(err, HS2G_ERR_EXTERIOR, 2, p);
    const double all = gzl + gzh + gyl + gyh + gxl + gxh;
    if (!(all == all) || isinf(all)) record_error(err, HS2G_ERR_ARG, 3, p);
  }
}

// ---------------------------------------------------------------------------------------------------------
// Per-line LU of the stage matrices (M - G/2 along the stage axis), in the reference's row order and
// normalisation (tridiag.pyx:25-41): piv_r = d_r - u_{r-1}*lo_r, u_r = hi_r/piv_r, with
// d = M + (G_lo+G_hi)/2, lo = -G_lo/2, hi = -G_hi/2 for computed voxels and the identity row for fixed ones.
//
// The step is the Douglas scheme in delta form,
//     (M - Lx/2) dT0 = L T + Q,   (M - Ly/2) dT1 = M dT0,   (M - Lz/2) dT2 = M dT1,   T' = T + dT2,
// which equals the reference's stage equations (alternatingdirection_c_pyx.pyx:483-493 with
// crank_subst_in_groups) exactly in real arithmetic.  Each stage's output is pre-multiplied by the diagonal
// scale the next stage's forward sweep applies to its input, so the y and z sweeps are one FMA per
// forward and back step:
//     s2 = M/piv2,  sigma = s2*M/piv1,   W0 = sigma*dT0,   W1 = s2*dT1.
// ---------------------------------------------------------------------------------------------------------
struct RowIn {
  double d, lo, hi;
};

__device__ __forceinline__ RowIn stage_row(bool comp, double M, double gl, double gh) {
  RowIn r;
  r.d = comp ? M + 0.5 * (gl + gh) : 1.0;
  r.lo = comp ? -(0.5 * gl) : 0.0;
  r.hi = comp ? -(0.5 * gh) : 0.0;
  return r;
}

// The six face conductances of voxel p as its own row sees them.  SharedFaces: one array per axis indexed by
// face, so the two rows of a face see the same value (the class and dense problems).  RowFaces: six
// (nz, ny, nx) arrays, one value per row and side, so a face may weigh differently in its two rows (the
// reference's curved-surface mode, where each row uses its own cell's edge lengths).
struct SharedFaces {
  const double *Gz, *Gy, *Gx;
  __device__ double zlo(const Dims& d, int64_t p, int64_t, int64_t, int64_t) const { return Gz[p]; }
  __device__ double zhi(const Dims& d, int64_t p, int64_t, int64_t, int64_t) const { return Gz[p + d.nxy()]; }
  __device__ double ylo(const Dims& d, int64_t, int64_t k, int64_t j, int64_t i) const {
    return Gy[(k * (d.ny + 1) + j) * d.nx + i];
  }
  __device__ double yhi(const Dims& d, int64_t, int64_t k, int64_t j, int64_t i) const {
    return Gy[(k * (d.ny + 1) + j + 1) * d.nx + i];
  }
  __device__ double xlo(const Dims& d, int64_t, int64_t k, int64_t j, int64_t i) const {
    return Gx[(k * d.ny + j) * (d.nx + 1) + i];
  }
  __device__ double xhi(const Dims& d, int64_t, int64_t k, int64_t j, int64_t i) const {
    return Gx[(k * d.ny + j) * (d.nx + 1) + i + 1];
  }
};
struct RowFaces {
  const double *zl, *zh, *yl, *yh, *xl, *xh;
  __device__ double zlo(const Dims&, int64_t p, int64_t, int64_t, int64_t) const { return zl[p]; }
  __device__ double zhi(const Dims&, int64_t p, int64_t, int64_t, int64_t) const { return zh[p]; }
  __device__ double ylo(const Dims&, int64_t p, int64_t, int64_t, int64_t) const { return yl[p]; }
  __device__ double yhi(const Dims&, int64_t p, int64_t, int64_t, int64_t) const { return yh[p]; }
  __device__ double xlo(const Dims&, int64_t p, int64_t, int64_t, int64_t) const { return xl[p]; }
  __device__ double xhi(const Dims&, int64_t p, int64_t, int64_t, int64_t) const { return xh[p]; }
};

// z lines (one thread per (j,i)): stage-2 coefficients and s2.
template <class F>
__global__ void factor_z_kernel(Dims d, F g, const double* __restrict__ M, const uint8_t* __restrict__ compute,
                                double* __restrict__ s2, double* __restrict__ a2, double* __restrict__ b2) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= d.nxy()) return;
  const int64_t j = t / d.nx, i = t - j * d.nx;
  double u_prev = 0.0;
  for (int64_t k = 0; k < d.nz; ++k) {
    const int64_t p = k * d.nxy() + t;
    const bool comp = compute[p] != 0;
    const RowIn r = stage_row(comp, M[p], comp ? g.zlo(d, p, k, j, i) : 0.0, comp ? g.zhi(d, p, k, j, i) : 0.0);
    const double piv = r.d - u_prev * r.lo;
    const double u = r.hi / piv;
    a2[p] = r.lo / piv;
    b2[p] = u;
    s2[p] = M[p] / piv;
    u_prev = u;
  }
}

// y lines (one thread per (k,i)): stage-1 coefficients and sigma.
template <class F>
__global__ void factor_y_kernel(Dims d, F g, const double* __restrict__ M, const uint8_t* __restrict__ compute,
                                const double* __restrict__ s2, double* __restrict__ sigma, double* __restrict__ a1,
                                double* __restrict__ b1, int64_t px) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= d.nz * d.nx) return;
  const int64_t k = t / d.nx, i = t - k * d.nx;
  double u_prev = 0.0, s2_prev = 1.0;
  for (int64_t j = 0; j < d.ny; ++j) {
    const int64_t p = (k * d.ny + j) * d.nx + i;
    const int64_t pp = (k * d.ny + j) * px + i;  // a1 / b1 row pitch
    const bool comp = compute[p] != 0;
    const RowIn r = stage_row(comp, M[p], comp ? g.ylo(d, p, k, j, i) : 0.0, comp ? g.yhi(d, p, k, j, i) : 0.0);
    const double piv = r.d - u_prev * r.lo;
    const double u = r.hi / piv;
    const double s2p = s2[p];
    sigma[p] = s2p * M[p] / piv;
    a1[pp] = (j > 0) ? s2p * r.lo / (piv * s2_prev) : 0.0;
    b1[pp] = (j + 1 < d.ny) ? s2p * u / s2[p + d.nx] : 0.0;
    u_prev = u;
    s2_prev = s2p;
  }
}

// x lines (one thread per (k,j)): stage-0 stencil, forward and back coefficients.
template <class F>
__global__ void factor_x_kernel(Dims d, F g, const double* __restrict__ M, const uint8_t* __restrict__ compute,
                                const double* __restrict__ sigma, Coeffs c) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= d.nz * d.ny) return;
  const int64_t k = t / d.ny, j = t - k * d.ny;
  double u_prev = 0.0, sg_prev = 1.0;
  for (int64_t i = 0; i < d.nx; ++i) {
    const int64_t p = t * d.nx + i;
    const bool comp = compute[p] != 0;
    const double gxl = comp ? g.xlo(d, p, k, j, i) : 0.0, gxh = comp ? g.xhi(d, p, k, j, i) : 0.0;
    const double gyl = comp ? g.ylo(d, p, k, j, i) : 0.0, gyh = comp ? g.yhi(d, p, k, j, i) : 0.0;
    const double gzl = comp ? g.zlo(d, p, k, j, i) : 0.0, gzh = comp ? g.zhi(d, p, k, j, i) : 0.0;
    const RowIn r = stage_row(comp, M[p], gxl, gxh);
    const double piv = r.d - u_prev * r.lo;
    const double u = r.hi / piv;
    const double sg = sigma[p];
    const double f0 = sg / piv;
    const double center = -(((gxl + gxh) + (gyl + gyh)) + (gzl + gzh));
    double* blk = c.xb + ((t * c.nchunks + i / 32) * kXBlockCoeffs) * 32 + (i % 32);
    blk[kWc * 32] = f0 * center;
    blk[kWxl * 32] = f0 * gxl;
    blk[kWxh * 32] = f0 * gxh;
    blk[kWyl * 32] = f0 * gyl;
    blk[kWyh * 32] = f0 * gyh;
    blk[kWzl * 32] = f0 * gzl;
    blk[kWzh * 32] = f0 * gzh;
    blk[kWq * 32] = comp ? f0 : 0.0;
    const double a0 = (i > 0) ? sg * r.lo / (piv * sg_prev) : 0.0;
    const double b0 = (i + 1 < d.nx) ? sg * u / sigma[p + 1] : 0.0;
    c.a0[p] = a0;
    c.b0[p] = b0;
    u_prev = u;
    sg_prev = sg;
  }
}

// per-row problem: capacities positive and finite, coefficients finite, exterior sides zero on computed
// voxels (the same rules as validate_dense_kernel); fixed voxels get the unit capacity of an identity row
__global__ void validate_rows_kernel(Dims d, RowFaces g, double* __restrict__ M, uint8_t* __restrict__ compute,
                                     unsigned long long* err) {
  const int64_t n = d.nvox();
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = p % d.nx, j = (p / d.nx) % d.ny, k = p / d.nxy();
    if (!compute[p]) {
      M[p] = 1.0;
      continue;
    }
    const double cap = M[p];
    if (!(cap > 0.0 && cap < INFINITY)) record_error(err, HS2G_ERR_CAPACITY, 3, p);
    if ((k == 0 && g.zl[p] != 0.0) || (k == d.nz - 1 && g.zh[p] != 0.0)) record_error(err, HS2G_ERR_EXTERIOR, 0, p);
    if ((j == 0 && g.yl[p] != 0.0) || (j == d.ny - 1 && g.yh[p] != 0.0)) record_error(err, HS2G_ERR_EXTERIOR, 1, p);
    if ((i == 0 && g.xl[p] != 0.0) || (i == d.nx - 1 && g.xh[p] != 0.0)) record_error(err, HS2G_ERR_EXTERIOR, 2, p);
    const double all = g.zl[p] + g.zh[p] + g.yl[p] + g.yh[p] + g.xl[p] + g.xh[p];
    if (!(all == all) || isinf(all)) record_error(err, HS2G_ERR_ARG, 3, p);
  }
}

inline unsigned grid_for(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > (1 << 20)) b = 1 << 20;
  return (unsigned)b;
}

}  // namespace

cudaError_t launch_faces(const Dims& d, int axis, const uint8_t* material, const uint8_t* bclass,
                         const hs2g_material* mats, int nmat, const hs2g_face_form* forms, int nbnd, double* G,
                         unsigned long long* err, cudaStream_t s) {
  const int64_t nfaces = (d.nz + (axis == 0)) * (d.ny + (axis == 1)) * (d.nx + (axis == 2));
  faces_kernel<<<grid_for(nfaces, kThreads), kThreads, 0, s>>>(d, axis, material, bclass, mats, nmat, forms, nbnd,
                                                               G, err);
  return cudaGetLastError();
}

cudaError_t launch_capacity_from_classes(const Dims& d, const uint8_t* material, const hs2g_material* mats,
                                         int nmat, double* M, uint8_t* compute, unsigned long long* err,
                                         cudaStream_t s) {
  capacity_kernel<<<grid_for(d.nvox(), kThreads), kThreads, 0, s>>>(d, material, mats, nmat, M, compute, err);
  return cudaGetLastError();
}

cudaError_t launch_validate_dense(const Dims& d, const double* Gz, const double* Gy, const double* Gx, double* M,
                                  uint8_t* compute, unsigned long long* err, cudaStream_t s) {
  validate_dense_kernel<<<grid_for(d.nvox(), kThreads), kThreads, 0, s>>>(d, Gz, Gy, Gx, M, compute, err);
  return cudaGetLastError();
}

template <class F>
cudaError_t launch_factor_with(const Dims& d, F g, const double* M, const uint8_t* compute, double* s2,
                               double* sigma, const Coeffs& c, cudaStream_t s) {
  const int th = 128;
  factor_z_kernel<F><<<grid_for(d.nxy(), th), th, 0, s>>>(d, g, M, compute, s2, c.a2, c.b2);
  factor_y_kernel<F><<<grid_for(d.nz * d.nx, th), th, 0, s>>>(d, g, M, compute, s2, sigma, c.a1, c.b1,
                                                                c.px ? c.px : d.nx);
  factor_x_kernel<F><<<grid_for(d.nz * d.ny, th), th, 0, s>>>(d, g, M, compute, sigma, c);
  return cudaGetLastError();
}

cudaError_t launch_factor(const Dims& d, const double* Gz, const double* Gy, const double* Gx, const double* M,
                          const uint8_t* compute, double* s2, double* sigma, const Coeffs& c, cudaStream_t s) {
  return launch_factor_with(d, SharedFaces{Gz, Gy, Gx}, M, compute, s2, sigma, c, s);
}

cudaError_t launch_factor_rows(const Dims& d, const double* const rows[6], const double* M, const uint8_t* compute,
                               double* s2, double* sigma, const Coeffs& c, cudaStream_t s) {
  const RowFaces g{rows[0], rows[1], rows[2], rows[3], rows[4], rows[5]};
  return launch_factor_with(d, g, M, compute, s2, sigma, c, s);
}

cudaError_t launch_validate_rows(const Dims& d, const double* const rows[6], double* M, uint8_t* compute,
                                 unsigned long long* err, cudaStream_t s) {
  const RowFaces g{rows[0], rows[1], rows[2], rows[3], rows[4], rows[5]};
  validate_rows_kernel<<<grid_for(d.nvox(), kThreads), kThreads, 0, s>>>(d, g, M, compute, err);
  return cudaGetLastError();
}

}  // namespace hs2g
