// Internal declarations shared by the hs2g translation units (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/hs2g.h"

namespace hs2g {

// Grid dimensions; voxel p = (k*ny + j)*nx + i.
struct Dims {
  int64_t nz, ny, nx;
  __host__ __device__ int64_t nvox() const { return nz * ny * nx; }
  __host__ __device__ int64_t nxy() const { return ny * nx; }
};

// Per-voxel coefficients of the scaled delta-form Douglas step.
//   stage 0 (x lines):  z_i = wc*T + wxl*T[i-1] + wxh*T[i+1] + wyl*T[j-1] + wyh*T[j+1] + wzl*T[k-1]
//                             + wzh*T[k+1] + wq*Q - a0*z_{i-1};   W0_i = z_i - b0*W0_{i+1}
//   stage 1 (y lines):  z_j = W0_j - a1*z_{j-1};                   W1_j = z_j - b1*W1_{j+1}
//   stage 2 (z lines):  z_k = W1_k - a2*z_{k-1};                   dT_k = z_k - b2*dT_{k+1};  T' = T + dT
// The eight stage-0 stencil coefficients are chunk-blocked: for x-line L = k*ny + j and 32-column chunk ch,
// block (L*nchunks + ch) holds [wc, wxl, wxh, wyl, wyh, wzl, wzh, wq] x 32 columns (2 KB, zero-padded past
// nx), so a warp's stencil reads one contiguous stream instead of eight.  The other coefficients are
// (nz, ny, nx) arrays in voxel order, a1 and b1 (and the stage buffers W0, W1) with row pitch px.
constexpr int kXBlockCoeffs = 8;
enum XCoeff { kWc = 0, kWxl, kWxh, kWyl, kWyh, kWzl, kWzh, kWq };
struct Coeffs {
  double* xb;   // stage-0 stencil blocks, nz*ny*nchunks*8*32 doubles
  int64_t nchunks;
  // Row pitch of the arrays the y sweep moves with TMA tiles (W0, W1, a1, b1): nx, or nx rounded up so that
  // the rows start on 16-byte boundaries (an odd nx gets one pad column).  All other arrays have pitch nx.
  int64_t px;
  double* a0;
  double* b0;
  double* a1;
  double* b1;
  double* a2;
  double* b2;
};
constexpr int kNumCoeffArrays = 6;  // voxel-order arrays besides xb

struct QTable {
  double q[HS2G_MAX_CLASSES];
};

// Device-resident source schedule of a handle, read by the x sweep of a step with a source.  The host writes
// every field: the rows, their flags and the shape field when the schedule or the shapes change, `step` (the
// row of the next step with a source) before such a step is queued, `row` (the history row of the next step)
// at the start of a run; the history kernel then advances `row` after each step.
struct DevSchedule {
  const double* q;         // [n][HS2G_MAX_CLASSES] class source values (W/m^3)
  const uint8_t* active;   // [n] 1 when row s has a non-zero value
  const double* shape;     // per-voxel multiplier of the class sources, or null when no class has a shape
  int64_t n;               // rows; steps at or beyond n have no source
  int64_t step;
  int64_t row;
  unsigned int hist_done;  // CTAs of the current history kernel that have finished (the last one advances row)
};

// L2 eviction policies (createpolicy) and stores that carry one: evict-first for data streamed once, evict-last
// for a value the same thread block reads back soon (a sweep's forward values), and dropping a 128-byte line
// without writing it back (its contents are undefined until written again).
__device__ __forceinline__ uint64_t l2_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void st_hint(double* p, double v, uint64_t policy) {
  asm volatile("st.global.L2::cache_hint.f64 [%0], %1, %2;" ::"l"(p), "d"(v), "l"(policy) : "memory");
}
__device__ __forceinline__ void st_hint(float* p, float v, uint64_t policy) {
  asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(policy) : "memory");
}
__device__ __forceinline__ void l2_discard_line(const void* p) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
}

// Programmatic dependent launch inside the captured step graphs: a sweep launched with the attribute may be set
// up on the SMs while the sweep before it on the stream completes (no kernel triggers early, so that happens
// only once every CTA of the previous sweep has exited, and the CTAs of the new one spread over the whole GPU as
// in an ordinary launch).  Each sweep waits here, before it touches memory the previous one reads or writes,
// until that sweep has completed and its writes are visible.  A no-op in a kernel launched without the
// attribute.
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Kernel launch with the programmatic-serialization attribute when pdl is set (an ordinary launch otherwise).
template <typename... P, typename... A>
cudaError_t launch_kernel(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, bool pdl,
                          A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<A&&>(args)...);
}

// Record the message hs2g_last_error() returns for this thread (hs2g_api.cu); returns code.
int set_last_error(int code, const char* message);

// First error recorded by a device kernel: (code << 56) | (axis << 54) | index, 0 when none.
__device__ __forceinline__ void record_error(unsigned long long* err, int code, int axis, int64_t index) {
  unsigned long long v = ((unsigned long long)(-code) << 56) | ((unsigned long long)axis << 54) |
                         ((unsigned long long)index & ((1ull << 54) - 1));
  atomicCAS(err, 0ull, v);
}

// setup kernels (hs2g_compile.cu)
cudaError_t launch_faces(const Dims& d, int axis, const uint8_t* material, const uint8_t* bclass,
                         const hs2g_material* mats, int nmat, const hs2g_face_form* forms, int nbnd, double* G,
                         unsigned long long* err, cudaStream_t s);
cudaError_t launch_capacity_from_classes(const Dims& d, const uint8_t* material, const hs2g_material* mats,
                                         int nmat, double* M, uint8_t* compute, unsigned long long* err,
                                         cudaStream_t s);
cudaError_t launch_validate_dense(const Dims& d, const double* Gz, const double* Gy, const double* Gx,
                                  double* M, uint8_t* compute, unsigned long long* err, cudaStream_t s);
cudaError_t launch_factor(const Dims& d, const double* Gz, const double* Gy, const double* Gx, const double* M,
                          const uint8_t* compute, double* s2, double* sigma, const Coeffs& c, cudaStream_t s);
// per-row problems: rows = {z lo, z hi, y lo, y hi, x lo, x hi}, each (nz, ny, nx)
cudaError_t launch_validate_rows(const Dims& d, const double* const rows[6], double* M, uint8_t* compute,
                                 unsigned long long* err, cudaStream_t s);
cudaError_t launch_factor_rows(const Dims& d, const double* const rows[6], const double* M, const uint8_t* compute,
                               double* s2, double* sigma, const Coeffs& c, cudaStream_t s);

// per-voxel source shapes (hs2g_sources.cu)
cudaError_t launch_fill(double* p, int64_t n, double v, cudaStream_t s);
cudaError_t launch_zdecay_shape(int64_t n, const uint8_t* vclass, int cls, const double* zgrid, double direction,
                                double offset, double ddz, double jpm2, double length, double dt, double* shape,
                                cudaStream_t s);
int64_t point_shape_tiles(int64_t n);
cudaError_t launch_point_shape(int64_t n, const uint8_t* vclass, int cls, int64_t* tile_scratch, const double* joules,
                               int64_t count, const double* volumes, double volume, double dt, double* shape,
                               cudaStream_t s);

// step kernels (hs2g_sweep.cu)
struct StepArgs {
  Dims d;
  const double* T_in;
  double* T_out;
  double* W0;
  double* W1;
  const uint8_t* vclass;
  const double* qdense;  // may be null
  const double* qshape;  // per-voxel multiplier of the class sources (null: 1 everywhere)
  bool has_qtab;
  int* status;           // device word: 0, or HS2G_ERR_TIMEOUT when a bounded wait in a kernel ran out
  bool bulk_y, bulk_z;   // use the TMA tensor-tile line sweeps (hs2g_lines.cu) for y / z
  bool z_discard;        // the plain z sweep drops its forward values from L2 after reading them
  struct TensorMapCache* tmaps;
  bool pdl;              // launch the y and z sweeps with programmatic dependent launch (captured step graphs)
  bool pdl_x;            // the same for the x sweep (not for the first kernel of a graph)
};

// TMA tensor-tile line sweeps (hs2g_lines.cu); axis 1 = y, 2 = z.
struct TensorMapCache;
TensorMapCache* tensor_map_cache_create();
void tensor_map_cache_destroy(TensorMapCache* c);
bool lines_bulk_supported(const Dims& d, int axis, int64_t px);
cudaError_t lines_bulk_prepare();
// axis 1 (y): A, alpha, scratch, beta and out have row pitch px; axis 2 (z): every array has pitch nx (px = nx)
cudaError_t launch_lines_bulk(const Dims& d, int axis, const double* A, const double* alpha, double* scratch,
                              const double* beta, const double* T_in, double* out, int* status,
                              TensorMapCache* cache, cudaStream_t s, int64_t px, bool pdl = false);
cudaError_t launch_step(const StepArgs& a, const Coeffs& c, const QTable& q, cudaStream_t s);
// the same three kernels with an event recorded before each and after the last (ev[0..3])
cudaError_t launch_step_events(const StepArgs& a, const Coeffs& c, const QTable& q, cudaStream_t s,
                               cudaEvent_t ev[4]);
// One step whose class sources are row ds->step of the device schedule (no source when that row is inactive or
// past the schedule's end): the x sweep reads the row on the device.  Used for the steps with a source in the
// captured step graphs of hs2g_run; the steps without one use launch_step with no table.
cudaError_t launch_step_row(const StepArgs& a, const Coeffs& c, const DevSchedule* ds, cudaStream_t s);
// History of the step just taken into hist[ds->row][ny][nx]: layer `layer` of T (dz2 <= 0) or the insulating
// z = 0 surface estimate from layers 0 and 1 with dz2 = dz**2 (dz2 > 0); the kernel's last CTA advances
// ds->row.
cudaError_t launch_history_row(const Dims& d, const double* T, int layer, double dz2, double* hist, DevSchedule* ds,
                               cudaStream_t s, bool pdl = false);
// the reference's dz**2.0 (the C library's pow)
double surface_dz2(double dz);
// one flag per schedule row: active[s] = any of q[s][0..nclass-1] non-zero
cudaError_t launch_schedule_flags(const double* q, int64_t nrows, uint8_t* active, cudaStream_t s);
cudaError_t fp64_fma_rate(double* fma_per_s);
cudaError_t launch_copy_layer(const Dims& d, const double* T, int layer, double* dst, cudaStream_t s);
// insulating z = 0 surface temperature from layers 0 and 1 of T (an nxy-element plane each) into dst[nxy]
cudaError_t launch_surface_estimate(int64_t nxy, const double* T, double dz, double* dst, cudaStream_t s);
// one bounded mbarrier wait on a barrier that receives its arrival (arrive != 0) or none (hs2g_lines.cu)
cudaError_t wait_selftest(uint64_t limit_ns, int arrive, int* status_dev, cudaStream_t s);
// the step in pieces, for overlapping host copies with it: the x sweep over x-lines [line_begin, line_end)
// (line = k*ny + j) with 32, 16 or 8 x-lines per CTA, the whole y sweep, the plain z sweep over columns
// [col_begin, col_end) (col = j*nx + i)
cudaError_t launch_x_range(const StepArgs& a, const Coeffs& c, const QTable& q, int64_t line_begin,
                           int64_t line_end, int lines_per_cta, cudaStream_t s);
cudaError_t launch_y(const StepArgs& a, const Coeffs& c, cudaStream_t s);
cudaError_t launch_z_range(const StepArgs& a, const Coeffs& c, int64_t col_begin, int64_t col_end, cudaStream_t s);

}  // namespace hs2g
