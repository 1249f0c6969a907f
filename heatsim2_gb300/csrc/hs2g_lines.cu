// y and z sweeps with TMA tensor-tile prefetch.
//
// A y or z line sweep is a first-order recurrence down each line, forward (z_r = A_r - alpha_r z_{r-1}) then
// back (x_r = Z_r - beta_r x_{r+1}).  One thread owns one line; the 64 lines of a CTA are 64 consecutive
// elements of a row, so a box of kRows consecutive rows x 64 lines of any array is one 2-D tile of the
// (nz, ny, nx) array (y sweep: rows along y at fixed z; z sweep: rows along z of the flattened (z, y*x) view).
// With one FMA per element the sweep is bound by bytes in flight, so one thread (the producer) keeps kSlots
// tiles of every input array in flight with cp.async.bulk.tensor copies, each slot's copies completing on the
// slot's mbarrier (transaction count = tile bytes).  All threads wait on the slot, run the recurrence down
// its rows and store their elements of the output rows directly.  Rows outside the array (the last tile of a
// line, or the first tile of the back sweep) are zero-filled by the TMA unit and never stored.
//
// Every mbarrier wait is bounded by %globaltimer (kWaitNs).  A wait that runs out sets the CTA's abort flag;
// the CTA then stops, its producer waits (again bounded) for the copies it still has in flight, and the
// kernel reports HS2G_ERR_TIMEOUT through the status word.
//
// Requirements (checked on the host, which otherwise uses the plain kernels of hs2g_sweep.cu): arrays
// 16-byte aligned and row pitches even, so every global stride is a multiple of 16 B.  The y sweep's arrays are
// allocated with an even row pitch px (one pad column for an odd nx); the z sweep needs ny*nx even.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

#include "hs2g_internal.cuh"
#include "hs2g_ring.h"

namespace hs2g {
namespace {

constexpr int kNL = 64;        // lines per CTA (threads)
constexpr int kRows = 16;      // rows per tile
constexpr int kSlots = 2;      // tiles in flight per array (32 KB of shared memory per y CTA, so all 520
                               // CTAs of a 65 x 512 x 512 y sweep are resident at once: 119.5 us, against
                               // 129.5 us with 6 slots of 8 rows and 122 us with 4 slots of 8 rows)
constexpr uint64_t kWaitNs = 2000000000ull;
constexpr uint32_t kTileBytes = kNL * kRows * 8;

__device__ __forceinline__ uint32_t saddr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(saddr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(saddr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(saddr(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns = kWaitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t deadline = now_ns() + limit_ns;
  while (!mbar_try_wait(bar, parity))
    if (now_ns() > deadline) return false;
  return true;
}
// Self-test of the bounded wait: one thread waits, for at most limit_ns, on an mbarrier that expects one
// arrival, which it makes itself (arrive != 0) or which never comes.  A wait that gives up reports
// HS2G_ERR_TIMEOUT through the status word, as a sweep whose copies never complete does; nothing is in
// flight, so the kernel ends cleanly either way.
__global__ void wait_selftest_kernel(uint64_t limit_ns, int arrive, int* status) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  if (arrive) mbar_arrive(&bar);
  *status = mbar_wait_bounded(&bar, 0, limit_ns) ? HS2G_OK : HS2G_ERR_TIMEOUT;
}

// 3-D tile load (x = line index within the row, y = row, z = plane); coordinates may lie outside the array.
// HINT: the copy carries an L2 cache policy (evict-first for data read for the last time in the step).
template <bool HINT = false>
__device__ __forceinline__ void tile_load(void* dst, const CUtensorMap* map, int c0, int c1, int c2, uint64_t* bar,
                                          uint64_t policy = 0) {
  if (HINT)
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint [%0], "
        "[%1, {%2, %3, %4}], [%5], %6;" ::"r"(saddr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(saddr(bar)), "l"(policy)
        : "memory");
  else
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(saddr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(saddr(bar))
        : "memory");
}
// store of a value the same kernel reads back soon (the forward sweep's scratch): kept in L2 with HINT
template <bool HINT>
__device__ __forceinline__ void st_keep(double* p, double v, uint64_t policy) {
  if (HINT)
    st_hint(p, v, policy);
  else
    *p = v;
}

struct Geometry {
  int64_t groups;        // CTAs per plane
  int64_t plane_stride;  // element offset between planes (y sweep: ny*nx, z sweep: 0)
  int64_t width;         // lines per plane (y sweep: nx, z sweep: ny*nx)
  int64_t stride;        // element offset between consecutive rows of a line
  int64_t nrows;         // line length
};

template <bool ADD_T>
__host__ __device__ constexpr int num_arrays() {
  return ADD_T ? 3 : 2;
}

template <bool ADD_T, int SLOTS = kSlots>
__host__ __device__ constexpr size_t smem_bytes() {
  return 128 /*alignment slack*/ + (size_t)SLOTS * num_arrays<ADD_T>() * kTileBytes + 8 * SLOTS + 16;
}

// Forward inputs A, alpha -> scratch; back inputs scratch, beta (and T_in when ADD_T) -> out.
// out may equal scratch (y sweep writes W1 in place) and T_in may equal out (in-place timestep).
template <bool ADD_T, bool HINT = false, int kSlots = hs2g::kSlots>
__global__ void __launch_bounds__(kNL) line_sweep_tma_kernel(Geometry g, const __grid_constant__ CUtensorMap mA,
                                                             const __grid_constant__ CUtensorMap mAlpha,
                                                             const __grid_constant__ CUtensorMap mScratch,
                                                             const __grid_constant__ CUtensorMap mBeta,
                                                             const __grid_constant__ CUtensorMap mT, double* scratch,
                                                             double* out, int* status) {
  constexpr int NA = num_arrays<ADD_T>();
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base_ptr = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  double* tiles = reinterpret_cast<double*>(base_ptr);
  uint64_t* bars = reinterpret_cast<uint64_t*>(base_ptr + (size_t)kSlots * NA * kTileBytes);
  int* abort_flag = reinterpret_cast<int*>(bars + kSlots);

  const int tid = threadIdx.x;
  const int64_t plane = blockIdx.x / g.groups;
  const int64_t i0 = (blockIdx.x - plane * g.groups) * kNL;
  const int w = (int)min((int64_t)kNL, g.width - i0);
  const int64_t base = plane * g.plane_stride + i0;
  const int64_t n = g.nrows;
  const int64_t ntiles = (n + kRows - 1) / kRows;
  auto tile = [&](int s, int arr) { return tiles + ((int64_t)s * NA + arr) * (kNL * kRows); };

  if (tid == 0) {
    // fetch the tensor-map descriptors while the barriers are set up (the first copies would wait for them)
    asm volatile("prefetch.tensormap [%0];" ::"l"(&mA) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&mAlpha) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&mScratch) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(&mBeta) : "memory");
    if (ADD_T) asm volatile("prefetch.tensormap [%0];" ::"l"(&mT) : "memory");
    for (int s = 0; s < kSlots; ++s) mbar_init(&bars[s], 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  wait_prior_grid();  // the inputs come from the previous sweep; the outputs overwrite what it read
  __syncthreads();

  SlotRing ring;  // slot phases; pending slots are tracked by the producer (tid 0), which issues every copy
  const int cx = (int)i0, cz = (int)plane;
  const uint64_t pol_first = HINT ? l2_evict_first() : 0;
  const uint64_t pol_last = HINT ? l2_evict_last() : 0;

  auto issue_fwd = [&](int64_t q) {  // tile q covers rows [q*kRows, q*kRows + kRows)
    const int s = (int)(q % kSlots);
    const int r0 = (int)(q * kRows);
    mbar_expect_tx(&bars[s], 2u * kTileBytes);
    tile_load<HINT>(tile(s, 0), &mA, cx, r0, cz, &bars[s], pol_first);
    tile_load<HINT>(tile(s, 1), &mAlpha, cx, r0, cz, &bars[s], pol_first);
    ring.issued(s);
  };
  auto issue_back = [&](int64_t q) {  // back tile q covers rows [n - (q+1)*kRows, n - q*kRows)
    const int s = (int)(q % kSlots);
    const int r0 = (int)(n - (q + 1) * kRows);
    mbar_expect_tx(&bars[s], (uint32_t)NA * kTileBytes);
    tile_load<HINT>(tile(s, 0), &mScratch, cx, r0, cz, &bars[s], pol_first);
    tile_load<HINT>(tile(s, 1), &mBeta, cx, r0, cz, &bars[s], pol_first);
    if (ADD_T) tile_load<HINT>(tile(s, 2), &mT, cx, r0, cz, &bars[s], pol_first);
    ring.issued(s);
  };

  bool aborted = false;
  // ---- forward ----
  if (tid == 0)
    for (int64_t q = 0; q < min(ntiles, (int64_t)kSlots); ++q) issue_fwd(q);
  double z = 0.0;
  for (int64_t q = 0; q < ntiles && !aborted; ++q) {
    const int s = (int)(q % kSlots);
    const bool done = mbar_wait_bounded(&bars[s], ring.phase(s));
    if (!done) *abort_flag = 1;
    ring.waited(s, done);
    const double* tA = tile(s, 0);
    const double* tAl = tile(s, 1);
    const int64_t r0 = q * kRows;
    const int nr = (int)min((int64_t)kRows, n - r0);
    if (tid < w) {
      double* dst = scratch + base + r0 * g.stride + tid;
#pragma unroll
      for (int rr = 0; rr < kRows; ++rr) {
        if (rr < nr) {
          z = fma(-tAl[rr * kNL + tid], z, tA[rr * kNL + tid]);
          st_keep<HINT>(dst + rr * g.stride, z, pol_last);
        }
      }
    }
    __syncthreads();
    aborted = *abort_flag != 0;
    if (!aborted && tid == 0 && q + kSlots < ntiles) issue_fwd(q + kSlots);
  }
  // the back sweep reads the forward values through the async proxy: order the generic stores before it
  asm volatile("fence.proxy.async.global;" ::: "memory");
  __syncthreads();
  // ---- back ----
  if (!aborted && tid == 0)
    for (int64_t q = 0; q < min(ntiles, (int64_t)kSlots); ++q) issue_back(q);
  double x = 0.0;
  for (int64_t q = 0; q < ntiles && !aborted; ++q) {
    const int s = (int)(q % kSlots);
    const bool done = mbar_wait_bounded(&bars[s], ring.phase(s));
    if (!done) *abort_flag = 1;
    ring.waited(s, done);
    const double* tZ = tile(s, 0);
    const double* tB = tile(s, 1);
    const double* tT = tile(s, ADD_T ? 2 : 0);
    const int64_t r0 = n - (q + 1) * kRows;  // may be negative for the last tile
    if (tid < w) {
#pragma unroll
      for (int rr = kRows - 1; rr >= 0; --rr) {
        const int64_t r = r0 + rr;
        if (r >= 0) {
          x = fma(-tB[rr * kNL + tid], x, tZ[rr * kNL + tid]);
          out[base + r * g.stride + tid] = ADD_T ? tT[rr * kNL + tid] + x : x;
        }
      }
    }
    __syncthreads();
    aborted = *abort_flag != 0;
    if (!aborted && tid == 0 && q + kSlots < ntiles) issue_back(q + kSlots);
  }
  if (aborted && tid == 0) {
    // drain: wait (bounded) for every copy still in flight into this CTA's shared memory, including a slot
    // whose wait above gave up (its phase was not advanced)
    for (int s = 0; s < kSlots; ++s)
      if (ring.in_flight(s)) mbar_wait_bounded(&bars[s], ring.phase(s));
    atomicExch(status, HS2G_ERR_TIMEOUT);
  }
}

// ---- host: tensor maps -----------------------------------------------------------------------------------
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, []() {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// (nz, ny, nx) array seen as rows of lines: y sweep {x: nx, y: ny, z: nz} with row pitch px (px >= nx, the
// columns past nx never read), z sweep {x: ny*nx, y: nz, z: 1}
bool encode(CUtensorMap* m, const Dims& d, int axis, const void* ptr, int64_t px) {
  PFN_cuTensorMapEncodeTiled_v12000 fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3], strides[2];
  if (axis == 1) {
    dims[0] = (cuuint64_t)d.nx;
    dims[1] = (cuuint64_t)d.ny;
    dims[2] = (cuuint64_t)d.nz;
    strides[0] = (cuuint64_t)px * 8;
    strides[1] = (cuuint64_t)(d.ny * px) * 8;
  } else {
    dims[0] = (cuuint64_t)d.nxy();
    dims[1] = (cuuint64_t)d.nz;
    dims[2] = 1;
    strides[0] = (cuuint64_t)d.nxy() * 8;
    strides[1] = (cuuint64_t)d.nvox() * 8;
  }
  const cuuint32_t box[3] = {(cuuint32_t)kNL, (cuuint32_t)kRows, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, const_cast<void*>(ptr), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

// Per-handle cache of encoded tensor maps, keyed by (array pointer, axis).
struct TensorMapCache {
  std::map<std::pair<const void*, int>, CUtensorMap> maps;
  bool get(const Dims& d, int axis, const void* ptr, int64_t px, CUtensorMap* out) {
    auto key = std::make_pair(ptr, axis);  // one pitch per handle, so the pointer and axis identify the map
    auto it = maps.find(key);
    if (it == maps.end()) {
      CUtensorMap m;
      if (!encode(&m, d, axis, ptr, px)) return false;
      if (maps.size() > 64) maps.clear();
      it = maps.emplace(key, m).first;
    }
    *out = it->second;
    return true;
  }
};

TensorMapCache* tensor_map_cache_create() { return new TensorMapCache(); }
void tensor_map_cache_destroy(TensorMapCache* c) { delete c; }

bool lines_bulk_supported(const Dims& d, int axis, int64_t px) {
  if (!encode_fn()) return false;
  if (axis == 1) return (px % 2 == 0) && px < (1ll << 31) && d.ny < (1ll << 31) && d.nz < (1ll << 31);
  return (d.nxy() % 2 == 0) && d.nxy() < (1ll << 31) && d.nz < (1ll << 31);
}

// Raise the dynamic shared-memory limit of the tile kernels on the current device (once per device, before
// the first launch; called when a handle is created).
cudaError_t lines_bulk_prepare() {
  cudaError_t e = cudaFuncSetAttribute(line_sweep_tma_kernel<false, true>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes<false>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(line_sweep_tma_kernel<false, true, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_bytes<false, 3>());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(line_sweep_tma_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem_bytes<true>());
  return e;
}

cudaError_t launch_lines_bulk(const Dims& d, int axis, const double* A, const double* alpha, double* scratch,
                              const double* beta, const double* T_in, double* out, int* status,
                              TensorMapCache* cache, cudaStream_t s, int64_t px, bool pdl) {
  if (!aligned16(A) || !aligned16(alpha) || !aligned16(scratch) || !aligned16(beta) || !aligned16(out) ||
      (T_in && !aligned16(T_in)) || !cache)
    return cudaErrorMisalignedAddress;
  CUtensorMap mA, mAl, mS, mB, mT;
  if (axis != 1) px = d.nx;
  const bool ok = cache->get(d, axis, A, px, &mA) && cache->get(d, axis, alpha, px, &mAl) &&
                  cache->get(d, axis, scratch, px, &mS) && cache->get(d, axis, beta, px, &mB) &&
                  (T_in ? cache->get(d, axis, T_in, px, &mT) : cache->get(d, axis, A, px, &mT));
  if (!ok) return cudaErrorInvalidValue;
  Geometry g;
  if (axis == 1) {
    g.groups = (d.nx + kNL - 1) / kNL;
    g.plane_stride = d.ny * px;
    g.width = d.nx;
    g.stride = px;
    g.nrows = d.ny;
    const char* slots = getenv("HS2G_Y_SLOTS");
    if (slots && strcmp(slots, "3") == 0)
      return launch_kernel(line_sweep_tma_kernel<false, true, 3>, dim3((unsigned)(d.nz * g.groups)), dim3(kNL),
                           smem_bytes<false, 3>(), s, pdl, g, mA, mAl, mS, mB, mT, scratch, out, status);
    return launch_kernel(line_sweep_tma_kernel<false, true>, dim3((unsigned)(d.nz * g.groups)), dim3(kNL),
                         smem_bytes<false>(), s, pdl, g, mA, mAl, mS, mB, mT, scratch, out, status);
  } else {
    g.groups = (d.nxy() + kNL - 1) / kNL;
    g.plane_stride = 0;
    g.width = d.nxy();
    g.stride = d.nxy();
    g.nrows = d.nz;
    return launch_kernel(line_sweep_tma_kernel<true>, dim3((unsigned)g.groups), dim3(kNL), smem_bytes<true>(), s, pdl,
                         g, mA, mAl, mS, mB, mT, scratch, out, status);
  }
}


cudaError_t wait_selftest(uint64_t limit_ns, int arrive, int* status_dev, cudaStream_t s) {
  wait_selftest_kernel<<<1, 32, 0, s>>>(limit_ns, arrive, status_dev);
  return cudaGetLastError();
}

}  // namespace hs2g
