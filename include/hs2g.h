/*
 * hs2g -- GB300-native ADI Crank-Nicolson heat-conduction timestep (heatsim2's hot path), C ABI.
 *
 * This is the native boundary that replaces the reference's Cython extension modules
 * (heatsim2/alternatingdirection_c_pyx.pyx, heatsim2/crank_nicolson.pyx, heatsim2/tridiag.pyx) and its
 * hand-written C assembler (heatsim2/alternatingdirection_c.h:50-54).  Plain pointers and sizes only; the
 * library owns every device allocation it makes, the caller owns every buffer it passes in.
 *
 * Conventions
 *   - every entry point returns HS2G_OK (0) or a negative HS2G_ERR_* code and never exits or aborts
 *     (the reference's add_equation calls exit(1) on an out-of-domain stencil, alternatingdirection_c.c:160-163);
 *     hs2g_last_error() describes the last failure of the calling thread;
 *   - arrays are C-contiguous, z slowest and x fastest: T[k][j][i] with shape (nz, ny, nx), z faces
 *     (nz+1, ny, nx), y faces (nz, ny+1, nx), x faces (nz, ny, nx+1) (heatsim2/__init__.py:191-197);
 *   - a handle is used by one host thread at a time; distinct handles may be used concurrently;
 *   - work is queued on the handle's stream (hs2g_set_stream); HS2G_SYNC waits for it before returning.
 */
#ifndef HS2G_H
#define HS2G_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HS2G_ABI_VERSION 1

#define HS2G_OK 0
#define HS2G_ERR_ARG (-1)        /* bad argument (shape, pointer, class index out of range) */
#define HS2G_ERR_CUDA (-2)       /* a CUDA runtime call failed */
#define HS2G_ERR_NOMEM (-3)      /* device or pinned-host allocation failed */
#define HS2G_ERR_EXTERIOR (-4)   /* a compute voxel has a non-insulating face on the grid's exterior */
#define HS2G_ERR_KTYPE (-5)      /* a boundary class needs scalar k but the material has a matrix, or reverse */
#define HS2G_ERR_UNALIGNED (-6)  /* a face flux couples across axes (anisotropy not aligned with the grid) */
#define HS2G_ERR_FORM (-7)       /* a face flux is not a conservative Crank-Nicolson two-point difference */
#define HS2G_ERR_CAPACITY (-8)   /* a computed voxel has rho*c/dt <= 0 or not finite */
#define HS2G_ERR_STATE (-9)      /* handle not in a state that allows this call */
#define HS2G_ERR_TIMEOUT (-10)   /* a bounded wait inside a kernel ran out; the step's output is invalid */

/* flags */
#define HS2G_DEVICE 1            /* T_in / T_out / qdense / history are device pointers (no copies) */
#define HS2G_SYNC 2              /* synchronise the handle's stream before returning */
#define HS2G_REUSE 4             /* hs2g_source_*: use the device copy of the per-voxel array kept from the
                                    previous call for the same class (the caller's array is unchanged) */
#define HS2G_SCHEDULED 8         /* hs2g_run: class sources from the handle's device schedule at its clock */

/* material kinds (heatsim2/__init__.py:42-43) */
#define HS2G_TEMPERATURE_COMPUTE 0
#define HS2G_TEMPERATURE_FIXED 1

/* source kinds evaluated per class by hs2g_source_table (heatsim2/__init__.py:46-50) */
#define HS2G_NO_SOURCE 0
#define HS2G_IMPULSE_SOURCE 1
#define HS2G_STEPPED_SOURCE 2
#define HS2G_IMPULSE_POINT_SOURCE_JOULES 3
/* a class whose per-voxel values come from the handle's source shape (hs2g_source_zdecay, hs2g_source_point):
   hs2g_source_table gives it 1 at t == params[0] exactly and 0 otherwise (no kind of this number in the
   reference, whose numpy loop evaluates these sources on every call, alternatingdirection_c_pyx.pyx:307-384) */
#define HS2G_SHAPED_IMPULSE 5

/*
 * A face flux coefficient as an affine form in the conductivity entries of the two materials that meet at the
 * face (after the reference's neighbour-k fallback, crank_nicolson.pyx:298-338):
 *     value = f[0] + sum_e f[1+e] * k_lo[e] + sum_e f[1+HS2G_K_ENTRIES+e] * k_hi[e]
 * k entry 0 is a scalar conductivity, entries 1..9 the 3x3 tensor (row-major, z,y,x order).  A material holds
 * NaN in the representation it does not have; a form with a non-zero coefficient on such an entry raises
 * HS2G_ERR_KTYPE for the faces that use it.
 */
#define HS2G_K_ENTRIES 10
#define HS2G_FORM_LEN (1 + 2 * HS2G_K_ENTRIES)
#define HS2G_MAX_ZERO_FORMS 24
#define HS2G_MAX_CLASSES 256

typedef struct {
  int32_t kind;                     /* HS2G_TEMPERATURE_COMPUTE / _FIXED */
  double k[HS2G_K_ENTRIES];         /* scalar k in k[0] or tensor in k[1..9]; NaN where absent */
  double capacity;                  /* rho * c * (1/dt) in W/m^3/K (crank_nicolson.pyx:378) */
} hs2g_material;

/*
 * A boundary class evaluated on one axis (0 = z, 1 = y, 2 = x): the heat-balance conductance of the face,
 * G (W/m^3/K) = normal . [1, k_lo, k_hi], i.e. the flux divided by the cell size is -G * (T_hi - T_lo)
 * (crank_nicolson.pyx:359-363).  zero[z] are forms that must vanish on every face that uses the class
 * (cross-axis terms, unbalanced two-point terms, terms outside a Crank-Nicolson group, constant fluxes);
 * zero_code[z] is the HS2G_ERR_* raised when one does not.
 */
typedef struct {
  double normal[HS2G_FORM_LEN];
  int32_t nzero;
  int32_t zero_code[HS2G_MAX_ZERO_FORMS];
  double zero[HS2G_MAX_ZERO_FORMS][HS2G_FORM_LEN];
} hs2g_face_form;

/* Problem described by class arrays: what heatsim2.setup receives (crank_nicolson.pyx:128-142). */
typedef struct {
  int64_t nz, ny, nx;
  int32_t nmat, nbnd;
  const hs2g_material* materials;   /* [nmat] */
  const hs2g_face_form* forms;      /* [nbnd][3] */
  const uint8_t* material;          /* (nz, ny, nx) */
  const uint8_t* boundary_z;        /* (nz+1, ny, nx) */
  const uint8_t* boundary_y;        /* (nz, ny+1, nx) */
  const uint8_t* boundary_x;        /* (nz, ny, nx+1) */
  const uint8_t* volumetric;        /* (nz, ny, nx) source class of each voxel */
} hs2g_class_problem;

/* Problem described by per-face conductances and per-voxel capacities (continuous, per-voxel k / rho*c).
   Faces of fixed voxels are ignored; exterior faces of computed voxels must be zero. */
typedef struct {
  int64_t nz, ny, nx;
  const double* Gz;                 /* (nz+1, ny, nx) W/m^3/K */
  const double* Gy;                 /* (nz, ny+1, nx) */
  const double* Gx;                 /* (nz, ny, nx+1) */
  const double* capacity;           /* (nz, ny, nx) rho*c/dt, W/m^3/K */
  const uint8_t* fixed;             /* (nz, ny, nx) 1 = fixed temperature, or NULL for none */
  const uint8_t* volumetric;        /* (nz, ny, nx) source classes, or NULL for class 0 everywhere */
} hs2g_dense_problem;

/* Problem described by per-row face conductances: for every voxel, the conductance of each of its six faces
   as that voxel's own heat balance weighs it (W/m^3/K), so the two rows of a face may differ.  This is the
   reference's curved-surface mode (crank_nicolson.pyx:388-457) after each row is divided by its cell volume:
   face areas and edge lengths follow the cell's depth and the surface curvature.  Exterior sides of computed
   voxels must be zero. */
typedef struct {
  int64_t nz, ny, nx;
  const double* zlo;                /* (nz, ny, nx) each: the low and high face of every voxel on z, y, x */
  const double* zhi;
  const double* ylo;
  const double* yhi;
  const double* xlo;
  const double* xhi;
  const double* capacity;           /* (nz, ny, nx) rho*c/dt */
  const uint8_t* fixed;             /* (nz, ny, nx) 1 = fixed temperature, or NULL for none */
  const uint8_t* volumetric;        /* (nz, ny, nx) source classes, or NULL for class 0 everywhere */
} hs2g_rows_problem;

typedef struct hs2g_handle hs2g_handle;

int hs2g_abi_version(void);
const char* hs2g_last_error(void);

/* Compile a problem onto device `device` (replaces setup's voxel loop and per-stage assembly + LU:
   crank_nicolson.pyx:272-496, alternatingdirection_c.c:56-199 create_adi_step/add_equation,
   alternatingdirection_c_pyx.pyx:212-282 finalize, tridiag.pyx:9-43 tridiaglu). */
int hs2g_create_classes(const hs2g_class_problem* problem, int device, hs2g_handle** out);
int hs2g_create_dense(const hs2g_dense_problem* problem, int device, hs2g_handle** out);
int hs2g_create_rows(const hs2g_rows_problem* problem, int device, hs2g_handle** out);
/* Free every device buffer of the handle (replaces delete_adi_step, alternatingdirection_c.c:14-54). */
void hs2g_destroy(hs2g_handle* h);

/* Queue subsequent work on `stream` (a cudaStream_t; NULL = the CUDA legacy default stream, as everywhere in
   CUDA).  A new handle uses a non-blocking stream of its own until this is called. */
int hs2g_set_stream(hs2g_handle* h, void* stream);
int hs2g_shape(const hs2g_handle* h, int64_t shape[3]);

/*
 * One timestep T_out = ADI(T_in) (replaces run_adi_steps' stage loop, alternatingdirection_c_pyx.pyx:387-416,
 * and tridiagsolve, tridiag.pyx:46-69).
 *   qtab      host array of HS2G_MAX_CLASSES source values (W/m^3) per volumetric class for this step,
 *             or NULL when no class source is active;
 *   qdense    per-voxel source added to the class sources (W/m^3), or NULL;
 *   volumetric  replacement (nz,ny,nx) source-class map (host), or NULL to keep the current one.
 * T_out may equal T_in.  Fixed-temperature voxels keep T_in.
 */
int hs2g_step(hs2g_handle* h, const double* T_in, double* T_out, const double* qtab, const double* qdense,
              const uint8_t* volumetric, int flags);

/*
 * nsteps timesteps on the device (replaces the reference's run_adi_steps loop over a run's times,
 * alternatingdirection_c_pyx.pyx:387-416).  After the first step (queued directly when T_in != T_out) the steps
 * are replays of captured CUDA graphs of the in-place step: a step whose schedule row has a source replays a
 * one-step graph whose x sweep reads that row of the handle's device schedule (hs2g_set_schedule) on the
 * device, and runs of steps without one replay a graph of four steps (or one); graphs are kept per (T buffer,
 * history buffer, layer) and reused by later calls.
 *   qtabs  host array [nsteps][HS2G_MAX_CLASSES] of per-step class sources: replaces the handle's schedule
 *          (as hs2g_set_schedule with these rows, clock 0) before the steps; or NULL: with HS2G_SCHEDULED the
 *          steps take rows from the schedule already set, from its clock on (rows past its end: no source),
 *          and without it no class source.
 * When history is not NULL, the layer z = record_layer of T after every step is written to
 * history[nsteps][ny][nx].
 */
int hs2g_run(hs2g_handle* h, int nsteps, const double* T_in, double* T_out, const double* qtabs,
             int record_layer, double* history, int flags);

/*
 * hs2g_run recording, after every step, the temperature of the z = 0 surface as the reference's
 * insulating_z_min_surface_temperature(T, dz) estimates it from layers 0 and 1 (heatsim2/surface_temperature.py:4-36;
 * the reference evaluates it in numpy on each step's returned T): history[nsteps][ny][nx].  Needs nz >= 2 and
 * dz > 0 (m, the layers' thickness).
 */
int hs2g_run_surface(hs2g_handle* h, int nsteps, const double* T_in, double* T_out, const double* qtabs, double dz,
                     double* history, int flags);

/*
 * The same surface estimate of one (nz, ny, nx) temperature field, no handle needed: out[ny][nx] from T's layers
 * 0 and 1 on `device`, on `stream` (NULL: the default stream).  With HS2G_DEVICE T and out are device pointers
 * and the call returns after queuing (unless HS2G_SYNC); otherwise host pointers, copied through temporary
 * device buffers, and the call synchronises.
 */
int hs2g_surface_temperature(int device, int64_t nz, int64_t ny, int64_t nx, const double* T, double dz,
                             double* out, void* stream, int flags);

/*
 * hs2g_run without history, timing each sweep kernel with CUDA events on the handle's stream.
 * kernel_ms[0..2] receive the summed device time of the x, y and z sweeps over the nsteps steps and
 * kernel_ms[3] the device time from the first event to the last.  Takes device pointers (HS2G_DEVICE).
 */
int hs2g_run_timed(hs2g_handle* h, int nsteps, const double* T_in, double* T_out, const double* qtabs, int flags,
                   double* kernel_ms);

/* Measured FP64 fused-multiply-add issue rate of `device` (FMA/s): a register-only kernel with 8 independent
   chains per thread on every SM, timed with CUDA events.  The FP64 roofline denominator for the sweeps. */
int hs2g_fp64_fma_rate(int device, double* fma_per_s);

/* Per-class source values at time t (alternatingdirection_c_pyx.pyx:294-319 for the class-uniform kinds):
   kind[c] in HS2G_*_SOURCE, params[c*4 .. c*4+3] = the tuple's numbers after the kind;
   volume = dz*dy*dx for IMPULSE_POINT_SOURCE_JOULES.  Writes qtab[0..HS2G_MAX_CLASSES-1]; returns the
   number of classes with a non-zero value (>= 0) or an error. */
int hs2g_source_table(int nsrc, const int32_t* kind, const double* params, double t, double dt, double volume,
                      double* qtab);

/*
 * Device-resident source schedule of a handle (the batched form's hs2g_batch_set_sources for one problem):
 * qtabs[nsteps][HS2G_MAX_CLASSES] class source values (W/m^3) for steps 0 .. nsteps-1, a host array or, with
 * HS2G_DEVICE, a device array, copied on the handle's stream.  One flag per row (any non-zero value) is kept on
 * the host, from which hs2g_run picks each step's graph: for device rows the call computes them on the device
 * and waits for the stream to read them back.  Sets the clock to 0; a
 * scheduled step takes row `clock` (none when clock >= nsteps; nsteps = 0 clears the schedule) and advances the
 * clock.  Row values multiply the per-voxel source shapes as hs2g_step's qtab does (hs2g_source_zdecay /
 * hs2g_source_point, as they stand when the run is queued).  Steps queued earlier read the rows they were
 * queued with.
 */
int hs2g_set_schedule(hs2g_handle* h, int64_t nsteps, const double* qtabs, int flags);
/* Set or read the schedule clock: the row of the next scheduled step, counted by the steps queued (no device
   work). */
int hs2g_set_clock(hs2g_handle* h, int64_t step);
int hs2g_get_clock(hs2g_handle* h, int64_t* step);

/*
 * Per-voxel source shapes: the source kinds whose value differs between the voxels of a class are evaluated on
 * the device into a per-voxel multiplier S of the handle (1 for every voxel not given a shape).  On every step
 * the x sweep adds table[class] * S to each voxel's source, so a class given a shape and a table value of 1 on
 * its firing step (HS2G_SHAPED_IMPULSE) receives exactly the shape's values, and class-uniform sources are
 * unchanged.  A shape is written for the voxels of its class in the handle's current source-class map; a new
 * map (hs2g_set_source_classes, or hs2g_step's volumetric argument) resets S to 1 and drops every shape.
 * Arrays are host pointers (copied into a device buffer of the handle kept per class), device pointers
 * (HS2G_DEVICE, used in place and needed only until the call's work has run), or, with HS2G_REUSE, the device
 * copy kept from the previous call for the class.  Work is queued on the handle's stream.
 */
/* Replace the source-class map (nz, ny, nx) on the device (host, or device with HS2G_DEVICE). */
int hs2g_set_source_classes(hs2g_handle* h, const uint8_t* volumetric, int flags);
/* Spatially z-decaying impulse of class cls (alternatingdirection_c_pyx.pyx:320-384): zgrid (nz, ny, nx) holds
   each cell's z coordinate; with d = zgrid * direction - offset (direction +1 or -1, the reference's +z or -z
   unit vector) the cell between d - ddz/2 and d + ddz/2 (clipped at 0) receives the share
   exp(-a / length) - exp(-b / length) of joules_per_m2, divided by ddz * dt (W/m^3); cells with
   d + ddz/2 <= 0 receive nothing. */
int hs2g_source_zdecay(hs2g_handle* h, int cls, const double* zgrid, double direction, double offset, double ddz,
                       double joules_per_m2, double length, double dt, int flags);
/* Point-joules impulse of class cls (alternatingdirection_c_pyx.pyx:307-319): joules per cell / (V * dt), the
   joules one value for every cell (count == 1) or one per cell of the class in C order (count = the class's
   voxel count), V the cell volume `volume` or, with volumes != NULL, each cell's own (nz, ny, nx) volume (the
   curved-surface mode). */
int hs2g_source_point(hs2g_handle* h, int cls, const double* joules, int64_t count, const double* volumes,
                      double volume, double dt, int flags);

/*
 * One timestep that allocates nothing: no counterpart in the reference.
 *
 * For callers that cannot allocate device memory -- a plugin whose host application owns every device
 * allocation and forbids its plugins from calling cudaMalloc (a fixed device-memory budget, or a pool
 * allocator that must not be bypassed).  Such callers cannot create a handle, so this call takes the problem
 * itself in caller-owned device memory: face conductances Gz (nz+1,ny,nx), Gy (nz,ny+1,nx), Gx (nz,ny,nx+1)
 * in W/m^3/K, capacities rho*c/dt (nz,ny,nx), the fixed-temperature mask (or NULL), the per-voxel source in
 * W/m^3 (or NULL) and T_in; it writes T_out (which may equal T_in).  Faces on the grid's exterior are treated
 * as insulating.  Each line is factorised as it is swept, so the call does more FP64 work per step than
 * hs2g_step on a compiled handle.
 *
 * The intermediate fields live in a static device array sized for HS2G_STATIC_MAX_VOXELS voxels (24 MiB),
 * held by every GPU that loads the library until the process exits; larger grids return HS2G_ERR_ARG.
 * Every call shares that array: calls that overlap on the GPU race and must be serialised by the caller.
 * The first call on a device takes the array's device address (cudaGetSymbolAddress), and so does the first
 * call after the device's context changed (cudaDeviceReset); make that call before any stream capture.
 * Work runs on `stream` (a cudaStream_t, NULL = default stream) and the call waits for it: a computed voxel
 * whose capacity is not positive and finite returns HS2G_ERR_CAPACITY (the output is then not a valid step).
 * A launch failure returns HS2G_ERR_CUDA; a sticky error left in the context by earlier work (an illegal
 * address, say) surfaces here too, because every later launch in that context fails.
 */
#define HS2G_STATIC_MAX_VOXELS (1 << 20)
int hs2g_step_static(int64_t nz, int64_t ny, int64_t nx, const double* Gz, const double* Gy, const double* Gx,
                     const double* capacity, const uint8_t* fixed, const double* Q, const double* T_in,
                     double* T_out, void* stream);

/*
 * Batched form: n independent problems of uneven size advanced together (no counterpart in the reference,
 * whose time loop handles one problem; a loop over run_adi_steps calls is what it replaces).  All instances
 * live in one concatenated state: instance i's (nz_i, ny_i, nx_i) field starts at voxel offsets[i] (see
 * hs2g_batch_layout).  precision 64 stores and computes in double (per instance equal to hs2g_step bit for
 * bit); precision 32 compiles in double and stores / sweeps in float.  A timestep is three persistent sweep
 * kernels over flattened line lists, captured once in a CUDA graph and replayed.
 */
typedef struct hs2g_batch hs2g_batch;
int hs2g_batch_create(int n, const hs2g_class_problem* problems, int precision, int device, hs2g_batch** out);
void hs2g_batch_destroy(hs2g_batch* b);
/* offsets[n+1] voxel offsets of the instances, dims[n][3] their (nz, ny, nx); either may be NULL. */
int hs2g_batch_layout(const hs2g_batch* b, int64_t* offsets, int64_t* dims);
int64_t hs2g_batch_device_bytes(const hs2g_batch* b);
/* Temperature of all instances, concatenated (offsets[n] doubles), host or device (HS2G_DEVICE).  With
   precision 32, pass temperatures as offsets from an ambient value (the step maps a uniform field to itself,
   so offsets evolve exactly like temperatures) to spend float resolution on the changes. */
int hs2g_batch_set_temperature(hs2g_batch* b, const double* T, int flags);
int hs2g_batch_get_temperature(hs2g_batch* b, double* T, int flags);
/* Source schedule: qtabs[nsteps][n][nclass] per-class source values (W/m^3) of every instance at every step
   (host); resets the step clock to 0.  Steps beyond the schedule have no source. */
int hs2g_batch_set_sources(hs2g_batch* b, int nsteps, int nclass, const double* qtabs);
int hs2g_batch_set_clock(hs2g_batch* b, int step);
/* Advance every instance by nsteps (graph replays on the batch's stream).  elapsed_ms (or NULL) receives the
   device time of the replays measured with CUDA events; HS2G_SYNC waits for completion. */
int hs2g_batch_run(hs2g_batch* b, int nsteps, int flags, double* elapsed_ms);
/* Time candidate launch shapes per axis on this batch and keep the fastest; writes a report. */
int hs2g_batch_autotune(hs2g_batch* b, char* report, int report_len);

/*
 * Adjoint (no counterpart in the reference, which has no derivatives): gradients of a top-surface misfit
 *     J_i = sum_{n < nsteps} sum_{y,x} (T_{n+1}[0, y, x] - obs_i[n, y, x])^2
 * with respect to per-voxel conductivity k (W/m/K), volumetric heat capacity C = rho*c (J/m^3/K), source
 * amplitude q (W/m^3, applied at step n as schedule[n] * q) and the initial temperature, for n instances of
 * uneven size in one concatenated state (a single problem is n = 1).  Each instance is a box insulating
 * outside, its interior faces conducting with the arithmetic face mean of boundary_conducting
 * (boundary_conducting.py:7-71) unless hs2g_adjoint_set_faces gives face classes (insulating, thin-layer and
 * any other affine scalar-k form) and fixed voxels; the step is the same Douglas delta form as hs2g_step.
 * k must be >= 0 and C > 0.  The forward pass checkpoints T every `ckpt` steps; the backward pass recomputes one segment at a
 * time from its checkpoint and runs the transposed tridiagonal solves in reverse order (z, y, x).  Every
 * kernel of a sweep covers all instances in one launch.
 */
typedef struct {
  int64_t nz, ny, nx;
  double dz, dy, dx;                /* m */
} hs2g_adjoint_grid;
typedef struct hs2g_adjoint hs2g_adjoint;
int hs2g_adjoint_create(int n, const hs2g_adjoint_grid* grids, double dt, int device, hs2g_adjoint** out);
void hs2g_adjoint_destroy(hs2g_adjoint* a);
/* Queue work on a caller's cudaStream_t (NULL = legacy default stream) instead of the handle's own stream. */
int hs2g_adjoint_set_stream(hs2g_adjoint* a, void* stream);
/* offsets[n+1]: instance i's (nz, ny, nx) fields start at voxel offsets[i] of every concatenated array. */
int hs2g_adjoint_layout(const hs2g_adjoint* a, int64_t* offsets);
int64_t hs2g_adjoint_device_bytes(const hs2g_adjoint* a);
/* k, C, q: offsets[n] doubles each, host or device (HS2G_DEVICE); compiles conductances and line factors. */
int hs2g_adjoint_set_parameters(hs2g_adjoint* a, const double* k, const double* C, const double* q, int flags);
/* T0: offsets[n] doubles; obs: per instance in order, nsteps * ny_i * nx_i doubles (host or device, flags);
   schedule[nsteps] host.  loss[n] receives J_i; T_out (offsets[n] doubles, or NULL) the final temperature;
   elapsed_ms (or NULL) the device time of the steps. */
int hs2g_adjoint_forward(hs2g_adjoint* a, int nsteps, const double* schedule, const double* T0, const double* obs,
                         int ckpt, double* loss, double* T_out, int flags, double* elapsed_ms);
/* Face classes and fixed-temperature voxels, in place of the default (every interior face conducting with the
   arithmetic mean of k, every voxel computed).  forms[i][c][a][0..2] = (f0, flo, fhi): a face of class c on
   axis a (0 = z, 1 = y, 2 = x) of instance i conducts f0 + flo * k_lo + fhi * k_hi (W/m^3/K), k_lo and k_hi the
   conductivities of the voxels below and above it, a fixed voxel's replaced by its computed neighbour's
   (crank_nicolson.pyx:298-338): the affine form a boundary class has for scalar k (conducting: flo = fhi =
   1 / (2 d^2); insulating: 0; thin insulating layer: f0 = h / d).  face_z, face_y, face_x (offsets[n] bytes,
   host or device per flags): the class of each voxel's low face on that axis (ignored on the first layer, the
   exterior).  fixed (offsets[n] bytes, or NULL): 1 marks a fixed-temperature voxel, which keeps its
   temperature and whose k, C and q get no gradient.  nclass = 0 (arrays NULL) restores the default.  Applies
   from the next hs2g_adjoint_set_parameters. */
int hs2g_adjoint_set_faces(hs2g_adjoint* a, int nclass, const double* forms, const uint8_t* face_z,
                           const uint8_t* face_y, const uint8_t* face_x, const uint8_t* fixed, int flags);
/* dJ_i/dk, dJ_i/dC, dJ_i/dq and (gT0 not NULL) dJ_i/dT0 of the last forward pass, offsets[n] doubles each. */
int hs2g_adjoint_backward(hs2g_adjoint* a, double* gk, double* gC, double* gq, double* gT0, int flags,
                          double* elapsed_ms);

/* Self-test of the bounded waits inside the TMA sweeps (failure detection without a fault): one thread waits
   at most limit_ns (<= 10 s) on an mbarrier that receives its one arrival (arrive != 0) or none.  *status
   receives HS2G_OK, or HS2G_ERR_TIMEOUT -- the status a sweep reports when its copies never complete -- and
   the device stays usable either way. */
int hs2g_selftest_wait(int device, int64_t limit_ns, int arrive, int* status);

/* Copy the compiled face conductances and capacities to host buffers (any may be NULL).  A handle made by
   hs2g_create_rows has no shared face conductances: asking for Gz, Gy or Gx returns HS2G_ERR_STATE. */
int hs2g_get_faces(hs2g_handle* h, double* Gz, double* Gy, double* Gx, double* capacity, uint8_t* fixed);

/* Device bytes held by the handle. */
int64_t hs2g_device_bytes(const hs2g_handle* h);

#ifdef __cplusplus
}
#endif
#endif
