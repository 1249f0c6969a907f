#!/usr/bin/env python
"""Benchmark of heatsim2's ADI Crank-Nicolson timestep on GB300: voxel-steps/s and roofline fractions.

Workload (one GPU): the composite panel -- 64 x 512 x 512 computed voxels at 0.5 mm under a fixed-temperature
ambient layer (grid 65 x 512 x 512), anisotropic composite over aluminium, three seeded delaminations, flash
2e9 W/m^3 for the first 5 ms step, dt = 5 ms.  A "step" is one ADI timestep over the whole grid; the default
K = 1000 steps is the whole simulated job (t = 0 .. 5 s), timed from t = 0 after W warm-up steps on a
throw-away copy.  Synthetic, seeded input (heatsim2_gb300.workloads.composite_panel(seed=1)).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line.  ``value`` counts computed voxels (64*512*512) per second with the state resident in
HBM; ``e2e`` is the same metric through the C ABI with host buffers (host->device copy of T, the step,
device->host copy of T, every step); ``roofline`` is the dominant sweep kernel against the measured HBM copy
bandwidth, on the algorithmic bytes of a sweep that reads each array it needs once with the face conductances
and capacities re-read in every sweep (x 56, y 40, z 40 B per voxel: 136 B per step), with this
implementation's own bytes (x 88 B: T, nine step coefficients, W0) and the ncu-measured DRAM traffic beside
it; ``kernel_hbm_frac`` gives the same for every sweep; ``step_hbm`` the whole step against the bandwidth
(both accountings); ``fp64_roofline`` the whole step against the measured FP64 FMA rate;
``cpu_baseline`` the reference (or, where it cannot be built, the oracle) on the host cores.  ``batched`` is
the 256-instance uneven batch (FP64 and FP32) against a per-instance loop of the plain path; ``adjoint`` the
gradient evaluations per second of the (32,128,128) steel inverse problem and of the 32-instance batched
adjoint against a loop of single-instance adjoints; ``curved`` the benchmark grid in the curved-surface mode.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "voxel-steps/s"
SEED = 1
# algorithmic bytes and FP64 operations per grid voxel, per kernel (dense coefficient layout, no source active):
#   sweep_x  reads T and 9 coefficient arrays (wc wxl wxh wyl wyh wzl wzh a0 b0), writes W0
#   sweep_y  reads W0, a1, b1, writes W1
#   sweep_z  reads W1, a2, b2, T, writes T'
BYTES_PER_VOXEL = {"sweep_x": 8 + 9 * 8 + 8, "sweep_y": 4 * 8, "sweep_z": 5 * 8}
# the algorithmic bytes the roofline is reported on: each sweep touching each array it needs once, with the face
# conductances and capacities re-read in every sweep (136 B per voxel and step):
#   sweep_x  reads T, M, Gx, Gy, Gz, Q, writes T*0 (7 arrays)
#   sweep_y  reads T, T*0, M, Gy, writes T*1 (5)
#   sweep_z  reads T, T*1, M, Gz, writes T' (5)
ROOFLINE_BYTES_PER_VOXEL = {"sweep_x": 7 * 8, "sweep_y": 5 * 8, "sweep_z": 5 * 8}
FP64_OPS_PER_VOXEL = {"sweep_x": 9, "sweep_y": 2, "sweep_z": 3}
KERNELS = ("sweep_x", "sweep_y", "sweep_z")
# adjoint: arrays touched per voxel and step (8 B each), from the kernels of hs2g_adjoint.cu
#   forward step (forward pass, and again as the recompute of the backward pass): x stage reads T, gx, gy, gz,
#   D, q, lo0, ip0, u0 and writes y0 (10); y stage reads y0, lo1, mip1, u1 (mip = M / piv), writes y1 (5); z stage
#   reads y1, lo2, mip2, u2, T, writes y2, T' (7)                                             -> 22 arrays
#   reverse step: transposed z reads lambda, u2, lo2, ip2, writes mu2 (5); transposed y reads mu2, u1, lo1,
#   mip1, writes mu1 (5); transposed x the same for mu0 (5); update reads gx, gy, gz, T, y0, y1, y2, mu0, mu1,
#   mu2, lambda and the five accumulators and writes lambda and the accumulators (22)          -> 37 arrays
# so one gradient evaluation moves (22 + 22 + 37) * 8 = 648 B (the x stage also reads the diagonal D) and does
# about 18 + 18 + (3 + 3 + 3 + 34) = 79 FP64 operations per voxel and step (forward step, recompute,
# transposed solves and update).
ADJ_BYTES_PER_VOXEL_STEP = (22 + 22 + 37) * 8
ADJ_FP64_OPS_PER_VOXEL_STEP = 79


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--shape", type=int, nargs=3, default=[64, 512, 512], metavar=("NZ", "NY", "NX"),
                    help="computed voxels (an ambient layer is added on top)")
    ap.add_argument("--e2e-steps", type=int, default=30)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batch-instances", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=100)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-curved", action="store_true")
    ap.add_argument("--adjoint-steps", type=int, default=None,
                    help="steps of both adjoint workloads (default: their own 500 and 400; smaller for profiling)")
    ap.add_argument("--adjoint-loop", type=int, default=32,
                    help="instances of the batched adjoint workload timed as a loop of single-instance adjoints")
    ap.add_argument("--cpu-worker", default=None, help=argparse.SUPPRESS)
    return ap.parse_args()


def workload(shape, nsteps):
    from heatsim2_gb300 import workloads as W
    nz, ny, nx = shape
    wr = (min(10, ny, nx), min(60, ny, nx))
    dr = (min(4, nz - 1), min(40, nz - 1))
    return W.composite_panel(seed=SEED, nz=nz, ny=ny, nx=nx, nsteps=nsteps, width_range=wr, depth_range=dr)


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def read_traffic():
    """DRAM bytes per grid voxel per launch measured by ncu (profiles/dram_traffic.txt), or {}."""
    out = {}
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    try:
        with open(path) as fh:
            for line in fh:
                parts = line.split()
                if len(parts) >= 2 and not line.startswith("#"):
                    out[parts[0]] = float(parts[1])
    except OSError:
        pass
    return out


class ClockSampler(object):
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None, "samples": len(sm), "reasons": sorted(reasons)}


# ------------------------------------------------------------------------------------------------------------
# CPU baseline (the reference built in oracle/_ref, else the oracle) -- a bounded sample, own process
# ------------------------------------------------------------------------------------------------------------
CPU_SAMPLE_SHAPE = (64, 64, 64)


def _cpu_impl():
    import build_ref
    if build_ref.available():
        try:
            return "reference", build_ref.import_reference()
        except Exception:
            pass
    import oracle
    from oracle_shim import HS
    return "port", (oracle, HS)


def cpu_worker(kind_req, seconds, max_steps, barrier=None, result=None, warm=1):
    """Time one CPU implementation on the composite panel at CPU_SAMPLE_SHAPE after `warm` untimed steps;
    returns a dict."""
    import contextlib
    import io
    from heatsim2_gb300 import workloads as W
    kind, impl = _cpu_impl()
    spec = workload(CPU_SAMPLE_SHAPE, max_steps)
    if kind == "reference":
        hsr = impl
        with contextlib.redirect_stdout(io.StringIO()):
            P, S = hsr.setup(*W.setup_args(hsr, spec))
        step = lambda t, T: hsr.run_adi_steps(P, S, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
        vol = W.volumetric_tuple(hsr, spec)
    else:
        orc, HS = impl
        P, _ = orc.setup(*W.setup_args(HS, spec))
        vol = W.volumetric_tuple(HS, spec)
        step = lambda t, T: orc.run_adi_steps(P, None, t, spec["dt"], T, spec["arrays"]["volumetric"], vol)
    T = W.initial_temperature(spec)
    times = W.step_times(spec, max_steps)
    for t in times[:warm]:         # warm-up
        T = step(t, T)
    if barrier is not None:
        barrier.wait()
    t0 = time.perf_counter()
    n = 0
    for t in times[warm:]:
        T = step(t, T)
        n += 1
        if seconds and time.perf_counter() - t0 >= seconds:
            break
    el = time.perf_counter() - t0
    nz, ny, nx = CPU_SAMPLE_SHAPE
    out = {"kind": kind, "steps": n, "seconds": el, "voxels": nz * ny * nx,
           "value": nz * ny * nx * n / el if el > 0 else 0.0}
    if result is not None:
        result.put(out)
    return out


def run_cpu_baseline(seconds):
    cmd = [sys.executable, os.path.abspath(__file__), "--cpu-worker", "auto", "--cpu-seconds", str(seconds)]
    try:
        out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
        d = json.loads(out.stdout.strip().splitlines()[-1])
    except Exception as e:
        return {"value": None, "unit": METRIC, "cores": 1, "kind": "port", "sample": "failed: %s" % (e,)}
    nz, ny, nx = CPU_SAMPLE_SHAPE
    return {"value": d["value"], "unit": METRIC, "cores": 1, "kind": d["kind"],
            "sample": "composite panel %dx%dx%d (+ambient layer), %d steps after setup, %.1f s, 1 thread "
                      "(the reference is single-threaded); cpu: %s" % (nz, ny, nx, d["steps"], d["seconds"],
                                                                     cpu_model())}


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip() + " x%d" % os.cpu_count()
    except OSError:
        pass
    return "%d cores" % os.cpu_count()


# ------------------------------------------------------------------------------------------------------------
# reference arm: the reference CPU implementation on all host cores (one process per core)
# ------------------------------------------------------------------------------------------------------------
def reference_arm(args, world, rank):
    if rank != 0:
        return
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    nproc = os.cpu_count() or 1
    barrier = ctx.Barrier(nproc)
    q = ctx.Queue()
    steps = max(1, args.steps)
    warm = max(1, args.warmup)
    procs = [ctx.Process(target=cpu_worker, args=("auto", 0.0, steps + warm, barrier, q, warm))
             for _ in range(nproc)]
    for p in procs:
        p.start()
    res = [q.get() for _ in procs]
    for p in procs:
        p.join()
    el = max(r["seconds"] for r in res)
    total = sum(r["voxels"] * r["steps"] for r in res)
    value = total / el
    nz, ny, nx = CPU_SAMPLE_SHAPE
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
        "steps": steps, "warmup": warm, "ms_per_step": 1e3 * el / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "composite panel %dx%dx%d (+ambient), one independent instance per host core"
                               % (nz, ny, nx), "processes": nproc},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": nproc, "kind": res[0]["kind"],
                         "sample": "%d processes x %d steps of the composite panel %dx%dx%d after setup; cpu: %s"
                                   % (nproc, steps, nz, ny, nx, cpu_model())},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------------------------
# batched form (uneven instances) against a loop of the single-problem path
# ------------------------------------------------------------------------------------------------------------
def batched_measurement(args, world, rank, dev):
    """256 uneven instances (nz 16..64, ny,nx 64..256; steel or composite; one flaw; flash), seed 2.
    FP64 and FP32 batches (autotuned, one CUDA graph per step) against a per-instance loop of hs2g_run."""
    import ctypes
    import numpy as np
    import torch
    import heatsim2_gb300 as hs
    from heatsim2_gb300 import _native, workloads as W
    from heatsim2_gb300.batch import Batch, shard
    from heatsim2_gb300.alternatingdirection import _ClassSources, source_table

    L = _native.load()
    specs_all = W.uneven_batch(seed=2, n=args.batch_instances)
    sizes = [W.voxels(s) for s in specs_all]
    specs = [specs_all[i] for i in shard(sizes, world, rank)]
    steps = args.batch_steps
    dt = specs[0]["dt"]
    times = W.step_times(specs[0], steps)
    computed = sum(s.get("compute_voxels", W.voxels(s)) for s in specs)
    out = {"workload": "%d uneven instances (seed 2), %d steps of dt=%g" % (len(specs_all), steps, dt),
           "instances": len(specs), "computed_voxels": computed}
    results = {}
    for prec in (64, 32):
        t0 = time.perf_counter()
        b = Batch([W.setup_args(hs, s) for s in specs], precision=prec)
        setup_s = time.perf_counter() - t0
        b.set_temperature([W.initial_temperature(s) for s in specs])
        tune = b.autotune()
        b.set_sources(times, dt)
        b.run(0)
        torch.cuda.synchronize()
        ms = b.run(steps)
        results[prec] = b.get_temperature()
        out["fp%d" % prec] = {"value": computed * steps / (ms * 1e-3), "ms_per_step": ms / steps,
                              "setup_s": setup_s, "device_bytes": b.device_bytes,
                              "tuning": tune.strip().splitlines()[-1]}
        del b
    out["fp32_max_rel_err_vs_fp64"] = max(
        float(np.abs(a - c).max() / np.abs(a).max()) for a, c in zip(results[64], results[32]))
    # per-instance loop of the single-problem path on the same instances, one stream, device time
    handles = []
    for s in specs:
        P, S = hs.setup(*W.setup_args(hs, s))
        src = _ClassSources(W.volumetric_tuple(hs, s))
        q = np.ascontiguousarray([source_table(src, t, dt, P.volume_array)[0] for t in times])
        T = torch.from_numpy(W.initial_temperature(s)).to(dev)
        handles.append((P, q, T))
    stream = torch.cuda.Stream(device=dev)
    for P, _, _ in handles:
        _native.check(L.hs2g_set_stream(P.handle.ptr, ctypes.c_void_p(stream.cuda_stream)))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for P, q, T in handles:
        _native.check(L.hs2g_run(P.handle.ptr, steps, T.data_ptr(), T.data_ptr(), q.ctypes.data, 0, None,
                                 _native.DEVICE))
    e1.record(stream)
    torch.cuda.synchronize()
    loop_ms = e0.elapsed_time(e1)
    worst = max(float(np.abs(T.cpu().numpy() - r).max() / np.abs(r).max())
                for (_, _, T), r in zip(handles, results[64]))
    out["plain_loop"] = {"value": computed * steps / (loop_ms * 1e-3), "ms_per_step": loop_ms / steps,
                         "max_rel_diff_vs_batch_fp64": worst}
    if world > 1:
        for key in ("fp64", "fp32", "plain_loop"):
            t = torch.tensor([out[key]["ms_per_step"]], device=dev, dtype=torch.float64)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            c = torch.tensor([float(computed)], device=dev, dtype=torch.float64)
            torch.distributed.all_reduce(c)
            out[key]["value"] = float(c.item()) / (float(t.item()) * 1e-3)
    out["speedup_fp64_vs_loop"] = out["fp64"]["value"] / out["plain_loop"]["value"]
    del handles
    return out


def curved_measurement(args, dev, steps=200):
    """The reference's curved-surface mode (crank_nicolson.pyx:388-457) on the benchmark grid: the composite
    panel under uniform surface curvatures of 2 /m along y and 1 /m along x (radii 0.5 m and 1 m), compiled
    from per-row conductances (hs2g_create_rows); setup time and voxel-steps/s over ``steps`` steps."""
    import ctypes
    import numpy as np
    import torch
    import heatsim2_gb300 as hs
    from heatsim2_gb300 import _native, workloads as W
    from heatsim2_gb300.alternatingdirection import _ClassSources, source_table

    L = _native.load()
    spec = W.curved(workload(args.shape, steps), ky=2.0, kx=1.0)
    t0 = time.perf_counter()
    P, S = hs.setup(*W.setup_args(hs, spec), **W.setup_kwargs(spec))
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    src = _ClassSources(W.volumetric_tuple(hs, spec), True)
    qtabs = np.ascontiguousarray([source_table(src, t, spec["dt"], P.volume_array)[0]
                                  for t in W.step_times(spec, steps)])
    T0 = torch.from_numpy(W.initial_temperature(spec)).to(dev)
    T = T0.clone()
    stream = torch.cuda.Stream(device=dev)
    h = P.handle.ptr
    _native.check(L.hs2g_set_stream(h, ctypes.c_void_p(stream.cuda_stream)))
    # as the main measurement: the schedule on the device, the same in-place call warmed up, then timed
    _native.check(L.hs2g_set_schedule(h, steps, qtabs.ctypes.data, 0))
    _native.check(L.hs2g_run(h, min(steps, 10), T.data_ptr(), T.data_ptr(), None, 0, None,
                             _native.DEVICE | _native.SCHEDULED))
    _native.check(L.hs2g_set_clock(h, 0))
    T.copy_(T0)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    _native.check(L.hs2g_run(h, steps, T.data_ptr(), T.data_ptr(), None, 0, None, _native.DEVICE | _native.SCHEDULED))
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = float(ev0.elapsed_time(ev1))
    return {"workload": "composite panel %dx%dx%d, surface curvatures 2 /m (y) and 1 /m (x), %d steps"
                        % (tuple(args.shape) + (steps,)),
            "value": spec["compute_voxels"] * steps / (ms * 1e-3), "unit": METRIC,
            "ms_per_step": ms / steps, "setup_s": setup_s}


def adjoint_measurement(args, world, rank, dev):
    """Gradient evaluations (forward pass + checkpointed backward pass) per second.

    steel: one (32,128,128) steel instance, per-voxel lognormal k, 500 steps of 10 ms, checkpoint every 50.
    batched: 32 uneven two-phase instances (nz 24..48, ny,nx 96..192), 400 steps of 5 ms, checkpoint every 40,
    all in one concatenated state (one launch per sweep over every instance), against a loop of the
    single-instance adjoint over the same instances.  Device time from CUDA events around the steps."""
    import ctypes
    import numpy as np
    import torch
    from heatsim2_gb300 import _native, workloads as W
    from heatsim2_gb300.adjoint import Adjoint
    from heatsim2_gb300.batch import shard

    out = {}
    steps_kw = {} if args.adjoint_steps is None else {"nsteps": args.adjoint_steps}
    w = W.adjoint_steel(**steps_kw)
    a = Adjoint([(w["shape"], w["spacing"])], w["dt"])
    a.set_parameters(w["k"], w["C"], w["q"])
    for _ in range(2):  # warm-up, then the timed evaluation
        a.forward(w["T0"], w["obs"], w["schedule"], w["ckpt"])
        a.backward()
    fwd, bwd = a.forward_ms, a.backward_ms
    vox = int(np.prod(w["shape"]))
    hbm_peak, _ = read_peaks()
    fma_rate = ctypes.c_double(0.0)
    _native.check(_native.load().hs2g_fp64_fma_rate(torch.cuda.current_device(), ctypes.byref(fma_rate)))

    def fracs(voxel_steps, ms):
        return {"bytes_per_voxel_step": ADJ_BYTES_PER_VOXEL_STEP,
                "fp64_ops_per_voxel_step": ADJ_FP64_OPS_PER_VOXEL_STEP,
                "hbm_frac": ADJ_BYTES_PER_VOXEL_STEP * voxel_steps / (ms * 1e-3) / (hbm_peak * 1e9),
                "fp64_frac": ADJ_FP64_OPS_PER_VOXEL_STEP * voxel_steps / (ms * 1e-3) / fma_rate.value}
    out["steel"] = {"workload": "steel (32,128,128) lognormal k, %d steps dt=10 ms, checkpoint %d"
                                % (w["nsteps"], w["ckpt"]),
                    "gradient_evals_per_s": 1e3 / (fwd + bwd), "forward_ms": fwd, "backward_ms": bwd,
                    "forward_voxel_steps_per_s": vox * w["nsteps"] / (fwd * 1e-3),
                    "roofline": fracs(vox * w["nsteps"], fwd + bwd), "device_bytes": a.device_bytes}
    del a
    insts_all = W.adjoint_batch(**steps_kw)
    sizes = [int(np.prod(x["shape"])) for x in insts_all]
    insts = [insts_all[i] for i in shard(sizes, world, rank)]
    b = Adjoint([(x["shape"], x["spacing"]) for x in insts], insts[0]["dt"])
    b.set_parameters([x["k"] for x in insts], [x["C"] for x in insts], [x["q"] for x in insts])
    args_f = ([x["T0"] for x in insts], [x["obs"] for x in insts], insts[0]["schedule"], insts[0]["ckpt"])
    for _ in range(2):
        b.forward(*args_f)
        gb = b.backward()
    batch_ms = b.forward_ms + b.backward_ms
    bytes_b = b.device_bytes
    del b
    torch.cuda.empty_cache()
    loop_ms, worst = 0.0, 0.0
    nloop = min(args.adjoint_loop, len(insts))
    for i, x in enumerate(insts[:nloop]):
        s = Adjoint([(x["shape"], x["spacing"])], x["dt"])
        s.set_parameters(x["k"], x["C"], x["q"])
        s.forward(x["T0"], x["obs"], x["schedule"], x["ckpt"])
        g = s.backward()
        loop_ms += s.forward_ms + s.backward_ms
        worst = max(worst, max(float(np.abs(u - v[i]).max() / max(np.abs(v[i]).max(), 1e-300))
                               for u, v in zip(g, gb)))
        del s
    loop_ms *= len(insts) / nloop
    batch_evals = len(insts) / (batch_ms * 1e-3)
    loop_evals = len(insts) / (loop_ms * 1e-3)
    if world > 1:
        t = torch.tensor([batch_ms, loop_ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        batch_evals = len(insts_all) / (float(t[0]) * 1e-3)
        loop_evals = len(insts_all) / (float(t[1]) * 1e-3)
    out["batched"] = {"workload": "%d uneven two-phase instances (nz 24..48, ny,nx 96..192), %d steps dt=5 ms, "
                                  "checkpoint %d" % (len(insts_all), insts[0]["nsteps"], insts[0]["ckpt"]),
                      "voxels": sum(sizes), "gradient_evals_per_s": batch_evals, "ms_per_eval_batch": batch_ms,
                      "roofline": fracs(sum(int(np.prod(x["shape"])) for x in insts) * insts[0]["nsteps"],
                                        batch_ms),
                      "device_bytes": bytes_b,
                      "single_loop": {"gradient_evals_per_s": loop_evals, "instances_timed": nloop,
                                      "max_rel_diff_vs_batch": worst},
                      "speedup_vs_loop": batch_evals / loop_evals}
    return out


# ------------------------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------------------------
def gpu_arm(args, world, rank, local_rank):
    import ctypes
    import numpy as np
    import torch
    import heatsim2_gb300 as hs
    from heatsim2_gb300 import _native, workloads as W
    from heatsim2_gb300.alternatingdirection import _ClassSources, source_table

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    L = _native.load()
    K, Wm = args.steps, args.warmup
    spec = workload(args.shape, K)
    t0 = time.perf_counter()
    P, S = hs.setup(*W.setup_args(hs, spec))
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    nz, ny, nx = spec["grid"]["nz"], spec["grid"]["ny"], spec["grid"]["nx"]
    grid_vox = nz * ny * nx
    compute_vox = spec["compute_voxels"]
    src = _ClassSources(W.volumetric_tuple(hs, spec))
    times = W.step_times(spec, max(K, Wm))
    qtabs = np.zeros((len(times), _native.MAX_CLASSES))
    for s, t in enumerate(times):
        qtabs[s], _ = source_table(src, t, spec["dt"], P.volume_array)
    T0 = torch.from_numpy(W.initial_temperature(spec)).to(dev)
    T = T0.clone()
    stream = torch.cuda.Stream(device=dev)
    h = P.handle.ptr
    _native.check(L.hs2g_set_stream(h, ctypes.c_void_p(stream.cuda_stream)))
    kms = np.zeros(4)
    # warm-up on a throw-away state
    qw = np.ascontiguousarray(qtabs[:Wm])
    _native.check(L.hs2g_run_timed(h, Wm, T0.data_ptr(), T.data_ptr(), qw.ctypes.data, _native.DEVICE,
                                   kms.ctypes.data))
    fma_rate = ctypes.c_double(0.0)
    _native.check(L.hs2g_fp64_fma_rate(local_rank, ctypes.byref(fma_rate)))
    # per-kernel device times: the same K steps launched from the host (each step's table a kernel parameter)
    # with CUDA events around every sweep
    qk = np.ascontiguousarray(qtabs[:K])
    T.copy_(T0)
    torch.cuda.synchronize()
    _native.check(L.hs2g_run_timed(h, K, T.data_ptr(), T.data_ptr(), qk.ctypes.data, _native.DEVICE,
                                   kms.ctypes.data))
    host_launched_ms = float(kms[3])
    # timed region: K steps from t = 0 as hs2g_run executes them -- the schedule's rows on the device, the
    # flash step as a replay of the one-step source graph and the others as replays of the four-step graph
    # without a source (x, y and z sweeps); the warm-up runs the same in-place call for W steps (at least 10: the
    # flash, two four-step graphs and a one-step graph, so that every graph the timed call replays is captured
    # before it), then the clock is rewound to row 0
    _native.check(L.hs2g_set_schedule(h, K, qk.ctypes.data, 0))
    T.copy_(T0)
    _native.check(L.hs2g_run(h, min(K, max(Wm, 10)), T.data_ptr(), T.data_ptr(), None, 0, None,
                             _native.DEVICE | _native.SCHEDULED))
    _native.check(L.hs2g_set_clock(h, 0))
    T.copy_(T0)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    _native.check(L.hs2g_run(h, K, T.data_ptr(), T.data_ptr(), None, 0, None, _native.DEVICE | _native.SCHEDULED))
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    total_ms = float(ev0.elapsed_time(ev1))
    if world > 1:
        t = torch.tensor([total_ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    value = world * compute_vox * K / (total_ms * 1e-3)
    per_kernel_ms = {k: float(kms[i]) / K for i, k in enumerate(KERNELS)}
    # roofline of the dominant kernel
    hbm_peak, peak_src = read_peaks()
    dom = max(per_kernel_ms, key=per_kernel_ms.get)
    achieved_gbs = ROOFLINE_BYTES_PER_VOXEL[dom] * grid_vox / (per_kernel_ms[dom] * 1e-3) / 1e9
    impl_gbs = BYTES_PER_VOXEL[dom] * grid_vox / (per_kernel_ms[dom] * 1e-3) / 1e9
    traffic = read_traffic()
    roofline = {"kernel": dom, "bound": "hbm", "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved_gbs / hbm_peak, "peak_source": peak_src + " (MEASURED_PEAKS.json hbm_gbs)",
                "algorithmic_bytes_per_voxel": ROOFLINE_BYTES_PER_VOXEL[dom],
                "algorithmic_bytes_per_launch": ROOFLINE_BYTES_PER_VOXEL[dom] * grid_vox,
                "traffic": traffic[dom] * grid_vox if dom in traffic else None,
                "implementation_bytes_per_voxel": BYTES_PER_VOXEL[dom], "implementation_achieved": impl_gbs,
                "implementation_frac": impl_gbs / hbm_peak}
    step_ops = sum(FP64_OPS_PER_VOXEL.values()) * grid_vox
    fp64 = {"bound": "fp64", "achieved": step_ops / (total_ms * 1e-3 / K) / 1e12,
            "peak": fma_rate.value / 1e12, "unit": "TFMA/s", "ops_per_voxel_step": sum(FP64_OPS_PER_VOXEL.values()),
            "peak_source": "measured (hs2g_fp64_fma_rate, register-only FMA chains)"}
    fp64["frac"] = fp64["achieved"] / fp64["peak"] if fp64["peak"] else None
    per_kernel_fp64 = {k: FP64_OPS_PER_VOXEL[k] * grid_vox / (per_kernel_ms[k] * 1e-3) / fma_rate.value
                       for k in KERNELS}
    # the whole step against HBM: with this implementation's algorithmic bytes (160 per grid voxel), and with
    # the 136-byte accounting of a step that re-reads T, M and the face conductances in every sweep (17 arrays)
    step_s = total_ms * 1e-3 / K
    step_hbm = {"bytes_per_voxel_step": sum(BYTES_PER_VOXEL.values()),
                "achieved_gbs": sum(BYTES_PER_VOXEL.values()) * grid_vox / step_s / 1e9,
                "frac": sum(BYTES_PER_VOXEL.values()) * grid_vox / step_s / 1e9 / hbm_peak,
                "frac_136_bytes": 136 * compute_vox / step_s / 1e9 / hbm_peak, "peak": hbm_peak}
    per_kernel_hbm = {k: ROOFLINE_BYTES_PER_VOXEL[k] * grid_vox / (per_kernel_ms[k] * 1e-3) / 1e9 / hbm_peak
                      for k in KERNELS}
    per_kernel_hbm_impl = {k: BYTES_PER_VOXEL[k] * grid_vox / (per_kernel_ms[k] * 1e-3) / 1e9 / hbm_peak
                           for k in KERNELS}
    per_kernel_traffic = {k: traffic[k] * grid_vox / (per_kernel_ms[k] * 1e-3) / 1e9 / hbm_peak
                          for k in KERNELS if k in traffic}
    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        E = max(2, min(args.e2e_steps, K))
        hin = torch.from_numpy(W.initial_temperature(spec)).pin_memory()
        hout = torch.empty_like(hin).pin_memory()
        _native.check(L.hs2g_set_stream(h, None))
        for s in range(2):
            _native.check(L.hs2g_step(h, hin.data_ptr(), hout.data_ptr(), qtabs[s].ctypes.data, None, None, 0))
        hin.copy_(torch.from_numpy(W.initial_temperature(spec)))
        te = time.perf_counter()
        a, b = hin, hout
        for s in range(E):
            _native.check(L.hs2g_step(h, a.data_ptr(), b.data_ptr(), qtabs[s % len(qtabs)].ctypes.data, None, None,
                                      0))
            a, b = b, a
        el = time.perf_counter() - te
        e2e = {"value": world * compute_vox * E / el, "unit": METRIC, "h2d_bytes_per_step": grid_vox * 8,
               "d2h_bytes_per_step": grid_vox * 8, "steps": E,
               "path": "hs2g_step with pinned host buffers (copy in, 3 sweeps, copy out, sync) per step"}
    state_bytes = P.device_bytes
    batched = None
    if not args.no_batched:
        del P, S
        torch.cuda.empty_cache()
        batched = batched_measurement(args, world, rank, dev)
    curved = None
    if not args.no_curved:
        torch.cuda.empty_cache()
        curved = curved_measurement(args, dev)
    adjoint = None
    if not args.no_adjoint:
        torch.cuda.empty_cache()
        adjoint = adjoint_measurement(args, world, rank, dev)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = run_cpu_baseline(args.cpu_seconds)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": K, "warmup": Wm,
            "ms_per_step": total_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "composite panel %dx%dx%d computed voxels (+1 fixed ambient layer), 0.5 mm, "
                                   "anisotropic composite over aluminium, 3 delaminations, flash at t=0, dt=5 ms"
                                   % tuple(args.shape),
                       "grid": [nz, ny, nx], "computed_voxels": compute_vox, "seed": SEED,
                       "l2": "inputs larger than L2 (T %.0f MB, device state %.0f MB)"
                             % (grid_vox * 8 / 1e6, state_bytes / 1e6),
                       "kernels": "x: CTA-staged stencil + warp recurrence; y: TMA tensor-tile ring; z: per-line; "
                                  "timed as hs2g_run: schedule rows on the device, one step-graph replay per step",
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": roofline, "fp64_roofline": fp64, "step_hbm": step_hbm,
            "kernel_ms_per_step": per_kernel_ms, "kernel_fp64_frac": per_kernel_fp64,
            "kernel_hbm_frac": per_kernel_hbm, "kernel_hbm_frac_implementation_bytes": per_kernel_hbm_impl,
            "kernel_dram_frac_measured_traffic": per_kernel_traffic,
            "host_launched_ms_per_step": host_launched_ms / K,
            "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": 3 * K, "clocks": clk, "setup_s": setup_s,
            "device_bytes": state_bytes, "batched": batched, "adjoint": adjoint, "curved": curved,
        }
        print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.cpu_worker:
        print(json.dumps(cpu_worker(args.cpu_worker, args.cpu_seconds, 100000)), flush=True)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        reference_arm(args, world, rank)
        return
    if world > 1:
        import torch
        torch.cuda.set_device(local_rank)
        torch.distributed.init_process_group("nccl")
    gpu_arm(args, world, rank, local_rank)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
