"""Batched form: many independent heatsim2 problems of uneven size advanced together on one GPU.

The reference advances one problem per ``run_adi_steps`` call; a user with many specimens loops over them.
``Batch`` takes a list of problems given as ``heatsim2.setup`` argument tuples, compiles them into one
concatenated device state (libhs2g ``hs2g_batch_create``) and advances all of them per step with three
persistent sweep kernels captured in one CUDA graph.  ``precision=64`` gives, per instance, exactly the
result of ``setup`` + ``run_adi_steps``; ``precision=32`` stores and sweeps in float (coefficients compiled in
double) for throughput, with its error against double left to the caller to measure.
"""
import ctypes

import numpy as np

from . import _native
from .crank_nicolson import ClassProblem, raise_compile_error, current_device
from .alternatingdirection import _ClassSources, source_table


def shard(sizes, world, rank):
    """Instances (indices into ``sizes``, the voxel counts) that rank ``rank`` of ``world`` advances.

    Instances are independent, so a multi-GPU run splits them across ranks with no collective on the data
    path.  Greedy longest-processing-time assignment: largest instance first, each to the least-loaded rank
    (ties to the lower rank), which keeps every rank within one instance of the mean load.  Deterministic, so
    every rank computes the same split without communicating."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad world / rank")
    load = [0] * world
    mine = []
    for i in sorted(range(len(sizes)), key=lambda i: (-sizes[i], i)):
        r = min(range(world), key=lambda r: (load[r], r))
        load[r] += sizes[i]
        if r == rank:
            mine.append(i)
    return sorted(mine)


class Batch(object):
    def __init__(self, problems, precision=64, device=None):
        """problems: sequence of setup-argument tuples (positional arguments of ``heatsim2.setup``)."""
        if precision not in (32, 64):
            raise ValueError("precision must be 64 or 32")
        self.precision = precision
        self.device = current_device() if device is None else device
        self.problems = [ClassProblem(*p) for p in problems]
        if any(p.curvature is not None for p in self.problems):
            raise NotImplementedError("curved-surface problems are not provided in the batched form")
        n = len(self.problems)
        if n < 1:
            raise ValueError("empty batch")
        arr = (_native.ClassProblem * n)(*[p.struct for p in self.problems])
        L = _native.load()
        h = ctypes.c_void_p()
        rc = L.hs2g_batch_create(n, arr, precision, self.device, ctypes.byref(h))
        if rc != _native.OK:
            raise_compile_error(rc)
        self._h = h
        self.n = n
        self.offsets = np.zeros(n + 1, dtype=np.int64)
        dims = np.zeros((n, 3), dtype=np.int64)
        _native.check(L.hs2g_batch_layout(h, self.offsets.ctypes.data, dims.ctypes.data))
        self.shapes = [tuple(int(v) for v in r) for r in dims]
        self.voxels = int(sum(a * b * c for a, b, c in self.shapes))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _native._lib is not None:
            _native._lib.hs2g_batch_destroy(h)
            self._h = None

    @property
    def device_bytes(self):
        return int(_native.load().hs2g_batch_device_bytes(self._h))

    def _concat(self, fields):
        buf = np.zeros(int(self.offsets[-1]))
        for i, f in enumerate(fields):
            f = np.ascontiguousarray(f, dtype="d")
            if f.shape != self.shapes[i]:
                raise ValueError("instance %d: shape %s, expected %s" % (i, f.shape, self.shapes[i]))
            buf[self.offsets[i]:self.offsets[i] + f.size] = f.reshape(-1)
        return buf

    def set_temperature(self, fields):
        """fields: one (nz,ny,nx) array per instance.

        With precision 32 the device holds each instance's temperature as an offset from that instance's
        initial mean: the step is linear and maps a uniform field to itself, so the offset evolves exactly as
        the temperature does, while float resolution goes to the changes instead of to ~300 K."""
        fields = [np.asarray(f, dtype="d") for f in fields]
        if self.precision == 32:
            self.reference = [float(f.mean()) for f in fields]
            fields = [f - r for f, r in zip(fields, self.reference)]
        else:
            self.reference = [0.0] * self.n
        buf = self._concat(fields)
        _native.check(_native.load().hs2g_batch_set_temperature(self._h, buf.ctypes.data, 0))

    def get_temperature(self):
        buf = np.empty(int(self.offsets[-1]))
        _native.check(_native.load().hs2g_batch_get_temperature(self._h, buf.ctypes.data, 0))
        ref = getattr(self, "reference", [0.0] * self.n)
        return [buf[self.offsets[i]:self.offsets[i] + int(np.prod(s))].reshape(s) + ref[i]
                for i, s in enumerate(self.shapes)]

    def set_sources(self, times, dt):
        """Per-step source tables for the t values ``times`` (one step each) with each instance's own
        ``volumetric`` tuple and class map; resets the step clock."""
        srcs = [_ClassSources(p.volumetric) for p in self.problems]
        if any(s.shaped for s in srcs):
            raise NotImplementedError("per-voxel sources (point joules with an array, z-decaying impulse) are "
                                      "not provided in the batched form")
        nclass = max(1, max(len(p.volumetric) for p in self.problems))
        q = np.zeros((len(times), self.n, nclass))
        for s, t in enumerate(times):
            for i, (src, p) in enumerate(zip(srcs, self.problems)):
                dz, dy, dx = p.spacing
                tab, _ = source_table(src, t, dt, dz * dy * dx)
                q[s, i, :] = tab[:nclass]
        _native.check(_native.load().hs2g_batch_set_sources(self._h, len(times), nclass, q.ctypes.data))

    def run(self, nsteps, sync=True):
        """Advance every instance by nsteps; returns the device time of the graph replays in ms."""
        ms = ctypes.c_double(0.0)
        _native.check(_native.load().hs2g_batch_run(self._h, int(nsteps), _native.SYNC if sync else 0,
                                                    ctypes.byref(ms)))
        return ms.value

    def autotune(self):
        """Time candidate launch shapes per axis on this batch, keep the fastest; returns the report."""
        buf = ctypes.create_string_buffer(8192)
        _native.check(_native.load().hs2g_batch_autotune(self._h, buf, len(buf)))
        return buf.value.decode()
