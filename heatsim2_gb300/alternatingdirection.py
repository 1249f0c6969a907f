"""``run_adi_steps``: one ADI Crank-Nicolson timestep on the GPU, and the objects ``setup`` returns.

Mirrors ``heatsim2.alternatingdirection_c_pyx.run_adi_steps`` (reference alternatingdirection_c_pyx.pyx:287-416):
same arguments, a fresh array returned, the source classes evaluated at ``t`` with ``dt``
(pyx:294-386), the step's coefficients fixed by ``setup``'s dt.  ``Tarray`` may be a numpy array (copied to
and from the device each call) or a float64 CUDA ``torch.Tensor`` on the problem's device (no copies; the
result is a new tensor).  ``run`` advances many steps on the device in one call.
"""
import ctypes
import numbers

import numpy as np

from . import _native

NO_SOURCE = 0
IMPULSE_SOURCE = 1
STEPPED_SOURCE = 2
IMPULSE_POINT_SOURCE_JOULES = 3
SPATIALLY_Z_DECAYING_TEMPORAL_IMPULSE = 4


class adi_params(object):
    """Compiled problem (the reference's ADI_params, alternatingdirection_c_pyx.pyx:75-85): ``shape``,
    ``volume_array`` (cell volume), plus the device handle that owns the step coefficients."""

    shape = None
    volume_array = None

    def __init__(self, **kwargs):
        for key, val in kwargs.items():
            setattr(self, key, val)

    @property
    def device_bytes(self):
        return int(_native.load().hs2g_device_bytes(self.handle.ptr))

    def faces(self):
        """(Gz, Gy, Gx, capacity, fixed) as compiled: per-face conductances (W/m^3/K), rho*c/dt per voxel
        (1 for fixed voxels) and the fixed-temperature mask."""
        nz, ny, nx = self.shape
        Gz = np.empty((nz + 1, ny, nx))
        Gy = np.empty((nz, ny + 1, nx))
        Gx = np.empty((nz, ny, nx + 1))
        M = np.empty((nz, ny, nx))
        fixed = np.empty((nz, ny, nx), dtype=np.uint8)
        L = _native.load()
        _native.check(L.hs2g_get_faces(self.handle.ptr, Gz.ctypes.data, Gy.ctypes.data, Gx.ctypes.data,
                                       M.ctypes.data, fixed.ctypes.data))
        return Gz, Gy, Gx, M, fixed


class adi_step(object):
    """One ADI stage (the reference's pyadi_step, alternatingdirection_c_pyx.pyx:120-284): stage ``stepnum``
    solves along the last axis of ``permuteorder``.  ``Amat``, ``Bmat``, ``Cmats``, ``Dvec``, ``Lmat`` and
    ``Umat`` are rebuilt on demand from the compiled face conductances in the reference's matrix form (rows in
    the permuted order), for inspection; the timestep itself never uses them."""

    def __init__(self, params, permuteorder, stepnum):
        self.ADI_params = params
        self.permuteorder = tuple(permuteorder)
        inv = [0, 0, 0]
        for ind, pord in enumerate(permuteorder):
            inv[pord] = ind
        self.invpermuteorder = tuple(inv)
        self.permutedshape = [params.shape[i] for i in permuteorder]
        self.stepnum = stepnum
        self._mats = None

    def _build(self):
        if self._mats is None:
            from .introspect import stage_matrices
            self._mats = stage_matrices(self.ADI_params, self.stepnum)
        return self._mats

    Amat = property(lambda self: self._build()["A"])
    Bmat = property(lambda self: self._build()["B"])
    Cmats = property(lambda self: self._build()["C"])
    Dvec = property(lambda self: self._build()["D"])
    Lmat = property(lambda self: self._build()["L"])
    Umat = property(lambda self: self._build()["U"])


# --------------------------------------------------------------------------------------------------------
# sources
# --------------------------------------------------------------------------------------------------------
class _ClassSources(object):
    """The sources of a ``volumetric`` tuple, packed for hs2g_source_table.  Class-uniform kinds are evaluated
    per class; the kinds whose value differs between a class's voxels (point joules with per-voxel values or
    per-cell volumes, the z-decaying impulse) become HS2G_SHAPED_IMPULSE classes whose per-voxel values the
    device evaluates into the handle's source shape (``_prepare_shapes``)."""

    def __init__(self, volumetric, per_voxel_volume=False):
        """per_voxel_volume: the problem's cells differ in volume (curved-surface mode), so point-joules sources
        are evaluated per voxel (J / (V dt), pyx:309-313)."""
        n = len(volumetric)
        if n > _native.MAX_CLASSES:
            raise ValueError("at most 256 source classes")
        self.kind = np.zeros(max(n, 1), dtype=np.int32)
        self.params = np.zeros((max(n, 1), 4))
        self.shaped = []                    # (class index, source tuple) evaluated per voxel on the device
        for c, src in enumerate(volumetric):
            k = src[0]
            if k in (NO_SOURCE, IMPULSE_SOURCE, STEPPED_SOURCE):
                self.kind[c] = k
                vals = [float(v) for v in src[1:]]
                self.params[c, :len(vals)] = vals
            elif k == IMPULSE_POINT_SOURCE_JOULES:
                if isinstance(src[2], numbers.Number) and not per_voxel_volume:
                    self.kind[c] = k
                    self.params[c, :2] = (float(src[1]), float(src[2]))
                else:
                    self.kind[c] = _native.SHAPED_IMPULSE
                    self.params[c, 0] = float(src[1])
                    self.shaped.append((c, src))
            elif k == SPATIALLY_Z_DECAYING_TEMPORAL_IMPULSE:
                self.kind[c] = _native.SHAPED_IMPULSE
                self.params[c, 0] = float(src[1])
                self.shaped.append((c, src))
            else:
                raise ValueError("unknown volumetric source kind %r (class %d)" % (k, c))
        self.n = n


def _same_array(P, key, a):
    """True when ``a`` is the array last uploaded under ``key`` for this problem (same object, same memory),
    so the device keeps its copy; records ``a`` otherwise."""
    cache = P.__dict__.setdefault("_shape_arrays", {})
    old = cache.get(key)
    if old is not None and old[0] is a and old[1] == a.ctypes.data:
        return True
    cache[key] = (a, a.ctypes.data)
    return False


def _prepare_shapes(P, sources, times, dt, volumetric_elements):
    """Evaluate on the device the source shapes of the shaped classes that fire at one of ``times``
    (pyx:307-384).  A shape is re-evaluated when its source tuple, dt or the device's class map changed since
    it was evaluated; its per-voxel inputs (z coordinates, per-voxel joules, cell volumes) are uploaded once
    and kept on the device while the same arrays are passed."""
    if not sources.shaped:
        return
    L = _native.load()
    done = P.__dict__.setdefault("_shapes", {})
    tset = set(float(t) for t in times)
    for c, src in sources.shaped:
        if float(src[1]) not in tset:
            continue
        key = (tuple(id(v) for v in src), tuple(float(v) for v in src if isinstance(v, numbers.Number)), float(dt),
               id(P.compiled_volumetric))
        if done.get(c) == key:
            continue
        if src[0] == SPATIALLY_Z_DECAYING_TEMPORAL_IMPULSE:
            (_, t_imp, direc, offset, zgrid, ddz, jpm2, length) = src
            direc = np.asarray(direc, dtype="d")
            if not ((direc == np.array([1.0, 0.0, 0.0])).all() or (direc == np.array([-1.0, 0.0, 0.0])).all()):
                raise AssertionError("decay direction must be +z or -z")
            length = float(length)
            if not length > 0:
                raise AssertionError("characteristic length must be positive")
            z = np.asarray(zgrid, dtype="d")
            if z.shape != tuple(P.shape):
                z = np.broadcast_to(z, tuple(P.shape))
            z = np.ascontiguousarray(z)
            flags = _native.REUSE if _same_array(P, ("z", c), z) else 0
            _native.check(L.hs2g_source_zdecay(P.handle.ptr, c, z.ctypes.data, float(direc[0]), float(offset),
                                               abs(float(ddz)), float(jpm2), length, float(dt), flags))
        else:
            J = src[2]
            nsel = None
            if isinstance(J, numbers.Number):
                Ja = np.array([float(J)])
            else:
                Ja = np.ascontiguousarray(np.asarray(J, dtype="d").reshape(-1))
                if Ja.size != 1:
                    nsel = int(np.count_nonzero(np.asarray(volumetric_elements) == c))
                    if Ja.size != nsel:
                        raise ValueError("point source of class %d has %d values for %d voxels"
                                         % (c, Ja.size, nsel))
            flags = _native.REUSE if _same_array(P, ("J", c), Ja) else 0
            vols, volume = None, 1.0
            if np.ndim(P.volume_array) > 0:
                V = np.ascontiguousarray(P.volume_array, dtype="d")
                if not _same_array(P, ("V", c), V):
                    flags &= ~_native.REUSE      # joules and volumes are reused together or not at all
                vols = V.ctypes.data
            else:
                volume = float(P.volume_array)
            _native.check(L.hs2g_source_point(P.handle.ptr, c, Ja.ctypes.data, int(Ja.size), vols, volume,
                                              float(dt), flags))
        done[c] = key


def source_table(sources, t, dt, volume):
    """(qtab ndarray[256], any_active) for the class-uniform sources at time t."""
    qtab = np.zeros(_native.MAX_CLASSES)
    L = _native.load()
    # with per-cell volumes the point-joules sources are per voxel, so the table needs no volume
    vol = float(volume) if np.ndim(volume) == 0 else 1.0
    active = _native.check(L.hs2g_source_table(sources.n, sources.kind.ctypes.data, sources.params.ctypes.data,
                                               float(t), float(dt), vol, qtab.ctypes.data))
    return qtab, active > 0


# --------------------------------------------------------------------------------------------------------
# stepping
# --------------------------------------------------------------------------------------------------------
def _is_torch_cuda(x):
    try:
        import torch
    except ImportError:
        return False
    return isinstance(x, torch.Tensor) and x.is_cuda


def _class_map_update(P, volumetric_elements):
    """The host source-class map to upload when it differs from the one on the device, else None.  The caller
    records it as the device's map (``_class_map_uploaded``) only once the native call that uploads it has
    succeeded, so a failed call leaves the map to be uploaded again."""
    if volumetric_elements is None or volumetric_elements is P.compiled_volumetric:
        return None
    ve = np.ascontiguousarray(volumetric_elements, dtype=np.uint8)
    if ve.shape != tuple(P.shape):
        raise ValueError("volumetric_elements has shape %s, expected %s" % (ve.shape, tuple(P.shape)))
    if np.array_equal(ve, P.compiled_volumetric):
        return None
    return ve.copy()


def _class_map_uploaded(P, newmap):
    if newmap is not None:
        P.compiled_volumetric = newmap
        P.__dict__.pop("_shapes", None)     # the device dropped every source shape with the old map


def _upload_class_map(P, newmap):
    """Replace the device's source-class map before anything that reads it (the source shapes)."""
    if newmap is not None:
        _native.check(_native.load().hs2g_set_source_classes(P.handle.ptr, newmap.ctypes.data, 0))
        _class_map_uploaded(P, newmap)


def run_adi_steps(ADI_params, ADI_steps, t, dt, Tarray, volumetric_elements, volumetric):
    """Advance ``Tarray`` by one timestep; returns a new array (numpy in, numpy out; CUDA tensor in, tensor out)."""
    P = ADI_params
    L = _native.load()
    sources = _ClassSources(volumetric, np.ndim(P.volume_array) > 0)
    qtab, active = source_table(sources, t, dt, P.volume_array)
    on_dev = _is_torch_cuda(Tarray)
    if on_dev:
        import torch
        T = Tarray
        if T.dtype != torch.float64:
            raise ValueError("Tarray must be float64")
        if tuple(T.shape) != tuple(P.shape):
            raise ValueError("Tarray has shape %s, expected %s" % (tuple(T.shape), tuple(P.shape)))
        if T.device.index != P.device:
            raise ValueError("Tarray is on cuda:%d, the problem on cuda:%d" % (T.device.index, P.device))
        T = T.contiguous()
        stream = torch.cuda.current_stream(T.device)
        _native.check(L.hs2g_set_stream(P.handle.ptr, ctypes.c_void_p(stream.cuda_stream)))
    else:
        T = np.ascontiguousarray(Tarray, dtype="d")
        if T.shape != tuple(P.shape):
            raise ValueError("Tarray has shape %s, expected %s" % (T.shape, tuple(P.shape)))
        _native.check(L.hs2g_set_stream(P.handle.ptr, None))
    if active:
        # the step's sources read the device's class map (and, for shaped classes, their shapes): both are
        # brought up to date first, on the step's stream
        _upload_class_map(P, _class_map_update(P, volumetric_elements))
        _prepare_shapes(P, sources, (t,), dt, volumetric_elements)
    qptr = qtab.ctypes.data if active else None
    if on_dev:
        out = torch.empty_like(T)
        _native.check(L.hs2g_step(P.handle.ptr, T.data_ptr(), out.data_ptr(), qptr, None, None, _native.DEVICE))
        return out
    out = np.empty_like(T)
    _native.check(L.hs2g_step(P.handle.ptr, T.ctypes.data, out.ctypes.data, qptr, None, None, 0))
    return out


def run(ADI_params, Tarray, times, dt, volumetric_elements, volumetric, record_layer=None, record_surface=False):
    """Advance ``Tarray`` through one step per value in ``times`` (the t passed to each step), on the device.

    Equivalent to calling run_adi_steps once per t, with every step queued in one native call (the per-voxel
    source kinds included: their shapes are evaluated on the device before the first step).  Returns ``T``, or ``(T, history)`` of shape (len(times), ny, nx) recorded after every step:
    the layer z=record_layer with ``record_layer``, or with ``record_surface=True`` the z = 0 surface
    temperature as the reference's ``insulating_z_min_surface_temperature(T, dz)`` estimates it
    (heatsim2_gb300.surface_temperature)."""
    P = ADI_params
    L = _native.load()
    sources = _ClassSources(volumetric, np.ndim(P.volume_array) > 0)
    nz, ny, nx = P.shape
    if record_surface and record_layer is not None:
        raise ValueError("record_layer and record_surface are exclusive")
    if record_surface and nz < 2:
        raise ValueError("the surface estimate needs nz >= 2")
    recording = record_layer is not None or bool(record_surface)
    dz = float(P.spacing[0])
    times = [float(t) for t in times]
    n = len(times)
    on_dev = _is_torch_cuda(Tarray)
    if on_dev:
        import torch
        T = Tarray.contiguous().clone()
        hist = torch.empty((n, ny, nx), dtype=torch.float64, device=T.device) if recording else None
        stream = torch.cuda.current_stream(T.device)
        _native.check(L.hs2g_set_stream(P.handle.ptr, ctypes.c_void_p(stream.cuda_stream)))
        ptr = T.data_ptr()
        flags = _native.DEVICE
    else:
        T = np.ascontiguousarray(Tarray, dtype="d").copy()
        hist = np.empty((n, ny, nx)) if recording else None
        _native.check(L.hs2g_set_stream(P.handle.ptr, None))
        ptr = T.ctypes.data
        flags = 0
    qtabs = np.zeros((n, _native.MAX_CLASSES))
    any_active = False
    for s, t in enumerate(times):
        qtabs[s], act = source_table(sources, t, dt, P.volume_array)
        any_active |= act
    if any_active:
        # a changed source-class map and the shapes of the shaped classes that fire within the run are set on
        # the device first; the steps then run in one native call, firing steps included
        _upload_class_map(P, _class_map_update(P, volumetric_elements))
        _prepare_shapes(P, sources, times, dt, volumetric_elements)
    if hist is not None:
        hptr = hist.data_ptr() if on_dev else hist.ctypes.data
        if record_surface:
            _native.check(L.hs2g_run_surface(P.handle.ptr, n, ptr, ptr, qtabs.ctypes.data, dz, hptr, flags))
        else:
            _native.check(L.hs2g_run(P.handle.ptr, n, ptr, ptr, qtabs.ctypes.data, int(record_layer), hptr, flags))
    else:
        _native.check(L.hs2g_run(P.handle.ptr, n, ptr, ptr, qtabs.ctypes.data, 0, None, flags))
    if on_dev:
        stream.synchronize()
    return (T, hist) if recording else T
