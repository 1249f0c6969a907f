"""Gradients of a surface-temperature misfit through the ADI step (libhs2g hs2g_adjoint_*).

No counterpart in the reference, which has no derivatives.  The model is the per-voxel form of the
reference's step: a box with per-voxel conductivity k (W/m/K), volumetric heat capacity C = rho*c (J/m^3/K)
and source amplitude q (W/m^3, scaled per step by a schedule), insulating outside and conducting inside with
the arithmetic face mean of boundary_conducting.py:7-71, or (``Adjoint.set_faces``) with the face classes of
a class problem -- conducting, insulating, thin insulating layers, any class affine in a scalar k -- and
fixed-temperature voxels.  The loss of an instance is
    J = sum_n sum_{y,x} (T_{n+1}[0, y, x] - obs[n, y, x])^2
(layer 0 is the heated surface).  The forward pass checkpoints T every ``ckpt`` steps; the backward pass
recomputes one segment at a time and runs the transposed tridiagonal solves in reverse order on the GPU.

Temperatures enter the device as offsets from the mean of T0 (observations shifted alike).  The step maps a
uniform field to itself and the misfit only sees differences, so loss and gradients are unchanged, while
double rounding applies to the temperature changes instead of to ~300 K.

``Adjoint`` drives the C ABI with numpy arrays (one instance or a batch of uneven instances in one
concatenated state; every sweep is one launch over all of them).  ``surface_misfit`` and
``batch_surface_misfit`` are the ``torch.autograd.Function`` forms on CUDA float64 tensors.
"""
import ctypes
import threading

import numpy as np

from . import _native
from .crank_nicolson import current_device


def _grid_structs(grids):
    out = (_native.AdjointGrid * len(grids))()
    for i, (shape, spacing) in enumerate(grids):
        nz, ny, nx = (int(v) for v in shape)
        dz, dy, dx = (float(v) for v in spacing)
        out[i] = _native.AdjointGrid(nz, ny, nx, dz, dy, dx)
    return out


class Adjoint(object):
    """One instance or a batch: ``grids`` is a list of ((nz, ny, nx), (dz, dy, dx)) pairs."""

    def __init__(self, grids, dt, device=None):
        self.grids = [(tuple(int(v) for v in g[0]), tuple(float(v) for v in g[1])) for g in grids]
        if not self.grids:
            raise ValueError("no instances")
        self.dt = float(dt)
        self.device = current_device() if device is None else int(device)
        L = _native.load()
        h = ctypes.c_void_p()
        _native.check(L.hs2g_adjoint_create(len(self.grids), _grid_structs(self.grids), self.dt, self.device,
                                            ctypes.byref(h)))
        self._h = h
        self.n = len(self.grids)
        self.offsets = np.zeros(self.n + 1, dtype=np.int64)
        _native.check(L.hs2g_adjoint_layout(h, self.offsets.ctypes.data))
        self.voxels = int(self.offsets[-1])
        self.nsteps = 0

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _native._lib is not None:
            _native._lib.hs2g_adjoint_destroy(h)
            self._h = None

    @property
    def device_bytes(self):
        return int(_native.load().hs2g_adjoint_device_bytes(self._h))

    def set_stream(self, stream):
        _native.check(_native.load().hs2g_adjoint_set_stream(self._h, stream))

    # -- numpy interface -------------------------------------------------------------------------------
    def _concat(self, fields, what):
        if self.n == 1 and not isinstance(fields, (list, tuple)):
            fields = [fields]
        if len(fields) != self.n:
            raise ValueError("%s: %d fields for %d instances" % (what, len(fields), self.n))
        buf = np.empty(self.voxels)
        for i, f in enumerate(fields):
            f = np.asarray(f, dtype="d")
            if f.shape != self.grids[i][0]:
                raise ValueError("%s of instance %d: shape %s, expected %s" % (what, i, f.shape, self.grids[i][0]))
            buf[self.offsets[i]:self.offsets[i + 1]] = f.reshape(-1)
        return buf

    def _split(self, buf):
        out = [buf[self.offsets[i]:self.offsets[i + 1]].reshape(self.grids[i][0]) for i in range(self.n)]
        return out[0] if self.n == 1 else out

    def set_faces(self, faces=None, fixed=None):
        """Face classes and fixed voxels (call before ``set_parameters``); None restores the default (every
        interior face conducting with the arithmetic mean of k, every voxel computed).

        ``faces``: per instance ``(boundaries, boundary_z_elements, boundary_y_elements, boundary_x_elements)``
        as ``heatsim2.setup`` takes them: a tuple of boundary classes ``(module, *extra)`` and uint8 class arrays
        of shapes (nz+1, ny, nx), (nz, ny+1, nx), (nz, ny, nx+1).  Each class is evaluated for scalar k into its
        affine face form (``face_forms``).  ``fixed``: per instance a (nz, ny, nx) mask of fixed-temperature
        voxels, or None.  Lists of them for a batch."""
        L = _native.load()
        if faces is None and fixed is None:
            _native.check(L.hs2g_adjoint_set_faces(self._h, 0, None, None, None, None, None, 0))
            return
        if faces is None:
            faces = [None] * self.n
        elif self.n == 1 and not isinstance(faces, list):
            faces = [faces]
        if fixed is not None and self.n == 1 and not isinstance(fixed, list):
            fixed = [fixed]
        if len(faces) != self.n or (fixed is not None and len(fixed) != self.n):
            raise ValueError("faces / fixed: one entry per instance")
        per = []
        for i, spec in enumerate(faces):
            shape, spacing = self.grids[i]
            fx_i = None if fixed is None or fixed[i] is None else np.asarray(fixed[i]).astype(bool)
            if fx_i is not None and fx_i.shape != shape:
                raise ValueError("fixed of instance %d: shape %s, expected %s" % (i, fx_i.shape, shape))
            per.append(face_classes(shape, spacing, spec, fx_i))
        nclass = max(f.shape[0] for f, _ in per)
        forms = np.zeros((self.n, nclass, 3, 3))
        for i, (f, _) in enumerate(per):
            forms[i, :f.shape[0]] = f
        cls = [np.empty(self.voxels, dtype=np.uint8) for _ in range(3)]
        for i, (_, low) in enumerate(per):
            for a in range(3):
                cls[a][self.offsets[i]:self.offsets[i + 1]] = low[a].reshape(-1)
        fixed_buf = None
        if fixed is not None:
            fixed_buf = np.zeros(self.voxels, dtype=np.uint8)
            for i, m in enumerate(fixed):
                if m is not None:
                    fixed_buf[self.offsets[i]:self.offsets[i + 1]] = np.asarray(m).astype(bool).reshape(-1)
        forms = np.ascontiguousarray(forms)
        _native.check(L.hs2g_adjoint_set_faces(self._h, nclass, forms.ctypes.data, cls[0].ctypes.data,
                                               cls[1].ctypes.data, cls[2].ctypes.data,
                                               None if fixed_buf is None else fixed_buf.ctypes.data, 0))

    def set_parameters(self, k, C, q):
        """Per-voxel k, C = rho*c and q: one (nz, ny, nx) array each, or lists of them for a batch."""
        bufs = [self._concat(a, w) for a, w in ((k, "k"), (C, "C"), (q, "q"))]
        if not all(np.isfinite(b).all() for b in bufs):
            raise ValueError("non-finite parameters")
        if (bufs[0] < 0).any() or (bufs[1] <= 0).any():
            raise ValueError("k must be >= 0 and C > 0")
        self._params = bufs  # keeps the host buffers alive until the copies finish (the call synchronises)
        _native.check(_native.load().hs2g_adjoint_set_parameters(self._h, *[b.ctypes.data for b in bufs], 0))

    def forward(self, T0, obs, schedule, ckpt=50, return_state=False):
        """Loss per instance (array of n).  obs: (nsteps, ny, nx) array per instance; schedule: nsteps source
        multipliers shared by all instances."""
        schedule = np.ascontiguousarray(schedule, dtype="d").reshape(-1)
        nsteps = schedule.size
        if nsteps < 1:
            raise ValueError("empty schedule")
        if self.n == 1 and not isinstance(obs, (list, tuple)):
            obs = [obs]
        if len(obs) != self.n:
            raise ValueError("obs: %d arrays for %d instances" % (len(obs), self.n))
        parts = []
        for i, o in enumerate(obs):
            o = np.asarray(o, dtype="d")
            nz, ny, nx = self.grids[i][0]
            if o.shape != (nsteps, ny, nx):
                raise ValueError("obs of instance %d: shape %s, expected %s" % (i, o.shape, (nsteps, ny, nx)))
            parts.append(o.reshape(-1))
        T0_buf = self._concat(T0, "T0")
        shift = [float(T0_buf[self.offsets[i]:self.offsets[i + 1]].mean()) for i in range(self.n)]
        for i in range(self.n):
            T0_buf[self.offsets[i]:self.offsets[i + 1]] -= shift[i]
            parts[i] = parts[i] - shift[i]
        obs_buf = np.concatenate(parts)
        loss = np.zeros(self.n)
        T_out = np.empty(self.voxels) if return_state else None
        ms = ctypes.c_double(0.0)
        _native.check(_native.load().hs2g_adjoint_forward(
            self._h, nsteps, schedule.ctypes.data, T0_buf.ctypes.data, obs_buf.ctypes.data, int(ckpt),
            loss.ctypes.data, None if T_out is None else T_out.ctypes.data, 0, ctypes.byref(ms)))
        self.nsteps = nsteps
        self.forward_ms = ms.value
        if return_state:
            for i in range(self.n):
                T_out[self.offsets[i]:self.offsets[i + 1]] += shift[i]
            return loss, self._split(T_out)
        return loss

    def backward(self):
        """(dJ/dk, dJ/dC, dJ/dq, dJ/dT0) of the last forward pass; lists for a batch."""
        out = [np.empty(self.voxels) for _ in range(4)]
        ms = ctypes.c_double(0.0)
        _native.check(_native.load().hs2g_adjoint_backward(self._h, *[b.ctypes.data for b in out], 0,
                                                           ctypes.byref(ms)))
        self.backward_ms = ms.value
        return tuple(self._split(b) for b in out)

    # -- device interface (torch CUDA float64 tensors, flat concatenated, no temperature shift); work is
    # queued on torch's current stream so it is ordered after the kernels that produced the tensors ----------
    def _torch_stream(self):
        import torch
        self.set_stream(torch.cuda.current_stream(self.device).cuda_stream)

    def set_parameters_device(self, k, C, q):
        self._torch_stream()
        _native.check(_native.load().hs2g_adjoint_set_parameters(self._h, k.data_ptr(), C.data_ptr(),
                                                                 q.data_ptr(), _native.DEVICE))

    def forward_device(self, T0, obs, schedule, ckpt):
        self._torch_stream()
        schedule = np.ascontiguousarray(schedule, dtype="d").reshape(-1)
        loss = np.zeros(self.n)
        ms = ctypes.c_double(0.0)
        _native.check(_native.load().hs2g_adjoint_forward(
            self._h, schedule.size, schedule.ctypes.data, T0.data_ptr(), obs.data_ptr(), int(ckpt),
            loss.ctypes.data, None, _native.DEVICE, ctypes.byref(ms)))
        self.nsteps = schedule.size
        self.forward_ms = ms.value
        return loss

    def backward_device(self, gk, gC, gq, gT0):
        self._torch_stream()
        ms = ctypes.c_double(0.0)
        _native.check(_native.load().hs2g_adjoint_backward(self._h, gk.data_ptr(), gC.data_ptr(), gq.data_ptr(),
                                                           gT0.data_ptr(), _native.DEVICE, ctypes.byref(ms)))
        self.backward_ms = ms.value


def face_forms(boundaries, spacing):
    """[nclass][3][3] affine scalar-k face forms (f0, flo, fhi) per class and axis (z, y, x): the conductance
    G = f0 + flo k_lo + fhi k_hi (W/m^3/K) each boundary class gives a face, from the same symbolic evaluation
    as ``setup`` (heatsim2_gb300.crank_nicolson.compile_boundary_forms).  Classes that use a conductivity
    tensor, or whose flux is not a two-point difference for every scalar k, raise ValueError."""
    from .crank_nicolson import compile_boundary_forms
    dz, dy, dx = spacing
    ff = compile_boundary_forms(boundaries, dz, dy, dx)
    K = _native.K_ENTRIES
    out = np.zeros((len(boundaries), 3, 3))
    for b in range(len(boundaries)):
        for a in range(3):
            f = ff[3 * b + a]
            normal = np.array(f.normal[:])
            if np.any(normal[2:1 + K]) or np.any(normal[2 + K:]):
                raise ValueError("boundary class %d: the adjoint takes a scalar k per voxel, this class uses the "
                                 "conductivity tensor" % b)
            for z in range(f.nzero):
                zf = np.array(f.zero[z][:])
                if zf[0] or zf[1] or zf[1 + K]:
                    raise ValueError("boundary class %d: its flux is not a two-point difference for scalar k "
                                     "(error %d)" % (b, f.zero_code[z]))
            out[b, a] = (normal[0], normal[1], normal[1 + K])
    return out


def face_classes(shape, spacing, spec, fixed=None):
    """(forms, (low_z, low_y, low_x)) of one instance: the class forms and each voxel's low-face class per axis.
    spec None: every interior face conducting (boundary_conducting's form).  Exterior faces next to a computed
    voxel must conduct nothing, as in the reference (alternatingdirection_c.c:158-163)."""
    nz, ny, nx = shape
    if spec is None:
        dz, dy, dx = spacing
        forms = np.zeros((1, 3, 3))
        for a, d in enumerate((dz, dy, dx)):
            forms[0, a] = (0.0, 0.5 / (d * d), 0.5 / (d * d))
        zeros = np.zeros(shape, dtype=np.uint8)
        return forms, (zeros, zeros, zeros)
    boundaries, bz, by, bx = spec
    forms = face_forms(boundaries, spacing)
    arrs = []
    for name, arr, want in (("boundary_z_elements", bz, (nz + 1, ny, nx)), ("boundary_y_elements", by, (nz, ny + 1, nx)),
                            ("boundary_x_elements", bx, (nz, ny, nx + 1))):
        arr = np.asarray(arr)
        if arr.dtype != np.uint8 or arr.shape != want:
            raise ValueError("%s must be a uint8 array of shape %s" % (name, want))
        if int(arr.max(initial=0)) >= len(boundaries):
            raise ValueError("%s holds a class past the boundaries tuple" % name)
        arrs.append(arr)
    bz, by, bx = arrs
    comp = np.ones(shape, dtype=bool) if fixed is None else ~np.asarray(fixed, dtype=bool)
    conducts = np.any(forms != 0.0, axis=2)     # [class][axis]
    # each exterior face class with the voxels beside it: low and high side of z, y, x
    exterior = ((0, bz[0], comp[0]), (0, bz[nz], comp[-1]), (1, by[:, 0], comp[:, 0]), (1, by[:, ny], comp[:, -1]),
                (2, bx[..., 0], comp[..., 0]), (2, bx[..., nx], comp[..., -1]))
    for a, outer, beside in exterior:
        if np.any(conducts[outer, a] & beside):
            raise ValueError("a computed voxel has a conducting exterior face (axis %d); the reference requires "
                             "exterior faces to be insulating" % a)
    low = (np.ascontiguousarray(bz[:nz]), np.ascontiguousarray(by[:, :ny]), np.ascontiguousarray(bx[:, :, :nx]))
    return forms, low


# handles idle between a forward and its backward are not shared; finished ones are reused per layout
_pool = {}
_pool_lock = threading.Lock()


def _take(key, grids, dt, device):
    with _pool_lock:
        free = _pool.get(key)
        if free:
            return free.pop()
    return Adjoint(grids, dt, device)


def _give(key, a):
    with _pool_lock:
        _pool.setdefault(key, []).append(a)


def _autograd_function():
    import torch

    class _BatchMisfit(torch.autograd.Function):
        """Flat concatenated k, C, q, T0 (float64, CUDA), obs concatenated per instance -> loss per instance."""

        @staticmethod
        def forward(ctx, k, C, q, T0, obs, grids, schedule, dt, ckpt, faces=None, fixed=None):
            for name, t in (("k", k), ("C", C), ("q", q), ("T0", T0), ("obs", obs)):
                if not t.is_cuda or t.dtype != torch.float64:
                    raise TypeError("%s must be a CUDA float64 tensor" % name)
            device = k.device.index if k.device.index is not None else torch.cuda.current_device()
            key = (tuple(grids), float(dt), device)
            a = _take(key, list(grids), dt, device)
            if a.voxels != k.numel() or T0.numel() != a.voxels or C.numel() != a.voxels or q.numel() != a.voxels:
                _give(key, a)
                raise ValueError("parameter sizes do not match the grids")
            nobs = sum(g[0][1] * g[0][2] for g in grids) * len(schedule)
            if obs.numel() != nobs:
                _give(key, a)
                raise ValueError("obs has %d values, expected %d" % (obs.numel(), nobs))
            with torch.cuda.device(device):
                k, C, q = (t.detach().contiguous() for t in (k, C, q))
                shift = T0.detach().mean()
                T0s = (T0.detach() - shift).contiguous()
                obss = (obs.detach() - shift).contiguous()
                a.set_faces(faces, fixed)          # pooled handles: the faces of this call, or the default
                a.set_parameters_device(k, C, q)
                loss = a.forward_device(T0s, obss, schedule, ckpt)
            ctx.adj, ctx.key = a, key
            return torch.tensor(loss, dtype=torch.float64, device=k.device)

        @staticmethod
        def backward(ctx, grad_loss):
            a = ctx.adj
            if a is None:
                raise RuntimeError("the adjoint of this forward pass was already taken (retain_graph is not "
                                   "supported)")
            ctx.adj = None
            dev = grad_loss.device
            g = [torch.empty(a.voxels, dtype=torch.float64, device=dev) for _ in range(4)]
            with torch.cuda.device(dev):
                a.backward_device(*g)
            _give(ctx.key, a)
            # scale each instance's gradient by its loss's incoming gradient
            scale = torch.repeat_interleave(grad_loss.to(torch.float64),
                                            torch.tensor(np.diff(a.offsets), device=dev))
            gk, gC, gq, gT0 = (t * scale for t in g)
            return gk, gC, gq, gT0, None, None, None, None, None, None, None

    return _BatchMisfit


_fn = None


def _function():
    global _fn
    if _fn is None:
        _fn = _autograd_function()
    return _fn


def batch_surface_misfit(k, C, q, T0, obs, schedule, spacing, dt, ckpt=50, faces=None, fixed=None):
    """Losses (tensor of n) of n instances; k, C, q, T0 lists of (nz_i, ny_i, nx_i) CUDA float64 tensors, obs a
    list of (nsteps, ny_i, nx_i) tensors, spacing one (dz, dy, dx) or a list of them.  Differentiable with
    respect to k, C, q and T0.  Temperatures are shifted by the mean of all T0 on the device.  faces / fixed:
    per instance, face classes and fixed voxels as ``Adjoint.set_faces`` takes them (lists, or None)."""
    import torch
    n = len(k)
    spacing = list(spacing) if isinstance(spacing[0], (list, tuple)) else [tuple(spacing)] * n
    grids = tuple((tuple(int(v) for v in k[i].shape), tuple(float(v) for v in spacing[i])) for i in range(n))
    flat = [torch.cat([t.reshape(-1) for t in arr]) for arr in (k, C, q, T0)]
    ob = torch.cat([o.reshape(-1) for o in obs])
    sched = tuple(float(v) for v in np.asarray(schedule, dtype="d").reshape(-1))
    return _function().apply(flat[0], flat[1], flat[2], flat[3], ob, grids, sched, float(dt), int(ckpt), faces,
                             fixed)


def surface_misfit(k, C, q, T0, obs, schedule, spacing, dt, ckpt=50, faces=None, fixed=None):
    """Loss (0-d tensor) of one instance: k, C, q, T0 (nz, ny, nx) and obs (nsteps, ny, nx) CUDA float64
    tensors.  Differentiable with respect to k, C, q and T0.  faces / fixed as ``Adjoint.set_faces``."""
    return batch_surface_misfit([k], [C], [q], [T0], [obs], schedule, spacing, dt, ckpt,
                                None if faces is None else [faces], None if fixed is None else [fixed])[0]
