"""Surface temperature of an insulating z = 0 face (reference heatsim2/surface_temperature.py:4-36), on the device.

The reference estimates the temperature of the z = 0 surface, which lies half a layer above the centre of layer
0, from the first two layers of T[z, y, x]: a quadratic with zero slope at the surface (the face is
insulating) through the layer centres at dz/2 and 3 dz/2 gives

    a = (T1 - T0) / (2 dz^2),   c = T0 - 0.25 a dz^2,

a linear extrapolation gives T0 - (T1 - T0)/2, and the estimate is the mean of the two.  Here the same
operations, in the same order, run in a CUDA kernel (libhs2g ``hs2g_surface_temperature``); ``run(...,
record_surface=True)`` records the estimate after every step on the device (``hs2g_run_surface``), so a long
run need not copy the volume back.
"""
import ctypes

import numpy as np

from . import _native


def _device_index():
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.current_device()
    except ImportError:
        pass
    return 0


def insulating_z_min_surface_temperature(T, dz):
    """(ny, nx) temperature of the z = 0 surface estimated from T's layers 0 and 1.

    T: (nz, ny, nx) with nz >= 2, a numpy array (numpy result) or a float64 CUDA tensor (tensor result, computed
    on the tensor's device and current stream); dz: the layer thickness in m."""
    L = _native.load()
    dz = float(dz)
    if hasattr(T, "is_cuda") and T.is_cuda:
        import torch
        if T.dtype != torch.float64 or T.dim() != 3 or T.shape[0] < 2:
            raise ValueError("T must be a float64 (nz, ny, nx) tensor with nz >= 2")
        T = T.contiguous()
        out = torch.empty(tuple(T.shape[1:]), dtype=torch.float64, device=T.device)
        stream = torch.cuda.current_stream(T.device)
        _native.check(L.hs2g_surface_temperature(T.device.index, T.shape[0], T.shape[1], T.shape[2], T.data_ptr(),
                                                 dz, out.data_ptr(), ctypes.c_void_p(stream.cuda_stream),
                                                 _native.DEVICE))
        return out
    T = np.ascontiguousarray(T, dtype="d")
    if T.ndim != 3 or T.shape[0] < 2:
        raise ValueError("T must be (nz, ny, nx) with nz >= 2")
    out = np.empty(T.shape[1:])
    _native.check(L.hs2g_surface_temperature(_device_index(), T.shape[0], T.shape[1], T.shape[2], T.ctypes.data, dz,
                                             out.ctypes.data, None, 0))
    return out
