"""heatsim2_gb300: heatsim2's ADI Crank-Nicolson heat-conduction timestep on NVIDIA GB300 (sm_103a).

Drop-in for the reference package's hot path (isuthermography/heatsim2, heatsim2/__init__.py):

    import heatsim2_gb300 as heatsim2
    (ADI_params, ADI_steps) = heatsim2.setup(z0, y0, x0, dz, dy, dx, nz, ny, nx, dt, materials, boundaries,
                                             volumetric, material_elements, boundary_z_elements,
                                             boundary_y_elements, boundary_x_elements, volumetric_elements)
    T = heatsim2.run_adi_steps(ADI_params, ADI_steps, t, dt, T, volumetric_elements, volumetric)

Same material / boundary / source tuples, the same four boundary-class modules and the same uint8 class
arrays.  ``install_as_heatsim2()`` registers this package under the name ``heatsim2`` so existing scripts and
user boundary classes that import ``heatsim2.expression.group`` run unchanged.  ``setup`` also takes the
reference's surface-curvature arrays (curved-surface mode, ``heatsim2_gb300.curvature``).

Beside the drop-in: ``heatsim2_gb300.batch.Batch`` advances many problems of uneven size together (FP64, or
FP32 with its error against FP64 measured), and ``heatsim2_gb300.adjoint`` gives gradients of a surface
misfit with respect to per-voxel conductivity, heat capacity and source (``torch.autograd.Function`` forms).
"""
import os
import sys

import numpy as np

from . import boundary_conducting  # noqa: F401
from . import boundary_conducting_anisotropic  # noqa: F401
from . import boundary_insulating  # noqa: F401
from . import boundary_thininsulatinglayer  # noqa: F401
from . import expression  # noqa: F401
from . import crank_nicolson  # noqa: F401
from . import alternatingdirection  # noqa: F401
from . import surface_temperature  # noqa: F401
from .crank_nicolson import setup, UnalignedAnisotropyError  # noqa: F401
from .alternatingdirection import run_adi_steps, run  # noqa: F401

__version__ = "0.1.0"

# material[0] (heatsim2/__init__.py:42-43 in the reference)
TEMPERATURE_COMPUTE = 0
TEMPERATURE_FIXED = 1

# volumetric[0] (heatsim2/__init__.py:46-50)
NO_SOURCE = 0
IMPULSE_SOURCE = 1
STEPPED_SOURCE = 2
IMPULSE_POINT_SOURCE_JOULES = 3
SPATIALLY_Z_DECAYING_TEMPORAL_IMPULSE = 4


def _meshgrids(z_bnd, y_bnd, x_bnd, z, y, x):
    zb = np.meshgrid(z_bnd, y, x, indexing="ij")
    yb = np.meshgrid(z, y_bnd, x, indexing="ij")
    xb = np.meshgrid(z, y, x_bnd, indexing="ij")
    zgrid, ygrid, xgrid = np.meshgrid(z, y, x, indexing="ij")
    r3d = np.sqrt(xgrid ** 2 + ygrid ** 2 + zgrid ** 2)
    r2d = np.sqrt(xgrid ** 2 + ygrid ** 2)
    return zgrid, ygrid, xgrid, zb, yb, xb, r3d, r2d


def build_grid(minz, maxz, nz, miny, maxy, ny, minx, maxx, nx):
    """Grid with cell boundaries at min..max on each axis (reference heatsim2/__init__.py:53-99).

    Returns (dz,dy,dx, z,y,x, zgrid,ygrid,xgrid, z_bnd,y_bnd,x_bnd, z_bnd_z,z_bnd_y,z_bnd_x,
    y_bnd_z,y_bnd_y,y_bnd_x, x_bnd_z,x_bnd_y,x_bnd_x, r3d,r2d)."""
    z_bnd, dz = np.linspace(minz, maxz, num=nz + 1, retstep=True)
    y_bnd, dy = np.linspace(miny, maxy, num=ny + 1, retstep=True)
    x_bnd, dx = np.linspace(minx, maxx, num=nx + 1, retstep=True)
    z = z_bnd[:-1] + dz / 2.0
    y = y_bnd[:-1] + dy / 2.0
    x = x_bnd[:-1] + dx / 2.0
    zgrid, ygrid, xgrid, zb, yb, xb, r3d, r2d = _meshgrids(z_bnd, y_bnd, x_bnd, z, y, x)
    return (dz, dy, dx, z, y, x, zgrid, ygrid, xgrid, z_bnd, y_bnd, x_bnd) + tuple(zb) + tuple(yb) + tuple(xb) + \
        (r3d, r2d)


def _grid_from_bounds(z_bnd, y_bnd, x_bnd, dz, dy, dx):
    z = z_bnd[:-1] + dz / 2.0
    y = y_bnd[:-1] + dy / 2.0
    x = x_bnd[:-1] + dx / 2.0
    zgrid, ygrid, xgrid, zb, yb, xb, r3d, r2d = _meshgrids(z_bnd, y_bnd, x_bnd, z, y, x)
    return (z, y, x, zgrid, ygrid, xgrid, z_bnd, y_bnd, x_bnd) + tuple(zb) + tuple(yb) + tuple(xb) + (r3d, r2d)


def build_grid_min_step(minzcenter, dz, nz, minycenter, dy, ny, minxcenter, dx, nx):
    """Grid from the first cell centre and the step on each axis (reference heatsim2/__init__.py:102-142)."""
    z_bnd = minzcenter - dz / 2.0 + np.arange(nz + 1, dtype="d") * dz
    y_bnd = minycenter - dy / 2.0 + np.arange(ny + 1, dtype="d") * dy
    x_bnd = minxcenter - dx / 2.0 + np.arange(nx + 1, dtype="d") * dx
    return _grid_from_bounds(z_bnd, y_bnd, x_bnd, dz, dy, dx)


def build_grid_min_step_edge(minzedge, dz, nz, minyedge, dy, ny, minxedge, dx, nx):
    """Grid from the first cell edge and the step on each axis (reference heatsim2/__init__.py:147-185)."""
    z_bnd = minzedge + np.arange(nz + 1, dtype="d") * dz
    y_bnd = minyedge + np.arange(ny + 1, dtype="d") * dy
    x_bnd = minxedge + np.arange(nx + 1, dtype="d") * dx
    return _grid_from_bounds(z_bnd, y_bnd, x_bnd, dz, dy, dx)


def zero_elements(nz, ny, nx):
    """uint8 class arrays: material (nz,ny,nx), boundary z (nz+1,ny,nx), y (nz,ny+1,nx), x (nz,ny,nx+1) and
    volumetric (nz,ny,nx) (reference heatsim2/__init__.py:191-197)."""
    return (np.zeros((nz, ny, nx), dtype="u1"), np.zeros((nz + 1, ny, nx), dtype="u1"),
            np.zeros((nz, ny + 1, nx), dtype="u1"), np.zeros((nz, ny, nx + 1), dtype="u1"),
            np.zeros((nz, ny, nx), dtype="u1"))


def install_as_heatsim2():
    """Make ``import heatsim2`` (and ``heatsim2.expression`` etc.) resolve to this package."""
    me = sys.modules[__name__]
    sys.modules["heatsim2"] = me
    for sub in ("expression", "crank_nicolson", "alternatingdirection", "boundary_conducting",
                "boundary_conducting_anisotropic", "boundary_insulating", "boundary_thininsulatinglayer",
                "surface_temperature"):
        sys.modules["heatsim2." + sub] = sys.modules[__name__ + "." + sub]
    sys.modules["heatsim2.alternatingdirection_c_pyx"] = sys.modules[__name__ + ".alternatingdirection"]
    return me


def native_library_path():
    from . import _native
    return _native.lib_path()
