"""A module-like object with the reference API's public names, for driving the oracle from a spec.

The oracle recognises boundary classes by module name, so name-only stand-ins suffice."""
import types


class _HS(object):
    TEMPERATURE_COMPUTE = 0
    TEMPERATURE_FIXED = 1
    NO_SOURCE = 0
    IMPULSE_SOURCE = 1
    STEPPED_SOURCE = 2
    IMPULSE_POINT_SOURCE_JOULES = 3
    SPATIALLY_Z_DECAYING_TEMPORAL_IMPULSE = 4

    def __init__(self):
        for n in ("insulating", "conducting", "conducting_anisotropic", "thininsulatinglayer"):
            setattr(self, "boundary_" + n, types.ModuleType("oracle_shim.boundary_" + n))


HS = _HS()
