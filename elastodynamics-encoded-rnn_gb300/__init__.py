"""GB300-native ERNN propagation: the time-recurrent anisotropic elastic FD cell
and its hand-written adjoint, running in libernn_gb300.so (sm_103a).

Public surface:
  CFRPWaveSimulatorRicker, SpatiallyVaryingAnisotropicSimulator
      drop-in replacements of the reference's simulator modules;
  ShotGatherSimulator, DegradationSimulator
      receiver-trace and degradation-map forms;
  ErnnPropagate / propagate, Geometry
      the autograd Function over the C ABI;
  elastic_operator_with_force
      one application of the operator;
  series_misfit, parameter_loss, damage_loss
      the inverters' objectives as fused device passes (loss and adjoint source);
  sources, materials, configs, harness
      source signals and loads, in-plane rotation and stability, benchmark
      configurations (numpy only) and the inversion iteration built on them.
"""
from . import _lib, autotune, configs, fem, formats, materials, misfit, sources
from ._lib import PATH_AUTO, PATH_RESIDENT, PATH_STEP, PATH_TILED
from .propagate import (MODE_DFIELD, MODE_FIELDS, MODE_SCALAR, RECORD_FIELDS,
                        RECORD_RECEIVERS, ErnnPropagate, Geometry, check_device_status,
                        elastic_operator_with_force, propagate)
from .simulators import (CFRPWaveSimulatorRicker, DegradationSimulator, ShotGatherSimulator,
                         SpatiallyVaryingAnisotropicSimulator, damage_loss, parameter_loss,
                         total_variation_2d)
from .misfit import series_misfit

__all__ = [
    "CFRPWaveSimulatorRicker", "SpatiallyVaryingAnisotropicSimulator", "ShotGatherSimulator",
    "DegradationSimulator", "damage_loss", "parameter_loss", "series_misfit",
    "total_variation_2d", "ErnnPropagate", "Geometry", "propagate", "elastic_operator_with_force",
    "sources", "materials", "configs", "formats", "fem", "autotune", "misfit", "MODE_SCALAR", "MODE_DFIELD",
    "MODE_FIELDS", "RECORD_FIELDS", "RECORD_RECEIVERS", "PATH_AUTO", "PATH_STEP",
    "PATH_RESIDENT", "PATH_TILED", "check_device_status", "load_library",
]


def load_library():
    """Load (building in-tree if needed) libernn_gb300.so; raises if unavailable."""
    return _lib.load()
