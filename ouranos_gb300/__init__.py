"""GB300-native transport-sweep operator for discontinuous-Galerkin S_N
radiative transfer (a drop-in for the RadiativeTransfer operator of
Rombur/ouranos).  The compute path is the CUDA library built from
ouranos_gb300/csrc; see include/ouranos_gb300.h for the C-ABI."""
from . import _capi
from .problem import (Problem, Quadrature, SplitMix64, batch_2d, build_quadrature, config_small,
                      heterogeneous_2d, pulse_strength, thick_3d, time_dependent_3d, uniform_problem,
                      zorder_cells)
from .transport import RadiativeTransfer
from .batch import Batch

__all__ = ["Problem", "Quadrature", "SplitMix64", "RadiativeTransfer", "Batch", "build_quadrature",
           "config_small", "heterogeneous_2d", "thick_3d", "batch_2d", "time_dependent_3d", "pulse_strength",
           "uniform_problem", "zorder_cells"]


def build(force=False, verbose=False):
    """Compile the CUDA library in-tree (nvcc, sm_103a)."""
    from .build import build as _build
    return _build(force=force, verbose=verbose)
