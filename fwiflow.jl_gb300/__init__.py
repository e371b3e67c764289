"""fwiflow_gb300: GB300-native elastic FWI operator with FwiFlow.jl's surface.

The directory is `fwiflow.jl_gb300/`; it is imported under the module name
`fwiflow_gb300` (see `load_package` in __graft_entry__.py).
"""
from .utils import (FWIGeometry, default_nPad, padding, paraGen, sourceGene, surveyGen, surveyGen_shots,
                    velocity_to_moduli)
from .fwi import (FWI, FwiContext, FwiOpFunction, compute_misfit, compute_observation, fwi_obs_op, fwi_op,
                  fwi_op_grad)
from ._lib import FwiError, LIB_PATH
from . import gradcheck, inversion, precond, shots, synthetic

__all__ = [
    "FWI", "FwiContext", "FwiOpFunction", "FwiError", "FWIGeometry", "LIB_PATH", "compute_misfit",
    "compute_observation", "default_nPad", "fwi_obs_op", "fwi_op", "fwi_op_grad", "padding", "paraGen",
    "sourceGene", "surveyGen", "surveyGen_shots", "velocity_to_moduli",
]
