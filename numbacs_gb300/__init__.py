"""numbacs_gb300: GB300-native (sm_103a) flow-map -> FTLE -> ridge path.

A drop-in for NumbaCS's ``flowmap_grid_2D`` -> ``ftle_grid_2D`` / ``C_eig_2D``
-> ``ftle_ridge_pts`` / ``ftle_ridges`` path with the reference's call
signatures.  The compute runs in hand-written CUDA kernels (libnbcs.so, C ABI
in include/nbcs.h); there is no CPU fallback.
"""
from . import diagnostics, extraction, flows, integration  # noqa: F401
from .diagnostics import (C_eig_2D, C_eig_aux_2D, C_tensor_2D, ftle_evec_2D,  # noqa: F401
                          ftle_from_eig, ftle_grid_2D)
from .extraction import ftle_ordered_ridges, ftle_ridge_pts, ftle_ridges  # noqa: F401
from .flows import Flow, get_flow_2D, get_interp_arrays_2D, get_predefined_flow  # noqa: F401
from .integration import (UCGrid, flowmap, flowmap_aux_grid_2D, flowmap_composition,  # noqa: F401
                          flowmap_composition_initial, flowmap_composition_step, flowmap_grid_2D,
                          flowmap_grid_ND, flowmap_n, flowmap_n_grid_2D)

__version__ = "0.1.0"
