"""GB300-native lattice Boltzmann solver core with the reference's LBM interface.

The compute path is the sm_103a CUDA library behind include/lbm_capi.h (built in-tree by
``fluidx3d_gb300.build``); this package is its Python host mirror. There is no CPU fallback.
"""
from .setups import TYPE_S, TYPE_E, TYPE_T, TYPE_F, TYPE_I, TYPE_G, TYPE_X, TYPE_Y  # noqa: F401
from ._capi import LBMError, relaxation_rate  # noqa: F401
from .lbm import LBM, Field  # noqa: F401
from .mesh import Mesh, read_stl, write_stl, ellipsoid_mesh, sphere_mesh  # noqa: F401
from .units import Units, units  # noqa: F401

__all__ = ["LBM", "Field", "LBMError", "Mesh", "read_stl", "write_stl", "ellipsoid_mesh", "sphere_mesh", "relaxation_rate", "Units", "units",
           "TYPE_S", "TYPE_E", "TYPE_T", "TYPE_F", "TYPE_I", "TYPE_G", "TYPE_X", "TYPE_Y"]
