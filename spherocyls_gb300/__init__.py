"""spherocyls_gb300 -- GB300 (sm_103a) implementation of the overdamped-dynamics hot
path of tmarschall/spherocyls: 2D bidisperse spherocylinder packings under
Lees-Edwards shear, pure shear and affine box resize, plus energy minimisation.

The work is done by ``libspherocyl`` (C++ host runtime + hand-written CUDA kernels,
C ABI in ``include/spherocyl.h``); this package binds it with ctypes.
"""
from ._lib import ScError, lib
from .box import (BoxBatch, SpherocylBox, generate_config, generate_config_rect, generate_packing,
                  generate_packing_device, read_positions, trim_memory, write_positions)

__all__ = ["BoxBatch", "SpherocylBox", "generate_config", "generate_config_rect",
           "generate_packing", "generate_packing_device", "read_positions", "trim_memory",
           "write_positions", "ScError", "lib"]
