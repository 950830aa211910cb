"""openswpc_gb300 -- GB300-native (sm_103a) time loop of OpenSWPC's swpc_3d.

The CUDA kernels and the C ABI (include/swpc_gpu.h) live in
``openswpc_gb300/csrc`` and build into ``_build/libswpc_gb300.so``;
``openswpc_gb300.gpu`` binds that ABI, ``openswpc_gb300.configs`` writes the
synthetic benchmark inputs.
"""
from .gpu import Simulation, SwpcError, make_dims, lib  # noqa: F401

__version__ = "0.1.0"
