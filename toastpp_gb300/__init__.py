"""GB300-native FEM diffusion forward path (assembly, multi-source Krylov
solve, ProjectAll, nodal Jacobian) behind a C ABI, include/toastgpu.h."""
from .capi import (DATA_LIN, DATA_LOG, MEM_DEVICE, MEM_HOST, FwdSolver, Links, Mesh, ToastGPUError,  # noqa: F401
                   optical_coefficients, omega_of)
