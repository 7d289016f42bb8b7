"""GB300 GP-MOOD: one FP64 SSP-RK3 step of GP-MOOD on one GPU.

Package layout:
  csrc/        CUDA kernels (sm_103a) and the C ABI of libgpmood.so
  gpmood.py    ctypes binding mirroring the reference's time_stepping/Setdt/Boundary_C,
               plus the batched (Batch) and adjoint (Adjoint) entry points
  adjoint.py   torch.autograd front end of the adjoint (imports torch on use)
  nn_train.py  training of the a-priori MLP gate on the GPU kernels
  ic.py        initial conditions of the benchmark problems
  build.py     in-tree build of libgpmood.so
"""
from .gpmood import (DIRICHLET, DMR, DOUBLE_MACH800, FE, FOG, KH, MACH800, RMI, RT, FP_EXACT, FP_FAST, GP_MOOD, GP_SE, HLL, HLLC, LLF, NEUMANN, NGC, NN_GP_MOOD,
                     NN_GP_MOOD_CC, POL_MOOD, UNLIM_POL,
                     PERIODIC, REFLECTIVE, SSP_RK2, SSP_RK3, SSP_RK4, UNSPLIT, Adjoint, Batch, GpmoodError, Params,
                     Solver, default_params, gp_weights, load_library, padded, probe_fp64)

__all__ = ["DIRICHLET", "DMR", "DOUBLE_MACH800", "FE", "FOG", "KH", "MACH800", "RMI", "RT", "FP_EXACT", "FP_FAST", "GP_MOOD", "GP_SE", "HLL", "HLLC", "LLF", "NEUMANN", "NGC",
           "NN_GP_MOOD", "NN_GP_MOOD_CC", "POL_MOOD", "UNLIM_POL", "PERIODIC", "REFLECTIVE", "SSP_RK2", "SSP_RK3", "SSP_RK4", "UNSPLIT", "Adjoint", "Batch",
           "GpmoodError", "Params", "Solver", "default_params", "gp_weights", "load_library", "padded", "probe_fp64"]
