"""GB300-native matrix-free frequency-domain CSEM solve.

A drop-in for the hot path of yangpl/demo_matrixfree_csem (fdfd.c, solver.c,
cdotprod.c, airbc_init_free.c, inject_extract.c, gmres_init_free.c): hand-written
sm_103a CUDA kernels behind a C ABI (include/csem_gpu.h, include/csem_host.h), a host
layer in C that keeps the reference's key=value driver, float32 model files and
emf_NNNN.txt output, and Python bindings (api.py).
"""
from .api import (CHANNELS, STATUS, CsemError, Ctx, Grid, cdot, device_count, iom_of,  # noqa: F401
                  launch_count, lib, partition_systems, profile, profile_read, solve_batch,
                  solve_batch_multi, solve_batches)
