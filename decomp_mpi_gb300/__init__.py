"""decomp_mpi_gb300: single-GPU GB300 (sm_103a) implementation of Decomp_MPI's
decomposition-driven reshape and split 3D FFT.

The product is the C-ABI shared library ``libdecomp_gb300.so`` (headers in
``include/``); this package builds it and mirrors its interface in Python.
"""
from .api import (Comm, Decomp, DecompError, ReshapePlan, SplitPlan, build_parallel_plan,  # noqa: F401
                  decomp_from_spec, processor_grid, propose_parallel_plan)
from .build import LIB_PATH, build  # noqa: F401
