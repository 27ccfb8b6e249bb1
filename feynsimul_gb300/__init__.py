"""feynsimul_gb300 -- GB300-native path-integral Monte Carlo behind FeynSimul's plugin API.

Modules mirror the reference package: ``kernel_args`` (KernelArgs), ``kernel``
(PIMCKernel), ``pimc_utils`` (modN), ``physical_systems``.  The compute path is the CUDA
library ``libfeynsimul_gb300.so`` (include/feynsimul.h), built by
``python -m feynsimul_gb300.build``.
"""
__all__ = ["kernel", "kernel_args", "pimc_utils"]
__version__ = "0.1.0"
