"""blamm_gb300: GB300-native (sm_103a) PWM scan for blamm's dict/hist/scan pipeline.

The compute path is libblamm_gpu.so (CUDA, C ABI in include/blamm_gpu.h); the
host side (motif files, PWMs, histograms, FASTA streaming, output) is C++ in
libblamm_host.so and the `blamm` command line.  This package holds the build
script, ctypes bindings and the synthetic workload generators.
"""
from ._native import (BLAMM_ERR_OVERFLOW, BLAMM_OK, HIT_DTYPE, MODES, BlammError, GpuScanner, Server,
                      gpu_lib)

__all__ = ["GpuScanner", "Server", "BlammError", "gpu_lib", "HIT_DTYPE", "MODES", "BLAMM_OK",
           "BLAMM_ERR_OVERFLOW"]
