"""sps_gb300 -- GB300 (sm_103a) implementation of the Stress-Particle SPH step.

The product is the native pair libsps_gb300.so (CUDA + the C-ABI of include/sps.h) and
libsph_host.so (set-up, include/sph_host.h).  This package is the Python binding over
them: `Problem` builds the initial module state, `Solver` advances it on the GPU.
"""
from ._abi import SPS_PREC_FP64_PLAIN, SPS_PREC_FP32_FAST  # noqa: F401
from .build import build_all, build_cuda, build_host, lib_path  # noqa: F401
from .problem import Problem, partition_by_size  # noqa: F401
from .context import autotune, Batch, Solver, StepContext, SpsError, gpu_lib, stream_of, kernels_per_step, profile_steps, selftest_division, selftest_convert, selftest_cone, set_surface_detection, lookahead, prefetch, set_lookahead, set_prefetch  # noqa: F401
