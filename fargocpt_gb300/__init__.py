"""fargocpt_gb300: GB300 (sm_103a) engine for FargoCPT's per-timestep gas step.

The hot path is CUDA behind a C ABI (include/fargocpt_gb300.h,
libfargocpt_gb300.so); this package holds its Python front end
(:mod:`.engine`), the host-side mirror of FargoCPT's run loop
(:mod:`.simulation`), the ctypes ABI mirror (:mod:`.abi`) and the build
(:mod:`.build`).
"""
from .abi import FgpuBody, FgpuParams, params_from_dict, params_to_dict  # noqa: F401

__all__ = ["FgpuBody", "FgpuParams", "params_from_dict", "params_to_dict"]
