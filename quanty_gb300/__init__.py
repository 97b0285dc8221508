"""GB300 (sm_103a) engine for second-quantized operators on Slater-determinant wavefunctions.

The numerical work runs in libqgpu.so (C ABI in include/qgpu.h, CUDA sources in csrc/);
``api`` mirrors the reference's operator/wavefunction interface on top of it.  Nothing here
falls back to the CPU: without the built library or a GPU the calls raise.
"""
from . import qgpu  # noqa: F401

__all__ = ["qgpu", "api", "build"]
