"""GB300 (sm_103a) implementation of the QS3 matrix-free Lanczos hot path.

The compute path is libqs3g.so (ed_gb300/csrc, C ABI in include/qs3g.h);
``ed_gb300.capi`` binds it with ctypes and ``ed_gb300.inputs`` reads the QS3
input.dat / list_* formats.
"""
from . import inputs  # noqa: F401

__all__ = ["capi", "inputs", "build"]
