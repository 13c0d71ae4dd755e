"""GB300 Brownian-dynamics engine for the ccp chromatin model.

The engine is the C-ABI library libccpgpu.so (include/ccpgpu.h) built from
tfm_gb300/csrc by tfm_gb300/build.py; tfm_gb300.ccpgpu binds it with ctypes.
"""
__all__ = ["ccpgpu", "build"]
