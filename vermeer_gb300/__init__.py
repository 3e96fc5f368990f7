"""vermeer_gb300 - GB300-native (sm_103a) traversal and rendering path for
Vermeer scenes.

The compute path is libvmr (hand-written CUDA behind the C ABI in
include/vmr.h).  This package builds and binds it; there is no CPU fallback:
every entry point raises if the library or a CUDA device is missing.
"""
from .api import (BUILD_AUTO, BUILD_DEVICE, BUILD_HOST, MOTION_FAITHFUL, MOTION_FIXED, MNODE_DTYPE,  # noqa: F401
                  NODE_DTYPE, Context, VmrError)
from . import scenes  # noqa: F401

__all__ = ["Context", "VmrError", "NODE_DTYPE", "MNODE_DTYPE", "MOTION_FAITHFUL", "MOTION_FIXED", "BUILD_AUTO",
           "BUILD_HOST", "BUILD_DEVICE", "scenes"]
