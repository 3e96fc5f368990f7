"""vermeer_gb300 - GB300-native (sm_103a) traversal and rendering path for
Vermeer scenes.

The compute path is libvmr (hand-written CUDA behind the C ABI in
include/vmr.h).  This package builds and binds it; there is no CPU fallback:
every entry point raises if the library or a CUDA device is missing.
"""
from .api import (BUILD_AUTO, BUILD_DEVICE, BUILD_HOST, FILTER_AIRY, FILTER_BOX, FILTER_GAUSSIAN,  # noqa: F401
                  MOTION_FAITHFUL, MOTION_FIXED, MNODE_DTYPE, NODE_DTYPE, Context, VmrError, pixel_filter_warp,
                  render_path_split, render_split, split_rows, transform_keys_at, write_float)
from . import scenes  # noqa: F401

__all__ = ["Context", "VmrError", "NODE_DTYPE", "MNODE_DTYPE", "MOTION_FAITHFUL", "MOTION_FIXED", "BUILD_AUTO",
           "BUILD_HOST", "BUILD_DEVICE", "FILTER_BOX", "FILTER_GAUSSIAN", "FILTER_AIRY", "pixel_filter_warp", "transform_keys_at", "write_float",
           "split_rows", "render_split", "render_path_split", "scenes"]
