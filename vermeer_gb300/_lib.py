"""ctypes declarations of libvmr's C ABI (include/vmr.h)."""
from __future__ import annotations

import ctypes
import os

from . import build as _build

P = ctypes.c_void_p
U32 = ctypes.c_uint32
I32 = ctypes.c_int32


class QbvhNode(ctypes.Structure):
    """qbvh.Node (qbvh/qbvh.go:31-36)."""
    _fields_ = [("boxes", ctypes.c_float * 24), ("axis0", U32), ("axis1", U32), ("axis2", U32),
                ("children", I32 * 4), ("parent", I32)]


class MqbvhNode(ctypes.Structure):
    """qbvh.MotionNode (qbvh/mqbvh.go:24-29)."""
    _fields_ = [("axis0", I32), ("axis1", I32), ("axis2", I32), ("children", I32 * 4), ("parent", I32),
                ("pad", U32 * 2)]


class MeshInput(ctypes.Structure):
    _fields_ = [("verts", P), ("n_verts", U32), ("motion_keys", U32), ("idxp", P), ("n_tris", U32),
                ("ray_bias", ctypes.c_float), ("motion_mode", ctypes.c_int), ("shader_idx", P)]


class MeshDesc(ctypes.Structure):
    _fields_ = [("verts", P), ("n_verts", U32), ("motion_keys", U32), ("idxp", P), ("n_tris", U32),
                ("accel_idx", P), ("ray_bias", ctypes.c_float), ("motion_mode", ctypes.c_int),
                ("nodes", P), ("n_nodes", U32), ("mnodes", P), ("n_mnodes", U32), ("mboxes", P),
                ("bounds", P), ("shader_idx", P)]


class Rays(ctypes.Structure):
    _fields_ = [(n, P) for n in ("px", "py", "pz", "dx", "dy", "dz", "tmax", "time")]


class Hits(ctypes.Structure):
    _fields_ = [(n, P) for n in ("prim", "geom", "t", "u", "v", "w")]


class Tuning(ctypes.Structure):
    _fields_ = [("kernel", ctypes.c_int), ("block", ctypes.c_int), ("blocks_per_sm", ctypes.c_int),
                ("refill_min", ctypes.c_int), ("walk_tail", ctypes.c_int), ("sort_bits", ctypes.c_int)]


class TraceJob(ctypes.Structure):
    _fields_ = [("geom", U32), ("pad", U32), ("n", ctypes.c_size_t), ("rays", Rays), ("hits", Hits)]


class TraceStats(ctypes.Structure):
    _fields_ = [("rays", ctypes.c_uint64), ("node_visits", ctypes.c_uint64), ("leaf_visits", ctypes.c_uint64),
                ("tri_tests", ctypes.c_uint64), ("kernel_ms", ctypes.c_float)]


class ShaderStd(ctypes.Structure):
    """vmr_shader_std (builtin/shader/std.go:25-47)."""
    _fields_ = [("flags", U32), ("emission_colour", ctypes.c_float * 3), ("emission_strength", ctypes.c_float),
                ("diffuse_colour", ctypes.c_float * 3), ("diffuse_strength", ctypes.c_float),
                ("diffuse_roughness", ctypes.c_float), ("spec1_colour", ctypes.c_float * 3),
                ("spec1_strength", ctypes.c_float), ("spec1_roughness", ctypes.c_float),
                ("spec1_fresnel", ctypes.c_int), ("spec1_fresnel_refl", ctypes.c_float * 3),
                ("spec1_fresnel_edge", ctypes.c_float * 3), ("ior", ctypes.c_float)]


class TriLight(ctypes.Structure):
    _fields_ = [("p0", ctypes.c_float * 3), ("p1", ctypes.c_float * 3), ("p2", ctypes.c_float * 3),
                ("samples", ctypes.c_int), ("shader", U32), ("geom", U32)]


class DiskLight(ctypes.Structure):
    _fields_ = [("P", ctypes.c_float * 3), ("up", ctypes.c_float * 3), ("lookat", ctypes.c_float * 3),
                ("radius", ctypes.c_float), ("samples", ctypes.c_int), ("shader", U32), ("geom", U32)]


class SphereLight(ctypes.Structure):
    _fields_ = [("P", ctypes.c_float * 3), ("radius", ctypes.c_float), ("samples", ctypes.c_int), ("shader", U32),
                ("geom", U32)]


class Camera(ctypes.Structure):
    _fields_ = [("m", ctypes.c_float * 16), ("tan_theta_focal", ctypes.c_float), ("aspect", ctypes.c_float),
                ("focal", ctypes.c_float), ("radius", ctypes.c_float)]


class PixelFilter(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("res", ctypes.c_int), ("width", ctypes.c_float), ("peak", ctypes.c_float)]


FILTER_BOX, FILTER_GAUSSIAN, FILTER_AIRY = 0, 1, 2
IO_DEVICE_IN, IO_DEVICE_OUT = 1, 2


class VnfInfo(ctypes.Structure):
    _fields_ = [("width", U32), ("height", U32), ("max_iter", ctypes.c_int), ("n_geoms", U32),
                ("n_shaders", U32), ("n_lights", U32), ("camera", ctypes.c_char * 64),
                ("output_hdr", ctypes.c_char * 256), ("output_float", ctypes.c_char * 256)]


VNF_MOTION_FIXED = 1


class RenderParams(ctypes.Structure):
    _fields_ = [("width", U32), ("height", U32), ("iter_begin", U32), ("iter_count", U32),
                ("seed", ctypes.c_uint64), ("max_batch_samples", U32), ("row_begin", U32), ("row_count", U32),
                ("flags", U32)]


class RenderStats(ctypes.Structure):
    _fields_ = [("samples", ctypes.c_uint64), ("camera_rays", ctypes.c_uint64), ("shadow_rays", ctypes.c_uint64),
                ("ms", ctypes.c_float)]


class QuadLight(ctypes.Structure):
    _fields_ = [("p0", ctypes.c_float * 3), ("e1", ctypes.c_float * 3), ("e2", ctypes.c_float * 3),
                ("shader", U32), ("geom", U32)]


class PathParams(ctypes.Structure):
    _fields_ = [("width", U32), ("height", U32), ("iter_begin", U32), ("iter_count", U32),
                ("seed", ctypes.c_uint64), ("max_depth", U32), ("rr_depth", U32), ("max_batch_samples", U32),
                ("flags", U32), ("fb64", P), ("guide_fraction", ctypes.c_float), ("train_steps", U32),
                ("train_batch", U32), ("train_lr", ctypes.c_float), ("guide_depth", U32), ("row_begin", U32),
                ("row_count", U32)]


class PathStats(ctypes.Structure):
    _fields_ = [("samples", ctypes.c_uint64), ("rays", ctypes.c_uint64), ("shadow_rays", ctypes.c_uint64),
                ("graph_replays", U32), ("ms", ctypes.c_float), ("train_records", ctypes.c_uint64),
                ("train_steps", U32), ("train_loss", ctypes.c_float)]


class PathJob(ctypes.Structure):
    _fields_ = [("geom", U32), ("width", U32), ("height", U32), ("camera", Camera), ("fb", P)]


PATH_NO_GRAPH = 1
PATH_GUIDED = 2
PATH_TRAIN = 4
PATH_SORT_QUEUES = 8
PATH_FIXED_SELECTION = 16
PATH_TWO_LEVEL = 32

GUIDE_WEIGHTS = 20032
GUIDE_OUTPUTS = 41


class Adam(ctypes.Structure):
    _fields_ = [("lr", ctypes.c_float), ("beta1", ctypes.c_float), ("beta2", ctypes.c_float), ("eps", ctypes.c_float)]

SHADER_FLAGS = {"emission_colour": 1, "emission_strength": 2, "diffuse_colour": 4, "diffuse_strength": 8,
                "diffuse_roughness": 16, "spec1_colour": 32, "spec1_strength": 64, "spec1_roughness": 128,
                "spec1_fresnel_refl": 256, "spec1_fresnel_edge": 512, "ior": 1024}
RENDER_F32 = 1  # vmr_render_params.flags
SH_DEBUG = 2048  # DebugShader: a shader dict with "debug": True and diffuse_colour = Colour

assert ctypes.sizeof(QbvhNode) == 128 and ctypes.sizeof(MqbvhNode) == 40

# name -> (restype, argtypes)
SIGNATURES = {
    "vmr_abi_version": (ctypes.c_int, []),
    "vmr_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(P)]),
    "vmr_destroy": (ctypes.c_int, [P]),
    "vmr_last_error": (ctypes.c_char_p, [P]),
    "vmr_set_stream": (ctypes.c_int, [P, P]),
    "vmr_sync": (ctypes.c_int, [P]),
    "vmr_set_tuning": (ctypes.c_int, [P, ctypes.POINTER(Tuning)]),
    "vmr_get_tuning": (ctypes.c_int, [P, ctypes.POINTER(Tuning)]),
    "vmr_trace_timing": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    "vmr_mesh_build": (ctypes.c_int, [P, ctypes.POINTER(MeshInput), ctypes.POINTER(U32)]),
    "vmr_set_builder": (ctypes.c_int, [P, ctypes.c_int]),
    "vmr_mesh_upload": (ctypes.c_int, [P, ctypes.POINTER(MeshDesc), ctypes.POINTER(U32)]),
    "vmr_mesh_info": (ctypes.c_int, [P, U32, P, P, P, P]),
    "vmr_mesh_export": (ctypes.c_int, [P, U32, P, P, P, P, P, P]),
    "vmr_scene_build": (ctypes.c_int, [P, P, U32]),
    "vmr_scene_upload": (ctypes.c_int, [P, P, U32, P, U32, P, U32, P, U32]),
    "vmr_scene_export": (ctypes.c_int, [P, P, P, P, P, P, P, P]),
    "vmr_trace_mesh": (ctypes.c_int, [P, U32, ctypes.POINTER(Rays), ctypes.c_size_t, ctypes.c_int,
                                      ctypes.POINTER(Hits), ctypes.POINTER(TraceStats)]),
    "vmr_trace_scene": (ctypes.c_int, [P, ctypes.POINTER(Rays), ctypes.c_size_t, ctypes.c_int,
                                       ctypes.POINTER(Hits), ctypes.POINTER(TraceStats)]),
    "vmr_set_shaders": (ctypes.c_int, [P, P, U32]),
    "vmr_mesh_set_shading": (ctypes.c_int, [P, U32, P, U32, P]),
    "vmr_mesh_set_motion_normals": (ctypes.c_int, [P, U32, P, U32, U32]),
    "vmr_set_lights": (ctypes.c_int, [P, P, U32]),
    "vmr_set_disk_lights": (ctypes.c_int, [P, P, U32]),
    "vmr_set_sphere_lights": (ctypes.c_int, [P, P, U32]),
    "vmr_sphere_add": (ctypes.c_int, [P, P, ctypes.c_float, ctypes.POINTER(U32)]),
    "vmr_set_camera": (ctypes.c_int, [P, ctypes.POINTER(Camera)]),
    "vmr_set_pixel_filter": (ctypes.c_int, [P, ctypes.POINTER(PixelFilter)]),
    "vmr_pixel_filter_warp": (ctypes.c_int, [ctypes.POINTER(PixelFilter), P, P, ctypes.c_size_t, P, P]),
    "vmr_encode_rgbe": (ctypes.c_int, [P, P, U32, U32, ctypes.c_int, P]),
    "vmr_load_vnf": (ctypes.c_int, [P, ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(VnfInfo)]),
    "vmr_get_camera": (ctypes.c_int, [P, ctypes.POINTER(Camera)]),
    "vmr_render": (ctypes.c_int, [P, ctypes.POINTER(RenderParams), P, ctypes.POINTER(RenderStats)]),
    "vmr_set_quad_lights": (ctypes.c_int, [P, P, U32]),
    "vmr_set_env_light": (ctypes.c_int, [P, P]),
    "vmr_render_path": (ctypes.c_int, [P, ctypes.POINTER(PathParams), P, ctypes.POINTER(PathStats)]),
    "vmr_render_path_jobs": (ctypes.c_int, [P, P, U32, ctypes.POINTER(PathParams), ctypes.POINTER(PathStats)]),
    "vmr_set_path_batch": (ctypes.c_int, [P, U32]),
    "vmr_mesh_set_transform": (ctypes.c_int, [P, U32, P]),
    "vmr_mesh_set_transform_keys": (ctypes.c_int, [P, U32, P, U32]),
    "vmr_instance_add": (ctypes.c_int, [P, U32, P, U32, P, P, ctypes.POINTER(U32)]),
    "vmr_proc_add": (ctypes.c_int, [P, P, U32, P, U32, P, P, ctypes.POINTER(U32)]),
    "vmr_set_camera_keys": (ctypes.c_int, [P, P, U32]),
    "vmr_transform_keys_at": (ctypes.c_int, [P, U32, ctypes.c_float, ctypes.c_int, P]),
    "vmr_get_camera_keys": (ctypes.c_int, [P, P, U32, ctypes.POINTER(U32)]),
    "vmr_render_split": (ctypes.c_int, [P, U32, ctypes.POINTER(RenderParams), P, ctypes.POINTER(RenderStats)]),
    "vmr_render_path_split": (ctypes.c_int, [P, U32, ctypes.POINTER(PathParams), P, ctypes.POINTER(PathStats)]),
    "vmr_split_rows": (ctypes.c_int, [U32, U32, P, P]),
    "vmr_selftest_wait": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_float)]),
    "vmr_get_path_batch": (ctypes.c_int, [P, ctypes.POINTER(U32)]),
    "vmr_autotune_path": (ctypes.c_int, [P, ctypes.POINTER(PathParams), P, P, ctypes.POINTER(U32),
                                         ctypes.POINTER(U32)]),
    "vmr_guide_init": (ctypes.c_int, [P, ctypes.c_uint64]),
    "vmr_guide_set_weights": (ctypes.c_int, [P, P]),
    "vmr_guide_get_weights": (ctypes.c_int, [P, P]),
    "vmr_guide_forward": (ctypes.c_int, [P, P, P, P, ctypes.c_size_t, P, P, P]),
    "vmr_guide_gradient": (ctypes.c_int, [P, P, P, P, P, P, P, ctypes.c_float, ctypes.c_size_t, P, P, P,
                                          ctypes.POINTER(ctypes.c_float)]),
    "vmr_guide_train_step": (ctypes.c_int, [P, P, P, P, P, P, P, ctypes.c_float, ctypes.c_size_t, P, P,
                                            ctypes.POINTER(Adam), ctypes.POINTER(ctypes.c_float)]),
    "vmr_autotune": (ctypes.c_int, [P, U32, ctypes.POINTER(Rays), ctypes.c_size_t, ctypes.c_int,
                                    ctypes.POINTER(Tuning), ctypes.POINTER(ctypes.c_float), ctypes.POINTER(U32)]),
    "vmr_clear_tuning": (ctypes.c_int, [P, U32]),
    "vmr_trace_jobs": (ctypes.c_int, [P, P, U32, ctypes.c_int, ctypes.POINTER(TraceStats)]),
    "vmr_trace_mesh_noalloc": (ctypes.c_int, [P, U32, ctypes.POINTER(Rays), ctypes.c_size_t, ctypes.c_int,
                                              ctypes.POINTER(Hits)]),
}

_lib = None


def load(build_if_missing: bool = True):
    """Load libvmr.  Raises if it cannot be built or loaded: there is no
    fallback implementation."""
    global _lib
    if _lib is None:
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"libvmr not built ({path}); run vermeer_gb300.build.build()")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def shader_struct(d: dict) -> ShaderStd:
    """A ShaderStd parameter dict (keys as in SHADER_FLAGS, plus
    'spec1_fresnel': 'Dielectric' | 'Metal') as the C struct."""
    sh = ShaderStd()
    flags = 0
    for k, bit in SHADER_FLAGS.items():
        if k in d:
            flags |= bit
            v = d[k]
            if isinstance(getattr(sh, k), float):
                setattr(sh, k, float(v))
            else:
                for i in range(3):
                    getattr(sh, k)[i] = float(v[i])
    sh.flags = flags | (SH_DEBUG if d.get("debug") else 0)
    sh.spec1_fresnel = 1 if d.get("spec1_fresnel") == "Metal" else 0
    return sh


def exported_symbols():
    return list(SIGNATURES)


def extra_symbols():
    """Declared functions bound by other modules of the package."""
    return []
