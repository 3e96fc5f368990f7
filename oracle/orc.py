"""ctypes wrapper of the CPU oracle (oracle/_build/liborc.so).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path.  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import
this module.  The product package ``vermeer_gb300`` never does.

Every entry point restates a reference function; the C++ sources cite the
file:line of each (oracle/orc_core.cpp, oracle/orc_ldseq.cpp,
oracle/orc_render.cpp).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liborc.so")
_lib = None

ORC_NODE_DTYPE = np.dtype([
    ("boxes", "<f4", (24,)),
    ("axis", "<u4", (3,)),
    ("children", "<i4", (4,)),
    ("parent", "<i4"),
])
ORC_MNODE_DTYPE = np.dtype([
    ("axis", "<i4", (3,)),
    ("children", "<i4", (4,)),
    ("parent", "<i4"),
    ("pad", "<u4", (2,)),
])
assert ORC_NODE_DTYPE.itemsize == 128 and ORC_MNODE_DTYPE.itemsize == 40


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, -ffp-contract=off); make
    rebuilds only when a source is newer than the library."""
    subprocess.run(["make", "-s", "-C", _HERE] + (["-B"] if force else []), check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        L.orc_mesh_create.restype = P
        L.orc_mesh_create.argtypes = [P, ctypes.c_uint32, ctypes.c_uint32, P, ctypes.c_uint32,
                                      ctypes.c_float, ctypes.c_int]
        L.orc_mesh_destroy.argtypes = [P]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_mesh_info.argtypes = [P, P, P, P]
        L.orc_mesh_export.argtypes = [P, P, P, P, P, P]
        L.orc_trace_mesh.restype = ctypes.c_int
        L.orc_trace_mesh.argtypes = [P, P, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                     P, P, P, P, P, P]
        L.orc_scene_create.restype = P
        L.orc_scene_create.argtypes = [P, ctypes.c_uint32]
        L.orc_scene_destroy.argtypes = [P]
        L.orc_scene_info.argtypes = [P, P, P, P]
        L.orc_scene_export.argtypes = [P, P, P, P, P]
        L.orc_trace_scene.restype = ctypes.c_int
        L.orc_trace_scene.argtypes = [P, P, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                                      P, P, P, P, P, P, P]
        L.orc_vdc.restype = ctypes.c_uint64
        L.orc_vdc.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.orc_sobol.restype = ctypes.c_uint64
        L.orc_sobol.argtypes = [ctypes.c_uint64, ctypes.c_uint64]
        L.orc_raster_xy.restype = ctypes.c_uint64
        L.orc_raster_xy.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                    ctypes.c_uint32, ctypes.c_uint64, ctypes.c_uint64,
                                    ctypes.POINTER(ctypes.c_double),
                                    ctypes.POINTER(ctypes.c_double)]
        L.orc_vdc_sobol_tables.argtypes = [ctypes.c_uint32, P, P]
        L.orc_scene_create_ids.restype = P
        L.orc_scene_create_ids.argtypes = [P, P, ctypes.c_uint32]
        L.orc_mesh_set_transform_keys.argtypes = [P, P, ctypes.c_uint32]
        L.orc_instance_create.restype = P
        L.orc_instance_create.argtypes = [P, P, ctypes.c_uint32, P, P]
        L.orc_proc_create.restype = P
        L.orc_proc_create.argtypes = [P, P, ctypes.c_uint32, P, ctypes.c_uint32, P, P]
        L.orc_decompose.argtypes = [P, P]
        L.orc_keyed_matrix.restype = ctypes.c_int
        L.orc_keyed_matrix.argtypes = [P, ctypes.c_uint32, ctypes.c_float, ctypes.c_int, P]
        L.orc_render_set_camera_keys.restype = ctypes.c_int
        L.orc_render_set_camera_keys.argtypes = [P, P, ctypes.c_uint32]
        L.orc_set_normalize_mode.argtypes = [ctypes.c_int, ctypes.c_uint64]
        _register_render(L)
        _lib = L
    return _lib


class OrcShader(ctypes.Structure):
    _fields_ = [("flags", ctypes.c_uint32), ("emission_colour", ctypes.c_float * 3),
                ("emission_strength", ctypes.c_float), ("diffuse_colour", ctypes.c_float * 3),
                ("diffuse_strength", ctypes.c_float), ("diffuse_roughness", ctypes.c_float),
                ("spec1_colour", ctypes.c_float * 3), ("spec1_strength", ctypes.c_float),
                ("spec1_roughness", ctypes.c_float), ("spec1_fresnel", ctypes.c_int),
                ("spec1_fresnel_refl", ctypes.c_float * 3), ("spec1_fresnel_edge", ctypes.c_float * 3),
                ("ior", ctypes.c_float)]


class OrcTriLight(ctypes.Structure):
    _fields_ = [("p0", ctypes.c_float * 3), ("p1", ctypes.c_float * 3), ("p2", ctypes.c_float * 3),
                ("samples", ctypes.c_int), ("shader", ctypes.c_uint32), ("mesh", ctypes.c_uint32)]


class OrcDiskLight(ctypes.Structure):
    _fields_ = [("P", ctypes.c_float * 3), ("up", ctypes.c_float * 3), ("lookat", ctypes.c_float * 3),
                ("radius", ctypes.c_float), ("samples", ctypes.c_int), ("shader", ctypes.c_uint32),
                ("mesh", ctypes.c_uint32)]


class OrcSphereLight(ctypes.Structure):
    _fields_ = [("P", ctypes.c_float * 3), ("radius", ctypes.c_float), ("samples", ctypes.c_int),
                ("shader", ctypes.c_uint32), ("mesh", ctypes.c_uint32)]


class OrcCamera(ctypes.Structure):
    _fields_ = [("m", ctypes.c_float * 16), ("tan_theta_focal", ctypes.c_float), ("aspect", ctypes.c_float),
                ("focal", ctypes.c_float), ("radius", ctypes.c_float)]


_SH_FLAGS = {"emission_colour": 1, "emission_strength": 2, "diffuse_colour": 4, "diffuse_strength": 8,
             "diffuse_roughness": 16, "spec1_colour": 32, "spec1_strength": 64, "spec1_roughness": 128,
             "spec1_fresnel_refl": 256, "spec1_fresnel_edge": 512, "ior": 1024}
_SH_DEBUG = 2048  # DebugShader: {"debug": True, "diffuse_colour": Colour}


def _keys16(keys):
    a = np.ascontiguousarray(keys, np.float32).reshape(-1, 16)
    return a, a.shape[0]


def decompose(m):
    """TransformDecompMatrix4 of a column-major 4x4: (T[3], R[4] xyzw, S[16])."""
    out = np.zeros(23, np.float32)
    lib().orc_decompose(_ptr(np.ascontiguousarray(m, np.float32).reshape(16)), _ptr(out))
    return out[:3], out[3:7], out[7:]


def keyed_matrix(keys, time, blend_one=False):
    """The decomposed keys blended at time and rebuilt (column-major 16)."""
    a, n = _keys16(keys)
    out = np.zeros(16, np.float32)
    if lib().orc_keyed_matrix(_ptr(a), n, float(time), int(bool(blend_one)), _ptr(out)) != 0:
        raise ValueError("time outside the keys")
    return out


def set_normalize_mode(mode, seed=0):
    """Vec3Normalize of the reference-mode renderer: 0 exact, 1 the RSQRTSS
    emulation (process-wide)."""
    lib().orc_set_normalize_mode(int(mode), int(seed))


def _register_render(L):
    P = ctypes.c_void_p
    L.orc_mesh_set_shading.restype = ctypes.c_int
    L.orc_mesh_set_shading.argtypes = [P, P, P]
    L.orc_mesh_set_motion_normals.restype = ctypes.c_int
    L.orc_mesh_set_motion_normals.argtypes = [P, P, ctypes.c_uint32, ctypes.c_uint32]
    L.orc_render_create.restype = P
    L.orc_render_create.argtypes = [P, P, ctypes.c_uint32, P, P, P, P, ctypes.c_uint32, P, ctypes.c_uint32, P]
    L.orc_render_destroy.argtypes = [P]
    L.orc_render_add_disk_lights.restype = ctypes.c_int
    L.orc_render_add_disk_lights.argtypes = [P, P, ctypes.c_uint32]
    L.orc_render_add_sphere_lights.restype = ctypes.c_int
    L.orc_render_add_sphere_lights.argtypes = [P, P, ctypes.c_uint32]
    L.orc_sphere_create.restype = P
    L.orc_sphere_create.argtypes = [P, ctypes.c_float]
    L.orc_render_run.restype = ctypes.c_int
    L.orc_render_run.argtypes = [P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.c_uint64, P, ctypes.c_int]
    L.orc_scramble.restype = ctypes.c_uint64
    L.orc_scramble.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32]
    L.orc_pt_run.restype = ctypes.c_int
    L.orc_pt_run.argtypes = [P, P, ctypes.c_uint32, P, P, P, ctypes.c_int, ctypes.c_int]
    L.orc_pt_run_rows.restype = ctypes.c_int
    L.orc_pt_run_rows.argtypes = [P, P, ctypes.c_uint32, P, ctypes.c_uint32, ctypes.c_uint32, P, P, ctypes.c_int,
                                  ctypes.c_int]
    L.orc_render_run_rows.restype = ctypes.c_int
    L.orc_render_run_rows.argtypes = [P, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                      ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64, P, ctypes.c_int]
    L.orc_pt_rnd.restype = ctypes.c_float
    L.orc_pt_rnd.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32]
    L.orc_sincos_turns.argtypes = [P, ctypes.c_size_t, P, P]
    L.orc_mesh_set_transform.argtypes = [P, P]
    L.orc_guide_n_weights.restype = ctypes.c_int
    L.orc_guide_features.argtypes = [P, P, P, P, P, ctypes.c_int, P]
    L.orc_guide_forward.argtypes = [P, P, ctypes.c_int, ctypes.c_int, P]
    L.orc_guide_pdf.restype = ctypes.c_double
    L.orc_guide_pdf.argtypes = [P, P]
    L.orc_guide_out_grad.argtypes = [P, P, ctypes.c_double, ctypes.c_double, ctypes.c_double, P, P]
    L.orc_guide_loss_grad.restype = ctypes.c_double
    L.orc_guide_loss_grad.argtypes = [P, P, P, P, P, ctypes.c_double, ctypes.c_int, ctypes.c_int, P]
    L.orc_filter_warp.restype = ctypes.c_int
    L.orc_filter_warp.argtypes = [P, P, P, ctypes.c_size_t, P, P]
    L.orc_filter_tables.restype = ctypes.c_int
    L.orc_filter_tables.argtypes = [P, P, P]
    L.orc_render_set_filter.restype = ctypes.c_int
    L.orc_render_set_filter.argtypes = [P, P]
    L.orc_encode_rgbe.restype = ctypes.c_int
    L.orc_encode_rgbe.argtypes = [P, ctypes.c_uint32, ctypes.c_uint32, P]


class OrcPixelFilter(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("res", ctypes.c_int), ("width", ctypes.c_float), ("peak", ctypes.c_float)]


FILTER_DEFAULTS = {1: dict(res=17, width=2.0, peak=0.0), 2: dict(res=49, width=6.0, peak=4.0)}


def _pixel_filter(d):
    """A pixel-filter dict (kind 1 GaussianFilter, 2 AiryFilter; res, width,
    peak default to the nodes' defaults) as the C struct."""
    kind = int(d["kind"])
    dflt = FILTER_DEFAULTS.get(kind, dict(res=0, width=0.0, peak=0.0))
    return OrcPixelFilter(kind, int(d.get("res", dflt["res"])), float(d.get("width", dflt["width"])),
                          float(d.get("peak", dflt["peak"])))


def sincos_turns(u):
    """sin and cos of 2*pi*u (float32 u in [0, 1)) as the extended path
    tracer's sampling computes them: (sin, cos) float32 arrays."""
    u = np.ascontiguousarray(u, np.float32)
    s = np.empty_like(u)
    c = np.empty_like(u)
    lib().orc_sincos_turns(_ptr(u), u.size, _ptr(s), _ptr(c))
    return s, c


def filter_warp(f, r0, r1):
    """Sampler.WarpSample over arrays r0, r1 in [0, 1): returns (u, v)."""
    r0 = np.ascontiguousarray(r0, np.float64)
    r1 = np.ascontiguousarray(r1, np.float64)
    u = np.empty_like(r0)
    v = np.empty_like(r0)
    pf = _pixel_filter(f)
    if lib().orc_filter_warp(ctypes.byref(pf), _ptr(r0), _ptr(r1), r0.size, _ptr(u), _ptr(v)) != 0:
        raise ValueError("bad pixel filter")
    return u, v


def encode_rgbe(fb):
    """OutputHDR's pixel bytes of a float framebuffer [h, w, 3]: [h, w, 4]
    uint8 in file order (bottom row first)."""
    fb = np.ascontiguousarray(fb, np.float32)
    h, w = fb.shape[:2]
    out = np.empty((h, w, 4), np.uint8)
    lib().orc_encode_rgbe(_ptr(fb), w, h, _ptr(out))
    return out


def filter_tables(f):
    """CreateSampler's (cdfV [res], cdfVU [res, res])."""
    pf = _pixel_filter(f)
    a = np.empty(pf.res, np.float64)
    b = np.empty((pf.res, pf.res), np.float64)
    if lib().orc_filter_tables(ctypes.byref(pf), _ptr(a), _ptr(b)) != 0:
        raise ValueError("bad pixel filter")
    return a, b


class Guide:
    """The path-guiding network's oracle (orc_mlp.cpp)."""

    N_IN, N_OUT = 80, 41

    @staticmethod
    def n_weights():
        return lib().orc_guide_n_weights()

    @staticmethod
    def features(pos, nrm, wo, lo, hi):
        pos, nrm, wo = (np.ascontiguousarray(a, np.float32) for a in (pos, nrm, wo))
        lo, hi = np.ascontiguousarray(lo, np.float32), np.ascontiguousarray(hi, np.float32)
        n = pos.shape[0]
        f = np.zeros((n, 80), np.float64)
        lib().orc_guide_features(_ptr(pos), _ptr(nrm), _ptr(wo), _ptr(lo), _ptr(hi), n, _ptr(f))
        return f

    @staticmethod
    def forward(W, feat, precision=64):
        W = np.ascontiguousarray(W, np.float32)
        feat = np.ascontiguousarray(feat, np.float64)
        out = np.zeros((feat.shape[0], 41), np.float64)
        lib().orc_guide_forward(_ptr(W), _ptr(feat), feat.shape[0], int(precision), _ptr(out))
        return out

    @staticmethod
    def pdf(out41, w):
        """The vMF mixture's density at the unit direction w."""
        o = np.ascontiguousarray(out41, np.float64)
        w = np.ascontiguousarray(w, np.float64)
        return lib().orc_guide_pdf(_ptr(o), _ptr(w))

    @staticmethod
    def alpha(out41, amax):
        """The probability of sampling the guide: amax * sigmoid(s)."""
        return amax / (1.0 + np.exp(-np.asarray(out41, np.float64)[..., 40]))

    @staticmethod
    def out_grad(out41, w, weight, pb=-1.0, amax=0.5):
        """Loss and its gradient at the outputs; pb < 0: no BSDF density."""
        o = np.ascontiguousarray(out41, np.float64)
        w = np.ascontiguousarray(w, np.float64)
        g = np.zeros(41, np.float64)
        loss = ctypes.c_double()
        lib().orc_guide_out_grad(_ptr(o), _ptr(w), float(weight), float(pb), float(amax), _ptr(g), ctypes.byref(loss))
        return g, loss.value

    @staticmethod
    def loss_grad(W, feat, omega, weight, precision=64, bsdf_pdf=None, amax=0.5):
        W = np.ascontiguousarray(W, np.float32)
        feat = np.ascontiguousarray(feat, np.float64)
        omega = np.ascontiguousarray(omega, np.float32)
        weight = np.ascontiguousarray(weight, np.float32)
        pb = None if bsdf_pdf is None else np.ascontiguousarray(bsdf_pdf, np.float32)
        g = np.zeros(W.size, np.float64)
        loss = lib().orc_guide_loss_grad(_ptr(W), _ptr(feat), _ptr(omega), _ptr(weight),
                                         None if pb is None else _ptr(pb), float(amax), feat.shape[0],
                                         int(precision), _ptr(g))
        return loss, g


class OrcQuadLight(ctypes.Structure):
    _fields_ = [("p0", ctypes.c_float * 3), ("e1", ctypes.c_float * 3), ("e2", ctypes.c_float * 3),
                ("shader", ctypes.c_uint32), ("mesh", ctypes.c_uint32)]


class OrcPtParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("iter_begin", ctypes.c_uint32),
                ("iter_count", ctypes.c_uint32), ("seed", ctypes.c_uint64), ("max_depth", ctypes.c_uint32),
                ("rr_depth", ctypes.c_uint32), ("env", ctypes.c_float * 3)]


class Render:
    """The oracle's reference-mode renderer over a render scene
    (vermeer_gb300.scenes format)."""

    def __init__(self, scene):
        self.meshes = build_geoms(scene["meshes"])
        self.scene = scene_of(scene["meshes"], self.meshes)
        # an instance shades with the shaders of the geom it instances
        lists = [scene["meshes"][m["instance"]]["shaders"] if "instance" in m else m["shaders"]
                 for m in scene["meshes"]]
        counts = np.asarray([len(x) for x in lists], np.uint32)
        offs = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint32)
        lst = np.asarray([s for x in lists for s in x], np.uint32)
        shs = (OrcShader * len(scene["shaders"]))()
        for i, d in enumerate(scene["shaders"]):
            fl = 0
            for k, bit in _SH_FLAGS.items():
                if k in d:
                    fl |= bit
                    if isinstance(getattr(shs[i], k), float):
                        setattr(shs[i], k, float(d[k]))
                    else:
                        for c in range(3):
                            getattr(shs[i], k)[c] = float(d[k][c])
            shs[i].flags = fl | (_SH_DEBUG if d.get("debug") else 0)
            shs[i].spec1_fresnel = 1 if d.get("spec1_fresnel") == "Metal" else 0
        lts = (OrcTriLight * len(scene["lights"]))()
        for i, d in enumerate(scene["lights"]):
            for k in ("p0", "p1", "p2"):
                for c in range(3):
                    getattr(lts[i], k)[c] = float(d[k][c])
            lts[i].samples, lts[i].shader, lts[i].mesh = int(d.get("samples", 1)), int(d["shader"]), int(d["mesh"])
        cam = OrcCamera()
        for i in range(16):
            cam.m[i] = float(scene["camera"]["m"][i])
        c = scene["camera"]
        cam.tan_theta_focal, cam.aspect, cam.focal, cam.radius = (float(c[k]) for k in
                                                               ("tan_theta_focal", "aspect", "focal", "radius"))
        qs = scene.get("quad_lights", [])
        self._quads = (OrcQuadLight * len(qs))()
        for i, d in enumerate(qs):
            for k in ("p0", "e1", "e2"):
                for c in range(3):
                    getattr(self._quads[i], k)[c] = float(d[k][c])
            self._quads[i].shader, self._quads[i].mesh = int(d["shader"]), int(d["mesh"])
        self._env = tuple(float(x) for x in scene.get("env", (0.0, 0.0, 0.0)))
        arr = (ctypes.c_void_p * len(self.meshes))(*[m.h for m in self.meshes])
        self._keep = (counts, offs, lst, shs, lts, cam, arr)
        self.h = lib().orc_render_create(self.scene.h, arr, len(self.meshes), _ptr(offs), _ptr(counts), _ptr(lst),
                                         shs, len(scene["shaders"]), lts, len(scene["lights"]), ctypes.byref(cam))
        if scene["camera"].get("keys") is not None:
            self._cam_keys, nk = _keys16(scene["camera"]["keys"])
            lib().orc_render_set_camera_keys(self.h, _ptr(self._cam_keys), nk)
        dls = scene.get("disk_lights", [])
        if dls:
            darr = (OrcDiskLight * len(dls))()
            for i, d in enumerate(dls):
                for k in ("P", "up", "lookat"):
                    for c in range(3):
                        getattr(darr[i], k)[c] = float(d[k][c])
                darr[i].radius = float(d["radius"])
                darr[i].samples, darr[i].shader, darr[i].mesh = int(d.get("samples", 1)), int(d["shader"]), int(d["mesh"])
            lib().orc_render_add_disk_lights(self.h, darr, len(dls))
        sls = scene.get("sphere_lights", [])
        if sls:
            sarr = (OrcSphereLight * len(sls))()
            for i, d in enumerate(sls):
                for c in range(3):
                    sarr[i].P[c] = float(d["P"][c])
                sarr[i].radius = float(d["radius"])
                sarr[i].samples, sarr[i].shader, sarr[i].mesh = int(d.get("samples", 1)), int(d["shader"]), int(d["mesh"])
            lib().orc_render_add_sphere_lights(self.h, sarr, len(sls))
        if scene.get("pixel_filter"):
            self._filter = _pixel_filter(scene["pixel_filter"])
            if lib().orc_render_set_filter(self.h, ctypes.byref(self._filter)) != 0:
                raise ValueError("bad pixel filter")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_render_destroy(self.h)
            self.h = None

    def run_path(self, width, height, iter_begin, iter_count, seed, max_depth=4, rr_depth=3, precision=32, fb=None,
                 fb64=None, nthreads=0, rows=None):
        """The extended path tracer (orc_pt.cpp) over this scene plus its
        'quad_lights' and 'env'; rows = (row_begin, row_count): that band
        only.  Returns (fb float32, fb64 float64)."""
        r0, nr = rows if rows is not None else (0, 0)
        hb = nr if rows is not None else height
        if fb is None:
            fb = np.zeros((hb, width, 3), np.float32)
        if fb64 is None:
            fb64 = np.zeros((hb, width, 3), np.float64)
        fb = np.ascontiguousarray(fb, np.float32)
        fb64 = np.ascontiguousarray(fb64, np.float64)
        quads = self._quads
        p = OrcPtParams(width, height, iter_begin, iter_count, seed, max_depth, rr_depth,
                        (ctypes.c_float * 3)(*[float(x) for x in self._env]))
        rc = lib().orc_pt_run_rows(self.h, quads, len(quads), ctypes.byref(p), r0, nr, _ptr(fb), _ptr(fb64),
                                   int(precision), int(nthreads))
        if rc != 0:
            raise RuntimeError("orc_pt_run failed")
        return fb, fb64

    def run(self, width, height, iter_begin, iter_count, seed, fb=None, nthreads=0, rows=None):
        """Reference-mode render; rows = (row_begin, row_count) renders that
        band only (fb then holds row_count rows)."""
        r0, nr = rows if rows is not None else (0, 0)
        if fb is None:
            fb = np.zeros((nr if rows is not None else height, width, 3), np.float32)
        fb = np.ascontiguousarray(fb, np.float32)
        if lib().orc_render_run_rows(self.h, width, height, r0, nr, iter_begin, iter_count, seed, _ptr(fb),
                                     int(nthreads)) != 0:
            raise ValueError("row band outside the image")
        return fb


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def build_geoms(entries):
    """Oracle geoms for a scene's mesh list (vermeer_gb300.scenes format):
    meshes (optionally 'transform' or 'transform_keys'), spheres, instances
    ({'instance': i, 'keys', 'bmin', 'bmax'}) and Procs ({'proc': [child
    indices], 'keys' (optional), 'bmin', 'bmax'}); entry i reports id i."""
    geoms = [None] * len(entries)
    for i, m in enumerate(entries):
        if "sphere" in m:
            geoms[i] = Sphere(m["sphere"][:3], m["sphere"][3])
        elif "verts" in m:
            om = Mesh(m["verts"], m["idxp"], keys=m.get("keys", 1), motion_fixed=m.get("motion_mode", 0) == 1)
            fs = None if m.get("face_shader") is None else np.ascontiguousarray(m["face_shader"], np.uint8)
            nr = None if m.get("normals") is None else np.ascontiguousarray(m["normals"], np.float32)
            lib().orc_mesh_set_shading(om.h, _ptr(fs), _ptr(nr))
            if m.get("motion_normals") is not None:
                om.set_motion_normals(m["motion_normals"])
            if m.get("transform_keys") is not None:
                om.set_transform_keys(m["transform_keys"])
            elif m.get("transform") is not None:
                om.set_transform(m["transform"])
            geoms[i] = om
    for i, m in enumerate(entries):
        if "instance" in m:
            geoms[i] = Instance(geoms[m["instance"]], m["keys"], m["bmin"], m["bmax"])
        elif "proc" in m:
            geoms[i] = Proc([geoms[c] for c in m["proc"]], m["proc"], m.get("keys"), m["bmin"], m["bmax"])
    return geoms


def scene_of(entries, geoms):
    """The scene's top level: every geom but a Proc's children, each
    reporting its index in the list."""
    children = {c for m in entries if "proc" in m for c in m["proc"]}
    top = [i for i in range(len(entries)) if i not in children]
    return Scene([geoms[i] for i in top], ids=top)


class Instance:
    """GeomInstance (builtin/geom/instance/instance.go) of an oracle geom."""

    def __init__(self, of, keys, bmin, bmax):
        self.of = of
        self._k, n = _keys16(keys)
        self._b = (np.asarray(bmin, np.float32), np.asarray(bmax, np.float32))
        self.h = lib().orc_instance_create(of.h, _ptr(self._k), n, _ptr(self._b[0]), _ptr(self._b[1]))
        if not self.h:
            raise ValueError(lib().orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mesh_destroy(self.h)
            self.h = None


class Proc:
    """Proc (builtin/geom/proc/proc.go) over oracle geoms; a hit in child k
    reports ids[k]."""

    def __init__(self, children, ids, keys, bmin, bmax):
        self.children = list(children)
        arr = (ctypes.c_void_p * len(children))(*[c.h for c in children])
        self._ids = np.ascontiguousarray(ids, np.int32)
        self._k, n = (None, 0) if keys is None else _keys16(keys)
        self._b = (np.asarray(bmin, np.float32), np.asarray(bmax, np.float32))
        self._arr = arr
        self.h = lib().orc_proc_create(arr, _ptr(self._ids), len(children), _ptr(self._k), n, _ptr(self._b[0]),
                                       _ptr(self._b[1]))
        if not self.h:
            raise ValueError(lib().orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mesh_destroy(self.h)
            self.h = None


class Mesh:
    """A PolyMesh with its accelerator built by the oracle."""

    def __init__(self, verts, idxp, keys=1, ray_bias=0.0, motion_fixed=False):
        verts = np.ascontiguousarray(verts, dtype=np.float32)
        idxp = np.ascontiguousarray(idxp, dtype=np.uint32)
        assert verts.size % (3 * keys) == 0 and idxp.size % 3 == 0
        self.nverts = verts.size // (3 * keys)
        self.keys = keys
        self.ntris = idxp.size // 3
        self.verts, self.idxp_in = verts, idxp
        self.h = lib().orc_mesh_create(_ptr(verts), self.nverts, keys, _ptr(idxp), self.ntris,
                                       float(ray_bias), int(bool(motion_fixed)))
        if not self.h:
            raise ValueError(lib().orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mesh_destroy(self.h)
            self.h = None

    def set_transform_keys(self, keys):
        """PolyMesh.Transform of n keys ([n, 16] column-major)."""
        self._xk, n = _keys16(keys)
        lib().orc_mesh_set_transform_keys(self.h, _ptr(self._xk), n)

    def set_motion_normals(self, normals):
        """PolyMesh.Normals of a motion mesh with as many keys as its
        vertices: [keys, n, 3], n >= 3 x triangles; a hit on element e reads
        rows 3e .. 3e + 2 of each key (trace.go:694-712).  None clears them."""
        if normals is None:
            lib().orc_mesh_set_motion_normals(self.h, None, 0, 0)
            return
        a = np.ascontiguousarray(normals, np.float32)
        assert a.ndim == 3 and a.shape[2] == 3
        if lib().orc_mesh_set_motion_normals(self.h, _ptr(a), a.shape[1], a.shape[0]) != 0:
            raise ValueError("motion normals need the mesh's key count and at least 3 rows per triangle")

    def set_transform(self, m):
        """PolyMesh.Transform: a column-major 4x4 (16 floats) or None."""
        if m is None:
            lib().orc_mesh_set_transform(self.h, None)
        else:
            self._xf = np.ascontiguousarray(m, np.float32).reshape(16)
            lib().orc_mesh_set_transform(self.h, _ptr(self._xf))

    def info(self):
        n = ctypes.c_uint32()
        nm = ctypes.c_uint32()
        b = np.zeros(6, np.float32)
        lib().orc_mesh_info(self.h, ctypes.byref(n), ctypes.byref(nm), _ptr(b))
        return n.value, nm.value, b

    def export(self):
        n, nm, b = self.info()
        nodes = np.zeros(n, ORC_NODE_DTYPE)
        accel_idx = np.zeros(self.ntris, np.int32)
        idxp = np.zeros(self.ntris * 3, np.uint32)
        mnodes = np.zeros(nm, ORC_MNODE_DTYPE)
        mboxes = np.zeros((self.keys if nm else 0, nm, 24), np.float32)
        lib().orc_mesh_export(self.h, _ptr(nodes), _ptr(accel_idx), _ptr(idxp), _ptr(mnodes),
                              _ptr(mboxes))
        return dict(nodes=nodes, accel_idx=accel_idx, idxp=idxp, mnodes=mnodes, mboxes=mboxes,
                    bounds=b)

    def trace(self, rays, shadow=False, nthreads=0, counters=False):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        u = np.empty(n, np.float32)
        v = np.empty(n, np.float32)
        w = np.empty(n, np.float32)
        cnt = np.empty((n, 3), np.uint32) if counters else None
        st = lib().orc_trace_mesh(self.h, _ptr(rays), n, int(bool(shadow)), int(nthreads),
                                  _ptr(prim), _ptr(t), _ptr(u), _ptr(v), _ptr(w), _ptr(cnt))
        out = dict(prim=prim, t=t, u=u, v=v, w=w, status=st)
        if counters:
            out["counters"] = cnt
        return out


class Sphere:
    """An analytic sphere geom (builtin/geom/sphere), usable as a scene
    member like Mesh."""

    def __init__(self, center, radius):
        c = np.ascontiguousarray(center, np.float32)
        self.h = lib().orc_sphere_create(_ptr(c), float(radius))
        self._keep = c

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mesh_destroy(self.h)
            self.h = None


class Scene:
    """The two-level scene of builtin/scene over oracle meshes (hits report
    ids[i] for meshes[i], default i)."""

    def __init__(self, meshes, ids=None):
        self.meshes = list(meshes)
        arr = (ctypes.c_void_p * len(self.meshes))(*[m.h for m in self.meshes])
        self._ids = None if ids is None else np.ascontiguousarray(ids, np.int32)
        self.h = lib().orc_scene_create_ids(arr, _ptr(self._ids), len(self.meshes))
        if not self.h:
            raise ValueError(lib().orc_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_scene_destroy(self.h)
            self.h = None

    def export(self):
        n = ctypes.c_uint32()
        nm = ctypes.c_uint32()
        keys = ctypes.c_uint32()
        lib().orc_scene_info(self.h, ctypes.byref(n), ctypes.byref(nm), ctypes.byref(keys))
        nodes = np.zeros(n.value, ORC_NODE_DTYPE)
        order = np.zeros(len(self.meshes), np.int32)
        mnodes = np.zeros(nm.value, ORC_MNODE_DTYPE)
        mboxes = np.zeros((keys.value if nm.value else 0, nm.value, 24), np.float32)
        lib().orc_scene_export(self.h, _ptr(nodes), _ptr(order), _ptr(mnodes), _ptr(mboxes))
        return dict(nodes=nodes, geom_order=order, mnodes=mnodes, mboxes=mboxes, keys=keys.value)

    def trace(self, rays, shadow=False, nthreads=0, counters=False):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        n = rays.shape[0]
        prim = np.empty(n, np.int32)
        geom = np.empty(n, np.int32)
        t = np.empty(n, np.float32)
        u = np.empty(n, np.float32)
        v = np.empty(n, np.float32)
        w = np.empty(n, np.float32)
        cnt = np.empty((n, 3), np.uint32) if counters else None
        st = lib().orc_trace_scene(self.h, _ptr(rays), n, int(bool(shadow)), int(nthreads),
                                   _ptr(prim), _ptr(geom), _ptr(t), _ptr(u), _ptr(v), _ptr(w),
                                   _ptr(cnt))
        out = dict(prim=prim, geom=geom, t=t, u=u, v=v, w=w, status=st)
        if counters:
            out["counters"] = cnt
        return out


def vdc(i, scramble=0):
    return lib().orc_vdc(i, scramble)


def sobol(i, scramble=0):
    return lib().orc_sobol(i, scramble)


def raster_xy(m, frame, px, py, sx=0, sy=0):
    rx = ctypes.c_double()
    ry = ctypes.c_double()
    idx = lib().orc_raster_xy(m, frame, px, py, sx, sy, ctypes.byref(rx), ctypes.byref(ry))
    return idx, rx.value, ry.value


def vdc_sobol_tables(m):
    f = np.zeros(52, np.uint64)
    v = np.zeros(52, np.uint64)
    lib().orc_vdc_sobol_tables(m, _ptr(f), _ptr(v))
    return f, v
