"""Host-side interface over libvmr's C ABI.

Mirrors the reference's traversal boundary: a PolyMesh is built
(PolyMesh.PreRender -> initAccel, builtin/geom/polymesh/buildqbvh.go:14-144)
or uploaded with a reference-built QBVH, a Scene gets its top level
(Scene.PreRender -> initAccel, builtin/scene/scene.go:131-203), and rays are
traced closest-hit or as shadow rays (qbvh.Trace, qbvh/intersect.go:91;
Scene.Trace, scene.go:30).  Errors raise VmrError carrying the vmr_status.

Ray batches are float32 arrays of shape [n, 8] (px py pz dx dy dz tmax time)
in host memory, or CUDA tensors of shape [8, n] (one row per field, already
in HBM) for the device path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib

STATUS = {0: "VMR_OK", -1: "VMR_ERR_INVALID", -2: "VMR_ERR_CUDA", -3: "VMR_ERR_OOM", -4: "VMR_ERR_TIMEOUT",
          -5: "VMR_ERR_STACK_OVERFLOW", -6: "VMR_ERR_QUEUE_OVERFLOW", -7: "VMR_ERR_UNSUPPORTED"}
TRACE_ANY_HIT, TRACE_DEVICE, TRACE_COUNT = 1, 2, 4
MOTION_FAITHFUL, MOTION_FIXED = 0, 1
BUILD_AUTO, BUILD_HOST, BUILD_DEVICE = 0, 1, 2

NODE_DTYPE = np.dtype([("boxes", "<f4", (24,)), ("axis", "<u4", (3,)), ("children", "<i4", (4,)),
                       ("parent", "<i4")])
MNODE_DTYPE = np.dtype([("axis", "<i4", (3,)), ("children", "<i4", (4,)), ("parent", "<i4"),
                        ("pad", "<u4", (2,))])


class VmrError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


FILTER_BOX, FILTER_GAUSSIAN, FILTER_AIRY = _lib.FILTER_BOX, _lib.FILTER_GAUSSIAN, _lib.FILTER_AIRY


def pixel_filter_warp(kind: int, r0, r1, res: int = 0, width: float = 0.0, peak: float = 0.0):
    """The pixel filter's Sampler.WarpSample on the host (no GPU): offsets
    (u, v) from the pixel centre for sample positions (r0, r1) in [0, 1)."""
    L = _lib.load()
    r0 = np.ascontiguousarray(r0, np.float64)
    r1 = np.ascontiguousarray(r1, np.float64)
    u = np.empty_like(r0)
    v = np.empty_like(r0)
    f = _lib.PixelFilter(int(kind), int(res), float(width), float(peak))
    rc = L.vmr_pixel_filter_warp(ctypes.byref(f), _p(r0), _p(r1), r0.size, _p(u), _p(v))
    if rc != 0:
        raise VmrError(rc, "bad pixel filter")
    return u, v


def transform_keys_at(keys, time: float, blend_one: bool = False):
    """libvmr's matrix for decomposed transform keys ([n, 16] column-major)
    at a time, on the host (no GPU): TransformDecompMatrix4 per key,
    TransformDecompLerp of the keys around time, TransformDecompToMatrix4."""
    L = _lib.load()
    k = np.ascontiguousarray(keys, np.float32).reshape(-1, 16)
    out = np.zeros(16, np.float32)
    rc = L.vmr_transform_keys_at(_p(k), k.shape[0], float(time), int(bool(blend_one)), _p(out))
    if rc != 0:
        raise VmrError(rc, "time outside the keys")
    return out


def split_rows(height: int, n: int):
    """The row bands libvmr's split renders use (vmr_split_rows): a list of
    (row_begin, row_count), one per device."""
    L = _lib.load()
    b = np.zeros(n, np.uint32)
    c = np.zeros(n, np.uint32)
    rc = L.vmr_split_rows(height, n, _p(b), _p(c))
    if rc != 0:
        raise VmrError(rc, "bad split")
    return [(int(x), int(y)) for x, y in zip(b, c)]


def render_split(ctxs, width: int, height: int, iter_begin: int, iter_count: int, seed: int, fb=None,
                 max_batch_samples: int = 0):
    """vmr_render_split: one reference-mode image over several contexts (one
    per GPU, each holding the same scene); returns (fb, stats)."""
    L = _lib.load()
    if fb is None:
        fb = np.zeros((height, width, 3), np.float32)
    fb = np.ascontiguousarray(fb, np.float32)
    arr = (ctypes.c_void_p * len(ctxs))(*[c.h for c in ctxs])
    p = _lib.RenderParams(width, height, iter_begin, iter_count, seed, max_batch_samples, 0, 0)
    st = _lib.RenderStats()
    rc = L.vmr_render_split(arr, len(ctxs), ctypes.byref(p), _p(fb), ctypes.byref(st))
    if rc != 0:
        raise VmrError(rc, " / ".join(L.vmr_last_error(c.h).decode() for c in ctxs))
    return fb, dict(samples=st.samples, camera_rays=st.camera_rays, shadow_rays=st.shadow_rays, ms=st.ms)


def render_path_split(ctxs, width: int, height: int, iter_begin: int, iter_count: int, seed: int, fb=None,
                      fb64=None, **kw):
    """vmr_render_path_split: one path-traced image over several contexts;
    keyword arguments as Context.render_path (train excluded)."""
    L = _lib.load()
    if fb is None:
        fb = np.zeros((height, width, 3), np.float32)
    fb = np.ascontiguousarray(fb, np.float32)
    p = Context._path_params(width, height, iter_begin, iter_count, seed, fb64=fb64, **kw)
    arr = (ctypes.c_void_p * len(ctxs))(*[c.h for c in ctxs])
    st = _lib.PathStats()
    rc = L.vmr_render_path_split(arr, len(ctxs), ctypes.byref(p), _p(fb), ctypes.byref(st))
    if rc != 0:
        raise VmrError(rc, " / ".join(L.vmr_last_error(c.h).decode() for c in ctxs))
    return fb, dict(samples=st.samples, rays=st.rays, shadow_rays=st.shadow_rays, ms=st.ms)


def write_float(path: str, fb):
    """The OutputFloat driver (builtin/driver/outputfloat.go): the float32
    framebuffer [h, w, 3] as raw little-endian floats."""
    np.ascontiguousarray(fb, "<f4").tofile(path)


def _p(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)
    return ctypes.c_void_p(a.data_ptr())  # torch tensor


class Context:
    """One libvmr context on one GPU (vmr_create)."""

    def __init__(self, device: int = 0):
        self.L = _lib.load()
        h = ctypes.c_void_p()
        rc = self.L.vmr_create(int(device), ctypes.byref(h))
        if rc != 0:
            raise VmrError(rc, "vmr_create failed (no usable CUDA device?)")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.L.vmr_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc: int):
        if rc != 0:
            raise VmrError(rc, self.L.vmr_last_error(self.h).decode(errors="replace"))

    def set_stream(self, stream_handle: int | None):
        self._check(self.L.vmr_set_stream(self.h, ctypes.c_void_p(stream_handle) if stream_handle else None))

    def sync(self):
        self._check(self.L.vmr_sync(self.h))

    def set_tuning(self, kernel: int = 45, block: int = 0, blocks_per_sm: int = 0, refill_min: int = 0,
                   walk_tail: int = 8, sort_bits: int = 0):
        """Launch parameters of the traversal kernels (vmr_set_tuning)."""
        t = _lib.Tuning(kernel, block, blocks_per_sm, refill_min, walk_tail, sort_bits)
        self._check(self.L.vmr_set_tuning(self.h, ctypes.byref(t)))

    def autotune(self, geom: int, rays, shadow: bool = False):
        """vmr_autotune on a sample (numpy [n, 8] or CUDA tensor [8, n]);
        returns (tuning dict, best_ms, candidates tried)."""
        flags = TRACE_ANY_HIT if shadow else 0
        if isinstance(rays, np.ndarray):
            soa = np.ascontiguousarray(np.ascontiguousarray(rays, np.float32).reshape(-1, 8).T)
            n = soa.shape[1]
            r = _lib.Rays(*[_p(soa[k]) for k in range(8)])
        else:
            n = rays.shape[1]
            r = _lib.Rays(*[ctypes.c_void_p(rays[k].data_ptr()) for k in range(8)])
            flags |= TRACE_DEVICE
        t = _lib.Tuning()
        ms = ctypes.c_float()
        nt = ctypes.c_uint32()
        self._check(self.L.vmr_autotune(self.h, geom, ctypes.byref(r), n, flags, ctypes.byref(t), ctypes.byref(ms),
                                        ctypes.byref(nt)))
        return (dict(kernel=t.kernel, block=t.block, blocks_per_sm=t.blocks_per_sm, refill_min=t.refill_min,
                     walk_tail=t.walk_tail, sort_bits=t.sort_bits), ms.value, nt.value)

    def clear_tuning(self, geom: int):
        self._check(self.L.vmr_clear_tuning(self.h, geom))

    def trace_jobs(self, jobs, shadow: bool = False, outputs=("prim", "t", "u", "v", "w")):
        """vmr_trace_jobs: jobs = [(geom, CUDA tensor [8, n]), ...], all in one
        launch.  Returns (list of hit dicts, stats)."""
        import torch
        arr = (_lib.TraceJob * len(jobs))()
        outs = []
        for i, (geom, rays) in enumerate(jobs):
            assert rays.is_cuda and rays.dtype == torch.float32 and rays.shape[0] == 8 and rays.is_contiguous()
            n = rays.shape[1]
            out = {k: torch.empty(n, dtype=torch.int32 if k in ("prim", "geom") else torch.float32,
                                  device=rays.device) for k in outputs}
            arr[i].geom = geom
            arr[i].n = n
            arr[i].rays = _lib.Rays(*[ctypes.c_void_p(rays[k].data_ptr()) for k in range(8)])
            arr[i].hits = _lib.Hits(*[_p(out.get(k)) for k in ("prim", "geom", "t", "u", "v", "w")])
            outs.append(out)
        st = _lib.TraceStats()
        flags = TRACE_DEVICE | (TRACE_ANY_HIT if shadow else 0)
        self._check(self.L.vmr_trace_jobs(self.h, arr, len(jobs), flags, ctypes.byref(st)))
        return outs, dict(rays=st.rays, kernel_ms=st.kernel_ms)

    def trace_timing(self):
        """(sort_ms, traverse_ms) of the last trace call (vmr_trace_timing)."""
        a, b = ctypes.c_float(), ctypes.c_float()
        self._check(self.L.vmr_trace_timing(self.h, ctypes.byref(a), ctypes.byref(b)))
        return a.value, b.value

    def get_tuning(self):
        t = _lib.Tuning()
        self._check(self.L.vmr_get_tuning(self.h, ctypes.byref(t)))
        return dict(kernel=t.kernel, block=t.block, blocks_per_sm=t.blocks_per_sm, refill_min=t.refill_min,
                    walk_tail=t.walk_tail, sort_bits=t.sort_bits)

    # ------------------------------------------------------------ meshes
    def set_builder(self, builder: int):
        """BUILD_AUTO (device for meshes of >= 16384 triangles), BUILD_HOST or
        BUILD_DEVICE: the QBVH builder of mesh_build (same result either way)."""
        self._check(self.L.vmr_set_builder(self.h, builder))

    def mesh_build(self, verts, idxp, keys: int = 1, ray_bias: float = 0.0, motion_mode: int = MOTION_FAITHFUL,
                   shader_idx=None) -> int:
        verts = np.ascontiguousarray(verts, np.float32)
        idxp = np.ascontiguousarray(idxp, np.uint32)
        sidx = None if shader_idx is None else np.ascontiguousarray(shader_idx, np.uint8)
        mi = _lib.MeshInput(_p(verts), verts.size // (3 * keys), keys, _p(idxp), idxp.size // 3,
                            float(ray_bias), int(motion_mode), _p(sidx))
        g = ctypes.c_uint32()
        self._check(self.L.vmr_mesh_build(self.h, ctypes.byref(mi), ctypes.byref(g)))
        return g.value

    def mesh_upload(self, verts, idxp, accel_idx, nodes=None, mnodes=None, mboxes=None, bounds=None, keys: int = 1,
                    ray_bias: float = 0.0, motion_mode: int = MOTION_FAITHFUL) -> int:
        verts = np.ascontiguousarray(verts, np.float32)
        idxp = np.ascontiguousarray(idxp, np.uint32)
        accel_idx = np.ascontiguousarray(accel_idx, np.int32)
        nodes = None if nodes is None else np.ascontiguousarray(nodes, NODE_DTYPE)
        mnodes = None if mnodes is None else np.ascontiguousarray(mnodes, MNODE_DTYPE)
        mboxes = None if mboxes is None else np.ascontiguousarray(mboxes, np.float32)
        bounds = None if bounds is None else np.ascontiguousarray(bounds, np.float32)
        d = _lib.MeshDesc(_p(verts), verts.size // (3 * keys), keys, _p(idxp), idxp.size // 3, _p(accel_idx),
                          float(ray_bias), int(motion_mode), _p(nodes), 0 if nodes is None else len(nodes),
                          _p(mnodes), 0 if mnodes is None else len(mnodes), _p(mboxes), _p(bounds), None)
        g = ctypes.c_uint32()
        self._check(self.L.vmr_mesh_upload(self.h, ctypes.byref(d), ctypes.byref(g)))
        return g.value

    def mesh_info(self, geom: int):
        a, b, c, d = (ctypes.c_uint32() for _ in range(4))
        self._check(self.L.vmr_mesh_info(self.h, geom, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                         ctypes.byref(d)))
        return dict(n_nodes=a.value, n_mnodes=b.value, n_tris=c.value, keys=d.value)

    def mesh_export(self, geom: int):
        i = self.mesh_info(geom)
        nodes = np.zeros(i["n_nodes"], NODE_DTYPE)
        mnodes = np.zeros(i["n_mnodes"], MNODE_DTYPE)
        mboxes = np.zeros((i["keys"] if i["n_mnodes"] else 0, i["n_mnodes"], 24), np.float32)
        accel_idx = np.zeros(i["n_tris"], np.int32)
        idxp = np.zeros(i["n_tris"] * 3, np.uint32)
        bounds = np.zeros(6 * i["keys"], np.float32)
        self._check(self.L.vmr_mesh_export(self.h, geom, _p(nodes), _p(accel_idx), _p(idxp), _p(mnodes),
                                           _p(mboxes), _p(bounds)))
        return dict(nodes=nodes, accel_idx=accel_idx, idxp=idxp, mnodes=mnodes, mboxes=mboxes, bounds=bounds)

    # ------------------------------------------------------------- scene
    def scene_build(self, geoms):
        g = np.ascontiguousarray(geoms, np.uint32)
        self._check(self.L.vmr_scene_build(self.h, _p(g), g.size))

    def scene_upload(self, geom_order, nodes=None, mnodes=None, mboxes=None, keys: int = 1):
        order = np.ascontiguousarray(geom_order, np.uint32)
        nodes = None if nodes is None else np.ascontiguousarray(nodes, NODE_DTYPE)
        mnodes = None if mnodes is None else np.ascontiguousarray(mnodes, MNODE_DTYPE)
        mboxes = None if mboxes is None else np.ascontiguousarray(mboxes, np.float32)
        self._check(self.L.vmr_scene_upload(self.h, _p(nodes), 0 if nodes is None else len(nodes), _p(mnodes),
                                            0 if mnodes is None else len(mnodes), _p(mboxes), keys, _p(order),
                                            order.size))

    def scene_export(self, n_geoms: int):
        nn, nm, k = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        self._check(self.L.vmr_scene_export(self.h, None, None, None, None, ctypes.byref(nn), ctypes.byref(nm),
                                            ctypes.byref(k)))
        order = np.zeros(n_geoms, np.uint32)
        nodes = np.zeros(nn.value, NODE_DTYPE)
        mnodes = np.zeros(nm.value, MNODE_DTYPE)
        mboxes = np.zeros((k.value if nm.value else 0, nm.value, 24), np.float32)
        self._check(self.L.vmr_scene_export(self.h, _p(order), _p(nodes), _p(mnodes), _p(mboxes), None, None, None))
        return dict(geom_order=order, nodes=nodes, mnodes=mnodes, mboxes=mboxes, keys=k.value)

    # ------------------------------------------------------------- trace
    def _trace(self, geom, rays, shadow, counters, outputs):
        flags = (TRACE_ANY_HIT if shadow else 0) | (TRACE_COUNT if counters else 0)
        st = _lib.TraceStats()
        if isinstance(rays, np.ndarray):
            rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
            n = rays.shape[0]
            soa = np.ascontiguousarray(rays.T)
            r = _lib.Rays(*[_p(soa[k]) for k in range(8)])
            out = {k: np.empty(n, np.int32 if k in ("prim", "geom") else np.float32) for k in outputs}
            h = _lib.Hits(*[_p(out.get(k)) for k in ("prim", "geom", "t", "u", "v", "w")])
        else:  # CUDA tensor [8, n], rows already in HBM
            import torch
            assert rays.is_cuda and rays.dtype == torch.float32 and rays.shape[0] == 8 and rays.is_contiguous()
            n = rays.shape[1]
            r = _lib.Rays(*[ctypes.c_void_p(rays[k].data_ptr()) for k in range(8)])
            out = {k: torch.empty(n, dtype=torch.int32 if k in ("prim", "geom") else torch.float32,
                                  device=rays.device) for k in outputs}
            h = _lib.Hits(*[_p(out.get(k)) for k in ("prim", "geom", "t", "u", "v", "w")])
            flags |= TRACE_DEVICE
        if geom is None:
            rc = self.L.vmr_trace_scene(self.h, ctypes.byref(r), n, flags, ctypes.byref(h), ctypes.byref(st))
        else:
            rc = self.L.vmr_trace_mesh(self.h, geom, ctypes.byref(r), n, flags, ctypes.byref(h), ctypes.byref(st))
        self._check(rc)
        out["stats"] = dict(rays=st.rays, node_visits=st.node_visits, leaf_visits=st.leaf_visits,
                            tri_tests=st.tri_tests, kernel_ms=st.kernel_ms)
        return out

    def trace_mesh(self, geom: int, rays, shadow: bool = False, counters: bool = False,
                   outputs=("prim", "t", "u", "v", "w")):
        """PolyMesh.Trace over one mesh: closest hit, or any hit for shadow rays."""
        return self._trace(geom, rays, shadow, counters, outputs)

    def trace_scene(self, rays, shadow: bool = False, counters: bool = False,
                    outputs=("prim", "geom", "t", "u", "v", "w")):
        """Scene.Trace over the two-level scene."""
        return self._trace(None, rays, shadow, counters, outputs)

    # ------------------------------------------------------------ render
    def set_shaders(self, shaders):
        """Material table: ShaderStd parameter dicts (see _lib.SHADER_FLAGS)."""
        arr = (_lib.ShaderStd * len(shaders))(*[_lib.shader_struct(d) for d in shaders])
        self._check(self.L.vmr_set_shaders(self.h, arr, len(shaders)))

    def mesh_set_shading(self, geom: int, shader_ids, normals=None):
        ids = np.ascontiguousarray(shader_ids, np.uint32)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32)
        self._check(self.L.vmr_mesh_set_shading(self.h, geom, _p(ids), ids.size, _p(nrm)))

    def mesh_set_motion_normals(self, geom: int, normals):
        """vmr_mesh_set_motion_normals: [keys, n, 3] corner normals of a motion
        mesh (n >= 3 x triangles; a hit on element e reads rows 3e .. 3e + 2
        of each key), or None to remove them."""
        if normals is None:
            self._check(self.L.vmr_mesh_set_motion_normals(self.h, geom, None, 0, 0))
            return
        a = np.ascontiguousarray(normals, np.float32)
        assert a.ndim == 3 and a.shape[2] == 3
        self._check(self.L.vmr_mesh_set_motion_normals(self.h, geom, _p(a), a.shape[1], a.shape[0]))

    def set_lights(self, lights):
        """TriLights: dicts with p0, p1, p2, samples, shader, geom."""
        arr = (_lib.TriLight * len(lights))()
        for i, d in enumerate(lights):
            for k in ("p0", "p1", "p2"):
                for c in range(3):
                    getattr(arr[i], k)[c] = float(d[k][c])
            arr[i].samples, arr[i].shader, arr[i].geom = int(d.get("samples", 1)), int(d["shader"]), int(d["geom"])
        self._check(self.L.vmr_set_lights(self.h, arr, len(lights)))

    def sphere_add(self, center, radius: float) -> int:
        """An analytic sphere geom (vmr_sphere_add); returns its geom id."""
        c = (ctypes.c_float * 3)(*[float(x) for x in center])
        g = ctypes.c_uint32()
        self._check(self.L.vmr_sphere_add(self.h, c, float(radius), ctypes.byref(g)))
        return g.value

    def set_sphere_lights(self, lights):
        """SphereLights: dicts with P, radius, samples, shader, geom."""
        arr = (_lib.SphereLight * len(lights))()
        for i, d in enumerate(lights):
            for c in range(3):
                arr[i].P[c] = float(d["P"][c])
            arr[i].radius = float(d["radius"])
            arr[i].samples, arr[i].shader, arr[i].geom = int(d.get("samples", 1)), int(d["shader"]), int(d["geom"])
        self._check(self.L.vmr_set_sphere_lights(self.h, arr, len(lights)))

    def set_disk_lights(self, lights):
        """DiskLights: dicts with P, up, lookat, radius, samples, shader, geom."""
        arr = (_lib.DiskLight * len(lights))()
        for i, d in enumerate(lights):
            for k in ("P", "up", "lookat"):
                for c in range(3):
                    getattr(arr[i], k)[c] = float(d[k][c])
            arr[i].radius = float(d["radius"])
            arr[i].samples, arr[i].shader, arr[i].geom = int(d.get("samples", 1)), int(d["shader"]), int(d["geom"])
        self._check(self.L.vmr_set_disk_lights(self.h, arr, len(lights)))

    def set_quad_lights(self, lights):
        """Quad lights: dicts with p0, e1, e2, shader, geom."""
        arr = (_lib.QuadLight * len(lights))()
        for i, d in enumerate(lights):
            for k in ("p0", "e1", "e2"):
                for c in range(3):
                    getattr(arr[i], k)[c] = float(d[k][c])
            arr[i].shader, arr[i].geom = int(d["shader"]), int(d["geom"])
        self._check(self.L.vmr_set_quad_lights(self.h, arr, len(lights)))

    def set_env_light(self, radiance):
        r = (ctypes.c_float * 3)(*[float(x) for x in radiance])
        self._check(self.L.vmr_set_env_light(self.h, r))

    def render_path(self, width: int, height: int, iter_begin: int, iter_count: int, seed: int, max_depth: int = 4,
                    rr_depth: int = 3, fb=None, fb64=None, max_batch_samples: int = 0, graph: bool = True,
                    guided: bool = False, train: bool = False, guide_fraction: float = 0.0, train_steps: int = 0,
                    train_batch: int = 0, train_lr: float = 0.0, sort_queues: bool = False, guide_depth: int = 0,
                    rows=None, fixed_selection: bool = False, two_level: bool = False):
        """The extended path tracer: iterations [iter_begin, iter_begin +
        iter_count) folded into fb (float32 [height, width, 3]) and, when
        given, fb64 (float64).  guided: sample the guide network too; train:
        train it online; guide_depth: guide only the first vertices of each
        path (0: all); guide_fraction: alpha_max of the learned selection
        (0: 0.9), or with fixed_selection the guide's probability at every
        vertex (0: 0.5); sort_queues: trace each queue in ray-key order;
        two_level: trace the two-level scene even when it can be flattened;
        rows: (row_begin, row_count), a band of the image (fb then holds
        row_count rows).  Returns (fb, stats)."""
        r0, nr = rows if rows is not None else (0, 0)
        hb = nr if rows is not None else height
        if fb is None:
            fb = np.zeros((hb, width, 3), np.float32)
        fb = np.ascontiguousarray(fb, np.float32)
        if fb64 is not None:
            assert fb64.dtype == np.float64 and fb64.flags.c_contiguous and fb64.shape == (hb, width, 3)
        p = self._path_params(width, height, iter_begin, iter_count, seed, max_depth, rr_depth, fb64,
                              max_batch_samples, graph, guided, train, guide_fraction, train_steps, train_batch,
                              train_lr, sort_queues, guide_depth, r0, nr, fixed_selection, two_level)
        st = _lib.PathStats()
        self._check(self.L.vmr_render_path(self.h, ctypes.byref(p), _p(fb), ctypes.byref(st)))
        return fb, dict(samples=st.samples, rays=st.rays, shadow_rays=st.shadow_rays,
                        graph_replays=st.graph_replays, ms=st.ms, train_records=st.train_records,
                        train_steps=st.train_steps, train_loss=st.train_loss)

    @staticmethod
    def _path_params(width, height, iter_begin, iter_count, seed, max_depth=4, rr_depth=3, fb64=None,
                     max_batch_samples=0, graph=True, guided=False, train=False, guide_fraction=0.0, train_steps=0,
                     train_batch=0, train_lr=0.0, sort_queues=False, guide_depth=0, row_begin=0, row_count=0,
                     fixed_selection=False, two_level=False):
        flags = (0 if graph else _lib.PATH_NO_GRAPH) | (_lib.PATH_GUIDED if guided else 0) | \
                (_lib.PATH_TRAIN if train else 0) | (_lib.PATH_SORT_QUEUES if sort_queues else 0) | \
                (_lib.PATH_FIXED_SELECTION if fixed_selection else 0) | (_lib.PATH_TWO_LEVEL if two_level else 0)
        return _lib.PathParams(width, height, iter_begin, iter_count, seed, max_depth, rr_depth, max_batch_samples,
                               flags, None if fb64 is None else _p(fb64), guide_fraction, train_steps, train_batch,
                               train_lr, guide_depth, row_begin, row_count)

    # ------------------------------------------------------------ guide ---
    def guide_init(self, seed: int = 0):
        self._check(self.L.vmr_guide_init(self.h, int(seed)))

    def guide_set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        assert w.size == _lib.GUIDE_WEIGHTS
        self._check(self.L.vmr_guide_set_weights(self.h, _p(w)))

    def guide_get_weights(self):
        w = np.zeros(_lib.GUIDE_WEIGHTS, np.float32)
        self._check(self.L.vmr_guide_get_weights(self.h, _p(w)))
        return w

    @staticmethod
    def _rows(*arrs):
        return [np.ascontiguousarray(a, np.float32) for a in arrs]

    def guide_forward(self, pos, nrm, wo, lo, hi):
        """The network's 41 outputs per vertex (8 lobes x 5, then the
        selection logit)."""
        pos, nrm, wo, lo, hi = self._rows(pos, nrm, wo, lo, hi)
        n = pos.shape[0]
        out = np.zeros((n, _lib.GUIDE_OUTPUTS), np.float32)
        self._check(self.L.vmr_guide_forward(self.h, _p(pos), _p(nrm), _p(wo), n, _p(lo), _p(hi), _p(out)))
        return out

    def guide_gradient(self, pos, nrm, wo, omega, weight, lo, hi, bsdf_pdf=None, alpha_max=0.9):
        """Gradient and loss of a batch (vmr_guide_gradient); bsdf_pdf: the
        BSDF's density of each direction, for the full sampling density's
        loss that also trains the selection."""
        pos, nrm, wo, omega, weight, lo, hi = self._rows(pos, nrm, wo, omega, weight, lo, hi)
        pb = None if bsdf_pdf is None else np.ascontiguousarray(bsdf_pdf, np.float32)
        g = np.zeros(_lib.GUIDE_WEIGHTS, np.float32)
        loss = ctypes.c_float()
        self._check(self.L.vmr_guide_gradient(self.h, _p(pos), _p(nrm), _p(wo), _p(omega), _p(weight), _p(pb),
                                              float(alpha_max), pos.shape[0], _p(lo), _p(hi), _p(g),
                                              ctypes.byref(loss)))
        return g.astype(np.float64), loss.value

    def guide_train_step(self, pos, nrm, wo, omega, weight, lo, hi, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8,
                         bsdf_pdf=None, alpha_max=0.9):
        pos, nrm, wo, omega, weight, lo, hi = self._rows(pos, nrm, wo, omega, weight, lo, hi)
        pb = None if bsdf_pdf is None else np.ascontiguousarray(bsdf_pdf, np.float32)
        a = _lib.Adam(lr, beta1, beta2, eps)
        loss = ctypes.c_float()
        self._check(self.L.vmr_guide_train_step(self.h, _p(pos), _p(nrm), _p(wo), _p(omega), _p(weight), _p(pb),
                                                float(alpha_max), pos.shape[0], _p(lo), _p(hi), ctypes.byref(a),
                                                ctypes.byref(loss)))
        return loss.value

    @staticmethod
    def _camera(cam: dict):
        c = _lib.Camera()
        for i in range(16):
            c.m[i] = float(cam["m"][i])
        c.tan_theta_focal, c.aspect, c.focal, c.radius = (float(cam[k]) for k in
                                                         ("tan_theta_focal", "aspect", "focal", "radius"))
        return c

    def set_camera(self, cam: dict):
        """vmr_set_camera; cam may carry 'keys' ([n, 16] LocalToWorld motion
        keys, vmr_set_camera_keys)."""
        c = self._camera(cam)
        self._check(self.L.vmr_set_camera(self.h, ctypes.byref(c)))
        if cam.get("keys") is not None:
            k = np.ascontiguousarray(cam["keys"], np.float32).reshape(-1, 16)
            self._check(self.L.vmr_set_camera_keys(self.h, _p(k), k.shape[0]))

    def set_path_batch(self, paths: int):
        """Paths per wavefront batch of later render_path calls that give no
        max_batch_samples (0: the default)."""
        self._check(self.L.vmr_set_path_batch(self.h, int(paths)))

    def get_path_batch(self) -> int:
        v = ctypes.c_uint32()
        self._check(self.L.vmr_get_path_batch(self.h, ctypes.byref(v)))
        return v.value

    def autotune_path(self, width: int, height: int, iter_count: int, seed: int = 0, max_depth: int = 4,
                      rr_depth: int = 3, guided: bool = False, guide_fraction: float = 0.0, sort_queues: bool = False):
        """vmr_autotune_path: time the render at each candidate queue
        capacity and keep the fastest for this context.  Returns (best,
        {capacity: device ms})."""
        flags = (_lib.PATH_GUIDED if guided else 0) | (_lib.PATH_SORT_QUEUES if sort_queues else 0)
        p = _lib.PathParams(width, height, 0, iter_count, seed, max_depth, rr_depth, 0, flags, None,
                            guide_fraction, 0, 0, 0.0)
        cand = np.zeros(8, np.uint32)  # room for the 8 candidates
        ms = np.zeros(8, np.float32)
        n, best = ctypes.c_uint32(), ctypes.c_uint32()
        self._check(self.L.vmr_autotune_path(self.h, ctypes.byref(p), _p(cand), _p(ms), ctypes.byref(n),
                                             ctypes.byref(best)))
        return best.value, {int(c): float(m) for c, m in zip(cand[:n.value], ms[:n.value])}

    def render_path_jobs(self, jobs, iter_begin: int, iter_count: int, seed: int, max_depth: int = 4,
                         rr_depth: int = 3, max_batch_samples: int = 0, graph: bool = True):
        """Batched path-traced jobs (vmr_render_path_jobs): jobs are dicts
        with geom, width, height, camera and optionally fb (float32
        [height, width, 3], folded into).  Returns (images, stats)."""
        arr = (_lib.PathJob * len(jobs))()
        fbs = []
        for i, j in enumerate(jobs):
            fb = j.get("fb")
            if fb is None:
                fb = np.zeros((j["height"], j["width"], 3), np.float32)
            fb = np.ascontiguousarray(fb, np.float32)
            fbs.append(fb)
            arr[i].geom, arr[i].width, arr[i].height = int(j["geom"]), int(j["width"]), int(j["height"])
            arr[i].camera = self._camera(j["camera"])
            arr[i].fb = _p(fb)
        p = _lib.PathParams(0, 0, iter_begin, iter_count, seed, max_depth, rr_depth, max_batch_samples,
                            0 if graph else _lib.PATH_NO_GRAPH, None, 0.0, 0, 0, 0.0)
        st = _lib.PathStats()
        self._check(self.L.vmr_render_path_jobs(self.h, arr, len(jobs), ctypes.byref(p), ctypes.byref(st)))
        return fbs, dict(samples=st.samples, rays=st.rays, shadow_rays=st.shadow_rays,
                         graph_replays=st.graph_replays, ms=st.ms)

    def render(self, width: int, height: int, iter_begin: int, iter_count: int, seed: int, fb=None,
               max_batch_samples: int = 0, rows=None, f32: bool = False):
        """core.Render iterations [iter_begin, iter_begin+iter_count) folded
        into fb (float32 [height, width, 3]; with rows = (row_begin,
        row_count) the band of those rows, [row_count, width, 3]); f32: the
        float32-transcendental shading (VMR_RENDER_F32).  Returns (fb,
        stats)."""
        r0, nr = rows if rows is not None else (0, 0)
        if fb is None:
            fb = np.zeros((nr if rows is not None else height, width, 3), np.float32)
        fb = np.ascontiguousarray(fb, np.float32)
        p = _lib.RenderParams(width, height, iter_begin, iter_count, seed, max_batch_samples, r0, nr,
                              _lib.RENDER_F32 if f32 else 0)
        st = _lib.RenderStats()
        self._check(self.L.vmr_render(self.h, ctypes.byref(p), _p(fb), ctypes.byref(st)))
        return fb, dict(samples=st.samples, camera_rays=st.camera_rays, shadow_rays=st.shadow_rays, ms=st.ms)

    def mesh_set_transform(self, geom: int, m):
        """PolyMesh.Transform (vmr_mesh_set_transform): a column-major 4x4
        as 16 floats (math.Matrix4 order), or None to remove it."""
        if m is None:
            self._check(self.L.vmr_mesh_set_transform(self.h, geom, None))
            return
        a = np.ascontiguousarray(m, np.float32).reshape(16)
        self._check(self.L.vmr_mesh_set_transform(self.h, geom, _p(a)))

    def mesh_set_transform_keys(self, geom: int, keys):
        """PolyMesh.Transform with motion keys (vmr_mesh_set_transform_keys):
        [n, 16] column-major matrices."""
        k = np.ascontiguousarray(keys, np.float32).reshape(-1, 16)
        self._check(self.L.vmr_mesh_set_transform_keys(self.h, geom, _p(k), k.shape[0]))

    def instance_add(self, of: int, keys, bmin, bmax) -> int:
        """GeomInstance of geom `of` (vmr_instance_add); returns its geom id."""
        k = np.ascontiguousarray(keys, np.float32).reshape(-1, 16)
        lo, hi = np.asarray(bmin, np.float32), np.asarray(bmax, np.float32)
        out = ctypes.c_uint32()
        self._check(self.L.vmr_instance_add(self.h, of, _p(k), k.shape[0], _p(lo), _p(hi), ctypes.byref(out)))
        return out.value

    def proc_add(self, children, keys, bmin, bmax) -> int:
        """Proc over the child geoms (vmr_proc_add); keys None: identity."""
        ch = np.ascontiguousarray(children, np.uint32)
        k = None if keys is None else np.ascontiguousarray(keys, np.float32).reshape(-1, 16)
        lo, hi = np.asarray(bmin, np.float32), np.asarray(bmax, np.float32)
        out = ctypes.c_uint32()
        self._check(self.L.vmr_proc_add(self.h, _p(ch), ch.size, None if k is None else _p(k),
                                        0 if k is None else k.shape[0], _p(lo), _p(hi), ctypes.byref(out)))
        return out.value

    def load_scene(self, scene: dict):
        """Upload a render scene (vermeer_gb300.scenes format): meshes with
        their shading (and 'transform' or 'transform_keys'), spheres,
        instances ({'instance': i, 'keys', 'bmin', 'bmax'}) and Procs
        ({'proc': [child indices], 'keys', 'bmin', 'bmax'}), the two-level
        scene over every entry but a Proc's children, materials, lights,
        camera.  Returns the geom ids (one per entry)."""
        ids = [None] * len(scene["meshes"])
        for i, m in enumerate(scene["meshes"]):
            if "sphere" in m:  # an analytic sphere geom: (cx, cy, cz, radius)
                ids[i] = self.sphere_add(m["sphere"][:3], m["sphere"][3])
            elif "verts" in m:
                g = self.mesh_build(m["verts"], m["idxp"], keys=m.get("keys", 1),
                                    ray_bias=m.get("ray_bias", 0.0),
                                    motion_mode=m.get("motion_mode", MOTION_FAITHFUL),
                                    shader_idx=m.get("face_shader"))
                if m.get("transform_keys") is not None:
                    self.mesh_set_transform_keys(g, m["transform_keys"])
                elif m.get("transform") is not None:
                    self.mesh_set_transform(g, m["transform"])
                ids[i] = g
        for i, m in enumerate(scene["meshes"]):
            if "instance" in m:
                ids[i] = self.instance_add(ids[m["instance"]], m["keys"], m["bmin"], m["bmax"])
            elif "proc" in m:
                ids[i] = self.proc_add([ids[c] for c in m["proc"]], m.get("keys"), m["bmin"], m["bmax"])
        children = {c for m in scene["meshes"] if "proc" in m for c in m["proc"]}
        self.scene_build([g for i, g in enumerate(ids) if i not in children])
        self.set_shaders(scene["shaders"])
        for g, m in zip(ids, scene["meshes"]):
            if "instance" not in m and "proc" not in m:
                self.mesh_set_shading(g, m["shaders"], m.get("normals"))
                if m.get("motion_normals") is not None:
                    self.mesh_set_motion_normals(g, m["motion_normals"])
        self.set_lights([dict(l, geom=ids[l["mesh"]]) for l in scene["lights"]])
        self.set_disk_lights([dict(d, geom=ids[d["mesh"]]) for d in scene.get("disk_lights", [])])
        self.set_sphere_lights([dict(d, geom=ids[d["mesh"]]) for d in scene.get("sphere_lights", [])])
        self.set_quad_lights([dict(q, geom=ids[q["mesh"]]) for q in scene.get("quad_lights", [])])
        self.set_env_light(scene.get("env", (0.0, 0.0, 0.0)))
        self.set_camera(scene["camera"])
        self.set_pixel_filter(**scene.get("pixel_filter", {"kind": _lib.FILTER_BOX}))
        return ids

    def load_vnf(self, path: str, motion_fixed: bool = False) -> dict:
        """Load a .vnf scene file (vmr_load_vnf): geometry, materials,
        lights, camera and pixel filter.  Returns the Globals and output
        settings the file gives (width, height, max_iter, outputs)."""
        info = _lib.VnfInfo()
        self._check(self.L.vmr_load_vnf(self.h, str(path).encode(), _lib.VNF_MOTION_FIXED if motion_fixed else 0,
                                        ctypes.byref(info)))
        return dict(width=info.width, height=info.height, max_iter=info.max_iter, n_geoms=info.n_geoms,
                    n_shaders=info.n_shaders, n_lights=info.n_lights, camera=info.camera.decode(),
                    output_hdr=info.output_hdr.decode(), output_float=info.output_float.decode())

    def get_camera_keys(self) -> np.ndarray:
        """The camera's LocalToWorld keys ([n, 16] column-major)."""
        n = ctypes.c_uint32()
        self._check(self.L.vmr_get_camera_keys(self.h, None, 0, ctypes.byref(n)))
        out = np.zeros((n.value, 16), np.float32)
        self._check(self.L.vmr_get_camera_keys(self.h, _p(out), n.value, ctypes.byref(n)))
        return out

    def get_camera(self) -> dict:
        c = _lib.Camera()
        self._check(self.L.vmr_get_camera(self.h, ctypes.byref(c)))
        return dict(m=np.array(c.m[:], np.float32), tan_theta_focal=np.float32(c.tan_theta_focal),
                    aspect=np.float32(c.aspect), focal=np.float32(c.focal), radius=np.float32(c.radius))

    def encode_rgbe(self, fb):
        """OutputHDR's pixel bytes of a float framebuffer [h, w, 3] (numpy
        on the host, or a CUDA torch tensor), encoded on the GPU: uint8
        [h, w, 4] in file order (scanline 0 = the bottom image row)."""
        if hasattr(fb, "is_cuda") and fb.is_cuda:
            import torch
            t = fb.contiguous().float()
            h, w = t.shape[:2]
            out = torch.empty((h, w, 4), dtype=torch.uint8, device=t.device)
            self._check(self.L.vmr_encode_rgbe(self.h, ctypes.c_void_p(t.data_ptr()), w, h,
                                               _lib.IO_DEVICE_IN | _lib.IO_DEVICE_OUT, ctypes.c_void_p(out.data_ptr())))
            return out
        fb = np.ascontiguousarray(fb, np.float32)
        h, w = fb.shape[:2]
        out = np.empty((h, w, 4), np.uint8)
        self._check(self.L.vmr_encode_rgbe(self.h, _p(fb), w, h, 0, _p(out)))
        return out

    def write_hdr(self, path: str, fb):
        """The OutputHDR driver (builtin/driver/outputhdr.go): a Radiance
        .hdr file of the framebuffer, pixels encoded on the GPU."""
        px = self.encode_rgbe(fb)
        if not isinstance(px, np.ndarray):
            px = px.cpu().numpy()
        h, w = px.shape[:2]
        with open(path, "wb") as f:
            f.write(f"#?RADIANCE\n# vermeer_gb300\nFORMAT=32-bit_rle_rgbe\n\n+Y {h} +X {w}\n".encode())
            f.write(px.tobytes())

    def set_pixel_filter(self, kind: int, res: int = 0, width: float = 0.0, peak: float = 0.0):
        """The render's pixel filter (GaussianFilter / AiryFilter node):
        kind FILTER_BOX (none), FILTER_GAUSSIAN or FILTER_AIRY; res, width
        and peak <= 0 take the nodes' defaults."""
        f = _lib.PixelFilter(int(kind), int(res), float(width), float(peak))
        self._check(self.L.vmr_set_pixel_filter(self.h, ctypes.byref(f)))
