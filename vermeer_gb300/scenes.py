"""Seeded synthetic inputs with the shapes of the benchmark workloads.

No scene files ship with the reference, so every workload is generated here
from a seed.  The generator is defined once and used by the tests, the
benchmark and the smoke check, so the CUDA path and the CPU oracle always
consume the same float32 bits.

PRNG: SplitMix64 seeded per stream.  A uniform float is the top 24 bits of a
64-bit draw times 2^-24 (exact in float32).  Directions uniform on the
sphere use z = 1-2u, phi = 2*pi*v in float64, rounded to float32 at the end.
"""
from __future__ import annotations

import numpy as np

_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """n draws of SplitMix64 started at state seed*2^32 + stream."""
    with np.errstate(over="ignore"):
        base = np.uint64((seed << 32) + stream)
        z = base + _GOLD * np.arange(1, n + 1, dtype=np.uint64)
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, n: int, stream: int = 0) -> np.ndarray:
    """Uniform float64 in [0,1) with 24 random bits (exact in float32)."""
    return (splitmix64(seed, n, stream) >> np.uint64(40)).astype(np.float64) * (2.0 ** -24)


def unit_sphere(seed: int, n: int, stream: int) -> np.ndarray:
    u = uniform(seed, n, stream)
    v = uniform(seed, n, stream + 1)
    z = 1.0 - 2.0 * u
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = 2.0 * np.pi * v
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1)


def triangle_soup(n_tris: int, seed: int, lo=0.0, hi=1.0, edge=0.005) -> tuple[np.ndarray, np.ndarray]:
    """A soup of n_tris triangles: centroid uniform in [lo,hi)^3, each vertex
    at centroid + edge * (a direction uniform on the sphere).  Returns
    (verts float32 [3n,3], idxp uint32 [3n]) - the PolyMesh form without
    FaceIdx, whose face i uses vertices 3i..3i+2 (polymesh/init.go:108-130)."""
    c = lo + (hi - lo) * np.stack([uniform(seed, n_tris, s) for s in range(3)], axis=1)
    verts = np.empty((n_tris, 3, 3), np.float64)
    for k in range(3):
        verts[:, k, :] = c + edge * unit_sphere(seed, n_tris, 10 + 2 * k)
    verts = verts.astype(np.float32).reshape(-1, 3)
    return verts, np.arange(verts.shape[0], dtype=np.uint32)


def incoherent_rays(n: int, seed: int, lo=0.0, hi=1.0) -> np.ndarray:
    """n rays [n,8] = px py pz dx dy dz tmax time: origins uniform in the
    cube, directions uniform on the sphere, tmax = +inf, time = 0."""
    o = lo + (hi - lo) * np.stack([uniform(seed, n, 100 + s) for s in range(3)], axis=1)
    d = unit_sphere(seed, n, 110)
    rays = np.empty((n, 8), np.float32)
    rays[:, 0:3] = o
    rays[:, 3:6] = d
    rays[:, 6] = np.inf
    rays[:, 7] = 0.0
    return rays


def coherent_rays(res: int, eye=(0.5, 0.5, -1.2), target=(0.5, 0.5, 0.5), fov_deg=40.0) -> np.ndarray:
    """res x res pinhole primaries through pixel centres, directions
    normalised in float64 then rounded to float32, tmax = +inf."""
    eye = np.asarray(eye, np.float64)
    w = eye - np.asarray(target, np.float64)
    w /= np.linalg.norm(w)
    up = np.array([0.0, 1.0, 0.0])
    u = np.cross(up, w)
    u /= np.linalg.norm(u)
    v = np.cross(w, u)
    tanh = np.tan(np.radians(fov_deg) / 2)
    s = (np.arange(res) + 0.5) / res * 2.0 - 1.0
    sx, sy = np.meshgrid(s, -s)
    d = sx[..., None] * tanh * u + sy[..., None] * tanh * v - w
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    rays = np.empty((res * res, 8), np.float32)
    rays[:, 0:3] = eye
    rays[:, 3:6] = d.reshape(-1, 3)
    rays[:, 6] = np.inf
    rays[:, 7] = 0.0
    return rays


def motion_soup(n_tris: int, seed: int, velocity=0.05, edge=0.005):
    """Two-key linear motion: key 1 = key 0 + a per-triangle velocity drawn
    uniformly in a ball of radius `velocity`.  Returns verts [2*3n,3]
    (key-major PointArray layout) and idxp."""
    v0, idxp = triangle_soup(n_tris, seed, edge=edge)
    d = unit_sphere(seed, n_tris, 40) * (velocity * np.cbrt(uniform(seed, n_tris, 42)))[:, None]
    v1 = (v0.reshape(n_tris, 3, 3).astype(np.float64) + d[:, None, :]).astype(np.float32).reshape(-1, 3)
    return np.concatenate([v0, v1], axis=0), idxp


# ---------------------------------------------------------------- renders ---
def lookat_camera(eye, target, up, fov_deg: float, aspect: float, focal: float = 12.0) -> dict:
    """Camera node of type LookAt with one key (builtin/camera/camera.go:
    80-98, 109-193): W = normalize(From - To), u = normalize(Up x W),
    v = normalize(u x W), LocalToWorld = Translate(From) * Basis(u, v, W)
    (column-major), TanThetaFocal = tan(degToRad(Fov/2)) * Focal."""
    f32 = np.float32
    eye, target, up = (np.asarray(a, f32) for a in (eye, target, up))

    def norm(a):
        a = a.astype(f32)
        return (a * (f32(1.0) / np.sqrt(np.dot(a, a), dtype=f32))).astype(f32)

    W = norm(eye - target)
    u = norm(np.cross(up, W).astype(f32))
    v = norm(np.cross(u, W).astype(f32))
    m = np.zeros(16, f32)
    m[0:3], m[4:7], m[8:11], m[12:15], m[15] = u, v, W, eye, 1.0
    pi = f32(3.14159265358)
    half = f32(fov_deg) / f32(2)
    tan = f32(np.tan(np.float64(half * pi / f32(180.0))))
    return dict(m=m, tan_theta_focal=f32(tan * f32(focal)), aspect=f32(aspect), focal=f32(focal), radius=f32(0))


def _tri_light_mesh(p0, p1, p2):
    """The emissive mesh a TriLight adds (builtin/light/triangle.go:537-565):
    three vertices with the face normal at each."""
    p = np.asarray([p0, p1, p2], np.float32)
    n = np.cross(p[1] - p[0], p[2] - p[0]).astype(np.float32)
    n = n / np.sqrt(np.dot(n, n), dtype=np.float32)
    return p, np.arange(3, dtype=np.uint32), np.tile(n, (3, 1)).astype(np.float32)


def _rect_y(x0, z0, x1, z1, y):
    """Two triangles of the rectangle [x0,x1] x [z0,z1] at height y, wound so
    their geometric normal points down (-y)."""
    return [(x0, y, z0), (x1, y, z0), (x1, y, z1), (x0, y, z0), (x1, y, z1), (x0, y, z1)]


def small_room(n_tris: int = 16384, seed: int = 1, res: int = 256, n_albedo: int = 8, light_samples: int = 1) -> dict:
    """The small-room configuration: a closed 2x2x2 box (open at the camera
    side) with an 0.8 x 0.5 opening in the ceiling, a soup of n_tris
    triangles with centroids uniform in the inner 1.6^3 box and vertices at
    centroid + 0.02 x a direction on the sphere, two TriLight panels (0.3 x
    0.4 right triangles, normals down) of radiance 10 recessed above the
    opening at heights 1.05 and 1.10, Lambert (ShaderStd with
    DiffuseRoughness 0) albedos uniform in [0.3, 0.8], and a pinhole camera at
    fov 40.

    The layout keeps clear of two properties of the reference.  A shading
    point in or near a light's plane gives sampleSphericalTriangle
    (builtin/light/triangle.go:380-418) a degenerate spherical triangle whose
    float32 side-to-angle conversion takes the square root of a negative
    number, so the sample is NaN; no surface here crosses either panel's
    plane, and the panels are at different heights so that neither samples
    the other edge-on.  And two geoms with the same box centroid make the
    top-level split of qbvh/build.go:34-43 (pivot n/2+1 for flat centroid
    bounds) recurse forever, so the panels are not the two halves of one
    quad."""
    f = np.float32
    hx, hz = 0.4, 0.25
    tris = []
    tris += [(-1, -1, -1), (-1, -1, 1), (1, -1, 1), (-1, -1, -1), (1, -1, 1), (1, -1, -1)]  # floor, up
    for x0, z0, x1, z1 in ((-1, -1, 1, -hz), (-1, hz, 1, 1), (-1, -hz, -hx, hz), (hx, -hz, 1, hz)):
        tris += _rect_y(x0, z0, x1, z1, 1.0)  # ceiling around the opening, down
    tris += [(-1, -1, 1), (-1, 1, 1), (1, 1, 1), (-1, -1, 1), (1, 1, 1), (1, -1, 1)]  # back, -z
    tris += [(-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, -1), (-1, 1, 1), (-1, -1, 1)]  # left, +x
    tris += [(1, -1, -1), (1, -1, 1), (1, 1, 1), (1, -1, -1), (1, 1, 1), (1, 1, -1)]  # right, -x
    rv = np.asarray(tris, f)
    face_shader = np.asarray([0] * 2 + [1] * 8 + [2] * 2 + [3] * 2 + [4] * 2, np.uint8)
    room = dict(verts=rv, idxp=np.arange(rv.shape[0], dtype=np.uint32), face_shader=face_shader,
                shaders=[0, 1, 2, 3, 4])
    sv, sidx = triangle_soup(n_tris, seed, lo=-0.8, hi=0.8, edge=0.02)
    soup = dict(verts=sv, idxp=sidx, shaders=list(range(5, 5 + n_albedo)),
                face_shader=(splitmix64(seed, n_tris, 300) % np.uint64(n_albedo)).astype(np.uint8))
    alb = 0.3 + 0.5 * np.stack([uniform(seed, 5 + n_albedo, 310 + k) for k in range(3)], axis=1)
    shaders = [dict(diffuse_colour=alb[i], diffuse_strength=1.0, diffuse_roughness=0.0) for i in range(5 + n_albedo)]
    light_shader = len(shaders)
    shaders.append(dict(emission_colour=(1.0, 1.0, 1.0), emission_strength=10.0, diffuse_colour=(0.0, 0.0, 0.0),
                        diffuse_strength=1.0, diffuse_roughness=0.0))
    y0, y1 = f(1.05), f(1.10)
    panels = (((-0.35, y0, -0.2), (-0.05, y0, -0.2), (-0.05, y0, 0.2)),
              ((0.05, y1, -0.2), (0.35, y1, 0.2), (0.05, y1, 0.2)))
    meshes = [room, soup]
    lights = []
    for tri in panels:
        pv, pi, pn = _tri_light_mesh(*tri)
        meshes.append(dict(verts=pv, idxp=pi, normals=pn, shaders=[light_shader]))
        lights.append(dict(p0=pv[0], p1=pv[1], p2=pv[2], samples=light_samples, shader=light_shader,
                           mesh=len(meshes) - 1))
    cam = lookat_camera((0.0, 0.0, -3.4), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0, 1.0)
    return dict(meshes=meshes, shaders=shaders, lights=lights, camera=cam, res=res)
